// FP64 peak probe: the denominator of the plain path's roofline.  GB300's
// FP64 rate is not among the measured peaks, so the benchmark
// measures it in the same run with these two kernels: independent DFMA
// chains on the CUDA cores, and independent m8n8k4 DMMA accumulators on the
// FP64 tensor path.  Both run a fixed, in-bounds amount of work per thread.
#include "api_internal.h"
#include "common.cuh"

namespace uvt {
namespace {

__global__ void __launch_bounds__(256) probe_dfma(double *out, double seed, int iters) {
  double x[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) x[i] = seed + threadIdx.x * 1e-9 + i;
  const double m = 0.999999, c = 1e-7;
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int i = 0; i < 16; ++i) x[i] = fma(x[i], m, c);
  double s = 0;
#pragma unroll
  for (int i = 0; i < 16; ++i) s += x[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void __launch_bounds__(256) probe_dmma(double *out, double seed, int iters) {
  double d[4][2];
#pragma unroll
  for (int j = 0; j < 4; ++j) d[j][0] = d[j][1] = 0.0;
  const double a = seed + threadIdx.x * 1e-9, b = seed - threadIdx.x * 1e-9;
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int j = 0; j < 4; ++j)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                   : "+d"(d[j][0]), "+d"(d[j][1])
                   : "d"(a), "d"(b));
  double s = 0;
#pragma unroll
  for (int j = 0; j < 4; ++j) s += d[j][0] + d[j][1];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace
}  // namespace uvt

using namespace uvt;

extern "C" UVATRMM_API int uvatrmm_probe_fp64_peak(uvatrmm_handle_t h, int engine, double *tflops) {
  if (!(h = resolve(h))) return uvatrmm_last_status();
  if (!tflops || (engine != UVATRMM_ENGINE_DFMA && engine != UVATRMM_ENGINE_DMMA))
    return fail(UVATRMM_EINVAL, "invalid arguments");
  std::lock_guard<std::mutex> g(h->mu);
  const int blocks = h->num_sms * 8, threads = 256;
  double *out = static_cast<double *>(workspace(h, 3, (size_t)blocks * threads * 8));
  if (!out) return uvatrmm_last_status();
  // flops per thread per iteration: DFMA 16 chains x 2; DMMA 4 x (8*8*4*2)/32.
  // About 100 ms per launch at GB300's FP64 rate, best of three after a
  // warm-up launch, so the clocks have settled.
  const double fpt = engine == UVATRMM_ENGINE_DFMA ? 32.0 : 64.0;
  const int iters = engine == UVATRMM_ENGINE_DFMA ? 12000 : 6000;
  auto launch = [&](int it) {
    if (engine == UVATRMM_ENGINE_DFMA) probe_dfma<<<blocks, threads, 0, h->stream>>>(out, 1.0, it);
    else probe_dmma<<<blocks, threads, 0, h->stream>>>(out, 1.0, it);
  };
  launch(iters / 10);
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(h->ev0, h->stream);
    launch(iters);
    cudaEventRecord(h->ev1, h->stream);
    cudaError_t e = cudaEventSynchronize(h->ev1);
    if (e != cudaSuccess) return cuda_fail(e, "fp64 probe");
    float ms;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    if (ms < best) best = ms;
  }
  *tflops = fpt * (double)blocks * threads * iters / (best * 1e-3) / 1e12;
  return ok();
}
