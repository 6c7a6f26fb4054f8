// uvatrmm_dtrmm_device_noalloc: the plain FP64 TRMM for callers that cannot
// allocate device memory.
//
// The in-place device TRMM needs scratch: a copy of B for the kernel to read
// while it writes the result into B, A when A is not 16-byte aligned with an
// even leading dimension, and two control words (the tile counter of the
// dynamic schedule and the kernel's status word).  The ordinary entry point
// takes that scratch from the handle's workspace (cudaMalloc).  This one
// takes it from g_noalloc_scratch, a fixed file-scope device array, so a call
// allocates nothing: no cudaMalloc, no cudaFree, no allocating library call.
//
// The array is part of this file's device module, so a GPU reserves it when
// the library's device code is loaded there -- at the first call on that
// device under CUDA's default lazy module loading, at context creation under
// CUDA_MODULE_LOADING=EAGER -- and holds it until the process exits.  Its
// device address is looked up once per device (cudaGetSymbolAddress, with
// that device current) on the first call there; make that first call before
// any stream capture.  All calls on a device share the array and it keeps the last
// call's contents: the control words are cleared by each call, and calls
// whose work overlaps on the GPU (different streams, or host threads without
// ordering between them) race on it.
#include <mutex>
#include <string>

#include "api_internal.h"
#include "common.cuh"
#include "trmm_fp64.cuh"

namespace uvt {
namespace {

constexpr size_t kNoAllocBytes = size_t(64) << 20;  // 64 MiB per device
constexpr size_t kNoAllocCtl = 256;                  // control words, then staged operands
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
unsigned char *g_noalloc_addr[kMaxDevices] = {};

// Device address of the scratch array on device `dev` (the current device).
int noalloc_scratch(int dev, unsigned char **addr) {
  std::lock_guard<std::mutex> g(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "no-allocation scratch lookup (cudaGetSymbolAddress)");
    g_noalloc_addr[dev] = static_cast<unsigned char *>(p);
  }
  *addr = g_noalloc_addr[dev];
  return UVATRMM_OK;
}

}  // namespace
}  // namespace uvt

using namespace uvt;

extern "C" UVATRMM_API int uvatrmm_dtrmm_device_noalloc(int layout, int side, int uplo, int transa, int diag,
                                                        int64_t m, int64_t n, double alpha, const double *dA,
                                                        int64_t lda, double *dB, int64_t ldb, void *stream) {
  if (int bad = check_args(layout, side, uplo, transa, diag, m, n, lda, ldb))
    return fail(UVATRMM_EINVAL, "parameter " + std::to_string(bad) + " had an illegal value");
  const Trmm t = normalise(layout, side, uplo, transa, diag, m, n, alpha);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (t.m == 0 || t.n == 0) return ok();
  const int64_t ka = t.side == CblasLeft ? t.m : t.n;
  const bool stage_a = (reinterpret_cast<uintptr_t>(dA) % 16 != 0) || (lda % 2 != 0);
  // Every dimension is bounded by a division before any size is multiplied
  // out, so no product below can overflow.
  const int64_t avail = (int64_t)(kNoAllocBytes - kNoAllocCtl);
  bool fits = t.m <= avail / 8 && ka <= avail / 8;
  const int64_t lb = fits ? round_up(t.m, 16) : 0, la = fits ? round_up(ka, 16) : 0;
  fits = fits && t.n <= avail / (8 * lb) && (!stage_a || ka <= avail / (8 * la));
  const size_t b_bytes = fits ? (size_t)round_up(lb * t.n * 8, 256) : 0;
  const size_t a_bytes = fits && stage_a ? (size_t)la * ka * 8 : 0;
  fits = fits && kNoAllocCtl + b_bytes + a_bytes <= kNoAllocBytes;
  if (alpha != 0.0 && !fits)
    return fail(UVATRMM_EINVAL, "no-allocation TRMM: the problem needs more scratch than the fixed " +
                                    std::to_string(kNoAllocBytes) +
                                    " bytes (B staged as round_up(rows,16) x cols doubles, plus A when it is not "
                                    "16-byte aligned with an even leading dimension)");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return fail(UVATRMM_EUNSUPPORTED, "device index out of range");
  int major = 0, minor = 0, sms = 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (major != 10 || minor != 3) return fail(UVATRMM_EUNSUPPORTED, "device is not sm_103 (GB300)");
  if (alpha == 0.0) {
    e = cudaMemset2DAsync(dB, ldb * 8, 0, t.m * 8, t.n, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? ok() : cuda_fail(e, "zero fill");
  }
  unsigned char *base = nullptr;
  if (int rc = noalloc_scratch(dev, &base)) return rc;
  int *ctl = reinterpret_cast<int *>(base);  // [0] tile counter, [1] status word
  double *Bs = reinterpret_cast<double *>(base + kNoAllocCtl);
  double *As = reinterpret_cast<double *>(base + kNoAllocCtl + b_bytes);
  e = cudaMemsetAsync(ctl, 0, 2 * sizeof(int), st);
  if (e == cudaSuccess)
    e = cudaMemcpy2DAsync(Bs, lb * 8, dB, ldb * 8, t.m * 8, t.n, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess && stage_a)
    e = cudaMemcpy2DAsync(As, la * 8, dA, lda * 8, ka * 8, ka, cudaMemcpyDeviceToDevice, st);
  if (e != cudaSuccess) return cuda_fail(e, "staging into the no-allocation scratch");
  const double *A = stage_a ? As : dA;
  const int64_t lA = stage_a ? la : lda;

  Fp64Launch L;
  const bool lower = (t.uplo == CblasLower) != (t.trans != 0);
  L.M = t.m;
  L.N = t.n;
  L.K = ka;
  L.alpha = t.alpha;
  L.C = dB;
  L.ldc = ldb;
  L.unit = t.unit;
  L.tri_lower = lower;
  if (t.side == CblasLeft) {
    L.tri_left = true;
    L.xl = MatRef{A, ka, ka, lA};
    L.lft_kmajor = t.trans != 0;
    L.xr = MatRef{Bs, t.m, t.n, lb};
    L.rgt_kmajor = true;
  } else {
    L.tri_left = false;
    L.xl = MatRef{Bs, t.m, t.n, lb};
    L.lft_kmajor = false;
    L.xr = MatRef{A, ka, ka, lA};
    L.rgt_kmajor = t.trans == 0;
  }
  L.engine = UVATRMM_ENGINE_DFMA;
  L.schedule = UVATRMM_SCHED_DYNAMIC;
  L.shape = UVATRMM_SHAPE_TRAPEZOID;
  L.tile = 0;
  L.counter = ctl;
  L.status = ctl + 1;
  L.num_sms = sms;
  const char *why = nullptr;
  int rc = launch_trmm_fp64(L, st, &why);
  if (rc != UVATRMM_OK) return fail(rc, why ? why : "kernel launch failed");
  int flags = 0;
  e = cudaMemcpyAsync(&flags, ctl + 1, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "no-allocation TRMM");
  if (flags & KERR_WAIT_TIMEOUT) return fail(UVATRMM_ETIMEOUT, "a kernel wait expired (bounded spin limit)");
  if (flags) return fail(UVATRMM_EDEVICE, "kernel reported error flags " + std::to_string(flags));
  return ok();
}
