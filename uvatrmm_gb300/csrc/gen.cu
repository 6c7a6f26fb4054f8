// Input generators, ||C||_inf, error norms and the reference's row mappings.
#include <cmath>
#include <cstdint>

#include "api_internal.h"
#include "common.cuh"

namespace uvt {
namespace {

// Element (i, j) of the reference's n x n row-major input
// (UVaTRMM/src/mm_triangular_common.c:1782-1805, -DMININUMS=1): the
// reciprocal of ((i*n + j) mod 2341) + 1, and 0 above the diagonal of the
// triangular A.  Indices are 64-bit (the reference's int overflows from n = 46341).
__global__ void gen_consecutive_kernel(int64_t n, int triangular, double *d) {
  const int64_t total = n * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / n, j = e - i * n;
    double v = 0.0;
    if (!(triangular && j > i)) v = 1.0 / (double)((i * n + j) % 2341 + 1);
    d[e] = v;
  }
}

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

// Counter-based uniform[-1,1): splitmix64 finaliser over a (seed, stream)
// key plus (idx+1) * golden ratio; top 53 bits scaled to [0,1), then 2u-1.
// Optional exponent in [-spread, spread] from an independent key.
__global__ void gen_uniform_kernel(uint64_t seed, uint64_t stream, int64_t rows, int64_t cols, double *d,
                                   int64_t rs, int64_t cs, int tri, double fill, int spread) {
  const uint64_t key = mix64(seed * 0x9E3779B97F4A7C15ULL + stream * 0xD1B54A32D192ED03ULL + 0x632BE59BD9B4E019ULL);
  const uint64_t key2 = mix64(seed * 0x9E3779B97F4A7C15ULL + stream * 0xD1B54A32D192ED03ULL + 0x2545F4914F6CDD1DULL);
  const int64_t total = rows * cols;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    // Walk in storage order so writes coalesce for either layout.
    int64_t i, j;
    if (cs == 1 || rs >= cs) { i = e / cols; j = e - i * cols; }
    else { j = e / rows; i = e - j * rows; }
    const bool keep = tri == 0 || (tri == 'L' && j <= i) || (tri == 'U' && j >= i);
    double v = fill;
    if (keep) {
      const uint64_t idx = (uint64_t)(i * cols + j);
      const uint64_t z = mix64(key + (idx + 1) * 0x9E3779B97F4A7C15ULL);
      v = (double)(z >> 11) * 0x1.0p-53 * 2.0 - 1.0;
      if (spread > 0) {
        const uint64_t z2 = mix64(key2 + (idx + 1) * 0x9E3779B97F4A7C15ULL);
        v = ldexp(v, (int)(z2 % (uint64_t)(2 * spread + 1)) - spread);
      }
    }
    d[i * rs + j * cs] = v;
  }
}

// One warp per row: sum of |C[i, :]|, then a max via the ordered bit
// pattern of non-negative doubles.
__global__ void row_abs_max_kernel(int64_t rows, int64_t cols, const double *C, int64_t ldc,
                                   unsigned long long *out) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x / 32);
  for (int64_t i = blockIdx.x * (int64_t)(blockDim.x / 32) + threadIdx.x / 32; i < rows; i += warps) {
    double s = 0.0;
    for (int64_t j = lane; j < cols; j += 32) s += fabs(C[i * ldc + j]);
#pragma unroll
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) atomicMax(out, (unsigned long long)__double_as_longlong(s));
  }
}

// Sums of (X - R)^2 and R^2 over a column-major rows x cols block.
__global__ void diff_norms_kernel(int64_t rows, int64_t cols, const double *X, int64_t ldx, const double *R,
                                  int64_t ldr, double *out) {
  double se = 0.0, sr = 0.0;
  const int64_t total = rows * cols;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = e / rows, i = e - j * rows;
    const double r = R[i + j * ldr], x = X[i + j * ldx];
    se += (x - r) * (x - r);
    sr += r * r;
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    se += __shfl_xor_sync(0xffffffffu, se, o);
    sr += __shfl_xor_sync(0xffffffffu, sr, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(out, se);
    atomicAdd(out + 1, sr);
  }
}

int grid_for(int64_t work, uvatrmm_handle_t h) {
  int64_t g = (work + 255) / 256;
  int64_t cap = (int64_t)h->num_sms * 8;
  return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

}  // namespace

// Frobenius error of X against R (column-major device blocks); host helper
// used by the Ozaki path's error report.
int rel_frobenius(uvatrmm_handle_t h, int64_t rows, int64_t cols, const double *X, int64_t ldx, const double *R,
                  int64_t ldr, double *rel) {
  double *acc = static_cast<double *>(workspace(h, 3, 64));
  if (!acc) return UVATRMM_ENOMEM;
  cudaMemsetAsync(acc, 0, 16, h->stream);
  diff_norms_kernel<<<grid_for(rows * cols, h), 256, 0, h->stream>>>(rows, cols, X, ldx, R, ldr, acc);
  double host[2] = {0, 0};
  cudaError_t e = cudaMemcpyAsync(host, acc, 16, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return cuda_fail(e, "error norm");
  *rel = host[1] > 0 ? std::sqrt(host[0] / host[1]) : std::sqrt(host[0]);
  return UVATRMM_OK;
}

}  // namespace uvt

using namespace uvt;

namespace {

// get_rows_before (UVaTRMM/src/mm_mapping.c:177-181).
uint64_t rows_before(double ideal, int k) {
  double num = -1.0 + std::sqrt(1.0 + 8.0 * (k * ideal));
  return num > 0 ? (uint64_t)(std::floor(num) / 2.0) : 0;
}

}  // namespace

extern "C" {

// map_regular (UVaTRMM/src/mm_mapping.c:27-67) and map_balanced
// (UVaTRMM/src/mm_mapping.c:319-366, helpers :120-181), with the
// reference's integer widths: the triangle's element count is an unsigned
// int and the ideal block is ceil(count / P) as an unsigned int.
UVATRMM_API int uvatrmm_map_rows(int schedule, uint64_t n, uint32_t P, uint32_t idx, uint64_t *begin,
                                 uint64_t *size) {
  if (!begin || !size || P == 0 || idx >= P) return fail(UVATRMM_EINVAL, "invalid mapping arguments");
  if (schedule == UVATRMM_SCHED_REG) {
    uint64_t eq = n / P, rem = n % P;
    if (eq < 1) eq = 1;
    if (P != 1 && eq * P > n) return fail(UVATRMM_EINVAL, "too few rows for map_regular");
    *begin = (uint64_t)idx * eq;
    *size = eq + (idx == P - 1 ? rem : 0);
    return ok();
  }
  if (schedule == UVATRMM_SCHED_BALANCED) {
    unsigned int count = (unsigned int)(0.5 * (double)(n * (n + 1)));
    double ideal_d = (double)count / (double)P;
    if (ideal_d < 1) return fail(UVATRMM_EINVAL, "ideal block size smaller than one");
    unsigned int ideal = (unsigned int)std::ceil(ideal_d);
    unsigned int rb = (unsigned int)rows_before((double)ideal, (int)idx);
    unsigned int re = (unsigned int)rows_before((double)ideal, (int)idx + 1);
    uint64_t b = rb, s = (unsigned int)(re - rb);
    if (idx == 0) {
      b = 0;
      s = P > 1 ? rows_before((double)ideal, 1) : n;
    }
    if (n > 1 && idx == P - 1) s = n - b;
    if (s == 0) return fail(UVATRMM_EINVAL, "empty block in map_balanced");
    *begin = b;
    *size = s;
    return ok();
  }
  return fail(UVATRMM_EINVAL, "schedule must be REG or BALANCED");
}

UVATRMM_API int uvatrmm_gen_consecutive(uvatrmm_handle_t h, int64_t n, int triangular, double *d) {
  if (!(h = resolve(h))) return uvatrmm_last_status();
  if (n < 0 || (!d && n > 0)) return fail(UVATRMM_EINVAL, "invalid arguments");
  if (n == 0) return ok();
  gen_consecutive_kernel<<<grid_for(n * n, h), 256, 0, h->stream>>>(n, triangular, d);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? ok() : cuda_fail(e, "gen_consecutive");
}

UVATRMM_API int uvatrmm_gen_uniform(uvatrmm_handle_t h, uint64_t seed, uint64_t stream, int64_t rows, int64_t cols,
                                    double *d, int64_t rs, int64_t cs, int tri, double fill, int spread) {
  if (!(h = resolve(h))) return uvatrmm_last_status();
  if (rows < 0 || cols < 0 || spread < 0 || spread > 1000 || (tri != 0 && tri != 'L' && tri != 'U'))
    return fail(UVATRMM_EINVAL, "invalid arguments");
  if (rows == 0 || cols == 0) return ok();
  gen_uniform_kernel<<<grid_for(rows * cols, h), 256, 0, h->stream>>>(seed, stream, rows, cols, d, rs, cs, tri, fill,
                                                                       spread);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? ok() : cuda_fail(e, "gen_uniform");
}

UVATRMM_API int uvatrmm_inf_norm(uvatrmm_handle_t h, int64_t rows, int64_t cols, const double *dC, int64_t ldc,
                                 double *norm) {
  if (!(h = resolve(h))) return uvatrmm_last_status();
  if (!norm || rows < 0 || cols < 0 || ldc < cols) return fail(UVATRMM_EINVAL, "invalid arguments");
  *norm = 0.0;
  if (rows == 0 || cols == 0) return ok();
  std::lock_guard<std::mutex> g(h->mu);
  unsigned long long *acc = static_cast<unsigned long long *>(workspace(h, 3, 64));
  if (!acc) return uvatrmm_last_status();
  cudaMemsetAsync(acc, 0, 8, h->stream);
  row_abs_max_kernel<<<grid_for(rows * 32, h), 256, 0, h->stream>>>(rows, cols, dC, ldc, acc);
  unsigned long long bits = 0;
  cudaError_t e = cudaMemcpyAsync(&bits, acc, 8, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return cuda_fail(e, "inf norm");
  double v;
  memcpy(&v, &bits, 8);
  *norm = v;
  return ok();
}

}  // extern "C"
