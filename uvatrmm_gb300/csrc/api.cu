// C ABI of libuvatrmm.so: handles, argument checking, CBLAS row-major
// normalisation, operand staging, and the plain FP64 TRMM entry points.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "api_internal.h"
#include "common.cuh"
#include "trmm_fp64.cuh"

namespace uvt {

static thread_local int tl_status = UVATRMM_OK;
static thread_local std::string tl_msg;
static thread_local uvatrmm_handle_t tl_default[64] = {};

int fail(int status, const std::string &msg) {
  tl_status = status;
  tl_msg = msg;
  return status;
}
int ok() {
  tl_status = UVATRMM_OK;
  tl_msg.clear();
  return UVATRMM_OK;
}
int cuda_fail(cudaError_t e, const char *what) {
  // A failed call such as an allocation that did not fit also sets the
  // runtime's last-error state; consume it so the check after this thread's
  // next kernel launch does not report it a second time.  (Sticky errors,
  // which leave the context unusable, are not cleared by this.)
  cudaGetLastError();
  return fail(e == cudaErrorMemoryAllocation ? UVATRMM_ENOMEM : UVATRMM_EDEVICE,
              std::string(what) + ": " + cudaGetErrorString(e));
}

uvatrmm_handle_t resolve(uvatrmm_handle_t h) {
  if (h) return h;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
    fail(UVATRMM_EDEVICE, "no CUDA device");
    return nullptr;
  }
  if (!tl_default[dev]) {
    uvatrmm_handle_t nh = nullptr;
    if (uvatrmm_create(&nh) != UVATRMM_OK) return nullptr;
    tl_default[dev] = nh;
  }
  return tl_default[dev];
}

void *workspace(uvatrmm_handle_t h, int slot, size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (h->ws_cap[slot] >= bytes) return h->ws[slot];
  if (h->ws[slot]) {
    cudaStreamSynchronize(h->stream);
    cudaFree(h->ws[slot]);
    h->ws[slot] = nullptr;
    h->ws_cap[slot] = 0;
  }
  size_t cap = (size_t)round_up((int64_t)bytes, 1 << 21);
  cudaError_t e = cudaMalloc(&h->ws[slot], cap);
  if (e != cudaSuccess) {
    h->ws[slot] = nullptr;
    cuda_fail(e, "workspace allocation");
    return nullptr;
  }
  h->ws_cap[slot] = cap;
  return h->ws[slot];
}

int collect_status(uvatrmm_handle_t h) {
  int st = 0;
  cudaError_t e = cudaMemcpyAsync(&st, h->dctl + 1, sizeof(int), cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return cuda_fail(e, "kernel execution");
  if (st) {
    cudaMemsetAsync(h->dctl + 1, 0, sizeof(int), h->stream);
    cudaStreamSynchronize(h->stream);
    if (st & KERR_WAIT_TIMEOUT) return fail(UVATRMM_ETIMEOUT, "a kernel wait expired (bounded spin limit)");
    return fail(UVATRMM_EDEVICE, "kernel reported error flags " + std::to_string(st));
  }
  return UVATRMM_OK;
}

// ------------------------------------------------------------------ TRMM core

// Argument checks in the order (and with the parameter numbers) of the
// reference BLAS cblas_dtrmm; returns 0 or the 1-based index of the first
// bad argument (as xerbla reports it).
int check_args(int layout, int side, int uplo, int transa, int diag, int64_t m, int64_t n, int64_t lda,
               int64_t ldb) {
  if (layout != CblasRowMajor && layout != CblasColMajor) return 1;
  if (side != CblasLeft && side != CblasRight) return 2;
  if (uplo != CblasUpper && uplo != CblasLower) return 3;
  if (transa != CblasNoTrans && transa != CblasTrans && transa != CblasConjTrans) return 4;
  if (diag != CblasUnit && diag != CblasNonUnit) return 5;
  if (m < 0) return 6;
  if (n < 0) return 7;
  const int64_t ka = side == CblasLeft ? m : n;
  if (lda < (ka > 1 ? ka : 1)) return 10;
  const int64_t brows = layout == CblasColMajor ? m : n;
  if (ldb < (brows > 1 ? brows : 1)) return 12;
  return 0;
}

Trmm normalise(int layout, int side, int uplo, int transa, int diag, int64_t m, int64_t n, double alpha) {
  Trmm t;
  t.side = side;
  t.uplo = uplo;
  t.m = m;
  t.n = n;
  if (layout == CblasRowMajor) {
    // Row-major X is column-major X^T: C^T = B^T op(A)^T swaps the side,
    // flips the stored triangle and exchanges m and n.
    t.side = side == CblasLeft ? CblasRight : CblasLeft;
    t.uplo = uplo == CblasUpper ? CblasLower : CblasUpper;
    t.m = n;
    t.n = m;
  }
  t.trans = transa != CblasNoTrans;
  t.unit = diag == CblasUnit;
  t.alpha = alpha;
  return t;
}

namespace {

bool tma_ok(const void *p, int64_t ld) { return (reinterpret_cast<uintptr_t>(p) % 16 == 0) && (ld % 2 == 0); }

// Launches C := alpha*op(A)*B or alpha*B*op(A) on device buffers, all
// column-major; A and B must satisfy tma_ok.
int run_fp64(uvatrmm_handle_t h, const Trmm &t, const double *A, int64_t lda, const double *B, int64_t ldb,
             double *C, int64_t ldc, int schedule, int shape, double beta = 0.0) {
  Fp64Launch L;
  const int64_t ka = t.side == CblasLeft ? t.m : t.n;
  const bool lower = (t.uplo == CblasLower) != (t.trans != 0);
  L.M = t.m;
  L.N = t.n;
  L.K = ka;
  L.alpha = t.alpha;
  L.beta = beta;
  L.C = C;
  L.ldc = ldc;
  L.unit = t.unit;
  L.tri_lower = lower;
  if (t.side == CblasLeft) {
    L.tri_left = true;
    L.xl = MatRef{A, ka, ka, lda};
    L.lft_kmajor = t.trans != 0;
    L.xr = MatRef{B, t.m, t.n, ldb};
    L.rgt_kmajor = true;
  } else {
    L.tri_left = false;
    L.xl = MatRef{B, t.m, t.n, ldb};
    L.lft_kmajor = false;
    L.xr = MatRef{A, ka, ka, lda};
    L.rgt_kmajor = t.trans == 0;
  }
  L.engine = h->engine;
  L.schedule = schedule;
  L.shape = shape;
  L.tile = h->tile;
  L.counter = h->dctl;
  L.status = h->dctl + 1;
  L.num_sms = h->num_sms;
  L.expiry_test_polls = h->expiry_test_polls;
  const char *why = nullptr;
  int rc = launch_trmm_fp64(L, h->stream, &why);
  if (rc != UVATRMM_OK) return fail(rc, why ? why : "kernel launch failed");
  return UVATRMM_OK;
}

// alpha == 0: B := 0 without reading A (BLAS semantics).
int zero_device(uvatrmm_handle_t h, double *dB, int64_t ldb, int64_t rows, int64_t cols) {
  cudaError_t e = cudaMemset2DAsync(dB, ldb * 8, 0, rows * 8, cols, h->stream);
  return e == cudaSuccess ? UVATRMM_OK : cuda_fail(e, "zero fill");
}

}  // namespace

// Device-side core shared by the in-place and out-of-place entry points.
// dC receives the result (may equal dB only when `in_place`).
int device_trmm(uvatrmm_handle_t h, int layout, int side, int uplo, int transa, int diag, int64_t m, int64_t n,
                double alpha, const double *dA, int64_t lda, const double *dB, int64_t ldb, double *dC,
                int64_t ldc, bool in_place, int schedule, int shape, double beta) {
  if (int bad = check_args(layout, side, uplo, transa, diag, m, n, lda, ldb))
    return fail(UVATRMM_EINVAL, "parameter " + std::to_string(bad) + " had an illegal value");
  if (!in_place) {
    const int64_t crows = layout == CblasColMajor ? m : n;
    if (ldc < (crows > 1 ? crows : 1)) return fail(UVATRMM_EINVAL, "parameter ldc had an illegal value");
  }
  Trmm t = normalise(layout, side, uplo, transa, diag, m, n, alpha);
  if (t.m == 0 || t.n == 0) return ok();
  if (alpha == 0.0) {
    if (beta == 0.0) return zero_device(h, dC, ldc, t.m, t.n) == UVATRMM_OK ? ok() : tl_status;
    return scale_device(h, dC, ldc, t.m, t.n, beta) == UVATRMM_OK ? ok() : tl_status;
  }
  const int64_t ka = t.side == CblasLeft ? t.m : t.n;
  const double *A = dA;
  int64_t la = lda;
  if (!tma_ok(dA, lda)) {
    la = round_up(ka, 16);
    double *w = static_cast<double *>(workspace(h, 0, (size_t)la * ka * 8));
    if (!w) return tl_status;
    cudaError_t e = cudaMemcpy2DAsync(w, la * 8, dA, lda * 8, ka * 8, ka, cudaMemcpyDeviceToDevice, h->stream);
    if (e != cudaSuccess) return cuda_fail(e, "staging A");
    A = w;
  }
  const double *B = dB;
  int64_t lb = ldb;
  if (in_place || !tma_ok(dB, ldb)) {
    lb = round_up(t.m, 16);
    double *w = static_cast<double *>(workspace(h, 1, (size_t)lb * t.n * 8));
    if (!w) return tl_status;
    cudaError_t e = cudaMemcpy2DAsync(w, lb * 8, dB, ldb * 8, t.m * 8, t.n, cudaMemcpyDeviceToDevice, h->stream);
    if (e != cudaSuccess) return cuda_fail(e, "staging B");
    B = w;
  }
  int rc = run_fp64(h, t, A, la, B, lb, dC, ldc, schedule, shape, beta);
  return rc == UVATRMM_OK ? ok() : rc;
}

// The host-pointer TRMM: A and B copied in, C := alpha op(A) B (or B op(A))
// computed out of place, C copied back into B.  `async`: A and B must lie in
// uvatrmm_host_alloc memory, everything is enqueued on the handle's stream
// and the status is collected by uvatrmm_sync.
int host_trmm(uvatrmm_handle_t h, int layout, int side, int uplo, int transa, int diag, int64_t m, int64_t n,
              double alpha, const double *A, int64_t lda, double *B, int64_t ldb, bool async) {
  if (int bad = check_args(layout, side, uplo, transa, diag, m, n, lda, ldb))
    return fail(UVATRMM_EINVAL, "parameter " + std::to_string(bad) + " had an illegal value");
  Trmm t = normalise(layout, side, uplo, transa, diag, m, n, alpha);
  if (t.m == 0 || t.n == 0) return ok();
  const int64_t ka = t.side == CblasLeft ? t.m : t.n;
  if (async && (!host_alloc_contains(A, (size_t)(lda * (ka - 1) + ka) * 8) ||
                !host_alloc_contains(B, (size_t)(ldb * (t.n - 1) + t.m) * 8)))
    return fail(UVATRMM_EINVAL, "asynchronous host operands must lie in uvatrmm_host_alloc memory");
  if (alpha == 0.0) {
    if (async) {
      cudaError_t e = cudaStreamSynchronize(h->stream);  // earlier calls may still write B
      if (e != cudaSuccess) return cuda_fail(e, "stream synchronise");
    }
    for (int64_t j = 0; j < t.n; ++j) memset(B + j * ldb, 0, (size_t)t.m * 8);
    return ok();
  }
  const int64_t la = round_up(ka, 16), lb = round_up(t.m, 16);
  double *dA = static_cast<double *>(workspace(h, 0, (size_t)la * ka * 8));
  double *dB = static_cast<double *>(workspace(h, 1, (size_t)lb * t.n * 8));
  double *dC = static_cast<double *>(workspace(h, 2, (size_t)lb * t.n * 8));
  if (!dA || !dB || !dC) return tl_status;
  cudaError_t e = copy_triangle_h2d(h, dA, la, A, lda, ka, t.uplo == CblasLower);
  if (e == cudaSuccess) e = host_copy2d(h, dB, lb * 8, B, ldb * 8, t.m * 8, t.n, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "host to device copy");
  int rc = run_fp64(h, t, dA, la, dB, lb, dC, lb, h->schedule, h->shape);
  if (rc != UVATRMM_OK) return rc;
  e = host_copy2d(h, B, ldb * 8, dC, lb * 8, t.m * 8, t.n, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "device to host copy");
  if (async) return ok();
  rc = collect_status(h);
  return rc == UVATRMM_OK ? ok() : rc;
}

}  // namespace uvt

using namespace uvt;

extern "C" {

UVATRMM_API const char *uvatrmm_version(void) { return "uvatrmm-gb300 0.1 (sm_103a)"; }
UVATRMM_API const char *uvatrmm_last_error(void) { return tl_msg.c_str(); }
UVATRMM_API int uvatrmm_last_status(void) { return tl_status; }

UVATRMM_API int uvatrmm_create(uvatrmm_handle_t *handle) {
  if (!handle) return fail(UVATRMM_EINVAL, "handle pointer is NULL");
  *handle = nullptr;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  cudaDeviceProp prop;
  e = cudaGetDeviceProperties(&prop, dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceProperties");
  if (prop.major != 10 || prop.minor != 3)
    return fail(UVATRMM_EUNSUPPORTED, std::string("device is not sm_103 (GB300): ") + prop.name);
  auto *h = new uvatrmm_handle_st();
  h->device = dev;
  h->num_sms = prop.multiProcessorCount;
  e = cudaMalloc(&h->dctl, 64);
  if (e == cudaSuccess) e = cudaMemset(h->dctl, 0, 64);
  if (e == cudaSuccess) e = cudaEventCreate(&h->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&h->ev1);
  if (e != cudaSuccess) {
    delete h;
    return cuda_fail(e, "handle setup");
  }
  *handle = h;
  return ok();
}

UVATRMM_API int uvatrmm_destroy(uvatrmm_handle_t h) {
  if (!h) return ok();
  cudaStreamSynchronize(h->stream);
  for (int i = 0; i < uvatrmm_handle_st::kSlots; ++i)
    if (h->ws[i]) cudaFree(h->ws[i]);
  if (h->dctl) cudaFree(h->dctl);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  release_host_staging(h);
  for (auto &ev : h->sev)
    if (ev) cudaEventDestroy(ev);
  for (auto &d : tl_default)
    if (d == h) d = nullptr;
  delete h;
  return ok();
}

UVATRMM_API int uvatrmm_set_stream(uvatrmm_handle_t h, void *stream) {
  if (!(h = resolve(h))) return tl_status;
  h->stream = static_cast<cudaStream_t>(stream);
  return ok();
}

UVATRMM_API int uvatrmm_set_option(uvatrmm_handle_t h, int option, int value) {
  if (!(h = resolve(h))) return tl_status;
  switch (option) {
    case UVATRMM_OPT_ENGINE:
      if (value != UVATRMM_ENGINE_DFMA && value != UVATRMM_ENGINE_DMMA) break;
      h->engine = value;
      return ok();
    case UVATRMM_OPT_SCHEDULE:
      if (value < UVATRMM_SCHED_DYNAMIC || value > UVATRMM_SCHED_BALANCED) break;
      h->schedule = value;
      return ok();
    case UVATRMM_OPT_SHAPE:
      if (value != UVATRMM_SHAPE_TRAPEZOID && value != UVATRMM_SHAPE_BOXES) break;
      h->shape = value;
      return ok();
    case UVATRMM_OPT_TILE:
      if (value != 0 && value != 64 && value != 128) break;
      h->tile = value;
      return ok();
    case UVATRMM_OPT_OZAKI_SCRATCH_MB:
      if (value < 64) break;
      h->ozaki_scratch_mb = value;
      return ok();
    case UVATRMM_OPT_OZAKI_RASTER:
      if (value < 0 || value > 64) break;
      h->oz_raster = value;
      return ok();
    case UVATRMM_OPT_HOST_STAGE_KB:
      if (value != 0 && value < 64) break;
      h->hstage_bytes = (size_t)(value ? value : 262144) << 10;
      return ok();
    case UVATRMM_OPT_OZAKI_ERR_HOST:
      if (value != 0 && value != 1) break;
      h->oz_err_host = value != 0;
      return ok();
    case UVATRMM_OPT_WAIT_EXPIRY_TEST:
      if (value < 0 || value > (int)kSpinLimit) break;
      h->expiry_test_polls = (uint32_t)value;
      return ok();
    case UVATRMM_OPT_AUTOTUNE:
      if (value != 0 && value != 1) break;
      h->autotune = value != 0;
      return ok();
    case UVATRMM_OPT_STAGE_TIMING:
      if (value != 0 && value != 1) break;
      if (value && !h->sev[0])
        for (auto &ev : h->sev)
          if (cudaEventCreate(&ev) != cudaSuccess) return cuda_fail(cudaGetLastError(), "stage events");
      h->stage_timing = value != 0;
      return ok();
    default:
      return fail(UVATRMM_EINVAL, "unknown option");
  }
  return fail(UVATRMM_EINVAL, "invalid value for option " + std::to_string(option));
}

UVATRMM_API int uvatrmm_sync(uvatrmm_handle_t h) {
  if (!(h = resolve(h))) return tl_status;
  int rc = collect_status(h);
  return rc == UVATRMM_OK ? ok() : rc;
}

UVATRMM_API int uvatrmm_dtrmm_device(uvatrmm_handle_t h, int layout, int side, int uplo, int transa, int diag,
                                     int64_t m, int64_t n, double alpha, const double *dA, int64_t lda, double *dB,
                                     int64_t ldb) {
  if (!(h = resolve(h))) return tl_status;
  std::lock_guard<std::mutex> g(h->mu);
  return device_trmm(h, layout, side, uplo, transa, diag, m, n, alpha, dA, lda, dB, ldb, dB, ldb, true,
                     h->schedule, h->shape);
}

UVATRMM_API int uvatrmm_dtrmm_device_oop(uvatrmm_handle_t h, int layout, int side, int uplo, int transa, int diag,
                                         int64_t m, int64_t n, double alpha, const double *dA, int64_t lda,
                                         const double *dB, int64_t ldb, double *dC, int64_t ldc) {
  if (!(h = resolve(h))) return tl_status;
  std::lock_guard<std::mutex> g(h->mu);
  return device_trmm(h, layout, side, uplo, transa, diag, m, n, alpha, dA, lda, dB, ldb, dC, ldc, false,
                     h->schedule, h->shape);
}

UVATRMM_API int uvatrmm_dtrmm(uvatrmm_handle_t h, int layout, int side, int uplo, int transa, int diag, int64_t m,
                              int64_t n, double alpha, const double *A, int64_t lda, double *B, int64_t ldb) {
  if (!(h = resolve(h))) return tl_status;
  std::lock_guard<std::mutex> g(h->mu);
  return host_trmm(h, layout, side, uplo, transa, diag, m, n, alpha, A, lda, B, ldb, false);
}

UVATRMM_API int uvatrmm_dtrmm_async(uvatrmm_handle_t h, int layout, int side, int uplo, int transa, int diag,
                                    int64_t m, int64_t n, double alpha, const double *A, int64_t lda, double *B,
                                    int64_t ldb) {
  if (!(h = resolve(h))) return tl_status;
  std::lock_guard<std::mutex> g(h->mu);
  return host_trmm(h, layout, side, uplo, transa, diag, m, n, alpha, A, lda, B, ldb, true);
}

UVATRMM_API void cblas_dtrmm(CBLAS_LAYOUT layout, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transa,
                             CBLAS_DIAG diag, int M, int N, double alpha, const double *A, int lda, double *B,
                             int ldb) {
  if (int bad = check_args(layout, side, uplo, transa, diag, M, N, lda, ldb)) {
    fprintf(stderr, " ** On entry to cblas_dtrmm parameter number %d had an illegal value\n", bad);
    fail(UVATRMM_EINVAL, "parameter " + std::to_string(bad) + " had an illegal value");
    return;
  }
  int rc = uvatrmm_dtrmm(nullptr, layout, side, uplo, transa, diag, M, N, alpha, A, lda, B, ldb);
  if (rc != UVATRMM_OK) fprintf(stderr, "cblas_dtrmm (uvatrmm): %s\n", uvatrmm_last_error());
}

UVATRMM_API int uvatrmm_product(uvatrmm_handle_t h, int64_t n, int schedule, int shape, const double *dA,
                                const double *dB, double *dC, double *mult_seconds) {
  if (!(h = resolve(h))) return tl_status;
  std::lock_guard<std::mutex> g(h->mu);
  if (n < 1) return fail(UVATRMM_EINVAL, "n must be positive");
  if (schedule < UVATRMM_SCHED_DYNAMIC || schedule > UVATRMM_SCHED_BALANCED)
    return fail(UVATRMM_EINVAL, "unknown schedule");
  if (shape != UVATRMM_SHAPE_TRAPEZOID && shape != UVATRMM_SHAPE_BOXES) return fail(UVATRMM_EINVAL, "unknown shape");
  cudaEventRecord(h->ev0, h->stream);
  // Row-major C = tril(A) * B, as UVaTRMM/src/mm_triangular.c:319-410 computes it.
  int rc = device_trmm(h, CblasRowMajor, CblasLeft, CblasLower, CblasNoTrans, CblasNonUnit, n, n, 1.0, dA, n, dB,
                       n, dC, n, false, schedule, shape);
  if (rc != UVATRMM_OK) return rc;
  cudaEventRecord(h->ev1, h->stream);
  rc = collect_status(h);
  if (rc != UVATRMM_OK) return rc;
  if (mult_seconds) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    *mult_seconds = ms * 1e-3;
  }
  return ok();
}

UVATRMM_API int uvatrmm_device_alloc(size_t bytes, void **ptr) {
  if (!ptr) return fail(UVATRMM_EINVAL, "ptr is NULL");
  *ptr = nullptr;
  cudaError_t e = cudaMalloc(ptr, bytes ? bytes : 16);
  return e == cudaSuccess ? ok() : cuda_fail(e, "cudaMalloc");
}

UVATRMM_API int uvatrmm_device_free(void *ptr) {
  cudaError_t e = cudaFree(ptr);
  return e == cudaSuccess ? ok() : cuda_fail(e, "cudaFree");
}

UVATRMM_API int uvatrmm_copy(uvatrmm_handle_t h, void *dst, const void *src, size_t bytes, int kind) {
  if (!(h = resolve(h))) return tl_status;
  cudaMemcpyKind k = kind == 1 ? cudaMemcpyHostToDevice
                     : kind == 2 ? cudaMemcpyDeviceToHost
                     : kind == 3 ? cudaMemcpyDeviceToDevice
                                 : cudaMemcpyDefault;
  if (kind < 1 || kind > 3) return fail(UVATRMM_EINVAL, "copy kind must be 1, 2 or 3");
  cudaError_t e = cudaMemcpyAsync(dst, src, bytes, k, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  return e == cudaSuccess ? ok() : cuda_fail(e, "copy");
}

}  // extern "C"
