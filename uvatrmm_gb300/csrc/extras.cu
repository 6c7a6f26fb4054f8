// The reference's other local call (GEMM) on the FP64 tile engine, one stage
// of its product loop, its binary result files, and ScaLAPACK block-cyclic
// layout adapters.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "api_internal.h"
#include "common.cuh"
#include "trmm_fp64.cuh"

namespace uvt {
namespace {

__global__ void scale_kernel(double *C, int64_t ldc, int64_t rows, int64_t cols, double beta) {
  const int64_t total = rows * cols;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = e / rows, i = e - j * rows;
    double *c = C + i + j * ldc;
    *c = beta == 0.0 ? 0.0 : beta * *c;
  }
}

int grid_of(uvatrmm_handle_t h, int64_t work) {
  int64_t g = (work + 255) / 256, cap = (int64_t)h->num_sms * 8;
  return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

bool tma_aligned(const void *p, int64_t ld) { return reinterpret_cast<uintptr_t>(p) % 16 == 0 && ld % 2 == 0; }

// Argument checks in the order and numbering of the reference CBLAS dgemm.
int check_gemm(int layout, int ta, int tb, int64_t m, int64_t n, int64_t k, int64_t lda, int64_t ldb, int64_t ldc) {
  auto okt = [](int t) { return t == CblasNoTrans || t == CblasTrans || t == CblasConjTrans; };
  if (layout != CblasRowMajor && layout != CblasColMajor) return 1;
  if (!okt(ta)) return 2;
  if (!okt(tb)) return 3;
  if (m < 0) return 4;
  if (n < 0) return 5;
  if (k < 0) return 6;
  const bool col = layout == CblasColMajor;
  const bool na = ta == CblasNoTrans, nb = tb == CblasNoTrans;
  const int64_t need_a = col ? (na ? m : k) : (na ? k : m);
  const int64_t need_b = col ? (nb ? k : n) : (nb ? n : k);
  const int64_t need_c = col ? m : n;
  if (lda < (need_a > 1 ? need_a : 1)) return 9;
  if (ldb < (need_b > 1 ? need_b : 1)) return 11;
  if (ldc < (need_c > 1 ? need_c : 1)) return 14;
  return 0;
}

// C := alpha*op(A)*op(B) + beta*C on device buffers (any layout).
int device_gemm(uvatrmm_handle_t h, int layout, int ta, int tb, int64_t m, int64_t n, int64_t k, double alpha,
                const double *A, int64_t lda, const double *B, int64_t ldb, double beta, double *C, int64_t ldc) {
  if (int bad = check_gemm(layout, ta, tb, m, n, k, lda, ldb, ldc))
    return fail(UVATRMM_EINVAL, "parameter " + std::to_string(bad) + " had an illegal value");
  if (layout == CblasRowMajor) {
    // C^T = op(B)^T op(A)^T: the column-major call with A and B exchanged.
    std::swap(ta, tb);
    std::swap(m, n);
    std::swap(A, B);
    std::swap(lda, ldb);
  }
  if (m == 0 || n == 0) return ok();
  if (alpha == 0.0 || k == 0) return scale_device(h, C, ldc, m, n, beta) == UVATRMM_OK ? ok() : uvatrmm_last_status();
  const bool at = ta != CblasNoTrans, bt = tb != CblasNoTrans;
  int64_t ar = at ? k : m, ac = at ? m : k, br = bt ? n : k, bc = bt ? k : n;
  if (!tma_aligned(A, lda)) {
    const int64_t la = round_up(ar, 16);
    double *w = static_cast<double *>(workspace(h, 0, (size_t)la * ac * 8));
    if (!w) return uvatrmm_last_status();
    cudaError_t e = cudaMemcpy2DAsync(w, la * 8, A, lda * 8, ar * 8, ac, cudaMemcpyDeviceToDevice, h->stream);
    if (e != cudaSuccess) return cuda_fail(e, "staging A");
    A = w;
    lda = la;
  }
  if (!tma_aligned(B, ldb)) {
    const int64_t lb = round_up(br, 16);
    double *w = static_cast<double *>(workspace(h, 1, (size_t)lb * bc * 8));
    if (!w) return uvatrmm_last_status();
    cudaError_t e = cudaMemcpy2DAsync(w, lb * 8, B, ldb * 8, br * 8, bc, cudaMemcpyDeviceToDevice, h->stream);
    if (e != cudaSuccess) return cuda_fail(e, "staging B");
    B = w;
    ldb = lb;
  }
  Fp64Launch L;
  L.M = m;
  L.N = n;
  L.K = k;
  L.alpha = alpha;
  L.beta = beta;
  L.C = C;
  L.ldc = ldc;
  L.tri_none = true;
  L.tri_left = true;
  L.tri_lower = true;
  L.unit = false;
  L.xl = MatRef{A, ar, ac, lda};
  L.lft_kmajor = at;
  L.xr = MatRef{B, br, bc, ldb};
  L.rgt_kmajor = !bt;
  L.engine = h->engine;
  L.schedule = UVATRMM_SCHED_DYNAMIC;
  L.shape = UVATRMM_SHAPE_TRAPEZOID;
  L.tile = h->tile;
  L.counter = h->dctl;
  L.status = h->dctl + 1;
  L.num_sms = h->num_sms;
  const char *why = nullptr;
  int rc = launch_trmm_fp64(L, h->stream, &why);
  if (rc != UVATRMM_OK) return fail(rc, why ? why : "GEMM launch failed");
  return ok();
}

// One mb x nb block of the global matrix per CTA iteration.  Global block
// (bi, bj) lives on process (bi mod nprow, bj mod npcol) at local block
// (bi div nprow, bj div npcol); its columns are contiguous runs of mb doubles
// in both layouts, so a warp moves 256 consecutive bytes per column.
constexpr int kBcRows = 32, kBcCols = 8;

__global__ void __launch_bounds__(kBcRows *kBcCols)
    bc_kernel(int64_t m, int64_t n, int64_t mb, int64_t nb, int nprow, int npcol, double *const *locals,
              const int64_t *lld, double *global, int64_t ldg, int to_global) {
  const int64_t nbr = (m + mb - 1) / mb, nbc = (n + nb - 1) / nb;
  for (int64_t blk = blockIdx.x; blk < nbr * nbc; blk += gridDim.x) {
    const int64_t bi = blk % nbr, bj = blk / nbr;
    const int pq = (int)(bi % nprow) * npcol + (int)(bj % npcol);
    const int64_t ld = lld[pq];
    double *loc = locals[pq] + (bi / nprow) * mb + (bj / npcol) * nb * ld;
    double *glb = global + bi * mb + bj * nb * ldg;
    const int64_t rows = min(mb, m - bi * mb), cols = min(nb, n - bj * nb);
    const double *__restrict__ src = to_global ? loc : glb;
    double *__restrict__ dst = to_global ? glb : loc;
    const int64_t lds = to_global ? ld : ldg, ldd = to_global ? ldg : ld;
    for (int64_t c = threadIdx.y; c < cols; c += kBcCols) {
#pragma unroll 4
      for (int64_t r = threadIdx.x; r < rows; r += kBcRows) dst[r + c * ldd] = src[r + c * lds];
    }
  }
}

int bc_move(uvatrmm_handle_t h, int64_t m, int64_t n, int64_t mb, int64_t nb, int nprow, int npcol,
            double *const *locals, const int64_t *lld, double *global, int64_t ldg, bool to_global) {
  if (m < 0 || n < 0 || mb < 1 || nb < 1 || nprow < 1 || npcol < 1 || !locals || !lld || ldg < (m > 1 ? m : 1))
    return fail(UVATRMM_EINVAL, "invalid block-cyclic arguments");
  if (m == 0 || n == 0) return ok();
  const int np = nprow * npcol;
  for (int pq = 0; pq < np; ++pq) {
    const int64_t rows = uvatrmm_numroc(m, mb, pq / npcol, 0, nprow);
    if (lld[pq] < (rows > 1 ? rows : 1)) return fail(UVATRMM_EINVAL, "local leading dimension too small");
  }
  std::lock_guard<std::mutex> g(h->mu);
  char *tab = static_cast<char *>(workspace(h, 7, (size_t)np * 16 + 256));
  if (!tab) return uvatrmm_last_status();
  double **dptr = reinterpret_cast<double **>(tab);
  int64_t *dlld = reinterpret_cast<int64_t *>(tab + (size_t)np * 8);
  cudaError_t e = cudaMemcpyAsync(dptr, locals, (size_t)np * 8, cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dlld, lld, (size_t)np * 8, cudaMemcpyHostToDevice, h->stream);
  if (e != cudaSuccess) return cuda_fail(e, "block-cyclic tables");
  const int64_t blocks = ((m + mb - 1) / mb) * ((n + nb - 1) / nb);
  const int grid = (int)std::min<int64_t>(blocks, (int64_t)h->num_sms * 8);
  bc_kernel<<<grid, dim3(kBcRows, kBcCols), 0, h->stream>>>(m, n, mb, nb, nprow, npcol, dptr, dlld, global, ldg,
                                                            to_global ? 1 : 0);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);  // the host tables may go away after return
  return e == cudaSuccess ? ok() : cuda_fail(e, "block-cyclic copy");
}

}  // namespace

int scale_device(uvatrmm_handle_t h, double *C, int64_t ldc, int64_t rows, int64_t cols, double beta) {
  if (rows <= 0 || cols <= 0) return UVATRMM_OK;
  scale_kernel<<<grid_of(h, rows * cols), 256, 0, h->stream>>>(C, ldc, rows, cols, beta);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? UVATRMM_OK : cuda_fail(e, "scale");
}

}  // namespace uvt

using namespace uvt;

extern "C" {

UVATRMM_API int uvatrmm_dgemm_device(uvatrmm_handle_t h, int layout, int transa, int transb, int64_t m, int64_t n,
                                     int64_t k, double alpha, const double *dA, int64_t lda, const double *dB,
                                     int64_t ldb, double beta, double *dC, int64_t ldc) {
  if (int bad = check_gemm(layout, transa, transb, m, n, k, lda, ldb, ldc))
    return fail(UVATRMM_EINVAL, "parameter " + std::to_string(bad) + " had an illegal value");
  if (!(h = resolve(h))) return uvatrmm_last_status();
  std::lock_guard<std::mutex> g(h->mu);
  return device_gemm(h, layout, transa, transb, m, n, k, alpha, dA, lda, dB, ldb, beta, dC, ldc);
}

UVATRMM_API int uvatrmm_dgemm(uvatrmm_handle_t h, int layout, int transa, int transb, int64_t m, int64_t n,
                              int64_t k, double alpha, const double *A, int64_t lda, const double *B, int64_t ldb,
                              double beta, double *C, int64_t ldc) {
  if (int bad = check_gemm(layout, transa, transb, m, n, k, lda, ldb, ldc))
    return fail(UVATRMM_EINVAL, "parameter " + std::to_string(bad) + " had an illegal value");
  if (!(h = resolve(h))) return uvatrmm_last_status();
  std::lock_guard<std::mutex> g(h->mu);
  // Column-major view of the three host matrices.
  const bool col = layout == CblasColMajor;
  const bool na = transa == CblasNoTrans, nb = transb == CblasNoTrans;
  const int64_t ar = col ? (na ? m : k) : (na ? k : m), acn = col ? (na ? k : m) : (na ? m : k);
  const int64_t br = col ? (nb ? k : n) : (nb ? n : k), bcn = col ? (nb ? n : k) : (nb ? k : n);
  const int64_t cr = col ? m : n, ccn = col ? n : m;
  if (m == 0 || n == 0) return ok();
  const int64_t la = round_up(ar > 0 ? ar : 1, 16), lb = round_up(br > 0 ? br : 1, 16);
  const int64_t lc = round_up(cr > 0 ? cr : 1, 16);
  double *dA = static_cast<double *>(workspace(h, 0, (size_t)la * acn * 8 + 16));
  double *dB = static_cast<double *>(workspace(h, 1, (size_t)lb * bcn * 8 + 16));
  double *dC = static_cast<double *>(workspace(h, 2, (size_t)lc * ccn * 8 + 16));
  if (!dA || !dB || !dC) return uvatrmm_last_status();
  cudaError_t e = cudaSuccess;
  if (ar && acn) e = host_copy2d(h, dA, la * 8, A, lda * 8, ar * 8, acn, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && br && bcn)
    e = host_copy2d(h, dB, lb * 8, B, ldb * 8, br * 8, bcn, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && beta != 0.0)
    e = host_copy2d(h, dC, lc * 8, C, ldc * 8, cr * 8, ccn, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "host to device copy");
  int rc = device_gemm(h, layout, transa, transb, m, n, k, alpha, dA, la, dB, lb, beta, dC, lc);
  if (rc != UVATRMM_OK) return rc;
  e = host_copy2d(h, C, ldc * 8, dC, lc * 8, cr * 8, ccn, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "device to host copy");
  rc = collect_status(h);
  return rc == UVATRMM_OK ? ok() : rc;
}

UVATRMM_API void cblas_dgemm(CBLAS_LAYOUT layout, CBLAS_TRANSPOSE transa, CBLAS_TRANSPOSE transb, int M, int N,
                             int K, double alpha, const double *A, int lda, const double *B, int ldb, double beta,
                             double *C, int ldc) {
  if (int bad = check_gemm(layout, transa, transb, M, N, K, lda, ldb, ldc)) {
    fprintf(stderr, " ** On entry to cblas_dgemm parameter number %d had an illegal value\n", bad);
    fail(UVATRMM_EINVAL, "parameter " + std::to_string(bad) + " had an illegal value");
    return;
  }
  int rc = uvatrmm_dgemm(nullptr, layout, transa, transb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
  if (rc != UVATRMM_OK) fprintf(stderr, "cblas_dgemm (uvatrmm): %s\n", uvatrmm_last_error());
}

UVATRMM_API int uvatrmm_stage(uvatrmm_handle_t h, int64_t n, int64_t w, int64_t b, int64_t hr, const double *dAblk,
                              int64_t lda, const double *dB, int64_t ldb, double *dC, int64_t ldc) {
  if (!(h = resolve(h))) return uvatrmm_last_status();
  if (n < 1 || w < 0 || b < 0 || hr < 1 || b + hr > n || lda < b + hr || ldb < w || ldc < w)
    return fail(UVATRMM_EINVAL, "invalid stage arguments");
  std::lock_guard<std::mutex> g(h->mu);
  if (w == 0) return ok();
  // dgemm: C[b:b+h] = Ablk[:, 0:b+1] * B[0:b+1]  (UVaTRMM/src/mm_triangular.c:347-360)
  int rc = device_gemm(h, CblasRowMajor, CblasNoTrans, CblasNoTrans, hr, w, b + 1, 1.0, dAblk, lda, dB, ldb, 0.0,
                       dC + b * ldc, ldc);
  if (rc != UVATRMM_OK || hr == 1) return rc;
  // dtrmm + add: C[b+1:b+h] += tril(Ablk[1:h, b+1:b+h]) * B[b+1:b+h]  (:374-393)
  rc = device_trmm(h, CblasRowMajor, CblasLeft, CblasLower, CblasNoTrans, CblasNonUnit, hr - 1, w, 1.0,
                   dAblk + lda + (b + 1), lda, dB + (b + 1) * ldb, ldb, dC + (b + 1) * ldc, ldc, false,
                   UVATRMM_SCHED_DYNAMIC, UVATRMM_SHAPE_TRAPEZOID, 1.0);
  return rc == UVATRMM_OK ? ok() : rc;
}

UVATRMM_API int uvatrmm_write_result(const char *path, int rows, int cols, int row_begin, int nrows, int col_begin,
                                     int ncols, const double *block, int64_t ld) {
  if (!path || rows < 0 || cols < 0 || nrows < 0 || ncols < 0 || (nrows && ncols && (!block || ld < ncols)))
    return fail(UVATRMM_EINVAL, "invalid result-file arguments");
  FILE *f = fopen(path, "wb");
  if (!f) return fail(UVATRMM_EINVAL, std::string("cannot open ") + path);
  const int hdr[6] = {rows, cols, row_begin, nrows, col_begin, ncols};
  bool good = fwrite(hdr, sizeof(int), 6, f) == 6;
  for (int i = 0; good && i < nrows; ++i)
    good = fwrite(block + (int64_t)i * ld, sizeof(double), (size_t)ncols, f) == (size_t)ncols;
  good = (fclose(f) == 0) && good;
  return good ? ok() : fail(UVATRMM_EDEVICE, std::string("write failed: ") + path);
}

UVATRMM_API int uvatrmm_read_result(const char *path, int hdr[6], double *out, int64_t capacity) {
  if (!path || !hdr) return fail(UVATRMM_EINVAL, "invalid arguments");
  FILE *f = fopen(path, "rb");
  if (!f) return fail(UVATRMM_EINVAL, std::string("cannot open ") + path);
  bool good = fread(hdr, sizeof(int), 6, f) == 6;
  const int64_t count = good ? (int64_t)hdr[3] * hdr[5] : 0;
  if (good && (hdr[3] < 0 || hdr[5] < 0 || count > capacity || (count && !out))) good = false;
  if (good && count) good = fread(out, sizeof(double), (size_t)count, f) == (size_t)count;
  fclose(f);
  return good ? ok() : fail(UVATRMM_EINVAL, std::string("malformed result file or buffer too small: ") + path);
}

UVATRMM_API int64_t uvatrmm_numroc(int64_t n, int64_t nb, int iproc, int isrcproc, int nprocs) {
  if (n <= 0 || nb <= 0 || nprocs <= 0) return 0;
  const int mydist = ((iproc - isrcproc) % nprocs + nprocs) % nprocs;
  const int64_t nblocks = n / nb;
  int64_t r = (nblocks / nprocs) * nb;
  const int64_t extra = nblocks % nprocs;
  if (mydist < extra) r += nb;
  else if (mydist == extra) r += n % nb;
  return r;
}

UVATRMM_API int uvatrmm_bc_gather(uvatrmm_handle_t h, int64_t m, int64_t n, int64_t mb, int64_t nb, int nprow,
                                  int npcol, const double *const *locals, const int64_t *lld, double *dglobal,
                                  int64_t ldg) {
  if (!(h = resolve(h))) return uvatrmm_last_status();
  return bc_move(h, m, n, mb, nb, nprow, npcol, const_cast<double *const *>(locals), lld, dglobal, ldg, true);
}

UVATRMM_API int uvatrmm_bc_scatter(uvatrmm_handle_t h, int64_t m, int64_t n, int64_t mb, int64_t nb, int nprow,
                                   int npcol, const double *dglobal, int64_t ldg, double *const *locals,
                                   const int64_t *lld) {
  if (!(h = resolve(h))) return uvatrmm_last_status();
  return bc_move(h, m, n, mb, nb, nprow, npcol, locals, lld, const_cast<double *>(dglobal), ldg, false);
}

}  // extern "C"
