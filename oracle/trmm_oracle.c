/*
 * CPU oracle for the TRMM hot path  --  TEST INFRASTRUCTURE ONLY.
 *
 * This file restates, in plain C, the reference's algorithm for the path
 * B := alpha * op(A) * B (A triangular, FP64), so that tests/, the smoke
 * check and bench.py's CPU-baseline leg can check and time the CUDA product
 * against it.  Nothing in the product (uvatrmm_gb300/, include/) links,
 * loads or calls it.  Built by oracle/Makefile into oracle/_build/liboracle.so.
 *
 * Contents, each citing the reference lines it follows:
 *   orc_map_regular / orc_map_balanced    UVaTRMM/src/mm_mapping.c:27-67, :120-181, :319-366
 *   orc_gen_consecutive                   UVaTRMM/src/mm_triangular_common.c:1782-1805
 *   orc_inf_norm                          UVaTRMM/src/mm_triangular_common.c:2936-2991
 *   orc_uvatrmm_product                   UVaTRMM/src/mm_triangular.c:88-99, :319-403
 *                                         (every rank's column slice, run in one process)
 *   orc_dtrmm_naive / orc_dtrmm_dd        cblas_dtrmm semantics (called by the reference at
 *                                         UVaTRMM/src/mm_triangular.c:374-387); naive FP64 loops
 *                                         and a double-double (compensated) variant used as the
 *                                         high-accuracy reference for error reports
 *   orc_blas_dtrmm / orc_blas_dgemm       the third-party arithmetic the reference links
 *                                         (MKL there; OpenBLAS 0.3.34 as bundled by scipy here),
 *                                         resolved at run time with dlopen
 *   orc_fill_uniform / orc_fill_wide      seeded synthetic inputs (counter-based splitmix64);
 *                                         the product has its own device generator that must
 *                                         produce the same bytes
 *
 * Parity status: pinned.  The mapping, the generator and the product norms are
 * checked against the reference itself (oracle/_ref, built by
 * oracle/build_ref.sh) through the fixtures in tests/golden/.
 */
#include <dlfcn.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define ORC_EXPORT __attribute__((visibility("default")))

/* CBLAS enumerations (standard values). */
enum { ORC_ROW = 101, ORC_COL = 102 };
enum { ORC_NOTRANS = 111, ORC_TRANS = 112, ORC_CONJTRANS = 113 };
enum { ORC_UPPER = 121, ORC_LOWER = 122 };
enum { ORC_NONUNIT = 131, ORC_UNIT = 132 };
enum { ORC_LEFT = 141, ORC_RIGHT = 142 };

/* ------------------------------------------------------------------------ */
/* Row mappings.                                                            */
/* ------------------------------------------------------------------------ */

/* map_regular (UVaTRMM/src/mm_mapping.c:27-67): floor(n/P) rows per block,
 * remainder to the last block.  Returns 0, or -1 where the reference aborts
 * (P > n with P != 1). */
ORC_EXPORT int orc_map_regular(uint64_t n, uint32_t P, uint32_t idx, uint64_t *begin, uint64_t *size) {
  uint64_t eq = n / P, rem = n % P;
  if (eq < 1) eq = 1;
  if (P != 1 && eq * P > n) return -1;
  *begin = (uint64_t)idx * eq;
  *size = eq + (idx == P - 1 ? rem : 0);
  return 0;
}

/* get_rows_before (UVaTRMM/src/mm_mapping.c:177-181): rows r with
 * r(r+1)/2 <= k*ideal, i.e. floor(-1+sqrt(1+8k*ideal)) / 2, truncated. */
static uint64_t orc_rows_before(double ideal, int k) {
  double num = -1.0 + sqrt(1.0 + 8.0 * (k * ideal));
  return num > 0 ? (uint64_t)(floor(num) / 2.0) : 0;
}

/* map_balanced (UVaTRMM/src/mm_mapping.c:319-366 with helpers :120-170):
 * equal counts of lower-triangle elements per block.  The element count is
 * held in an unsigned int (:127-128) and the ideal block size is
 * ceil(count/P) as an unsigned int (:330).  Returns -1 where the reference
 * aborts (ideal < 1, or an empty block). */
ORC_EXPORT int orc_map_balanced(uint64_t n, uint32_t P, uint32_t idx, uint64_t *begin, uint64_t *size) {
  unsigned int count = (unsigned int)(0.5 * (double)(n * (n + 1)));
  double ideal_d = (double)count / (double)P;
  if (ideal_d < 1) return -1;
  unsigned int ideal = (unsigned int)ceil(ideal_d);
  unsigned int rb = (unsigned int)orc_rows_before((double)ideal, (int)idx);
  unsigned int re = (unsigned int)orc_rows_before((double)ideal, (int)idx + 1);
  uint64_t b = rb, s = (unsigned int)(re - rb);
  if (idx == 0) {
    b = 0;
    s = P > 1 ? orc_rows_before((double)ideal, 1) : n;
  }
  if (n > 1 && idx == P - 1) s = n - b;
  if (s == 0) return -1;
  *begin = b;
  *size = s;
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Input generators.                                                        */
/* ------------------------------------------------------------------------ */

/* mat_consecutive_values (UVaTRMM/src/mm_triangular_common.c:1782-1805):
 * element (i, j) of a block whose first row is rows_begin and first column
 * cols_begin, in a matrix with n_global columns, is
 *   1 / (((rows_begin + i) * n_global + cols_begin + j) mod 2341 + 1)
 * (the reciprocal is taken with -DMININUMS=1, UVaTRMM/Makefile:14), and 0
 * above the diagonal when `triangular`.  Indices are 64-bit here; the
 * reference's int arithmetic overflows from n = 46341 on. */
ORC_EXPORT void orc_gen_consecutive(int64_t n_global, int64_t rows_begin, int64_t rows, int64_t cols_begin,
                                    int64_t cols, int triangular, int mininums, double *out) {
  for (int64_t i = 0; i < rows; i++)
    for (int64_t j = 0; j < cols; j++) {
      int64_t g = rows_begin + i, c = cols_begin + j;
      double v;
      if (triangular && c > g) v = 0.0;
      else {
        v = (double)((g * n_global + c) % 2341 + 1);
        if (mininums) v = 1.0 / v;
      }
      out[i * cols + j] = v;
    }
}

static inline uint64_t orc_mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

/* Counter-based uniform[-1,1) value for element `idx` of stream `stream`
 * under `seed`: splitmix64 finaliser over (key(seed,stream) + (idx+1)*phi),
 * top 53 bits scaled to [0,1), mapped by 2u-1 (exact in FP64). */
static inline double orc_uniform(uint64_t seed, uint64_t stream, uint64_t idx) {
  uint64_t key = orc_mix64(seed * 0x9E3779B97F4A7C15ULL + stream * 0xD1B54A32D192ED03ULL + 0x632BE59BD9B4E019ULL);
  uint64_t z = orc_mix64(key + (idx + 1) * 0x9E3779B97F4A7C15ULL);
  return (double)(z >> 11) * 0x1.0p-53 * 2.0 - 1.0;
}

/* Exponent in [-spread, spread] for element idx (second, independent stream). */
static inline int orc_exponent(uint64_t seed, uint64_t stream, uint64_t idx, int spread) {
  uint64_t key = orc_mix64(seed * 0x9E3779B97F4A7C15ULL + stream * 0xD1B54A32D192ED03ULL + 0x2545F4914F6CDD1DULL);
  uint64_t z = orc_mix64(key + (idx + 1) * 0x9E3779B97F4A7C15ULL);
  return (int)(z % (uint64_t)(2 * spread + 1)) - spread;
}

/* Fill a rows x cols matrix (element (i,j) at out[i*rs + j*cs]) with the
 * seeded uniform[-1,1) values of logical index i*cols + j.  `tri` keeps
 * only one triangle (0 none, 'L' lower incl. diagonal, 'U' upper incl.
 * diagonal) and writes `fill` elsewhere. */
ORC_EXPORT void orc_fill_uniform(uint64_t seed, uint64_t stream, int64_t rows, int64_t cols, double *out,
                                 int64_t rs, int64_t cs, int tri, double fill) {
  for (int64_t i = 0; i < rows; i++)
    for (int64_t j = 0; j < cols; j++) {
      int keep = tri == 0 || (tri == 'L' && j <= i) || (tri == 'U' && j >= i);
      out[i * rs + j * cs] = keep ? orc_uniform(seed, stream, (uint64_t)(i * cols + j)) : fill;
    }
}

/* As orc_fill_uniform, times 2^k with k uniform in [-spread, spread]. */
ORC_EXPORT void orc_fill_wide(uint64_t seed, uint64_t stream, int64_t rows, int64_t cols, double *out,
                              int64_t rs, int64_t cs, int tri, double fill, int spread) {
  for (int64_t i = 0; i < rows; i++)
    for (int64_t j = 0; j < cols; j++) {
      int keep = tri == 0 || (tri == 'L' && j <= i) || (tri == 'U' && j >= i);
      uint64_t idx = (uint64_t)(i * cols + j);
      out[i * rs + j * cs] =
          keep ? ldexp(orc_uniform(seed, stream, idx), orc_exponent(seed, stream, idx, spread)) : fill;
    }
}

/* ------------------------------------------------------------------------ */
/* Naive TRMM (cblas_dtrmm semantics), FP64 and double-double.              */
/* ------------------------------------------------------------------------ */

/* Element (i,j) of op(A) for a column-major triangular A, with the
 * triangle and unit diagonal applied (the other triangle is never read). */
static inline double orc_opA(const double *A, int64_t lda, int upper, int trans, int unit, int64_t i, int64_t j) {
  int64_t r = trans ? j : i, c = trans ? i : j;
  if (r == c) return unit ? 1.0 : A[r + c * lda];
  if (upper ? (r > c) : (r < c)) return 0.0;
  return A[r + c * lda];
}

/* Normalise to column-major: a row-major call is the column-major call on
 * the transposed matrices, i.e. with side and uplo swapped and M, N
 * exchanged (the standard CBLAS reduction). */
static void orc_to_colmajor(int layout, int *side, int *uplo, int64_t *m, int64_t *n) {
  if (layout == ORC_ROW) {
    *side = *side == ORC_LEFT ? ORC_RIGHT : ORC_LEFT;
    *uplo = *uplo == ORC_UPPER ? ORC_LOWER : ORC_UPPER;
    int64_t t = *m; *m = *n; *n = t;
  }
}

/* B := alpha * op(A) * B (side L) or alpha * B * op(A) (side R), naive
 * triple loop with FP64 accumulation, out of place into a scratch copy. */
ORC_EXPORT int orc_dtrmm_naive(int layout, int side, int uplo, int transa, int diag, int64_t m, int64_t n,
                               double alpha, const double *A, int64_t lda, double *B, int64_t ldb) {
  orc_to_colmajor(layout, &side, &uplo, &m, &n);
  int upper = uplo == ORC_UPPER, trans = transa != ORC_NOTRANS, unit = diag == ORC_UNIT;
  double *C = (double *)malloc((size_t)(m * n > 0 ? m * n : 1) * sizeof(double));
  if (!C) return -1;
  for (int64_t j = 0; j < n; j++)
    for (int64_t i = 0; i < m; i++) {
      double s = 0.0;
      if (side == ORC_LEFT)
        for (int64_t k = 0; k < m; k++) s += orc_opA(A, lda, upper, trans, unit, i, k) * B[k + j * ldb];
      else
        for (int64_t k = 0; k < n; k++) s += B[i + k * ldb] * orc_opA(A, lda, upper, trans, unit, k, j);
      C[i + j * m] = alpha * s;
    }
  for (int64_t j = 0; j < n; j++)
    for (int64_t i = 0; i < m; i++) B[i + j * ldb] = C[i + j * m];
  free(C);
  return 0;
}

/* Error-free transformations (Knuth TwoSum, FMA-based TwoProd). */
static inline void orc_two_sum(double a, double b, double *s, double *e) {
  double x = a + b, z = x - a;
  *s = x;
  *e = (a - (x - z)) + (b - z);
}
static inline void orc_dd_add_prod(double *hi, double *lo, double a, double b) {
  double p = a * b, pe = fma(a, b, -p), s, e;
  orc_two_sum(*hi, p, &s, &e);
  e += *lo + pe;
  orc_two_sum(s, e, hi, lo);
}

/* Same contract as orc_dtrmm_naive, but each dot product is accumulated in
 * double-double (about 106 bits) and rounded once: the high-accuracy
 * reference for relative-error reports.  Rows in [row0,row1) and columns in
 * [col0,col1) of the (column-major-normalised) result only; the outputs
 * land in C (ldc), B is not modified. */
ORC_EXPORT int orc_dtrmm_dd(int layout, int side, int uplo, int transa, int diag, int64_t m, int64_t n,
                            double alpha, const double *A, int64_t lda, const double *B, int64_t ldb,
                            int64_t row0, int64_t row1, int64_t col0, int64_t col1, double *C, int64_t ldc) {
  orc_to_colmajor(layout, &side, &uplo, &m, &n);
  int upper = uplo == ORC_UPPER, trans = transa != ORC_NOTRANS, unit = diag == ORC_UNIT;
  if (row1 > m) row1 = m;
  if (col1 > n) col1 = n;
#pragma omp parallel for collapse(2) schedule(dynamic, 4)
  for (int64_t j = col0; j < col1; j++)
    for (int64_t i = row0; i < row1; i++) {
      double hi = 0.0, lo = 0.0;
      if (side == ORC_LEFT)
        for (int64_t k = 0; k < m; k++) orc_dd_add_prod(&hi, &lo, orc_opA(A, lda, upper, trans, unit, i, k), B[k + j * ldb]);
      else
        for (int64_t k = 0; k < n; k++) orc_dd_add_prod(&hi, &lo, B[i + k * ldb], orc_opA(A, lda, upper, trans, unit, k, j));
      C[(i - row0) + (j - col0) * ldc] = alpha * (hi + lo);
    }
  return 0;
}

/* ------------------------------------------------------------------------ */
/* OpenBLAS (the reference's BLAS arithmetic), resolved at run time.        */
/* ------------------------------------------------------------------------ */

typedef void (*orc_dgemm_fn)(int, int, int, int, int, int, double, const double *, int, const double *, int,
                             double, double *, int);
typedef void (*orc_dtrmm_fn)(int, int, int, int, int, int, int, double, const double *, int, double *, int);
typedef void (*orc_setnt_fn)(int);
static orc_dgemm_fn orc_dgemm_p;
static orc_dtrmm_fn orc_dtrmm_p;
static orc_setnt_fn orc_setnt_p;

/* Load the CBLAS library at `path` (the scipy-bundled OpenBLAS, whose
 * exported names carry a `scipy_` prefix, or any plain CBLAS). */
ORC_EXPORT int orc_blas_load(const char *path) {
  void *h = dlopen(path, RTLD_NOW | RTLD_GLOBAL);
  if (!h) return -1;
  orc_dgemm_p = (orc_dgemm_fn)dlsym(h, "scipy_cblas_dgemm");
  orc_dtrmm_p = (orc_dtrmm_fn)dlsym(h, "scipy_cblas_dtrmm");
  orc_setnt_p = (orc_setnt_fn)dlsym(h, "scipy_goto_set_num_threads");
  if (!orc_dgemm_p) orc_dgemm_p = (orc_dgemm_fn)dlsym(h, "cblas_dgemm");
  if (!orc_dtrmm_p) orc_dtrmm_p = (orc_dtrmm_fn)dlsym(h, "cblas_dtrmm");
  if (!orc_setnt_p) orc_setnt_p = (orc_setnt_fn)dlsym(h, "openblas_set_num_threads");
  return (orc_dgemm_p && orc_dtrmm_p) ? 0 : -2;
}

ORC_EXPORT void orc_blas_threads(int t) {
  if (orc_setnt_p) orc_setnt_p(t);
}

ORC_EXPORT int orc_blas_dtrmm(int layout, int side, int uplo, int transa, int diag, int m, int n, double alpha,
                              const double *A, int lda, double *B, int ldb) {
  if (!orc_dtrmm_p) return -1;
  orc_dtrmm_p(layout, side, uplo, transa, diag, m, n, alpha, A, lda, B, ldb);
  return 0;
}

ORC_EXPORT int orc_blas_dgemm(int layout, int ta, int tb, int m, int n, int k, double alpha, const double *A,
                              int lda, const double *B, int ldb, double beta, double *C, int ldc) {
  if (!orc_dgemm_p) return -1;
  orc_dgemm_p(layout, ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C, ldc);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* The reference's per-rank decomposition, all ranks in one process.        */
/* ------------------------------------------------------------------------ */

/* C = tril(A) * B for the reference's row-major n x n problem, computed the
 * way P ranks of uvatrmm.x compute it (UVaTRMM/src/mm_triangular.c:88-99,
 * :319-403):
 *   rank r owns columns map_regular(n, P, r) of B and C (:90);
 *   for each row block s = [b, b+h) of A given by `balanced ? map_balanced
 *   : map_regular` (:88), with the rank's B slice Bl (n x w, ld w):
 *     save rows [b, b+h) of Bl (:334-344, only when P > 1);
 *     C[b:b+h] = A[b:b+h, 0:b+1] * Bl[0:b+1]                 (dgemm, :347-360)
 *     Bl[b+1:b+h] := tril(A[b+1:b+h, b+1:b+h]) * Bl[b+1:b+h]   (dtrmm, :374-387)
 *     C[b+1:b+h] += Bl[b+1:b+h]                               (:388-393)
 *     restore the saved rows (:395-403, only when P > 1).
 * A (n x n, ld n) and B (n x n, ld n) are row-major full matrices; C
 * receives the n x n row-major result.  The message shape (boxes or
 * trapezoid) only changes which bytes MPI moves, never the arithmetic, so
 * it is not a parameter.  Ranks [r0, r1) only (their column slices of C are
 * written, the rest of C is left as is).  Returns -1 where the reference aborts. */
ORC_EXPORT int orc_uvatrmm_ranks(int64_t n, uint32_t P, int balanced, uint32_t r0, uint32_t r1, const double *A,
                                 const double *B, double *C) {
  if (!orc_dgemm_p || !orc_dtrmm_p) return -3;
  if (n < (int64_t)P || r1 > P || r0 > r1) return -1;
  for (uint32_t r = r0; r < r1; r++) {
    uint64_t cb, w;
    if (orc_map_regular((uint64_t)n, P, r, &cb, &w)) return -1;
    double *Bl = (double *)malloc((size_t)n * w * sizeof(double) + 8);
    double *Cl = (double *)calloc((size_t)n * w + 1, sizeof(double));
    if (!Bl || !Cl) return -2;
    for (int64_t i = 0; i < n; i++) memcpy(Bl + i * w, B + i * n + cb, w * sizeof(double));
    for (uint32_t s = 0; s < P; s++) {
      uint64_t b, h;
      int rc = balanced ? orc_map_balanced((uint64_t)n, P, s, &b, &h) : orc_map_regular((uint64_t)n, P, s, &b, &h);
      if (rc) { free(Bl); free(Cl); return -1; }
      double *save = NULL;
      if (P > 1) {
        save = (double *)malloc(h * w * sizeof(double) + 8);
        memcpy(save, Bl + b * w, h * w * sizeof(double));
      }
      /* A row block s as the rank receives it: h x n, ld n. */
      const double *As = A + b * n;
      orc_dgemm_p(ORC_ROW, ORC_NOTRANS, ORC_NOTRANS, (int)h, (int)w, (int)(b + 1), 1.0, As, (int)n, Bl, (int)w, 0.0,
                  Cl + b * w, (int)w);
      int64_t tri = (int64_t)h - 1;
      if (tri > n) tri = n;
      if (tri < 0) tri = 0;
      int64_t bcols = (int64_t)w < n ? (int64_t)w : n;
      int64_t left = (int64_t)(b + h) - tri; /* = b + 1 */
      int64_t above = (int64_t)h - tri;      /* = 1 */
      if (tri > 0)
        orc_dtrmm_p(ORC_ROW, ORC_LEFT, ORC_LOWER, ORC_NOTRANS, ORC_NONUNIT, (int)tri, (int)bcols, 1.0,
                    As + above * n + left, (int)n, Bl + left * w, (int)w);
      for (int64_t f = left; f < left + tri; f++)
        for (int64_t c = 0; c < bcols; c++) Cl[f * w + c] += Bl[f * w + c];
      if (P > 1) {
        memcpy(Bl + b * w, save, h * w * sizeof(double));
        free(save);
      }
    }
    for (int64_t i = 0; i < n; i++) memcpy(C + i * n + cb, Cl + i * w, w * sizeof(double));
    free(Bl);
    free(Cl);
  }
  return 0;
}

/* All P ranks (the whole product). */
ORC_EXPORT int orc_uvatrmm_product(int64_t n, uint32_t P, int balanced, const double *A, const double *B,
                                   double *C) {
  return orc_uvatrmm_ranks(n, P, balanced, 0, P, A, B, C);
}

/* matrix_rangeInfinityNorm (UVaTRMM/src/mm_triangular_common.c:2936-2991):
 * max over rows of the sum of |C[i, :]| for a row-major rows x cols C. */
ORC_EXPORT double orc_inf_norm(int64_t rows, int64_t cols, const double *C, int64_t ldc) {
  double norm = 0.0;
  for (int64_t i = 0; i < rows; i++) {
    double s = 0.0;
    for (int64_t j = 0; j < cols; j++) s += fabs(C[i * ldc + j]);
    if (s > norm) norm = s;
  }
  return norm;
}
