// Internal host-side pieces shared by the C-ABI translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>

#include "uvatrmm.h"

struct uvatrmm_handle_st {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  int engine = UVATRMM_ENGINE_DFMA;
  int schedule = UVATRMM_SCHED_DYNAMIC;
  int shape = UVATRMM_SHAPE_TRAPEZOID;
  int tile = 0;
  int64_t ozaki_scratch_mb = 49152;  // residue-plane budget per pass (MiB)
  bool autotune = true;
  int oz_raster = 0;  // residue-GEMM raster group of single Ozaki calls (0 = default)
  uint32_t expiry_test_polls = 0;  // UVATRMM_OPT_WAIT_EXPIRY_TEST (0 = off)
  bool oz_err_host = false;        // UVATRMM_OPT_OZAKI_ERR_HOST
  // Grow-only device workspace slots: 0-2 plain-path and GEMM staging,
  // 3 reductions, 4 Ozaki scales, 5 Ozaki residue planes, 6 Ozaki product
  // residues, 7 Ozaki error-estimate scratch and the block-cyclic pointer
  // tables.  Calls on a handle are serialised by `mu` and a slot's contents
  // live only within one call (a slot that grows first drains the stream).
  static constexpr int kSlots = 8;
  void *ws[kSlots] = {};
  size_t ws_cap[kSlots] = {};
  int *dctl = nullptr;  // [0] tile counter, [1] kernel status word
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // Per-stage GPU timing of the last Ozaki call (UVATRMM_OPT_STAGE_TIMING):
  // events bracket scaling, each pass's slicing and GEMM, and reassembly.
  bool stage_timing = false;
  static constexpr int kStageEvents = 48;
  cudaEvent_t sev[kStageEvents] = {};
  int n_sev = 0;
  int sev_kind[kStageEvents] = {};  // stage the interval ending at this event belongs to
  // Host staging for host operands outside uvatrmm_host_alloc memory: two
  // page-locked huge-page buffers used alternately (host_mem.cu).
  size_t hstage_bytes = (size_t)256 << 20;  // chunk size (UVATRMM_OPT_HOST_STAGE_KB)
  void *hstage[2] = {};
  size_t hstage_cap = 0;
  cudaEvent_t hstage_ev[2] = {};
  std::mutex mu;
};

namespace uvt {

// Thread-local error reporting.
int fail(int status, const std::string &msg);
int ok();
int cuda_fail(cudaError_t e, const char *what);

// Returns the handle to use (the argument, or the calling thread's default
// handle on the current device); nullptr and an error set on failure.
uvatrmm_handle_t resolve(uvatrmm_handle_t h);

// Ensures workspace slot `slot` holds at least `bytes`; returns its pointer or nullptr.
void *workspace(uvatrmm_handle_t h, int slot, size_t bytes);

// Host <-> device 2-D copy (`width` bytes x `height` lines) for the host
// entry points, ordered on h->stream.  Host memory from uvatrmm_host_alloc
// is copied directly; other host memory goes through the handle's staging
// buffers, packed by several CPU threads while the previous chunk's DMA
// runs.  A device-to-host copy has landed in `dst` when this returns.
cudaError_t host_copy2d(uvatrmm_handle_t h, void *dst, size_t dpitch, const void *src, size_t spitch, size_t width,
                        size_t height, cudaMemcpyKind kind);
// Host-to-device copy of the referenced triangle of the ka x ka
// column-major A (lower: rows j..ka-1 of column j; upper: rows 0..j), in
// blocks of kTriCopyCols columns, each block the rectangle over its part of
// the triangle.  The device copy's other entries are left as they were: the
// kernels never use the unreferenced triangle's values.
constexpr int64_t kTriCopyCols = 256;
cudaError_t copy_triangle_h2d(uvatrmm_handle_t h, double *dA, int64_t la, const double *A, int64_t lda, int64_t ka,
                              bool lower);
// True when [p, p + bytes) lies inside one uvatrmm_host_alloc region.
bool host_alloc_contains(const void *p, size_t bytes);
// Frees the handle's staging buffers and events.
void release_host_staging(uvatrmm_handle_t h);

// Reads and clears the kernel status word (synchronising the stream).
int collect_status(uvatrmm_handle_t h);

inline int64_t round_up(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

// Column-major normalised TRMM description (CBLAS row-major calls are
// turned into the column-major call on the transposed matrices).
struct Trmm {
  int side, uplo, trans, unit;  // CBLAS enum values; trans/unit as 0/1
  int64_t m, n;                 // B is m x n
  double alpha;
};
int check_args(int layout, int side, int uplo, int transa, int diag, int64_t m, int64_t n, int64_t lda,
               int64_t ldb);
Trmm normalise(int layout, int side, int uplo, int transa, int diag, int64_t m, int64_t n, double alpha);

// Plain FP64 TRMM on device buffers (stages misaligned operands, and B when
// in place, through workspace slots 0 and 1).
int device_trmm(uvatrmm_handle_t h, int layout, int side, int uplo, int transa, int diag, int64_t m, int64_t n,
                double alpha, const double *dA, int64_t lda, const double *dB, int64_t ldb, double *dC,
                int64_t ldc, bool in_place, int schedule, int shape, double beta = 0.0);

// Ozaki emulated TRMM on device buffers, in place on dB (ozaki_api.cu).
int ozaki_device(uvatrmm_handle_t h, int layout, int side, int uplo, int transa, int diag, int64_t m, int64_t n,
                 double alpha, const double *dA, int64_t lda, double *dB, int64_t ldb, int moduli, double *relerr,
                 int *bits_out);

// Relative Frobenius error of S sampled result vectors `got` against a
// compensated FP64 host computation from op(A) (host memory, column-major
// view of the normalised call) and the S sampled input vectors `b` (both
// stored vector after vector, m entries each for side Left, n for side
// Right); ozaki_err.cu.
double host_ref_relerr(const Trmm &t, const double *A, int64_t lda, int S, const double *b, const double *got);

// Autotuner (tune.cu): tuned tile edge (FP64) or raster group (Ozaki) for a
// problem shape; measures and caches a missing bucket when h->autotune.
int tune_choice(uvatrmm_handle_t h, int tier, int side, int64_t m, int64_t n, int *choice);

// C := beta * C over a column-major rows x cols device block (extras.cu).
int scale_device(uvatrmm_handle_t h, double *C, int64_t ldc, int64_t rows, int64_t cols, double beta);

// ||X - R||_F / ||R||_F over column-major device blocks.
int rel_frobenius(uvatrmm_handle_t h, int64_t rows, int64_t cols, const double *X, int64_t ldx, const double *R,
                  int64_t ldr, double *rel);

}  // namespace uvt
