/*
 * uvatrmm -- FP64 triangular matrix multiply (TRMM) on one NVIDIA GB300.
 *
 * C ABI of libuvatrmm.so.  Plain C types only (no CUDA or torch types): a
 * stream is passed as `void *` holding a cudaStream_t, device buffers as
 * plain pointers.  Every `int`-returning entry point returns a
 * uvatrmm_status; `uvatrmm_last_error()` gives the message of the calling
 * thread's most recent failure.
 *
 * What each entry point replaces in the reference (uva-trasgo/UVaTRMM):
 *   cblas_dtrmm            the MKL cblas_dtrmm the reference links
 *                          (UVaTRMM/src/mm_triangular.c:374-387, UVaTRMM/Makefile:20)
 *   uvatrmm_dtrmm*         the same operation with a status return, on host
 *                          or device buffers
 *   uvatrmm_product        the reference's per-rank product loop
 *                          (UVaTRMM/src/mm_triangular.c:319-410) for the whole
 *                          n x n problem, with its row mapping
 *                          (UVaTRMM/src/mm_mapping.c:27-67, :319-366) and
 *                          message shape (UVaTRMM/src/mm_triangular_common.c:434-511,
 *                          :1071-1126) selecting the GPU tile schedule and tile geometry
 *   uvatrmm_gen_*          the reference's input generator
 *                          (UVaTRMM/src/mm_triangular_common.c:1782-1805) and seeded inputs
 *   uvatrmm_inf_norm       matrix_rangeInfinityNorm
 *                          (UVaTRMM/src/mm_triangular_common.c:2936-2991)
 *   uvatrmm_map_rows       map_regular / map_balanced (UVaTRMM/src/mm_mapping.c:27-67, :319-366)
 */
#ifndef UVATRMM_H
#define UVATRMM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define UVATRMM_API __declspec(dllexport)
#else
#define UVATRMM_API __attribute__((visibility("default")))
#endif

/* ---------------------------------------------------------------- status */
typedef enum {
  UVATRMM_OK = 0,
  UVATRMM_EINVAL = -1,      /* invalid argument (as the reference's INVALID_ARGS) */
  UVATRMM_ENOMEM = -2,      /* device or pinned host allocation failed */
  UVATRMM_EDEVICE = -3,     /* a CUDA call failed */
  UVATRMM_ETIMEOUT = -4,    /* a kernel's bounded wait ran out; the context is still usable */
  UVATRMM_EUNSUPPORTED = -5,/* valid but not supported (e.g. no sm_103a device) */
  UVATRMM_EBUSY = -6,       /* serving: admission refused (HBM budget or slots) */
  UVATRMM_ENOTREADY = -7    /* serving: request still in flight */
} uvatrmm_status;

/* ---------------------------------------------------------------- CBLAS enums */
/* Standard CBLAS values.  Declared here unless a CBLAS header came first. */
#if !defined(CBLAS_H) && !defined(__mkl_cblas_h__) && !defined(UVATRMM_ORACLE_MKL_SHIM_H) && \
    !defined(CBLAS_ENUM_DEFINED_H)
typedef enum { CblasRowMajor = 101, CblasColMajor = 102 } CBLAS_LAYOUT;
typedef enum { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 } CBLAS_TRANSPOSE;
typedef enum { CblasUpper = 121, CblasLower = 122 } CBLAS_UPLO;
typedef enum { CblasNonUnit = 131, CblasUnit = 132 } CBLAS_DIAG;
typedef enum { CblasLeft = 141, CblasRight = 142 } CBLAS_SIDE;
#endif

/* Drop-in for cblas_dtrmm (LP64): B := alpha*op(A)*B (side Left) or
 * alpha*B*op(A) (side Right), A triangular, in place on the host buffer B.
 * Same argument meaning as the reference's MKL call
 * (UVaTRMM/src/mm_triangular.c:374-387).  Errors are reported like BLAS
 * xerbla: a message on stderr and B left unchanged; the status is also
 * available from uvatrmm_last_status(). */
UVATRMM_API void cblas_dtrmm(CBLAS_LAYOUT layout, CBLAS_SIDE side, CBLAS_UPLO uplo, CBLAS_TRANSPOSE transa,
                             CBLAS_DIAG diag, int M, int N, double alpha, const double *A, int lda, double *B,
                             int ldb);

/* ---------------------------------------------------------------- handle */
typedef struct uvatrmm_handle_st *uvatrmm_handle_t;

/* Creates a handle bound to the current CUDA device.  A handle owns its
 * workspace and stream setting; use one handle per host thread. */
UVATRMM_API int uvatrmm_create(uvatrmm_handle_t *handle);
UVATRMM_API int uvatrmm_destroy(uvatrmm_handle_t handle);
/* Stream (a cudaStream_t) for the handle's device work; NULL = legacy default stream. */
UVATRMM_API int uvatrmm_set_stream(uvatrmm_handle_t handle, void *stream);

/* Tuning options. */
typedef enum {
  UVATRMM_OPT_ENGINE = 1,   /* UVATRMM_ENGINE_*   FP64 arithmetic engine */
  UVATRMM_OPT_SCHEDULE = 2, /* UVATRMM_SCHED_*    tile-to-SM assignment */
  UVATRMM_OPT_SHAPE = 3,    /* UVATRMM_SHAPE_*    diagonal tile geometry */
  UVATRMM_OPT_TILE = 4,     /* 0 = automatic, 64 or 128: output tile edge */
  UVATRMM_OPT_OZAKI_SCRATCH_MB = 5, /* Ozaki residue-plane budget per pass, MiB (default 49152) */
  UVATRMM_OPT_STAGE_TIMING = 6,     /* 1: time the stages of each Ozaki call (uvatrmm_stage_times) */
  UVATRMM_OPT_AUTOTUNE = 7,         /* 1 (default): measure untuned shape buckets; 0: defaults only */
  UVATRMM_OPT_OZAKI_RASTER = 8,     /* Ozaki residue GEMM of single calls: major tiles per raster
                                       group (0 = default: 2; or 1..64) */
  UVATRMM_OPT_HOST_STAGE_KB = 9,    /* chunk of the host staging used for host operands outside
                                       uvatrmm_host_alloc memory, KiB (0 = default 262144; >= 64) */
  UVATRMM_OPT_WAIT_EXPIRY_TEST = 10,/* tests of the failure path only: 0 = off (default); N > 0 makes
                                       the plain FP64 kernels of this handle wait N polls on a barrier
                                       that nothing completes, so they end with UVATRMM_ETIMEOUT at the
                                       next uvatrmm_sync (the context stays usable) */
  UVATRMM_OPT_OZAKI_ERR_HOST = 11   /* 1: uvatrmm_ozaki_dtrmm_device's relerr_out is measured against
                                       the host FP64 reference (A and the samples copied to the host),
                                       as uvatrmm_ozaki_dtrmm's always is; 0 (default): against the
                                       plain FP64 kernel on the device */
} uvatrmm_option;
typedef enum { UVATRMM_ENGINE_DFMA = 0, UVATRMM_ENGINE_DMMA = 1 } uvatrmm_engine;
/* DYNAMIC: persistent CTAs pull tiles from a counter, in bands of 1024
 * columns of the non-triangular operand, longest row tiles first in a band.
 * REG / BALANCED: the reference's row mappings (map_regular / map_balanced)
 * applied to row tiles; each CTA owns one row block x one column panel. */
typedef enum { UVATRMM_SCHED_DYNAMIC = 0, UVATRMM_SCHED_REG = 1, UVATRMM_SCHED_BALANCED = 2 } uvatrmm_schedule;
/* TRAPEZOID: diagonal tiles skip the zero half (the reference's exact
 * trapezoid message).  BOXES: diagonal tiles are computed as full boxes with
 * the zero half masked (the reference's bounding-box message). */
typedef enum { UVATRMM_SHAPE_TRAPEZOID = 0, UVATRMM_SHAPE_BOXES = 1 } uvatrmm_shape;
UVATRMM_API int uvatrmm_set_option(uvatrmm_handle_t handle, int option, int value);

/* ---------------------------------------------------------------- TRMM */
/* Host buffers, in place on B, with status.  handle may be NULL (a
 * per-thread default handle on the current device is used). */
UVATRMM_API int uvatrmm_dtrmm(uvatrmm_handle_t handle, int layout, int side, int uplo, int transa, int diag,
                              int64_t m, int64_t n, double alpha, const double *A, int64_t lda, double *B,
                              int64_t ldb);

/* Asynchronous uvatrmm_dtrmm for pipelines: enqueues the copies of A and B
 * to the device, the product and the copy of the result into B on the
 * handle's stream, and returns.  A and B must lie in uvatrmm_host_alloc
 * memory (else UVATRMM_EINVAL) and stay untouched until uvatrmm_sync(handle),
 * which waits and reports the kernel status.  Calls on one handle run in
 * order; calls on two handles whose streams are distinct non-blocking
 * streams (uvatrmm_set_stream; a new handle uses the legacy default stream)
 * overlap one problem's copies with the other's product. */
UVATRMM_API int uvatrmm_dtrmm_async(uvatrmm_handle_t handle, int layout, int side, int uplo, int transa, int diag,
                                    int64_t m, int64_t n, double alpha, const double *A, int64_t lda, double *B,
                                    int64_t ldb);
/* Device buffers, in place on dB, ordered on the handle's stream (returns
 * once the work is enqueued; errors from kernels surface at the next
 * synchronising call or uvatrmm_sync). */
UVATRMM_API int uvatrmm_dtrmm_device(uvatrmm_handle_t handle, int layout, int side, int uplo, int transa,
                                     int diag, int64_t m, int64_t n, double alpha, const double *dA, int64_t lda,
                                     double *dB, int64_t ldb);

/* Device buffers, out of place: dC := alpha*op(A)*dB (or dB*op(A)); dB unchanged. */
UVATRMM_API int uvatrmm_dtrmm_device_oop(uvatrmm_handle_t handle, int layout, int side, int uplo, int transa,
                                         int diag, int64_t m, int64_t n, double alpha, const double *dA,
                                         int64_t lda, const double *dB, int64_t ldb, double *dC, int64_t ldc);

/* The in-place device TRMM of uvatrmm_dtrmm_device for callers that cannot
 * allocate device memory, e.g. a process whose device memory is all handed
 * to its own pool or arena allocator, or a latency-bound loop that must not
 * take the device-wide synchronisation of cudaMalloc/cudaFree.  No
 * counterpart in the reference (which runs MKL on host memory).
 *
 * No handle: the call allocates nothing.  Its scratch (the staged copy of B,
 * A when dA is not 16-byte aligned with an even lda, and two control words)
 * lives in one fixed 64 MiB device array, so it rejects, with
 * UVATRMM_EINVAL and a message, problems whose staged B (round_up(rows, 16)
 * x cols doubles of the column-major view) plus any staged A exceed it.
 * A device reserves the array when the library's device code is loaded
 * there (the first call on that device under CUDA's default lazy module
 * loading; context creation under CUDA_MODULE_LOADING=EAGER) and holds it
 * until the process exits.  The first call on a device also looks up the
 * array's device address and should come before any stream capture.  All calls on a device share the
 * array: calls whose work overlaps on the GPU race.  Ordered on `stream` (a
 * cudaStream_t, NULL = legacy default stream); returns after the result is
 * in dB, with the kernel's status.  Plain DFMA engine, dynamic schedule. */
UVATRMM_API int uvatrmm_dtrmm_device_noalloc(int layout, int side, int uplo, int transa, int diag, int64_t m,
                                            int64_t n, double alpha, const double *dA, int64_t lda, double *dB,
                                            int64_t ldb, void *stream);

/* ---------------------------------------------------------------- GEMM and the reference's stage */
/* Drop-in for cblas_dgemm (LP64): C := alpha*op(A)*op(B) + beta*C on host
 * buffers, the reference's other local call (UVaTRMM/src/mm_triangular.c:347-360),
 * on the same FP64 tile engine as the TRMM.  Errors as cblas_dtrmm. */
UVATRMM_API void cblas_dgemm(CBLAS_LAYOUT layout, CBLAS_TRANSPOSE transa, CBLAS_TRANSPOSE transb, int M, int N,
                             int K, double alpha, const double *A, int lda, const double *B, int ldb, double beta,
                             double *C, int ldc);
/* The same with a status (host buffers / device buffers on the handle's stream). */
UVATRMM_API int uvatrmm_dgemm(uvatrmm_handle_t handle, int layout, int transa, int transb, int64_t m, int64_t n,
                              int64_t k, double alpha, const double *A, int64_t lda, const double *B, int64_t ldb,
                              double beta, double *C, int64_t ldc);
UVATRMM_API int uvatrmm_dgemm_device(uvatrmm_handle_t handle, int layout, int transa, int transb, int64_t m,
                                     int64_t n, int64_t k, double alpha, const double *dA, int64_t lda,
                                     const double *dB, int64_t ldb, double beta, double *dC, int64_t ldc);
/* One stage of the reference's product loop (UVaTRMM/src/mm_triangular.c:319-410)
 * for one column slice, on device buffers, all row-major: with the row block
 * [b, b+h) of the lower-triangular n x n A as the rank receives it (dAblk, h
 * rows, lda >= b+h), the slice B (n x w, ldb) and C (ldc):
 *   C[b:b+h, :]    = Ablk[:, 0:b+1] * B[0:b+1, :]                   (the dgemm)
 *   C[b+1:b+h, :] += tril(Ablk[1:h, b+1:b+h]) * B[b+1:b+h, :]        (dtrmm + add)
 * B is not modified (the reference saves and restores it around its
 * in-place dtrmm).  A caller that receives row blocks (e.g. over MPI/NCCL)
 * feeds them stage by stage. */
UVATRMM_API int uvatrmm_stage(uvatrmm_handle_t handle, int64_t n, int64_t w, int64_t b, int64_t h,
                              const double *dAblk, int64_t lda, const double *dB, int64_t ldb, double *dC,
                              int64_t ldc);

/* ---------------------------------------------------------------- result files and layouts */
/* The reference's binary result file (print_output_results_generic,
 * UVaTRMM/src/mm_triangular_common.c:2134-2163): int rows, int cols, int
 * {row_begin, nrows, col_begin, ncols}, then nrows rows of ncols doubles
 * (host, row-major block with leading dimension ld). */
UVATRMM_API int uvatrmm_write_result(const char *path, int rows, int cols, int row_begin, int nrows, int col_begin,
                                     int ncols, const double *block, int64_t ld);
/* Reads such a file: header into hdr[6], data into out (capacity doubles). */
UVATRMM_API int uvatrmm_read_result(const char *path, int hdr[6], double *out, int64_t capacity);
/* ScaLAPACK's numroc: rows (or columns) of an n-long dimension split in
 * blocks of nb owned by process iproc of nprocs when the first block sits
 * on isrcproc (the layout of ScaLAPACK/scalapack_sample_trmm.c:66-121). */
UVATRMM_API int64_t uvatrmm_numroc(int64_t n, int64_t nb, int iproc, int isrcproc, int nprocs);
/* 2-D block-cyclic pieces <-> one column-major matrix on the device.
 * locals[p*npcol + q] is process (p, q)'s column-major local matrix with
 * leading dimension lld[p*npcol + q] (both host arrays of device pointers /
 * sizes); blocks are mb x nb, the first block on process (0, 0). */
UVATRMM_API int uvatrmm_bc_gather(uvatrmm_handle_t handle, int64_t m, int64_t n, int64_t mb, int64_t nb, int nprow,
                                  int npcol, const double *const *locals, const int64_t *lld, double *dglobal,
                                  int64_t ldg);
UVATRMM_API int uvatrmm_bc_scatter(uvatrmm_handle_t handle, int64_t m, int64_t n, int64_t mb, int64_t nb, int nprow,
                                   int npcol, const double *dglobal, int64_t ldg, double *const *locals,
                                   const int64_t *lld);

/* ---------------------------------------------------------------- Ozaki (emulated FP64) */
/* The same TRMM computed exactly in integer arithmetic on the bf16 tensor
 * cores and rounded once to FP64 (Ozaki-style splitting with `moduli`
 * residue slices; 0 = automatic, 2..20).  Same arguments and in-place
 * semantics as uvatrmm_dtrmm_device / uvatrmm_dtrmm; there is no reference
 * counterpart (the reference runs FP64 MKL only).  When relerr_out is not
 * NULL it receives the relative Frobenius error of the result over 8 evenly
 * spaced result columns (side Left) or rows (side Right), and the call
 * synchronises.  The reference for that error is FP64 arithmetic on the
 * host: every sampled entry a compensated (Dot2) dot product of op(A) with
 * the sampled input, computed on the host cores from the caller's own A and
 * B for uvatrmm_ozaki_dtrmm, and for uvatrmm_ozaki_dtrmm_device from host
 * copies when UVATRMM_OPT_OZAKI_ERR_HOST is 1 (else from the plain FP64
 * kernel on the device).  *bits_out (if not NULL) receives the bits kept per
 * scaled operand entry. */
UVATRMM_API int uvatrmm_ozaki_dtrmm_device(uvatrmm_handle_t handle, int layout, int side, int uplo, int transa,
                                          int diag, int64_t m, int64_t n, double alpha, const double *dA,
                                          int64_t lda, double *dB, int64_t ldb, int moduli, double *relerr_out,
                                          int *bits_out);
UVATRMM_API int uvatrmm_ozaki_dtrmm(uvatrmm_handle_t handle, int layout, int side, int uplo, int transa, int diag,
                                   int64_t m, int64_t n, double alpha, const double *A, int64_t lda, double *B,
                                   int64_t ldb, int moduli, double *relerr_out, int *bits_out);
/* GPU milliseconds of the last Ozaki call's stages: [0] scaling, [1] residue
 * slicing, [2] residue GEMMs, [3] CRT reassembly (needs
 * UVATRMM_OPT_STAGE_TIMING = 1; synchronises). */
UVATRMM_API int uvatrmm_stage_times(uvatrmm_handle_t handle, double *ms4);
/* Residue slices the automatic choice uses for inner dimension k, and the
 * bits per scaled entry that `moduli` slices give for it. */
UVATRMM_API int uvatrmm_ozaki_plan(int64_t k, int moduli, int *moduli_out, int *bits_out);

/* ---------------------------------------------------------------- grouped batches */
/* No counterpart in the reference (one TRMM per process there).  Many TRMMs
 * of any shape, side, uplo, trans and accuracy tier run as grouped
 * persistent launches (one for every FP64 tile shape in use, one residue
 * GEMM per Ozaki wave) captured once into a CUDA graph. */
typedef enum { UVATRMM_TIER_FP64 = 0, UVATRMM_TIER_OZAKI = 1 } uvatrmm_tier;
typedef struct {
  int layout, side, uplo, transa, diag; /* CBLAS values */
  int64_t m, n;
  double alpha;
  const double *A; /* device */
  int64_t lda;
  double *B; /* device, overwritten with the result */
  int64_t ldb;
  int tier;   /* uvatrmm_tier */
  int moduli; /* Ozaki slices, 0 = automatic */
} uvatrmm_trmm_problem;

typedef struct uvatrmm_group_st *uvatrmm_group_t;
/* Plans the batch: checks every problem, picks its tile shape (autotuner),
 * sizes one workspace arena (Ozaki problems are processed in waves that fit
 * UVATRMM_OPT_OZAKI_SCRATCH_MB), uploads the descriptors and captures the
 * whole batch into a CUDA graph on the handle's stream.  The problems'
 * buffers must stay valid while the group lives; every run recomputes each
 * problem from the current contents of its buffers. */
UVATRMM_API int uvatrmm_group_create(uvatrmm_handle_t handle, const uvatrmm_trmm_problem *problems, int count,
                                    uvatrmm_group_t *group);
/* Launches the captured graph on the handle's stream (asynchronous; use
 * uvatrmm_sync for completion and kernel status). */
UVATRMM_API int uvatrmm_group_run(uvatrmm_group_t group);
/* Plan facts: total m^2 n (or n^2 m) flops, kernel launches per run, FP64
 * tiles, Ozaki residue tiles, Ozaki waves, arena bytes. */
UVATRMM_API int uvatrmm_group_stats(uvatrmm_group_t group, double *flops, int *launches, int64_t *fp64_tiles,
                                   int64_t *ozaki_tiles, int *ozaki_waves, int64_t *arena_bytes);
UVATRMM_API int uvatrmm_group_destroy(uvatrmm_group_t group);

/* ---------------------------------------------------------------- serving */
/* No counterpart in the reference.  A request loop with continuous
 * batching: a server thread admits submitted TRMMs (FIFO) as slots and
 * device memory under the HBM budget free up, and runs "ticks": grouped
 * launches over tile ranges taken from every active request, so requests
 * that arrive while others run join the next tick and share the device
 * with them.  Each output tile is computed whole inside one launch, so a
 * result is bitwise the same alone and in any mix. */
typedef struct uvatrmm_server_st *uvatrmm_server_t;
typedef struct {
  int64_t hbm_budget_bytes; /* device memory for admitted requests' working buffers (default 120e9) */
  int max_active;           /* requests admitted at once (default 512) */
  double tick_fp64_gflop;   /* FP64-tier work per tick (default 12) */
  double tick_ozaki_gflop;  /* bf16 residue-GEMM work per tick (default 3000) */
} uvatrmm_server_config;
typedef struct {
  int64_t submitted, completed, failed, cancelled, refused, ticks;
  double p50_ms, p99_ms, mean_ms, max_ms; /* submit -> result ready, completed requests */
  double served_flops;                    /* sum of m^2 n (side L) / n^2 m (side R) completed */
  double first_submit_s, last_done_s;     /* monotonic seconds */
  int64_t peak_bytes;                     /* largest pool use */
} uvatrmm_server_stats;
/* cfg may be NULL (defaults).  The server has its own streams on the
 * handle's device; the handle is only read at creation. */
UVATRMM_API int uvatrmm_server_create(uvatrmm_handle_t handle, const uvatrmm_server_config *cfg,
                                     uvatrmm_server_t *server);
/* Queues one TRMM and returns its id at once.  operands_on_device != 0: A
 * and B are device pointers that must stay valid (B receives the result);
 * else host pointers, copied in at admission and the result copied back
 * into B.  A request whose working set exceeds the whole budget is refused
 * (UVATRMM_EBUSY). */
UVATRMM_API int uvatrmm_server_submit(uvatrmm_server_t server, const uvatrmm_trmm_problem *problem,
                                     int operands_on_device, int64_t *id);
/* Waits up to timeout_s (< 0: forever) for request `id`: UVATRMM_OK when its
 * result is in B, UVATRMM_ENOTREADY on timeout, or the request's error. */
UVATRMM_API int uvatrmm_server_wait(uvatrmm_server_t server, int64_t id, double timeout_s);
/* Withdraws a request that has not been admitted yet. */
UVATRMM_API int uvatrmm_server_cancel(uvatrmm_server_t server, int64_t id);
UVATRMM_API int uvatrmm_server_get_stats(uvatrmm_server_t server, uvatrmm_server_stats *stats);
/* Latency of completed request `id` in ms (submit -> result ready);
 * UVATRMM_ENOTREADY while it is in flight, its error if it failed. */
UVATRMM_API int uvatrmm_server_latency(uvatrmm_server_t server, int64_t id, double *ms);
/* Finishes every queued request, then stops the server thread. */
UVATRMM_API int uvatrmm_server_destroy(uvatrmm_server_t server);

/* ---------------------------------------------------------------- autotuner */
/* The tuned choice for a problem shape: FP64 tier -> output tile edge (64 or
 * 128); Ozaki tier -> residue-GEMM raster group (1, 2 or 3).  Shapes are
 * bucketed by (tier, side, ceil(log2 m), ceil(log2 n)); a missing bucket is
 * measured on the device (when UVATRMM_OPT_AUTOTUNE is 1, the default) and
 * cached in the file named by $UVATRMM_TUNE_CACHE (default
 * $HOME/.cache/uvatrmm_tune.txt). */
UVATRMM_API int uvatrmm_tune(uvatrmm_handle_t handle, int tier, int side, int64_t m, int64_t n, int *choice);

/* Waits for the handle's stream and reports any kernel-side error
 * (UVATRMM_ETIMEOUT for an expired bounded wait). */
UVATRMM_API int uvatrmm_sync(uvatrmm_handle_t handle);

/* ---------------------------------------------------------------- reference-shaped helpers */
/* Row block `idx` of `nblocks` over `n` rows, by the reference's mapping
 * (schedule UVATRMM_SCHED_REG or UVATRMM_SCHED_BALANCED).  Returns
 * UVATRMM_EINVAL where the reference aborts. */
UVATRMM_API int uvatrmm_map_rows(int schedule, uint64_t n, uint32_t nblocks, uint32_t idx, uint64_t *begin,
                                 uint64_t *size);

/* The reference program's whole product on device buffers: C = tril(A)*B
 * for row-major n x n A, B, C (lda = ldb = ldc = n), with the reference's
 * mapping (reg/balanced) and message shape (boxes/trapezoid) selecting the
 * tile schedule and diagonal-tile geometry.  Returns the GPU time of the
 * multiply in *mult_seconds when non-NULL. */
UVATRMM_API int uvatrmm_product(uvatrmm_handle_t handle, int64_t n, int schedule, int shape, const double *dA,
                                const double *dB, double *dC, double *mult_seconds);

/* Device input generators (bit-identical to the oracle's CPU versions).
 * consecutive: element (i,j) of the n x n row-major matrix is
 *   1/(((i*n + j) mod 2341) + 1), zero above the diagonal when triangular.
 * uniform: element (i,j) of a rows x cols matrix (at d[i*rs + j*cs]) is a
 *   seeded counter-based uniform[-1,1) value of index i*cols+j, times 2^k
 *   with k uniform in [-spread, spread] when spread > 0; tri = 0, 'L' or 'U'
 *   keeps one triangle (incl. diagonal) and writes `fill` elsewhere. */
UVATRMM_API int uvatrmm_gen_consecutive(uvatrmm_handle_t handle, int64_t n, int triangular, double *d);
UVATRMM_API int uvatrmm_gen_uniform(uvatrmm_handle_t handle, uint64_t seed, uint64_t stream, int64_t rows,
                                    int64_t cols, double *d, int64_t rs, int64_t cs, int tri, double fill,
                                    int spread);

/* ||C||_inf of a row-major rows x cols device matrix (max row sum of |C|). */
UVATRMM_API int uvatrmm_inf_norm(uvatrmm_handle_t handle, int64_t rows, int64_t cols, const double *dC,
                                 int64_t ldc, double *norm);

/* ---------------------------------------------------------------- memory */
/* Device memory and copies for C callers that do not include CUDA headers.
 * kind: 1 = host to device, 2 = device to host, 3 = device to device.
 * Copies are ordered on the handle's stream and complete before return. */
UVATRMM_API int uvatrmm_device_alloc(size_t bytes, void **ptr);
UVATRMM_API int uvatrmm_device_free(void *ptr);
UVATRMM_API int uvatrmm_copy(uvatrmm_handle_t handle, void *dst, const void *src, size_t bytes, int kind);
/* Page-locked host memory for the operands of the host entry points
 * (uvatrmm_dtrmm, cblas_dtrmm, ...): zeroed, aligned to the transparent-huge-
 * page size and backed by huge pages where the kernel grants them.  On GB300
 * hosts such buffers keep their full copy rate (2 GiB in ~10 ms) where
 * cudaHostAlloc'd or malloc'd buffers slow down as they age.  Free with
 * uvatrmm_host_free (NULL is accepted; other pointers give UVATRMM_EINVAL). */
UVATRMM_API int uvatrmm_host_alloc(size_t bytes, void **ptr);
UVATRMM_API int uvatrmm_host_free(void *ptr);

/* ---------------------------------------------------------------- errors */
UVATRMM_API const char *uvatrmm_last_error(void);
UVATRMM_API int uvatrmm_last_status(void);
UVATRMM_API const char *uvatrmm_version(void);

#ifdef __cplusplus
}
#endif

#endif /* UVATRMM_H */
