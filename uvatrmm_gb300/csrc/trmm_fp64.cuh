// Plain FP64 TRMM: launch descriptor shared by the kernel file and the API.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace uvt {

// One operand source: a column-major matrix X (rows x cols, leading
// dimension ld, in elements).  16-byte aligned base and even ld (the TMA
// rules for FP64); the API layer stages anything else into workspace.
struct MatRef {
  const double *ptr;
  int64_t rows, cols, ld;
};

// Canonical problem, column-major:  C (M x N) = alpha * Lft (M x K) * Rgt (K x N).
//   side Left : Lft = op(A) (triangular, M = K), Rgt = B.
//   side Right: Lft = B, Rgt = op(A) (triangular, K = N).
// Lft is read from X_L with Lft[i,k] = lft_kmajor ? X_L[k,i] : X_L[i,k];
// Rgt is read from X_R with Rgt[k,j] = rgt_kmajor ? X_R[k,j] : X_R[j,k].
struct Fp64Launch {
  MatRef xl, xr;
  double *C;
  int64_t ldc;
  int64_t M, N, K;
  double alpha;
  bool lft_kmajor, rgt_kmajor;
  bool tri_left;   // the triangular operand is Lft (side Left) or Rgt (side Right)
  bool tri_lower;  // op(A) is lower triangular
  bool unit;       // unit diagonal
  int engine;      // UVATRMM_ENGINE_*
  int schedule;    // UVATRMM_SCHED_*
  int shape;       // UVATRMM_SHAPE_*
  int tile;        // 0 auto, 64, 128
  int *counter;    // device int, dynamic schedule (zeroed by the launcher)
  int *status;     // device int, kernel error flags (KERR_*)
  int num_sms;
  double beta = 0.0;     // C = alpha*op*B + beta*C (0: C is only written)
  bool tri_none = false;  // plain GEMM: neither operand triangular
  // Tests of the failure path only (0 = off): the consumers first wait, with
  // this many polls, on a barrier that nothing completes, and every wait on
  // work uses the same limit, so the launch ends with KERR_WAIT_TIMEOUT; the
  // producer's final drain of its copies in flight keeps the default limit.
  uint32_t expiry_test_polls = 0;
};

// Enqueues the kernel on `stream`.  Returns a uvatrmm_status.
int launch_trmm_fp64(const Fp64Launch &L, cudaStream_t stream, const char **why);

// What the kernel's tile walk, engines and epilogue need about one problem.
struct TileProb {
  int64_t M, N, K, ldc;
  double alpha, beta;  // C = alpha * Lft * Rgt + beta * C (C is not read when beta == 0)
  double *C;
  int tri_left, tri_lower, unit, trapezoid;
  int tri_none;                     // no triangular operand: a plain GEMM over all of K
  int n_major, n_minor, major_rev;  // tiles along the triangular dimension / the other one
  int band;                         // minor tiles per band of the dynamic order (1..n_minor)
};

// Minor tiles per band of the dynamic tile order for a problem with inner
// dimension K and n_minor minor tiles of edge BN.
int fp64_dynamic_band(int64_t K, int BN, int n_minor);

// One problem of a grouped launch, as the device reads it (128-byte aligned
// like CUtensorMap: the tensor maps are read by TMA from global memory).
struct alignas(128) Fp64GroupProb {
  CUtensorMap tmL, tmR;
  TileProb tp;
  int lk, rk;
  int tile_begin, tile_count;
  int tile_offset;  // first of the problem's own tiles this launch covers
};

// Fills `out` for problem L with tile edge BM (tile_begin left to the caller).
int fp64_group_prob(const Fp64Launch &L, int BM, Fp64GroupProb *out, const char **why);
// Sets the grouped kernel's launch attributes (call before a stream capture).
int fp64_group_prepare(int BM, int engine);
// One persistent launch over `nprob` problems (device array `dprobs`, sorted
// by tile_begin, tiles [0, total_tiles)); `counter` is zeroed here.
int launch_trmm_fp64_group(const Fp64GroupProb *dprobs, int nprob, int total_tiles, int BM, int engine,
                           int *counter, int *status, int num_sms, cudaStream_t stream, const char **why);

// Tile edge the automatic choice picks for this problem.
int fp64_auto_tile(int64_t M, int64_t N, int64_t K, int num_sms);

}  // namespace uvt
