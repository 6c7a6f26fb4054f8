// Plain FP64 TRMM: launch descriptor shared by the kernel file and the API.
#pragma once

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
};

// Enqueues the kernel on `stream`.  Returns a uvatrmm_status.
int launch_trmm_fp64(const Fp64Launch &L, cudaStream_t stream, const char **why);

// Tile edge the automatic choice picks for this problem.
int fp64_auto_tile(int64_t M, int64_t N, int64_t K, int num_sms);

}  // namespace uvt
