// Ozaki-style split-precision FP64 TRMM on GB300's bf16 tensor cores.
//
// The emulated product C = alpha * Lft * Rgt (the same canonical GEMM view as
// the plain path, one operand triangular) is computed exactly in integers and
// rounded once:
//   1. scaling  - each row p of Lft and column p of Rgt gets a power-of-two
//      scale so its entries become integers of at most t bits
//      (Lft'[i,k] = rint(Lft[i,k] * 2^(t - e_i)), likewise Rgt');
//   2. slicing  - every integer is cut into its residues modulo N pairwise
//      coprime moduli m_l <= 363; each residue, balanced into [-181, 181],
//      is exactly representable in bf16 (integers up to 256 are);
//   3. products - for every modulus, one bf16 x bf16 -> fp32 tcgen05 GEMM of
//      the residue matrices.  Products are at most 181^2 and every K chunk
//      of 512 is reduced modulo m_l in the fp32 accumulator (in TMEM) before
//      the next (512 * 181^2 + 184 < 2^24), so every accumulated value is an
//      integer below 2^24 and the accumulation is exact.  The kernel stores
//      y_l = u_l C' mod m_l as 16-bit words, u_l = (M/m_l)^-1 mod m_l
//      (M = prod m_l);
//   4. reassembly - the Chinese remainder theorem rebuilds C' (|C'| < M/4)
//      per element as S - k M with S = sum_l y_l (M/m_l) and k = rint(S/M),
//      which is rounded once to FP64 and scaled back by
//      2^(e_i + d_j - 2t) * alpha.
// Moduli of about 8.4 bits (rather than 8 with m_l <= 256) give the 121 bits
// that 54-bit entries need at K = 32768 with 15 products instead of 16.
// N (the slice count) sets M and hence t; see ozaki_bits().
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

namespace uvt {

constexpr int kMaxModuli = 20;
// Pairwise coprime, largest first (greedy from 363 down): 3*11^2, 2*181, 19^2,
// 359, 5*71, 353, 349, 347, 7^3, 337, 331, 317, 313, 311, 307, 13*23, 293,
// 17^2, 283, 281.
constexpr int kModuli[kMaxModuli] = {363, 362, 361, 359, 355, 353, 349, 347, 343, 337,
                                     331, 317, 313, 311, 307, 299, 293, 289, 283, 281};

// u_l = (M/m_l)^-1 mod m_l for the first n moduli, M = prod_{j<n} m_j.
constexpr int crt_u(int n, int l) {
  const int m = kModuli[l];
  int prod = 1;
  for (int j = 0; j < n; ++j)
    if (j != l) prod = prod * (kModuli[j] % m) % m;
  // Extended Euclid: prod * u = 1 (mod m).
  int r0 = m, r1 = prod, t0 = 0, t1 = 1;
  while (r1) {
    const int q = r0 / r1, r2 = r0 - q * r1, t2 = t0 - q * t1;
    r0 = r1; r1 = r2; t0 = t1; t1 = t2;
  }
  return t0 < 0 ? t0 + m : t0;
}

// Bits t kept per scaled operand entry for n moduli and inner dimension K:
// the largest t with K * 2^(2t) < M / 4.
int ozaki_bits(int n_moduli, int64_t K);
// Slice count the automatic choice uses for inner dimension K (t >= 52).
int ozaki_auto_moduli(int64_t K);

// One operand of the emulated product as the residue kernels see it:
// P[p, k] = kcontig ? X[k + p*ld] : X[p + k*ld], p < P, k < K.
// `tri` = 0: dense; 1: this operand is op(A); then the triangle test uses
// (r, c) = p_is_row ? (p, k) : (k, p).
struct OzOperand {
  const double *X;
  int64_t ld;
  int64_t P, K;
  bool kcontig;
  bool tri, p_is_row, lower, unit;
};

struct OzPlan {
  int n_moduli;       // N
  int bits;           // t
  int64_t M, N, K;    // canonical GEMM sizes
  int64_t Mp, Np, Kp; // padded: Mp % 256 == 0, Np % 256 == 0, Kp % 64 == 0
};

// Padded extents of the residue planes: the residue GEMM's CTA pairs cover
// 256 rows (two 128-row tiles) x 256 columns, its K slabs are 64 wide.  The
// K range of a pair (triangular Lft) or of a column tile (triangular Rgt) is
// set per block of kOzBlock rows of the triangular operand: [0, b + 256) when
// its nonzeros lie at k <= p, [b, K) when at k >= p (b = the block's first
// row); the slicing skips the residue tiles outside it.
constexpr int kOzBlock = 256;
inline int64_t oz_pad_rows(int64_t M) { return (M + 255) / 256 * 256; }
inline int64_t oz_pad_cols(int64_t N) { return (N + 255) / 256 * 256; }

// Device pieces (ozaki_prep.cu).
// Row/column exponents: e[p] = max over valid k of (ilogb|P[p,k]| + 1).
int oz_scales(const OzOperand &op, int *e, cudaStream_t st);
// Residues of moduli [l0, l1) as bf16 planes R[l - l0][p][k] (p < Pp, k < Kp).
int oz_residues(const OzOperand &op, const int *e, int bits, int l0, int l1, int64_t Pp, int64_t Kp, uint16_t *R,
                cudaStream_t st);
// CRT reassembly of C (column-major, ldc) from residue planes
// res[l][j][i] (uint16, plane stride Mp*Np, ld Mp).
int oz_reassemble(const OzPlan &plan, const uint16_t *res, const int *e_row, const int *e_col, double alpha,
                  double *C, int64_t ldc, cudaStream_t st);

// Grouped slicing and reassembly for a wave of problems (one launch per
// stage): scales (each block covers all of K, so no prior fill), residue
// planes of all moduli, and the CRT reassembly into C.
struct OzWaveItem {
  OzOperand L, R;
  int *e_row, *e_col;
  OzPlan plan;
  uint16_t *LR, *RR;
  const uint16_t *res;
  double alpha;
  double *C;
  int64_t ldc;
};
struct OzWaveTables {
  void *scale, *resid, *crt;
  int n_scale, n_resid, n_crt;
  int64_t b_scale, b_resid, b_crt;
};
size_t oz_wave_table_bytes(int nitems);
// Builds the job tables of `n` items into device memory `dev` (synchronous copies).
int oz_wave_tables(const OzWaveItem *items, int n, void *dev, OzWaveTables *out);
// The same tables as a host image (oz_wave_table_bytes(n) bytes) that the
// caller copies to `dev`; `out` already points into `dev`.
void oz_wave_image(const OzWaveItem *items, int n, void *dev, std::vector<char> &image, OzWaveTables *out);
int oz_wave_prep(const OzWaveTables &t, cudaStream_t st);
int oz_wave_reassemble(const OzWaveTables &t, cudaStream_t st);

// The tcgen05 residue GEMM (ozaki_gemm.cu): for moduli [l0, l1), with residue
// planes LR[l-l0][i][k] (Mp x Kp) and RR[l-l0][j][k] (Np x Kp), writes
// res[l][j][i] = (sum_k LR*RR) mod m_l.  K range per output tile follows the
// triangle (tri_left: rows of Lft; else columns of Rgt).
struct OzGroupProb;
struct OzGemmLaunch {
  const uint16_t *LR, *RR;
  uint16_t *res;
  int64_t Mp, Np, Kp, M, N, K;
  int l0, l1;
  int n_moduli = 0;  // moduli of the CRT set (sets u_l of the stored residues)
  bool tri_left, tri_lower;
  int raster_group = 0;          // major tiles per raster group (0 = default: 4 from m, n >= 16384, else 2)
  OzGroupProb *desc = nullptr;   // device slot for the descriptor (single launches)
  int *status;
  int num_sms;
};
int launch_oz_gemm(const OzGemmLaunch &L, cudaStream_t st, const char **why);

// One residue GEMM of a grouped launch as the device reads it (128-byte
// aligned like CUtensorMap; TMA reads the two tensor maps from global memory).
struct alignas(128) OzGroupProb {
  CUtensorMap tmA, tmB;
  int64_t Mp, Np, M, N, K;
  int l0, l1;
  int tri_left, tri_lower, grows;
  int tiles_m, tiles_n, tiles_per_mod, group;
  uint16_t *res;
  int64_t plane;
  int tile_begin, tile_count;
  int tile_offset;  // first of the problem's own tiles this launch covers
  int nmod;         // moduli of the problem's CRT set
};
// Fills the descriptor of one residue GEMM (tile_begin left to the caller).
int oz_group_prob(const OzGemmLaunch &L, OzGroupProb *out, const char **why);
// Sets the residue GEMM's launch attributes (call before a stream capture).
int oz_gemm_prepare();
// One persistent launch over nprob residue GEMMs (device array sorted by tile_begin).
int launch_oz_gemm_group(const OzGroupProb *dprobs, int nprob, int total_tiles, int *status, int num_sms,
                         cudaStream_t st, const char **why);

}  // namespace uvt
