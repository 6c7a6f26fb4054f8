// Plain FP64 TRMM on GB300: one persistent, warp-specialised kernel.
//
// The reference computes each rank's column slice as, per row block of A, a
// cblas_dgemm over the rectangle left of the diagonal plus a cblas_dtrmm of
// the diagonal triangle and an add (UVaTRMM/src/mm_triangular.c:319-410).
// Here the whole product is one launch: every output tile (BM x BN) of
// C = alpha * Lft * Rgt runs a K loop over 16-wide slabs, clipped to the
// triangle, with dense slabs off the diagonal and masked slabs on it.
//
// * Staging: one producer warp issues 2-D TMA loads (cp.async.bulk.tensor)
//   of the Lft and Rgt slabs into a STAGES-deep shared-memory ring guarded by
//   full/empty mbarriers; K-contiguous slabs use the 128-byte swizzle so the
//   consumers' strided reads stay (nearly) conflict-free.
// * Compute: eight consumer warps.  Engine DFMA: each thread owns a
//   (BM/16) x (BN/16) register tile (rows ty+16*ii, columns tx+16*jj).
//   Engine DMMA: each warp owns a 2x4 share of the tile in m8n8k4 FP64
//   tensor-core fragments (mma.sync ... f64).  On GB300 the FP64 pipe
//   behind DFMA measures faster than DMMA, so DFMA is the default.
// * Diagonal slabs: elements outside the triangle are selected to 0 (the
//   unreferenced triangle may hold anything), the diagonal to 1 for unit
//   diag.  Shape TRAPEZOID skips the register rows / fragments that lie
//   entirely in the zero half (the reference's exact trapezoid message,
//   UVaTRMM/src/mm_triangular_common.c:1071-1126); shape BOXES computes the
//   full bounding box (UVaTRMM/src/mm_triangular_common.c:434-511).
// * Schedule: DYNAMIC = CTAs pull tiles from an atomic counter, band by band
//   of the non-triangular dimension's tiles (a band's panels stay in L2) and
//   longest-first inside a band;
//   REG / BALANCED = each CTA owns one block of the reference's row mapping
//   (UVaTRMM/src/mm_mapping.c:27-67, :319-366) applied to tiles, times one
//   column panel of its column split (UVaTRMM/src/mm_triangular.c:90).
// * Every mbarrier wait is bounded; on expiry the kernel records
//   KERR_WAIT_TIMEOUT, drains its own copies in flight and returns.
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "common.cuh"
#include "tmap.cuh"
#include "trmm_fp64.cuh"

namespace uvt {
namespace {

constexpr int kBK = 16;
constexpr int kMaxBlocks = 256;

enum : int { SF_FIRST = 1, SF_LAST = 2 };

struct StageInfo {
  int ti, tj, kt, flags;  // ti < 0 marks the end of the work
  int prob;               // problem of a grouped launch (0 otherwise)
  int pad[3];
};

struct KParams : TileProb {
  int *counter, *status;
  uint32_t spin;    // poll limit of the waits on work (kSpinLimit unless testing expiry)
  int expiry_test;  // consumers first wait on a barrier that nothing completes
  int sched_static, Q, CP;
  int qb[kMaxBlocks + 1];  // work-rank bounds of the Q major blocks
  int cb[kMaxBlocks + 1];  // bounds of the CP minor panels
};

template <int BM>
struct Cfg {
  static constexpr int BN = BM;
  // Consumer warps: 8 for 64-wide tiles (2 CTAs per SM), 16 for 128-wide
  // tiles; plus one producer warp.  Thread grid 16 (columns) x TY (rows).
  static constexpr int NCW = BM == 128 ? 16 : 8;
  static constexpr int THREADS = (NCW + 1) * 32;
  static constexpr int TY = NCW * 32 / 16;
  static constexpr int TM = BM / TY, TN = BN / 16;
  static constexpr int STAGES = BM == 128 ? 4 : 6;
  static constexpr int L_ELEMS = BM * kBK, R_ELEMS = BN * kBK;
  static constexpr uint32_t STAGE_BYTES = (L_ELEMS + R_ELEMS) * 8u;
  static constexpr int MIN_BLOCKS = BM == 128 ? 1 : 2;
  // Ring, full/empty barriers, stage records, and one barrier that only the
  // expiry test waits on.
  static constexpr size_t SMEM =
      1024 + STAGES * (size_t)STAGE_BYTES + STAGES * 16 + STAGES * sizeof(StageInfo) + 16;
};

// Slab element readers.  K-major slabs were written by TMA with the 128-byte
// swizzle: element (row r, k) of a 16-double row sits in 16-byte chunk
// (k/2) XOR (r mod 8).
template <int BM, bool LK>
__device__ __forceinline__ double ldL(const double *Ls, int i, int k) {
  if constexpr (LK)
    return Ls[i * 16 + ((((k >> 1) ^ (i & 7))) << 1) + (k & 1)];
  else
    return Ls[k * BM + i];
}
template <int BN, bool RK>
__device__ __forceinline__ double ldR(const double *Rs, int k, int j) {
  if constexpr (RK)
    return Rs[j * 16 + ((((k >> 1) ^ (j & 7))) << 1) + (k & 1)];
  else
    return Rs[k * BN + j];
}

// Triangle test for op(A)[r, c]: returns 0 outside, 1 inside, 2 on the diagonal.
__device__ __forceinline__ int tri_class(int64_t r, int64_t c, int lower) {
  if (r == c) return 2;
  return lower ? (c < r) : (c > r);
}

__device__ __forceinline__ double tri_select(double v, int cls, int unit) {
  return cls == 0 ? 0.0 : (cls == 2 && unit ? 1.0 : v);
}

__device__ __forceinline__ void tile_kslabs(const TileProb &p, int ti, int tj, int BM, int &kt0, int &kt1) {
  int64_t kb, ke;
  if (p.tri_none) {
    kb = 0;
    ke = p.K;
  } else if (p.tri_left) {
    int64_t i0 = (int64_t)ti * BM;
    if (p.tri_lower) { kb = 0; ke = min(i0 + BM, p.K); }
    else { kb = i0; ke = p.K; }
  } else {
    int64_t j0 = (int64_t)tj * BM;
    if (p.tri_lower) { kb = j0; ke = p.K; }
    else { kb = 0; ke = min(j0 + BM, p.K); }
  }
  kt0 = (int)(kb / kBK);
  kt1 = (int)((ke + kBK - 1) / kBK);
}

// Epilogue store: alpha * acc, plus beta * C when beta != 0 (C unread otherwise).
__device__ __forceinline__ void out_store(const TileProb &p, int64_t i, int64_t j, double acc) {
  double *c = p.C + i + j * p.ldc;
  *c = p.beta != 0.0 ? fma(p.beta, *c, p.alpha * acc) : p.alpha * acc;
}

__device__ __forceinline__ void decode_major(const TileProb &p, int r, int minor, int &ti, int &tj) {
  int major = p.major_rev ? (p.n_major - 1 - r) : r;
  if (p.tri_left) { ti = major; tj = minor; }
  else { ti = minor; tj = major; }
}

// Tile t of the dynamic order.  The minor tiles are cut into bands of
// p.band; a band's tiles run longest major first, all of a major's tiles in
// the band together.  The band's panels of the minor-side operand (K x
// band*BN) then stay in L2 while the major-side panels stream past, instead
// of every minor panel being read again for each major tile.
__device__ __forceinline__ void decode_dynamic(const TileProb &p, int t, int &ti, int &tj) {
  const int per_band = p.n_major * p.band;
  const int b = t / per_band;
  const int local = t - b * per_band;
  const int w = min(p.band, p.n_minor - b * p.band);
  decode_major(p, p.n_major - 1 - local / w, b * p.band + local % w, ti, tj);
}

// ---------------------------------------------------------------- DFMA engine
// Thread (tx, ty) owns rows ty + TY*ii and columns tx + 16*jj of the tile.
// The slab layouts (LK, RK) are template arguments of the slab functions, so
// one engine (one set of accumulator registers) serves every layout.
template <int BM>
struct DfmaEngine {
  using C = Cfg<BM>;
  double acc[C::TM][C::TN];
  int tx, ty;
  int nii, njj;  // register-row blocks / column blocks of this warp inside the tile's valid part

  __device__ void init(int tid) { tx = tid & 15; ty = tid >> 4; }
  // Valid part of the current tile (rows x cols of BM x BN).  A warp owns
  // rows tw + TY*ii and tw + 1 + TY*ii (tw = ty & ~1) and every column block,
  // so both counts are the same in all its lanes.
  __device__ void extent(int rows, int cols) {
    const int tw = ty & ~1;
    nii = rows > tw ? min(C::TM, (rows - tw + C::TY - 1) / C::TY) : 0;
    njj = min(C::TN, (cols + 15) / 16);
  }
  __device__ void zero() {
#pragma unroll
    for (int ii = 0; ii < C::TM; ++ii)
#pragma unroll
      for (int jj = 0; jj < C::TN; ++jj) acc[ii][jj] = 0.0;
  }
  template <bool LK, bool RK>
  __device__ void slab(const double *Ls, const double *Rs) {
#pragma unroll
    for (int k = 0; k < kBK; ++k) {
      double a[C::TM];
#pragma unroll
      for (int ii = 0; ii < C::TM; ++ii) a[ii] = ldL<BM, LK>(Ls, ty + C::TY * ii, k);
#pragma unroll
      for (int jj = 0; jj < C::TN; ++jj) {
        const double b = ldR<C::BN, RK>(Rs, k, tx + 16 * jj);
#pragma unroll
        for (int ii = 0; ii < C::TM; ++ii) acc[ii][jj] = fma(a[ii], b, acc[ii][jj]);
      }
    }
  }
  // Part of a slab: register rows [LO, HI) only and column blocks below
  // njj; with SEL, a diagonal slab (k in [c0, c0 + 16) of the tile's
  // diagonal block) whose triangle lies on the left operand.  Rows left out
  // never issue their FMAs: a predicated-off DFMA still holds the FP64 pipe
  // (measured: per-lane skip predicates saved no time), so the row range is
  // a template argument and the column blocks are left by a branch.
  template <bool LK, bool RK, int LO, int HI, bool SEL>
  __device__ void part(const double *Ls, const double *Rs, int c0, bool lower, bool unit) {
#pragma unroll 1
    for (int k = 0; k < kBK; ++k) {
      double a[C::TM];
#pragma unroll
      for (int ii = LO; ii < HI; ++ii) {
        const int r = ty + C::TY * ii;
        a[ii] = ldL<BM, LK>(Ls, r, k);
        if (SEL) a[ii] = tri_select(a[ii], tri_class(r, c0 + k, lower), unit);
      }
#pragma unroll
      for (int jj = 0; jj < C::TN; ++jj) {
        if (jj >= njj) break;
        const double b = ldR<C::BN, RK>(Rs, k, tx + 16 * jj);
#pragma unroll
        for (int ii = LO; ii < HI; ++ii) acc[ii][jj] = fma(a[ii], b, acc[ii][jj]);
      }
    }
  }
  template <bool LK, bool RK, bool SEL>
  __device__ void part_rows(const double *Ls, const double *Rs, int lo, int hi, int c0, bool lower, bool unit) {
    static_assert(C::TM == 4, "row-range dispatch covers four register rows");
    switch (lo * 8 + hi) {
#define UVT_PART(L, H) \
  case L * 8 + H: part<LK, RK, L, H, SEL>(Ls, Rs, c0, lower, unit); break;
      UVT_PART(0, 1) UVT_PART(0, 2) UVT_PART(0, 3) UVT_PART(0, 4)
      UVT_PART(1, 2) UVT_PART(1, 3) UVT_PART(1, 4)
      UVT_PART(2, 3) UVT_PART(2, 4)
      UVT_PART(3, 4)
#undef UVT_PART
      default: break;  // no rows of this warp hold work in this slab
    }
  }
  // A slab of a tile that overhangs the matrix: only the register rows and
  // column blocks that hold valid outputs are computed (the others would
  // only multiply the zero fill of the out-of-range TMA boxes).
  template <bool LK, bool RK>
  __device__ void slab_edge(const double *Ls, const double *Rs) {
    part_rows<LK, RK, false>(Ls, Rs, 0, nii, 0, false, false);
  }
  // Diagonal slab `s` (k in [16s, 16s+16) of the tile's diagonal block,
  // whose rows and columns share the same origin).
  template <bool LK, bool RK>
  __device__ void slab_diag(const double *Ls, const double *Rs, int s, const TileProb &p) {
    const bool trap = p.trapezoid, lower = p.tri_lower, unit = p.unit;
    const int c0 = 16 * s;
    if (!p.tri_left) {
#pragma unroll 1
      for (int k = 0; k < kBK; ++k) {
        double a[C::TM];
#pragma unroll
        for (int ii = 0; ii < C::TM; ++ii) a[ii] = ldL<BM, LK>(Ls, ty + C::TY * ii, k);
#pragma unroll
        for (int jj = 0; jj < C::TN; ++jj) {
          if (jj >= njj) break;
          // op(A)[c0 + k, c] with c = tx + 16*jj; with TRAPEZOID, column
          // blocks wholly right (lower) or left (upper) of the slab are
          // skipped (the same in all lanes: c0 is a multiple of 16).
          const int c = tx + 16 * jj;
          const double b = tri_select(ldR<C::BN, RK>(Rs, k, c), tri_class(c0 + k, c, lower), unit);
          if (trap && (lower ? (c > c0 + kBK - 1) : (c < c0))) continue;
#pragma unroll
          for (int ii = 0; ii < C::TM; ++ii) {
            if (ii >= nii) break;
            acc[ii][jj] = fma(a[ii], b, acc[ii][jj]);
          }
        }
      }
      return;
    }
    // op(A)[r, c0 + k] with r = ty + TY*ii.  With TRAPEZOID, register rows
    // wholly above (lower) or below (upper) the slab are skipped; a warp's
    // two rows tw, tw + 1 (tw even, c0 a multiple of 16) always fall on the
    // same side, so the row range is the same in all its lanes.
    const int tw = ty & ~1;
    int lo = 0, hi = nii;
    if (trap) {
      if (lower) lo = c0 - tw - 1 > 0 ? (c0 - tw - 1 + C::TY - 1) / C::TY : 0;
      else hi = c0 + kBK - 1 - tw < 0 ? 0 : min(hi, (c0 + kBK - 1 - tw) / C::TY + 1);
    }
    part_rows<LK, RK, true>(Ls, Rs, lo, hi, c0, lower, unit);
  }
  __device__ void store(const TileProb &p, int64_t i0, int64_t j0) {
#pragma unroll
    for (int jj = 0; jj < C::TN; ++jj) {
      int64_t j = j0 + tx + 16 * jj;
      if (j >= p.N) continue;
#pragma unroll
      for (int ii = 0; ii < C::TM; ++ii) {
        int64_t i = i0 + ty + C::TY * ii;
        if (i < p.M) out_store(p, i, j, acc[ii][jj]);
      }
    }
  }
};

// ---------------------------------------------------------------- DMMA engine
__device__ __forceinline__ void dmma884(double &c0, double &c1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
               : "+d"(c0), "+d"(c1)
               : "d"(a), "d"(b));
}

template <int BM>
struct DmmaEngine {
  using C = Cfg<BM>;
  // Warp grid (NCW/4) rows x 4 columns; warp tile WM x WN in m8n8 fragments.
  static constexpr int WM = BM / (C::NCW / 4), WN = C::BN / 4;
  static constexpr int FM = WM / 8, FN = WN / 8;
  double acc[FM][FN][2];
  int r0, c0, g, t;
  int nf, nh;  // row / column fragments of this warp inside the tile's valid part

  __device__ void init(int tid) {
    int w = tid >> 5, lane = tid & 31;
    r0 = (w >> 2) * WM;
    c0 = (w & 3) * WN;
    g = lane >> 2;
    t = lane & 3;
  }
  // Valid part of the current tile; a fragment is a warp's, so both counts
  // are the same in all its lanes.
  __device__ void extent(int rows, int cols) {
    nf = rows > r0 ? min(FM, (rows - r0 + 7) / 8) : 0;
    nh = cols > c0 ? min(FN, (cols - c0 + 7) / 8) : 0;
  }
  // Fragments [0, NF) x [0, NH) of a slab: the fragment counts are template
  // arguments, so the MMAs of fragments outside the matrix are never issued.
  template <bool LK, bool RK, int NF, int NH>
  __device__ void part(const double *Ls, const double *Rs) {
#pragma unroll 1
    for (int k = 0; k < kBK; k += 4) {
      double a[FM], b[FN];
#pragma unroll
      for (int f = 0; f < NF; ++f) a[f] = ldL<BM, LK>(Ls, r0 + 8 * f + g, k + t);
#pragma unroll
      for (int h = 0; h < NH; ++h) b[h] = ldR<C::BN, RK>(Rs, k + t, c0 + 8 * h + g);
#pragma unroll
      for (int f = 0; f < NF; ++f)
#pragma unroll
        for (int h = 0; h < NH; ++h) dmma884(acc[f][h][0], acc[f][h][1], a[f], b[h]);
    }
  }
  template <bool LK, bool RK>
  __device__ void slab_edge(const double *Ls, const double *Rs) {
    static_assert(FM <= 4 && FN <= 4, "fragment-count dispatch covers up to four fragments each way");
    switch (nf * 8 + nh) {
#define UVT_FRAGS(F, H)                                             \
  case F * 8 + H:                                                   \
    if constexpr (F <= FM && H <= FN) part<LK, RK, F, H>(Ls, Rs); \
    break;
      UVT_FRAGS(1, 1) UVT_FRAGS(1, 2) UVT_FRAGS(1, 3) UVT_FRAGS(1, 4)
      UVT_FRAGS(2, 1) UVT_FRAGS(2, 2) UVT_FRAGS(2, 3) UVT_FRAGS(2, 4)
      UVT_FRAGS(3, 1) UVT_FRAGS(3, 2) UVT_FRAGS(3, 3) UVT_FRAGS(3, 4)
      UVT_FRAGS(4, 1) UVT_FRAGS(4, 2) UVT_FRAGS(4, 3) UVT_FRAGS(4, 4)
#undef UVT_FRAGS
      default: break;  // no fragment of this warp inside the matrix
    }
  }
  __device__ void zero() {
#pragma unroll
    for (int f = 0; f < FM; ++f)
#pragma unroll
      for (int h = 0; h < FN; ++h) acc[f][h][0] = acc[f][h][1] = 0.0;
  }
  template <bool LK, bool RK>
  __device__ void slab(const double *Ls, const double *Rs) {
#pragma unroll
    for (int k = 0; k < kBK; k += 4) {
      double a[FM], b[FN];
#pragma unroll
      for (int f = 0; f < FM; ++f) a[f] = ldL<BM, LK>(Ls, r0 + 8 * f + g, k + t);
#pragma unroll
      for (int h = 0; h < FN; ++h) b[h] = ldR<C::BN, RK>(Rs, k + t, c0 + 8 * h + g);
#pragma unroll
      for (int f = 0; f < FM; ++f)
#pragma unroll
        for (int h = 0; h < FN; ++h) dmma884(acc[f][h][0], acc[f][h][1], a[f], b[h]);
    }
  }
  template <bool LK, bool RK>
  __device__ void slab_diag(const double *Ls, const double *Rs, int s, const TileProb &p) {
    const bool trap = p.trapezoid, lower = p.tri_lower, unit = p.unit;
#pragma unroll 1
    for (int k = 0; k < kBK; k += 4) {
      double a[FM], b[FN];
#pragma unroll
      for (int f = 0; f < FM; ++f) a[f] = ldL<BM, LK>(Ls, r0 + 8 * f + g, k + t);
#pragma unroll
      for (int h = 0; h < FN; ++h) b[h] = ldR<C::BN, RK>(Rs, k + t, c0 + 8 * h + g);
      const int kk = 16 * s + k;  // slab-relative k of this step's first column
      if (p.tri_left) {
#pragma unroll
        for (int f = 0; f < FM; ++f) a[f] = tri_select(a[f], tri_class(r0 + 8 * f + g, kk + t, lower), unit);
#pragma unroll
        for (int f = 0; f < FM; ++f) {
          if (f >= nf) break;
          const int rb = r0 + 8 * f;  // fragment rows [rb, rb+8), k columns [kk, kk+4)
          if (trap && (lower ? (kk > rb + 7) : (kk + 3 < rb))) continue;
#pragma unroll
          for (int h = 0; h < FN; ++h) {
            if (h >= nh) break;
            dmma884(acc[f][h][0], acc[f][h][1], a[f], b[h]);
          }
        }
      } else {
#pragma unroll
        for (int h = 0; h < FN; ++h) b[h] = tri_select(b[h], tri_class(kk + t, c0 + 8 * h + g, lower), unit);
#pragma unroll
        for (int h = 0; h < FN; ++h) {
          if (h >= nh) break;
          const int cb = c0 + 8 * h;  // fragment columns [cb, cb+8)
          if (trap && (lower ? (kk + 3 < cb) : (kk > cb + 7))) continue;
#pragma unroll
          for (int f = 0; f < FM; ++f) {
            if (f >= nf) break;
            dmma884(acc[f][h][0], acc[f][h][1], a[f], b[h]);
          }
        }
      }
    }
  }
  __device__ void store(const TileProb &p, int64_t i0, int64_t j0) {
#pragma unroll
    for (int f = 0; f < FM; ++f)
#pragma unroll
      for (int h = 0; h < FN; ++h) {
        int64_t i = i0 + r0 + 8 * f + g;
        int64_t j = j0 + c0 + 8 * h + 2 * t;
        if (i < p.M) {
          if (j < p.N) out_store(p, i, j, acc[f][h][0]);
          if (j + 1 < p.N) out_store(p, i, j + 1, acc[f][h][1]);
        }
      }
  }
};

// ---------------------------------------------------------------- kernel
template <int BM, bool LK, bool RK, template <int> class EngineT>
__global__ void __launch_bounds__(Cfg<BM>::THREADS, Cfg<BM>::MIN_BLOCKS)
    trmm_fp64_kernel(const __grid_constant__ CUtensorMap tmL, const __grid_constant__ CUtensorMap tmR,
                     const __grid_constant__ KParams p) {
  using C = Cfg<BM>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t *full = reinterpret_cast<uint64_t *>(base + C::STAGES * C::STAGE_BYTES);
  uint64_t *empty = full + C::STAGES;
  StageInfo *info = reinterpret_cast<StageInfo *>(empty + C::STAGES);
  uint64_t *never = reinterpret_cast<uint64_t *>(info + C::STAGES);  // nothing arrives on it
  auto Lst = [&](int s) { return reinterpret_cast<double *>(base + s * C::STAGE_BYTES); };
  auto Rst = [&](int s) { return reinterpret_cast<double *>(base + s * C::STAGE_BYTES) + C::L_ELEMS; };

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < C::STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], C::NCW);
    }
    mbar_init(never, 1);
    fence_barrier_init();
  }
  __syncthreads();

  if (warp == C::NCW) {
    // ------------------------------------------------------------ producer
    if (lane == 0) {
      tma_prefetch_desc(&tmL);
      tma_prefetch_desc(&tmR);
      int s = 0;
      uint32_t ph = 0;
      bool ok = true;
      uint32_t issued = 0;
      uint32_t last_ph[C::STAGES];
      auto claim = [&]() -> bool {  // wait until stage s is free
        if (!mbar_wait_bounded(&empty[s], ph ^ 1, p.spin)) {
          record_error(p.status, KERR_WAIT_TIMEOUT);
          return false;
        }
        return true;
      };
      auto advance = [&]() {
        if (++s == C::STAGES) { s = 0; ph ^= 1; }
      };
      auto issue_tile = [&](int ti, int tj) -> bool {
        int kt0, kt1;
        tile_kslabs(p, ti, tj, BM, kt0, kt1);
        const int i0 = ti * BM, j0 = tj * C::BN;
        for (int kt = kt0; kt < kt1; ++kt) {
          if (!claim()) return false;
          info[s] = StageInfo{ti, tj, kt, (kt == kt0 ? SF_FIRST : 0) | (kt == kt1 - 1 ? SF_LAST : 0), 0, {}};
          mbar_arrive_expect_tx(&full[s], C::STAGE_BYTES);
          const int k0 = kt * kBK;
          if constexpr (LK) tma_load_2d(Lst(s), &tmL, k0, i0, &full[s]);
          else tma_load_2d(Lst(s), &tmL, i0, k0, &full[s]);
          if constexpr (RK) tma_load_2d(Rst(s), &tmR, k0, j0, &full[s]);
          else tma_load_2d(Rst(s), &tmR, j0, k0, &full[s]);
          issued |= 1u << s;
          last_ph[s] = ph;
          advance();
        }
        return true;
      };
      if (!p.sched_static) {
        const int total = p.n_major * p.n_minor;
        while (ok) {
          int t = atomicAdd(p.counter, 1);
          if (t >= total) break;
          int ti, tj;
          decode_dynamic(p, t, ti, tj);
          ok = issue_tile(ti, tj);
        }
      } else if ((int)blockIdx.x < p.Q * p.CP) {
        const int q = blockIdx.x / p.CP, c = blockIdx.x % p.CP;
        for (int r = p.qb[q + 1] - 1; ok && r >= p.qb[q]; --r)
          for (int m = p.cb[c]; ok && m < p.cb[c + 1]; ++m) {
            int ti, tj;
            decode_major(p, r, m, ti, tj);
            ok = issue_tile(ti, tj);
          }
      }
      // End-of-work marker (a plain arrive completes the phase).
      if (claim()) {
        info[s] = StageInfo{-1, -1, 0, 0, 0, {}};
        mbar_arrive(&full[s]);
        issued |= 1u << s;
        last_ph[s] = ph;
      }  // else: no stage came free; the consumers' own bounded waits end them
      // Drain: every copy this thread issued must have landed before exit.
      for (int st = 0; st < C::STAGES; ++st)
        if ((issued >> st) & 1u)
          if (!mbar_wait_bounded(&full[st], last_ph[st])) record_error(p.status, KERR_WAIT_TIMEOUT);
    }
  } else {
    // ------------------------------------------------------------ consumers
    EngineT<BM> eng;
    eng.init(threadIdx.x);
    int s = 0;
    uint32_t ph = 0;
    bool go = true;
    if (p.expiry_test && !mbar_wait_bounded(never, 0, p.spin)) {
      record_error(p.status, KERR_WAIT_TIMEOUT);
      go = false;
    }
    while (go) {
      if (!mbar_wait_bounded(&full[s], ph, p.spin)) {
        record_error(p.status, KERR_WAIT_TIMEOUT);
        break;
      }
      const volatile StageInfo *vi = &info[s];
      const StageInfo inf{vi->ti, vi->tj, vi->kt, vi->flags};
      if (inf.ti < 0) break;
      const int64_t i0 = (int64_t)inf.ti * BM, j0 = (int64_t)inf.tj * C::BN;
      const bool edge = i0 + BM > p.M || j0 + C::BN > p.N;
      if (inf.flags & SF_FIRST) {
        eng.zero();
        eng.extent((int)min((int64_t)BM, p.M - i0), (int)min((int64_t)C::BN, p.N - j0));
      }
      const int64_t k0 = (int64_t)inf.kt * kBK;
      const int64_t d0 = p.tri_left ? i0 : j0;
      if (!p.tri_none && k0 >= d0 && k0 < d0 + BM)
        eng.template slab_diag<LK, RK>(Lst(s), Rst(s), (int)((k0 - d0) / kBK), p);
      else if (edge)
        eng.template slab_edge<LK, RK>(Lst(s), Rst(s));
      else
        eng.template slab<LK, RK>(Lst(s), Rst(s));
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[s]);
      if (inf.flags & SF_LAST) eng.store(p, i0, j0);
      if (++s == C::STAGES) { s = 0; ph ^= 1; }
    }
  }
  __syncthreads();
}

// ---------------------------------------------------------------- grouped kernel
// Many TRMMs in one persistent launch: the problems' tiles form one list
// (problem p owns tiles [tile_begin, tile_begin + tile_count)), pulled from
// an atomic counter; inside a problem, in the dynamic order of the
// single-problem kernel (bands, longest tiles first in a band).  Each problem
// carries its own tensor maps (in global memory) and slab layouts, which
// the consumers dispatch on at run time.
__device__ __forceinline__ void tmap_acquire(const CUtensorMap *m) {
  asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(reinterpret_cast<uint64_t>(m))
               : "memory");
}

__device__ __forceinline__ int find_problem(const Fp64GroupProb *probs, int nprob, int t) {
  int lo = 0, hi = nprob - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (probs[mid].tile_begin <= t) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

template <int BM, template <int> class EngineT>
__global__ void __launch_bounds__(Cfg<BM>::THREADS, Cfg<BM>::MIN_BLOCKS)
    trmm_fp64_group_kernel(const Fp64GroupProb *__restrict__ probs, int nprob, int total_tiles, int *counter,
                           int *status) {
  using C = Cfg<BM>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t *full = reinterpret_cast<uint64_t *>(base + C::STAGES * C::STAGE_BYTES);
  uint64_t *empty = full + C::STAGES;
  StageInfo *info = reinterpret_cast<StageInfo *>(empty + C::STAGES);
  auto Lst = [&](int s) { return reinterpret_cast<double *>(base + s * C::STAGE_BYTES); };
  auto Rst = [&](int s) { return reinterpret_cast<double *>(base + s * C::STAGE_BYTES) + C::L_ELEMS; };

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < C::STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], C::NCW);
    }
    fence_barrier_init();
  }
  __syncthreads();

  if (warp == C::NCW) {
    if (lane == 0) {
      int s = 0;
      uint32_t ph = 0, issued = 0;
      uint32_t last_ph[C::STAGES];
      bool ok = true;
      while (ok) {
        const int t = atomicAdd(counter, 1);
        if (t >= total_tiles) break;
        const int pi = find_problem(probs, nprob, t);
        const Fp64GroupProb &P = probs[pi];
        const TileProb tp = P.tp;
        const int r = t - P.tile_begin + P.tile_offset;
        int ti, tj, kt0, kt1;
        decode_dynamic(tp, r, ti, tj);
        tile_kslabs(tp, ti, tj, BM, kt0, kt1);
        tmap_acquire(&P.tmL);
        tmap_acquire(&P.tmR);
        const int i0 = ti * BM, j0 = tj * C::BN;
        for (int kt = kt0; kt < kt1; ++kt) {
          if (!mbar_wait_bounded(&empty[s], ph ^ 1)) {
            record_error(status, KERR_WAIT_TIMEOUT);
            ok = false;
            break;
          }
          info[s] = StageInfo{ti, tj, kt, (kt == kt0 ? SF_FIRST : 0) | (kt == kt1 - 1 ? SF_LAST : 0), pi, {}};
          mbar_arrive_expect_tx(&full[s], C::STAGE_BYTES);
          const int k0 = kt * kBK;
          if (P.lk) tma_load_2d(Lst(s), &P.tmL, k0, i0, &full[s]);
          else tma_load_2d(Lst(s), &P.tmL, i0, k0, &full[s]);
          if (P.rk) tma_load_2d(Rst(s), &P.tmR, k0, j0, &full[s]);
          else tma_load_2d(Rst(s), &P.tmR, j0, k0, &full[s]);
          issued |= 1u << s;
          last_ph[s] = ph;
          if (++s == C::STAGES) { s = 0; ph ^= 1; }
        }
      }
      if (mbar_wait_bounded(&empty[s], ph ^ 1)) {
        info[s] = StageInfo{-1, -1, 0, 0, 0, {}};
        mbar_arrive(&full[s]);
        issued |= 1u << s;
        last_ph[s] = ph;
      } else {
        record_error(status, KERR_WAIT_TIMEOUT);
      }
      for (int st = 0; st < C::STAGES; ++st)
        if ((issued >> st) & 1u)
          if (!mbar_wait_bounded(&full[st], last_ph[st])) record_error(status, KERR_WAIT_TIMEOUT);
    }
  } else {
    EngineT<BM> eng;
    eng.init(threadIdx.x);
    int s = 0;
    uint32_t ph = 0;
    while (true) {
      if (!mbar_wait_bounded(&full[s], ph)) {
        record_error(status, KERR_WAIT_TIMEOUT);
        break;
      }
      const volatile StageInfo *vi = &info[s];
      const StageInfo inf{vi->ti, vi->tj, vi->kt, vi->flags, vi->prob, {}};
      if (inf.ti < 0) break;
      const Fp64GroupProb &P = probs[inf.prob];
      const TileProb tp = P.tp;
      const int64_t i0 = (int64_t)inf.ti * BM, j0 = (int64_t)inf.tj * C::BN;
      const bool edge = i0 + BM > tp.M || j0 + C::BN > tp.N;
      if (inf.flags & SF_FIRST) {
        eng.zero();
        eng.extent((int)min((int64_t)BM, tp.M - i0), (int)min((int64_t)C::BN, tp.N - j0));
      }
      const int64_t k0 = (int64_t)inf.kt * kBK;
      const int64_t d0 = tp.tri_left ? i0 : j0;
      const double *Ls = Lst(s), *Rs = Rst(s);
      const int lay = (P.lk ? 2 : 0) | (P.rk ? 1 : 0);
      if (!tp.tri_none && k0 >= d0 && k0 < d0 + BM) {
        const int sd = (int)((k0 - d0) / kBK);
        switch (lay) {
          case 3: eng.template slab_diag<true, true>(Ls, Rs, sd, tp); break;
          case 2: eng.template slab_diag<true, false>(Ls, Rs, sd, tp); break;
          case 1: eng.template slab_diag<false, true>(Ls, Rs, sd, tp); break;
          default: eng.template slab_diag<false, false>(Ls, Rs, sd, tp); break;
        }
      } else if (edge) {
        switch (lay) {
          case 3: eng.template slab_edge<true, true>(Ls, Rs); break;
          case 2: eng.template slab_edge<true, false>(Ls, Rs); break;
          case 1: eng.template slab_edge<false, true>(Ls, Rs); break;
          default: eng.template slab_edge<false, false>(Ls, Rs); break;
        }
      } else {
        switch (lay) {
          case 3: eng.template slab<true, true>(Ls, Rs); break;
          case 2: eng.template slab<true, false>(Ls, Rs); break;
          case 1: eng.template slab<false, true>(Ls, Rs); break;
          default: eng.template slab<false, false>(Ls, Rs); break;
        }
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[s]);
      if (inf.flags & SF_LAST) eng.store(tp, i0, j0);
      if (++s == C::STAGES) { s = 0; ph ^= 1; }
    }
  }
  __syncthreads();
}

template <int BM, bool LK, bool RK, template <int> class EngineT>
int launch_variant(const CUtensorMap &tmL, const CUtensorMap &tmR, const KParams &kp, int grid,
                   cudaStream_t stream) {
  auto kern = trmm_fp64_kernel<BM, LK, RK, EngineT>;
  static bool attr_set = false;  // per instantiation
  if (!attr_set) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Cfg<BM>::SMEM) !=
        cudaSuccess)
      return UVATRMM_EDEVICE;
    attr_set = true;
  }
  kern<<<grid, Cfg<BM>::THREADS, Cfg<BM>::SMEM, stream>>>(tmL, tmR, kp);
  return cudaGetLastError() == cudaSuccess ? UVATRMM_OK : UVATRMM_EDEVICE;
}

template <int BM, template <int> class EngineT>
int dispatch_layout(bool lk, bool rk, const CUtensorMap &tmL, const CUtensorMap &tmR, const KParams &kp, int grid,
                    cudaStream_t st) {
  if (lk && rk) return launch_variant<BM, true, true, EngineT>(tmL, tmR, kp, grid, st);
  if (lk && !rk) return launch_variant<BM, true, false, EngineT>(tmL, tmR, kp, grid, st);
  if (!lk && rk) return launch_variant<BM, false, true, EngineT>(tmL, tmR, kp, grid, st);
  return launch_variant<BM, false, false, EngineT>(tmL, tmR, kp, grid, st);
}

// map_regular / map_balanced over `n` units into `P` blocks (the C restatement
// lives beside the public uvatrmm_map_rows); fills bounds[0..P].
int fill_bounds(int schedule, int n, int P, int *bounds) {
  bounds[0] = 0;
  for (int q = 0; q < P; ++q) {
    uint64_t b, s;
    if (uvatrmm_map_rows(schedule, (uint64_t)n, (uint32_t)P, (uint32_t)q, &b, &s) != UVATRMM_OK) return -1;
    if ((int)b != bounds[q]) return -1;
    bounds[q + 1] = (int)(b + s);
  }
  return bounds[P] == n ? 0 : -1;
}

// Block counts of the static schedules: the (Q, CP) with Q*CP <= slots that
// minimises the largest CTA's work, where major tile of work rank r costs
// r + 1 slabs-units (the triangle) and a CTA's work is its row block's cost
// times its panel's width.  The reference mapping decides where the blocks
// split; only their number is chosen here.  Results are cached per shape.
void static_grid(int schedule, int n_major, int n_minor, int slots, int *Q_out, int *CP_out) {
  static std::mutex mu;
  static std::map<std::tuple<int, int, int, int>, std::pair<int, int>> cache;
  const auto key = std::make_tuple(schedule, n_major, n_minor, slots);
  {
    std::lock_guard<std::mutex> g(mu);
    auto it = cache.find(key);
    if (it != cache.end()) {
      *Q_out = it->second.first;
      *CP_out = it->second.second;
      return;
    }
  }
  std::vector<int> qb(kMaxBlocks + 1), cb(kMaxBlocks + 1);
  int bestQ = 1, bestCP = 1;
  double best = -1.0;
  for (int CP = 1; CP <= std::min(n_minor, kMaxBlocks) && CP <= slots; CP *= 2) {
    if (fill_bounds(UVATRMM_SCHED_REG, n_minor, CP, cb.data()) != 0) continue;
    int wmax = 0;
    for (int c = 0; c < CP; ++c) wmax = std::max(wmax, cb[c + 1] - cb[c]);
    for (int Q = 1; Q <= std::min(std::min(slots / CP, n_major), kMaxBlocks); ++Q) {
      if (fill_bounds(schedule, n_major, Q, qb.data()) != 0) continue;
      double rmax = 0.0;
      for (int q = 0; q < Q; ++q) {
        // sum of (r + 1) over ranks r in [qb[q], qb[q+1])
        const double a = qb[q], b = qb[q + 1];
        rmax = std::max(rmax, 0.5 * (b * (b + 1) - a * (a + 1)));
      }
      const double span = rmax * wmax;
      if (best < 0 || span < best * (1.0 - 1e-9)) {
        best = span;
        bestQ = Q;
        bestCP = CP;
      }
    }
  }
  std::lock_guard<std::mutex> g(mu);
  cache[key] = {bestQ, bestCP};
  *Q_out = bestQ;
  *CP_out = bestCP;
}

}  // namespace

int fp64_auto_tile(int64_t M, int64_t N, int64_t K, int num_sms) {
  // The FP64 pipe, not memory, bounds this kernel on GB300, so the 64-wide
  // tile (two CTAs per SM, no register spills) is the default everywhere;
  // 128 stays selectable through UVATRMM_OPT_TILE.
  (void)M; (void)N; (void)K; (void)num_sms;
  return 64;
}

// A band is 1024 columns (16 panels of 64) of the minor-side operand, cut
// to fewer panels where K x band*BN doubles would exceed 128 MB (the L2).
// Measured DRAM bytes per launch (m = n, side L) were lowest with this rule
// among fixed byte budgets of 16-256 MB at m = 4096, 8192 and 16384.
int fp64_dynamic_band(int64_t K, int BN, int n_minor) {
  constexpr int64_t kBandBytes = 128ll << 20;
  const int64_t panel = std::max<int64_t>(1, K) * BN * 8;
  const int64_t w = std::min<int64_t>(1024 / BN, kBandBytes / panel);
  return (int)std::max<int64_t>(1, std::min<int64_t>(n_minor, w));
}

int launch_trmm_fp64(const Fp64Launch &L, cudaStream_t stream, const char **why) {
  *why = nullptr;
  if (L.M <= 0 || L.N <= 0 || L.K <= 0) return UVATRMM_OK;
  const int BM = L.tile ? L.tile : fp64_auto_tile(L.M, L.N, L.K, L.num_sms);
  if (BM != 64 && BM != 128) {
    *why = "tile must be 0, 64 or 128";
    return UVATRMM_EINVAL;
  }
  if (L.M > INT32_MAX / 2 || L.N > INT32_MAX / 2 || L.K > INT32_MAX / 2) {
    *why = "dimension too large";
    return UVATRMM_EINVAL;
  }
  CUtensorMap tmL, tmR;
  const uint32_t boxL_in = L.lft_kmajor ? kBK : BM, boxL_out = L.lft_kmajor ? BM : kBK;
  const uint32_t boxR_in = L.rgt_kmajor ? kBK : BM, boxR_out = L.rgt_kmajor ? BM : kBK;
  if (make_tmap_2d(&tmL, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 8, L.xl.ptr, L.xl.rows, L.xl.cols, L.xl.ld * 8, boxL_in,
                   boxL_out, L.lft_kmajor) ||
      make_tmap_2d(&tmR, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 8, L.xr.ptr, L.xr.rows, L.xr.cols, L.xr.ld * 8, boxR_in,
                   boxR_out, L.rgt_kmajor)) {
    *why = "tensor map encoding failed (alignment or driver)";
    return UVATRMM_EDEVICE;
  }

  KParams kp;
  memset(&kp, 0, sizeof(kp));
  kp.M = L.M; kp.N = L.N; kp.K = L.K; kp.ldc = L.ldc;
  kp.alpha = L.alpha; kp.beta = L.beta; kp.C = L.C; kp.counter = L.counter; kp.status = L.status;
  kp.spin = L.expiry_test_polls ? L.expiry_test_polls : kSpinLimit;
  kp.expiry_test = L.expiry_test_polls != 0;
  kp.tri_left = L.tri_left; kp.tri_lower = L.tri_lower; kp.unit = L.unit;
  kp.tri_none = L.tri_none;
  kp.trapezoid = L.shape == UVATRMM_SHAPE_TRAPEZOID;
  const int tiles_m = (int)((L.M + BM - 1) / BM), tiles_n = (int)((L.N + BM - 1) / BM);
  kp.n_major = L.tri_left ? tiles_m : tiles_n;
  kp.n_minor = L.tri_left ? tiles_n : tiles_m;
  // Work grows with the major index for (left, lower) and (right, upper).
  const bool grows = L.tri_left ? L.tri_lower : !L.tri_lower;
  kp.major_rev = grows ? 0 : 1;
  kp.band = fp64_dynamic_band(L.K, BM, kp.n_minor);

  const int per_sm = BM == 128 ? Cfg<128>::MIN_BLOCKS : Cfg<64>::MIN_BLOCKS;
  int grid;
  if (L.schedule == UVATRMM_SCHED_DYNAMIC) {
    grid = std::min<int64_t>((int64_t)L.num_sms * per_sm, (int64_t)tiles_m * tiles_n);
    if (cudaMemsetAsync(L.counter, 0, sizeof(int), stream) != cudaSuccess) return UVATRMM_EDEVICE;
  } else {
    // Q row blocks (reference mapping over the major tiles) x CP column
    // panels (map_regular over the minor tiles), Q*CP <= CTAs resident.
    const int slots = L.num_sms * per_sm;
    int Q = 1, CP = 1;
    static_grid(L.schedule, kp.n_major, kp.n_minor, slots, &Q, &CP);
    if (fill_bounds(L.schedule, kp.n_major, Q, kp.qb) != 0 ||
        fill_bounds(UVATRMM_SCHED_REG, kp.n_minor, CP, kp.cb) != 0) {
      *why = "row mapping rejected the tile counts";
      return UVATRMM_EINVAL;
    }
    kp.sched_static = 1;
    kp.Q = Q;
    kp.CP = CP;
    grid = Q * CP;
  }
  const bool lk = L.lft_kmajor, rk = L.rgt_kmajor;
  if (L.engine == UVATRMM_ENGINE_DMMA) {
    if (BM == 128) return dispatch_layout<128, DmmaEngine>(lk, rk, tmL, tmR, kp, grid, stream);
    return dispatch_layout<64, DmmaEngine>(lk, rk, tmL, tmR, kp, grid, stream);
  }
  if (BM == 128) return dispatch_layout<128, DfmaEngine>(lk, rk, tmL, tmR, kp, grid, stream);
  return dispatch_layout<64, DfmaEngine>(lk, rk, tmL, tmR, kp, grid, stream);
}

int fp64_group_prob(const Fp64Launch &L, int BM, Fp64GroupProb *out, const char **why) {
  *why = nullptr;
  memset(out, 0, sizeof(*out));
  if (BM != 64 && BM != 128) {
    *why = "tile must be 64 or 128";
    return UVATRMM_EINVAL;
  }
  if (L.M <= 0 || L.N <= 0 || L.K <= 0 || L.M > INT32_MAX / 2 || L.N > INT32_MAX / 2 || L.K > INT32_MAX / 2) {
    *why = "dimension out of range for a grouped problem";
    return UVATRMM_EINVAL;
  }
  const uint32_t boxL_in = L.lft_kmajor ? kBK : BM, boxL_out = L.lft_kmajor ? BM : kBK;
  const uint32_t boxR_in = L.rgt_kmajor ? kBK : BM, boxR_out = L.rgt_kmajor ? BM : kBK;
  if (make_tmap_2d(&out->tmL, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 8, L.xl.ptr, L.xl.rows, L.xl.cols, L.xl.ld * 8,
                   boxL_in, boxL_out, L.lft_kmajor) ||
      make_tmap_2d(&out->tmR, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 8, L.xr.ptr, L.xr.rows, L.xr.cols, L.xr.ld * 8,
                   boxR_in, boxR_out, L.rgt_kmajor)) {
    *why = "tensor map encoding failed (alignment or driver)";
    return UVATRMM_EDEVICE;
  }
  TileProb &tp = out->tp;
  tp.M = L.M; tp.N = L.N; tp.K = L.K; tp.ldc = L.ldc;
  tp.alpha = L.alpha; tp.beta = L.beta; tp.C = L.C;
  tp.tri_left = L.tri_left; tp.tri_lower = L.tri_lower; tp.unit = L.unit;
  tp.tri_none = L.tri_none;
  tp.trapezoid = L.shape == UVATRMM_SHAPE_TRAPEZOID;
  const int tiles_m = (int)((L.M + BM - 1) / BM), tiles_n = (int)((L.N + BM - 1) / BM);
  tp.n_major = L.tri_left ? tiles_m : tiles_n;
  tp.n_minor = L.tri_left ? tiles_n : tiles_m;
  const bool grows = L.tri_left ? L.tri_lower : !L.tri_lower;
  tp.major_rev = grows ? 0 : 1;
  tp.band = fp64_dynamic_band(L.K, BM, tp.n_minor);
  out->lk = L.lft_kmajor;
  out->rk = L.rgt_kmajor;
  out->tile_count = tiles_m * tiles_n;
  return UVATRMM_OK;
}

namespace {
template <int BM, template <int> class EngineT>
int group_attr() {
  static bool attr_set = false;
  if (!attr_set) {
    if (cudaFuncSetAttribute(trmm_fp64_group_kernel<BM, EngineT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)Cfg<BM>::SMEM) != cudaSuccess)
      return UVATRMM_EDEVICE;
    attr_set = true;
  }
  return UVATRMM_OK;
}

template <int BM, template <int> class EngineT>
int launch_group_variant(const Fp64GroupProb *dprobs, int nprob, int total, int *counter, int *status, int grid,
                         cudaStream_t st) {
  if (int rc = group_attr<BM, EngineT>()) return rc;
  trmm_fp64_group_kernel<BM, EngineT><<<grid, Cfg<BM>::THREADS, Cfg<BM>::SMEM, st>>>(dprobs, nprob, total, counter,
                                                                                      status);
  return cudaGetLastError() == cudaSuccess ? UVATRMM_OK : UVATRMM_EDEVICE;
}
}  // namespace

int fp64_group_prepare(int BM, int engine) {
  if (engine == UVATRMM_ENGINE_DMMA) return BM == 128 ? group_attr<128, DmmaEngine>() : group_attr<64, DmmaEngine>();
  return BM == 128 ? group_attr<128, DfmaEngine>() : group_attr<64, DfmaEngine>();
}

int launch_trmm_fp64_group(const Fp64GroupProb *dprobs, int nprob, int total_tiles, int BM, int engine,
                           int *counter, int *status, int num_sms, cudaStream_t st, const char **why) {
  *why = nullptr;
  if (nprob <= 0 || total_tiles <= 0) return UVATRMM_OK;
  if (BM != 64 && BM != 128) {
    *why = "tile must be 64 or 128";
    return UVATRMM_EINVAL;
  }
  if (cudaMemsetAsync(counter, 0, sizeof(int), st) != cudaSuccess) return UVATRMM_EDEVICE;
  const int per_sm = BM == 128 ? Cfg<128>::MIN_BLOCKS : Cfg<64>::MIN_BLOCKS;
  const int grid = std::min(num_sms * per_sm, total_tiles);
  int rc;
  if (engine == UVATRMM_ENGINE_DMMA)
    rc = BM == 128 ? launch_group_variant<128, DmmaEngine>(dprobs, nprob, total_tiles, counter, status, grid, st)
                   : launch_group_variant<64, DmmaEngine>(dprobs, nprob, total_tiles, counter, status, grid, st);
  else
    rc = BM == 128 ? launch_group_variant<128, DfmaEngine>(dprobs, nprob, total_tiles, counter, status, grid, st)
                   : launch_group_variant<64, DfmaEngine>(dprobs, nprob, total_tiles, counter, status, grid, st);
  if (rc != UVATRMM_OK) *why = "grouped FP64 kernel launch failed";
  return rc;
}

}  // namespace uvt
