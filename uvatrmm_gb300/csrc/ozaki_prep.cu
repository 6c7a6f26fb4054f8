// Ozaki path, memory-bound stages: per-row/column power-of-two scales, the
// residue planes (slicing), and the CRT reassembly to FP64.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "api_internal.h"
#include "common.cuh"
#include "ozaki.cuh"

namespace uvt {
namespace {

constexpr int kExpNone = (int)0x80808080;  // "no nonzero entry" (memset byte 0x80)
constexpr int kMaxBits = 120;              // keeps every shifted mantissa inside 128 bits

// ---------------------------------------------------------------- element access
__device__ __forceinline__ double load_elem(const OzOperand &op, int64_t p, int64_t k) {
  if (p >= op.P || k >= op.K) return 0.0;
  if (op.tri) {
    const int64_t r = op.p_is_row ? p : k, c = op.p_is_row ? k : p;
    if (r == c) return op.unit ? 1.0 : (op.kcontig ? op.X[k + p * op.ld] : op.X[p + k * op.ld]);
    if (op.lower ? (c > r) : (c < r)) return 0.0;
  }
  return op.kcontig ? op.X[k + p * op.ld] : op.X[p + k * op.ld];
}

// ilogb(|v|) + 1 for v != 0 (so |v| < 2^result), from the bit pattern.
__device__ __forceinline__ int exp_above(double v) {
  const uint64_t b = (uint64_t)__double_as_longlong(v);
  const int be = (int)((b >> 52) & 0x7FF);
  if (be) return be - 1023 + 1;
  const uint64_t f = b & ((1ull << 52) - 1);  // subnormal: |v| = f * 2^-1074
  return f ? (63 - __clzll((long long)f)) - 1074 + 1 : kExpNone;
}

// Tiles of 32 (p) x 64 (k) per 256-thread block; grid.y splits K.
constexpr int TP = 32, TK = 64;
static_assert(kOzBlock % TP == 0 && kOzBlock % TK == 0, "a residue tile lies in one K-range block");

// Rows [32 bx, 32 bx + 32) of the operand over k in [by * kpb, (by+1) * kpb):
// the maximum exponent per row.  `direct`: this block covers all of K, so it
// writes e[p] itself (no prior fill, no atomics across blocks).
__device__ __forceinline__ void scale_body(const OzOperand &op, int *e, int64_t bx, int64_t by, int64_t k_per_block,
                                           bool direct) {
  __shared__ int red[TP];
  const int tid = threadIdx.x;
  if (tid < TP) red[tid] = kExpNone;
  __syncthreads();
  const int64_t p0 = bx * TP;
  const int64_t kb = by * k_per_block, ke = min(op.K, kb + k_per_block);
  int best = kExpNone;
  if (op.kcontig) {
    // warp w handles rows p0 + w, p0 + w + 8, ...; lanes stride over k
    const int w = tid >> 5, ln = tid & 31;
    for (int pp = w; pp < TP; pp += 8) {
      int b2 = kExpNone;
      for (int64_t k = kb + ln; k < ke; k += 32) {
        const double v = load_elem(op, p0 + pp, k);
        if (__double_as_longlong(v) << 1) b2 = max(b2, exp_above(v));
      }
#pragma unroll
      for (int o = 16; o; o >>= 1) b2 = max(b2, __shfl_xor_sync(0xffffffffu, b2, o));
      if (ln == 0) atomicMax(&red[pp], b2);
    }
  } else {
    const int pp = tid & 31, ky = tid >> 5;
    for (int64_t k = kb + ky; k < ke; k += 8) {
      const double v = load_elem(op, p0 + pp, k);
      if (__double_as_longlong(v) << 1) best = max(best, exp_above(v));
    }
    atomicMax(&red[pp], best);
  }
  __syncthreads();
  if (tid < TP && p0 + tid < op.P) {
    if (direct) e[p0 + tid] = red[tid];
    else if (red[tid] != kExpNone) atomicMax(&e[p0 + tid], red[tid]);
  }
}

__global__ void __launch_bounds__(256) scale_kernel(OzOperand op, int *e, int64_t k_per_block) {
  scale_body(op, e, blockIdx.x, blockIdx.y, k_per_block, false);
}

// ---------------------------------------------------------------- residues
constexpr uint32_t pow2mod(int e, uint32_t m) {
  uint32_t r = 1 % m;
  for (int i = 0; i < e; ++i) r = (r * 2) % m;
  return r;
}

// Balanced residue of x (as four 32-bit words, most significant last) for
// modulus kModuli[L], negated when `neg`, as bf16 bits.
template <int L>
__device__ __forceinline__ uint16_t residue_bf16(const uint32_t (&w)[4], bool neg) {
  constexpr uint32_t m = (uint32_t)kModuli[L];
  constexpr uint32_t c32 = pow2mod(32, m), c64 = pow2mod(64, m), c96 = pow2mod(96, m);
  uint32_t r = ((w[3] % m) * c96 + (w[2] % m) * c64 + (w[1] % m) * c32 + (w[0] % m)) % m;
  if (neg && r) r = m - r;
  const int rs = (int)r > (int)(m / 2) ? (int)r - (int)m : (int)r;
  return __bfloat16_as_ushort(__float2bfloat16_rn((float)rs));
}

template <int L>
__device__ __forceinline__ void store_residues(const uint32_t (&w)[4], bool neg, int l0, int l1, uint16_t *out,
                                               int64_t plane) {
  if constexpr (L < kMaxModuli) {
    if (L >= l0 && L < l1) out[(int64_t)(L - l0) * plane] = residue_bf16<L>(w, neg);
    store_residues<L + 1>(w, neg, l0, l1, out, plane);
  }
}

// Integers below 2^63 (every automatic slice count) go through the FP32
// pipe: x = sum_i d_i 2^(11 i) with six 11-bit digits, so x is congruent to
// s = sum_i d_i (2^(11 i) mod m) < 6 * 2^11 * 363 < 2^23 modulo m, exact in
// fp32.  r = s - m * rint(s / m), rounding by the 1.5 * 2^23 constant in one
// fma, is congruent to x: the quotient's error, at most (s/m) 2^-24 < 0.00074,
// is below the gap 1/(2m) between s/m and a half-integer for the odd moduli,
// and the even modulus 362 only has the tie +-181 either way, so |r| <= 181
// as the residue GEMM's exactness bound requires.

// Digits d_0 .. d_5 of x as exact floats.
__device__ __forceinline__ void digits11(uint64_t x, float (&d)[6]) {
  const uint32_t lo = (uint32_t)x, hi = (uint32_t)(x >> 32);
  const uint32_t v[6] = {lo & 0x7FFu, (lo >> 11) & 0x7FFu, __funnelshift_r(lo, hi, 22) & 0x7FFu,
                         (hi >> 1) & 0x7FFu, (hi >> 12) & 0x7FFu, hi >> 23};
#pragma unroll
  for (int i = 0; i < 6; ++i) d[i] = __int_as_float((int)(0x4B000000u | v[i])) - 8388608.0f;
}

// bf16 bits of a residue of the integer with digits d, modulo kModuli[L].
template <int L>
__device__ __forceinline__ uint32_t residue_bits(const float (&d)[6]) {
  constexpr int m = kModuli[L];
  constexpr float mf = (float)m, inv = 1.0f / (float)m;
  constexpr float c1 = (float)pow2mod(11, m), c2 = (float)pow2mod(22, m), c3 = (float)pow2mod(33, m),
                  c4 = (float)pow2mod(44, m), c5 = (float)pow2mod(55, m);
  float s = fmaf(d[1], c1, d[0]);
  s = fmaf(d[2], c2, s);
  s = fmaf(d[3], c3, s);
  s = fmaf(d[4], c4, s);
  s = fmaf(d[5], c5, s);
  const float q = fmaf(s, inv, 12582912.0f) - 12582912.0f;
  const float r = fmaf(-q, mf, s);
  return __float_as_uint(r) >> 16;  // |r| <= 181: exact in bf16
}

// Residues of four consecutive-k entries for moduli [l0, l1), one 8-byte
// store per plane; sg holds each entry's sign bit at bit 15 of its half.
template <int L>
__device__ __forceinline__ void store4_residues(const float (&d)[4][6], const uint32_t (&sg)[2], int l0, int l1,
                                                uint16_t *out, int64_t plane) {
  if constexpr (L < kMaxModuli) {
    if (L >= l0 && L < l1) {
      uint2 v;
      v.x = (residue_bits<L>(d[0]) | (residue_bits<L>(d[1]) << 16)) ^ sg[0];
      v.y = (residue_bits<L>(d[2]) | (residue_bits<L>(d[3]) << 16)) ^ sg[1];
      *reinterpret_cast<uint2 *>(out + (int64_t)(L - l0) * plane) = v;
    }
    store4_residues<L + 1>(d, sg, l0, l1, out, plane);
  }
}

// The 32 (p) x 64 (k) residue tile (bx = k tile, by = p tile).
__device__ __forceinline__ void residue_body(const OzOperand &op, const int *e, int bits, int l0, int l1, int64_t Pp,
                                             int64_t Kp, uint16_t *R, int64_t bx, int64_t by) {
  __shared__ double tile[TP][TK + 1];
  const int tid = threadIdx.x;
  const int64_t p0 = by * TP, k0 = bx * TK;
  if (op.tri) {
    // The residue GEMM never reads this tile when its K slab is outside the
    // range of the kOzBlock-row block holding it (see kOzBlock).
    const int64_t b = p0 / kOzBlock * kOzBlock;
    const bool k_le_p = op.p_is_row == op.lower;  // nonzeros at k <= p
    if (k_le_p ? k0 >= b + kOzBlock : k0 + TK <= b) return;
  }
  // Load (coalesced along the contiguous dimension of X).
  for (int idx = tid; idx < TP * TK; idx += 256) {
    int pp, kk;
    if (op.kcontig) { kk = idx % TK; pp = idx / TK; }
    else { pp = idx % TP; kk = idx / TP; }
    tile[pp][kk] = load_elem(op, p0 + pp, k0 + kk);
  }
  __syncthreads();
  const int64_t plane = Pp * Kp;
  if (bits <= 63) {
    // Each thread: four consecutive k of rows tid/16 and tid/16 + 16.
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      const int pp = (tid >> 4) + half * (TP / 2), kk0 = (tid & 15) * 4;
      const int ep = e[p0 + pp];
      uint64_t x[4];
      uint32_t sg[2] = {0, 0};
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const double v = tile[pp][kk0 + q];
        x[q] = 0;
        if ((__double_as_longlong(v) << 1) && ep != kExpNone) {
          const uint64_t b = (uint64_t)__double_as_longlong(v);
          const int be = (int)((b >> 52) & 0x7FF);
          const uint64_t mant = be ? ((b & ((1ull << 52) - 1)) | (1ull << 52)) : (b & ((1ull << 52) - 1));
          const int s = (be ? be - 1075 : -1074) + bits - ep;  // scaled integer = mant * 2^s < 2^bits
          if (s >= 0) x[q] = mant << s;
          else if (s > -64) x[q] = (mant + (1ull << (-s - 1))) >> (-s);
          if (b >> 63) sg[q >> 1] |= 0x8000u << (16 * (q & 1));
        }
      }
      float dg[4][6];
#pragma unroll
      for (int q = 0; q < 4; ++q) digits11(x[q], dg[q]);
      store4_residues<0>(dg, sg, l0, l1, R + (p0 + pp) * Kp + (k0 + kk0), plane);
    }
    return;
  }
  for (int idx = tid; idx < TP * TK; idx += 256) {
    const int kk = idx % TK, pp = idx / TK;
    const double v = tile[pp][kk];
    uint32_t w[4] = {0, 0, 0, 0};
    bool neg = false;
    const int ep = e[p0 + pp];
    if ((__double_as_longlong(v) << 1) && ep != kExpNone) {
      const uint64_t b = (uint64_t)__double_as_longlong(v);
      neg = (b >> 63) != 0;
      const int be = (int)((b >> 52) & 0x7FF);
      const uint64_t mant = be ? ((b & ((1ull << 52) - 1)) | (1ull << 52)) : (b & ((1ull << 52) - 1));
      const int ex2 = be ? be - 1075 : -1074;  // |v| = mant * 2^ex2
      const int s = ex2 + bits - ep;            // scaled integer = mant * 2^s
      unsigned __int128 x = 0;
      if (s >= 0) x = (unsigned __int128)mant << s;
      else if (s > -64) x = (mant + (1ull << (-s - 1))) >> (-s);
      w[0] = (uint32_t)x;
      w[1] = (uint32_t)(x >> 32);
      w[2] = (uint32_t)(x >> 64);
      w[3] = (uint32_t)(x >> 96);
    }
    store_residues<0>(w, neg, l0, l1, R + (p0 + pp) * Kp + (k0 + kk), plane);
  }
}

// Six blocks per SM (40 registers, a few bytes spilled to L1): the slicing
// warps mostly wait on the tile's global loads, and the extra blocks hide
// that latency (m = n = 32768: 25.3 against 30.0 ms at four blocks per SM,
// bit-identical residues).
__global__ void __launch_bounds__(256, 6) residue_kernel(OzOperand op, const int *e, int bits, int l0, int l1,
                                                      int64_t Pp, int64_t Kp, uint16_t *R) {
  residue_body(op, e, bits, l0, l1, Pp, Kp, R, blockIdx.x, blockIdx.y);
}

// ---------------------------------------------------------------- reassembly
// The residue GEMM stores y_l = u_l C' mod m_l (0 <= y_l < m_l), so
// S = sum_l y_l P_l with P_l = M/m_l is congruent to C' modulo M and
// S/M = sum_l y_l/m_l < n.  With |C'| <= K 2^(2t) < M/4, C' = S - k M for
// k = rint(S/M), and any estimate of S/M within 1/4 gives that k.  C' is
// formed in L 32-bit limbs (least significant first) in two's complement,
// M < 2^(32L), so limbs above L never matter.  S's limb sums are < 20 * 363 * 2^32.
constexpr int kLimbs = 6;  // L for 20 moduli (M < 2^168)

struct CrtConst {
  int n;
  int bits;
  int limbs;                       // L
  float c_hi, c_lo;                // 2^(32(L-1)) / M, 2^(32(L-2)) / M
  uint32_t P[kMaxModuli][kLimbs];  // P_l = M / m_l
  uint32_t Mw[kLimbs];
};

// d * 2^k, exact when the result is a normal double.
__device__ __forceinline__ double times_pow2(double d, int k) {
  if (k >= -1022 && k <= 1023) return d * __longlong_as_double((long long)(k + 1023) << 52);
  return ldexp(d, k);
}

// One element from its residues (16-bit field `f` of the pairs rw[l]) -> C value (alpha applied).
template <int L, int NM>
__device__ __forceinline__ double crt_element(const CrtConst &cc, const uint2 (&rw)[NM], int f, int er,
                                              int ec, double alpha, bool unit_alpha) {
  uint64_t acc[L];
#pragma unroll
  for (int k = 0; k < L; ++k) acc[k] = 0;
#pragma unroll
  for (int l = 0; l < NM; ++l) {
    if (l < cc.n) {
      const uint32_t y = ((f < 2 ? rw[l].x : rw[l].y) >> (16 * (f & 1))) & 0xFFFFu;
#pragma unroll
      for (int k = 0; k < L; ++k) acc[k] += (uint64_t)y * cc.P[l][k];
    }
  }
  // k from the two top limb sums: the limbs below add less than 2^-20 to S/M
  // and the fp32 rounding stays below 2^-18.
  const float sm = fmaf((float)acc[L - 1], cc.c_hi, (float)acc[L - 2] * cc.c_lo);
  const uint32_t kq = (uint32_t)(sm + 0.5f);
  // X = S - k M in two's complement, then sign and magnitude.
  uint32_t X[L];
  int64_t c = 0;
#pragma unroll
  for (int k = 0; k < L; ++k) {
    c += (int64_t)acc[k] - (int64_t)((uint64_t)kq * cc.Mw[k]);
    X[k] = (uint32_t)c;
    c >>= 32;
  }
  const bool neg = (X[L - 1] >> 31) != 0;
  if (neg) {
    uint32_t cy = 1;
#pragma unroll
    for (int k = 0; k < L; ++k) {
      const uint64_t t = (uint64_t)(~X[k]) + cy;
      X[k] = (uint32_t)t;
      cy = (uint32_t)(t >> 32);
    }
  }
  // Round the magnitude to FP64 once: a 64-bit window below the top bit,
  // with a sticky bit for everything under it.
  int t = 0;
#pragma unroll
  for (int k = 1; k < L; ++k)
    if (X[k]) t = k;
  uint64_t top;
  int ex;
  if (t == 0) {
    top = X[0];
    ex = 0;
  } else {
    const int lz = __clz(X[t]);
    const uint64_t w = ((uint64_t)X[t] << 32) | X[t - 1];
    const uint32_t below = t >= 2 ? X[t - 2] : 0u;
    top = lz ? (w << lz) | (below >> (32 - lz)) : w;
    bool sticky = (lz ? (below << lz) : below) != 0u;
#pragma unroll
    for (int k = 0; k < L - 3; ++k)
      if (k < t - 2 && X[k]) sticky = true;
    if (t < 2) sticky = false;
    top |= sticky ? 1ull : 0ull;
    ex = 32 * (t - 1) - lz;
  }
  // top * 2^e2 as a double, rounded to nearest even in integer arithmetic
  // (GB300's FP64 pipe is narrow); results outside the normal range take
  // the floating-point path.
  const int e2 = ex + er + ec - 2 * cc.bits;
  uint64_t bitsd = 0;
  if (top) {
    const int lzt = __clzll((long long)top);
    const uint64_t x = top << lzt;  // leading one at bit 63
    uint64_t mant = x >> 11;        // the 53 bits FP64 keeps
    const uint64_t rem = x & 0x7FFu;
    if (rem > 0x400u || (rem == 0x400u && (mant & 1u))) ++mant;
    int e = e2 - lzt + 63;  // exponent of the leading bit
    if (mant >> 53) {
      mant >>= 1;
      ++e;
    }
    if (e >= -1022 && e <= 1023) {
      bitsd = ((uint64_t)(e + 1023) << 52) | (mant & ((1ull << 52) - 1));
    } else {
      const double d = times_pow2(__ull2double_rn(top), e2);
      bitsd = (uint64_t)__double_as_longlong(d);
    }
  }
  if (neg) bitsd ^= 1ull << 63;
  const double d = __longlong_as_double((long long)bitsd);
  return unit_alpha ? d : alpha * d;
}

// Rows [1024 bx, 1024 bx + 1024) of columns j0, j0 + jstep, ... of C; each
// thread takes four consecutive rows (one 8-byte load per residue plane).
constexpr int kCrtRows = 4;

// NM >= n bounds the unrolled modulus loops (the CRT set's size rounded up to
// a multiple of 4 for single calls, kMaxModuli for grouped ones).
template <int L, int NM>
__device__ __forceinline__ void reassemble_body(const CrtConst &cc, const uint16_t *res, int64_t Mp, int64_t plane,
                                                int64_t M, int64_t N, const int *e_row, const int *e_col,
                                                double alpha, double *C, int64_t ldc, int64_t bx, int64_t j0,
                                                int64_t jstep) {
  const int64_t i0 = (bx * blockDim.x + threadIdx.x) * kCrtRows;
  if (i0 >= M) return;
  const bool unit_alpha = alpha == 1.0;
  const int4 er4 = *reinterpret_cast<const int4 *>(e_row + i0);
  const int er[kCrtRows] = {er4.x, er4.y, er4.z, er4.w};
  for (int64_t j = j0; j < N; j += jstep) {
    const int ec = e_col[j];
    uint2 rw[NM];
    const uint16_t *rp = res + j * Mp + i0;
#pragma unroll
    for (int l = 0; l < NM; ++l)
      rw[l] = l < cc.n ? *reinterpret_cast<const uint2 *>(rp + l * plane) : make_uint2(0u, 0u);
    // One row at a time: interleaving the four rows' limb sums doubles the
    // registers and halves the resident blocks.
#pragma unroll 1
    for (int q = 0; q < kCrtRows; ++q) {
      if (i0 + q >= M) break;
      const int erq = q == 0 ? er[0] : q == 1 ? er[1] : q == 2 ? er[2] : er[3];
      double v;
      if (erq == kExpNone || ec == kExpNone) v = alpha * 0.0;
      else v = crt_element<L, NM>(cc, rw, q, erq, ec, alpha, unit_alpha);
      C[i0 + q + j * ldc] = v;
    }
  }
}

template <int L, int NM>
__global__ void __launch_bounds__(256) reassemble_kernel(const __grid_constant__ CrtConst cc, const uint16_t *res,
                                                         int64_t Mp, int64_t plane, int64_t M, int64_t N,
                                                         const int *e_row, const int *e_col, double alpha,
                                                         double *C, int64_t ldc) {
  reassemble_body<L, NM>(cc, res, Mp, plane, M, N, e_row, e_col, alpha, C, ldc, blockIdx.x, blockIdx.y, gridDim.y);
}

// ---------------------------------------------------------------- grouped (wave) kernels
// One launch per stage for all problems of a wave: block b belongs to the
// job whose [block_begin, block_begin + blocks) holds it.
struct ScaleJob {
  OzOperand op;
  int *e;
  int64_t block_begin;
};
struct ResidueJob {
  OzOperand op;
  const int *e;
  int bits, nmod;
  int64_t Pp, Kp, gx;
  uint16_t *R;
  int64_t block_begin;
};
struct CrtJob {
  CrtConst cc;
  const uint16_t *res;
  int64_t Mp, plane, M, N, gx;
  const int *e_row, *e_col;
  double alpha;
  double *C;
  int64_t ldc;
  int64_t block_begin;
};

template <class J>
__device__ __forceinline__ int find_job(const J *jobs, int n, int64_t b) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (jobs[mid].block_begin <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ int64_t flat_block() { return (int64_t)blockIdx.y * gridDim.x + blockIdx.x; }

__global__ void __launch_bounds__(256) scale_wave_kernel(const ScaleJob *jobs, int n, int64_t total) {
  const int64_t b = flat_block();
  if (b >= total) return;
  const ScaleJob &J = jobs[find_job(jobs, n, b)];
  scale_body(J.op, J.e, b - J.block_begin, 0, J.op.K, true);
}

__global__ void __launch_bounds__(256, 6) residue_wave_kernel(const ResidueJob *jobs, int n, int64_t total) {
  const int64_t b = flat_block();
  if (b >= total) return;
  const ResidueJob &J = jobs[find_job(jobs, n, b)];
  const int64_t lb = b - J.block_begin;
  residue_body(J.op, J.e, J.bits, 0, J.nmod, J.Pp, J.Kp, J.R, lb % J.gx, lb / J.gx);
}

__global__ void __launch_bounds__(256) reassemble_wave_kernel(const CrtJob *jobs, int n, int64_t total) {
  const int64_t b = flat_block();
  if (b >= total) return;
  const CrtJob &J = jobs[find_job(jobs, n, b)];
  const int64_t lb = b - J.block_begin;
  const CrtConst &cc = J.cc;
  switch (cc.limbs) {
#define UVT_CRT_CASE(L)                                                                                           \
  case L:                                                                                                         \
    reassemble_body<L, kMaxModuli>(cc, J.res, J.Mp, J.plane, J.M, J.N, J.e_row, J.e_col, J.alpha, J.C, J.ldc, \
                                   lb % J.gx, lb / J.gx, J.N);                                                   \
    break;
    UVT_CRT_CASE(2) UVT_CRT_CASE(3) UVT_CRT_CASE(4) UVT_CRT_CASE(5) UVT_CRT_CASE(6)
#undef UVT_CRT_CASE
    default: break;
  }
}

dim3 flat_grid(int64_t total) {
  const int64_t gx = std::min<int64_t>(total, 1 << 20);
  return dim3((unsigned)std::max<int64_t>(gx, 1), (unsigned)((total + gx - 1) / std::max<int64_t>(gx, 1)));
}

// ---------------------------------------------------------------- host bigint helpers
struct Big {
  uint64_t w[3] = {0, 0, 0};
};
Big big_mul_small(const Big &a, uint64_t s) {
  Big r;
  unsigned __int128 c = 0;
  for (int i = 0; i < 3; ++i) {
    c += (unsigned __int128)a.w[i] * s;
    r.w[i] = (uint64_t)c;
    c >>= 64;
  }
  return r;
}
Big big_div_small(const Big &a, uint64_t s, uint64_t *rem) {
  Big q;
  unsigned __int128 r = 0;
  for (int i = 2; i >= 0; --i) {
    r = (r << 64) | a.w[i];
    q.w[i] = (uint64_t)(r / s);
    r %= s;
  }
  *rem = (uint64_t)r;
  return q;
}
double big_to_double(const Big &a) {
  return (double)a.w[2] * 0x1p128 + (double)a.w[1] * 0x1p64 + (double)a.w[0];
}
double big_log2(const Big &a) {
  double v = (double)a.w[2] * 0x1p128 + (double)a.w[1] * 0x1p64 + (double)a.w[0];
  return std::log2(v);
}
Big modulus_product(int n) {
  Big M;
  M.w[0] = 1;
  for (int l = 0; l < n; ++l) M = big_mul_small(M, (uint64_t)kModuli[l]);
  return M;
}

}  // namespace

int ozaki_bits(int n_moduli, int64_t K) {
  const double lm = big_log2(modulus_product(n_moduli));
  const double lk = std::log2((double)std::max<int64_t>(K, 1));
  int t = (int)std::floor((lm - lk - 2.0) / 2.0);
  return std::max(1, std::min(t, kMaxBits));
}

int ozaki_auto_moduli(int64_t K) {
  // 52 bits per scaled entry keep the result several times below a 1e-14
  // relative Frobenius error even for entries spread over 2^+-20 (measured:
  // 2.2e-16 at K = 32768 with 54 bits, 3.5e-15 with 50 bits).
  for (int n = 2; n <= kMaxModuli; ++n)
    if (ozaki_bits(n, K) >= 52) return n;
  return kMaxModuli;
}

int oz_scales(const OzOperand &op, int *e, cudaStream_t st) {
  if (op.P <= 0) return UVATRMM_OK;
  if (cudaMemsetAsync(e, 0x80, (size_t)op.P * sizeof(int), st) != cudaSuccess) return UVATRMM_EDEVICE;
  if (op.K <= 0) return UVATRMM_OK;
  const int64_t kpb = 4096;
  dim3 grid((unsigned)((op.P + TP - 1) / TP), (unsigned)((op.K + kpb - 1) / kpb));
  scale_kernel<<<grid, 256, 0, st>>>(op, e, kpb);
  return cudaGetLastError() == cudaSuccess ? UVATRMM_OK : UVATRMM_EDEVICE;
}

int oz_residues(const OzOperand &op, const int *e, int bits, int l0, int l1, int64_t Pp, int64_t Kp, uint16_t *R,
                cudaStream_t st) {
  if (Pp % TP || Kp % TK) return UVATRMM_EINVAL;
  dim3 grid((unsigned)(Kp / TK), (unsigned)(Pp / TP));
  if (grid.y > 65535u) return UVATRMM_EINVAL;
  residue_kernel<<<grid, 256, 0, st>>>(op, e, bits, l0, l1, Pp, Kp, R);
  return cudaGetLastError() == cudaSuccess ? UVATRMM_OK : UVATRMM_EDEVICE;
}

namespace {
// CRT constants for the first n moduli: P_l = M/m_l, M, the limb count L
// (smallest >= 2 with M < 2^(32L)) and the scales of the k estimate.
CrtConst make_crt(const OzPlan &plan) {
  CrtConst cc;
  memset(&cc, 0, sizeof(cc));
  cc.n = plan.n_moduli;
  cc.bits = plan.bits;
  const Big M = modulus_product(plan.n_moduli);
  auto limb = [](const Big &v, int k) { return (uint32_t)(v.w[k / 2] >> (32 * (k % 2))); };
  int top = 0;
  for (int k = 0; k < kLimbs; ++k) {
    cc.Mw[k] = limb(M, k);
    if (cc.Mw[k]) top = k;
  }
  cc.limbs = std::max(2, top + 1);
  for (int l = 0; l < plan.n_moduli; ++l) {
    uint64_t rem;
    const Big Pl = big_div_small(M, (uint64_t)kModuli[l], &rem);
    for (int k = 0; k < kLimbs; ++k) cc.P[l][k] = limb(Pl, k);
  }
  const double mf = big_to_double(M);
  cc.c_hi = (float)(std::ldexp(1.0, 32 * (cc.limbs - 1)) / mf);
  cc.c_lo = (float)(std::ldexp(1.0, 32 * (cc.limbs - 2)) / mf);
  return cc;
}
}  // namespace

size_t oz_wave_table_bytes(int nitems) {
  auto r = [](size_t b) { return (b + 255) / 256 * 256; };
  return r(2 * (size_t)nitems * sizeof(ScaleJob)) + r(2 * (size_t)nitems * sizeof(ResidueJob)) +
         r((size_t)nitems * sizeof(CrtJob));
}

int oz_wave_tables(const OzWaveItem *items, int n, void *dev, OzWaveTables *out) {
  std::vector<char> image;
  oz_wave_image(items, n, dev, image, out);
  return cudaMemcpy(dev, image.data(), image.size(), cudaMemcpyHostToDevice) == cudaSuccess ? UVATRMM_OK
                                                                                          : UVATRMM_EDEVICE;
}

void oz_wave_image(const OzWaveItem *items, int n, void *dev, std::vector<char> &image, OzWaveTables *out) {
  std::vector<ScaleJob> sj(2 * n);
  std::vector<ResidueJob> rj(2 * n);
  std::vector<CrtJob> cj(n);
  int64_t bs = 0, br = 0, bc = 0;
  for (int i = 0; i < n; ++i) {
    const OzWaveItem &it = items[i];
    const OzPlan &pl = it.plan;
    for (int s = 0; s < 2; ++s) {
      const OzOperand &op = s ? it.R : it.L;
      sj[2 * i + s] = ScaleJob{op, s ? it.e_col : it.e_row, bs};
      bs += (op.P + TP - 1) / TP;
      const int64_t Pp = s ? pl.Np : pl.Mp;
      const int64_t gx = pl.Kp / TK;
      rj[2 * i + s] = ResidueJob{op, s ? it.e_col : it.e_row, pl.bits, pl.n_moduli, Pp, pl.Kp, gx,
                                 s ? it.RR : it.LR, br};
      br += gx * (Pp / TP);
    }
    CrtJob &c = cj[i];
    c.cc = make_crt(pl);
    c.res = it.res;
    c.Mp = pl.Mp;
    c.plane = pl.Mp * pl.Np;
    c.M = pl.M;
    c.N = pl.N;
    c.gx = (pl.M + 256 * kCrtRows - 1) / (256 * kCrtRows);
    c.e_row = it.e_row;
    c.e_col = it.e_col;
    c.alpha = it.alpha;
    c.C = it.C;
    c.ldc = it.ldc;
    c.block_begin = bc;
    bc += c.gx * pl.N;
  }
  auto r = [](size_t b) { return (b + 255) / 256 * 256; };
  char *base = static_cast<char *>(dev);
  out->scale = base;
  out->resid = base + r(sj.size() * sizeof(ScaleJob));
  out->crt = static_cast<char *>(out->resid) + r(rj.size() * sizeof(ResidueJob));
  out->n_scale = out->n_resid = 2 * n;
  out->n_crt = n;
  out->b_scale = bs;
  out->b_resid = br;
  out->b_crt = bc;
  image.assign(oz_wave_table_bytes(n), 0);
  memcpy(image.data(), sj.data(), sj.size() * sizeof(ScaleJob));
  memcpy(image.data() + (static_cast<char *>(out->resid) - base), rj.data(), rj.size() * sizeof(ResidueJob));
  memcpy(image.data() + (static_cast<char *>(out->crt) - base), cj.data(), cj.size() * sizeof(CrtJob));
}

int oz_wave_prep(const OzWaveTables &t, cudaStream_t st) {
  if (t.b_scale > 0)
    scale_wave_kernel<<<flat_grid(t.b_scale), 256, 0, st>>>(static_cast<const ScaleJob *>(t.scale), t.n_scale,
                                                            t.b_scale);
  if (t.b_resid > 0)
    residue_wave_kernel<<<flat_grid(t.b_resid), 256, 0, st>>>(static_cast<const ResidueJob *>(t.resid), t.n_resid,
                                                              t.b_resid);
  return cudaGetLastError() == cudaSuccess ? UVATRMM_OK : UVATRMM_EDEVICE;
}

int oz_wave_reassemble(const OzWaveTables &t, cudaStream_t st) {
  if (t.b_crt > 0)
    reassemble_wave_kernel<<<flat_grid(t.b_crt), 256, 0, st>>>(static_cast<const CrtJob *>(t.crt), t.n_crt,
                                                               t.b_crt);
  return cudaGetLastError() == cudaSuccess ? UVATRMM_OK : UVATRMM_EDEVICE;
}

int oz_reassemble(const OzPlan &plan, const uint16_t *res, const int *e_row, const int *e_col, double alpha,
                  double *C, int64_t ldc, cudaStream_t st) {
  const CrtConst cc = make_crt(plan);
  if (plan.M <= 0 || plan.N <= 0) return UVATRMM_OK;
  dim3 grid((unsigned)((plan.M + 256 * kCrtRows - 1) / (256 * kCrtRows)), (unsigned)std::min<int64_t>(plan.N, 65535));
  const int nm = (cc.n + 3) / 4 * 4;
  switch (nm * 8 + cc.limbs) {
#define UVT_CRT_LAUNCH(NM, L)                                                                                     \
  case NM * 8 + L:                                                                                                \
    reassemble_kernel<L, NM><<<grid, 256, 0, st>>>(cc, res, plan.Mp, plan.Mp * plan.Np, plan.M, plan.N, e_row,    \
                                                   e_col, alpha, C, ldc);                                         \
    break;
    UVT_CRT_LAUNCH(4, 2) UVT_CRT_LAUNCH(8, 2) UVT_CRT_LAUNCH(8, 3) UVT_CRT_LAUNCH(12, 3) UVT_CRT_LAUNCH(12, 4)
    UVT_CRT_LAUNCH(16, 4) UVT_CRT_LAUNCH(16, 5) UVT_CRT_LAUNCH(20, 5) UVT_CRT_LAUNCH(20, 6)
#undef UVT_CRT_LAUNCH
    default: return UVATRMM_EINVAL;
  }
  return cudaGetLastError() == cudaSuccess ? UVATRMM_OK : UVATRMM_EDEVICE;
}

}  // namespace uvt
