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
  int myp;
  if (op.kcontig) {
    // warp w handles rows p0 + w, p0 + w + 8, ...; lanes stride over k
    const int w = tid >> 5, ln = tid & 31;
    for (int pp = w; pp < TP; pp += 8) {
      int b2 = kExpNone;
      for (int64_t k = kb + ln; k < ke; k += 32) {
        const double v = load_elem(op, p0 + pp, k);
        if (v != 0.0) b2 = max(b2, exp_above(v));
      }
#pragma unroll
      for (int o = 16; o; o >>= 1) b2 = max(b2, __shfl_xor_sync(0xffffffffu, b2, o));
      if (ln == 0) atomicMax(&red[pp], b2);
    }
    myp = -1;
  } else {
    const int pp = tid & 31, ky = tid >> 5;
    for (int64_t k = kb + ky; k < ke; k += 8) {
      const double v = load_elem(op, p0 + pp, k);
      if (v != 0.0) best = max(best, exp_above(v));
    }
    atomicMax(&red[pp], best);
    myp = pp;
  }
  (void)myp;
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

// The 32 (p) x 64 (k) residue tile (bx = k tile, by = p tile).
__device__ __forceinline__ void residue_body(const OzOperand &op, const int *e, int bits, int l0, int l1, int64_t Pp,
                                             int64_t Kp, uint16_t *R, int64_t bx, int64_t by) {
  __shared__ double tile[TP][TK + 1];
  const int tid = threadIdx.x;
  const int64_t p0 = by * TP, k0 = bx * TK;
  // Load (coalesced along the contiguous dimension of X).
  for (int idx = tid; idx < TP * TK; idx += 256) {
    int pp, kk;
    if (op.kcontig) { kk = idx % TK; pp = idx / TK; }
    else { pp = idx % TP; kk = idx / TP; }
    tile[pp][kk] = load_elem(op, p0 + pp, k0 + kk);
  }
  __syncthreads();
  const int64_t plane = Pp * Kp;
  for (int idx = tid; idx < TP * TK; idx += 256) {
    const int kk = idx % TK, pp = idx / TK;
    const double v = tile[pp][kk];
    uint32_t w[4] = {0, 0, 0, 0};
    bool neg = false;
    const int ep = e[p0 + pp];
    if (v != 0.0 && ep != kExpNone) {
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

__global__ void __launch_bounds__(256) residue_kernel(OzOperand op, const int *e, int bits, int l0, int l1,
                                                      int64_t Pp, int64_t Kp, uint16_t *R) {
  residue_body(op, e, bits, l0, l1, Pp, Kp, R, blockIdx.x, blockIdx.y);
}

// ---------------------------------------------------------------- reassembly
struct CrtConst {
  int n;
  int bits;
  uint64_t W[kMaxModuli][3];  // W_l = (M/m_l) * ((M/m_l)^-1 mod m_l)
  uint64_t Mw[3], halfM[3];
  float Mf;                   // M / 2^128
};

__device__ __forceinline__ bool ge3(const uint64_t a[3], const uint64_t b[3]) {
  if (a[2] != b[2]) return a[2] > b[2];
  if (a[1] != b[1]) return a[1] > b[1];
  return a[0] >= b[0];
}
__device__ __forceinline__ void sub3(uint64_t a[3], const uint64_t b[3]) {
  unsigned __int128 t = (unsigned __int128)a[0] - b[0];
  a[0] = (uint64_t)t;
  uint64_t br = (uint64_t)(t >> 64) ? 1 : 0;
  t = (unsigned __int128)a[1] - b[1] - br;
  a[1] = (uint64_t)t;
  br = (uint64_t)(t >> 64) ? 1 : 0;
  a[2] = a[2] - b[2] - br;
}
__device__ __forceinline__ void add3(uint64_t a[3], const uint64_t b[3]) {
  unsigned __int128 t = (unsigned __int128)a[0] + b[0];
  a[0] = (uint64_t)t;
  t = (unsigned __int128)a[1] + b[1] + (uint64_t)(t >> 64);
  a[1] = (uint64_t)t;
  a[2] = a[2] + b[2] + (uint64_t)(t >> 64);
}

// Rows [256 bx, 256 bx + 256) of columns j0, j0 + jstep, ... of C.
__device__ __forceinline__ void reassemble_body(const CrtConst &cc, const uint8_t *res, int64_t Mp, int64_t plane,
                                                int64_t M, int64_t N, const int *e_row, const int *e_col,
                                                double alpha, double *C, int64_t ldc, int64_t bx, int64_t j0,
                                                int64_t jstep) {
  const int64_t i = bx * blockDim.x + threadIdx.x;
  if (i >= M) return;
  const int er = e_row[i];
  for (int64_t j = j0; j < N; j += jstep) {
  const int ec = e_col[j];
  if (er == kExpNone || ec == kExpNone) {
    C[i + j * ldc] = alpha * 0.0;
    continue;
  }
  // S = sum_l r_l W_l  (< 2^146: three 64-bit words)
  uint64_t S[3] = {0, 0, 0};
  const uint8_t *rp = res + j * Mp + i;
  for (int l = 0; l < cc.n; ++l) {
    const uint64_t r = rp[(int64_t)l * plane];
    unsigned __int128 t = (unsigned __int128)r * cc.W[l][0] + S[0];
    S[0] = (uint64_t)t;
    t = (unsigned __int128)r * cc.W[l][1] + S[1] + (uint64_t)(t >> 64);
    S[1] = (uint64_t)t;
    S[2] = S[2] + r * cc.W[l][2] + (uint64_t)(t >> 64);
  }
  // R = S mod M via an fp32 quotient estimate and one correction each way.
  const float sf = (float)S[2] + (float)S[1] * 5.42101086e-20f;  // S / 2^128
  uint32_t q = (uint32_t)floorf(sf / cc.Mf);
  uint64_t qM[3];
  {
    unsigned __int128 t = (unsigned __int128)q * cc.Mw[0];
    qM[0] = (uint64_t)t;
    t = (unsigned __int128)q * cc.Mw[1] + (uint64_t)(t >> 64);
    qM[1] = (uint64_t)t;
    qM[2] = q * cc.Mw[2] + (uint64_t)(t >> 64);
  }
  if (!ge3(S, qM)) add3(S, cc.Mw);  // estimate one too high
  sub3(S, qM);
  if (ge3(S, cc.Mw)) sub3(S, cc.Mw);  // estimate one too low
  // Signed value in (-M/2, M/2].
  bool neg = false;
  if (ge3(S, cc.halfM) && !(S[0] == cc.halfM[0] && S[1] == cc.halfM[1] && S[2] == cc.halfM[2])) {
    uint64_t t[3] = {cc.Mw[0], cc.Mw[1], cc.Mw[2]};
    sub3(t, S);
    S[0] = t[0]; S[1] = t[1]; S[2] = t[2];
    neg = true;
  }
  // Round the magnitude to FP64 once: top 64 bits with a sticky bit.
  uint64_t top;
  int shift;
  if (S[2]) {
    const int lz = __clzll((long long)S[2]);
    top = lz ? (S[2] << lz) | (S[1] >> (64 - lz)) : S[2];
    const bool sticky = (lz ? (S[1] << lz) : S[1]) != 0 || S[0] != 0;
    top |= sticky ? 1ull : 0ull;
    shift = 128 - lz;
  } else if (S[1]) {
    const int lz = __clzll((long long)S[1]);
    top = lz ? (S[1] << lz) | (S[0] >> (64 - lz)) : S[1];
    const bool sticky = (lz ? (S[0] << lz) : 0ull) != 0;
    top |= sticky ? 1ull : 0ull;
    shift = 64 - lz;
  } else {
    top = S[0];
    shift = 0;
  }
  double d = __ull2double_rn(top);
  d = ldexp(d, shift + er + ec - 2 * cc.bits);
  C[i + j * ldc] = alpha * (neg ? -d : d);
  }
}

__global__ void __launch_bounds__(256) reassemble_kernel(const __grid_constant__ CrtConst cc, const uint8_t *res,
                                                         int64_t Mp, int64_t plane, int64_t M, int64_t N,
                                                         const int *e_row, const int *e_col, double alpha,
                                                         double *C, int64_t ldc) {
  reassemble_body(cc, res, Mp, plane, M, N, e_row, e_col, alpha, C, ldc, blockIdx.x, blockIdx.y, gridDim.y);
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
  const uint8_t *res;
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

__global__ void __launch_bounds__(256) residue_wave_kernel(const ResidueJob *jobs, int n, int64_t total) {
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
  reassemble_body(J.cc, J.res, J.Mp, J.plane, J.M, J.N, J.e_row, J.e_col, J.alpha, J.C, J.ldc, lb % J.gx, lb / J.gx,
                  J.N);
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
double big_log2(const Big &a) {
  double v = (double)a.w[2] * 0x1p128 + (double)a.w[1] * 0x1p64 + (double)a.w[0];
  return std::log2(v);
}
int64_t inv_mod(int64_t a, int64_t m) {
  int64_t g = m, x = 0, x1 = 1, a1 = a % m;
  while (a1) {
    int64_t q = g / a1, t = g - q * a1;
    g = a1;
    a1 = t;
    t = x - q * x1;
    x = x1;
    x1 = t;
  }
  return ((x % m) + m) % m;
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
// CRT constants for the first n moduli: W_l = (M/m_l) * ((M/m_l)^-1 mod m_l).
CrtConst make_crt(const OzPlan &plan) {
  CrtConst cc;
  memset(&cc, 0, sizeof(cc));
  cc.n = plan.n_moduli;
  cc.bits = plan.bits;
  const Big M = modulus_product(plan.n_moduli);
  for (int l = 0; l < plan.n_moduli; ++l) {
    uint64_t rem;
    const Big Ml = big_div_small(M, (uint64_t)kModuli[l], &rem);
    uint64_t mlm;
    big_div_small(Ml, (uint64_t)kModuli[l], &mlm);
    const int64_t inv = inv_mod((int64_t)mlm, kModuli[l]);
    const Big W = big_mul_small(Ml, (uint64_t)inv);
    for (int k = 0; k < 3; ++k) cc.W[l][k] = W.w[k];
  }
  uint64_t r2;
  const Big half = big_div_small(M, 2, &r2);
  for (int k = 0; k < 3; ++k) {
    cc.Mw[k] = M.w[k];
    cc.halfM[k] = half.w[k];
  }
  cc.Mf = (float)((double)M.w[2] + (double)M.w[1] * 0x1p-64 + (double)M.w[0] * 0x1p-128);
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
    c.gx = (pl.M + 255) / 256;
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

int oz_reassemble(const OzPlan &plan, const uint8_t *res, const int *e_row, const int *e_col, double alpha,
                  double *C, int64_t ldc, cudaStream_t st) {
  const CrtConst cc = make_crt(plan);
  if (plan.M <= 0 || plan.N <= 0) return UVATRMM_OK;
  dim3 grid((unsigned)((plan.M + 255) / 256), (unsigned)std::min<int64_t>(plan.N, 65535));
  reassemble_kernel<<<grid, 256, 0, st>>>(cc, res, plan.Mp, plan.Mp * plan.Np, plan.M, plan.N, e_row, e_col,
                                           alpha, C, ldc);
  return cudaGetLastError() == cudaSuccess ? UVATRMM_OK : UVATRMM_EDEVICE;
}

}  // namespace uvt
