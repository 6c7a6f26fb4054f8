// Exact residue GEMM on the 5th-generation tensor cores (tcgen05, sm_103a).
//
// For every modulus m_l and output block of 256 x 256 the K loop runs over
// 128-deep bf16 slabs, each two 64-wide atoms staged by TMA (128-byte
// swizzle, K-major), in a 3-stage shared-memory ring; one thread issues
// tcgen05.mma.kind::f16 (bf16 x bf16 -> fp32 in TMEM, K=16 per instruction,
// eight per slab).  Every 4 slabs (a K chunk of 512) the accumulator is handed
// to the epilogue warps, which reduce
// it modulo m_l in place (tcgen05.ld -> fp32 fold -> tcgen05.st) while the
// MMA thread fills the other TMEM accumulator with the next chunk; the next
// chunk for that accumulator then adds on top of the folded value.  Residues
// are at most 181 in magnitude (moduli up to 363) and a folded value at most
// a few units past m/2, so every value the accumulator ever holds is an
// integer below 512 * 181^2 + 184 < 2^24 and fp32 accumulation is exact.
// The last two chunks are combined and the tile's residues r are written as
// the 16-bit words u_l r mod m_l (u_l = (M/m_l)^-1 mod m_l, for the CRT).
//
// CTA pairs and the 2-SM MMA.  The kernel runs in clusters of two CTAs on
// two SMs.  The pair computes a 256 x 256 block with tcgen05.mma.cta_group::2
// (M = 256, N = 256): each CTA stages its own 128 rows of A and its own half
// (128 rows) of the B tile in its own shared memory, and the MMA, issued by
// one thread of the even CTA (the leader), reads A and B from both CTAs and
// accumulates each CTA's 128 rows in that CTA's TMEM.  Per 16-wide K step an
// SM thus stages and reads 8 KB of operands for 128 x 256 outputs, where a
// single-CTA M = 128 MMA over the whole B tile needs 12 KB, and no copy needs
// to be multicast to share B.  Both CTAs' copies complete on the
// leader's "full" barrier (the .cta_group::2 form of the TMA load); the
// leader's commits free the stage in both CTAs ("empty") and hand each
// finished chunk to both CTAs' epilogues ("cdone"), whose warps release the
// accumulator on the leader's "afree" barrier.  No load is multicast: every
// copy lands in the shared memory of the CTA that issued it.  The pair's K
// range is the union of its two row tiles' ranges (the extra slabs of the
// shorter range only meet zeros of the triangle).
//
// The accumulators alternate across tiles (chunk g of a pair uses buffer
// g & 1).  The second-to-last chunk of a tile is reduced to residues (low
// bytes in shared memory, the ninth bits in a per-thread word per 32
// columns) and its buffer released at once, so the next tile's first chunk
// runs while the last chunk is combined and stored.
//
// Warp roles (320 threads, one CTA per SM): warp 0 TMA producer, warp 1 TMEM
// owner (both CTAs allocate the pair's columns together) and, in the leader,
// MMA issuer; warps 2-9 epilogue (each bound to its TMEM lane quadrant,
// warp % 4, and to half of the columns).  Tiles go to clusters round-robin
// in a raster of pair-row groups (see decode()).  All mbarrier waits are
// bounded; on expiry the kernel records KERR_WAIT_TIMEOUT, drains its copies
// and MMAs, frees TMEM and exits (after the pair's closing cluster barrier).
#include <algorithm>
#include <cstring>

#include "common.cuh"
#include "ozaki.cuh"
#include "tmap.cuh"

namespace uvt {
namespace {

constexpr int BM = 128, BN = 256, BK = 64;
constexpr int PAIR = 2;          // CTAs per cluster, stacked along M; one 2-SM MMA per K step
static_assert(PAIR * BM == kOzBlock && BN == kOzBlock, "the slicing skips tiles by this K-range geometry");
constexpr int BH = BN / PAIR;    // rows of the B tile each CTA stages (its half of N)
// Two 64-wide swizzle atoms per stage: per 128-deep slab the producer, the
// MMA thread and the barriers hand off once for eight MMAs (measured 5-10 %
// faster than 64-deep slabs in a 4-stage ring, bit-identical results).
constexpr int ATOMS = 2;
constexpr int SLAB = ATOMS * BK;         // K per stage
constexpr int STAGES = 3;
constexpr int CHUNK_SLABS = 512 / SLAB;  // K chunk of 512 between modular folds
constexpr uint32_t ATOM_A = BM * BK * 2, ATOM_B = BH * BK * 2;
constexpr uint32_t A_BYTES = ATOMS * ATOM_A, BH_BYTES = ATOMS * ATOM_B;
constexpr uint32_t STAGE_BYTES = A_BYTES + BH_BYTES;  // one CTA's share of a stage
constexpr uint32_t PAIR_TX = PAIR * STAGE_BYTES;      // bytes landing on the leader's full barrier
// Warp 0: TMA producer; warp 1: MMA issuer; warps 2..9: epilogue, two warps
// per TMEM lane quarter (warp & 3), each taking half of the 256 columns, so a
// tile's last-chunk epilogue stays within one chunk of MMAs.
constexpr int EPI_WARPS = 8;
constexpr int CB_PER_WARP = BN / 32 / (EPI_WARPS / 4);  // 32-column blocks per epilogue warp
constexpr int NUM_THREADS = 32 * (2 + EPI_WARPS);
constexpr uint32_t TMEM_COLS = 2 * BN;  // two fp32 accumulators of 256 columns
// Low bytes of a tile's second-to-last chunk residues, [column word][row] (32 KB).
constexpr uint32_t R1_BYTES = BM * BN;
constexpr size_t SMEM = 1024 + (size_t)STAGES * STAGE_BYTES + 256 + R1_BYTES;
// kind::f16 instruction descriptor: D fp32 (bits 4-5 = 1), A and B bf16
// (bits 7-9 = 1, 10-12 = 1), both K-major, N/8 at bits 17-22, M/16 at 24-28
// with M = 256, the pair's rows.
constexpr uint32_t IDESC =
    (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)((PAIR * BM) >> 4) << 24);

// Launch-wide parameters; the problems themselves are OzGroupProb entries in
// global memory (their tensor maps are read by TMA from there).
struct GParams {
  int nprob, total_tiles;  // tiles = CTA-pair tiles (256 x 256 per modulus)
  int *status;
  float mod_f[kMaxModuli];
  float inv_f[kMaxModuli];
  float u_f[kMaxModuli + 1][kMaxModuli];  // u_f[n][l] = crt_u(n, l)
};

struct Tile {
  int l, tp, tj, ks0, ks1;  // modulus, pair row tile, column tile, K slab range
};

__device__ __forceinline__ void tmap_acquire(const CUtensorMap *m) {
  asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(reinterpret_cast<uint64_t>(m))
               : "memory");
}

// Problem owning global tile t (problems sorted by tile_begin).
__device__ __forceinline__ int find_problem(const OzGroupProb *probs, int nprob, int t) {
  int lo = 0, hi = nprob - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (probs[mid].tile_begin <= t) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Local pair tile t of problem p: modulus, tile coordinates and K slab range.
__device__ __forceinline__ Tile decode(const OzGroupProb &p, int t, int nclusters) {
  Tile T;
  T.l = p.l0 + t / p.tiles_per_mod;
  int r = t % p.tiles_per_mod;
  const int tpm = p.tiles_m / PAIR;
  const int n_maj = p.tri_left ? tpm : p.tiles_n, n_min = p.tri_left ? p.tiles_n : tpm;
  // Raster: groups of `group` major tiles in longest-first order; inside a
  // group the minor index is outer, so the clusters of one wave (tiles
  // c + k * nclusters) form a group x (nclusters / group) block sharing both
  // panels.  The major tile of a minor index is rotated by the wave, so a
  // cluster cycles through the group's (triangle-shortened) major tiles
  // instead of keeping the shortest or longest one and drifting out of step
  // with the clusters it shares panels with.
  const int gspan = p.group * n_min;
  const int g = r / gspan, within = r % gspan;
  const int gsize = min(p.group, n_maj - g * p.group);
  const int mi = within / gsize;
  const int per_wave = max(1, nclusters / gsize);  // minor tiles per wave
  const int rank = g * p.group + (within % gsize + mi / per_wave) % gsize;
  const int ma = p.grows ? (n_maj - 1 - rank) : rank;
  T.tp = p.tri_left ? ma : mi;
  T.tj = p.tri_left ? mi : ma;
  int64_t kb, ke;
  if (p.tri_left) {
    const int64_t i0 = (int64_t)T.tp * (PAIR * BM);
    if (p.tri_lower) { kb = 0; ke = min(i0 + PAIR * BM, p.K); }
    else { kb = i0; ke = p.K; }
  } else {
    const int64_t j0 = (int64_t)T.tj * BN;
    if (p.tri_lower) { kb = j0; ke = p.K; }
    else { kb = 0; ke = min(j0 + BN, p.K); }
  }
  T.ks0 = (int)(kb / SLAB);
  T.ks1 = (int)((ke + SLAB - 1) / SLAB);
  return T;
}

// ---------------------------------------------------------------- cluster helpers
__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t cluster_index() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint32_t cluster_count() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%nclusterid.x;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Address of the same shared-memory location in CTA `rank` of the cluster.
__device__ __forceinline__ uint32_t mapa(uint32_t saddr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(saddr), "r"(rank));
  return r;
}

// 2-D TMA load into this CTA's shared memory whose completion is counted on
// the mbarrier at cluster address `bar` (this CTA's or its pair peer's: the
// .cta_group::2 form).
__device__ __forceinline__ void tma_load_2d_pair(void *smem_dst, const CUtensorMap *m, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(smem_dst)),
      "l"(reinterpret_cast<uint64_t>(m)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// Arrive on the mbarrier at cluster address `bar` (this CTA's or the pair
// peer's).  The default semantics (release at CTA scope) suffice: what the
// arrive hands over is TMEM, ordered by tcgen05.wait + tcgen05.fence around
// it, not ordinary memory, so it need not wait for the warp's earlier global
// stores to become visible across the cluster.
__device__ __forceinline__ void mbar_arrive_remote(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cluster.b64 _, [%0];" ::"r"(bar) : "memory");
}

// ---------------------------------------------------------------- packed fp32 fold
__device__ __forceinline__ uint64_t pack2(float f) {
  uint64_t r;
  asm("mov.b64 %0, {%1, %1};" : "=l"(r) : "f"(f));
  return r;
}
// (a, b) := (a, b) - m * q with q = x * fl(1/m) rounded to an integer: the
// fma with 1.5 * 2^23 rounds the exact product once (|x / m| < 2^22 for the
// |x| < 2^24 held here) and x - q * m is exact; fl(1/m) is off by at most
// 2^-24 relative, so |result| <= m/2 + 2.
__device__ __forceinline__ void fold2(uint32_t &a, uint32_t &b, uint64_t inv2, uint64_t negm2) {
  uint64_t x, q;
  asm("mov.b64 %0, {%1, %2};" : "=l"(x) : "r"(a), "r"(b));
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(q) : "l"(x), "l"(inv2), "l"(0x4B4000004B400000ull));
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(q) : "l"(q), "l"(0x4B4000004B400000ull));
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(x) : "l"(q), "l"(negm2), "l"(x));
  asm("mov.b64 {%0, %1}, %2;" : "=r"(a), "=r"(b) : "l"(x));
}

// ---------------------------------------------------------------- tcgen05 wrappers
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)(16u >> 4) << 16;    // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024u >> 4) << 32;  // stride byte offset: 8 rows x 128 B
  d |= (uint64_t)1 << 46;             // descriptor version
  d |= (uint64_t)2 << 61;             // 128-byte swizzle
  return d;
}

// One 2-SM MMA: D[256 x 256] (+)= A[256 x 16] * B[16 x 256]^T, A's rows and
// B's columns split between the pair's shared memories at the same offsets.
__device__ __forceinline__ void umma_bf16_pair(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(IDESC), "r"(acc)
      : "memory");
}

// Arrive-once on the mbarrier at cluster address `bar` when this thread's
// earlier 2-SM MMAs have completed.
__device__ __forceinline__ void umma_commit_pair(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
        "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
        "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
        "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr)
      : "memory");
}

__device__ __forceinline__ void tmem_st32(uint32_t taddr, const uint32_t (&v)[32]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
      "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(taddr),
      "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]), "r"(v[8]),
      "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15]), "r"(v[16]), "r"(v[17]),
      "r"(v[18]), "r"(v[19]), "r"(v[20]), "r"(v[21]), "r"(v[22]), "r"(v[23]), "r"(v[24]), "r"(v[25]), "r"(v[26]),
      "r"(v[27]), "r"(v[28]), "r"(v[29]), "r"(v[30]), "r"(v[31])
      : "memory");
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// r = v mod m in [0, m) for an fp32 integer v (|v| < 2^25).
__device__ __forceinline__ float mod_pos(float v, float m, float inv) {
  float q = floorf(v * inv);
  float r = fmaf(-q, m, v);
  if (r < 0.f) r += m;
  if (r >= m) r -= m;
  return r;
}

// ---------------------------------------------------------------- kernel
__global__ void __cluster_dims__(PAIR, 1, 1) __launch_bounds__(NUM_THREADS, 1)
    oz_gemm_kernel(const OzGroupProb *__restrict__ probs, const __grid_constant__ GParams p) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t *bars = reinterpret_cast<uint64_t *>(base + STAGES * STAGE_BYTES);
  uint64_t *full = bars, *empty = bars + STAGES;
  uint64_t *cdone = bars + 2 * STAGES, *afree = cdone + 2, *drain = afree + 2;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(drain + 1);
  uint32_t *r1s = reinterpret_cast<uint32_t *>(base + STAGES * STAGE_BYTES + 256);
  auto smA = [&](int s) { return base + s * STAGE_BYTES; };
  auto smB = [&](int s) { return base + s * STAGE_BYTES + A_BYTES; };

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t rank = cluster_rank();
  const bool leader = rank == 0;  // issues the pair's MMAs; its barriers pace the pair
  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);   // leader: its expect_tx arrival, then both CTAs' bytes
      mbar_init(&empty[s], 1);  // the leader's commit after the stage's MMAs
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&cdone[b], 1);                 // the leader's commit at a chunk's end
      mbar_init(&afree[b], PAIR * EPI_WARPS);  // leader: every epilogue warp of the pair
    }
    mbar_init(drain, 1);
    fence_barrier_init();
  }
  if (warp == 1) {
    // The pair allocates its accumulator columns together (one warp of each CTA).
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
    tc_fence_before();
  }
  // Both CTAs' barriers are initialised before either CTA's copies or
  // commits can reach them.
  cluster_sync();
  tc_fence_after();
  const uint32_t tmem_base = *reinterpret_cast<volatile uint32_t *>(tmem_slot);

  if (warp == 0) {
    // ------------------------------------------------------------ TMA producer
    if (lane == 0) {
      int s = 0;
      uint32_t ph = 0, issued = 0, last_ph[STAGES] = {};
      bool ok = true;
      int cur = -1;
      for (int t = (int)cluster_index(); ok && t < p.total_tiles; t += (int)cluster_count()) {
        const int pi = find_problem(probs, p.nprob, t);
        const OzGroupProb &P = probs[pi];
        if (pi != cur) {
          tmap_acquire(&P.tmA);
          tmap_acquire(&P.tmB);
          cur = pi;
        }
        const Tile T = decode(P, t - P.tile_begin + P.tile_offset, (int)cluster_count());
        const int ya = (int)((T.l - P.l0) * P.Mp + ((int64_t)T.tp * PAIR + rank) * BM);
        const int yb = (int)((T.l - P.l0) * P.Np + (int64_t)T.tj * BN + rank * BH);
        for (int ks = T.ks0; ks < T.ks1; ++ks) {
          if (!mbar_wait_bounded(&empty[s], ph ^ 1)) {
            record_error(p.status, KERR_WAIT_TIMEOUT);
            ok = false;
            break;
          }
          // This CTA's A tile and its half of B, both counted on the leader's
          // full barrier, which expects both CTAs' bytes.
          const uint32_t fb = mapa(smem_u32(&full[s]), 0);
          if (leader) mbar_arrive_expect_tx(&full[s], PAIR_TX);
#pragma unroll
          for (int a = 0; a < ATOMS; ++a) {
            tma_load_2d_pair(smA(s) + a * ATOM_A, &P.tmA, ks * SLAB + a * BK, ya, fb);
            tma_load_2d_pair(smB(s) + a * ATOM_B, &P.tmB, ks * SLAB + a * BK, yb, fb);
          }
          issued |= 1u << s;
          last_ph[s] = ph;
          if (++s == STAGES) { s = 0; ph ^= 1; }
        }
      }
      // Drain.  The leader's full barriers count both CTAs' copies, so once
      // its last phases have completed nothing is in flight into either CTA.
      // The peer cannot see that barrier; it waits instead until the
      // leader's MMAs have released every stage it filled (which they do
      // only after its copies landed), so it never leaves with a copy in
      // flight into its own shared memory.
      for (int st = 0; st < STAGES; ++st)
        if ((issued >> st) & 1u)
          if (!mbar_wait_bounded(leader ? &full[st] : &empty[st], last_ph[st]))
            record_error(p.status, KERR_WAIT_TIMEOUT);
    }
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer (leader)
    if (lane == 0 && leader) {
      int s = 0;
      uint32_t ph = 0, gc = 0;
      bool ok = true, any = false;
      const uint32_t peer = rank ^ 1u;
      for (int t = (int)cluster_index(); ok && t < p.total_tiles; t += (int)cluster_count()) {
        const OzGroupProb &P = probs[find_problem(probs, p.nprob, t)];
        const Tile T = decode(P, t - P.tile_begin + P.tile_offset, (int)cluster_count());
        const int nslab = T.ks1 - T.ks0;
        const int nchunk = (nslab + CHUNK_SLABS - 1) / CHUNK_SLABS;
        for (int c = 0; ok && c < nchunk; ++c, ++gc) {
          const uint32_t b = gc & 1u, u = gc >> 1;
          if (!mbar_wait_bounded(&afree[b], (u & 1u) ^ 1u)) {
            record_error(p.status, KERR_WAIT_TIMEOUT);
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t d_tmem = tmem_base + b * (uint32_t)BN;
          const int sl0 = c * CHUNK_SLABS, sl1 = min(nslab, sl0 + CHUNK_SLABS);
          for (int sl = sl0; sl < sl1; ++sl) {
            if (!mbar_wait_bounded(&full[s], ph)) {
              record_error(p.status, KERR_WAIT_TIMEOUT);
              ok = false;
              break;
            }
            tc_fence_after();
            const uint32_t a0 = smem_u32(smA(s)), b0 = smem_u32(smB(s));
#pragma unroll
            for (int kk = 0; kk < SLAB / 16; ++kk) {
              const uint32_t acc = (c >= 2 || sl > sl0 || kk > 0) ? 1u : 0u;
              const uint32_t a = (uint32_t)(kk / (BK / 16)), w = (uint32_t)(kk % (BK / 16));
              umma_bf16_pair(d_tmem, sw128_desc(a0 + a * ATOM_A + w * 32), sw128_desc(b0 + a * ATOM_B + w * 32), acc);
            }
            // Stage s is free in both CTAs once these MMAs have read it.
            umma_commit_pair(smem_u32(&empty[s]));
            umma_commit_pair(mapa(smem_u32(&empty[s]), peer));
            any = true;
            if (++s == STAGES) { s = 0; ph ^= 1; }
          }
          if (!ok) break;
          umma_commit_pair(smem_u32(&cdone[b]));
          umma_commit_pair(mapa(smem_u32(&cdone[b]), peer));
        }
      }
      // Drain: all MMAs this thread issued complete before TMEM is freed.
      if (any) {
        umma_commit_pair(smem_u32(drain));
        if (!mbar_wait_bounded(drain, 0)) record_error(p.status, KERR_WAIT_TIMEOUT);
      }
    }
  } else {
    // ------------------------------------------------------------ epilogue
    const int quad = warp & 3;
    const int cb0 = ((warp - 2) >> 2) * CB_PER_WARP;  // this warp's first 32-column block
    const int row = quad * 32 + lane;
    const uint32_t lane_base = tmem_base + ((uint32_t)(quad * 32) << 16);
    uint32_t gc = 0;
    bool ok = true;
    for (int t = (int)cluster_index(); ok && t < p.total_tiles; t += (int)cluster_count()) {
      const OzGroupProb &P = probs[find_problem(probs, p.nprob, t)];
      const Tile T = decode(P, t - P.tile_begin + P.tile_offset, (int)cluster_count());
      const int nslab = T.ks1 - T.ks0;
      const int nchunk = (nslab + CHUNK_SLABS - 1) / CHUNK_SLABS;
      const float m = p.mod_f[T.l], inv = p.inv_f[T.l], cu = p.u_f[P.nmod][T.l];
      const uint64_t inv2 = pack2(inv), negm2 = pack2(-m);
      // This thread's row of the tile's residue output (column stride Mp).
      uint16_t *out = P.res + (int64_t)T.l * P.plane + ((int64_t)T.tp * PAIR + rank) * BM + row;
      uint32_t *r1 = r1s + row;  // this row's words of r1s, stride BM (each thread touches only its own)
      uint32_t hib[CB_PER_WARP];  // ninth bits of the second-to-last chunk's residues
      for (int c = 0; c < nchunk; ++c, ++gc) {
        const uint32_t b = gc & 1u, u = gc >> 1;
        if (!mbar_wait_bounded(&cdone[b], u & 1u)) {
          record_error(p.status, KERR_WAIT_TIMEOUT);
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t tb = lane_base + b * (uint32_t)BN;
        if (c + 2 < nchunk) {
          // Fold: acc := acc - m * q, q = x / m rounded to nearest, exact in
          // fp32, two values per packed instruction.
#pragma unroll 1
          for (int cb = cb0; cb < cb0 + CB_PER_WARP; ++cb) {
            uint32_t v[32];
            tmem_ld32(tb + (uint32_t)(cb * 32), v);
            tmem_wait_ld();
#pragma unroll
            for (int e = 0; e < 32; e += 2) fold2(v[e], v[e + 1], inv2, negm2);
            tmem_st32(tb + (uint32_t)(cb * 32), v);
          }
          tmem_wait_st();
        } else if (c + 2 == nchunk) {
          // Second-to-last chunk: its residues move aside, the buffer is freed now.
#pragma unroll 1
          for (int cb = cb0; cb < cb0 + CB_PER_WARP; ++cb) {
            uint32_t v[32];
            tmem_ld32(tb + (uint32_t)(cb * 32), v);
            tmem_wait_ld();
            uint32_t hi = 0;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
              uint32_t w = 0;
#pragma unroll
              for (int e = 0; e < 4; ++e) {
                const uint32_t r = (uint32_t)(int)mod_pos(__uint_as_float(v[q * 4 + e]), m, inv);
                w |= (r & 255u) << (8 * e);
                hi |= (r >> 8) << (q * 4 + e);
              }
              r1[(cb * 8 + q) * BM] = w;
            }
            hib[cb - cb0] = hi;
          }
        } else {
          // Last chunk: with v this chunk's sum and p the parked residue, the
          // stored 16-bit word is u_l (v + p) mod m_l.  v is folded to
          // |v'| <= 184 first, so x = (v' + p) u_l has |x| < 546 * 362 < 2^18
          // (exact); floor(x / m) in fp32 is exact except that a multiple of m
          // may come out one low, which the single correction handles.
          const bool two = nchunk >= 2;
#pragma unroll 1
          for (int cb = cb0; cb < cb0 + CB_PER_WARP; ++cb) {
            uint32_t v[32];
            tmem_ld32(tb + (uint32_t)(cb * 32), v);
            tmem_wait_ld();
            const int64_t j0 = (int64_t)T.tj * BN + cb * 32;
            const uint32_t hi = two ? hib[cb - cb0] : 0u;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
              const uint32_t w = two ? r1[(cb * 8 + q) * BM] : 0u;
#pragma unroll
              for (int e = 0; e < 4; ++e) {
                const uint32_t prev = ((w >> (8 * e)) & 255u) | (((hi >> (q * 4 + e)) & 1u) << 8);
                const float a = __uint_as_float(v[q * 4 + e]);
                const float x = (fmaf(-rintf(a * inv), m, a) + (float)prev) * cu;
                float y = fmaf(-floorf(x * inv), m, x);
                if (y >= m) y -= m;
                out[(j0 + q * 4 + e) * P.Mp] = (uint16_t)(int)y;
              }
            }
          }
        }
        tc_fence_before();
        __syncwarp();
        // The accumulator is free once every epilogue warp of the pair has
        // arrived on the leader's barrier.
        if (lane == 0) mbar_arrive_remote(mapa(smem_u32(&afree[b]), 0));
      }
    }
  }
  __syncthreads();
  // Neither CTA leaves while the other may still read its shared memory
  // through the pair's MMAs or arrive on its barriers.
  cluster_sync();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem_base), "r"(TMEM_COLS)
                 : "memory");
  }
}

int g_max_clusters = 0;  // co-resident CTA pairs of oz_gemm_kernel (set by oz_gemm_prepare)

}  // namespace

int oz_group_prob(const OzGemmLaunch &L, OzGroupProb *out, const char **why) {
  *why = nullptr;
  memset(out, 0, sizeof(*out));
  if (L.l1 <= L.l0 || L.M <= 0 || L.N <= 0 || L.K <= 0) {
    *why = "empty residue GEMM";
    return UVATRMM_EINVAL;
  }
  if (L.Mp % (PAIR * BM) || L.Np % BN || L.Kp % BK) {
    *why = "residue planes are not padded to the tile sizes";
    return UVATRMM_EINVAL;
  }
  if (L.l0 < 0 || L.l1 > L.n_moduli || L.n_moduli > kMaxModuli) {
    *why = "residue GEMM moduli outside the CRT set";
    return UVATRMM_EINVAL;
  }
  const int nmod = L.l1 - L.l0;
  if ((int64_t)nmod * L.Mp > INT32_MAX || (int64_t)nmod * L.Np > INT32_MAX || L.Kp > INT32_MAX) {
    *why = "problem too large for one residue pass";
    return UVATRMM_EINVAL;
  }
  if (make_tmap_2d(&out->tmA, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, L.LR, L.Kp, nmod * L.Mp, L.Kp * 2, BK, BM,
                   true) ||
      make_tmap_2d(&out->tmB, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, L.RR, L.Kp, nmod * L.Np, L.Kp * 2, BK, BH,
                   true)) {
    *why = "tensor map encoding failed for the residue planes";
    return UVATRMM_EDEVICE;
  }
  out->Mp = L.Mp; out->Np = L.Np; out->M = L.M; out->N = L.N; out->K = L.K;
  out->l0 = L.l0; out->l1 = L.l1;
  out->tri_left = L.tri_left;
  out->tri_lower = L.tri_lower;
  out->grows = L.tri_left ? L.tri_lower : !L.tri_lower;
  out->tiles_m = (int)(L.Mp / BM);
  out->tiles_n = (int)(L.Np / BN);
  out->tiles_per_mod = (out->tiles_m / PAIR) * out->tiles_n;
  out->tile_count = out->tiles_per_mod * nmod;
  // Default raster group: 2 pair rows (measured best with 128-deep slabs at
  // m = n = 8192 .. 32768 against 3; 3 was best with 64-deep slabs).
  out->group = L.raster_group > 0 ? L.raster_group : 2;
  out->res = L.res;
  out->plane = L.Mp * L.Np;
  out->nmod = L.n_moduli;
  return UVATRMM_OK;
}

int oz_gemm_prepare() {
  static bool done = false;
  if (!done) {
    if (cudaFuncSetAttribute(oz_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM) != cudaSuccess)
      return UVATRMM_EDEVICE;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(sms / PAIR * PAIR), 1, 1);
    cfg.blockDim = dim3(NUM_THREADS, 1, 1);
    cfg.dynamicSmemBytes = SMEM;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, oz_gemm_kernel, &cfg) != cudaSuccess || n <= 0) {
      cudaGetLastError();
      n = sms / PAIR;
    }
    g_max_clusters = n;
    done = true;
  }
  return UVATRMM_OK;
}

int launch_oz_gemm_group(const OzGroupProb *dprobs, int nprob, int total_tiles, int *status, int num_sms,
                         cudaStream_t st, const char **why) {
  *why = nullptr;
  if (nprob <= 0 || total_tiles <= 0) return UVATRMM_OK;
  GParams g;
  memset(&g, 0, sizeof(g));
  g.nprob = nprob;
  g.total_tiles = total_tiles;
  g.status = status;
  for (int l = 0; l < kMaxModuli; ++l) {
    g.mod_f[l] = (float)kModuli[l];
    g.inv_f[l] = 1.0f / (float)kModuli[l];
    for (int n = l + 1; n <= kMaxModuli; ++n) g.u_f[n][l] = (float)crt_u(n, l);
  }
  if (oz_gemm_prepare() != UVATRMM_OK) {
    *why = "cannot reserve shared memory for the residue GEMM";
    return UVATRMM_EDEVICE;
  }
  const int clusters = std::min(std::min(g_max_clusters, num_sms / PAIR), total_tiles);
  oz_gemm_kernel<<<std::max(clusters, 1) * PAIR, NUM_THREADS, SMEM, st>>>(dprobs, g);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    *why = cudaGetErrorString(e);
    return UVATRMM_EDEVICE;
  }
  return UVATRMM_OK;
}

int launch_oz_gemm(const OzGemmLaunch &L, cudaStream_t st, const char **why) {
  *why = nullptr;
  if (L.l1 <= L.l0 || L.M <= 0 || L.N <= 0 || L.K <= 0) return UVATRMM_OK;
  if (!L.desc) {
    *why = "no device slot for the residue GEMM descriptor";
    return UVATRMM_EINVAL;
  }
  OzGroupProb hp;
  if (int rc = oz_group_prob(L, &hp, why)) return rc;
  hp.tile_begin = 0;
  // A pageable-source async copy stages the descriptor before returning.
  cudaError_t e = cudaMemcpyAsync(L.desc, &hp, sizeof(hp), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) {
    *why = cudaGetErrorString(e);
    return UVATRMM_EDEVICE;
  }
  return launch_oz_gemm_group(L.desc, 1, hp.tile_count, L.status, L.num_sms, st, why);
}

}  // namespace uvt
