// Grouped batches: many TRMMs planned once and captured into one CUDA graph.
//
// Plan (uvatrmm_group_create):
//   * FP64-tier problems: each is staged like the in-place device call (B, and
//     A when it is not 16-byte aligned with an even lda, into the group's
//     arena), gets its tile edge from the autotuner, and becomes one
//     Fp64GroupProb; problems of the same tile edge share one persistent
//     grouped launch (trmm_fp64_group_kernel), longest problems first.
//   * Ozaki-tier problems: each gets its scales, residue planes and residue
//     output in the arena; they are packed into waves that fit the Ozaki
//     scratch budget; a wave is the slicing kernels of its problems, ONE
//     grouped residue-GEMM launch over all their tiles, then the CRT
//     reassembly of each problem.
//   * Everything is captured on the handle's stream into a CUDA graph; a run
//     replays it.  Descriptors are uploaded before the capture.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "api_internal.h"
#include "common.cuh"
#include "ozaki.cuh"
#include "trmm_fp64.cuh"

struct uvatrmm_group_st {
  uvatrmm_handle_t h = nullptr;
  void *arena = nullptr;
  size_t arena_bytes = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  double flops = 0.0;
  int launches = 0, waves = 0;
  int64_t fp64_tiles = 0, oz_tiles = 0;
};

namespace uvt {

// The two residue operands of a normalised TRMM (ozaki_api.cu).
void ozaki_operands(const Trmm &t, const double *dA, int64_t lda, const double *dB, int64_t ldb, OzOperand &L,
                    OzOperand &R);

namespace {

struct ArenaPlan {
  size_t used = 0;
  size_t take(size_t bytes, size_t align = 256) {
    used = (used + align - 1) / align * align;
    const size_t off = used;
    used += bytes;
    return off;
  }
};

struct F64Item {
  Trmm t;
  const double *A;
  int64_t lda;
  double *B;
  int64_t ldb;
  int tile;
  bool stage_a;
  int64_t la, lb;
  size_t offA = 0, offB = 0;
  int64_t work = 0;  // slabs of the largest tile, for the longest-first order
};

struct OzItem {
  Trmm t;
  const double *A;
  int64_t lda;
  double *B;
  int64_t ldb;
  OzPlan plan;
  int raster;
  size_t bytes = 0;           // scales + planes + residues
  size_t offE = 0, offP = 0, offR = 0;  // inside the wave region
  int wave = 0;
};

bool tma_aligned(const void *p, int64_t ld) { return (reinterpret_cast<uintptr_t>(p) % 16 == 0) && (ld % 2 == 0); }

Fp64Launch fp64_launch(const Trmm &t, const double *A, int64_t lda, const double *B, int64_t ldb, double *C,
                       int64_t ldc, int tile) {
  Fp64Launch L;
  const int64_t ka = t.side == CblasLeft ? t.m : t.n;
  L.M = t.m;
  L.N = t.n;
  L.K = ka;
  L.alpha = t.alpha;
  L.C = C;
  L.ldc = ldc;
  L.unit = t.unit;
  L.tri_lower = (t.uplo == CblasLower) != (t.trans != 0);
  if (t.side == CblasLeft) {
    L.tri_left = true;
    L.xl = MatRef{A, ka, ka, lda};
    L.lft_kmajor = t.trans != 0;
    L.xr = MatRef{B, t.m, t.n, ldb};
    L.rgt_kmajor = true;
  } else {
    L.tri_left = false;
    L.xl = MatRef{B, t.m, t.n, ldb};
    L.lft_kmajor = false;
    L.xr = MatRef{A, ka, ka, lda};
    L.rgt_kmajor = t.trans == 0;
  }
  L.engine = UVATRMM_ENGINE_DFMA;
  L.schedule = UVATRMM_SCHED_DYNAMIC;
  L.shape = UVATRMM_SHAPE_TRAPEZOID;
  L.tile = tile;
  return L;
}

void destroy_group(uvatrmm_group_t g) {
  if (!g) return;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  if (g->arena) cudaFree(g->arena);
  delete g;
}

int build(uvatrmm_group_t g, const uvatrmm_trmm_problem *probs, int count) {
  uvatrmm_handle_t h = g->h;
  std::vector<F64Item> f64;
  std::vector<OzItem> oz;
  std::vector<std::pair<double *, Trmm>> zeros;
  std::vector<int64_t> zero_ld;
  for (int i = 0; i < count; ++i) {
    const uvatrmm_trmm_problem &p = probs[i];
    if (int bad = check_args(p.layout, p.side, p.uplo, p.transa, p.diag, p.m, p.n, p.lda, p.ldb))
      return fail(UVATRMM_EINVAL, "problem " + std::to_string(i) + ": parameter " + std::to_string(bad) +
                                      " had an illegal value");
    if (p.tier != UVATRMM_TIER_FP64 && p.tier != UVATRMM_TIER_OZAKI)
      return fail(UVATRMM_EINVAL, "problem " + std::to_string(i) + ": unknown tier");
    if (p.tier == UVATRMM_TIER_OZAKI && p.moduli != 0 && (p.moduli < 2 || p.moduli > kMaxModuli))
      return fail(UVATRMM_EINVAL, "problem " + std::to_string(i) + ": moduli out of range");
    if (!p.B || (!p.A && p.m && p.n)) return fail(UVATRMM_EINVAL, "problem " + std::to_string(i) + ": NULL buffer");
    const Trmm t = normalise(p.layout, p.side, p.uplo, p.transa, p.diag, p.m, p.n, p.alpha);
    if (t.m == 0 || t.n == 0) continue;
    g->flops += t.side == CblasLeft ? (double)t.m * t.m * t.n : (double)t.n * t.n * t.m;
    if (t.alpha == 0.0) {
      zeros.push_back({p.B, t});
      zero_ld.push_back(p.ldb);
      continue;
    }
    if (p.tier == UVATRMM_TIER_FP64) {
      F64Item it;
      it.t = t;
      it.A = p.A;
      it.lda = p.lda;
      it.B = p.B;
      it.ldb = p.ldb;
      if (int rc = tune_choice(h, UVATRMM_TIER_FP64, t.side, t.m, t.n, &it.tile)) return rc;
      const int64_t ka = t.side == CblasLeft ? t.m : t.n;
      it.stage_a = !tma_aligned(p.A, p.lda);
      it.la = round_up(ka, 16);
      it.lb = round_up(t.m, 16);
      it.work = (ka + it.tile - 1) / it.tile;
      f64.push_back(it);
    } else {
      OzItem it;
      it.t = t;
      it.A = p.A;
      it.lda = p.lda;
      it.B = p.B;
      it.ldb = p.ldb;
      OzPlan &pl = it.plan;
      pl.M = t.m;
      pl.N = t.n;
      pl.K = t.side == CblasLeft ? t.m : t.n;
      pl.n_moduli = p.moduli ? p.moduli : ozaki_auto_moduli(pl.K);
      pl.bits = ozaki_bits(pl.n_moduli, pl.K);
      pl.Mp = oz_pad_rows(pl.M);
      pl.Np = oz_pad_cols(pl.N);
      pl.Kp = round_up(pl.K, 64);
      if (int rc = tune_choice(h, UVATRMM_TIER_OZAKI, t.side, t.m, t.n, &it.raster)) return rc;
      ArenaPlan a;
      it.offE = a.take((size_t)(pl.Mp + pl.Np) * sizeof(int));
      it.offP = a.take((size_t)pl.n_moduli * (pl.Mp + pl.Np) * pl.Kp * 2);
      it.offR = a.take((size_t)pl.n_moduli * pl.Mp * pl.Np * sizeof(uint16_t));
      it.bytes = round_up((int64_t)a.used, 256);
      oz.push_back(it);
    }
  }

  // ---- arena layout: control words, FP64 descriptors + staging, Ozaki waves
  ArenaPlan A;
  const size_t off_ctl = A.take(256);
  std::sort(f64.begin(), f64.end(), [](const F64Item &x, const F64Item &y) { return x.work > y.work; });
  std::vector<int> classes;  // tile edges in use
  for (auto &it : f64)
    if (std::find(classes.begin(), classes.end(), it.tile) == classes.end()) classes.push_back(it.tile);
  std::vector<size_t> off_desc(classes.size());
  std::vector<std::vector<int>> members(classes.size());
  for (size_t c = 0; c < classes.size(); ++c) {
    for (int i = 0; i < (int)f64.size(); ++i)
      if (f64[i].tile == classes[c]) members[c].push_back(i);
    off_desc[c] = A.take(members[c].size() * sizeof(Fp64GroupProb), 64);
  }
  for (auto &it : f64) {
    it.offB = A.take((size_t)it.lb * it.t.n * 8);
    if (it.stage_a) it.offA = A.take((size_t)it.la * (it.t.side == CblasLeft ? it.t.m : it.t.n) * 8);
  }
  // Ozaki waves: greedy packing under the scratch budget.
  const size_t budget = (size_t)h->ozaki_scratch_mb << 20;
  std::vector<std::vector<int>> waves;
  size_t wave_bytes = 0, max_wave = 0;
  for (int i = 0; i < (int)oz.size(); ++i) {
    if (waves.empty() || (wave_bytes + oz[i].bytes > budget && !waves.back().empty())) {
      waves.emplace_back();
      wave_bytes = 0;
    }
    oz[i].wave = (int)waves.size() - 1;
    oz[i].offE += wave_bytes;
    oz[i].offP += wave_bytes;
    oz[i].offR += wave_bytes;
    wave_bytes += oz[i].bytes;
    waves.back().push_back(i);
    max_wave = std::max(max_wave, wave_bytes);
  }
  std::vector<size_t> off_wdesc(waves.size()), off_wtab(waves.size());
  for (size_t w = 0; w < waves.size(); ++w) {
    off_wdesc[w] = A.take(waves[w].size() * sizeof(OzGroupProb), 64);
    off_wtab[w] = A.take(oz_wave_table_bytes((int)waves[w].size()));
  }
  const size_t off_wave = A.take(max_wave);
  g->arena_bytes = A.used;
  cudaError_t e = cudaMalloc(&g->arena, std::max<size_t>(g->arena_bytes, 256));
  if (e != cudaSuccess) {
    const std::string what = "group arena (" + std::to_string(g->arena_bytes) + " bytes)";
    return cuda_fail(e, what.c_str());
  }
  char *base = static_cast<char *>(g->arena);
  int *ctl = reinterpret_cast<int *>(base + off_ctl);
  cudaMemset(ctl, 0, 256);

  // ---- descriptors (host-built, uploaded before capture)
  const char *why = nullptr;
  std::vector<int> class_total(classes.size(), 0);
  for (size_t c = 0; c < classes.size(); ++c) {
    std::vector<Fp64GroupProb> hd(members[c].size());
    int begin = 0;
    for (size_t k = 0; k < members[c].size(); ++k) {
      const F64Item &it = f64[members[c][k]];
      const double *Ause = it.stage_a ? reinterpret_cast<double *>(base + it.offA) : it.A;
      const int64_t ldA = it.stage_a ? it.la : it.lda;
      const double *Bs = reinterpret_cast<double *>(base + it.offB);
      Fp64Launch L = fp64_launch(it.t, Ause, ldA, Bs, it.lb, it.B, it.ldb, it.tile);
      if (int rc = fp64_group_prob(L, it.tile, &hd[k], &why)) return fail(rc, why ? why : "FP64 descriptor");
      hd[k].tile_begin = begin;
      begin += hd[k].tile_count;
    }
    class_total[c] = begin;
    g->fp64_tiles += begin;
    e = cudaMemcpy(base + off_desc[c], hd.data(), hd.size() * sizeof(Fp64GroupProb), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "FP64 descriptors");
    if (int rc = fp64_group_prepare(classes[c], UVATRMM_ENGINE_DFMA)) return fail(rc, "FP64 kernel attributes");
  }
  std::vector<int> wave_total(waves.size(), 0);
  std::vector<OzWaveTables> wave_tab(waves.size());
  for (size_t w = 0; w < waves.size(); ++w) {
    std::vector<OzGroupProb> hd(waves[w].size());
    std::vector<OzWaveItem> items(waves[w].size());
    int begin = 0;
    for (size_t k = 0; k < waves[w].size(); ++k) {
      const OzItem &it = oz[waves[w][k]];
      const OzPlan &pl = it.plan;
      OzWaveItem &wi = items[k];
      ozaki_operands(it.t, it.A, it.lda, it.B, it.ldb, wi.L, wi.R);
      wi.e_row = reinterpret_cast<int *>(base + off_wave + it.offE);
      wi.e_col = wi.e_row + pl.Mp;
      wi.plan = pl;
      wi.LR = reinterpret_cast<uint16_t *>(base + off_wave + it.offP);
      wi.RR = wi.LR + (int64_t)pl.n_moduli * pl.Mp * pl.Kp;
      wi.res = reinterpret_cast<uint16_t *>(base + off_wave + it.offR);
      wi.alpha = it.t.alpha;
      wi.C = it.B;
      wi.ldc = it.ldb;
      OzGemmLaunch L;
      L.LR = reinterpret_cast<uint16_t *>(base + off_wave + it.offP);
      L.RR = L.LR + (int64_t)pl.n_moduli * pl.Mp * pl.Kp;
      L.res = reinterpret_cast<uint16_t *>(base + off_wave + it.offR);
      L.Mp = pl.Mp; L.Np = pl.Np; L.Kp = pl.Kp; L.M = pl.M; L.N = pl.N; L.K = pl.K;
      L.l0 = 0; L.l1 = pl.n_moduli;
      L.n_moduli = pl.n_moduli;
      L.tri_left = it.t.side == CblasLeft;
      L.tri_lower = (it.t.uplo == CblasLower) != (it.t.trans != 0);
      L.raster_group = it.raster;
      L.status = h->dctl + 1;
      L.num_sms = h->num_sms;
      if (int rc = oz_group_prob(L, &hd[k], &why)) return fail(rc, why ? why : "Ozaki descriptor");
      hd[k].tile_begin = begin;
      begin += hd[k].tile_count;
    }
    wave_total[w] = begin;
    g->oz_tiles += begin;
    e = cudaMemcpy(base + off_wdesc[w], hd.data(), hd.size() * sizeof(OzGroupProb), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "Ozaki descriptors");
    if (int rc = oz_wave_tables(items.data(), (int)items.size(), base + off_wtab[w], &wave_tab[w]))
      return fail(rc, "Ozaki wave job tables");
  }
  if (!waves.empty())
    if (int rc = oz_gemm_prepare()) return fail(rc, "residue GEMM attributes");
  g->waves = (int)waves.size();

  // ---- capture
  cudaStream_t st = h->stream;
  bool own_stream = false;
  if (!st) {  // the legacy default stream cannot be captured
    if ((e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking)) != cudaSuccess)
      return cuda_fail(e, "capture stream");
    own_stream = true;
  }
  e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    if (own_stream) cudaStreamDestroy(st);
    return cuda_fail(e, "cudaStreamBeginCapture");
  }
  int rc = UVATRMM_OK;
  for (size_t z = 0; z < zeros.size() && rc == UVATRMM_OK; ++z)
    if (cudaMemset2DAsync(zeros[z].first, zero_ld[z] * 8, 0, zeros[z].second.m * 8, zeros[z].second.n, st) !=
        cudaSuccess)
      rc = UVATRMM_EDEVICE;
  // Per wave: grouped scales + residues (2 launches), one grouped residue
  // GEMM, one grouped reassembly.
  for (size_t w = 0; w < waves.size() && rc == UVATRMM_OK; ++w) {
    rc = oz_wave_prep(wave_tab[w], st);
    if (rc == UVATRMM_OK)
      rc = launch_oz_gemm_group(reinterpret_cast<OzGroupProb *>(base + off_wdesc[w]), (int)waves[w].size(),
                                wave_total[w], h->dctl + 1, h->num_sms, st, &why);
    if (rc == UVATRMM_OK) rc = oz_wave_reassemble(wave_tab[w], st);
    g->launches += 4;
  }
  for (auto &it : f64) {
    if (rc != UVATRMM_OK) break;
    e = cudaMemcpy2DAsync(base + it.offB, it.lb * 8, it.B, it.ldb * 8, it.t.m * 8, it.t.n, cudaMemcpyDeviceToDevice,
                          st);
    const int64_t ka = it.t.side == CblasLeft ? it.t.m : it.t.n;
    if (e == cudaSuccess && it.stage_a)
      e = cudaMemcpy2DAsync(base + it.offA, it.la * 8, it.A, it.lda * 8, ka * 8, ka, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) rc = UVATRMM_EDEVICE;
  }
  for (size_t c = 0; c < classes.size() && rc == UVATRMM_OK; ++c) {
    rc = launch_trmm_fp64_group(reinterpret_cast<Fp64GroupProb *>(base + off_desc[c]), (int)members[c].size(),
                                class_total[c], classes[c], UVATRMM_ENGINE_DFMA, ctl + (int)c, h->dctl + 1,
                                h->num_sms, st, &why);
    g->launches += 1;
  }
  cudaGraph_t graph = nullptr;
  e = cudaStreamEndCapture(st, &graph);
  if (own_stream) cudaStreamDestroy(st);
  if (rc != UVATRMM_OK) {
    if (graph) cudaGraphDestroy(graph);
    return fail(rc, why ? why : "capturing the group failed");
  }
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
  g->graph = graph;
  e = cudaGraphInstantiate(&g->exec, graph, 0);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
  return UVATRMM_OK;
}

}  // namespace
}  // namespace uvt

using namespace uvt;

extern "C" {

UVATRMM_API int uvatrmm_group_create(uvatrmm_handle_t h, const uvatrmm_trmm_problem *problems, int count,
                                    uvatrmm_group_t *group) {
  if (!group) return fail(UVATRMM_EINVAL, "group pointer is NULL");
  *group = nullptr;
  if (!(h = resolve(h))) return uvatrmm_last_status();
  if (count < 0 || (count > 0 && !problems)) return fail(UVATRMM_EINVAL, "invalid problem list");
  std::lock_guard<std::mutex> lk(h->mu);
  auto *g = new uvatrmm_group_st();
  g->h = h;
  int rc = build(g, problems, count);
  if (rc != UVATRMM_OK) {
    destroy_group(g);
    return rc;
  }
  *group = g;
  return ok();
}

UVATRMM_API int uvatrmm_group_run(uvatrmm_group_t g) {
  if (!g) return fail(UVATRMM_EINVAL, "group is NULL");
  std::lock_guard<std::mutex> lk(g->h->mu);
  cudaError_t e = cudaGraphLaunch(g->exec, g->h->stream);
  return e == cudaSuccess ? ok() : cuda_fail(e, "cudaGraphLaunch");
}

UVATRMM_API int uvatrmm_group_stats(uvatrmm_group_t g, double *flops, int *launches, int64_t *fp64_tiles,
                                   int64_t *ozaki_tiles, int *ozaki_waves, int64_t *arena_bytes) {
  if (!g) return fail(UVATRMM_EINVAL, "group is NULL");
  if (flops) *flops = g->flops;
  if (launches) *launches = g->launches;
  if (fp64_tiles) *fp64_tiles = g->fp64_tiles;
  if (ozaki_tiles) *ozaki_tiles = g->oz_tiles;
  if (ozaki_waves) *ozaki_waves = g->waves;
  if (arena_bytes) *arena_bytes = (int64_t)g->arena_bytes;
  return ok();
}

UVATRMM_API int uvatrmm_group_destroy(uvatrmm_group_t g) {
  if (!g) return ok();
  {
    std::lock_guard<std::mutex> lk(g->h->mu);
    cudaStreamSynchronize(g->h->stream);
  }
  destroy_group(g);
  return ok();
}

}  // extern "C"
