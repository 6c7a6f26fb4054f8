// Request loop with continuous batching (see the serving section of uvatrmm.h).
//
// One server thread owns the device work:
//   admit  - FIFO: the head request is admitted when a slot is free and the
//            pool (one cudaMalloc of the HBM budget, first-fit) has room for
//            its working set; host-mode operands are copied in on a copy
//            stream;
//   tick   - one grouped launch per kind over tile ranges taken from every
//            active request (Ozaki slicing of newly admitted requests, the
//            residue GEMM, Ozaki reassembly of requests whose last GEMM tiles
//            are in this tick, then the FP64 TRMM), alternating between two
//            compute streams with two ticks in flight, so one tick's tail
//            overlaps the next tick and the device never waits for the host;
//   retire - when a tick's Ozaki work completes, the Ozaki requests
//            reassembled in it are finished; when the whole tick completes,
//            its FP64 requests are (host mode: after their result's copy
//            back); their memory returns to the pool and waiters are woken.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "api_internal.h"
#include "common.cuh"
#include "ozaki.cuh"
#include "trmm_fp64.cuh"

namespace uvt {
void ozaki_operands(const Trmm &t, const double *dA, int64_t lda, const double *dB, int64_t ldb, OzOperand &L,
                    OzOperand &R);
}

namespace {

using namespace uvt;

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// First-fit allocator over [0, size) with 256-byte granularity.
class Pool {
 public:
  void init(size_t size) {
    size_ = size;
    free_.clear();
    free_[0] = size;
    used_ = peak_ = 0;
  }
  bool alloc(size_t bytes, size_t *off) {
    bytes = (bytes + 255) / 256 * 256;
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= bytes) {
        *off = it->first;
        const size_t rest = it->second - bytes, at = it->first + bytes;
        free_.erase(it);
        if (rest) free_[at] = rest;
        used_ += bytes;
        peak_ = std::max(peak_, used_);
        return true;
      }
    }
    return false;
  }
  void release(size_t off, size_t bytes) {
    bytes = (bytes + 255) / 256 * 256;
    used_ -= bytes;
    auto it = free_.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
  size_t peak() const { return peak_; }

 private:
  size_t size_ = 0, used_ = 0, peak_ = 0;
  std::map<size_t, size_t> free_;
};

enum ReqState { PENDING, ACTIVE, DONE, FAILED, CANCELLED };

struct Req {
  int64_t id = 0;
  uvatrmm_trmm_problem p{};
  bool on_device = false;
  Trmm t{};
  double flops = 0.0;
  ReqState state = PENDING;
  int status = UVATRMM_OK;
  double t_submit = 0.0, t_done = 0.0;
  size_t bytes = 0, off = 0;
  // device view of the operands (user buffers or pool copies)
  const double *A = nullptr;
  int64_t lda = 0;
  double *Bin = nullptr;  // FP64: staged input copy; Ozaki: the buffer sliced and overwritten
  int64_t ldbin = 0;
  double *Cout = nullptr;  // where the result lands on the device
  int64_t ldc = 0;
  // host mode: copy-in finished
  cudaEvent_t h2d = nullptr;
  bool h2d_pending = false;
  // FP64 tier
  Fp64GroupProb fd{};
  // Ozaki tier
  OzPlan plan{};
  OzGroupProb od{};
  int *e_row = nullptr, *e_col = nullptr;
  uint16_t *LR = nullptr, *RR = nullptr;
  uint16_t *res = nullptr;
  bool prepped = false;
  // tile progress
  int total = 0, next = 0;
  double tile_cost = 0.0;  // work per tile (flops of its tier)
  int64_t last_tick = -1;
  bool copy_back = false;
  cudaEvent_t d2h = nullptr;
};

struct TickSlot {
  char *dev = nullptr;
  char *host = nullptr;  // pinned mirror
  cudaEvent_t done = nullptr;
  cudaEvent_t prepped = nullptr;  // this tick's Ozaki slicing finished
  cudaEvent_t gemm_done = nullptr;  // this tick's residue GEMM (and slicing) finished
  cudaEvent_t oz_done = nullptr;    // this tick's Ozaki work finished (before its FP64 launch)
  bool has_prep = false;
  bool oz_retired = false;          // finishing_oz already retired
  int64_t id = -1;
  std::vector<int64_t> finishing;     // FP64-tier requests whose last work is in this tick
  std::vector<int64_t> finishing_oz;  // Ozaki-tier requests reassembled in this tick
};

}  // namespace

struct uvatrmm_server_st {
  uvatrmm_handle_t h = nullptr;  // internal handle (status word, SM count)
  int device = 0;
  uvatrmm_server_config cfg{};
  // Ticks alternate between two compute streams, so one tick's tail overlaps
  // the next tick's start; cross-tick order comes from events.
  cudaStream_t cstream[2] = {nullptr, nullptr};
  cudaStream_t copy = nullptr;
  char *arena = nullptr;
  Pool pool;
  // tick descriptor slots
  static constexpr int kSlots = 4;
  TickSlot slots[kSlots];
  size_t off_f64 = 0, off_oz = 0, off_prep = 0, off_reas = 0, slot_bytes = 0;
  int64_t tick_counter = 0;
  std::deque<int64_t> inflight;  // tick ids in order
  // requests
  std::mutex mu;
  std::condition_variable cv_submit, cv_done;
  std::unordered_map<int64_t, std::unique_ptr<Req>> reqs;
  std::deque<int64_t> pending;
  std::vector<int64_t> active;
  int64_t next_id = 1;
  bool stop = false;
  std::thread worker;
  // stats
  std::vector<double> lat_ms;
  uvatrmm_server_stats st{};
};

namespace {

size_t working_bytes(const Req &r) {
  const Trmm &t = r.t;
  const int64_t ka = t.side == CblasLeft ? t.m : t.n;
  size_t b = 0;
  auto add = [&](size_t x) { b += (x + 255) / 256 * 256; };
  const bool tier_oz = r.p.tier == UVATRMM_TIER_OZAKI;
  const bool stage_a = !r.on_device || reinterpret_cast<uintptr_t>(r.p.A) % 16 || r.p.lda % 2;
  if (stage_a || !r.on_device) add((size_t)round_up(ka, 16) * ka * 8);
  if (!tier_oz) {
    add((size_t)round_up(t.m, 16) * t.n * 8);            // staged input B
    if (!r.on_device) add((size_t)round_up(t.m, 16) * t.n * 8);  // output C
  } else {
    const OzPlan &pl = r.plan;
    if (!r.on_device) add((size_t)round_up(t.m, 16) * t.n * 8);  // B copy, overwritten
    add((size_t)(pl.Mp + pl.Np) * sizeof(int));
    add((size_t)pl.n_moduli * (pl.Mp + pl.Np) * pl.Kp * 2);
    add((size_t)pl.n_moduli * pl.Mp * pl.Np * sizeof(uint16_t));
  }
  return b;
}

// Lays out the request's pool block and builds its descriptors.
int setup(uvatrmm_server_t s, Req &r) {
  const Trmm &t = r.t;
  const int64_t ka = t.side == CblasLeft ? t.m : t.n;
  char *base = s->arena + r.off;
  size_t cur = 0;
  auto take = [&](size_t x) {
    char *p = base + cur;
    cur += (x + 255) / 256 * 256;
    return p;
  };
  const bool tier_oz = r.p.tier == UVATRMM_TIER_OZAKI;
  const bool stage_a = !r.on_device || reinterpret_cast<uintptr_t>(r.p.A) % 16 || r.p.lda % 2;
  const int64_t la = round_up(ka, 16), lb = round_up(t.m, 16);
  if (stage_a || !r.on_device) {
    double *dA = reinterpret_cast<double *>(take((size_t)la * ka * 8));
    const cudaMemcpyKind kind = r.on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (cudaMemcpy2DAsync(dA, la * 8, r.p.A, r.p.lda * 8, ka * 8, ka, kind, s->copy) != cudaSuccess)
      return UVATRMM_EDEVICE;
    r.A = dA;
    r.lda = la;
    r.h2d_pending = true;
  } else {
    r.A = r.p.A;
    r.lda = r.p.lda;
  }
  if (!tier_oz) {
    r.Bin = reinterpret_cast<double *>(take((size_t)lb * t.n * 8));
    r.ldbin = lb;
    const cudaMemcpyKind kind = r.on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (cudaMemcpy2DAsync(r.Bin, lb * 8, r.p.B, r.p.ldb * 8, t.m * 8, t.n, kind, s->copy) != cudaSuccess)
      return UVATRMM_EDEVICE;
    r.h2d_pending = true;
    if (r.on_device) {
      r.Cout = r.p.B;
      r.ldc = r.p.ldb;
    } else {
      r.Cout = reinterpret_cast<double *>(take((size_t)lb * t.n * 8));
      r.ldc = lb;
      r.copy_back = true;
    }
    Fp64Launch L;
    L.M = t.m;
    L.N = t.n;
    L.K = ka;
    L.alpha = t.alpha;
    L.C = r.Cout;
    L.ldc = r.ldc;
    L.unit = t.unit;
    L.tri_lower = (t.uplo == CblasLower) != (t.trans != 0);
    if (t.side == CblasLeft) {
      L.tri_left = true;
      L.xl = MatRef{r.A, ka, ka, r.lda};
      L.lft_kmajor = t.trans != 0;
      L.xr = MatRef{r.Bin, t.m, t.n, r.ldbin};
      L.rgt_kmajor = true;
    } else {
      L.tri_left = false;
      L.xl = MatRef{r.Bin, t.m, t.n, r.ldbin};
      L.lft_kmajor = false;
      L.xr = MatRef{r.A, ka, ka, r.lda};
      L.rgt_kmajor = t.trans == 0;
    }
    L.engine = UVATRMM_ENGINE_DFMA;
    L.schedule = UVATRMM_SCHED_DYNAMIC;
    L.shape = UVATRMM_SHAPE_TRAPEZOID;
    L.tile = 64;
    const char *why = nullptr;
    if (int rc = fp64_group_prob(L, 64, &r.fd, &why)) return rc;
    r.total = r.fd.tile_count;
    r.tile_cost = r.flops / std::max(1, r.total);
  } else {
    if (r.on_device) {
      r.Bin = r.p.B;
      r.ldbin = r.p.ldb;
    } else {
      r.Bin = reinterpret_cast<double *>(take((size_t)lb * t.n * 8));
      r.ldbin = lb;
      if (cudaMemcpy2DAsync(r.Bin, lb * 8, r.p.B, r.p.ldb * 8, t.m * 8, t.n, cudaMemcpyHostToDevice, s->copy) !=
          cudaSuccess)
        return UVATRMM_EDEVICE;
      r.h2d_pending = true;
      r.copy_back = true;
    }
    r.Cout = r.Bin;
    r.ldc = r.ldbin;
    const OzPlan &pl = r.plan;
    r.e_row = reinterpret_cast<int *>(take((size_t)(pl.Mp + pl.Np) * sizeof(int)));
    r.e_col = r.e_row + pl.Mp;
    r.LR = reinterpret_cast<uint16_t *>(take((size_t)pl.n_moduli * (pl.Mp + pl.Np) * pl.Kp * 2));
    r.RR = r.LR + (int64_t)pl.n_moduli * pl.Mp * pl.Kp;
    r.res = reinterpret_cast<uint16_t *>(take((size_t)pl.n_moduli * pl.Mp * pl.Np * sizeof(uint16_t)));
    OzGemmLaunch L;
    L.LR = r.LR;
    L.RR = r.RR;
    L.res = r.res;
    L.Mp = pl.Mp; L.Np = pl.Np; L.Kp = pl.Kp; L.M = pl.M; L.N = pl.N; L.K = pl.K;
    L.l0 = 0;
    L.l1 = pl.n_moduli;
    L.n_moduli = pl.n_moduli;
    L.tri_left = t.side == CblasLeft;
    L.tri_lower = (t.uplo == CblasLower) != (t.trans != 0);
    L.raster_group = 0;
    L.status = s->h->dctl + 1;
    L.num_sms = s->h->num_sms;
    const char *why = nullptr;
    if (int rc = oz_group_prob(L, &r.od, &why)) return rc;
    r.total = r.od.tile_count;
    r.tile_cost = (double)pl.n_moduli * 2.0 * pl.Mp * pl.Np * (pl.Kp / 2 + 64) / std::max(1, r.total);
  }
  if (r.h2d_pending) {
    if (cudaEventCreateWithFlags(&r.h2d, cudaEventDisableTiming) != cudaSuccess) return UVATRMM_EDEVICE;
    cudaEventRecord(r.h2d, s->copy);
  }
  return cur <= r.bytes ? UVATRMM_OK : UVATRMM_EINVAL;
}

void finish(uvatrmm_server_t s, Req &r, int status) {
  r.state = status == UVATRMM_OK ? DONE : FAILED;
  r.status = status;
  r.t_done = now_s();
  if (r.bytes) s->pool.release(r.off, r.bytes);
  r.bytes = 0;
  if (r.h2d) cudaEventDestroy(r.h2d);
  if (r.d2h) cudaEventDestroy(r.d2h);
  r.h2d = r.d2h = nullptr;
  if (status == UVATRMM_OK) {
    s->st.completed++;
    s->st.served_flops += r.flops;
    s->lat_ms.push_back((r.t_done - r.t_submit) * 1e3);
    s->st.last_done_s = std::max(s->st.last_done_s, r.t_done);
  } else {
    s->st.failed++;
  }
}

// Builds and enqueues one tick; returns false when there was nothing to do.
bool launch_tick(uvatrmm_server_t s, std::vector<Req *> &act) {
  const int64_t id = s->tick_counter;
  TickSlot &slot = s->slots[id % uvatrmm_server_st::kSlots];
  // the slot's previous tick must be retired (inflight holds at most 2 < kSlots)
  std::vector<Req *> prep, reas;
  std::vector<Fp64GroupProb> fdesc;
  std::vector<OzGroupProb> odesc;
  std::vector<Req *> touched;
  double f_budget = s->cfg.tick_fp64_gflop * 1e9, o_budget = s->cfg.tick_ozaki_gflop * 1e9;
  int f_begin = 0, o_begin = 0;
  // Order: the oldest request of each tier first, with at most a quarter of
  // the tier's tick (so nothing starves), then shortest remaining work first
  // (small requests are not stuck behind large ones).
  std::vector<Req *> order;
  std::vector<Req *> rest;
  Req *oldest[2] = {nullptr, nullptr};
  for (Req *r : act)
    if (r->next < r->total) {
      const int k = r->p.tier == UVATRMM_TIER_OZAKI;
      if (!oldest[k]) oldest[k] = r;
      else rest.push_back(r);
    }
  std::stable_sort(rest.begin(), rest.end(), [](const Req *a, const Req *b) {
    return (a->total - a->next) * a->tile_cost < (b->total - b->next) * b->tile_cost;
  });
  for (Req *r : oldest)
    if (r) order.push_back(r);
  order.insert(order.end(), rest.begin(), rest.end());
  // Tiles per request: first the shares above; then the tick is made
  // work-conserving -- budget nobody else could use goes to the requests in
  // the same order (the oldest first), so a request running with little
  // company is not held to a quarter of the device.
  std::vector<int> takes(order.size(), 0);
  int n_oz = 0, n_f64 = 0;
  for (size_t i = 0; i < order.size(); ++i) {
    Req *r = order[i];
    const bool oz = r->p.tier == UVATRMM_TIER_OZAKI;
    double &budget = oz ? o_budget : f_budget;
    if (budget <= 0) continue;
    if ((oz ? n_oz : n_f64) >= s->cfg.max_active) continue;
    const double share = r == oldest[oz ? 1 : 0] ? 0.25 * (oz ? s->cfg.tick_ozaki_gflop : s->cfg.tick_fp64_gflop) * 1e9
                                                 : budget;
    const int take = (int)std::min<double>(r->total - r->next, std::max(1.0, std::ceil(share / r->tile_cost)));
    budget -= take * r->tile_cost;
    takes[i] = take;
    (oz ? n_oz : n_f64)++;
  }
  for (size_t i = 0; i < order.size(); ++i) {
    Req *r = order[i];
    if (!takes[i]) continue;
    double &budget = r->p.tier == UVATRMM_TIER_OZAKI ? o_budget : f_budget;
    const int more = (int)std::min<double>(r->total - r->next - takes[i], std::floor(budget / r->tile_cost));
    if (more <= 0) continue;
    takes[i] += more;
    budget -= more * r->tile_cost;
  }
  for (size_t i = 0; i < order.size(); ++i) {
    Req *r = order[i];
    const int take = takes[i];
    if (!take) continue;
    const bool oz = r->p.tier == UVATRMM_TIER_OZAKI;
    if (oz) {
      if (!r->prepped) {
        prep.push_back(r);
        r->prepped = true;
      }
      OzGroupProb d = r->od;
      d.tile_begin = o_begin;
      d.tile_count = take;
      d.tile_offset = r->next;
      o_begin += take;
      odesc.push_back(d);
    } else {
      Fp64GroupProb d = r->fd;
      d.tile_begin = f_begin;
      d.tile_count = take;
      d.tile_offset = r->next;
      f_begin += take;
      fdesc.push_back(d);
    }
    r->next += take;
    touched.push_back(r);
    if (r->next >= r->total) {
      if (oz) reas.push_back(r);
      r->last_tick = id;
    }
  }
  if (touched.empty()) return false;
  cudaStream_t cs = s->cstream[id & 1];
  const TickSlot *prev = id > 0 ? &s->slots[(id - 1) % uvatrmm_server_st::kSlots] : nullptr;
  // Wait for the staging copies of the requests in this tick.
  for (Req *r : touched)
    if (r->h2d_pending) {
      cudaStreamWaitEvent(cs, r->h2d, 0);
      r->h2d_pending = false;
    }
  // Descriptor image -> pinned slot -> device slot.
  OzWaveTables tprep{}, treas{};
  std::vector<char> img_prep, img_reas;
  auto items = [&](const std::vector<Req *> &v) {
    std::vector<OzWaveItem> it(v.size());
    for (size_t k = 0; k < v.size(); ++k) {
      Req &r = *v[k];
      ozaki_operands(r.t, r.A, r.lda, r.Bin, r.ldbin, it[k].L, it[k].R);
      it[k].e_row = r.e_row;
      it[k].e_col = r.e_col;
      it[k].plan = r.plan;
      it[k].LR = r.LR;
      it[k].RR = r.RR;
      it[k].res = r.res;
      it[k].alpha = r.t.alpha;
      it[k].C = r.Cout;
      it[k].ldc = r.ldc;
    }
    return it;
  };
  if (!prep.empty()) {
    auto it = items(prep);
    oz_wave_image(it.data(), (int)it.size(), slot.dev + s->off_prep, img_prep, &tprep);
  }
  if (!reas.empty()) {
    auto it = items(reas);
    oz_wave_image(it.data(), (int)it.size(), slot.dev + s->off_reas, img_reas, &treas);
  }
  memcpy(slot.host + s->off_f64, fdesc.data(), fdesc.size() * sizeof(Fp64GroupProb));
  memcpy(slot.host + s->off_oz, odesc.data(), odesc.size() * sizeof(OzGroupProb));
  memcpy(slot.host + s->off_prep, img_prep.data(), img_prep.size());
  memcpy(slot.host + s->off_reas, img_reas.data(), img_reas.size());
  cudaMemcpyAsync(slot.dev, slot.host, s->slot_bytes, cudaMemcpyHostToDevice, cs);
  const char *why = nullptr;
  int rc = UVATRMM_OK;
  if (!prep.empty()) {
    rc = oz_wave_prep(tprep, cs);
    cudaEventRecord(slot.prepped, cs);
  }
  slot.has_prep = !prep.empty();
  // Residue tiles of a request sliced in the previous tick (other stream).
  if (prev && prev->has_prep && !odesc.empty()) cudaStreamWaitEvent(cs, prev->prepped, 0);
  if (rc == UVATRMM_OK && !odesc.empty())
    rc = launch_oz_gemm_group(reinterpret_cast<OzGroupProb *>(slot.dev + s->off_oz), (int)odesc.size(), o_begin,
                              s->h->dctl + 1, s->h->num_sms, cs, &why);
  cudaEventRecord(slot.gemm_done, cs);
  // The tick's Ozaki work comes before its FP64 tiles, so Ozaki requests that
  // finish here retire on oz_done without waiting for those tiles.
  if (rc == UVATRMM_OK && !reas.empty()) {
    // Earlier residue tiles of these requests ran in previous ticks: the one
    // before this (other stream) up to its residue GEMM; older ticks retired.
    if (prev) cudaStreamWaitEvent(cs, prev->gemm_done, 0);
    rc = oz_wave_reassemble(treas, cs);
  }
  cudaEventRecord(slot.oz_done, cs);
  if (rc == UVATRMM_OK && !fdesc.empty())
    rc = launch_trmm_fp64_group(reinterpret_cast<Fp64GroupProb *>(slot.dev + s->off_f64), (int)fdesc.size(),
                                f_begin, 64, UVATRMM_ENGINE_DFMA, s->h->dctl + 2 + (int)(id % 2), s->h->dctl + 1,
                                s->h->num_sms, cs, &why);
  // A tick retires only after the previous one, so completion is in order.
  if (prev) cudaStreamWaitEvent(cs, prev->done, 0);
  cudaEventRecord(slot.done, cs);
  slot.id = id;
  slot.finishing.clear();
  slot.finishing_oz.clear();
  slot.oz_retired = false;
  for (Req *r : touched)
    if (r->last_tick == id) {
      const bool oz = r->p.tier == UVATRMM_TIER_OZAKI;
      (oz ? slot.finishing_oz : slot.finishing).push_back(r->id);
      if (r->copy_back) {
        cudaEventCreateWithFlags(&r->d2h, cudaEventDisableTiming);
        cudaStreamWaitEvent(s->copy, oz ? slot.oz_done : slot.done, 0);
        cudaMemcpy2DAsync(r->p.B, r->p.ldb * 8, r->Cout, r->ldc * 8, r->t.m * 8, r->t.n, cudaMemcpyDeviceToHost,
                          s->copy);
        cudaEventRecord(r->d2h, s->copy);
      }
    }
  if (rc != UVATRMM_OK)
    for (Req *r : touched) r->status = rc;
  s->inflight.push_back(id);
  s->tick_counter++;
  s->st.ticks++;
  return true;
}

void worker(uvatrmm_server_t s) {
  cudaSetDevice(s->device);
  std::vector<Req *> act;
  std::vector<int64_t> done_wait;  // host-mode requests waiting for their copy back
  while (true) {
    bool did = false;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      // admit (FIFO)
      while (!s->pending.empty() && (int)s->active.size() < s->cfg.max_active) {
        Req &r = *s->reqs[s->pending.front()];
        if (r.state == CANCELLED) {
          s->pending.pop_front();
          continue;
        }
        size_t off;
        if (!s->pool.alloc(r.bytes, &off)) break;
        r.off = off;
        s->pending.pop_front();
        r.state = ACTIVE;
        int rc = setup(s, r);
        if (rc != UVATRMM_OK) {
          finish(s, r, rc);
          s->cv_done.notify_all();
          continue;
        }
        s->active.push_back(r.id);
        did = true;
      }
      s->st.peak_bytes = (int64_t)s->pool.peak();
      act.clear();
      for (int64_t id : s->active) act.push_back(s->reqs[id].get());
      if (s->stop && s->pending.empty() && s->active.empty() && s->inflight.empty() && done_wait.empty()) break;
    }
    // launch while fewer than two ticks are in flight
    if (s->inflight.size() < 2 && launch_tick(s, act)) did = true;
    // Retire: the Ozaki requests of any tick in flight once its Ozaki work
    // is done; the oldest tick (with its FP64 requests) once it is done.
    auto retire = [&](const std::vector<int64_t> &ids, cudaError_t q) {
      std::lock_guard<std::mutex> lk(s->mu);
      for (int64_t rid : ids) {
        Req &r = *s->reqs[rid];
        s->active.erase(std::find(s->active.begin(), s->active.end(), rid));
        if (r.d2h) done_wait.push_back(rid);
        else finish(s, r, q == cudaSuccess ? r.status : UVATRMM_EDEVICE);
      }
      s->cv_done.notify_all();
    };
    for (int64_t tid : s->inflight) {
      TickSlot &slot = s->slots[tid % uvatrmm_server_st::kSlots];
      if (slot.oz_retired) continue;
      const cudaError_t q = cudaEventQuery(slot.oz_done);
      if (q == cudaErrorNotReady) continue;
      slot.oz_retired = true;
      if (!slot.finishing_oz.empty()) {
        retire(slot.finishing_oz, q);
        did = true;
      }
    }
    if (!s->inflight.empty()) {
      TickSlot &slot = s->slots[s->inflight.front() % uvatrmm_server_st::kSlots];
      cudaError_t q = cudaEventQuery(slot.done);
      if (q != cudaErrorNotReady) {
        s->inflight.pop_front();
        if (!slot.oz_retired) {
          slot.oz_retired = true;
          retire(slot.finishing_oz, q);
        }
        retire(slot.finishing, q);
        did = true;
      }
    }
    if (!done_wait.empty()) {
      std::lock_guard<std::mutex> lk(s->mu);
      for (size_t k = 0; k < done_wait.size();) {
        Req &r = *s->reqs[done_wait[k]];
        cudaError_t q = cudaEventQuery(r.d2h);
        if (q != cudaErrorNotReady) {
          finish(s, r, q == cudaSuccess ? r.status : UVATRMM_EDEVICE);
          done_wait.erase(done_wait.begin() + k);
          did = true;
        } else {
          ++k;
        }
      }
      s->cv_done.notify_all();
    }
    if (!did) {
      std::unique_lock<std::mutex> lk(s->mu);
      s->cv_submit.wait_for(lk, std::chrono::microseconds(50));
    }
  }
}

}  // namespace

using namespace uvt;

extern "C" {

UVATRMM_API int uvatrmm_server_create(uvatrmm_handle_t h, const uvatrmm_server_config *cfg, uvatrmm_server_t *out) {
  if (!out) return fail(UVATRMM_EINVAL, "server pointer is NULL");
  *out = nullptr;
  if (!(h = resolve(h))) return uvatrmm_last_status();
  auto *s = new uvatrmm_server_st();
  s->cfg.hbm_budget_bytes = (int64_t)120e9;
  s->cfg.max_active = 512;
  s->cfg.tick_fp64_gflop = 12.0;
  s->cfg.tick_ozaki_gflop = 3000.0;
  if (cfg) {
    if (cfg->hbm_budget_bytes > 0) s->cfg.hbm_budget_bytes = cfg->hbm_budget_bytes;
    if (cfg->max_active > 0) s->cfg.max_active = cfg->max_active;
    if (cfg->tick_fp64_gflop > 0) s->cfg.tick_fp64_gflop = cfg->tick_fp64_gflop;
    if (cfg->tick_ozaki_gflop > 0) s->cfg.tick_ozaki_gflop = cfg->tick_ozaki_gflop;
  }
  s->device = h->device;
  uvatrmm_handle_t ih = nullptr;
  int rc = uvatrmm_create(&ih);
  if (rc != UVATRMM_OK) {
    delete s;
    return rc;
  }
  s->h = ih;
  cudaError_t e = cudaStreamCreateWithFlags(&s->cstream[0], cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->cstream[1], cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->copy, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&s->arena, (size_t)s->cfg.hbm_budget_bytes);
  // tick slots: FP64 descriptors, Ozaki descriptors, two wave-table areas
  const size_t na = (size_t)s->cfg.max_active;
  auto r = [](size_t b) { return (b + 255) / 256 * 256; };
  s->off_f64 = 0;
  s->off_oz = r(na * sizeof(Fp64GroupProb));
  s->off_prep = s->off_oz + r(na * sizeof(OzGroupProb));
  s->off_reas = s->off_prep + r(oz_wave_table_bytes((int)na));
  s->slot_bytes = s->off_reas + r(oz_wave_table_bytes((int)na));
  for (auto &sl : s->slots) {
    if (e == cudaSuccess) e = cudaMalloc(&sl.dev, s->slot_bytes);
    if (e == cudaSuccess) e = cudaMallocHost(&sl.host, s->slot_bytes);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.prepped, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.gemm_done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.oz_done, cudaEventDisableTiming);
  }
  if (e == cudaSuccess && (fp64_group_prepare(64, UVATRMM_ENGINE_DFMA) || oz_gemm_prepare())) e = cudaErrorUnknown;
  if (e != cudaSuccess) {
    const int code = cuda_fail(e, "server setup");
    uvatrmm_server_destroy(s);
    return code;
  }
  s->pool.init((size_t)s->cfg.hbm_budget_bytes);
  s->worker = std::thread(worker, s);
  *out = s;
  return ok();
}

UVATRMM_API int uvatrmm_server_submit(uvatrmm_server_t s, const uvatrmm_trmm_problem *p, int operands_on_device,
                                     int64_t *id) {
  if (!s || !p || !id) return fail(UVATRMM_EINVAL, "invalid arguments");
  if (int bad = check_args(p->layout, p->side, p->uplo, p->transa, p->diag, p->m, p->n, p->lda, p->ldb))
    return fail(UVATRMM_EINVAL, "parameter " + std::to_string(bad) + " had an illegal value");
  if (p->tier != UVATRMM_TIER_FP64 && p->tier != UVATRMM_TIER_OZAKI) return fail(UVATRMM_EINVAL, "unknown tier");
  if (p->tier == UVATRMM_TIER_OZAKI && p->moduli != 0 && (p->moduli < 2 || p->moduli > kMaxModuli))
    return fail(UVATRMM_EINVAL, "moduli out of range");
  auto r = std::make_unique<Req>();
  r->p = *p;
  r->on_device = operands_on_device != 0;
  r->t = normalise(p->layout, p->side, p->uplo, p->transa, p->diag, p->m, p->n, p->alpha);
  const Trmm &t = r->t;
  r->flops = t.side == CblasLeft ? (double)t.m * t.m * t.n : (double)t.n * t.n * t.m;
  if (p->tier == UVATRMM_TIER_OZAKI) {
    OzPlan &pl = r->plan;
    pl.M = t.m;
    pl.N = t.n;
    pl.K = t.side == CblasLeft ? t.m : t.n;
    pl.n_moduli = p->moduli ? p->moduli : ozaki_auto_moduli(pl.K);
    pl.bits = ozaki_bits(pl.n_moduli, pl.K);
    pl.Mp = oz_pad_rows(pl.M);
    pl.Np = oz_pad_cols(pl.N);
    pl.Kp = round_up(pl.K, 64);
  }
  if (t.m == 0 || t.n == 0 || t.alpha == 0.0) {
    // Nothing for the device to multiply: served at once.
    if (t.alpha == 0.0 && t.m && t.n) {
      if (r->on_device) {
        cudaMemset2D(p->B, p->ldb * 8, 0, t.m * 8, t.n);
      } else {
        for (int64_t j = 0; j < t.n; ++j) memset(p->B + j * p->ldb, 0, (size_t)t.m * 8);
      }
    }
    std::lock_guard<std::mutex> lk(s->mu);
    r->id = s->next_id++;
    r->t_submit = now_s();
    if (s->st.submitted == 0) s->st.first_submit_s = r->t_submit;
    s->st.submitted++;
    *id = r->id;
    Req &rr = *r;
    s->reqs[rr.id] = std::move(r);
    finish(s, rr, UVATRMM_OK);
    s->cv_done.notify_all();
    return ok();
  }
  r->bytes = working_bytes(*r);
  std::lock_guard<std::mutex> lk(s->mu);
  if (s->stop) return fail(UVATRMM_EINVAL, "server is stopping");
  if ((int64_t)r->bytes > s->cfg.hbm_budget_bytes) {
    s->st.refused++;
    return fail(UVATRMM_EBUSY, "request needs " + std::to_string(r->bytes) + " bytes, more than the HBM budget");
  }
  r->id = s->next_id++;
  r->t_submit = now_s();
  if (s->st.submitted == 0) s->st.first_submit_s = r->t_submit;
  s->st.submitted++;
  *id = r->id;
  s->pending.push_back(r->id);
  s->reqs[r->id] = std::move(r);
  s->cv_submit.notify_one();
  return ok();
}

UVATRMM_API int uvatrmm_server_wait(uvatrmm_server_t s, int64_t id, double timeout_s) {
  if (!s) return fail(UVATRMM_EINVAL, "server is NULL");
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return fail(UVATRMM_EINVAL, "unknown request id");
  Req &r = *it->second;
  auto finished = [&] { return r.state == DONE || r.state == FAILED || r.state == CANCELLED; };
  if (timeout_s < 0) s->cv_done.wait(lk, finished);
  else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), finished))
    return fail(UVATRMM_ENOTREADY, "request still in flight");
  if (r.state == CANCELLED) return fail(UVATRMM_EINVAL, "request was cancelled");
  if (r.state == FAILED) return fail(r.status, "request failed");
  return ok();
}

UVATRMM_API int uvatrmm_server_cancel(uvatrmm_server_t s, int64_t id) {
  if (!s) return fail(UVATRMM_EINVAL, "server is NULL");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return fail(UVATRMM_EINVAL, "unknown request id");
  Req &r = *it->second;
  if (r.state != PENDING) return fail(UVATRMM_EBUSY, "request already admitted");
  r.state = CANCELLED;
  s->pending.erase(std::find(s->pending.begin(), s->pending.end(), id));
  s->st.cancelled++;
  s->cv_done.notify_all();
  return ok();
}

UVATRMM_API int uvatrmm_server_latency(uvatrmm_server_t s, int64_t id, double *ms) {
  if (!s || !ms) return fail(UVATRMM_EINVAL, "invalid arguments");
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->reqs.find(id);
  if (it == s->reqs.end()) return fail(UVATRMM_EINVAL, "unknown request id");
  const Req &r = *it->second;
  if (r.state != DONE) return fail(r.state == FAILED ? r.status : UVATRMM_ENOTREADY, "request not completed");
  *ms = (r.t_done - r.t_submit) * 1e3;
  return ok();
}

UVATRMM_API int uvatrmm_server_get_stats(uvatrmm_server_t s, uvatrmm_server_stats *out) {
  if (!s || !out) return fail(UVATRMM_EINVAL, "invalid arguments");
  std::lock_guard<std::mutex> lk(s->mu);
  *out = s->st;
  std::vector<double> v = s->lat_ms;
  if (!v.empty()) {
    std::sort(v.begin(), v.end());
    auto pct = [&](double q) { return v[std::min(v.size() - 1, (size_t)(q * (v.size() - 1) + 0.5))]; };
    out->p50_ms = pct(0.5);
    out->p99_ms = pct(0.99);
    out->max_ms = v.back();
    double sum = 0;
    for (double x : v) sum += x;
    out->mean_ms = sum / v.size();
  }
  out->peak_bytes = (int64_t)s->pool.peak();
  return ok();
}

UVATRMM_API int uvatrmm_server_destroy(uvatrmm_server_t s) {
  if (!s) return ok();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    s->cv_submit.notify_all();
  }
  if (s->worker.joinable()) s->worker.join();
  for (auto cs : s->cstream)
    if (cs) cudaStreamSynchronize(cs);
  if (s->copy) cudaStreamSynchronize(s->copy);
  for (auto &sl : s->slots) {
    if (sl.dev) cudaFree(sl.dev);
    if (sl.host) cudaFreeHost(sl.host);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.prepped) cudaEventDestroy(sl.prepped);
    if (sl.gemm_done) cudaEventDestroy(sl.gemm_done);
    if (sl.oz_done) cudaEventDestroy(sl.oz_done);
  }
  if (s->arena) cudaFree(s->arena);
  for (auto cs : s->cstream)
    if (cs) cudaStreamDestroy(cs);
  if (s->copy) cudaStreamDestroy(s->copy);
  if (s->h) uvatrmm_destroy(s->h);
  delete s;
  return ok();
}

}  // extern "C"
