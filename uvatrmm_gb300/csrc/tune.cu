// Autotuner: per shape bucket, the FP64 output tile edge (64 or 128) and the
// Ozaki residue-GEMM raster group (1, 2 or 3), measured on the device and
// cached in a small text file ("tier side log2m log2n choice" per line).
#include <sys/stat.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <string>
#include <tuple>

#include "api_internal.h"
#include "common.cuh"

namespace uvt {
namespace {

using Key = std::tuple<int, int, int, int>;  // tier, side (0 L / 1 R), ceil log2 m, ceil log2 n
std::mutex g_mu;
std::map<Key, int> g_cache;
bool g_loaded = false;

std::string cache_path() {
  if (const char *p = getenv("UVATRMM_TUNE_CACHE")) return p;
  const char *home = getenv("HOME");
  return std::string(home ? home : "/tmp") + "/.cache/uvatrmm_tune.txt";
}

void load() {
  g_loaded = true;
  FILE *f = fopen(cache_path().c_str(), "r");
  if (!f) return;
  int t, s, bm, bn, c;
  while (fscanf(f, "%d %d %d %d %d", &t, &s, &bm, &bn, &c) == 5) g_cache[Key{t, s, bm, bn}] = c;
  fclose(f);
}

void save() {
  const std::string path = cache_path();
  const size_t slash = path.rfind('/');
  if (slash != std::string::npos) mkdir(path.substr(0, slash).c_str(), 0755);
  const std::string tmp = path + ".tmp";
  FILE *f = fopen(tmp.c_str(), "w");
  if (!f) return;
  for (auto &kv : g_cache)
    fprintf(f, "%d %d %d %d %d\n", std::get<0>(kv.first), std::get<1>(kv.first), std::get<2>(kv.first),
            std::get<3>(kv.first), kv.second);
  fclose(f);
  rename(tmp.c_str(), path.c_str());
}

int ceil_log2(int64_t x) {
  int b = 0;
  while ((int64_t(1) << b) < x) ++b;
  return b;
}

// Best-of-3 time of one configuration on a representative problem.
int measure(uvatrmm_handle_t h, int tier, int side, int64_t m, int64_t n, int choice, const double *dA,
            double *dB, double *dC, float *best_ms) {
  const int64_t ka = side == CblasLeft ? m : n;
  *best_ms = 1e30f;
  const int saved_tile = h->tile, saved_raster = h->oz_raster;
  if (tier == UVATRMM_TIER_FP64) h->tile = choice;
  else h->oz_raster = choice;
  int rc = UVATRMM_OK;
  for (int rep = 0; rep < 4 && rc == UVATRMM_OK; ++rep) {
    cudaEventRecord(h->ev0, h->stream);
    if (tier == UVATRMM_TIER_FP64)
      rc = device_trmm(h, CblasColMajor, side, CblasLower, CblasNoTrans, CblasNonUnit, m, n, 1.0, dA, ka, dB, m,
                       dC, m, false, UVATRMM_SCHED_DYNAMIC, UVATRMM_SHAPE_TRAPEZOID);
    else
      rc = ozaki_device(h, CblasColMajor, side, CblasLower, CblasNoTrans, CblasNonUnit, m, n, 1.0, dA, ka, dC, m, 0,
                        nullptr, nullptr);
    cudaEventRecord(h->ev1, h->stream);
    if (rc == UVATRMM_OK && cudaEventSynchronize(h->ev1) != cudaSuccess) rc = UVATRMM_EDEVICE;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->ev0, h->ev1);
    if (rep > 0 && ms < *best_ms) *best_ms = ms;  // first run warms up
  }
  h->tile = saved_tile;
  h->oz_raster = saved_raster;
  if (rc == UVATRMM_OK) rc = collect_status(h);
  return rc;
}

}  // namespace

int tune_choice(uvatrmm_handle_t h, int tier, int side, int64_t m, int64_t n, int *choice) {
  if (tier != UVATRMM_TIER_FP64 && tier != UVATRMM_TIER_OZAKI) return fail(UVATRMM_EINVAL, "unknown tier");
  if (side != CblasLeft && side != CblasRight) return fail(UVATRMM_EINVAL, "unknown side");
  const Key key{tier, side == CblasLeft ? 0 : 1, ceil_log2(std::max<int64_t>(m, 1)),
                ceil_log2(std::max<int64_t>(n, 1))};
  const int fallback = tier == UVATRMM_TIER_FP64 ? 64 : 8;
  {
    std::lock_guard<std::mutex> g(g_mu);
    if (!g_loaded) load();
    auto it = g_cache.find(key);
    if (it != g_cache.end()) {
      *choice = it->second;
      return UVATRMM_OK;
    }
  }
  *choice = fallback;
  if (!h->autotune) return UVATRMM_OK;
  // Representative problem of the bucket, capped so a trial stays short.
  const int64_t rm = std::min<int64_t>(int64_t(1) << std::get<2>(key), 2048);
  const int64_t rn = std::min<int64_t>(int64_t(1) << std::get<3>(key), 2048);
  const int64_t ka = side == CblasLeft ? rm : rn;
  double *dA = nullptr, *dB = nullptr, *dC = nullptr;
  cudaError_t e = cudaMalloc(&dA, (size_t)ka * ka * 8);
  if (e == cudaSuccess) e = cudaMalloc(&dB, (size_t)rm * rn * 8);
  if (e == cudaSuccess) e = cudaMalloc(&dC, (size_t)rm * rn * 8);
  if (e != cudaSuccess) {
    cudaFree(dA);
    cudaFree(dB);
    return cuda_fail(e, "autotuner buffers");
  }
  uvatrmm_gen_uniform(h, 99, 0, ka, ka, dA, 1, ka, 0, 0.0, 0);
  uvatrmm_gen_uniform(h, 99, 1, rm, rn, dB, 1, rm, 0, 0.0, 0);
  const int cand_fp64[2] = {64, 128}, cand_oz[3] = {1, 2, 3};
  const int *cand = tier == UVATRMM_TIER_FP64 ? cand_fp64 : cand_oz;
  const int ncand = tier == UVATRMM_TIER_FP64 ? 2 : 3;
  float best = 1e30f;
  int pick = fallback, rc = UVATRMM_OK;
  for (int c = 0; c < ncand && rc == UVATRMM_OK; ++c) {
    if (tier == UVATRMM_TIER_OZAKI)
      cudaMemcpyAsync(dC, dB, (size_t)rm * rn * 8, cudaMemcpyDeviceToDevice, h->stream);
    float ms;
    rc = measure(h, tier, side, rm, rn, cand[c], dA, dB, dC, &ms);
    if (rc == UVATRMM_OK && ms < best) {
      best = ms;
      pick = cand[c];
    }
  }
  cudaStreamSynchronize(h->stream);
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dC);
  if (rc != UVATRMM_OK) return rc;
  *choice = pick;
  std::lock_guard<std::mutex> g(g_mu);
  g_cache[key] = pick;
  save();
  return UVATRMM_OK;
}

}  // namespace uvt

using namespace uvt;

extern "C" UVATRMM_API int uvatrmm_tune(uvatrmm_handle_t h, int tier, int side, int64_t m, int64_t n, int *choice) {
  if (!(h = resolve(h))) return uvatrmm_last_status();
  if (!choice || m < 0 || n < 0) return fail(UVATRMM_EINVAL, "invalid arguments");
  std::lock_guard<std::mutex> g(h->mu);
  int rc = tune_choice(h, tier, side, m, n, choice);
  return rc == UVATRMM_OK ? ok() : rc;
}
