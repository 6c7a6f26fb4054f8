// Internal host-side pieces shared by the C-ABI translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>

#include "uvatrmm.h"

struct uvatrmm_handle_st {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  int engine = UVATRMM_ENGINE_DFMA;
  int schedule = UVATRMM_SCHED_DYNAMIC;
  int shape = UVATRMM_SHAPE_TRAPEZOID;
  int tile = 0;
  // Grow-only device workspace slots.
  void *ws[4] = {nullptr, nullptr, nullptr, nullptr};
  size_t ws_cap[4] = {0, 0, 0, 0};
  int *dctl = nullptr;  // [0] tile counter, [1] kernel status word
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::mutex mu;
};

namespace uvt {

// Thread-local error reporting.
int fail(int status, const std::string &msg);
int ok();
int cuda_fail(cudaError_t e, const char *what);

// Returns the handle to use (the argument, or the calling thread's default
// handle on the current device); nullptr and an error set on failure.
uvatrmm_handle_t resolve(uvatrmm_handle_t h);

// Ensures workspace slot `slot` holds at least `bytes`; returns its pointer or nullptr.
void *workspace(uvatrmm_handle_t h, int slot, size_t bytes);

// Reads and clears the kernel status word (synchronising the stream).
int collect_status(uvatrmm_handle_t h);

inline int64_t round_up(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

}  // namespace uvt
