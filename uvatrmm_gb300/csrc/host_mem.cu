// Page-locked host memory for the operands of the host entry points.
//
// On GB300 hosts (Arm, 64 KB base pages) a 2 GiB page-locked buffer from
// cudaHostAlloc copies at 10 ms when it was just used, but its first copy
// after a pause grows with the buffer's age (to 200+ ms for 2 GiB after a
// minute of alternating compute and copies), while a buffer backed by
// transparent huge pages copies at the same 10 ms throughout.  This
// allocator maps anonymous memory aligned to the huge-page size, asks for
// huge pages (MADV_HUGEPAGE), touches it and page-locks it with
// cudaHostRegister.  Where the kernel offers no huge pages the memory is
// still page-locked and usable.
//
// The host entry points copy operands in such memory directly; other host
// buffers (malloc'd, as the reference's, or page-locked elsewhere) are packed
// into two staging buffers of this kind by several CPU threads, each chunk's
// DMA overlapping the packing of the next (host_copy2d).
#include <sys/mman.h>
#include <unistd.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "api_internal.h"

namespace uvt {
namespace {

std::mutex g_host_mu;
std::map<void *, size_t> g_host_maps;  // base -> mapped length

// The transparent-huge-page size the kernel reports, else 2 MiB.
size_t huge_page_bytes() {
  static size_t hp = [] {
    size_t v = 0;
    if (FILE *f = fopen("/sys/kernel/mm/transparent_hugepage/hpage_pmd_size", "r")) {
      unsigned long long x = 0;
      if (fscanf(f, "%llu", &x) == 1) v = (size_t)x;
      fclose(f);
    }
    const size_t page = (size_t)sysconf(_SC_PAGESIZE);
    if (v < page || (v & (v - 1))) v = (size_t)2 << 20;
    return v;
  }();
  return hp;
}

// True when [p, p + bytes) lies inside one uvatrmm_host_alloc region.
bool in_host_alloc(const void *p, size_t bytes) {
  std::lock_guard<std::mutex> g(g_host_mu);
  auto it = g_host_maps.upper_bound(const_cast<void *>(p));
  if (it == g_host_maps.begin()) return false;
  --it;
  const uintptr_t base = reinterpret_cast<uintptr_t>(it->first), a = reinterpret_cast<uintptr_t>(p);
  return a >= base && a + bytes <= base + it->second;
}

int map_region(size_t bytes, void **out, size_t *len_out) {
  const size_t hp = huge_page_bytes();
  const size_t len = ((bytes ? bytes : 1) + hp - 1) / hp * hp;
  if (len < bytes) return fail(UVATRMM_EINVAL, "size overflows");
  // Over-map by one huge page and trim, so the region starts on a huge-page boundary.
  void *raw = mmap(nullptr, len + hp, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
  if (raw == MAP_FAILED) return fail(UVATRMM_ENOMEM, "mmap of " + std::to_string(len + hp) + " bytes failed");
  const uintptr_t a = reinterpret_cast<uintptr_t>(raw), b = (a + hp - 1) / hp * hp;
  if (b > a) munmap(raw, b - a);
  munmap(reinterpret_cast<void *>(b + len), a + hp - b);
  void *p = reinterpret_cast<void *>(b);
  madvise(p, len, MADV_HUGEPAGE);  // advisory: ignored where huge pages are off
  memset(p, 0, len);               // fault the pages in (as huge pages where granted)
  cudaError_t e = cudaHostRegister(p, len, cudaHostRegisterDefault);
  if (e != cudaSuccess) {
    munmap(p, len);
    return cuda_fail(e, "cudaHostRegister");
  }
  {
    std::lock_guard<std::mutex> g(g_host_mu);
    g_host_maps[p] = len;
  }
  *out = p;
  *len_out = len;
  return UVATRMM_OK;
}

// Copies `lines` lines of `width` bytes with up to 16 threads.
void par_copy(void *dst, size_t dpitch, const void *src, size_t spitch, size_t width, size_t lines) {
  char *d = static_cast<char *>(dst);
  const char *s = static_cast<const char *>(src);
  const size_t total = width * lines;
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t nt = std::min<size_t>({16, hw, std::max<size_t>(1, total >> 22)});  // >= 4 MiB per thread
  auto part = [&](size_t i) {
    if (dpitch == width && spitch == width) {
      const size_t b0 = total * i / nt, b1 = total * (i + 1) / nt;
      memcpy(d + b0, s + b0, b1 - b0);
    } else {
      for (size_t l = lines * i / nt, l1 = lines * (i + 1) / nt; l < l1; ++l)
        memcpy(d + l * dpitch, s + l * spitch, width);
    }
  };
  std::vector<std::thread> th;
  size_t started = 1;
  try {
    for (; started < nt; ++started) th.emplace_back(part, started);
  } catch (...) {  // no thread available: the caller copies the remaining parts
  }
  part(0);
  for (size_t i = started; i < nt; ++i) part(i);
  for (auto &t : th) t.join();
}

}  // namespace

bool host_alloc_contains(const void *p, size_t bytes) { return in_host_alloc(p, bytes); }

cudaError_t copy_triangle_h2d(uvatrmm_handle_t h, double *dA, int64_t la, const double *A, int64_t lda, int64_t ka,
                              bool lower) {
  for (int64_t j0 = 0; j0 < ka; j0 += kTriCopyCols) {
    const int64_t w = std::min<int64_t>(kTriCopyCols, ka - j0);
    const int64_t r0 = lower ? j0 : 0, r1 = lower ? ka : j0 + w;
    const cudaError_t e = host_copy2d(h, dA + r0 + j0 * la, (size_t)la * 8, A + r0 + j0 * lda, (size_t)lda * 8,
                                      (size_t)(r1 - r0) * 8, (size_t)w, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t host_copy2d(uvatrmm_handle_t h, void *dst, size_t dpitch, const void *src, size_t spitch, size_t width,
                        size_t height, cudaMemcpyKind kind) {
  if (width == 0 || height == 0) return cudaSuccess;
  const bool h2d = kind == cudaMemcpyHostToDevice;
  const void *host = h2d ? src : dst;
  const size_t hpitch = h2d ? spitch : dpitch;
  const size_t extent = hpitch * (height - 1) + width;
  const bool flat = dpitch == width && spitch == width;
  // Direct DMA: operands in uvatrmm_host_alloc memory, small copies, or lines
  // longer than a staging chunk.
  if (in_host_alloc(host, extent) || width * height < ((size_t)1 << 20) || (!flat && width > h->hstage_bytes)) {
    if (flat) return cudaMemcpyAsync(dst, src, width * height, kind, h->stream);
    return cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, height, kind, h->stream);
  }
  if (h->hstage_cap < h->hstage_bytes) {
    release_host_staging(h);
    size_t len = 0;
    for (int b = 0; b < 2; ++b) {
      if (map_region(h->hstage_bytes, &h->hstage[b], &len) != UVATRMM_OK) return cudaErrorMemoryAllocation;
      cudaError_t e = cudaEventCreateWithFlags(&h->hstage_ev[b], cudaEventDisableTiming);
      if (e != cudaSuccess) return e;
    }
    h->hstage_cap = h->hstage_bytes;
  }
  // A chunk is `lpc` lines (or, for a flat copy, `lpc` bytes of one line).
  const size_t unit = flat ? 1 : width, count = flat ? width * height : height;
  const size_t lpc = std::max<size_t>(1, h->hstage_bytes / unit);
  const size_t nchunk = (count + lpc - 1) / lpc;
  auto rows = [&](size_t k) { return std::min(lpc, count - k * lpc); };
  cudaError_t e = cudaSuccess;
  if (h2d) {
    const char *s = static_cast<const char *>(src);
    char *d = static_cast<char *>(dst);
    for (size_t k = 0; k < nchunk && e == cudaSuccess; ++k) {
      const int b = (int)(k & 1);
      e = cudaEventSynchronize(h->hstage_ev[b]);  // the DMA that last read this buffer
      if (e != cudaSuccess) break;
      const size_t n = rows(k);
      if (flat) {
        par_copy(h->hstage[b], n, s + k * lpc, n, n, 1);
        e = cudaMemcpyAsync(d + k * lpc, h->hstage[b], n, kind, h->stream);
      } else {
        par_copy(h->hstage[b], width, s + k * lpc * spitch, spitch, width, n);
        e = cudaMemcpy2DAsync(d + k * lpc * dpitch, dpitch, h->hstage[b], width, width, n, kind, h->stream);
      }
      if (e == cudaSuccess) e = cudaEventRecord(h->hstage_ev[b], h->stream);
    }
    return e;
  }
  const char *s = static_cast<const char *>(src);
  char *d = static_cast<char *>(dst);
  auto issue = [&](size_t k) {
    const int b = (int)(k & 1);
    const size_t n = rows(k);
    cudaError_t r = flat ? cudaMemcpyAsync(h->hstage[b], s + k * lpc, n, kind, h->stream)
                         : cudaMemcpy2DAsync(h->hstage[b], width, s + k * lpc * spitch, spitch, width, n, kind,
                                             h->stream);
    return r == cudaSuccess ? cudaEventRecord(h->hstage_ev[b], h->stream) : r;
  };
  e = issue(0);
  for (size_t k = 0; k < nchunk && e == cudaSuccess; ++k) {
    if (k + 1 < nchunk) e = issue(k + 1);  // into the buffer unpacked at step k - 1
    if (e == cudaSuccess) e = cudaEventSynchronize(h->hstage_ev[k & 1]);
    if (e != cudaSuccess) break;
    const size_t n = rows(k);
    if (flat) par_copy(d + k * lpc, n, h->hstage[k & 1], n, n, 1);
    else par_copy(d + k * lpc * dpitch, dpitch, h->hstage[k & 1], width, width, n);
  }
  return e;
}

void release_host_staging(uvatrmm_handle_t h) {
  for (int b = 0; b < 2; ++b) {
    if (h->hstage_ev[b]) {
      cudaEventSynchronize(h->hstage_ev[b]);
      cudaEventDestroy(h->hstage_ev[b]);
      h->hstage_ev[b] = nullptr;
    }
    if (h->hstage[b]) {
      uvatrmm_host_free(h->hstage[b]);
      h->hstage[b] = nullptr;
    }
  }
  h->hstage_cap = 0;
}

}  // namespace uvt

using namespace uvt;

extern "C" {

UVATRMM_API int uvatrmm_host_alloc(size_t bytes, void **ptr) {
  if (!ptr) return fail(UVATRMM_EINVAL, "ptr is NULL");
  *ptr = nullptr;
  size_t len = 0;
  const int rc = map_region(bytes, ptr, &len);
  return rc == UVATRMM_OK ? ok() : rc;
}

UVATRMM_API int uvatrmm_host_free(void *ptr) {
  if (!ptr) return ok();
  size_t len = 0;
  {
    std::lock_guard<std::mutex> g(g_host_mu);
    auto it = g_host_maps.find(ptr);
    if (it == g_host_maps.end()) return fail(UVATRMM_EINVAL, "pointer was not returned by uvatrmm_host_alloc");
    len = it->second;
    g_host_maps.erase(it);
  }
  cudaError_t e = cudaHostUnregister(ptr);
  munmap(ptr, len);
  return e == cudaSuccess ? ok() : cuda_fail(e, "cudaHostUnregister");
}

}  // extern "C"
