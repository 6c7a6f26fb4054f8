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
#include <sys/mman.h>
#include <unistd.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>

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

}  // namespace
}  // namespace uvt

using namespace uvt;

extern "C" {

UVATRMM_API int uvatrmm_host_alloc(size_t bytes, void **ptr) {
  if (!ptr) return fail(UVATRMM_EINVAL, "ptr is NULL");
  *ptr = nullptr;
  const size_t hp = huge_page_bytes();
  const size_t len = ((bytes ? bytes : 1) + hp - 1) / hp * hp;
  if (len < bytes) return fail(UVATRMM_EINVAL, "size overflows");
  // Over-map by one huge page and trim, so the region starts on a huge-page boundary.
  void *raw = mmap(nullptr, len + hp, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
  if (raw == MAP_FAILED) return fail(UVATRMM_ENOMEM, "mmap of " + std::to_string(len + hp) + " bytes failed");
  const uintptr_t a = reinterpret_cast<uintptr_t>(raw), b = (a + hp - 1) / hp * hp;
  if (b > a) munmap(raw, b - a);
  if (b + len < a + len + hp) munmap(reinterpret_cast<void *>(b + len), a + len + hp - (b + len));
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
  *ptr = p;
  return ok();
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
