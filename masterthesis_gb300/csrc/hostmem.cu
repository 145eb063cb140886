// Pinned host memory backed by huge pages, for the host arrays of uploads
// and downloads.
//
// A copy engine that reads or writes pinned host memory translates its
// pages through the GPU's page tables.  With 64 KB base pages a 1 GiB
// field spans 16 384 pages; after a long solve the translations are no
// longer cached, and the first copy of such a buffer measured 45 - 160 ms
// on GB300 against 5.2 ms for the same copy with warm translations (the
// link rate).  Memory that the kernel backs with transparent huge pages
// (512 MB on a 64 KB-page kernel, 2 MB on a 4 KB-page one) needs a
// handful of translations per field and keeps the link rate after long
// solves.  scafes_host_alloc maps anonymous memory aligned to the huge
// page size, asks for huge pages (madvise), touches it and registers it
// with CUDA (page-locked, usable by cudaMemcpyAsync).
#include <cuda_runtime.h>
#include <sys/mman.h>
#include <unistd.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>

#include "../../include/scafes_gb300.h"

namespace scafes {
void set_last_error(const char* msg);
}

namespace {

struct Mapping {
    void* base;
    size_t length;
};

std::mutex g_mutex;
std::map<uintptr_t, Mapping> g_maps;  // user pointer -> its mapping

size_t huge_page_bytes() {
    size_t v = 0;
    if (FILE* f = std::fopen("/sys/kernel/mm/transparent_hugepage/hpage_pmd_size", "r")) {
        unsigned long long x = 0;
        if (std::fscanf(f, "%llu", &x) == 1) v = (size_t)x;
        std::fclose(f);
    }
    return v >= 4096 ? v : (size_t)2 << 20;
}

int reject(int code, const char* msg) {
    scafes::set_last_error(msg);
    return code;
}

}  // namespace

extern "C" int scafes_host_alloc(size_t bytes, void** out) {
    if (!out || bytes == 0) return reject(SCAFES_ERR_ARG, "scafes_host_alloc: bytes == 0 or out is NULL");
    *out = nullptr;
    const size_t hp = huge_page_bytes();
    const size_t len = (bytes + hp - 1) / hp * hp;
    const size_t map_len = len + hp;  // room to align the start to a huge page
    void* base = mmap(nullptr, map_len, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
    if (base == MAP_FAILED) return reject(SCAFES_ERR_NOMEM, "scafes_host_alloc: mmap failed");
    const uintptr_t start = ((uintptr_t)base + hp - 1) / hp * hp;
    void* p = reinterpret_cast<void*>(start);
#ifdef MADV_HUGEPAGE
    madvise(p, len, MADV_HUGEPAGE);  // advisory: without huge pages the memory still works
#endif
    std::memset(p, 0, len);          // fault the pages in before registering them
    if (cudaHostRegister(p, len, cudaHostRegisterDefault) != cudaSuccess) {
        munmap(base, map_len);
        cudaGetLastError();
        return reject(SCAFES_ERR_CUDA, "scafes_host_alloc: cudaHostRegister failed");
    }
    std::lock_guard<std::mutex> lock(g_mutex);
    g_maps[start] = Mapping{base, map_len};
    *out = p;
    return SCAFES_OK;
}

extern "C" void scafes_host_free(void* p) {
    if (!p) return;
    Mapping m{};
    {
        std::lock_guard<std::mutex> lock(g_mutex);
        const auto it = g_maps.find(reinterpret_cast<uintptr_t>(p));
        if (it == g_maps.end()) return;
        m = it->second;
        g_maps.erase(it);
    }
    cudaHostUnregister(p);
    munmap(m.base, m.length);
}
