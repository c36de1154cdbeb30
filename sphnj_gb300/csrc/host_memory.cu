// Pinned, device-mapped host memory (sphnj_host_alloc / sphnj_host_free) and
// the registry of its ranges that the transfers consult.
//
// An allocation is made with cudaHostAllocMapped | cudaHostAllocPortable, so
// every device can address it; with unified addressing its device address is
// its host address (checked at allocation).  A transfer hands a host array to
// a kernel only when the whole array lies inside one registered allocation,
// so no kernel ever reads or writes past the memory the caller owns; any
// other pointer goes through the copy engines, which check it themselves.
#include "sphnj.h"
#include "kernels.h"

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <map>
#include <mutex>

namespace sphnj {

namespace {

std::mutex g_mutex;
std::map<uintptr_t, size_t> g_ranges;  // first byte -> size

}  // namespace

bool host_mapped(const void *ptr, size_t bytes) {
    if (!ptr || bytes == 0) return false;
    const uintptr_t a = reinterpret_cast<uintptr_t>(ptr);
    std::lock_guard<std::mutex> lock(g_mutex);
    auto it = g_ranges.upper_bound(a);
    if (it == g_ranges.begin()) return false;
    --it;
    const uintptr_t off = a - it->first;  // a >= it->first
    return off < it->second && bytes <= it->second - off;
}

}  // namespace sphnj

extern "C" {

int sphnj_host_alloc(uint64_t bytes, void **out) {
    if (!out) return SPHNJ_ERR_ARG;
    *out = nullptr;
    if (bytes == 0 || bytes > (uint64_t)SIZE_MAX) return SPHNJ_ERR_ARG;
    void *p = nullptr;
    if (cudaHostAlloc(&p, (size_t)bytes, cudaHostAllocMapped | cudaHostAllocPortable) != cudaSuccess) {
        cudaGetLastError();
        return SPHNJ_ERR_CUDA;
    }
    void *dev = nullptr;
    if (cudaHostGetDevicePointer(&dev, p, 0) != cudaSuccess || dev != p) {
        cudaGetLastError();
        cudaFreeHost(p);
        return SPHNJ_ERR_UNSUPPORTED;
    }
    std::memset(p, 0, (size_t)bytes);
    {
        std::lock_guard<std::mutex> lock(sphnj::g_mutex);
        sphnj::g_ranges[reinterpret_cast<uintptr_t>(p)] = (size_t)bytes;
    }
    *out = p;
    return SPHNJ_OK;
}

int sphnj_host_free(void *ptr) {
    if (!ptr) return SPHNJ_OK;
    {
        std::lock_guard<std::mutex> lock(sphnj::g_mutex);
        auto it = sphnj::g_ranges.find(reinterpret_cast<uintptr_t>(ptr));
        if (it == sphnj::g_ranges.end()) return SPHNJ_ERR_ARG;
        sphnj::g_ranges.erase(it);
    }
    return cudaFreeHost(ptr) == cudaSuccess ? SPHNJ_OK : SPHNJ_ERR_CUDA;
}

}  // extern "C"
