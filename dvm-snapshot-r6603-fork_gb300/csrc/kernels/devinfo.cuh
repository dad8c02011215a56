// Per-device facts the kernel launchers size their grids by, looked up once
// per device ordinal (a process may drive more than one GPU, one after the
// other, and GPUs of one machine need not have the same SM count).
#pragma once

#include <cuda_runtime.h>

#include <atomic>

namespace gbdev {

constexpr int MAX_DEVICES = 64;

// the current device's ordinal, or -1
inline int current() {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return -1;
    return dev;
}

// SM count of the current device (152 on GB300 if the query fails)
inline int smCount() {
    static std::atomic<int> cache[MAX_DEVICES];
    const int dev = current();
    if (dev < 0) return 152;
    int n = cache[dev].load(std::memory_order_relaxed);
    if (n <= 0) {
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
        cache[dev].store(n, std::memory_order_relaxed);
    }
    return n;
}

// CTAs of `kernel` (threads per CTA, dynamic shared memory) that are resident
// on one SM of the current device; the dynamic shared memory limit is raised
// first where it exceeds the default.  Cached per (device, cache) slot:
// one `cache` array per kernel/configuration.
template <typename K>
int residentCtas(std::atomic<int> (&cache)[MAX_DEVICES], K kernel, int threads, size_t smem) {
    const int dev = current();
    if (dev < 0) return 1;
    int occ = cache[dev].load(std::memory_order_relaxed);
    if (occ <= 0) {
        if (smem > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, threads, smem) != cudaSuccess || occ < 1)
            occ = 1;
        cache[dev].store(occ, std::memory_order_relaxed);
    }
    return occ;
}

}  // namespace gbdev
