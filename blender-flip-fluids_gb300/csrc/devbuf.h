// Device buffer that grows on demand (cudaMalloc), freed with its owner.
#pragma once
#include <cuda_runtime.h>

#include <atomic>

#include "common.cuh"

namespace ffgpu {

// Failure injection for the allocation path: when positive, the countdown-th next device
// allocation fails as if the device were out of memory (one shot).
inline std::atomic<long long> g_alloc_fail_countdown{0};

template <typename T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    // grows (never shrinks); contents are not preserved
    void reserve(size_t count) {
        if (count <= n) return;
        release();
        if (g_alloc_fail_countdown.load() > 0 && --g_alloc_fail_countdown == 0)
            throw std::runtime_error("Error: device allocation of " + std::to_string(count * sizeof(T)) +
                                     " bytes failed (injected).\n");
        FFGPU_CUDA(cudaMalloc(&p, count * sizeof(T)));
        n = count;
    }
    operator T *() const { return p; }
};

}  // namespace ffgpu
