// Device buffer that grows on demand (cudaMalloc), freed with its owner.
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"

namespace ffgpu {

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
        FFGPU_CUDA(cudaMalloc(&p, count * sizeof(T)));
        n = count;
    }
    operator T *() const { return p; }
};

}  // namespace ffgpu
