// Allocation-free entry point: layered velocity extrapolation on caller-owned device
// buffers, with its scratch (two per-face status grids) in a fixed file-scope device array.
//
// It serves callers that must not allocate device memory while they run: hosts whose
// device memory is owned by another framework's pool (a renderer or game engine that hands
// out buffers and treats any cudaMalloc behind its back as a leak), and real-time loops that
// forbid allocator calls after set-up because an allocation can block for milliseconds.
// The array below is part of the library image: every GPU that loads the library holds
// it until the process exits.
#include <mutex>
#include <stdexcept>
#include <string>

#include "capi_internal.h"

namespace ffgpu {

// Largest grid (cells) the allocation-free extrapolation accepts: 4 Mi cells, e.g. a
// 161^3 face grid.  Scratch = two status bytes per cell = 8 MiB of device memory.
constexpr size_t NOALLOC_MAX_CELLS = (size_t)4 << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[2 * NOALLOC_MAX_CELLS];

// Device address of the scratch array, looked up once per device (host code cannot use
// the symbol itself: on the host it is only a stand-in, not a device address).  The cache
// lives as long as the process: after cudaDeviceReset the module may load elsewhere, so a
// caller that resets a device must not call this entry point on it again.
static unsigned char *scratch_for_current_device() {
    static std::mutex mu;
    static unsigned char *addr[64] = {nullptr};
    int dev = 0;
    FFGPU_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) throw std::runtime_error("Error: device index out of range.\n");
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess)
            throw std::runtime_error(std::string("Error: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e) + "\n");
        addr[dev] = static_cast<unsigned char *>(p);
    }
    return addr[dev];
}

}  // namespace ffgpu

using namespace ffgpu;

extern "C" {

void ffgpu_extrapolate_noalloc(int w, int h, int d, float *grid, const unsigned char *valid, int layers,
                               void *stream, int *err) {
    guarded(err, [&] {
        if (w < 1 || h < 1 || d < 1 || layers < 0) throw std::domain_error("Error: bad extrapolation arguments.\n");
        size_t n = (size_t)w * h * d;
        if (n > NOALLOC_MAX_CELLS)
            throw std::length_error("Error: ffgpu_extrapolate_noalloc accepts at most " +
                                    std::to_string(NOALLOC_MAX_CELLS) + " cells (got " + std::to_string(n) + ").\n");
        if (!grid || !valid) throw std::invalid_argument("Error: null device buffer.\n");
        // An error left by an earlier, unrelated CUDA call would otherwise be read back after
        // the launch below and reported as this call's failure: refuse to run and name it.
        const cudaError_t pending = cudaGetLastError();
        if (pending != cudaSuccess)
            throw std::runtime_error(std::string("Error: a CUDA error from an earlier call was pending (") +
                                     cudaGetErrorString(pending) + "); nothing was launched.\n");
        unsigned char *s = scratch_for_current_device();
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        // every status byte is written by the first kernel, so nothing needs clearing
        launch_extrapolate(w, h, d, grid, valid, layers, s, s + NOALLOC_MAX_CELLS, st);
        FFGPU_CUDA(cudaGetLastError());
    });
}

}  // extern "C"
