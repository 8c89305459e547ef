// Shared device/host helpers for the GB300 FLIP substep library.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>
#include <stdexcept>
#include <string>

namespace ffgpu {

#define FFGPU_CUDA(call)                                                                   \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess)                                                             \
            throw std::runtime_error(std::string("CUDA error: ") + cudaGetErrorString(e_) + \
                                     " at " __FILE__ ":" + std::to_string(__LINE__));     \
    } while (0)

// Error-word bits a kernel may raise (read by the host after the stage that can set them).
enum ErrorBits : unsigned int {
    ERR_NONE = 0,
    ERR_WAIT_TIMEOUT = 1u << 0,      // a bounded spin-wait gave up
    ERR_INDEX = 1u << 1,             // an index check failed (access skipped)
    ERR_NONFINITE = 1u << 2,         // NaN/Inf met where finite values are required
    ERR_CAPACITY = 1u << 3,          // a fixed-capacity buffer would overflow
};

struct Dims {
    int ni, nj, nk;
    __host__ __device__ size_t cells() const { return (size_t)ni * nj * nk; }
    __host__ __device__ size_t faces(int c) const {
        return (size_t)(ni + (c == 0)) * (nj + (c == 1)) * (nk + (c == 2));
    }
};

__host__ __device__ inline size_t flat3(int i, int j, int k, int w, int h) {
    return (size_t)i + (size_t)w * ((size_t)j + (size_t)h * (size_t)k);
}

// Order-preserving float <-> int mapping for integer atomicMin on floats.
__device__ inline int float_to_ordered(float f) {
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
__device__ inline float ordered_to_float(int i) {
    return __int_as_float(i >= 0 ? i : i ^ 0x7FFFFFFF);
}

inline unsigned int ceil_div(size_t a, size_t b) { return (unsigned int)((a + b - 1) / b); }

// Division by a launch-constant divisor d >= 1 for numerators n < 2^31 (Granlund and
// Montgomery, "Division by invariant integers using multiplication", 1994): with
// l = ceil(log2 d) and m = ceil(2^(31+l) / d) <= 2^32, n / d = (n m) >> (31 + l) exactly.
struct FastDiv {
    unsigned long long m;
    int s;
    __device__ unsigned int div(unsigned int n) const { return (unsigned int)(((unsigned long long)n * m) >> s); }
};
inline FastDiv fastdiv(unsigned int d) {
    int l = 0;
    while ((1ull << l) < d) l++;
    return FastDiv{((1ull << (31 + l)) + d - 1) / d, 31 + l};
}

// (i, j, k) of a linear x-fastest index t < 2^31 into a w x h x d grid.
struct GridDecode {
    FastDiv dw, dh;
    unsigned int w, h;
    __device__ void operator()(unsigned int t, int &i, int &j, int &k) const {
        const unsigned int r = dw.div(t), kk = dh.div(r);
        i = (int)(t - r * w);
        j = (int)(r - kk * h);
        k = (int)kk;
    }
};
inline GridDecode grid_decode(int w, int h, int d) {
    if ((unsigned long long)w * h * d >= (1ull << 31)) throw std::runtime_error("Error: grid exceeds 2^31 entries.\n");
    return GridDecode{fastdiv((unsigned int)w), fastdiv((unsigned int)h), (unsigned int)w, (unsigned int)h};
}

// Sized grid for a 1-D launch: at most `cap` blocks (grid-stride loops cover the rest).
inline unsigned int grid_for(size_t n, int block, unsigned int cap = 152u * 16u) {
    size_t g = (n + block - 1) / block;
    if (g < 1) g = 1;
    return (unsigned int)(g < cap ? g : cap);
}

// Deterministic block reduction of doubles (fixed tree order, warp shuffles then smem).
template <int BLOCK>
__device__ inline double block_sum(double v, double *smem) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) smem[wid] = v;
    __syncthreads();
    double r = 0.0;
    if (wid == 0) {
        r = lane < BLOCK / 32 ? smem[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
    }
    __syncthreads();
    return r;   // valid in thread 0
}

template <int BLOCK>
__device__ inline double block_max(double v, double *smem) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) smem[wid] = v;
    __syncthreads();
    double r = 0.0;
    if (wid == 0) {
        r = lane < BLOCK / 32 ? smem[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) r = fmax(r, __shfl_down_sync(0xffffffffu, r, o));
    }
    __syncthreads();
    return r;
}

// floor((double)v * D) as the reference evaluates it, for a float v and a double D.  The float
// product p carries a relative error below 2^-23 against the double one, so when p lies farther
// than twice that from every integer both floors agree; otherwise (or for huge p) the double
// product is formed.
static __device__ __noinline__ int floor_fd_exact(float v, double D) { return (int)floor((double)v * D); }
static __device__ inline int floor_fd(float v, double D, float Df) {
    const float p = v * Df;
    const float fp = floorf(p);
    const float m = fabsf(p) * 2.5e-7f;
    // a real branch (the exact path is not inlined), so the double product is formed only when needed
    if (fabsf(p) < 4.0e6f && p - fp > m && (fp + 1.0f) - p > m) return (int)fp;
    return floor_fd_exact(v, D);
}

}  // namespace ffgpu
