// Pieces of the MIC(0) wavefront (mic_wavefront.cu): the tile bookkeeping, the tagged tile-face
// exchange words, the cell-pair and quad types, and the host-side helpers of a sweep pair.
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"
#include "kernels.h"
#include "pcg.h"

namespace ffgpu {

constexpr long long WF_SPIN_LIMIT = 1 << 21;       // ~1-2 s of polling

// The four cells of a solver thread's 2 x 2 block, in memory order (x-pair index + 2 row).
template <typename T> struct alignas(4 * sizeof(T)) Quad { T v[4]; };

// Two adjacent cells of one row, moved as one 8- or 16-byte access.
template <typename T> struct Pair2;
template <> struct Pair2<float> { using type = float2; };
template <> struct Pair2<double> { using type = double2; };
template <typename T> __device__ inline typename Pair2<T>::type make_pair2(T a, T b) { return {a, b}; }

struct WfTiles {
    const int *done;            // PCG converged flag: the sweep is skipped when set (may be null)
    int A, B;                   // tiles along x, y
    int x0;                     // grid x of the tiles' low edge (even, at or below the box's)
    const short2 *order;        // tile coordinates in ticket order (diagonal-major)
    unsigned long long *xchg;   // face words: x faces [tile][diagonal][row], then y faces [tile][diagonal][col]
    unsigned int epoch;         // this sweep's tag (high half of every word it writes), set in the kernel
    unsigned int *epoch_ctr;    // device: the last sweep's tag; a sweep tags with the next value and its
                                // last CTA to leave stores it back (so captured sweeps replay with new tags)
    unsigned int *ticket;       // [0] tile ticket, [1] CTAs that have left; zero between sweeps
    unsigned int *error;
    long long spin_limit;       // polls before a face wait gives up
    double *dot_part;           // forward sweep with the dot: 4 q.q partials per tile (staging warps)
    PcgScalars *dot_sc;         // and the PCG scalars its last CTA updates (rho, or beta and rho)
    int dot_first;
};

__device__ inline unsigned long long ld_relaxed_u64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];\n" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ inline void st_relaxed_u64(unsigned long long *p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;\n" ::"l"(p), "l"(v) : "memory");
}

// One face value as WfWords<T>::N tagged words.
template <typename T> struct WfWords {
    static constexpr int N = sizeof(T) / 4;
    unsigned long long w[N];
};
template <typename T> __device__ inline void face_put(unsigned long long *p, T v, unsigned int epoch) {
    const unsigned long long tag = (unsigned long long)epoch << 32;
    if constexpr (sizeof(T) == 4) {
        st_relaxed_u64(p, tag | __float_as_uint(v));
    } else {
        const unsigned long long bits = (unsigned long long)__double_as_longlong(v);
        st_relaxed_u64(p, tag | (bits & 0xffffffffull));
        st_relaxed_u64(p + 1, tag | (bits >> 32));
    }
}
template <typename T> __device__ inline void face_load(WfWords<T> &f, const unsigned long long *p) {
#pragma unroll
    for (int h = 0; h < WfWords<T>::N; h++) f.w[h] = ld_relaxed_u64(p + h);
}
template <typename T> __device__ inline bool face_ready(const WfWords<T> &f, unsigned int epoch) {
    bool ok = true;
#pragma unroll
    for (int h = 0; h < WfWords<T>::N; h++) ok = ok && (unsigned int)(f.w[h] >> 32) == epoch;
    return ok;
}
template <typename T> __device__ inline T face_value(const WfWords<T> &f) {
    if constexpr (sizeof(T) == 4) return __uint_as_float((unsigned int)f.w[0]);
    else return __longlong_as_double((long long)((f.w[1] << 32) | (f.w[0] & 0xffffffffull)));
}
// Returns the face value once it carries this sweep's epoch; false on timeout or on an error
// raised elsewhere (the value is then meaningless).
template <typename T>
__device__ inline bool face_get(WfWords<T> &f, const unsigned long long *p, const WfTiles &w, T &v) {
    long long it = 0;
    while (!face_ready(f, w.epoch)) {
        face_load(f, p);
        if ((++it & 63) == 0) {
            if (it > w.spin_limit || *((volatile unsigned int *)w.error) != 0) {
                atomicOr(w.error, (unsigned int)ERR_WAIT_TIMEOUT);
                return false;
            }
            __nanosleep(64);
        }
    }
    v = face_value(f);
    return true;
}


// Host side of a sweep pair: the diagonal tile order table (uploaded when the tile grid changes)
// and the next sweep epoch (never 0; the exchange buffer and the device counter are cleared when the
// counter wraps).  The host count mirrors the device counter, which the sweeps advance themselves.
void wf_upload_order(const WfWork &ww, int A, int B, cudaStream_t st);
unsigned int wf_next_epoch(const WfWork &ww, cudaStream_t st);

}  // namespace ffgpu
