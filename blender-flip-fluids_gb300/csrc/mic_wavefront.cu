// MIC(0) preconditioner application (pcgsolver.h:212-241) as a pipelined wavefront.
//
// The box of pressure cells is cut into tiles of TX x TY columns in the (x, y) plane; a
// thread owns one column and sweeps z.  Thread (tx, ty) processes plane z at step
// t = z + tx + ty, so the -x and -y neighbours of its cell were finished one step earlier
// by the neighbouring threads, which hand over their factor products L*q through shared
// memory (one barrier per step).  Every cell therefore performs exactly the reference's
// operations in the reference's order:
//   forward   q(c) = (((r(c) - Lz(c-z) q(c-z)) - Ly(c-y) q(c-y)) - Lx(c-x) q(c-x)) * inv(c)
//   backward  z(c) = (((q(c) - Lx(c) z(c+x)) - Ly(c) z(c+y)) - Lz(c) z(c+z)) * inv(c)
// which is the same as evaluating the i+j+k hyperplanes one after another.
//
// Tiles depend on their -x and -y neighbour tiles (+x/+y for the backward sweep).
// Persistent CTAs take tiles from an atomic ticket in diagonal order, so every tile a CTA
// waits for already belongs to a running CTA: progress is guaranteed whatever the number
// of resident CTAs.  A tile publishes how many planes it has finished (release store after
// a barrier and a fence); its successors poll that counter with acquire loads.  Every wait
// is bounded: on timeout the kernel raises ERR_WAIT_TIMEOUT in the error word and the CTA
// abandons its tiles, so the launch always terminates and the host reports the failure.
#include <cuda/atomic>

#include <algorithm>
#include <stdexcept>
#include <vector>

#include "common.cuh"
#include "kernels.h"
#include "pcg.h"

namespace ffgpu {

constexpr int WF_TX = 16, WF_TY = 16;
constexpr int WF_PUBLISH = 4;             // publish progress every 4 steps
constexpr long long WF_SPIN_LIMIT = 1 << 21;   // ~1-2 s of polling

struct WfTiles {
    const int *done;       // PCG converged flag: the sweep is skipped when set (may be null)
    int A, B;              // tiles along x, y
    const short2 *order;   // tile coordinates in ticket order (diagonal-major)
    int *progress;         // planes finished per tile (indexed a + A*b)
    unsigned int *ticket;
    unsigned int *error;
};

__device__ inline int ld_acquire(const int *p) {
    cuda::atomic_ref<const int, cuda::thread_scope_device> r(*p);
    return r.load(cuda::memory_order_acquire);
}
__device__ inline void st_release(int *p, int v) {
    cuda::atomic_ref<int, cuda::thread_scope_device> r(*p);
    r.store(v, cuda::memory_order_release);
}

// Waits until progress[tile] >= need; returns false on timeout (error raised).
__device__ inline bool wait_progress(const WfTiles &w, int tile, int need, int &cached) {
    if (cached >= need) return true;
    long long it = 0;
    int v = ld_acquire(w.progress + tile);
    while (v < need) {
        if (++it > WF_SPIN_LIMIT || *((volatile unsigned int *)w.error) != 0) {
            atomicOr(w.error, (unsigned int)ERR_WAIT_TIMEOUT);
            return false;
        }
        __nanosleep(32);
        v = ld_acquire(w.progress + tile);
    }
    cached = v;
    return true;
}

template <typename T, bool FORWARD>
__global__ void __launch_bounds__(WF_TX *WF_TY) k_mic_wavefront(Dims d, Bbox bb, FactorView<T> F,
                                                                const T *__restrict__ rin, T *q, WfTiles w) {
    __shared__ T sx[2][WF_TY][WF_TX];
    __shared__ T sy[2][WF_TY][WF_TX];
    __shared__ int s_tile, s_abort;
    __shared__ int s_cx, s_cy;
    const int tx = threadIdx.x % WF_TX, ty = threadIdx.x / WF_TX;
    const int I = bb.i1 - bb.i0 + 1, J = bb.j1 - bb.j0 + 1, K = bb.k1 - bb.k0 + 1;
    const size_t sl = (size_t)d.ni * d.nj;
    const int ntiles = w.A * w.B;
    const int steps = K + WF_TX + WF_TY - 2;
    if (w.done && *w.done) return;
    for (;;) {
        if (threadIdx.x == 0) {
            unsigned int tk = atomicAdd(w.ticket, 1u);
            s_tile = (int)tk;
            s_abort = 0;
            s_cx = s_cy = -1;
        }
        __syncthreads();
        const int tk = s_tile;
        if (tk >= ntiles) return;
        const short2 ab = w.order[FORWARD ? tk : ntiles - 1 - tk];
        const int a = ab.x, b = ab.y;
        const int tile = a + w.A * b;
        // upstream tiles: -x/-y (forward) or +x/+y (backward)
        const int upx = FORWARD ? (a > 0 ? tile - 1 : -1) : (a < w.A - 1 ? tile + 1 : -1);
        const int upy = FORWARD ? (b > 0 ? tile - w.A : -1) : (b < w.B - 1 ? tile + w.A : -1);
        // this thread's column (local position mirrored for the backward sweep)
        const int lx_ = FORWARD ? tx : WF_TX - 1 - tx;
        const int ly_ = FORWARD ? ty : WF_TY - 1 - ty;
        const int xi = a * WF_TX + lx_, yj = b * WF_TY + ly_;
        const bool col = xi < I && yj < J;
        const int i = bb.i0 + xi, j = bb.j0 + yj;
        T carry = T(0);   // product handed along z by this thread
        for (int t = 0; t < steps; t++) {
            if (threadIdx.x == 0) {
                int need = min(t + 1, K);
                int cx = s_cx, cy = s_cy;
                bool ok = true;
                if (upx >= 0) ok = wait_progress(w, upx, need, cx);
                if (ok && upy >= 0) ok = wait_progress(w, upy, need, cy);
                s_cx = cx; s_cy = cy;
                if (!ok) s_abort = 1;
            }
            __syncthreads();
            if (s_abort) break;
            const int s = t - tx - ty;          // planes done before this thread's current one
            if (col && s >= 0 && s < K) {
                const int kk = FORWARD ? s : K - 1 - s;
                const int k = bb.k0 + kk;
                const size_t c = flat3(i, j, k, d.ni, d.nj);
                T v = FORWARD ? rin[c] : q[c];
                if (FORWARD) {
                    if (s > 0) v -= carry;                                        // Lz(c-z) q(c-z)
                    if (ty > 0) v -= sy[(t - 1) & 1][ty - 1][tx];                 // Ly(c-y) q(c-y)
                    else if (yj > 0) v -= __ldcg(F.ly + c - d.ni) * __ldcg(q + c - d.ni);
                    if (tx > 0) v -= sx[(t - 1) & 1][ty][tx - 1];                 // Lx(c-x) q(c-x)
                    else if (xi > 0) v -= __ldcg(F.lx + c - 1) * __ldcg(q + c - 1);
                    const T qv = v * F.inv[c];
                    q[c] = qv;
                    sx[t & 1][ty][tx] = F.lx[c] * qv;
                    sy[t & 1][ty][tx] = F.ly[c] * qv;
                    carry = F.lz[c] * qv;
                } else {
                    const T Lx = F.lx[c], Ly = F.ly[c], Lz = F.lz[c];
                    if (tx > 0) v -= Lx * sx[(t - 1) & 1][ty][tx - 1];            // Lx(c) z(c+x)
                    else if (xi < I - 1) v -= Lx * __ldcg(q + c + 1);
                    if (ty > 0) v -= Ly * sy[(t - 1) & 1][ty - 1][tx];            // Ly(c) z(c+y)
                    else if (yj < J - 1) v -= Ly * __ldcg(q + c + d.ni);
                    if (s > 0) v -= Lz * carry;                                   // Lz(c) z(c+z)
                    const T zv = v * F.inv[c];
                    q[c] = zv;
                    sx[t & 1][ty][tx] = zv;
                    sy[t & 1][ty][tx] = zv;
                    carry = zv;
                }
            }
            // publish: planes finished by every thread of the tile
            const int done = t - (WF_TX - 1) - (WF_TY - 1) + 1;
            if (done > 0 && (done % WF_PUBLISH == 0 || done >= K || t == steps - 1)) {
                __syncthreads();
                if (threadIdx.x == 0) {
                    __threadfence();
                    st_release(w.progress + tile, min(done, K));
                }
            }
        }
        __syncthreads();
        if (s_abort) return;
    }
}

template <typename T>
void mic_wavefront(Dims d, Bbox bb, FactorView<T> F, const T *r, T *z, WfWork ww, cudaStream_t st) {
    const int I = bb.i1 - bb.i0 + 1, J = bb.j1 - bb.j0 + 1;
    WfTiles w;
    w.A = (I + WF_TX - 1) / WF_TX;
    w.B = (J + WF_TY - 1) / WF_TY;
    const int nt = w.A * w.B;
    if (nt > ww.max_tiles) throw std::runtime_error("Error: wavefront tile table too small.\n");
    w.order = ww.order; w.progress = ww.progress; w.ticket = ww.ticket; w.error = ww.error;
    w.done = ww.done;
    // tile order (diagonal-major), uploaded once per box shape
    if (*ww.order_key != ((long long)w.A << 32 | w.B)) {
        std::vector<short2> ord;
        ord.reserve(nt);
        for (int dg = 0; dg <= w.A + w.B - 2; dg++)
            for (int a = 0; a < w.A; a++) {
                int b = dg - a;
                if (b >= 0 && b < w.B) ord.push_back(make_short2((short)a, (short)b));
            }
        FFGPU_CUDA(cudaMemcpyAsync(ww.order, ord.data(), nt * sizeof(short2), cudaMemcpyHostToDevice, st));
        FFGPU_CUDA(cudaStreamSynchronize(st));
        *ww.order_key = ((long long)w.A << 32 | w.B);
    }
    int grid = std::min(nt, ww.resident_ctas);
    // forward sweep: r -> z, then backward sweep in place on z
    FFGPU_CUDA(cudaMemsetAsync(ww.progress, 0, nt * sizeof(int), st));
    FFGPU_CUDA(cudaMemsetAsync(ww.ticket, 0, sizeof(unsigned int), st));
    k_mic_wavefront<T, true><<<grid, WF_TX * WF_TY, 0, st>>>(d, bb, F, r, z, w);
    FFGPU_CUDA(cudaMemsetAsync(ww.progress, 0, nt * sizeof(int), st));
    FFGPU_CUDA(cudaMemsetAsync(ww.ticket, 0, sizeof(unsigned int), st));
    k_mic_wavefront<T, false><<<grid, WF_TX * WF_TY, 0, st>>>(d, bb, F, r, z, w);
}

int mic_wavefront_resident_ctas() {
    int dev = 0, sms = 0, per = 0;
    FFGPU_CUDA(cudaGetDevice(&dev));
    FFGPU_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    FFGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_mic_wavefront<double, true>, WF_TX * WF_TY, 0));
    return std::max(1, sms * std::max(per, 1));
}

template void mic_wavefront<double>(Dims, Bbox, FactorView<double>, const double *, double *, WfWork, cudaStream_t);
template void mic_wavefront<float>(Dims, Bbox, FactorView<float>, const float *, float *, WfWork, cudaStream_t);

}  // namespace ffgpu
