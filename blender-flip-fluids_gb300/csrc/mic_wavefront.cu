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
// Memory access.  Because of the skew, the 32 lanes of a warp work on different z planes
// at any step, so loading each lane's operands directly would touch 32 cache lines per
// instruction.  Instead a warp copies whole planes of its own columns (coalesced rows of TX
// cells) with cp.async a few steps before its first lane needs them, into per-lane delay
// lines in shared memory; results go to a second delay line and are written back one full
// plane at a time.  Each lane only ever reads back its own slots, so the delay lines need
// no barrier.  Results on the tile's downstream faces (last row and column) are also
// stored at once, because the next tiles read them.
//
// Tiles depend on their -x and -y neighbour tiles (+x/+y for the backward sweep).  The values
// that cross a tile face (forward: the products Lx*q, Ly*q; backward: z) are passed through an
// exchange buffer, one 64-bit word per value and plane, whose high half holds the epoch of the
// sweep that wrote it (FP64 values take two words, one per half).  Value and epoch land in one
// single-copy-atomic store, so the consumer needs no fence: it loads the word a few steps ahead
// and, if the epoch is not yet the current one, polls until it is.
// Persistent CTAs take tiles from an atomic ticket in diagonal order, so every tile a CTA
// waits for already belongs to a running CTA: progress is guaranteed whatever the number
// of resident CTAs.  Every wait is bounded: on timeout the kernel raises ERR_WAIT_TIMEOUT in
// the error word (which also releases every other waiter), the CTA drains its copies and
// abandons its tiles, so the launch always terminates and the host reports the failure.
#include <cuda/atomic>

#include <algorithm>
#include <atomic>
#include <stdexcept>
#include <vector>

#include "common.cuh"
#include "kernels.h"
#include "pcg.h"

namespace ffgpu {

constexpr int WF_TX = 16;                          // tile width (x); a warp covers 32 / WF_TX rows
constexpr int WF_RPW = 32 / WF_TX;                 // rows per warp
constexpr int WF_DIN = 3;                          // own operands are copied this many steps ahead
constexpr int WF_RIN = WF_DIN + WF_TX + WF_RPW - 1;   // input delay line depth (planes)
constexpr int WF_ROUT = WF_TX + WF_RPW - 1;        // output delay line depth (planes)
constexpr int WF_DE = 4;                           // tile-face words are loaded this many steps ahead
constexpr long long WF_SPIN_LIMIT = 1 << 21;       // ~1-2 s of polling

// Tile height: 16 rows for FP32, 8 for FP64 (the delay lines then take the same 121 KB).
template <typename T> constexpr int wf_ty() { return sizeof(T) == 4 ? 16 : 8; }

template <typename T, int TY> struct WfSmem {
    T in[WF_RIN][5][WF_TX * TY];   // [plane slot][r-or-q, inv, lx, ly, lz][thread]
    T out[WF_ROUT][WF_TX * TY];    // [plane slot][thread]
    T sx[2][TY][WF_TX];            // hand-over to the +x neighbour thread
    T sy[2][TY][WF_TX];            // hand-over to the +y neighbour thread
};

struct WfTiles {
    const int *done;            // PCG converged flag: the sweep is skipped when set (may be null)
    int A, B;                   // tiles along x, y
    const short2 *order;        // tile coordinates in ticket order (diagonal-major)
    unsigned long long *xchg;   // face words: x faces [tile][row][plane], then y faces [tile][col][plane]
    unsigned int epoch;         // this sweep's tag (high half of every word it writes)
    unsigned int *ticket;
    unsigned int *error;
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
        if (++it > WF_SPIN_LIMIT || *((volatile unsigned int *)w.error) != 0) {
            atomicOr(w.error, (unsigned int)ERR_WAIT_TIMEOUT);
            return false;
        }
        if (it > 32) __nanosleep(64);
        face_load(f, p);
    }
    v = face_value(f);
    return true;
}

template <typename T> __device__ inline void cp_async_elem(T *dst, const T *src) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
    if constexpr (sizeof(T) == 4)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(src) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(src) : "memory");
}
__device__ inline void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ inline void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }
__device__ inline void cp_async_drain() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

template <typename T, bool FORWARD, int TY>
__global__ void __launch_bounds__(WF_TX *TY) k_mic_wavefront(Dims d, Bbox bb, FactorView<T> F,
                                                             const T *__restrict__ rin, T *q, WfTiles w) {
    extern __shared__ __align__(16) unsigned char wf_smem_raw[];
    WfSmem<T, TY> &S = *reinterpret_cast<WfSmem<T, TY> *>(wf_smem_raw);
    constexpr int NW = WfWords<T>::N;
    __shared__ int s_tile;
    __shared__ int s_abort[2];   // set during step t into slot (t + 1) & 1, read after the barrier of step t + 1
    const int tid = threadIdx.x;
    const int tx = tid % WF_TX, ty = tid / WF_TX;
    const int wrow = (tid / 32) * WF_RPW;   // first tile row of this thread's warp
    const int I = bb.i1 - bb.i0 + 1, J = bb.j1 - bb.j0 + 1, K = bb.k1 - bb.k0 + 1;
    const int ntiles = w.A * w.B;
    const int steps = K + WF_TX + TY - 2;
    const size_t yface0 = (size_t)ntiles * TY * K;   // first y-face word index (in values)
    if (w.done && *w.done) return;
    for (;;) {
        if (tid == 0) {
            unsigned int tk = atomicAdd(w.ticket, 1u);
            s_tile = (int)tk;
            s_abort[0] = s_abort[1] = 0;
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
        const int ly_ = FORWARD ? ty : TY - 1 - ty;
        const int xi = a * WF_TX + lx_, yj = b * TY + ly_;
        const bool col = xi < I && yj < J;
        const int i = bb.i0 + xi, j = bb.j0 + yj;
        // values crossing the tile faces: consumed from the upstream tiles, produced for the downstream ones
        const bool hasx = col && tx == 0 && (FORWARD ? xi > 0 : xi < I - 1);
        const bool hasy = col && ty == 0 && (FORWARD ? yj > 0 : yj < J - 1);
        const bool putx = col && tx == WF_TX - 1 && (FORWARD ? xi < I - 1 : xi > 0);
        const bool puty = col && ty == TY - 1 && (FORWARD ? yj < J - 1 : yj > 0);
        const unsigned long long *gx = w.xchg + NW * (((size_t)(upx < 0 ? 0 : upx) * TY + ty) * K);
        const unsigned long long *gy = w.xchg + NW * (yface0 + ((size_t)(upy < 0 ? 0 : upy) * WF_TX + tx) * K);
        unsigned long long *px = w.xchg + NW * (((size_t)tile * TY + ty) * K);
        unsigned long long *py = w.xchg + NW * (yface0 + ((size_t)tile * WF_TX + tx) * K);
        auto cell = [&](int s) {
            return flat3(i, j, bb.k0 + (FORWARD ? s : K - 1 - s), d.ni, d.nj);
        };
        // the warp copies plane p of its columns into the input delay line (one group per call)
        auto stage = [&](int p) {
            if (col && p >= 0 && p < K) {
                const size_t c = cell(p);
                const int sl = p % WF_RIN;
                cp_async_elem(&S.in[sl][0][tid], (FORWARD ? rin : (const T *)q) + c);
                cp_async_elem(&S.in[sl][1][tid], F.inv + c);
                cp_async_elem(&S.in[sl][2][tid], F.lx + c);
                cp_async_elem(&S.in[sl][3][tid], F.ly + c);
                cp_async_elem(&S.in[sl][4][tid], F.lz + c);
            }
            cp_async_commit();
        };
        // face words of step tt (plane tt - tx - ty), loaded ahead; checked when used
        auto fetch_face = [&](WfWords<T> &fx, WfWords<T> &fy, int tt) {
            const int s = tt - tx - ty;
            if (s < 0 || s >= K) return;
            if (hasx) face_load(fx, gx + (size_t)NW * s);
            if (hasy) face_load(fy, gy + (size_t)NW * s);
        };

        for (int t = -WF_DIN; t < 0; t++) stage(t - wrow + WF_DIN);
        WfWords<T> fx[WF_DE] = {}, fy[WF_DE] = {};
#pragma unroll
        for (int u = 0; u < WF_DE; u++) fetch_face(fx[u], fy[u], u);
        T carry = T(0);   // product handed along z by this thread
        bool abort = false;
        for (int t0 = 0; t0 < steps && !abort; t0 += WF_DE) {
#pragma unroll
            for (int u = 0; u < WF_DE; u++) {
                const int t = t0 + u;
                if (t >= steps) break;
                cp_async_wait<WF_DIN - 1>();   // this lane's operands of step t have landed
                __syncthreads();   // step t-1 finished everywhere; its hand-over values are in shared memory
                if (s_abort[t & 1]) { abort = true; break; }
                const int s = t - tx - ty;
                if (col && s >= 0 && s < K) {
                    const int sl = s % WF_RIN;
                    const T in = S.in[sl][0][tid], inv = S.in[sl][1][tid];
                    const T Lx = S.in[sl][2][tid], Ly = S.in[sl][3][tid], Lz = S.in[sl][4][tid];
                    T ex = T(0), ey = T(0);
                    bool ok = true;
                    if (hasx) ok = face_get(fx[u], gx + (size_t)NW * s, w, ex);
                    if (ok && hasy) ok = face_get(fy[u], gy + (size_t)NW * s, w, ey);
                    if (!ok) s_abort[(t + 1) & 1] = 1;
                    T v = in, res;
                    if (FORWARD) {
                        if (s > 0) v -= carry;                                  // Lz(c-z) q(c-z)
                        if (ty > 0) v -= S.sy[(t - 1) & 1][ty - 1][tx];         // Ly(c-y) q(c-y)
                        else if (hasy) v -= ey;
                        if (tx > 0) v -= S.sx[(t - 1) & 1][ty][tx - 1];         // Lx(c-x) q(c-x)
                        else if (hasx) v -= ex;
                        res = v * inv;
                        const T hx = Lx * res, hy = Ly * res;
                        S.sx[t & 1][ty][tx] = hx;
                        S.sy[t & 1][ty][tx] = hy;
                        if (putx) face_put(px + (size_t)NW * s, hx, w.epoch);
                        if (puty) face_put(py + (size_t)NW * s, hy, w.epoch);
                        carry = Lz * res;
                    } else {
                        if (tx > 0) v -= Lx * S.sx[(t - 1) & 1][ty][tx - 1];    // Lx(c) z(c+x)
                        else if (hasx) v -= Lx * ex;
                        if (ty > 0) v -= Ly * S.sy[(t - 1) & 1][ty - 1][tx];    // Ly(c) z(c+y)
                        else if (hasy) v -= Ly * ey;
                        if (s > 0) v -= Lz * carry;                             // Lz(c) z(c+z)
                        res = v * inv;
                        S.sx[t & 1][ty][tx] = res;
                        S.sy[t & 1][ty][tx] = res;
                        if (putx) face_put(px + (size_t)NW * s, res, w.epoch);
                        if (puty) face_put(py + (size_t)NW * s, res, w.epoch);
                        carry = res;
                    }
                    S.out[s % WF_ROUT][tid] = res;
                }
                stage(t - wrow + WF_DIN);
                // every lane of the warp has finished plane po: write it back as whole rows
                const int po = t - (WF_TX + WF_RPW - 2) - wrow;
                if (col && po >= 0 && po < K) q[cell(po)] = S.out[po % WF_ROUT][tid];
                if (t + WF_DE < steps) fetch_face(fx[u], fy[u], t + WF_DE);
            }
        }
        cp_async_drain();
        if (abort) return;   // every thread saw the same flag after the same barrier
        __syncthreads();     // a timeout in the last step is seen here
        if (s_abort[steps & 1]) return;
    }
}

template <typename T>
static int wf_setup(size_t smem) {   // per device: opt in to the shared memory, count resident CTAs
    constexpr int TY = wf_ty<T>();
    static std::atomic<int> cached[64];
    int dev = 0;
    FFGPU_CUDA(cudaGetDevice(&dev));
    if (dev < 64 && cached[dev].load() > 0) return cached[dev].load();
    FFGPU_CUDA(cudaFuncSetAttribute(k_mic_wavefront<T, true, TY>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    FFGPU_CUDA(cudaFuncSetAttribute(k_mic_wavefront<T, false, TY>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int sms = 0, per = 0;
    FFGPU_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    FFGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_mic_wavefront<T, true, TY>, WF_TX * TY, smem));
    const int r = std::max(1, sms * std::max(per, 1));
    if (dev < 64) cached[dev].store(r);
    return r;
}

int mic_wavefront_max_tiles(int I, int J) {
    return ((I + WF_TX - 1) / WF_TX) * ((J + wf_ty<double>() - 1) / wf_ty<double>());
}

template <typename T> static size_t xchg_words_for(int I, int J, int K) {
    constexpr int TY = wf_ty<T>();
    const size_t tiles = (size_t)((I + WF_TX - 1) / WF_TX) * ((J + TY - 1) / TY);
    return WfWords<T>::N * tiles * (WF_TX + TY) * (size_t)K;
}

size_t mic_wavefront_xchg_words(int I, int J, int K) {
    return std::max(xchg_words_for<float>(I, J, K), xchg_words_for<double>(I, J, K));
}

template <typename T>
void mic_wavefront(Dims d, Bbox bb, FactorView<T> F, const T *r, T *z, WfWork ww, cudaStream_t st) {
    constexpr int TY = wf_ty<T>();
    const size_t smem = sizeof(WfSmem<T, TY>);
    const int resident = wf_setup<T>(smem);
    const int I = bb.i1 - bb.i0 + 1, J = bb.j1 - bb.j0 + 1;
    WfTiles w;
    w.A = (I + WF_TX - 1) / WF_TX;
    w.B = (J + TY - 1) / TY;
    const int nt = w.A * w.B;
    if (nt > ww.max_tiles) throw std::runtime_error("Error: wavefront tile table too small.\n");
    const int K = bb.k1 - bb.k0 + 1;
    if (xchg_words_for<T>(I, J, K) > ww.xchg_words)
        throw std::runtime_error("Error: wavefront exchange buffer too small.\n");
    w.order = ww.order; w.xchg = ww.xchg; w.ticket = ww.ticket; w.error = ww.error;
    w.done = ww.done;
    // tile order (diagonal-major), uploaded once per tile-grid shape
    const long long key = (long long)w.A << 32 | w.B;
    if (*ww.order_key != key) {
        std::vector<short2> ord;
        ord.reserve(nt);
        for (int dg = 0; dg <= w.A + w.B - 2; dg++)
            for (int a = 0; a < w.A; a++) {
                int b = dg - a;
                if (b >= 0 && b < w.B) ord.push_back(make_short2((short)a, (short)b));
            }
        FFGPU_CUDA(cudaMemcpyAsync(ww.order, ord.data(), nt * sizeof(short2), cudaMemcpyHostToDevice, st));
        FFGPU_CUDA(cudaStreamSynchronize(st));
        *ww.order_key = key;
    }
    const int grid = std::min(nt, resident);
    // every sweep tags its face words with a new epoch; words left by earlier sweeps never match
    auto next_epoch = [&] {
        if (++*ww.epoch == 0) {   // wrapped: clear the buffer so no stale word carries a reused tag
            FFGPU_CUDA(cudaMemsetAsync(ww.xchg, 0, ww.xchg_words * sizeof(unsigned long long), st));
            *ww.epoch = 1;
        }
        return *ww.epoch;
    };
    // forward sweep: r -> z, then backward sweep in place on z
    w.epoch = next_epoch();
    FFGPU_CUDA(cudaMemsetAsync(ww.ticket, 0, sizeof(unsigned int), st));
    k_mic_wavefront<T, true, TY><<<grid, WF_TX * TY, smem, st>>>(d, bb, F, r, z, w);
    w.epoch = next_epoch();
    FFGPU_CUDA(cudaMemsetAsync(ww.ticket, 0, sizeof(unsigned int), st));
    k_mic_wavefront<T, false, TY><<<grid, WF_TX * TY, smem, st>>>(d, bb, F, r, z, w);
}

template void mic_wavefront<double>(Dims, Bbox, FactorView<double>, const double *, double *, WfWork, cudaStream_t);
template void mic_wavefront<float>(Dims, Bbox, FactorView<float>, const float *, float *, WfWork, cudaStream_t);

}  // namespace ffgpu
