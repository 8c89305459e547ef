// MIC(0) preconditioner application (pcgsolver.h:212-241) as a pipelined wavefront.
//
// The box of pressure cells is cut into tiles of 16 x 16 columns in the (x, y) plane.  A tile
// is swept by 8 x 8 solver threads; each owns a 2 x 2 block of columns and walks z.  Thread
// (tx, ty) processes plane z of its block at step t = z + tx + ty, visiting its four cells in
// the order (0,0), (1,0), (0,1), (1,1), so every cell's -x, -y and -z neighbours (the upstream
// ones) are final when it is computed: inside the block they were just computed by the same
// thread, across blocks they were computed one step earlier by the neighbouring thread,
// which hands its factor products L*q over through shared memory (one barrier per step).
// Every cell therefore performs exactly the reference's operations in the reference's order:
//   forward   q(c) = (((r(c) - Lz(c-z) q(c-z)) - Ly(c-y) q(c-y)) - Lx(c-x) q(c-x)) * inv(c)
//   backward  z(c) = (((q(c) - Lx(c) z(c+x)) - Ly(c) z(c+y)) - Lz(c) z(c+z)) * inv(c)
// which is the same as evaluating the i+j+k hyperplanes one after another.  A neighbour outside
// the box of pressure cells has no matrix entry and contributes nothing, as in the reference.
// The backward sweep runs the same code on mirrored tiles (+x/+y/+z are upstream).
//
// Memory access.  Because of the skew, the solver threads work on different z planes at any
// step.  Dedicated staging threads therefore copy whole planes of the tile (rows of 16 cells,
// coalesced) with cp.async several steps before they are first needed into a delay line in
// shared memory, laid out so that each solver thread reads its own slots without bank
// conflicts, and write results back one full plane at a time once the last solver thread
// finished it.  The staging threads also move the tile-face values (below), so the solver
// threads run nothing but the dependent arithmetic, without branches.
//
// Tiles depend on their upstream neighbour tiles.  The values that cross a tile face (forward:
// the products Lx*q, Ly*q; backward: z) are passed through an exchange buffer, one 64-bit word
// per value and plane, whose high half holds the epoch of the sweep that wrote it (FP64 values
// take two words, one per half).  Value and epoch land in one single-copy-atomic store, so the
// consumer needs no fence: a staging lane loads the word a few steps ahead and, if the epoch is
// not yet the current one, polls until it is, then places the value where the solver thread on
// the tile's first column / row reads its neighbour's hand-over.
// Persistent CTAs take tiles from an atomic ticket in diagonal order, so every tile a CTA waits
// for already belongs to a running CTA: progress is guaranteed whatever the number of resident
// CTAs.  Every wait is bounded: on timeout the kernel raises ERR_WAIT_TIMEOUT in the error word
// (which also releases every other waiter), the CTA drains its copies and abandons its tiles,
// so the launch always terminates and the host reports the failure.
#include <algorithm>
#include <atomic>
#include <climits>
#include <cstdint>
#include <stdexcept>
#include <vector>

#include "common.cuh"
#include "kernels.h"
#include "mic_wavefront.cuh"
#include "pcg.h"

namespace ffgpu {

#ifndef FFGPU_WF_DE
#define FFGPU_WF_DE 2
#endif
constexpr int WF_NX = 8, WF_NY = 8;                // solver threads per tile (x, y)
constexpr int WF_NT = WF_NX * WF_NY;
constexpr int WF_NCOPY = 128;                      // staging threads per tile
constexpr int WF_NFACE = 64;                       // face threads per tile (deliver, publish)
constexpr int WF_THREADS = WF_NT + WF_NCOPY + WF_NFACE;
constexpr int WF_TC = 16;                          // tile edge in cells (2 x 2 cells per solver thread)
constexpr int WF_ROUT = WF_NX + WF_NY;             // output delay line depth (planes)
constexpr int WF_DE = FFGPU_WF_DE;                 // tile-face words are loaded this many steps ahead

// Planes staged ahead (D) and input delay line depth: a plane is read by the solver threads for
// WF_NX + WF_NY - 1 steps after the step it is first needed.  FP64 stays within 227 KB.
#ifndef FFGPU_WF_D32
#define FFGPU_WF_D32 8
#endif
template <typename T> struct WfShape {
    static constexpr int D = sizeof(T) == 4 ? FFGPU_WF_D32 : 3;
    static constexpr int RIN = D + WF_NX + WF_NY - 1;
};


template <typename T> struct WfSmem {
    Quad<T> in[WfShape<T>::RIN][5][WF_NT];   // [plane slot][r-or-q, inv, lx, ly, lz][solver thread]
    Quad<T> out[WF_ROUT][WF_NT];             // [plane slot][solver thread]
    T hx[2][2][WF_NT];                    // [step parity][block row]: hand-over to the +x neighbour thread
    T hy[2][2][WF_NT];                    // [step parity][block column]: hand-over to the +y neighbour thread
    T fx[2][2][WF_NT];                    // [step parity][block row]: x-face values for the first thread column
    T fy[2][2][WF_NT];                    // [step parity][block column]: y-face values for the first thread row
};

template <typename T> __device__ inline void cp_async_elem(T *dst, const T *src) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
    if constexpr (sizeof(T) == 4)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(src) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(src) : "memory");
}
// Two adjacent cells (8 or 16 bytes, aligned to their size).
template <typename T> __device__ inline void cp_async_pair(T *dst, const T *src) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
    if constexpr (sizeof(T) == 4)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(src) : "memory");
    else
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(src) : "memory");
}
template <typename T> __device__ inline void store_pair(T *g, const T *s) {
    if constexpr (sizeof(T) == 4) *reinterpret_cast<float2 *>(g) = *reinterpret_cast<const float2 *>(s);
    else *reinterpret_cast<double2 *>(g) = *reinterpret_cast<const double2 *>(s);
}
__device__ inline void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ inline void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }
__device__ inline void cp_async_drain() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Compensated FP32 sum of squares (TwoProduct through fmaf, then TwoSum), as the PCG's FP32 dots.
struct SqAcc {
    float hi = 0.0f, lo = 0.0f;
    __device__ void add(float a) {
        const float p = a * a, e = fmaf(a, a, -p);
        const float s = hi + p, bb = s - hi;
        const float err = (hi - (s - bb)) + (p - bb);
        hi = s;
        lo += err + e;
    }
    __device__ double value() const { return (double)hi + (double)lo; }
};
__device__ inline double warp_sum_xor(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
// The q.q partials summed by one block of BLOCK threads in a fixed order, then rho (first) or beta
// and rho updated as the z.r dot kernel updates them (FP64 step scalars).
template <int BLOCK>
__device__ inline void dotq_final(const double *part, int P, PcgScalars *sc, int first, double *sm) {
    double s = 0.0;
    for (int q = threadIdx.x; q < P; q += BLOCK) s += __ldcg(part + q);
    const double tot = block_sum<BLOCK>(s, sm);
    if (threadIdx.x == 0) {
        if (first) {
            sc->rho = tot;
        } else {
            sc->beta = tot / sc->rho;
            sc->beta_used = sc->beta;
            sc->rho = tot;
        }
    }
}

// running ring index: i mod n for i = i0, i0 + 1, ...
struct RingIdx {
    int v;
    __device__ RingIdx(int i0, int n) : v(((i0 % n) + n) % n) {}
    __device__ void next(int n) { v = v + 1 == n ? 0 : v + 1; }
};

// DOTQ (FP32 forward sweep): the staging threads also sum the squares of the results they write back,
// each staging warp's sum goes to w.dot_part[4 tile + warp], and the last CTA to leave sums them all
// and updates the PCG scalars (rho = z.r = q.q for M = L L^T).
template <typename T, bool FORWARD, bool PAIRS, bool DOTQ = false>
__global__ void __launch_bounds__(WF_THREADS) k_mic_wavefront(Dims d, Bbox bb, FactorView<T> F, const T *__restrict__ rin,
                                                              T *q, WfTiles w) {
    static_assert(!DOTQ || (FORWARD && sizeof(T) == 4), "the dot rides on the FP32 forward sweep");
    extern __shared__ __align__(32) unsigned char wf_smem_raw[];
    WfSmem<T> &S = *reinterpret_cast<WfSmem<T> *>(wf_smem_raw);
    constexpr int NW = WfWords<T>::N;
    constexpr int D = WfShape<T>::D, RIN = WfShape<T>::RIN;
    constexpr int sg = FORWARD ? 1 : -1;      // sweep direction along every axis
    constexpr int SKEW = WF_NX + WF_NY - 2;   // steps between the solver's first and last thread on one plane
    __shared__ int s_tile;
    __shared__ int s_abort[2];   // set during step t into slot (t + 1) & 1, read after the barrier of step t + 1
    __shared__ unsigned int s_epoch;
    const int tid = threadIdx.x;
    // this sweep's tag: one past the last sweep's (0 is never a tag)
    if (tid == 0) {
        const unsigned int e = *reinterpret_cast<volatile unsigned int *>(w.epoch_ctr) + 1u;
        s_epoch = e == 0u ? 1u : e;
    }
    __syncthreads();
    w.epoch = s_epoch;
    const int K = bb.k1 - bb.k0 + 1;
    const int ntiles = w.A * w.B;
    const int steps = K + SKEW;
    // Face values are stored by diagonal: row / column r of plane s sits at diagonal s + r / 2, the
    // step on which the consumer needs it, so the 16 values of one step share one line.
    const int KD = K + WF_NX - 1;                        // diagonals of a face
    const size_t yface0 = (size_t)ntiles * WF_TC * KD;   // first y-face value
    const int ni = d.ni, slab = d.ni * d.nj;
    const int dk = sg * slab;
    // The last CTA to leave resets the ticket pair for the next sweep (stream order makes the
    // reset visible to it).
    // With DOTQ every thread of the CTA calls it (uniformly): the last CTA then sums the partials,
    // unless the sweep was skipped or gave up (reduce false).
    __shared__ int s_last;
    __shared__ double s_red[WF_THREADS / 32];
    auto leave = [&](bool reduce) {
        if (tid == 0) {
            if (DOTQ) __threadfence();   // this CTA's partials before its count
            const bool last = atomicAdd(w.ticket + 1, 1u) == gridDim.x - 1;
            s_last = last ? 1 : 0;
            if (last) {
                w.ticket[0] = 0;
                w.ticket[1] = 0;
                *w.epoch_ctr = w.epoch;   // every CTA read the counter before it left
            }
        }
        if constexpr (DOTQ) {
            __syncthreads();
            if (s_last && reduce) {
                __threadfence();
                dotq_final<WF_THREADS>(w.dot_part, 4 * ntiles, w.dot_sc, w.dot_first, s_red);
            }
        }
    };
    if (w.done && *w.done) { leave(false); return; }
    for (;;) {
        if (tid == 0) {
            unsigned int tk = atomicAdd(w.ticket, 1u);
            s_tile = (int)tk;
            s_abort[0] = s_abort[1] = 0;
        }
        __syncthreads();
        const int tk = s_tile;
        if (tk >= ntiles) { leave(true); return; }
        const short2 ab = w.order[FORWARD ? tk : ntiles - 1 - tk];
        const int a = ab.x, b = ab.y;
        const int tile = a + w.A * b;
        const int upx = FORWARD ? (a > 0 ? tile - 1 : -1) : (a < w.A - 1 ? tile + 1 : -1);
        const int upy = FORWARD ? (b > 0 ? tile - w.A : -1) : (b < w.B - 1 ? tile + w.A : -1);
        // grid coordinates of tile-local position (lx, ly); tiles are mirrored for the backward sweep
        auto gxl = [&](int lx) { return w.x0 + a * WF_TC + (FORWARD ? lx : WF_TC - 1 - lx); };
        auto gyl = [&](int ly) { return bb.j0 + b * WF_TC + (FORWARD ? ly : WF_TC - 1 - ly); };
        auto inx = [&](int x) { return x >= bb.i0 && x <= bb.i1; };
        auto iny = [&](int y) { return y >= bb.j0 && y <= bb.j1; };
        bool abort = false;
        if (tid < WF_NT) {
            // ---- solver thread: the 2 x 2 block (2 tx .. 2 tx + 1, 2 ty .. 2 ty + 1), tile-local ----
            const int tx = tid % WF_NX, ty = tid / WF_NX;
            bool cv[4];
#pragma unroll
            for (int cc = 0; cc < 4; cc++) cv[cc] = inx(gxl(2 * tx + (cc & 1))) && iny(gyl(2 * ty + (cc >> 1)));
            // upstream values of the block's first column / row: the neighbour thread's hand-over,
            // or on the tile's first column / row the face values the staging threads deliver
            const T *xsrc = tx > 0 ? &S.hx[0][0][tid - 1] : &S.fx[0][0][tid];
            const T *ysrc = ty > 0 ? &S.hy[0][0][tid - WF_NX] : &S.fy[0][0][tid];
            RingIdx rs(-(tx + ty), RIN), ro(-(tx + ty), WF_ROUT);
            T carry[4] = {T(0), T(0), T(0), T(0)};   // z hand-over of each block cell
            for (int t = 0; t < steps; t++) {
                __syncthreads();   // step t-1 done everywhere: hand-overs, faces and planes <= t are in shared memory
                if (s_abort[t & 1]) { abort = true; break; }
                const int s = t - tx - ty;
                if (s >= 0 && s < K) {
                    const int pb = ((t - 1) & 1) * 2 * WF_NT, cb = t & 1;
                    // block cells are stored in memory order: x-pair index (cx, or 1 - cx backward) + 2 cy
                    const Quad<T> qin = S.in[rs.v][0][tid], qinv = S.in[rs.v][1][tid];
                    const Quad<T> qlx = S.in[rs.v][2][tid], qly = S.in[rs.v][3][tid], qlz = S.in[rs.v][4][tid];
                    const T nx0 = xsrc[pb], nx1 = xsrc[pb + WF_NT], ny0 = ysrc[pb], ny1 = ysrc[pb + WF_NT];
                    T hxo[4], hyo[4], res[4];   // hand-overs to the downstream x / y neighbour; results
#pragma unroll
                    for (int cc = 0; cc < 4; cc++) {
                        const int cx = cc & 1, cy = cc >> 1;
                        const int e = (FORWARD ? cx : 1 - cx) + 2 * cy;
                        const T nx = cx ? hxo[cc - 1] : (cy ? nx1 : nx0);
                        const T ny = cy ? hyo[cc - 2] : (cx ? ny1 : ny0);
                        T v = qin.v[e];
                        // a neighbour outside the box hands over +0 (and has a +0 coefficient), so the
                        // subtraction leaves v unchanged bit for bit, as the reference's missing entry;
                        // cells outside the box (their staged operands are arbitrary) produce exactly +0
                        if (FORWARD) {
                            v -= carry[cc];   // Lz(c-z) q(c-z)
                            v -= ny;          // Ly(c-y) q(c-y)
                            v -= nx;          // Lx(c-x) q(c-x)
                            res[cc] = cv[cc] ? v * qinv.v[e] : T(0);
                            hxo[cc] = cv[cc] ? qlx.v[e] * res[cc] : T(0);
                            hyo[cc] = cv[cc] ? qly.v[e] * res[cc] : T(0);
                            carry[cc] = cv[cc] ? qlz.v[e] * res[cc] : T(0);
                        } else {
                            v -= qlx.v[e] * nx;          // Lx(c) z(c+x)
                            v -= qly.v[e] * ny;          // Ly(c) z(c+y)
                            v -= qlz.v[e] * carry[cc];   // Lz(c) z(c+z)
                            res[cc] = cv[cc] ? v * qinv.v[e] : T(0);
                            hxo[cc] = hyo[cc] = carry[cc] = res[cc];
                        }
                    }
                    Quad<T> qo;
#pragma unroll
                    for (int cc = 0; cc < 4; cc++) qo.v[(FORWARD ? (cc & 1) : 1 - (cc & 1)) + 2 * (cc >> 1)] = res[cc];
                    S.out[ro.v][tid] = qo;
                    S.hx[cb][0][tid] = hxo[1];
                    S.hx[cb][1][tid] = hxo[3];
                    S.hy[cb][0][tid] = hyo[2];
                    S.hy[cb][1][tid] = hyo[3];
                }
                rs.next(RIN);
                ro.next(WF_ROUT);
            }
            if (!abort) __syncthreads();   // the staging threads may publish and write back the last step
        } else if (tid < WF_NT + WF_NCOPY) {
            // ---- staging threads ----
            const int ctid = tid - WF_NT;
            // Each staging thread owns one cell pair of the tile: tile-local row ly (solver frame) = ctid / 8,
            // memory-order pair pm = ctid % 8 (cells 2 pm, 2 pm + 1 counted from the tile's low-x edge).
            // It stages the pair of all five arrays every plane (consecutive lanes copy consecutive
            // 8-cell rows, coalesced) and writes the pair's results back.
            const int ly = ctid / 8, pm = ctid % 8;
            const int xlo = w.x0 + a * WF_TC + 2 * pm, ypair = gyl(ly);
            const int stx = FORWARD ? pm : WF_NX - 1 - pm;   // solver thread column owning the pair
            const bool plo = iny(ypair) && inx(xlo), phi_ = iny(ypair) && inx(xlo + 1);
            const bool pv = plo || phi_;
            const int goff = xlo + ni * ypair + slab * (FORWARD ? bb.k0 : bb.k1);   // grid offset on plane 0
            const int sdst = (stx + WF_NX * (ly >> 1)) * 4 + 2 * (ly & 1);          // element in a [slot][array] row
            const T *src[5] = {FORWARD ? rin : (const T *)q, F.inv, F.lx, F.ly, F.lz};
            T *in0 = &S.in[0][0][0].v[0];
            const T *out0 = &S.out[0][0].v[0];
            int pst = 0, slot = 0;   // next plane to stage and its slot
            auto stage = [&]() {
                if (pv && pst < K) {
                    const int c = goff + pst * dk;
#pragma unroll
                    for (int m = 0; m < 5; m++) {
                        T *dstp = in0 + (size_t)(slot * 5 + m) * WF_NT * 4 + sdst;
                        if (PAIRS) {
                            cp_async_pair(dstp, src[m] + c);
                        } else {
                            if (plo) cp_async_elem(dstp, src[m] + c);
                            if (phi_) cp_async_elem(dstp + 1, src[m] + c + 1);
                        }
                    }
                }
                cp_async_commit();
                ++pst;
                slot = slot + 1 == RIN ? 0 : slot + 1;
            };
            // plane po is complete once the solver's last thread did it, SKEW steps after the first
            int po = -(SKEW + 1);
            RingIdx rpo(po, WF_ROUT);
            SqAcc qq;   // DOTQ: the pair's squares over the planes in sweep order
            auto write_back = [&]() {
                if (pv && po >= 0 && po < K) {
                    const T *o = out0 + (size_t)rpo.v * WF_NT * 4 + sdst;
                    T *g = q + (goff + po * dk);
                    if (PAIRS && plo && phi_) {
                        store_pair(g, o);
                    } else {
                        if (plo) g[0] = o[0];
                        if (phi_) g[1] = o[1];
                    }
                    if constexpr (DOTQ) {
                        if (plo) qq.add(o[0]);
                        if (phi_) qq.add(o[1]);
                    }
                }
                ++po;
                rpo.next(WF_ROUT);
            };
            for (int p = 0; p < D; p++) stage();
            cp_async_wait<D - 1>();   // plane 0 has landed
            for (int t = 0; t < steps; t++) {
                __syncthreads();   // step t-1 done everywhere
                if (s_abort[t & 1]) { abort = true; break; }
                stage();        // plane t + D
                write_back();   // plane t - SKEW - 1
                cp_async_wait<D - 1>();   // plane t + 1 has landed
            }
            cp_async_drain();
            if (!abort) {
                __syncthreads();   // the solver finished its last step
                while (po < K) write_back();
                if constexpr (DOTQ) {
                    const double v = warp_sum_xor(qq.value());
                    if ((ctid & 31) == 0) {
                        w.dot_part[4 * (size_t)tile + (ctid >> 5)] = v;
                        __threadfence();
                    }
                }
            }
        } else {
            // ---- face threads: lane r of the first warp (x rows r < 16, y columns r - 16) delivers the
            // upstream tiles' values, lane r of the second publishes this tile's.  Row / column r of a
            // face belongs to block cell r % 2 of solver thread r / 2 in the tile's first (consumer) or
            // last (producer) thread column / row.
            const int fwarp = (tid - WF_NT - WF_NCOPY) / 32, lane = tid % 32;
            const bool xr = lane < 16;
            const int r = lane & 15;
            const int sid = xr ? WF_NX * (r >> 1) : (r >> 1);                                         // consumer
            const int pid = xr ? (WF_NX - 1) + WF_NX * (r >> 1) : (r >> 1) + WF_NX * (WF_NY - 1);   // producer
            bool get = false, put = false;
            const unsigned long long *gsrc = nullptr;
            unsigned long long *pdst = nullptr;
            T *gdst = nullptr;
            const T *psrc = nullptr;
            if (fwarp == 0) {
                const int x = gxl(xr ? 0 : r), y = gyl(xr ? r : 0);
                const int up = xr ? upx : upy;
                get = up >= 0 && inx(x) && iny(y) && (xr ? inx(x - sg) : iny(y - sg));
                gsrc = w.xchg + NW * ((xr ? 0 : yface0) + (size_t)(up < 0 ? 0 : up) * WF_TC * KD + r);
                gdst = xr ? &S.fx[0][r & 1][sid] : &S.fy[0][r & 1][sid];
            } else {
                const int x = gxl(xr ? WF_TC - 1 : r), y = gyl(xr ? r : WF_TC - 1);
                put = inx(x) && iny(y) && (xr ? inx(x + sg) : iny(y + sg));
                pdst = w.xchg + NW * ((xr ? 0 : yface0) + (size_t)tile * WF_TC * KD + r);
                psrc = xr ? &S.hx[0][r & 1][pid] : &S.hy[0][r & 1][pid];
            }
            // deliver the face value the consumer uses at solver step tt (plane tt - r / 2) into parity (tt - 1) & 1
            WfWords<T> gw[WF_DE] = {};
            // the words a step needs (diagonal tt, every row) share one line
            auto get_load = [&](WfWords<T> &g, int tt) {
                const int s = tt - (r >> 1);
                if (get && s >= 0 && s < K) face_load(g, gsrc + (size_t)NW * WF_TC * tt);
            };
            auto deliver = [&](WfWords<T> &g, int tt) {
                const int s = tt - (r >> 1);
                T v = T(0);
                if (get && s >= 0 && s < K && !face_get(g, gsrc + (size_t)NW * WF_TC * tt, w, v)) s_abort[tt & 1] = 1;
                gdst[((tt - 1) & 1) * 2 * WF_NT] = v;
            };
            // publish the value the producer handed over at solver step tt (plane tt - (WF_NX - 1) - r / 2)
            auto publish = [&](int tt) {
                const int s = tt - (WF_NX - 1) - (r >> 1);
                if (put && s >= 0 && s < K)
                    face_put(pdst + (size_t)NW * WF_TC * (s + (r >> 1)), psrc[(tt & 1) * 2 * WF_NT], w.epoch);
            };
            if (fwarp == 0) {
#pragma unroll
                for (int u = 0; u < WF_DE; u++) get_load(gw[u], u);
                WfWords<T> g0 = gw[0];   // faces of solver step 0
                deliver(g0, 0);
                get_load(gw[0], WF_DE);
                for (int t0 = 0; t0 < steps && !abort; t0 += WF_DE) {
#pragma unroll
                    for (int u = 0; u < WF_DE; u++) {
                        const int t = t0 + u;
                        if (t >= steps) break;
                        __syncthreads();   // step t-1 done everywhere
                        if (s_abort[t & 1]) { abort = true; break; }
                        if (t + 1 < steps) {
                            // slot (u + 1) % WF_DE holds the words of step t + 1
                            deliver(gw[(u + 1) % WF_DE], t + 1);
                            if (t + 1 + WF_DE < steps) get_load(gw[(u + 1) % WF_DE], t + 1 + WF_DE);
                        }
                    }
                }
                if (!abort) __syncthreads();
            } else {
                for (int t = 0; t < steps; t++) {
                    __syncthreads();   // step t-1 done everywhere: its hand-overs are in shared memory
                    if (s_abort[t & 1]) { abort = true; break; }
                    if (t > 0) publish(t - 1);
                }
                if (!abort) {
                    __syncthreads();   // the solver finished its last step
                    publish(steps - 1);
                }
            }
        }
        if (abort || s_abort[steps & 1]) { leave(false); return; }   // every thread saw the same flags after the same barriers
    }
}

template <typename T, bool PAIRS>
static int wf_setup(size_t smem) {   // per device: opt in to the shared memory, count resident CTAs
    static std::atomic<int> cached[64];
    int dev = 0;
    FFGPU_CUDA(cudaGetDevice(&dev));
    if (dev < 64 && cached[dev].load() > 0) return cached[dev].load();
    FFGPU_CUDA(cudaFuncSetAttribute(k_mic_wavefront<T, true, PAIRS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    FFGPU_CUDA(cudaFuncSetAttribute(k_mic_wavefront<T, false, PAIRS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if constexpr (sizeof(T) == 4)
        FFGPU_CUDA(cudaFuncSetAttribute(k_mic_wavefront<T, true, PAIRS, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem));
    int sms = 0, per = 0;
    FFGPU_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    FFGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_mic_wavefront<T, true, PAIRS>, WF_THREADS, smem));
    const int r = std::max(1, sms * std::max(per, 1));
    if (dev < 64) cached[dev].store(r);
    return r;
}

template <typename T, bool PAIRS>
static void wf_launch(int grid, size_t smem, Dims d, Bbox bb, FactorView<T> F, const T *r, T *z, WfTiles w,
                      unsigned int e_fwd, unsigned int e_bwd, unsigned int *ticket, cudaStream_t st) {
    // forward sweep: r -> z, then backward sweep in place on z (each sweep leaves the ticket at 0)
    w.epoch = e_fwd;
    k_mic_wavefront<T, true, PAIRS><<<grid, WF_THREADS, smem, st>>>(d, bb, F, r, z, w);
    w.epoch = e_bwd;
    k_mic_wavefront<T, false, PAIRS><<<grid, WF_THREADS, smem, st>>>(d, bb, F, r, z, w);
}

int mic_wavefront_max_tiles(int I, int J) { return ((I + 1 + WF_TC - 1) / WF_TC) * ((J + WF_TC - 1) / WF_TC); }

size_t mic_wavefront_xchg_words(int I, int J, int K) {
    return 2 * (size_t)mic_wavefront_max_tiles(I, J) * (2 * WF_TC) * (size_t)(K + WF_NX);   // FP64: two words a value
}

void wf_upload_order(const WfWork &ww, int A, int B, cudaStream_t st) {
    const long long key = (long long)A << 32 | B;
    if (*ww.order_key == key) return;
    const int nt = A * B;
    std::vector<short2> ord;
    ord.reserve(nt);
    for (int dg = 0; dg <= A + B - 2; dg++)
        for (int a = 0; a < A; a++) {
            int b = dg - a;
            if (b >= 0 && b < B) ord.push_back(make_short2((short)a, (short)b));
        }
    FFGPU_CUDA(cudaMemcpyAsync(ww.order, ord.data(), nt * sizeof(short2), cudaMemcpyHostToDevice, st));
    FFGPU_CUDA(cudaStreamSynchronize(st));
    *ww.order_key = key;
}

static void wf_clear_epochs(const WfWork &ww, cudaStream_t st) {
    // no stale word may carry a reused tag: clear the words and restart both counters at 0
    FFGPU_CUDA(cudaMemsetAsync(ww.xchg, 0, ww.xchg_words * sizeof(unsigned long long), st));
    FFGPU_CUDA(cudaMemsetAsync(ww.epoch_dev, 0, sizeof(unsigned int), st));
    *ww.epoch = 0;
}

unsigned int wf_next_epoch(const WfWork &ww, cudaStream_t st) {
    if (*ww.epoch == UINT_MAX) wf_clear_epochs(ww, st);
    return ++*ww.epoch;
}

void wf_reserve_epochs(const WfWork &ww, unsigned int n, cudaStream_t st) {
    if (*ww.epoch > UINT_MAX - n) wf_clear_epochs(ww, st);
}

// Launch shape of a sweep over box bb of grid d: tiles, CTAs, shared memory, pair copies.
template <typename T> struct WfPlan {
    WfTiles w;
    int grid;
    size_t smem;
    bool pairs;
};

template <typename T>
static WfPlan<T> wf_plan(Dims d, Bbox bb, FactorView<T> F, const T *r, const T *z, WfWork ww, cudaStream_t st) {
    // cell indices are 32-bit inside the kernels (block offsets reach one slab past the box)
    if (d.cells() + 2 * (size_t)d.ni * d.nj >= (size_t)INT_MAX)
        throw std::runtime_error("Error: grid too large for the wavefront preconditioner.\n");
    WfPlan<T> p;
    p.smem = sizeof(WfSmem<T>);
    // Cell pairs move as one 8- or 16-byte copy when every row starts on a pair boundary: the
    // tiles start at an even x, so that needs an even row length and pair-aligned arrays.
    auto aligned = [](const void *q) { return reinterpret_cast<uintptr_t>(q) % (2 * sizeof(T)) == 0; };
    p.pairs = d.ni % 2 == 0 && aligned(F.inv) && aligned(F.lx) && aligned(F.ly) && aligned(F.lz) &&
              (r == nullptr || aligned(r)) && aligned(z);
    const int resident = p.pairs ? wf_setup<T, true>(p.smem) : wf_setup<T, false>(p.smem);
    const int x0 = bb.i0 & ~1;
    const int I = bb.i1 - x0 + 1, J = bb.j1 - bb.j0 + 1, K = bb.k1 - bb.k0 + 1;
    WfTiles &w = p.w;
    w.A = (I + WF_TC - 1) / WF_TC;
    w.B = (J + WF_TC - 1) / WF_TC;
    w.x0 = x0;
    const int nt = w.A * w.B;
    if (nt > ww.max_tiles) throw std::runtime_error("Error: wavefront tile table too small.\n");
    if ((size_t)WfWords<T>::N * nt * (2 * WF_TC) * (K + WF_NX) > ww.xchg_words)
        throw std::runtime_error("Error: wavefront exchange buffer too small.\n");
    w.order = ww.order; w.xchg = ww.xchg; w.ticket = ww.ticket; w.error = ww.error;
    w.epoch_ctr = ww.epoch_dev;
    w.spin_limit = ww.spin_limit > 0 ? ww.spin_limit : WF_SPIN_LIMIT;
    w.done = ww.done;
    w.dot_part = ww.dot_part;
    w.dot_sc = nullptr;
    w.dot_first = 0;
    wf_upload_order(ww, w.A, w.B, st);
    p.grid = std::min(nt, resident);
    return p;
}

template <typename T>
void mic_wavefront(Dims d, Bbox bb, FactorView<T> F, const T *r, T *z, WfWork ww, cudaStream_t st) {
    const WfPlan<T> p = wf_plan<T>(d, bb, F, r, z, ww, st);
    const unsigned int e1 = wf_next_epoch(ww, st), e2 = wf_next_epoch(ww, st);
    if (p.pairs) wf_launch<T, true>(p.grid, p.smem, d, bb, F, r, z, p.w, e1, e2, ww.ticket, st);
    else wf_launch<T, false>(p.grid, p.smem, d, bb, F, r, z, p.w, e1, e2, ww.ticket, st);
}

template <typename T>
void mic_wavefront_sweep(Dims d, Bbox bb, FactorView<T> F, const T *r, T *q, WfWork ww, bool forward, cudaStream_t st) {
    WfPlan<T> p = wf_plan<T>(d, bb, F, forward ? r : nullptr, q, ww, st);
    p.w.epoch = wf_next_epoch(ww, st);
    if (forward) {
        if (p.pairs) k_mic_wavefront<T, true, true><<<p.grid, WF_THREADS, p.smem, st>>>(d, bb, F, r, q, p.w);
        else k_mic_wavefront<T, true, false><<<p.grid, WF_THREADS, p.smem, st>>>(d, bb, F, r, q, p.w);
    } else {
        if (p.pairs) k_mic_wavefront<T, false, true><<<p.grid, WF_THREADS, p.smem, st>>>(d, bb, F, q, q, p.w);
        else k_mic_wavefront<T, false, false><<<p.grid, WF_THREADS, p.smem, st>>>(d, bb, F, q, q, p.w);
    }
    FFGPU_CUDA(cudaGetLastError());
}

// The forward sweep's q.q from q in memory, in the sweep's order: block = tile, thread = staging thread
// (the same cell pair, planes in order, the same compensated sum and warp tree).
__global__ void __launch_bounds__(WF_NCOPY) k_dotq_tiles(Dims d, Bbox bb, int x0, int A, const float *__restrict__ q,
                                                         double *part, const PcgScalars *sc) {
    if (sc->done) return;
    const int tile = blockIdx.x, a = tile % A, b = tile / A;
    const int ctid = threadIdx.x, ly = ctid / 8, pm = ctid % 8;
    const int xlo = x0 + a * WF_TC + 2 * pm, ypair = bb.j0 + b * WF_TC + ly;
    const bool yin = ypair >= bb.j0 && ypair <= bb.j1;
    const bool plo = yin && xlo >= bb.i0 && xlo <= bb.i1, phi_ = yin && xlo + 1 >= bb.i0 && xlo + 1 <= bb.i1;
    const int K = bb.k1 - bb.k0 + 1, slab = d.ni * d.nj;
    const int goff = xlo + d.ni * ypair + slab * bb.k0;
    SqAcc qq;
    if (plo || phi_)
        for (int po = 0; po < K; po++) {
            const float *g = q + (goff + po * slab);
            if (plo) qq.add(g[0]);
            if (phi_) qq.add(g[1]);
        }
    const double v = warp_sum_xor(qq.value());
    if ((ctid & 31) == 0) part[4 * (size_t)tile + (ctid >> 5)] = v;
}

__global__ void __launch_bounds__(256) k_dotq_final(const double *part, int P, PcgScalars *sc, int first) {
    __shared__ double sm[256 / 32];
    if (sc->done) return;
    dotq_final<256>(part, P, sc, first, sm);
}

void mic_dotq_tiles(Dims d, Bbox bb, const float *q, double *part, int max_tiles, PcgScalars *sc, int first,
                    cudaStream_t st) {
    const int x0 = bb.i0 & ~1;
    const int A = (bb.i1 - x0 + 1 + WF_TC - 1) / WF_TC, B = (bb.j1 - bb.j0 + 1 + WF_TC - 1) / WF_TC;
    if (A * B > max_tiles) throw std::runtime_error("Error: wavefront tile table too small.\n");
    k_dotq_tiles<<<A * B, WF_NCOPY, 0, st>>>(d, bb, x0, A, q, part, sc);
    k_dotq_final<<<1, 256, 0, st>>>(part, 4 * A * B, sc, first);
    FFGPU_CUDA(cudaGetLastError());
}

void mic_wavefront_dot(Dims d, Bbox bb, FactorView<float> F, const float *r, float *z, WfWork ww, PcgScalars *sc,
                       int first, cudaStream_t st) {
    WfPlan<float> p = wf_plan<float>(d, bb, F, r, z, ww, st);
    if (!ww.dot_part) throw std::runtime_error("Error: no buffer for the preconditioner's dot partials.\n");
    p.w.dot_sc = sc;
    p.w.dot_first = first;
    p.w.epoch = wf_next_epoch(ww, st);
    if (p.pairs) {
        k_mic_wavefront<float, true, true, true><<<p.grid, WF_THREADS, p.smem, st>>>(d, bb, F, r, z, p.w);
    } else {
        k_mic_wavefront<float, true, false, true><<<p.grid, WF_THREADS, p.smem, st>>>(d, bb, F, r, z, p.w);
    }
    p.w.epoch = wf_next_epoch(ww, st);
    if (p.pairs) k_mic_wavefront<float, false, true><<<p.grid, WF_THREADS, p.smem, st>>>(d, bb, F, z, z, p.w);
    else k_mic_wavefront<float, false, false><<<p.grid, WF_THREADS, p.smem, st>>>(d, bb, F, z, z, p.w);
    FFGPU_CUDA(cudaGetLastError());
}

// A wait that nothing ends: one warp waits with face_get for an epoch-1 word that stays zero, under
// the given limit, so the wait gives up, raises ERR_WAIT_TIMEOUT in the error word and returns.
__global__ void k_wait_probe(const unsigned long long *word, unsigned int *error, long long limit) {
    WfTiles w{};
    w.error = error;
    w.epoch = 1;
    w.spin_limit = limit;
    WfWords<float> f{};
    float v = 0.0f;
    face_get(f, word, w, v);
}

unsigned int wait_probe(long long limit, cudaStream_t st) {
    unsigned long long *word = nullptr;
    unsigned int *error = nullptr;
    FFGPU_CUDA(cudaMalloc(&word, sizeof(unsigned long long) + sizeof(unsigned int)));
    error = reinterpret_cast<unsigned int *>(word + 1);
    unsigned int bits = 0;
    cudaError_t e = cudaMemsetAsync(word, 0, sizeof(unsigned long long) + sizeof(unsigned int), st);
    if (e == cudaSuccess) {
        k_wait_probe<<<1, 32, 0, st>>>(word, error, limit);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&bits, error, sizeof(unsigned int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(word);
    FFGPU_CUDA(e);
    return bits;
}

template void mic_wavefront<double>(Dims, Bbox, FactorView<double>, const double *, double *, WfWork, cudaStream_t);
template void mic_wavefront<float>(Dims, Bbox, FactorView<float>, const float *, float *, WfWork, cudaStream_t);
template void mic_wavefront_sweep<float>(Dims, Bbox, FactorView<float>, const float *, float *, WfWork, bool,
                                         cudaStream_t);

}  // namespace ffgpu
