// K6 particle-to-grid FLIP transfer, K7 layered velocity extrapolation, K8 constant body
// force and K16 solid-face constraint.  Compiled with -fmad=false so the transfer
// weights match the reference's float arithmetic for every particle/face pair.
#include <cstdint>
#include <stdexcept>

#include "common.cuh"
#include "kernels.h"

namespace ffgpu {

constexpr int CW = 10;   // block frame of the reference transfer (velocityadvector.h:187)

// ---------------------------------------------------------------------------------
// K6: one thread per face of component `comp`.  The face gathers every sorted particle of
// the 2x3x3 cells around it and evaluates, in the reference's block-local float frame
// (10^3 face blocks), the smooth kernel w = 1 - 4/9 d^6/r^6 + 17/9 d^4/r^4 - 22/9 d^2/r^2
// for d^2 < r^2 (velocityadvector.cpp:467-536).  The reference also clips each particle
// to its blocks and search window (sr = r + 1e-6, :293-353, :497-507); d^2 < r^2 already
// implies both with a 1e-6 margin against float rounding of ~1e-8, so the pair set is the
// reference's.  Sums run in cell order, then particle order: deterministic, no atomics.
// ---------------------------------------------------------------------------------
// With REC (the differentiable substep) the kernel also accumulates the same transfer with
// the kernel weight in its factored form w = (1 - s)^2 (1 - 4 s / 9), s = d^2 / r^2, which is
// algebraically identical to the expanded polynomial but keeps its relative precision near
// the kernel radius, where the expanded form cancels.  These accurate sums (wsum) and
// transfer outputs (uacc, on valid faces) feed the transposed transfer.
template <bool REC>
__global__ void __launch_bounds__(256) k_p2g(Dims d, double dx, float r, float sr, int comp, GridDecode dec,
                                             const int *__restrict__ cell_start, const float *__restrict__ spx,
                                             const float *__restrict__ spy, const float *__restrict__ spz,
                                             const float *__restrict__ svel, const float *__restrict__ gpos,
                                             const float *__restrict__ bpos, float *field, unsigned char *valid,
                                             float *wsum, float *uacc) {
    const int fw = d.ni + (comp == 0), fh = d.nj + (comp == 1), fd = d.nk + (comp == 2);
    const unsigned int nf = (unsigned int)fw * fh * fd;
    const float hdx = (float)(0.5 * dx);
    const float ofx = comp == 0 ? 0.0f : hdx, ofy = comp == 1 ? 0.0f : hdx, ofz = comp == 2 ? 0.0f : hdx;
    const float rsq = r * r;
    const float coef1 = (4.0f / 9.0f) * (1.0f / (r * r * r * r * r * r));
    const float coef2 = (17.0f / 9.0f) * (1.0f / (r * r * r * r));
    const float coef3 = (22.0f / 9.0f) * (1.0f / (r * r));
    const float inv_rsq = 1.0f / rsq;
    const float eps = 1e-6f;
    for (unsigned int f = blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += gridDim.x * blockDim.x) {
        int fi, fj, fk;
        dec(f, fi, fj, fk);
        int A = fi / CW, B = fj / CW, C = fk / CW;
        int li = fi - CW * A, lj = fj - CW * B, lk = fk - CW * C;
        // (float)((double)(float)A * chunkdx) and (float)((double)(float)li * dx), from tables
        const float bx = __ldg(bpos + A), by = __ldg(bpos + B), bz = __ldg(bpos + C);
        const float gx = __ldg(gpos + li + 1), gy = __ldg(gpos + lj + 1), gz = __ldg(gpos + lk + 1);
        // candidate cells: the face's own axis spans 2 cells, the others 3
        int i0 = comp == 0 ? fi - 1 : fi - 1, i1 = comp == 0 ? fi : fi + 1;
        int j0 = fj - 1, j1 = comp == 1 ? fj : fj + 1;
        int k0 = fk - 1, k1 = comp == 2 ? fk : fk + 1;
        i0 = max(i0, 0); j0 = max(j0, 0); k0 = max(k0, 0);
        i1 = min(i1, d.ni - 1); j1 = min(j1, d.nj - 1); k1 = min(k1, d.nk - 1);
        float S = 0.0f, W = 0.0f, Sa = 0.0f, Wa = 0.0f;
        for (int ck = k0; ck <= k1; ck++)
            for (int cj = j0; cj <= j1; cj++) {
                size_t base = flat3(0, cj, ck, d.ni, d.nj);
                int p0 = cell_start[base + i0], p1 = cell_start[base + i1 + 1];
                for (int p = p0; p < p1; p++) {
                    // block-local frame of the face's block (velocityadvector.cpp:492-496)
                    float lx = (__ldg(spx + p) - ofx) - bx, ly = (__ldg(spy + p) - ofy) - by, lz = (__ldg(spz + p) - ofz) - bz;
                    float vx = gx - lx, vy = gy - ly, vz = gz - lz;
                    float d2 = vx * vx + vy * vy + vz * vz;
                    if (d2 < rsq) {
                        const float vp = __ldg(svel + p);
                        float wgt = 1.0f - coef1 * d2 * d2 * d2 + coef2 * d2 * d2 - coef3 * d2;
                        S += wgt * vp;
                        W += wgt;
                        if (REC) {
                            const float sq = d2 * inv_rsq, om = 1.0f - sq;
                            const float wa = om * om * (1.0f - (4.0f / 9.0f) * sq);
                            Sa += wa * vp;
                            Wa += wa;
                        }
                    }
                }
            }
        bool ok = W > eps;
        field[f] = ok ? S / W : S;
        valid[f] = ok ? 1 : 0;
        if (REC) {   // kept for the transposed transfer
            wsum[f] = Wa;
            uacc[f] = ok ? Sa / Wa : S;
        }
    }
}

// The three components in one pass: one thread per grid index (i, j, k) transfers to the faces
// u(i, j, k), v(i, j, k) and w(i, j, k) that exist, walking the sorted particles of the 3 x 3 x 3
// cells around (i, j, k) once (each particle loaded once for the three faces).  The three faces
// share the block frame; each takes its own half-cell offsets.  A face's own 2 x 3 x 3 window is a
// subset of the walk, visited in the one-component kernel's cell and particle order, and every
// particle of the other cells lies at least a cell width from the face (d^2 >= dx^2 > r^2), so
// each face's sums are that kernel's, bit for bit.  (Testing each face against its own window only,
// cell by cell, measured slower: 3.42 against 2.84 ms at 256^3.)
__global__ void __launch_bounds__(256) k_p2g3(Dims d, double dx, float r, GridDecode dec,
                                              const int *__restrict__ cell_start, const float *__restrict__ spx,
                                              const float *__restrict__ spy, const float *__restrict__ spz,
                                              const float *__restrict__ svx, const float *__restrict__ svy,
                                              const float *__restrict__ svz, const float *__restrict__ gpos,
                                              const float *__restrict__ bpos, float *fu, float *fv, float *fw,
                                              unsigned char *vu, unsigned char *vv, unsigned char *vw) {
    const unsigned int n = (unsigned int)(d.ni + 1) * (d.nj + 1) * (d.nk + 1);
    const float hdx = (float)(0.5 * dx);
    const float rsq = r * r;
    const float coef1 = (4.0f / 9.0f) * (1.0f / (r * r * r * r * r * r));
    const float coef2 = (17.0f / 9.0f) * (1.0f / (r * r * r * r));
    const float coef3 = (22.0f / 9.0f) * (1.0f / (r * r));
    const float eps = 1e-6f;
    for (unsigned int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int fi, fj, fk;
        dec(t, fi, fj, fk);
        const bool hu = fj < d.nj && fk < d.nk, hv = fi < d.ni && fk < d.nk, hw = fi < d.ni && fj < d.nj;
        const int A = fi / CW, B = fj / CW, C = fk / CW;
        const int li = fi - CW * A, lj = fj - CW * B, lk = fk - CW * C;
        const float bx = __ldg(bpos + A), by = __ldg(bpos + B), bz = __ldg(bpos + C);
        const float gx = __ldg(gpos + li + 1), gy = __ldg(gpos + lj + 1), gz = __ldg(gpos + lk + 1);
        const int i0 = max(fi - 1, 0), i1 = min(fi + 1, d.ni - 1);
        const int j0 = max(fj - 1, 0), j1 = min(fj + 1, d.nj - 1);
        const int k0 = max(fk - 1, 0), k1 = min(fk + 1, d.nk - 1);
        float Su = 0.0f, Wu = 0.0f, Sv = 0.0f, Wv = 0.0f, Sw = 0.0f, Ww = 0.0f;
        auto weight = [&](float d2) { return 1.0f - coef1 * d2 * d2 * d2 + coef2 * d2 * d2 - coef3 * d2; };
        for (int ck = k0; ck <= k1; ck++)
            for (int cj = j0; cj <= j1; cj++) {
                const size_t base = flat3(0, cj, ck, d.ni, d.nj);
                const int p0 = cell_start[base + i0], p1 = cell_start[base + i1 + 1];
                for (int p = p0; p < p1; p++) {
                    const float px = __ldg(spx + p), py = __ldg(spy + p), pz = __ldg(spz + p);
                    // block-local frame (velocityadvector.cpp:492-496): on the face's own axis the
                    // face sits at the grid position, on the others half a cell in
                    const float lx0 = (px - 0.0f) - bx, ly0 = (py - 0.0f) - by, lz0 = (pz - 0.0f) - bz;
                    const float lx1 = (px - hdx) - bx, ly1 = (py - hdx) - by, lz1 = (pz - hdx) - bz;
                    const float ax0 = gx - lx0, ay0 = gy - ly0, az0 = gz - lz0;
                    const float ax1 = gx - lx1, ay1 = gy - ly1, az1 = gz - lz1;
                    const float du = ax0 * ax0 + ay1 * ay1 + az1 * az1;
                    const float dv = ax1 * ax1 + ay0 * ay0 + az1 * az1;
                    const float dw = ax1 * ax1 + ay1 * ay1 + az0 * az0;
                    if (hu && du < rsq) { const float wg = weight(du); Su += wg * __ldg(svx + p); Wu += wg; }
                    if (hv && dv < rsq) { const float wg = weight(dv); Sv += wg * __ldg(svy + p); Wv += wg; }
                    if (hw && dw < rsq) { const float wg = weight(dw); Sw += wg * __ldg(svz + p); Ww += wg; }
                }
            }
        if (hu) {
            const size_t f = (size_t)fi + (size_t)(d.ni + 1) * ((size_t)fj + (size_t)d.nj * fk);
            const bool ok = Wu > eps;
            fu[f] = ok ? Su / Wu : Su;
            vu[f] = ok ? 1 : 0;
        }
        if (hv) {
            const size_t f = (size_t)fi + (size_t)d.ni * ((size_t)fj + (size_t)(d.nj + 1) * fk);
            const bool ok = Wv > eps;
            fv[f] = ok ? Sv / Wv : Sv;
            vv[f] = ok ? 1 : 0;
        }
        if (hw) {
            const size_t f = (size_t)fi + (size_t)d.ni * ((size_t)fj + (size_t)d.nj * fk);
            const bool ok = Ww > eps;
            fw[f] = ok ? Sw / Ww : Sw;
            vw[f] = ok ? 1 : 0;
        }
    }
}

void launch_p2g3(Dims d, double dx, double radius, const int *cell_start, const float *spx, const float *spy,
                 const float *spz, const float *svx, const float *svy, const float *svz, const float *gpos,
                 const float *bpos, float *u, float *v, float *w, unsigned char *vu, unsigned char *vv,
                 unsigned char *vw, cudaStream_t st) {
    const size_t n = (size_t)(d.ni + 1) * (d.nj + 1) * (d.nk + 1);
    const GridDecode dec = grid_decode(d.ni + 1, d.nj + 1, d.nk + 1);
    k_p2g3<<<grid_for(n, 256, 152u * 64u), 256, 0, st>>>(d, dx, (float)radius, dec, cell_start, spx, spy, spz, svx, svy,
                                                         svz, gpos, bpos, u, v, w, vu, vv, vw);
}

void launch_p2g(Dims d, double dx, double radius, int comp, const int *cell_start, const float *spx,
                const float *spy, const float *spz, const float *svel, const float *gpos, const float *bpos,
                float *field, unsigned char *valid, cudaStream_t st, float *wsum, float *uacc) {
    size_t nf = d.faces(comp);
    float r = (float)radius;
    float sr = (float)(radius + 1e-6f);
    const GridDecode dec = grid_decode(d.ni + (comp == 0), d.nj + (comp == 1), d.nk + (comp == 2));
    if (wsum)
        k_p2g<true><<<grid_for(nf, 256, 152u * 64u), 256, 0, st>>>(d, dx, r, sr, comp, dec, cell_start, spx, spy, spz,
                                                                   svel, gpos, bpos, field, valid, wsum, uacc);
    else
        k_p2g<false><<<grid_for(nf, 256, 152u * 64u), 256, 0, st>>>(d, dx, r, sr, comp, dec, cell_start, spx, spy, spz,
                                                                    svel, gpos, bpos, field, valid, nullptr, nullptr);
}

// ---------------------------------------------------------------------------------
// K7: layered extrapolation (gridutils.h:43-163, gridutils.cpp:99-170).  Status codes:
// 0 unknown, 1 waiting, 2 known, 3 done.  Border cells start done, valid cells known.
// Each layer: known -> done and their unknown 6-neighbours -> waiting (status pass), then
// every waiting cell takes the mean of its done neighbours in +x,-x,+y,-y,+z,-z order and
// becomes known (value pass).  Waiting cells read only done cells, so the value pass is
// race free and matches the reference bit for bit.
// ---------------------------------------------------------------------------------
// Record kept for the transposed extrapolation: layer index (5 bits) and the number of done
// neighbours the value was averaged over, minus one (3 bits); 0xFF = not extrapolated.
__device__ inline unsigned char extrap_record(int layer, int count) {
    return (unsigned char)(layer | ((count - 1) << 5));
}

__global__ void k_extrap_init(int w, int h, int dd, const unsigned char *__restrict__ valid, unsigned char *st) {
    size_t n = (size_t)w * h * dd;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        int i = (int)(t % w), j = (int)((t / w) % h), k = (int)(t / ((size_t)w * h));
        bool border = i == 0 || j == 0 || k == 0 || i == w - 1 || j == h - 1 || k == dd - 1;
        st[t] = border ? 3 : (valid[t] ? 2 : 0);
    }
}

__global__ void k_extrap_status(int w, int h, int dd, const unsigned char *__restrict__ st, unsigned char *st2) {
    size_t n = (size_t)w * h * dd;
    size_t sl = (size_t)w * h;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        unsigned char s = st[t];
        if (s == 2) s = 3;
        else if (s == 0) {
            // unknown cells are never on the border, so all 6 neighbours exist
            if (st[t + 1] == 2 || st[t - 1] == 2 || st[t + w] == 2 || st[t - w] == 2 || st[t + sl] == 2 || st[t - sl] == 2)
                s = 1;
        }
        st2[t] = s;
    }
}

__global__ void k_extrap_value(int w, int h, int dd, unsigned char *st2, float *grid, int last, int layer,
                               unsigned char *layer_of) {
    size_t n = (size_t)w * h * dd;
    size_t sl = (size_t)w * h;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        if (st2[t] != 1) continue;
        float sum = 0.0f;
        int count = 0;
        size_t nb[6] = {t + 1, t - 1, t + w, t - w, t + sl, t - sl};
        for (int q = 0; q < 6; q++)
            if (st2[nb[q]] == 3) { sum += grid[nb[q]]; count++; }
        grid[t] = sum / (float)count;
        if (layer_of) layer_of[t] = extrap_record(layer, count);
        if (!last) st2[t] = 2;
    }
}

void launch_extrapolate(int w, int h, int dd, float *grid, const unsigned char *valid, int layers,
                        unsigned char *status, unsigned char *status2, cudaStream_t st, unsigned char *layer_of) {
    size_t n = (size_t)w * h * dd;
    unsigned int g = grid_for(n, 256, 152u * 32u);
    k_extrap_init<<<g, 256, 0, st>>>(w, h, dd, valid, status);
    if (layer_of) FFGPU_CUDA(cudaMemsetAsync(layer_of, 0xff, n, st));
    unsigned char *a = status, *b = status2;
    for (int l = 0; l < layers; l++) {
        k_extrap_status<<<g, 256, 0, st>>>(w, h, dd, a, b);
        k_extrap_value<<<g, 256, 0, st>>>(w, h, dd, b, grid, l == layers - 1, l, layer_of);
        unsigned char *t = a; a = b; b = t;
    }
}

// K7, frontier form.  Same layers, statuses and per-face arithmetic as above, but after the
// first (dense) status pass only the faces that change are visited: layer l's waiting faces
// are kept in a list, which the next status pass turns done while it claims their unknown
// neighbours (byte compare-and-swap 0 -> 1) into the next list.  A face's value depends only
// on its done neighbours, never on the order in which the list is processed, so the result is
// bit-identical to the dense passes.
__device__ inline bool claim_unknown(unsigned char *st, size_t g) {
    unsigned int *wp = reinterpret_cast<unsigned int *>(reinterpret_cast<uintptr_t>(st + g) & ~(uintptr_t)3);
    const int sh = (int)((reinterpret_cast<uintptr_t>(st + g) & 3) * 8);
    unsigned int old = *reinterpret_cast<volatile unsigned int *>(wp), assumed;
    do {
        if (((old >> sh) & 0xffu) != 0) return false;
        assumed = old;
        old = atomicCAS(wp, assumed, assumed | (1u << sh));
    } while (old != assumed);
    return true;
}

// warp-aggregated append of t to list (every lane of the warp calls it)
__device__ inline void list_append(bool want, unsigned int t, unsigned int *list, unsigned int *count) {
    const unsigned int act = __activemask();
    const unsigned int m = __ballot_sync(act, want);
    if (!m) return;
    const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
    unsigned int base = 0;
    if (lane == leader) base = atomicAdd(count, (unsigned int)__popc(m));
    base = __shfl_sync(act, base, leader);
    if (want) list[base + __popc(m & ((1u << lane) - 1))] = t;
}

// first status pass straight from the valid flags: border and valid faces end done, unknown
// faces next to a valid non-border face become waiting (listed)
__global__ void k_front_first(int w, int h, int dd, const unsigned char *__restrict__ valid, unsigned char *st,
                              unsigned int *list, unsigned int *count) {
    const int lane = threadIdx.x & 31;
    const int gw = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), nw = (int)((gridDim.x * blockDim.x) >> 5);
    const size_t sl = (size_t)w * h;
    for (int rw = gw; rw < h * dd; rw += nw) {
        const int j = rw % h, k = rw / h;
        const size_t row = (size_t)w * rw;
        const bool rowb = j == 0 || k == 0 || j == h - 1 || k == dd - 1;
        for (int i0 = 0; i0 < w; i0 += 32) {
            const int i = i0 + lane;
            bool wait = false;
            if (i < w) {
                const size_t t = row + i;
                unsigned char sv;
                if (rowb || i == 0 || i == w - 1) sv = 3;
                else if (valid[t]) sv = 3;
                else {
                    // a neighbour seeds the layer when it is valid and not on the border
                    wait = (valid[t + 1] && i + 1 != w - 1) || (valid[t - 1] && i - 1 != 0) ||
                           (valid[t + w] && j + 1 != h - 1) || (valid[t - w] && j - 1 != 0) ||
                           (valid[t + sl] && k + 1 != dd - 1) || (valid[t - sl] && k - 1 != 0);
                    sv = wait ? 1 : 0;
                }
                st[t] = sv;
            }
            list_append(wait, (unsigned int)(row + i), list, count);
        }
    }
}

// value pass over the waiting list
__global__ void k_front_values(const unsigned int *__restrict__ list, const unsigned int *__restrict__ count, int w,
                               size_t sl, unsigned char *st, float *grid, int last, int layer,
                               unsigned char *layer_of) {
    const unsigned int n = *count;
    for (unsigned int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const size_t t = list[q];
        float sum = 0.0f;
        int cnt = 0;
        const size_t nb[6] = {t + 1, t - 1, t + w, t - w, t + sl, t - sl};
        for (int e = 0; e < 6; e++)
            if (st[nb[e]] == 3) { sum += grid[nb[e]]; cnt++; }
        grid[t] = sum / (float)cnt;
        if (layer_of) layer_of[t] = extrap_record(layer, cnt);
        if (!last) st[t] = 2;
    }
}

// next status pass: the listed (known) faces become done, their unknown neighbours waiting
__global__ void k_front_advance(const unsigned int *__restrict__ list, const unsigned int *__restrict__ count, int w,
                                size_t sl, unsigned char *st, unsigned int *next, unsigned int *ncount) {
    const unsigned int n = *count;
    const unsigned int stride = gridDim.x * blockDim.x;
    // every lane of a warp runs the same number of rounds (list_append is warp-collective)
    const unsigned int rounds = (n + stride - 1) / stride;
    for (unsigned int rd = 0; rd < rounds; rd++) {
        const unsigned int q = rd * stride + blockIdx.x * blockDim.x + threadIdx.x;
        size_t t = 0;
        bool have = q < n;
        if (have) {
            t = list[q];
            st[t] = 3;
        }
        const long long off[6] = {1, -1, w, -(long long)w, (long long)sl, -(long long)sl};
        for (int e = 0; e < 6; e++) {
            const size_t g = t + off[e];
            const bool got = have && st[g] == 0 && claim_unknown(st, g);
            list_append(got, (unsigned int)g, next, ncount);
        }
    }
}

void launch_extrapolate_front(int w, int h, int dd, float *grid, const unsigned char *valid, int layers, ExtrapFront f,
                              cudaStream_t st, unsigned char *layer_of) {
    const size_t n = (size_t)w * h * dd, sl = (size_t)w * h;
    if (n >= 0xffffffffull) throw std::runtime_error("Error: face grid too large for the extrapolation lists.\n");
    if (layer_of) FFGPU_CUDA(cudaMemsetAsync(layer_of, 0xff, n, st));
    FFGPU_CUDA(cudaMemsetAsync(f.count, 0, 2 * sizeof(unsigned int), st));
    k_front_first<<<grid_for((size_t)h * dd, 256 / 32, 152u * 32u), 256, 0, st>>>(w, h, dd, valid, f.status, f.list[0],
                                                                                    f.count);
    const unsigned int g = 152u * 4u;
    int cur = 0;
    for (int l = 0; l < layers; l++) {
        k_front_values<<<g, 256, 0, st>>>(f.list[cur], f.count + cur, w, sl, f.status, grid, l == layers - 1, l,
                                          layer_of);
        if (l == layers - 1) break;
        FFGPU_CUDA(cudaMemsetAsync(f.count + (1 - cur), 0, sizeof(unsigned int), st));
        k_front_advance<<<g, 256, 0, st>>>(f.list[cur], f.count + cur, w, sl, f.status, f.list[1 - cur],
                                           f.count + (1 - cur));
        cur = 1 - cur;
    }
}

// K8: u += (float)(g * dt) on every face (fluidsimulation.cpp:5837-5876, no inflows).
__global__ void k_add(size_t n, float *f, float a) {
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) f[t] += a;
}

void launch_body_force(size_t n, float *field, float add, cudaStream_t st) {
    k_add<<<grid_for(n, 256), 256, 0, st>>>(n, field, add);
}

// K16: faces with zero open weight take the (static, zero) solid velocity; partially open
// faces keep f*0 + (1-f)*u = u for zero friction (fluidsimulation.cpp:6391-6442).
__global__ void k_constrain(size_t n, const float *__restrict__ wgt, float *f) {
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
        if (wgt[t] == 0.0f) f[t] = 0.0f;
}

void launch_constrain(size_t n, const float *weight, float *field, cudaStream_t st) {
    k_constrain<<<grid_for(n, 256), 256, 0, st>>>(n, weight, field);
}

}  // namespace ffgpu
