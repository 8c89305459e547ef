// Pressure system on the MAC grid: K5 pressure-cell classification, K9 system build,
// K10 MIC(0) factorisation and K15 pressure application.  Dense cell-grid storage; all
// kernels work inside the bounding box of the pressure cells, and every neighbour read
// outside that box is a structural zero.  Compiled with -fmad=false: the FP64 system,
// factor and projection reproduce the reference's rounding step by step.
#include <climits>

#include <cooperative_groups.h>

#include <algorithm>

#include "common.cuh"
#include "kernels.h"
#include "tension.cuh"

namespace ffgpu {
namespace cg = cooperative_groups;

// K5: pressure cells = interior cells (1..n-2 on every axis) with liquid phi < 0,
// pressuresolver.cpp:138-147.  Also reduces their bounding box.
__global__ void k_classify(Dims d, const float *__restrict__ phi, unsigned char *fluid, int *bb) {
    size_t n = d.cells();
    int lo[3] = {INT_MAX, INT_MAX, INT_MAX}, hi[3] = {-1, -1, -1};
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        int i = (int)(t % d.ni), j = (int)((t / d.ni) % d.nj), k = (int)(t / ((size_t)d.ni * d.nj));
        bool f = i >= 1 && j >= 1 && k >= 1 && i < d.ni - 1 && j < d.nj - 1 && k < d.nk - 1 && phi[t] < 0;
        fluid[t] = f ? 1 : 0;
        if (f) {
            lo[0] = min(lo[0], i); lo[1] = min(lo[1], j); lo[2] = min(lo[2], k);
            hi[0] = max(hi[0], i); hi[1] = max(hi[1], j); hi[2] = max(hi[2], k);
        }
    }
    for (int a = 0; a < 3; a++) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[a] = min(lo[a], __shfl_down_sync(0xffffffffu, lo[a], o));
            hi[a] = max(hi[a], __shfl_down_sync(0xffffffffu, hi[a], o));
        }
    }
    if ((threadIdx.x & 31) == 0) {
        for (int a = 0; a < 3; a++) {
            if (hi[a] >= 0) { atomicMin(&bb[a], lo[a]); atomicMax(&bb[3 + a], hi[a]); }
        }
    }
}

void launch_classify(Dims d, const float *phi, unsigned char *fluid, int *bbox6, cudaStream_t st) {
    int init[6] = {INT_MAX, INT_MAX, INT_MAX, -1, -1, -1};
    FFGPU_CUDA(cudaMemcpyAsync(bbox6, init, sizeof(init), cudaMemcpyHostToDevice, st));
    k_classify<<<grid_for(d.cells(), 256), 256, 0, st>>>(d, phi, fluid, bbox6);
    FFGPU_CUDA(cudaGetLastError());
}

struct BoxIt {
    Bbox b;
    int I, J, K;
    __device__ bool in(int i, int j, int k) const {
        return i >= b.i0 && j >= b.j0 && k >= b.k0 && i <= b.i1 && j <= b.j1 && k <= b.k1;
    }
};

inline BoxIt boxit(Bbox b) { return BoxIt{b, b.i1 - b.i0 + 1, b.j1 - b.j0 + 1, b.k1 - b.k0 + 1}; }

// K9: rhs = negative divergence (pressuresolver.cpp:624-713) and matrix coefficients
// (:767-867) for unit density and static solids.  Row c keeps A(c,c) and the couplings
// A(c,c+x), A(c,c+y), A(c,c+z); couplings exist only between two pressure cells.
__global__ void k_build(Dims d, double dx, double dt, BoxIt bx, const float *__restrict__ phi,
                        const float *__restrict__ wu, const float *__restrict__ wv, const float *__restrict__ ww,
                        const float *__restrict__ u, const float *__restrict__ v, const float *__restrict__ w,
                        const unsigned char *__restrict__ fluid, PressureSystem sys, unsigned long long *maxabs,
                        TensionDev ten) {
    size_t n = (size_t)bx.I * bx.J * bx.K;
    const double factor = 1.0 / dx, mfac = dt / (dx * dx), eps = 1e-9, maxtheta = 25;
    double lm = 0.0;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        int i = bx.b.i0 + (int)(t % bx.I), j = bx.b.j0 + (int)((t / bx.I) % bx.J), k = bx.b.k0 + (int)(t / ((size_t)bx.I * bx.J));
        size_t c = flat3(i, j, k, d.ni, d.nj);
        if (!fluid[c]) {
            sys.diag[c] = 0; sys.ax[c] = 0; sys.ay[c] = 0; sys.az[c] = 0; sys.b[c] = 0;
            continue;
        }
        int uw = d.ni + 1, uh = d.nj, vw_ = d.ni, vh = d.nj + 1;
        double vr = wu[flat3(i + 1, j, k, uw, uh)], vl = wu[flat3(i, j, k, uw, uh)];
        double vt = wv[flat3(i, j + 1, k, vw_, vh)], vb = wv[flat3(i, j, k, vw_, vh)];
        double vf = ww[flat3(i, j, k + 1, d.ni, d.nj)], vk = ww[flat3(i, j, k, d.ni, d.nj)];
        double div = 0.0;
        div += -factor * vr * (double)u[flat3(i + 1, j, k, uw, uh)];
        div += factor * vl * (double)u[flat3(i, j, k, uw, uh)];
        div += -factor * vt * (double)v[flat3(i, j + 1, k, vw_, vh)];
        div += factor * vb * (double)v[flat3(i, j, k, vw_, vh)];
        div += -factor * vf * (double)w[flat3(i, j, k + 1, d.ni, d.nj)];
        div += factor * vk * (double)w[flat3(i, j, k, d.ni, d.nj)];
        if (ten.on) {   // surface tension at the air neighbours, +x, -x, +y, -y, +z, -z (pressuresolver.cpp:659-709)
            const double stfactor = dt / (dx * dx);
            const double pcen = phi[c];
            const int ti[6] = {i + 1, i - 1, i, i, i, i}, tj[6] = {j, j, j + 1, j - 1, j, j}, tk[6] = {k, k, k, k, k + 1, k - 1};
            const double tvol[6] = {vr, vl, vt, vb, vf, vk};
            for (int q = 0; q < 6; q++) {
                const double pn = phi[flat3(ti[q], tj[q], tk[q], d.ni, d.nj)];
                if (pn >= 0.0) {
                    const double tension = tension_term(ten, d, dx, i, j, k, ti[q], tj[q], tk[q]);
                    double theta = (pcen - pn) / (pcen + eps);
                    theta = theta < -maxtheta ? -maxtheta : (theta > maxtheta ? maxtheta : theta);
                    div += stfactor * tvol[q] * theta * tension;
                }
            }
        }
        sys.b[c] = div;
        lm = fmax(lm, fabs(div));

        const double rho = 1.0;
        double pc = phi[c];
        double diag = (vr / rho + vl / rho + vt / rho + vb / rho + vf / rho + vk / rho) * mfac;
        const int ni_[6] = {i + 1, i - 1, i, i, i, i}, nj_[6] = {j, j, j + 1, j - 1, j, j}, nk_[6] = {k, k, k, k, k + 1, k - 1};
        const double vol[6] = {vr, vl, vt, vb, vf, vk};
        double cpl[3] = {0.0, 0.0, 0.0};
        for (int q = 0; q < 6; q++) {
            size_t cn = flat3(ni_[q], nj_[q], nk_[q], d.ni, d.nj);
            double pn = phi[cn];
            if (pn < 0.0) {
                // keymap: a liquid neighbour that is not a pressure cell (grid border) adds nothing
                if ((q & 1) == 0 && fluid[cn]) cpl[q >> 1] = -(vol[q] / rho) * mfac;
            } else {
                double th = pn / (pc + eps);
                th = th < -maxtheta ? -maxtheta : (th > maxtheta ? maxtheta : th);
                diag -= (vol[q] / rho) * mfac * th;
            }
        }
        sys.diag[c] = fmax(diag, 0.0);
        sys.ax[c] = cpl[0]; sys.ay[c] = cpl[1]; sys.az[c] = cpl[2];
    }
    for (int o = 16; o > 0; o >>= 1) lm = fmax(lm, __shfl_down_sync(0xffffffffu, lm, o));
    if ((threadIdx.x & 31) == 0) atomicMax(maxabs, (unsigned long long)__double_as_longlong(lm));
}

void launch_build_system(Dims d, double dx, double dt, Bbox bb, const float *phi, const float *wu,
                         const float *wv, const float *ww, const float *u, const float *v, const float *w,
                         PressureSystem sys, double *, unsigned int *, double *maxabs_b, cudaStream_t st,
                         const TensionDev *tension) {
    FFGPU_CUDA(cudaMemsetAsync(maxabs_b, 0, sizeof(double), st));
    BoxIt bx = boxit(bb);
    size_t n = (size_t)bx.I * bx.J * bx.K;
    const TensionDev ten = tension ? *tension : TensionDev{nullptr, nullptr, nullptr, 0.0, 0};
    k_build<<<grid_for(n, 256), 256, 0, st>>>(d, dx, dt, bx, phi, wu, wv, ww, u, v, w, sys.fluid, sys,
                                              (unsigned long long *)maxabs_b, ten);
    FFGPU_CUDA(cudaGetLastError());
}

// K10: modified incomplete Cholesky level 0 (pcgsolver.h:68-205) for the 7-point
// operator, one i+j+k hyperplane of the box per launch.  For each pressure cell the
// pivot receives, in column order (c-z, c-y, c-x), -L^2 and -0.97*L*(sum of the other
// two factor entries of that column), then the 0.25*A(c,c) safeguard.  Column entries:
// L(c+x,c) = A(c,c+x) / sqrt(pivot).
__device__ inline void mic0_level(Dims d, const BoxIt &bx, int level, PressureSystem &sys) {
    int IJ = bx.I * bx.J;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < IJ; t += gridDim.x * blockDim.x) {
        int ii = t % bx.I, jj = t / bx.I, kk = level - ii - jj;
        if (kk < 0 || kk >= bx.K) continue;
        int i = bx.b.i0 + ii, j = bx.b.j0 + jj, k = bx.b.k0 + kk;
        size_t c = flat3(i, j, k, d.ni, d.nj);
        if (!sys.fluid[c]) { sys.inv[c] = 0; sys.lx[c] = 0; sys.ly[c] = 0; sys.lz[c] = 0; continue; }
        const double tau = 0.97, sigma = 0.25;
        double a = sys.diag[c];
        if (a < 1e-9) a = 0;
        double e = a;
        size_t sl = (size_t)d.ni * d.nj;
        if (bx.in(i, j, k - 1) && sys.fluid[c - sl] && sys.diag[c - sl] >= 1e-9) {
            size_t q = c - sl;
            double L = sys.lz[q];
            e -= L * L;
            e -= tau * L * ((0.0 + sys.lx[q]) + sys.ly[q]);
        }
        if (bx.in(i, j - 1, k) && sys.fluid[c - d.ni] && sys.diag[c - d.ni] >= 1e-9) {
            size_t q = c - d.ni;
            double L = sys.ly[q];
            e -= L * L;
            e -= tau * L * ((0.0 + sys.lx[q]) + sys.lz[q]);
        }
        if (bx.in(i - 1, j, k) && sys.fluid[c - 1] && sys.diag[c - 1] >= 1e-9) {
            size_t q = c - 1;
            double L = sys.lx[q];
            e -= L * L;
            e -= tau * L * ((0.0 + sys.ly[q]) + sys.lz[q]);
        }
        double inv;
        if (a == 0) {
            // null row/column: the reference skips this column entirely (pcgsolver.h:148-151),
        // so it neither finalises it nor eliminates it from later columns (checked above)
            inv = e;
            sys.lx[c] = sys.ax[c]; sys.ly[c] = sys.ay[c]; sys.lz[c] = sys.az[c];
        } else {
            inv = (e < sigma * a) ? 1 / sqrt(a) : 1 / sqrt(e);
            sys.lx[c] = sys.ax[c] * inv; sys.ly[c] = sys.ay[c] * inv; sys.lz[c] = sys.az[c] * inv;
        }
        sys.inv[c] = inv;
    }
}

__global__ void k_mic0_level(Dims d, BoxIt bx, int level, PressureSystem sys) { mic0_level(d, bx, level, sys); }

// All hyperplanes in one cooperative launch: the grid synchronises between planes.
__global__ void __launch_bounds__(256) k_mic0_planes(Dims d, BoxIt bx, PressureSystem sys) {
    cg::grid_group g = cg::this_grid();
    const int levels = bx.I + bx.J + bx.K - 2;
    for (int l = 0; l < levels; l++) {
        mic0_level(d, bx, l, sys);
        g.sync();
    }
}

// The same factorization as a tiled wavefront: one CTA per MF_T x MF_T column tile of the box,
// one thread per column, sweeping z on a skewed schedule (cell k of column (tx, ty) at step
// k + tx + ty), so that a cell's -x and -y neighbours were finished one step earlier by the
// neighbouring threads (double-buffered shared memory) and its -z neighbour by itself.  Across
// tile edges the neighbour tile's results are read from global memory once that tile has
// published (release / acquire) a step count of at least s + MF_T + 1: one step more than the
// cell needs, so that the edge threads load the next cell's neighbour values a step ahead.  Every cell performs the
// operations of mic0_level in the same order, so the factor is bit-identical.  The launch is
// cooperative, so all tiles are co-resident; every wait is bounded and raises
// ERR_WAIT_TIMEOUT on expiry, after which all tiles stop.
#ifndef FFGPU_MF_TILE
#define FFGPU_MF_TILE 8
#endif
constexpr int MF_T = FFGPU_MF_TILE;   // tile edge in columns
constexpr long long MF_SPIN_LIMIT = 1 << 22;

__device__ inline unsigned int mf_ld_acquire(const unsigned int *p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ inline void mf_st_release(unsigned int *p, unsigned int v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;\n" ::"l"(p), "r"(v) : "memory");
}

__global__ void __launch_bounds__(MF_T * MF_T) k_mic0_wavefront(Dims d, BoxIt bx, PressureSystem sys, int ntx,
                                                                unsigned int *progress, unsigned int *error,
                                                                long long spin_limit) {
    __shared__ double slx[2][MF_T * MF_T], sly[2][MF_T * MF_T], slz[2][MF_T * MF_T];
    __shared__ int sok[2][MF_T * MF_T];
    __shared__ int stop;
    const int t = threadIdx.x, tx = t % MF_T, ty = t / MF_T;
    const int bxt = blockIdx.x % ntx, byt = blockIdx.x / ntx;
    const int i = bx.b.i0 + MF_T * bxt + tx, j = bx.b.j0 + MF_T * byt + ty;
    const bool col = i <= bx.b.i1 && j <= bx.b.j1;
    const int S = bx.K + 2 * (MF_T - 1);
    const int upx = bxt > 0 ? (int)blockIdx.x - 1 : -1, upy = byt > 0 ? (int)blockIdx.x - ntx : -1;
    const double tau = 0.97, sigma = 0.25;
    unsigned int seen_x = 0, seen_y = 0;
    if (t == 0) stop = 0;
    // the column's previous cell (the -z neighbour of the next one)
    double plx = 0, ply = 0, plz = 0;
    int pok = 0;
    // inputs of the column's next cell, loaded one step ahead
    unsigned char nfl = 0;
    double nd = 0, nax = 0, nay = 0, naz = 0;
    // on the tile's first row / column: the -y / -x neighbour tile's results (ok flag, lx, ly, lz)
    // for plane pyk / pxk, loaded a step ahead
    int pyk = -1, pxk = -1, pyok = 0, pxok = 0;
    double pyq[3] = {0, 0, 0}, pxq[3] = {0, 0, 0};
    auto nb_load = [&](size_t q, int &ok, double (&v)[3]) {
        const unsigned char f = sys.fluid[q];
        const double dd = sys.diag[q];
        v[0] = __ldcg(sys.lx + q); v[1] = __ldcg(sys.ly + q); v[2] = __ldcg(sys.lz + q);
        ok = f && dd >= 1e-9;
    };
    auto fetch = [&](int k) {
        if (col && k >= 0 && k < bx.K) {
            const size_t c = flat3(i, j, bx.b.k0 + k, d.ni, d.nj);
            nfl = sys.fluid[c]; nd = sys.diag[c]; nax = sys.ax[c]; nay = sys.ay[c]; naz = sys.az[c];
        }
    };
    fetch(-tx - ty);
    for (int s = 0; s <= S; s++) {
        __syncthreads();   // step s-1 finished: its shared and global writes are done
        if (t == 0) {
            if ((s & 3) == 0 || s == S) {
                __threadfence();
                mf_st_release(progress + blockIdx.x, (unsigned int)s);
            }
            if (s < S) {
                const unsigned int need = (unsigned int)min(s + MF_T + 1, S);
                long long it = 0;
                while ((upx >= 0 && seen_x < need) || (upy >= 0 && seen_y < need)) {
                    if (upx >= 0 && seen_x < need) seen_x = mf_ld_acquire(progress + upx);
                    if (upy >= 0 && seen_y < need) seen_y = mf_ld_acquire(progress + upy);
                    if ((++it & 63) == 0) {
                        if (it > spin_limit || *((volatile unsigned int *)error) != 0) {
                            atomicOr(error, (unsigned int)ERR_WAIT_TIMEOUT);
                            stop = 1;
                            break;
                        }
                        __nanosleep(32);
                    }
                }
            }
        }
        __syncthreads();   // the neighbour tiles' results for this step are visible
        if (stop || s == S) break;
        const int k = s - tx - ty;
        const int cur = s & 1, prv = cur ^ 1;
        const unsigned char fl = nfl;
        const double dg = nd, ax = nax, ay = nay, az = naz;
        fetch(k + 1);
        if (col && k >= 0 && k < bx.K) {
            const size_t c = flat3(i, j, bx.b.k0 + k, d.ni, d.nj);
            double olx = 0, oly = 0, olz = 0, inv = 0;
            int ook = 0;
            if (fl) {
                double a = dg;
                if (a < 1e-9) a = 0;
                double e = a;
                if (k > 0 && pok) {   // -z
                    const double L = plz;
                    e -= L * L;
                    e -= tau * L * ((0.0 + plx) + ply);
                }
                {   // -y
                    int ok = 0;
                    double qx = 0, qy = 0, qz = 0;
                    if (ty > 0) {
                        ok = sok[prv][t - MF_T]; qx = slx[prv][t - MF_T]; qy = sly[prv][t - MF_T]; qz = slz[prv][t - MF_T];
                    } else if (j - 1 >= bx.b.j0) {
                        if (pyk != k) { nb_load(c - d.ni, pyok, pyq); pyk = k; }
                        ok = pyok;
                        if (ok) { qx = pyq[0]; qy = pyq[1]; qz = pyq[2]; }
                    }
                    if (ok) {
                        const double L = qy;
                        e -= L * L;
                        e -= tau * L * ((0.0 + qx) + qz);
                    }
                }
                {   // -x
                    int ok = 0;
                    double qx = 0, qy = 0, qz = 0;
                    if (tx > 0) {
                        ok = sok[prv][t - 1]; qx = slx[prv][t - 1]; qy = sly[prv][t - 1]; qz = slz[prv][t - 1];
                    } else if (i - 1 >= bx.b.i0) {
                        if (pxk != k) { nb_load(c - 1, pxok, pxq); pxk = k; }
                        ok = pxok;
                        if (ok) { qx = pxq[0]; qy = pxq[1]; qz = pxq[2]; }
                    }
                    if (ok) {
                        const double L = qx;
                        e -= L * L;
                        e -= tau * L * ((0.0 + qy) + qz);
                    }
                }
                if (a == 0) {
                    inv = e;
                    olx = ax; oly = ay; olz = az;
                } else {
                    inv = (e < sigma * a) ? 1 / sqrt(a) : 1 / sqrt(e);
                    olx = ax * inv; oly = ay * inv; olz = az * inv;
                    ook = 1;
                }
            }
            sys.inv[c] = inv; sys.lx[c] = olx; sys.ly[c] = oly; sys.lz[c] = olz;
            sok[cur][t] = ook; slx[cur][t] = olx; sly[cur][t] = oly; slz[cur][t] = olz;
            pok = ook; plx = olx; ply = oly; plz = olz;
        }
        // the neighbour tiles' results for the next cell (their producers finished that plane by step
        // s + MF_T, which the acquire above covers)
        const int kn = k + 1;
        if (col && kn >= 0 && kn < bx.K) {
            const size_t cn = flat3(i, j, bx.b.k0 + kn, d.ni, d.nj);
            if (ty == 0 && j - 1 >= bx.b.j0) { nb_load(cn - d.ni, pyok, pyq); pyk = kn; }
            if (tx == 0 && i - 1 >= bx.b.i0) { nb_load(cn - 1, pxok, pxq); pxk = kn; }
        }
    }
}

// Tiles the wavefront factorization needs for a box of I x J columns.
int mic0_factor_tiles(int I, int J) { return ((I + MF_T - 1) / MF_T) * ((J + MF_T - 1) / MF_T); }

void launch_mic0_factor(Dims d, Bbox bb, PressureSystem sys, unsigned int *progress, unsigned int *error,
                        cudaStream_t st, long long spin_limit) {
    if (spin_limit <= 0) spin_limit = MF_SPIN_LIMIT;
    BoxIt bx = boxit(bb);
    int levels = bx.I + bx.J + bx.K - 2;
    int IJ = bx.I * bx.J;
    {
        static int wf_blocks[64] = {0};   // co-resident wavefront CTAs per device (0: not yet known)
        int dev = 0;
        FFGPU_CUDA(cudaGetDevice(&dev));
        int cap = dev < 64 ? wf_blocks[dev] : 0;
        if (cap == 0) {
            int coop = 0, sms = 0, per = 0;
            FFGPU_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
            FFGPU_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
            FFGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_mic0_wavefront, MF_T * MF_T, 0));
            cap = coop ? std::max(1, sms * per) : -1;
            if (dev < 64) wf_blocks[dev] = cap;
        }
        const int ntx = (bx.I + MF_T - 1) / MF_T, tiles = mic0_factor_tiles(bx.I, bx.J);
        if (progress && cap > 0 && tiles <= cap) {
            FFGPU_CUDA(cudaMemsetAsync(progress, 0, (size_t)tiles * sizeof(unsigned int), st));
            void *args[] = {&d, &bx, &sys, (void *)&ntx, &progress, &error, &spin_limit};
            FFGPU_CUDA(cudaLaunchCooperativeKernel((void *)k_mic0_wavefront, dim3(tiles), dim3(MF_T * MF_T), args, 0,
                                                   st));
            FFGPU_CUDA(cudaGetLastError());
            return;
        }
    }
    static int coop_blocks[64] = {0};   // co-resident blocks per device (0: not yet known)
    int dev = 0;
    FFGPU_CUDA(cudaGetDevice(&dev));
    int maxb = dev < 64 ? coop_blocks[dev] : 0;
    if (maxb == 0) {
        int coop = 0, sms = 0, per = 0;
        FFGPU_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
        FFGPU_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        FFGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_mic0_planes, 256, 0));
        maxb = coop ? std::max(1, sms * per) : -1;
        if (dev < 64) coop_blocks[dev] = maxb;
    }
    if (maxb > 0) {
        unsigned int g = std::min((unsigned int)maxb, grid_for(IJ, 256, 152u * 8u));
        void *args[] = {&d, &bx, &sys};
        FFGPU_CUDA(cudaLaunchCooperativeKernel((void *)k_mic0_planes, dim3(g), dim3(256), args, 0, st));
    } else {
        unsigned int g = grid_for(IJ, 128, 152u * 8u);
        for (int l = 0; l < levels; l++) k_mic0_level<<<g, 128, 0, st>>>(d, bx, l, sys);
    }
    FFGPU_CUDA(cudaGetLastError());
}

// FP32 copies of the operator and factor for the mixed-precision solver.
__global__ void k_to_float(Dims d, BoxIt bx, PressureSystem sys) {
    size_t n = (size_t)bx.I * bx.J * bx.K;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        int i = bx.b.i0 + (int)(t % bx.I), j = bx.b.j0 + (int)((t / bx.I) % bx.J), k = bx.b.k0 + (int)(t / ((size_t)bx.I * bx.J));
        size_t c = flat3(i, j, k, d.ni, d.nj);
        const float dh = (float)sys.diag[c], xh = (float)sys.ax[c], yh = (float)sys.ay[c], zh = (float)sys.az[c];
        sys.diag32[c] = dh; sys.ax32[c] = xh; sys.ay32[c] = yh; sys.az32[c] = zh;
        sys.diag32lo[c] = (float)(sys.diag[c] - (double)dh); sys.ax32lo[c] = (float)(sys.ax[c] - (double)xh);
        sys.ay32lo[c] = (float)(sys.ay[c] - (double)yh); sys.az32lo[c] = (float)(sys.az[c] - (double)zh);
        sys.inv32[c] = (float)sys.inv[c]; sys.lx32[c] = (float)sys.lx[c];
        sys.ly32[c] = (float)sys.ly[c]; sys.lz32[c] = (float)sys.lz[c];
    }
}

void launch_to_float(Dims d, Bbox bb, PressureSystem sys, cudaStream_t st) {
    BoxIt bx = boxit(bb);
    size_t n = (size_t)bx.I * bx.J * bx.K;
    k_to_float<<<grid_for(n, 256), 256, 0, st>>>(d, bx, sys);
}

// K15 (pressuresolver.cpp:1047-1205): tension 0, unit density.  Faces 0 and n-1 along the
// component axis keep their value (as the reference); valid flags are rebuilt.
__global__ void k_apply_pressure(Dims d, float factor, const float *__restrict__ phi, const float *__restrict__ wu,
                                 const float *__restrict__ wv, const float *__restrict__ ww,
                                 const float *__restrict__ pr, float *u, float *v, float *w,
                                 unsigned char *vu, unsigned char *vv, unsigned char *vw, TensionDev ten, double dx) {
    size_t nu = d.faces(0), nv = d.faces(1), nw = d.faces(2);
    size_t total = nu + nv + nw;
    const float eps = 1e-6f;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        int comp;
        size_t q;
        if (t < nu) { comp = 0; q = t; } else if (t < nu + nv) { comp = 1; q = t - nu; } else { comp = 2; q = t - nu - nv; }
        int fw = d.ni + (comp == 0), fh = d.nj + (comp == 1);
        int i = (int)(q % fw), j = (int)((q / fw) % fh), k = (int)(q / ((size_t)fw * fh));
        int ax = comp == 0 ? i : (comp == 1 ? j : k);
        int na = comp == 0 ? d.ni : (comp == 1 ? d.nj : d.nk);
        float *vel = comp == 0 ? u : (comp == 1 ? v : w);
        unsigned char *val = comp == 0 ? vu : (comp == 1 ? vv : vw);
        const float *wg = comp == 0 ? wu : (comp == 1 ? wv : ww);
        val[q] = 0;
        if (ax == 0 || ax == na - 1) continue;
        int i1 = i - (comp == 0), j1 = j - (comp == 1), k1 = k - (comp == 2);
        bool in2 = ax < na;   // upper cell exists
        size_t c1 = flat3(i1, j1, k1, d.ni, d.nj);
        size_t c2 = in2 ? flat3(i, j, k, d.ni, d.nj) : c1;
        bool f1 = phi[c1] < 0.0, f2 = in2 && phi[c2] < 0.0;
        if (wg[q] > 0 && (f1 || f2)) {
            float p1, p2;
            if (f1 && f2) { p1 = pr[c1]; p2 = pr[c2]; }
            else {
                float phi1 = phi[c1], phi2 = in2 ? phi[c2] : 1.0f;
                // p_ghost = thetaTension * tension + thetaPressure * p, evaluated in double as the
                // reference (keeps the sign of zero identical); the tension term of the face's lower
                // and upper cell, in that order (:1076, :1127, :1177), 0 without surface tension
                const double tension = (ten.on && in2) ? tension_term(ten, d, dx, i1, j1, k1, i, j, k) : 0.0;
                if (f1) {
                    float th = phi2 / (phi1 + eps);
                    th = (float)fmin(fmax((double)th, -25.0), 25.0);
                    float tt = (phi1 - phi2) / (phi1 + eps);
                    tt = (float)fmin(fmax((double)tt, -25.0), 25.0);
                    p1 = pr[c1];
                    p2 = (float)((double)tt * tension + (double)(th * p1));
                } else {
                    float th = phi1 / (phi2 + eps);
                    th = (float)fmin(fmax((double)th, -25.0), 25.0);
                    float tt = (phi2 - phi1) / (phi2 + eps);
                    tt = (float)fmin(fmax((double)tt, -25.0), 25.0);
                    p2 = pr[c2];
                    p1 = (float)((double)tt * tension + (double)(th * p2));
                }
            }
            float rho = (1.0f + 1.0f) / 2.0f;
            vel[q] += -factor * (p2 - p1) / rho;
            val[q] = 1;
        } else {
            vel[q] = 0.0f;
        }
    }
}

void launch_apply_pressure(Dims d, double dx, double dt, const float *phi, const float *wu, const float *wv,
                           const float *ww, const float *pressure, float *u, float *v, float *w,
                           unsigned char *vu, unsigned char *vv, unsigned char *vw, cudaStream_t st,
                           const TensionDev *tension) {
    size_t total = d.faces(0) + d.faces(1) + d.faces(2);
    const TensionDev ten = tension ? *tension : TensionDev{nullptr, nullptr, nullptr, 0.0, 0};
    k_apply_pressure<<<grid_for(total, 256), 256, 0, st>>>(d, (float)(dt / dx), phi, wu, wv, ww, pressure, u, v,
                                                           w, vu, vv, vw, ten, dx);
}

// ---- diagnostics: errors of a solve against an FP64 reference solve ----

// Largest |D_c| over the pressure cells, D_c = (1/dx) * sum over the six faces of +-w_f u_f:
// the weighted divergence the rhs holds before the solve (pressuresolver.cpp:624-713) and the
// residual the projection leaves after it.  Stored as the bits of a non-negative double.
__global__ void k_divergence_max(Dims d, double dx, const unsigned char *__restrict__ fluid,
                                 const float *__restrict__ wu, const float *__restrict__ wv,
                                 const float *__restrict__ ww, const float *__restrict__ u,
                                 const float *__restrict__ v, const float *__restrict__ w,
                                 unsigned long long *maxbits) {
    const double factor = 1.0 / dx;
    double m = 0.0;
    const size_t n = d.cells();
    const int uw = d.ni + 1, uh = d.nj, vw_ = d.ni, vh = d.nj + 1;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        if (!fluid[t]) continue;
        const int i = (int)(t % d.ni), j = (int)((t / d.ni) % d.nj), k = (int)(t / ((size_t)d.ni * d.nj));
        double div = 0.0;
        div += factor * (double)wu[flat3(i + 1, j, k, uw, uh)] * (double)u[flat3(i + 1, j, k, uw, uh)];
        div -= factor * (double)wu[flat3(i, j, k, uw, uh)] * (double)u[flat3(i, j, k, uw, uh)];
        div += factor * (double)wv[flat3(i, j + 1, k, vw_, vh)] * (double)v[flat3(i, j + 1, k, vw_, vh)];
        div -= factor * (double)wv[flat3(i, j, k, vw_, vh)] * (double)v[flat3(i, j, k, vw_, vh)];
        div += factor * (double)ww[flat3(i, j, k + 1, d.ni, d.nj)] * (double)w[flat3(i, j, k + 1, d.ni, d.nj)];
        div -= factor * (double)ww[flat3(i, j, k, d.ni, d.nj)] * (double)w[flat3(i, j, k, d.ni, d.nj)];
        m = fmax(m, fabs(div));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(maxbits, (unsigned long long)__double_as_longlong(m));
}

double divergence_max(Dims d, double dx, const unsigned char *fluid, const float *wu, const float *wv,
                      const float *ww, const float *u, const float *v, const float *w,
                      unsigned long long *maxbits, double *host, cudaStream_t st) {
    FFGPU_CUDA(cudaMemsetAsync(maxbits, 0, sizeof(unsigned long long), st));
    k_divergence_max<<<grid_for(d.cells(), 256), 256, 0, st>>>(d, dx, fluid, wu, wv, ww, u, v, w, maxbits);
    FFGPU_CUDA(cudaGetLastError());
    FFGPU_CUDA(cudaMemcpyAsync(host, maxbits, sizeof(double), cudaMemcpyDeviceToHost, st));
    FFGPU_CUDA(cudaStreamSynchronize(st));
    return host[0];
}

// Per block: sum over t with mask[t] != 0 (every t when mask is null) of (a - b)^2 and b^2.
constexpr int DIFF_BLOCKS = 1024;
template <typename A, typename B>
__global__ void k_diff_sq(size_t n, const A *__restrict__ a, const B *__restrict__ b,
                          const unsigned char *__restrict__ mask, double *part) {
    double e2 = 0.0, r2 = 0.0;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        if (mask && !mask[t]) continue;
        const double bt = (double)b[t], dt_ = (double)a[t] - bt;
        e2 += dt_ * dt_;
        r2 += bt * bt;
    }
    __shared__ double s[2][32];
    for (int o = 16; o > 0; o >>= 1) {
        e2 += __shfl_down_sync(0xffffffffu, e2, o);
        r2 += __shfl_down_sync(0xffffffffu, r2, o);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { s[0][wid] = e2; s[1][wid] = r2; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double te = 0.0, tr = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) { te += s[0][q]; tr += s[1][q]; }
        part[2 * blockIdx.x] = te;
        part[2 * blockIdx.x + 1] = tr;
    }
}

template <typename A, typename B>
void diff_sq(size_t n, const A *a, const B *b, const unsigned char *mask, double *part, double *host_part,
             double &e2, double &r2, cudaStream_t st) {
    e2 = 0.0; r2 = 0.0;
    if (n == 0) return;
    const int blocks = (int)std::min<size_t>(DIFF_BLOCKS, (n + 255) / 256);
    k_diff_sq<A, B><<<blocks, 256, 0, st>>>(n, a, b, mask, part);
    FFGPU_CUDA(cudaGetLastError());
    FFGPU_CUDA(cudaMemcpyAsync(host_part, part, 2 * blocks * sizeof(double), cudaMemcpyDeviceToHost, st));
    FFGPU_CUDA(cudaStreamSynchronize(st));
    for (int q = 0; q < blocks; q++) { e2 += host_part[2 * q]; r2 += host_part[2 * q + 1]; }
}
template void diff_sq<double, double>(size_t, const double *, const double *, const unsigned char *, double *,
                                      double *, double &, double &, cudaStream_t);
template void diff_sq<float, float>(size_t, const float *, const float *, const unsigned char *, double *, double *,
                                    double &, double &, cudaStream_t);

}  // namespace ffgpu
