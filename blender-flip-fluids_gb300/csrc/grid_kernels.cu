// Grid-side kernels of the FLIP substep: solid level set of the closed domain, face
// weights, near-solid coarse grid, and the liquid signed distance field (K4) with its
// post-process.  Compiled with -fmad=false: every float/double expression here follows
// the reference engine's rounding step by step (no fused multiply-add).
#include <cmath>

#include "common.cuh"
#include "kernels.h"

namespace ffgpu {

// ---------------------------------------------------------------------------------
// Solid level set: closed domain box (inset as FluidSimulation::_getBoundaryAABB,
// fluidsimulation.cpp:5175-5180) unioned with analytic spheres.  Positive inside the
// fluid region, negative in solids; nodal (ni+1)(nj+1)(nk+1).
// ---------------------------------------------------------------------------------
__global__ void k_solid_phi(Dims d, double dx, float lox, float loy, float loz,
                            double hix, double hiy, double hiz, int nsph, SphereList sph, float *phi) {
    int w = d.ni + 1, h = d.nj + 1;
    size_t n = (size_t)w * h * (d.nk + 1);
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        int i = (int)(t % w), j = (int)((t / w) % h), k = (int)(t / ((size_t)w * h));
        double x[3] = {(double)i * dx, (double)j * dx, (double)k * dx};
        double lo[3] = {lox, loy, loz}, hi[3] = {hix, hiy, hiz};
        double din = 1e30, dout2 = 0.0;
        bool inside = true;
        for (int a = 0; a < 3; a++) {
            double dl = x[a] - lo[a], dh = hi[a] - x[a];
            din = fmin(din, fmin(dl, dh));
            if (dl < 0) { inside = false; dout2 += dl * dl; }
            if (dh < 0) { inside = false; dout2 += dh * dh; }
        }
        double v = inside ? din : -sqrt(dout2);
        for (int s = 0; s < nsph; s++) {
            double ex = x[0] - sph.s[s][0], ey = x[1] - sph.s[s][1], ez = x[2] - sph.s[s][2];
            v = fmin(v, sqrt(ex * ex + ey * ey + ez * ez) - sph.s[s][3]);
        }
        phi[t] = (float)v;
    }
}

void launch_solid_phi(Dims d, double dx, const SphereList &sph, int nsph, float *phi, cudaStream_t st) {
    // boundary box: AABB(0,0,0, n*dx).expand(-3dx - 1e-4) -> shift by half (aabb.cpp:122-128)
    double hv = 0.5 * (-3 * dx - 1e-4);
    float lo = 0.0f - (float)hv;
    double wi = d.ni * dx + (-3 * dx - 1e-4), wj = d.nj * dx + (-3 * dx - 1e-4), wk = d.nk * dx + (-3 * dx - 1e-4);
    double hix = (double)(float)(lo + wi), hiy = (double)(float)(lo + wj), hiz = (double)(float)(lo + wk);
    size_t n = (size_t)(d.ni + 1) * (d.nj + 1) * (d.nk + 1);
    k_solid_phi<<<grid_for(n, 256), 256, 0, st>>>(d, dx, lo, lo, lo, hix, hiy, hiz, nsph, sph, phi);
}

__global__ void k_unite_spheres(Dims d, double dx, int nsph, SphereList sph, float *phi) {
    const int w = d.ni + 1, h = d.nj + 1;
    const size_t n = (size_t)w * h * (d.nk + 1);
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(t % w), j = (int)((t / w) % h), k = (int)(t / ((size_t)w * h));
        const double x = (double)i * dx, y = (double)j * dx, z = (double)k * dx;
        double v = phi[t];
        for (int s = 0; s < nsph; s++) {
            const double ex = x - sph.s[s][0], ey = y - sph.s[s][1], ez = z - sph.s[s][2];
            v = fmin(v, sqrt(ex * ex + ey * ey + ez * ez) - sph.s[s][3]);
        }
        phi[t] = (float)v;
    }
}

void launch_unite_spheres(Dims d, double dx, const SphereList &sph, int nsph, float *phi, cudaStream_t st) {
    const size_t n = (size_t)(d.ni + 1) * (d.nj + 1) * (d.nk + 1);
    k_unite_spheres<<<grid_for(n, 256), 256, 0, st>>>(d, dx, nsph, sph, phi);
}

// ---------------------------------------------------------------------------------
// Face weights: 1 - fractionInside of the 4 solid corners, clamped to [0,1]
// (fluidsimulation.cpp:6110-6150, meshlevelset.cpp:357-395, levelsetutils.cpp:39-141).
// ---------------------------------------------------------------------------------
__device__ inline float frac2(float l, float r) {
    if (l < 0 && r < 0) return 1;
    if (l < 0 && r >= 0) return l / (l - r);
    if (l >= 0 && r < 0) return r / (r - l);
    return 0;
}

__device__ inline void cycle4(float *a) { float t = a[0]; a[0] = a[1]; a[1] = a[2]; a[2] = a[3]; a[3] = t; }

__device__ float frac4(float bl, float br, float tl, float tr) {
    int inside = (bl < 0) + (tl < 0) + (br < 0) + (tr < 0);
    float L[4] = {bl, br, tr, tl};
    if (inside == 4) return 1;
    if (inside == 3) {
        for (int g = 0; g < 4 && L[0] < 0; g++) cycle4(L);
        float s0 = 1 - frac2(L[0], L[3]);
        float s1 = 1 - frac2(L[0], L[1]);
        return 1.0f - 0.5f * s0 * s1;
    }
    if (inside == 2) {
        for (int g = 0; g < 4 && (L[0] >= 0 || !(L[1] < 0 || L[2] < 0)); g++) cycle4(L);
        if (L[1] < 0) return 0.5f * (frac2(L[0], L[3]) + frac2(L[1], L[2]));
        float mid = 0.25f * (L[0] + L[1] + L[2] + L[3]);
        if (mid < 0) {
            float area = 0;
            float s1 = 1 - frac2(L[0], L[3]);
            float s3 = 1 - frac2(L[2], L[3]);
            area += 0.5f * s1 * s3;
            float s2 = 1 - frac2(L[2], L[1]);
            float s0 = 1 - frac2(L[0], L[1]);
            area += 0.5f * s0 * s2;
            return 1.0f - area;
        }
        float area = 0;
        float s0 = frac2(L[0], L[1]);
        float s1 = frac2(L[0], L[3]);
        area += 0.5f * s0 * s1;
        float s2 = frac2(L[2], L[1]);
        float s3 = frac2(L[2], L[3]);
        area += 0.5f * s2 * s3;
        return area;
    }
    if (inside == 1) {
        for (int g = 0; g < 4 && L[0] >= 0; g++) cycle4(L);
        return 0.5f * frac2(L[0], L[3]) * frac2(L[0], L[1]);
    }
    return 0;
}

__device__ inline float clamp01(float x) { return x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x); }

__global__ void k_face_weights(Dims d, const float *__restrict__ s, float *wu, float *wv, float *ww) {
    int sw = d.ni + 1, sh = d.nj + 1;
    size_t nu = d.faces(0), nv = d.faces(1), nw = d.faces(2);
    size_t total = nu + nv + nw;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        if (t < nu) {
            int w = d.ni + 1, h = d.nj;
            int i = (int)(t % w), j = (int)((t / w) % h), k = (int)(t / ((size_t)w * h));
            wu[t] = clamp01(1.0f - frac4(s[flat3(i, j, k, sw, sh)], s[flat3(i, j + 1, k, sw, sh)],
                                         s[flat3(i, j, k + 1, sw, sh)], s[flat3(i, j + 1, k + 1, sw, sh)]));
        } else if (t < nu + nv) {
            size_t q = t - nu;
            int w = d.ni, h = d.nj + 1;
            int i = (int)(q % w), j = (int)((q / w) % h), k = (int)(q / ((size_t)w * h));
            wv[q] = clamp01(1.0f - frac4(s[flat3(i, j, k, sw, sh)], s[flat3(i, j, k + 1, sw, sh)],
                                         s[flat3(i + 1, j, k, sw, sh)], s[flat3(i + 1, j, k + 1, sw, sh)]));
        } else {
            size_t q = t - nu - nv;
            int w = d.ni, h = d.nj;
            int i = (int)(q % w), j = (int)((q / w) % h), k = (int)(q / ((size_t)w * h));
            ww[q] = clamp01(1.0f - frac4(s[flat3(i, j, k, sw, sh)], s[flat3(i, j + 1, k, sw, sh)],
                                         s[flat3(i + 1, j, k, sw, sh)], s[flat3(i + 1, j + 1, k, sw, sh)]));
        }
    }
}

void launch_face_weights(Dims d, const float *solid, float *wu, float *wv, float *ww, cudaStream_t st) {
    size_t total = d.faces(0) + d.faces(1) + d.faces(2);
    k_face_weights<<<grid_for(total, 256), 256, 0, st>>>(d, solid, wu, wv, ww);
}

// ---------------------------------------------------------------------------------
// Near-solid coarse grid (fluidsimulation.cpp:5448-5480): coarse cell (3 dx) is marked
// when a node it covers has |solid phi| < 3 dx, then dilated over 6 neighbours
// ceil(CFL/3) times.
// ---------------------------------------------------------------------------------
__global__ void k_near_mark(Dims d, double dx, NearGrid ng, const float *__restrict__ s, unsigned char *g) {
    float maxd = (float)(3 * dx);
    size_t n = d.cells();
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        int i = (int)(t % d.ni), j = (int)((t / d.ni) % d.nj), k = (int)(t / ((size_t)d.ni * d.nj));
        if (fabsf(s[flat3(i, j, k, d.ni + 1, d.nj + 1)]) < maxd)
            g[flat3(i / 3, j / 3, k / 3, ng.w, ng.h)] = 1;   // benign same-value race
    }
}

__global__ void k_near_dilate(NearGrid ng, const unsigned char *src, unsigned char *dst) {
    size_t n = (size_t)ng.w * ng.h * ng.d;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        int i = (int)(t % ng.w), j = (int)((t / ng.w) % ng.h), k = (int)(t / ((size_t)ng.w * ng.h));
        unsigned char v = src[t];
        if (!v) {
            if (i > 0 && src[t - 1]) v = 1;
            else if (i < ng.w - 1 && src[t + 1]) v = 1;
            else if (j > 0 && src[t - ng.w]) v = 1;
            else if (j < ng.h - 1 && src[t + ng.w]) v = 1;
            else if (k > 0 && src[t - (size_t)ng.w * ng.h]) v = 1;
            else if (k < ng.d - 1 && src[t + (size_t)ng.w * ng.h]) v = 1;
        }
        dst[t] = v;
    }
}

void launch_near_solid(Dims d, double dx, int cfl, const float *solid, NearGrid ng, unsigned char *g,
                       unsigned char *tmp, cudaStream_t st) {
    size_t n = (size_t)ng.w * ng.h * ng.d;
    FFGPU_CUDA(cudaMemsetAsync(g, 0, n, st));
    k_near_mark<<<grid_for(d.cells(), 256), 256, 0, st>>>(d, dx, ng, solid, g);
    int layers = (int)ceilf((float)cfl / 3.0f);
    for (int l = 0; l < layers; l++) {
        k_near_dilate<<<grid_for(n, 256), 256, 0, st>>>(ng, g, tmp);
        FFGPU_CUDA(cudaMemcpyAsync(g, tmp, n, cudaMemcpyDeviceToDevice, st));
    }
}

// ---------------------------------------------------------------------------------
// K4 liquid SDF (particlelevelset.cpp:335-666, post-process :170-194).  The reference
// assigns each particle to the 10^3 cell blocks of its block frame that its search box
// touches (:507-551) and keeps, per cell of a block, the minimum of |c - p| - r over the
// assigned particles whose cell window covers the cell, all in block-local float arithmetic
// (:618-666).  Here one CTA per block gathers that minimum per cell (a minimum does not
// depend on the order of its terms, so the result is bit-identical).  A cell visits the
// particles whose sort cell lies within `reach` cells of it (and inside the block's
// candidate region); those in the 3x3x3 neighbourhood go first, and since a particle two or
// more cells away lies at least 1.5 cells from the cell centre, the outer shell is visited
// only while the minimum is not yet below 1.5 dx - r.  The post-process against the solid
// level set is fused into the write-back.
//
// Each particle's assignment and windows do not depend on the cell, so a first pass packs
// them into 64 bits per particle (cell-sorted order):
//   bits  0-20  first assigned block index per axis (7 bits each, x, y, z)
//   bits 21-23  whether the particle is also assigned to the next block, per axis
//   bits 24-53  per axis a and block slot s (first / next block), 5 bits at 24 + 5 (2a + s):
//               low 4 bits = first window cell + 4 (block-local), bit 4 = last - first - 3
//   bit  63     the decision does not fit this form; the gather evaluates the pair directly
// ---------------------------------------------------------------------------------
constexpr int SDF_BW = 10;

struct SdfFrame {
    int A, B, C;
    float sr, r, fblockdx, inv_fbf, inv_dxf, ox, oy, oz;
    double inv_fb, inv_dx;
};

__device__ inline void sdf_pair(const SdfFrame &f, const float *cc, int li, int lj, int lk, float x, float y, float z,
                                int &best) {
    const int a = floor_fd(x, f.inv_fb, f.inv_fbf), b = floor_fd(y, f.inv_fb, f.inv_fbf), c = floor_fd(z, f.inv_fb, f.inv_fbf);
    const float bx = (float)a * f.fblockdx, by = (float)b * f.fblockdx, bz = (float)c * f.fblockdx;
    bool assigned;
    if (x - f.sr > bx && y - f.sr > by && z - f.sr > bz && x + f.sr < bx + f.fblockdx && y + f.sr < by + f.fblockdx &&
        z + f.sr < bz + f.fblockdx) {
        assigned = (a == f.A && b == f.B && c == f.C);
    } else {
        assigned = floor_fd(x - f.sr, f.inv_fb, f.inv_fbf) <= f.A && f.A <= floor_fd(x + f.sr, f.inv_fb, f.inv_fbf) &&
                   floor_fd(y - f.sr, f.inv_fb, f.inv_fbf) <= f.B && f.B <= floor_fd(y + f.sr, f.inv_fb, f.inv_fbf) &&
                   floor_fd(z - f.sr, f.inv_fb, f.inv_fbf) <= f.C && f.C <= floor_fd(z + f.sr, f.inv_fb, f.inv_fbf);
    }
    if (!assigned) return;
    const float lx = x - f.ox, ly = y - f.oy, lz = z - f.oz;
    if (floor_fd(lx - f.sr, f.inv_dx, f.inv_dxf) > li || floor_fd(lx + f.sr, f.inv_dx, f.inv_dxf) < li) return;
    if (floor_fd(ly - f.sr, f.inv_dx, f.inv_dxf) > lj || floor_fd(ly + f.sr, f.inv_dx, f.inv_dxf) < lj) return;
    if (floor_fd(lz - f.sr, f.inv_dx, f.inv_dxf) > lk || floor_fd(lz + f.sr, f.inv_dx, f.inv_dxf) < lk) return;
    const float vx = cc[li] - lx, vy = cc[lj] - ly, vz = cc[lk] - lz;
    const float dist = __fsqrt_rn(vx * vx + vy * vy + vz * vz) - f.r;
    best = min(best, float_to_ordered(dist));
}

// The block-independent part of the frame.
__host__ __device__ inline void sdf_frame_common(SdfFrame &f, double dx, float r) {
    f.sr = 2.0f * r;
    f.r = r;
    f.fblockdx = (float)(SDF_BW * dx);
    f.inv_fb = 1.0 / (double)f.fblockdx;
    f.inv_fbf = (float)f.inv_fb;
    f.inv_dx = 1.0 / dx;
    f.inv_dxf = (float)f.inv_dx;
}

constexpr unsigned long long SDF_REC_EXACT = 1ull << 63;

// Packs one particle's block assignment and per-block cell windows (layout above) with the
// same expressions sdf_pair evaluates.
__global__ void k_sdf_records(SdfFrame f, double bdx, int np, const float *__restrict__ spx,
                              const float *__restrict__ spy, const float *__restrict__ spz, unsigned long long *rec) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < np; q += gridDim.x * blockDim.x) {
        const float p[3] = {spx[q], spy[q], spz[q]};
        int a[3], lo[3], hi[3];
        for (int ax = 0; ax < 3; ax++) a[ax] = floor_fd(p[ax], f.inv_fb, f.inv_fbf);
        bool interior = true;
        for (int ax = 0; ax < 3; ax++) {
            const float b0 = (float)a[ax] * f.fblockdx;
            interior = interior && p[ax] - f.sr > b0 && p[ax] + f.sr < b0 + f.fblockdx;
        }
        for (int ax = 0; ax < 3; ax++) {
            lo[ax] = interior ? a[ax] : floor_fd(p[ax] - f.sr, f.inv_fb, f.inv_fbf);
            hi[ax] = interior ? a[ax] : floor_fd(p[ax] + f.sr, f.inv_fb, f.inv_fbf);
        }
        unsigned long long R = 0;
        bool exact = false;
        for (int ax = 0; ax < 3; ax++) {
            const int span = hi[ax] - lo[ax];
            if (lo[ax] + 1 < 0 || lo[ax] + 1 > 127 || span < 0 || span > 1) { exact = true; break; }
            R |= (unsigned long long)(lo[ax] + 1) << (7 * ax);
            R |= (unsigned long long)span << (21 + ax);
            for (int sl = 0; sl <= span; sl++) {
                const int A = lo[ax] + sl;
                if (A < 0) continue;   // no block of the grid; never asked for
                const float o = (float)((double)(float)A * bdx);
                const float l = p[ax] - o;
                const int wlo = floor_fd(l - f.sr, f.inv_dx, f.inv_dxf), whi = floor_fd(l + f.sr, f.inv_dx, f.inv_dxf);
                if (wlo < -4 || wlo > 11 || whi - wlo < 3 || whi - wlo > 4) { exact = true; break; }
                R |= (unsigned long long)((wlo + 4) | ((whi - wlo - 3) << 4)) << (24 + 5 * (2 * ax + sl));
            }
            if (exact) break;
        }
        rec[q] = exact ? SDF_REC_EXACT : R;
    }
}

// the rare pairs whose particle record could not be packed
static __device__ __noinline__ int sdf_pair_slow(SdfFrame f, const float *cc, int li, int lj, int lk, float x, float y,
                                                 float z, int best) {
    sdf_pair(f, cc, li, lj, lk, x, y, z, best);
    return best;
}

// sdf_pair with the assignment and window decisions read from the particle's record
__device__ inline void sdf_pair_rec(const SdfFrame &f, const float *cc, int li, int lj, int lk, int q,
                                    const float *__restrict__ spx, const float *__restrict__ spy,
                                    const float *__restrict__ spz, const unsigned long long *__restrict__ rec,
                                    int &best) {
    const unsigned long long R = __ldg(rec + q);
    if (R & SDF_REC_EXACT) {
        best = sdf_pair_slow(f, cc, li, lj, lk, __ldg(spx + q), __ldg(spy + q), __ldg(spz + q), best);
        return;
    }
    const unsigned sx = (unsigned)(f.A + 1 - (int)(R & 127)), sy = (unsigned)(f.B + 1 - (int)((R >> 7) & 127)),
                   sz = (unsigned)(f.C + 1 - (int)((R >> 14) & 127));
    if (sx > ((R >> 21) & 1) || sy > ((R >> 22) & 1) || sz > ((R >> 23) & 1)) return;
    const int wx = (int)(R >> (24 + 5 * sx)) & 31, wy = (int)(R >> (34 + 5 * sy)) & 31,
              wz = (int)(R >> (44 + 5 * sz)) & 31;
    const int xlo = (wx & 15) - 4, ylo = (wy & 15) - 4, zlo = (wz & 15) - 4;
    if (li < xlo || li > xlo + 3 + (wx >> 4) || lj < ylo || lj > ylo + 3 + (wy >> 4) || lk < zlo ||
        lk > zlo + 3 + (wz >> 4))
        return;
    const float lx = __ldg(spx + q) - f.ox, ly = __ldg(spy + q) - f.oy, lz = __ldg(spz + q) - f.oz;
    const float vx = cc[li] - lx, vy = cc[lj] - ly, vz = cc[lk] - lz;
    const float dist = __fsqrt_rn(vx * vx + vy * vy + vz * vz) - f.r;
    best = min(best, float_to_ordered(dist));
}

__global__ void __launch_bounds__(256) k_liquid_sdf_gather(Dims d, double dx, float r, int reach,
                                                           const int *__restrict__ cell_start,
                                                           const float *__restrict__ spx, const float *__restrict__ spy,
                                                           const float *__restrict__ spz,
                                                           const unsigned long long *__restrict__ rec,
                                                           const float *__restrict__ solid, int do_post, float *phi) {
    __shared__ float cc[SDF_BW];
    __shared__ int any;
    const int nbi = (d.ni + SDF_BW - 1) / SDF_BW, nbj = (d.nj + SDF_BW - 1) / SDF_BW;
    SdfFrame f;
    f.A = blockIdx.x % nbi; f.B = (blockIdx.x / nbi) % nbj; f.C = blockIdx.x / (nbi * nbj);
    const float maxd = (float)(3.0 * dx);
    const int imaxd = float_to_ordered(maxd);
    const double hw = 0.5 * dx;
    if (threadIdx.x < SDF_BW) cc[threadIdx.x] = (float)((double)(float)threadIdx.x * dx + hw);
    if (threadIdx.x == 0) any = 0;
    // the block's candidate region (cells within two of the block), clipped to the grid
    const int ri0 = max(SDF_BW * f.A - 2, 0), ri1 = min(SDF_BW * f.A + SDF_BW + 1, d.ni - 1);
    const int rj0 = max(SDF_BW * f.B - 2, 0), rj1 = min(SDF_BW * f.B + SDF_BW + 1, d.nj - 1);
    const int rk0 = max(SDF_BW * f.C - 2, 0), rk1 = min(SDF_BW * f.C + SDF_BW + 1, d.nk - 1);
    __syncthreads();
    {   // skip blocks without a particle in the region
        const int nh = rj1 - rj0 + 1, nrow = nh * (rk1 - rk0 + 1);
        int found = 0;
        for (int rw = threadIdx.x; rw < nrow; rw += blockDim.x) {
            const size_t c = flat3(ri0, rj0 + rw % nh, rk0 + rw / nh, d.ni, d.nj);
            found |= cell_start[c + (ri1 - ri0 + 1)] > cell_start[c];
        }
        if (__syncthreads_or(found) && threadIdx.x == 0) any = 1;
        __syncthreads();
    }
    sdf_frame_common(f, dx, r);
    const double bdx = SDF_BW * dx;
    f.ox = (float)((double)(float)f.A * bdx); f.oy = (float)((double)(float)f.B * bdx); f.oz = (float)((double)(float)f.C * bdx);
    // a particle whose sort cell is two or more cells away gives at least this distance
    const int ibound = float_to_ordered((float)(1.5 * dx) - r - (float)(1e-4 * dx));
    // and one in a neighbouring sort cell at least this one (half a cell from the centre)
    const int iface = float_to_ordered((float)(0.5 * dx) - r - (float)(1e-4 * dx));
    const float eps = (float)(0.005 * dx);
    const int sw = d.ni + 1, sh = d.nj + 1;
    for (int t = threadIdx.x; t < SDF_BW * SDF_BW * SDF_BW; t += blockDim.x) {
        const int li = t % SDF_BW, lj = (t / SDF_BW) % SDF_BW, lk = t / (SDF_BW * SDF_BW);
        const int gi = f.A * SDF_BW + li, gj = f.B * SDF_BW + lj, gk = f.C * SDF_BW + lk;
        if (gi >= d.ni || gj >= d.nj || gk >= d.nk) continue;
        int best = imaxd;
        if (any) {
            // rows of sort cells [x0, x1] x {jj} x {kk}; `shell` excludes the inner x range (gi +- 1) on
            // the inner rows, `hole` the target's own sort cell on its row
            auto scan = [&](int x0, int x1, int y0, int y1, int z0, int z1, bool shell, bool hole) {
                for (int kk = z0; kk <= z1; kk++)
                    for (int jj = y0; jj <= y1; jj++) {
                        const bool inner = shell && kk >= gk - 1 && kk <= gk + 1 && jj >= gj - 1 && jj <= gj + 1;
                        const bool own = hole && kk == gk && jj == gj;
                        const size_t row = flat3(0, jj, kk, d.ni, d.nj);
                        // one or two particle ranges of the row
                        int ra0 = x0, ra1 = x1, rb0 = 1, rb1 = 0;
                        if (inner) { ra1 = gi - 2; rb0 = gi + 2; rb1 = x1; }
                        if (own) { ra1 = gi - 1; rb0 = gi + 1; rb1 = x1; }
                        if (ra0 <= ra1)
                            for (int p = cell_start[row + ra0], pe = cell_start[row + ra1 + 1]; p < pe; p++)
                                sdf_pair_rec(f, cc, li, lj, lk, p, spx, spy, spz, rec, best);
                        if (rb0 <= rb1)
                            for (int p = cell_start[row + rb0], pe = cell_start[row + rb1 + 1]; p < pe; p++)
                                sdf_pair_rec(f, cc, li, lj, lk, p, spx, spy, spz, rec, best);
                    }
            };
            // the target's own sort cell first: a particle of a neighbouring one lies at least half a
            // cell from the centre, so once the minimum is below that bound the neighbours cannot lower it
            scan(gi, gi, gj, gj, gk, gk, false, false);
            if (best >= iface)
                scan(max(gi - 1, ri0), min(gi + 1, ri1), max(gj - 1, rj0), min(gj + 1, rj1), max(gk - 1, rk0),
                     min(gk + 1, rk1), false, true);
            if (best >= ibound && reach > 1)
                scan(max(gi - reach, ri0), min(gi + reach, ri1), max(gj - reach, rj0), min(gj + reach, rj1),
                     max(gk - reach, rk0), min(gk + reach, rk1), true, false);
        }
        float v = ordered_to_float(best);
        if (do_post) {
            if (v < 0.5 * dx) {
                float sc = 0.125f * (solid[flat3(gi, gj, gk, sw, sh)] + solid[flat3(gi + 1, gj, gk, sw, sh)] +
                                     solid[flat3(gi, gj + 1, gk, sw, sh)] + solid[flat3(gi + 1, gj + 1, gk, sw, sh)] +
                                     solid[flat3(gi, gj, gk + 1, sw, sh)] + solid[flat3(gi + 1, gj, gk + 1, sw, sh)] +
                                     solid[flat3(gi, gj + 1, gk + 1, sw, sh)] + solid[flat3(gi + 1, gj + 1, gk + 1, sw, sh)]);
                if (sc < 0) v = (float)(-0.5f * dx);
            }
            if (fabsf(v) < eps) v = v > 0 ? eps : -eps;
        }
        phi[flat3(gi, gj, gk, d.ni, d.nj)] = v;
    }
}

void launch_liquid_sdf(Dims d, double dx, double radius, int np, const int *cell_start, const float *spx,
                       const float *spy, const float *spz, unsigned long long *rec, const float *solid, int do_post,
                       float *phi, cudaStream_t st) {
    int nb = ((d.ni + SDF_BW - 1) / SDF_BW) * ((d.nj + SDF_BW - 1) / SDF_BW) * ((d.nk + SDF_BW - 1) / SDF_BW);
    // sort cells a contributing particle can lie in, around the target cell: the window reaches
    // ceil(2r / dx) cells beyond the particle's own, plus one for the sort / block frame rounding
    const int reach = (int)std::ceil(2.0 * radius / dx) + 1;
    SdfFrame f{};
    sdf_frame_common(f, dx, (float)radius);
    if (np > 0) k_sdf_records<<<grid_for(np, 256), 256, 0, st>>>(f, SDF_BW * dx, np, spx, spy, spz, rec);
    k_liquid_sdf_gather<<<nb, 256, 0, st>>>(d, dx, (float)radius, reach, cell_start, spx, spy, spz, rec, solid,
                                            do_post, phi);
}

}  // namespace ffgpu
