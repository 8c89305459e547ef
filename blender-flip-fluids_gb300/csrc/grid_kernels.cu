// Grid-side kernels of the FLIP substep: solid level set of the closed domain, face
// weights, near-solid coarse grid, and the liquid signed distance field (K4) with its
// post-process.  Compiled with -fmad=false: every float/double expression here follows
// the reference engine's rounding step by step (no fused multiply-add).
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
// K4 liquid SDF.  One CTA per 10^3 cell block of the reference's block frame
// (particlelevelset.cpp:618-666).  The CTA visits every particle whose cell lies within
// two cells of the block, decides exactly as the reference whether that particle was
// assigned to this block (:507-551), and scatters min(|c - p| - r) over its search window
// into a shared-memory block with integer atomicMin (min is order independent, so the
// result is bit-identical to the reference).  The post-process against the solid level
// set (:170-194) is fused into the write-back.
// ---------------------------------------------------------------------------------
constexpr int SDF_BW = 10;

__global__ void __launch_bounds__(256) k_liquid_sdf(Dims d, double dx, float r, const int *__restrict__ cell_start,
                                                    const float *__restrict__ spx, const float *__restrict__ spy,
                                                    const float *__restrict__ spz, const float *__restrict__ solid,
                                                    int do_post, float *phi) {
    __shared__ int blk[SDF_BW * SDF_BW * SDF_BW];
    __shared__ float cc[SDF_BW];
    const int nbi = (d.ni + SDF_BW - 1) / SDF_BW, nbj = (d.nj + SDF_BW - 1) / SDF_BW;
    const int A = blockIdx.x % nbi, B = (blockIdx.x / nbi) % nbj, C = blockIdx.x / (nbi * nbj);
    const float maxd = (float)(3.0 * dx);
    const int imaxd = float_to_ordered(maxd);
    for (int t = threadIdx.x; t < SDF_BW * SDF_BW * SDF_BW; t += blockDim.x) blk[t] = imaxd;
    const double hw = 0.5 * dx;
    if (threadIdx.x < SDF_BW) cc[threadIdx.x] = (float)((double)(float)threadIdx.x * dx + hw);
    __syncthreads();

    const float sr = 2.0f * r;
    const float fblockdx = (float)(SDF_BW * dx);
    const double inv_fb = 1.0 / (double)fblockdx;
    const double bdx = SDF_BW * dx;
    const double inv_dx = 1.0 / dx;
    const float ox = (float)((double)(float)A * bdx), oy = (float)((double)(float)B * bdx), oz = (float)((double)(float)C * bdx);

    // candidate cells: [10A-2, 10A+11] per axis, clipped to the grid
    const int ci0 = max(SDF_BW * A - 2, 0), ci1 = min(SDF_BW * A + SDF_BW + 1, d.ni - 1);
    const int cj0 = max(SDF_BW * B - 2, 0), cj1 = min(SDF_BW * B + SDF_BW + 1, d.nj - 1);
    const int ck0 = max(SDF_BW * C - 2, 0), ck1 = min(SDF_BW * C + SDF_BW + 1, d.nk - 1);
    const int cw = ci1 - ci0 + 1, chh = cj1 - cj0 + 1, cd = ck1 - ck0 + 1;
    // one warp per candidate cell row; lanes set up that row's particles 32 at a time
    const int nrows = chh * cd;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (int row = warp; row < nrows; row += nwarps) {
        int cj = cj0 + row % chh, ck = ck0 + row / chh;
        size_t base = flat3(ci0, cj, ck, d.ni, d.nj);
        int p0 = cell_start[base], p1 = cell_start[base + cw];
        for (int pb = p0; pb < p1; pb += 32) {
            // per lane: one particle's exact block assignment and search window
            const int p = pb + lane;
            bool assigned = false;
            float lx = 0.0f, ly = 0.0f, lz = 0.0f;
            int i0 = 0, i1 = -1, j0 = 0, j1 = -1, k0 = 0, k1 = -1;
            if (p < p1) {
                float x = spx[p], y = spy[p], z = spz[p];
                int a = (int)floor(x * inv_fb), b = (int)floor(y * inv_fb), c = (int)floor(z * inv_fb);
                float bx = (float)((double)(float)a * (double)fblockdx);
                float by = (float)((double)(float)b * (double)fblockdx);
                float bz = (float)((double)(float)c * (double)fblockdx);
                if (x - sr > bx && y - sr > by && z - sr > bz &&
                    x + sr < bx + fblockdx && y + sr < by + fblockdx && z + sr < bz + fblockdx) {
                    assigned = (a == A && b == B && c == C);
                } else {
                    assigned = (int)floor((double)(x - sr) * inv_fb) <= A && A <= (int)floor((double)(x + sr) * inv_fb) &&
                               (int)floor((double)(y - sr) * inv_fb) <= B && B <= (int)floor((double)(y + sr) * inv_fb) &&
                               (int)floor((double)(z - sr) * inv_fb) <= C && C <= (int)floor((double)(z + sr) * inv_fb);
                }
                if (assigned) {
                    lx = x - ox; ly = y - oy; lz = z - oz;
                    i0 = max((int)floor((double)(lx - sr) * inv_dx), 0); i1 = min((int)floor((double)(lx + sr) * inv_dx), SDF_BW - 1);
                    j0 = max((int)floor((double)(ly - sr) * inv_dx), 0); j1 = min((int)floor((double)(ly + sr) * inv_dx), SDF_BW - 1);
                    k0 = max((int)floor((double)(lz - sr) * inv_dx), 0); k1 = min((int)floor((double)(lz + sr) * inv_dx), SDF_BW - 1);
                    assigned = i0 <= i1 && j0 <= j1 && k0 <= k1;
                }
            }
            // warp-cooperative scatter: one particle at a time, lanes over its window cells,
            // so every atomicMin of an instruction targets a distinct cell
            unsigned int todo = __ballot_sync(0xffffffffu, assigned);
            while (todo) {
                const int src = __ffs(todo) - 1;
                todo &= todo - 1;
                const float sx = __shfl_sync(0xffffffffu, lx, src), sy = __shfl_sync(0xffffffffu, ly, src),
                            sz = __shfl_sync(0xffffffffu, lz, src);
                const int a0 = __shfl_sync(0xffffffffu, i0, src), a1 = __shfl_sync(0xffffffffu, i1, src);
                const int b0 = __shfl_sync(0xffffffffu, j0, src), b1 = __shfl_sync(0xffffffffu, j1, src);
                const int c0 = __shfl_sync(0xffffffffu, k0, src), c1 = __shfl_sync(0xffffffffu, k1, src);
                const int nx = a1 - a0 + 1, ny = b1 - b0 + 1, nz = c1 - c0 + 1;
                const int ncell = nx * ny * nz;
                for (int q = lane; q < ncell; q += 32) {
                    const int i = a0 + q % nx, j = b0 + (q / nx) % ny, k = c0 + q / (nx * ny);
                    const float vx = cc[i] - sx, vy = cc[j] - sy, vz = cc[k] - sz;
                    const float dist = __fsqrt_rn(vx * vx + vy * vy + vz * vz) - r;
                    atomicMin(&blk[i + SDF_BW * (j + SDF_BW * k)], float_to_ordered(dist));
                }
            }
        }
    }
    __syncthreads();
    const float eps = (float)(0.005 * dx);
    const int sw = d.ni + 1, sh = d.nj + 1;
    for (int t = threadIdx.x; t < SDF_BW * SDF_BW * SDF_BW; t += blockDim.x) {
        int i = t % SDF_BW, j = (t / SDF_BW) % SDF_BW, k = t / (SDF_BW * SDF_BW);
        int gi = A * SDF_BW + i, gj = B * SDF_BW + j, gk = C * SDF_BW + k;
        if (gi >= d.ni || gj >= d.nj || gk >= d.nk) continue;
        float v = ordered_to_float(blk[t]);
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

void launch_liquid_sdf(Dims d, double dx, double radius, const int *cell_start, const float *spx,
                       const float *spy, const float *spz, const float *solid, int do_post, float *phi,
                       cudaStream_t st) {
    int nb = ((d.ni + SDF_BW - 1) / SDF_BW) * ((d.nj + SDF_BW - 1) / SDF_BW) * ((d.nk + SDF_BW - 1) / SDF_BW);
    k_liquid_sdf<<<nb, 256, 0, st>>>(d, dx, (float)radius, cell_start, spx, spy, spz, solid, do_post, phi);
}

}  // namespace ffgpu
