// K17 grid-to-particle PIC/FLIP update, K18 RK3 marker advection with solid collision
// handling, K19 marker removal and stable compaction, and the max-speed reduction used
// by the CFL substep count.  Compiled with -fmad=false: the collision and removal logic
// follow the reference's float/double rounding step by step.  MAC sampling runs in FP32
// (cell fractions formed with one fused x - i*dx), where the reference samples in double.
#include "common.cuh"
#include "kernels.h"
#include "mac_sample.cuh"

namespace ffgpu {

// K17 (fluidsimulation.cpp:6771-6789)
__global__ void k_g2p(MacDev cur, MacDev saved, float a, float b, int np, const float *__restrict__ px,
                      const float *__restrict__ py, const float *__restrict__ pz, float *vx, float *vy, float *vz) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        float x = px[p], y = py[p], z = pz[p];
        float cx, cy, cz, sx, sy, sz;
        sample_mac(cur, x, y, z, cx, cy, cz);
        sample_mac(saved, x, y, z, sx, sy, sz);
        float fx = vx[p] + cx - sx, fy = vy[p] + cy - sy, fz = vz[p] + cz - sz;
        vx[p] = a * cx + b * fx;
        vy[p] = a * cy + b * fy;
        vz[p] = a * cz + b * fz;
    }
}

void launch_g2p(Dims d, double dx, float pic, int np, const float *px, const float *py, const float *pz,
                float *vx, float *vy, float *vz, MacView cur, MacView saved, cudaStream_t st) {
    if (np == 0) return;
    float a = pic, b = (float)(1.0 - (double)pic);
    k_g2p<<<grid_for(np, 256), 256, 0, st>>>(make_mac(d, dx, cur), make_mac(d, dx, saved), a, b, np, px, py, pz,
                                             vx, vy, vz);
}

// ---- solid level set sampling, reference rounding (interpolation.cpp:72-110, 200-260) ----
struct SolidDev {
    const float *phi;
    int w, h, d;
    double dx;
};

__device__ inline float sget(const SolidDev &s, int i, int j, int k) {
    return (i >= 0 && j >= 0 && k >= 0 && i < s.w && j < s.h && k < s.d) ? __ldg(s.phi + flat3(i, j, k, s.w, s.h)) : 0.0f;
}

__device__ inline void solid_frac(const SolidDev &s, float x, float y, float z, int &i, int &j, int &k,
                                  double &ix, double &iy, double &iz) {
    double inv = 1.0 / s.dx;
    const float invf = (float)inv;
    i = floor_fd(x, inv, invf); j = floor_fd(y, inv, invf); k = floor_fd(z, inv, invf);
    float gx = (float)((double)(float)i * s.dx), gy = (float)((double)(float)j * s.dx), gz = (float)((double)(float)k * s.dx);
    ix = (double)(x - gx) * inv; iy = (double)(y - gy) * inv; iz = (double)(z - gz) * inv;
}

__device__ float solid_trilinear(const SolidDev &s, float x, float y, float z) {
    int i, j, k;
    double ix, iy, iz;
    solid_frac(s, x, y, z, i, j, k, ix, iy, iz);
    double p0 = sget(s, i, j, k), p1 = sget(s, i + 1, j, k), p2 = sget(s, i, j + 1, k), p3 = sget(s, i, j, k + 1);
    double p4 = sget(s, i + 1, j, k + 1), p5 = sget(s, i, j + 1, k + 1), p6 = sget(s, i + 1, j + 1, k), p7 = sget(s, i + 1, j + 1, k + 1);
    double r = p0 * (1 - ix) * (1 - iy) * (1 - iz) + p1 * ix * (1 - iy) * (1 - iz) + p2 * (1 - ix) * iy * (1 - iz) +
               p3 * (1 - ix) * (1 - iy) * iz + p4 * ix * (1 - iy) * iz + p5 * (1 - ix) * iy * iz +
               p6 * ix * iy * (1 - iz) + p7 * ix * iy * iz;
    return (float)r;
}

// (solid level set < 0) exactly as solid_trilinear(...) < 0.  The trilinear weights are
// non-negative, so with no negative corner the value cannot be negative and the double-precision
// evaluation is skipped; otherwise v receives the exact value.
__device__ inline bool solid_below(const SolidDev &s, float x, float y, float z, float &v) {
    const double inv = 1.0 / s.dx;
    const float invf = (float)inv;
    const int i = floor_fd(x, inv, invf), j = floor_fd(y, inv, invf), k = floor_fd(z, inv, invf);
    const float c0 = sget(s, i, j, k), c1 = sget(s, i + 1, j, k), c2 = sget(s, i, j + 1, k), c3 = sget(s, i, j, k + 1);
    const float c4 = sget(s, i + 1, j, k + 1), c5 = sget(s, i, j + 1, k + 1), c6 = sget(s, i + 1, j + 1, k);
    const float c7 = sget(s, i + 1, j + 1, k + 1);
    if (fminf(fminf(fminf(c0, c1), fminf(c2, c3)), fminf(fminf(c4, c5), fminf(c6, c7))) >= 0.0f) {
        v = 0.0f;
        return false;
    }
    v = solid_trilinear(s, x, y, z);
    return v < 0.0f;
}

__device__ inline double bilerp(double v00, double v10, double v01, double v11, double ix, double iy) {
    double l1 = (1 - ix) * v00 + ix * v10;
    double l2 = (1 - ix) * v01 + ix * v11;
    return (1 - iy) * l1 + iy * l2;
}

__device__ void solid_gradient(const SolidDev &s, float x, float y, float z, float &gx, float &gy, float &gz) {
    int i, j, k;
    double ix, iy, iz;
    solid_frac(s, x, y, z, i, j, k, ix, iy, iz);
    float v000 = sget(s, i, j, k), v100 = sget(s, i + 1, j, k), v010 = sget(s, i, j + 1, k), v001 = sget(s, i, j, k + 1);
    float v101 = sget(s, i + 1, j, k + 1), v011 = sget(s, i, j + 1, k + 1), v110 = sget(s, i + 1, j + 1, k), v111 = sget(s, i + 1, j + 1, k + 1);
    gx = (float)bilerp(v100 - v000, v110 - v010, v101 - v001, v111 - v011, iy, iz);
    gy = (float)bilerp(v010 - v000, v110 - v100, v011 - v001, v111 - v101, ix, iz);
    gz = (float)bilerp(v001 - v000, v101 - v100, v011 - v010, v111 - v110, ix, iy);
}

struct BoxDev {   // AABB with float corner and double extents (aabb.h)
    float px, py, pz;
    double w, h, d;
    __device__ bool inside(float x, float y, float z) const {
        return x >= px && y >= py && z >= pz && x < px + w && y < py + h && z < pz + d;
    }
    __device__ void nearest(float &x, float &y, float &z) const {   // aabb.cpp:501-518
        if (inside(x, y, z)) return;
        float mx = px + (float)w, my = py + (float)h, mz = pz + (float)d;
        x = fmaxf(x, px); y = fmaxf(y, py); z = fmaxf(z, pz);
        x = (float)fmin((double)x, (double)mx - 1e-6);
        y = (float)fmin((double)y, (double)my - 1e-6);
        z = (float)fmin((double)z, (double)mz - 1e-6);
    }
};

__device__ inline float vlen(float x, float y, float z) { return __fsqrt_rn(x * x + y * y + z * z); }

// K18 (fluidsimulation.cpp:7616-7721)
__global__ void __launch_bounds__(128, 8) k_advect(MacDev m, SolidDev s, BoxDev bnd, NearGrid ng, const unsigned char *__restrict__ near,
                         double dt, float maxdist, int np, const float *__restrict__ px, const float *__restrict__ py,
                         const float *__restrict__ pz, float *ox, float *oy, float *oz, unsigned char *collided) {
    const float h1 = (float)(0.5 * dt), h2 = (float)(0.75 * dt), h3 = (float)(dt / 9.0f);
    const double ncinv = 1.0 / ng.cell, dinv = 1.0 / m.ddx;
    const float ncinvf = (float)ncinv, dinvf = (float)dinv;   // float-first floors, exact (floor_fd)
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        float x0 = px[p], y0 = py[p], z0 = pz[p];
        float k1x, k1y, k1z, k2x, k2y, k2z, k3x, k3y, k3z;
        sample_mac(m, x0, y0, z0, k1x, k1y, k1z);
        sample_mac(m, x0 + h1 * k1x, y0 + h1 * k1y, z0 + h1 * k1z, k2x, k2y, k2z);
        sample_mac(m, x0 + h2 * k2x, y0 + h2 * k2y, z0 + h2 * k2z, k3x, k3y, k3z);
        float nx = x0 + h3 * (2.0f * k1x + 3.0f * k2x + 4.0f * k3x);
        float ny = y0 + h3 * (2.0f * k1y + 3.0f * k2y + 4.0f * k3y);
        float nz = z0 + h3 * (2.0f * k1z + 3.0f * k2z + 4.0f * k3z);
        const float rx0 = nx, ry0 = ny, rz0 = nz;
        // _resolveCollision
        int gi = floor_fd(nx, dinv, dinvf), gj = floor_fd(ny, dinv, dinvf), gk = floor_fd(nz, dinv, dinvf);
        if (!(gi >= 0 && gj >= 0 && gk >= 0 && gi < m.d.ni && gj < m.d.nj && gk < m.d.nk)) bnd.nearest(nx, ny, nz);
        int oi = floor_fd(x0, ncinv, ncinvf), oj = floor_fd(y0, ncinv, ncinvf), ok = floor_fd(z0, ncinv, ncinvf);
        int ni2 = floor_fd(nx, ncinv, ncinvf), nj2 = floor_fd(ny, ncinv, ncinvf), nk2 = floor_fd(nz, ncinv, ncinvf);
        auto nearat = [&](int a, int b, int c) -> bool {
            if (a < 0 || b < 0 || c < 0 || a >= ng.w || b >= ng.h || c >= ng.d) return false;
            return near[flat3(a, b, c, ng.w, ng.h)] != 0;
        };
        if (nearat(oi, oj, ok) || nearat(ni2, nj2, nk2)) {
            const float eps = 1e-6f;
            float step = 0.1f * (float)m.ddx;
            float dxv = nx - x0, dyv = ny - y0, dzv = nz - z0;
            float travel = vlen(dxv, dyv, dzv);
            if (travel >= eps) {
                int nsteps = (int)ceilf(travel / step);
                float inv = (float)(1.0 / travel);
                float sx = dxv * inv, sy = dyv * inv, sz = dzv * inv;
                float lx = x0, ly = y0, lz = z0, cx = x0, cy = y0, cz = z0;
                bool hit = false;
                float hitphi = 0.0f;
                for (int q = 0; q < nsteps; q++) {
                    if (q == nsteps - 1) { cx = nx; cy = ny; cz = nz; }
                    else {
                        float f = (float)(q + 1) * step;
                        cx = x0 + f * sx; cy = y0 + f * sy; cz = z0 + f * sz;
                    }
                    float phi;
                    const bool below = solid_below(s, cx, cy, cz, phi);
                    if (below || !bnd.inside(cx, cy, cz)) {
                        // the hit value is needed exactly (also when only the domain box was left)
                        hitphi = below ? phi : solid_trilinear(s, cx, cy, cz);
                        hit = true;
                        break;
                    }
                    lx = cx; ly = cy; lz = cz;
                }
                if (hit) {
                    float rx, ry, rz;
                    float gx, gy, gz;
                    solid_gradient(s, cx, cy, cz, gx, gy, gz);
                    float gl = vlen(gx, gy, gz);
                    if (gl > eps) {
                        float ginv = (float)(1.0 / gl);
                        gx = gx * ginv; gy = gy * ginv; gz = gz * ginv;
                        float sc = (float)((double)hitphi - (double)0.2f * m.ddx);
                        rx = cx - sc * gx; ry = cy - sc * gy; rz = cz - sc * gz;
                        float rphi = solid_trilinear(s, rx, ry, rz);
                        float rdist = vlen(rx - cx, ry - cy, rz - cz);
                        if (rphi < 0 || rdist > maxdist) { rx = lx; ry = ly; rz = lz; }
                    } else {
                        rx = lx; ry = ly; rz = lz;
                    }
                    if (!bnd.inside(rx, ry, rz)) {
                        float qx = rx, qy = ry, qz = rz;
                        bnd.nearest(rx, ry, rz);
                        float rphi = solid_trilinear(s, rx, ry, rz);
                        float rdist = vlen(rx - qx, ry - qy, rz - qz);
                        if (rphi < 0.0f || rdist > maxdist) { rx = lx; ry = ly; rz = lz; }
                    }
                    nx = rx; ny = ry; nz = rz;
                }
            }
        }
        ox[p] = nx; oy[p] = ny; oz[p] = nz;
        if (collided) collided[p] = (nx != rx0 || ny != ry0 || nz != rz0) ? 1 : 0;
    }
}

static BoxDev boundary(Dims d, double dx) {
    // _getBoundaryAABB (fluidsimulation.cpp:5175-5180) then expand(-0.2 dx) (:7639-7640)
    BoxDev b;
    double v1 = -3 * dx - 1e-4;
    float h1 = (float)(0.5 * v1);
    b.px = 0.0f - h1; b.py = 0.0f - h1; b.pz = 0.0f - h1;
    b.w = d.ni * dx + v1; b.h = d.nj * dx + v1; b.d = d.nk * dx + v1;
    double v2 = -(double)0.2f * dx;
    float h2 = (float)(0.5 * v2);
    b.px = b.px - h2; b.py = b.py - h2; b.pz = b.pz - h2;
    b.w += v2; b.h += v2; b.d += v2;
    return b;
}

void launch_advect(Dims d, double dx, double dt, int cfl, int np, const float *px, const float *py,
                   const float *pz, float *ox, float *oy, float *oz, MacView vel, const float *solid,
                   NearGrid ng, const unsigned char *near, cudaStream_t st, unsigned char *collided) {
    if (np == 0) return;
    SolidDev s{solid, d.ni + 1, d.nj + 1, d.nk + 1, dx};
    k_advect<<<grid_for(np, 128, 152u * 32u), 128, 0, st>>>(make_mac(d, dx, vel), s, boundary(d, dx), ng, near, dt,
                                                            (float)(cfl * dx), np, px, py, pz, ox, oy, oz, collided);
}

// ---- K19 removal (fluidsimulation.cpp:7773-7851) ----
__global__ void k_remove_mark(Dims d, double dx, SolidDev s, int np, const float *__restrict__ px,
                              const float *__restrict__ py, const float *__restrict__ pz, int *keep, int *key,
                              int *count, int *maxc) {
    double inv = 1.0 / dx;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        float x = px[p], y = py[p], z = pz[p];
        int i = min(max((int)floor(x * inv), 0), d.ni - 1);
        int j = min(max((int)floor(y * inv), 0), d.nj - 1);
        int k = min(max((int)floor(z * inv), 0), d.nk - 1);
        int c = (int)flat3(i, j, k, d.ni, d.nj);
        key[p] = c;
        float sv;
        if (solid_below(s, x, y, z, sv)) { keep[p] = 0; continue; }
        keep[p] = 1;
        int v = atomicAdd(&count[c], 1) + 1;
        atomicMax(maxc, v);
    }
}

void launch_remove_mark(Dims d, double dx, int np, const float *px, const float *py, const float *pz,
                        const float *solid, int *keep, int *key, int *cell_count, int *max_count, cudaStream_t st) {
    if (np == 0) return;
    SolidDev s{solid, d.ni + 1, d.nj + 1, d.nk + 1, dx};
    k_remove_mark<<<grid_for(np, 256), 256, 0, st>>>(d, dx, s, np, px, py, pz, keep, key, cell_count, max_count);
}

// Per-cell cap in particle order: walk each cell's stably sorted list, keep the first
// max_per_cell surviving particles.
__global__ void k_cap(size_t nc, const int *__restrict__ cell_start, const int *__restrict__ idx,
                      const int *__restrict__ keep_in, int *keep_out, int cap) {
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < nc; c += (size_t)gridDim.x * blockDim.x) {
        // keep_in: 0 removed (solid), 1 kept, 2 counted but removed for speed
        int kept = 0;
        for (int q = cell_start[c]; q < cell_start[c + 1]; q++) {
            int p = idx[q];
            if (!keep_in[p]) { keep_out[p] = 0; continue; }
            keep_out[p] = (kept < cap && keep_in[p] == 1) ? 1 : 0;
            kept++;
        }
    }
}

void launch_cap_per_cell(size_t ncells, const int *cell_start, const int *sorted_idx, const int *keep_in,
                         int *keep_out, int max_per_cell, cudaStream_t st) {
    k_cap<<<grid_for(ncells, 256), 256, 0, st>>>(ncells, cell_start, sorted_idx, keep_in, keep_out, max_per_cell);
}

constexpr int MAX_COMPACT_ATTRS = 16;
struct CPack { const float *src[MAX_COMPACT_ATTRS]; float *dst[MAX_COMPACT_ATTRS]; };

__global__ void k_compact(int np, const int *__restrict__ keep, const int *__restrict__ off, CPack pk, int nattr) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        if (!keep[p]) continue;
        int o = off[p];
        for (int a = 0; a < nattr; a++) pk.dst[a][o] = pk.src[a][p];
    }
}

void launch_compact(int np, const int *keep, const int *offset, const float *const *src, float *const *dst,
                    int nattr, cudaStream_t st) {
    if (nattr < 0 || nattr > MAX_COMPACT_ATTRS) throw std::invalid_argument("Error: too many particle attributes to compact.\n");
    if (np == 0) return;
    CPack pk;
    for (int a = 0; a < nattr; a++) { pk.src[a] = src[a]; pk.dst[a] = dst[a]; }
    k_compact<<<grid_for(np, 256), 256, 0, st>>>(np, keep, offset, pk, nattr);
}

// max |v|^2 over particles, float dot as the reference (fluidsimulation.cpp:10189-10203);
// non-negative floats order like their bit patterns, so an integer atomicMax is exact.
__global__ void k_max_speed_sq(int np, const float *__restrict__ vx, const float *__restrict__ vy,
                               const float *__restrict__ vz, unsigned int *out) {
    float m = 0.0f;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        float x = vx[p], y = vy[p], z = vz[p];
        m = fmaxf(m, x * x + y * y + z * z);
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}

void launch_max_speed_sq(int np, const float *vx, const float *vy, const float *vz, double *, unsigned int *out,
                         double *, cudaStream_t st) {
    FFGPU_CUDA(cudaMemsetAsync(out, 0, sizeof(unsigned int), st));
    if (np == 0) return;
    k_max_speed_sq<<<grid_for(np, 256), 256, 0, st>>>(np, vx, vy, vz, out);
}


// ---- extreme-speed rule (fluidsimulation.cpp:7723-7771) ----
__global__ void k_speed_hist(int np, const float *__restrict__ vx, const float *__restrict__ vy,
                             const float *__restrict__ vz, double step, int nb, int *bins, unsigned long long *maxbits) {
    double m = 0.0;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        float x = vx[p], y = vy[p], z = vz[p];
        double speed = (double)__fsqrt_rn(x * x + y * y + z * z);
        int bin = (int)fmin(floor(speed / step), (double)(nb - 1));
        atomicAdd(&bins[bin], 1);
        m = fmax(m, speed);
    }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(maxbits, (unsigned long long)__double_as_longlong(m));
}

void launch_speed_hist(int np, const float *vx, const float *vy, const float *vz, double step, int nbins,
                       int *bins, unsigned long long *maxbits, cudaStream_t st) {
    if (np == 0) return;
    k_speed_hist<<<grid_for(np, 256), 256, 0, st>>>(np, vx, vy, vz, step, nbins, bins, maxbits);
}

__global__ void k_speed_outliers(int np, const float *__restrict__ vx, const float *__restrict__ vy,
                                 const float *__restrict__ vz, double lower, double upper, int *counts) {
    int a = 0, b = 0;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        float x = vx[p], y = vy[p], z = vz[p];
        double speed = (double)__fsqrt_rn(x * x + y * y + z * z);
        if (speed >= lower && speed < upper) a++;
        if (speed >= upper) b++;
    }
    for (int o = 16; o > 0; o >>= 1) { a += __shfl_down_sync(0xffffffffu, a, o); b += __shfl_down_sync(0xffffffffu, b, o); }
    if ((threadIdx.x & 31) == 0) { atomicAdd(&counts[0], a); atomicAdd(&counts[1], b); }
}

void launch_speed_outliers(int np, const float *vx, const float *vy, const float *vz, double lower, double upper,
                           int *counts, cudaStream_t st) {
    FFGPU_CUDA(cudaMemsetAsync(counts, 0, 2 * sizeof(int), st));
    if (np == 0) return;
    k_speed_outliers<<<grid_for(np, 256), 256, 0, st>>>(np, vx, vy, vz, lower, upper, counts);
}

// keep: 0 inside a solid, 2 faster than the speed limit (still counted per cell), 1 kept
__global__ void k_remove_mark2(Dims d, double dx, SolidDev s, int np, const float *__restrict__ px,
                               const float *__restrict__ py, const float *__restrict__ pz,
                               const float *__restrict__ vx, const float *__restrict__ vy,
                               const float *__restrict__ vz, double maxspeedsq, int *keep, int *key,
                               int *count, int *maxc) {
    double inv = 1.0 / dx;
    // every lane of a warp runs the same number of rounds (the maximum is reduced per warp)
    const int stride = gridDim.x * blockDim.x;
    const int rounds = (np + stride - 1) / stride;
    int wmax = 0;
    for (int rd = 0; rd < rounds; rd++) {
        const int p = rd * stride + blockIdx.x * blockDim.x + threadIdx.x;
        if (p < np) {
            float x = px[p], y = py[p], z = pz[p];
            const float invf = (float)inv;
            int i = min(max(floor_fd(x, inv, invf), 0), d.ni - 1);
            int j = min(max(floor_fd(y, inv, invf), 0), d.nj - 1);
            int k = min(max(floor_fd(z, inv, invf), 0), d.nk - 1);
            int c = (int)flat3(i, j, k, d.ni, d.nj);
            key[p] = c;
            float sv;
            if (solid_below(s, x, y, z, sv)) {
                keep[p] = 0;
            } else {
                float ux = vx[p], uy = vy[p], uz = vz[p];
                float v2 = ux * ux + uy * uy + uz * uz;
                keep[p] = (maxspeedsq >= 0.0 && (double)v2 > maxspeedsq) ? 2 : 1;
                wmax = max(wmax, atomicAdd(&count[c], 1) + 1);
            }
        }
    }
    wmax = __reduce_max_sync(0xffffffffu, wmax);
    if ((threadIdx.x & 31) == 0 && wmax > 0) atomicMax(maxc, wmax);
}

void launch_remove_mark2(Dims d, double dx, int np, const float *px, const float *py, const float *pz,
                         const float *vx, const float *vy, const float *vz, const float *solid, double maxspeedsq,
                         int *keep, int *key, int *cell_count, int *max_count, cudaStream_t st) {
    if (np == 0) return;
    SolidDev s{solid, d.ni + 1, d.nj + 1, d.nk + 1, dx};
    k_remove_mark2<<<grid_for(np, 256), 256, 0, st>>>(d, dx, s, np, px, py, pz, vx, vy, vz, maxspeedsq, keep, key,
                                                      cell_count, max_count);
}

__global__ void k_keep01(int np, const int *__restrict__ keep, int *out) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) out[p] = keep[p] == 1;
}

void launch_keep01(int np, const int *keep, int *keep01, cudaStream_t st) {
    if (np == 0) return;
    k_keep01<<<grid_for(np, 256), 256, 0, st>>>(np, keep, keep01);
}


// ---- particle I/O: interleaved xyz (the C API's layout) <-> device SoA ----
__global__ void k_deinterleave(int np, const float *__restrict__ aos, float *x, float *y, float *z) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        x[p] = aos[3 * (size_t)p]; y[p] = aos[3 * (size_t)p + 1]; z[p] = aos[3 * (size_t)p + 2];
    }
}

__global__ void k_interleave(int np, const float *__restrict__ x, const float *__restrict__ y,
                             const float *__restrict__ z, float *aos) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        aos[3 * (size_t)p] = x[p]; aos[3 * (size_t)p + 1] = y[p]; aos[3 * (size_t)p + 2] = z[p];
    }
}

void launch_deinterleave(int np, const float *aos, float *x, float *y, float *z, cudaStream_t st) {
    if (np == 0) return;
    k_deinterleave<<<grid_for(np, 256), 256, 0, st>>>(np, aos, x, y, z);
}

// deinterleave that also checks every record: positions (hi != null) inside [0, hi) per axis,
// compared in double as the load filter does; velocities (hi == null) finite.  A failing record
// sets `bit` in *flag.
__global__ void k_deinterleave_checked(int np, const float *__restrict__ aos, float *x, float *y, float *z,
                                       double hx, double hy, double hz, int positions, unsigned int bit,
                                       unsigned int *flag) {
    bool bad = false;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        const float a = aos[3 * (size_t)p], b = aos[3 * (size_t)p + 1], c = aos[3 * (size_t)p + 2];
        x[p] = a; y[p] = b; z[p] = c;
        if (positions) bad = bad || !(a >= 0.0f && b >= 0.0f && c >= 0.0f && a < hx && b < hy && c < hz);
        else bad = bad || !(isfinite(a) && isfinite(b) && isfinite(c));
    }
    if (bad) atomicOr(flag, bit);
}

void launch_deinterleave_checked(int np, const float *aos, float *x, float *y, float *z, const double *hi,
                                 unsigned int bit, unsigned int *flag, cudaStream_t st) {
    if (np == 0) return;
    k_deinterleave_checked<<<grid_for(np, 256), 256, 0, st>>>(np, aos, x, y, z, hi ? hi[0] : 0.0, hi ? hi[1] : 0.0,
                                                              hi ? hi[2] : 0.0, hi ? 1 : 0, bit, flag);
}

void launch_interleave(int np, const float *x, const float *y, const float *z, float *aos, cudaStream_t st) {
    if (np == 0) return;
    k_interleave<<<grid_for(np, 256), 256, 0, st>>>(np, x, y, z, aos);
}

}  // namespace ffgpu
