// K6a / K17a: the APIC velocity transfer.
//   P2G: VelocityAdvector::_advectionAPICProducerThread (velocityadvector.cpp:543-623) over the
//        block assignment of :239-353; every particle adds w (v + a . (x_node - x_p)) and w to
//        the nodes of its trilinear stencil that lie inside each block it is assigned to.
//   G2P: FluidSimulation::_updatePICAPICMarkerParticleVelocitiesThread
//        (fluidsimulation.cpp:6791-6843): the PIC velocity and, per component, the affine
//        vector sum_q grad(w_q) u_q from _getIndicesAndGradientWeights.
// Compiled with -fmad=false so every weight is the reference's float expression.
#include <cmath>

#include "common.cuh"
#include "kernels.h"
#include "mac_sample.cuh"

namespace ffgpu {

namespace {

constexpr int CW = 10;   // velocityadvector.h:187 (_chunkWidth)

// The double product decides; kept out of line so the compiler cannot evaluate it on the
// common path (FP64 issue is scarce on this GPU).
__device__ __noinline__ int floor_dp(float v, double inv) { return (int)floor((double)v * inv); }

// floor((double)v * inv) for a float v, where inv = 1 / h in double and invf its float value
// 1 / (float)h.  The float product lies within 3e-7 |t| of the double one, so away from an
// integer the float floor is the double floor; near one the double product decides.
__device__ inline int exact_floor(float v, float invf, double inv) {
    const float t = v * invf;
    const float fl = floorf(t);
    const float fr = t - fl;
    const float margin = 1e-5f + 1e-6f * fabsf(t);
    if (fr > margin && fr < 1.0f - margin) return (int)fl;
    return floor_dp(v, inv);
}

// Transfer frame of one component: cell and block widths with their double and float inverses,
// the assignment half-width sr and the face offsets (velocityadvector.cpp:177-188, 293-300).
struct ApicFrame {
    double inv_dx, inv_fb, fblockdx_d;
    float fblockdx, sr, invf_dx, invf_fb, invf;
    float ofx, ofy, ofz;
};

ApicFrame make_frame(double dx, double radius, int comp) {
    ApicFrame F;
    F.inv_dx = 1.0 / dx;
    F.fblockdx = (float)(dx * CW);
    F.fblockdx_d = (double)F.fblockdx;
    F.inv_fb = 1.0 / F.fblockdx_d;
    F.sr = (float)(radius + 1e-6f);
    F.invf_dx = (float)F.inv_dx;
    F.invf_fb = (float)F.inv_fb;
    F.invf = (float)(1.0 / (double)(float)dx);   // vec3 / float (vmath.cpp:100-103)
    const float hdx = (float)(0.5 * dx);
    F.ofx = comp == 0 ? 0.0f : hdx;
    F.ofy = comp == 1 ? 0.0f : hdx;
    F.ofz = comp == 2 ? 0.0f : hdx;
    return F;
}

// Block assignment record of one particle for one component (velocityadvector.cpp:293-353):
// per axis the first block plus one (16 bits) and whether the range spans the next block
// (1 bit).  A particle whose radius-sr box lies strictly inside its own block is assigned to
// that block alone; any other to every block the box overlaps (at most two per axis, as
// 2 sr < one block).
__device__ inline unsigned long long axis_rec(float x, const ApicFrame &F, bool interior, int own) {
    int a0 = own, a1 = own;
    if (!interior) {
        a0 = exact_floor(x - F.sr, F.invf_fb, F.inv_fb);
        a1 = exact_floor(x + F.sr, F.invf_fb, F.inv_fb);
    }
    return (unsigned long long)((unsigned)(a0 + 1) & 0xFFFFu) | ((unsigned long long)(a1 > a0) << 16);
}

__global__ void k_apic_records(ApicFrame F0, ApicFrame F1, ApicFrame F2, int np, const float *__restrict__ spx,
                               const float *__restrict__ spy, const float *__restrict__ spz,
                               unsigned long long *rec) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        const float px = spx[p], py = spy[p], pz = spz[p];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const ApicFrame &F = c == 0 ? F0 : (c == 1 ? F1 : F2);
            const float x = px - F.ofx, y = py - F.ofy, z = pz - F.ofz;
            const int a = exact_floor(x, F.invf_fb, F.inv_fb), b = exact_floor(y, F.invf_fb, F.inv_fb),
                      cc = exact_floor(z, F.invf_fb, F.inv_fb);
            const float bxa = (float)((double)(float)a * F.fblockdx_d), bya = (float)((double)(float)b * F.fblockdx_d),
                        bza = (float)((double)(float)cc * F.fblockdx_d);
            const bool interior = x - F.sr > bxa && y - F.sr > bya && z - F.sr > bza && x + F.sr < bxa + F.fblockdx &&
                                  y + F.sr < bya + F.fblockdx && z + F.sr < bza + F.fblockdx;
            rec[(size_t)c * np + p] = axis_rec(x, F, interior, a) | (axis_rec(y, F, interior, b) << 17) |
                                      (axis_rec(z, F, interior, cc) << 34);
        }
    }
}

__device__ inline bool rec_has(unsigned long long r, int shift, int blk) {
    const int a0 = (int)((r >> shift) & 0xFFFFu) - 1;
    const unsigned span = (unsigned)((r >> (shift + 16)) & 1u);
    return (unsigned)(blk - a0) <= span;
}

// The trilinear weight factor of node `l` along one axis for a particle at block-local
// coordinate lx; false when the node is not in the particle's stencil.
__device__ inline bool stencil_factor(float lx, int l, float invf_dx, double inv_dx, const float *__restrict__ gpos,
                                      float invf, float &wgt) {
    const int g = exact_floor(lx, invf_dx, inv_dx);
    if (l != g && l != g + 1) return false;   // so -1 <= g <= CW - 1
    const float gp = __ldg(gpos + g + 1);
    const float t = (lx - gp) * invf;
    wgt = l == g ? 1.0f - t : t;
    return true;
}

// One thread per face: gathers the particles of the 2x3x3 cells around it (the only ones
// whose stencil can hold the face), keeps those assigned to the face's block and sums their
// APIC contributions in the block's float frame.  Sums run in cell order, then particle
// order: deterministic, no atomics.
__global__ void __launch_bounds__(256) k_p2g_apic(Dims d, ApicFrame F, int comp, GridDecode dec,
                                                  const int *__restrict__ cell_start, const float *__restrict__ spx,
                                                  const float *__restrict__ spy, const float *__restrict__ spz,
                                                  const float *__restrict__ svel, const float *__restrict__ sax,
                                                  const float *__restrict__ say, const float *__restrict__ saz,
                                                  const unsigned long long *__restrict__ rec,
                                                  const float *__restrict__ gpos, const float *__restrict__ bpos,
                                                  float *field, unsigned char *valid) {
    const int fw = d.ni + (comp == 0), fh = d.nj + (comp == 1), fd = d.nk + (comp == 2);
    const unsigned int nf = (unsigned int)fw * fh * fd;
    const float eps = 1e-6f;
    const float invf_dx = F.invf_dx, invf = F.invf;
    const double inv_dx = F.inv_dx;
    for (unsigned int f = blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += gridDim.x * blockDim.x) {
        int fi, fj, fk;
        dec(f, fi, fj, fk);
        const int A = fi / CW, B = fj / CW, C = fk / CW;
        const int li = fi - CW * A, lj = fj - CW * B, lk = fk - CW * C;
        const float bx = __ldg(bpos + A), by = __ldg(bpos + B), bz = __ldg(bpos + C);   // (float)((double)(float)A * chunkdx)
        const float nx = __ldg(gpos + li + 1), ny = __ldg(gpos + lj + 1), nz = __ldg(gpos + lk + 1);
        int i0 = fi - 1, i1 = comp == 0 ? fi : fi + 1;
        int j0 = fj - 1, j1 = comp == 1 ? fj : fj + 1;
        int k0 = fk - 1, k1 = comp == 2 ? fk : fk + 1;
        i0 = max(i0, 0); j0 = max(j0, 0); k0 = max(k0, 0);
        i1 = min(i1, d.ni - 1); j1 = min(j1, d.nj - 1); k1 = min(k1, d.nk - 1);
        float S = 0.0f, W = 0.0f;
        for (int ck = k0; ck <= k1; ck++)
            for (int cj = j0; cj <= j1; cj++) {
                const size_t base = flat3(0, cj, ck, d.ni, d.nj);
                const int p0 = cell_start[base + i0], p1 = cell_start[base + i1 + 1];
                for (int p = p0; p < p1; p++) {
                    const unsigned long long r = __ldg(rec + p);
                    if (!rec_has(r, 0, A) || !rec_has(r, 17, B) || !rec_has(r, 34, C)) continue;
                    // block-local frame (velocityadvector.cpp:565-569)
                    const float lx = (__ldg(spx + p) - F.ofx) - bx, ly = (__ldg(spy + p) - F.ofy) - by,
                                lz = (__ldg(spz + p) - F.ofz) - bz;
                    float wx, wy, wz;
                    if (!stencil_factor(lx, li, invf_dx, inv_dx, gpos, invf, wx) ||
                        !stencil_factor(ly, lj, invf_dx, inv_dx, gpos, invf, wy) ||
                        !stencil_factor(lz, lk, invf_dx, inv_dx, gpos, invf, wz))
                        continue;
                    const float wgt = wx * wy * wz;
                    const float apic = __ldg(sax + p) * (nx - lx) + __ldg(say + p) * (ny - ly) + __ldg(saz + p) * (nz - lz);
                    S += wgt * (__ldg(svel + p) + apic);
                    W += wgt;
                }
            }
        const bool ok = W > eps;
        field[f] = ok ? S / W : S;
        valid[f] = ok ? 1 : 0;
    }
}

// Gradient weights of the 8 stencil nodes (fluidsimulation.cpp:6731-6769), node q = (q & 1,
// q >> 1 & 1, q >> 2), and the affine vector of one component.
__device__ inline float node_pos(int g, const float *__restrict__ gpos, int gmax, double dx) {
    return (g >= -1 && g <= gmax) ? __ldg(gpos + g + 1) : (float)((double)(float)g * dx);
}

__device__ inline void affine_of(const float *__restrict__ g, int gw, int gh, int gd, float qx, float qy, float qz,
                                 double dx, double inv, float invf_dx, float invf, float invdx,
                                 const float *__restrict__ gpos, int gmax, float &a0, float &a1, float &a2) {
    const int gi = exact_floor(qx, invf_dx, inv), gj = exact_floor(qy, invf_dx, inv), gk = exact_floor(qz, invf_dx, inv);
    const float gx = node_pos(gi, gpos, gmax, dx), gy = node_pos(gj, gpos, gmax, dx), gz = node_pos(gk, gpos, gmax, dx);
    const float ix = (qx - gx) * invf, iy = (qy - gy) * invf, iz = (qz - gz) * invf;
    const float wts[8][3] = {
        {-invdx * (1.0f - iy) * (1.0f - iz), -invdx * (1.0f - ix) * (1.0f - iz), -invdx * (1.0f - ix) * (1.0f - iy)},
        {invdx * (1.0f - iy) * (1.0f - iz), ix * (-invdx) * (1.0f - iz), ix * (1.0f - iy) * (-invdx)},
        {(-invdx) * iy * (1.0f - iz), (1.0f - ix) * invdx * (1.0f - iz), (1.0f - ix) * iy * (-invdx)},
        {invdx * iy * (1.0f - iz), ix * invdx * (1.0f - iz), ix * iy * (-invdx)},
        {(-invdx) * (1.0f - iy) * iz, (1.0f - ix) * (-invdx) * iz, (1.0f - ix) * (1.0f - iy) * invdx},
        {invdx * (1.0f - iy) * iz, ix * (-invdx) * iz, ix * (1.0f - iy) * invdx},
        {(-invdx) * iy * iz, (1.0f - ix) * invdx * iz, (1.0f - ix) * iy * invdx},
        {invdx * iy * iz, ix * invdx * iz, ix * iy * invdx}};
    a0 = 0.0f; a1 = 0.0f; a2 = 0.0f;
#pragma unroll
    for (int q = 0; q < 8; q++) {
        const int i = gi + (q & 1), j = gj + ((q >> 1) & 1), k = gk + (q >> 2);
        if (i < 0 || j < 0 || k < 0 || i >= gw || j >= gh || k >= gd) continue;
        const float val = __ldg(g + flat3(i, j, k, gw, gh));
        a0 += wts[q][0] * val; a1 += wts[q][1] * val; a2 += wts[q][2] * val;
    }
}

struct AffPtrs { float *a[9]; };

// One thread per particle: the affine vectors from the gradient weights (in double-floor
// node indices, float weights) and the PIC velocity (FP32 MAC sampling).
__global__ void k_g2p_apic(MacDev m, float invf, float invdx, int np, const float *__restrict__ px,
                           const float *__restrict__ py, const float *__restrict__ pz, float *vx, float *vy, float *vz,
                           AffPtrs A, const float *__restrict__ gpos, int gmax) {
    const double inv = 1.0 / m.ddx;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        const float x = px[p], y = py[p], z = pz[p];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const float *g = c == 0 ? m.f.u : (c == 1 ? m.f.v : m.f.w);
            const int gw = m.d.ni + (c == 0), gh = m.d.nj + (c == 1), gd = m.d.nk + (c == 2);
            const float qx = x - (c == 0 ? 0.0f : m.hdx), qy = y - (c == 1 ? 0.0f : m.hdx), qz = z - (c == 2 ? 0.0f : m.hdx);
            float a0, a1, a2;
            affine_of(g, gw, gh, gd, qx, qy, qz, m.ddx, inv, m.inv, invf, invdx, gpos, gmax, a0, a1, a2);
            A.a[3 * c][p] = a0; A.a[3 * c + 1][p] = a1; A.a[3 * c + 2][p] = a2;
        }
        float ox, oy, oz;
        sample_mac(m, x, y, z, ox, oy, oz);
        vx[p] = ox; vy[p] = oy; vz[p] = oz;
    }
}

}  // namespace

void launch_apic_records(Dims, double dx, double radius, int np, const float *spx, const float *spy, const float *spz,
                         unsigned long long *rec, cudaStream_t st) {
    if (np == 0) return;
    k_apic_records<<<grid_for(np, 256, 152u * 32u), 256, 0, st>>>(make_frame(dx, radius, 0), make_frame(dx, radius, 1),
                                                                  make_frame(dx, radius, 2), np, spx, spy, spz, rec);
}

void launch_p2g_apic(Dims d, double dx, double radius, int comp, const int *cell_start, const float *spx,
                     const float *spy, const float *spz, const float *svel, const float *const *saff,
                     const unsigned long long *rec, int np, const float *gpos, const float *bpos, float *field,
                     unsigned char *valid, cudaStream_t st) {
    const size_t nf = d.faces(comp);
    const GridDecode dec = grid_decode(d.ni + (comp == 0), d.nj + (comp == 1), d.nk + (comp == 2));
    k_p2g_apic<<<grid_for(nf, 256, 152u * 64u), 256, 0, st>>>(d, make_frame(dx, radius, comp), comp, dec, cell_start,
                                                              spx, spy, spz, svel, saff[0], saff[1], saff[2],
                                                              rec + (size_t)comp * np, gpos, bpos, field, valid);
}

void launch_g2p_apic(Dims d, double dx, int np, const float *px, const float *py, const float *pz, float *vx,
                     float *vy, float *vz, float *const *aff, MacView vel, const float *gpos, int gmax,
                     cudaStream_t st) {
    if (np == 0) return;
    AffPtrs A;
    for (int q = 0; q < 9; q++) A.a[q] = aff[q];
    const float invf = (float)(1.0 / (double)(float)dx);
    const float invdx = (float)(1.0 / dx);   // 1.0f / _dx with a double _dx
    k_g2p_apic<<<grid_for(np, 256), 256, 0, st>>>(make_mac(d, dx, vel), invf, invdx, np, px, py, pz, vx, vy, vz, A,
                                                  gpos, gmax);
}

}  // namespace ffgpu
