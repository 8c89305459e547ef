// K20 the variational viscosity solve applied before the pressure projection
// (FluidSimulation::_applyViscosityToVelocityField, fluidsimulation.cpp:5983-6064;
// ViscositySolver, viscositysolver.cpp:53-901), reference-exact:
//   face states from the solid distance at cell centres, liquid cells dilated twice, subcell
//   volume fractions from the liquid level set averaged onto centre/face/edge grids, the
//   15-point system over the faces with a positive volume nearby (rows sorted by column,
//   stored as 16-slot rows), the general MIC(0) factor and its triangular solves by levels,
//   and PCG in float.
// Levels: the unknowns are ordered U faces, then V, then W, each x-fastest; every coupling of
// a row to a lower row lies at a strictly lower level when U(i,j,k) sits at level i+j+k,
// V(i,j,k) at i+j+k+2 and W(i,j,k) at i+j+k+4.  Rows of one level are independent, so the
// factor, the forward and the backward solve run one launch per level (no waits between
// blocks), each row pulling from its lower (or upper) rows in ascending column order: the
// reference's operation order per entry.
// Compiled with -fmad=false: every coefficient is the reference's float expression.
#include <cmath>
#include <stdexcept>
#include <vector>

#include <cooperative_groups.h>

#include "common.cuh"
#include "kernels.h"
#include "viscosity.h"

namespace ffgpu {

namespace cg = cooperative_groups;

namespace {

constexpr unsigned char FS_FLUID = 1, FS_SOLID = 2;
constexpr int SLOTS = VISC_SLOTS;
// entry s of row r (rows of 16 slots, row after row)
#define SL(r, s) ((size_t)(r) * SLOTS + (size_t)(s))

struct FaceDims {
    int ni, nj, nk;
    size_t nu, nv, nw;
    __host__ __device__ size_t U(int i, int j, int k) const { return (size_t)i + (size_t)(ni + 1) * (j + (size_t)nj * k); }
    __host__ __device__ size_t V(int i, int j, int k) const { return nu + i + (size_t)ni * (j + (size_t)(nj + 1) * k); }
    __host__ __device__ size_t W(int i, int j, int k) const { return nu + nv + i + (size_t)ni * (j + (size_t)nj * k); }
};

FaceDims face_dims(Dims d) {
    FaceDims f;
    f.ni = d.ni; f.nj = d.nj; f.nk = d.nk;
    f.nu = d.faces(0); f.nv = d.faces(1); f.nw = d.faces(2);
    return f;
}

__device__ inline float get3(const float *g, int w, int h, int d, int i, int j, int k) {
    return (i >= 0 && j >= 0 && k >= 0 && i < w && j < h && k < d) ? g[flat3(i, j, k, w, h)] : 0.0f;
}

// ---- face states (viscositysolver.cpp:144-207, meshlevelset.cpp:152-162) ----
__global__ void k_face_state(FaceDims F, const float *__restrict__ solid, unsigned char *state) {
    const int ni = F.ni, nj = F.nj, nk = F.nk;
    const size_t nf = F.nu + F.nv + F.nw;
    auto scp = [&](int i, int j, int k) {
        auto s = [&](int a, int b, int c) { return solid[flat3(a, b, c, ni + 1, nj + 1)]; };
        return 0.125f * (s(i, j, k) + s(i + 1, j, k) + s(i, j + 1, k) + s(i + 1, j + 1, k) + s(i, j, k + 1) +
                         s(i + 1, j, k + 1) + s(i, j + 1, k + 1) + s(i + 1, j + 1, k + 1));
    };
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < nf; t += (size_t)gridDim.x * blockDim.x) {
        bool solid_face;
        if (t < F.nu) {
            const int i = (int)(t % (ni + 1)), j = (int)((t / (ni + 1)) % nj), k = (int)(t / ((size_t)(ni + 1) * nj));
            solid_face = i == 0 || i == ni || scp(i - 1, j, k) + scp(i, j, k) <= 0;
        } else if (t < F.nu + F.nv) {
            const size_t q = t - F.nu;
            const int i = (int)(q % ni), j = (int)((q / ni) % (nj + 1)), k = (int)(q / ((size_t)ni * (nj + 1)));
            solid_face = j == 0 || j == nj || scp(i, j - 1, k) + scp(i, j, k) <= 0;
        } else {
            const size_t q = t - F.nu - F.nv;
            const int i = (int)(q % ni), j = (int)((q / ni) % nj), k = (int)(q / ((size_t)ni * nj));
            solid_face = k == 0 || k == nk || scp(i, j, k - 1) + scp(i, j, k) <= 0;
        }
        state[t] = solid_face ? FS_SOLID : FS_FLUID;
    }
}

// ---- liquid cells dilated twice over the (n+1)^3 grid (viscositysolver.cpp:209-238) ----
__global__ void k_valid_init(Dims d, const float *__restrict__ liquid, unsigned char *valid) {
    const int w = d.ni + 1, h = d.nj + 1, dd = d.nk + 1;
    const size_t n = (size_t)w * h * dd;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(t % w), j = (int)((t / w) % h), k = (int)(t / ((size_t)w * h));
        valid[t] = (i < d.ni && j < d.nj && k < d.nk && liquid[flat3(i, j, k, d.ni, d.nj)] < 0) ? 1 : 0;
    }
}

__global__ void k_valid_dilate(Dims d, const unsigned char *__restrict__ src, unsigned char *dst) {
    const int w = d.ni + 1, h = d.nj + 1, dd = d.nk + 1;
    const size_t n = (size_t)w * h * dd;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(t % w), j = (int)((t / w) % h), k = (int)(t / ((size_t)w * h));
        unsigned char v = src[t];
        if (i > 0) v |= src[t - 1];
        if (i < w - 1) v |= src[t + 1];
        if (j > 0) v |= src[t - w];
        if (j < h - 1) v |= src[t + w];
        if (k > 0) v |= src[t - (size_t)w * h];
        if (k < dd - 1) v |= src[t + (size_t)w * h];
        dst[t] = v;
    }
}

// ---- subcell volume fractions (viscositysolver.cpp:287-346, levelsetutils.cpp:213-258) ----
// trilinear sample of the cell-centred liquid level set (particlelevelset.cpp:136-138,
// interpolation.cpp:61-112): index floor and weights in double, corner order 000, 100, 010,
// 001, 101, 011, 110, 111
__device__ float sample_liquid(const float *__restrict__ phi, Dims d, double dx, double inv, float sh, float px,
                               float py, float pz) {
    const float x = px - sh, y = py - sh, z = pz - sh;
    const int i = (int)floor((double)x * inv), j = (int)floor((double)y * inv), k = (int)floor((double)z * inv);
    const float gx = (float)((double)(float)i * dx), gy = (float)((double)(float)j * dx), gz = (float)((double)(float)k * dx);
    const double ix = (double)(x - gx) * inv, iy = (double)(y - gy) * inv, iz = (double)(z - gz) * inv;
    const double p0 = get3(phi, d.ni, d.nj, d.nk, i, j, k), p1 = get3(phi, d.ni, d.nj, d.nk, i + 1, j, k),
                 p2 = get3(phi, d.ni, d.nj, d.nk, i, j + 1, k), p3 = get3(phi, d.ni, d.nj, d.nk, i, j, k + 1),
                 p4 = get3(phi, d.ni, d.nj, d.nk, i + 1, j, k + 1), p5 = get3(phi, d.ni, d.nj, d.nk, i, j + 1, k + 1),
                 p6 = get3(phi, d.ni, d.nj, d.nk, i + 1, j + 1, k), p7 = get3(phi, d.ni, d.nj, d.nk, i + 1, j + 1, k + 1);
    const double r = p0 * (1 - ix) * (1 - iy) * (1 - iz) + p1 * ix * (1 - iy) * (1 - iz) + p2 * (1 - ix) * iy * (1 - iz) +
                     p3 * (1 - ix) * (1 - iy) * iz + p4 * ix * (1 - iy) * iz + p5 * (1 - ix) * iy * iz +
                     p6 * ix * iy * (1 - iz) + p7 * ix * iy * iz;
    return (float)r;
}

__device__ inline void swapf(float &a, float &b) { const float c = a; a = b; b = c; }

__device__ float vf4(float p0, float p1, float p2, float p3) {
    if (p0 > p1) swapf(p0, p1);
    if (p2 > p3) swapf(p2, p3);
    if (p0 > p2) swapf(p0, p2);
    if (p1 > p3) swapf(p1, p3);
    if (p1 > p2) swapf(p1, p2);
    if (p3 <= 0) return 1;
    if (p2 <= 0) return 1 - p3 * p3 * p3 / ((p3 - p2) * (p3 - p1) * (p3 - p0));
    if (p1 <= 0) {
        const float a = p0 / (p0 - p2), b = p0 / (p0 - p3), c = p1 / (p1 - p3), dd = p1 / (p1 - p2);
        return a * b * (1 - dd) + b * (1 - c) * dd + c * dd;
    }
    if (p0 <= 0) return p0 * p0 * p0 / ((p0 - p1) * (p0 - p2) * (p0 - p3));
    return 0;
}

__global__ void k_subcell(Dims d, double ddx, float dxf, const unsigned char *__restrict__ valid,
                          const float *__restrict__ phi, float *sub) {
    const int w = 2 * d.ni, h = 2 * d.nj, dd = 2 * d.nk;
    const size_t n = (size_t)w * h * dd;
    const float cs = 0.25f * dxf, sdx = 0.5f * dxf, hh = 0.5f * sdx;
    const float sh = (float)(0.5 * ddx);
    const double inv = 1.0 / ddx;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(t % w), j = (int)((t / w) % h), k = (int)(t / ((size_t)w * h));
        if (!valid[flat3(i / 2, j / 2, k / 2, d.ni + 1, d.nj + 1)]) { sub[t] = 0.0f; continue; }
        const float cx = cs + i * sdx, cy = cs + j * sdx, cz = cs + k * sdx;
        const float xm = cx + (-hh), xp = cx + hh, ym = cy + (-hh), yp = cy + hh, zm = cz + (-hh), zp = cz + hh;
        const float p000 = sample_liquid(phi, d, ddx, inv, sh, xm, ym, zm), p001 = sample_liquid(phi, d, ddx, inv, sh, xm, ym, zp),
                    p010 = sample_liquid(phi, d, ddx, inv, sh, xm, yp, zm), p011 = sample_liquid(phi, d, ddx, inv, sh, xm, yp, zp),
                    p100 = sample_liquid(phi, d, ddx, inv, sh, xp, ym, zm), p101 = sample_liquid(phi, d, ddx, inv, sh, xp, ym, zp),
                    p110 = sample_liquid(phi, d, ddx, inv, sh, xp, yp, zm), p111 = sample_liquid(phi, d, ddx, inv, sh, xp, yp, zp);
        sub[t] = (vf4(p000, p001, p101, p011) + vf4(p000, p101, p100, p110) + vf4(p000, p010, p011, p110) +
                  vf4(p101, p011, p111, p110) + 2 * vf4(p000, p011, p101, p110) + vf4(p100, p101, p001, p111) +
                  vf4(p100, p001, p000, p010) + vf4(p100, p110, p111, p010) + vf4(p001, p111, p011, p010) +
                  2 * vf4(p100, p111, p001, p010)) / 12.0f;
    }
}

// centre, U, V, W, edgeU, edgeV, edgeW volumes of the valid cells (i, j, k) in [1, n-1]^3 as the
// mean of 8 subcells (viscositysolver.cpp:348-373); the caller zeroes the grids first
__global__ void k_volumes(Dims d, const unsigned char *__restrict__ valid, const float *__restrict__ sub, ViscVolumes V) {
    const int m = (d.ni - 1), mj = (d.nj - 1), mk = (d.nk - 1);
    if (m <= 0 || mj <= 0 || mk <= 0) return;
    const size_t n = (size_t)m * mj * mk;
    const int sw = 2 * d.ni, sh = 2 * d.nj;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        const int i = 1 + (int)(t % m), j = 1 + (int)((t / m) % mj), k = 1 + (int)(t / ((size_t)m * mj));
        if (!valid[flat3(i, j, k, d.ni + 1, d.nj + 1)]) continue;
        const int off[7][3] = {{0, 0, 0}, {-1, 0, 0}, {0, -1, 0}, {0, 0, -1}, {0, -1, -1}, {-1, 0, -1}, {-1, -1, 0}};
        const int gw[7] = {d.ni, d.ni + 1, d.ni, d.ni, d.ni, d.ni + 1, d.ni + 1};
        const int gh[7] = {d.nj, d.nj, d.nj + 1, d.nj, d.nj + 1, d.nj, d.nj + 1};
        float *grids[7] = {V.center, V.u, V.v, V.w, V.eu, V.ev, V.ew};
#pragma unroll
        for (int g = 0; g < 7; g++) {
            const int bi = 2 * i + off[g][0], bj = 2 * j + off[g][1], bk = 2 * k + off[g][2];
            float acc = 0.0f;
            for (int ko = 0; ko < 2; ko++)
                for (int jo = 0; jo < 2; jo++)
                    for (int io = 0; io < 2; io++) acc += sub[flat3(bi + io, bj + jo, bk + ko, sw, sh)];
            grids[g][flat3(i, j, k, gw[g], gh[g])] = 0.125f * acc;
        }
    }
}

// ---- rows of the system: faces in (1..n-1)^3, fluid, with a positive volume nearby ----
struct VolView {
    const float *c, *u, *v, *w, *eu, *ev, *ew;
    int ni, nj, nk;
    __device__ float C(int i, int j, int k) const { return get3(c, ni, nj, nk, i, j, k); }
    __device__ float U(int i, int j, int k) const { return get3(u, ni + 1, nj, nk, i, j, k); }
    __device__ float Vv(int i, int j, int k) const { return get3(v, ni, nj + 1, nk, i, j, k); }
    __device__ float W(int i, int j, int k) const { return get3(w, ni, nj, nk + 1, i, j, k); }
    __device__ float EU(int i, int j, int k) const { return get3(eu, ni, nj + 1, nk + 1, i, j, k); }
    __device__ float EV(int i, int j, int k) const { return get3(ev, ni + 1, nj, nk + 1, i, j, k); }
    __device__ float EW(int i, int j, int k) const { return get3(ew, ni + 1, nj + 1, nk, i, j, k); }
};

VolView vol_view(Dims d, const ViscVolumes &V) {
    return VolView{V.center, V.u, V.v, V.w, V.eu, V.ev, V.ew, d.ni, d.nj, d.nk};
}

__device__ inline bool face_decode(const FaceDims &F, size_t t, int &comp, int &i, int &j, int &k) {
    if (t < F.nu) {
        comp = 0; i = (int)(t % (F.ni + 1)); j = (int)((t / (F.ni + 1)) % F.nj); k = (int)(t / ((size_t)(F.ni + 1) * F.nj));
    } else if (t < F.nu + F.nv) {
        const size_t q = t - F.nu;
        comp = 1; i = (int)(q % F.ni); j = (int)((q / F.ni) % (F.nj + 1)); k = (int)(q / ((size_t)F.ni * (F.nj + 1)));
    } else {
        const size_t q = t - F.nu - F.nv;
        comp = 2; i = (int)(q % F.ni); j = (int)((q / F.ni) % F.nj); k = (int)(q / ((size_t)F.ni * F.nj));
    }
    return true;
}

// viscositysolver.cpp:363-471
__global__ void k_row_flags(FaceDims F, VolView V, const unsigned char *__restrict__ state, int *flag) {
    const size_t nf = F.nu + F.nv + F.nw;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < nf; t += (size_t)gridDim.x * blockDim.x) {
        int comp, i, j, k;
        face_decode(F, t, comp, i, j, k);
        bool in = false;
        if (i >= 1 && j >= 1 && k >= 1 && i < F.ni && j < F.nj && k < F.nk && state[t] == FS_FLUID) {
            if (comp == 0)
                in = V.U(i, j, k) > 0 || V.C(i, j, k) > 0 || V.C(i - 1, j, k) > 0 || V.EW(i, j + 1, k) > 0 ||
                     V.EW(i, j, k) > 0 || V.EV(i, j, k + 1) > 0 || V.EV(i, j, k) > 0;
            else if (comp == 1)
                in = V.Vv(i, j, k) > 0 || V.EW(i + 1, j, k) > 0 || V.EW(i, j, k) > 0 || V.C(i, j, k) > 0 ||
                     V.C(i, j - 1, k) > 0 || V.EU(i, j, k + 1) > 0 || V.EU(i, j, k) > 0;
            else
                in = V.W(i, j, k) > 0 || V.EV(i + 1, j, k) > 0 || V.EV(i, j, k) > 0 || V.EU(i, j + 1, k) > 0 ||
                     V.EU(i, j, k) > 0 || V.C(i, j, k) > 0 || V.C(i, j, k - 1) > 0;
        }
        flag[t] = in ? 1 : 0;
    }
}

__global__ void k_row_index(size_t nf, const int *__restrict__ flag, const int *__restrict__ scan, int *index,
                            int *rowface) {
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < nf; t += (size_t)gridDim.x * blockDim.x) {
        if (flag[t]) {
            index[t] = scan[t];
            rowface[scan[t]] = (int)t;
        } else {
            index[t] = -1;
        }
    }
}

struct Coupling { int col; float coef; };

// one row (viscositysolver.cpp:556-829); returns the rhs, writes the sorted row and its level
__global__ void k_rows(FaceDims F, VolView V, float dxf, float dtf, float visc, const unsigned char *__restrict__ state,
                       const int *__restrict__ index, const int *__restrict__ rowface, int n, const float *__restrict__ u,
                       const float *__restrict__ v, const float *__restrict__ w, int *col, float *val,
                       float *rhs, int *level, float *x0) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        int comp, i, j, k;
        face_decode(F, (size_t)rowface[r], comp, i, j, k);
        const float invdx = 1.0f / dxf;
        const float factor = dtf * invdx * invdx;
        const float avg = 0.25f * (visc + visc + visc + visc);   // mean of four grid values of the constant field
        float fR, fL, fT, fB, fF, fK, vol, vel;
        auto stU = [&](int a, int b, int c) -> unsigned char {
            return (a >= 0 && b >= 0 && c >= 0 && a <= F.ni && b < F.nj && c < F.nk) ? state[F.U(a, b, c)] : 0;
        };
        auto stV = [&](int a, int b, int c) -> unsigned char {
            return (a >= 0 && b >= 0 && c >= 0 && a < F.ni && b <= F.nj && c < F.nk) ? state[F.V(a, b, c)] : 0;
        };
        auto stW = [&](int a, int b, int c) -> unsigned char {
            return (a >= 0 && b >= 0 && c >= 0 && a < F.ni && b < F.nj && c <= F.nk) ? state[F.W(a, b, c)] : 0;
        };
        if (comp == 0) {
            fR = 2 * factor * visc * V.C(i, j, k);
            fL = 2 * factor * visc * V.C(i - 1, j, k);
            fT = factor * avg * V.EW(i, j + 1, k);
            fB = factor * avg * V.EW(i, j, k);
            fF = factor * avg * V.EV(i, j, k + 1);
            fK = factor * avg * V.EV(i, j, k);
            vol = V.U(i, j, k); vel = u[F.U(i, j, k)];
        } else if (comp == 1) {
            fR = factor * avg * V.EW(i + 1, j, k);
            fL = factor * avg * V.EW(i, j, k);
            fT = 2 * factor * visc * V.C(i, j, k);
            fB = 2 * factor * visc * V.C(i, j - 1, k);
            fF = factor * avg * V.EU(i, j, k + 1);
            fK = factor * avg * V.EU(i, j, k);
            vol = V.Vv(i, j, k); vel = v[F.V(i, j, k) - F.nu];
        } else {
            fR = factor * avg * V.EV(i + 1, j, k);
            fL = factor * avg * V.EV(i, j, k);
            fT = factor * avg * V.EU(i, j + 1, k);
            fB = factor * avg * V.EU(i, j, k);
            fF = 2 * factor * visc * V.C(i, j, k);
            fK = 2 * factor * visc * V.C(i, j, k - 1);
            vol = V.W(i, j, k); vel = w[F.W(i, j, k) - F.nu - F.nv];
        }
        Coupling cs[SLOTS];
        int nc = 0;
        cs[nc++] = Coupling{r, vol + fR + fL + fT + fB + fF + fK};
        float rv = vol * vel;
        auto add = [&](int fc, int a, int b, int c, float coef) {
            const unsigned char st = fc == 0 ? stU(a, b, c) : (fc == 1 ? stV(a, b, c) : stW(a, b, c));
            if (st == FS_FLUID) {
                const size_t t = fc == 0 ? F.U(a, b, c) : (fc == 1 ? F.V(a, b, c) : F.W(a, b, c));
                const int cc = index[t];
                if (cc >= 0) cs[nc++] = Coupling{cc, coef};   // SparseMatrix::add skips index -1
            } else if (st == FS_SOLID) {
                const float vv = fc == 0 ? u[F.U(a, b, c)] : (fc == 1 ? v[F.V(a, b, c) - F.nu] : w[F.W(a, b, c) - F.nu - F.nv]);
                rv -= coef * vv;
            }
        };
        if (comp == 0) {
            add(0, i + 1, j, k, -fR); add(0, i - 1, j, k, -fL); add(0, i, j + 1, k, -fT); add(0, i, j - 1, k, -fB);
            add(0, i, j, k + 1, -fF); add(0, i, j, k - 1, -fK);
            add(1, i, j + 1, k, -fT); add(1, i - 1, j + 1, k, fT); add(1, i, j, k, fB); add(1, i - 1, j, k, -fB);
            add(2, i, j, k + 1, -fF); add(2, i - 1, j, k + 1, fF); add(2, i, j, k, fK); add(2, i - 1, j, k, -fK);
        } else if (comp == 1) {
            add(1, i + 1, j, k, -fR); add(1, i - 1, j, k, -fL); add(1, i, j + 1, k, -fT); add(1, i, j - 1, k, -fB);
            add(1, i, j, k + 1, -fF); add(1, i, j, k - 1, -fK);
            add(0, i + 1, j, k, -fR); add(0, i + 1, j - 1, k, fR); add(0, i, j, k, fL); add(0, i, j - 1, k, -fL);
            add(2, i, j, k + 1, -fF); add(2, i, j - 1, k + 1, fF); add(2, i, j, k, fK); add(2, i, j - 1, k, -fK);
        } else {
            add(2, i + 1, j, k, -fR); add(2, i - 1, j, k, -fL); add(2, i, j + 1, k, -fT); add(2, i, j - 1, k, -fB);
            add(2, i, j, k + 1, -fF); add(2, i, j, k - 1, -fK);
            add(0, i + 1, j, k, -fR); add(0, i + 1, j, k - 1, fR); add(0, i, j, k, fL); add(0, i, j, k - 1, -fL);
            add(1, i, j + 1, k, -fT); add(1, i, j + 1, k - 1, fT); add(1, i, j, k, fB); add(1, i, j, k - 1, -fB);
        }
        // columns are distinct: insertion sort by column
        for (int a = 1; a < nc; a++) {
            const Coupling c = cs[a];
            int b = a - 1;
            while (b >= 0 && cs[b].col > c.col) { cs[b + 1] = cs[b]; b--; }
            cs[b + 1] = c;
        }
        for (int s = 0; s < SLOTS; s++) {
            col[SL(r, s)] = s < nc ? cs[s].col : -1;
            val[SL(r, s)] = s < nc ? cs[s].coef : 0.0f;
        }
        rhs[r] = rv;
        x0[r] = vel;   // the field before the solve: the warm start
        level[r] = i + j + k + 2 * comp;
    }
}

// level bookkeeping: counts, then rows grouped by level
__global__ void k_level_count(int n, const int *__restrict__ level, int *count) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) atomicAdd(count + level[r], 1);
}

__global__ void k_level_scatter(int n, const int *__restrict__ level, const int *__restrict__ start, int *cursor,
                                int *rows) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const int L = level[r];
        rows[start[L] + atomicAdd(cursor + L, 1)] = r;
    }
}

// for every lower entry (r, c < r) the slot of r in row c
__global__ void k_transpose_slots(int n, const int *__restrict__ col, unsigned char *tpos) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        for (int s = 0; s < SLOTS; s++) {
            const int c = col[SL(r, s)];
            unsigned char t = 0xFF;
            if (c >= 0 && c < r)
                for (int q = 0; q < SLOTS; q++)
                    if (col[SL(c, q)] == r) { t = (unsigned char)q; break; }
            tpos[SL(r, s)] = t;
        }
    }
}

// initial factor values (pcgsolver.h:76-117): the diagonal (below 1e-9 -> 0) and the upper part
__global__ void k_factor_init(int n, const int *__restrict__ col, const float *__restrict__ val,
                              float *invdiag, float *adiag, float *lval) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        for (int s = 0; s < SLOTS; s++) {
            const int c = col[SL(r, s)];
            const float a = val[SL(r, s)];
            if (c == r) {
                const float d = a < 1e-9f ? 0.0f : a;
                invdiag[r] = d;
                adiag[r] = d;
            }
            lval[SL(r, s)] = c > r ? a : 0.0f;
        }
    }
}

// One level of the MIC(0) factorization (pcgsolver.h:119-205), pulled per column j: for each
// earlier column k (ascending) with an entry in row j, the updates that k's elimination makes
// to column j, in the reference's order; then the pivot and the scaling of column j.
// A half-warp takes one row j, lane t holding slot t of row j and, in turn, slot t of each row k
// (16-lane loads of whole rows).  Per k the updates are: the pivot's (the entry of k's column at
// row j), each kept lower entry of j's (one entry of k's column each), and the dropped entries
// summed in k's slot order -- the same float operations in the same order as one thread
// walking the slots.
constexpr int FL_THREADS = 128;
__global__ void __launch_bounds__(FL_THREADS) k_factor_level(const int *__restrict__ rows, int cnt,
                                                             const int *__restrict__ col,
                                                             const unsigned char *__restrict__ tpos,
                                                             const float *__restrict__ adiag, float *invdiag,
                                                             float *lval) {
    const float mod = 0.97f, mdr = 0.25f;
    const int t = threadIdx.x & 15;
    const unsigned hmask = 0xffffu << (threadIdx.x & 16);
    const int nh = gridDim.x * (FL_THREADS / 16);
    for (int q = (blockIdx.x * FL_THREADS + threadIdx.x) >> 4; q < cnt; q += nh) {
        const int j = rows[q];
        const int cjt = col[SL(j, t)];
        float myL = lval[SL(j, t)];
        const int tpj = tpos[SL(j, t)];
        int cj[SLOTS];
#pragma unroll
        for (int b = 0; b < SLOTS; b++) cj[b] = __shfl_sync(hmask, cjt, b, 16);
        float invd = invdiag[j];
        for (int s = 0; s < SLOTS; s++) {
            const int k = __shfl_sync(hmask, cjt, s, 16);
            if (k < 0 || k >= j) break;   // columns ascend: the lower ones come first
            const unsigned tp = (unsigned)__shfl_sync(hmask, tpj, s, 16);
            const int rr = col[SL(k, t)];
            const float lv = lval[SL(k, t)];
            if (adiag[k] == 0) continue;          // a null column eliminates nothing
            if (tp >= (unsigned)SLOTS) continue;  // the pattern is symmetric; kept for memory safety
            const float mult = __shfl_sync(hmask, lv, (int)tp, 16);
            // my slot t of row k: below k? the pivot's entry? kept in row j (at slot mb)? dropped?
            const bool lower = rr > k;
            int mb = -1;
#pragma unroll
            for (int b = 0; b < SLOTS; b++)
                if (cj[b] == rr) mb = b;
            const bool piv = lower && rr == j;
            const bool kept = lower && !piv && mb >= 0 && rr > j;
            const bool dropped = lower && !piv && mb < 0;
            const float prod = mult * lv;
            // the pivot update
            const unsigned pm = __ballot_sync(hmask, piv) >> (threadIdx.x & 16);
            if (pm) invd -= __shfl_sync(hmask, prod, __ffs(pm) - 1, 16);
            // the kept entries: lane mb takes the product of the slot that matched it
#pragma unroll
            for (int u = 0; u < SLOTS; u++) {
                const int tb = __shfl_sync(hmask, kept ? mb : -1, u, 16);
                const float pv = __shfl_sync(hmask, prod, u, 16);
                if (tb == t) myL -= pv;
            }
            // the dropped entries, summed in k's slot order
            const float term = dropped ? lv : 0.0f;
            float missing = 0.0f;
#pragma unroll
            for (int u = 0; u < SLOTS; u++) missing += __shfl_sync(hmask, term, u, 16);
            invd -= mod * mult * missing;
        }
        const float ad = adiag[j];
        if (ad != 0) {
            invd = invd < mdr * ad ? (float)(1.0 / sqrt((double)ad)) : (float)(1.0 / sqrt((double)invd));
            if (cjt > j) myL *= invd;
        }
        if (t == 0) invdiag[j] = invd;
        if (cjt > j) lval[SL(j, t)] = myL;
    }
}

// L z = r for one row (pcgsolver.h:212-225, pulled in ascending column order)
__device__ inline void lower_row(int i, const int *__restrict__ col, const unsigned char *__restrict__ tpos,
                                 const float *__restrict__ lval, const float *__restrict__ invdiag,
                                 const float *__restrict__ r, float *z) {
    float x = r[i];
    for (int s = 0; s < SLOTS; s++) {
        const int c = col[SL(i, s)];
        const unsigned tp = tpos[SL(i, s)];
        if (c < 0 || c >= i || tp >= (unsigned)SLOTS) continue;
        x -= lval[SL(c, tp)] * z[c];
    }
    z[i] = x * invdiag[i];
}

// L^T z = z for one row (pcgsolver.h:228-241)
__device__ inline void upper_row(int i, const int *__restrict__ col, const float *__restrict__ lval,
                                 const float *__restrict__ invdiag, float *z) {
    float x = z[i];
    for (int s = 0; s < SLOTS; s++) {
        const int c = col[SL(i, s)];
        if (c <= i) continue;
        x -= lval[SL(i, s)] * z[c];
    }
    z[i] = x * invdiag[i];
}

__global__ void k_lower_level(const int *__restrict__ rows, int cnt, const int *__restrict__ col,
                              const unsigned char *__restrict__ tpos, const float *__restrict__ lval,
                              const float *__restrict__ invdiag, const float *__restrict__ r, float *z) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < cnt; q += gridDim.x * blockDim.x)
        lower_row(rows[q], col, tpos, lval, invdiag, r, z);
}

__global__ void k_upper_level(const int *__restrict__ rows, int cnt, const int *__restrict__ col,
                              const float *__restrict__ lval, const float *__restrict__ invdiag, float *z) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < cnt; q += gridDim.x * blockDim.x)
        upper_row(rows[q], col, lval, invdiag, z);
}

// Both sweeps in one cooperative launch: the grid walks the levels in order with a grid-wide
// barrier between levels (all blocks co-resident by the cooperative launch).
constexpr int PC_THREADS = 256;
__global__ void __launch_bounds__(PC_THREADS) k_precond_coop(const int *__restrict__ rows, const int *__restrict__ start,
                                                             int nlev, const int *__restrict__ col,
                                                             const unsigned char *__restrict__ tpos,
                                                             const float *__restrict__ lval,
                                                             const float *__restrict__ invdiag,
                                                             const float *__restrict__ r, float *z) {
    cg::grid_group g = cg::this_grid();
    const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
    for (int L = 0; L < nlev; L++) {
        const int b = start[L], e = start[L + 1];
        for (int q = b + tid; q < e; q += nth) lower_row(rows[q], col, tpos, lval, invdiag, r, z);
        g.sync();
    }
    for (int L = nlev - 1; L >= 0; L--) {
        const int b = start[L], e = start[L + 1];
        for (int q = b + tid; q < e; q += nth) upper_row(rows[q], col, lval, invdiag, z);
        if (L > 0) g.sync();
    }
}

// ---- the PCG on dense boxes, the preconditioner as three tiled wavefront blocks ----
// The rows of one component couple among themselves only through their +-x, +-y, +-z neighbours
// of the same component (a 7-point pattern), and every U row precedes every V row, which precedes
// every W row.  L z = r therefore solves the U block first, then V, then W, each block a 7-point
// lower triangular solve whose right-hand side first loses the couplings to the components
// solved before it.  Per row that is the reference's order exactly: the columns of the earlier
// components are the row's smallest (subtracted by the fold, ascending), then its own -z, -y, -x
// neighbours (the wavefront's order), then the pivot.  L^T z = q runs W, V, U; there the
// reference subtracts a row's own +x, +y, +z neighbours before the later components' couplings,
// while the fold subtracts those couplings first: the same operator with another rounding order.
//
// Each component's rows live in a dense copy of their box (axes possibly reordered so that the
// wavefront sweeps the box's shortest axis); every PCG vector, the operator (its 15 entries per row
// in the reference's column order), the factor and the couplings between components are stored
// there, so the SpMV and the folds are stencils with coalesced loads.  A cell of the box that holds
// no row keeps +0 in every field: each product with it is exactly +0 and subtracting or adding it
// leaves any value unchanged bit for bit (a sum that starts at +0 is never -0), as a missing entry.

struct Nb { signed char comp, di, dj, dk; };
// the entries of a row of component c in the reference's column order (U rows, then V, then W,
// each x fastest): (component, offset); the own component's seven sit at 0 / 4 / 8
__constant__ Nb c_nb[3][15] = {
    {{0, 0, 0, -1}, {0, 0, -1, 0}, {0, -1, 0, 0}, {0, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1},
     {1, -1, 0, 0}, {1, 0, 0, 0}, {1, -1, 1, 0}, {1, 0, 1, 0},
     {2, -1, 0, 0}, {2, 0, 0, 0}, {2, -1, 0, 1}, {2, 0, 0, 1}},
    {{0, 0, -1, 0}, {0, 1, -1, 0}, {0, 0, 0, 0}, {0, 1, 0, 0},
     {1, 0, 0, -1}, {1, 0, -1, 0}, {1, -1, 0, 0}, {1, 0, 0, 0}, {1, 1, 0, 0}, {1, 0, 1, 0}, {1, 0, 0, 1},
     {2, 0, -1, 0}, {2, 0, 0, 0}, {2, 0, -1, 1}, {2, 0, 0, 1}},
    {{0, 0, 0, -1}, {0, 1, 0, -1}, {0, 0, 0, 0}, {0, 1, 0, 0},
     {1, 0, 0, -1}, {1, 0, 1, -1}, {1, 0, 0, 0}, {1, 0, 1, 0},
     {2, 0, 0, -1}, {2, 0, -1, 0}, {2, -1, 0, 0}, {2, 0, 0, 0}, {2, 1, 0, 0}, {2, 0, 1, 0}, {2, 0, 0, 1}}};
__host__ __device__ inline int nb_own(int c) { return 4 * c; }
// couplings to the other components, as fields X0..X7 of the row's component: forward (L(row, col)
// of the earlier components' columns, entries 0 ..) and backward (L(col, row) of the later ones)
//   U: X0..X7 = backward entries 7..14;  V: X0..X3 = forward 0..3, X4..X7 = backward 11..14;
//   W: X0..X7 = forward 0..7
__host__ __device__ inline int xf_count(int c) { return 4 * c; }
__host__ __device__ inline int xb_count(int c) { return 8 - 4 * c; }
__host__ __device__ inline int xb_first(int c) { return c == 0 ? 7 : 11; }   // table entry of the first
__host__ __device__ inline int xb_field(int c) { return c == 0 ? 0 : 4; }    // field X of the first

struct DenseMap {
    int i0, j0, k0;     // box origin in the component's face grid
    int e[3];           // box extent along the face grid's axes
    int perm[3];        // dense axis a runs along the face grid's axis perm[a]
    int pitch, rows;    // dense row length (padded) and rows per plane
    int planes;         // planes (along the swept axis)
    size_t base;        // offset of the component in every dense field
    size_t cells;       // pitch * rows * planes
};
struct DenseMaps { DenseMap m[3]; };

// dense position of face (i, j, k) of the map's component, or -1 outside its box
__device__ inline long long dense_pos(const DenseMap &M, int i, int j, int k) {
    const int l[3] = {i - M.i0, j - M.j0, k - M.k0};
    if ((unsigned)l[0] >= (unsigned)M.e[0] || (unsigned)l[1] >= (unsigned)M.e[1] || (unsigned)l[2] >= (unsigned)M.e[2])
        return -1;
    return (long long)(M.base + (size_t)l[M.perm[0]] + (size_t)M.pitch * ((size_t)l[M.perm[1]] + (size_t)M.rows * l[M.perm[2]]));
}
// face of dense cell q (offset within the component); false for the row padding
__device__ inline bool dense_face(const DenseMap &M, size_t q, int &i, int &j, int &k) {
    const int a0 = (int)(q % M.pitch), a1 = (int)((q / M.pitch) % M.rows), a2 = (int)(q / ((size_t)M.pitch * M.rows));
    if (a0 >= M.e[M.perm[0]]) return false;
    int l[3];
    l[M.perm[0]] = a0; l[M.perm[1]] = a1; l[M.perm[2]] = a2;
    i = M.i0 + l[0]; j = M.j0 + l[1]; k = M.k0 + l[2];
    return true;
}

enum DenseField {
    DF_INV = 0, DF_LX, DF_LY, DF_LZ,   // pivot and own factor entries towards +x', +y', +z' (dense axes)
    DF_A0 = 4,                         // 15 operator entries in the row's column order
    DF_X0 = DF_A0 + 15,                // 8 couplings to the other components
    DF_B = DF_X0 + 8, DF_XV, DF_R, DF_S, DF_Q, DF_RIN, DF_AZ,
    DF_COUNT
};

__global__ void k_boxes_init(int *b) {
    const int t = threadIdx.x;
    if (t < 19) b[t] = t == 18 ? 0 : ((t % 6) < 3 ? INT_MAX : INT_MIN);
}

// row box of every component (min and max of i, j, k over its rows)
__global__ void __launch_bounds__(256) k_comp_boxes(FaceDims F, int n, const int *__restrict__ rowface, int *b) {
    __shared__ int sb[18];
    if (threadIdx.x < 18) sb[threadIdx.x] = (threadIdx.x % 6) < 3 ? INT_MAX : INT_MIN;
    __syncthreads();
    int lo[9], hi[9];
#pragma unroll
    for (int q = 0; q < 9; q++) { lo[q] = INT_MAX; hi[q] = INT_MIN; }
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        int comp, i, j, k;
        face_decode(F, (size_t)rowface[r], comp, i, j, k);
#pragma unroll
        for (int c = 0; c < 3; c++)
            if (comp == c) {
                lo[3 * c] = min(lo[3 * c], i); lo[3 * c + 1] = min(lo[3 * c + 1], j); lo[3 * c + 2] = min(lo[3 * c + 2], k);
                hi[3 * c] = max(hi[3 * c], i); hi[3 * c + 1] = max(hi[3 * c + 1], j); hi[3 * c + 2] = max(hi[3 * c + 2], k);
            }
    }
#pragma unroll
    for (int q = 0; q < 9; q++) {
        const int l = __reduce_min_sync(0xffffffffu, lo[q]), h = __reduce_max_sync(0xffffffffu, hi[q]);
        if ((threadIdx.x & 31) == 0) {
            atomicMin(&sb[6 * (q / 3) + q % 3], l);
            atomicMax(&sb[6 * (q / 3) + 3 + q % 3], h);
        }
    }
    __syncthreads();
    if (threadIdx.x < 18) {
        if ((threadIdx.x % 6) < 3) atomicMin(b + threadIdx.x, sb[threadIdx.x]);
        else atomicMax(b + threadIdx.x, sb[threadIdx.x]);
    }
}

// Every row's dense copy: its position, pivot, own factor entries towards the +x', +y', +z'
// neighbours, the 15 operator entries, the couplings to the other components and the rhs.  The
// entries are matched to the neighbour table in column order; a row whose columns do not match
// raises bit 0 of *bad (the system would not be the 15-point pattern).
__global__ void k_dense_fill(FaceDims F, int n, const int *__restrict__ rowface, const int *__restrict__ index,
                             const int *__restrict__ col, const float *__restrict__ val,
                             const float *__restrict__ lval, const unsigned char *__restrict__ tpos,
                             const float *__restrict__ invdiag, const float *__restrict__ rhs, DenseMaps D,
                             float *dense, size_t dtot, int *pos, int *bad) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        int comp, i, j, k;
        face_decode(F, (size_t)rowface[r], comp, i, j, k);
        const DenseMap &M = D.m[comp];
        const long long pl = dense_pos(M, i, j, k);
        if (pl < 0) { atomicOr(bad, 1); continue; }
        const size_t p = (size_t)pl;
        pos[r] = (int)p;
        auto row_at = [&](int c, int a, int b_, int d) -> int {
            // rows lie in 1 .. n-1 along every axis
            if (a < 1 || b_ < 1 || d < 1 || a >= F.ni || b_ >= F.nj || d >= F.nk) return -1;
            const size_t t = c == 0 ? F.U(a, b_, d) : (c == 1 ? F.V(a, b_, d) : F.W(a, b_, d));
            return index[t];
        };
        float A[15], L[15];
        int slot = 0;
#pragma unroll
        for (int e = 0; e < 15; e++) {
            const Nb nb = c_nb[comp][e];
            const int nr = row_at(nb.comp, i + nb.di, j + nb.dj, k + nb.dk);
            A[e] = 0.0f;
            L[e] = 0.0f;
            if (nr >= 0) {
                if (slot < SLOTS && col[SL(r, slot)] == nr) {
                    A[e] = val[SL(r, slot)];
                    if (nr > r) L[e] = lval[SL(r, slot)];   // L(nr, r): row r holds its column
                    else if (nr < r) {
                        const unsigned tp = tpos[SL(r, slot)];
                        if (tp < (unsigned)SLOTS) L[e] = lval[SL(nr, tp)];   // L(r, nr): held by row nr
                    }
                    slot++;
                } else {
                    atomicOr(bad, 1);
                }
            }
        }
        if (slot < SLOTS && col[SL(r, slot)] >= 0) atomicOr(bad, 1);   // an entry the table does not hold
        const int o = nb_own(comp);
        const float lv[3] = {L[o + 4], L[o + 5], L[o + 6]};   // towards +x, +y, +z of the face grid
        dense[DF_INV * dtot + p] = invdiag[r];
        dense[DF_LX * dtot + p] = lv[M.perm[0]];
        dense[DF_LY * dtot + p] = lv[M.perm[1]];
        dense[DF_LZ * dtot + p] = lv[M.perm[2]];
#pragma unroll
        for (int e = 0; e < 15; e++) dense[(DF_A0 + e) * dtot + p] = A[e];
#pragma unroll
        for (int m = 0; m < 8; m++) {
            float x = 0.0f;
            if (m < xf_count(comp)) x = L[m];
            else if (comp < 2 && m >= xb_field(comp)) x = L[xb_first(comp) + m - xb_field(comp)];
            dense[(DF_X0 + m) * dtot + p] = x;
        }
        dense[DF_B * dtot + p] = rhs[r];
    }
}

// Dense kernels walk one component's box line by line (a line: fixed dense y' and z', cells along
// x').  Every component's box uses the same axis order, so a neighbour entry (component c', offset
// d) of a cell at dense (a0, a1, a2) sits at dense (a0 + t0, a1 + t1, a2 + t2) of c' with
// t = d + (origin_c - origin_c') in dense axes: per line, each entry is a row base and an x' range.
struct LineEntry {
    long long base;   // dense index of c' at x' = 0 of the entry's line, shifted by t0 (may be negative)
    int lo, hi;       // the entry exists for lo <= a0 < hi (an empty range: not on this line)
};
__device__ inline LineEntry line_entry(const DenseMaps &D, int c, int e, int a1, int a2) {
    const DenseMap &M = D.m[c];
    const Nb nb = c_nb[c][e];
    const DenseMap &T = D.m[nb.comp];
    const int d[3] = {nb.di + M.i0 - T.i0, nb.dj + M.j0 - T.j0, nb.dk + M.k0 - T.k0};
    const int t0 = d[M.perm[0]], t1 = d[M.perm[1]], t2 = d[M.perm[2]];
    const int b1 = a1 + t1, b2 = a2 + t2;
    LineEntry L;
    if (b1 < 0 || b1 >= T.e[T.perm[1]] || b2 < 0 || b2 >= T.e[T.perm[2]]) {
        L.base = 0; L.lo = 0; L.hi = 0;
        return L;
    }
    L.base = (long long)T.base + (long long)T.pitch * ((long long)b1 + (long long)T.rows * b2) + t0;
    L.lo = -t0;
    L.hi = T.e[T.perm[0]] - t0;
    return L;
}

// The dense kernels give each warp one line at a time; a lane takes 4 consecutive cells (16-byte
// loads of the entries, which start on 16-byte boundaries: the row length is a multiple of 4 and
// every field and component starts on a 64-element boundary).  Cells of the row padding compute +0.
constexpr int DL_WARPS = 4;

// z = A s over component c's box: each row's entries in its column order (the reference's
// FixedSparseMatrix product order)
__global__ void __launch_bounds__(32 * DL_WARPS) k_dense_spmv(DenseMaps D, int c, const float *__restrict__ dense,
                                                              size_t dtot, const float *__restrict__ s, float *z,
                                                              const int *done) {
    if (done && *done) return;
    const DenseMap &M = D.m[c];
    const int nx = M.e[M.perm[0]], lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ LineEntry L[DL_WARPS][15];
    const int nlines = M.rows * M.planes;
    for (int line = blockIdx.x * DL_WARPS + warp; line < nlines; line += gridDim.x * DL_WARPS) {
        if (lane < 15) L[warp][lane] = line_entry(D, c, lane, line % M.rows, line / M.rows);
        __syncwarp();
        const size_t row = M.base + (size_t)M.pitch * line;
        for (int a0 = 4 * lane; a0 < nx; a0 += 128) {
            const size_t p = row + a0;
            float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
            for (int e = 0; e < 15; e++) {
                const LineEntry le = L[warp][e];
                const float4 a = *reinterpret_cast<const float4 *>(dense + (DF_A0 + e) * dtot + p);
                const float av[4] = {a.x, a.y, a.z, a.w};
                const float *sp = s + le.base;
#pragma unroll
                for (int k = 0; k < 4; k++)
                    if (a0 + k >= le.lo && a0 + k < le.hi) acc[k] += av[k] * sp[a0 + k];
            }
            *reinterpret_cast<float4 *>(z + p) = make_float4(acc[0], acc[1], acc[2], acc[3]);
        }
        __syncwarp();
    }
}

// forward: rin = r minus the couplings to the earlier components (component c = 1, 2), ascending
template <int C>
__global__ void __launch_bounds__(32 * DL_WARPS) k_dense_fold_fwd(DenseMaps D, const float *__restrict__ dense,
                                                                  size_t dtot, const float *__restrict__ r,
                                                                  const float *__restrict__ q, float *rin,
                                                                  const int *done) {
    if (done && *done) return;
    constexpr int NE = 4 * C;
    const DenseMap &M = D.m[C];
    const int nx = M.e[M.perm[0]], lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ LineEntry L[DL_WARPS][NE];
    const int nlines = M.rows * M.planes;
    for (int line = blockIdx.x * DL_WARPS + warp; line < nlines; line += gridDim.x * DL_WARPS) {
        if (lane < NE) L[warp][lane] = line_entry(D, C, lane, line % M.rows, line / M.rows);
        __syncwarp();
        const size_t row = M.base + (size_t)M.pitch * line;
        for (int a0 = 4 * lane; a0 < nx; a0 += 128) {
            const size_t p = row + a0;
            const float4 r4 = *reinterpret_cast<const float4 *>(r + p);
            float x[4] = {r4.x, r4.y, r4.z, r4.w};
#pragma unroll
            for (int m = 0; m < NE; m++) {
                const LineEntry le = L[warp][m];
                const float4 a = *reinterpret_cast<const float4 *>(dense + (DF_X0 + m) * dtot + p);
                const float av[4] = {a.x, a.y, a.z, a.w};
                const float *qp = q + le.base;
#pragma unroll
                for (int k = 0; k < 4; k++)
                    if (a0 + k >= le.lo && a0 + k < le.hi) x[k] -= av[k] * qp[a0 + k];
            }
            *reinterpret_cast<float4 *>(rin + p) = make_float4(x[0], x[1], x[2], x[3]);
        }
        __syncwarp();
    }
}

// backward: q of component c (0, 1) minus its couplings to the later components, ascending
template <int C>
__global__ void __launch_bounds__(32 * DL_WARPS) k_dense_fold_bwd(DenseMaps D, const float *__restrict__ dense,
                                                                  size_t dtot, float *q, const int *done) {
    if (done && *done) return;
    constexpr int NE = 8 - 4 * C, E0 = C == 0 ? 7 : 11, F0 = C == 0 ? 0 : 4;
    const DenseMap &M = D.m[C];
    const int nx = M.e[M.perm[0]], lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ LineEntry L[DL_WARPS][NE];
    const int nlines = M.rows * M.planes;
    for (int line = blockIdx.x * DL_WARPS + warp; line < nlines; line += gridDim.x * DL_WARPS) {
        if (lane < NE) L[warp][lane] = line_entry(D, C, E0 + lane, line % M.rows, line / M.rows);
        __syncwarp();
        const size_t row = M.base + (size_t)M.pitch * line;
        for (int a0 = 4 * lane; a0 < nx; a0 += 128) {
            const size_t p = row + a0;
            const float4 q4 = *reinterpret_cast<const float4 *>(q + p);
            float x[4] = {q4.x, q4.y, q4.z, q4.w};
#pragma unroll
            for (int m = 0; m < NE; m++) {
                const LineEntry le = L[warp][m];
                const float4 a = *reinterpret_cast<const float4 *>(dense + (DF_X0 + F0 + m) * dtot + p);
                const float av[4] = {a.x, a.y, a.z, a.w};
                const float *qp = q + le.base;
#pragma unroll
                for (int k = 0; k < 4; k++)
                    if (a0 + k >= le.lo && a0 + k < le.hi) x[k] -= av[k] * qp[a0 + k];
            }
            *reinterpret_cast<float4 *>(q + p) = make_float4(x[0], x[1], x[2], x[3]);
        }
        __syncwarp();
    }
}

__global__ void k_gather_rows(int n, const int *__restrict__ pos, const float *__restrict__ src, float *dst) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) dst[r] = src[pos[r]];
}

__global__ void k_scatter_rows(int n, const int *__restrict__ pos, const float *__restrict__ src, float *dst) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) dst[pos[r]] = src[r];
}

// out = a - b
__global__ void k_sub(size_t n, const float *__restrict__ a, const float *__restrict__ b, float *out) {
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
        out[t] = a[t] - b[t];
}

// ---- PCG vectors (pcgsolver.h:268-322): float vectors, FP64 dot products ----
__global__ void k_spmv(int n, const int *__restrict__ col, const float *__restrict__ val,
                       const float *__restrict__ s, float *z) {
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        float acc = 0.0f;   // FixedSparseMatrix multiply: row entries in column order
        for (int t = 0; t < SLOTS; t++) {
            const int c = col[SL(r, t)];
            if (c >= 0) acc += val[SL(r, t)] * s[c];
        }
        z[r] = acc;
    }
}

constexpr int RB = 256;
constexpr int RED_BLOCKS = 1024;

// Dot products: each thread sums its products in float over runs of 8 and adds the run sums in
// FP64 (FP64 issue is scarce on this part: one FP64 add per 8 elements), then the block and the
// partials are summed in FP64 in a fixed order.
__global__ void __launch_bounds__(RB) k_dot_partial(int n, const float *__restrict__ a, const float *__restrict__ b,
                                                    double *part, const int *done) {
    if (done && *done) return;
    __shared__ double sm[RB / 32];
    double acc = 0.0;
    const bool v4 = (reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b)) % 16 == 0;
    const int n4 = v4 ? n / 4 : 0;
    // 4 products a thread step (16-byte loads), two steps to a float run
    for (int i = blockIdx.x * RB + threadIdx.x; i < n4; i += 2 * gridDim.x * RB) {
        const float4 x = reinterpret_cast<const float4 *>(a)[i], y = reinterpret_cast<const float4 *>(b)[i];
        float run = x.x * y.x + x.y * y.y + x.z * y.z + x.w * y.w;
        const int i2 = i + gridDim.x * RB;
        if (i2 < n4) {
            const float4 x2 = reinterpret_cast<const float4 *>(a)[i2], y2 = reinterpret_cast<const float4 *>(b)[i2];
            run += x2.x * y2.x + x2.y * y2.y + x2.z * y2.z + x2.w * y2.w;
        }
        acc += (double)run;
    }
    for (int i = 4 * n4 + blockIdx.x * RB + threadIdx.x; i < n; i += gridDim.x * RB) acc += (double)(a[i] * b[i]);
    const double t = block_sum<RB>(acc, sm);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

__global__ void __launch_bounds__(RB) k_absmax_partial(int n, const float *__restrict__ a, double *part) {
    __shared__ double sm[RB / 32];
    float m = 0.0f;   // a max is exact in float
    for (int i = blockIdx.x * RB + threadIdx.x; i < n; i += gridDim.x * RB) m = fmaxf(m, fabsf(a[i]));
    const double t = block_max<RB>((double)m, sm);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// sums (or maxes) the partials in a fixed order into out[slot]; with slot 1 (s.z) also the step
// alpha = rho / (s.z) into out[4], with slot 2 (rho_new) beta = rho_new / rho into out[5].  With ctl
// (device convergence control: [0] done, [1] residual checks) it does nothing once done, and slot 3
// (|r|inf) counts a check and sets done when the float residual is <= out[6] (the stop).
__global__ void __launch_bounds__(RB) k_finish(const double *__restrict__ part, int nb, int is_max, double *out,
                                               int slot, int *ctl) {
    if (ctl && ctl[0]) return;
    __shared__ double sm[RB / 32];
    double acc = 0.0;
    for (int i = threadIdx.x; i < nb; i += RB) acc = is_max ? fmax(acc, part[i]) : acc + part[i];
    const double t = is_max ? block_max<RB>(acc, sm) : block_sum<RB>(acc, sm);
    if (threadIdx.x == 0) {
        out[slot] = t;
        if (slot == 1) out[4] = out[0] / t;
        if (slot == 2) out[5] = t / out[0];
        if (ctl && slot == 3) {
            ctl[1] += 1;
            if ((double)(float)t <= out[6]) ctl[0] = 1;
        }
    }
}

// x += alpha s; r -= alpha z (pcgsolver.h:299-301); with part, also the block maxima of |r|
__global__ void __launch_bounds__(RB) k_update_xr(int n, const double *__restrict__ sc, const float *__restrict__ s,
                                                  const float *__restrict__ z, float *x, float *r, double *part,
                                                  const int *done) {
    if (done && *done) return;
    __shared__ double sm[RB / 32];
    const double alpha = sc[4];
    const float a = (float)alpha, na = (float)-alpha;
    float m = 0.0f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        x[i] += a * s[i];
        const float ri = r[i] + na * z[i];
        r[i] = ri;
        m = fmaxf(m, fabsf(ri));
    }
    if (part) {
        const double t = block_max<RB>((double)m, sm);
        if (threadIdx.x == 0) part[blockIdx.x] = t;
    }
}

// s = z + beta s (pcgsolver.h:313-316)
__global__ void k_update_s(int n, const double *__restrict__ sc, const float *__restrict__ z, float *s,
                           const int *done) {
    if (done && *done) return;
    const float beta = (float)sc[5];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) s[i] = z[i] + beta * s[i];
}

__global__ void k_rho_shift(double *sc, const int *done) {
    if (!(done && *done)) sc[0] = sc[2];
}

// _applySolutionToVelocityField (viscositysolver.cpp:869-901): every face cleared, rows set
__global__ void k_apply_solution(FaceDims F, const int *__restrict__ index, const float *__restrict__ x, float *u,
                                 float *v, float *w) {
    const size_t nf = F.nu + F.nv + F.nw;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < nf; t += (size_t)gridDim.x * blockDim.x) {
        const int r = index[t];
        const float val = r >= 0 ? x[r] : 0.0f;
        if (t < F.nu) u[t] = val;
        else if (t < F.nu + F.nv) v[t - F.nu] = val;
        else w[t - F.nu - F.nv] = val;
    }
}

}  // namespace

// ------------------------------------------------------------------------------------------
void ViscWork::reserve_grids(Dims d) {
    const size_t nf = d.faces(0) + d.faces(1) + d.faces(2);
    const size_t nn = (size_t)(d.ni + 1) * (d.nj + 1) * (d.nk + 1);
    state.reserve(nf); flag.reserve(nf); scan.reserve(nf + 1); index.reserve(nf);
    valid.reserve(nn); valid2.reserve(nn);
    sub.reserve(8 * d.cells());
    const size_t vn = d.cells() + d.faces(0) + d.faces(1) + d.faces(2) + (size_t)d.ni * (d.nj + 1) * (d.nk + 1) +
                      (size_t)(d.ni + 1) * d.nj * (d.nk + 1) + (size_t)(d.ni + 1) * (d.nj + 1) * d.nk;
    vol.reserve(vn);
    scan_tmp.reserve(scan_scratch_ints(nf + 1) + 64);
    partials.reserve(RED_BLOCKS);
    scalars.reserve(8);
}

ViscVolumes ViscWork::volumes(Dims d) const {
    ViscVolumes V;
    float *p = vol.p;
    V.center = p; p += d.cells();
    V.u = p; p += d.faces(0);
    V.v = p; p += d.faces(1);
    V.w = p; p += d.faces(2);
    V.eu = p; p += (size_t)d.ni * (d.nj + 1) * (d.nk + 1);
    V.ev = p; p += (size_t)(d.ni + 1) * d.nj * (d.nk + 1);
    V.ew = p;
    return V;
}

void ViscWork::reserve_rows(int n) {
    const size_t m = (size_t)std::max(n, 1);
    rowface.reserve(m); col.reserve(m * SLOTS); val.reserve(m * SLOTS); lval.reserve(m * SLOTS);
    tpos.reserve(m * SLOTS); rhs.reserve(m); invdiag.reserve(m); adiag.reserve(m); level.reserve(m);
    lrows.reserve(m); x.reserve(m); r.reserve(m); z.reserve(m); s.reserve(m); x0.reserve(m);
}

// Builds the system for (u, v, w) (already constrained); returns the number of rows.
int visc_build(Dims d, double dx, double dt, float visc, const float *liquid, const float *solid, const float *u,
               const float *v, const float *w, ViscWork &W, int *host_int, cudaStream_t st, unsigned long long &launches) {
    const FaceDims F = face_dims(d);
    const size_t nf = F.nu + F.nv + F.nw;
    const size_t nn = (size_t)(d.ni + 1) * (d.nj + 1) * (d.nk + 1);
    W.reserve_grids(d);
    k_face_state<<<grid_for(nf, 256, 152u * 32u), 256, 0, st>>>(F, solid, W.state);
    k_valid_init<<<grid_for(nn, 256, 152u * 32u), 256, 0, st>>>(d, liquid, W.valid);
    k_valid_dilate<<<grid_for(nn, 256, 152u * 32u), 256, 0, st>>>(d, W.valid, W.valid2);
    k_valid_dilate<<<grid_for(nn, 256, 152u * 32u), 256, 0, st>>>(d, W.valid2, W.valid);
    k_subcell<<<grid_for(8 * d.cells(), 128, 152u * 64u), 128, 0, st>>>(d, dx, (float)dx, W.valid, liquid, W.sub);
    const ViscVolumes V = W.volumes(d);
    FFGPU_CUDA(cudaMemsetAsync(W.vol.p, 0, W.vol.n * sizeof(float), st));
    k_volumes<<<grid_for(d.cells(), 128, 152u * 32u), 128, 0, st>>>(d, W.valid, W.sub, V);
    const VolView VV = vol_view(d, V);
    k_row_flags<<<grid_for(nf, 256, 152u * 32u), 256, 0, st>>>(F, VV, W.state, W.flag);
    launch_exclusive_scan(W.flag, W.scan, nf, W.scan_tmp, st);
    // rows: U faces, then V, then W
    FFGPU_CUDA(cudaMemcpyAsync(host_int, W.scan.p + nf, sizeof(int), cudaMemcpyDeviceToHost, st));
    FFGPU_CUDA(cudaMemcpyAsync(host_int + 1, W.scan.p + F.nu, sizeof(int), cudaMemcpyDeviceToHost, st));
    FFGPU_CUDA(cudaMemcpyAsync(host_int + 2, W.scan.p + F.nu + F.nv, sizeof(int), cudaMemcpyDeviceToHost, st));
    FFGPU_CUDA(cudaStreamSynchronize(st));
    const int n = host_int[0];
    launches += 12;
    W.n = n;
    W.grid = d;
    W.first[0] = 0; W.first[1] = host_int[1]; W.first[2] = host_int[2]; W.first[3] = n;
    if (n == 0) return 0;
    W.reserve_rows(n);
    k_row_index<<<grid_for(nf, 256, 152u * 32u), 256, 0, st>>>(nf, W.flag, W.scan, W.index, W.rowface);
    k_rows<<<grid_for(n, 128, 152u * 32u), 128, 0, st>>>(F, VV, (float)dx, (float)dt, visc, W.state, W.index, W.rowface, n,
                                                         u, v, w, W.col, W.val, W.rhs, W.level, W.x0);
    // levels: U at i+j+k, V at +2, W at +4
    const int nlev = (d.ni - 1) + (d.nj - 1) + (d.nk - 1) + 4 + 1;
    W.lcount.reserve((size_t)nlev + 1);
    W.lcursor.reserve((size_t)nlev + 1);
    FFGPU_CUDA(cudaMemsetAsync(W.lcount.p, 0, (size_t)(nlev + 1) * sizeof(int), st));
    FFGPU_CUDA(cudaMemsetAsync(W.lcursor.p, 0, (size_t)(nlev + 1) * sizeof(int), st));
    k_level_count<<<grid_for(n, 256, 152u * 16u), 256, 0, st>>>(n, W.level, W.lcount);
    std::vector<int> cnt((size_t)nlev);
    FFGPU_CUDA(cudaMemcpyAsync(cnt.data(), W.lcount.p, (size_t)nlev * sizeof(int), cudaMemcpyDeviceToHost, st));
    FFGPU_CUDA(cudaStreamSynchronize(st));
    W.lstart.assign((size_t)nlev + 1, 0);
    for (int L = 0; L < nlev; L++) W.lstart[L + 1] = W.lstart[L] + cnt[L];
    FFGPU_CUDA(cudaMemcpyAsync(W.lcount.p, W.lstart.data(), (size_t)(nlev + 1) * sizeof(int), cudaMemcpyHostToDevice,
                               st));
    k_level_scatter<<<grid_for(n, 256, 152u * 16u), 256, 0, st>>>(n, W.level, W.lcount, W.lcursor, W.lrows);
    k_transpose_slots<<<grid_for(n, 128, 152u * 32u), 128, 0, st>>>(n, W.col, W.tpos);
    launches += 6;
    return n;
}

void visc_factor(ViscWork &W, cudaStream_t st, unsigned long long &launches) {
    const int n = W.n;
    k_factor_init<<<grid_for(n, 256, 152u * 16u), 256, 0, st>>>(n, W.col, W.val, W.invdiag, W.adiag, W.lval);
    launches++;
    const int nlev = (int)W.lstart.size() - 1;
    for (int L = 0; L < nlev; L++) {
        const int c = W.lstart[L + 1] - W.lstart[L];
        if (!c) continue;
        k_factor_level<<<grid_for((size_t)c * 16, FL_THREADS, 152u * 32u), FL_THREADS, 0, st>>>(W.lrows.p + W.lstart[L], c, W.col, W.tpos, W.adiag,
                                                                   W.invdiag, W.lval);
        launches++;
    }
}

// co-resident blocks of the cooperative preconditioner on this device (-1: no cooperative launch)
static int coop_precond_blocks() {
    static int cached[64] = {0};
    int dev = 0;
    FFGPU_CUDA(cudaGetDevice(&dev));
    int b = dev < 64 ? cached[dev] : 0;
    if (b == 0) {
        int coop = 0, sms = 0, per = 0;
        FFGPU_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
        FFGPU_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        FFGPU_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_precond_coop, PC_THREADS, 0));
        b = (coop && per > 0) ? sms * per : -1;
        if (dev < 64) cached[dev] = b;
    }
    return b;
}

bool visc_precondition_coop(ViscWork &W, const float *r, float *z, cudaStream_t st, unsigned long long &launches) {
    const int maxb = coop_precond_blocks();
    if (maxb <= 0) return false;
    int nlev = (int)W.lstart.size() - 1;
    int widest = 0;
    for (int L = 0; L < nlev; L++) widest = std::max(widest, W.lstart[L + 1] - W.lstart[L]);
    // one block per SM at most: the grid barrier between levels costs more with more blocks, and a
    // level holds at most a few tens of thousands of rows
    int dev = 0, sms = 1;
    FFGPU_CUDA(cudaGetDevice(&dev));
    FFGPU_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int g = std::max(1, std::min(std::min(maxb, sms), (widest + PC_THREADS - 1) / PC_THREADS));
    const int *rows = W.lrows.p, *start = W.lcount.p, *col = W.col.p;
    const unsigned char *tpos = W.tpos.p;
    const float *lval = W.lval.p, *inv = W.invdiag.p;
    void *args[] = {(void *)&rows, (void *)&start, (void *)&nlev, (void *)&col, (void *)&tpos, (void *)&lval,
                    (void *)&inv, (void *)&r, (void *)&z};
    FFGPU_CUDA(cudaLaunchCooperativeKernel((void *)k_precond_coop, dim3(g), dim3(PC_THREADS), args, 0, st));
    launches++;
    return true;
}

void visc_precondition(ViscWork &W, const float *r, float *z, cudaStream_t st, unsigned long long &launches,
                       int sweeps) {
    const int nlev = (int)W.lstart.size() - 1;
    for (int L = 0; L < nlev; L++) {
        const int c = W.lstart[L + 1] - W.lstart[L];
        if (!c) continue;
        k_lower_level<<<grid_for(c, 128, 152u * 32u), 128, 0, st>>>(W.lrows.p + W.lstart[L], c, W.col, W.tpos, W.lval,
                                                                    W.invdiag, r, z);
        launches++;
    }
    for (int L = nlev - 1; L >= 0 && sweeps > 1; L--) {
        const int c = W.lstart[L + 1] - W.lstart[L];
        if (!c) continue;
        k_upper_level<<<grid_for(c, 128, 152u * 32u), 128, 0, st>>>(W.lrows.p + W.lstart[L], c, W.col, W.lval,
                                                                    W.invdiag, z);
        launches++;
    }
}

// blocks of DL_WARPS lines covering a dense box (at most 152 x 32 blocks; the kernels loop)
static unsigned line_blocks(Dims dc) {
    const size_t lines = (size_t)dc.nj * dc.nk;
    return (unsigned)std::max<size_t>(1, std::min<size_t>((lines + DL_WARPS - 1) / DL_WARPS, 152u * 32u));
}

static DenseMaps dense_maps(const ViscWork &W) {
    DenseMaps D;
    for (int c = 0; c < 3; c++) {
        const ViscWork::Box &bx = W.cbox[c];
        DenseMap &M = D.m[c];
        M.i0 = bx.i0; M.j0 = bx.j0; M.k0 = bx.k0;
        M.e[0] = bx.i1 - bx.i0 + 1; M.e[1] = bx.j1 - bx.j0 + 1; M.e[2] = bx.k1 - bx.k0 + 1;
        for (int a = 0; a < 3; a++) M.perm[a] = W.cperm[c][a];
        M.pitch = std::max(W.cdim[c].ni, 1);
        M.rows = std::max(W.cdim[c].nj, 1);
        M.planes = W.cdim[c].nk;
        M.base = W.cbase[c];
        M.cells = W.cdim[c].cells();
    }
    return D;
}

void visc_wavefront_setup(ViscWork &W, cudaStream_t st, unsigned long long &launches) {
    const FaceDims F = face_dims(W.grid);
    const int n = W.n;
    W.boxes.reserve(19);
    k_boxes_init<<<1, 32, 0, st>>>(W.boxes);
    k_comp_boxes<<<grid_for(n, 256, 152u * 4u), 256, 0, st>>>(F, n, W.rowface, W.boxes);
    int b[18];
    FFGPU_CUDA(cudaMemcpyAsync(b, W.boxes.p, sizeof(b), cudaMemcpyDeviceToHost, st));
    FFGPU_CUDA(cudaStreamSynchronize(st));
    launches += 2;
    // One axis order for the three boxes (so a neighbour of another component is a fixed dense
    // offset away): the grid's, or (axis_order) the union box's shortest axis swept, as the pressure
    // solve's mixed copy does (a shorter wavefront chain for boxes long in z).
    AxisMap m{{0, 1, 2}};
    if (W.axis_order) {
        Bbox u{INT_MAX, INT_MAX, INT_MAX, INT_MIN, INT_MIN, INT_MIN};
        for (int c = 0; c < 3; c++) {
            if (W.first[c + 1] <= W.first[c]) continue;
            u.i0 = std::min(u.i0, b[6 * c]); u.j0 = std::min(u.j0, b[6 * c + 1]); u.k0 = std::min(u.k0, b[6 * c + 2]);
            u.i1 = std::max(u.i1, b[6 * c + 3]); u.j1 = std::max(u.j1, b[6 * c + 4]); u.k1 = std::max(u.k1, b[6 * c + 5]);
        }
        Dims du;
        Bbox pu;
        m = choose_axis_map(u, du, pu);
    }
    size_t tot = 0;
    for (int c = 0; c < 3; c++) {
        const bool any = W.first[c + 1] > W.first[c];
        ViscWork::Box bx = any ? ViscWork::Box{b[6 * c], b[6 * c + 1], b[6 * c + 2], b[6 * c + 3], b[6 * c + 4], b[6 * c + 5]}
                               : ViscWork::Box{0, 0, 0, -1, -1, -1};
        W.cbox[c] = bx;
        Dims dc{0, 0, 0};
        Bbox pb{0, 0, 0, -1, -1, -1};
        if (any) {
            const int e[3] = {bx.i1 - bx.i0 + 1, bx.j1 - bx.j0 + 1, bx.k1 - bx.k0 + 1};
            const int ne[3] = {e[m.perm[0]], e[m.perm[1]], e[m.perm[2]]};
            pb = Bbox{0, 0, 0, ne[0] - 1, ne[1] - 1, ne[2] - 1};
            dc = Dims{(ne[0] + 3) / 4 * 4, ne[1], ne[2]};
        }
        W.cdim[c] = dc;
        W.cpbox[c] = pb;
        for (int a = 0; a < 3; a++) W.cperm[c][a] = m.perm[a];
        W.cbase[c] = tot;
        tot += (dc.cells() + 63) / 64 * 64;
        if (any) {
            const int cap = mic_wavefront_max_tiles(pb.i1 + 1, pb.j1 + 1);
            if (cap > W.order_cap[c]) {
                W.order[c].reserve((size_t)cap);
                W.order_cap[c] = cap;
                W.order_key[c] = -1;   // new storage: the table is uploaded again
            }
        }
    }
    if (tot >= (size_t)INT_MAX) throw std::runtime_error("Error: viscosity system too large for the wavefront form.\n");
    W.dtot = std::max<size_t>(tot, 64);
    W.dense.reserve(DF_COUNT * W.dtot);
    W.pos.reserve((size_t)std::max(n, 1));
    FFGPU_CUDA(cudaMemsetAsync(W.dense.p, 0, DF_COUNT * W.dtot * sizeof(float), st));
    k_dense_fill<<<grid_for(n, 128, 1u << 20), 128, 0, st>>>(F, n, W.rowface, W.index, W.col, W.val, W.lval, W.tpos,
                                                              W.invdiag, W.rhs, dense_maps(W), W.dense, W.dtot, W.pos,
                                                              W.boxes.p + 18);
    int bad = 0;
    FFGPU_CUDA(cudaMemcpyAsync(&bad, W.boxes.p + 18, sizeof(int), cudaMemcpyDeviceToHost, st));
    FFGPU_CUDA(cudaStreamSynchronize(st));
    launches++;
    if (bad) throw std::runtime_error("Error: viscosity system rows do not match the 15-point pattern.\n");
}

// z = M^-1 r on the dense boxes (r, z: dense vectors); sweeps = 1 stops after L z = r
static void visc_precondition_dense(ViscWork &W, const float *r, float *z, const WfWork &ww, int sweeps,
                                    cudaStream_t st, unsigned long long &launches, const int *done = nullptr) {
    float *const f = W.dense.p;
    float *const rin = f + DF_RIN * W.dtot;
    const DenseMaps D = dense_maps(W);
    auto rows = [&](int c) { return W.first[c + 1] - W.first[c]; };
    auto sweep = [&](int c, bool forward, const float *in) {
        const size_t o = W.cbase[c];
        const FactorView<float> Fc{f + DF_INV * W.dtot + o, f + DF_LX * W.dtot + o, f + DF_LY * W.dtot + o,
                                   f + DF_LZ * W.dtot + o};
        WfWork w = ww;
        w.order = W.order[c];
        w.order_key = &W.order_key[c];
        w.max_tiles = W.order_cap[c];
        w.done = done;
        mic_wavefront_sweep<float>(W.cdim[c], W.cpbox[c], Fc, in ? in + o : nullptr, z + o, w, forward, st);
        launches++;
    };
    for (int c = 0; c < 3; c++) {
        if (!rows(c)) continue;
        if (c > 0) {
            const unsigned nb = line_blocks(W.cdim[c]);
            if (c == 1) k_dense_fold_fwd<1><<<nb, 32 * DL_WARPS, 0, st>>>(D, f, W.dtot, r, z, rin, done);
            else k_dense_fold_fwd<2><<<nb, 32 * DL_WARPS, 0, st>>>(D, f, W.dtot, r, z, rin, done);
            launches++;
        }
        sweep(c, true, c > 0 ? rin : r);
    }
    if (sweeps < 2) return;
    for (int c = 2; c >= 0; c--) {
        if (!rows(c)) continue;
        if (c < 2) {
            const unsigned nb = line_blocks(W.cdim[c]);
            if (c == 0) k_dense_fold_bwd<0><<<nb, 32 * DL_WARPS, 0, st>>>(D, f, W.dtot, z, done);
            else k_dense_fold_bwd<1><<<nb, 32 * DL_WARPS, 0, st>>>(D, f, W.dtot, z, done);
            launches++;
        }
        sweep(c, false, nullptr);
    }
}

void visc_precondition_wf(ViscWork &W, const float *r, float *z, const WfWork &ww, int sweeps, cudaStream_t st,
                          unsigned long long &launches) {
    // rows -> dense (the rhs field is reused as the input), apply, dense -> rows
    float *const f = W.dense.p;
    float *const rd = f + DF_R * W.dtot, *const qd = f + DF_Q * W.dtot;
    k_scatter_rows<<<grid_for(W.n, 256, 152u * 16u), 256, 0, st>>>(W.n, W.pos, r, rd);
    visc_precondition_dense(W, rd, qd, ww, sweeps, st, launches);
    k_gather_rows<<<grid_for(W.n, 256, 152u * 16u), 256, 0, st>>>(W.n, W.pos, qd, z);
    launches += 2;
}

static void reduce(int n, const float *a, const float *b, double *part, double *out, int slot, cudaStream_t st,
                   int *ctl = nullptr) {
    const int nb = (int)std::min<size_t>(RED_BLOCKS, std::max<size_t>(1, ((size_t)n + RB - 1) / RB));
    if (b) k_dot_partial<<<nb, RB, 0, st>>>(n, a, b, part, ctl);
    else k_absmax_partial<<<nb, RB, 0, st>>>(n, a, part);
    k_finish<<<1, RB, 0, st>>>(part, nb, b ? 0 : 1, out, slot, ctl);
}

// PCGSolver<float>::solve (pcgsolver.h:268-322) on the built system; x starts at 0.  Scalars
// slots: 0 rho, 1 s.z, 2 rho_new, 3 |r|inf.  Returns success; iterations and residual out.
bool visc_solve(ViscWork &W, double tol, int maxit, double *host_dbl, int *host_int, const WfWork &ww, int &iters,
                float &residual, bool &wait_failed, cudaStream_t st, unsigned long long &launches,
                cudaEvent_t factored) {
    wait_failed = false;
    const int n = W.n;
    const unsigned g = grid_for(n, 256, 152u * 16u);
    FFGPU_CUDA(cudaMemsetAsync(W.x.p, 0, (size_t)n * sizeof(float), st));
    FFGPU_CUDA(cudaMemcpyAsync(W.r.p, W.rhs.p, (size_t)n * sizeof(float), cudaMemcpyDeviceToDevice, st));
    reduce(n, W.r, nullptr, W.partials, W.scalars, 3, st);
    FFGPU_CUDA(cudaMemcpyAsync(host_dbl, W.scalars.p + 3, sizeof(double), cudaMemcpyDeviceToHost, st));
    FFGPU_CUDA(cudaStreamSynchronize(st));
    launches += 2;
    residual = (float)host_dbl[0];
    iters = 0;
    if (residual == 0.0f) {
        if (factored) FFGPU_CUDA(cudaEventRecord(factored, st));
        return true;
    }
    const float tolf = std::max((float)tol, 1e-30f);
    const double tolr = (double)(tolf * residual);
    const double stop = std::min(tolr, 1.0);
    visc_factor(W, st, launches);
    // The preconditioner: the tiled wavefront blocks, with the whole PCG on the dense boxes; or, in
    // row order, one launch per level and sweep (captured once as a graph and replayed) or one
    // cooperative launch per application.
    const bool wf = W.precond == ViscWork::VP_WAVEFRONT || W.precond == ViscWork::VP_WAVEFRONT_GRID_AXES;
    W.axis_order = W.precond == ViscWork::VP_WAVEFRONT ? 1 : 0;
    const bool coop = W.precond == ViscWork::VP_COOP && coop_precond_blocks() > 0;
    unsigned long long per_apply = 0;
    cudaGraphExec_t exec = nullptr;
    if (wf) visc_wavefront_setup(W, st, launches);
    if (factored) FFGPU_CUDA(cudaEventRecord(factored, st));
    if (!coop && !wf) {
        cudaGraph_t graph = nullptr;
        FFGPU_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        visc_precondition(W, W.r, W.z, st, per_apply);
        FFGPU_CUDA(cudaStreamEndCapture(st, &graph));
        FFGPU_CUDA(cudaGraphInstantiate(&exec, graph, 0));
        FFGPU_CUDA(cudaGraphDestroy(graph));
    }
    struct ExecGuard {
        cudaGraphExec_t e;
        ~ExecGuard() { if (e) cudaGraphExecDestroy(e); }
    } guard{exec};
    // the vectors: rows (n) or dense boxes (dtot; cells without a row stay +0)
    float *const f = W.dense.p;
    const int nv = wf ? (int)W.dtot : n;
    float *const vx = wf ? f + DF_XV * W.dtot : W.x.p;
    float *const vr = wf ? f + DF_R * W.dtot : W.r.p;
    float *const vs = wf ? f + DF_S * W.dtot : W.s.p;
    float *const vz = wf ? f + DF_Q * W.dtot : W.z.p;    // M^-1 r
    float *const va = wf ? f + DF_AZ * W.dtot : W.z.p;   // A s
    const unsigned gv = grid_for((size_t)nv, 256, 152u * 16u);
    const DenseMaps D = wf ? dense_maps(W) : DenseMaps{};
    if (wf) FFGPU_CUDA(cudaMemcpyAsync(vr, f + DF_B * W.dtot, W.dtot * sizeof(float), cudaMemcpyDeviceToDevice, st));
    if (W.warm) {
        // start from the field before the solve (x0, one value per row) instead of zero: r = b - A x0.
        // The stop stays tol |b|inf, the zero start's.
        if (wf) {
            k_scatter_rows<<<g, 256, 0, st>>>(n, W.pos, W.x0, vx);   // cells without a row stay +0
            for (int c = 0; c < 3; c++)
                if (W.first[c + 1] > W.first[c])
                    k_dense_spmv<<<line_blocks(W.cdim[c]), 32 * DL_WARPS, 0, st>>>(D, c, f, W.dtot, vx, va, nullptr);
            k_sub<<<gv, 256, 0, st>>>((size_t)nv, f + DF_B * W.dtot, va, vr);
        } else {
            FFGPU_CUDA(cudaMemcpyAsync(W.x.p, W.x0.p, (size_t)n * sizeof(float), cudaMemcpyDeviceToDevice, st));
            k_spmv<<<g, 256, 0, st>>>(n, W.col, W.val, W.x, W.z);
            k_sub<<<gv, 256, 0, st>>>((size_t)n, W.rhs, W.z, W.r);
        }
        launches += 5;
    }
    auto apply = [&]() {
        if (wf) {
            visc_precondition_dense(W, vr, vz, ww, 2, st, launches);
        } else if (coop) {
            visc_precondition_coop(W, W.r, W.z, st, launches);
        } else {
            FFGPU_CUDA(cudaGraphLaunch(exec, st));
            launches += per_apply;
        }
    };
    auto finish = [&]() {   // the solution in row order
        if (wf) {
            k_gather_rows<<<g, 256, 0, st>>>(n, W.pos, vx, W.x);
            launches++;
        }
    };
    apply();
    reduce(nv, vz, vr, W.partials, W.scalars, 0, st);
    FFGPU_CUDA(cudaMemcpyAsync(vs, vz, (size_t)nv * sizeof(float), cudaMemcpyDeviceToDevice, st));
    FFGPU_CUDA(cudaMemcpyAsync(host_dbl, W.scalars.p, sizeof(double), cudaMemcpyDeviceToHost, st));
    FFGPU_CUDA(cudaStreamSynchronize(st));
    launches += 2;
    const double rho0 = host_dbl[0];
    if (rho0 == 0 || rho0 != rho0) {
        finish();
        return false;
    }
    // one iteration (pcgsolver.h:296-318); with ctl, every kernel does nothing once the device has
    // seen the residual at or below the stop
    auto iteration = [&](int *ctl) {
        if (wf) {
            for (int c = 0; c < 3; c++)
                if (W.first[c + 1] > W.first[c])
                    k_dense_spmv<<<line_blocks(W.cdim[c]), 32 * DL_WARPS, 0, st>>>(D, c, f, W.dtot, vs, va, ctl);
            launches += 2;
        } else {
            k_spmv<<<g, 256, 0, st>>>(n, W.col, W.val, vs, va);
        }
        reduce(nv, vs, va, W.partials, W.scalars, 1, st, ctl);
        {   // the update and |r|inf in one pass: block maxima, then the fixed-order maximum
            const int nb = (int)std::min<size_t>(RED_BLOCKS, std::max<size_t>(1, ((size_t)nv + RB - 1) / RB));
            k_update_xr<<<nb, RB, 0, st>>>(nv, W.scalars, vs, va, vx, vr, W.partials, ctl);
            k_finish<<<1, RB, 0, st>>>(W.partials, nb, 1, W.scalars, 3, ctl);
        }
        launches += 5;
    };
    auto second_half = [&](int *ctl) {
        if (wf) visc_precondition_dense(W, vr, vz, ww, 2, st, launches, ctl);
        else apply();
        reduce(nv, vz, vr, W.partials, W.scalars, 2, st, ctl);
        k_update_s<<<gv, 256, 0, st>>>(nv, W.scalars, vz, vs, ctl);
        k_rho_shift<<<1, 1, 0, st>>>(W.scalars, ctl);
        launches += 4;
    };
    if (wf) {
        // Device-side stopping: batches of 8 iterations between host checks, replayed from a graph
        // captured once per solve (the sweeps take their tags from the device counter); the stop
        // (the float residual against tol |b|inf, pcgsolver.h:300-305) is tested by the device.
        W.ctl.reserve(2);
        FFGPU_CUDA(cudaMemsetAsync(W.ctl.p, 0, 2 * sizeof(int), st));
        host_dbl[1] = stop;
        FFGPU_CUDA(cudaMemcpyAsync(W.scalars.p + 6, host_dbl + 1, sizeof(double), cudaMemcpyHostToDevice, st));
        constexpr int BATCH = 8;
        struct GraphGuard {
            cudaGraphExec_t e = nullptr;
            ~GraphGuard() { if (e) cudaGraphExecDestroy(e); }
        } gb;
        unsigned long long per_batch = 0;
        unsigned int sweeps = 0;
        for (int enq = 0; enq < maxit;) {
            const int batch = std::min(BATCH, maxit - enq);
            if (batch == BATCH) {
                if (!gb.e) {
                    wf_reserve_epochs(ww, 6u * BATCH, st);
                    const unsigned int tag = *ww.epoch;
                    const unsigned long long l0 = launches;
                    cudaGraph_t gr = nullptr;
                    FFGPU_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
                    for (int q = 0; q < BATCH; q++) { iteration(W.ctl); second_half(W.ctl); }
                    FFGPU_CUDA(cudaStreamEndCapture(st, &gr));
                    const cudaError_t ie = cudaGraphInstantiate(&gb.e, gr, 0);
                    cudaGraphDestroy(gr);
                    FFGPU_CUDA(ie);
                    sweeps = *ww.epoch - tag;   // the sweeps one batch runs
                    *ww.epoch = tag;            // nothing ran yet
                    per_batch = launches - l0;
                    launches = l0;
                }
                wf_reserve_epochs(ww, sweeps, st);
                FFGPU_CUDA(cudaGraphLaunch(gb.e, st));
                *ww.epoch += sweeps;
                launches += per_batch;
            } else {
                for (int q = 0; q < batch; q++) { iteration(W.ctl); second_half(W.ctl); }
            }
            enq += batch;
            FFGPU_CUDA(cudaMemcpyAsync(host_int + 4, W.ctl.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
            FFGPU_CUDA(cudaMemcpyAsync(host_dbl, W.scalars.p + 3, sizeof(double), cudaMemcpyDeviceToHost, st));
            FFGPU_CUDA(cudaMemcpyAsync(host_int + 3, ww.error, sizeof(unsigned int), cudaMemcpyDeviceToHost, st));
            FFGPU_CUDA(cudaStreamSynchronize(st));
            if (host_int[3] != 0) {   // a face wait gave up: the preconditioned vectors are meaningless
                wait_failed = true;
                iters = host_int[5];
                return false;
            }
            residual = (float)host_dbl[0];
            if (host_int[4]) {
                iters = host_int[5];
                finish();
                return true;
            }
        }
        iters = maxit;
        finish();
        return false;
    }
    for (int it = 0; it < maxit; it++) {
        iteration(nullptr);
        FFGPU_CUDA(cudaMemcpyAsync(host_dbl, W.scalars.p + 3, sizeof(double), cudaMemcpyDeviceToHost, st));
        FFGPU_CUDA(cudaStreamSynchronize(st));
        residual = (float)host_dbl[0];
        if ((double)residual <= stop) {
            iters = it + 1;
            return true;
        }
        second_half(nullptr);
    }
    iters = maxit;
    return false;
}

void visc_apply(Dims d, ViscWork &W, float *u, float *v, float *w, cudaStream_t st) {
    const FaceDims F = face_dims(d);
    k_apply_solution<<<grid_for(F.nu + F.nv + F.nw, 256, 152u * 32u), 256, 0, st>>>(F, W.index, W.x, u, v, w);
}

}  // namespace ffgpu
