// Oracle (test infrastructure only): grid-to-particle PIC/FLIP update, RK3 marker
// advection with solid collision handling, marker removal, solid-face constraint.
//   MAC sampling: MACVelocityField::_interpolateLinear{U,V,W} (macvelocityfield.cpp:519-645),
//                 in double like the reference.
//   G2P: _updatePICFLIPMarkerParticleVelocitiesThread (fluidsimulation.cpp:6771-6789).
//   RK3: _RK3 (:7616-7623); collisions: _resolveMarkerParticleCollisions/_resolveCollision
//        (:7636-7721) with the near-solid grid of _updateNearSolidGrid (:5448-5480).
//   Removal: _removeMarkerParticles (:7773-7851), extreme-speed rule (:7723-7771).
//   Constraint: _constrainVelocityFieldThread (:6391-6442), static solids.
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <vector>

using namespace oracle;

namespace {

struct Mac {
    int ni, nj, nk;
    double dx;
    const float *u, *v, *w;
};

inline double tri(const double p[8], double x, double y, double z) {
    return p[0] * (1 - x) * (1 - y) * (1 - z) + p[1] * x * (1 - y) * (1 - z) +
           p[2] * (1 - x) * y * (1 - z) + p[3] * (1 - x) * (1 - y) * z +
           p[4] * x * (1 - y) * z + p[5] * (1 - x) * y * z +
           p[6] * x * y * (1 - z) + p[7] * x * y * z;
}

inline bool in_grid(const Mac &m, double x, double y, double z) {   // grid3d.h:134-136
    return x >= 0 && y >= 0 && z >= 0 && x < m.dx * m.ni && y < m.dx * m.nj && z < m.dx * m.nk;
}

// comp 0/1/2 -> face grid dims and offsets
double interp(const Mac &m, int comp, double x, double y, double z) {
    if (!in_grid(m, x, y, z)) return 0.0;
    const float *g = comp == 0 ? m.u : (comp == 1 ? m.v : m.w);
    int gw = m.ni + (comp == 0), gh = m.nj + (comp == 1), gd = m.nk + (comp == 2);
    if (comp != 0) x -= 0.5 * m.dx;
    if (comp != 1) y -= 0.5 * m.dx;
    if (comp != 2) z -= 0.5 * m.dx;
    double inv = 1.0 / m.dx;
    int i = (int)std::floor(x * inv), j = (int)std::floor(y * inv), k = (int)std::floor(z * inv);
    double gx = (double)i * m.dx, gy = (double)j * m.dx, gz = (double)k * m.dx;
    double inv_dx = 1 / m.dx;
    double ix = (x - gx) * inv_dx, iy = (y - gy) * inv_dx, iz = (z - gz) * inv_dx;
    double p[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const int off[8][3] = {{0,0,0},{1,0,0},{0,1,0},{0,0,1},{1,0,1},{0,1,1},{1,1,0},{1,1,1}};
    for (int c = 0; c < 8; c++) {
        int a = i + off[c][0], b = j + off[c][1], e = k + off[c][2];
        if (a >= 0 && b >= 0 && e >= 0 && a < gw && b < gh && e < gd) p[c] = g[flat(a, b, e, gw, gh)];
    }
    return tri(p, ix, iy, iz);
}

V3 eval(const Mac &m, V3 p) {   // macvelocityfield.cpp:635-645
    double x = p.x, y = p.y, z = p.z;
    if (!in_grid(m, x, y, z)) return v3(0, 0, 0);
    return v3((float)interp(m, 0, x, y, z), (float)interp(m, 1, x, y, z), (float)interp(m, 2, x, y, z));
}

struct Near {
    int w, h, d;
    double cell;
    std::vector<char> g;
    bool at(int i, int j, int k) const {
        if (i < 0 || j < 0 || k < 0 || i >= w || j >= h || k >= d) return false;
        return g[flat(i, j, k, w, h)] != 0;
    }
};

Near near_solid(int ni, int nj, int nk, double dx, int cfl, const float *solid) {   // :5448-5480
    Near N;
    const int factor = 3;
    N.cell = factor * dx;
    N.w = (int)std::ceil(ni * dx / N.cell);
    N.h = (int)std::ceil(nj * dx / N.cell);
    N.d = (int)std::ceil(nk * dx / N.cell);
    N.g.assign((size_t)N.w * N.h * N.d, 0);
    float maxd = (float)(3 * dx);
    for (int k = 0; k < nk; k++)
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++)
                if (std::fabs(solid[flat(i, j, k, ni + 1, nj + 1)]) < maxd)
                    N.g[flat(i / factor, j / factor, k / factor, N.w, N.h)] = 1;
    int layers = (int)std::ceil((float)cfl / (float)factor);
    for (int l = 0; l < layers; l++) {   // featherGrid6 (gridutils.cpp:229-262)
        std::vector<char> src = N.g;
        for (int k = 0; k < N.d; k++)
            for (int j = 0; j < N.h; j++)
                for (int i = 0; i < N.w; i++) {
                    if (!src[flat(i, j, k, N.w, N.h)]) continue;
                    const int nb[6][3] = {{-1,0,0},{1,0,0},{0,-1,0},{0,1,0},{0,0,-1},{0,0,1}};
                    for (auto &o : nb) {
                        int a = i + o[0], b = j + o[1], c = k + o[2];
                        if (a >= 0 && b >= 0 && c >= 0 && a < N.w && b < N.h && c < N.d) N.g[flat(a, b, c, N.w, N.h)] = 1;
                    }
                }
    }
    return N;
}

inline void pidx(V3 p, double dx, int &i, int &j, int &k) {
    double inv = 1.0 / dx;
    i = (int)std::floor(p.x * inv); j = (int)std::floor(p.y * inv); k = (int)std::floor(p.z * inv);
}

V3 resolve(V3 oldp, V3 newp, const Box &boundary, const Near &N, const Grid &solid, int ni, int nj, int nk,
           double dx, int cfl) {   // fluidsimulation.cpp:7646-7721
    int gi, gj, gk;
    pidx(newp, dx, gi, gj, gk);
    if (!(gi >= 0 && gj >= 0 && gk >= 0 && gi < ni && gj < nj && gk < nk)) newp = boundary.nearest_inside(newp);
    int oi, oj, ok, ni2, nj2, nk2;
    pidx(oldp, N.cell, oi, oj, ok);
    pidx(newp, N.cell, ni2, nj2, nk2);
    if (!N.at(oi, oj, ok) && !N.at(ni2, nj2, nk2)) return newp;
    const float eps = 1e-6f;
    float step = 0.1f * (float)dx;
    float travel = vlength(newp - oldp);
    if (travel < eps) return newp;
    int nsteps = (int)std::ceil(travel / step);
    V3 dir = (newp - oldp) / vlength(newp - oldp);
    V3 last = oldp, cur = oldp;
    bool hit = false;
    float hitphi = 0.0f;
    for (int s = 0; s < nsteps; s++) {
        if (s == nsteps - 1) cur = newp;
        else cur = oldp + ((float)(s + 1) * step) * dir;
        float phi = solid_trilinear(solid, dx, cur);
        if (phi < 0.0f || !boundary.inside(cur)) { hitphi = phi; hit = true; break; }
        last = cur;
    }
    if (!hit) return newp;
    V3 res;
    float maxdist = (float)(cfl * dx);
    V3 grad = solid_gradient(solid, dx, cur);
    if (vlength(grad) > eps) {
        grad = grad / vlength(grad);
        float s = (float)((double)hitphi - (double)0.2f * dx);
        res = cur - s * grad;
        float rphi = solid_trilinear(solid, dx, res);
        float rdist = vlength(res - cur);
        if (rphi < 0 || rdist > maxdist) res = last;
    } else {
        res = last;
    }
    if (!boundary.inside(res)) {
        V3 orig = res;
        res = boundary.nearest_inside(res);
        float rphi = solid_trilinear(solid, dx, res);
        float rdist = vlength(res - orig);
        if (rphi < 0.0f || rdist > maxdist) res = last;
    }
    return res;
}

}  // namespace

extern "C" {

// vel <- pic*PIC + (1-pic)*(vel + PIC - saved) with PIC, saved sampled at pos.
void oracle_g2p(int ni, int nj, int nk, double dx, double pic, int np, const float *pos, float *vel,
                const float *u, const float *v, const float *w,
                const float *su, const float *sv, const float *sw) {
    Mac m{ni, nj, nk, dx, u, v, w}, s{ni, nj, nk, dx, su, sv, sw};
    float a = (float)pic, b = (float)(1 - pic);
#pragma omp parallel for
    for (int p = 0; p < np; p++) {
        V3 x = v3(pos[3 * p], pos[3 * p + 1], pos[3 * p + 2]);
        V3 ve = v3(vel[3 * p], vel[3 * p + 1], vel[3 * p + 2]);
        V3 vpic = eval(m, x);
        V3 vflip = ve + vpic - eval(s, x);
        V3 r = a * vpic + b * vflip;
        vel[3 * p] = r.x; vel[3 * p + 1] = r.y; vel[3 * p + 2] = r.z;
    }
}

// APIC particle update (_updatePICAPICMarkerParticleVelocitiesThread,
// fluidsimulation.cpp:6791-6843, gradient weights _getIndicesAndGradientWeights :6709-6769):
// the velocity is the PIC sample; each component's affine vector sums the trilinear weight
// gradients (float) times the face values of the 8 stencil nodes in range.
// aff: 9 floats per particle (x, y, z component vectors).
void oracle_g2p_apic(int ni, int nj, int nk, double dx, int np, const float *pos, float *vel, float *aff,
                     const float *u, const float *v, const float *w) {
    Mac m{ni, nj, nk, dx, u, v, w};
    const float h = (float)(0.5 * dx);
    const float invf = (float)(1.0 / (double)(float)dx);   // vec3 / float
    const float invdx = (float)(1.0 / dx);                  // 1.0f / _dx
    const double inv = 1.0 / dx;
#pragma omp parallel for
    for (int p = 0; p < np; p++) {
        const V3 x = v3(pos[3 * p], pos[3 * p + 1], pos[3 * p + 2]);
        for (int c = 0; c < 3; c++) {
            const float *g = c == 0 ? u : (c == 1 ? v : w);
            const int gw = ni + (c == 0), gh = nj + (c == 1), gd = nk + (c == 2);
            const float qx = x.x - (c == 0 ? 0.0f : h), qy = x.y - (c == 1 ? 0.0f : h), qz = x.z - (c == 2 ? 0.0f : h);
            const int gi = (int)std::floor((double)qx * inv), gj = (int)std::floor((double)qy * inv),
                      gk = (int)std::floor((double)qz * inv);
            const float gx = (float)((double)(float)gi * dx), gy = (float)((double)(float)gj * dx),
                        gz = (float)((double)(float)gk * dx);
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
            float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f;
            for (int q = 0; q < 8; q++) {
                const int i = gi + (q & 1), j = gj + ((q >> 1) & 1), k = gk + (q >> 2);
                if (i < 0 || j < 0 || k < 0 || i >= gw || j >= gh || k >= gd) continue;
                const float val = g[flat(i, j, k, gw, gh)];
                a0 += wts[q][0] * val; a1 += wts[q][1] * val; a2 += wts[q][2] * val;
            }
            aff[9 * p + 3 * c] = a0; aff[9 * p + 3 * c + 1] = a1; aff[9 * p + 3 * c + 2] = a2;
        }
        const V3 r = eval(m, x);
        vel[3 * p] = r.x; vel[3 * p + 1] = r.y; vel[3 * p + 2] = r.z;
    }
}

// MAC sample of one field at np points (float result per component).
void oracle_sample_mac(int ni, int nj, int nk, double dx, int np, const float *pos,
                       const float *u, const float *v, const float *w, float *out) {
    Mac m{ni, nj, nk, dx, u, v, w};
    for (int p = 0; p < np; p++) {
        V3 r = eval(m, v3(pos[3 * p], pos[3 * p + 1], pos[3 * p + 2]));
        out[3 * p] = r.x; out[3 * p + 1] = r.y; out[3 * p + 2] = r.z;
    }
}

// RK3 advection + collision resolution; writes new positions into out.
void oracle_advect(int ni, int nj, int nk, double dx, double dt, int cfl, int np, const float *pos,
                   const float *u, const float *v, const float *w, const float *solid_phi, float *out) {
    Mac m{ni, nj, nk, dx, u, v, w};
    Domain dm{ni, nj, nk, dx};
    Box boundary = expand(boundary_box(dm), -(double)0.2f * dx);
    Near N = near_solid(ni, nj, nk, dx, cfl, solid_phi);
    Grid solid{ni + 1, nj + 1, nk + 1, const_cast<float *>(solid_phi)};
    float h1 = (float)(0.5 * dt), h2 = (float)(0.75 * dt), h3 = (float)(dt / 9.0f);
#pragma omp parallel for
    for (int p = 0; p < np; p++) {
        V3 p0 = v3(pos[3 * p], pos[3 * p + 1], pos[3 * p + 2]);
        V3 k1 = eval(m, p0);
        V3 k2 = eval(m, p0 + h1 * k1);
        V3 k3 = eval(m, p0 + h2 * k2);
        V3 p1 = p0 + h3 * (2.0f * k1 + 3.0f * k2 + 4.0f * k3);
        V3 r = resolve(p0, p1, boundary, N, solid, ni, nj, nk, dx, cfl);
        out[3 * p] = r.x; out[3 * p + 1] = r.y; out[3 * p + 2] = r.z;
    }
}

// Marker removal: inside solid, more than max_per_cell per cell (in particle order).
// Compacts pos/vel in place, keeping order; returns the new count.
// oracle_remove that also compacts a per-particle attribute of `na` floats (may be null).
int oracle_remove_attr(int ni, int nj, int nk, double dx, int np, float *pos, float *vel, float *attr, int na,
                       const float *solid_phi, int max_per_cell) {
    Grid solid{ni + 1, nj + 1, nk + 1, const_cast<float *>(solid_phi)};
    std::vector<int> count((size_t)ni * nj * nk, 0);
    int out = 0;
    for (int p = 0; p < np; p++) {
        V3 x = v3(pos[3 * p], pos[3 * p + 1], pos[3 * p + 2]);
        if (solid_trilinear(solid, dx, x) < 0.0f) continue;
        int i, j, k;
        pidx(x, dx, i, j, k);
        size_t c = flat(i, j, k, ni, nj);
        if (count[c] >= max_per_cell) continue;
        count[c]++;
        for (int q = 0; q < 3; q++) { pos[3 * out + q] = pos[3 * p + q]; vel[3 * out + q] = vel[3 * p + q]; }
        if (attr)
            for (int q = 0; q < na; q++) attr[(size_t)na * out + q] = attr[(size_t)na * p + q];
        out++;
    }
    return out;
}

int oracle_remove(int ni, int nj, int nk, double dx, int np, float *pos, float *vel,
                  const float *solid_phi, int max_per_cell) {
    Grid solid{ni + 1, nj + 1, nk + 1, const_cast<float *>(solid_phi)};
    std::vector<int> count((size_t)ni * nj * nk, 0);
    int out = 0;
    for (int p = 0; p < np; p++) {
        V3 x = v3(pos[3 * p], pos[3 * p + 1], pos[3 * p + 2]);
        if (solid_trilinear(solid, dx, x) < 0.0f) continue;
        int i, j, k;
        pidx(x, dx, i, j, k);
        size_t c = flat(i, j, k, ni, nj);
        if (count[c] >= max_per_cell) continue;
        count[c]++;
        for (int q = 0; q < 3; q++) { pos[3 * out + q] = pos[3 * p + q]; vel[3 * out + q] = vel[3 * p + q]; }
        out++;
    }
    return out;
}

// FluidSimulation::_getMarkerParticleSpeedLimit (fluidsimulation.cpp:7723-7771): a histogram of
// particle speeds in steps of CFL*dx/frame_dt, one bin per allowed substep; the limit rises past
// the top bins while they hold at most min(0.05 % of the particles, 35) particles, and drops to
// 0.99999 of the fastest speed when at most 6 particles lie in each outlier band.  Constants
// are the reference's defaults (fluidsimulation.h:2452-2457).
float oracle_speed_limit(int np, const float *vel, double cfl, double dx, double frame_dt, int max_steps) {
    double maxps = 0.0;
    const double step = cfl * dx / frame_dt;
    std::vector<int> bins(max_steps, 0);
    auto speed_of = [&](int p) {
        const float x = vel[3 * p], y = vel[3 * p + 1], z = vel[3 * p + 2];
        return (double)std::sqrt(x * x + y * y + z * z);   // vec3::length, float
    };
    for (int p = 0; p < np; p++) {
        const double sp = speed_of(p);
        bins[(int)std::fmin(std::floor(sp / step), max_steps - 1)]++;
        maxps = std::max(sp, maxps);
    }
    const int maxrem = (int)std::fmin((int)((double)np * 0.0005), 35);
    double maxspeed = max_steps * step;
    int cur = 0;
    for (int i = max_steps - 1; i > 0; i--) {
        if (cur + bins[i] > maxrem) break;
        cur += bins[i];
        maxspeed = std::max(i + 4, max_steps) * step;
    }
    const double lower = 0.90 * maxps, upper = 0.99999 * maxps;
    int nlow = 0, nup = 0;
    for (int p = 0; p < np; p++) {
        const double sp = speed_of(p);
        if (sp >= lower && sp < upper) nlow++;
        if (sp >= upper) nup++;
    }
    if (nup <= 6 && nlow <= 6) maxspeed = std::min(upper, maxspeed);
    return (float)maxspeed;
}

// _removeMarkerParticles (:7773-7851) with extreme-velocity removal on: a particle inside a
// solid is dropped; otherwise it takes its cell's count (and is dropped beyond max_per_cell),
// then is dropped when |v|^2 (float) exceeds limit^2 (float product, compared in double).
int oracle_remove_extreme(int ni, int nj, int nk, double dx, int np, float *pos, float *vel,
                          const float *solid_phi, int max_per_cell, float limit) {
    Grid solid{ni + 1, nj + 1, nk + 1, const_cast<float *>(solid_phi)};
    std::vector<int> count((size_t)ni * nj * nk, 0);
    const double maxspeedsq = limit * limit;
    int out = 0;
    for (int p = 0; p < np; p++) {
        V3 x = v3(pos[3 * p], pos[3 * p + 1], pos[3 * p + 2]);
        if (solid_trilinear(solid, dx, x) < 0.0f) continue;
        int i, j, k;
        pidx(x, dx, i, j, k);
        size_t c = flat(i, j, k, ni, nj);
        if (count[c] >= max_per_cell) continue;
        count[c]++;
        const float vx = vel[3 * p], vy = vel[3 * p + 1], vz = vel[3 * p + 2];
        if ((double)(vx * vx + vy * vy + vz * vz) > maxspeedsq) continue;
        for (int q = 0; q < 3; q++) { pos[3 * out + q] = pos[3 * p + q]; vel[3 * out + q] = vel[3 * p + q]; }
        out++;
    }
    return out;
}

// Solid-face constraint with zero solid velocity and zero friction: faces with weight 0
// take the solid velocity (0); partially open faces keep f*0 + (1-f)*u = u.
void oracle_constrain(int ni, int nj, int nk, const float *wu, const float *wv, const float *ww,
                      float *u, float *v, float *w) {
    size_t nu = (size_t)(ni + 1) * nj * nk, nv = (size_t)ni * (nj + 1) * nk, nw = (size_t)ni * nj * (nk + 1);
    for (size_t t = 0; t < nu; t++) if (wu[t] == 0) u[t] = 0.0f;
    for (size_t t = 0; t < nv; t++) if (wv[t] == 0) v[t] = 0.0f;
    for (size_t t = 0; t < nw; t++) if (ww[t] == 0) w[t] = 0.0f;
}

}  // extern "C"
