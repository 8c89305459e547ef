// Oracle (test infrastructure only): the variational viscosity solve applied before the
// pressure projection (FluidSimulation::_applyViscosityToVelocityField,
// fluidsimulation.cpp:5983-6064; ViscositySolver, viscositysolver.cpp:53-901).
//   Face states: _computeFaceStateGridThread (:144-188) from the solid distance at cell
//                centres (MeshLevelSet::getDistanceAtCellCenter, meshlevelset.cpp:152-162).
//   Volumes:     _computeVolumeGrid (:209-285) - liquid cells dilated twice, subcell volume
//                fractions from the liquid level set (LevelsetUtils::volumeFraction,
//                levelsetutils.cpp:213-258, levelsetutils.h:63-100; trilinear sampling,
//                interpolation.cpp:61-112) averaged onto centre/face/edge grids.
//   System:      _computeMatrixIndexTable (:363-471) and _initializeLinearSystemThread{U,V,W}
//                (:556-829), rows sorted by column (SparseMatrix::set/add, sparsematrix.h:72-111).
//   Solve:       PCGSolver<float> with the MIC(0) factor (pcgsolver.h:68-322) and single-thread
//                BLAS (blaswrapper.h), then _applySolutionToVelocityField (:869-901).
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <utility>
#include <vector>

using namespace oracle;

namespace {

enum : char { FS_AIR = 0, FS_FLUID = 1, FS_SOLID = 2 };

struct F3 {   // float Array3d with out-of-range reads returning 0
    int w = 0, h = 0, d = 0;
    std::vector<float> a;
    F3() = default;
    F3(int w_, int h_, int d_) : w(w_), h(h_), d(d_), a((size_t)w_ * h_ * d_, 0.0f) {}
    bool in(int i, int j, int k) const { return i >= 0 && j >= 0 && k >= 0 && i < w && j < h && k < d; }
    float get(int i, int j, int k) const { return in(i, j, k) ? a[flat(i, j, k, w, h)] : 0.0f; }
    float &at(int i, int j, int k) { return a[flat(i, j, k, w, h)]; }
};

struct S3 {   // face states; out-of-range reads as air (neither fluid nor solid)
    int w = 0, h = 0, d = 0;
    std::vector<char> a;
    S3() = default;
    S3(int w_, int h_, int d_) : w(w_), h(h_), d(d_), a((size_t)w_ * h_ * d_, FS_AIR) {}
    char get(int i, int j, int k) const {
        return (i >= 0 && j >= 0 && k >= 0 && i < w && j < h && k < d) ? a[flat(i, j, k, w, h)] : FS_AIR;
    }
};

// trilinear sample of a cell-centred float grid (Interpolation::trilinearInterpolate with the
// ParticleLevelSet half-cell shift, particlelevelset.cpp:136-138)
float sample_phi(const F3 &phi, double dx, float px, float py, float pz) {
    const float sh = (float)(0.5 * dx);
    const float x = px - sh, y = py - sh, z = pz - sh;
    const double inv = 1.0 / dx;
    const int i = (int)std::floor(x * inv), j = (int)std::floor(y * inv), k = (int)std::floor(z * inv);
    const float gx = (float)((double)(float)i * dx), gy = (float)((double)(float)j * dx), gz = (float)((double)(float)k * dx);
    const double ix = (double)(x - gx) * inv, iy = (double)(y - gy) * inv, iz = (double)(z - gz) * inv;
    const double p0 = phi.get(i, j, k), p1 = phi.get(i + 1, j, k), p2 = phi.get(i, j + 1, k), p3 = phi.get(i, j, k + 1),
                 p4 = phi.get(i + 1, j, k + 1), p5 = phi.get(i, j + 1, k + 1), p6 = phi.get(i + 1, j + 1, k),
                 p7 = phi.get(i + 1, j + 1, k + 1);
    const double r = p0 * (1 - ix) * (1 - iy) * (1 - iz) + p1 * ix * (1 - iy) * (1 - iz) + p2 * (1 - ix) * iy * (1 - iz) +
                     p3 * (1 - ix) * (1 - iy) * iz + p4 * ix * (1 - iy) * iz + p5 * (1 - ix) * iy * iz +
                     p6 * ix * iy * (1 - iz) + p7 * ix * iy * iz;
    return (float)r;
}

inline void sort4(float &a, float &b, float &c, float &d) {
    if (a > b) std::swap(a, b);
    if (c > d) std::swap(c, d);
    if (a > c) std::swap(a, c);
    if (b > d) std::swap(b, d);
    if (b > c) std::swap(b, c);
}

inline float tet_fraction(float p0, float p1, float p2, float p3) {
    return p0 * p0 * p0 / ((p0 - p1) * (p0 - p2) * (p0 - p3));
}

inline float prism_fraction(float p0, float p1, float p2, float p3) {
    const float a = p0 / (p0 - p2), b = p0 / (p0 - p3), c = p1 / (p1 - p3), d = p1 / (p1 - p2);
    return a * b * (1 - d) + b * (1 - c) * d + c * d;
}

float vf4(float p0, float p1, float p2, float p3) {
    sort4(p0, p1, p2, p3);
    if (p3 <= 0) return 1;
    if (p2 <= 0) return 1 - tet_fraction(p3, p2, p1, p0);
    if (p1 <= 0) return prism_fraction(p0, p1, p2, p3);
    if (p0 <= 0) return tet_fraction(p0, p1, p2, p3);
    return 0;
}

float vf8(float p000, float p100, float p010, float p110, float p001, float p101, float p011, float p111) {
    return (vf4(p000, p001, p101, p011) + vf4(p000, p101, p100, p110) + vf4(p000, p010, p011, p110) +
            vf4(p101, p011, p111, p110) + 2 * vf4(p000, p011, p101, p110) + vf4(p100, p101, p001, p111) +
            vf4(p100, p001, p000, p010) + vf4(p100, p110, p111, p010) + vf4(p001, p111, p011, p010) +
            2 * vf4(p100, p111, p001, p010)) / 12.0f;
}

struct Visc {
    int ni, nj, nk;
    float dx, dt;   // ViscositySolverParameters holds float cell width and time step
    double ddx;     // the liquid level set's own (double) cell width
    S3 su, sv, sw;
    F3 center, vu, vv, vw, eu, ev, ew;
    std::vector<int> index;   // face (U, V, W blocks, x fastest) -> matrix row, -1 if none
    int n = 0;
    int U(int i, int j, int k) const { return (i < 0 || j < 0 || k < 0 || i > ni || j >= nj || k >= nk) ? -1 : index[flat(i, j, k, ni + 1, nj)]; }
    int V(int i, int j, int k) const {
        return (i < 0 || j < 0 || k < 0 || i >= ni || j > nj || k >= nk) ? -1
                                                                          : index[(size_t)(ni + 1) * nj * nk + flat(i, j, k, ni, nj + 1)];
    }
    int W(int i, int j, int k) const {
        return (i < 0 || j < 0 || k < 0 || i >= ni || j >= nj || k > nk)
                   ? -1
                   : index[(size_t)(ni + 1) * nj * nk + (size_t)ni * (nj + 1) * nk + flat(i, j, k, ni, nj)];
    }
};

void face_states(Visc &S, const float *solid) {
    const int ni = S.ni, nj = S.nj, nk = S.nk;
    F3 scp(ni, nj, nk);
    auto sp = [&](int i, int j, int k) { return solid[flat(i, j, k, ni + 1, nj + 1)]; };
    for (int k = 0; k < nk; k++)
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++)
                scp.at(i, j, k) = 0.125f * (sp(i, j, k) + sp(i + 1, j, k) + sp(i, j + 1, k) + sp(i + 1, j + 1, k) +
                                            sp(i, j, k + 1) + sp(i + 1, j, k + 1) + sp(i, j + 1, k + 1) +
                                            sp(i + 1, j + 1, k + 1));
    S.su = S3(ni + 1, nj, nk); S.sv = S3(ni, nj + 1, nk); S.sw = S3(ni, nj, nk + 1);
    for (int k = 0; k < nk; k++)
        for (int j = 0; j < nj; j++)
            for (int i = 0; i <= ni; i++)
                S.su.a[flat(i, j, k, ni + 1, nj)] =
                    (i == 0 || i == ni || scp.get(i - 1, j, k) + scp.get(i, j, k) <= 0) ? FS_SOLID : FS_FLUID;
    for (int k = 0; k < nk; k++)
        for (int j = 0; j <= nj; j++)
            for (int i = 0; i < ni; i++)
                S.sv.a[flat(i, j, k, ni, nj + 1)] =
                    (j == 0 || j == nj || scp.get(i, j - 1, k) + scp.get(i, j, k) <= 0) ? FS_SOLID : FS_FLUID;
    for (int k = 0; k <= nk; k++)
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++)
                S.sw.a[flat(i, j, k, ni, nj)] =
                    (k == 0 || k == nk || scp.get(i, j, k - 1) + scp.get(i, j, k) <= 0) ? FS_SOLID : FS_FLUID;
}

void volumes(Visc &S, const float *liquid) {
    const int ni = S.ni, nj = S.nj, nk = S.nk;
    const int vw = ni + 1, vh = nj + 1, vd = nk + 1;
    std::vector<char> valid((size_t)vw * vh * vd, 0);
    for (int k = 0; k < nk; k++)
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++)
                if (liquid[flat(i, j, k, ni, nj)] < 0) valid[flat(i, j, k, vw, vh)] = 1;
    for (int layer = 0; layer < 2; layer++) {
        std::vector<char> t = valid;
        for (int k = 0; k < vd; k++)
            for (int j = 0; j < vh; j++)
                for (int i = 0; i < vw; i++) {
                    if (!valid[flat(i, j, k, vw, vh)]) continue;
                    const int nb[6][3] = {{i - 1, j, k}, {i + 1, j, k}, {i, j - 1, k}, {i, j + 1, k}, {i, j, k - 1}, {i, j, k + 1}};
                    for (auto &q : nb)
                        if (q[0] >= 0 && q[1] >= 0 && q[2] >= 0 && q[0] < vw && q[1] < vh && q[2] < vd)
                            t[flat(q[0], q[1], q[2], vw, vh)] = 1;
                }
        valid = t;
    }
    F3 phi(ni, nj, nk);
    phi.a.assign(liquid, liquid + (size_t)ni * nj * nk);
    const double ddx = S.ddx;
    F3 sub(2 * ni, 2 * nj, 2 * nk);
    const float cs = 0.25f * S.dx, sdx = 0.5f * S.dx, h = 0.5f * sdx;
    for (int k = 0; k < 2 * nk; k++)
        for (int j = 0; j < 2 * nj; j++)
            for (int i = 0; i < 2 * ni; i++) {
                if (!valid[flat(i / 2, j / 2, k / 2, vw, vh)]) continue;
                const float cx = cs + i * sdx, cy = cs + j * sdx, cz = cs + k * sdx;
                auto s = [&](float ox, float oy, float oz) { return sample_phi(phi, ddx, cx + ox, cy + oy, cz + oz); };
                const float p000 = s(-h, -h, -h), p001 = s(-h, -h, +h), p010 = s(-h, +h, -h), p011 = s(-h, +h, +h),
                            p100 = s(+h, -h, -h), p101 = s(+h, -h, +h), p110 = s(+h, +h, -h), p111 = s(+h, +h, +h);
                sub.at(i, j, k) = vf8(p000, p100, p010, p110, p001, p101, p011, p111);
            }
    S.center = F3(ni, nj, nk); S.vu = F3(ni + 1, nj, nk); S.vv = F3(ni, nj + 1, nk); S.vw = F3(ni, nj, nk + 1);
    S.eu = F3(ni, nj + 1, nk + 1); S.ev = F3(ni + 1, nj, nk + 1); S.ew = F3(ni + 1, nj + 1, nk);
    struct G { F3 *g; int oi, oj, ok; };
    const G groups[7] = {{&S.center, 0, 0, 0}, {&S.vu, -1, 0, 0}, {&S.vv, 0, -1, 0}, {&S.vw, 0, 0, -1},
                         {&S.eu, 0, -1, -1},   {&S.ev, -1, 0, -1}, {&S.ew, -1, -1, 0}};
    for (const G &g : groups)
        for (int k = 1; k < nk; k++)
            for (int j = 1; j < nj; j++)
                for (int i = 1; i < ni; i++) {
                    if (!valid[flat(i, j, k, vw, vh)]) continue;
                    float acc = 0.0f;
                    for (int ko = 0; ko < 2; ko++)
                        for (int jo = 0; jo < 2; jo++)
                            for (int io = 0; io < 2; io++)
                                acc += sub.get(2 * i + g.oi + io, 2 * j + g.oj + jo, 2 * k + g.ok + ko);
                    g.g->at(i, j, k) = 0.125f * acc;
                }
}

void matrix_index(Visc &S) {
    const int ni = S.ni, nj = S.nj, nk = S.nk;
    const size_t nu = (size_t)(ni + 1) * nj * nk, nv = (size_t)ni * (nj + 1) * nk, nw = (size_t)ni * nj * (nk + 1);
    std::vector<char> in(nu + nv + nw, 0);
    for (int k = 1; k < nk; k++)
        for (int j = 1; j < nj; j++)
            for (int i = 1; i < ni; i++) {
                if (S.su.get(i, j, k) == FS_FLUID &&
                    (S.vu.get(i, j, k) > 0 || S.center.get(i, j, k) > 0 || S.center.get(i - 1, j, k) > 0 ||
                     S.ew.get(i, j + 1, k) > 0 || S.ew.get(i, j, k) > 0 || S.ev.get(i, j, k + 1) > 0 || S.ev.get(i, j, k) > 0))
                    in[flat(i, j, k, ni + 1, nj)] = 1;
                if (S.sv.get(i, j, k) == FS_FLUID &&
                    (S.vv.get(i, j, k) > 0 || S.ew.get(i + 1, j, k) > 0 || S.ew.get(i, j, k) > 0 || S.center.get(i, j, k) > 0 ||
                     S.center.get(i, j - 1, k) > 0 || S.eu.get(i, j, k + 1) > 0 || S.eu.get(i, j, k) > 0))
                    in[nu + flat(i, j, k, ni, nj + 1)] = 1;
                if (S.sw.get(i, j, k) == FS_FLUID &&
                    (S.vw.get(i, j, k) > 0 || S.ev.get(i + 1, j, k) > 0 || S.ev.get(i, j, k) > 0 || S.eu.get(i, j + 1, k) > 0 ||
                     S.eu.get(i, j, k) > 0 || S.center.get(i, j, k) > 0 || S.center.get(i, j, k - 1) > 0))
                    in[nu + nv + flat(i, j, k, ni, nj)] = 1;
            }
    S.index.assign(in.size(), -1);
    int m = 0;
    for (size_t t = 0; t < in.size(); t++)
        if (in[t]) S.index[t] = m++;
    S.n = m;
}

struct Row { std::vector<std::pair<int, float>> e; };

// One row of the system; comp 0/1/2 = U/V/W (viscositysolver.cpp:556-829).
void build_row(const Visc &S, const F3 &visc, const float *u, const float *v, const float *w, int comp, int i, int j,
               int k, Row &row, float &rhs) {
    const int ni = S.ni, nj = S.nj;
    const float invdx = 1.0f / S.dx;
    const float factor = S.dt * invdx * invdx;
    auto vi = [&](int a, int b, int c) { return visc.get(a, b, c); };
    auto U = [&](int a, int b, int c) { return u[flat(a, b, c, ni + 1, nj)]; };
    auto V = [&](int a, int b, int c) { return v[flat(a, b, c, ni, nj + 1)]; };
    auto Wf = [&](int a, int b, int c) { return w[flat(a, b, c, ni, nj)]; };
    float fR, fL, fT, fB, fF, fK, vol, vel;
    int r;
    if (comp == 0) {
        const float vR = vi(i, j, k), vL = vi(i - 1, j, k);
        const float vT = 0.25f * (vi(i - 1, j + 1, k) + vi(i - 1, j, k) + vi(i, j + 1, k) + vi(i, j, k));
        const float vB = 0.25f * (vi(i - 1, j, k) + vi(i - 1, j - 1, k) + vi(i, j, k) + vi(i, j - 1, k));
        const float vF = 0.25f * (vi(i - 1, j, k + 1) + vi(i - 1, j, k) + vi(i, j, k + 1) + vi(i, j, k));
        const float vK = 0.25f * (vi(i - 1, j, k) + vi(i - 1, j, k - 1) + vi(i, j, k) + vi(i, j, k - 1));
        fR = 2 * factor * vR * S.center.get(i, j, k);
        fL = 2 * factor * vL * S.center.get(i - 1, j, k);
        fT = factor * vT * S.ew.get(i, j + 1, k);
        fB = factor * vB * S.ew.get(i, j, k);
        fF = factor * vF * S.ev.get(i, j, k + 1);
        fK = factor * vK * S.ev.get(i, j, k);
        vol = S.vu.get(i, j, k); vel = U(i, j, k); r = S.U(i, j, k);
    } else if (comp == 1) {
        const float vR = 0.25f * (vi(i, j - 1, k) + vi(i + 1, j - 1, k) + vi(i, j, k) + vi(i + 1, j, k));
        const float vL = 0.25f * (vi(i, j - 1, k) + vi(i - 1, j - 1, k) + vi(i, j, k) + vi(i - 1, j, k));
        const float vT = vi(i, j, k), vB = vi(i, j - 1, k);
        const float vF = 0.25f * (vi(i, j - 1, k) + vi(i, j - 1, k + 1) + vi(i, j, k) + vi(i, j, k + 1));
        const float vK = 0.25f * (vi(i, j - 1, k) + vi(i, j - 1, k - 1) + vi(i, j, k) + vi(i, j, k - 1));
        fR = factor * vR * S.ew.get(i + 1, j, k);
        fL = factor * vL * S.ew.get(i, j, k);
        fT = 2 * factor * vT * S.center.get(i, j, k);
        fB = 2 * factor * vB * S.center.get(i, j - 1, k);
        fF = factor * vF * S.eu.get(i, j, k + 1);
        fK = factor * vK * S.eu.get(i, j, k);
        vol = S.vv.get(i, j, k); vel = V(i, j, k); r = S.V(i, j, k);
    } else {
        const float vR = 0.25f * (vi(i, j, k) + vi(i, j, k - 1) + vi(i + 1, j, k) + vi(i + 1, j, k - 1));
        const float vL = 0.25f * (vi(i, j, k) + vi(i, j, k - 1) + vi(i - 1, j, k) + vi(i - 1, j, k - 1));
        const float vT = 0.25f * (vi(i, j, k) + vi(i, j, k - 1) + vi(i, j + 1, k) + vi(i, j + 1, k - 1));
        const float vB = 0.25f * (vi(i, j, k) + vi(i, j, k - 1) + vi(i, j - 1, k) + vi(i, j - 1, k - 1));
        const float vF = vi(i, j, k), vK = vi(i, j, k - 1);
        fR = factor * vR * S.ev.get(i + 1, j, k);
        fL = factor * vL * S.ev.get(i, j, k);
        fT = factor * vT * S.eu.get(i, j + 1, k);
        fB = factor * vB * S.eu.get(i, j, k);
        fF = 2 * factor * vF * S.center.get(i, j, k);
        fK = 2 * factor * vK * S.center.get(i, j, k - 1);
        vol = S.vw.get(i, j, k); vel = Wf(i, j, k); r = S.W(i, j, k);
    }
    (void)r;
    row.e.clear();
    row.e.push_back({-2, vol + fR + fL + fT + fB + fF + fK});   // the diagonal, column filled in below
    float rv = vol * vel;
    // (state grid, face index, coefficient, velocity) per coupling, in the reference's order
    struct C { int st; int col; float coef; float vel; };
    std::vector<C> cs;
    auto cu = [&](int a, int b, int c, float f) { cs.push_back({S.su.get(a, b, c), S.U(a, b, c), f, S.su.get(a, b, c) == FS_SOLID ? U(a, b, c) : 0.0f}); };
    auto cv = [&](int a, int b, int c, float f) { cs.push_back({S.sv.get(a, b, c), S.V(a, b, c), f, S.sv.get(a, b, c) == FS_SOLID ? V(a, b, c) : 0.0f}); };
    auto cw = [&](int a, int b, int c, float f) { cs.push_back({S.sw.get(a, b, c), S.W(a, b, c), f, S.sw.get(a, b, c) == FS_SOLID ? Wf(a, b, c) : 0.0f}); };
    if (comp == 0) {
        cu(i + 1, j, k, -fR); cu(i - 1, j, k, -fL); cu(i, j + 1, k, -fT); cu(i, j - 1, k, -fB); cu(i, j, k + 1, -fF); cu(i, j, k - 1, -fK);
        cv(i, j + 1, k, -fT); cv(i - 1, j + 1, k, fT); cv(i, j, k, fB); cv(i - 1, j, k, -fB);
        cw(i, j, k + 1, -fF); cw(i - 1, j, k + 1, fF); cw(i, j, k, fK); cw(i - 1, j, k, -fK);
    } else if (comp == 1) {
        cv(i + 1, j, k, -fR); cv(i - 1, j, k, -fL); cv(i, j + 1, k, -fT); cv(i, j - 1, k, -fB); cv(i, j, k + 1, -fF); cv(i, j, k - 1, -fK);
        cu(i + 1, j, k, -fR); cu(i + 1, j - 1, k, fR); cu(i, j, k, fL); cu(i, j - 1, k, -fL);
        cw(i, j, k + 1, -fF); cw(i, j - 1, k + 1, fF); cw(i, j, k, fK); cw(i, j - 1, k, -fK);
    } else {
        cw(i + 1, j, k, -fR); cw(i - 1, j, k, -fL); cw(i, j + 1, k, -fT); cw(i, j - 1, k, -fB); cw(i, j, k + 1, -fF); cw(i, j, k - 1, -fK);
        cu(i + 1, j, k, -fR); cu(i + 1, j, k - 1, fR); cu(i, j, k, fL); cu(i, j, k - 1, -fL);
        cv(i, j + 1, k, -fT); cv(i, j + 1, k - 1, fT); cv(i, j, k, fB); cv(i, j, k - 1, -fB);
    }
    for (const C &c : cs) {
        if (c.st == FS_FLUID && c.col >= 0) row.e.push_back({c.col, c.coef});   // SparseMatrix::add skips index -1
        else if (c.st == FS_SOLID) rv -= c.coef * c.vel;
    }
    rhs = rv;
}

// Sparse symmetric matrix, rows sorted by column (SparseMatrix<float>)
struct Sparse {
    int n = 0;
    std::vector<std::vector<int>> idx;
    std::vector<std::vector<float>> val;
};

struct Lower {   // SparseColumnLowerFactor<float> (pcgsolver.h:30-58)
    std::vector<float> invdiag, adiag, value;
    std::vector<unsigned> colstart, rowindex;
};

// factorModifiedIncompleteColesky0 (pcgsolver.h:68-205), tau = 0.97, minDiagonalRatio = 0.25
void mic0(const Sparse &A, Lower &L) {
    const unsigned n = (unsigned)A.n;
    const float mod = 0.97f, mdr = 0.25f, eps = 1e-9f;
    L.invdiag.assign(n, 0.0f); L.adiag.assign(n, 0.0f); L.value.clear(); L.rowindex.clear(); L.colstart.assign(n + 1, 0);
    for (unsigned i = 0; i < n; i++) {
        L.colstart[i] = (unsigned)L.rowindex.size();
        for (size_t t = 0; t < A.idx[i].size(); t++) {
            const unsigned c = (unsigned)A.idx[i][t];
            if (c > i) { L.rowindex.push_back(c); L.value.push_back(A.val[i][t]); }
            else if (c == i) {
                float value = A.val[i][t];
                if (value < eps) value = 0;
                L.invdiag[i] = L.adiag[i] = value;
            }
        }
    }
    L.colstart[n] = (unsigned)L.rowindex.size();
    for (unsigned k = 0; k < n; k++) {
        if (L.adiag[k] == 0) continue;
        // unqualified sqrt of a float resolves to the double ::sqrt: the pivot is formed in double
        if (L.invdiag[k] < mdr * L.adiag[k]) L.invdiag[k] = (float)(1 / std::sqrt((double)L.adiag[k]));
        else L.invdiag[k] = (float)(1 / std::sqrt((double)L.invdiag[k]));
        for (unsigned p = L.colstart[k]; p < L.colstart[k + 1]; p++) L.value[p] *= L.invdiag[k];
        for (unsigned p = L.colstart[k]; p < L.colstart[k + 1]; p++) {
            const unsigned j = L.rowindex[p];
            const float mult = L.value[p];
            float missing = 0;
            unsigned a = L.colstart[k];
            size_t b = 0;
            while (a < L.colstart[k + 1] && L.rowindex[a] < j) {
                while (b < A.idx[j].size()) {
                    if ((unsigned)A.idx[j][b] < L.rowindex[a]) b++;
                    else if ((unsigned)A.idx[j][b] == L.rowindex[a]) break;
                    else { missing += L.value[a]; break; }
                }
                a++;
            }
            if (a < L.colstart[k + 1] && L.rowindex[a] == j) L.invdiag[j] -= mult * L.value[a];
            a++;
            unsigned bb = L.colstart[j];
            while (a < L.colstart[k + 1] && bb < L.colstart[j + 1]) {
                if (L.rowindex[bb] < L.rowindex[a]) bb++;
                else if (L.rowindex[bb] == L.rowindex[a]) { L.value[bb] -= mult * L.value[a]; a++; bb++; }
                else { missing += L.value[a]; a++; }
            }
            while (a < L.colstart[k + 1]) { missing += L.value[a]; a++; }
            L.invdiag[j] -= mod * mult * missing;
        }
    }
}

void apply_precond(const Lower &L, const std::vector<float> &r, std::vector<float> &z) {   // pcgsolver.h:212-241
    const unsigned n = (unsigned)r.size();
    z = r;
    for (unsigned i = 0; i < n; i++) {
        z[i] *= L.invdiag[i];
        for (unsigned j = L.colstart[i]; j < L.colstart[i + 1]; j++) z[L.rowindex[j]] -= L.value[j] * z[i];
    }
    unsigned i = n;
    do {
        i--;
        for (unsigned j = L.colstart[i]; j < L.colstart[i + 1]; j++) z[i] -= L.value[j] * z[L.rowindex[j]];
        z[i] *= L.invdiag[i];
    } while (i != 0);
}

float fdot(const std::vector<float> &x, const std::vector<float> &y) {
    float s = 0;
    for (size_t i = 0; i < x.size(); i++) s += x[i] * y[i];
    return s;
}

float fabsmax(const std::vector<float> &x) {
    int mi = 0;
    float mv = 0;
    for (size_t i = 0; i < x.size(); i++)
        if (std::fabs(x[i]) > mv) { mv = std::fabs(x[i]); mi = (int)i; }
    return std::fabs(x[mi]);
}

void axpy(float a, const std::vector<float> &x, std::vector<float> &y) {
    for (size_t i = 0; i < x.size(); i++) y[i] += a * x[i];
}

// PCGSolver<float>::solve (pcgsolver.h:268-322)
bool pcg(const Sparse &A, const std::vector<float> &rhs, std::vector<float> &x, float tolf, int maxit, const Lower &L,
         float &res, int &iters) {
    const size_t n = rhs.size();
    std::vector<float> r = rhs, z(n), s(n), q(n);
    res = fabsmax(r);
    if (res == 0) { iters = 0; return true; }
    const double tol = (double)(std::max(tolf, 1e-30f) * res);   // float product, then widened
    apply_precond(L, r, z);
    double rho = fdot(z, r);
    if (rho == 0 || rho != rho) { iters = 0; return false; }
    s = z;
    int it;
    for (it = 0; it < maxit; it++) {
        for (size_t i = 0; i < n; i++) {
            float acc = 0;
            for (size_t t = 0; t < A.idx[i].size(); t++) acc += A.val[i][t] * s[A.idx[i][t]];
            z[i] = acc;
        }
        const double alpha = rho / (double)fdot(s, z);
        axpy((float)alpha, s, x);
        axpy((float)-alpha, z, r);
        res = fabsmax(r);
        if (res <= std::min(tol, 1.0)) { iters = it + 1; return true; }
        apply_precond(L, r, z);
        const double rhoNew = fdot(z, r);
        const double beta = rhoNew / rho;
        axpy((float)beta, s, z);
        s.swap(z);
        rho = rhoNew;
    }
    iters = it;
    return false;
}

}  // namespace

extern "C" {

// Applies the viscosity solve to (u, v, w) in place.  liquid: cell-centred liquid level set
// (ni*nj*nk); solid: nodal solid level set ((ni+1)(nj+1)(nk+1)); visc: (ni+1)(nj+1)(nk+1)
// viscosity grid.  stats <- {matrix size, iterations, success}; *err <- final residual.
// Optional outputs (null to skip): vol7 = centre, U, V, W, edgeU, edgeV, edgeW volume grids
// concatenated; index = face -> row table (U, V, W faces); rowstart/col/val = the system as
// CSR (n + 1, 15 n, 15 n entries at most) and rhs; ic_invdiag/ic_colstart/ic_rowindex/ic_value
// = the MIC(0) factor; soln = the solution.
void oracle_viscosity(int ni, int nj, int nk, double dx, double dt, const float *liquid, const float *solid,
                      const float *visc, double tol, int maxit, float *u, float *v, float *w, int *stats, float *err,
                      float *vol7, int *index, unsigned *rowstart, unsigned *col, float *val, float *rhs_out,
                      float *ic_invdiag, unsigned *ic_colstart, unsigned *ic_rowindex, float *ic_value, float *soln_out) {
    Visc S;
    S.ni = ni; S.nj = nj; S.nk = nk;
    S.dx = (float)dx; S.dt = (float)dt; S.ddx = dx;
    face_states(S, solid);
    volumes(S, liquid);
    matrix_index(S);
    if (vol7) {
        float *o = vol7;
        for (const F3 *g : {&S.center, &S.vu, &S.vv, &S.vw, &S.eu, &S.ev, &S.ew}) { std::copy(g->a.begin(), g->a.end(), o); o += g->a.size(); }
    }
    if (index) std::copy(S.index.begin(), S.index.end(), index);
    stats[0] = S.n; stats[1] = 0; stats[2] = 1;
    *err = 0.0f;
    if (S.n == 0) return;
    F3 vg(ni + 1, nj + 1, nk + 1);
    vg.a.assign(visc, visc + vg.a.size());
    Sparse A;
    A.n = S.n;
    A.idx.assign(S.n, {}); A.val.assign(S.n, {});
    std::vector<float> rhs(S.n, 0.0f);
    Row row;
    for (int comp = 0; comp < 3; comp++)
        for (int k = 1; k < nk; k++)
            for (int j = 1; j < nj; j++)
                for (int i = 1; i < ni; i++) {
                    const S3 &st = comp == 0 ? S.su : (comp == 1 ? S.sv : S.sw);
                    const int r = comp == 0 ? S.U(i, j, k) : (comp == 1 ? S.V(i, j, k) : S.W(i, j, k));
                    if (st.get(i, j, k) != FS_FLUID || r < 0) continue;
                    float rv;
                    build_row(S, vg, u, v, w, comp, i, j, k, row, rv);
                    row.e[0].first = r;
                    std::sort(row.e.begin(), row.e.end(), [](const std::pair<int, float> &a, const std::pair<int, float> &b) {
                        return a.first < b.first;
                    });
                    for (auto &e : row.e) { A.idx[r].push_back(e.first); A.val[r].push_back(e.second); }
                    rhs[r] = rv;
                }
    if (rowstart) {
        unsigned t = 0;
        for (int r = 0; r < S.n; r++) {
            rowstart[r] = t;
            for (size_t q = 0; q < A.idx[r].size(); q++, t++) { col[t] = (unsigned)A.idx[r][q]; val[t] = A.val[r][q]; }
        }
        rowstart[S.n] = t;
    }
    if (rhs_out) std::copy(rhs.begin(), rhs.end(), rhs_out);
    Lower L;
    mic0(A, L);
    if (ic_invdiag) {
        std::copy(L.invdiag.begin(), L.invdiag.end(), ic_invdiag);
        std::copy(L.colstart.begin(), L.colstart.end(), ic_colstart);
        std::copy(L.rowindex.begin(), L.rowindex.end(), ic_rowindex);
        std::copy(L.value.begin(), L.value.end(), ic_value);
    }
    std::vector<float> x(S.n, 0.0f);
    float res = 0.0f;
    int it = 0;
    const bool conv = pcg(A, rhs, x, (float)tol, maxit, L, res, it);
    // ViscositySolver::_solveLinearSystem (:832-867): the iteration limit with a residual below
    // the acceptable tolerance (10) still counts as success
    const bool ok = conv || (it == maxit && res < 10.0f);
    if (soln_out) std::copy(x.begin(), x.end(), soln_out);
    stats[1] = it; stats[2] = ok ? 1 : 0;
    *err = res;
    if (!ok) return;   // applyViscosityToVelocityField leaves the field unchanged on failure
    // _applySolutionToVelocityField: every face cleared, faces in the system set
    const size_t nu = (size_t)(ni + 1) * nj * nk, nv = (size_t)ni * (nj + 1) * nk, nw = (size_t)ni * nj * (nk + 1);
    for (size_t t = 0; t < nu; t++) u[t] = S.index[t] >= 0 ? x[S.index[t]] : 0.0f;
    for (size_t t = 0; t < nv; t++) v[t] = S.index[nu + t] >= 0 ? x[S.index[nu + t]] : 0.0f;
    for (size_t t = 0; t < nw; t++) w[t] = S.index[nu + nv + t] >= 0 ? x[S.index[nu + nv + t]] : 0.0f;
}

}  // extern "C"
