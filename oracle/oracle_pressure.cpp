// Oracle (test infrastructure only): variational pressure projection.
//   System: PressureSolver::_initialize, _calculateNegativeDivergenceVectorThread,
//           _calculateMatrixCoefficientsThread (pressuresolver.cpp:118-158, 624-713, 767-867),
//           for unit density and static (zero-velocity) solids; with surface tension through
//           oracle_pressure_solve_tension (cluster status and the ghost-fluid tension term).
//   Solver: PCGSolver<double> with modified incomplete Cholesky level 0
//           (pcgsolver/pcgsolver.h:68-322, blaswrapper.h:35-157, sparsematrix.h:187-215).
//   Apply:  PressureSolver::_applyPressureToVelocityFieldThread (pressuresolver.cpp:1047-1205).
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <vector>

using namespace oracle;

namespace {

struct Sys {
    int n = 0;
    std::vector<int> ci, cj, ck;               // pressure cells in k-j-i order
    std::vector<int> key;                       // dense cell -> row, -1 if none
    std::vector<std::vector<int>> idx;          // sorted column indices per row
    std::vector<std::vector<double>> val;
    std::vector<double> rhs;
};

void rowset(Sys &s, int r, int c, double v) {   // SparseMatrix::set/add (sparsematrix.h:60-108)
    if (r < 0 || c < 0) return;
    auto &I = s.idx[r];
    auto &V = s.val[r];
    for (size_t q = 0; q < I.size(); q++) {
        if (I[q] == c) { V[q] = v; return; }
        if (I[q] > c) { I.insert(I.begin() + q, c); V.insert(V.begin() + q, v); return; }
    }
    I.push_back(c); V.push_back(v);
}

inline double clampd(double x, double lo, double hi) { return x < lo ? lo : (x > hi ? hi : x); }

void build(Sys &s, int ni, int nj, int nk, double dx, double dt, const float *phi,
           const float *wu, const float *wv, const float *ww,
           const float *u, const float *v, const float *w) {
    s.key.assign((size_t)ni * nj * nk, -1);
    for (int k = 1; k < nk - 1; k++)
        for (int j = 1; j < nj - 1; j++)
            for (int i = 1; i < ni - 1; i++)
                if (phi[flat(i, j, k, ni, nj)] < 0) {
                    s.key[flat(i, j, k, ni, nj)] = (int)s.ci.size();
                    s.ci.push_back(i); s.cj.push_back(j); s.ck.push_back(k);
                }
    s.n = (int)s.ci.size();
    s.idx.assign(s.n, {});
    s.val.assign(s.n, {});
    s.rhs.assign(s.n, 0.0);
    auto U = [&](int i, int j, int k) { return (double)u[flat(i, j, k, ni + 1, nj)]; };
    auto V = [&](int i, int j, int k) { return (double)v[flat(i, j, k, ni, nj + 1)]; };
    auto W = [&](int i, int j, int k) { return (double)w[flat(i, j, k, ni, nj)]; };
    auto WU = [&](int i, int j, int k) { return (double)wu[flat(i, j, k, ni + 1, nj)]; };
    auto WV = [&](int i, int j, int k) { return (double)wv[flat(i, j, k, ni, nj + 1)]; };
    auto WW = [&](int i, int j, int k) { return (double)ww[flat(i, j, k, ni, nj)]; };
    auto P = [&](int i, int j, int k) { return (double)phi[flat(i, j, k, ni, nj)]; };
    auto K = [&](int i, int j, int k) { return s.key[flat(i, j, k, ni, nj)]; };
    const double factor = 1.0 / dx;
    const double mfac = dt / (dx * dx);
    const double eps = 1e-9, maxtheta = 25;
    for (int r = 0; r < s.n; r++) {
        int i = s.ci[r], j = s.cj[r], k = s.ck[r];
        double vr = WU(i + 1, j, k), vl = WU(i, j, k), vt = WV(i, j + 1, k), vb = WV(i, j, k);
        double vf = WW(i, j, k + 1), vk = WW(i, j, k);
        double div = 0.0;
        div += -factor * vr * U(i + 1, j, k);
        div += factor * vl * U(i, j, k);
        div += -factor * vt * V(i, j + 1, k);
        div += factor * vb * V(i, j, k);
        div += -factor * vf * W(i, j, k + 1);
        div += factor * vk * W(i, j, k);
        s.rhs[r] = div;

        const double rho = 1.0;
        double pc = P(i, j, k);
        double diag = (vr / rho + vl / rho + vt / rho + vb / rho + vf / rho + vk / rho) * mfac;
        struct Nb { int i, j, k; double vol; };
        Nb nbs[6] = {{i + 1, j, k, vr}, {i - 1, j, k, vl}, {i, j + 1, k, vt},
                     {i, j - 1, k, vb}, {i, j, k + 1, vf}, {i, j, k - 1, vk}};
        for (auto &nb : nbs) {
            double pn = P(nb.i, nb.j, nb.k);
            if (pn < 0.0) {
                rowset(s, r, K(nb.i, nb.j, nb.k), -(nb.vol / rho) * mfac);
            } else {
                double theta = clampd(pn / (pc + eps), -maxtheta, maxtheta);
                diag -= (nb.vol / rho) * mfac * theta;
            }
        }
        diag = std::max(diag, 0.0);
        rowset(s, r, r, diag);
    }
}

// ---- surface tension (pressuresolver.cpp:314-605, 659-749) ----
enum : char { CS_UNSET = 0x00, CS_OK_IN = 0x01, CS_OK_OUT = 0x02, CS_BAD_IN = 0x04, CS_BAD_OUT = 0x08, CS_BORDER = 0x10 };

// _initializeSurfaceTensionClusterData with one thread: 4^3 block status, cell status, surface
// cells, then a breadth-first search per surface cell over its phase, marking clusters that
// reach fewer than 36 cells without touching a classified cell as bad.
std::vector<char> cluster_status(int ni, int nj, int nk, const float *phi) {
    const int bw = 4, bi = ni / bw, bj = nj / bw, bk = nk / bw;
    std::vector<char> block((size_t)bi * bj * bk, 0);
    for (int k = 0; k < nk; k++)
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++) {
                const int a = i / bw, b = j / bw, c = k / bw;
                if (a >= bi || b >= bj || c >= bk) continue;
                block[flat(a, b, c, bi, bj)] |= phi[flat(i, j, k, ni, nj)] < 0 ? 0x01 : 0x02;
            }
    std::vector<char> st((size_t)ni * nj * nk, CS_UNSET);
    auto border = [&](int i, int j, int k) { return i == 0 || j == 0 || k == 0 || i == ni - 1 || j == nj - 1 || k == nk - 1; };
    for (int k = 0; k < nk; k++)
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++) {
                const size_t t = flat(i, j, k, ni, nj);
                if (border(i, j, k)) { st[t] = CS_BORDER; continue; }
                const int a = i / bw, b = j / bw, c = k / bw;
                if (a >= bi || b >= bj || c >= bk) continue;
                const char bs = block[flat(a, b, c, bi, bj)];
                if ((bs & 0x01) && !(bs & 0x02)) st[t] = CS_OK_IN;
                else if (!(bs & 0x01) && (bs & 0x02)) st[t] = CS_OK_OUT;
            }
    auto P = [&](int i, int j, int k) { return phi[flat(i, j, k, ni, nj)]; };
    std::vector<int> surface;
    for (int k = 0; k < nk; k++)
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++) {
                if (border(i, j, k) || st[flat(i, j, k, ni, nj)] != CS_UNSET) continue;
                const bool fl = P(i, j, k) < 0.0f;
                const int nb[6][3] = {{i + 1, j, k}, {i - 1, j, k}, {i, j + 1, k}, {i, j - 1, k}, {i, j, k + 1}, {i, j, k - 1}};
                for (auto &q : nb) {
                    const float nd = P(q[0], q[1], q[2]);
                    if (fl ? nd >= 0.0f : nd < 0.0f) { surface.push_back((int)flat(i, j, k, ni, nj)); break; }
                }
            }
    std::vector<char> processed(st.size(), 0);
    std::vector<int> queue;
    const int threshold = 36;   // _surfaceTensionClusterThreshold
    for (int seed : surface) {
        if (st[seed] != CS_UNSET) continue;
        queue.clear();
        queue.push_back(seed);
        processed[seed] = 1;
        const bool fl = phi[seed] < 0.0f;
        char result = CS_UNSET;
        bool stop = false;
        for (size_t f = 0; f < queue.size() && !stop; f++) {
            const int g = queue[f];
            const int i = g % ni, j = (g / ni) % nj, k = g / (ni * nj);
            const int nb[6][3] = {{i + 1, j, k}, {i - 1, j, k}, {i, j + 1, k}, {i, j - 1, k}, {i, j, k + 1}, {i, j, k - 1}};
            for (auto &q : nb) {
                const int n = (int)flat(q[0], q[1], q[2], ni, nj);
                if (processed[n]) continue;
                if (!(fl ? phi[n] < 0.0f : phi[n] >= 0.0f)) continue;
                const char ns = st[n];
                if (ns == CS_BORDER) continue;
                if (ns != CS_UNSET) { result = ns; stop = true; break; }
                queue.push_back(n);
                processed[n] = 1;
                if ((int)queue.size() == threshold) result = fl ? CS_OK_IN : CS_OK_OUT;
            }
        }
        if (result == CS_UNSET && (int)queue.size() < threshold) result = fl ? CS_BAD_IN : CS_BAD_OUT;
        for (int q : queue) { st[q] = result; processed[q] = 0; }
    }
    return st;
}

// Interpolation::trilinearInterpolate of a cell-centred float grid at p - dx/2, in double
double sample_centred(const float *g, int ni, int nj, int nk, double dx, float px, float py, float pz) {
    const float sh = (float)(0.5 * dx);
    const float x = px - sh, y = py - sh, z = pz - sh;
    const double inv = 1.0 / dx;
    const int i = (int)std::floor(x * inv), j = (int)std::floor(y * inv), k = (int)std::floor(z * inv);
    const float gx = (float)((double)(float)i * dx), gy = (float)((double)(float)j * dx), gz = (float)((double)(float)k * dx);
    const double ix = (double)(x - gx) * inv, iy = (double)(y - gy) * inv, iz = (double)(z - gz) * inv;
    auto G = [&](int a, int b, int c) -> double {
        return (a >= 0 && b >= 0 && c >= 0 && a < ni && b < nj && c < nk) ? g[flat(a, b, c, ni, nj)] : 0.0;
    };
    const double p0 = G(i, j, k), p1 = G(i + 1, j, k), p2 = G(i, j + 1, k), p3 = G(i, j, k + 1), p4 = G(i + 1, j, k + 1),
                 p5 = G(i, j + 1, k + 1), p6 = G(i + 1, j + 1, k), p7 = G(i + 1, j + 1, k + 1);
    return p0 * (1 - ix) * (1 - iy) * (1 - iz) + p1 * ix * (1 - iy) * (1 - iz) + p2 * (1 - ix) * iy * (1 - iz) +
           p3 * (1 - ix) * (1 - iy) * iz + p4 * ix * (1 - iy) * iz + p5 * (1 - ix) * iy * iz + p6 * ix * iy * (1 - iz) +
           p7 * ix * iy * iz;
}

// PressureSolver::_getSurfaceTensionTerm (pressuresolver.cpp:715-749)
double tension_term(int ni, int nj, int nk, double dx, const float *phi, const float *curv, double k_st,
                    const std::vector<char> &st, int i1, int j1, int k1, int i2, int j2, int k2) {
    const char s = st[flat(i1, j1, k1, ni, nj)] | st[flat(i2, j2, k2, ni, nj)];
    if ((s & CS_BAD_IN) || (s & CS_BAD_OUT)) return 0.0;
    const double hw = 0.5 * dx;   // GridIndexToCellCenter (grid3d.h:86-103), in double, then float
    const float p1x = (float)((double)i1 * dx + hw), p1y = (float)((double)j1 * dx + hw), p1z = (float)((double)k1 * dx + hw);
    const float p2x = (float)((double)i2 * dx + hw), p2y = (float)((double)j2 * dx + hw), p2z = (float)((double)k2 * dx + hw);
    const float phi1 = phi[flat(i1, j1, k1, ni, nj)], phi2 = phi[flat(i2, j2, k2, ni, nj)];
    if ((phi1 < 0.0f && phi2 < 0.0f) || (phi1 >= 0.0f && phi2 >= 0.0f)) return 0.0;
    float px, py, pz;
    if (std::abs(phi2 - phi1) < 1e-6f) {
        px = p1x + 0.5f * (p2x - p1x); py = p1y + 0.5f * (p2y - p1y); pz = p1z + 0.5f * (p2z - p1z);
    } else {
        const float th = phi1 / (phi1 - phi2);
        px = p1x + th * (p2x - p1x); py = p1y + th * (p2y - p1y); pz = p1z + th * (p2z - p1z);
    }
    const double curvature = sample_centred(curv, ni, nj, nk, dx, px, py, pz);
    return k_st * curvature;
}

// adds the surface tension terms to the rhs of a built system (pressuresolver.cpp:659-709)
void add_tension(Sys &s, int ni, int nj, int nk, double dx, double dt, const float *phi, const float *wu,
                 const float *wv, const float *ww, const float *curv, double k_st) {
    const std::vector<char> st = cluster_status(ni, nj, nk, phi);
    const double stfactor = dt / (dx * dx), eps = 1e-9, maxtheta = 25;
    auto P = [&](int i, int j, int k) { return (double)phi[flat(i, j, k, ni, nj)]; };
    for (int r = 0; r < s.n; r++) {
        const int i = s.ci[r], j = s.cj[r], k = s.ck[r];
        const double vol[6] = {wu[flat(i + 1, j, k, ni + 1, nj)], wu[flat(i, j, k, ni + 1, nj)],
                               wv[flat(i, j + 1, k, ni, nj + 1)], wv[flat(i, j, k, ni, nj + 1)],
                               ww[flat(i, j, k + 1, ni, nj)],     ww[flat(i, j, k, ni, nj)]};
        const int nb[6][3] = {{i + 1, j, k}, {i - 1, j, k}, {i, j + 1, k}, {i, j - 1, k}, {i, j, k + 1}, {i, j, k - 1}};
        const double pc = P(i, j, k);
        double div = s.rhs[r];
        for (int q = 0; q < 6; q++) {
            const double pn = P(nb[q][0], nb[q][1], nb[q][2]);
            if (pn >= 0.0) {
                const double tension = tension_term(ni, nj, nk, dx, phi, curv, k_st, st, i, j, k, nb[q][0], nb[q][1], nb[q][2]);
                const double theta = clampd((pc - pn) / (pc + eps), -maxtheta, maxtheta);
                div += stfactor * vol[q] * theta * tension;
            }
        }
        s.rhs[r] = div;
    }
}

struct Factor {   // SparseColumnLowerFactor (pcgsolver.h:30-58)
    std::vector<double> invdiag, value, adiag;
    std::vector<int> rowindex, colstart;
};

void mic0(const Sys &A, Factor &F, double tau = 0.97, double sigma = 0.25) {   // pcgsolver.h:68-205
    int n = A.n;
    F.invdiag.assign(n, 0.0); F.adiag.assign(n, 0.0);
    F.value.clear(); F.rowindex.clear(); F.colstart.assign(n + 1, 0);
    const double eps = 1e-9;
    for (int i = 0; i < n; i++) {
        F.colstart[i] = (int)F.rowindex.size();
        for (size_t q = 0; q < A.idx[i].size(); q++) {
            int c = A.idx[i][q];
            if (c > i) { F.rowindex.push_back(c); F.value.push_back(A.val[i][q]); }
            else if (c == i) {
                double d = A.val[i][q];
                if (d < eps) d = 0;
                F.invdiag[i] = F.adiag[i] = d;
            }
        }
    }
    F.colstart[n] = (int)F.rowindex.size();
    for (int k = 0; k < n; k++) {
        if (F.adiag[k] == 0) continue;
        if (F.invdiag[k] < sigma * F.adiag[k]) F.invdiag[k] = 1 / std::sqrt(F.adiag[k]);
        else F.invdiag[k] = 1 / std::sqrt(F.invdiag[k]);
        for (int p = F.colstart[k]; p < F.colstart[k + 1]; p++) F.value[p] *= F.invdiag[k];
        for (int p = F.colstart[k]; p < F.colstart[k + 1]; p++) {
            int j = F.rowindex[p];
            double mult = F.value[p];
            double missing = 0;
            int a = F.colstart[k];
            size_t b = 0;
            while (a < F.colstart[k + 1] && F.rowindex[a] < j) {
                while (b < A.idx[j].size()) {
                    if (A.idx[j][b] < F.rowindex[a]) b++;
                    else if (A.idx[j][b] == F.rowindex[a]) break;
                    else { missing += F.value[a]; break; }
                }
                a++;
            }
            if (a < F.colstart[k + 1] && F.rowindex[a] == j) F.invdiag[j] -= mult * F.value[a];
            a++;
            int bb = F.colstart[j];
            while (a < F.colstart[k + 1] && bb < F.colstart[j + 1]) {
                if (F.rowindex[bb] < F.rowindex[a]) bb++;
                else if (F.rowindex[bb] == F.rowindex[a]) { F.value[bb] -= mult * F.value[a]; a++; bb++; }
                else { missing += F.value[a]; a++; }
            }
            while (a < F.colstart[k + 1]) { missing += F.value[a]; a++; }
            F.invdiag[j] -= tau * mult * missing;
        }
    }
}

void apply_precon(const Factor &F, const std::vector<double> &x, std::vector<double> &res) {  // pcgsolver.h:212-241
    int n = (int)F.invdiag.size();
    res = x;
    for (int i = 0; i < n; i++) {
        res[i] *= F.invdiag[i];
        for (int q = F.colstart[i]; q < F.colstart[i + 1]; q++) res[F.rowindex[q]] -= F.value[q] * res[i];
    }
    for (int i = n - 1; i >= 0; i--) {
        for (int q = F.colstart[i]; q < F.colstart[i + 1]; q++) res[i] -= F.value[q] * res[F.rowindex[q]];
        res[i] *= F.invdiag[i];
    }
}

double dotv(const std::vector<double> &a, const std::vector<double> &b) {
    double s = 0;
    for (size_t i = 0; i < a.size(); i++) s += a[i] * b[i];
    return s;
}
double absmax(const std::vector<double> &a) {
    double m = 0;
    for (double x : a) if (std::fabs(x) > m) m = std::fabs(x);
    return m;
}
void spmv(const Sys &A, const std::vector<double> &x, std::vector<double> &y) {
    y.assign(A.n, 0.0);
    for (int i = 0; i < A.n; i++) {
        double s = 0;
        for (size_t q = 0; q < A.idx[i].size(); q++) s += A.val[i][q] * x[A.idx[i][q]];
        y[i] = s;
    }
}

// PCGSolver::solve (pcgsolver.h:268-322).  float_scalars reproduces addScaled(float alpha, ...).
bool pcg(const Sys &A, std::vector<double> &x, double tol_factor, int maxit, bool float_scalars,
         double &resid_out, int &iters_out) {
    int n = A.n;
    std::vector<double> r = A.rhs, z, s, t;
    resid_out = absmax(r);
    if (resid_out == 0) { iters_out = 0; return true; }
    double tol = tol_factor * resid_out;
    Factor F;
    mic0(A, F);
    apply_precon(F, r, z);
    double rho = dotv(z, r);
    if (rho == 0 || rho != rho) { iters_out = 0; return false; }
    s = z;
    auto sc = [&](double a) { return float_scalars ? (double)(float)a : a; };
    int it;
    for (it = 0; it < maxit; it++) {
        spmv(A, s, z);
        double alpha = rho / dotv(s, z);
        double fa = sc(alpha), fna = sc(-alpha);
        for (int i = 0; i < n; i++) x[i] += fa * s[i];
        for (int i = 0; i < n; i++) r[i] += fna * z[i];
        resid_out = absmax(r);
        if (resid_out <= std::min(tol, 1.0)) { iters_out = it + 1; return true; }
        apply_precon(F, r, z);
        double rhonew = dotv(z, r);
        double beta = rhonew / rho;
        double fb = sc(beta);
        for (int i = 0; i < n; i++) z[i] += fb * s[i];
        s.swap(z);
        rho = rhonew;
    }
    iters_out = it;
    return false;
}

}  // namespace

extern "C" {

// Solves the pressure system for one substep.  Writes the cell pressure grid (ni*nj*nk,
// zero outside pressure cells) and returns {iterations, success} in stats and the final
// recursive inf-norm residual in *err_out.  float_scalars=1 reproduces the reference's
// float-truncated step lengths; 0 keeps them in double.
int oracle_pressure_solve(int ni, int nj, int nk, double dx, double dt, const float *phi,
                          const float *wu, const float *wv, const float *ww,
                          const float *u, const float *v, const float *w,
                          double tol, int maxit, int float_scalars,
                          float *pressure, int *stats, double *err_out) {
    Sys A;
    build(A, ni, nj, nk, dx, dt, phi, wu, wv, ww, u, v, w);
    size_t nc = (size_t)ni * nj * nk;
    for (size_t c = 0; c < nc; c++) pressure[c] = 0.0f;
    double maxabs = absmax(A.rhs);
    if (maxabs < tol) { stats[0] = 0; stats[1] = 1; *err_out = 0.0; return A.n; }
    std::vector<double> x(A.n, 0.0);
    double resid; int iters;
    bool ok = pcg(A, x, tol, maxit, float_scalars != 0, resid, iters);
    for (int r = 0; r < A.n; r++) pressure[flat(A.ci[r], A.cj[r], A.ck[r], ni, nj)] = (float)x[r];
    bool success = ok || (iters == maxit && (float)resid < 1.0);   // pressuresolver.cpp:892-915
    stats[0] = iters; stats[1] = success ? 1 : 0;
    *err_out = resid;
    return A.n;
}

// Surface-tension cluster status per cell (pressuresolver.cpp:314-605, one thread): 0x01/0x02 ok
// inside/outside, 0x04/0x08 bad inside/outside, 0x10 border, 0 unset.
void oracle_cluster_status(int ni, int nj, int nk, const float *phi, char *status) {
    const std::vector<char> st = cluster_status(ni, nj, nk, phi);
    std::copy(st.begin(), st.end(), status);
}

// The same solve with surface tension (pressuresolver.cpp:314-605, 659-749): curv is the surface
// curvature grid (ni*nj*nk) and k_st the surface tension constant.
int oracle_pressure_solve_tension(int ni, int nj, int nk, double dx, double dt, const float *phi,
                                  const float *wu, const float *wv, const float *ww,
                                  const float *u, const float *v, const float *w, const float *curv, double k_st,
                                  double tol, int maxit, int float_scalars,
                                  float *pressure, int *stats, double *err_out) {
    Sys A;
    build(A, ni, nj, nk, dx, dt, phi, wu, wv, ww, u, v, w);
    add_tension(A, ni, nj, nk, dx, dt, phi, wu, wv, ww, curv, k_st);
    size_t nc = (size_t)ni * nj * nk;
    for (size_t c = 0; c < nc; c++) pressure[c] = 0.0f;
    double maxabs = absmax(A.rhs);
    if (maxabs < tol) { stats[0] = 0; stats[1] = 1; *err_out = 0.0; return A.n; }
    std::vector<double> x(A.n, 0.0);
    double resid; int iters;
    bool ok = pcg(A, x, tol, maxit, float_scalars != 0, resid, iters);
    for (int r = 0; r < A.n; r++) pressure[flat(A.ci[r], A.cj[r], A.ck[r], ni, nj)] = (float)x[r];
    bool success = ok || (iters == maxit && (float)resid < 1.0);
    stats[0] = iters; stats[1] = success ? 1 : 0;
    *err_out = resid;
    return A.n;
}

// FP64 check of a pressure grid against the FP64 system: returns ||b - A p||_inf / ||b||_inf
// and writes the relative L2 norm into *rel_l2.
double oracle_pressure_residual(int ni, int nj, int nk, double dx, double dt, const float *phi,
                                const float *wu, const float *wv, const float *ww,
                                const float *u, const float *v, const float *w,
                                const double *pressure64, double *rel_l2) {
    Sys A;
    build(A, ni, nj, nk, dx, dt, phi, wu, wv, ww, u, v, w);
    std::vector<double> x(A.n), y;
    for (int r = 0; r < A.n; r++) x[r] = pressure64[flat(A.ci[r], A.cj[r], A.ck[r], ni, nj)];
    spmv(A, x, y);
    double bn = absmax(A.rhs), rn = 0, b2 = 0, r2 = 0;
    for (int r = 0; r < A.n; r++) {
        double e = A.rhs[r] - y[r];
        rn = std::max(rn, std::fabs(e));
        r2 += e * e; b2 += A.rhs[r] * A.rhs[r];
    }
    *rel_l2 = b2 > 0 ? std::sqrt(r2 / b2) : 0.0;
    return bn > 0 ? rn / bn : 0.0;
}

// Exports the FP64 system (rows in k-j-i order) for dense checks on small grids:
// cells[3*n], rhs[n], and a dense n x n matrix if dense != nullptr.  Returns n.
int oracle_pressure_system(int ni, int nj, int nk, double dx, double dt, const float *phi,
                           const float *wu, const float *wv, const float *ww,
                           const float *u, const float *v, const float *w,
                           int maxn, int *cells, double *rhs, double *dense) {
    Sys A;
    build(A, ni, nj, nk, dx, dt, phi, wu, wv, ww, u, v, w);
    if (A.n > maxn) return A.n;
    for (int r = 0; r < A.n; r++) {
        cells[3 * r] = A.ci[r]; cells[3 * r + 1] = A.cj[r]; cells[3 * r + 2] = A.ck[r];
        rhs[r] = A.rhs[r];
        if (dense) {
            for (int c = 0; c < A.n; c++) dense[(size_t)r * A.n + c] = 0.0;
            for (size_t q = 0; q < A.idx[r].size(); q++) dense[(size_t)r * A.n + A.idx[r][q]] = A.val[r][q];
        }
    }
    return A.n;
}

// pressuresolver.cpp:94-112 and :1047-1205 (unit density).  Resets and sets the valid flags;
// faces 0 and n-1 along the component axis are left untouched.  With curv != null the ghost
// pressure at an air neighbour adds thetaTension * tension, the surface tension term of the
// face's lower and upper cell (in that order, :1076, :1127, :1177); otherwise that term is 0.
void oracle_apply_pressure_tension(int ni, int nj, int nk, double dx, double dt, const float *phi,
                                   const float *wu, const float *wv, const float *ww, const float *pressure,
                                   const float *curv, double k_st, float *u, float *v, float *w,
                                   unsigned char *vu, unsigned char *vv, unsigned char *vw) {
    std::vector<char> st;
    if (curv) st = cluster_status(ni, nj, nk, phi);
    auto tension_of = [&](int i1, int j1, int k1, int i2, int j2, int k2) {
        return curv ? tension_term(ni, nj, nk, dx, phi, curv, k_st, st, i1, j1, k1, i2, j2, k2) : 0.0;
    };
    const float factor = (float)(dt / dx);
    const float eps = 1e-6f;
    const double maxtheta = 25;
    auto inr = [&](int i, int j, int k) { return i >= 0 && j >= 0 && k >= 0 && i < ni && j < nj && k < nk; };
    auto fluid = [&](int i, int j, int k) { return inr(i, j, k) && phi[flat(i, j, k, ni, nj)] < 0.0; };
    auto P = [&](int i, int j, int k) { return inr(i, j, k) ? pressure[flat(i, j, k, ni, nj)] : 0.0f; };
    // cells beyond the grid edge read as air (the closed domain never opens an edge face)
    auto L = [&](int i, int j, int k) { return inr(i, j, k) ? phi[flat(i, j, k, ni, nj)] : 1.0f; };
    for (size_t t = 0; t < (size_t)(ni + 1) * nj * nk; t++) vu[t] = 0;
    for (size_t t = 0; t < (size_t)ni * (nj + 1) * nk; t++) vv[t] = 0;
    for (size_t t = 0; t < (size_t)ni * nj * (nk + 1); t++) vw[t] = 0;
    // generic face update between cells c1 (lower) and c2 (upper)
    auto face = [&](float wgt, bool border, int i1, int j1, int k1, int i2, int j2, int k2,
                    float &vel, unsigned char &valid) {
        bool f1 = fluid(i1, j1, k1);
        bool f2 = fluid(i2, j2, k2);
        (void)border;
        if (wgt > 0 && (f1 || f2)) {
            float p1 = 0.0f, p2 = 0.0f;
            if (f1 && f2) { p1 = P(i1, j1, k1); p2 = P(i2, j2, k2); }
            else {
                float phi1 = L(i1, j1, k1), phi2 = L(i2, j2, k2);
                const double tension = tension_of(i1, j1, k1, i2, j2, k2);
                if (f1) {
                    float th = phi2 / (phi1 + eps);
                    th = (float)clampd((double)th, -maxtheta, maxtheta);
                    float tt = (phi1 - phi2) / (phi1 + eps);
                    tt = (float)clampd((double)tt, -maxtheta, maxtheta);
                    p1 = P(i1, j1, k1);
                    p2 = (float)((double)tt * tension + (double)(th * p1));
                } else {
                    float th = phi1 / (phi2 + eps);
                    th = (float)clampd((double)th, -maxtheta, maxtheta);
                    float tt = (phi2 - phi1) / (phi2 + eps);
                    tt = (float)clampd((double)tt, -maxtheta, maxtheta);
                    p2 = P(i2, j2, k2);
                    p1 = (float)((double)tt * tension + (double)(th * p2));
                }
            }
            float rho = (1.0f + 1.0f) / 2.0f;
            vel += -factor * (p2 - p1) / rho;
            valid = 1;
        } else {
            vel = 0.0f;
        }
    };
    for (int k = 0; k < nk; k++)
        for (int j = 0; j < nj; j++)
            for (int i = 0; i <= ni; i++) {
                if (i == 0 || i == ni - 1) continue;
                size_t f = flat(i, j, k, ni + 1, nj);
                face(wu[f], false, i - 1, j, k, i, j, k, u[f], vu[f]);
            }
    for (int k = 0; k < nk; k++)
        for (int j = 0; j <= nj; j++)
            for (int i = 0; i < ni; i++) {
                if (j == 0 || j == nj - 1) continue;
                size_t f = flat(i, j, k, ni, nj + 1);
                face(wv[f], false, i, j - 1, k, i, j, k, v[f], vv[f]);
            }
    for (int k = 0; k <= nk; k++)
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++) {
                if (k == 0 || k == nk - 1) continue;
                size_t f = flat(i, j, k, ni, nj);
                face(ww[f], false, i, j, k - 1, i, j, k, w[f], vw[f]);
            }
}

void oracle_apply_pressure(int ni, int nj, int nk, double dx, double dt, const float *phi,
                           const float *wu, const float *wv, const float *ww, const float *pressure,
                           float *u, float *v, float *w,
                           unsigned char *vu, unsigned char *vv, unsigned char *vw) {
    oracle_apply_pressure_tension(ni, nj, nk, dx, dt, phi, wu, wv, ww, pressure, nullptr, 0.0, u, v, w, vu, vv, vw);
}

}  // extern "C"
