// Oracle (test infrastructure only): the liquid surface curvature grid that feeds the
// surface-tension term (ParticleLevelSet::calculateCurvatureGrid, particlelevelset.cpp:196-291):
//   band of nodes with |phi| < 2 dx, widened to 6^3 blocks and one block layer
//   (GridUtils::featherGrid6, gridutils.cpp:229-262); upwind re-initialisation of the level set
//   over that band (LevelSetSolver::reinitializeUpwind, levelsetsolver.cpp:82-170, 317-390);
//   nodes outside the band set to 5 dx; curvature at the nodes whose 6 neighbours lie within
//   2 dx of the surface (_getValidCurvatureNodes, _getCurvature, particlelevelset.cpp:692-800);
//   three extrapolation layers (GridUtils::extrapolateGrid).
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <limits>
#include <vector>

using namespace oracle;

extern "C" void oracle_extrapolate(int w, int h, int d, float *grid, const unsigned char *valid, int layers);

namespace {

struct CGrid {
    int w, h, d;
    std::vector<float> a;
    float get(int i, int j, int k) const { return a[flat(i, j, k, w, h)]; }
};

inline float sq(float x) { return x * x; }

// LevelSetSolver::_sign: the distance in double, dx squared in float
inline float sign_of(const CGrid &g, float dx, int i, int j, int k) {
    const double d = g.get(i, j, k);
    return (float)(d / std::sqrt(d * d + dx * dx));
}

// LevelSetSolver::reinitializeUpwind (levelsetsolver.cpp:82-138); cells are the solver cells in
// the reference's order (duplicates included)
void reinit_upwind(const CGrid &in, float dx, float maxdist, const std::vector<int> &cells, CGrid &out) {
    const float max_cfl = 0.5f;
    float maxS = -std::numeric_limits<float>::max();
    for (int k = 0; k < in.d; k++)
        for (int j = 0; j < in.h; j++)
            for (int i = 0; i < in.w; i++) maxS = std::max(sign_of(in, dx, i, j, k), maxS);
    float dtau = max_cfl * dx;
    while (dtau * maxS / dx > max_cfl) dtau *= 0.5;
    const int iters = (int)std::ceil(maxdist / dtau);
    // outputSDF = inputSDF; tempSDF is allocated and never filled (levelsetsolver.cpp:95), and cells
    // outside the band are read from it from the second iteration on: in the reference's allocation
    // sequence that memory is a freed copy of the input level set, which is what is modelled here
    CGrid bufA = in;
    CGrid bufB = in;
    CGrid *outp = &bufA, *tmpp = &bufB;
    const float invdx = 1.0f / dx;
    float last = -1.0f;
    for (int n = 0; n < iters; n++) {
        for (int c : cells) {
            const int i = c % in.w, j = (c / in.w) % in.h, k = c / (in.w * in.h);
            const float s = sign_of(*outp, dx, i, j, k);
            const int im1 = i < 1 ? 0 : i - 1, ip1 = std::min(i + 1, in.w - 1);
            const int jm1 = j < 1 ? 0 : j - 1, jp1 = std::min(j + 1, in.h - 1);
            const int km1 = k < 1 ? 0 : k - 1, kp1 = std::min(k + 1, in.d - 1);
            const float c0 = outp->get(i, j, k);
            const float dx0 = invdx * (c0 - outp->get(im1, j, k)), dx1 = invdx * (outp->get(ip1, j, k) - c0);
            const float dy0 = invdx * (c0 - outp->get(i, jm1, k)), dy1 = invdx * (outp->get(i, jp1, k) - c0);
            const float dz0 = invdx * (c0 - outp->get(i, j, km1)), dz1 = invdx * (outp->get(i, j, kp1) - c0);
            const float val =
                c0 -
                dtau * std::max(s, 0.0f) *
                    (std::sqrt(sq(std::max(dx0, 0.0f)) + sq(std::min(dx1, 0.0f)) + sq(std::max(dy0, 0.0f)) +
                               sq(std::min(dy1, 0.0f)) + sq(std::max(dz0, 0.0f)) + sq(std::min(dz1, 0.0f))) -
                     1.0f) -
                dtau * std::min(s, 0.0f) *
                    (std::sqrt(sq(std::min(dx0, 0.0f)) + sq(std::max(dx1, 0.0f)) + sq(std::min(dy0, 0.0f)) +
                               sq(std::max(dy1, 0.0f)) + sq(std::min(dz0, 0.0f)) + sq(std::max(dz1, 0.0f))) -
                     1.0f);
            tmpp->a[c] = val;
        }
        float maxdiff = 0;
        for (int c : cells) maxdiff = std::max(std::abs(tmpp->a[c] - outp->a[c]), maxdiff);
        std::swap(tmpp, outp);
        if (std::abs(maxdiff - last) < 0.01f * dx) break;
        last = maxdiff;
    }
    out.a = outp->a;
}

// ParticleLevelSet::_getCurvature (particlelevelset.cpp:728-800, the active variant)
float curvature_at(const CGrid &p, double dx, int i, int j, int k) {
    if (i == 0 || j == 0 || k == 0 || i == p.w - 1 || j == p.h - 1 || k == p.d - 1) return 0.0f;
    const float x = 0.5f * (p.get(i + 1, j, k) - p.get(i - 1, j, k));
    const float y = 0.5f * (p.get(i, j + 1, k) - p.get(i, j - 1, k));
    const float z = 0.5f * (p.get(i, j, k + 1) - p.get(i, j, k - 1));
    const float xx = p.get(i + 1, j, k) - 2.0f * p.get(i, j, k) + p.get(i - 1, j, k);
    const float yy = p.get(i, j + 1, k) - 2.0f * p.get(i, j, k) + p.get(i, j - 1, k);
    const float zz = p.get(i, j, k + 1) - 2.0f * p.get(i, j, k) + p.get(i, j, k - 1);
    const float xy = 0.25f * (p.get(i + 1, j + 1, k) - p.get(i - 1, j + 1, k) - p.get(i + 1, j - 1, k) + p.get(i - 1, j - 1, k));
    const float xz = 0.25f * (p.get(i + 1, j, k + 1) - p.get(i - 1, j, k + 1) - p.get(i + 1, j, k - 1) + p.get(i - 1, j, k - 1));
    const float yz = 0.25f * (p.get(i, j + 1, k + 1) - p.get(i, j - 1, k + 1) - p.get(i, j + 1, k - 1) + p.get(i, j - 1, k - 1));
    float den = x * x + y * y + z * z;
    den = (float)std::sqrt((double)(den * den * den));   // unqualified sqrt of a float: the double one
    if (den < 1e-9f) return 0.0f;
    float curv = (float)(((xx * (y * y + z * z) + yy * (x * x + z * z) + zz * (x * x + y * y) - 2 * xy * x * y -
                           2 * xz * x * z - 2 * yz * y * z) / den) / dx);
    curv = std::min(curv, 1.0f / (float)dx);
    curv = std::max(curv, -1.0f / (float)dx);
    return curv;
}

}  // namespace

extern "C" {

// phi: the (post-processed) liquid level set, ni*nj*nk; surface_phi, kgrid: outputs of the same size.
void oracle_curvature_grid(int ni, int nj, int nk, double dx, const float *phi, float *surface_phi, float *kgrid) {
    const size_t n = (size_t)ni * nj * nk;
    const int band = 3;                                           // _curvatureGridExactBand
    const float maxsurf = (float)(2.0f * dx);
    std::vector<char> valid(n, 0);
    for (size_t t = 0; t < n; t++) valid[t] = std::abs(phi[t]) < maxsurf;
    const int bw = 2 * band;
    const int bi = (ni + bw - 1) / bw, bj = (nj + bw - 1) / bw, bk = (nk + bw - 1) / bw;
    std::vector<char> vb((size_t)bi * bj * bk, 0);
    for (int k = 0; k < nk; k++)
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++)
                if (valid[flat(i, j, k, ni, nj)]) vb[flat(i / bw, j / bw, k / bw, bi, bj)] = 1;
    {   // featherGrid6: one layer of face neighbours, read from a copy
        std::vector<char> src = vb;
        for (int k = 0; k < bk; k++)
            for (int j = 0; j < bj; j++)
                for (int i = 0; i < bi; i++) {
                    if (!src[flat(i, j, k, bi, bj)]) continue;
                    const int nb[6][3] = {{i - 1, j, k}, {i + 1, j, k}, {i, j - 1, k}, {i, j + 1, k}, {i, j, k - 1}, {i, j, k + 1}};
                    for (auto &q : nb)
                        if (q[0] >= 0 && q[1] >= 0 && q[2] >= 0 && q[0] < bi && q[1] < bj && q[2] < bk)
                            vb[flat(q[0], q[1], q[2], bi, bj)] = 1;
                }
    }
    int nvalid = 0;
    for (int k = 0; k < nk; k++)
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++)
                if (vb[flat(i / bw, j / bw, k / bw, bi, bj)]) { valid[flat(i, j, k, ni, nj)] = 1; nvalid++; }
    // std::vector<GridIndex> solverGridCells(numValid) holds numValid default (0, 0, 0) entries
    // before the valid nodes are appended (particlelevelset.cpp:250-258)
    std::vector<int> cells((size_t)nvalid, 0);
    for (int k = 0; k < nk; k++)
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++)
                if (valid[flat(i, j, k, ni, nj)]) cells.push_back((int)flat(i, j, k, ni, nj));
    CGrid src{ni, nj, nk, std::vector<float>(phi, phi + n)};
    CGrid out{ni, nj, nk, std::vector<float>()};
    reinit_upwind(src, (float)dx, (float)(band * dx), cells, out);
    const float oor = (float)(5.0f * dx);                         // _outOfRangeDistance * _dx
    for (size_t t = 0; t < n; t++)
        if (!valid[t]) out.a[t] = oor;
    // _getValidCurvatureNodes
    const float ub = (float)((band - 1) * dx);
    std::vector<char> tv(n, 0);
    for (size_t t = 0; t < n; t++) tv[t] = std::abs(out.a[t]) < ub;
    std::vector<unsigned char> vn(n, 0);
    for (int k = 1; k < nk - 1; k++)
        for (int j = 1; j < nj - 1; j++)
            for (int i = 1; i < ni - 1; i++) {
                const size_t t = flat(i, j, k, ni, nj);
                if (!tv[t]) continue;
                if (tv[flat(i + 1, j, k, ni, nj)] && tv[flat(i - 1, j, k, ni, nj)] && tv[flat(i, j + 1, k, ni, nj)] &&
                    tv[flat(i, j - 1, k, ni, nj)] && tv[flat(i, j, k + 1, ni, nj)] && tv[flat(i, j, k - 1, ni, nj)])
                    vn[t] = 1;
            }
    for (size_t t = 0; t < n; t++) kgrid[t] = 0.0f;
    for (int k = 0; k < nk; k++)
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++)
                if (vn[flat(i, j, k, ni, nj)]) kgrid[flat(i, j, k, ni, nj)] = curvature_at(out, dx, i, j, k);
    oracle_extrapolate(ni, nj, nk, kgrid, vn.data(), 3);          // _curvatureGridExtrapolationLayers
    std::copy(out.a.begin(), out.a.end(), surface_phi);
}

}  // extern "C"
