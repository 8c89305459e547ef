// Oracle (test infrastructure only): geometry helpers, solid level set, face weights,
// liquid signed distance field.  See oracle.h for the contract.
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace oracle {

float vlength(V3 a) {
    float s = a.x * a.x + a.y * a.y + a.z * a.z;
    return std::sqrt(s);
}

bool Box::inside(V3 p) const {  // aabb.cpp:130-133
    return p.x >= px && p.y >= py && p.z >= pz &&
           p.x < px + w && p.y < py + h && p.z < pz + d;
}

V3 Box::nearest_inside(V3 p) const {  // aabb.cpp:501-518
    if (inside(p)) return p;
    const double eps = 1e-6;
    float maxx = px + (float)w, maxy = py + (float)h, maxz = pz + (float)d;
    p.x = (float)std::fmax(p.x, px);
    p.y = (float)std::fmax(p.y, py);
    p.z = (float)std::fmax(p.z, pz);
    p.x = (float)std::fmin((double)p.x, (double)maxx - eps);
    p.y = (float)std::fmin((double)p.y, (double)maxy - eps);
    p.z = (float)std::fmin((double)p.z, (double)maxz - eps);
    return p;
}

Box expand(Box b, double v) {  // aabb.cpp:122-128
    double hv = 0.5 * v;
    float fh = (float)hv;
    b.px = b.px - fh; b.py = b.py - fh; b.pz = b.pz - fh;
    b.w += v; b.h += v; b.d += v;
    return b;
}

Box boundary_box(const Domain &dm) {  // fluidsimulation.cpp:5175-5180
    Box b;
    b.px = 0.0f; b.py = 0.0f; b.pz = 0.0f;
    b.w = dm.ni * dm.dx; b.h = dm.nj * dm.dx; b.d = dm.nk * dm.dx;
    return expand(b, -3 * dm.dx - 1e-4);
}

static inline void pos_to_index(V3 p, double dx, int &i, int &j, int &k) {  // grid3d.h:55-60
    double inv = 1.0 / dx;
    i = (int)std::floor(p.x * inv);
    j = (int)std::floor(p.y * inv);
    k = (int)std::floor(p.z * inv);
}

static inline double trilerp(const double p[8], double x, double y, double z) {
    // corner order {000,100,010,001,101,011,110,111} (interpolation.cpp:59-70)
    return p[0] * (1 - x) * (1 - y) * (1 - z) +
           p[1] * x * (1 - y) * (1 - z) +
           p[2] * (1 - x) * y * (1 - z) +
           p[3] * (1 - x) * (1 - y) * z +
           p[4] * x * (1 - y) * z +
           p[5] * (1 - x) * y * z +
           p[6] * x * y * (1 - z) +
           p[7] * x * y * z;
}

float solid_trilinear(const Grid &phi, double dx, V3 p) {  // interpolation.cpp:72-110
    int i, j, k;
    pos_to_index(p, dx, i, j, k);
    float gx = (float)((double)(float)i * dx), gy = (float)((double)(float)j * dx), gz = (float)((double)(float)k * dx);
    double inv = 1.0 / dx;
    double ix = (p.x - gx) * inv, iy = (p.y - gy) * inv, iz = (p.z - gz) * inv;
    double pts[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const int off[8][3] = {{0,0,0},{1,0,0},{0,1,0},{0,0,1},{1,0,1},{0,1,1},{1,1,0},{1,1,1}};
    for (int c = 0; c < 8; c++) {
        int a = i + off[c][0], b = j + off[c][1], e = k + off[c][2];
        if (phi.in(a, b, e)) pts[c] = phi.at(a, b, e);
    }
    return (float)trilerp(pts, ix, iy, iz);
}

static inline double bilerp(double v00, double v10, double v01, double v11, double ix, double iy) {
    double l1 = (1 - ix) * v00 + ix * v10;   // interpolation.cpp:194-199
    double l2 = (1 - ix) * v01 + ix * v11;
    return (1 - iy) * l1 + iy * l2;
}

V3 solid_gradient(const Grid &phi, double dx, V3 p) {  // interpolation.cpp:200-260
    int i, j, k;
    pos_to_index(p, dx, i, j, k);
    float gx = (float)((double)(float)i * dx), gy = (float)((double)(float)j * dx), gz = (float)((double)(float)k * dx);
    double inv = 1.0 / dx;
    double ix = (p.x - gx) * inv, iy = (p.y - gy) * inv, iz = (p.z - gz) * inv;
    auto g = [&](int a, int b, int e) -> float { return phi.in(a, b, e) ? phi.at(a, b, e) : 0.0f; };
    float v000 = g(i, j, k), v100 = g(i + 1, j, k), v010 = g(i, j + 1, k), v001 = g(i, j, k + 1);
    float v101 = g(i + 1, j, k + 1), v011 = g(i, j + 1, k + 1), v110 = g(i + 1, j + 1, k), v111 = g(i + 1, j + 1, k + 1);
    float ddx00 = v100 - v000, ddx10 = v110 - v010, ddx01 = v101 - v001, ddx11 = v111 - v011;
    float dvdx = (float)bilerp(ddx00, ddx10, ddx01, ddx11, iy, iz);
    float ddy00 = v010 - v000, ddy10 = v110 - v100, ddy01 = v011 - v001, ddy11 = v111 - v101;
    float dvdy = (float)bilerp(ddy00, ddy10, ddy01, ddy11, ix, iz);
    float ddz00 = v001 - v000, ddz10 = v101 - v100, ddz01 = v011 - v010, ddz11 = v111 - v110;
    float dvdz = (float)bilerp(ddz00, ddz10, ddz01, ddz11, ix, iy);
    return v3(dvdx, dvdy, dvdz);
}

// ---- face weights (levelsetutils.cpp:39-141, meshlevelset.cpp:357-395) ----

static float frac2(float l, float r) {
    if (l < 0 && r < 0) return 1;
    if (l < 0 && r >= 0) return l / (l - r);
    if (l >= 0 && r < 0) return r / (r - l);
    return 0;
}

static void cycle4(float *a) {
    float t = a[0]; a[0] = a[1]; a[1] = a[2]; a[2] = a[3]; a[3] = t;
}

static float frac4(float bl, float br, float tl, float tr) {
    int inside = (bl < 0) + (tl < 0) + (br < 0) + (tr < 0);
    float L[4] = {bl, br, tr, tl};
    if (inside == 4) return 1;
    if (inside == 3) {
        while (L[0] < 0) cycle4(L);
        float s0 = 1 - frac2(L[0], L[3]);
        float s1 = 1 - frac2(L[0], L[1]);
        return 1.0f - 0.5f * s0 * s1;
    }
    if (inside == 2) {
        while (L[0] >= 0 || !(L[1] < 0 || L[2] < 0)) cycle4(L);
        if (L[1] < 0) {
            float sl = frac2(L[0], L[3]);
            float sr = frac2(L[1], L[2]);
            return 0.5f * (sl + sr);
        }
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
        while (L[0] >= 0) cycle4(L);
        float s0 = frac2(L[0], L[3]);
        float s1 = frac2(L[0], L[1]);
        return 0.5f * s0 * s1;
    }
    return 0;
}

static inline float clamp01(float x) { return x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x); }

}  // namespace oracle

using namespace oracle;

extern "C" {

// Nodal solid phi of the closed domain: positive inside the boundary box
// (fluidsimulation.cpp:5175-5180 inset box, negated mesh SDF at :5277-5286),
// unioned (min) with analytic spheres (cx, cy, cz, r) given in `spheres`.
void oracle_solid_phi(int ni, int nj, int nk, double dx, int nspheres, const double *spheres, float *phi) {
    Domain dm{ni, nj, nk, dx};
    Box b = boundary_box(dm);
    double lo[3] = {b.px, b.py, b.pz};
    double hi[3] = {(double)(float)(b.px + b.w), (double)(float)(b.py + b.h), (double)(float)(b.pz + b.d)};
    for (int k = 0; k <= nk; k++)
        for (int j = 0; j <= nj; j++)
            for (int i = 0; i <= ni; i++) {
                double x[3] = {(double)i * dx, (double)j * dx, (double)k * dx};
                double din = 1e30, dout2 = 0.0;
                bool inside = true;
                for (int a = 0; a < 3; a++) {
                    double dl = x[a] - lo[a], dh = hi[a] - x[a];
                    din = std::min(din, std::min(dl, dh));
                    if (dl < 0) { inside = false; dout2 += dl * dl; }
                    if (dh < 0) { inside = false; dout2 += dh * dh; }
                }
                double v = inside ? din : -std::sqrt(dout2);
                for (int s = 0; s < nspheres; s++) {
                    const double *sp = spheres + 4 * s;
                    double ex = x[0] - sp[0], ey = x[1] - sp[1], ez = x[2] - sp[2];
                    double ds = std::sqrt(ex * ex + ey * ey + ez * ez) - sp[3];
                    v = std::min(v, ds);
                }
                phi[flat(i, j, k, ni + 1, nj + 1)] = (float)v;
            }
}

// Face open fractions 1 - fractionInside(solid corners), clamped to [0, 1]
// (fluidsimulation.cpp:6110-6150 with meshlevelset.cpp:357-395).
void oracle_face_weights(int ni, int nj, int nk, const float *solid_phi, float *wu, float *wv, float *ww) {
    Grid s{ni + 1, nj + 1, nk + 1, const_cast<float *>(solid_phi)};
    for (int k = 0; k < nk; k++)
        for (int j = 0; j < nj; j++)
            for (int i = 0; i <= ni; i++)
                wu[flat(i, j, k, ni + 1, nj)] = clamp01(1.0f - frac4(s.at(i, j, k), s.at(i, j + 1, k), s.at(i, j, k + 1), s.at(i, j + 1, k + 1)));
    for (int k = 0; k < nk; k++)
        for (int j = 0; j <= nj; j++)
            for (int i = 0; i < ni; i++)
                wv[flat(i, j, k, ni, nj + 1)] = clamp01(1.0f - frac4(s.at(i, j, k), s.at(i, j, k + 1), s.at(i + 1, j, k), s.at(i + 1, j, k + 1)));
    for (int k = 0; k <= nk; k++)
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++)
                ww[flat(i, j, k, ni, nj)] = clamp01(1.0f - frac4(s.at(i, j, k), s.at(i, j + 1, k), s.at(i + 1, j, k), s.at(i + 1, j + 1, k)));
}

}  // extern "C"
