// Oracle (test infrastructure only): particle-to-grid FLIP velocity transfer,
// layered velocity extrapolation and constant body forces.
//   P2G: VelocityAdvector::_advectGrid and helpers (velocityadvector.cpp:74-536), with the
//        reference's per-block float frame and per-face summation in particle order.
//   Extrapolation: GridUtils::extrapolateGrid (gridutils.h:43-163, gridutils.cpp:99-170).
//   Body force: FluidSimulation::_applyConstantBodyForces (fluidsimulation.cpp:5837-5876).
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <vector>

using namespace oracle;

namespace {
const int CW = 10;   // velocityadvector.h:187 (_chunkWidth)
inline int ifloor(double v) { return (int)std::floor(v); }
}

// Particle-to-block assignment shared by the FLIP and APIC transfers
// (velocityadvector.cpp:239-353): positions in the face-offset frame, and for every active
// block the particles assigned to it, in particle order.
struct P2GBlocks {
    int fw, fh, fd, bi, bj, bk;
    std::vector<float> sp;
    std::vector<std::vector<int>> bucket;
};

static P2GBlocks p2g_blocks(int ni, int nj, int nk, double dx, double radius, int np, const float *pos, int dir) {
    P2GBlocks B;
    int fw = ni + (dir == 0), fh = nj + (dir == 1), fd = nk + (dir == 2);
    B.fw = fw; B.fh = fh; B.fd = fd;

    float hdx = (float)(0.5 * dx);
    float ox = dir == 0 ? 0.0f : hdx, oy = dir == 1 ? 0.0f : hdx, oz = dir == 2 ? 0.0f : hdx;  // :177-188
    std::vector<float> &sp = B.sp;
    sp.resize(3 * (size_t)np);
    for (int p = 0; p < np; p++) {
        sp[3 * p] = pos[3 * p] - ox; sp[3 * p + 1] = pos[3 * p + 1] - oy; sp[3 * p + 2] = pos[3 * p + 2] - oz;
    }
    int bi = (fw + CW - 1) / CW, bj = (fh + CW - 1) / CW, bk = (fd + CW - 1) / CW;
    B.bi = bi; B.bj = bj; B.bk = bk;
    auto bid = [&](int a, int b, int c) -> long long {
        if (a < 0 || b < 0 || c < 0 || a >= bi || b >= bj || c >= bk) return -1;
        return a + (long long)bi * (b + (long long)bj * c);
    };
    size_t nb = (size_t)bi * bj * bk;
    const double chunkdx = dx * CW;
    // active blocks (:239-250) then featherGrid26
    std::vector<char> act(nb, 0), act2;
    for (int p = 0; p < np; p++) {
        double inv = 1.0 / chunkdx;
        long long id = bid(ifloor(sp[3 * p] * inv), ifloor(sp[3 * p + 1] * inv), ifloor(sp[3 * p + 2] * inv));
        if (id >= 0) act[id] = 1;
    }
    act2 = act;
    for (int c = 0; c < bk; c++)
        for (int b = 0; b < bj; b++)
            for (int a = 0; a < bi; a++) {
                if (!act[bid(a, b, c)]) continue;
                for (int z = -1; z <= 1; z++)
                    for (int y = -1; y <= 1; y++)
                        for (int x = -1; x <= 1; x++) {
                            long long id = bid(a + x, b + y, c + z);
                            if (id >= 0) act2[id] = 1;
                        }
            }
    // block assignment (:293-353), buckets keep particle order
    const float eps = 1e-6f;
    const float sr = (float)(radius + eps);
    const float fblockdx = (float)chunkdx;
    const double inv_fb = 1.0 / (double)fblockdx;
    std::vector<std::vector<int>> &bucket = B.bucket;
    bucket.assign(nb, std::vector<int>());
    for (int p = 0; p < np; p++) {
        float x = sp[3 * p], y = sp[3 * p + 1], z = sp[3 * p + 2];
        int a = ifloor(x * inv_fb), b = ifloor(y * inv_fb), c = ifloor(z * inv_fb);
        float bx = (float)((double)(float)a * (double)fblockdx);
        float by = (float)((double)(float)b * (double)fblockdx);
        float bz = (float)((double)(float)c * (double)fblockdx);
        if (x - sr > bx && y - sr > by && z - sr > bz &&
            x + sr < bx + fblockdx && y + sr < by + fblockdx && z + sr < bz + fblockdx) {
            long long id = bid(a, b, c);
            if (id >= 0 && act2[id]) bucket[id].push_back(p);
        } else {
            int a0 = ifloor((double)(x - sr) * inv_fb), b0 = ifloor((double)(y - sr) * inv_fb), c0 = ifloor((double)(z - sr) * inv_fb);
            int a1 = ifloor((double)(x + sr) * inv_fb), b1 = ifloor((double)(y + sr) * inv_fb), c1 = ifloor((double)(z + sr) * inv_fb);
            for (int cc = c0; cc <= c1; cc++)
                for (int bb = b0; bb <= b1; bb++)
                    for (int aa = a0; aa <= a1; aa++) {
                        long long id = bid(aa, bb, cc);
                        if (id >= 0 && act2[id]) bucket[id].push_back(p);
                    }
        }
    }
    return B;
}

extern "C" {

// dir: 0 = U, 1 = V, 2 = W.  Face grid dims: U (ni+1, nj, nk), V (ni, nj+1, nk), W (ni, nj, nk+1).
void oracle_p2g_component(int ni, int nj, int nk, double dx, double radius, int np,
                          const float *pos, const float *vel, int dir,
                          float *field, unsigned char *valid) {
    int fw = ni + (dir == 0), fh = nj + (dir == 1), fd = nk + (dir == 2);
    size_t nf = (size_t)fw * fh * fd;
    for (size_t t = 0; t < nf; t++) { field[t] = 0.0f; valid[t] = 0; }
    if (np == 0) return;
    P2GBlocks B = p2g_blocks(ni, nj, nk, dx, radius, np, pos, dir);
    const std::vector<float> &sp = B.sp;
    const std::vector<std::vector<int>> &bucket = B.bucket;
    const int bi = B.bi, bj = B.bj;
    const size_t nb = bucket.size();
    const double chunkdx = dx * CW;
    const float eps = 1e-6f;
    const float sr = (float)(radius + eps);
    // accumulation (:467-536)
    const float r = (float)radius;
    const float rsq = r * r;
    const float coef1 = (4.0f / 9.0f) * (1.0f / (r * r * r * r * r * r));
    const float coef2 = (17.0f / 9.0f) * (1.0f / (r * r * r * r));
    const float coef3 = (22.0f / 9.0f) * (1.0f / (r * r));
    const double inv_dx = 1.0 / dx;
    float gp[CW];
    for (int l = 0; l < CW; l++) gp[l] = (float)((double)(float)l * dx);
#pragma omp parallel for schedule(dynamic, 4)
    for (long long id = 0; id < (long long)nb; id++) {
        if (bucket[id].empty()) continue;
        int a = (int)(id % bi), b = (int)((id / bi) % bj), c = (int)(id / ((long long)bi * bj));
        float bx = (float)((double)(float)a * chunkdx), by = (float)((double)(float)b * chunkdx), bz = (float)((double)(float)c * chunkdx);
        float S[CW * CW * CW], W[CW * CW * CW];
        for (int t = 0; t < CW * CW * CW; t++) { S[t] = 0.0f; W[t] = 0.0f; }
        for (int p : bucket[id]) {
            float x = sp[3 * p] - bx, y = sp[3 * p + 1] - by, z = sp[3 * p + 2] - bz;
            float v = vel[3 * p + dir];
            int i0 = std::max(ifloor((double)(x - sr) * inv_dx), 0), i1 = std::min(ifloor((double)(x + sr) * inv_dx), CW - 1);
            int j0 = std::max(ifloor((double)(y - sr) * inv_dx), 0), j1 = std::min(ifloor((double)(y + sr) * inv_dx), CW - 1);
            int k0 = std::max(ifloor((double)(z - sr) * inv_dx), 0), k1 = std::min(ifloor((double)(z + sr) * inv_dx), CW - 1);
            for (int k = k0; k <= k1; k++)
                for (int j = j0; j <= j1; j++)
                    for (int i = i0; i <= i1; i++) {
                        float vx = gp[i] - x, vy = gp[j] - y, vz = gp[k] - z;
                        float d2 = vx * vx + vy * vy + vz * vz;
                        if (d2 < rsq) {
                            float wgt = 1.0f - coef1 * d2 * d2 * d2 + coef2 * d2 * d2 - coef3 * d2;
                            int t = i + CW * (j + CW * k);
                            S[t] += wgt * v;
                            W[t] += wgt;
                        }
                    }
        }
        for (int k = 0; k < CW; k++)
            for (int j = 0; j < CW; j++)
                for (int i = 0; i < CW; i++) {
                    int t = i + CW * (j + CW * k);
                    if (W[t] > eps) S[t] /= W[t];
                    int gi = a * CW + i, gj = b * CW + j, gk = c * CW + k;
                    if (gi < fw && gj < fh && gk < fd) {
                        size_t f = flat(gi, gj, gk, fw, fh);
                        field[f] = S[t];
                        if (W[t] > eps) valid[f] = 1;
                    }
                }
    }
}

// APIC transfer for one component (VelocityAdvector::_advectionAPICProducerThread,
// velocityadvector.cpp:543-623): the same block assignment as FLIP; in each block, every
// assigned particle adds w (v + a . (x_node - x)) and w to the nodes of its trilinear stencil
// that lie inside the block (a = its affine vector for this component, w = trilinear weight,
// all in the block's float frame), and nodes with a weight sum above 1e-6 are normalised.
// aff9: 9 floats per particle, the x, y and z components' affine vectors.
void oracle_p2g_apic_component(int ni, int nj, int nk, double dx, double radius, int np, const float *pos,
                               const float *vel, const float *aff9, int dir, float *field, unsigned char *valid) {
    int fw = ni + (dir == 0), fh = nj + (dir == 1), fd = nk + (dir == 2);
    size_t nf = (size_t)fw * fh * fd;
    for (size_t t = 0; t < nf; t++) { field[t] = 0.0f; valid[t] = 0; }
    if (np == 0) return;
    P2GBlocks B = p2g_blocks(ni, nj, nk, dx, radius, np, pos, dir);
    const std::vector<float> &sp = B.sp;
    const int bi = B.bi, bj = B.bj;
    const size_t nb = B.bucket.size();
    const double chunkdx = dx * CW;
    const float eps = 1e-6f;
    const double inv_dx = 1.0 / dx;
    const float invf = (float)(1.0 / (double)(float)dx);   // vec3 / float (vmath.cpp:100-103)
#pragma omp parallel for schedule(dynamic, 4)
    for (long long id = 0; id < (long long)nb; id++) {
        if (B.bucket[id].empty()) continue;
        int a = (int)(id % bi), b = (int)((id / bi) % bj), c = (int)(id / ((long long)bi * bj));
        float bx = (float)((double)(float)a * chunkdx), by = (float)((double)(float)b * chunkdx), bz = (float)((double)(float)c * chunkdx);
        float S[CW * CW * CW], W[CW * CW * CW];
        for (int t = 0; t < CW * CW * CW; t++) { S[t] = 0.0f; W[t] = 0.0f; }
        for (int p : B.bucket[id]) {
            const float x = sp[3 * p] - bx, y = sp[3 * p + 1] - by, z = sp[3 * p + 2] - bz;
            const float v = vel[3 * p + dir];
            const float ax = aff9[9 * p + 3 * dir], ay = aff9[9 * p + 3 * dir + 1], az = aff9[9 * p + 3 * dir + 2];
            const int gi = ifloor((double)x * inv_dx), gj = ifloor((double)y * inv_dx), gk = ifloor((double)z * inv_dx);
            const float gx = (float)((double)(float)gi * dx), gy = (float)((double)(float)gj * dx), gz = (float)((double)(float)gk * dx);
            const float ix = (x - gx) * invf, iy = (y - gy) * invf, iz = (z - gz) * invf;
            const float wt[8] = {(1.0f - ix) * (1.0f - iy) * (1.0f - iz), ix * (1.0f - iy) * (1.0f - iz),
                                 (1.0f - ix) * iy * (1.0f - iz),          ix * iy * (1.0f - iz),
                                 (1.0f - ix) * (1.0f - iy) * iz,          ix * (1.0f - iy) * iz,
                                 (1.0f - ix) * iy * iz,                   ix * iy * iz};
            for (int q = 0; q < 8; q++) {
                const int i = gi + (q & 1), j = gj + ((q >> 1) & 1), k = gk + (q >> 2);
                if (i < 0 || j < 0 || k < 0 || i >= CW || j >= CW || k >= CW) continue;
                const float nx = (float)((double)(float)i * dx), ny = (float)((double)(float)j * dx),
                            nz = (float)((double)(float)k * dx);
                const float apic = ax * (nx - x) + ay * (ny - y) + az * (nz - z);
                const int t = i + CW * (j + CW * k);
                S[t] += wt[q] * (v + apic);
                W[t] += wt[q];
            }
        }
        for (int k = 0; k < CW; k++)
            for (int j = 0; j < CW; j++)
                for (int i = 0; i < CW; i++) {
                    int t = i + CW * (j + CW * k);
                    if (W[t] > eps) S[t] /= W[t];
                    int gi = a * CW + i, gj = b * CW + j, gk = c * CW + k;
                    if (gi < fw && gj < fh && gk < fd) {
                        size_t f = flat(gi, gj, gk, fw, fh);
                        field[f] = S[t];
                        if (W[t] > eps) valid[f] = 1;
                    }
                }
    }
}

// Layered extrapolation of `grid` (w x h x d) from cells flagged in `valid`.
void oracle_extrapolate(int w, int h, int d, float *grid, const unsigned char *valid, int layers) {
    const char UNKNOWN = 0, WAITING = 1, KNOWN = 2, DONE = 3;
    size_t n = (size_t)w * h * d;
    std::vector<char> st(n, UNKNOWN);
    for (int k = 0; k < d; k++)
        for (int j = 0; j < h; j++)
            for (int i = 0; i < w; i++) {
                size_t t = flat(i, j, k, w, h);
                if (i == 0 || j == 0 || k == 0 || i == w - 1 || j == h - 1 || k == d - 1) st[t] = DONE;
                else if (valid[t]) st[t] = KNOWN;
            }
    const long long nb[6] = {1, -1, (long long)w, -(long long)w, (long long)w * h, -(long long)w * h};
    std::vector<size_t> cells;
    for (int layer = 0; layer < layers; layer++) {
        cells.clear();
        for (size_t t = 0; t < n; t++) {
            if (st[t] != KNOWN) continue;
            for (int q = 0; q < 6; q++) {
                size_t u = (size_t)((long long)t + nb[q]);
                if (st[u] == UNKNOWN) { st[u] = WAITING; cells.push_back(u); }
            }
            st[t] = DONE;
        }
        for (size_t c : cells) {
            float sum = 0.0f;
            int count = 0;
            for (int q = 0; q < 6; q++) {
                size_t u = (size_t)((long long)c + nb[q]);
                if (st[u] == DONE) { sum += grid[u]; count++; }
            }
            grid[c] = sum / (float)count;
        }
        if (layer != layers - 1)
            for (size_t c : cells) st[c] = KNOWN;
    }
}

void oracle_body_force(int ni, int nj, int nk, double dt, float gx, float gy, float gz,
                       float *u, float *v, float *w) {
    const float eps = 1e-6f;
    if (std::fabs(gx) > eps) { float a = (float)(gx * dt); size_t n = (size_t)(ni + 1) * nj * nk; for (size_t t = 0; t < n; t++) u[t] += a; }
    if (std::fabs(gy) > eps) { float a = (float)(gy * dt); size_t n = (size_t)ni * (nj + 1) * nk; for (size_t t = 0; t < n; t++) v[t] += a; }
    if (std::fabs(gz) > eps) { float a = (float)(gz * dt); size_t n = (size_t)ni * nj * (nk + 1); for (size_t t = 0; t < n; t++) w[t] += a; }
}

}  // extern "C"
