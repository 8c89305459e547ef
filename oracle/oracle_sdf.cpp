// Oracle (test infrastructure only): liquid signed distance field from marker particles
// and its post-process against the solid level set.  Restates
// ParticleLevelSet::_computeSignedDistanceFromParticles and its helpers
// (particlelevelset.cpp:335-666) and postProcessSignedDistanceField (:170-194),
// reproducing the reference's block-local float frame (10^3 blocks) bit for bit.
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <vector>

using namespace oracle;

namespace {

const int BW = 10;   // particlelevelset.h:147 (_blockwidth)

inline int ifloor(double v) { return (int)std::floor(v); }

struct BlockDims {
    int bi, bj, bk;
    int id(int a, int b, int c) const {
        if (a < 0 || b < 0 || c < 0 || a >= bi || b >= bj || c >= bk) return -1;
        return a + bi * (b + bj * c);
    }
};

}  // namespace

extern "C" {

// Raw particle SDF at cell centres (before post-processing).  radius is the particle
// radius in world units (0.5*sqrt(3)*dx for the engine defaults, fluidsimulation.cpp:4351).
void oracle_liquid_sdf(int ni, int nj, int nk, double dx, double radius, int np, const float *pos, float *phi) {
    const float maxd = (float)(3.0 * dx);                      // particlelevelset.cpp:331
    const size_t nc = (size_t)ni * nj * nk;
    for (size_t c = 0; c < nc; c++) phi[c] = maxd;
    if (np == 0) return;

    BlockDims bd{(ni + BW - 1) / BW, (nj + BW - 1) / BW, (nk + BW - 1) / BW};
    const size_t nb = (size_t)bd.bi * bd.bj * bd.bk;
    const float fblockdx = (float)(BW * dx);                   // float blockdx (:459, :517)
    const double inv_fb = 1.0 / (double)fblockdx;

    // active blocks: those holding a particle, feathered over 26 neighbours (:415-446)
    std::vector<char> act(nb, 0), act2;
    for (int p = 0; p < np; p++) {
        int a = ifloor(pos[3 * p] * inv_fb), b = ifloor(pos[3 * p + 1] * inv_fb), c = ifloor(pos[3 * p + 2] * inv_fb);
        int id = bd.id(a, b, c);
        if (id >= 0) act[id] = 1;
    }
    act2 = act;
    for (int c = 0; c < bd.bk; c++)
        for (int b = 0; b < bd.bj; b++)
            for (int a = 0; a < bd.bi; a++) {
                if (!act[bd.id(a, b, c)]) continue;
                for (int dz = -1; dz <= 1; dz++)
                    for (int dy = -1; dy <= 1; dy++)
                        for (int dxx = -1; dxx <= 1; dxx++) {
                            int id = bd.id(a + dxx, b + dy, c + dz);
                            if (id >= 0) act2[id] = 1;
                        }
            }

    // assign particles to blocks (:507-551)
    const float r = (float)radius;
    const float sr = 2.0f * r;                                 // _searchRadiusFactor (particlelevelset.h:149)
    std::vector<std::vector<int>> bucket(nb);
    for (int p = 0; p < np; p++) {
        float x = pos[3 * p], y = pos[3 * p + 1], z = pos[3 * p + 2];
        int a = ifloor(x * inv_fb), b = ifloor(y * inv_fb), c = ifloor(z * inv_fb);
        float bx = (float)((double)(float)a * (double)fblockdx);
        float by = (float)((double)(float)b * (double)fblockdx);
        float bz = (float)((double)(float)c * (double)fblockdx);
        if (x - sr > bx && y - sr > by && z - sr > bz &&
            x + sr < bx + fblockdx && y + sr < by + fblockdx && z + sr < bz + fblockdx) {
            int id = bd.id(a, b, c);
            if (id >= 0 && act2[id]) bucket[id].push_back(p);
        } else {
            int a0 = ifloor((double)(x - sr) * inv_fb), b0 = ifloor((double)(y - sr) * inv_fb), c0 = ifloor((double)(z - sr) * inv_fb);
            int a1 = ifloor((double)(x + sr) * inv_fb), b1 = ifloor((double)(y + sr) * inv_fb), c1 = ifloor((double)(z + sr) * inv_fb);
            for (int cc = c0; cc <= c1; cc++)
                for (int bb = b0; bb <= b1; bb++)
                    for (int aa = a0; aa <= a1; aa++) {
                        int id = bd.id(aa, bb, cc);
                        if (id >= 0 && act2[id]) bucket[id].push_back(p);
                    }
        }
    }

    // per-block exact band (:618-666), in the block-local float frame
    const double bdx = BW * dx;
    const double inv_dx = 1.0 / dx;
    const double hw = 0.5 * dx;
    float cc_[BW];
    for (int l = 0; l < BW; l++) cc_[l] = (float)((double)(float)l * dx + hw);
#pragma omp parallel for schedule(dynamic, 4)
    for (long long id = 0; id < (long long)nb; id++) {
        if (bucket[id].empty()) continue;
        int a = (int)(id % bd.bi), b = (int)((id / bd.bi) % bd.bj), c = (int)(id / ((size_t)bd.bi * bd.bj));
        float ox = (float)((double)(float)a * bdx), oy = (float)((double)(float)b * bdx), oz = (float)((double)(float)c * bdx);
        float blk[BW * BW * BW];
        for (int t = 0; t < BW * BW * BW; t++) blk[t] = maxd;
        for (int p : bucket[id]) {
            float x = pos[3 * p] - ox, y = pos[3 * p + 1] - oy, z = pos[3 * p + 2] - oz;
            int i0 = std::max(ifloor((double)(x - sr) * inv_dx), 0), i1 = std::min(ifloor((double)(x + sr) * inv_dx), BW - 1);
            int j0 = std::max(ifloor((double)(y - sr) * inv_dx), 0), j1 = std::min(ifloor((double)(y + sr) * inv_dx), BW - 1);
            int k0 = std::max(ifloor((double)(z - sr) * inv_dx), 0), k1 = std::min(ifloor((double)(z + sr) * inv_dx), BW - 1);
            for (int k = k0; k <= k1; k++)
                for (int j = j0; j <= j1; j++)
                    for (int i = i0; i <= i1; i++) {
                        V3 d = v3(cc_[i] - x, cc_[j] - y, cc_[k] - z);
                        float dist = vlength(d) - r;
                        int t = i + BW * (j + BW * k);
                        if (dist < blk[t]) blk[t] = dist;
                    }
        }
        for (int k = 0; k < BW; k++)
            for (int j = 0; j < BW; j++)
                for (int i = 0; i < BW; i++) {
                    int gi = a * BW + i, gj = b * BW + j, gk = c * BW + k;
                    if (gi < ni && gj < nj && gk < nk) phi[flat(gi, gj, gk, ni, nj)] = blk[i + BW * (j + BW * k)];
                }
    }
}

// particlelevelset.cpp:170-194 with meshlevelset.cpp:152-162 (solid phi at cell centre)
void oracle_postprocess_sdf(int ni, int nj, int nk, double dx, const float *solid_phi, float *phi) {
    const float eps = (float)(0.005 * dx);
    const int sw = ni + 1, sh = nj + 1;
    for (int k = 0; k < nk; k++)
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++) {
                float &v = phi[flat(i, j, k, ni, nj)];
                if (v < 0.5 * dx) {
                    const float *s = solid_phi;
                    float sc = 0.125f * (s[flat(i, j, k, sw, sh)] + s[flat(i + 1, j, k, sw, sh)] +
                                         s[flat(i, j + 1, k, sw, sh)] + s[flat(i + 1, j + 1, k, sw, sh)] +
                                         s[flat(i, j, k + 1, sw, sh)] + s[flat(i + 1, j, k + 1, sw, sh)] +
                                         s[flat(i, j + 1, k + 1, sw, sh)] + s[flat(i + 1, j + 1, k + 1, sw, sh)]);
                    if (sc < 0) v = (float)(-0.5f * dx);
                }
                float val = v;
                if (std::fabs(val) < eps) v = val > 0 ? eps : -eps;
            }
}

}  // extern "C"
