// Surface tension term of the pressure solve (pressuresolver.cpp:659-749, :1047-1205): the
// device-side pieces shared by the system build and the pressure application.
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"
#include "kernels.h"

namespace ffgpu {

// cluster status of a cell (pressuresolver.cpp:314-605): ok / bad inside or outside the liquid
enum ClusterStatus : unsigned char {
    CS_UNSET = 0x00, CS_OK_IN = 0x01, CS_OK_OUT = 0x02, CS_BAD_IN = 0x04, CS_BAD_OUT = 0x08, CS_BORDER = 0x10
};

// What the build and the application need to add the surface tension term; on == 0: no term.
struct TensionDev {
    const float *phi;              // post-processed liquid level set (cell centres)
    const float *curv;             // surface curvature grid (cell centres)
    const unsigned char *status;   // cluster status per cell
    double k;                      // surface tension constant
    int on;
};

// Interpolation::trilinearInterpolate of a cell-centred grid at p - dx/2 (interpolation.cpp:61-112),
// in double with the reference's corner order; cells outside the grid read 0
__device__ inline double sample_centred(const float *g, Dims d, double dx, float px, float py, float pz) {
    const float sh = (float)(0.5 * dx);
    const float x = px - sh, y = py - sh, z = pz - sh;
    const double inv = 1.0 / dx;
    const int i = (int)floor((double)x * inv), j = (int)floor((double)y * inv), k = (int)floor((double)z * inv);
    const float gx = (float)((double)(float)i * dx), gy = (float)((double)(float)j * dx), gz = (float)((double)(float)k * dx);
    const double ix = (double)(x - gx) * inv, iy = (double)(y - gy) * inv, iz = (double)(z - gz) * inv;
    auto G = [&](int a, int b, int c) -> double {
        return (a >= 0 && b >= 0 && c >= 0 && a < d.ni && b < d.nj && c < d.nk) ? (double)g[flat3(a, b, c, d.ni, d.nj)]
                                                                               : 0.0;
    };
    const double p0 = G(i, j, k), p1 = G(i + 1, j, k), p2 = G(i, j + 1, k), p3 = G(i, j, k + 1), p4 = G(i + 1, j, k + 1),
                 p5 = G(i, j + 1, k + 1), p6 = G(i + 1, j + 1, k), p7 = G(i + 1, j + 1, k + 1);
    return p0 * (1 - ix) * (1 - iy) * (1 - iz) + p1 * ix * (1 - iy) * (1 - iz) + p2 * (1 - ix) * iy * (1 - iz) +
           p3 * (1 - ix) * (1 - iy) * iz + p4 * ix * (1 - iy) * iz + p5 * (1 - ix) * iy * iz + p6 * ix * iy * (1 - iz) +
           p7 * ix * iy * iz;
}

// PressureSolver::_getSurfaceTensionTerm(g1, g2) (pressuresolver.cpp:715-749): k times the curvature
// at the interface point between the two cell centres, 0 when either cell lies in a bad cluster
// or both are on the same side of the surface.  The argument order matters for the rounding.
__device__ inline double tension_term(const TensionDev &t, Dims d, double dx, int i1, int j1, int k1, int i2, int j2,
                                      int k2) {
    const size_t c1 = flat3(i1, j1, k1, d.ni, d.nj), c2 = flat3(i2, j2, k2, d.ni, d.nj);
    const unsigned char s = t.status[c1] | t.status[c2];
    if ((s & CS_BAD_IN) || (s & CS_BAD_OUT)) return 0.0;
    const double hw = 0.5 * dx;   // GridIndexToCellCenter (grid3d.h:86-103): double, then float
    const float p1x = (float)((double)i1 * dx + hw), p1y = (float)((double)j1 * dx + hw), p1z = (float)((double)k1 * dx + hw);
    const float p2x = (float)((double)i2 * dx + hw), p2y = (float)((double)j2 * dx + hw), p2z = (float)((double)k2 * dx + hw);
    const float phi1 = t.phi[c1], phi2 = t.phi[c2];
    if ((phi1 < 0.0f && phi2 < 0.0f) || (phi1 >= 0.0f && phi2 >= 0.0f)) return 0.0;
    float px, py, pz;
    if (fabsf(phi2 - phi1) < 1e-6f) {
        px = p1x + 0.5f * (p2x - p1x); py = p1y + 0.5f * (p2y - p1y); pz = p1z + 0.5f * (p2z - p1z);
    } else {
        const float th = phi1 / (phi1 - phi2);
        px = p1x + th * (p2x - p1x); py = p1y + th * (p2y - p1y); pz = p1z + th * (p2z - p1z);
    }
    return t.k * sample_centred(t.curv, d, dx, px, py, pz);
}

}  // namespace ffgpu
