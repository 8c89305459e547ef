// FP32 trilinear MAC velocity sampling (macvelocityfield.cpp:519-645 semantics, FP32
// arithmetic: cell fractions formed with one fused x - i*dx) and its Jacobian, shared by the
// G2P / RK3 kernels and their adjoints.
#pragma once
#include <cmath>
#include <limits>

#include "common.cuh"
#include "kernels.h"

namespace ffgpu {

struct MacDev {
    Dims d;
    float dx, inv, hdx;
    double ddx;
    float xmax, ymax, zmax;   // smallest floats >= ni dx, nj dx, nk dx (exact domain test)
    MacView f;
};

// Smallest float >= b: for a float x, (double)x < b exactly when x < float_at_least(b).
inline float float_at_least(double b) {
    float f = (float)b;
    if ((double)f < b) f = std::nextafter(f, std::numeric_limits<float>::infinity());
    return f;
}

inline MacDev make_mac(Dims d, double dx, MacView v) {
    MacDev m;
    m.d = d; m.dx = (float)dx; m.inv = (float)(1.0 / dx); m.hdx = (float)(0.5 * dx); m.ddx = dx; m.f = v;
    m.xmax = float_at_least(dx * d.ni); m.ymax = float_at_least(dx * d.nj); m.zmax = float_at_least(dx * d.nk);
    return m;
}

__device__ inline float corner(const float *g, int gw, int gh, int gd, int i, int j, int k) {
    return (i >= 0 && j >= 0 && k >= 0 && i < gw && j < gh && k < gd) ? __ldg(g + flat3(i, j, k, gw, gh)) : 0.0f;
}

// The 8 corner values of one component around a point and the point's cell fractions.
struct MacCell {
    float c000, c100, c010, c110, c001, c101, c011, c111, ix, iy, iz;
};

__device__ inline MacCell mac_cell(const MacDev &m, int comp, float x, float y, float z) {
    const float *g = comp == 0 ? m.f.u : (comp == 1 ? m.f.v : m.f.w);
    int gw = m.d.ni + (comp == 0), gh = m.d.nj + (comp == 1), gd = m.d.nk + (comp == 2);
    if (comp != 0) x = x - m.hdx;
    if (comp != 1) y = y - m.hdx;
    if (comp != 2) z = z - m.hdx;
    int i = (int)floorf(x * m.inv), j = (int)floorf(y * m.inv), k = (int)floorf(z * m.inv);
    MacCell c;
    c.ix = fmaf(-(float)i, m.dx, x) * m.inv;
    c.iy = fmaf(-(float)j, m.dx, y) * m.inv;
    c.iz = fmaf(-(float)k, m.dx, z) * m.inv;
    c.c000 = corner(g, gw, gh, gd, i, j, k); c.c100 = corner(g, gw, gh, gd, i + 1, j, k);
    c.c010 = corner(g, gw, gh, gd, i, j + 1, k); c.c110 = corner(g, gw, gh, gd, i + 1, j + 1, k);
    c.c001 = corner(g, gw, gh, gd, i, j, k + 1); c.c101 = corner(g, gw, gh, gd, i + 1, j, k + 1);
    c.c011 = corner(g, gw, gh, gd, i, j + 1, k + 1); c.c111 = corner(g, gw, gh, gd, i + 1, j + 1, k + 1);
    return c;
}

__device__ inline float sample_comp(const MacDev &m, int comp, float x, float y, float z) {
    const MacCell c = mac_cell(m, comp, x, y, z);
    float a00 = c.c000 + c.ix * (c.c100 - c.c000), a10 = c.c010 + c.ix * (c.c110 - c.c010);
    float a01 = c.c001 + c.ix * (c.c101 - c.c001), a11 = c.c011 + c.ix * (c.c111 - c.c011);
    float b0 = a00 + c.iy * (a10 - a00), b1 = a01 + c.iy * (a11 - a01);
    return b0 + c.iz * (b1 - b0);
}

// Gradient of the sampled component with respect to the sample point (piecewise: the
// derivative of the trilinear interpolant inside the point's cell).
__device__ inline void sample_comp_grad(const MacDev &m, int comp, float x, float y, float z, float &gx, float &gy,
                                        float &gz) {
    const MacCell c = mac_cell(m, comp, x, y, z);
    const float uy = 1.0f - c.iy, uz = 1.0f - c.iz;
    float a00 = c.c000 + c.ix * (c.c100 - c.c000), a10 = c.c010 + c.ix * (c.c110 - c.c010);
    float a01 = c.c001 + c.ix * (c.c101 - c.c001), a11 = c.c011 + c.ix * (c.c111 - c.c011);
    float b0 = a00 + c.iy * (a10 - a00), b1 = a01 + c.iy * (a11 - a01);
    float dix = uy * uz * (c.c100 - c.c000) + c.iy * uz * (c.c110 - c.c010) + uy * c.iz * (c.c101 - c.c001) +
                c.iy * c.iz * (c.c111 - c.c011);
    float diy = uz * (a10 - a00) + c.iz * (a11 - a01);
    float diz = b1 - b0;
    gx = dix * m.inv; gy = diy * m.inv; gz = diz * m.inv;
}

// isPositionInGrid (grid3d.h:134-136): 0 <= x < n dx with the bound in double, evaluated
// exactly in float through the precomputed float bounds
__device__ inline bool mac_inside(const MacDev &m, float x, float y, float z) {
    return x >= 0.0f && y >= 0.0f && z >= 0.0f && x < m.xmax && y < m.ymax && z < m.zmax;
}

__device__ inline void sample_mac(const MacDev &m, float x, float y, float z, float &ox, float &oy, float &oz) {
    if (!mac_inside(m, x, y, z)) {
        ox = oy = oz = 0.0f;
        return;
    }
    ox = sample_comp(m, 0, x, y, z);
    oy = sample_comp(m, 1, x, y, z);
    oz = sample_comp(m, 2, x, y, z);
}

// J(p)^T g for the sampled velocity u(p): (sum_c g_c du_c/dx, .../dy, .../dz); zero outside the grid.
__device__ inline void sample_mac_jt(const MacDev &m, float x, float y, float z, float gu, float gv, float gw,
                                     float &jx, float &jy, float &jz) {
    jx = jy = jz = 0.0f;
    if (!mac_inside(m, x, y, z)) return;
    const float g[3] = {gu, gv, gw};
#pragma unroll
    for (int c = 0; c < 3; c++) {
        float ax, ay, az;
        sample_comp_grad(m, c, x, y, z, ax, ay, az);
        jx += g[c] * ax; jy += g[c] * ay; jz += g[c] * az;
    }
}

}  // namespace ffgpu
