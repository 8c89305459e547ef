// Surface tension inputs of the pressure solve:
//   the surface curvature grid, ParticleLevelSet::calculateCurvatureGrid (particlelevelset.cpp:196-291)
//   the cluster status, PressureSolver::_initializeSurfaceTensionClusterData (pressuresolver.cpp:314-605)
//
// Curvature grid.  The nodes with |phi| < 2 dx mark their 6^3 blocks; one layer of face neighbours
// is added (GridUtils::featherGrid6, gridutils.cpp:229-262) and every node of a marked block joins
// the solver band.  LevelSetSolver::reinitializeUpwind (levelsetsolver.cpp:82-138) then updates the
// band Jacobi style from one buffer into the other: its list of solver cells starts with as many
// default (0, 0, 0) entries as there are band nodes (particlelevelset.cpp:250-258), so node
// (0, 0, 0) is updated too, and the nodes outside the band keep the input level set in both
// buffers (the reference's temporary grid there holds a freed copy of the input).  The step length
// and count come from the largest sign of the input; a step is the reference's float arithmetic
// node by node, so the order of the nodes does not matter, and the early stop compares the largest
// change with the previous one (a max-reduction per step, read back by the host).  Nodes outside
// the band become 5 dx; the curvature (ParticleLevelSet::_getCurvature, particlelevelset.cpp:728-800)
// is computed at the interior nodes whose six neighbours lie within 2 dx of the surface and
// extrapolated over three layers with the velocity extrapolation kernels.
//
// Cluster status.  Border cells are "border"; cells of 4^3 blocks that are wholly liquid or
// wholly air are "ok".  The reference then runs a breadth-first search from every surface cell
// over its phase.  Its result does not depend on the search order: a connected same-phase
// component of the remaining cells is bad when it has fewer than 36 cells and touches no
// classified cell of its phase, else ok.  Here the components come from a union-find over the
// cells' same-phase face neighbours (hooking the larger root under the smaller with compare-and-
// swap, path halving on the finds), then a size count and a touch flag per root.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <stdexcept>

#include "common.cuh"
#include "kernels.h"
#include "tension.cuh"

namespace ffgpu {

namespace {
constexpr int CURV_BAND = 3;      // ParticleLevelSet::_curvatureGridExactBand
constexpr int CURV_BLOCK = 2 * CURV_BAND;
constexpr int CLUSTER_BLOCK = 4;  // pressuresolver.cpp:318
constexpr int CLUSTER_MIN = 36;   // _surfaceTensionClusterThreshold
constexpr long long UF_LIMIT = 1 << 24;   // steps of a find or a hook before an index error is raised

// non-negative and negative floats as unsigned integers that compare like the floats
__device__ inline unsigned int ordered_bits(float f) {
    const unsigned int b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
inline float from_ordered(unsigned int u) {
    const unsigned int b = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
    float f;
    std::memcpy(&f, &b, 4);
    return f;
}

// LevelSetSolver::_sign: the distance in double, dx squared in float
__device__ inline float sign_of(float v, float dxf) {
    const double dd = v;
    return (float)(dd / sqrt(dd * dd + (double)(dxf * dxf)));
}

__device__ inline float sq(float x) { return x * x; }
// std::max / std::min: the first argument unless the second is strictly larger / smaller, so the
// sign of a zero is kept as the reference's float code keeps it
__device__ inline float smax(float a, float b) { return (a < b) ? b : a; }
__device__ inline float smin(float a, float b) { return (b < a) ? b : a; }

// marks the 6^3 blocks of nodes near the surface; both buffers start as the input; largest sign
__global__ void k_curv_mark(Dims d, float dxf, float maxsurf, const float *__restrict__ phi, float *a, float *b_,
                            unsigned char *blocks0, int bi, int bj, unsigned int *maxs) {
    unsigned int m = 0;
    const size_t n = d.cells();
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        const float v = phi[t];
        a[t] = v;
        b_[t] = v;
        m = max(m, ordered_bits(sign_of(v, dxf)));
        if (fabsf(v) < maxsurf) {
            const int i = (int)(t % d.ni), j = (int)((t / d.ni) % d.nj), k = (int)(t / ((size_t)d.ni * d.nj));
            blocks0[flat3(i / CURV_BLOCK, j / CURV_BLOCK, k / CURV_BLOCK, bi, bj)] = 1;
        }
    }
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(maxs, m);
}

__global__ void k_feather6(int bi, int bj, int bk, const unsigned char *__restrict__ src, unsigned char *dst) {
    const size_t n = (size_t)bi * bj * bk;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(t % bi), j = (int)((t / bi) % bj), k = (int)(t / ((size_t)bi * bj));
        bool v = src[t];
        v = v || (i > 0 && src[t - 1]) || (i < bi - 1 && src[t + 1]);
        v = v || (j > 0 && src[t - bi]) || (j < bj - 1 && src[t + bi]);
        v = v || (k > 0 && src[t - (size_t)bi * bj]) || (k < bk - 1 && src[t + (size_t)bi * bj]);
        dst[t] = v;
    }
}

__global__ void k_curv_band(Dims d, const unsigned char *__restrict__ blocks, int bi, int bj, unsigned char *valid,
                            unsigned int *count) {
    unsigned int c = 0;
    const size_t n = d.cells();
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(t % d.ni), j = (int)((t / d.ni) % d.nj), k = (int)(t / ((size_t)d.ni * d.nj));
        const unsigned char v = blocks[flat3(i / CURV_BLOCK, j / CURV_BLOCK, k / CURV_BLOCK, bi, bj)];
        valid[t] = v;
        c += v;
    }
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
}

// one upwind step (levelsetsolver.cpp:317-390) of every band node and of node 0 when the band is
// not empty: dst = step(src); the largest |dst - src| of those nodes into *maxdiff (float bits)
__global__ void k_reinit(Dims d, float dxf, float dtau, int with_origin, const unsigned char *__restrict__ valid,
                         const float *__restrict__ src, float *dst, unsigned int *maxdiff) {
    unsigned int m = 0;
    const size_t n = d.cells();
    const float invdx = 1.0f / dxf;
    const int slab = d.ni * d.nj;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        if (!valid[t] && !(t == 0 && with_origin)) continue;
        const int i = (int)(t % d.ni), j = (int)((t / d.ni) % d.nj), k = (int)(t / ((size_t)d.ni * d.nj));
        const float c0 = src[t];
        const float s = sign_of(c0, dxf);
        const float xm = src[t - (i > 0 ? 1 : 0)], xp = src[t + (i < d.ni - 1 ? 1 : 0)];
        const float ym = src[t - (j > 0 ? d.ni : 0)], yp = src[t + (j < d.nj - 1 ? d.ni : 0)];
        const float zm = src[t - (k > 0 ? slab : 0)], zp = src[t + (k < d.nk - 1 ? slab : 0)];
        const float dx0 = invdx * (c0 - xm), dx1 = invdx * (xp - c0);
        const float dy0 = invdx * (c0 - ym), dy1 = invdx * (yp - c0);
        const float dz0 = invdx * (c0 - zm), dz1 = invdx * (zp - c0);
        const float gp = sqrtf(sq(smax(dx0, 0.0f)) + sq(smin(dx1, 0.0f)) + sq(smax(dy0, 0.0f)) + sq(smin(dy1, 0.0f)) +
                               sq(smax(dz0, 0.0f)) + sq(smin(dz1, 0.0f)));
        const float gm = sqrtf(sq(smin(dx0, 0.0f)) + sq(smax(dx1, 0.0f)) + sq(smin(dy0, 0.0f)) + sq(smax(dy1, 0.0f)) +
                               sq(smin(dz0, 0.0f)) + sq(smax(dz1, 0.0f)));
        const float val = c0 - dtau * smax(s, 0.0f) * (gp - 1.0f) - dtau * smin(s, 0.0f) * (gm - 1.0f);
        dst[t] = val;
        m = max(m, __float_as_uint(fabsf(val - c0)));
    }
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(maxdiff, m);
}

// ParticleLevelSet::_getCurvature (particlelevelset.cpp:728-800)
__device__ inline float curvature_at(const float *__restrict__ p, Dims d, double dx, int i, int j, int k) {
    const size_t c = flat3(i, j, k, d.ni, d.nj);
    const size_t sx = 1, sy = (size_t)d.ni, sz = (size_t)d.ni * d.nj;
    const float x = 0.5f * (p[c + sx] - p[c - sx]);
    const float y = 0.5f * (p[c + sy] - p[c - sy]);
    const float z = 0.5f * (p[c + sz] - p[c - sz]);
    const float xx = p[c + sx] - 2.0f * p[c] + p[c - sx];
    const float yy = p[c + sy] - 2.0f * p[c] + p[c - sy];
    const float zz = p[c + sz] - 2.0f * p[c] + p[c - sz];
    const float xy = 0.25f * (p[c + sx + sy] - p[c - sx + sy] - p[c + sx - sy] + p[c - sx - sy]);
    const float xz = 0.25f * (p[c + sx + sz] - p[c - sx + sz] - p[c + sx - sz] + p[c - sx - sz]);
    const float yz = 0.25f * (p[c + sy + sz] - p[c - sy + sz] - p[c + sy - sz] + p[c - sy - sz]);
    float den = x * x + y * y + z * z;
    den = (float)sqrt((double)(den * den * den));   // the reference's unqualified sqrt of a float: double
    if (den < 1e-9f) return 0.0f;
    float curv = (float)(((xx * (y * y + z * z) + yy * (x * x + z * z) + zz * (x * x + y * y) - 2 * xy * x * y -
                           2 * xz * x * z - 2 * yz * y * z) / den) / dx);
    curv = smin(curv, 1.0f / (float)dx);
    curv = smax(curv, -1.0f / (float)dx);
    return curv;
}

// band nodes keep the re-initialised value, the others 5 dx (surface level set)
__global__ void k_curv_finish(Dims d, float oor, const unsigned char *__restrict__ valid, const float *__restrict__ res,
                              float *surface) {
    const size_t n = d.cells();
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
        surface[t] = valid[t] ? res[t] : oor;
}

// _getValidCurvatureNodes (particlelevelset.cpp:692-726) and the curvature there, 0 elsewhere
__global__ void k_curv_nodes(Dims d, double dx, float ub, const float *__restrict__ surface, unsigned char *vn,
                             float *kgrid) {
    const size_t n = d.cells();
    const size_t sy = (size_t)d.ni, sz = (size_t)d.ni * d.nj;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(t % d.ni), j = (int)((t / d.ni) % d.nj), k = (int)(t / ((size_t)d.ni * d.nj));
        bool ok = i > 0 && j > 0 && k > 0 && i < d.ni - 1 && j < d.nj - 1 && k < d.nk - 1;
        ok = ok && fabsf(surface[t]) < ub && fabsf(surface[t + 1]) < ub && fabsf(surface[t - 1]) < ub &&
             fabsf(surface[t + sy]) < ub && fabsf(surface[t - sy]) < ub && fabsf(surface[t + sz]) < ub &&
             fabsf(surface[t - sz]) < ub;
        vn[t] = ok ? 1 : 0;
        kgrid[t] = ok ? curvature_at(surface, d, dx, i, j, k) : 0.0f;
    }
}

// ---- cluster status ----

__device__ inline bool border_cell(Dims d, int i, int j, int k) {
    return i == 0 || j == 0 || k == 0 || i == d.ni - 1 || j == d.nj - 1 || k == d.nk - 1;
}

// block phase bits: 1 some liquid cell, 2 some air cell (full 4^3 blocks only)
__global__ void k_cluster_blocks(Dims d, const float *__restrict__ phi, unsigned int *blocks, int bi, int bj, int bk) {
    const size_t n = d.cells();
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(t % d.ni), j = (int)((t / d.ni) % d.nj), k = (int)(t / ((size_t)d.ni * d.nj));
        const int a = i / CLUSTER_BLOCK, b_ = j / CLUSTER_BLOCK, c = k / CLUSTER_BLOCK;
        if (a >= bi || b_ >= bj || c >= bk) continue;
        const unsigned int bit = phi[t] < 0.0f ? 1u : 2u;
        unsigned int *p = blocks + flat3(a, b_, c, bi, bj);
        if (!(*p & bit)) atomicOr(p, bit);
    }
}

// initial status (border, ok from pure blocks, unset) and union-find parents of the unset cells
__global__ void k_cluster_init(Dims d, const unsigned int *__restrict__ blocks, int bi, int bj, int bk,
                               unsigned char *status, int *parent, int *count, unsigned char *touch) {
    const size_t n = d.cells();
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(t % d.ni), j = (int)((t / d.ni) % d.nj), k = (int)(t / ((size_t)d.ni * d.nj));
        unsigned char s = CS_UNSET;
        if (border_cell(d, i, j, k)) {
            s = CS_BORDER;
        } else {
            const int a = i / CLUSTER_BLOCK, b_ = j / CLUSTER_BLOCK, c = k / CLUSTER_BLOCK;
            if (a < bi && b_ < bj && c < bk) {
                const unsigned int bs = blocks[flat3(a, b_, c, bi, bj)];
                if (bs == 1) s = CS_OK_IN;
                else if (bs == 2) s = CS_OK_OUT;
            }
        }
        status[t] = s;
        parent[t] = (int)t;
        count[t] = 0;
        touch[t] = 0;
    }
}

__device__ inline int uf_find(int *parent, int x, unsigned int *error) {
    int p = parent[x];
    long long it = 0;
    while (p != x) {
        const int gp = parent[p];
        if (gp < p) parent[x] = gp;   // path halving (benign races: every value written is an ancestor)
        x = p;
        p = gp;
        if (++it > UF_LIMIT) { atomicOr(error, (unsigned int)ERR_INDEX); return x; }
    }
    return x;
}

// joins every unset cell with its unset same-phase +x, +y, +z neighbours
__global__ void k_cluster_union(Dims d, const float *__restrict__ phi, const unsigned char *__restrict__ status,
                                int *parent, unsigned int *error) {
    const size_t n = d.cells();
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        if (status[t] != CS_UNSET) continue;
        const int i = (int)(t % d.ni), j = (int)((t / d.ni) % d.nj), k = (int)(t / ((size_t)d.ni * d.nj));
        const bool fl = phi[t] < 0.0f;
        const size_t nb[3] = {i + 1 < d.ni ? t + 1 : t, j + 1 < d.nj ? t + d.ni : t,
                              k + 1 < d.nk ? t + (size_t)d.ni * d.nj : t};
        for (int q = 0; q < 3; q++) {
            const size_t u = nb[q];
            if (u == t || status[u] != CS_UNSET || (phi[u] < 0.0f) != fl) continue;
            int a = uf_find(parent, (int)t, error), b_ = uf_find(parent, (int)u, error);
            long long it = 0;
            while (a != b_) {   // hook the larger root under the smaller
                if (a < b_) { const int sw = a; a = b_; b_ = sw; }
                const int old = atomicCAS(&parent[a], a, b_);
                if (old == a) break;
                a = uf_find(parent, old, error);
                if (++it > UF_LIMIT) { atomicOr(error, (unsigned int)ERR_INDEX); break; }
            }
        }
    }
}

// roots of the unset cells, component sizes and touch flags
__global__ void k_cluster_measure(Dims d, const float *__restrict__ phi, const unsigned char *__restrict__ status,
                                  int *parent, int *count, unsigned char *touch, unsigned int *error) {
    const size_t n = d.cells();
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        if (status[t] != CS_UNSET) continue;
        const int r = uf_find(parent, (int)t, error);
        atomicAdd(&count[r], 1);
        const int i = (int)(t % d.ni), j = (int)((t / d.ni) % d.nj), k = (int)(t / ((size_t)d.ni * d.nj));
        const bool fl = phi[t] < 0.0f;
        const int ni_[6] = {i + 1, i - 1, i, i, i, i}, nj_[6] = {j, j, j + 1, j - 1, j, j}, nk_[6] = {k, k, k, k, k + 1, k - 1};
        for (int q = 0; q < 6; q++) {
            if (ni_[q] < 0 || nj_[q] < 0 || nk_[q] < 0 || ni_[q] >= d.ni || nj_[q] >= d.nj || nk_[q] >= d.nk) continue;
            const size_t u = flat3(ni_[q], nj_[q], nk_[q], d.ni, d.nj);
            const unsigned char su = status[u];
            if (su != CS_UNSET && su != CS_BORDER && (phi[u] < 0.0f) == fl) touch[r] = 1;
        }
    }
}

__global__ void k_cluster_final(Dims d, const float *__restrict__ phi, unsigned char *status, int *parent,
                                const int *__restrict__ count, const unsigned char *__restrict__ touch,
                                unsigned int *error) {
    const size_t n = d.cells();
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        if (status[t] != CS_UNSET) continue;
        const int r = uf_find(parent, (int)t, error);
        const bool fl = phi[t] < 0.0f;
        const bool bad = count[r] < CLUSTER_MIN && !touch[r];
        status[t] = bad ? (fl ? CS_BAD_IN : CS_BAD_OUT) : (fl ? CS_OK_IN : CS_OK_OUT);
    }
}
}  // namespace

int launch_curvature_grid(Dims d, double dx, const float *phi, float *surface_phi, float *curvature, TensionWork w,
                          cudaStream_t st) {
    const size_t n = d.cells();
    const float dxf = (float)dx;
    const float maxsurf = (float)(2.0f * dx);
    const int bi = (d.ni + CURV_BLOCK - 1) / CURV_BLOCK, bj = (d.nj + CURV_BLOCK - 1) / CURV_BLOCK,
              bk = (d.nk + CURV_BLOCK - 1) / CURV_BLOCK;
    const size_t nb = (size_t)bi * bj * bk;
    int launches = 0;
    FFGPU_CUDA(cudaMemsetAsync(w.blocks0, 0, nb, st));
    FFGPU_CUDA(cudaMemsetAsync(w.scal, 0, 4 * sizeof(unsigned int), st));
    float *a = surface_phi, *b_ = w.buf;   // the two re-initialisation buffers
    k_curv_mark<<<grid_for(n, 256), 256, 0, st>>>(d, dxf, maxsurf, phi, a, b_, w.blocks0, bi, bj, w.scal);
    k_feather6<<<grid_for(nb, 256), 256, 0, st>>>(bi, bj, bk, w.blocks0, w.blocks1);
    k_curv_band<<<grid_for(n, 256), 256, 0, st>>>(d, w.blocks1, bi, bj, w.valid, w.scal + 1);
    launches += 3;
    FFGPU_CUDA(cudaMemcpyAsync(w.host, w.scal, 2 * sizeof(unsigned int), cudaMemcpyDeviceToHost, st));
    FFGPU_CUDA(cudaStreamSynchronize(st));
    const float maxS = from_ordered((unsigned int)w.host[0]);
    const unsigned int nvalid = (unsigned int)w.host[1];
    // LevelSetSolver::reinitializeUpwind step length and count (levelsetsolver.cpp:82-95)
    const float max_cfl = 0.5f;
    float dtau = max_cfl * dxf;
    while (dtau * maxS / dxf > max_cfl) dtau *= 0.5;
    const float maxdist = (float)(CURV_BAND * dx);
    const int iters = (int)std::ceil(maxdist / dtau);
    float last = -1.0f;
    for (int it = 0; it < iters; it++) {
        FFGPU_CUDA(cudaMemsetAsync(w.scal + 2, 0, sizeof(unsigned int), st));
        k_reinit<<<grid_for(n, 256), 256, 0, st>>>(d, dxf, dtau, nvalid > 0 ? 1 : 0, w.valid, a, b_, w.scal + 2);
        launches++;
        FFGPU_CUDA(cudaMemcpyAsync(w.host + 2, w.scal + 2, sizeof(unsigned int), cudaMemcpyDeviceToHost, st));
        FFGPU_CUDA(cudaStreamSynchronize(st));
        float maxdiff;
        std::memcpy(&maxdiff, &w.host[2], 4);
        std::swap(a, b_);
        if (std::fabs(maxdiff - last) < 0.01f * dxf) break;
        last = maxdiff;
    }
    // a holds the result; the surface level set goes into surface_phi (one of the buffers)
    const float oor = (float)(5.0f * dx);   // _outOfRangeDistance * dx
    k_curv_finish<<<grid_for(n, 256), 256, 0, st>>>(d, oor, w.valid, a, a == surface_phi ? surface_phi : w.buf);
    if (a != surface_phi)
        FFGPU_CUDA(cudaMemcpyAsync(surface_phi, w.buf, n * sizeof(float), cudaMemcpyDeviceToDevice, st));
    const float ub = (float)((CURV_BAND - 1) * dx);
    k_curv_nodes<<<grid_for(n, 256), 256, 0, st>>>(d, dx, ub, surface_phi, w.vn, curvature);
    launch_extrapolate(d.ni, d.nj, d.nk, curvature, w.vn, 3, w.xst1, w.xst2, st);   // _curvatureGridExtrapolationLayers
    FFGPU_CUDA(cudaGetLastError());
    return launches + 3;
}

int launch_cluster_status(Dims d, const float *phi, unsigned char *status, TensionWork w, cudaStream_t st) {
    const size_t n = d.cells();
    const int bi = d.ni / CLUSTER_BLOCK, bj = d.nj / CLUSTER_BLOCK, bk = d.nk / CLUSTER_BLOCK;
    const size_t nb = (size_t)bi * bj * bk;
    if (nb) FFGPU_CUDA(cudaMemsetAsync(w.cblocks, 0, nb * sizeof(unsigned int), st));
    FFGPU_CUDA(cudaMemsetAsync(w.scal + 3, 0, sizeof(unsigned int), st));
    if (nb) k_cluster_blocks<<<grid_for(n, 256), 256, 0, st>>>(d, phi, w.cblocks, bi, bj, bk);
    k_cluster_init<<<grid_for(n, 256), 256, 0, st>>>(d, w.cblocks, bi, bj, bk, status, w.parent, w.count, w.touch);
    k_cluster_union<<<grid_for(n, 256), 256, 0, st>>>(d, phi, status, w.parent, w.scal + 3);
    k_cluster_measure<<<grid_for(n, 256), 256, 0, st>>>(d, phi, status, w.parent, w.count, w.touch, w.scal + 3);
    k_cluster_final<<<grid_for(n, 256), 256, 0, st>>>(d, phi, status, w.parent, w.count, w.touch, w.scal + 3);
    FFGPU_CUDA(cudaMemcpyAsync(w.host + 3, w.scal + 3, sizeof(unsigned int), cudaMemcpyDeviceToHost, st));
    FFGPU_CUDA(cudaStreamSynchronize(st));
    if (w.host[3]) throw std::runtime_error("Error: cluster status search exceeded its step limit.\n");
    return 5;
}

}  // namespace ffgpu
