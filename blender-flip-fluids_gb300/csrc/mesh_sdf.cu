// Solid level set of static triangle-mesh obstacles (see mesh_sdf.h for the reference mapping).
//
// A "part" is one MeshLevelSet of the reference: a box of nodes of the domain grid (its origin
// node g and its cells ni x nj x nk), the triangles it is computed from and its upper bound
// (ni + nj + nk + 3) dx.  For each part:
//   1. every node starts at the upper bound;
//   2. k_band: one CTA per triangle walks the triangle's node box and lowers each node to its
//      exact distance (atomicMin on the float bits: all values are non-negative).  The block form
//      (meshlevelset.cpp:878-918, 1115-1163) takes the box from the triangle's float bounding box
//      and measures in the coordinates of the node's 10^3 block; the island form (:1165-1234)
//      takes it from the vertices' truncated grid coordinates and measures in part coordinates;
//   3. inside tests (meshutils.cpp:57-245, 356-437): the mesh, shifted by half a cell and moved to
//      the cell grid of its bounding box, is crossed by +z lines through the cell centres (offset
//      by the jitter); k_cross_count / k_cross_fill record each column's crossing heights and
//      k_inside marks the nodes with an odd number of crossings below them, in columns with an
//      even total.  A mesh that leaves the part's box is split into its islands first (those
//      inside are tested together, each crossing one alone; meshutils.cpp:382-462);
//   4. k_finish negates the marked nodes and unites the part into its target (min), or for the
//      domain box writes the negated level set.
// Distances and crossings use the reference's float/double mix operation by operation; the
// library is built without contraction, so the results are those of the reference's x86-64 build.
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "kernels.h"
#include "mesh_sdf.h"

namespace ffgpu {
namespace {

constexpr int EXACT_BAND = 3;         // FluidSimulation::_solidLevelSetExactBand (fluidsimulation.h:2235)
constexpr int BLOCK_WIDTH = 10;       // MeshLevelSet::_blockwidth (meshlevelset.h:369)
constexpr int ISLAND_TRIGGER = 25;    // MeshObject::_numIslandsForFractureOptimizationTrigger (meshobject.h:222)

struct F3 { float x, y, z; };
__host__ __device__ inline F3 f3(float x, float y, float z) { F3 r; r.x = x; r.y = y; r.z = z; return r; }
__host__ __device__ inline F3 fd3(double x, double y, double z) { return f3((float)x, (float)y, (float)z); }
__host__ __device__ inline F3 operator+(F3 a, F3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ inline F3 operator-(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ inline F3 operator*(float s, F3 a) { return f3(s * a.x, s * a.y, s * a.z); }
__host__ __device__ inline F3 neg(F3 a) { return f3(-a.x, -a.y, -a.z); }
__host__ __device__ inline float dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ inline F3 cross(F3 a, F3 b) {
    return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__host__ __device__ inline float len(F3 a) { return sqrtf(a.x * a.x + a.y * a.y + a.z * a.z); }
// vmath's vector / float: multiply by the float of the double reciprocal (vmath.cpp:100-103)
__host__ __device__ inline F3 divf(F3 a, float s) { const float r = (float)(1.0 / s); return f3(a.x * r, a.y * r, a.z * r); }

// Grid3d::GridIndexToPosition / GridIndexToCellCenter (grid3d.h:76-108)
__host__ __device__ inline F3 node_at(int i, int j, int k, double h) { return fd3((float)i * h, (float)j * h, (float)k * h); }
__host__ __device__ inline F3 centre_at(int i, int j, int k, double h) {
    const double hw = 0.5 * h;
    return fd3((float)i * h + hw, (float)j * h + hw, (float)k * h + hw);
}
__host__ __device__ inline int floor_index(float p, double inv) { return (int)floor(p * inv); }
__host__ __device__ inline double clamp01d(double v) { return v < 0.0 ? 0.0 : (v > 1.0 ? 1.0 : v); }

// bounding box of a triangle with the reference's float corner and double extents (aabb.cpp:84-112)
struct Box3 {
    F3 lo;
    double w, h, d;
    __host__ __device__ F3 hi() const { return lo + fd3(w, h, d); }
};
__host__ __device__ inline Box3 tri_box(F3 a, F3 b, F3 c) {
    double mn[3] = {a.x, a.y, a.z}, mx[3] = {a.x, a.y, a.z};
    const F3 p[3] = {a, b, c};
    for (int q = 0; q < 3; q++) {
        mn[0] = fmin((double)p[q].x, mn[0]); mn[1] = fmin((double)p[q].y, mn[1]); mn[2] = fmin((double)p[q].z, mn[2]);
        mx[0] = fmax((double)p[q].x, mx[0]); mx[1] = fmax((double)p[q].y, mx[1]); mx[2] = fmax((double)p[q].z, mx[2]);
    }
    Box3 r;
    r.lo = fd3(mn[0], mn[1], mn[2]);
    r.w = mx[0] - mn[0] + 1e-9; r.h = mx[1] - mn[1] + 1e-9; r.d = mx[2] - mn[2] + 1e-9;
    return r;
}

// Collision::findClosestPointOnTriangle (collision.cpp:161-270): float dot products, the
// barycentric parameters in double, the point assembled in float
__device__ F3 closest_point(F3 p0, F3 v0, F3 v1, F3 v2) {
    const F3 e0 = v1 - v0, e1 = v2 - v0, pv = v0 - p0;
    const double a = dot(e0, e0), b = dot(e0, e1), c = dot(e1, e1), d = dot(e0, pv), e = dot(e1, pv);
    const double det = a * c - b * b;
    if (fabs(det) < 1e-9) {
        const float feps = 1e-6f;
        const float l1 = len(v0 - v1), l2 = len(v1 - v2), l3 = len(v2 - v0);
        if (l1 < feps && l2 < feps && l3 < feps) return v0;
        F3 s0, s1;
        if (l1 < feps) { s0 = v0; s1 = v2; }
        else if (l2 < feps) { s0 = v1; s1 = v0; }
        else { s0 = v2; s1 = v1; }
        const float num = dot(p0 - s0, s1 - s0), den = dot(s1 - s0, s1 - s0);
        if (fabsf(den) < feps) return v0;
        const float lam = num / den;
        if (lam <= 0.0f) return s0;
        if (lam >= 1.0f) return s1;
        return s0 + lam * (s1 - s0);
    }
    double s = b * e - c * d, t = b * d - a * e;
    if (s + t < det) {
        if (s < 0.0) {
            if (t < 0.0) {
                if (d < 0.0) { s = clamp01d(-d / a); t = 0.0; }
                else { s = 0.0; t = clamp01d(-e / c); }
            } else {
                s = 0.0; t = clamp01d(-e / c);
            }
        } else if (t < 0.0) {
            s = clamp01d(-d / a); t = 0.0;
        } else {
            const double r = 1.0 / det;
            s *= r; t *= r;
        }
    } else if (s < 0.0) {
        const double u0 = b + d, u1 = c + e;
        if (u1 > u0) { s = clamp01d((u1 - u0) / (a - 2 * b + c)); t = 1 - s; }
        else { t = clamp01d(-e / c); s = 0.0; }
    } else if (t < 0.0) {
        if (a + d > b + e) { s = clamp01d((c + e - b - d) / (a - 2 * b + c)); t = 1 - s; }
        else { s = clamp01d(-e / c); t = 0.0; }
    } else {
        s = clamp01d((c + e - b - d) / (a - 2 * b + c)); t = 1.0 - s;
    }
    return (v0 + (float)s * e0) + (float)t * e1;
}

// Collision::lineIntersectsTriangle (collision.cpp:79-114) for the +z line through o
__device__ bool crosses(F3 o, F3 v0, F3 v1, F3 v2, float &z) {
    const F3 dir = f3(0.0f, 0.0f, 1.0f);
    const F3 e1 = v1 - v0, e2 = v2 - v0;
    const F3 h = cross(dir, e2);
    const float a = dot(e1, h);
    if (fabs((double)a) < 10e-9) return false;
    const float f = 1 / a;
    const F3 s = o - v0;
    const float u = f * dot(s, h);
    if (u < 0.0 || u > 1.0) return false;
    const F3 q = cross(s, e1);
    const float v = f * dot(dir, q);
    if (v < 0.0 || u + v > 1.0) return false;
    const double t = f * dot(e2, q);
    z = (o + (float)t * dir).z;
    return true;
}

__device__ inline F3 vert(const float *v, int i) { return f3(v[3 * i], v[3 * i + 1], v[3 * i + 2]); }

struct BandArgs {
    const float *v;   // absolute vertex coordinates
    const int *t;
    int nt;
    int ni, nj, nk;   // part cells
    F3 off;           // part origin (position of its first node)
    double dx;
    int serial;       // 1: island form, 0: block form
};

__global__ void k_band(BandArgs P, float *phi) {
    const double inv = 1.0 / P.dx;
    const int W = P.ni + 1, H = P.nj + 1;
    for (int tri = blockIdx.x; tri < P.nt; tri += gridDim.x) {
        const F3 a = vert(P.v, P.t[3 * tri]), b = vert(P.v, P.t[3 * tri + 1]), c = vert(P.v, P.t[3 * tri + 2]);
        const F3 p = a - P.off, q = b - P.off, r = c - P.off;
        int lo[3], hi[3];
        const int top[3] = {P.ni, P.nj, P.nk};
        if (!P.serial) {   // meshlevelset.cpp:878-918
            Box3 bb = tri_box(a, b, c);
            bb.lo = bb.lo - P.off;
            const F3 mx = bb.hi();
            lo[0] = floor_index(bb.lo.x, inv) - EXACT_BAND; lo[1] = floor_index(bb.lo.y, inv) - EXACT_BAND;
            lo[2] = floor_index(bb.lo.z, inv) - EXACT_BAND;
            hi[0] = floor_index(mx.x, inv) + EXACT_BAND + 1; hi[1] = floor_index(mx.y, inv) + EXACT_BAND + 1;
            hi[2] = floor_index(mx.z, inv) + EXACT_BAND + 1;
            bool out = false;
            for (int e = 0; e < 3; e++) out = out || hi[e] < 0 || lo[e] >= top[e] + 1;
            if (out) continue;
            for (int e = 0; e < 3; e++) { lo[e] = max(lo[e], 0); hi[e] = min(hi[e], top[e]); }
        } else {           // meshlevelset.cpp:1180-1198: truncated grid coordinates
            const double fp[3] = {(double)p.x * inv, (double)p.y * inv, (double)p.z * inv};
            const double fq[3] = {(double)q.x * inv, (double)q.y * inv, (double)q.z * inv};
            const double fr[3] = {(double)r.x * inv, (double)r.y * inv, (double)r.z * inv};
            for (int e = 0; e < 3; e++) {
                const int l = int(fmin(fp[e], fmin(fq[e], fr[e]))) - EXACT_BAND;
                const int h = int(fmax(fp[e], fmax(fq[e], fr[e]))) + EXACT_BAND + 1;
                lo[e] = l < 0 ? 0 : (l > top[e] ? top[e] : l);
                hi[e] = h < 0 ? 0 : (h > top[e] ? top[e] : h);
            }
        }
        const long long ex = hi[0] - lo[0] + 1, ey = hi[1] - lo[1] + 1, ez = hi[2] - lo[2] + 1;
        if (ex <= 0 || ey <= 0 || ez <= 0) continue;
        const long long vol = ex * ey * ez;
        for (long long s = threadIdx.x; s < vol; s += blockDim.x) {
            const int i = lo[0] + (int)(s % ex), j = lo[1] + (int)((s / ex) % ey), k = lo[2] + (int)(s / (ex * ey));
            float dist;
            if (!P.serial) {
                const int bi = i / BLOCK_WIDTH, bj = j / BLOCK_WIDTH, bk = k / BLOCK_WIDTH;
                const F3 bo = node_at(bi, bj, bk, BLOCK_WIDTH * P.dx);
                const F3 x = node_at(i - BLOCK_WIDTH * bi, j - BLOCK_WIDTH * bj, k - BLOCK_WIDTH * bk, P.dx);
                dist = len(closest_point(x, p - bo, q - bo, r - bo) - x);
            } else {
                const F3 x = node_at(i, j, k, P.dx);
                dist = len(closest_point(x, p, q, r) - x);
            }
            unsigned int *cell = reinterpret_cast<unsigned int *>(phi + (size_t)i + (size_t)W * ((size_t)j + (size_t)H * k));
            if (dist < __uint_as_float(*((volatile unsigned int *)cell))) atomicMin(cell, __float_as_uint(dist));
        }
    }
}

struct CrossArgs {
    const float *v;   // vertices on the test's cell grid
    const int *t;
    int nt;
    int ci, cj, ck;   // test grid cells
    F3 jit;
    double dx;
};

// fill = 0: count the crossings of every column; fill = 1: write their heights
__global__ void k_cross(CrossArgs T, int *count, const int *off, int *cursor, float *zs, int fill) {
    const double inv = 1.0 / T.dx;
    for (int tri = blockIdx.x; tri < T.nt; tri += gridDim.x) {
        const F3 a = vert(T.v, T.t[3 * tri]), b = vert(T.v, T.t[3 * tri + 1]), c = vert(T.v, T.t[3 * tri + 2]);
        const Box3 bb = tri_box(a, b, c);
        const F3 mx = bb.hi();
        const int i0 = max(floor_index(bb.lo.x, inv), 0), j0 = max(floor_index(bb.lo.y, inv), 0);
        const int i1 = min(floor_index(mx.x, inv), T.ci - 1), j1 = min(floor_index(mx.y, inv), T.cj - 1);
        if (i1 < i0 || j1 < j0) continue;
        const int ex = i1 - i0 + 1, n = ex * (j1 - j0 + 1);
        for (int s = threadIdx.x; s < n; s += blockDim.x) {
            const int i = i0 + s % ex, j = j0 + s / ex;
            const F3 o = centre_at(i, j, -1, T.dx) + T.jit;
            float z;
            if (!crosses(o, a, b, c, z)) continue;
            const int col = i + T.ci * j;
            if (!fill) atomicAdd(&count[col], 1);
            else zs[off[col] + atomicAdd(&cursor[col], 1)] = z;
        }
    }
}

// nodes of the part below an odd number of crossings of an even-count column
__global__ void k_inside(CrossArgs T, int gi, int gj, int gk, int ni, int nj, int nk, const int *off,
                         const float *zs, unsigned char *mark) {
    const size_t n = (size_t)T.ci * T.cj * T.ck;
    for (size_t s = blockIdx.x * (size_t)blockDim.x + threadIdx.x; s < n; s += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(s % T.ci), j = (int)((s / T.ci) % T.cj), k = (int)(s / ((size_t)T.ci * T.cj));
        const int a = i + gi, b = j + gj, c = k + gk;
        if (a < 0 || b < 0 || c < 0 || a > ni || b > nj || c > nk) continue;
        const int col = i + T.ci * j;
        const int z0 = off[col], z1 = off[col + 1];
        if ((z1 - z0) % 2 != 0) continue;
        const float zc = centre_at(i, j, k, T.dx).z;
        int below = 0;
        for (int q = z0; q < z1; q++) below += zs[q] < zc;
        if (below % 2 == 1) mark[(size_t)a + (size_t)(ni + 1) * ((size_t)b + (size_t)(nj + 1) * c)] = 1;
    }
}

// the part's signed values into the target: mode 0 min, mode 1 the negated values (the domain box)
__global__ void k_finish(const float *phi, const unsigned char *mark, int ni, int nj, int nk, int gi, int gj, int gk,
                         float *target, int ti, int tj, int tk, int mode) {
    const size_t n = (size_t)(ni + 1) * (nj + 1) * (nk + 1);
    for (size_t s = blockIdx.x * (size_t)blockDim.x + threadIdx.x; s < n; s += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(s % (ni + 1)), j = (int)((s / (ni + 1)) % (nj + 1)), k = (int)(s / ((size_t)(ni + 1) * (nj + 1)));
        const int a = i + gi, b = j + gj, c = k + gk;
        if (a < 0 || b < 0 || c < 0 || a > ti || b > tj || c > tk) continue;
        const float v = mark[s] ? -phi[s] : phi[s];
        float &dst = target[(size_t)a + (size_t)(ti + 1) * ((size_t)b + (size_t)(tj + 1) * c)];
        if (mode == 1) dst = -v;
        else if (v < dst) dst = v;
    }
}

__global__ void k_fill(float *a, size_t n, float v) {
    for (size_t s = blockIdx.x * (size_t)blockDim.x + threadIdx.x; s < n; s += (size_t)gridDim.x * blockDim.x) a[s] = v;
}

// solid = min(solid, -inv): the inverted obstacles (fluidsimulation.cpp:5318-5332)
__global__ void k_unite_negated(float *solid, const float *inv, size_t n) {
    for (size_t s = blockIdx.x * (size_t)blockDim.x + threadIdx.x; s < n; s += (size_t)gridDim.x * blockDim.x) {
        const float v = -inv[s];
        if (v < solid[s]) solid[s] = v;
    }
}

// ---- host side ----

struct HostMesh {
    std::vector<F3> v;
    std::vector<int> t;
    int ntri() const { return (int)(t.size() / 3); }
};

// AABB of a vertex list (aabb.cpp:54-82)
Box3 points_box(const std::vector<F3> &pts) {
    double mn[3] = {pts[0].x, pts[0].y, pts[0].z}, mx[3] = {pts[0].x, pts[0].y, pts[0].z};
    for (const F3 &p : pts) {
        mn[0] = std::fmin((double)p.x, mn[0]); mn[1] = std::fmin((double)p.y, mn[1]); mn[2] = std::fmin((double)p.z, mn[2]);
        mx[0] = std::fmax((double)p.x, mx[0]); mx[1] = std::fmax((double)p.y, mx[1]); mx[2] = std::fmax((double)p.z, mx[2]);
    }
    Box3 r;
    r.lo = fd3(mn[0], mn[1], mn[2]);
    r.w = mx[0] - mn[0] + 1e-9; r.h = mx[1] - mn[1] + 1e-9; r.d = mx[2] - mn[2] + 1e-9;
    return r;
}

// AABB::isPointInside (aabb.cpp:130-133) for a box with its corner at the origin
bool in_box(const Box3 &b, F3 p) {
    return p.x >= b.lo.x && p.y >= b.lo.y && p.z >= b.lo.z && p.x < b.lo.x + b.w && p.y < b.lo.y + b.h &&
           p.z < b.lo.z + b.d;
}

// AABB::getIntersection (aabb.cpp:170-190): true when the overlap has a positive extent
bool overlaps(const Box3 &a, const Box3 &b) {
    const F3 l1 = a.lo, l2 = b.lo, h1 = a.hi(), h2 = b.hi();
    if (l1.x > h2.x || l1.y > h2.y || l1.z > h2.z || h1.x < l2.x || h1.y < l2.y || h1.z < l2.z) return false;
    const F3 lo = fd3(std::fmax(l1.x, l2.x), std::fmax(l1.y, l2.y), std::fmax(l1.z, l2.z));
    const F3 hi = fd3(std::fmin(h1.x, h2.x), std::fmin(h1.y, h2.y), std::fmin(h1.z, h2.z));
    return (double)hi.x - (double)lo.x > 0.0 || (double)hi.y - (double)lo.y > 0.0 || (double)hi.z - (double)lo.z > 0.0;
}

Box3 grid_box(int ni, int nj, int nk, double dx) {
    Box3 b;
    b.lo = f3(0.0f, 0.0f, 0.0f);
    b.w = ni * dx; b.h = nj * dx; b.d = nk * dx;
    return b;
}

// vertex-connected components (meshutils.cpp:464-572): triangles in mesh order, vertices in
// order of first use
std::vector<HostMesh> islands_of(const HostMesh &m) {
    const int nv = (int)m.v.size();
    std::vector<int> head(nv + 1, 0), adj;
    for (int x : m.t) head[x + 1] += 2;
    for (int q = 0; q < nv; q++) head[q + 1] += head[q];
    adj.resize(head[nv]);
    std::vector<int> fillp(head.begin(), head.end() - 1);
    for (int t = 0; t < m.ntri(); t++)
        for (int q = 0; q < 3; q++) {
            const int a = m.t[3 * t + q];
            adj[fillp[a]++] = m.t[3 * t + (q + 1) % 3];
            adj[fillp[a]++] = m.t[3 * t + (q + 2) % 3];
        }
    std::vector<int> group(nv, -1), stack;
    int ng = 0;
    for (int s = 0; s < nv; s++) {
        if (group[s] != -1) continue;
        group[s] = ng;
        stack.assign(1, s);
        while (!stack.empty()) {
            const int x = stack.back();
            stack.pop_back();
            for (int q = head[x]; q < head[x + 1]; q++)
                if (group[adj[q]] == -1) { group[adj[q]] = ng; stack.push_back(adj[q]); }
        }
        ng++;
    }
    std::vector<HostMesh> out(ng);
    std::vector<int> remap(nv, -1);
    for (int t = 0; t < m.ntri(); t++) {
        HostMesh &isl = out[group[m.t[3 * t]]];
        for (int q = 0; q < 3; q++) {
            const int vi = m.t[3 * t + q];
            if (remap[vi] == -1) { remap[vi] = (int)isl.v.size(); isl.v.push_back(m.v[vi]); }
            isl.t.push_back(remap[vi]);
        }
    }
    return out;
}

void append_mesh(HostMesh &a, const HostMesh &b) {
    const int base = (int)a.v.size();
    a.v.insert(a.v.end(), b.v.begin(), b.v.end());
    for (int x : b.t) a.t.push_back(x + base);
}

// MeshObject::_expandMeshIsland (meshobject.cpp:710-736)
void expand(HostMesh &m, float expansion) {
    F3 sum = f3(0.0f, 0.0f, 0.0f);
    for (const F3 &p : m.v) sum = sum + p;
    const F3 cen = divf(sum, (float)m.v.size());
    const float e = 0.5f * expansion, eps = 1e-9f;
    for (F3 &p : m.v) {
        F3 d = p - cen;
        if (std::fabs(d.x) < eps && std::fabs(d.y) < eps && std::fabs(d.z) < eps) continue;
        d = divf(d, len(d));
        p = p + e * d;
    }
}

// closed-domain box mesh: the domain's AABB expanded by -(3 dx + 1e-4) (fluidsimulation.cpp:5175-5186)
HostMesh domain_mesh(int ni, int nj, int nk, double dx) {
    const double v = -3 * dx - 1e-4, hv = 0.5 * v;
    const F3 p = f3(0.0f, 0.0f, 0.0f) - fd3(hv, hv, hv);
    const double w = ni * dx + v, h = nj * dx + v, d = nk * dx + v;
    HostMesh m;
    m.v = {fd3(p.x, p.y, p.z), fd3(p.x + w, p.y, p.z), fd3(p.x + w, p.y, p.z + d), fd3(p.x, p.y, p.z + d),
           fd3(p.x, p.y + h, p.z), fd3(p.x + w, p.y + h, p.z), fd3(p.x + w, p.y + h, p.z + d), fd3(p.x, p.y + h, p.z + d)};
    m.t = {0, 1, 2, 0, 2, 3, 4, 7, 6, 4, 6, 5, 0, 3, 7, 0, 7, 4, 1, 5, 6, 1, 6, 2, 0, 4, 5, 0, 5, 1, 3, 2, 6, 3, 6, 7};
    return m;
}

}  // namespace

struct SolidBuilder::Part {
    HostMesh mesh;            // absolute coordinates
    int ni, nj, nk;           // cells
    int gi, gj, gk;           // origin node in the domain grid
    F3 off;
    bool serial;
    double dx;
    float upper() const { return (float)((ni + 1 + nj + 1 + nk + 1) * dx); }   // meshlevelset.cpp:769-771
    size_t nodes() const { return (size_t)(ni + 1) * (nj + 1) * (nk + 1); }
};

void SolidBuilder::next_jitter(double dx, float j[3]) {
    if (jitter_list && jitter_used < jitter_n) {
        std::memcpy(j, jitter_list + 3 * jitter_used, 3 * sizeof(float));
    } else {
        // jit + u (-jit - jit), jit = 0.001 dx (meshutils.cpp:95-114), with fixed u = r / 2147483647
        // for r = 536870912, 1503238554, 858993459: distinct components keep the lines off the
        // diagonals of grid-aligned faces
        const double jit = 0.001 * dx, rmax = 2147483647.0;
        j[0] = (float)(jit + (536870912.0 / rmax) * (-jit - jit));
        j[1] = (float)(jit + (1503238554.0 / rmax) * (-jit - jit));
        j[2] = (float)(jit + (858993459.0 / rmax) * (-jit - jit));
    }
    jitter_used++;
}

void SolidBuilder::level_set(const Part &p, cudaStream_t st) {
    const size_t nn = p.nodes();
    part.reserve(nn);
    mark.reserve(nn);
    k_fill<<<grid_for(nn, 256), 256, 0, st>>>(part, nn, p.upper());
    FFGPU_CUDA(cudaMemsetAsync(mark, 0, nn, st));
    launches++;
    const HostMesh &m = p.mesh;
    if (m.t.empty()) return;
    verts.reserve(3 * m.v.size());
    tris.reserve(m.t.size());
    FFGPU_CUDA(cudaMemcpyAsync(verts, m.v.data(), m.v.size() * sizeof(F3), cudaMemcpyHostToDevice, st));
    FFGPU_CUDA(cudaMemcpyAsync(tris, m.t.data(), m.t.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    BandArgs B{verts, tris, m.ntri(), p.ni, p.nj, p.nk, p.off, p.dx, p.serial ? 1 : 0};
    k_band<<<(unsigned)std::min(m.ntri(), 152 * 64), 128, 0, st>>>(B, part);
    launches++;
    // the sign (meshlevelset.cpp:1298-1318): the mesh in part coordinates, split into islands when it
    // leaves the part's box (meshutils.cpp:382-437)
    HostMesh tm = m;
    for (F3 &v : tm.v) v = v + neg(p.off);
    const Box3 box = grid_box(p.ni, p.nj, p.nk, p.dx);
    bool contained = true;
    for (const F3 &v : tm.v)
        if (!in_box(box, v)) { contained = false; break; }
    std::vector<HostMesh> tests;
    if (contained) {
        tests.push_back(std::move(tm));
    } else {
        HostMesh inner;
        std::vector<HostMesh> crossing;
        for (HostMesh &isl : islands_of(tm)) {
            if (isl.v.empty()) continue;
            const Box3 ib = points_box(isl.v);
            if (in_box(box, ib.lo) && in_box(box, ib.hi())) append_mesh(inner, isl);
            else if (overlaps(box, ib)) crossing.push_back(std::move(isl));
        }
        tests.push_back(std::move(inner));
        for (HostMesh &c : crossing) tests.push_back(std::move(c));
    }
    // MeshUtils::getGridNodesInsideTriangleMesh, list form (meshutils.cpp:356-380), per test mesh
    for (HostMesh &t : tests) {
        float jit[3];
        next_jitter(p.dx, jit);
        if (t.v.empty() || t.t.empty()) continue;
        // shifted by half a cell and moved to the cell grid of its box (meshutils.cpp:358-372)
        const float hw = (float)(0.5 * p.dx);
        for (F3 &v : t.v) v = v + f3(hw, hw, hw);
        Box3 bb = points_box(t.v);
        const double inv = 1.0 / p.dx;
        const int go[3] = {floor_index(bb.lo.x, inv), floor_index(bb.lo.y, inv), floor_index(bb.lo.z, inv)};
        const F3 o = node_at(go[0], go[1], go[2], p.dx);
        for (F3 &v : t.v) v = v + neg(o);
        bb.lo = bb.lo - o;
        const F3 mx = bb.hi();
        const int ci = floor_index(mx.x, inv) + 1, cj = floor_index(mx.y, inv) + 1, ck = floor_index(mx.z, inv) + 1;
        if (ci <= 0 || cj <= 0 || ck <= 0) continue;
        const size_t ncol = (size_t)ci * cj;
        verts.reserve(3 * t.v.size());
        tris.reserve(t.t.size());
        FFGPU_CUDA(cudaMemcpyAsync(verts, t.v.data(), t.v.size() * sizeof(F3), cudaMemcpyHostToDevice, st));
        FFGPU_CUDA(cudaMemcpyAsync(tris, t.t.data(), t.t.size() * sizeof(int), cudaMemcpyHostToDevice, st));
        col_count.reserve(ncol + 1);
        col_off.reserve(ncol + 1);
        col_cursor.reserve(ncol);
        scan_tmp.reserve(scan_scratch_ints(ncol + 1) + 64);
        FFGPU_CUDA(cudaMemsetAsync(col_count, 0, (ncol + 1) * sizeof(int), st));
        FFGPU_CUDA(cudaMemsetAsync(col_cursor, 0, ncol * sizeof(int), st));
        CrossArgs C{verts, tris, t.ntri(), ci, cj, ck, f3(jit[0], jit[1], jit[2]), p.dx};
        const unsigned g = (unsigned)std::min(t.ntri(), 152 * 64);
        k_cross<<<g, 128, 0, st>>>(C, col_count, nullptr, nullptr, nullptr, 0);
        launch_exclusive_scan(col_count, col_off, ncol, scan_tmp, st);
        int total = 0;
        FFGPU_CUDA(cudaMemcpyAsync(&total, col_off.p + ncol, sizeof(int), cudaMemcpyDeviceToHost, st));
        FFGPU_CUDA(cudaStreamSynchronize(st));
        launches += 2;
        if (total == 0) continue;
        zs.reserve(total);
        k_cross<<<g, 128, 0, st>>>(C, nullptr, col_off, col_cursor, zs, 1);
        k_inside<<<grid_for(ncol * ck, 256), 256, 0, st>>>(C, go[0], go[1], go[2], p.ni, p.nj, p.nk, col_off, zs,
                                                           mark);
        launches += 2;
    }
    FFGPU_CUDA(cudaGetLastError());
}

int SolidBuilder::build(Dims d, double dx, const std::vector<const Obstacle *> &obstacles, float *solid,
                        cudaStream_t st, const float *jitter, int njitter) {
    launches = 0;
    jitter_used = 0;
    jitter_list = jitter;
    jitter_n = njitter;
    const size_t nn = (size_t)(d.ni + 1) * (d.nj + 1) * (d.nk + 1);
    // the closed domain: the box mesh's level set over the whole grid, negated
    Part dom{domain_mesh(d.ni, d.nj, d.nk, dx), d.ni, d.nj, d.nk, 0, 0, 0, f3(0.0f, 0.0f, 0.0f), false, dx};
    level_set(dom, st);
    k_finish<<<grid_for(nn, 256), 256, 0, st>>>(part, mark, d.ni, d.nj, d.nk, 0, 0, 0, solid, d.ni, d.nj, d.nk, 1);
    launches++;
    const Box3 dombox = grid_box(d.ni, d.nj, d.nk, dx);
    const double rdx = 1.0 / dx;
    auto add_obstacle = [&](const Obstacle &ob, float *target) {
        // the static mesh at the frame time, v + f (v - v), and without unused vertices
        // (meshobject.cpp:158-177, 243-250)
        HostMesh m;
        std::vector<int> used(ob.v.size() / 3, -1);
        for (int x : ob.t) used[x] = 0;
        for (size_t q = 0; q < used.size(); q++)
            if (used[q] == 0) {
                used[q] = (int)m.v.size();
                m.v.push_back(f3(ob.v[3 * q], ob.v[3 * q + 1], ob.v[3 * q + 2]) + f3(0.0f, 0.0f, 0.0f));
            }
        for (int x : ob.t) m.t.push_back(used[x]);
        if (m.t.empty()) return;
        std::vector<HostMesh> isl;   // islands inside or crossing the domain (meshobject.cpp:633-665)
        for (HostMesh &i : islands_of(m)) {
            if (i.v.empty()) continue;
            const Box3 ib = points_box(i.v);
            if ((in_box(dombox, ib.lo) && in_box(dombox, ib.hi())) || overlaps(dombox, ib)) isl.push_back(std::move(i));
        }
        const bool per_island = (int)isl.size() >= ISLAND_TRIGGER;
        if (per_island && std::fabs(ob.expansion) >= 1e-9f)
            for (HostMesh &i : isl) expand(i, ob.expansion);
        std::vector<HostMesh> parts;
        if (per_island) parts = std::move(isl);
        else parts.push_back(std::move(m));
        for (HostMesh &pm : parts) {   // MeshObject::_getMeshIslandLevelSet (meshobject.cpp:667-701)
            const Box3 ib = points_box(pm.v);
            const F3 mx = ib.hi();
            const int lo[3] = {std::max(floor_index(ib.lo.x, rdx) - EXACT_BAND, 0),
                               std::max(floor_index(ib.lo.y, rdx) - EXACT_BAND, 0),
                               std::max(floor_index(ib.lo.z, rdx) - EXACT_BAND, 0)};
            const int hi[3] = {std::min(floor_index(mx.x, rdx) + EXACT_BAND + 1, d.ni - 1),
                               std::min(floor_index(mx.y, rdx) + EXACT_BAND + 1, d.nj - 1),
                               std::min(floor_index(mx.z, rdx) + EXACT_BAND + 1, d.nk - 1)};
            const int w = hi[0] - lo[0], h = hi[1] - lo[1], dd = hi[2] - lo[2];
            if (w <= 0 || h <= 0 || dd <= 0) continue;
            Part p{std::move(pm), w, h, dd, lo[0], lo[1], lo[2], node_at(lo[0], lo[1], lo[2], dx), per_island, dx};
            level_set(p, st);
            k_finish<<<grid_for(p.nodes(), 256), 256, 0, st>>>(part, mark, w, h, dd, lo[0], lo[1], lo[2], target, d.ni,
                                                               d.nj, d.nk, 0);
            launches++;
        }
    };
    for (const Obstacle *ob : obstacles)
        if (ob->enabled && !ob->inversed) add_obstacle(*ob, solid);
    bool any_inv = false;
    for (const Obstacle *ob : obstacles) any_inv = any_inv || (ob->enabled && ob->inversed);
    if (any_inv) {
        inv.reserve(nn);
        k_fill<<<grid_for(nn, 256), 256, 0, st>>>(inv, nn, dom.upper());
        for (const Obstacle *ob : obstacles)
            if (ob->enabled && ob->inversed) add_obstacle(*ob, inv);
        k_unite_negated<<<grid_for(nn, 256), 256, 0, st>>>(solid, inv, nn);
        launches += 2;
    }
    FFGPU_CUDA(cudaGetLastError());
    return launches;
}

}  // namespace ffgpu
