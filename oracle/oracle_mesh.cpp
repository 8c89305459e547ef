// Solid level set of triangle-mesh obstacles -- TEST INFRASTRUCTURE ONLY (CPU oracle).
//
// Restates, for static obstacles:
//   MeshLevelSet::fastCalculateSignedDistanceField (meshlevelset.cpp:572-601): exact distances in a
//     band around every triangle (block form :781-876 with the triangle boxes of :878-918 and the
//     block-local coordinates of :1115-1163; island form :1165-1234), then the inside test
//     (:1298-1318 with MeshUtils::getGridNodesInsideTriangleMesh, meshutils.cpp:57-245, 356-437);
//   the closest point on a triangle, Collision::findClosestPointOnTriangle (collision.cpp:161-270),
//     and the z-line crossing test, Collision::lineIntersectsTriangle (collision.cpp:79-114);
//   MeshObject::getMeshLevelSet (meshobject.cpp:239-264) with its islands (:633-736, :738-860);
//   FluidSimulation::_addStaticObjectsToSDF (fluidsimulation.cpp:5277-5333) with the closed-domain
//     box mesh (fluidsimulation.cpp:5175-5186 and _getTriangleMeshFromAABB) and
//     MeshLevelSet::calculateUnion (meshlevelset.cpp:603-638, 1759-1790).
//
// The inside test offsets its z lines by a jitter that the reference draws from the C library's
// rand(); here it is an argument (3 floats per inside test, in call order, or one fixed value).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "oracle.h"

namespace oracle {
namespace {

constexpr int EXACT_BAND = 3;         // FluidSimulation::_solidLevelSetExactBand (fluidsimulation.h:2235)
constexpr int BLOCK_WIDTH = 10;       // MeshLevelSet::_blockwidth (meshlevelset.h:369)
constexpr int ISLAND_TRIGGER = 25;    // MeshObject::_numIslandsForFractureOptimizationTrigger (meshobject.h:222)

struct Mesh {
    std::vector<V3> v;
    std::vector<int> t;   // three vertex indices per triangle
    int ntri() const { return (int)(t.size() / 3); }
};

inline float dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross3(V3 a, V3 b) { return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
inline V3 neg3(V3 a) { return v3(-a.x, -a.y, -a.z); }
inline V3 d3(double x, double y, double z) { return v3((float)x, (float)y, (float)z); }

// AABB with a float corner and double extents (aabb.h)
struct AB {
    V3 pos;
    double w = 0.0, h = 0.0, d = 0.0;
    V3 maxp() const { return pos + d3(w, h, d); }                       // aabb.cpp:493-495
    bool inside(V3 p) const {                                           // aabb.cpp:130-133
        return p.x >= pos.x && p.y >= pos.y && p.z >= pos.z && p.x < pos.x + w && p.y < pos.y + h &&
               p.z < pos.z + d;
    }
};

// aabb.cpp:54-82 (points) and :84-112 (one triangle): min corner, extents + 1e-9
AB bounds(const V3 *pts, const int *idx, int n) {
    const V3 &p0 = pts[idx ? idx[0] : 0];
    double lo[3] = {p0.x, p0.y, p0.z}, hi[3] = {p0.x, p0.y, p0.z};
    for (int q = 0; q < n; q++) {
        const V3 &p = pts[idx ? idx[q] : q];
        lo[0] = std::fmin(p.x, lo[0]); lo[1] = std::fmin(p.y, lo[1]); lo[2] = std::fmin(p.z, lo[2]);
        hi[0] = std::fmax(p.x, hi[0]); hi[1] = std::fmax(p.y, hi[1]); hi[2] = std::fmax(p.z, hi[2]);
    }
    AB b;
    b.pos = d3(lo[0], lo[1], lo[2]);
    b.w = hi[0] - lo[0] + 1e-9; b.h = hi[1] - lo[1] + 1e-9; b.d = hi[2] - lo[2] + 1e-9;
    return b;
}
AB mesh_bounds(const Mesh &m) { return bounds(m.v.data(), nullptr, (int)m.v.size()); }
AB tri_bounds(const Mesh &m, int t) { return bounds(m.v.data(), &m.t[3 * t], 3); }

// AABB::getIntersection (aabb.cpp:170-190): an empty box when disjoint
AB intersection(const AB &a, const AB &b) {
    V3 lo1 = a.pos, lo2 = b.pos, hi1 = a.maxp(), hi2 = b.maxp();
    AB r;
    if (lo1.x > hi2.x || lo1.y > hi2.y || lo1.z > hi2.z || hi1.x < lo2.x || hi1.y < lo2.y || hi1.z < lo2.z) {
        r.pos = v3(0, 0, 0);
        return r;
    }
    V3 lo = d3(std::fmax(lo1.x, lo2.x), std::fmax(lo1.y, lo2.y), std::fmax(lo1.z, lo2.z));
    V3 hi = d3(std::fmin(hi1.x, hi2.x), std::fmin(hi1.y, hi2.y), std::fmin(hi1.z, hi2.z));
    r.pos = lo;   // AABB(p1, p2), aabb.cpp:40-52: no eps
    r.w = (double)hi.x - (double)lo.x; r.h = (double)hi.y - (double)lo.y; r.d = (double)hi.z - (double)lo.z;
    return r;
}

struct I3 { int i, j, k; };
I3 to_index(V3 p, double dx) {   // Grid3d::positionToGridIndex (grid3d.h:55-60)
    const double inv = 1.0 / dx;
    return I3{(int)std::floor(p.x * inv), (int)std::floor(p.y * inv), (int)std::floor(p.z * inv)};
}
V3 node_pos(int i, int j, int k, double dx) {   // Grid3d::GridIndexToPosition (grid3d.h:76-78)
    return d3((float)i * dx, (float)j * dx, (float)k * dx);
}
V3 cell_center(int i, int j, int k, double dx) {   // Grid3d::GridIndexToCellCenter (grid3d.h:100-103)
    const double hw = 0.5 * dx;
    return d3((float)i * dx + hw, (float)j * dx + hw, (float)k * dx + hw);
}

double clampd(double v, double lo, double hi) { return v < lo ? lo : (v > hi ? hi : v); }

// Collision::findClosestPointOnTriangle (collision.cpp:161-270): dots in float, the parameters
// in double
V3 closest_on_triangle(V3 p0, V3 v0, V3 v1, V3 v2) {
    const V3 e0 = v1 - v0, e1 = v2 - v0, pv = v0 - p0;
    const double a = dot3(e0, e0), b = dot3(e0, e1), c = dot3(e1, e1), d = dot3(e0, pv), e = dot3(e1, pv);
    const double det = a * c - b * b;
    if (std::abs(det) < 1e-9) {   // degenerate: a segment or a point
        const float feps = 1e-6f;
        const float l1 = vlength(v0 - v1), l2 = vlength(v1 - v2), l3 = vlength(v2 - v0);
        if (l1 < feps && l2 < feps && l3 < feps) return v0;
        V3 dp, dq;
        if (l1 < feps) { dp = v0; dq = v2; }
        else if (l2 < feps) { dp = v1; dq = v0; }
        else { dp = v2; dq = v1; }
        const float num = dot3(p0 - dp, dq - dp), den = dot3(dq - dp, dq - dp);
        if (std::abs(den) < feps) return v0;
        const float lam = num / den;
        if (lam <= 0.0f) return dp;
        if (lam >= 1.0f) return dq;
        return dp + lam * (dq - dp);
    }
    double s = b * e - c * d, t = b * d - a * e;
    if (s + t < det) {
        if (s < 0.0) {
            if (t < 0.0) {
                if (d < 0.0) { s = clampd(-d / a, 0.0, 1.0); t = 0.0; }
                else { s = 0.0; t = clampd(-e / c, 0.0, 1.0); }
            } else {
                s = 0.0; t = clampd(-e / c, 0.0, 1.0);
            }
        } else if (t < 0.0) {
            s = clampd(-d / a, 0.0, 1.0); t = 0.0;
        } else {
            const double inv = 1.0 / det;
            s *= inv; t *= inv;
        }
    } else {
        if (s < 0.0) {
            const double t0 = b + d, t1 = c + e;
            if (t1 > t0) { s = clampd((t1 - t0) / (a - 2 * b + c), 0.0, 1.0); t = 1 - s; }
            else { t = clampd(-e / c, 0.0, 1.0); s = 0.0; }
        } else if (t < 0.0) {
            if (a + d > b + e) { s = clampd((c + e - b - d) / (a - 2 * b + c), 0.0, 1.0); t = 1 - s; }
            else { s = clampd(-e / c, 0.0, 1.0); t = 0.0; }
        } else {
            s = clampd((c + e - b - d) / (a - 2 * b + c), 0.0, 1.0); t = 1.0 - s;
        }
    }
    return (v0 + (float)s * e0) + (float)t * e1;
}

float tri_distance(V3 x, V3 a, V3 b, V3 c) { return vlength(closest_on_triangle(x, a, b, c) - x); }

// Collision::lineIntersectsTriangle (collision.cpp:79-114) for the +z line through p: the z of the
// crossing point
bool z_crossing(V3 p, V3 v0, V3 v1, V3 v2, float &z) {
    const V3 dir = v3(0.0f, 0.0f, 1.0f);
    const V3 e1 = v1 - v0, e2 = v2 - v0;
    const V3 h = cross3(dir, e2);
    const float a = dot3(e1, h);
    if (std::fabs(a) < 10e-9) return false;
    const float f = 1 / a;
    const V3 s = p - v0;
    const float u = f * dot3(s, h);
    if (u < 0.0 || u > 1.0) return false;
    const V3 q = cross3(s, e1);
    const float v = f * dot3(dir, q);
    if (v < 0.0 || u + v > 1.0) return false;
    const double t = f * dot3(e2, q);
    z = (p + (float)t * dir).z;
    return true;
}

// MeshUtils::_splitIntoMeshIslands (meshutils.cpp:464-572): vertex-connected components, each with
// its triangles in mesh order and its vertices in order of first use
std::vector<Mesh> split_islands(const Mesh &m) {
    const int nv = (int)m.v.size();
    std::vector<std::vector<int>> nb(nv);
    for (int t = 0; t < m.ntri(); t++)
        for (int q = 0; q < 3; q++) {
            nb[m.t[3 * t + q]].push_back(m.t[3 * t + (q + 1) % 3]);
            nb[m.t[3 * t + q]].push_back(m.t[3 * t + (q + 2) % 3]);
        }
    std::vector<int> group(nv, -1);
    int ng = 0;
    for (int s = 0; s < nv; s++) {
        if (group[s] != -1) continue;
        std::vector<int> stack{s};
        group[s] = ng;
        while (!stack.empty()) {
            int x = stack.back();
            stack.pop_back();
            for (int y : nb[x])
                if (group[y] == -1) { group[y] = ng; stack.push_back(y); }
        }
        ng++;
    }
    std::vector<Mesh> out(ng);
    std::vector<int> remap(nv, -1);
    for (int t = 0; t < m.ntri(); t++) {
        Mesh &isl = out[group[m.t[3 * t]]];
        for (int q = 0; q < 3; q++) {
            const int vi = m.t[3 * t + q];
            if (remap[vi] == -1) { remap[vi] = (int)isl.v.size(); isl.v.push_back(m.v[vi]); }
            isl.t.push_back(remap[vi]);
        }
    }
    return out;
}

void append(Mesh &a, const Mesh &b) {   // TriangleMesh::append (trianglemesh.cpp:883-900)
    const int off = (int)a.v.size();
    a.v.insert(a.v.end(), b.v.begin(), b.v.end());
    for (int x : b.t) a.t.push_back(x + off);
}

// MeshUtils::getGridNodesInsideTriangleMesh, the list form (meshutils.cpp:356-380): nodes whose
// +z line from below crosses the mesh an odd number of times, counted at cell centres of the mesh
// shifted by half a cell
void nodes_inside(Mesh m, double dx, V3 jitter, std::vector<I3> &out) {
    if (m.v.empty()) return;
    const float hw = (float)(0.5 * dx);
    for (V3 &p : m.v) p = p + v3(hw, hw, hw);
    AB bb = mesh_bounds(m);
    const I3 go = to_index(bb.pos, dx);
    const V3 off = node_pos(go.i, go.j, go.k, dx);
    for (V3 &p : m.v) p = p + neg3(off);
    bb.pos = bb.pos - off;
    const I3 g2 = to_index(bb.maxp(), dx);
    const int ci = g2.i + 1, cj = g2.j + 1, ck = g2.k + 1;
    if (ci <= 0 || cj <= 0 || ck <= 0) return;
    // triangles per column (meshutils.cpp:57-75)
    std::vector<std::vector<int>> col((size_t)ci * cj);
    for (int t = 0; t < m.ntri(); t++) {
        AB tb = tri_bounds(m, t);
        I3 a = to_index(tb.pos, dx), b = to_index(tb.maxp(), dx);
        a.i = std::max(a.i, 0); a.j = std::max(a.j, 0);
        b.i = std::min(b.i, ci - 1); b.j = std::min(b.j, cj - 1);
        for (int j = a.j; j <= b.j; j++)
            for (int i = a.i; i <= b.i; i++) col[(size_t)i + (size_t)ci * j].push_back(t);
    }
    for (int j = 0; j < cj; j++)
        for (int i = 0; i < ci; i++) {
            const std::vector<int> &ts = col[(size_t)i + (size_t)ci * j];
            if (ts.empty()) continue;
            const V3 o = cell_center(i, j, -1, dx) + jitter;
            std::vector<float> zs;
            for (int t : ts) {
                float z;
                if (z_crossing(o, m.v[m.t[3 * t]], m.v[m.t[3 * t + 1]], m.v[m.t[3 * t + 2]], z)) zs.push_back(z);
            }
            if (zs.size() % 2 != 0) continue;   // meshutils.cpp:205-207
            for (int k = 0; k < ck; k++) {
                const float zc = cell_center(i, j, k, dx).z;
                int below = 0;
                for (float z : zs) below += z < zc;
                if (below % 2 == 1) out.push_back(I3{i + go.i, j + go.j, k + go.k});
            }
        }
}

// Jitter of the c-th inside test: the caller's list, else the fixed draw jit + u (-jit - jit) of
// meshutils.cpp:95-97, 110-114 with jit = 0.001 dx and u = r / 2147483647 for the integers
// r = 536870912, 1503238554, 858993459 in x, y, z (distinct components keep the lines off the
// diagonals of grid-aligned faces)
struct Jitter {
    const float *list = nullptr;
    int n = 0, used = 0;
    double dx = 0.0;
    V3 next() {
        if (used < n) { const float *j = list + 3 * used++; return v3(j[0], j[1], j[2]); }
        used++;
        const double jit = 0.001 * dx, rmax = 2147483647.0;
        return d3(jit + (536870912.0 / rmax) * (-jit - jit), jit + (1503238554.0 / rmax) * (-jit - jit),
                  jit + (858993459.0 / rmax) * (-jit - jit));
    }
};

// A MeshLevelSet on a box of the domain: cells (ni, nj, nk) from node `go`, nodes stored x fastest
struct LevelSet {
    int ni, nj, nk;
    I3 go;
    V3 off;   // position of node go (MeshLevelSet::setGridOffset, meshlevelset.cpp:720-723)
    double dx;
    std::vector<float> phi;
    float upper() const { return (float)((ni + 1 + nj + 1 + nk + 1) * dx); }   // meshlevelset.cpp:769-771
    float &at(int i, int j, int k) { return phi[flat(i, j, k, ni + 1, nj + 1)]; }
    bool in(int i, int j, int k) const { return i >= 0 && j >= 0 && k >= 0 && i <= ni && j <= nj && k <= nk; }
    LevelSet(int a, int b, int c, I3 g, double h) : ni(a), nj(b), nk(c), go(g), dx(h) {
        off = node_pos(g.i, g.j, g.k, h);
        phi.assign((size_t)(ni + 1) * (nj + 1) * (nk + 1), upper());
    }
};

// exact band, block form: triangle boxes from the float AABB (meshlevelset.cpp:878-918), distances
// in the coordinates of each node's 10^3 block (:1115-1163)
void band_blocks(LevelSet &L, const Mesh &m, int band) {
    for (int t = 0; t < m.ntri(); t++) {
        AB tb = tri_bounds(m, t);
        tb.pos = tb.pos - L.off;
        I3 lo = to_index(tb.pos, L.dx), hi = to_index(tb.maxp(), L.dx);
        lo.i -= band; lo.j -= band; lo.k -= band;
        hi.i += band + 1; hi.j += band + 1; hi.k += band + 1;
        if (hi.i < 0 || lo.i >= L.ni + 1 || hi.j < 0 || lo.j >= L.nj + 1 || hi.k < 0 || lo.k >= L.nk + 1) continue;
        lo.i = std::max(lo.i, 0); lo.j = std::max(lo.j, 0); lo.k = std::max(lo.k, 0);
        hi.i = std::min(hi.i, L.ni); hi.j = std::min(hi.j, L.nj); hi.k = std::min(hi.k, L.nk);
        const V3 p = m.v[m.t[3 * t]] - L.off, q = m.v[m.t[3 * t + 1]] - L.off, r = m.v[m.t[3 * t + 2]] - L.off;
        for (int k = lo.k; k <= hi.k; k++)
            for (int j = lo.j; j <= hi.j; j++)
                for (int i = lo.i; i <= hi.i; i++) {
                    const int bi = i / BLOCK_WIDTH, bj = j / BLOCK_WIDTH, bk = k / BLOCK_WIDTH;
                    const V3 bo = node_pos(bi, bj, bk, BLOCK_WIDTH * L.dx);
                    const V3 x = node_pos(i - BLOCK_WIDTH * bi, j - BLOCK_WIDTH * bj, k - BLOCK_WIDTH * bk, L.dx);
                    const float dist = tri_distance(x, p - bo, q - bo, r - bo);
                    if (dist < L.at(i, j, k)) L.at(i, j, k) = dist;
                }
    }
}

// exact band, single-threaded form (meshlevelset.cpp:1165-1234): boxes from the vertices' grid
// coordinates (truncated), clamped to the nodes
void band_serial(LevelSet &L, const Mesh &m, int band) {
    const double inv = 1.0 / L.dx;
    auto clampi = [](int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); };
    for (int t = 0; t < m.ntri(); t++) {
        const V3 p = m.v[m.t[3 * t]] - L.off, q = m.v[m.t[3 * t + 1]] - L.off, r = m.v[m.t[3 * t + 2]] - L.off;
        const double fp[3] = {(double)p.x * inv, (double)p.y * inv, (double)p.z * inv};
        const double fq[3] = {(double)q.x * inv, (double)q.y * inv, (double)q.z * inv};
        const double fr[3] = {(double)r.x * inv, (double)r.y * inv, (double)r.z * inv};
        const int top[3] = {L.ni, L.nj, L.nk};
        int lo[3], hi[3];
        for (int a = 0; a < 3; a++) {
            lo[a] = clampi(int(std::fmin(fp[a], std::fmin(fq[a], fr[a]))) - band, 0, top[a]);
            hi[a] = clampi(int(std::fmax(fp[a], std::fmax(fq[a], fr[a]))) + band + 1, 0, top[a]);
        }
        for (int k = lo[2]; k <= hi[2]; k++)
            for (int j = lo[1]; j <= hi[1]; j++)
                for (int i = lo[0]; i <= hi[0]; i++) {
                    const float dist = tri_distance(node_pos(i, j, k, L.dx), p, q, r);
                    if (dist < L.at(i, j, k)) L.at(i, j, k) = dist;
                }
    }
}

// MeshLevelSet::_computeDistanceFieldSigns (meshlevelset.cpp:1298-1318) with the grid form of
// getGridNodesInsideTriangleMesh (meshutils.cpp:382-437): a mesh that leaves the box is split into
// islands, those inside tested together and each crossing one on its own
void signs(LevelSet &L, const Mesh &m, Jitter &jit) {
    Mesh tm = m;
    for (V3 &p : tm.v) p = p + neg3(L.off);
    AB box;
    box.pos = v3(0, 0, 0);
    box.w = L.ni * L.dx; box.h = L.nj * L.dx; box.d = L.nk * L.dx;
    bool contained = true;
    for (const V3 &p : tm.v)
        if (!box.inside(p)) { contained = false; break; }
    std::vector<I3> nodes;
    if (contained) {
        nodes_inside(tm, L.dx, jit.next(), nodes);
    } else {
        Mesh inner;
        std::vector<Mesh> crossing;
        for (Mesh &isl : split_islands(tm)) {
            if (isl.v.empty()) continue;
            AB ib = mesh_bounds(isl);
            if (box.inside(ib.pos) && box.inside(ib.maxp())) { append(inner, isl); continue; }
            AB x = intersection(box, ib);
            if (x.w > 0.0 || x.h > 0.0 || x.d > 0.0) crossing.push_back(isl);
        }
        nodes_inside(inner, L.dx, jit.next(), nodes);
        for (Mesh &c : crossing) nodes_inside(c, L.dx, jit.next(), nodes);
    }
    std::vector<char> mark(L.phi.size(), 0);
    for (const I3 &g : nodes)
        if (L.in(g.i, g.j, g.k)) mark[flat(g.i, g.j, g.k, L.ni + 1, L.nj + 1)] = 1;
    for (size_t c = 0; c < mark.size(); c++)
        if (mark[c]) L.phi[c] = -L.phi[c];
}

// MeshLevelSet::calculateUnion (meshlevelset.cpp:1759-1790), phi only
void unite(LevelSet &dst, const LevelSet &src) {
    for (int k = 0; k <= src.nk; k++)
        for (int j = 0; j <= src.nj; j++)
            for (int i = 0; i <= src.ni; i++) {
                const int a = i + src.go.i - dst.go.i, b = j + src.go.j - dst.go.j, c = k + src.go.k - dst.go.k;
                if (!dst.in(a, b, c)) continue;
                const float v = src.phi[flat(i, j, k, src.ni + 1, src.nj + 1)];
                if (v < dst.at(a, b, c)) dst.at(a, b, c) = v;
            }
}

// MeshObject::_expandMeshIsland (meshobject.cpp:710-736)
void expand_island(Mesh &m, float expansion) {
    if (m.v.empty()) return;
    V3 sum = v3(0, 0, 0);
    for (const V3 &p : m.v) sum = sum + p;
    const V3 cen = sum / (float)m.v.size();
    const float e = 0.5f * expansion, eps = 1e-9f;
    for (V3 &p : m.v) {
        V3 d = p - cen;
        if (std::fabs(d.x) < eps && std::fabs(d.y) < eps && std::fabs(d.z) < eps) continue;
        d = d / vlength(d);
        p = p + e * d;
    }
}

// MeshObject::getMeshLevelSet (meshobject.cpp:239-264) into `target` (union)
void obstacle_level_set(const Mesh &in, float expansion, int ni, int nj, int nk, double dx, Jitter &jit,
                        LevelSet &target) {
    // the static mesh at any frame time: v + f (v - v) (meshobject.cpp:158-177) turns -0 into +0
    Mesh m;
    std::vector<int> used(in.v.size(), -1);
    for (int x : in.t) used[x] = 0;
    for (size_t q = 0; q < in.v.size(); q++)   // TriangleMesh::removeExtraneousVertices
        if (used[q] == 0) { used[q] = (int)m.v.size(); m.v.push_back(in.v[q] + v3(0.0f, 0.0f, 0.0f)); }
    for (int x : in.t) m.t.push_back(used[x]);
    if (m.t.empty()) return;
    // islands inside or crossing the domain (meshobject.cpp:633-701)
    AB dom;
    dom.pos = v3(0, 0, 0);
    dom.w = ni * dx; dom.h = nj * dx; dom.d = nk * dx;
    std::vector<Mesh> islands;
    for (Mesh &isl : split_islands(m)) {
        if (isl.v.empty()) continue;
        AB ib = mesh_bounds(isl);
        if (dom.inside(ib.pos) && dom.inside(ib.maxp())) { islands.push_back(isl); continue; }
        AB x = intersection(dom, ib);
        if (x.w > 0.0 || x.h > 0.0 || x.d > 0.0) islands.push_back(isl);
    }
    const bool per_island = (int)islands.size() >= ISLAND_TRIGGER;
    if (per_island && std::fabs(expansion) >= 1e-9f)
        for (Mesh &isl : islands) expand_island(isl, expansion);
    std::vector<Mesh> parts = per_island ? islands : std::vector<Mesh>{m};
    for (const Mesh &part : parts) {   // _getMeshIslandLevelSet (meshobject.cpp:667-701)
        AB ib = mesh_bounds(part);
        I3 lo = to_index(ib.pos, dx), hi = to_index(ib.maxp(), dx);
        lo.i = (int)std::fmax(lo.i - EXACT_BAND, 0); lo.j = (int)std::fmax(lo.j - EXACT_BAND, 0);
        lo.k = (int)std::fmax(lo.k - EXACT_BAND, 0);
        hi.i = (int)std::fmin(hi.i + EXACT_BAND + 1, ni - 1); hi.j = (int)std::fmin(hi.j + EXACT_BAND + 1, nj - 1);
        hi.k = (int)std::fmin(hi.k + EXACT_BAND + 1, nk - 1);
        const int w = hi.i - lo.i, h = hi.j - lo.j, d = hi.k - lo.k;
        if (w <= 0 || h <= 0 || d <= 0) continue;
        LevelSet L(w, h, d, lo, dx);
        if (per_island) band_serial(L, part, EXACT_BAND);   // disableMultiThreading (meshobject.cpp:852)
        else band_blocks(L, part, EXACT_BAND);
        signs(L, part, jit);
        unite(target, L);
    }
}

Mesh box_mesh(int ni, int nj, int nk, double dx) {   // fluidsimulation.cpp:5175-5186 and the AABB mesh
    Domain dm{ni, nj, nk, dx};
    const Box b = boundary_box(dm);
    const V3 p = v3(b.px, b.py, b.pz);
    Mesh m;
    m.v = {d3(p.x, p.y, p.z), d3(p.x + b.w, p.y, p.z), d3(p.x + b.w, p.y, p.z + b.d), d3(p.x, p.y, p.z + b.d),
           d3(p.x, p.y + b.h, p.z), d3(p.x + b.w, p.y + b.h, p.z), d3(p.x + b.w, p.y + b.h, p.z + b.d),
           d3(p.x, p.y + b.h, p.z + b.d)};
    m.t = {0, 1, 2, 0, 2, 3, 4, 7, 6, 4, 6, 5, 0, 3, 7, 0, 7, 4, 1, 5, 6, 1, 6, 2, 0, 4, 5, 0, 5, 1, 3, 2, 6, 3, 6, 7};
    return m;
}

}  // namespace
}  // namespace oracle

using namespace oracle;

extern "C" {

// Solid level set of the closed domain and static mesh obstacles, nodes (ni+1)(nj+1)(nk+1)
// (FluidSimulation::_addStaticObjectsToSDF, fluidsimulation.cpp:5277-5333).  Object o has
// nverts[o] vertices (3 floats each, concatenated over the objects in `verts`), ntris[o]
// triangles (3 ints each, indices into its own vertices, concatenated in `tris`), flags[o]
// (bit0 inversed, bit1 disabled) and mesh expansion expansion[o].  jitter: 3 floats per inside
// test in call order (njitter of them), the fixed draw after that.
void oracle_solid_level_set(int ni, int nj, int nk, double dx, int nobj, const int *nverts, const int *ntris,
                            const float *verts, const int *tris, const int *flags, const float *expansion,
                            int njitter, const float *jitter, float *phi) {
    Jitter jit;
    jit.list = jitter; jit.n = njitter; jit.dx = dx;
    LevelSet dom(ni, nj, nk, I3{0, 0, 0}, dx);
    const Mesh box = box_mesh(ni, nj, nk, dx);
    band_blocks(dom, box, EXACT_BAND);
    signs(dom, box, jit);
    for (float &v : dom.phi) v = -v;
    std::vector<Mesh> meshes(nobj);
    size_t vo = 0, to = 0;
    for (int o = 0; o < nobj; o++) {
        for (int q = 0; q < nverts[o]; q++) meshes[o].v.push_back(v3(verts[3 * (vo + q)], verts[3 * (vo + q) + 1],
                                                                     verts[3 * (vo + q) + 2]));
        meshes[o].t.assign(tris + 3 * to, tris + 3 * (to + ntris[o]));
        vo += nverts[o];
        to += ntris[o];
    }
    for (int o = 0; o < nobj; o++) {
        if ((flags[o] & 2) || (flags[o] & 1)) continue;
        LevelSet tmp(ni, nj, nk, I3{0, 0, 0}, dx);
        obstacle_level_set(meshes[o], expansion[o], ni, nj, nk, dx, jit, tmp);
        unite(dom, tmp);
    }
    bool any_inv = false;
    for (int o = 0; o < nobj; o++) any_inv = any_inv || ((flags[o] & 1) && !(flags[o] & 2));
    if (any_inv) {
        LevelSet inv(ni, nj, nk, I3{0, 0, 0}, dx);
        for (int o = 0; o < nobj; o++) {
            if (!(flags[o] & 1) || (flags[o] & 2)) continue;
            LevelSet tmp(ni, nj, nk, I3{0, 0, 0}, dx);
            obstacle_level_set(meshes[o], expansion[o], ni, nj, nk, dx, jit, tmp);
            unite(inv, tmp);
        }
        for (float &v : inv.phi) v = -v;
        unite(dom, inv);
    }
    std::memcpy(phi, dom.phi.data(), dom.phi.size() * sizeof(float));
}

}  // extern "C"
