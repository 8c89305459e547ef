// CPU oracle for the FLIP substep hot path -- TEST INFRASTRUCTURE ONLY.
//
// A from-scratch restatement, in plain C++, of the reference engine's per-substep
// algorithm (rlguy/Blender-FLIP-Fluids 1.8.5, src/engine).  Every function cites the
// reference file:line it follows.  It is pinned against golden vectors produced by the
// reference engine itself (tests/golden/, generated by tests/golden/make_golden.py from
// oracle/ref_harness.cpp).  Only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline may load it; the product library never links or calls it.
//
// Float semantics follow the reference's x86-64 build: float arithmetic where the
// reference uses float, double where it uses double, no FMA contraction
// (compile with -ffp-contract=off).
#pragma once
#include <cstddef>
#include <cstdint>
#include <vector>

namespace oracle {

struct V3 { float x, y, z; };

inline V3 v3(float x, float y, float z) { V3 r; r.x = x; r.y = y; r.z = z; return r; }
inline V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator*(float s, V3 a) { return v3(s * a.x, s * a.y, s * a.z); }
// vmath.cpp:100-103: multiply by the float reciprocal computed in double
inline V3 operator/(V3 a, float s) { float inv = (float)(1.0 / s); return v3(a.x * inv, a.y * inv, a.z * inv); }
float vlength(V3 a);   // sqrt((x*x + y*y) + z*z) in float (vmath.h:85-91)

inline size_t flat(int i, int j, int k, int w, int h) {
    return (size_t)i + (size_t)w * ((size_t)j + (size_t)h * (size_t)k);
}

// Dense float grid, x fastest (array3d.h:774-777).
struct Grid {
    int w = 0, h = 0, d = 0;
    float *data = nullptr;
    bool in(int i, int j, int k) const { return i >= 0 && j >= 0 && k >= 0 && i < w && j < h && k < d; }
    float &at(int i, int j, int k) { return data[flat(i, j, k, w, h)]; }
    float at(int i, int j, int k) const { return data[flat(i, j, k, w, h)]; }
};

struct Domain {
    int ni, nj, nk;
    double dx;
};

// Axis-aligned box with the reference's mixed float/double members (aabb.h):
// float corner, double extents.
struct Box {
    float px, py, pz;
    double w, h, d;
    bool inside(V3 p) const;
    V3 nearest_inside(V3 p) const;   // aabb.cpp:501-518, eps 1e-6
};
Box boundary_box(const Domain &dm);     // fluidsimulation.cpp:5175-5180 (expand = shift by half)
Box expand(Box b, double v);            // aabb.cpp:122-128

// Nodal solid-phi helpers (meshlevelset.cpp:261, interpolation.cpp:75-110, 200-260)
float solid_trilinear(const Grid &phi, double dx, V3 p);
V3 solid_gradient(const Grid &phi, double dx, V3 p);

}  // namespace oracle
