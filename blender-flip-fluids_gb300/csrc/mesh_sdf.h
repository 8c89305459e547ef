// Solid level set of static triangle-mesh obstacles, built on the GPU:
//   MeshLevelSet::fastCalculateSignedDistanceField (meshlevelset.cpp:572-601) -- exact distances
//     to the triangles in a band of 3 cells around each, the rest at the level set's upper bound,
//     then the sign from an odd count of +z line crossings (meshlevelset.cpp:1298-1318,
//     meshutils.cpp:57-245, 356-437);
//   MeshObject::getMeshLevelSet (meshobject.cpp:239-264): one level set over the whole mesh's box,
//     or one per mesh island (with the mesh expansion) when the mesh has 25 islands or more;
//   FluidSimulation::_addStaticObjectsToSDF (fluidsimulation.cpp:5277-5333): the negated level set
//     of the closed-domain box mesh, unioned (min) with the obstacles, the inverted ones negated.
// Vertex and triangle bookkeeping (islands, boxes, offsets) runs on the host; the band distances,
// the line crossings and the unions run as kernels.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "common.cuh"
#include "devbuf.h"

namespace ffgpu {

// A static obstacle (the C ABI's MeshObject): vertices (x, y, z floats) and triangles (three
// vertex indices each), with the switches the solid level set reads.
struct Obstacle {
    std::vector<float> v;
    std::vector<int> t;
    bool enabled = true, inversed = false;
    float expansion = 0.0f;      // MeshObject::setMeshExpansion (meshobject.cpp:389-391)
    float friction = 0.0f;       // stored for the API; the substep does not read it
    unsigned long long version = 1;   // changes with every edit of the mesh or the switches
};

class SolidBuilder {
public:
    // Writes the nodal solid level set ((ni+1)(nj+1)(nk+1), x fastest) of the closed domain and
    // the enabled obstacles into `solid` on stream st.  jitter: njitter triples, the +z line offsets
    // of the inside tests in the order they run; later tests use the fixed offset.  Returns the
    // kernels launched.
    int build(Dims d, double dx, const std::vector<const Obstacle *> &obstacles, float *solid, cudaStream_t st,
              const float *jitter = nullptr, int njitter = 0);

private:
    DevBuf<float> verts, part, inv;
    DevBuf<int> tris, col_count, col_off, col_cursor, scan_tmp;
    DevBuf<float> zs;
    DevBuf<unsigned char> mark;
    int launches = 0;
    int jitter_used = 0;
    const float *jitter_list = nullptr;
    int jitter_n = 0;
    struct Part;
    void level_set(const Part &p, cudaStream_t st);
    void next_jitter(double dx, float j[3]);
};

}  // namespace ffgpu
