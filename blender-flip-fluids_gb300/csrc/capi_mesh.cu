// C ABI, part 3: mesh obstacles -- the MeshObject_* calls of the reference
// (src/engine/c_bindings/meshobject_c.cpp) that a static obstacle needs, and
// FluidSimulation_add/remove_mesh_obstacle(s) (fluidsimulation_c.cpp:3113-3134).  The mesh is
// copied on update; the solid level set is rebuilt on the GPU before the next substep.
#include <cstring>
#include <string>
#include <vector>

#include "capi_internal.h"

using namespace ffgpu;

namespace {

MeshObject &M(MeshObject *o) {
    if (!o) throw std::invalid_argument("Error: MeshObject handle is null.\n");
    return *o;
}

// MeshUtils::structToTriangleMesh (meshutils.cpp:36-55), with the indices checked
void copy_mesh(const TriangleMesh_t &m, Obstacle &ob) {
    if (m.numVertices < 0 || m.numTriangles < 0) throw std::domain_error("Error: negative mesh size.\n");
    if ((m.numVertices > 0 && !m.vertices) || (m.numTriangles > 0 && !m.triangles))
        throw std::invalid_argument("Error: mesh data pointer is null.\n");
    for (long long q = 0; q < 3LL * m.numTriangles; q++)
        if (m.triangles[q] < 0 || m.triangles[q] >= m.numVertices)
            throw std::out_of_range("Error: triangle vertex index out of range.\nindex: " + std::to_string(m.triangles[q]) +
                                    "\n");
    ob.v.assign(m.vertices, m.vertices + 3 * (size_t)m.numVertices);
    ob.t.assign(m.triangles, m.triangles + 3 * (size_t)m.numTriangles);
    ob.version++;
}

}  // namespace

extern "C" {

MeshObject *MeshObject_new(int i, int j, int k, double dx, int *err) {
    return guarded(err, [&]() -> MeshObject * {
        MeshObject *o = new MeshObject();
        o->ni = i; o->nj = j; o->nk = k; o->dx = dx;
        return o;
    });
}

void MeshObject_destroy(MeshObject *obj) { delete obj; }

void MeshObject_update_mesh_static(MeshObject *obj, TriangleMesh_t mesh_data, int *err) {
    guarded(err, [&] { copy_mesh(mesh_data, M(obj).ob); });
}

void MeshObject_update_mesh_animated(MeshObject *obj, TriangleMesh_t, TriangleMesh_t, TriangleMesh_t, int *err) {
    guarded(err, [&] {
        M(obj);
        throw std::runtime_error("Error: animated mesh obstacles are not part of the GB300 substep library.\n");
    });
}

void MeshObject_enable(MeshObject *obj, int *err) {
    guarded(err, [&] { Obstacle &o = M(obj).ob; if (!o.enabled) { o.enabled = true; o.version++; } });
}

void MeshObject_disable(MeshObject *obj, int *err) {
    guarded(err, [&] { Obstacle &o = M(obj).ob; if (o.enabled) { o.enabled = false; o.version++; } });
}

int MeshObject_is_enabled(MeshObject *obj, int *err) {
    return guarded(err, [&] { return M(obj).ob.enabled ? 1 : 0; });
}

void MeshObject_inverse(MeshObject *obj, int *err) {   // toggles (meshobject.cpp:332-334)
    guarded(err, [&] { Obstacle &o = M(obj).ob; o.inversed = !o.inversed; o.version++; });
}

int MeshObject_is_inversed(MeshObject *obj, int *err) {
    return guarded(err, [&] { return M(obj).ob.inversed ? 1 : 0; });
}

float MeshObject_get_friction(MeshObject *obj, int *err) {
    return guarded(err, [&] { return M(obj).ob.friction; });
}

void MeshObject_set_friction(MeshObject *obj, float f, int *err) {   // clamped to [0, 1] (meshobject.cpp:340-344)
    guarded(err, [&] { M(obj).ob.friction = std::fmax(std::fmin(f, 1.0f), 0.0f); });
}

float MeshObject_get_mesh_expansion(MeshObject *obj, int *err) {
    return guarded(err, [&] { return M(obj).ob.expansion; });
}

void MeshObject_set_mesh_expansion(MeshObject *obj, float ex, int *err) {
    guarded(err, [&] { Obstacle &o = M(obj).ob; o.expansion = ex; o.version++; });
}

void FluidSimulation_add_mesh_obstacle(FluidSimulation *obj, MeshObject *obstacle, int *err) {
    guarded(err, [&] { E(obj).add_obstacle(&M(obstacle).ob); });
}

void FluidSimulation_remove_mesh_obstacle(FluidSimulation *obj, MeshObject *obstacle, int *err) {
    guarded(err, [&] { E(obj).remove_obstacle(&M(obstacle).ob); });
}

void FluidSimulation_remove_mesh_obstacles(FluidSimulation *obj, int *err) {
    guarded(err, [&] { E(obj).remove_obstacles(); });
}

void ffgpu_solid_level_set(int ni, int nj, int nk, double dx, int nobj, const int *nverts, const int *ntris,
                           const float *verts, const int *tris, const int *flags, const float *expansion,
                           int njitter, const float *jitter, float *phi, int *err) {
    guarded(err, [&] {
        if (ni < 1 || nj < 1 || nk < 1 || !(dx > 0.0)) throw std::domain_error("Error: bad grid dimensions.\n");
        if (nobj < 0 || njitter < 0) throw std::domain_error("Error: negative count.\n");
        std::vector<Obstacle> obs(nobj);
        size_t vo = 0, to = 0;
        for (int o = 0; o < nobj; o++) {
            TriangleMesh_t m{const_cast<float *>(verts + 3 * vo), const_cast<int *>(tris + 3 * to), nverts[o], ntris[o]};
            copy_mesh(m, obs[o]);
            obs[o].inversed = (flags[o] & 1) != 0;
            obs[o].enabled = (flags[o] & 2) == 0;
            obs[o].expansion = expansion[o];
            vo += nverts[o];
            to += ntris[o];
        }
        std::vector<const Obstacle *> ptrs;
        for (const Obstacle &o : obs) ptrs.push_back(&o);
        const size_t nn = (size_t)(ni + 1) * (nj + 1) * (nk + 1);
        cudaStream_t st;
        FFGPU_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        try {
            SolidBuilder b;
            DevBuf<float> out;
            out.reserve(nn);
            b.build(Dims{ni, nj, nk}, dx, ptrs, out, st, jitter, njitter);
            FFGPU_CUDA(cudaMemcpyAsync(phi, out.p, nn * sizeof(float), cudaMemcpyDeviceToHost, st));
            FFGPU_CUDA(cudaStreamSynchronize(st));
        } catch (...) {
            cudaStreamDestroy(st);
            throw;
        }
        FFGPU_CUDA(cudaStreamDestroy(st));
    });
}

}  // extern "C"
