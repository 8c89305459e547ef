// Golden-vector harness for the reference engine (test infrastructure only).
//
// Links the unmodified reference engine (oracle/_ref/libffengine.so, built by
// oracle/build_ref.sh from rlguy/Blender-FLIP-Fluids src/engine) and drives one
// FluidSimulation through the per-substep hot path, writing every intermediate
// grid and particle array as raw little-endian binary files.  The stage order
// replicates FluidSimulation::_stepFluid (src/engine/fluidsimulation.cpp:10078-10121)
// so intermediate state can be captured between stages; the trajectory mode calls
// the public FluidSimulation::update (fluidsimulation.cpp:10410) unchanged.
//
// Input file layout (little endian):
//   int32 n, int32 num_particles, int32 mode_flags (bit0: sphere obstacle),
//   int32 num_substeps, float64 dx, float64 dt, float64 pic_ratio, int32 cfl,
//   float64 sphere_cx, cy, cz, r,
//   float32 positions[3*num_particles], float32 velocities[3*num_particles],
//   with mode_flags bit1 (APIC transfer): float32 affine[9*num_particles] (x, y, z
//   component vectors per particle); with mode_flags bit2 (viscosity): float64 viscosity;
//   mode_flags bit3 dumps the surface curvature grid (no payload); mode_flags bit4 (surface
//   tension, implies bit3): float64 surface tension constant, used by the pressure solve;
//   mode_flags bit5 (CFL substepping): int32 min, int32 max time steps per frame (otherwise
//   both 1); mode_flags bit6 turns extreme-velocity removal on (no payload); mode_flags bit7
//   (pressure tolerance): float64 PCG tolerance (otherwise the engine's 1e-9); mode_flags bit8
//   (FFP3 fluid-particle output): int32 output flags (bit0..2 surface, boundary, interior
//   output, bit3 velocity, bit4 speed attribute), float64 output amount, uint16 ids[num_particles]
//   (loaded with the particles); the trajectory mode then dumps the frame's FFP3 data and the
//   particle ids after every update
//
// Mesh mode (solid level set of static mesh obstacles) reads its own layout:
//   int32 n, float64 dx, int32 num_objects, then per object int32 flags (bit0 inversed,
//   bit1 disabled), float32 mesh expansion, int32 num_vertices, int32 num_triangles,
//   float32 vertices[3*num_vertices], int32 triangles[3*num_triangles].
// In that mode the harness's rand() cycles through three fixed values, assigned so that the
// z-line jitter of every inside test (meshutils.cpp:95-114), jit + u (-jit - jit) with
// u = rand() / RAND_MAX and jit = 0.001 dx, takes u = MESH_RAND_X / RAND_MAX in x (and Y, Z
// likewise) whatever else used the C library's generator; the other modes forward rand() to
// the C library.
//
// Usage: ref_harness stages|traj|mesh|time <input.bin> <outdir>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <string>
#include <vector>
#include <map>
#include <set>
#include <queue>
#include <thread>
#include <mutex>
#include <sstream>
#include <fstream>
#include <iostream>
#include <algorithm>
#include <limits>
#include <random>
#include <functional>
#include <memory>
#include <condition_variable>
#include <atomic>
#include <chrono>
#include <dlfcn.h>

// Stage-level access to the engine's private members (test harness only).
#define private public
#define protected public
#include "fluidsimulation.h"
#include "meshobject.h"
#include "trianglemesh.h"
#include "pressuresolver.h"
#include "velocityadvector.h"
#include "viscositysolver.h"
#undef private
#undef protected

// rand() of the process (the engine's calls bind to this definition): 0 in mesh mode, else the
// C library's generator
static const int MESH_RAND_X = 536870912, MESH_RAND_Y = 1503238554, MESH_RAND_Z = 858993459;
static bool g_mesh_rand = false;
static int g_rand_cycle[3] = {0, 0, 0}, g_rand_at = 0;
static long g_rand_calls = 0;
extern "C" int rand(void) {
    g_rand_calls++;
    if (g_mesh_rand) { int r = g_rand_cycle[g_rand_at]; g_rand_at = (g_rand_at + 1) % 3; return r; }
    static int (*libc_rand)(void) = (int (*)(void))dlsym(RTLD_NEXT, "rand");
    return libc_rand();
}

struct Input {
    int n = 0, np = 0, flags = 0, substeps = 1;
    double dx = 0, dt = 0, pic = 0.05;
    int cfl = 5;
    double scx = 0, scy = 0, scz = 0, sr = 0;
    std::vector<float> pos, vel, aff;
    double visc = 0.0;
    double tension = 0.0;
    int min_steps = 1, max_steps = 1;
    double tolerance = 0.0;
    int threads = 1;   // engine threads (time mode: all)
    int ffp_flags = 0;
    double ffp_amount = 1.0;
    std::vector<uint16_t> ids;
};

static Input readInput(const char *path) {
    Input in;
    FILE *f = fopen(path, "rb");
    if (!f) { fprintf(stderr, "cannot open %s\n", path); exit(2); }
    auto rd = [&](void *p, size_t s) { if (fread(p, 1, s, f) != s) { fprintf(stderr, "short read\n"); exit(2); } };
    rd(&in.n, 4); rd(&in.np, 4); rd(&in.flags, 4); rd(&in.substeps, 4);
    rd(&in.dx, 8); rd(&in.dt, 8); rd(&in.pic, 8); rd(&in.cfl, 4);
    rd(&in.scx, 8); rd(&in.scy, 8); rd(&in.scz, 8); rd(&in.sr, 8);
    in.pos.resize(3 * (size_t)in.np); in.vel.resize(3 * (size_t)in.np);
    rd(in.pos.data(), 4 * in.pos.size()); rd(in.vel.data(), 4 * in.vel.size());
    if (in.flags & 2) {
        in.aff.resize(9 * (size_t)in.np);
        rd(in.aff.data(), 4 * in.aff.size());
    }
    if (in.flags & 4) rd(&in.visc, 8);
    if (in.flags & 16) rd(&in.tension, 8);
    if (in.flags & 32) { rd(&in.min_steps, 4); rd(&in.max_steps, 4); }
    if (in.flags & 128) rd(&in.tolerance, 8);
    if (in.flags & 256) {
        rd(&in.ffp_flags, 4);
        rd(&in.ffp_amount, 8);
        in.ids.resize((size_t)in.np);
        rd(in.ids.data(), 2 * in.ids.size());
    }
    fclose(f);
    return in;
}

static std::string g_out;
static void dump(const std::string &name, const void *data, size_t bytes) {
    std::string p = g_out + "/" + name + ".bin";
    FILE *f = fopen(p.c_str(), "wb");
    if (!f) { fprintf(stderr, "cannot write %s\n", p.c_str()); exit(2); }
    fwrite(data, 1, bytes, f);
    fclose(f);
}
static void dumpArrayF(const std::string &name, Array3d<float> &a) {
    std::vector<float> v((size_t)a.width * a.height * a.depth);
    for (int k = 0; k < a.depth; k++)
        for (int j = 0; j < a.height; j++)
            for (int i = 0; i < a.width; i++)
                v[(size_t)i + (size_t)a.width * (j + (size_t)a.height * k)] = a(i, j, k);
    dump(name, v.data(), v.size() * 4);
}
static void dumpArrayB(const std::string &name, Array3d<bool> &a) {
    std::vector<unsigned char> v((size_t)a.width * a.height * a.depth);
    for (int k = 0; k < a.depth; k++)
        for (int j = 0; j < a.height; j++)
            for (int i = 0; i < a.width; i++)
                v[(size_t)i + (size_t)a.width * (j + (size_t)a.height * k)] = a(i, j, k) ? 1 : 0;
    dump(name, v.data(), v.size());
}
static void dumpMAC(const std::string &prefix, MACVelocityField &m) {
    dumpArrayF(prefix + "_u", *m.getArray3dU());
    dumpArrayF(prefix + "_v", *m.getArray3dV());
    dumpArrayF(prefix + "_w", *m.getArray3dW());
}
static void dumpValid(const std::string &prefix, ValidVelocityComponentGrid &g) {
    dumpArrayB(prefix + "_validu", g.validU);
    dumpArrayB(prefix + "_validv", g.validV);
    dumpArrayB(prefix + "_validw", g.validW);
}
static void dumpParticles(const std::string &prefix, FluidSimulation &sim) {
    std::vector<vmath::vec3> *p, *v;
    sim._markerParticles.getAttributeValues("POSITION", p);
    sim._markerParticles.getAttributeValues("VELOCITY", v);
    dump(prefix + "_pos", p->data(), p->size() * 12);
    dump(prefix + "_vel", v->data(), v->size() * 12);
    if (sim.isVelocityTransferMethodAPIC()) {
        std::vector<vmath::vec3> *ax, *ay, *az;
        sim._markerParticles.getAttributeValues("AFFINEX", ax);
        sim._markerParticles.getAttributeValues("AFFINEY", ay);
        sim._markerParticles.getAttributeValues("AFFINEZ", az);
        std::vector<float> a(9 * ax->size());
        for (size_t i = 0; i < ax->size(); i++) {
            const vmath::vec3 c[3] = {ax->at(i), ay->at(i), az->at(i)};
            for (int q = 0; q < 3; q++) { a[9 * i + 3 * q] = c[q].x; a[9 * i + 3 * q + 1] = c[q].y; a[9 * i + 3 * q + 2] = c[q].z; }
        }
        dump(prefix + "_aff", a.data(), a.size() * 4);
    }
}

// Icosphere (subdivided icosahedron) used as the static sphere obstacle mesh.
static TriangleMesh makeIcosphere(double cx, double cy, double cz, double r, int subdiv) {
    const double t = (1.0 + std::sqrt(5.0)) / 2.0;
    std::vector<std::array<double, 3>> v = {
        {-1, t, 0}, {1, t, 0}, {-1, -t, 0}, {1, -t, 0}, {0, -1, t}, {0, 1, t},
        {0, -1, -t}, {0, 1, -t}, {t, 0, -1}, {t, 0, 1}, {-t, 0, -1}, {-t, 0, 1}};
    std::vector<std::array<int, 3>> f = {
        {0, 11, 5}, {0, 5, 1}, {0, 1, 7}, {0, 7, 10}, {0, 10, 11}, {1, 5, 9}, {5, 11, 4},
        {11, 10, 2}, {10, 7, 6}, {7, 1, 8}, {3, 9, 4}, {3, 4, 2}, {3, 2, 6}, {3, 6, 8},
        {3, 8, 9}, {4, 9, 5}, {2, 4, 11}, {6, 2, 10}, {8, 6, 7}, {9, 8, 1}};
    for (auto &p : v) { double l = std::sqrt(p[0]*p[0] + p[1]*p[1] + p[2]*p[2]); for (auto &c : p) c /= l; }
    for (int s = 0; s < subdiv; s++) {
        std::map<std::pair<int, int>, int> mid;
        auto midpoint = [&](int a, int b) {
            auto key = std::make_pair(std::min(a, b), std::max(a, b));
            auto it = mid.find(key);
            if (it != mid.end()) return it->second;
            std::array<double, 3> m = {(v[a][0] + v[b][0]) / 2, (v[a][1] + v[b][1]) / 2, (v[a][2] + v[b][2]) / 2};
            double l = std::sqrt(m[0]*m[0] + m[1]*m[1] + m[2]*m[2]);
            for (auto &c : m) c /= l;
            v.push_back(m);
            mid[key] = (int)v.size() - 1;
            return (int)v.size() - 1;
        };
        std::vector<std::array<int, 3>> nf;
        for (auto &tr : f) {
            int a = midpoint(tr[0], tr[1]), b = midpoint(tr[1], tr[2]), c = midpoint(tr[2], tr[0]);
            nf.push_back({tr[0], a, c}); nf.push_back({tr[1], b, a});
            nf.push_back({tr[2], c, b}); nf.push_back({a, b, c});
        }
        f = nf;
    }
    TriangleMesh m;
    for (auto &p : v) m.vertices.push_back(vmath::vec3(cx + r * p[0], cy + r * p[1], cz + r * p[2]));
    for (auto &tr : f) m.triangles.push_back(Triangle(tr[0], tr[1], tr[2]));
    return m;
}

static FluidSimulation *makeSim(const Input &in, MeshObject **obstacle) {
    FluidSimulation *sim = new FluidSimulation(in.n, in.n, in.n, in.dx);
    // One engine thread: the reference's marker-removal pass writes a shared
    // std::vector<bool> from several threads (meshlevelset.h:333-338), which can drop
    // removal flags under load.  A single thread makes every golden run deterministic;
    // no result on the path depends on the thread count below 500k pressure cells.
    if (in.threads > 0) sim->setMaxThreadCount(in.threads);
    sim->disableConsoleOutput();
    sim->disableSurfaceReconstruction();
    if (in.flags & 128) sim->_pressureSolveTolerance = in.tolerance;
    if (in.flags & 2) sim->setVelocityTransferMethodAPIC();
    else sim->setVelocityTransferMethodFLIP();
    sim->setPICFLIPRatio(in.pic);
    sim->setCFLConditionNumber(in.cfl);
    sim->setMinTimeStepsPerFrame(in.min_steps);
    sim->setMaxTimeStepsPerFrame(in.max_steps);
    if (in.flags & 64) sim->enableExtremeVelocityRemoval();
    else sim->disableExtremeVelocityRemoval();
    sim->addBodyForce(0.0, -9.81, 0.0);
    if (in.flags & 4) sim->setViscosity(in.visc);
    if (in.flags & 16) sim->setSurfaceTension(in.tension);
    if (in.flags & 256) {
        sim->enableFluidParticleOutput();
        if (in.ffp_flags & 1) sim->enableFluidParticleSurfaceOutput(); else sim->disableFluidParticleSurfaceOutput();
        if (in.ffp_flags & 2) sim->enableFluidParticleBoundaryOutput(); else sim->disableFluidParticleBoundaryOutput();
        if (in.ffp_flags & 4) sim->enableFluidParticleInteriorOutput(); else sim->disableFluidParticleInteriorOutput();
        if (in.ffp_flags & 8) sim->enableFluidParticleVelocityAttribute();
        if (in.ffp_flags & 16) sim->enableFluidParticleSpeedAttribute();
        sim->setFluidParticleOutputAmount(in.ffp_amount);
    }
    *obstacle = nullptr;
    if (in.flags & 1) {
        MeshObject *ob = new MeshObject(in.n, in.n, in.n, in.dx);
        ob->updateMeshStatic(makeIcosphere(in.scx, in.scy, in.scz, in.sr, 4));
        sim->addMeshObstacle(ob);
        *obstacle = ob;
    }
    FluidSimulationMarkerParticleData d;
    d.size = in.np;
    d.positions = (char *)in.pos.data();
    d.velocities = (char *)in.vel.data();
    sim->loadMarkerParticleData(d);
    std::vector<vmath::vec3> affx, affy, affz;
    if (in.flags & 2) {
        for (int i = 0; i < in.np; i++) {
            affx.push_back(vmath::vec3(in.aff[9 * i], in.aff[9 * i + 1], in.aff[9 * i + 2]));
            affy.push_back(vmath::vec3(in.aff[9 * i + 3], in.aff[9 * i + 4], in.aff[9 * i + 5]));
            affz.push_back(vmath::vec3(in.aff[9 * i + 6], in.aff[9 * i + 7], in.aff[9 * i + 8]));
        }
        FluidSimulationMarkerParticleAffineData a;
        a.size = in.np;
        a.affineX = (char *)affx.data();
        a.affineY = (char *)affy.data();
        a.affineZ = (char *)affz.data();
        sim->loadMarkerParticleAffineData(a);
    }
    if (in.flags & 256) {
        FluidSimulationMarkerParticleIDData idd;
        idd.size = in.np;
        idd.id = (char *)in.ids.data();
        sim->loadMarkerParticleIDData(idd);
    }
    sim->initialize();
    return sim;
}

// One substep, stage by stage (fluidsimulation.cpp:10078-10121), with dumps.
static void runStages(const Input &in) {
    MeshObject *ob;
    FluidSimulation *simp = makeSim(in, &ob);
    FluidSimulation &sim = *simp;
    dumpParticles("p0", sim);
    double dt = in.dt;
    // Bookkeeping normally done by update() (fluidsimulation.cpp:10410-10470).
    sim._currentFrameDeltaTime = dt;
    sim._currentFrameDeltaTimeRemaining = 0.0;
    sim._currentFrameTimeStep = dt;
    sim._currentFrameTimeStepNumber = 0;
    sim._isSkippedFrame = false;
    sim._isLastFrameTimeStep = true;

    sim._updateObstacleObjects(dt);
    dumpArrayF("solid_phi", sim._solidSDF._phi);
    dumpArrayB("near_solid", sim._nearSolidGrid);

    sim._updateLiquidLevelSet();
    dumpArrayF("liquid_phi_raw", *sim._liquidSDF.getPhiGrid());
    sim._liquidSDF.postProcessSignedDistanceField(sim._solidSDF);
    dumpArrayF("liquid_phi", *sim._liquidSDF.getPhiGrid());
    Array3d<float> curvature(in.n, in.n, in.n, 0.0f);
    if (in.flags & 24) {   // ParticleLevelSet::calculateCurvatureGrid (particlelevelset.cpp:196-291)
        // LevelSetSolver::reinitializeUpwind reads its temporary grid (allocated with new float[],
        // never filled, levelsetsolver.cpp:95) outside the solver band from the second iteration
        // on; in this single-threaded call sequence the allocator hands it a freed copy of the
        // input level set, so the dump is deterministic.
        Array3d<float> surf(in.n, in.n, in.n, 0.0f);
        sim._liquidSDF.calculateCurvatureGrid(surf, curvature);
        dumpArrayF("surface_phi", surf);
        dumpArrayF("curvature", curvature);
    }

    // _advectVelocityField (fluidsimulation.cpp:5623-5661), split to expose P2G.
    sim._validVelocities.reset();
    sim._MACVelocity.clear();
    {
        VelocityAdvectorParameters params;
        params.particles = &sim._markerParticles;
        params.vfield = &sim._MACVelocity;
        params.validVelocities = &sim._validVelocities;
        params.particleRadius = sim._liquidSDFParticleRadius;
        params.velocityTransferMethod = (in.flags & 2) ? VelocityAdvectorTransferMethod::APIC
                                                        : VelocityAdvectorTransferMethod::FLIP;
        sim._velocityAdvector.advect(params);
    }
    dumpMAC("p2g", sim._MACVelocity);
    dumpValid("p2g", sim._validVelocities);
    sim._extrapolateFluidVelocities(sim._MACVelocity, sim._validVelocities);
    dumpMAC("adv", sim._MACVelocity);

    sim._saveVelocityField();
    sim._applyBodyForcesToVelocityField(dt);
    dumpMAC("body", sim._MACVelocity);

    // _applyViscosityToVelocityField (fluidsimulation.cpp:5983-6064), split to expose the
    // viscosity solver's volume grids, linear system, MIC(0) factor and solution
    // (viscositysolver.cpp:53-80).
    if (in.flags & 4) {
        sim._constrainVelocityField(sim._MACVelocity);
        dumpMAC("visc_in", sim._MACVelocity);
        ViscositySolverParameters params;
        params.cellwidth = sim._dx;
        params.deltaTime = dt;
        params.velocityField = &sim._MACVelocity;
        params.liquidSDF = &sim._liquidSDF;
        params.solidSDF = &sim._solidSDF;
        params.viscosity = &sim._viscosity;
        params.errorTolerance = sim._viscositySolverErrorTolerance;
        params.maxIterations = sim._maxViscositySolveIterations;
        ViscositySolver vs;
        vs._initialize(params);
        vs._computeFaceStateGrid();
        vs._computeVolumeGrid();
        vs._computeMatrixIndexTable();
        dumpArrayF("visc_vol_center", vs._volumes.center);
        dumpArrayF("visc_vol_u", vs._volumes.U);
        dumpArrayF("visc_vol_v", vs._volumes.V);
        dumpArrayF("visc_vol_w", vs._volumes.W);
        dumpArrayF("visc_vol_eu", vs._volumes.edgeU);
        dumpArrayF("visc_vol_ev", vs._volumes.edgeV);
        dumpArrayF("visc_vol_ew", vs._volumes.edgeW);
        dump("visc_index", vs._matrixIndex.indexTable.data(), vs._matrixIndex.indexTable.size() * 4);
        int matsize = vs._matrixIndex.matrixSize;
        int vstats[3] = {matsize, 0, 0};
        float verr = 0.0f;
        if (matsize > 0) {
            SparseMatrixf matrix(matsize, 15);
            std::vector<float> rhs(matsize, 0), soln(matsize, 0);
            vs._initializeLinearSystem(matrix, rhs);
            FixedSparseMatrix<float> fm;
            fm.fromMatrix(matrix);
            dump("visc_rowstart", fm.rowstart.data(), fm.rowstart.size() * 4);
            dump("visc_col", fm.colindex.data(), fm.colindex.size() * 4);
            dump("visc_val", fm.value.data(), fm.value.size() * 4);
            dump("visc_rhs", rhs.data(), rhs.size() * 4);
            SparseColumnLowerFactor<float> ic;
            factorModifiedIncompleteColesky0(matrix, ic);
            dump("visc_ic_invdiag", ic.invdiag.data(), ic.invdiag.size() * 4);
            dump("visc_ic_colstart", ic.colstart.data(), ic.colstart.size() * 4);
            dump("visc_ic_rowindex", ic.rowindex.data(), ic.rowindex.size() * 4);
            dump("visc_ic_value", ic.value.data(), ic.value.size() * 4);
            bool ok = vs._solveLinearSystem(matrix, rhs, soln);
            dump("visc_soln", soln.data(), soln.size() * 4);
            vstats[1] = vs.getIterations();
            vstats[2] = ok ? 1 : 0;
            verr = vs.getError();
            if (ok) vs._applySolutionToVelocityField(soln);
        }
        dump("visc_stats", vstats, sizeof(vstats));
        dump("visc_error", &verr, 4);
        dumpMAC("visc", sim._MACVelocity);
    }

    // _pressureSolve (fluidsimulation.cpp:6152-6280), split to expose the pressure grid.
    sim._updateWeightGrid();
    dumpArrayF("weight_u", sim._weightGrid.U);
    dumpArrayF("weight_v", sim._weightGrid.V);
    dumpArrayF("weight_w", sim._weightGrid.W);
    {
        Array3d<float> densityGrid(in.n, in.n, in.n, 1.0f);
        Array3d<float> pressureGrid(in.n, in.n, in.n, 0.0f);
        PressureSolverParameters params;
        params.cellwidth = sim._dx;
        params.deltaTime = dt;
        params.tolerance = sim._pressureSolveTolerance;
        params.acceptableTolerance = sim._pressureSolveAcceptableTolerance;
        params.maxIterations = sim._maxPressureSolveIterations;
        params.velocityFieldFluid = &sim._MACVelocity;
        params.velocityFieldSolid = &(sim._solidSDF.getVelocityDataGrid()->field);
        params.validVelocities = &sim._validVelocities;
        params.liquidSDF = sim._liquidSDF.getPhiGrid();
        params.weightGrid = &sim._weightGrid;
        params.pressureGrid = &pressureGrid;
        params.densityGrid = &densityGrid;
        params.isSurfaceTensionEnabled = (in.flags & 16) != 0;
        params.surfaceTensionConstant = in.tension;
        params.curvatureGrid = &curvature;
        // the solid velocity field (MAC) around the solve: the largest |u|, |v|, |w| before and after,
        // which shows what PressureSolver::_conditionSolidVelocityField (pressuresolver.cpp:161-288)
        // changed in it
        auto absmax = [&](float out[3]) {
            MACVelocityField &f = sim._solidSDF.getVelocityDataGrid()->field;
            out[0] = out[1] = out[2] = 0.0f;
            for (int k = 0; k < in.n; k++)
                for (int j = 0; j < in.n; j++)
                    for (int i = 0; i <= in.n; i++) {
                        out[0] = std::max(out[0], std::fabs(f.U(i, j, k)));
                        out[1] = std::max(out[1], std::fabs(f.V(j, i, k)));
                        out[2] = std::max(out[2], std::fabs(f.W(j, k, i)));
                    }
        };
        float solid_vel[6];
        absmax(solid_vel);
        PressureSolver psolver;
        bool success = psolver.solve(params);
        if (success) psolver.applySolutionToVelocityField();
        absmax(solid_vel + 3);
        dump("solid_velocity_absmax", solid_vel, sizeof(solid_vel));
        dumpArrayF("pressure", pressureGrid);
        int stats[2] = {psolver.getIterations(), success ? 1 : 0};
        float err = psolver.getError();
        dump("pressure_iters", stats, sizeof(stats));
        dump("pressure_error", &err, 4);
        dumpMAC("proj", sim._MACVelocity);
        dumpValid("proj", sim._validVelocities);
        sim._extrapolateFluidVelocities(sim._MACVelocity, sim._validVelocities);
        dumpMAC("projx", sim._MACVelocity);
    }

    sim._constrainVelocityFields();
    dumpMAC("cons", sim._MACVelocity);
    dumpMAC("saved", sim._savedVelocityField);

    sim._updateMarkerParticleVelocities();
    dumpParticles("g2p", sim);

    // RK3 + collision (fluidsimulation.cpp:7853-7904) before removal.
    {
        std::vector<vmath::vec3> *positions;
        sim._markerParticles.getAttributeValues("POSITION", positions);
        std::vector<vmath::vec3> copy = *positions;
        std::vector<vmath::vec3> out(copy.size());
        sim._advanceMarkerParticlesThread(dt, 0, (int)copy.size(), &copy, &out);
        dump("adv_pos", out.data(), out.size() * 12);
    }
    sim._deleteSavedVelocityField();
    if (in.flags & 64) {   // the speed limit the removal below applies (fluidsimulation.cpp:7723-7771)
        float limit = sim._getMarkerParticleSpeedLimit(sim._currentFrameDeltaTime);
        dump("speed_limit", &limit, 4);
    }
    sim._advanceMarkerParticles(dt);
    dumpParticles("p1", sim);
    delete simp;
    delete ob;
}

static void runTraj(const Input &in) {
    MeshObject *ob;
    FluidSimulation *sim = makeSim(in, &ob);
    std::vector<double> stats, steps, dts;
    for (int s = 0; s < in.substeps; s++) {
        sim->update(in.dt);
        if (s == 0) dumpArrayF("solid_phi", sim->_solidSDF._phi);
        FluidSimulationFrameStats fs = sim->getFrameStatsData();
        stats.push_back(fs.fluidParticles);
        stats.push_back(fs.pressureSolverIterations);
        stats.push_back(fs.pressureSolverError);
        stats.push_back(fs.pressureSolverSuccess);
        // substeps of this update and the exact length of its last one
        steps.push_back(fs.substeps);
        steps.push_back(sim->_currentFrameTimeStep);
        // every substep's length as the engine logged it ("Substep Time: <t>s", 6 digits,
        // fluidsimulation.cpp:10474-10483); the log is flushed into the output once per update
        std::string log(sim->_outputData.logfileData.begin(), sim->_outputData.logfileData.end());
        const std::string key = "Substep Time: ";
        for (size_t at = log.find(key); at != std::string::npos; at = log.find(key, at + 1))
            dts.push_back(std::atof(log.c_str() + at + key.size()));
        char name[64];
        snprintf(name, sizeof(name), "traj%03d", s + 1);
        dumpParticles(name, *sim);
        if (in.flags & 256) {
            const std::string pre(name);
            std::vector<uint16_t> *ids;
            sim->_markerParticles.getAttributeValues("ID", ids);
            dump(pre + "_ids", ids->data(), ids->size() * 2);
            auto out = [&](const char *tag, const std::vector<char> &v) { dump(pre + tag, v.data(), v.size()); };
            out("_ffp_pos", sim->_outputData.fluidParticleData);
            out("_ffp_id", sim->_outputData.fluidParticleIDAttributeData);
            if (in.ffp_flags & 8) out("_ffp_vel", sim->_outputData.fluidParticleVelocityAttributeData);
            if (in.ffp_flags & 16) out("_ffp_speed", sim->_outputData.fluidParticleSpeedAttributeData);
        }
    }
    dump("traj_stats", stats.data(), stats.size() * 8);
    dump("traj_steps", steps.data(), steps.size() * 8);
    dump("traj_dts", dts.data(), dts.size() * 8);
    delete sim;
    delete ob;
}

// Solid level set of the domain and static mesh obstacles after the first obstacle update
// (fluidsimulation.cpp:5387-5425).
static void runMesh(const char *path) {
    FILE *f = fopen(path, "rb");
    if (!f) { fprintf(stderr, "cannot open %s\n", path); exit(2); }
    auto rd = [&](void *p, size_t sz) { if (fread(p, 1, sz, f) != sz) { fprintf(stderr, "short read\n"); exit(2); } };
    int n = 0, nobj = 0;
    double dx = 0.0;
    rd(&n, 4); rd(&dx, 8); rd(&nobj, 4);
    FluidSimulation *sim = new FluidSimulation(n, n, n, dx);
    sim->setMaxThreadCount(1);
    sim->disableConsoleOutput();
    sim->disableSurfaceReconstruction();
    std::vector<MeshObject *> obs;
    for (int o = 0; o < nobj; o++) {
        int flags = 0, nv = 0, nt = 0;
        float expansion = 0.0f;
        rd(&flags, 4); rd(&expansion, 4); rd(&nv, 4); rd(&nt, 4);
        std::vector<float> v(3 * (size_t)nv);
        std::vector<int> t(3 * (size_t)nt);
        rd(v.data(), 4 * v.size()); rd(t.data(), 4 * t.size());
        TriangleMesh m;
        for (int q = 0; q < nv; q++) m.vertices.push_back(vmath::vec3(v[3 * q], v[3 * q + 1], v[3 * q + 2]));
        for (int q = 0; q < nt; q++) m.triangles.push_back(Triangle(t[3 * q], t[3 * q + 1], t[3 * q + 2]));
        MeshObject *ob = new MeshObject(n, n, n, dx);
        ob->updateMeshStatic(m);
        if (flags & 1) ob->inverse();
        if (flags & 2) ob->disable();
        ob->setMeshExpansion(expansion);
        sim->addMeshObstacle(ob);
        obs.push_back(ob);
    }
    fclose(f);
    // one marker particle: the solid level set is only built once there is liquid
    float p[3] = {(float)(0.5 * n * dx), (float)(0.5 * n * dx), (float)(0.5 * n * dx)}, vel[3] = {0, 0, 0};
    FluidSimulationMarkerParticleData d;
    d.size = 1;
    d.positions = (char *)p;
    d.velocities = (char *)vel;
    sim->loadMarkerParticleData(d);
    // the order in which this compiler evaluates the three draws of a vec3 built from three
    // calls, as meshutils.cpp:110-114 builds the jitter: the draw that lands in x gets MESH_RAND_X
    static int probe_calls = 0;
    auto probe = [](double, double) { return (double)probe_calls++; };
    vmath::vec3 order(probe(1.0, -1.0), probe(1.0, -1.0), probe(1.0, -1.0));
    g_rand_cycle[(int)order.x] = MESH_RAND_X;
    g_rand_cycle[(int)order.y] = MESH_RAND_Y;
    g_rand_cycle[(int)order.z] = MESH_RAND_Z;
    const double jit = 0.001 * dx;
    const float jitter[3] = {(float)(jit + ((double)MESH_RAND_X / (double)RAND_MAX) * (-jit - jit)),
                             (float)(jit + ((double)MESH_RAND_Y / (double)RAND_MAX) * (-jit - jit)),
                             (float)(jit + ((double)MESH_RAND_Z / (double)RAND_MAX) * (-jit - jit))};
    const float draw_order[3] = {order.x, order.y, order.z};
    dump("jitter", jitter, sizeof(jitter));
    dump("draw_order", draw_order, sizeof(draw_order));
    g_mesh_rand = true;
    g_rand_at = 0;
    g_rand_calls = 0;
    sim->initialize();
    const double dt = 1.0 / 240.0;
    sim->_currentFrameDeltaTime = dt;
    sim->_currentFrameDeltaTimeRemaining = 0.0;
    sim->_currentFrameTimeStep = dt;
    sim->_currentFrameTimeStepNumber = 0;
    sim->_isSkippedFrame = false;
    sim->_isLastFrameTimeStep = true;
    sim->_updateObstacleObjects(dt);
    dumpArrayF("solid_phi", sim->_solidSDF._phi);
    dump("rand_calls", &g_rand_calls, 8);
    delete sim;
    for (MeshObject *ob : obs) delete ob;
}

// Wall time of each update() with the engine's default thread count (the reference's own
// throughput on this host's cores): one JSON line on stdout.
static void runTime(Input in) {
    in.threads = 0;
    MeshObject *ob;
    FluidSimulation *sim = makeSim(in, &ob);
    std::vector<double> secs;
    int iters = 0;
    for (int s = 0; s < in.substeps; s++) {
        auto t0 = std::chrono::steady_clock::now();
        sim->update(in.dt);
        secs.push_back(std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
        iters = sim->getFrameStatsData().pressureSolverIterations;
    }
    printf("{\"update_s\": [");
    for (size_t q = 0; q < secs.size(); q++) printf("%s%.4f", q ? ", " : "", secs[q]);
    printf("], \"threads\": %d, \"particles\": %d, \"last_pressure_iterations\": %d}\n",
           (int)std::thread::hardware_concurrency(), (int)sim->getNumMarkerParticles(), iters);
    delete sim;
    delete ob;
}

int main(int argc, char **argv) {
    if (argc != 4) {
        fprintf(stderr, "usage: %s stages|traj|mesh|time <input.bin> <outdir>\n", argv[0]);
        return 2;
    }
    g_out = argv[3];
    if (std::string(argv[1]) == "mesh") { runMesh(argv[2]); return 0; }
    Input in = readInput(argv[2]);
    if (std::string(argv[1]) == "stages") runStages(in);
    else if (std::string(argv[1]) == "traj") runTraj(in);
    else if (std::string(argv[1]) == "time") runTime(in);
    else { fprintf(stderr, "unknown mode\n"); return 2; }
    return 0;
}
