// C ABI, part 2: GB300 extensions (no counterpart in the reference) and stage-level
// functions that run one kernel group on host arrays.  The stage functions build a
// scratch engine of the requested size, copy the inputs to the device, run the stage
// and copy the outputs back: they exist so that each kernel group can be checked
// against the CPU oracle on identical inputs.
#include <cstring>
#include <limits>
#include <memory>
#include <vector>

#include "capi_internal.h"

namespace ffgpu {

void launch_deinterleave(int np, const float *aos, float *x, float *y, float *z, cudaStream_t st);
void launch_interleave(int np, const float *x, const float *y, const float *z, float *aos, cudaStream_t st);

static void h2d(void *dst, const void *src, size_t bytes, cudaStream_t st) {
    FFGPU_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st));
}
static void d2h(void *dst, const void *src, size_t bytes, cudaStream_t st) {
    FFGPU_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st));
    FFGPU_CUDA(cudaStreamSynchronize(st));
}

static void check_dims(int ni, int nj, int nk, double dx) {
    if (ni < 1 || nj < 1 || nk < 1 || !(dx > 0))
        throw std::domain_error("Error: grid dimensions and cell size must be positive.\n");
}

// scratch engine with grids allocated and particles loaded (interleaved host arrays)
static std::unique_ptr<Engine> scratch(int ni, int nj, int nk, double dx, int np, const float *pos, const float *vel) {
    check_dims(ni, nj, nk, dx);
    if (np < 0) throw std::domain_error("Error: particle count must be non-negative.\n");
    auto e = std::make_unique<Engine>(ni, nj, nk, dx);
    e->initialize();
    if (np > 0) {
        std::vector<float> zero;
        if (!vel) { zero.assign(3 * (size_t)np, 0.0f); vel = zero.data(); }
        e->set_particles(pos, vel, np);
    }
    return e;
}

// 9 floats per particle (component c's affine vector at 3c .. 3c+2) <-> three xyz arrays
static void split_affine(int np, const float *aff9, std::vector<float> (&a)[3]) {
    for (int c = 0; c < 3; c++) {
        a[c].resize(3 * (size_t)np);
        for (int p = 0; p < np; p++)
            for (int e = 0; e < 3; e++) a[c][3 * (size_t)p + e] = aff9[9 * (size_t)p + 3 * c + e];
    }
}

static void read_affine9(const Engine &e, int np, float *aff9) {
    std::vector<float> a(3 * (size_t)np);
    for (int c = 0; c < 3; c++) {
        if (np) e.get_affine(c, a.data(), 0, np);
        for (int p = 0; p < np; p++)
            for (int k = 0; k < 3; k++) aff9[9 * (size_t)p + 3 * c + k] = a[3 * (size_t)p + k];
    }
}

// scratch engine with the APIC transfer and particles carrying affine vectors
static std::unique_ptr<Engine> scratch_apic(int ni, int nj, int nk, double dx, int np, const float *pos,
                                            const float *vel, const float *aff9) {
    check_dims(ni, nj, nk, dx);
    if (np < 0) throw std::domain_error("Error: particle count must be non-negative.\n");
    auto e = std::make_unique<Engine>(ni, nj, nk, dx);
    e->apic = true;
    e->initialize();
    if (np > 0) {
        std::vector<float> a[3];
        split_affine(np, aff9, a);
        const float *a3[3] = {a[0].data(), a[1].data(), a[2].data()};
        e->set_particles(pos, vel, np, a3);
    }
    return e;
}
}  // namespace ffgpu

using namespace ffgpu;

extern "C" {

void FluidSimulation_gb300_set_pressure_solver_mode(FluidSimulation *obj, int mode, int *err) {
    guarded(err, [&] {
        if (mode != 0 && mode != 1) throw std::domain_error("Error: solver mode must be 0 (FP64) or 1 (mixed).\n");
        E(obj).solver = mode == 0 ? SOLVER_FP64 : SOLVER_MIXED;
    });
}

void FluidSimulation_gb300_set_mixed_inner_tolerance(FluidSimulation *obj, double rel, int *err) {
    guarded(err, [&] {
        if (!(rel > 0 && rel < 1)) throw std::domain_error("Error: inner tolerance must lie in (0, 1).\n");
        E(obj).inner_tolerance = rel;
    });
}

void FluidSimulation_gb300_set_pressure_solver_tolerance(FluidSimulation *obj, double tol, int *err) {
    guarded(err, [&] {
        if (!(tol > 0)) throw std::domain_error("Error: tolerance must be positive.\n");
        E(obj).tolerance = tol;
    });
}

void FluidSimulation_gb300_add_sphere_obstacle(FluidSimulation *obj, double cx, double cy, double cz, double r, int *err) {
    guarded(err, [&] {
        Engine &e = E(obj);
        if (e.initialized()) throw std::runtime_error("Error: obstacles must be added before initialize.\n");
        if (e.nspheres >= MAX_SPHERES) throw std::runtime_error("Error: too many sphere obstacles.\n");
        if (!(r > 0)) throw std::domain_error("Error: sphere radius must be positive.\n");
        double *s = e.spheres.s[e.nspheres++];
        s[0] = cx; s[1] = cy; s[2] = cz; s[3] = r;
    });
}

void FluidSimulation_gb300_set_solid_level_set(FluidSimulation *obj, const float *phi, int *err) {
    guarded(err, [&] { E(obj).set_solid_phi(phi); });
}

void FluidSimulation_gb300_set_marker_particle_data(FluidSimulation *obj, FluidSimulationMarkerParticleData data, int *err) {
    guarded(err, [&] {
        Engine &e = E(obj);
        if (!e.initialized()) throw std::runtime_error("Error: FluidSimulation must be initialized first.\n");
        e.set_particles(reinterpret_cast<const float *>(data.positions), reinterpret_cast<const float *>(data.velocities),
                        data.size);
    });
}

void FluidSimulation_gb300_get_pressure_solver_stats(FluidSimulation *obj, double *out, int *err) {
    guarded(err, [&] {
        const SolveStats &s = E(obj).last_solve;
        out[0] = s.iterations; out[1] = s.success ? 1 : 0; out[2] = s.outer; out[3] = s.fluid_cells;
        out[4] = s.error; out[5] = s.rel_residual;
    });
}

void FluidSimulation_gb300_set_solve_check(FluidSimulation *obj, double reference_tolerance, int *err) {
    guarded(err, [&] {
        if (reference_tolerance < 0.0 || reference_tolerance != reference_tolerance)
            throw std::domain_error("Error: reference tolerance must be 0 (off) or positive.\n");
        E(obj).check_tolerance = reference_tolerance;
    });
}

void FluidSimulation_gb300_get_solve_check(FluidSimulation *obj, double *out8, int *err) {
    guarded(err, [&] {
        const Engine::SolveCheck &c = E(obj).last_check;
        out8[0] = c.valid ? 1 : 0; out8[1] = c.p_rel_l2; out8[2] = c.u_rel_l2; out8[3] = c.div_rel;
        out8[4] = c.div_ref_rel; out8[5] = c.bnorm; out8[6] = c.ref_iterations; out8[7] = c.ref_rel_residual;
    });
}

int FluidSimulation_gb300_get_frame_substep_times(FluidSimulation *obj, double *out, int capacity, int *err) {
    return guarded(err, [&] {
        const std::vector<double> &t = E(obj).frame_dts;
        if (out)
            for (int q = 0; q < (int)t.size() && q < capacity; q++) out[q] = t[q];
        return (int)t.size();
    });
}

void FluidSimulation_gb300_get_viscosity_solver_stats(FluidSimulation *obj, double *out, int *err) {
    guarded(err, [&] {
        const Engine::ViscStats &s = E(obj).last_visc;
        out[0] = s.rows; out[1] = s.iterations; out[2] = s.error; out[3] = s.success ? 1 : 0;
    });
}

void FluidSimulation_gb300_get_viscosity_solver_times(FluidSimulation *obj, float *out, int *err) {
    guarded(err, [&] {
        const Engine::ViscStats &s = E(obj).last_visc;
        out[0] = s.build_ms; out[1] = s.factor_ms; out[2] = s.pcg_ms;
    });
}

void FluidSimulation_gb300_write_marker_particle_file(FluidSimulation *obj, int attribute, const char *path,
                                                      int append, int *err) {
    guarded(err, [&] {
        if (!path) throw std::domain_error("Error: file path is null.\n");
        E(obj).write_attribute_file(attribute, path, append != 0);
    });
}

long long FluidSimulation_gb300_load_marker_particle_files(FluidSimulation *obj, const char *position_path,
                                                           const char *velocity_path, const char *affinex_path,
                                                           const char *affiney_path, const char *affinez_path,
                                                           int *err) {
    return guarded(err, [&] {
        if (!position_path || !velocity_path) throw std::domain_error("Error: file path is null.\n");
        return E(obj).load_attribute_files(position_path, velocity_path, affinex_path, affiney_path, affinez_path);
    });
}

void FluidSimulation_gb300_enable_stage_timing(FluidSimulation *obj, int enable, int *err) {
    guarded(err, [&] { E(obj).timing = enable != 0; });
}

void FluidSimulation_gb300_get_stage_times(FluidSimulation *obj, float *out, int *err) {
    guarded(err, [&] {
        const StageTimes &t = E(obj).last_times;
        float v[12] = {t.sort, t.sdf, t.p2g, t.extrap, t.pressure_build, t.factor, t.pcg, t.project, t.g2p, t.advect,
                       t.remove, t.total};
        std::memcpy(out, v, sizeof(v));
    });
}

unsigned long long FluidSimulation_gb300_get_kernel_launch_count(FluidSimulation *obj, int *err) {
    return guarded(err, [&] { return E(obj).launches; });
}

void FluidSimulation_gb300_substep(FluidSimulation *obj, double dt, int *err) {
    guarded(err, [&] {
        Engine &e = E(obj);
        if (!e.initialized()) throw std::runtime_error("Error: FluidSimulation must be initialized before update.\n");
        if (!(dt > 0)) throw std::domain_error("Error: delta time must be positive.\n");
        e.substep(dt);
    });
}

float FluidSimulation_gb300_run_substeps_timed(FluidSimulation *obj, int k, double dt, int *err) {
    return guarded(err, [&] {
        Engine &e = E(obj);
        if (!e.initialized()) throw std::runtime_error("Error: FluidSimulation must be initialized before update.\n");
        if (k < 0 || !(dt > 0)) throw std::domain_error("Error: bad substep count or delta time.\n");
        return e.run_substeps_timed(k, dt);
    });
}

float FluidSimulation_gb300_time_kernel(FluidSimulation *obj, int kernel_id, int reps, double *bytes, int *err) {
    return guarded(err, [&] { return E(obj).time_kernel(kernel_id, reps, bytes); });
}

void FluidSimulation_gb300_substep_differentiable(FluidSimulation *obj, double dt, int *err) {
    guarded(err, [&] {
        if (!(dt > 0)) throw std::domain_error("Error: delta time must be positive.\n");
        E(obj).substep_differentiable(dt);
    });
}

int FluidSimulation_gb300_adjoint(FluidSimulation *obj, const float *grad_v1, double loss_ymin, float *grad_v0,
                                  int *err) {
    return guarded(err, [&] {
        Engine &e = E(obj);
        if (!e.diff_ready) throw std::runtime_error("Error: run a differentiable substep before the adjoint.\n");
        int n = e.num_particles();
        cudaStream_t st = e.stream();
        int count = -1;
        if (grad_v1) {
            FFGPU_CUDA(cudaMemcpyAsync(e.stage.p, grad_v1, (size_t)n * 12, cudaMemcpyHostToDevice, st));
            launch_deinterleave(n, e.stage, e.gv1x, e.gv1y, e.gv1z, st);
            count = e.adjoint(std::numeric_limits<double>::quiet_NaN());
        } else {
            count = e.adjoint(loss_ymin);
        }
        if (grad_v0) {
            launch_interleave(n, e.gv0x, e.gv0y, e.gv0z, e.stage, st);
            FFGPU_CUDA(cudaMemcpyAsync(grad_v0, e.stage.p, (size_t)n * 12, cudaMemcpyDeviceToHost, st));
        }
        FFGPU_CUDA(cudaStreamSynchronize(st));
        return count;
    });
}

void FluidSimulation_gb300_rollout_forward(FluidSimulation *obj, int k, double dt, int *err) {
    guarded(err, [&] {
        if (k < 1 || !(dt > 0)) throw std::domain_error("Error: bad substep count or delta time.\n");
        E(obj).rollout_forward(k, dt);
    });
}

int FluidSimulation_gb300_rollout_adjoint(FluidSimulation *obj, const float *grad_xk, const float *grad_vk,
                                          double loss_ymin, float *grad_x0, float *grad_v0, int *err) {
    return guarded(err, [&] {
        Engine &e = E(obj);
        if (e.rollout_k < 1 || e.num_particles() != e.rollout_np)
            throw std::runtime_error("Error: run a rollout before its adjoint.\n");
        e.alloc_adjoint();
        int n = e.num_particles();
        cudaStream_t st = e.stream();
        if (grad_xk) {
            FFGPU_CUDA(cudaMemcpyAsync(e.stage.p, grad_xk, (size_t)n * 12, cudaMemcpyHostToDevice, st));
            launch_deinterleave(n, e.stage, e.gx1x, e.gx1y, e.gx1z, st);
        }
        if (grad_vk) {
            FFGPU_CUDA(cudaMemcpyAsync(e.stage.p, grad_vk, (size_t)n * 12, cudaMemcpyHostToDevice, st));
            launch_deinterleave(n, e.stage, e.gv1x, e.gv1y, e.gv1z, st);
        }
        int count = e.rollout_adjoint(grad_xk != nullptr,
                                      grad_vk ? std::numeric_limits<double>::quiet_NaN() : loss_ymin);
        if (grad_x0) {
            launch_interleave(n, e.gx0x, e.gx0y, e.gx0z, e.stage, st);
            FFGPU_CUDA(cudaMemcpyAsync(grad_x0, e.stage.p, (size_t)n * 12, cudaMemcpyDeviceToHost, st));
        }
        if (grad_v0) {
            launch_interleave(n, e.gv0x, e.gv0y, e.gv0z, e.stage, st);
            FFGPU_CUDA(cudaMemcpyAsync(grad_v0, e.stage.p, (size_t)n * 12, cudaMemcpyDeviceToHost, st));
        }
        FFGPU_CUDA(cudaStreamSynchronize(st));
        return count;
    });
}

float FluidSimulation_gb300_run_forward_adjoint_timed(FluidSimulation *obj, int k, double dt, double loss_ymin,
                                                      int *err) {
    return guarded(err, [&] {
        if (k < 0 || !(dt > 0)) throw std::domain_error("Error: bad substep count or delta time.\n");
        return E(obj).run_forward_adjoint_timed(k, dt, loss_ymin);
    });
}

void FluidSimulation_gb300_set_adjoint_tolerance(FluidSimulation *obj, double tol, int *err) {
    guarded(err, [&] {
        if (!(tol > 0)) throw std::domain_error("Error: tolerance must be positive.\n");
        E(obj).adjoint_tolerance = tol;
    });
}

// ---------------- stage-level functions ----------------
void ffgpu_solid_phi(int ni, int nj, int nk, double dx, int nspheres, const double *spheres, float *phi, int *err) {
    guarded(err, [&] {
        check_dims(ni, nj, nk, dx);
        if (nspheres < 0 || nspheres > MAX_SPHERES) throw std::domain_error("Error: bad sphere count.\n");
        Engine e(ni, nj, nk, dx);
        for (int s = 0; s < nspheres; s++)
            for (int q = 0; q < 4; q++) e.spheres.s[s][q] = spheres[4 * s + q];
        e.nspheres = nspheres;
        e.initialize();
        d2h(phi, e.solid.p, (size_t)(ni + 1) * (nj + 1) * (nk + 1) * 4, e.stream());
    });
}

void ffgpu_face_weights(int ni, int nj, int nk, const float *solid, float *wu, float *wv, float *ww, int *err) {
    guarded(err, [&] {
        auto e = scratch(ni, nj, nk, 1.0, 0, nullptr, nullptr);
        Dims d = e->dims();
        h2d(e->solid.p, solid, (size_t)(ni + 1) * (nj + 1) * (nk + 1) * 4, e->stream());
        launch_face_weights(d, e->solid, e->wu, e->wv, e->ww, e->stream());
        d2h(wu, e->wu.p, d.faces(0) * 4, e->stream());
        d2h(wv, e->wv.p, d.faces(1) * 4, e->stream());
        d2h(ww, e->ww.p, d.faces(2) * 4, e->stream());
    });
}

void ffgpu_sort_particles(int ni, int nj, int nk, double dx, int np, const float *pos, int *cell_start,
                          int *sorted_index, int *err) {
    guarded(err, [&] {
        auto e = scratch(ni, nj, nk, dx, np, pos, nullptr);
        e->stage_sort();
        d2h(cell_start, e->cell_start.p, (e->dims().cells() + 1) * 4, e->stream());
        if (np) d2h(sorted_index, e->sidx.p, (size_t)np * 4, e->stream());
    });
}

void ffgpu_liquid_sdf(int ni, int nj, int nk, double dx, int np, const float *pos, const float *solid,
                      int postprocess, float *phi, int *err) {
    guarded(err, [&] {
        auto e = scratch(ni, nj, nk, dx, np, pos, nullptr);
        if (solid) h2d(e->solid.p, solid, (size_t)(ni + 1) * (nj + 1) * (nk + 1) * 4, e->stream());
        e->stage_sort();
        e->stage_sdf(postprocess != 0);
        d2h(phi, e->phi.p, e->dims().cells() * 4, e->stream());
    });
}

void ffgpu_p2g(int ni, int nj, int nk, double dx, int np, const float *pos, const float *vel, float *u, float *v,
               float *w, unsigned char *vu, unsigned char *vv, unsigned char *vw, int *err) {
    guarded(err, [&] {
        auto e = scratch(ni, nj, nk, dx, np, pos, vel);
        Dims d = e->dims();
        e->stage_sort();
        e->stage_p2g();
        d2h(u, e->u.p, d.faces(0) * 4, e->stream());
        d2h(v, e->v.p, d.faces(1) * 4, e->stream());
        d2h(w, e->w.p, d.faces(2) * 4, e->stream());
        d2h(vu, e->vu.p, d.faces(0), e->stream());
        d2h(vv, e->vv.p, d.faces(1), e->stream());
        d2h(vw, e->vw.p, d.faces(2), e->stream());
    });
}

void ffgpu_p2g_components(int ni, int nj, int nk, double dx, int np, const float *pos, const float *vel, float *u,
                          float *v, float *w, unsigned char *vu, unsigned char *vv, unsigned char *vw, int *err) {
    guarded(err, [&] {
        auto e = scratch(ni, nj, nk, dx, np, pos, vel);
        Dims d = e->dims();
        e->stage_sort();
        e->stage_p2g_components();
        d2h(u, e->u.p, d.faces(0) * 4, e->stream());
        d2h(v, e->v.p, d.faces(1) * 4, e->stream());
        d2h(w, e->w.p, d.faces(2) * 4, e->stream());
        d2h(vu, e->vu.p, d.faces(0), e->stream());
        d2h(vv, e->vv.p, d.faces(1), e->stream());
        d2h(vw, e->vw.p, d.faces(2), e->stream());
    });
}

void ffgpu_extrapolate(int w, int h, int d, float *grid, const unsigned char *valid, int layers, int *err) {
    guarded(err, [&] {
        if (w < 1 || h < 1 || d < 1 || layers < 0) throw std::domain_error("Error: bad extrapolation arguments.\n");
        size_t n = (size_t)w * h * d;
        DevBuf<float> g;
        DevBuf<unsigned char> val, s1;
        DevBuf<unsigned int> l1, l2, cnt;
        g.reserve(n); val.reserve(n); s1.reserve(n); l1.reserve(n); l2.reserve(n); cnt.reserve(2);
        cudaStream_t st = 0;
        h2d(g.p, grid, n * 4, st);
        h2d(val.p, valid, n, st);
        launch_extrapolate_front(w, h, d, g, val, layers, ExtrapFront{s1.p, {l1.p, l2.p}, cnt.p}, st);
        d2h(grid, g.p, n * 4, st);
    });
}

void ffgpu_pressure_solve(int ni, int nj, int nk, double dx, double dt, const float *phi, const float *wu,
                          const float *wv, const float *ww, const float *u, const float *v, const float *w,
                          double tol, int maxit, int mode, float *pressure, double *pressure64, int *stats,
                          double *errs, int *err) {
    guarded(err, [&] {
        auto e = scratch(ni, nj, nk, dx, 0, nullptr, nullptr);
        Dims d = e->dims();
        cudaStream_t st = e->stream();
        h2d(e->phi.p, phi, d.cells() * 4, st);
        h2d(e->wu.p, wu, d.faces(0) * 4, st); h2d(e->wv.p, wv, d.faces(1) * 4, st); h2d(e->ww.p, ww, d.faces(2) * 4, st);
        h2d(e->u.p, u, d.faces(0) * 4, st); h2d(e->v.p, v, d.faces(1) * 4, st); h2d(e->w.p, w, d.faces(2) * 4, st);
        e->tolerance = tol;
        e->max_iterations = maxit;
        e->solver = (mode & 1) ? SOLVER_MIXED : SOLVER_FP64;
        e->mic_levels = (mode & 2) != 0;
        e->axis_order = (mode & 4) ? 0 : 1;
        bool ok = e->stage_pressure(dt);
        d2h(pressure, e->pressure.p, d.cells() * 4, st);
        if (pressure64) {
            std::vector<double> x(d.cells(), 0.0);
            if (e->have_fluid_cells && e->last_solve.bnorm >= tol) d2h(x.data(), e->x64.p, d.cells() * 8, st);
            // keep only pressure cells (the FP64 vector is dense over the box)
            std::vector<unsigned char> f(d.cells(), 0);
            if (e->have_fluid_cells) d2h(f.data(), e->fluid.p, d.cells(), st);
            for (size_t c = 0; c < d.cells(); c++) pressure64[c] = f[c] ? x[c] : 0.0;
        }
        const SolveStats &s = e->last_solve;
        stats[0] = s.iterations; stats[1] = ok ? 1 : 0; stats[2] = s.outer; stats[3] = s.fluid_cells;
        errs[0] = s.error; errs[1] = s.rel_residual; errs[2] = s.bnorm;
    });
}

void ffgpu_apply_pressure(int ni, int nj, int nk, double dx, double dt, const float *phi, const float *wu,
                          const float *wv, const float *ww, const float *pressure, float *u, float *v, float *w,
                          unsigned char *vu, unsigned char *vv, unsigned char *vw, int *err) {
    guarded(err, [&] {
        auto e = scratch(ni, nj, nk, dx, 0, nullptr, nullptr);
        Dims d = e->dims();
        cudaStream_t st = e->stream();
        h2d(e->phi.p, phi, d.cells() * 4, st);
        h2d(e->wu.p, wu, d.faces(0) * 4, st); h2d(e->wv.p, wv, d.faces(1) * 4, st); h2d(e->ww.p, ww, d.faces(2) * 4, st);
        h2d(e->pressure.p, pressure, d.cells() * 4, st);
        h2d(e->u.p, u, d.faces(0) * 4, st); h2d(e->v.p, v, d.faces(1) * 4, st); h2d(e->w.p, w, d.faces(2) * 4, st);
        e->stage_project(dt);
        d2h(u, e->u.p, d.faces(0) * 4, st); d2h(v, e->v.p, d.faces(1) * 4, st); d2h(w, e->w.p, d.faces(2) * 4, st);
        d2h(vu, e->vu.p, d.faces(0), st); d2h(vv, e->vv.p, d.faces(1), st); d2h(vw, e->vw.p, d.faces(2), st);
    });
}

void ffgpu_g2p(int ni, int nj, int nk, double dx, double pic, int np, const float *pos, float *vel, const float *u,
               const float *v, const float *w, const float *su, const float *sv, const float *sw, int *err) {
    guarded(err, [&] {
        auto e = scratch(ni, nj, nk, dx, np, pos, vel);
        Dims d = e->dims();
        cudaStream_t st = e->stream();
        h2d(e->u.p, u, d.faces(0) * 4, st); h2d(e->v.p, v, d.faces(1) * 4, st); h2d(e->w.p, w, d.faces(2) * 4, st);
        h2d(e->su.p, su, d.faces(0) * 4, st); h2d(e->sv.p, sv, d.faces(1) * 4, st); h2d(e->sw.p, sw, d.faces(2) * 4, st);
        e->pic_ratio = pic;
        e->stage_g2p();
        e->get_velocities(vel, 0, np);
    });
}

void ffgpu_advect(int ni, int nj, int nk, double dx, double dt, int cfl, int np, const float *pos, const float *u,
                  const float *v, const float *w, const float *solid, float *out, int *err) {
    guarded(err, [&] {
        auto e = scratch(ni, nj, nk, dx, np, pos, nullptr);
        Dims d = e->dims();
        cudaStream_t st = e->stream();
        e->cfl = cfl;
        if (solid) {
            e->set_solid_phi(solid);
        }
        h2d(e->u.p, u, d.faces(0) * 4, st); h2d(e->v.p, v, d.faces(1) * 4, st); h2d(e->w.p, w, d.faces(2) * 4, st);
        e->stage_advect(dt);
        e->get_positions(out, 0, np);
    });
}

int ffgpu_remove(int ni, int nj, int nk, double dx, int np, float *pos, float *vel, const float *solid,
                 int max_per_cell, int *err) {
    return guarded(err, [&] {
        auto e = scratch(ni, nj, nk, dx, np, pos, vel);
        if (solid) e->set_solid_phi(solid);
        e->extreme_velocity_removal = false;
        e->max_per_cell = max_per_cell;
        e->stage_remove();
        int n = e->num_particles();
        e->get_positions(pos, 0, n);
        e->get_velocities(vel, 0, n);
        return n;
    });
}

void FluidSimulation_gb300_set_pressure_axis_order(FluidSimulation *obj, int mode, int *err) {
    guarded(err, [&] {
        if (mode < 0 || mode > 1) throw std::domain_error("Error: axis order mode must be 0 or 1.\n");
        E(obj).axis_order = mode;
    });
}

void FluidSimulation_gb300_set_viscosity_preconditioner(FluidSimulation *obj, int form, int *err) {
    guarded(err, [&] {
        if (form < 0 || form > 3) throw std::domain_error("Error: viscosity preconditioner form must be 0, 1, 2 or 3.\n");
        E(obj).visc_work.precond = form;
    });
}

void FluidSimulation_gb300_set_viscosity_warm_start(FluidSimulation *obj, int on, int *err) {
    guarded(err, [&] { E(obj).visc_warm = on != 0; });
}

void FluidSimulation_gb300_set_pcg_graphs(FluidSimulation *obj, int on, int *err) {
    guarded(err, [&] { E(obj).pcg_graphs = on != 0; });
}

void FluidSimulation_gb300_set_pressure_warm_start(FluidSimulation *obj, int on, int *err) {
    guarded(err, [&] {
        if (on < 0 || on > 2) throw std::domain_error("Error: warm start must be 0, 1 or 2.\n");
        Engine &e = E(obj);
        e.warm_start = on;
        if (!on) { e.have_prev = false; e.last_setup_warm = false; e.adj_have_prev = false; }
    });
}

void FluidSimulation_gb300_set_wait_limit(FluidSimulation *obj, long long polls, int *err) {
    guarded(err, [&] {
        if (polls < 0) throw std::domain_error("Error: wait limit must be greater than or equal to 0.\n");
        E(obj).wait_limit = polls;
    });
}

int ffgpu_wait_probe(long long limit, int *err) {
    return guarded(err, [&] {
        if (limit < 1 || limit > (1LL << 24)) throw std::domain_error("Error: wait limit out of range.\n");
        cudaStream_t st;
        FFGPU_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        unsigned int bits = 0;
        try {
            bits = wait_probe(limit, st);
        } catch (...) {
            cudaStreamDestroy(st);
            throw;
        }
        FFGPU_CUDA(cudaStreamDestroy(st));
        return (int)bits;
    });
}

void ffgpu_inject_allocation_failure(long long after, int *err) {
    guarded(err, [&] {
        if (after < 0) throw std::domain_error("Error: allocation count must be greater than or equal to 0.\n");
        g_alloc_fail_countdown.store(after);
    });
}

void ffgpu_curvature_grid(int ni, int nj, int nk, double dx, const float *phi, float *surface_phi, float *curvature,
                          int *err) {
    guarded(err, [&] {
        auto e = scratch(ni, nj, nk, dx, 0, nullptr, nullptr);
        Dims d = e->dims();
        cudaStream_t st = e->stream();
        h2d(e->phi.p, phi, d.cells() * 4, st);
        TensionWork tw = e->tension_work();
        launch_curvature_grid(d, dx, e->phi, e->surf, e->curv, tw, st);
        d2h(surface_phi, e->surf.p, d.cells() * 4, st);
        d2h(curvature, e->curv.p, d.cells() * 4, st);
    });
}

void ffgpu_cluster_status(int ni, int nj, int nk, const float *phi, unsigned char *status, int *err) {
    guarded(err, [&] {
        auto e = scratch(ni, nj, nk, 1.0, 0, nullptr, nullptr);
        Dims d = e->dims();
        cudaStream_t st = e->stream();
        h2d(e->phi.p, phi, d.cells() * 4, st);
        TensionWork tw = e->tension_work();
        launch_cluster_status(d, e->phi, e->tstatus, tw, st);
        d2h(status, e->tstatus.p, d.cells(), st);
    });
}

// the tension inputs of a scratch engine: k_st, the curvature grid and the cluster status of its phi
static void set_tension(Engine &e, const float *curvature, double k_st) {
    Dims d = e.dims();
    cudaStream_t st = e.stream();
    e.surface_tension = k_st;
    TensionWork tw = e.tension_work();
    h2d(e.curv.p, curvature, d.cells() * 4, st);
    launch_cluster_status(d, e.phi, e.tstatus, tw, st);
}

void ffgpu_pressure_solve_tension(int ni, int nj, int nk, double dx, double dt, const float *phi, const float *wu,
                                  const float *wv, const float *ww, const float *u, const float *v, const float *w,
                                  const float *curvature, double k_st, double tol, int maxit, int mode,
                                  float *pressure, double *pressure64, int *stats, double *errs, int *err) {
    guarded(err, [&] {
        auto e = scratch(ni, nj, nk, dx, 0, nullptr, nullptr);
        Dims d = e->dims();
        cudaStream_t st = e->stream();
        h2d(e->phi.p, phi, d.cells() * 4, st);
        h2d(e->wu.p, wu, d.faces(0) * 4, st); h2d(e->wv.p, wv, d.faces(1) * 4, st); h2d(e->ww.p, ww, d.faces(2) * 4, st);
        h2d(e->u.p, u, d.faces(0) * 4, st); h2d(e->v.p, v, d.faces(1) * 4, st); h2d(e->w.p, w, d.faces(2) * 4, st);
        set_tension(*e, curvature, k_st);
        e->tolerance = tol;
        e->max_iterations = maxit;
        e->solver = (mode & 1) ? SOLVER_MIXED : SOLVER_FP64;
        e->mic_levels = (mode & 2) != 0;
        e->axis_order = (mode & 4) ? 0 : 1;
        bool ok = e->stage_pressure(dt);
        d2h(pressure, e->pressure.p, d.cells() * 4, st);
        if (pressure64) {
            std::vector<double> x(d.cells(), 0.0);
            if (e->have_fluid_cells && e->last_solve.bnorm >= tol) d2h(x.data(), e->x64.p, d.cells() * 8, st);
            std::vector<unsigned char> f(d.cells(), 0);
            if (e->have_fluid_cells) d2h(f.data(), e->fluid.p, d.cells(), st);
            for (size_t c = 0; c < d.cells(); c++) pressure64[c] = f[c] ? x[c] : 0.0;
        }
        const SolveStats &s = e->last_solve;
        stats[0] = s.iterations; stats[1] = ok ? 1 : 0; stats[2] = s.outer; stats[3] = s.fluid_cells;
        errs[0] = s.error; errs[1] = s.rel_residual; errs[2] = s.bnorm;
    });
}

void ffgpu_apply_pressure_tension(int ni, int nj, int nk, double dx, double dt, const float *phi, const float *wu,
                                  const float *wv, const float *ww, const float *pressure, const float *curvature,
                                  double k_st, float *u, float *v, float *w, unsigned char *vu, unsigned char *vv,
                                  unsigned char *vw, int *err) {
    guarded(err, [&] {
        auto e = scratch(ni, nj, nk, dx, 0, nullptr, nullptr);
        Dims d = e->dims();
        cudaStream_t st = e->stream();
        h2d(e->phi.p, phi, d.cells() * 4, st);
        h2d(e->wu.p, wu, d.faces(0) * 4, st); h2d(e->wv.p, wv, d.faces(1) * 4, st); h2d(e->ww.p, ww, d.faces(2) * 4, st);
        h2d(e->pressure.p, pressure, d.cells() * 4, st);
        h2d(e->u.p, u, d.faces(0) * 4, st); h2d(e->v.p, v, d.faces(1) * 4, st); h2d(e->w.p, w, d.faces(2) * 4, st);
        set_tension(*e, curvature, k_st);
        e->stage_project(dt);
        d2h(u, e->u.p, d.faces(0) * 4, st); d2h(v, e->v.p, d.faces(1) * 4, st); d2h(w, e->w.p, d.faces(2) * 4, st);
        d2h(vu, e->vu.p, d.faces(0), st); d2h(vv, e->vv.p, d.faces(1), st); d2h(vw, e->vw.p, d.faces(2), st);
    });
}

int ffgpu_remove_extreme(int ni, int nj, int nk, double dx, int np, float *pos, float *vel, const float *solid,
                         int max_per_cell, double frame_dt, int cfl, int max_substeps, float *limit, int *err) {
    return guarded(err, [&] {
        if (!(frame_dt > 0.0) || max_substeps < 1 || cfl < 1)
            throw std::domain_error("Error: bad speed-limit arguments.\n");
        auto e = scratch(ni, nj, nk, dx, np, pos, vel);
        if (solid) e->set_solid_phi(solid);
        e->extreme_velocity_removal = true;
        e->max_per_cell = max_per_cell;
        e->last_frame_dt = frame_dt;
        e->cfl = cfl;
        e->max_substeps = max_substeps;
        e->stage_remove();
        if (limit) *limit = e->last_speed_limit;
        int n = e->num_particles();
        e->get_positions(pos, 0, n);
        e->get_velocities(vel, 0, n);
        return n;
    });
}

void ffgpu_classify(int ni, int nj, int nk, const float *phi, unsigned char *fluid, int *bbox6, int *err) {
    guarded(err, [&] {
        auto e = scratch(ni, nj, nk, 1.0, 0, nullptr, nullptr);
        Dims d = e->dims();
        cudaStream_t st = e->stream();
        h2d(e->phi.p, phi, d.cells() * 4, st);
        e->fluid.reserve(d.cells());
        e->bbox_dev.reserve(6);
        launch_classify(d, e->phi, e->fluid, e->bbox_dev, st);
        FFGPU_CUDA(cudaGetLastError());
        d2h(fluid, e->fluid.p, d.cells(), st);
        d2h(bbox6, e->bbox_dev.p, 6 * sizeof(int), st);
    });
}

int ffgpu_substep(int ni, int nj, int nk, double dx, double dt, double pic, int cfl, float gx, float gy, float gz,
                  const float *solid, double tol, int maxit, int mode, int np, float *pos, float *vel, int *stats,
                  double *errs, int *err) {
    return guarded(err, [&] {
        auto e = scratch(ni, nj, nk, dx, np, pos, vel);
        e->pic_ratio = pic; e->cfl = cfl; e->gx = gx; e->gy = gy; e->gz = gz;
        e->tolerance = tol; e->max_iterations = maxit;
        e->solver = (mode & 1) ? SOLVER_MIXED : SOLVER_FP64;
        e->mic_levels = (mode & 2) != 0;
        e->axis_order = (mode & 4) ? 0 : 1;
        e->extreme_velocity_removal = false;
        if (solid) e->set_solid_phi(solid);
        e->substep(dt);
        int n = e->num_particles();
        e->get_positions(pos, 0, n);
        e->get_velocities(vel, 0, n);
        const SolveStats &s = e->last_solve;
        stats[0] = s.iterations; stats[1] = s.success ? 1 : 0; stats[2] = s.outer; stats[3] = s.fluid_cells;
        errs[0] = s.error; errs[1] = s.rel_residual; errs[2] = s.bnorm;
        return n;
    });
}

void ffgpu_p2g_apic(int ni, int nj, int nk, double dx, int np, const float *pos, const float *vel, const float *aff9,
                    float *u, float *v, float *w, unsigned char *vu, unsigned char *vv, unsigned char *vw, int *err) {
    guarded(err, [&] {
        auto e = scratch_apic(ni, nj, nk, dx, np, pos, vel, aff9);
        Dims d = e->dims();
        e->stage_sort();
        e->stage_p2g();
        d2h(u, e->u.p, d.faces(0) * 4, e->stream());
        d2h(v, e->v.p, d.faces(1) * 4, e->stream());
        d2h(w, e->w.p, d.faces(2) * 4, e->stream());
        d2h(vu, e->vu.p, d.faces(0), e->stream());
        d2h(vv, e->vv.p, d.faces(1), e->stream());
        d2h(vw, e->vw.p, d.faces(2), e->stream());
    });
}

void ffgpu_g2p_apic(int ni, int nj, int nk, double dx, int np, const float *pos, float *vel, float *aff9,
                    const float *u, const float *v, const float *w, int *err) {
    guarded(err, [&] {
        auto e = scratch_apic(ni, nj, nk, dx, np, pos, vel, aff9);
        Dims d = e->dims();
        cudaStream_t st = e->stream();
        h2d(e->u.p, u, d.faces(0) * 4, st); h2d(e->v.p, v, d.faces(1) * 4, st); h2d(e->w.p, w, d.faces(2) * 4, st);
        e->stage_g2p();
        e->get_velocities(vel, 0, np);
        read_affine9(*e, np, aff9);
    });
}

int ffgpu_substep_apic(int ni, int nj, int nk, double dx, double dt, int cfl, float gx, float gy, float gz,
                       const float *solid, double tol, int maxit, int mode, int np, float *pos, float *vel, float *aff9,
                       int *stats, double *errs, int *err) {
    return guarded(err, [&] {
        auto e = scratch_apic(ni, nj, nk, dx, np, pos, vel, aff9);
        e->cfl = cfl; e->gx = gx; e->gy = gy; e->gz = gz;
        e->tolerance = tol; e->max_iterations = maxit;
        e->solver = (mode & 1) ? SOLVER_MIXED : SOLVER_FP64;
        e->mic_levels = (mode & 2) != 0;
        e->axis_order = (mode & 4) ? 0 : 1;
        e->extreme_velocity_removal = false;
        if (solid) e->set_solid_phi(solid);
        e->substep(dt);
        int n = e->num_particles();
        e->get_positions(pos, 0, n);
        e->get_velocities(vel, 0, n);
        read_affine9(*e, n, aff9);
        const SolveStats &s = e->last_solve;
        stats[0] = s.iterations; stats[1] = s.success ? 1 : 0; stats[2] = s.outer; stats[3] = s.fluid_cells;
        errs[0] = s.error; errs[1] = s.rel_residual; errs[2] = s.bnorm;
        return n;
    });
}

// The FFP3 output of the given particles (positions inside the domain), as an update writes it after
// its first substep: the liquid level set (post-processed against solid), its surface level set,
// the classification and the grouped bytes.  flags: bit0..2 surface, boundary, interior output,
// bit3 velocity, bit4 speed attribute.  outs: four buffers of at least 16 + 12 * 65536 + 12 np
// bytes (positions, ids, velocities, speeds); sizes <- their byte counts (0: not produced);
// types (optional) <- per particle 0 surface, 1 boundary, 2 interior, 3 unset.
void ffgpu_ffp3(int ni, int nj, int nk, double dx, const float *solid, int np, const float *pos, const float *vel,
                const uint16_t *ids, int flags, double amount, char *out_pos, char *out_id, char *out_vel,
                char *out_speed, long long *sizes, unsigned char *types, int *err) {
    guarded(err, [&] {
        check_dims(ni, nj, nk, dx);
        if (np < 0) throw std::domain_error("Error: particle count must be non-negative.\n");
        auto e = std::make_unique<Engine>(ni, nj, nk, dx);
        e->ffp_output = true;
        e->initialize();
        if (solid) e->set_solid_phi(solid);
        std::vector<unsigned int> id32((size_t)np);
        for (int p = 0; p < np; p++) id32[(size_t)p] = ids[p];
        if (np) e->set_particles(pos, vel, np, nullptr, id32.data());
        e->ffp.enabled = flags & 7;
        e->ffp.velocity = (flags & 8) != 0;
        e->ffp.speed = (flags & 16) != 0;
        e->ffp_amount = amount;
        e->output_fluid_particles();
        char *outs[4] = {out_pos, out_id, out_vel, out_speed};
        for (int a = 0; a < 4; a++) {
            sizes[a] = (long long)e->ffp3_bytes(a);
            if (sizes[a] && outs[a]) e->read_ffp3(a, outs[a]);
        }
        if (types) e->read_ffp3_types(types);
    });
}

int ffgpu_viscosity_precondition(int ni, int nj, int nk, double dx, double dt, const float *liquid,
                                 const float *solid, double visc, const float *u, const float *v, const float *w,
                                 int form, int sweeps, float *z, int *err) {
    return guarded(err, [&] {
        if (form < 0 || form > 3) throw std::domain_error("Error: viscosity preconditioner form must be 0, 1, 2 or 3.\n");
        if (sweeps < 1 || sweeps > 2) throw std::domain_error("Error: sweeps must be 1 or 2.\n");
        if (form == ViscWork::VP_COOP && sweeps != 2)
            throw std::domain_error("Error: the cooperative form applies both sweeps.\n");
        auto e = scratch(ni, nj, nk, dx, 0, nullptr, nullptr);
        Dims d = e->dims();
        cudaStream_t st = e->stream();
        e->set_solid_phi(solid);
        h2d(e->phi.p, liquid, d.cells() * 4, st);
        h2d(e->u.p, u, d.faces(0) * 4, st); h2d(e->v.p, v, d.faces(1) * 4, st); h2d(e->w.p, w, d.faces(2) * 4, st);
        const int n = e->viscosity_precondition_probe(dt, (float)visc, form, sweeps);
        if (n > 0) d2h(z, e->visc_work.z.p, (size_t)n * 4, st);
        return n;
    });
}

void ffgpu_viscosity(int ni, int nj, int nk, double dx, double dt, const float *liquid, const float *solid,
                     double visc, double tol, int maxit, float *u, float *v, float *w, int *stats, float *res,
                     float *vol7, int *index, unsigned *rowstart, unsigned *col, float *val, float *rhs,
                     float *ic_invdiag, unsigned *ic_colstart, unsigned *ic_rowindex, float *ic_value, float *soln,
                     int *err) {
    guarded(err, [&] {
        auto e = scratch(ni, nj, nk, dx, 0, nullptr, nullptr);
        Dims d = e->dims();
        cudaStream_t st = e->stream();
        e->set_solid_phi(solid);
        h2d(e->phi.p, liquid, d.cells() * 4, st);
        h2d(e->u.p, u, d.faces(0) * 4, st); h2d(e->v.p, v, d.faces(1) * 4, st); h2d(e->w.p, w, d.faces(2) * 4, st);
        e->viscosity_enabled = true;
        e->viscosity = visc;
        e->visc_tolerance = tol;
        e->visc_max_iterations = maxit;
        e->visc_warm = false;   // the reference solver's zero start (its iteration count)
        e->stage_viscosity(dt);
        const ViscWork &W = e->visc_work;
        const int n = e->last_visc.rows;
        stats[0] = n; stats[1] = e->last_visc.iterations; stats[2] = e->last_visc.success ? 1 : 0;
        *res = e->last_visc.error;
        d2h(u, e->u.p, d.faces(0) * 4, st); d2h(v, e->v.p, d.faces(1) * 4, st); d2h(w, e->w.p, d.faces(2) * 4, st);
        const size_t nf = d.faces(0) + d.faces(1) + d.faces(2);
        if (vol7) d2h(vol7, W.vol.p, W.vol.n * 4, st);
        if (index) {
            if (n > 0) d2h(index, W.index.p, nf * 4, st);
            else std::fill(index, index + nf, -1);
        }
        if (n == 0) return;
        std::vector<int> c((size_t)n * VISC_SLOTS);
        std::vector<float> a((size_t)n * VISC_SLOTS), l((size_t)n * VISC_SLOTS);
        d2h(c.data(), W.col.p, c.size() * 4, st);
        d2h(a.data(), W.val.p, a.size() * 4, st);
        if (rowstart) {
            unsigned t = 0;
            for (int r = 0; r < n; r++) {
                rowstart[r] = t;
                for (int q = 0; q < VISC_SLOTS; q++)
                    if (c[(size_t)r * VISC_SLOTS + q] >= 0) { col[t] = (unsigned)c[(size_t)r * VISC_SLOTS + q]; val[t] = a[(size_t)r * VISC_SLOTS + q]; t++; }
            }
            rowstart[n] = t;
        }
        if (rhs) d2h(rhs, W.rhs.p, (size_t)n * 4, st);
        if (ic_invdiag) {
            d2h(ic_invdiag, W.invdiag.p, (size_t)n * 4, st);
            d2h(l.data(), W.lval.p, l.size() * 4, st);
            unsigned t = 0;
            for (int r = 0; r < n; r++) {
                ic_colstart[r] = t;
                for (int q = 0; q < VISC_SLOTS; q++)
                    if (c[(size_t)r * VISC_SLOTS + q] > r) { ic_rowindex[t] = (unsigned)c[(size_t)r * VISC_SLOTS + q]; ic_value[t] = l[(size_t)r * VISC_SLOTS + q]; t++; }
            }
            ic_colstart[n] = t;
        }
        if (soln) d2h(soln, W.x.p, (size_t)n * 4, st);
    });
}

}  // extern "C"
