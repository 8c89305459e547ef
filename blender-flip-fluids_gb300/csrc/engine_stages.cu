// Substep stages of the GB300 FLIP engine, in the reference's order
// (FluidSimulation::_stepFluid, fluidsimulation.cpp:10078-10121).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <stdexcept>

#include "engine.h"

namespace ffgpu {

void launch_speed_hist(int np, const float *vx, const float *vy, const float *vz, double step, int nbins,
                       int *bins, unsigned long long *maxbits, cudaStream_t st);
void launch_speed_outliers(int np, const float *vx, const float *vy, const float *vz, double lower, double upper,
                           int *counts, cudaStream_t st);
void launch_remove_mark2(Dims d, double dx, int np, const float *px, const float *py, const float *pz,
                         const float *vx, const float *vy, const float *vz, const float *solid, double maxspeedsq,
                         int *keep, int *key, int *cell_count, int *max_count, cudaStream_t st);
void launch_keep01(int np, const int *keep, int *keep01, cudaStream_t st);

PressureSystem Engine::sys_view() {
    PressureSystem s;
    s.diag = diag; s.ax = ax; s.ay = ay; s.az = az; s.inv = inv; s.lx = lx; s.ly = ly; s.lz = lz;
    s.diag32 = diag32; s.ax32 = ax32; s.ay32 = ay32; s.az32 = az32;
    s.inv32 = inv32; s.lx32 = lx32; s.ly32 = ly32; s.lz32 = lz32;
    s.b = b; s.fluid = fluid;
    return s;
}

void Engine::read_scalars() {
    FFGPU_CUDA(cudaMemcpyAsync(host_sc, scal.p, sizeof(PcgScalars), cudaMemcpyDeviceToHost, st));
    FFGPU_CUDA(cudaStreamSynchronize(st));
}

void Engine::stage_sort() {
    Dims d = dims();
    size_t nc = d.cells();
    FFGPU_CUDA(cudaMemsetAsync(cell_count.p, 0, (nc + 1) * sizeof(int), st));
    launch_cell_keys(d, dx, np, px, py, pz, key, rank, cell_count, st);
    launch_exclusive_scan(cell_count, cell_start, nc, scan_tmp, st);
    launch_scatter_sorted(np, key, rank, cell_start, sidx, st);
    launch_sort_within_cells(nc, cell_start, sidx, st);
    const float *src[6] = {px, py, pz, vx, vy, vz};
    float *dst[6] = {spx, spy, spz, svx, svy, svz};
    launch_gather_particles(np, sidx, src, dst, 6, st);
    launches += 9;
}

void Engine::stage_sdf(bool post) {
    launch_liquid_sdf(dims(), dx, radius(), cell_start, spx, spy, spz, solid, post ? 1 : 0, phi, st);
    launches++;
}

void Engine::stage_p2g() {
    Dims d = dims();
    launch_p2g(d, dx, radius(), 0, cell_start, spx, spy, spz, svx, u, vu, st);
    launch_p2g(d, dx, radius(), 1, cell_start, spx, spy, spz, svy, v, vv, st);
    launch_p2g(d, dx, radius(), 2, cell_start, spx, spy, spz, svz, w, vw, st);
    launches += 3;
}

void Engine::stage_extrapolate(int comp) {
    int layers = (int)std::ceil(std::sqrt(3) * cfl) + 3;   // fluidsimulation.cpp:6284
    int fw = ni + (comp == 0), fh = nj + (comp == 1), fd = nk + (comp == 2);
    float *f = comp == 0 ? u.p : (comp == 1 ? v.p : w.p);
    unsigned char *val = comp == 0 ? vu.p : (comp == 1 ? vv.p : vw.p);
    launch_extrapolate(fw, fh, fd, f, val, layers, st1, st2, st);
    launches += 1 + 2 * (size_t)layers;
}

void Engine::stage_extrapolate_all() {
    for (int c = 0; c < 3; c++) stage_extrapolate(c);
}

void Engine::stage_save_and_body_force(double dt) {
    Dims d = dims();
    FFGPU_CUDA(cudaMemcpyAsync(su.p, u.p, d.faces(0) * 4, cudaMemcpyDeviceToDevice, st));
    FFGPU_CUDA(cudaMemcpyAsync(sv.p, v.p, d.faces(1) * 4, cudaMemcpyDeviceToDevice, st));
    FFGPU_CUDA(cudaMemcpyAsync(sw.p, w.p, d.faces(2) * 4, cudaMemcpyDeviceToDevice, st));
    const float eps = 1e-6f;   // fluidsimulation.cpp:5837-5876
    if (std::fabs(gx) > eps) { launch_body_force(d.faces(0), u, (float)(gx * dt), st); launches++; }
    if (std::fabs(gy) > eps) { launch_body_force(d.faces(1), v, (float)(gy * dt), st); launches++; }
    if (std::fabs(gz) > eps) { launch_body_force(d.faces(2), w, (float)(gz * dt), st); launches++; }
}

bool Engine::stage_pressure(double dt) {
    Dims d = dims();
    size_t nc = d.cells();
    SolveStats s;
    launch_classify(d, phi, fluid, bbox_dev, st);
    launches++;
    FFGPU_CUDA(cudaMemcpyAsync(host_int, bbox_dev.p, 6 * sizeof(int), cudaMemcpyDeviceToHost, st));
    FFGPU_CUDA(cudaStreamSynchronize(st));
    FFGPU_CUDA(cudaMemsetAsync(pressure.p, 0, nc * 4, st));
    have_fluid_cells = host_int[3] >= 0;
    if (!have_fluid_cells) {
        last_solve = s;
        return true;
    }
    bbox = Bbox{host_int[0], host_int[1], host_int[2], host_int[3], host_int[4], host_int[5]};
    size_t nbox = (size_t)(bbox.i1 - bbox.i0 + 1) * (bbox.j1 - bbox.j0 + 1) * (bbox.k1 - bbox.k0 + 1);
    if (timing) FFGPU_CUDA(cudaEventRecord(ev[4], st));
    launch_build_system(d, dx, dt, bbox, phi, wu, wv, ww, u, v, w, sys_view(), nullptr, nullptr, maxabs_b, st);
    launches += 1;
    FFGPU_CUDA(cudaMemcpyAsync(host_dbl, maxabs_b.p, sizeof(double), cudaMemcpyDeviceToHost, st));
    FFGPU_CUDA(cudaStreamSynchronize(st));
    s.bnorm = host_dbl[0];
    s.fluid_cells = (int)nbox;
    if (s.bnorm < tolerance) {   // pressuresolver.cpp:61-74
        last_solve = s;
        return true;
    }
    if (timing) FFGPU_CUDA(cudaEventRecord(ev[5], st));
    launch_mic0_factor(d, bbox, sys_view(), st);
    launches += bbox.i1 - bbox.i0 + bbox.j1 - bbox.j0 + bbox.k1 - bbox.k0 + 1;
    if (solver == SOLVER_MIXED) { launch_to_float(d, bbox, sys_view(), st); launches++; }
    if (timing) FFGPU_CUDA(cudaEventRecord(ev[6], st));
    if (solver == SOLVER_FP64) solve_fp64(s);
    else solve_mixed(s);
    if (timing) FFGPU_CUDA(cudaEventRecord(ev[7], st));
    last_solve = s;
    return s.success;
}

// PCGSolver<double>::solve (pcgsolver.h:268-322) on the device
void Engine::solve_fp64(SolveStats &out) {
    Dims d = dims();
    PcgVecs<double> vec{x64, r64, s64, z64};
    OpView<double> A{diag, ax, ay, az};
    FactorView<double> F{inv, lx, ly, lz};
    PcgWork wk{partials, counter, scal};
    int levels = bbox.i1 - bbox.i0 + bbox.j1 - bbox.j0 + bbox.k1 - bbox.k0 + 1;
    pcg_init<double>(d, bbox, b, vec, st);
    double resid = out.bnorm;
    double tol = tolerance * resid;
    pcg_precondition<double>(d, bbox, F, r64, z64, st);
    pcg_dot_zr<double>(d, bbox, vec, wk, 1, 1, st);
    launches += 2 + 2 * (size_t)levels;
    read_scalars();
    double rho = host_sc->rho;
    if (rho == 0 || rho != rho) {
        out.iterations = 0; out.success = false; out.error = resid;
        pcg_store_pressure<double>(d, bbox, x64, pressure, st);
        return;
    }
    pcg_update_s<double>(d, bbox, vec, wk, 1, st);
    launches++;
    int it;
    bool conv = false;
    for (it = 0; it < max_iterations; it++) {
        pcg_spmv_dot<double>(d, bbox, A, vec, wk, 1, st);
        pcg_update_xr<double>(d, bbox, vec, wk, st);
        launches += 2;
        read_scalars();
        resid = host_sc->resid;
        if (resid <= std::min(tol, 1.0)) { conv = true; it++; break; }
        pcg_precondition<double>(d, bbox, F, r64, z64, st);
        pcg_dot_zr<double>(d, bbox, vec, wk, 0, 1, st);
        pcg_update_s<double>(d, bbox, vec, wk, 0, st);
        launches += 2 + 2 * (size_t)levels;
    }
    out.iterations = it;
    out.error = resid;
    out.success = conv || (it == max_iterations && (float)resid < acceptable_tolerance);
    out.rel_residual = out.bnorm > 0 ? resid / out.bnorm : 0.0;
    pcg_store_pressure<double>(d, bbox, x64, pressure, st);
    launches++;
}

// Mixed precision: FP32 PCG (FP32 operator and MIC(0) factor, FP64 dots) as the inner
// solver of an FP64 iterative refinement; convergence is tested on the FP64 true
// residual ||b - A x||_inf <= tolerance * ||b||_inf.
void Engine::solve_mixed(SolveStats &out) {
    Dims d = dims();
    PcgVecs<float> vf{x32, r32, s32, z32};
    OpView<float> A32{diag32, ax32, ay32, az32};
    FactorView<float> F32{inv32, lx32, ly32, lz32};
    OpView<double> A64{diag, ax, ay, az};
    PcgWork wk{partials, counter, scal};
    int levels = bbox.i1 - bbox.i0 + bbox.j1 - bbox.j0 + bbox.k1 - bbox.k0 + 1;
    // x = 0, r = b (FP64) and its FP32 copy in s64's float view
    pcg_zero(d, bbox, x64, st);
    float *rf = reinterpret_cast<float *>(s64.p);   // FP32 right-hand side of the inner solve
    pcg_true_residual(d, bbox, A64, b, x64, r64, rf, wk, st);
    launches += 2;
    read_scalars();
    double resid = host_sc->resid;
    const double target = tolerance * out.bnorm;
    int total_it = 0, outer = 0;
    bool ok = resid <= target;
    while (!ok && outer < max_outer && total_it < max_iterations) {
        pcg_init<float>(d, bbox, rf, vf, st);
        pcg_precondition<float>(d, bbox, F32, r32, z32, st);
        pcg_dot_zr<float>(d, bbox, vf, wk, 1, 0, st);
        launches += 2 + 2 * (size_t)levels;
        read_scalars();
        double rho = host_sc->rho;
        if (rho == 0 || rho != rho) break;
        pcg_update_s<float>(d, bbox, vf, wk, 1, st);
        launches++;
        double inner_tol = std::max(inner_tolerance * resid, 0.5 * target);
        for (int it = 0; it < max_iterations - total_it; it++) {
            pcg_spmv_dot<float>(d, bbox, A32, vf, wk, 0, st);
            pcg_update_xr<float>(d, bbox, vf, wk, st);
            launches += 2;
            read_scalars();
            total_it++;
            double ri = host_sc->resid;
            if (ri <= inner_tol || ri != ri) break;
            pcg_precondition<float>(d, bbox, F32, r32, z32, st);
            pcg_dot_zr<float>(d, bbox, vf, wk, 0, 0, st);
            pcg_update_s<float>(d, bbox, vf, wk, 0, st);
            launches += 2 + 2 * (size_t)levels;
        }
        pcg_refine(d, bbox, x32, x64, st);
        pcg_true_residual(d, bbox, A64, b, x64, r64, rf, wk, st);
        launches += 2;
        read_scalars();
        resid = host_sc->resid;
        outer++;
        ok = resid <= target;
    }
    out.iterations = total_it;
    out.outer = outer;
    out.error = resid;
    out.rel_residual = out.bnorm > 0 ? resid / out.bnorm : 0.0;
    out.success = ok || (total_it >= max_iterations && (float)resid < acceptable_tolerance);
    pcg_store_pressure<double>(d, bbox, x64, pressure, st);
    launches++;
}

void Engine::stage_project(double dt) {
    launch_apply_pressure(dims(), dx, dt, phi, wu, wv, ww, pressure, u, v, w, vu, vv, vw, st);
    launches++;
}

void Engine::stage_constrain() {
    Dims d = dims();
    launch_constrain(d.faces(0), wu, su, st); launch_constrain(d.faces(1), wv, sv, st); launch_constrain(d.faces(2), ww, sw, st);
    launch_constrain(d.faces(0), wu, u, st); launch_constrain(d.faces(1), wv, v, st); launch_constrain(d.faces(2), ww, w, st);
    launches += 6;
}

void Engine::stage_g2p() {
    launch_g2p(dims(), dx, (float)pic_ratio, np, px, py, pz, vx, vy, vz, MacView{u, v, w}, MacView{su, sv, sw}, st);
    launches++;
}

void Engine::stage_advect(double dt) {
    launch_advect(dims(), dx, dt, (int)cfl, np, px, py, pz, ox, oy, oz, MacView{u, v, w}, solid, ng, near, st);
    launches++;
    std::swap(px.p, ox.p); std::swap(py.p, oy.p); std::swap(pz.p, oz.p);
}

// FluidSimulation::_removeMarkerParticles (fluidsimulation.cpp:7773-7851)
void Engine::stage_remove() {
    if (np == 0) return;
    Dims d = dims();
    size_t nc = d.cells();
    double maxspeedsq = -1.0;
    if (extreme_velocity_removal) {
        // _getMarkerParticleSpeedLimit (:7723-7771) with the frame's delta time
        double frame_dt = last_frame_dt;
        double step = cfl * dx / frame_dt;
        int nb = std::max(max_substeps, 1);
        FFGPU_CUDA(cudaMemsetAsync(maxcount.p, 0, 4 * sizeof(int), st));
        int *bins = cell_count.p;   // scratch (re-zeroed below)
        FFGPU_CUDA(cudaMemsetAsync(bins, 0, (size_t)(nb + 4) * sizeof(int), st));
        unsigned long long *mb = reinterpret_cast<unsigned long long *>(maxabs_b.p);
        FFGPU_CUDA(cudaMemsetAsync(mb, 0, sizeof(unsigned long long), st));
        launch_speed_hist(np, vx, vy, vz, step, nb, bins, mb, st);
        std::vector<int> hb(nb);
        FFGPU_CUDA(cudaMemcpyAsync(hb.data(), bins, nb * sizeof(int), cudaMemcpyDeviceToHost, st));
        FFGPU_CUDA(cudaMemcpyAsync(host_dbl, mb, sizeof(double), cudaMemcpyDeviceToHost, st));
        FFGPU_CUDA(cudaStreamSynchronize(st));
        double maxps = host_dbl[0];
        int maxrem = std::min((int)((double)np * 0.0005), 35);
        double maxspeed = nb * step;
        int cur = 0;
        for (int i = nb - 1; i > 0; i--) {
            if (cur + hb[i] > maxrem) break;
            cur += hb[i];
            maxspeed = std::max(i + 4, nb) * step;
        }
        double lower = 0.90 * maxps, upper = 0.99999 * maxps;
        launch_speed_outliers(np, vx, vy, vz, lower, upper, bins + nb, st);
        FFGPU_CUDA(cudaMemcpyAsync(host_int, bins + nb, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
        FFGPU_CUDA(cudaStreamSynchronize(st));
        if (host_int[1] <= 6 && host_int[0] <= 6) maxspeed = std::min(upper, maxspeed);
        float fms = (float)maxspeed;
        maxspeedsq = (double)(fms * fms);
        launches += 2;
    }
    FFGPU_CUDA(cudaMemsetAsync(cell_count.p, 0, (nc + 1) * sizeof(int), st));
    FFGPU_CUDA(cudaMemsetAsync(maxcount.p, 0, sizeof(int), st));
    launch_remove_mark2(d, dx, np, px, py, pz, vx, vy, vz, solid, maxspeedsq, keep, key, cell_count, maxcount, st);
    launches++;
    FFGPU_CUDA(cudaMemcpyAsync(host_int, maxcount.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    FFGPU_CUDA(cudaStreamSynchronize(st));
    const int *final_keep;
    if (host_int[0] > max_per_cell) {
        // per-cell cap in particle order: stable sort of all particles by their new cell
        FFGPU_CUDA(cudaMemsetAsync(cell_count.p, 0, (nc + 1) * sizeof(int), st));
        launch_cell_keys(d, dx, np, px, py, pz, key, rank, cell_count, st);
        launch_exclusive_scan(cell_count, cell_start, nc, scan_tmp, st);
        launch_scatter_sorted(np, key, rank, cell_start, sidx, st);
        launch_sort_within_cells(nc, cell_start, sidx, st);
        launch_cap_per_cell(nc, cell_start, sidx, keep, keep2, max_per_cell, st);
        launches += 8;
        final_keep = keep2;
    } else {
        launch_keep01(np, keep, keep2, st);
        launches++;
        final_keep = keep2;
    }
    launch_exclusive_scan(final_keep, off, (size_t)np, scan_tmp, st);
    FFGPU_CUDA(cudaMemcpyAsync(host_int, off.p + np, sizeof(int), cudaMemcpyDeviceToHost, st));
    FFGPU_CUDA(cudaStreamSynchronize(st));
    int nnew = host_int[0];
    launches += 4;
    if (nnew == np) return;
    const float *src[6] = {px, py, pz, vx, vy, vz};
    float *dst[6] = {cpx, cpy, cpz, cvx, cvy, cvz};
    launch_compact(np, final_keep, off, src, dst, 6, st);
    launches++;
    std::swap(px.p, cpx.p); std::swap(py.p, cpy.p); std::swap(pz.p, cpz.p);
    std::swap(vx.p, cvx.p); std::swap(vy.p, cvy.p); std::swap(vz.p, cvz.p);
    np = nnew;
}

void Engine::substep(double dt) {
    if (!in_update) last_frame_dt = dt;
    if (np == 0) {
        last_solve = SolveStats();
        return;
    }
    if (timing) FFGPU_CUDA(cudaEventRecord(ev[0], st));
    stage_sort();
    if (timing) FFGPU_CUDA(cudaEventRecord(ev[1], st));
    stage_sdf(true);
    if (timing) FFGPU_CUDA(cudaEventRecord(ev[2], st));
    stage_p2g();
    stage_extrapolate_all();
    stage_save_and_body_force(dt);
    if (timing) FFGPU_CUDA(cudaEventRecord(ev[3], st));
    bool ok = stage_pressure(dt);
    if (timing) FFGPU_CUDA(cudaEventRecord(ev[8], st));
    if (ok) stage_project(dt);
    stage_extrapolate_all();
    stage_constrain();
    if (timing) FFGPU_CUDA(cudaEventRecord(ev[9], st));
    stage_g2p();
    if (timing) FFGPU_CUDA(cudaEventRecord(ev[10], st));
    stage_advect(dt);
    if (timing) FFGPU_CUDA(cudaEventRecord(ev[11], st));
    stage_remove();
    if (timing) {
        FFGPU_CUDA(cudaEventRecord(ev[12], st));
        FFGPU_CUDA(cudaEventSynchronize(ev[12]));
        auto el = [&](int a, int b_) { float ms = 0; cudaEventElapsedTime(&ms, ev[a], ev[b_]); return ms; };
        last_times.sort = el(0, 1);
        last_times.sdf = el(1, 2);
        last_times.p2g = el(2, 3);
        last_times.pcg = el(3, 8);
        last_times.project = el(8, 9);
        last_times.g2p = el(9, 10);
        last_times.advect = el(10, 11);
        last_times.remove = el(11, 12);
        last_times.total = el(0, 12);
    }
    FFGPU_CUDA(cudaGetLastError());
}

}  // namespace ffgpu

namespace ffgpu {
float Engine::run_substeps_timed(int k, double dt) {
    FFGPU_CUDA(cudaEventRecord(ev[13], st));
    for (int q = 0; q < k; q++) substep(dt);
    FFGPU_CUDA(cudaEventRecord(ev[14], st));
    FFGPU_CUDA(cudaEventSynchronize(ev[14]));
    float ms = 0.0f;
    FFGPU_CUDA(cudaEventElapsedTime(&ms, ev[13], ev[14]));
    return ms;
}
}  // namespace ffgpu
