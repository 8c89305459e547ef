// Differentiable substep: recording forward pass and adjoint sweep (see adjoint_kernels.cu).
#include <cmath>
#include <cstring>
#include <limits>
#include <stdexcept>

#include "adjoint.h"
#include "engine.h"

namespace ffgpu {

void Engine::alloc_adjoint() {
    Dims d = dims();
    size_t nu = d.faces(0), nv = d.faces(1), nw = d.faces(2);
    size_t nmax = std::max(nu, std::max(nv, nw));
    wsum_u.reserve(nu); wsum_v.reserve(nv); wsum_w.reserve(nw);
    gcu.reserve(nu); gcv.reserve(nv); gcw.reserve(nw);
    gsu.reserve(nu); gsv.reserve(nv); gsw.reserve(nw);
    gbu.reserve(nu); gbv.reserve(nv); gbw.reserve(nw);
    gtmp.reserve(nmax);
    lay1u.reserve(nu); lay1v.reserve(nv); lay1w.reserve(nw);
    lay2u.reserve(nu); lay2v.reserve(nv); lay2w.reserve(nw);
    val1u.reserve(nu); val1v.reserve(nv); val1w.reserve(nw);
    val2u.reserve(nu); val2v.reserve(nv); val2w.reserve(nw);
    for (DevBuf<float> *b_ : {&gv1x, &gv1y, &gv1z, &gv0x, &gv0y, &gv0z}) b_->reserve(std::max(cap, 1));
    loss_count.reserve(1);
}

void Engine::substep_differentiable(double dt) {
    if (!is_init) throw std::runtime_error("Error: FluidSimulation must be initialized before update.\n");
    alloc_adjoint();
    diff_ready = false;
    Dims d = dims();
    int layers = (int)std::ceil(std::sqrt(3) * cfl) + 3;
    stage_sort();
    stage_sdf(true);
    launch_p2g(d, dx, radius(), 0, cell_start, spx, spy, spz, svx, u, vu, st, wsum_u);
    launch_p2g(d, dx, radius(), 1, cell_start, spx, spy, spz, svy, v, vv, st, wsum_v);
    launch_p2g(d, dx, radius(), 2, cell_start, spx, spy, spz, svz, w, vw, st, wsum_w);
    FFGPU_CUDA(cudaMemcpyAsync(val1u.p, vu.p, d.faces(0), cudaMemcpyDeviceToDevice, st));
    FFGPU_CUDA(cudaMemcpyAsync(val1v.p, vv.p, d.faces(1), cudaMemcpyDeviceToDevice, st));
    FFGPU_CUDA(cudaMemcpyAsync(val1w.p, vw.p, d.faces(2), cudaMemcpyDeviceToDevice, st));
    launch_extrapolate_front(ni + 1, nj, nk, u, vu, layers, front(), st, lay1u);
    launch_extrapolate_front(ni, nj + 1, nk, v, vv, layers, front(), st, lay1v);
    launch_extrapolate_front(ni, nj, nk + 1, w, vw, layers, front(), st, lay1w);
    stage_save_and_body_force(dt);
    bool ok = stage_pressure(dt);
    if (!ok) throw std::runtime_error("Error: pressure solve failed in the differentiable substep.\n");
    stage_project(dt);
    FFGPU_CUDA(cudaMemcpyAsync(val2u.p, vu.p, d.faces(0), cudaMemcpyDeviceToDevice, st));
    FFGPU_CUDA(cudaMemcpyAsync(val2v.p, vv.p, d.faces(1), cudaMemcpyDeviceToDevice, st));
    FFGPU_CUDA(cudaMemcpyAsync(val2w.p, vw.p, d.faces(2), cudaMemcpyDeviceToDevice, st));
    launch_extrapolate_front(ni + 1, nj, nk, u, vu, layers, front(), st, lay2u);
    launch_extrapolate_front(ni, nj + 1, nk, v, vv, layers, front(), st, lay2v);
    launch_extrapolate_front(ni, nj, nk + 1, w, vw, layers, front(), st, lay2w);
    stage_constrain();
    stage_g2p();
    stage_advect(dt);
    launches += 3 + 6 * (2 * (size_t)layers);
    diff_dt = dt;
    diff_ready = true;
}

int Engine::adjoint(double loss_ymin) {
    if (!diff_ready) throw std::runtime_error("Error: run a differentiable substep before the adjoint.\n");
    Dims d = dims();
    int layers = (int)std::ceil(std::sqrt(3) * cfl) + 3;
    int count = -1;
    if (!std::isnan(loss_ymin)) {
        count = adj_loss_grad_vy2(np, loss_ymin, py, vy, gv1x, gv1y, gv1z, loss_count, host_int, st);
        launches += 2;
    }
    const float a = (float)pic_ratio, bb_ = (float)(1.0 - (double)pic_ratio);
    // direct FLIP path: v1 = ... + b v0
    adj_scale(np, gv1x, bb_, gv0x, st); adj_scale(np, gv1y, bb_, gv0y, st); adj_scale(np, gv1z, bb_, gv0z, st);
    // G2P^T at the start-of-substep positions (sorted copies, same cells as the forward)
    const float *g1[3] = {gv1x, gv1y, gv1z};
    float *gc[3] = {gcu, gcv, gcw}, *gs[3] = {gsu, gsv, gsw}, *gb[3] = {gbu, gbv, gbw};
    const float *wg[3] = {wu, wv, ww};
    for (int c = 0; c < 3; c++)
        adj_g2p_transpose(d, dx, c, cell_start, sidx, spx, spy, spz, g1[c], a + bb_, -bb_, gc[c], gs[c], st);
    // solid constraint (zeroes weight-0 faces) on both fields
    for (int c = 0; c < 3; c++) {
        launch_constrain(d.faces(c), wg[c], gc[c], st);
        launch_constrain(d.faces(c), wg[c], gs[c], st);
    }
    // second extrapolation^T
    adj_extrapolate_transpose(ni + 1, nj, nk, layers, val2u, lay2u, gcu, gtmp, st);
    adj_extrapolate_transpose(ni, nj + 1, nk, layers, val2v, lay2v, gcv, gtmp, st);
    adj_extrapolate_transpose(ni, nj, nk + 1, layers, val2w, lay2w, gcw, gtmp, st);
    // projection^T: g_b = mask g_up + D^T A^-1 (-factor G^T g_up)
    if (have_fluid_cells && last_solve.bnorm >= tolerance) {
        adj_pressure_grad(d, bbox, dx, diff_dt, phi, wu, wv, ww, gcu, gcv, gcw, fluid, b, st);
        // solve A g = gp with the forward's operator and MIC(0) factor
        SolveStats s;
        PcgWork wk{partials, counter, scal};
        pcg_zero(d, bbox, x64, st);
        float *rf = reinterpret_cast<float *>(s64.p);
        FFGPU_CUDA(cudaMemsetAsync(scal.p, 0, sizeof(PcgScalars), st));
        pcg_true_residual(d, bbox, OpView<double>{diag, ax, ay, az}, b, x64, r64, rf, wk, st);
        read_scalars();
        s.bnorm = host_sc->resid;
        double saved_tol = tolerance;
        tolerance = adjoint_tolerance;
        if (s.bnorm > 0) {
            if (solver == SOLVER_FP64) solve_fp64(s);
            else solve_mixed(s);
        }
        tolerance = saved_tol;
        for (int c = 0; c < 3; c++) adj_projection_faces(d, c, phi, wg[c], gc[c], gb[c], st);
        if (s.bnorm > 0)
            for (int c = 0; c < 3; c++) adj_div_transpose(d, c, dx, wg[c], fluid, x64, gb[c], st);
        launches += 8;
    } else {
        // no solve: every active face keeps its value
        for (int c = 0; c < 3; c++) adj_projection_faces(d, c, phi, wg[c], gc[c], gb[c], st);
    }
    // body force is affine; the saved field joins before the first extrapolation
    for (int c = 0; c < 3; c++) adj_add(d.faces(c), gs[c], gb[c], st);
    adj_extrapolate_transpose(ni + 1, nj, nk, layers, val1u, lay1u, gbu, gtmp, st);
    adj_extrapolate_transpose(ni, nj + 1, nk, layers, val1v, lay1v, gbv, gtmp, st);
    adj_extrapolate_transpose(ni, nj, nk + 1, layers, val1w, lay1w, gbw, gtmp, st);
    // P2G^T into dL/dv0
    float *g0[3] = {gv0x, gv0y, gv0z};
    for (int c = 0; c < 3; c++)
        adj_p2g_transpose(d, dx, radius(), c, np, sidx, spx, spy, spz, c == 0 ? wsum_u.p : (c == 1 ? wsum_v.p : wsum_w.p),
                          gb[c], g0[c], st);
    launches += 3 + 3 + 6 + 6 * (size_t)layers + 3 + 6 * (size_t)layers + 3;
    FFGPU_CUDA(cudaGetLastError());
    return count;
}

float Engine::run_forward_adjoint_timed(int k, double dt, double loss_ymin) {
    FFGPU_CUDA(cudaEventRecord(ev[13], st));
    for (int q = 0; q < k; q++) {
        substep_differentiable(dt);
        adjoint(loss_ymin);
    }
    FFGPU_CUDA(cudaEventRecord(ev[14], st));
    FFGPU_CUDA(cudaEventSynchronize(ev[14]));
    float ms = 0.0f;
    FFGPU_CUDA(cudaEventElapsedTime(&ms, ev[13], ev[14]));
    return ms;
}

}  // namespace ffgpu
