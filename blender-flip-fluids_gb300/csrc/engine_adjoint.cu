// Differentiable substep: recording forward pass, adjoint sweep over the particle state
// (x, v), and checkpointed multi-substep rollouts (see adjoint_kernels.cu for the map).
#include <cmath>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <utility>

#include "adjoint.h"
#include "engine.h"

namespace ffgpu {

void Engine::alloc_adjoint() {
    Dims d = dims();
    size_t nu = d.faces(0), nv = d.faces(1), nw = d.faces(2);
    size_t nmax = std::max(nu, std::max(nv, nw));
    size_t c = (size_t)std::max(cap, 1);
    wsum_u.reserve(nu); wsum_v.reserve(nv); wsum_w.reserve(nw);
    p2g_u.reserve(nu); p2g_v.reserve(nv); p2g_w.reserve(nw);
    gcu.reserve(nu); gcv.reserve(nv); gcw.reserve(nw);
    gsu.reserve(nu); gsv.reserve(nv); gsw.reserve(nw);
    gbu.reserve(nu); gbv.reserve(nv); gbw.reserve(nw);
    gtmp.reserve(nmax);
    lay1u.reserve(nu); lay1v.reserve(nv); lay1w.reserve(nw);
    lay2u.reserve(nu); lay2v.reserve(nv); lay2w.reserve(nw);
    val1u.reserve(nu); val1v.reserve(nv); val1w.reserve(nw);
    val2u.reserve(nu); val2v.reserve(nv); val2w.reserve(nw);
    for (DevBuf<float> *b_ : {&gv1x, &gv1y, &gv1z, &gv0x, &gv0y, &gv0z, &gx1x, &gx1y, &gx1z, &gx0x, &gx0y, &gx0z})
        b_->reserve(c);
    collided.reserve(c);
    adj_wc.reserve(3 * c); adj_ws.reserve(3 * c);
    adj_pt2.reserve(6 * c); adj_pt3.reserve(6 * c); adj_q.reserve(6 * c);
    cell_count2.reserve(d.cells() + 1); cell_start2.reserve(d.cells() + 1); sidx2.reserve(c);
    loss_count.reserve(1);
}

void Engine::substep_differentiable(double dt) {
    if (!is_init) throw std::runtime_error("Error: FluidSimulation must be initialized before update.\n");
    int layers = (int)std::ceil(std::sqrt(3) * cfl) + 3;
    if (layers > 31)   // the per-face extrapolation record keeps the layer in 5 bits
        throw std::domain_error("Error: the differentiable substep supports CFL numbers up to 16.\n");
    if (apic)   // the transposed maps are those of the PIC/FLIP transfer
        throw std::runtime_error("Error: the differentiable substep needs the FLIP velocity transfer method.\n");
    if (tension_on())   // no transposed curvature or tension term
        throw std::runtime_error("Error: the differentiable substep does not include surface tension.\n");
    if (viscosity_enabled && viscosity > 0)   // no transposed viscosity solve
        throw std::runtime_error("Error: the differentiable substep does not include the viscosity solve.\n");
    alloc_adjoint();
    diff_ready = false;
    Dims d = dims();
    stage_sort();
    stage_sdf(true);
    launch_p2g(d, dx, radius(), 0, cell_start, spx, spy, spz, svx, gridpos, blockpos, u, vu, st, wsum_u, p2g_u);
    launch_p2g(d, dx, radius(), 1, cell_start, spx, spy, spz, svy, gridpos, blockpos, v, vv, st, wsum_v, p2g_v);
    launch_p2g(d, dx, radius(), 2, cell_start, spx, spy, spz, svz, gridpos, blockpos, w, vw, st, wsum_w, p2g_w);
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
    launch_advect(d, dx, dt, (int)cfl, np, px, py, pz, ox, oy, oz, MacView{u, v, w}, solid, ng, near, st, collided);
    std::swap(px.p, ox.p); std::swap(py.p, oy.p); std::swap(pz.p, oz.p);
    launches += 4 + 6 * (2 * (size_t)layers);
    diff_dt = dt;
    diff_ready = true;
}

// Cell sort of the RK3 stage points pts (x, y, z, then three weights; 6 x cap floats) into
// cell_start2 and the sorted copies adj_q, stable in the points' own order, keyed by the float
// cell floor that FP32 MAC sampling uses.
void Engine::sort_points(const float *pts) {
    Dims d = dims();
    size_t nc = d.cells(), c = (size_t)cap;
    FFGPU_CUDA(cudaMemsetAsync(cell_count2.p, 0, (nc + 1) * sizeof(int), st));
    launch_cell_keys(d, dx, np, pts, pts + c, pts + 2 * c, key, rank, cell_count2, st, true);
    launch_exclusive_scan(cell_count2, cell_start2, nc, scan_tmp, st);
    launch_scatter_sorted(np, key, rank, cell_start2, sidx2, st);
    launch_sort_within_cells(nc, cell_start2, sidx2, st);
    const float *src[6];
    float *dst[6];
    for (int a = 0; a < 6; a++) { src[a] = pts + a * c; dst[a] = adj_q.p + a * c; }
    launch_gather_particles(np, sidx2, src, dst, 6, st);
    launches += 8;
}

void Engine::adjoint_core(bool with_x) {
    if (!diff_ready) throw std::runtime_error("Error: run a differentiable substep before the adjoint.\n");
    Dims d = dims();
    const size_t c = (size_t)cap;
    int layers = (int)std::ceil(std::sqrt(3) * cfl) + 3;
    const float a = (float)pic_ratio, bb_ = (float)(1.0 - (double)pic_ratio);
    // direct FLIP path: v1 = ... + b v0
    adj_scale(np, gv1x, bb_, gv0x, st); adj_scale(np, gv1y, bb_, gv0y, st); adj_scale(np, gv1z, bb_, gv0z, st);
    // RK3^T and the position part of G2P^T; sample weights at x0 and at the stage points
    const float *gx1[3] = {gx1x, gx1y, gx1z}, *gv1[3] = {gv1x, gv1y, gv1z};
    float *gx0[3] = {gx0x, gx0y, gx0z};
    adj_advect_transpose(d, dx, a, bb_, diff_dt, np, c, sidx, spx, spy, spz, with_x ? gx1 : nullptr, gv1, collided,
                         gx0, adj_wc, adj_ws, adj_pt2, adj_pt3, MacView{u, v, w}, MacView{su, sv, sw}, st);
    // transposed sampling at x0 (G2P, RK3 stage 1) into the current and saved fields
    float *gc[3] = {gcu, gcv, gcw}, *gs[3] = {gsu, gsv, gsw}, *gb[3] = {gbu, gbv, gbw};
    const float *wg[3] = {wu, wv, ww};
    for (int q = 0; q < 3; q++)
        adj_sample_transpose(d, dx, q, false, cell_start, spx, spy, spz, adj_wc.p + q * c, adj_ws.p + q * c, gc[q],
                             gs[q], false, st);
    launches += 4;
    if (with_x) {
        // RK3 stages 2 and 3: their sample points are sorted by cell first
        for (const float *pts : {adj_pt2.p, adj_pt3.p}) {
            sort_points(pts);
            for (int q = 0; q < 3; q++)
                adj_sample_transpose(d, dx, q, true, cell_start2, adj_q.p, adj_q.p + c, adj_q.p + 2 * c,
                                     adj_q.p + (3 + q) * c, nullptr, gc[q], nullptr, true, st);
            launches += 3;
        }
    }
    // solid constraint (zeroes weight-0 faces) on both fields
    for (int q = 0; q < 3; q++) {
        launch_constrain(d.faces(q), wg[q], gc[q], st);
        launch_constrain(d.faces(q), wg[q], gs[q], st);
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
            if (solver == SOLVER_FP64) {
                solve_fp64(s);
            } else {
                // start from the last adjoint solve's solution (scaled like the forward's warm start:
                // the unknown goes as 1/dt for the same right-hand side); the stopping rule stays
                // relative to ||g_p||_inf, and the forward's pressure grid is left alone
                const size_t nc = d.cells();
                const bool warm = warm_start != 0 && adj_have_prev && adj_prev.n >= nc && adj_prev_dt > 0.0;
                if (warm) {
                    pcg_warm_start(d, bbox, adj_prev, fluid, adj_prev_dt / diff_dt, x64, st);
                    launches++;
                }
                solve_from_x = true;   // x64: the warm start, or the zero the residual above was taken at
                try {
                    solve_mixed(s);
                } catch (...) {
                    solve_from_x = false;
                    adj_have_prev = false;
                    tolerance = saved_tol;
                    throw;
                }
                solve_from_x = false;
                adj_prev.reserve(nc);
                FFGPU_CUDA(cudaMemsetAsync(adj_prev.p, 0, nc * sizeof(float), st));
                pcg_store_pressure<double>(d, bbox, x64, adj_prev, st);
                launches++;
                adj_have_prev = s.success;
                adj_prev_dt = diff_dt;
            }
        }
        tolerance = saved_tol;
        for (int q = 0; q < 3; q++) adj_projection_faces(d, q, phi, wg[q], gc[q], gb[q], st);
        if (s.bnorm > 0)
            for (int q = 0; q < 3; q++) adj_div_transpose(d, q, dx, wg[q], fluid, x64, gb[q], st);
        launches += 8;
    } else {
        // no solve: every active face keeps its value
        for (int q = 0; q < 3; q++) adj_projection_faces(d, q, phi, wg[q], gc[q], gb[q], st);
    }
    // body force is affine; the saved field joins before the first extrapolation
    for (int q = 0; q < 3; q++) adj_add(d.faces(q), gs[q], gb[q], st);
    adj_extrapolate_transpose(ni + 1, nj, nk, layers, val1u, lay1u, gbu, gtmp, st);
    adj_extrapolate_transpose(ni, nj + 1, nk, layers, val1v, lay1v, gbv, gtmp, st);
    adj_extrapolate_transpose(ni, nj, nk + 1, layers, val1w, lay1w, gbw, gtmp, st);
    // P2G^T into dL/dv0 and dL/dx0
    float *g0[3] = {gv0x, gv0y, gv0z};
    const float *sv[3] = {svx, svy, svz}, *ws_[3] = {wsum_u, wsum_v, wsum_w}, *uf[3] = {p2g_u, p2g_v, p2g_w};
    const unsigned char *v1[3] = {val1u, val1v, val1w};
    for (int q = 0; q < 3; q++)
        adj_p2g_transpose(d, dx, radius(), q, np, sidx, spx, spy, spz, sv[q], ws_[q], uf[q], v1[q], gb[q], g0[q], gx0,
                          st);
    launches += 3 + 6 + 6 * (size_t)layers + 3 + 6 * (size_t)layers + 3;
    FFGPU_CUDA(cudaGetLastError());
}

int Engine::adjoint(double loss_ymin) {
    if (!diff_ready) throw std::runtime_error("Error: run a differentiable substep before the adjoint.\n");
    int count = -1;
    if (!std::isnan(loss_ymin)) {
        count = adj_loss_grad_vy2(np, loss_ymin, py, vy, gv1x, gv1y, gv1z, loss_count, host_int, st);
        launches += 2;
    }
    adjoint_core(false);
    return count;
}

void Engine::save_state(size_t slot) {
    const size_t c = (size_t)cap, bytes = (size_t)np * sizeof(float);
    const float *src[6] = {px, py, pz, vx, vy, vz};
    for (int a = 0; a < 6; a++)
        FFGPU_CUDA(cudaMemcpyAsync(ckpt.p + (slot * 6 + a) * c, src[a], bytes, cudaMemcpyDeviceToDevice, st));
}

void Engine::restore_state(size_t slot) {
    const size_t c = (size_t)cap, bytes = (size_t)np * sizeof(float);
    float *dst[6] = {px, py, pz, vx, vy, vz};
    for (int a = 0; a < 6; a++)
        FFGPU_CUDA(cudaMemcpyAsync(dst[a], ckpt.p + (slot * 6 + a) * c, bytes, cudaMemcpyDeviceToDevice, st));
}

void Engine::rollout_forward(int k, double dt) {
    if (!is_init) throw std::runtime_error("Error: FluidSimulation must be initialized before update.\n");
    if (k < 1) throw std::domain_error("Error: a rollout needs at least one substep.\n");
    if (apic) throw std::runtime_error("Error: the differentiable substep needs the FLIP velocity transfer method.\n");
    if (viscosity_enabled && viscosity > 0)
        throw std::runtime_error("Error: the differentiable substep does not include the viscosity solve.\n");
    rollout_k = 0;
    ckpt.reserve((size_t)(k + 1) * 6 * (size_t)std::max(cap, 1));
    for (int i = 0; i < k; i++) {
        save_state((size_t)i);
        substep_differentiable(dt);
    }
    save_state((size_t)k);
    rollout_k = k;
    rollout_np = np;
    rollout_dt = dt;
}

int Engine::rollout_adjoint(bool with_x, double loss_ymin) {
    if (rollout_k < 1 || np != rollout_np) throw std::runtime_error("Error: run a rollout before its adjoint.\n");
    alloc_adjoint();
    const int k = rollout_k;
    int count = -1;
    if (!std::isnan(loss_ymin)) {
        restore_state((size_t)k);
        count = adj_loss_grad_vy2(np, loss_ymin, py, vy, gv1x, gv1y, gv1z, loss_count, host_int, st);
        launches += 2;
    }
    if (!with_x) {
        adj_fill(np, 0.0f, gx1x, st); adj_fill(np, 0.0f, gx1y, st); adj_fill(np, 0.0f, gx1z, st);
        launches += 3;
    }
    for (int i = k - 1; i >= 0; i--) {
        restore_state((size_t)i);
        substep_differentiable(rollout_dt);   // recompute the records of substep i
        adjoint_core(true);
        if (i > 0) {   // this substep's input gradient is the previous substep's output gradient
            std::swap(gx1x.p, gx0x.p); std::swap(gx1y.p, gx0y.p); std::swap(gx1z.p, gx0z.p);
            std::swap(gv1x.p, gv0x.p); std::swap(gv1y.p, gv0y.p); std::swap(gv1z.p, gv0z.p);
        }
    }
    restore_state((size_t)k);
    diff_ready = false;   // the recorded substep is no longer the state's last one
    return count;
}

float Engine::run_forward_adjoint_timed(int k, double dt, double loss_ymin) {
    FFGPU_CUDA(cudaEventRecord(ev[13], st));
    for (int q = 0; q < k; q++) {
        substep_differentiable(dt);
        // the full adjoint of one substep of a rollout: a loss gradient on v1 and a non-zero
        // position cotangent, so that the RK3 stages are transposed as well
        adj_loss_grad_vy2(np, loss_ymin, py, vy, gv1x, gv1y, gv1z, loss_count, host_int, st);
        adj_fill(np, 1.0f, gx1x, st); adj_fill(np, 1.0f, gx1y, st); adj_fill(np, 1.0f, gx1z, st);
        launches += 5;
        adjoint_core(true);
    }
    FFGPU_CUDA(cudaEventRecord(ev[14], st));
    FFGPU_CUDA(cudaEventSynchronize(ev[14]));
    float ms = 0.0f;
    FFGPU_CUDA(cudaEventElapsedTime(&ms, ev[13], ev[14]));
    return ms;
}

}  // namespace ffgpu
