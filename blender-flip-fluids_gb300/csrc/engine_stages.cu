// Substep stages of the GB300 FLIP engine, in the reference's order
// (FluidSimulation::_stepFluid, fluidsimulation.cpp:10078-10121).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <stdexcept>

#include "engine.h"
#include "tension.cuh"

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
    s.diag32lo = diag32lo; s.ax32lo = ax32lo; s.ay32lo = ay32lo; s.az32lo = az32lo;
    s.inv32 = inv32; s.lx32 = lx32; s.ly32 = ly32; s.lz32 = lz32;
    s.b = b; s.fluid = fluid;
    return s;
}

void Engine::read_scalars() {
    FFGPU_CUDA(cudaMemcpyAsync(host_sc, scal.p, sizeof(PcgScalars), cudaMemcpyDeviceToHost, st));
    FFGPU_CUDA(cudaStreamSynchronize(st));
}

template <typename T>
void Engine::precondition(FactorView<T> F, const T *r, T *z) {
    precondition<T>(dims(), bbox, F, r, z);
}

template <typename T>
void Engine::precondition(Dims d, Bbox bb, FactorView<T> F, const T *r, T *z) {
    if (mic_levels) {
        pcg_precondition<T>(d, bb, F, r, z, st);
        launches += 2 * (size_t)(bb.i1 - bb.i0 + bb.j1 - bb.j0 + bb.k1 - bb.k0 + 1);
    } else {
        mic_wavefront<T>(d, bb, F, r, z, wf_work(reinterpret_cast<const int *>(&scal.p->done)), st);
        launches += 2;
    }
}

void Engine::precondition_dot(Dims d, Bbox bb, FactorView<float> F, const float *r, float *z, int first) {
    if (mic_levels) {
        // the hyperplane sweeps with the same q.q, summed in the wavefront's order
        pcg_precondition_fwd<float>(d, bb, F, r, z, st);
        mic_dotq_tiles(d, bb, z, wf_dot, (int)wf_order.n, scal, first, st);
        pcg_precondition_bwd<float>(d, bb, F, z, st);
        launches += 2 + 2 * (size_t)(bb.i1 - bb.i0 + bb.j1 - bb.j0 + bb.k1 - bb.k0 + 1);
    } else {
        mic_wavefront_dot(d, bb, F, r, z, wf_work(reinterpret_cast<const int *>(&scal.p->done)), scal, first, st);
        launches += 2;
    }
}

WfWork Engine::wf_work(const int *done) {
    return WfWork{wf_order, wf_xchg, wf_xchg.n, &wf_epoch, wf_ticket, errword, (int)wf_order.n, &wf_order_key, done,
                  wait_limit, wf_epoch_dev, wf_dot};
}

void Engine::check_error_word(const char *where) {
    unsigned int e = 0;
    FFGPU_CUDA(cudaMemcpyAsync(host_int, errword.p, sizeof(unsigned int), cudaMemcpyDeviceToHost, st));
    FFGPU_CUDA(cudaStreamSynchronize(st));
    e = (unsigned int)host_int[0];
    if (e) {
        FFGPU_CUDA(cudaMemsetAsync(errword.p, 0, sizeof(unsigned int), st));
        // a sweep that gave up may have left tiles untaken: start the next one from a clean ticket
        FFGPU_CUDA(cudaMemsetAsync(wf_ticket.p, 0, 2 * sizeof(unsigned int), st));
        throw std::runtime_error("Error: GPU kernel reported error bits 0x" + std::to_string(e) +
                                 " (1 = wavefront wait timed out) during the " + where + ".\n");
    }
}

void Engine::stage_sort() {
    ensure_affine();
    Dims d = dims();
    size_t nc = d.cells();
    FFGPU_CUDA(cudaMemsetAsync(cell_count.p, 0, (nc + 1) * sizeof(int), st));
    launch_cell_keys(d, dx, np, px, py, pz, key, rank, cell_count, st);
    launch_exclusive_scan(cell_count, cell_start, nc, scan_tmp, st);
    launch_scatter_sorted(np, key, rank, cell_start, sidx, st);
    launch_sort_within_cells(nc, cell_start, sidx, st);
    const float *src[15] = {px, py, pz, vx, vy, vz};
    float *dst[15] = {spx, spy, spz, svx, svy, svz};
    const int nattr = apic ? 15 : 6;   // APIC: the affine vectors travel with the particles
    for (int q = 0; apic && q < 9; q++) { src[6 + q] = aff[q]; dst[6 + q] = saff[q]; }
    launch_gather_particles(np, sidx, src, dst, nattr, st);
    launches += 9;
}

void Engine::stage_sdf(bool post, cudaStream_t on) {
    sdf_rec.reserve((size_t)std::max(cap, 1));
    launch_liquid_sdf(dims(), dx, radius(), np, cell_start, spx, spy, spz, sdf_rec, solid, post ? 1 : 0, phi,
                      on ? on : st);
    launches += 2;
}

// FLIP transfer one component per launch (the kernel the differentiable substep runs)
void Engine::stage_p2g_components() {
    Dims d = dims();
    launch_p2g(d, dx, radius(), 0, cell_start, spx, spy, spz, svx, gridpos, blockpos, u, vu, st);
    launch_p2g(d, dx, radius(), 1, cell_start, spx, spy, spz, svy, gridpos, blockpos, v, vv, st);
    launch_p2g(d, dx, radius(), 2, cell_start, spx, spy, spz, svz, gridpos, blockpos, w, vw, st);
    launches += 3;
}

void Engine::stage_p2g() {
    Dims d = dims();
    if (apic) {
        launch_apic_records(d, dx, radius(), np, spx, spy, spz, apic_rec, st);
        const float *sv[3] = {svx, svy, svz};
        float *fld[3] = {u, v, w};
        unsigned char *val[3] = {vu, vv, vw};
        for (int c = 0; c < 3; c++) {
            const float *sa[3] = {saff[3 * c], saff[3 * c + 1], saff[3 * c + 2]};
            launch_p2g_apic(d, dx, radius(), c, cell_start, spx, spy, spz, sv[c], sa, apic_rec, np, gridpos, blockpos,
                            fld[c], val[c], st);
        }
        launches += 4;
        return;
    }
    launch_p2g3(d, dx, radius(), cell_start, spx, spy, spz, svx, svy, svz, gridpos, blockpos, u, v, w, vu, vv, vw, st);
    launches++;
}

void Engine::stage_extrapolate(int comp) {
    int layers = (int)std::ceil(std::sqrt(3) * cfl) + 3;   // fluidsimulation.cpp:6284
    int fw = ni + (comp == 0), fh = nj + (comp == 1), fd = nk + (comp == 2);
    float *f = comp == 0 ? u.p : (comp == 1 ? v.p : w.p);
    unsigned char *val = comp == 0 ? vu.p : (comp == 1 ? vv.p : vw.p);
    launch_extrapolate_front(fw, fh, fd, f, val, layers, front(), st);
    launches += 2 * (size_t)layers;
}

// The three components at once: u on the engine's stream, v and w on two side streams that start
// after everything enqueued so far and that the engine's stream waits for (own frontier buffers).
void Engine::stage_extrapolate_all() {
    const int layers = (int)std::ceil(std::sqrt(3) * cfl) + 3;   // fluidsimulation.cpp:6284
    FFGPU_CUDA(cudaEventRecord(xevent[0], st));
    for (auto &s_ : xstream) FFGPU_CUDA(cudaStreamWaitEvent(s_, xevent[0], 0));
    launch_extrapolate_front(ni + 1, nj, nk, u, vu, layers, front(), st);
    launch_extrapolate_front(ni, nj + 1, nk, v, vv, layers, ExtrapFront{xst_v.p, {xl_v[0].p, xl_v[1].p}, xc_v.p},
                             xstream[0]);
    launch_extrapolate_front(ni, nj, nk + 1, w, vw, layers, ExtrapFront{xst_w.p, {xl_w[0].p, xl_w[1].p}, xc_w.p},
                             xstream[1]);
    for (int q = 0; q < 2; q++) {
        FFGPU_CUDA(cudaEventRecord(xevent[1 + q], xstream[q]));
        FFGPU_CUDA(cudaStreamWaitEvent(st, xevent[1 + q], 0));
    }
    launches += 6 * (size_t)layers;
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
    solve_warm = solver == SOLVER_MIXED && warm_start && have_prev && prev_dt > 0.0;
    solve_warm2 = false;
    if (solve_warm) {
        // The pressure unknown scales as 1/dt: y = p dt is what evolves smoothly.  One level:
        // y_n = y_{n-1}.  Two levels (the last setup was warm, so prev_pressure still holds p_{n-2}
        // of the substep before, dt0): y_n = y_{n-1} + (y_{n-1} - y_{n-2}) dt1 / dt0.
        const double dt1 = prev_dt, dt0 = last_setup_dt;
        solve_warm2 = warm_start == 2 && last_setup_warm && dt0 > 0.0 && prev_pressure.n >= nc;
        if (solve_warm2) {
            std::swap(prev_pressure.p, prev2_pressure.p);
            std::swap(prev_pressure.n, prev2_pressure.n);
            const double ratio = dt1 / dt0;
            warm_scale = dt1 * (1.0 + ratio) / dt;
            warm_scale2 = -dt0 * ratio / dt;
        } else {
            warm_scale = dt1 / dt;
        }
        prev_pressure.reserve(nc);
        FFGPU_CUDA(cudaMemcpyAsync(prev_pressure.p, pressure.p, nc * 4, cudaMemcpyDeviceToDevice, st));
        last_setup_dt = dt1;
    }
    last_setup_warm = solve_warm;
    FFGPU_CUDA(cudaMemsetAsync(pressure.p, 0, nc * 4, st));
    have_fluid_cells = host_int[3] >= 0;
    if (!have_fluid_cells) {
        last_solve = s;
        have_prev = false;   // no solution to start the next solve from
        mark(6); mark(7); mark(8);
        return true;
    }
    bbox = Bbox{host_int[0], host_int[1], host_int[2], host_int[3], host_int[4], host_int[5]};
    size_t nbox = (size_t)(bbox.i1 - bbox.i0 + 1) * (bbox.j1 - bbox.j0 + 1) * (bbox.k1 - bbox.k0 + 1);
    const TensionDev ten{phi.p, curv.p, tstatus.p, surface_tension, tension_on() ? 1 : 0};
    launch_build_system(d, dx, dt, bbox, phi, wu, wv, ww, u, v, w, sys_view(), nullptr, nullptr, maxabs_b, st, &ten);
    launches += 1;
    FFGPU_CUDA(cudaMemcpyAsync(host_dbl, maxabs_b.p, sizeof(double), cudaMemcpyDeviceToHost, st));
    FFGPU_CUDA(cudaStreamSynchronize(st));
    s.bnorm = host_dbl[0];
    s.fluid_cells = (int)nbox;
    mark(6);
    if (s.bnorm < tolerance) {   // pressuresolver.cpp:61-74
        last_solve = s;
        have_prev = false;
        mark(7); mark(8);
        return true;
    }
    mic_progress.reserve((size_t)mic0_factor_tiles(bbox.i1 - bbox.i0 + 1, bbox.j1 - bbox.j0 + 1));
    launch_mic0_factor(d, bbox, sys_view(), mic_levels ? nullptr : mic_progress.p, errword, st, wait_limit);
    launches += 1;   // one cooperative launch
    perm_ready = false;
    perm_active = false;
    if (solver == SOLVER_MIXED) {
        Dims pd;
        Bbox pbx;
        const AxisMap m = choose_axis_map(bbox, pd, pbx);
        perm_active = axis_order == 1 && (m.perm[0] != 0 || m.perm[1] != 1 || m.perm[2] != 2);
        if (perm_active) {
            perm_map = m; perm_dims = pd; perm_box = pbx;
        } else {
            launch_to_float(d, bbox, sys_view(), st);
            launches++;
        }
    }
    mark(7);
    if (solver == SOLVER_FP64) solve_fp64(s);
    else solve_mixed(s);
    solve_warm = false;
    have_prev = solver == SOLVER_MIXED && s.success;
    prev_dt = dt;
    mark(8);
    last_solve = s;
    return s.success;
}

// Resets the device solver scalars for a new (inner) solve with stopping threshold `tol`.
static void reset_scalars(PcgScalars *dev, PcgScalars *host, double tol, cudaStream_t st) {
    std::memset(host, 0, sizeof(PcgScalars));
    host->tol = tol;
    FFGPU_CUDA(cudaMemcpyAsync(dev, host, sizeof(PcgScalars), cudaMemcpyHostToDevice, st));
    FFGPU_CUDA(cudaStreamSynchronize(st));
}

// PCGSolver<double>::solve (pcgsolver.h:268-322) on the device.  Iterations are enqueued
// in batches; the residual update raises a device flag at convergence and every later
// kernel of the batch returns at entry, so the iterate is exactly the one the reference
// stops on while the host synchronises once per batch.
void Engine::solve_fp64(SolveStats &out) {
    Dims d = dims();
    PcgVecs<double> vec{x64, r64, s64, z64};
    OpView<double> A{diag, ax, ay, az};
    FactorView<double> F{inv, lx, ly, lz};
    PcgWork wk{partials, counter, scal};
    double resid = out.bnorm;
    double tol = std::min(tolerance * resid, 1.0);   // |r|_inf <= min(tol * |b|_inf, 1)
    reset_scalars(scal, host_sc, tol, st);
    pcg_init<double>(d, bbox, b, vec, st);
    precondition<double>(F, r64, z64);
    pcg_dot_zr<double>(d, bbox, vec, wk, 1, 1, st);
    launches += 2;
    read_scalars();
    double rho = host_sc->rho;
    if (rho == 0 || rho != rho) {
        out.iterations = 0; out.success = false; out.error = resid;
        pcg_store_pressure<double>(d, bbox, x64, pressure, st);
        return;
    }
    pcg_update_s<double>(d, bbox, vec, wk, 1, st);
    launches++;
    int enq = 0;
    while (enq < max_iterations) {
        int batch = std::min(pcg_batch, max_iterations - enq);
        for (int q = 0; q < batch; q++) {
            pcg_spmv_dot<double>(d, bbox, A, vec, wk, 1, st);
            pcg_update_xr<double>(d, bbox, vec, wk, st);
            precondition<double>(F, r64, z64);
            pcg_dot_zr<double>(d, bbox, vec, wk, 0, 1, st);
            pcg_update_s<double>(d, bbox, vec, wk, 0, st);
            launches += 4;
        }
        enq += batch;
        read_scalars();
        if (host_sc->done) break;
    }
    bool conv = host_sc->done != 0;
    int it = host_sc->iters;
    resid = host_sc->resid;
    out.iterations = it;
    out.error = resid;
    out.success = conv || (it == max_iterations && (float)resid < acceptable_tolerance);
    out.rel_residual = out.bnorm > 0 ? resid / out.bnorm : 0.0;
    pcg_store_pressure<double>(d, bbox, x64, pressure, st);
    launches++;
    check_error_word();
}

// Mixed precision: FP32 PCG (FP32 vectors, operator and MIC(0) factor, FP64 dot products)
// with reliable updates.  The FP32 iteration keeps its search direction throughout; whenever
// its recursive residual has dropped by `inner_tolerance` (or reached the target) the device
// folds the FP32 iterate into the FP64 solution and replaces the residual by the FP64 true
// residual b - A x.  The solve stops when ||b - A x||_inf <= tolerance * ||b||_inf, checked
// in FP64 on that true residual.
void Engine::solve_mixed(SolveStats &out) {
    Dims d = dims();
    const bool guess = solve_warm || solve_from_x;   // x64 holds the start
    if (!perm_active) {
        if (solve_warm)
            pcg_warm_start(d, bbox, prev_pressure, fluid, warm_scale, x64, st, solve_warm2 ? prev2_pressure.p : nullptr,
                           warm_scale2);
        MixedArrays m{d, bbox, OpView<float>{diag32, ax32, ay32, az32}, OpView<float>{diag32lo, ax32lo, ay32lo, az32lo},
                      FactorView<float>{inv32, lx32, ly32, lz32}, OpView<double>{diag, ax, ay, az}, b, x64, r64,
                      reinterpret_cast<float *>(s64.p), PcgVecs<float>{x32, r32, s32, z32}, guess};
        solve_mixed_on(m, out);
        if (!solve_from_x) {
            pcg_store_pressure<double>(d, bbox, x64, pressure, st);
            launches++;
        }
        return;
    }
    // the axis-ordered copy: operator and factor once per system, the right-hand side every solve
    const Dims pd = perm_dims;
    const size_t pn = pd.cells();
    for (DevBuf<double> *a : {&pdiag, &pax, &pay, &paz, &pb, &px64, &pr64}) a->reserve(pn);
    for (DevBuf<float> *a : {&pdiag32, &pax32, &pay32, &paz32, &pdiag32lo, &pax32lo, &pay32lo, &paz32lo, &pinv32,
                             &plx32, &ply32, &plz32, &px32, &pr32, &ps32, &pz32, &prf})
        a->reserve(pn);
    if (!perm_ready) {
        // rows of the padding columns stay zero (operator, factor and vectors alike)
        for (DevBuf<double> *a : {&pdiag, &pax, &pay, &paz, &pb, &px64, &pr64})
            FFGPU_CUDA(cudaMemsetAsync(a->p, 0, pn * sizeof(double), st));
        for (DevBuf<float> *a : {&pdiag32, &pax32, &pay32, &paz32, &pdiag32lo, &pax32lo, &pay32lo, &paz32lo, &pinv32,
                                 &plx32, &ply32, &plz32, &px32, &pr32, &ps32, &pz32, &prf})
            FFGPU_CUDA(cudaMemsetAsync(a->p, 0, pn * sizeof(float), st));
        PermutedSystem ps{pdiag, pax, pay, paz, pdiag32, pax32, pay32, paz32, pdiag32lo, pax32lo, pay32lo, paz32lo,
                          pinv32, plx32, ply32, plz32};
        launch_permute_system(d, bbox, perm_map, pd, sys_view(), ps, st);
        launches++;
        perm_ready = true;
    }
    launch_permute_box<double>(d, bbox, perm_map, pd, b, pb, 0, st);
    if (solve_warm) {
        pcg_warm_start(d, bbox, prev_pressure, fluid, warm_scale, x64, st, solve_warm2 ? prev2_pressure.p : nullptr,
                       warm_scale2);
        launches++;
    }
    if (guess) {
        launch_permute_box<double>(d, bbox, perm_map, pd, x64, px64, 0, st);
        launches++;
    }
    MixedArrays m{pd, perm_box, OpView<float>{pdiag32, pax32, pay32, paz32},
                  OpView<float>{pdiag32lo, pax32lo, pay32lo, paz32lo}, FactorView<float>{pinv32, plx32, ply32, plz32},
                  OpView<double>{pdiag, pax, pay, paz}, pb, px64, pr64, prf, PcgVecs<float>{px32, pr32, ps32, pz32},
                  guess};
    solve_mixed_on(m, out);
    // the solution back into the grid's box cells (the cells the grid-order solve writes)
    launch_permute_box<double>(d, bbox, perm_map, pd, px64, x64, 1, st);
    launches += 2;
    if (!solve_from_x) {
        pcg_store_pressure<double>(d, bbox, x64, pressure, st);
        launches++;
    }
}

void Engine::solve_mixed_on(const MixedArrays &M, SolveStats &out) {
    const Dims d = M.d;
    const Bbox bb = M.bb;
    PcgVecs<float> vf = M.vf;
    const OpView<float> A32 = M.A32, A32lo = M.A32lo;
    const FactorView<float> F32 = M.F32;
    const OpView<double> A64 = M.A64;
    const double *bv = M.b;
    double *xv = M.x64, *rv = M.r64;
    PcgWork wk{partials, counter, scal};
    // x = 0, r = b (FP64) and its FP32 copy
    if (!M.warm) pcg_zero(d, bb, xv, st);
    float *rf = M.rf;
    reset_scalars(scal, host_sc, 0.0, st);
    pcg_true_residual(d, bb, A64, bv, xv, rv, rf, wk, st);
    launches += 2;
    read_scalars();
    double resid = host_sc->resid;
    const double target = tolerance * out.bnorm;
    bool ok = resid <= target;
    int it = 0, updates = 0;
    if (!ok) {
        std::memset(host_sc, 0, sizeof(PcgScalars));
        host_sc->tol = target;
        host_sc->target = target;
        host_sc->delta = inner_tolerance;
        host_sc->rmax = resid;
        host_sc->reliable = 1;
        FFGPU_CUDA(cudaMemcpyAsync(scal.p, host_sc, sizeof(PcgScalars), cudaMemcpyHostToDevice, st));
        pcg_init<float>(d, bb, rf, vf, st);
        precondition_dot(d, bb, F32, vf.r, vf.z, 1);   // rho = z.r, as q.q
        launches += 1;
        read_scalars();
        double rho = host_sc->rho;
        if (rho == 0 || rho != rho) {
            out.iterations = 0; out.success = false; out.error = resid;
            return;
        }
        pcg_update_s<float>(d, bb, vf, wk, 1, st);
        launches++;
        auto iterations = [&](int count) {
            for (int q = 0; q < count; q++) {
                pcg_spmv_dot_split(d, bb, A32, A32lo, vf, wk, st);
                pcg_update_xr<float>(d, bb, vf, wk, st);
                pcg_reliable_update(d, bb, A64, bv, xv, vf.x, rv, vf.r, wk, st);
                precondition_dot(d, bb, F32, vf.r, vf.z, 0);   // and beta, rho from q.q
                pcg_update_s<float>(d, bb, vf, wk, 0, st);
                launches += 5;
            }
        };
        // Full batches replay a graph captured once per solve: the kernels' arguments are fixed for
        // the solve, the sweeps take their tags from the device counter, and the kernels after
        // convergence exit at entry.  The preconditioner order table is already uploaded (above).
        const bool graph = pcg_graphs && !mic_levels;
        struct ExecGuard {
            cudaGraphExec_t e = nullptr;
            ~ExecGuard() { if (e) cudaGraphExecDestroy(e); }
        } batch_graph;
        unsigned long long per_batch = 0;
        const WfWork ww = wf_work(nullptr);
        int enq = 0;
        // full batches replayed back to back before the first host check: the ones the last solve of
        // this kind needed, less two (a batch past convergence only runs kernels that exit at entry)
        int unchecked = graph ? std::max(0, last_mixed_iters[solve_from_x ? 1 : 0] / pcg_batch - 2) : 0;
        while (enq < max_iterations) {
            int batch = std::min(pcg_batch, max_iterations - enq);
            if (graph && batch == pcg_batch) {
                const unsigned int sweeps = 2u * (unsigned int)batch;
                wf_reserve_epochs(ww, sweeps, st);
                if (!batch_graph.e) {
                    const unsigned int tag = wf_epoch;
                    const unsigned long long l0 = launches;
                    cudaGraph_t g = nullptr;
                    FFGPU_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
                    iterations(batch);
                    FFGPU_CUDA(cudaStreamEndCapture(st, &g));
                    const cudaError_t ie = cudaGraphInstantiate(&batch_graph.e, g, 0);
                    cudaGraphDestroy(g);
                    FFGPU_CUDA(ie);
                    wf_epoch = tag;   // nothing ran yet
                    per_batch = launches - l0;
                    launches = l0;
                }
                FFGPU_CUDA(cudaGraphLaunch(batch_graph.e, st));
                wf_epoch += sweeps;
                launches += per_batch;
            } else {
                iterations(batch);
            }
            enq += batch;
            if (unchecked > 0 && batch == pcg_batch && enq < max_iterations) {
                unchecked--;
                continue;
            }
            read_scalars();
            if (host_sc->done || host_sc->resid != host_sc->resid) break;
        }
        it = host_sc->iters;
        last_mixed_iters[solve_from_x ? 1 : 0] = it;
        updates = host_sc->updates;
        ok = host_sc->done != 0;
        resid = host_sc->resid;
        if (!ok) {   // iteration limit: fold the last FP32 iterate in and measure the FP64 residual
            pcg_refine(d, bb, vf.x, xv, st);
            reset_scalars(scal, host_sc, 0.0, st);
            pcg_true_residual(d, bb, A64, bv, xv, rv, rf, wk, st);
            launches += 2;
            read_scalars();
            resid = host_sc->resid;
            ok = resid <= target;
        }
    }
    out.iterations = it;
    out.outer = updates;
    out.error = resid;
    out.rel_residual = out.bnorm > 0 ? resid / out.bnorm : 0.0;
    out.success = ok || (it >= max_iterations && (float)resid < acceptable_tolerance);
    check_error_word();
}

void Engine::check_solve(double dt) {
    last_check = SolveCheck();
    if (!have_fluid_cells || !(last_solve.bnorm >= tolerance)) return;
    Dims d = dims();
    const size_t nc = d.cells();
    chk_x.reserve(nc); chk_p.reserve(nc); chk_part.reserve(DIFF_PARTIALS); chk_max.reserve(1);
    chk_u.reserve(d.faces(0)); chk_v.reserve(d.faces(1)); chk_w.reserve(d.faces(2));
    chk_vu.reserve(d.faces(0)); chk_vv.reserve(d.faces(1)); chk_vw.reserve(d.faces(2));
    std::vector<double> hp(DIFF_PARTIALS);
    // keep the substep's own solution (FP64 iterate and float pressure grid)
    FFGPU_CUDA(cudaMemcpyAsync(chk_x.p, x64.p, nc * 8, cudaMemcpyDeviceToDevice, st));
    FFGPU_CUDA(cudaMemcpyAsync(chk_p.p, pressure.p, nc * 4, cudaMemcpyDeviceToDevice, st));
    const SolveStats own = last_solve;
    SolveStats ref;
    ref.bnorm = own.bnorm;
    ref.fluid_cells = own.fluid_cells;
    const double tol0 = tolerance;
    const int it0 = max_iterations;
    tolerance = check_tolerance;
    max_iterations = std::max(max_iterations, 20000);
    solve_fp64(ref);   // x64, pressure <- the reference solution
    tolerance = tol0;
    max_iterations = it0;
    double e2, r2;
    diff_sq<double, double>(nc, chk_x.p, x64.p, fluid.p, chk_part.p, hp.data(), e2, r2, st);
    last_check.p_rel_l2 = r2 > 0.0 ? std::sqrt(e2 / r2) : 0.0;
    // the field projected with the reference pressure
    FFGPU_CUDA(cudaMemcpyAsync(chk_u.p, u.p, d.faces(0) * 4, cudaMemcpyDeviceToDevice, st));
    FFGPU_CUDA(cudaMemcpyAsync(chk_v.p, v.p, d.faces(1) * 4, cudaMemcpyDeviceToDevice, st));
    FFGPU_CUDA(cudaMemcpyAsync(chk_w.p, w.p, d.faces(2) * 4, cudaMemcpyDeviceToDevice, st));
    const TensionDev ten{phi.p, curv.p, tstatus.p, surface_tension, tension_on() ? 1 : 0};
    launch_apply_pressure(d, dx, dt, phi, wu, wv, ww, pressure, chk_u, chk_v, chk_w, chk_vu, chk_vv, chk_vw, st, &ten);
    last_check.div_ref_rel = divergence_max(d, dx, fluid, wu, wv, ww, chk_u, chk_v, chk_w, chk_max, host_dbl, st) /
                             own.bnorm;
    // restore the substep's own solution
    FFGPU_CUDA(cudaMemcpyAsync(x64.p, chk_x.p, nc * 8, cudaMemcpyDeviceToDevice, st));
    FFGPU_CUDA(cudaMemcpyAsync(pressure.p, chk_p.p, nc * 4, cudaMemcpyDeviceToDevice, st));
    last_solve = own;
    last_check.bnorm = own.bnorm;
    last_check.ref_iterations = ref.iterations;
    last_check.ref_rel_residual = ref.rel_residual;
    last_check.valid = true;
    launches += 4;
}

void Engine::check_projection() {
    if (!last_check.valid) return;
    Dims d = dims();
    std::vector<double> hp(DIFF_PARTIALS);
    last_check.div_rel = divergence_max(d, dx, fluid, wu, wv, ww, u, v, w, chk_max, host_dbl, st) / last_check.bnorm;
    double e2 = 0.0, r2 = 0.0;
    const float *a[3] = {u.p, v.p, w.p}, *b_[3] = {chk_u.p, chk_v.p, chk_w.p};
    const unsigned char *m[3] = {vu.p, vv.p, vw.p};
    for (int c = 0; c < 3; c++) {
        double e, r;
        diff_sq<float, float>(d.faces(c), a[c], b_[c], m[c], chk_part.p, hp.data(), e, r, st);
        e2 += e; r2 += r;
    }
    last_check.u_rel_l2 = r2 > 0.0 ? std::sqrt(e2 / r2) : 0.0;
    launches += 4;
}

TensionWork Engine::tension_work() {
    Dims d = dims();
    const size_t nc = d.cells();
    const size_t nb6 = (size_t)((ni + 5) / 6) * ((nj + 5) / 6) * ((nk + 5) / 6);
    const size_t nb4 = (size_t)std::max(ni / 4, 1) * std::max(nj / 4, 1) * std::max(nk / 4, 1);
    surf.reserve(nc); curv.reserve(nc); tbuf.reserve(nc);
    tvalid.reserve(nc); tvn.reserve(nc); tstatus.reserve(nc); ttouch.reserve(nc);
    tblocks0.reserve(nb6); tblocks1.reserve(nb6); tcblocks.reserve(nb4); tscal.reserve(4);
    tparent.reserve(nc); tcount.reserve(nc);
    return TensionWork{tbuf, tvalid, tvn, tblocks0, tblocks1, tparent, tcount, ttouch, tcblocks, tscal, st1, st2,
                       host_int + 8};
}

// ParticleLevelSet::calculateCurvatureGrid (fluidsimulation.cpp:5704-5729, particlelevelset.cpp:196-291)
// and the cluster status of PressureSolver::solve (pressuresolver.cpp:314-605), both of the
// post-processed liquid level set
void Engine::stage_surface_tension() {
    if (!tension_on() || np == 0) return;
    Dims d = dims();
    TensionWork tw = tension_work();
    launches += launch_curvature_grid(d, dx, phi, surf, curv, tw, st);
    launches += launch_cluster_status(d, phi, tstatus, tw, st);
}

void Engine::stage_project(double dt) {
    const TensionDev ten{phi.p, curv.p, tstatus.p, surface_tension, tension_on() ? 1 : 0};
    launch_apply_pressure(dims(), dx, dt, phi, wu, wv, ww, pressure, u, v, w, vu, vv, vw, st, &ten);
    launches++;
}

void Engine::stage_constrain() {
    Dims d = dims();
    launch_constrain(d.faces(0), wu, su, st); launch_constrain(d.faces(1), wv, sv, st); launch_constrain(d.faces(2), ww, sw, st);
    launch_constrain(d.faces(0), wu, u, st); launch_constrain(d.faces(1), wv, v, st); launch_constrain(d.faces(2), ww, w, st);
    launches += 6;
}

// FluidSimulation::_applyViscosityToVelocityField (fluidsimulation.cpp:5983-6064) with a
// constant viscosity: velocity constraint, then ViscositySolver::applyViscosityToVelocityField
// (viscositysolver.cpp:53-80, 832-867); the field changes only when the solve succeeds (or ends at
// the iteration limit below the acceptable residual 10).
void Engine::stage_viscosity(double dt) {
    Dims d = dims();
    launch_constrain(d.faces(0), wu, u, st); launch_constrain(d.faces(1), wv, v, st); launch_constrain(d.faces(2), ww, w, st);
    launches += 3;
    if (timing) FFGPU_CUDA(cudaEventRecord(vev[0], st));
    const int n = visc_build(d, dx, dt, (float)viscosity, phi, solid, u, v, w, visc_work, host_int, st, launches);
    last_visc.rows = n;
    if (n == 0) return;
    if (timing) FFGPU_CUDA(cudaEventRecord(vev[1], st));
    int it = 0;
    float res = 0.0f;
    bool wait_failed = false;
    const WfWork ww = wf_work(nullptr);
    visc_work.warm = visc_warm;
    const bool conv = visc_solve(visc_work, visc_tolerance, visc_max_iterations, host_dbl, host_int, ww, it, res,
                                 wait_failed, st, launches, timing ? vev[2] : nullptr);
    if (timing) {
        FFGPU_CUDA(cudaEventRecord(vev[3], st));
        FFGPU_CUDA(cudaEventSynchronize(vev[3]));
        FFGPU_CUDA(cudaEventElapsedTime(&last_visc.build_ms, vev[0], vev[1]));
        FFGPU_CUDA(cudaEventElapsedTime(&last_visc.factor_ms, vev[1], vev[2]));
        FFGPU_CUDA(cudaEventElapsedTime(&last_visc.pcg_ms, vev[2], vev[3]));
    }
    if (wait_failed) check_error_word("viscosity solve");   // throws; the velocity field is unchanged
    const bool ok = conv || (it == visc_max_iterations && res < 10.0f);
    last_visc.iterations = it;
    last_visc.error = res;
    last_visc.success = ok;
    if (ok) {
        visc_apply(d, visc_work, u, v, w, st);
        launches++;
    }
}

// The viscosity system of the current fields, its factor and one preconditioner application to its
// right-hand side (into visc_work.z) in the given form; returns the rows.
int Engine::viscosity_precondition_probe(double dt, float visc, int form, int sweeps) {
    Dims d = dims();
    launch_constrain(d.faces(0), wu, u, st); launch_constrain(d.faces(1), wv, v, st); launch_constrain(d.faces(2), ww, w, st);
    ViscWork &W = visc_work;
    const int n = visc_build(d, dx, dt, visc, phi, solid, u, v, w, W, host_int, st, launches);
    if (n == 0) return 0;
    visc_factor(W, st, launches);
    if (form == ViscWork::VP_WAVEFRONT || form == ViscWork::VP_WAVEFRONT_GRID_AXES) {
        W.axis_order = form == ViscWork::VP_WAVEFRONT ? 1 : 0;
        const WfWork wk = wf_work(nullptr);
        visc_wavefront_setup(W, st, launches);
        visc_precondition_wf(W, W.rhs, W.z, wk, sweeps, st, launches);
    } else if (form == ViscWork::VP_LEVELS) {
        visc_precondition(W, W.rhs, W.z, st, launches, sweeps);
    } else if (!visc_precondition_coop(W, W.rhs, W.z, st, launches)) {
        throw std::runtime_error("Error: the device cannot launch the cooperative preconditioner.\n");
    }
    check_error_word("viscosity preconditioner");
    return n;
}

void Engine::stage_g2p(cudaStream_t on) {
    ensure_affine();
    cudaStream_t s_ = on ? on : st;
    if (apic) {
        float *a9[9];
        for (int q = 0; q < 9; q++) a9[q] = aff[q];
        launch_g2p_apic(dims(), dx, np, px, py, pz, vx, vy, vz, a9, MacView{u, v, w}, gridpos, gridpos_max(), s_);
        launches++;
        return;
    }
    launch_g2p(dims(), dx, (float)pic_ratio, np, px, py, pz, vx, vy, vz, MacView{u, v, w}, MacView{su, sv, sw}, s_);
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
    last_speed_limit = 0.0f;
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
        last_speed_limit = fms;
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
    const float *src[15] = {px, py, pz, vx, vy, vz};
    float *dst[15] = {cpx, cpy, cpz, cvx, cvy, cvz};
    const bool with_aff = aff_ready;
    for (int q = 0; with_aff && q < 9; q++) { src[6 + q] = aff[q]; dst[6 + q] = caff[q]; }
    launch_compact(np, final_keep, off, src, dst, with_aff ? 15 : 6, st);
    launches++;
    if (ids_on) {   // the ids move with the particles (32-bit slots copied bit for bit)
        const float *isrc[1] = {reinterpret_cast<const float *>(pid.p)};
        float *idst[1] = {reinterpret_cast<float *>(cpid.p)};
        launch_compact(np, final_keep, off, isrc, idst, 1, st);
        launches++;
        std::swap(pid.p, cpid.p);
    }
    std::swap(px.p, cpx.p); std::swap(py.p, cpy.p); std::swap(pz.p, cpz.p);
    std::swap(vx.p, cvx.p); std::swap(vy.p, cvy.p); std::swap(vz.p, cvz.p);
    for (int q = 0; with_aff && q < 9; q++) std::swap(aff[q].p, caff[q].p);
    np = nnew;
}

void Engine::substep(double dt) {
    if (!in_update) last_frame_dt = dt;
    if (np == 0) {
        last_solve = SolveStats();
        return;
    }
    refresh_solid();   // FluidSimulation::_updateObstacleObjects (fluidsimulation.cpp:5550-5580)
    ensure_affine();
    mark(0);
    stage_sort();
    mark(1);
    // the liquid level set on a side stream, beside P2G and the extrapolation on the engine's stream
    // (the first reads the sorted particles and writes phi; the others the grid velocities); the
    // engine's stream waits for it before the first use of phi
    FFGPU_CUDA(cudaEventRecord(xevent[3], st));
    FFGPU_CUDA(cudaStreamWaitEvent(xstream[2], xevent[3], 0));
    if (timing) FFGPU_CUDA(cudaEventRecord(tev[14], xstream[2]));
    stage_sdf(true, xstream[2]);
    if (timing) FFGPU_CUDA(cudaEventRecord(tev[15], xstream[2]));
    FFGPU_CUDA(cudaEventRecord(xevent[4], xstream[2]));
    mark(2);
    stage_p2g();
    mark(3);
    stage_extrapolate_all();
    FFGPU_CUDA(cudaStreamWaitEvent(st, xevent[4], 0));
    mark(4);
    stage_surface_tension();
    stage_save_and_body_force(dt);
    last_visc = ViscStats();
    if (viscosity_enabled && viscosity > 0) stage_viscosity(dt);
    mark(5);
    bool ok = stage_pressure(dt);   // marks 6 (system built), 7 (factored), 8 (solved)
    if (check_tolerance > 0.0) check_solve(dt);
    if (ok) stage_project(dt);
    if (check_tolerance > 0.0 && ok) check_projection();
    mark(9);
    stage_extrapolate_all();
    stage_constrain();
    mark(10);
    // G2P (particle velocities from the grid) on the side stream beside the RK3 advection (positions
    // from the grid): both read the old positions and the same grid; removal waits for both
    FFGPU_CUDA(cudaEventRecord(xevent[3], st));
    FFGPU_CUDA(cudaStreamWaitEvent(xstream[2], xevent[3], 0));
    if (timing) FFGPU_CUDA(cudaEventRecord(tev[16], xstream[2]));
    stage_g2p(xstream[2]);
    if (timing) FFGPU_CUDA(cudaEventRecord(tev[17], xstream[2]));
    FFGPU_CUDA(cudaEventRecord(xevent[4], xstream[2]));
    mark(11);
    stage_advect(dt);
    FFGPU_CUDA(cudaStreamWaitEvent(st, xevent[4], 0));
    mark(12);
    stage_remove();
    mark(13);
    if (timing) {
        FFGPU_CUDA(cudaEventSynchronize(tev[13]));
        auto el = [&](int a, int b_) { float ms = 0; cudaEventElapsedTime(&ms, tev[a], tev[b_]); return ms; };
        last_times.sort = el(0, 1);
        last_times.sdf = el(14, 15);   // on its own stream, beside P2G and the extrapolation
        last_times.p2g = el(2, 3);
        last_times.extrap = el(3, 4) + el(9, 10);
        last_times.pressure_build = el(5, 6);
        last_times.factor = el(6, 7);
        last_times.pcg = el(7, 8);
        last_times.project = el(8, 9);
        last_times.g2p = el(16, 17);   // on its own stream, beside the advection
        last_times.advect = el(11, 12);
        last_times.remove = el(12, 13);
        last_times.total = el(0, 13);
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

namespace ffgpu {
float Engine::time_kernel(int id, int reps, double *bytes) {
    if (!is_init) throw std::runtime_error("Error: FluidSimulation must be initialized first.\n");
    Dims d = dims();
    size_t nc = d.cells();
    size_t nbox = have_fluid_cells ? (size_t)(bbox.i1 - bbox.i0 + 1) * (bbox.j1 - bbox.j0 + 1) * (bbox.k1 - bbox.k0 + 1) : 0;
    double B = 0.0;
    auto run = [&]() {
        switch (id) {
        case 0:
            launch_p2g3(d, dx, radius(), cell_start, spx, spy, spz, svx, svy, svz, gridpos, blockpos, u, v, w, vu, vv, vw,
                        st);
            break;
        case 1:
            sdf_rec.reserve((size_t)std::max(cap, 1));
            launch_liquid_sdf(d, dx, radius(), np, cell_start, spx, spy, spz, sdf_rec, solid, 1, phi, st);
            break;
        // ids 2 and 3 run on the layout the last mixed solve used (the grid's own or the
        // axis-ordered copy)
        case 2:
            if (perm_active && perm_ready)
                pcg_spmv_dot_split(perm_dims, perm_box, OpView<float>{pdiag32, pax32, pay32, paz32},
                                   OpView<float>{pdiag32lo, pax32lo, pay32lo, paz32lo},
                                   PcgVecs<float>{px32, pr32, ps32, pz32}, PcgWork{partials, counter, scal}, st);
            else
                pcg_spmv_dot_split(d, bbox, OpView<float>{diag32, ax32, ay32, az32},
                                   OpView<float>{diag32lo, ax32lo, ay32lo, az32lo}, PcgVecs<float>{x32, r32, s32, z32},
                                   PcgWork{partials, counter, scal}, st);
            break;
        case 3:
            if (perm_active && perm_ready)
                precondition<float>(perm_dims, perm_box, FactorView<float>{pinv32, plx32, ply32, plz32}, pr32, pz32);
            else
                precondition<float>(FactorView<float>{inv32, lx32, ly32, lz32}, r32, z32);
            break;
        case 4: launch_extrapolate_front(ni + 1, nj, nk, u, vu, (int)std::ceil(std::sqrt(3) * cfl) + 3, front(), st); break;
        case 5: launch_g2p(d, dx, (float)pic_ratio, np, px, py, pz, cvx, cvy, cvz, MacView{u, v, w}, MacView{su, sv, sw}, st); break;
        case 6: launch_advect(d, dx, 1.0 / 240.0, (int)cfl, np, px, py, pz, ox, oy, oz, MacView{u, v, w}, solid, ng, near, st); break;
        case 7: stage_sort(); break;
        case 8: {
            launch_apic_records(d, dx, radius(), np, spx, spy, spz, apic_rec, st);
            const float *sa[3] = {saff[0], saff[1], saff[2]};
            launch_p2g_apic(d, dx, radius(), 0, cell_start, spx, spy, spz, svx, sa, apic_rec, np, gridpos, blockpos, u, vu, st);
            break;
        }
        case 9: {
            float *a9[9];
            for (int q = 0; q < 9; q++) a9[q] = caff[q];
            launch_g2p_apic(d, dx, np, px, py, pz, cvx, cvy, cvz, a9, MacView{u, v, w}, gridpos, gridpos_max(), st);
            break;
        }
        case 10: stage_viscosity(1.0 / 240.0); break;
        case 11: output_fluid_particles(); break;
        default: throw std::domain_error("Error: unknown kernel id.\n");
        }
    };
    switch (id) {
    case 0: B = 24.0 * np + 4.0 * nc + 5.0 * (double)(d.faces(0) + d.faces(1) + d.faces(2)); break;   // all three
    case 1: B = 12.0 * np + 8.0 * nc + 4.0 * (double)(ni + 1) * (nj + 1) * (nk + 1); break;
    case 2: B = 40.0 * nbox; break;   // s, z and the operator as hi + lo floats
    case 3: B = 48.0 * nbox; break;
    case 4: B = 0.0; break;   // frontier-dependent; reported as time only
    case 5: B = 36.0 * np + 2.0 * 4.0 * (d.faces(0) + d.faces(1) + d.faces(2)); break;
    case 6: B = 24.0 * np + 4.0 * (d.faces(0) + d.faces(1) + d.faces(2)); break;
    case 7: B = 52.0 * np + 12.0 * nc; break;
    case 8: B = 72.0 * np + 4.0 * nc + 5.0 * d.faces(0); break;   // records (12 in, 24 out) + gather (36 in)
    case 9: B = 60.0 * np + 4.0 * (d.faces(0) + d.faces(1) + d.faces(2)); break;
    case 10: B = 0.0; break;   // solve-dependent; reported as time only
    case 11: B = 0.0; break;   // set after the run: the output bytes plus the particle attributes read
    }
    if ((id == 8 || id == 9) && !(apic && aff_ready))
        throw std::runtime_error("Error: APIC kernels are timed after an APIC substep.\n");
    if ((id == 2 || id == 3) && (!have_fluid_cells || solver != SOLVER_MIXED))
        throw std::runtime_error("Error: FP32 solver kernels are timed after a mixed-precision substep.\n");
    if (id == 2 || id == 3) reset_scalars(scal, host_sc, -1.0, st);   // clear the converged flag
    if (id == 5) {
        FFGPU_CUDA(cudaMemcpyAsync(cvx.p, vx.p, (size_t)np * 4, cudaMemcpyDeviceToDevice, st));
        FFGPU_CUDA(cudaMemcpyAsync(cvy.p, vy.p, (size_t)np * 4, cudaMemcpyDeviceToDevice, st));
        FFGPU_CUDA(cudaMemcpyAsync(cvz.p, vz.p, (size_t)np * 4, cudaMemcpyDeviceToDevice, st));
    }
    // the viscosity solve is timed with viscosity 1 unless one is set; the setting is restored after
    const bool visc_was = viscosity_enabled;
    const double visc_value = viscosity;
    if (id == 10) {
        viscosity_enabled = true;
        if (!(viscosity > 0)) viscosity = 1.0;
    }
    run();   // warm
    FFGPU_CUDA(cudaEventRecord(ev[13], st));
    for (int q = 0; q < reps; q++) run();
    FFGPU_CUDA(cudaEventRecord(ev[14], st));
    FFGPU_CUDA(cudaEventSynchronize(ev[14]));
    viscosity_enabled = visc_was;
    viscosity = visc_value;
    float ms = 0.0f;
    FFGPU_CUDA(cudaEventElapsedTime(&ms, ev[13], ev[14]));
    if (id == 11)   // the FFP3 bytes written and the positions, velocities and ids read
        B = (double)(ffp_counts.bytes[0] + ffp_counts.bytes[1] + ffp_counts.bytes[2] + ffp_counts.bytes[3]) + 28.0 * np;
    if (bytes) *bytes = B;
    return ms / (float)std::max(reps, 1);
}
}  // namespace ffgpu
