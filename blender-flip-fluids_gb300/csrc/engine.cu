// Host engine of the GB300 FLIP substep (see engine.h).
#include "engine.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <stdexcept>

namespace ffgpu {

// speed-limit kernels (particle_kernels.cu)
void launch_speed_hist(int np, const float *vx, const float *vy, const float *vz, double step, int nbins,
                       int *bins, unsigned long long *maxbits, cudaStream_t st);
void launch_speed_outliers(int np, const float *vx, const float *vy, const float *vz, double lower, double upper,
                           int *counts, cudaStream_t st);
void launch_remove_mark2(Dims d, double dx, int np, const float *px, const float *py, const float *pz,
                         const float *vx, const float *vy, const float *vz, const float *solid, double maxspeedsq,
                         int *keep, int *key, int *cell_count, int *max_count, cudaStream_t st);
void launch_keep01(int np, const int *keep, int *keep01, cudaStream_t st);
void launch_deinterleave(int np, const float *aos, float *x, float *y, float *z, cudaStream_t st);
void launch_interleave(int np, const float *x, const float *y, const float *z, float *aos, cudaStream_t st);

Engine::Engine(int ni_, int nj_, int nk_, double dx_) : ni(ni_), nj(nj_), nk(nk_), dx(dx_) {
    if (ni <= 0 || nj <= 0 || nk <= 0)
        throw std::domain_error("Error: grid dimensions must be greater than 0.\n");
    if (!(dx > 0.0)) throw std::domain_error("Error: cell size must be greater than 0.\n");
    int dev = 0;
    FFGPU_CUDA(cudaGetDevice(&dev));
    FFGPU_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    FFGPU_CUDA(cudaMallocHost(&host_sc, sizeof(PcgScalars)));
    FFGPU_CUDA(cudaMallocHost(&host_int, 16 * sizeof(int)));
    FFGPU_CUDA(cudaMallocHost(&host_dbl, 16 * sizeof(double)));
    for (auto &e : ev) FFGPU_CUDA(cudaEventCreate(&e));
    for (auto &e : tev) FFGPU_CUDA(cudaEventCreate(&e));
}

Engine::~Engine() {
    if (st) cudaStreamSynchronize(st);
    for (auto &e : ev) cudaEventDestroy(e);
    for (auto &e : tev) cudaEventDestroy(e);
    if (host_sc) cudaFreeHost(host_sc);
    if (host_int) cudaFreeHost(host_int);
    if (host_dbl) cudaFreeHost(host_dbl);
    if (st) cudaStreamDestroy(st);
}

double Engine::radius() const { return 0.5 * 1.0 * dx * std::sqrt(3.0); }   // fluidsimulation.cpp:4351

void Engine::load_particles(const float *pos, const float *vel, int count) {
    if (count < 0) throw std::domain_error("Error: particle count must be non-negative.\n");
    pend_pos.insert(pend_pos.end(), pos, pos + 3 * (size_t)count);
    pend_vel.insert(pend_vel.end(), vel, vel + 3 * (size_t)count);
    if (is_init) {
        // particles loaded after initialisation join at the next update (as queued loads do)
        std::vector<float> hp, hv;
        int cur = np;
        hp.resize(3 * (size_t)cur); hv.resize(3 * (size_t)cur);
        if (cur) { get_positions(hp.data(), 0, cur); get_velocities(hv.data(), 0, cur); }
        hp.insert(hp.end(), pend_pos.begin(), pend_pos.end());
        hv.insert(hv.end(), pend_vel.begin(), pend_vel.end());
        pend_pos.clear(); pend_vel.clear();
        set_particles(hp.data(), hv.data(), (int)(hp.size() / 3));
    }
}

void Engine::alloc_grids() {
    Dims d = dims();
    size_t nc = d.cells(), nn = (size_t)(ni + 1) * (nj + 1) * (nk + 1);
    size_t nu = d.faces(0), nv = d.faces(1), nw = d.faces(2);
    size_t nfmax = std::max(nu, std::max(nv, nw));
    solid.reserve(nn); wu.reserve(nu); wv.reserve(nv); ww.reserve(nw);
    ng.cell = 3 * dx;
    ng.w = (int)std::ceil(ni * dx / ng.cell); ng.h = (int)std::ceil(nj * dx / ng.cell); ng.d = (int)std::ceil(nk * dx / ng.cell);
    near.reserve((size_t)ng.w * ng.h * ng.d * 2);
    phi.reserve(nc); pressure.reserve(nc);
    u.reserve(nu); v.reserve(nv); w.reserve(nw); su.reserve(nu); sv.reserve(nv); sw.reserve(nw);
    vu.reserve(nu); vv.reserve(nv); vw.reserve(nw); st1.reserve(nfmax); st2.reserve(nfmax);
    xlist1.reserve(nfmax); xlist2.reserve(nfmax); xcount.reserve(2);
    cell_count.reserve(nc + 1); cell_start.reserve(nc + 1);
    scan_tmp.reserve(scan_scratch_ints(std::max(nc + 1, (size_t)1 << 20)) + 64);
    for (DevBuf<double> *b_ : {&diag, &ax, &ay, &az, &inv, &lx, &ly, &lz, &b, &x64, &r64, &s64, &z64}) b_->reserve(nc);
    for (DevBuf<float> *b_ : {&diag32, &ax32, &ay32, &az32, &inv32, &lx32, &ly32, &lz32, &x32, &r32, &s32, &z32,
                              &diag32lo, &ax32lo, &ay32lo, &az32lo})
        b_->reserve(nc);
    fluid.reserve(nc);
    partials.reserve(MAX_RED_BLOCKS);
    {
        size_t tiles = (size_t)mic_wavefront_max_tiles(ni, nj) + 1;
        wf_order.reserve(tiles); wf_ticket.reserve(2); errword.reserve(1);
        FFGPU_CUDA(cudaMemsetAsync(wf_ticket.p, 0, 2 * sizeof(unsigned int), st));
        wf_xchg.reserve(mic_wavefront_xchg_words(ni, nj, nk));
        FFGPU_CUDA(cudaMemsetAsync(wf_xchg.p, 0, wf_xchg.n * sizeof(unsigned long long), st));
        wf_epoch = 0;
        FFGPU_CUDA(cudaMemsetAsync(errword.p, 0, sizeof(unsigned int), st));
    }
    counter.reserve(1);
    scal.reserve(1);
    bbox_dev.reserve(6);
    maxabs_b.reserve(1);
    maxcount.reserve(4);
    speedbits.reserve(4);
    FFGPU_CUDA(cudaMemsetAsync(counter.p, 0, sizeof(unsigned int), st));
    FFGPU_CUDA(cudaMemsetAsync(scal.p, 0, sizeof(PcgScalars), st));
    FFGPU_CUDA(cudaMemsetAsync(u.p, 0, nu * 4, st));
    FFGPU_CUDA(cudaMemsetAsync(v.p, 0, nv * 4, st));
    FFGPU_CUDA(cudaMemsetAsync(w.p, 0, nw * 4, st));
    FFGPU_CUDA(cudaMemsetAsync(pressure.p, 0, nc * 4, st));
}

void Engine::ensure_particle_capacity(int count) {
    if (count <= cap) return;
    int ncap = std::max(count, cap + cap / 4);
    // preserve current particle state across the reallocation
    std::vector<float> hp, hv;
    if (np) {
        hp.resize(3 * (size_t)np); hv.resize(3 * (size_t)np);
        get_positions(hp.data(), 0, np); get_velocities(hv.data(), 0, np);
    }
    for (DevBuf<float> *b_ : {&px, &py, &pz, &vx, &vy, &vz, &spx, &spy, &spz, &svx, &svy, &svz, &ox, &oy, &oz,
                              &cpx, &cpy, &cpz, &cvx, &cvy, &cvz})
        b_->reserve(ncap);
    for (DevBuf<int> *b_ : {&key, &rank, &sidx, &keep, &keep2}) b_->reserve(ncap);
    stage.reserve(3 * (size_t)ncap);
    off.reserve((size_t)ncap + 1);
    scan_tmp.reserve(scan_scratch_ints(std::max((size_t)ncap + 1, dims().cells() + 1)) + 64);
    cap = ncap;
    if (!hp.empty()) set_particles(hp.data(), hv.data(), (int)(hp.size() / 3));
}

void Engine::set_particles(const float *pos, const float *vel, int count) {
    if (count < 0) throw std::domain_error("Error: particle count must be non-negative.\n");
    if (count > cap) { np = 0; ensure_particle_capacity(count); }
    // interleaved host arrays -> staging -> SoA (a pinned caller buffer makes the copy async)
    if (count) {
        FFGPU_CUDA(cudaMemcpyAsync(stage.p, pos, (size_t)count * 12, cudaMemcpyHostToDevice, st));
        launch_deinterleave(count, stage, px, py, pz, st);
        FFGPU_CUDA(cudaMemcpyAsync(stage.p, vel, (size_t)count * 12, cudaMemcpyHostToDevice, st));
        launch_deinterleave(count, stage, vx, vy, vz, st);
        launches += 2;
    }
    FFGPU_CUDA(cudaStreamSynchronize(st));
    np = count;
}

void Engine::read_interleaved(const float *a, const float *b_, const float *c, float *out, int start, int end) const {
    int n = end - start;
    if (n <= 0) return;
    launch_interleave(n, a + start, b_ + start, c + start, stage, st);
    FFGPU_CUDA(cudaMemcpyAsync(out, stage.p, (size_t)n * 12, cudaMemcpyDeviceToHost, st));
    FFGPU_CUDA(cudaStreamSynchronize(st));
}

void Engine::get_positions(float *out, int start, int end) const {
    if (start < 0 || end > np || start > end) throw std::out_of_range("Error: particle range out of bounds.\n");
    read_interleaved(px, py, pz, out, start, end);
}

void Engine::get_velocities(float *out, int start, int end) const {
    if (start < 0 || end > np || start > end) throw std::out_of_range("Error: particle range out of bounds.\n");
    read_interleaved(vx, vy, vz, out, start, end);
}

void Engine::solid_changed() {
    Dims d = dims();
    launch_face_weights(d, solid, wu, wv, ww, st);
    launch_near_solid(d, dx, (int)cfl, solid, ng, near.p, near.p + (size_t)ng.w * ng.h * ng.d, st);
    launches += 3 + 2 * (size_t)std::ceil(cfl / 3.0);
}

void Engine::set_solid_phi(const float *host_phi) {
    if (!is_init) throw std::runtime_error("Error: FluidSimulation must be initialized before setting the solid level set.\n");
    size_t nn = (size_t)(ni + 1) * (nj + 1) * (nk + 1);
    FFGPU_CUDA(cudaMemcpyAsync(solid.p, host_phi, nn * 4, cudaMemcpyHostToDevice, st));
    custom_solid = true;
    solid_changed();
    FFGPU_CUDA(cudaStreamSynchronize(st));
}

void Engine::initialize() {
    if (is_init) return;
    alloc_grids();
    launch_solid_phi(dims(), dx, spheres, nspheres, solid, st);
    launches++;
    solid_changed();
    // particles outside the domain are dropped on load (fluidsimulation.cpp:5011-5016)
    std::vector<float> hp, hv;
    double W = ni * dx, H = nj * dx, D = nk * dx;
    for (size_t p = 0; p < pend_pos.size() / 3; p++) {
        float x = pend_pos[3 * p], y = pend_pos[3 * p + 1], z = pend_pos[3 * p + 2];
        if (x >= 0.0f && y >= 0.0f && z >= 0.0f && x < W && y < H && z < D) {
            hp.insert(hp.end(), {x, y, z});
            hv.insert(hv.end(), {pend_vel[3 * p], pend_vel[3 * p + 1], pend_vel[3 * p + 2]});
        }
    }
    pend_pos.clear(); pend_vel.clear();
    int count = (int)(hp.size() / 3);
    ensure_particle_capacity(std::max(count, 1024));
    if (count) set_particles(hp.data(), hv.data(), count);
    FFGPU_CUDA(cudaStreamSynchronize(st));
    is_init = true;
}

double Engine::max_particle_speed() {
    if (np == 0) return 0.0;
    launch_max_speed_sq(np, vx, vy, vz, nullptr, speedbits, nullptr, st);
    launches++;
    unsigned int bits;
    FFGPU_CUDA(cudaMemcpyAsync(host_int, speedbits.p, 4, cudaMemcpyDeviceToHost, st));
    FFGPU_CUDA(cudaStreamSynchronize(st));
    bits = (unsigned int)host_int[0];
    float f;
    std::memcpy(&f, &bits, 4);
    return std::sqrt((double)f);
}

// FluidSimulation::_calculateNextTimeStep (fluidsimulation.cpp:10231-10263), static solids
double Engine::next_timestep(double frame_dt) {
    double maxu;
    if (current_frame == 0 && frame_substeps == 0) {
        float gl = std::sqrt(gx * gx + gy * gy + gz * gz);
        maxu = (double)gl * frame_dt;   // _predictMaximumMarkerParticleSpeed, no inflows
    } else {
        maxu = max_particle_speed();
    }
    double eps = 1e-6;
    double ts = cfl * dx / (maxu + eps);
    int n = std::max((int)std::ceil(frame_dt / ts), 1);
    return frame_dt / n;
}

// FluidSimulation::update (fluidsimulation.cpp:10410-10543)
void Engine::update(double dt) {
    if (!is_init) throw std::runtime_error("Error: FluidSimulation must be initialized before update.\n");
    if (dt < 0.0) throw std::domain_error("Error: delta time must be greater than or equal to 0.\n");
    auto t0 = std::chrono::steady_clock::now();
    double epsdt = 1e-6;
    bool zero_len = dt < epsdt;
    dt = std::max(dt, epsdt);
    bool skipped = zero_len && current_frame > 0;
    double substep_time = dt / (double)min_substeps;
    last_frame_dt = dt;
    in_update = true;
    double remaining = dt;
    frame_substeps = 0;
    frame_solve = SolveStats();
    size_t processed = 0;
    double processed_time = 0.0;
    const double eps = 1e-9;
    do {
        auto s0 = std::chrono::steady_clock::now();
        double ts = std::fmin(next_timestep(dt), remaining);
        double completed = dt - remaining;
        double limit = (frame_substeps + 1) * substep_time;
        if (completed + ts > limit) ts = std::fmin(substep_time, remaining);
        if (frame_substeps == max_substeps - 1) ts = remaining;
        remaining -= ts;
        if (!skipped) {
            substep(ts);
            if (frame_substeps == 0) frame_solve = last_solve;
            else if (frame_solve.success && (!last_solve.success || last_solve.iterations > frame_solve.iterations))
                frame_solve = last_solve;
        }
        processed += (size_t)np;
        processed_time += std::chrono::duration<double>(std::chrono::steady_clock::now() - s0).count();
        frame_substeps++;
    } while (remaining > eps);
    in_update = false;
    frame_time = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    total_time += frame_time;
    performance_score = (processed == 0 || processed_time < 1e-9) ? -1 : (int)(((double)processed / processed_time) / 1000.0);
    current_frame++;
}

}  // namespace ffgpu
