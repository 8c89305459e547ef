// Host engine of the GB300 FLIP substep (see engine.h).
#include "engine.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
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
void launch_deinterleave_checked(int np, const float *aos, float *x, float *y, float *z, const double *hi,
                                 unsigned int bit, unsigned int *flag, cudaStream_t st);
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
    for (auto &e : vev) FFGPU_CUDA(cudaEventCreate(&e));
    for (auto &s_ : xstream) FFGPU_CUDA(cudaStreamCreateWithFlags(&s_, cudaStreamNonBlocking));
    // the level set (beside P2G and the extrapolation) and G2P (beside the advection) run on xstream[2]
    // at the highest priority: the first is the longer chain of its pair, the second the shorter
    {
        int least = 0, greatest = 0;
        FFGPU_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        FFGPU_CUDA(cudaStreamDestroy(xstream[2]));
        FFGPU_CUDA(cudaStreamCreateWithPriority(&xstream[2], cudaStreamNonBlocking, greatest));
    }
    for (auto &e : xevent) FFGPU_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
}

Engine::~Engine() {
    if (st) cudaStreamSynchronize(st);
    for (auto &e : ev) cudaEventDestroy(e);
    for (auto &e : tev) cudaEventDestroy(e);
    for (auto &e : vev) cudaEventDestroy(e);
    for (auto &s_ : xstream)
        if (s_) { cudaStreamSynchronize(s_); cudaStreamDestroy(s_); }
    for (auto &e : xevent)
        if (e) cudaEventDestroy(e);
    if (host_sc) cudaFreeHost(host_sc);
    if (host_int) cudaFreeHost(host_int);
    if (host_dbl) cudaFreeHost(host_dbl);
    for (float *b_ : host_io)
        if (b_) cudaFreeHost(b_);
    if (st) cudaStreamDestroy(st);
}

double Engine::radius() const { return 0.5 * 1.0 * dx * std::sqrt(3.0); }   // fluidsimulation.cpp:4351

bool Engine::in_domain(float x, float y, float z) const {
    // AABB(0, 0, 0, isize dx, jsize dx, ksize dx).isPointInside (fluidsimulation.cpp:5011-5016)
    double W = ni * dx, H = nj * dx, D = nk * dx;
    return x >= 0.0f && y >= 0.0f && z >= 0.0f && x < W && y < H && z < D;
}

// The reference queues a loaded batch in a FragmentedVector of 5e6-byte fragments
// (fluidsimulation.cpp:3829-3836, fluidsimulation.h:1628-1634, fragmentedvector.h:320) and reads it
// back with operator[] (fragmentedvector.h:147-152), which finds element i's fragment as
// (int)(i * (1.0 / E)) for E records per fragment but its place in the fragment as i % E.  Where
// that product rounds below an integer k (i = k E), element i reads the first record of fragment
// k - 1 instead of its own: the record is duplicated and record k E is lost.  Returns the input
// record that element i of a batch becomes.
static size_t fragment_source(int i, int record_bytes) {
    const int E = std::max(5000000 / record_bytes, 1);
    const double inv = 1.0 / (double)E;
    const int node = (int)(i * inv);
    return (size_t)node * E + (size_t)(i % E);
}

// A batch in the order the reference's load queue hands it over (see fragment_source).
template <typename T>
static std::vector<T> as_loaded(const T *src, int count, int record_bytes, int items_per_record) {
    std::vector<T> out((size_t)items_per_record * count);
    for (int i = 0; i < count; i++) {
        const size_t from = fragment_source(i, record_bytes);
        std::copy(src + items_per_record * from, src + items_per_record * (from + 1), out.begin() + (size_t)items_per_record * i);
    }
    return out;
}

void Engine::load_particles(const float *pos_in, const float *vel_in, int count) {
    if (count < 0) throw std::domain_error("Error: particle count must be non-negative.\n");
    // MarkerParticle records: position + velocity, 24 bytes
    const std::vector<float> lp = as_loaded(pos_in, count, 24, 3), lv = as_loaded(vel_in, count, 24, 3);
    const float *pos = lp.data(), *vel = lv.data();
    if (!is_init) {
        pend_pos.insert(pend_pos.end(), pos, pos + 3 * (size_t)count);
        pend_vel.insert(pend_vel.end(), vel, vel + 3 * (size_t)count);
        pend_counts.push_back(count);
        return;
    }
    // particles loaded after initialisation join at once (as queued loads do at the next
    // update), filtered to the domain like the initial load; an affine batch that follows
    // pairs with them
    std::vector<float> hp, hv, ha[3];
    int cur = np;
    hp.resize(3 * (size_t)cur); hv.resize(3 * (size_t)cur);
    if (cur) { get_positions(hp.data(), 0, cur); get_velocities(hv.data(), 0, cur); }
    if (aff_ready) read_affine_host(ha);
    std::vector<unsigned int> hid = ids_on ? read_ids_host() : std::vector<unsigned int>();
    join_kept.clear();
    for (int p = 0; p < count; p++) {
        if (!in_domain(pos[3 * p], pos[3 * p + 1], pos[3 * p + 2])) continue;
        join_kept.push_back(p);
        hp.insert(hp.end(), pos + 3 * p, pos + 3 * p + 3);
        hv.insert(hv.end(), vel + 3 * p, vel + 3 * p + 3);
        if (aff_ready)
            for (auto &h : ha) h.insert(h.end(), {0.0f, 0.0f, 0.0f});
    }
    if (ids_on) {   // random ids, unless an id batch of the same size follows
        const std::vector<unsigned int> r = random_ids((int)join_kept.size());
        hid.insert(hid.end(), r.begin(), r.end());
    }
    join_start = cur;
    join_size = count;
    join_id_size = count;
    const float *a3[3] = {ha[0].data(), ha[1].data(), ha[2].data()};
    set_particles(hp.data(), hv.data(), (int)(hp.size() / 3), aff_ready ? a3 : nullptr, ids_on ? hid.data() : nullptr);
}

// FluidSimulation::loadMarkerParticleAffineData (fluidsimulation.cpp:3841-3863) and its
// pairing with the particle batches in _loadParticles (:5077-5110)
void Engine::load_affine(const float *afx_in, const float *afy_in, const float *afz_in, int count) {
    if (count < 0) throw std::domain_error("Error: affine data count must be non-negative.\n");
    if (count == 0) return;   // an empty batch is not queued
    // MarkerParticleAffine records: three vec3, 36 bytes (read back like the particle queue)
    const std::vector<float> la = as_loaded(afx_in, count, 36, 3), lb = as_loaded(afy_in, count, 36, 3),
                             lc = as_loaded(afz_in, count, 36, 3);
    const float *afx = la.data(), *afy = lb.data(), *afz = lc.data();
    if (!is_init) {
        std::vector<float> b_(9 * (size_t)count);
        std::copy(afx, afx + 3 * (size_t)count, b_.begin());
        std::copy(afy, afy + 3 * (size_t)count, b_.begin() + 3 * (size_t)count);
        std::copy(afz, afz + 3 * (size_t)count, b_.begin() + 6 * (size_t)count);
        pend_aff.push_back(std::move(b_));
        return;
    }
    if (!apic || count != join_size) return;
    join_size = -1;
    ensure_affine();
    const int n = (int)join_kept.size();
    if (n == 0) return;
    std::vector<float> h(3 * (size_t)n);
    const float *srcs[3] = {afx, afy, afz};
    for (int c = 0; c < 3; c++) {
        for (int q = 0; q < n; q++)
            for (int e = 0; e < 3; e++) h[3 * (size_t)q + e] = srcs[c][3 * (size_t)join_kept[q] + e];
        FFGPU_CUDA(cudaMemcpyAsync(stage.p, h.data(), (size_t)n * 12, cudaMemcpyHostToDevice, st));
        launch_deinterleave(n, stage, aff[3 * c].p + join_start, aff[3 * c + 1].p + join_start,
                            aff[3 * c + 2].p + join_start, st);
        FFGPU_CUDA(cudaStreamSynchronize(st));   // the pageable source and the staging buffer are reused
        launches++;
    }
}

void Engine::load_ids(const uint16_t *ids_in, int count) {
    if (count < 0) throw std::domain_error("Error: id data count must be non-negative.\n");
    if (count == 0) return;   // an empty batch is not queued (fluidsimulation.cpp:4023-4025)
    // MarkerParticleID records: one uint16 (read back like the particle queue)
    std::vector<uint16_t> la = as_loaded(ids_in, count, 2, 1);
    if (!is_init) {
        pend_ids.push_back(std::move(la));
        return;
    }
    if (!ids_on || count != join_id_size) return;
    join_id_size = -1;
    const int n = (int)join_kept.size();
    if (n == 0) return;
    std::vector<unsigned int> h((size_t)n);
    for (int q = 0; q < n; q++) h[(size_t)q] = la[(size_t)join_kept[q]];
    FFGPU_CUDA(cudaMemcpyAsync(pid.p + join_start, h.data(), (size_t)n * 4, cudaMemcpyHostToDevice, st));
    FFGPU_CUDA(cudaStreamSynchronize(st));   // the pageable source is released on return
}

std::vector<unsigned int> Engine::random_ids(int count) {
    // std::mt19937 seeded from std::random_device, uniform over 0 .. 65535 (fluidsimulation.cpp:4358-4359)
    if (!id_rng_seeded) {
        std::random_device dev;
        id_rng = std::mt19937(dev());
        id_rng_seeded = true;
    }
    std::uniform_int_distribution<> dist(0, 65535);
    std::vector<unsigned int> r((size_t)std::max(count, 0));
    for (auto &v : r) v = (unsigned int)(uint16_t)dist(id_rng);
    return r;
}

std::vector<unsigned int> Engine::read_ids_host() const {
    std::vector<unsigned int> h((size_t)np);
    if (np && ids_on) {
        FFGPU_CUDA(cudaMemcpyAsync(h.data(), pid.p, (size_t)np * 4, cudaMemcpyDeviceToHost, st));
        FFGPU_CUDA(cudaStreamSynchronize(st));
    }
    return h;
}

void Engine::get_ids(uint16_t *out, int start, int end) const {
    if (start < 0 || end > np || start > end) throw std::out_of_range("Error: particle range out of bounds.\n");
    if (!ids_on) throw std::runtime_error("Error: Invalid ParticleSystemAttribute <name=ID>\n");
    const int n = end - start;
    if (n <= 0) return;
    std::vector<unsigned int> h((size_t)n);
    FFGPU_CUDA(cudaMemcpyAsync(h.data(), pid.p + start, (size_t)n * 4, cudaMemcpyDeviceToHost, st));
    FFGPU_CUDA(cudaStreamSynchronize(st));
    for (int q = 0; q < n; q++) out[q] = (uint16_t)h[(size_t)q];
}

// FluidSimulation::_outputFluidParticles (fluidsimulation.cpp:9678-9730): the liquid level set and
// the surface level set of the current particles, then the FFP3 data of positions, ids and the
// enabled attributes
void Engine::output_fluid_particles() {
    if (!ids_on) {   // output turned on after initialisation: the particles get random ids now
        const std::vector<unsigned int> r = random_ids(np);
        ids_on = true;
        pid.reserve((size_t)std::max(cap, 1));
        cpid.reserve((size_t)std::max(cap, 1));
        if (np) FFGPU_CUDA(cudaMemcpyAsync(pid.p, r.data(), (size_t)np * 4, cudaMemcpyHostToDevice, st));
        FFGPU_CUDA(cudaStreamSynchronize(st));
    }
    Dims d = dims();
    if (np > 0) {
        stage_sort();
        stage_sdf(true);
        TensionWork tw = tension_work();
        launches += launch_curvature_grid(d, dx, phi, surf, curv, tw, st);
    }
    Ffp3Params prm = ffp;
    prm.id_limit = (int)std::round(65536 * ffp_amount);   // _getFluidParticleOutputIDLimit
    ffp_counts = launch_ffp3(d, dx, surf, np, px, py, pz, vx, vy, vz, pid, prm, ffp_work, st, launches);
    ffp_ready = true;
}

size_t Engine::ffp3_bytes(int which) const {
    if (which < 0 || which > 3) throw std::domain_error("Error: fluid particle output must be 0..3.\n");
    return ffp_ready ? ffp_counts.bytes[which] : 0;
}

void Engine::read_ffp3(int which, char *out) const {
    const size_t b = ffp3_bytes(which);
    if (!b) return;
    FFGPU_CUDA(cudaMemcpyAsync(out, ffp_work.out[which].p, b, cudaMemcpyDeviceToHost, st));
    FFGPU_CUDA(cudaStreamSynchronize(st));
}

void Engine::read_ffp3_types(unsigned char *out) const {
    if (!ffp_ready || np == 0) return;
    FFGPU_CUDA(cudaMemcpyAsync(out, ffp_work.type.p, (size_t)np, cudaMemcpyDeviceToHost, st));
    FFGPU_CUDA(cudaStreamSynchronize(st));
}

void Engine::ensure_affine() {
    if (!apic || aff_ready) return;
    for (int q = 0; q < 9; q++) {
        aff[q].reserve((size_t)std::max(cap, 1));
        saff[q].reserve((size_t)std::max(cap, 1));
        caff[q].reserve((size_t)std::max(cap, 1));
        if (np) FFGPU_CUDA(cudaMemsetAsync(aff[q].p, 0, (size_t)np * 4, st));
    }
    apic_rec.reserve(3 * (size_t)std::max(cap, 1));
    aff_ready = true;
}

void Engine::read_affine_host(std::vector<float> (&ha)[3]) const {
    for (int c = 0; c < 3; c++) {
        ha[c].resize(3 * (size_t)np);
        if (np) read_interleaved(aff[3 * c], aff[3 * c + 1], aff[3 * c + 2], ha[c].data(), 0, np);
    }
}

namespace {
constexpr long long SAVE_STATE_CHUNK = 1LL << 21;   // particles per write / read (bake.py:2865, 2657)
struct File {
    FILE *f = nullptr;
    ~File() { if (f) fclose(f); }
};
}  // namespace

void Engine::write_attribute_file(int attribute, const char *path, bool append) {
    if (attribute < 0 || attribute > 4) throw std::domain_error("Error: particle attribute must be 0..4.\n");
    if (attribute >= 2 && !aff_ready)
        throw std::runtime_error(std::string("Error: Invalid ParticleSystemAttribute <name=AFFINE") +
                                 "XYZ"[attribute - 2] + ">\n");
    const float *a = attribute == 0 ? px.p : (attribute == 1 ? vx.p : aff[3 * (attribute - 2)].p);
    const float *b_ = attribute == 0 ? py.p : (attribute == 1 ? vy.p : aff[3 * (attribute - 2) + 1].p);
    const float *c = attribute == 0 ? pz.p : (attribute == 1 ? vz.p : aff[3 * (attribute - 2) + 2].p);
    File out;
    out.f = std::fopen(path, append ? "ab" : "wb");
    if (!out.f) throw std::runtime_error(std::string("Error: cannot open ") + path + " for writing.\n");
    const size_t chunk_bytes = (size_t)SAVE_STATE_CHUNK * 12;
    for (float *&h : host_io)
        if (!h) FFGPU_CUDA(cudaMallocHost(&h, chunk_bytes));
    long long prev_n = 0;
    int prev_buf = -1;
    for (long long start = 0, q = 0; start < np; start += SAVE_STATE_CHUNK, q++) {
        const long long n = std::min<long long>(SAVE_STATE_CHUNK, np - start);
        const int buf = (int)(q & 1);
        launch_interleave((int)n, a + start, b_ + start, c + start, stage, st);
        FFGPU_CUDA(cudaMemcpyAsync(host_io[buf], stage.p, (size_t)n * 12, cudaMemcpyDeviceToHost, st));
        FFGPU_CUDA(cudaEventRecord(ev[buf], st));
        launches++;
        if (prev_buf >= 0) {   // the previous chunk is on the host: write it while this one copies
            FFGPU_CUDA(cudaEventSynchronize(ev[prev_buf]));
            if (std::fwrite(host_io[prev_buf], 12, (size_t)prev_n, out.f) != (size_t)prev_n)
                throw std::runtime_error(std::string("Error: short write to ") + path + "\n");
        }
        prev_buf = buf;
        prev_n = n;
    }
    if (prev_buf >= 0) {
        FFGPU_CUDA(cudaEventSynchronize(ev[prev_buf]));
        if (std::fwrite(host_io[prev_buf], 12, (size_t)prev_n, out.f) != (size_t)prev_n)
            throw std::runtime_error(std::string("Error: short write to ") + path + "\n");
    }
    if (std::fflush(out.f) != 0) throw std::runtime_error(std::string("Error: cannot write ") + path + "\n");
}

long long Engine::load_attribute_files(const char *pos_path, const char *vel_path, const char *afx_path,
                                       const char *afy_path, const char *afz_path) {
    const bool with_aff = afx_path && afy_path && afz_path;
    const char *paths[5] = {pos_path, vel_path, afx_path, afy_path, afz_path};
    File in[5];
    long long n = -1;
    for (int t = 0; t < (with_aff ? 5 : 2); t++) {
        in[t].f = std::fopen(paths[t], "rb");
        if (!in[t].f) throw std::runtime_error(std::string("Error: cannot open ") + paths[t] + "\n");
        std::fseek(in[t].f, 0, SEEK_END);
        const long long bytes = std::ftell(in[t].f);
        std::fseek(in[t].f, 0, SEEK_SET);
        if (bytes < 0 || bytes % 12) throw std::runtime_error(std::string("Error: ") + paths[t] + " is not a vector file.\n");
        if (n >= 0 && bytes / 12 != n) throw std::runtime_error("Error: save-state files hold different particle counts.\n");
        n = bytes / 12;
    }
    std::vector<float> buf[5];
    for (long long start = 0; start <= n; start += SAVE_STATE_CHUNK) {   // num_reads = n // 2^21 + 1
        const long long m = std::min<long long>(SAVE_STATE_CHUNK, n - start);
        for (int t = 0; t < (with_aff ? 5 : 2); t++) {
            buf[t].resize(3 * (size_t)m);
            if (m && std::fread(buf[t].data(), 12, (size_t)m, in[t].f) != (size_t)m)
                throw std::runtime_error(std::string("Error: short read from ") + paths[t] + "\n");
        }
        if (m == 0) continue;   // an empty batch is not queued (load_marker_particle_data, size 0)
        load_particles(buf[0].data(), buf[1].data(), (int)m);
        if (with_aff) load_affine(buf[2].data(), buf[3].data(), buf[4].data(), (int)m);
    }
    return n;
}

void Engine::get_affine(int comp, float *out, int start, int end) const {
    if (comp < 0 || comp > 2) throw std::domain_error("Error: affine component must be 0, 1 or 2.\n");
    if (start < 0 || end > np || start > end) throw std::domain_error("Error: invalid range.\n");
    if (!aff_ready)   // the attribute exists only when APIC was selected (fluidsimulation.cpp:4147-4152)
        throw std::runtime_error(std::string("Error: Invalid ParticleSystemAttribute <name=AFFINE") + "XYZ"[comp] +
                                 ">\n");
    read_interleaved(aff[3 * comp], aff[3 * comp + 1], aff[3 * comp + 2], out, start, end);
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
    xst_v.reserve(nfmax); xst_w.reserve(nfmax);
    for (int q = 0; q < 2; q++) { xl_v[q].reserve(nfmax); xl_w[q].reserve(nfmax); }
    xc_v.reserve(2); xc_w.reserve(2);
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
        wf_dot.reserve(4 * tiles);
        FFGPU_CUDA(cudaMemsetAsync(wf_ticket.p, 0, 2 * sizeof(unsigned int), st));
        wf_xchg.reserve(mic_wavefront_xchg_words(ni, nj, nk));
        FFGPU_CUDA(cudaMemsetAsync(wf_xchg.p, 0, wf_xchg.n * sizeof(unsigned long long), st));
        wf_epoch = 0;
        wf_epoch_dev.reserve(1);
        FFGPU_CUDA(cudaMemsetAsync(wf_epoch_dev.p, 0, sizeof(unsigned int), st));
        FFGPU_CUDA(cudaMemsetAsync(errword.p, 0, sizeof(unsigned int), st));
    }
    {
        std::vector<float> gp((size_t)gridpos_max() + 2);
        for (int g = -1; g <= gridpos_max(); g++) gp[(size_t)(g + 1)] = (float)((double)(float)g * dx);
        gridpos.reserve(gp.size());
        FFGPU_CUDA(cudaMemcpy(gridpos.p, gp.data(), gp.size() * sizeof(float), cudaMemcpyHostToDevice));
        const double chunkdx = dx * 10;   // velocityadvector.h:187
        std::vector<float> bp((size_t)gridpos_max() / 10 + 2);
        for (size_t b_ = 0; b_ < bp.size(); b_++) bp[b_] = (float)((double)(float)b_ * chunkdx);
        blockpos.reserve(bp.size());
        FFGPU_CUDA(cudaMemcpy(blockpos.p, bp.data(), bp.size() * sizeof(float), cudaMemcpyHostToDevice));
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
    std::vector<float> hp, hv, ha[3];
    const bool keep_aff = aff_ready && np;
    std::vector<unsigned int> hid;
    if (np) {
        hp.resize(3 * (size_t)np); hv.resize(3 * (size_t)np);
        get_positions(hp.data(), 0, np); get_velocities(hv.data(), 0, np);
        if (keep_aff) read_affine_host(ha);
        if (ids_on) hid = read_ids_host();
    }
    for (DevBuf<float> *b_ : {&px, &py, &pz, &vx, &vy, &vz, &spx, &spy, &spz, &svx, &svy, &svz, &ox, &oy, &oz,
                              &cpx, &cpy, &cpz, &cvx, &cvy, &cvz})
        b_->reserve(ncap);
    for (DevBuf<int> *b_ : {&key, &rank, &sidx, &keep, &keep2}) b_->reserve(ncap);
    if (aff_ready) {
        for (int q = 0; q < 9; q++) { aff[q].reserve(ncap); saff[q].reserve(ncap); caff[q].reserve(ncap); }
        apic_rec.reserve(3 * (size_t)ncap);
    }
    stage.reserve(3 * (size_t)ncap);
    off.reserve((size_t)ncap + 1);
    scan_tmp.reserve(scan_scratch_ints(std::max((size_t)ncap + 1, dims().cells() + 1)) + 64);
    if (ids_on) { pid.reserve(ncap); cpid.reserve(ncap); }
    cap = ncap;
    const float *a3[3] = {ha[0].data(), ha[1].data(), ha[2].data()};
    if (!hp.empty())
        set_particles(hp.data(), hv.data(), (int)(hp.size() / 3), keep_aff ? a3 : nullptr, ids_on ? hid.data() : nullptr);
}

// Device view of a page-locked host buffer (cudaHostAlloc / cudaHostRegister; mapped under
// unified addressing), or null for pageable memory.
static const float *pinned_view(const void *host) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    return (a.type == cudaMemoryTypeHost && a.devicePointer) ? static_cast<const float *>(a.devicePointer) : nullptr;
}

void Engine::set_particles(const float *pos, const float *vel, int count, const float *const *aff3,
                           const unsigned int *ids) {
    if (count < 0) throw std::domain_error("Error: particle count must be non-negative.\n");
    if (count > cap) { np = 0; ensure_particle_capacity(count); }
    if (ids_on && count) {
        pid.reserve((size_t)std::max(cap, 1));
        cpid.reserve((size_t)std::max(cap, 1));
        std::vector<unsigned int> r;
        if (!ids) { r = random_ids(count); ids = r.data(); }
        FFGPU_CUDA(cudaMemcpyAsync(pid.p, ids, (size_t)count * 4, cudaMemcpyHostToDevice, st));
        FFGPU_CUDA(cudaStreamSynchronize(st));   // the host array may be released on return
    }
    // interleaved host arrays -> SoA: a page-locked caller buffer is read by the kernel itself over
    // the host link (one pass, at the copy engine's rate: 2.7 ms for 23.5M positions and velocities);
    // pageable memory goes through a copy into the staging buffer
    if (count) {
        // every position inside the domain and every velocity finite: anything else would put grid
        // indices out of range in the kernels that follow
        const float *hp = pinned_view(pos), *hv = pinned_view(vel);
        const double hi[3] = {ni * dx, nj * dx, nk * dx};
        loadflag.reserve(1);
        FFGPU_CUDA(cudaMemsetAsync(loadflag.p, 0, sizeof(unsigned int), st));
        if (!hp) FFGPU_CUDA(cudaMemcpyAsync(stage.p, pos, (size_t)count * 12, cudaMemcpyHostToDevice, st));
        launch_deinterleave_checked(count, hp ? hp : stage.p, px, py, pz, hi, 1u, loadflag, st);
        if (!hv) FFGPU_CUDA(cudaMemcpyAsync(stage.p, vel, (size_t)count * 12, cudaMemcpyHostToDevice, st));
        launch_deinterleave_checked(count, hv ? hv : stage.p, vx, vy, vz, nullptr, 2u, loadflag, st);
        launches += 2;
        if (aff_ready) {
            for (int c = 0; c < 3; c++) {
                if (aff3) {
                    FFGPU_CUDA(cudaMemcpyAsync(stage.p, aff3[c], (size_t)count * 12, cudaMemcpyHostToDevice, st));
                    launch_deinterleave(count, stage, aff[3 * c], aff[3 * c + 1], aff[3 * c + 2], st);
                    launches++;
                } else {
                    for (int e = 0; e < 3; e++)
                        FFGPU_CUDA(cudaMemsetAsync(aff[3 * c + e].p, 0, (size_t)count * 4, st));
                }
            }
        }
        FFGPU_CUDA(cudaMemcpyAsync(host_int + 12, loadflag.p, sizeof(unsigned int), cudaMemcpyDeviceToHost, st));
    }
    FFGPU_CUDA(cudaStreamSynchronize(st));
    const unsigned int bad = count ? (unsigned int)host_int[12] : 0u;
    if (bad) {
        np = 0;   // the device state holds the rejected records: clear it
        if (bad & 1u) throw std::domain_error("Error: marker particle position outside the domain or not finite.\n");
        throw std::domain_error("Error: marker particle velocity is not finite.\n");
    }
    np = count;
}

void Engine::read_interleaved(const float *a, const float *b_, const float *c, float *out, int start, int end) const {
    int n = end - start;
    if (n <= 0) return;
    // interleave on the device, then one copy-engine transfer: kernel stores of 12-byte records into
    // host memory reach a third of the copy engine's rate over the host link (58 against ~190 GB/s)
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

void Engine::add_obstacle(const Obstacle *ob) {
    if (!ob) throw std::invalid_argument("Error: MeshObject handle is null.\n");
    for (const Obstacle *o : obstacles)
        if (o == ob) throw std::runtime_error("Error: mesh obstacle has already been added.\n");
    obstacles.push_back(ob);
    solid_built = false;
}

void Engine::remove_obstacle(const Obstacle *ob) {
    auto it = std::find(obstacles.begin(), obstacles.end(), ob);
    if (it == obstacles.end()) {
        char buf[64];
        std::snprintf(buf, sizeof(buf), "%p", (const void *)ob);
        throw std::invalid_argument(std::string("Error: could not find mesh obstacle to remove.\nmesh obstacle: ") +
                                    buf + "\n");
    }
    obstacles.erase(it);
    solid_built = false;
}

void Engine::remove_obstacles() {
    obstacles.clear();
    solid_built = false;
}

void Engine::refresh_solid() {
    if (custom_solid) return;
    std::vector<unsigned long long> now;
    for (const Obstacle *o : obstacles) now.push_back(o->version);
    if (solid_built && now == solid_versions) return;
    launches += solid_builder.build(dims(), dx, obstacles, solid, st);
    if (nspheres > 0) {
        launch_unite_spheres(dims(), dx, spheres, nspheres, solid, st);
        launches++;
    }
    solid_versions = now;
    solid_built = true;
    solid_changed();
    FFGPU_CUDA(cudaStreamSynchronize(st));
}

void Engine::initialize() {
    if (is_init) return;
    alloc_grids();
    refresh_solid();
    // particles outside the domain are dropped on load (fluidsimulation.cpp:5011-5016); with
    // APIC a batch keeps the affine vectors of its paired affine batch, else zeros (:5077-5110)
    std::vector<float> hp, hv, ha[3];
    std::vector<unsigned int> hid;
    ids_on = ffp_output;   // the ID attribute (fluidsimulation.cpp:4180-4182)
    const bool queues_match = pend_aff.size() == pend_counts.size();
    const bool id_queues_match = pend_ids.size() == pend_counts.size();
    size_t first = 0;
    for (size_t bt = 0; bt < pend_counts.size(); bt++) {
        const int n = pend_counts[bt];
        const bool paired = apic && queues_match && pend_aff[bt].size() == 9 * (size_t)n;
        const bool ids_paired = ids_on && id_queues_match && pend_ids[bt].size() == (size_t)n;
        size_t kept = 0;
        for (int q = 0; q < n; q++) {
            const size_t p = first + q;
            float x = pend_pos[3 * p], y = pend_pos[3 * p + 1], z = pend_pos[3 * p + 2];
            if (!in_domain(x, y, z)) continue;
            hp.insert(hp.end(), {x, y, z});
            hv.insert(hv.end(), {pend_vel[3 * p], pend_vel[3 * p + 1], pend_vel[3 * p + 2]});
            if (apic)
                for (int c = 0; c < 3; c++)
                    for (int e = 0; e < 3; e++)
                        ha[c].push_back(paired ? pend_aff[bt][3 * (size_t)n * c + 3 * (size_t)q + e] : 0.0f);
            if (ids_paired) hid.push_back(pend_ids[bt][(size_t)q]);
            kept++;
        }
        if (ids_on && !ids_paired) {   // _generateRandomFluidParticleID for each kept particle
            const std::vector<unsigned int> r = random_ids((int)kept);
            hid.insert(hid.end(), r.begin(), r.end());
        }
        first += n;
    }
    pend_pos.clear(); pend_vel.clear(); pend_counts.clear(); pend_aff.clear(); pend_ids.clear();
    int count = (int)(hp.size() / 3);
    if (ids_on) { pid.reserve((size_t)std::max(count, 1024)); cpid.reserve((size_t)std::max(count, 1024)); }
    ensure_particle_capacity(std::max(count, 1024));
    ensure_affine();
    const float *a3[3] = {ha[0].data(), ha[1].data(), ha[2].data()};
    if (count) set_particles(hp.data(), hv.data(), count, apic ? a3 : nullptr, ids_on ? hid.data() : nullptr);
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
    if (tension_on() && np > 0) {   // the surface tension restriction (fluidsimulation.cpp:10248-10251)
        double restriction = std::sqrt(dx * dx * dx) * std::sqrt(1.0 / (surface_tension + eps));
        ts = std::min(ts, tension_cfl * restriction);
    }
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
    frame_dts.clear();
    frame_solve = SolveStats();
    frame_visc = ViscStats();
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
        frame_dts.push_back(ts);
        if (!skipped) {
            substep(ts);
            // _pressureSolve resets the frame's solver status at the start of every substep
            // (fluidsimulation.cpp:6157-6159) before its "first failure, else most iterations" rule
            // (:6253-6265), so the rule compares against the reset status: the frame reports the
            // last substep's solve, or the reset values when that solve succeeded in 0 iterations.
            if (frame_substeps == 0) {
                frame_solve = last_solve;
            } else {
                frame_solve = SolveStats();
                if (!last_solve.success || last_solve.iterations > 0) frame_solve = last_solve;
            }
            // viscosity statistics: the first substep, then the first failure or the most iterations
            if (frame_substeps == 0) frame_visc = last_visc;
            else if (frame_visc.success && (!last_visc.success || last_visc.iterations > frame_visc.iterations))
                frame_visc = last_visc;
            // the frame's output data after its first substep (fluidsimulation.cpp:10051-10066)
            if (frame_substeps == 0 && ffp_output) output_fluid_particles();
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
