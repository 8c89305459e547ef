// Host engine of the GB300 FLIP substep: owns device buffers, sequences the per-substep
// stages (FluidSimulation::_stepFluid, fluidsimulation.cpp:10078-10121) and the frame
// loop with CFL substepping (FluidSimulation::update, :10410-10543).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <random>
#include <string>
#include <vector>

#include "devbuf.h"
#include "ffp3.h"
#include "kernels.h"
#include "mesh_sdf.h"
#include "pcg.h"
#include "viscosity.h"

namespace ffgpu {


enum SolverMode { SOLVER_FP64 = 0, SOLVER_MIXED = 1 };

struct SolveStats {
    int iterations = 0;        // total inner PCG iterations
    int outer = 0;             // refinement passes (mixed mode)
    bool success = true;
    double error = 0.0;        // final inf-norm residual the solver stopped on (absolute)
    double rel_residual = 0.0; // final FP64 ||b - A p||_inf / ||b||_inf (mixed mode)
    int fluid_cells = 0;
    double bnorm = 0.0;
};

struct StageTimes {   // milliseconds per stage of the last substep (CUDA events)
    float sort = 0, sdf = 0, p2g = 0, extrap = 0, pressure_build = 0, factor = 0, pcg = 0, project = 0,
          g2p = 0, advect = 0, remove = 0, total = 0;
};

class Engine {
public:
    Engine(int ni, int nj, int nk, double dx);
    ~Engine();

    // ---- configuration (mirrors the reference setters) ----
    int ni, nj, nk;
    double dx;
    double pic_ratio = 0.05;            // fluidsimulation.h:2402
    double pic_apic_ratio = 0.0;        // :2403 (stored; the APIC update does not blend)
    bool apic = false;                  // velocity transfer method: APIC instead of PIC/FLIP
    double cfl = 5.0;                   // :2190
    int min_substeps = 1, max_substeps = 6;   // :2186-2187
    double tolerance = 1e-9;            // :2378
    double acceptable_tolerance = 1.0;  // :2379
    int max_iterations = 900;           // :2380
    float gx = 0.0f, gy = 0.0f, gz = 0.0f;
    bool extreme_velocity_removal = true;
    int max_per_cell = 250;             // :2447
    SolverMode solver = SOLVER_FP64;
    double inner_tolerance = 0.1;       // mixed mode: reliable-update factor of the FP32 residual
    int pcg_batch = 8;                  // PCG iterations enqueued per host synchronisation
    bool pcg_graphs = true;             // mixed solve: full batches replayed from a graph captured once per solve
    bool timing = false;
    bool mic_levels = false;   // factor and apply MIC(0) by i+j+k hyperplanes instead of the wavefront kernels
    long long wait_limit = 0;  // polls before a wavefront wait gives up and the solve reports it (0: about a second)
    double last_frame_dt = 1.0 / 30.0;   // frame delta time of the current update (speed limit)
    bool in_update = false;
    // viscosity solve before the pressure projection (fluidsimulation.cpp:2569-2601, 5983-6064)
    bool viscosity_enabled = false;
    double viscosity = 0.0;             // constant viscosity
    double visc_tolerance = 1e-4;       // fluidsimulation.h:2364
    bool visc_warm = true;              // the viscosity PCG starts from the field before the solve
    int visc_max_iterations = 900;      // :2365
    struct ViscStats {
        int rows = 0, iterations = 0;
        float error = 0.0f;
        bool success = true;
        float build_ms = 0, factor_ms = 0, pcg_ms = 0;   // with stage timing on: system, factor, PCG
    };
    ViscStats last_visc, frame_visc;    // last substep; frame: first failure, else most iterations
    // surface tension (fluidsimulation.cpp:2604-2621, 2715-2727): the curvature grid of the liquid
    // level set and the cluster status feed a ghost-fluid tension term in the pressure rhs and in the
    // pressure application; the substep length is limited by the tension condition number
    double surface_tension = 0.0;            // constant k; the term is on when k > 1e-6
    double tension_cfl = 10.0;               // fluidsimulation.h:2191
    bool tension_on() const { return surface_tension > 1e-6; }
    int nspheres = 0;                 // analytic spheres, united with the mesh level set
    SphereList spheres{};
    bool custom_solid = false;        // a caller-given solid level set replaces the mesh level set
    // static mesh obstacles (FluidSimulation::addMeshObstacle / removeMeshObstacle,
    // fluidsimulation.cpp:2990-3032); the caller owns them
    void add_obstacle(const Obstacle *ob);
    void remove_obstacle(const Obstacle *ob);
    void remove_obstacles();
    // rebuilds the solid level set when the obstacle list or an obstacle changed
    // (FluidSimulation::_updateSolidLevelSet, fluidsimulation.cpp:5387-5425)
    void refresh_solid();

    // ---- lifecycle ----
    void load_particles(const float *pos, const float *vel, int count);   // queued until initialize
    // Affine vectors of a loaded batch (ax, ay, az: count xyz triples each, the affine vector of
    // the x, y and z velocity component).  Before initialisation the i-th affine batch pairs
    // with the i-th particle batch when both queues have the same length and the batch sizes
    // agree; afterwards it pairs with the last batch given to load_particles.  Unpaired
    // particles start with zero affine vectors.
    void load_affine(const float *ax, const float *ay, const float *az, int count);
    void initialize();
    bool initialized() const { return is_init; }
    void set_solid_phi(const float *host_phi);   // nodal (ni+1)(nj+1)(nk+1), static solids
    void update(double frame_dt);
    void substep(double dt);
    float run_substeps_timed(int k, double dt);   // device time of k substeps (CUDA events, ms)
    // Re-runs one kernel group `reps` times on the current state; returns the mean device
    // time per launch group (ms) and its algorithmic bytes (each input read once, each
    // output written once).  Ids: 0 P2G (one component), 1 liquid SDF, 2 SpMV + dot (FP32, split operator),
    // 3 MIC(0) forward + backward substitution (FP32), 4 extrapolation (one component, all
    // layers), 5 G2P, 6 RK3 advection + collision, 7 particle sort, 8 APIC P2G (assignment records
    // and one component), 9 APIC G2P, 10 viscosity solve (system, factor, PCG, apply; time only,
    // viscosity 1 unless one is set).
    float time_kernel(int id, int reps, double *bytes);

    // ---- particle access ----
    int num_particles() const { return np; }
    void get_positions(float *out, int start, int end) const;   // interleaved xyz
    void get_velocities(float *out, int start, int end) const;
    void get_affine(int comp, float *out, int start, int end) const;   // comp 0/1/2: affine x/y/z
    // Save-state particle files (bake.py:2864-2905): attribute 0 position, 1 velocity, 2..4
    // affine x/y/z as interleaved float32 xyz in particle order, streamed from the device in
    // chunks of 2^21 particles through two pinned buffers (copy of one chunk overlaps the write
    // of the previous).  append adds to an existing file.
    void write_attribute_file(int attribute, const char *path, bool append);
    // The save-state loader's batches (bake.py:554-721): the files are read in chunks of 2^21
    // particles, each chunk one load_particles batch and, with affine files, one load_affine batch.
    // Returns the number of particles read.
    long long load_attribute_files(const char *pos_path, const char *vel_path, const char *afx_path,
                                   const char *afy_path, const char *afz_path);
    // replace device state (host buffers); aff3 (optional): the three affine arrays as in load_affine;
    // ids (optional, one per particle): the particle ids when the particles carry ids (else random ids)
    void set_particles(const float *pos, const float *vel, int count, const float *const *aff3 = nullptr,
                       const unsigned int *ids = nullptr);

    // ---- FFP3 fluid-particle output (fluidsimulation.cpp:9477-9800, 10051-10066) ----
    // enable_fluid_particle_output turns on the particles' uint16 id attribute (created at
    // initialisation; loaded with load_ids, else random) and an FFP3 output after the first substep
    // of every update: the liquid level set and its surface level set recomputed from the particles,
    // the particles classified and grouped, the bytes kept on the device until read.
    bool ffp_output = false;
    double ffp_amount = 1.0;           // set_fluid_particle_output_amount (id limit round(65536 amount))
    Ffp3Params ffp;                    // enabled types, widths, velocity / speed attributes
    Ffp3Counts ffp_counts;             // the last output
    bool ffp_ready = false;
    // FluidSimulation::loadMarkerParticleIDData (fluidsimulation.cpp:4019-4039): an id batch, paired
    // with the particle batch of the same position and size (:5077-5110), else random ids
    void load_ids(const uint16_t *ids, int count);
    void output_fluid_particles();
    size_t ffp3_bytes(int which) const;              // 0 positions, 1 ids, 2 velocities, 3 speeds
    void read_ffp3(int which, char *out) const;
    void read_ffp3_types(unsigned char *out) const;   // per particle of the last output: 0..3
    void get_ids(uint16_t *out, int start, int end) const;
    bool has_ids() const { return ids_on; }
    // device-resident particle arrays (SoA), valid until the next substep
    float *dev_px() { return px; }

    // ---- statistics ----
    int current_frame = 0;
    int frame_substeps = 0;
    std::vector<double> frame_dts;   // lengths of the last update's substeps, in order
    float last_speed_limit = 0.0f;   // extreme-velocity removal limit of the last substep (0: rule off)
    SolveStats last_solve;        // last substep
    SolveStats frame_solve;       // the frame's last substep (the reference resets it per solve)
    StageTimes last_times;
    double frame_time = 0.0;
    double total_time = 0.0;
    int performance_score = 0;
    unsigned long long launches = 0;   // kernels launched by this engine (all substeps)

    // ---- intermediate device state (read by the stage-level API) ----
    Dims dims() const { return Dims{ni, nj, nk}; }
    cudaStream_t stream() const { return st; }
    double radius() const;

    DevBuf<float> solid, wu, wv, ww;
    std::vector<const Obstacle *> obstacles;
    std::vector<unsigned long long> solid_versions;   // obstacle versions the solid was built from
    bool solid_built = false;
    SolidBuilder solid_builder;
    DevBuf<unsigned char> near;
    NearGrid ng{};
    DevBuf<float> phi, pressure;
    // surface tension: surface level set, curvature, cluster status and their work buffers
    DevBuf<float> surf, curv, tbuf;
    DevBuf<unsigned char> tvalid, tvn, tblocks0, tblocks1, tstatus, ttouch;
    DevBuf<unsigned int> tcblocks, tscal;
    DevBuf<int> tparent, tcount;
    void stage_surface_tension();            // curvature grid and cluster status of phi
    TensionWork tension_work();
    DevBuf<float> u, v, w, su, sv, sw;
    DevBuf<unsigned char> vu, vv, vw, st1, st2;
    DevBuf<unsigned int> xlist1, xlist2, xcount;   // frontier extrapolation lists
    // the v and w components' frontier buffers and side streams: the three components extrapolate
    // concurrently (their frontier kernels are small and latency bound)
    DevBuf<unsigned char> xst_v, xst_w;
    DevBuf<unsigned int> xl_v[2], xl_w[2], xc_v, xc_w;
    cudaStream_t xstream[3] = {nullptr, nullptr, nullptr};   // [2]: the liquid level set beside P2G
    cudaEvent_t xevent[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    ExtrapFront front() { return ExtrapFront{st1.p, {xlist1.p, xlist2.p}, xcount.p}; }
    DevBuf<int> cell_count, cell_start, scan_tmp;
    DevBuf<int> key, rank, sidx, keep, keep2, off;
    DevBuf<unsigned long long> sdf_rec;       // liquid SDF per-particle assignment records
    DevBuf<float> px, py, pz, vx, vy, vz;     // particle state, particle order
    DevBuf<float> spx, spy, spz, svx, svy, svz;   // cell-sorted copies
    DevBuf<float> ox, oy, oz;                 // advected positions
    DevBuf<float> cpx, cpy, cpz, cvx, cvy, cvz;   // compaction targets
    DevBuf<float> stage;                      // interleaved xyz staging for host I/O (3 x capacity)
    // APIC: affine vectors (component c's vector in aff[3c .. 3c+2]), their cell-sorted copies,
    // compaction targets and the per-component block assignment records of the sorted particles
    DevBuf<float> aff[9], saff[9], caff[9];
    DevBuf<unsigned long long> apic_rec;
    DevBuf<float> gridpos;   // node positions (float)((double)(float)g * dx), g = -1 .. gridpos_max()
    int gridpos_max() const { return std::max(std::max(ni, nj), std::max(nk, 10)) + 1; }
    DevBuf<float> blockpos;  // transfer block origins (float)((double)(float)b * (10 dx)), b = 0 .. gridpos_max() / 10 + 1
    bool aff_ready = false;
    void ensure_affine();
    // pressure system
    DevBuf<double> diag, ax, ay, az, inv, lx, ly, lz, b;
    DevBuf<float> diag32, ax32, ay32, az32, inv32, lx32, ly32, lz32;
    DevBuf<float> diag32lo, ax32lo, ay32lo, az32lo;
    DevBuf<unsigned char> fluid;
    DevBuf<double> x64, r64, s64, z64;
    DevBuf<float> x32, r32, s32, z32;
    // mixed solve in a box-sized copy whose shortest axis is swept by the MIC(0) wavefront
    // (pcg_permute.cu): 0 keeps the grid's axis order, 1 chooses per solve
    int axis_order = 1;
    // mixed solve started from the previous substep's pressure, scaled by the ratio of the substep
    // lengths, instead of zero (the stopping rule, relative to ||b||, is unchanged)
    int warm_start = 2;   // 0 zero start, 1 the last pressure, 2 linear extrapolation from the last two
    bool have_prev = false, solve_warm = false;
    double prev_dt = 0.0, warm_scale = 1.0;
    DevBuf<float> prev_pressure;
    // the pressure before the last one (valid when the last setup was warm): the second level of the
    // extrapolation, its substep's dt, and the coefficient of its term
    DevBuf<float> prev2_pressure;
    bool last_setup_warm = false, solve_warm2 = false;
    double last_setup_dt = 0.0, warm_scale2 = 0.0;
    // the mixed solve starts from x64 as the caller left it and leaves the pressure grid alone (the
    // adjoint's solve)
    bool solve_from_x = false;
    // iterations of the last forward / adjoint mixed solve: the batches before the first host check
    int last_mixed_iters[2] = {0, 0};
    // the last adjoint solve's solution (valid when adj_have_prev), the next one's start, and its dt
    DevBuf<float> adj_prev;
    bool adj_have_prev = false;
    double adj_prev_dt = 0.0;
    bool perm_active = false, perm_ready = false;   // this solve uses the copy / the copy holds the system
    AxisMap perm_map{{0, 1, 2}};
    Dims perm_dims{0, 0, 0};
    Bbox perm_box{};
    DevBuf<double> pdiag, pax, pay, paz, pb, px64, pr64;
    DevBuf<float> pdiag32, pax32, pay32, paz32, pdiag32lo, pax32lo, pay32lo, paz32lo, pinv32, plx32, ply32, plz32;
    DevBuf<float> px32, pr32, ps32, pz32, prf;
    DevBuf<double> partials;
    DevBuf<short2> wf_order;
    DevBuf<unsigned long long> wf_xchg;   // wavefront tile-face exchange words
    unsigned int wf_epoch = 0;               // tag of the last sweep (mirrors wf_epoch_dev)
    DevBuf<unsigned int> wf_epoch_dev;
    DevBuf<double> wf_dot;   // 4 per tile: the q.q partials of the mixed solve's preconditioner
    DevBuf<unsigned int> wf_ticket, errword;
    DevBuf<unsigned int> mic_progress;     // per-tile step counters of the MIC(0) factorization
    long long wf_order_key = -1;
    DevBuf<unsigned int> counter;
    DevBuf<PcgScalars> scal;
    DevBuf<int> bbox_dev;
    DevBuf<double> maxabs_b;
    DevBuf<int> maxcount;
    DevBuf<unsigned int> speedbits;

    // ---- diagnostics: each solve against an FP64 reference solve ----
    // With check_tolerance > 0, every substep also solves its pressure system with the FP64 PCG
    // (same operator, same FP64 MIC(0) factor) to that relative residual, projects the velocity
    // field with that pressure into separate buffers, and records the errors of the substep's
    // own solve against it.  The substep's result is unchanged (it keeps its own solve).
    double check_tolerance = 0.0;
    struct SolveCheck {
        bool valid = false;      // a system was solved this substep
        double p_rel_l2 = 0.0;   // ||p - p_ref||_2 / ||p_ref||_2 over the pressure cells
        double u_rel_l2 = 0.0;   // ||u - u_ref||_2 / ||u_ref||_2 over the faces the projection set
        double div_rel = 0.0;    // max |D(u)| / ||b||_inf after the projection (D: weighted divergence)
        double div_ref_rel = 0.0;   // the same for the field projected with p_ref
        double bnorm = 0.0;
        int ref_iterations = 0;
        double ref_rel_residual = 0.0;
    };
    SolveCheck last_check;
    DevBuf<double> chk_x, chk_part;
    DevBuf<float> chk_p, chk_u, chk_v, chk_w;
    DevBuf<unsigned char> chk_vu, chk_vv, chk_vw;
    DevBuf<unsigned long long> chk_max;
    void check_solve(double dt);        // after stage_pressure: the reference solve and p error
    void check_projection();            // after stage_project: velocity error and divergence

    // ---- differentiable substep (adjoint) ----
    // Forward substep without marker removal that records what the transposed maps need
    // (transfer weight sums and outputs, extrapolation layers and valid flags, solver
    // operator, which particles the collision handling moved).
    void substep_differentiable(double dt);
    // dL/dv0 from dL/dv1 (device SoA arrays gv1x..z -> gv0x..z) for the last differentiable
    // substep.  When `loss_ymin` is not NaN, dL/dv1 is first set to the gradient of L = mean
    // over particles with y > loss_ymin of vy^2 (state after the substep); returns the number
    // of those particles.
    int adjoint(double loss_ymin);
    // (dL/dx1, dL/dv1) -> (dL/dx0, dL/dv0) for the last differentiable substep: gx1*, gv1* ->
    // gx0*, gv0*.  Without `with_x` dL/dx1 is taken as zero.
    void adjoint_core(bool with_x);
    // k differentiable substeps from the current state, with a checkpoint of (x, v) before each
    void rollout_forward(int k, double dt);
    // (dL/dx_k, dL/dv_k) in gx1*, gv1* -> (dL/dx_0, dL/dv_0) in gx0*, gv0*, recomputing each
    // substep from its checkpoint; `loss_ymin` as in adjoint().  The state is left at x_k, v_k.
    int rollout_adjoint(bool with_x, double loss_ymin);
    float run_forward_adjoint_timed(int k, double dt, double loss_ymin);
    double adjoint_tolerance = 1e-6;
    bool diff_ready = false;
    double diff_dt = 0.0;
    DevBuf<float> wsum_u, wsum_v, wsum_w, gcu, gcv, gcw, gsu, gsv, gsw, gbu, gbv, gbw, gtmp;
    DevBuf<float> p2g_u, p2g_v, p2g_w;   // recorded transfer outputs (accurate form, valid faces)
    DevBuf<unsigned char> lay1u, lay1v, lay1w, lay2u, lay2v, lay2w, val1u, val1v, val1w, val2u, val2v, val2w;
    DevBuf<unsigned char> collided;
    DevBuf<float> gv1x, gv1y, gv1z, gv0x, gv0y, gv0z, gx1x, gx1y, gx1z, gx0x, gx0y, gx0z;
    DevBuf<float> adj_wc, adj_ws, adj_pt2, adj_pt3, adj_q;   // RK3^T sample weights and stage points
    DevBuf<int> cell_count2, cell_start2, sidx2;               // cell sort of the stage points
    DevBuf<float> ckpt;                                        // rollout checkpoints, 6 x cap per substep
    int rollout_k = 0, rollout_np = 0;
    double rollout_dt = 0.0;
    DevBuf<int> loss_count;
    void alloc_adjoint();
    void sort_points(const float *pts);          // stage points (x, y, z, w...) -> cell_start2, adj_q
    void save_state(size_t slot);
    void restore_state(size_t slot);

    // stage entry points (operate on the device state above)
    void stage_sort();
    void stage_sdf(bool post = true, cudaStream_t on = nullptr);   // on: a stream other than the engine's
    void stage_p2g();
    void stage_extrapolate_all();
    void stage_extrapolate(int comp);
    void stage_save_and_body_force(double dt);
    int viscosity_precondition_probe(double dt, float visc, int form, int sweeps);
    void stage_p2g_components();
    void stage_viscosity(double dt);         // constrain, build, MIC(0)-PCG in float, apply
    ViscWork visc_work;
    bool stage_pressure(double dt);          // build, factor, solve, store pressure grid
    void stage_project(double dt);           // apply pressure + extrapolate
    void stage_constrain();
    void stage_g2p(cudaStream_t on = nullptr);   // on: a stream other than the engine's
    void stage_advect(double dt);
    void stage_remove();
    Bbox bbox{};
    bool have_fluid_cells = false;

private:
    bool is_init = false;
    int np = 0, cap = 0;
    std::vector<float> pend_pos, pend_vel;
    std::vector<int> pend_counts;                  // particle batches queued before initialisation
    std::vector<std::vector<float>> pend_aff;      // affine batches (ax, ay, az concatenated)
    std::vector<int> join_kept;                    // last batch joined after initialisation: kept entries
    int join_start = 0, join_size = -1, join_id_size = -1;
    std::vector<std::vector<uint16_t>> pend_ids;   // id batches queued before initialisation
    bool ids_on = false;                           // the particles carry ids
    DevBuf<unsigned int> pid, cpid;                // ids (uint16 values in 32-bit slots) and the compaction copy
    Ffp3Work ffp_work;
    std::mt19937 id_rng;                           // FluidSimulation::_generateRandomFluidParticleID
    bool id_rng_seeded = false;
    std::vector<unsigned int> random_ids(int count);
    std::vector<unsigned int> read_ids_host() const;
    bool in_domain(float x, float y, float z) const;
    void read_affine_host(std::vector<float> (&ha)[3]) const;
    cudaStream_t st = nullptr;
    PcgScalars *host_sc = nullptr;   // pinned
    float *host_io[2] = {nullptr, nullptr};   // pinned chunk buffers of the save-state writer
    int *host_int = nullptr;         // pinned scratch (16 words: [8..11] tension, [12] particle load check)
    DevBuf<unsigned int> loadflag;   // particle load check bits (1 position, 2 velocity)
    double *host_dbl = nullptr;      // pinned scratch
    cudaEvent_t ev[16];
    cudaEvent_t tev[18];   // per-stage timing marks ([14, 15] the level set, [16, 17] G2P on the side stream)
    cudaEvent_t vev[4];    // viscosity solve marks: build, factor, PCG
    void mark(int i) { if (timing) FFGPU_CUDA(cudaEventRecord(tev[i], st)); }

    void alloc_grids();
    void read_interleaved(const float *a, const float *b, const float *c, float *out, int start, int end) const;
    void ensure_particle_capacity(int count);
    void solid_changed();
    PressureSystem sys_view();
    void solve_fp64(SolveStats &out);
    void solve_mixed(SolveStats &out);
    struct MixedArrays {   // one mixed solve's grid, box and arrays (the grid's own or the axis-ordered copy)
        Dims d;
        Bbox bb;
        OpView<float> A32, A32lo;
        FactorView<float> F32;
        OpView<double> A64;
        const double *b;
        double *x64, *r64;
        float *rf;
        PcgVecs<float> vf;
        bool warm;   // x64 holds the initial guess
    };
    void solve_mixed_on(const MixedArrays &m, SolveStats &out);
    double max_particle_speed();
    double next_timestep(double dt);
    void read_scalars();
    template <typename T> void precondition(FactorView<T> F, const T *r, T *z);
    template <typename T> void precondition(Dims d, Bbox bb, FactorView<T> F, const T *r, T *z);
    // z = M^-1 r and the PCG's rho (first) or beta and rho from q.q (= z.r), for the mixed solve
    void precondition_dot(Dims d, Bbox bb, FactorView<float> F, const float *r, float *z, int first);
    void check_error_word(const char *where = "pressure solve");
    WfWork wf_work(const int *done);   // the wavefront's buffers, with the PCG converged flag (or null)
};

}  // namespace ffgpu
