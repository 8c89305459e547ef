// Host-side launchers of the FLIP substep kernels (one group per .cu file).
#pragma once
#include <cuda_runtime.h>
#include "common.cuh"

namespace ffgpu {

constexpr int MAX_SPHERES = 8;
struct SphereList { double s[MAX_SPHERES][4]; };   // cx, cy, cz, r
struct NearGrid { int w, h, d; double cell; };

// ---- grid_kernels.cu ----
void launch_solid_phi(Dims d, double dx, const SphereList &sph, int nsph, float *phi, cudaStream_t st);
// phi = min(phi, distance to each sphere's surface) at the nodes (analytic sphere obstacles)
void launch_unite_spheres(Dims d, double dx, const SphereList &sph, int nsph, float *phi, cudaStream_t st);
void launch_face_weights(Dims d, const float *solid, float *wu, float *wv, float *ww, cudaStream_t st);
void launch_near_solid(Dims d, double dx, int cfl, const float *solid, NearGrid ng, unsigned char *g,
                       unsigned char *tmp, cudaStream_t st);
// rec: np 64-bit scratch words (per-particle block assignment and cell windows)
void launch_liquid_sdf(Dims d, double dx, double radius, int np, const int *cell_start, const float *spx,
                       const float *spy, const float *spz, unsigned long long *rec, const float *solid, int do_post,
                       float *phi, cudaStream_t st);

// ---- sort_kernels.cu ----
// Scan scratch: at most ceil(n / SCAN_TILE) partial sums.
constexpr int SCAN_TILE = 4096;
size_t scan_scratch_ints(size_t n);
void launch_exclusive_scan(const int *in, int *out, size_t n, int *scratch, cudaStream_t st);  // out[n] = total
void launch_cell_keys(Dims d, double dx, int np, const float *px, const float *py, const float *pz,
                      int *key, int *rank, int *count, cudaStream_t st, bool float_keys = false);
void launch_scatter_sorted(int np, const int *key, const int *rank, const int *cell_start, int *sorted_idx,
                           cudaStream_t st);
void launch_sort_within_cells(size_t ncells, const int *cell_start, int *sorted_idx, cudaStream_t st);
void launch_gather_particles(int np, const int *sorted_idx, const float *const *src, float *const *dst, int nattr,
                             cudaStream_t st);

// ---- p2g_kernels.cu ----
// wsum, uacc (optional, together): per-face weight sums and transfer outputs in the factored
// kernel form, kept for the transposed transfer
// gpos, bpos: node positions and transfer block origins, (float)((double)(float)g * dx) for
// g = -1 .. and (float)((double)(float)b * 10 dx) for b = 0 .. (indexed g + 1 and b)
// the three components in one pass (same sums as three launch_p2g calls)
void launch_p2g3(Dims d, double dx, double radius, const int *cell_start, const float *spx, const float *spy,
                 const float *spz, const float *svx, const float *svy, const float *svz, const float *gpos,
                 const float *bpos, float *u, float *v, float *w, unsigned char *vu, unsigned char *vv,
                 unsigned char *vw, cudaStream_t st);
void launch_p2g(Dims d, double dx, double radius, int comp, const int *cell_start, const float *spx,
                const float *spy, const float *spz, const float *svel, const float *gpos, const float *bpos,
                float *field, unsigned char *valid, cudaStream_t st, float *wsum = nullptr, float *uacc = nullptr);
// layer_of (optional): per cell, the layer at which it was extrapolated (low 5 bits) and the number
// of neighbours averaged minus one (high 3 bits); 255 = not extrapolated.  Needs layers <= 31.
// Work buffers of the frontier extrapolation: face statuses (w*h*dd bytes), two face lists
// (w*h*dd entries each) and two list counters.
struct ExtrapFront {
    unsigned char *status;
    unsigned int *list[2];
    unsigned int *count;
};
void launch_extrapolate_front(int w, int h, int dd, float *grid, const unsigned char *valid, int layers, ExtrapFront f,
                              cudaStream_t st, unsigned char *layer_of = nullptr);
void launch_extrapolate(int w, int h, int dd, float *grid, const unsigned char *valid, int layers,
                        unsigned char *status, unsigned char *status2, cudaStream_t st,
                        unsigned char *layer_of = nullptr);
void launch_body_force(size_t n, float *field, float add, cudaStream_t st);
void launch_constrain(size_t n, const float *weight, float *field, cudaStream_t st);

// ---- particle_kernels.cu ----
struct MacView { const float *u, *v, *w; };
void launch_g2p(Dims d, double dx, float pic, int np, const float *px, const float *py, const float *pz,
                float *vx, float *vy, float *vz, MacView cur, MacView saved, cudaStream_t st);
void launch_advect(Dims d, double dx, double dt, int cfl, int np, const float *px, const float *py,
                   const float *pz, float *ox, float *oy, float *oz, MacView vel, const float *solid,
                   NearGrid ng, const unsigned char *near, cudaStream_t st, unsigned char *collided = nullptr);
void launch_remove_mark(Dims d, double dx, int np, const float *px, const float *py, const float *pz,
                        const float *solid, int *keep, int *key, int *cell_count, int *max_count, cudaStream_t st);
void launch_cap_per_cell(size_t ncells, const int *cell_start, const int *sorted_idx, const int *keep_in,
                         int *keep_out, int max_per_cell, cudaStream_t st);
void launch_compact(int np, const int *keep, const int *offset, const float *const *src, float *const *dst,
                    int nattr, cudaStream_t st);
void launch_max_speed_sq(int np, const float *vx, const float *vy, const float *vz, double *partials,
                         unsigned int *counter, double *result, cudaStream_t st);

// ---- apic_kernels.cu ----
// gpos, bpos: as for launch_p2g; gpos[g + 1] = (float)((double)(float)g * dx) for -1 <= g <= gmax,
// with gmax >= max(ni, nj, nk, 10) + 1 (GridIndexToPosition, grid3d.h:80-84)
// rec: 3 np words, the per-component block assignment records of the sorted particles
void launch_apic_records(Dims d, double dx, double radius, int np, const float *spx, const float *spy,
                         const float *spz, unsigned long long *rec, cudaStream_t st);
// saff: the sorted affine vector (x, y, z arrays) of component comp
void launch_p2g_apic(Dims d, double dx, double radius, int comp, const int *cell_start, const float *spx,
                     const float *spy, const float *spz, const float *svel, const float *const *saff,
                     const unsigned long long *rec, int np, const float *gpos, const float *bpos, float *field,
                     unsigned char *valid, cudaStream_t st);
// aff: 9 particle-order arrays, component c's affine vector in aff[3c .. 3c+2]
void launch_g2p_apic(Dims d, double dx, int np, const float *px, const float *py, const float *pz, float *vx,
                     float *vy, float *vz, float *const *aff, MacView vel, const float *gpos, int gmax,
                     cudaStream_t st);

// ---- pressure_kernels.cu ----
struct Bbox { int i0, j0, k0, i1, j1, k1; };   // inclusive
struct PressureSystem {
    // all dense over the cell grid, zero outside pressure cells
    double *diag, *ax, *ay, *az;     // A(c,c), A(c,c+x), A(c,c+y), A(c,c+z)
    double *inv, *lx, *ly, *lz;      // MIC(0): 1/sqrt(pivot), L(c+x,c), L(c+y,c), L(c+z,c)
    float *diag32, *ax32, *ay32, *az32, *inv32, *lx32, *ly32, *lz32;
    float *diag32lo, *ax32lo, *ay32lo, *az32lo;   // FP32 roundings of A - (FP32 A)
    double *b;                       // right-hand side (negative divergence)
    unsigned char *fluid;            // pressure-cell flag
};
void launch_classify(Dims d, const float *phi, unsigned char *fluid, int *bbox6, cudaStream_t st);
struct TensionDev;   // tension.cuh: the surface tension term (null: none)
void launch_build_system(Dims d, double dx, double dt, Bbox bb, const float *phi, const float *wu,
                         const float *wv, const float *ww, const float *u, const float *v, const float *w,
                         PressureSystem sys, double *partials, unsigned int *counter, double *maxabs_b,
                         cudaStream_t st, const TensionDev *tension = nullptr);
// progress: mic0_factor_tiles(I, J) words for the tiled wavefront (null: hyperplane schedule);
// error: device error word (ERR_WAIT_TIMEOUT if a wait expires)
int mic0_factor_tiles(int I, int J);
// spin_limit: polls before a wait gives up (0: the default, about a second)
void launch_mic0_factor(Dims d, Bbox bb, PressureSystem sys, unsigned int *progress, unsigned int *error,
                        cudaStream_t st, long long spin_limit = 0);
void launch_to_float(Dims d, Bbox bb, PressureSystem sys, cudaStream_t st);
void launch_apply_pressure(Dims d, double dx, double dt, const float *phi, const float *wu, const float *wv,
                           const float *ww, const float *pressure, float *u, float *v, float *w,
                           unsigned char *vu, unsigned char *vv, unsigned char *vw, cudaStream_t st,
                           const TensionDev *tension = nullptr);

// Surface tension (tension_kernels.cu).  Work buffers of the curvature grid and cluster status,
// each of ni*nj*nk entries unless noted.
struct TensionWork {
    float *buf;                    // second re-initialisation buffer
    unsigned char *valid;          // solver band (cells of marked 6^3 blocks)
    unsigned char *vn;             // nodes with a computed curvature
    unsigned char *blocks0, *blocks1;   // 6^3 block marks before and after feathering (one per block)
    int *parent;                   // cluster status: union-find parents
    int *count;                    // cluster status: cells per component root
    unsigned char *touch;          // cluster status: the component touches a classified cell
    unsigned int *cblocks;         // cluster status: phase bits of the 4^3 blocks (one per block)
    unsigned int *scal;            // 4 device words
    unsigned char *xst1, *xst2;    // extrapolation status (ni*nj*nk each)
    int *host;                     // pinned host words (4)
};
// ParticleLevelSet::calculateCurvatureGrid (particlelevelset.cpp:196-291) of the post-processed
// liquid level set phi: surface_phi (the re-initialised band, 5 dx outside) and the curvature grid.
// Synchronises the stream once per re-initialisation step.  Returns the kernels launched.
int launch_curvature_grid(Dims d, double dx, const float *phi, float *surface_phi, float *curvature, TensionWork w,
                          cudaStream_t st);
// Cluster status per cell (pressuresolver.cpp:314-605) as connected components.  Returns the kernels launched.
int launch_cluster_status(Dims d, const float *phi, unsigned char *status, TensionWork w, cudaStream_t st);
// Diagnostics (pressure_build.cu): the largest weighted divergence |D_c| over the pressure
// cells, and masked sums of (a - b)^2 and b^2 (blocking: both read their result back).
double divergence_max(Dims d, double dx, const unsigned char *fluid, const float *wu, const float *wv,
                      const float *ww, const float *u, const float *v, const float *w,
                      unsigned long long *maxbits, double *host, cudaStream_t st);
constexpr int DIFF_PARTIALS = 2 * 1024;   // doubles of block partials diff_sq needs
template <typename A, typename B>
void diff_sq(size_t n, const A *a, const B *b, const unsigned char *mask, double *part, double *host_part,
             double &e2, double &r2, cudaStream_t st);

}  // namespace ffgpu
