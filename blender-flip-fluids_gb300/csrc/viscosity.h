// Viscosity solve (viscosity_kernels.cu): work buffers and host entry points.
#pragma once
#include <vector>

#include "common.cuh"
#include "kernels.h"
#include "pcg.h"

namespace ffgpu {

constexpr int VISC_SLOTS = 16;   // entries per system row (at most 15: the diagonal and 14 couplings)

struct ViscVolumes { float *center, *u, *v, *w, *eu, *ev, *ew; };

template <typename T>
struct VBuf {   // grow-only device array (contents not preserved)
    T *p = nullptr;
    size_t n = 0;
    VBuf() = default;
    VBuf(const VBuf &) = delete;
    VBuf &operator=(const VBuf &) = delete;
    ~VBuf() { if (p) cudaFree(p); }
    void reserve(size_t c) {
        if (c <= n) return;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        FFGPU_CUDA(cudaMalloc(&p, c * sizeof(T)));
        n = c;
    }
    operator T *() const { return p; }
};

struct ViscWork {
    // grids: face states (U, V, W faces), row flags / scan / face -> row index, valid cells,
    // subcell volume fractions (2n)^3, the seven volume grids
    VBuf<unsigned char> state, valid, valid2;
    VBuf<int> flag, scan, index, scan_tmp;
    VBuf<float> sub, vol;
    // rows: face of each row, 16-slot rows (columns ascending, -1 padded), values, the factor's
    // lower values stored with their column (slot of row k holding row r > k), the slot of r in
    // row c for every lower entry, rhs, pivots, levels
    VBuf<int> rowface, col, level, lrows, lcount, lcursor;
    VBuf<float> val, lval, rhs, invdiag, adiag, x, r, z, s;
    VBuf<float> x0;       // per row: the velocity before the solve (the warm start's x)
    bool warm = false;    // start the PCG from x0 instead of zero (the stop stays tol |b|inf)
    VBuf<unsigned char> tpos;
    VBuf<double> partials, scalars;
    std::vector<int> lstart;   // host: rows of level L are lrows[lstart[L] .. lstart[L+1])
    int n = 0;
    Dims grid{0, 0, 0};            // the grid the system was built on
    int first[4] = {0, 0, 0, 0};   // host: rows of component c (U, V, W) are [first[c], first[c+1])
    // Preconditioner form.  VP_WAVEFRONT: each component's block as a 7-point triangular solve on a
    // dense copy of its row box, swept by the pressure solve's tiled wavefront, with the couplings
    // to the other components subtracted between the sweeps; each box swept along its shortest
    // axis when that shortens the chain (VP_WAVEFRONT_GRID_AXES: always along the grid's z).
    // VP_LEVELS: one launch per level (replayed from a graph).  VP_COOP: the levels in one
    // cooperative launch with a grid barrier per level.
    enum { VP_WAVEFRONT = 0, VP_LEVELS = 1, VP_COOP = 2, VP_WAVEFRONT_GRID_AXES = 3 };
    int precond = VP_WAVEFRONT;
    // wavefront form: per component the row box (in its face grid) and the dense grid holding it
    // (row length padded to a multiple of 4, axes possibly reordered); the dense fields (factor,
    // operator, couplings, PCG vectors; each over all components, component c at cbase[c]); the
    // dense position of every row; tile order tables
    struct Box { int i0, j0, k0, i1, j1, k1; };
    Box cbox[3];
    Dims cdim[3];
    Bbox cpbox[3];   // the box in the dense grid (axes possibly reordered)
    int cperm[3][3] = {{0, 1, 2}, {0, 1, 2}, {0, 1, 2}};   // dense axis a runs along face axis cperm[c][a]
    int axis_order = 1;   // set from precond: 1 sweep each box's shortest axis when shorter; 0 the grid's axes
    size_t cbase[3] = {0, 0, 0}, dtot = 0;
    VBuf<float> dense;
    VBuf<int> pos, boxes, ctl;      // ctl: device stopping of the batched PCG ([0] done, [1] residual checks)
    VBuf<short2> order[3];
    long long order_key[3] = {-1, -1, -1};
    int order_cap[3] = {0, 0, 0};
    void reserve_grids(Dims d);
    void reserve_rows(int n);
    ViscVolumes volumes(Dims d) const;
};

// Builds the system for the (constrained) velocity field; returns the number of rows.
int visc_build(Dims d, double dx, double dt, float visc, const float *liquid, const float *solid, const float *u,
               const float *v, const float *w, ViscWork &W, int *host_int, cudaStream_t st,
               unsigned long long &launches);
void visc_factor(ViscWork &W, cudaStream_t st, unsigned long long &launches);
// one launch per level; sweeps = 1 stops after L z = r
void visc_precondition(ViscWork &W, const float *r, float *z, cudaStream_t st, unsigned long long &launches,
                       int sweeps = 2);
// the same application as one cooperative launch; false when the device cannot launch it
bool visc_precondition_coop(ViscWork &W, const float *r, float *z, cudaStream_t st, unsigned long long &launches);
// the wavefront form: visc_wavefront_setup once per factor (sizes the dense boxes, fills the factor
// copies), then any number of applications.  sweeps = 1 stops after the forward sweeps (L z = r).
// ww: the tile-face exchange buffers, ticket and error word shared with the pressure solve.
void visc_wavefront_setup(ViscWork &W, cudaStream_t st, unsigned long long &launches);
void visc_precondition_wf(ViscWork &W, const float *r, float *z, const WfWork &ww, int sweeps, cudaStream_t st,
                          unsigned long long &launches);
// MIC(0)-PCG in float from x = 0 (factor included); false when it does not converge or when a
// wavefront wait gave up (*wait_failed set; ww's error word holds the bits)
bool visc_solve(ViscWork &W, double tol, int maxit, double *host_dbl, int *host_int, const WfWork &ww, int &iters,
                float &residual, bool &wait_failed, cudaStream_t st, unsigned long long &launches,
                cudaEvent_t factored = nullptr);   // recorded once the factor is ready
// every face cleared, rows set from the solution
void visc_apply(Dims d, ViscWork &W, float *u, float *v, float *w, cudaStream_t st);

}  // namespace ffgpu
