// Viscosity solve (viscosity_kernels.cu): work buffers and host entry points.
#pragma once
#include <vector>

#include "common.cuh"
#include "kernels.h"

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
    VBuf<unsigned char> tpos;
    VBuf<double> partials, scalars;
    std::vector<int> lstart;   // host: rows of level L are lrows[lstart[L] .. lstart[L+1])
    int n = 0;
    // preconditioner as one cooperative launch with a grid barrier per level instead of per-level
    // launches replayed from a graph; the graph is faster on GB300 (1.15 s against 1.51 s per
    // viscous 256^3 substep: a grid-wide barrier costs about 6.5 us, a graph node about 4.9 us)
    bool use_coop = false;
    void reserve_grids(Dims d);
    void reserve_rows(int n);
    ViscVolumes volumes(Dims d) const;
};

// Builds the system for the (constrained) velocity field; returns the number of rows.
int visc_build(Dims d, double dx, double dt, float visc, const float *liquid, const float *solid, const float *u,
               const float *v, const float *w, ViscWork &W, int *host_int, cudaStream_t st,
               unsigned long long &launches);
void visc_factor(ViscWork &W, cudaStream_t st, unsigned long long &launches);
void visc_precondition(ViscWork &W, const float *r, float *z, cudaStream_t st, unsigned long long &launches);
// the same application as one cooperative launch; false when the device cannot launch it
bool visc_precondition_coop(ViscWork &W, const float *r, float *z, cudaStream_t st, unsigned long long &launches);
// MIC(0)-PCG in float from x = 0 (factor included); false when it does not converge
bool visc_solve(ViscWork &W, double tol, int maxit, double *host_dbl, int &iters, float &residual, cudaStream_t st,
                unsigned long long &launches);
// every face cleared, rows set from the solution
void visc_apply(Dims d, ViscWork &W, float *u, float *v, float *w, cudaStream_t st);

}  // namespace ffgpu
