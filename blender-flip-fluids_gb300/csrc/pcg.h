// PCG building blocks (pcg_kernels.cu).
#pragma once
#include "kernels.h"

namespace ffgpu {

#ifndef FFGPU_RED_BLOCKS
#define FFGPU_RED_BLOCKS (152u * 4u)
#endif
constexpr unsigned int MAX_RED_BLOCKS = FFGPU_RED_BLOCKS;   // partial-sum slots per reduction (grid cap)

template <typename T> struct OpView { const T *diag, *ax, *ay, *az; };
template <typename T> struct FactorView { const T *inv, *lx, *ly, *lz; };
template <typename T> struct PcgVecs { T *x, *r, *s, *z; };

// Device-resident solver scalars; kernels update them, the host reads `resid`/`rho`.
struct PcgScalars {
    double rho, sz, alpha, alpha_used, beta, beta_used, resid;
    double tol;      // stop when resid <= tol (inf-norm, absolute)
    int done;        // set by the residual update once resid <= tol; later PCG kernels exit at entry
    int iters;       // residual updates performed since the last reset
    // reliable updates (mixed precision): with `reliable` set, the residual update does not
    // stop at tol but requests an update (`update`) once the FP32 recursive residual is
    // <= tol or has dropped to `delta` times its maximum `rmax` since the last update; the
    // update folds x32 into x64, replaces r by the FP64 true residual and stops (`done`)
    // once that is <= `target`.
    double rmax, target, delta;
    int reliable, update, updates;
};

struct PcgWork {
    double *partials;        // MAX_RED_BLOCKS doubles
    unsigned int *counter;   // zero between launches
    PcgScalars *sc;
};

// Work buffers of the pipelined wavefront MIC(0) (mic_wavefront.cu).
struct WfWork {
    short2 *order;            // tile coordinates in ticket order
    unsigned long long *xchg; // tile-face exchange words (value bits | sweep epoch << 32), zeroed at allocation
    size_t xchg_words;        // capacity of xchg
    unsigned int *epoch;      // host: epoch of the last sweep (never 0 once used)
    unsigned int *ticket;     // tile ticket and exit counters (2 words, zero between sweeps)
    unsigned int *error;      // error word (ErrorBits)
    int max_tiles;
    long long *order_key;     // host: tile-grid shape the order table was built for
    const int *done;          // device PCG converged flag (sweeps are skipped once set), or null
    long long spin_limit;     // polls before a face wait gives up (0: WF_SPIN_LIMIT)
    unsigned int *epoch_dev;  // device: tag of the last sweep (advanced by the sweeps; mirrored by *epoch)
    double *dot_part = nullptr;   // 4 per tile: the staging warps' q.q partials of a sweep with the dot
};
// Makes room for n more sweeps before the epoch counter wraps (clearing the exchange buffer and
// both counters when it would), so that n sweeps can be enqueued, or replayed from a graph,
// without a clear between them.
void wf_reserve_epochs(const WfWork &ww, unsigned int n, cudaStream_t st);

template <typename T>
void mic_wavefront(Dims d, Bbox bb, FactorView<T> F, const T *r, T *z, WfWork ww, cudaStream_t st);
// The FP32 application with the PCG's rho = z.r taken as q.q, q = L^-1 r the forward sweep's result (with
// M = L L^T, r.M^-1 r = |L^-1 r|^2): the forward sweep's staging warps sum q.q per tile, and its last CTA
// sums the tiles and updates rho (first) or beta and rho, as the z.r dot kernel does (ww.dot_part: 4 per
// tile).  Skipped once the PCG has converged.
void mic_wavefront_dot(Dims d, Bbox bb, FactorView<float> F, const float *r, float *z, WfWork ww, PcgScalars *sc,
                       int first, cudaStream_t st);
// The same q.q, summed in the same order, from the forward result q held in memory (the forward
// sweep done elsewhere): per tile and staging warp, then the tiles, then the update of rho / beta.
void mic_dotq_tiles(Dims d, Bbox bb, const float *q, double *part, int max_tiles, PcgScalars *sc, int first,
                    cudaStream_t st);
template <typename T> void pcg_precondition_fwd(Dims d, Bbox bb, FactorView<T> F, const T *r, T *z, cudaStream_t st);
template <typename T> void pcg_precondition_bwd(Dims d, Bbox bb, FactorView<T> F, T *z, cudaStream_t st);
// One sweep of the same wavefront: forward r -> q, or backward in place on q (r unused).
template <typename T>
void mic_wavefront_sweep(Dims d, Bbox bb, FactorView<T> F, const T *r, T *q, WfWork ww, bool forward, cudaStream_t st);
int mic_wavefront_max_tiles(int I, int J);        // tile-table entries a box of I x J columns needs
// One wavefront face wait on a word nothing writes, bounded by `limit` polls: the error bits it
// raised (ERR_WAIT_TIMEOUT).  Synchronises the stream.
unsigned int wait_probe(long long limit, cudaStream_t st);
size_t mic_wavefront_xchg_words(int I, int J, int K);   // exchange words a box of I x J x K cells needs

template <typename T> void pcg_init(Dims d, Bbox bb, const T *b, PcgVecs<T> v, cudaStream_t st);
template <typename T> void pcg_spmv_dot(Dims d, Bbox bb, OpView<T> A, PcgVecs<T> v, PcgWork w, int float_scalars,
                                        cudaStream_t st);
// FP32 SpMV + dot with the operator as hi + lo floats and a compensated row sum (the FP64
// operator to about 48 bits); falls back to pcg_spmv_dot on rows that are not 16-byte aligned
void pcg_spmv_dot_split(Dims d, Bbox bb, OpView<float> A, OpView<float> Alo, PcgVecs<float> v, PcgWork w,
                        cudaStream_t st);
template <typename T> void pcg_update_xr(Dims d, Bbox bb, PcgVecs<T> v, PcgWork w, cudaStream_t st);
template <typename T> void pcg_precondition(Dims d, Bbox bb, FactorView<T> F, const T *r, T *z, cudaStream_t st);
template <typename T> void pcg_dot_zr(Dims d, Bbox bb, PcgVecs<T> v, PcgWork w, int first, int float_scalars,
                                      cudaStream_t st);
template <typename T> void pcg_update_s(Dims d, Bbox bb, PcgVecs<T> v, PcgWork w, int first, cudaStream_t st);

template <typename T> void pcg_store_pressure(Dims d, Bbox bb, const T *x, float *pressure, cudaStream_t st);
void pcg_true_residual(Dims d, Bbox bb, OpView<double> A, const double *b, const double *x, double *r, float *rf,
                       PcgWork w, cudaStream_t st);
void pcg_refine(Dims d, Bbox bb, const float *corr, double *x, cudaStream_t st);
void pcg_zero(Dims d, Bbox bb, double *x, cudaStream_t st);
// x = scale * prev (+ scale2 * prev2 when prev2 is not null) on pressure cells, 0 on the box's other cells
void pcg_warm_start(Dims d, Bbox bb, const float *prev, const unsigned char *fluid, double scale, double *x,
                    cudaStream_t st, const float *prev2 = nullptr, double scale2 = 0.0);
// Axis order of the mixed solve (pcg_permute.cu): new axis a of the copy is the box's axis perm[a].
struct AxisMap { int perm[3]; };
// Writable copies of the operator (FP64, FP32 hi + lo) and the FP32 MIC(0) factor.
struct PermutedSystem {
    double *diag, *ax, *ay, *az;
    float *diag32, *ax32, *ay32, *az32, *diag32lo, *ax32lo, *ay32lo, *az32lo;
    float *inv32, *lx32, *ly32, *lz32;
};
// The order that puts the box's shortest axis last when that is under 4/5 of its z extent (else
// the identity), with the copy's grid (row length padded to a multiple of 4) and its box.
AxisMap choose_axis_map(Bbox bb, Dims &dp, Bbox &pbox);
void launch_permute_system(Dims d, Bbox bb, AxisMap m, Dims dp, PressureSystem sys, PermutedSystem out,
                           cudaStream_t st);
// box values of a grid array into the copy (back = 0) or from it (back = 1)
template <typename T>
void launch_permute_box(Dims d, Bbox bb, AxisMap m, Dims dp, const T *src, T *dst, int back, cudaStream_t st);

// Reliable update, skipped unless the device flag `update` is set: x64 += x32, x32 = 0, then
// r64 = b - A64 x64 and r32 = (float) r64, |r64|_inf into resid / rmax, `done` once it is <= target.
void pcg_reliable_update(Dims d, Bbox bb, OpView<double> A, const double *b, double *x64, float *x32, double *r64,
                         float *r32, PcgWork w, cudaStream_t st);

}  // namespace ffgpu
