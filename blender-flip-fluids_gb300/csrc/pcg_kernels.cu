// K11-K14: preconditioned conjugate gradient on the 7-point pressure operator.
//   FP64 mode follows PCGSolver<double>::solve (pcgsolver.h:268-322): double vectors,
//   step lengths alpha/beta truncated to float as BLAS::addScaled does
//   (blaswrapper.h:135), MIC(0) applied by forward/backward substitution over i+j+k
//   hyperplanes (pcgsolver.h:212-241) with the reference's per-cell operation order.
//   FP32 mode keeps vectors, operator and factor in float with double dot products; it is
//   the inner solver of the mixed-precision iterative refinement.
// Reductions are deterministic: fixed-shape block trees, then the last block to finish
// sums the block partials in index order.
#include <stdexcept>
#include <type_traits>

#include "common.cuh"
#include "kernels.h"
#include "pcg.h"

#ifndef FFGPU_VEC_UNROLL
#define FFGPU_VEC_UNROLL 1
#endif
#define FFGPU_PRAGMA(x) _Pragma(#x)
#define FFGPU_UNROLL(n) FFGPU_PRAGMA(unroll n)

namespace ffgpu {

constexpr int RB = 256;   // reduction block size

struct BoxIt2 {
    Bbox b;
    int I, J, K;
    unsigned int n;   // I J K < 2^31
    FastDiv dI, dJ;
    __device__ bool in(int i, int j, int k) const {
        return i >= b.i0 && j >= b.j0 && k >= b.k0 && i <= b.i1 && j <= b.j1 && k <= b.k1;
    }
};
inline BoxIt2 boxit2(Bbox b) {
    BoxIt2 bx;
    bx.b = b;
    bx.I = b.i1 - b.i0 + 1; bx.J = b.j1 - b.j0 + 1; bx.K = b.k1 - b.k0 + 1;
    const unsigned long long n = (unsigned long long)bx.I * bx.J * bx.K;
    if (n >= (1ull << 31)) throw std::runtime_error("Error: pressure box exceeds 2^31 cells.\n");
    bx.n = (unsigned int)n;
    bx.dI = fastdiv((unsigned int)bx.I);
    bx.dJ = fastdiv((unsigned int)bx.J);
    return bx;
}

__device__ inline void box_cell(const BoxIt2 &bx, unsigned int t, int &i, int &j, int &k) {
    const unsigned int row = bx.dI.div(t), kk = bx.dJ.div(row);
    i = bx.b.i0 + (int)(t - row * (unsigned int)bx.I);
    j = bx.b.j0 + (int)(row - kk * (unsigned int)bx.J);
    k = bx.b.k0 + (int)kk;
}

// Sums v over the grid; the last block writes the total through `fin`.
template <typename Fin>
__device__ inline void grid_sum(double v, double *partials, unsigned int *counter, Fin fin) {
    __shared__ double sm[RB / 32];
    __shared__ bool last;
    double bs = block_sum<RB>(v, sm);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = bs;
        __threadfence();
        unsigned int ticket = atomicAdd(counter, 1u);
        last = ticket == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    double s = 0.0;
    for (unsigned int q = threadIdx.x; q < gridDim.x; q += RB) s += __ldcg(partials + q);
    double tot = block_sum<RB>(s, sm);
    if (threadIdx.x == 0) {
        fin(tot);
        *counter = 0;
    }
}

template <typename Fin>
__device__ inline void grid_max(double v, double *partials, unsigned int *counter, Fin fin) {
    __shared__ double sm[RB / 32];
    __shared__ bool last;
    double bs = block_max<RB>(v, sm);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = bs;
        __threadfence();
        unsigned int ticket = atomicAdd(counter, 1u);
        last = ticket == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    double s = 0.0;
    for (unsigned int q = threadIdx.x; q < gridDim.x; q += RB) s = fmax(s, __ldcg(partials + q));
    double tot = block_max<RB>(s, sm);
    if (threadIdx.x == 0) {
        fin(tot);
        *counter = 0;
    }
}

__device__ inline double step_scalar(double a, int float_scalars) { return float_scalars ? (double)(float)a : a; }

// Dot-product accumulator.  FP64 vectors: products and sums in double.  FP32 vectors: the
// compensated dot product of Ogita, Rump and Oishi ("Accurate sum and dot product", SIAM J.
// Sci. Comput. 26, 2005): each product is split exactly into p + e (TwoProduct through fmaf)
// and summed with TwoSum, so a thread's partial sum hi + lo keeps about 48 significant bits
// without FP64 arithmetic per cell (FP64 throughput on this GPU is a small fraction of FP32);
// the partial sums are then added in FP64 across threads and blocks.
template <typename T> struct DotAcc {
    double acc = 0.0;
    __device__ void add(T a, T b) { acc += (double)a * (double)b; }
    __device__ double value() const { return acc; }
};
template <> struct DotAcc<float> {
    float hi = 0.0f, lo = 0.0f;
    __device__ void add(float a, float b) {
        const float p = a * b, e = fmaf(a, b, -p);       // p + e = a b exactly
        const float s = hi + p, bb = s - hi;
        const float err = (hi - (s - bb)) + (p - bb);    // hi + p = s + err exactly
        hi = s;
        lo += err + e;
    }
    __device__ double value() const { return (double)hi + (double)lo; }
};

// |r|_inf accumulator: the maximum is exact in the vectors' own precision.
template <typename T> struct MaxAcc {
    T m = T(0);
    __device__ void add(T v) { m = v > m ? v : m; }
    __device__ double value() const { return (double)m; }
};

// ---- vector kernels over the box ----
template <typename T>
__global__ void __launch_bounds__(RB) k_pcg_init(Dims d, BoxIt2 bx, const T *__restrict__ b, T *x, T *r, T *s, T *z) {
    const unsigned int n = bx.n;
    for (unsigned int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int i, j, k;
        box_cell(bx, t, i, j, k);
        size_t c = flat3(i, j, k, d.ni, d.nj);
        x[c] = 0; r[c] = b[c]; s[c] = 0; z[c] = 0;
    }
}

template <typename T>
__device__ inline T nb(const BoxIt2 &bx, const T *a, size_t c, int i, int j, int k) {
    return bx.in(i, j, k) ? a[c] : T(0);
}

// z = A s (row sum in column order -z,-y,-x,c,+x,+y,+z as sparsematrix.h:187-215), and s.z
template <typename T>
__global__ void __launch_bounds__(RB) k_spmv_dot(Dims d, BoxIt2 bx, OpView<T> A, const T *__restrict__ s,
                                                 T *__restrict__ z,
                                                 double *partials, unsigned int *counter, PcgScalars *sc,
                                                 int float_scalars) {
    if (sc->done) return;
    const unsigned int n = bx.n;
    size_t sl = (size_t)d.ni * d.nj;
    DotAcc<T> acc;
    FFGPU_UNROLL(FFGPU_VEC_UNROLL)
    for (unsigned int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int i, j, k;
        box_cell(bx, t, i, j, k);
        size_t c = flat3(i, j, k, d.ni, d.nj);
        T res = 0;
        res += nb(bx, A.az, c - sl, i, j, k - 1) * nb(bx, s, c - sl, i, j, k - 1);
        res += nb(bx, A.ay, c - d.ni, i, j - 1, k) * nb(bx, s, c - d.ni, i, j - 1, k);
        res += nb(bx, A.ax, c - 1, i - 1, j, k) * nb(bx, s, c - 1, i - 1, j, k);
        res += A.diag[c] * s[c];
        res += A.ax[c] * nb(bx, s, c + 1, i + 1, j, k);
        res += A.ay[c] * nb(bx, s, c + d.ni, i, j + 1, k);
        res += A.az[c] * nb(bx, s, c + sl, i, j, k + 1);
        z[c] = res;
        acc.add(s[c], res);
    }
    grid_sum(acc.value(), partials, counter, [&](double tot) {
        sc->sz = tot;
        sc->alpha = sc->rho / tot;
        sc->alpha_used = step_scalar(sc->alpha, float_scalars);
    });
}

// x += alpha s ; r -= alpha z ; |r|_inf
template <typename T>
__global__ void __launch_bounds__(RB) k_update_xr(Dims d, BoxIt2 bx, const T *__restrict__ s, const T *__restrict__ z,
                                                  T *__restrict__ x, T *__restrict__ r, double *partials,
                                                  unsigned int *counter,
                                                  PcgScalars *sc) {
    if (sc->done) return;
    const unsigned int n = bx.n;
    const T a = (T)sc->alpha_used, na = (T)(-sc->alpha_used);
    MaxAcc<T> m;
    FFGPU_UNROLL(FFGPU_VEC_UNROLL)
    for (unsigned int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int i, j, k;
        box_cell(bx, t, i, j, k);
        size_t c = flat3(i, j, k, d.ni, d.nj);
        x[c] += a * s[c];
        T rr = r[c] + na * z[c];
        r[c] = rr;
        m.add(rr < T(0) ? -rr : rr);
    }
    grid_max(m.value(), partials, counter, [&](double tot) {
        sc->resid = tot;
        sc->iters += 1;
        if (!sc->reliable) {
            if (tot <= sc->tol) sc->done = 1;
        } else {
            sc->rmax = fmax(sc->rmax, tot);
            if (tot <= sc->tol || tot <= sc->delta * sc->rmax) sc->update = 1;
        }
    });
}

// forward substitution on hyperplane `level`: q(c) = (r - Lz q(c-z) - Ly q(c-y) - Lx q(c-x)) inv(c)
template <typename T>
__global__ void k_fwd_level(Dims d, BoxIt2 bx, int level, FactorView<T> F, const T *__restrict__ r, T *q) {
    int IJ = bx.I * bx.J;
    size_t sl = (size_t)d.ni * d.nj;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < IJ; t += gridDim.x * blockDim.x) {
        int ii = t % bx.I, jj = t / bx.I, kk = level - ii - jj;
        if (kk < 0 || kk >= bx.K) continue;
        int i = bx.b.i0 + ii, j = bx.b.j0 + jj, k = bx.b.k0 + kk;
        size_t c = flat3(i, j, k, d.ni, d.nj);
        T v = r[c];
        if (kk > 0) v -= F.lz[c - sl] * q[c - sl];
        if (jj > 0) v -= F.ly[c - d.ni] * q[c - d.ni];
        if (ii > 0) v -= F.lx[c - 1] * q[c - 1];
        q[c] = v * F.inv[c];
    }
}

// backward substitution (in place): z(c) = (q - Lx(c) z(c+x) - Ly(c) z(c+y) - Lz(c) z(c+z)) inv(c)
template <typename T>
__global__ void k_bwd_level(Dims d, BoxIt2 bx, int level, FactorView<T> F, T *z) {
    int IJ = bx.I * bx.J;
    size_t sl = (size_t)d.ni * d.nj;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < IJ; t += gridDim.x * blockDim.x) {
        int ii = t % bx.I, jj = t / bx.I, kk = level - ii - jj;
        if (kk < 0 || kk >= bx.K) continue;
        int i = bx.b.i0 + ii, j = bx.b.j0 + jj, k = bx.b.k0 + kk;
        size_t c = flat3(i, j, k, d.ni, d.nj);
        T v = z[c];
        if (ii < bx.I - 1) v -= F.lx[c] * z[c + 1];
        if (jj < bx.J - 1) v -= F.ly[c] * z[c + d.ni];
        if (kk < bx.K - 1) v -= F.lz[c] * z[c + sl];
        z[c] = v * F.inv[c];
    }
}

// rho_new = z.r ; beta = rho_new / rho ; rho = rho_new  (first call: rho = z.r only)
template <typename T>
__global__ void __launch_bounds__(RB) k_dot_zr(Dims d, BoxIt2 bx, const T *__restrict__ z, const T *__restrict__ r,
                                               double *partials, unsigned int *counter, PcgScalars *sc,
                                               int first, int float_scalars) {
    if (sc->done) return;
    const unsigned int n = bx.n;
    DotAcc<T> acc;
    FFGPU_UNROLL(FFGPU_VEC_UNROLL)
    for (unsigned int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int i, j, k;
        box_cell(bx, t, i, j, k);
        size_t c = flat3(i, j, k, d.ni, d.nj);
        acc.add(z[c], r[c]);
    }
    grid_sum(acc.value(), partials, counter, [&](double tot) {
        if (first) {
            sc->rho = tot;
        } else {
            sc->beta = tot / sc->rho;
            sc->beta_used = step_scalar(sc->beta, float_scalars);
            sc->rho = tot;
        }
    });
}

// s = z + beta s   (first: s = z)
template <typename T>
__global__ void __launch_bounds__(RB) k_update_s(Dims d, BoxIt2 bx, const T *__restrict__ z, T *__restrict__ s,
                                                 PcgScalars *sc,
                                                 int first) {
    if (sc->done) return;
    const unsigned int n = bx.n;
    const T b = first ? T(0) : (T)sc->beta_used;
    FFGPU_UNROLL(FFGPU_VEC_UNROLL)
    for (unsigned int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int i, j, k;
        box_cell(bx, t, i, j, k);
        size_t c = flat3(i, j, k, d.ni, d.nj);
        s[c] = first ? z[c] : z[c] + b * s[c];
    }
}

// ---- FP32 kernels over aligned 4-cell groups ----
// With ni a multiple of 4 every grid row starts on a 16-byte boundary, so cells 4g .. 4g+3 of
// a row form one aligned float4.  These kernels walk the box as such groups (the first and
// last group of a row may reach outside the box; those lanes are neither counted nor
// written) with 16-byte loads and stores, four times the bytes per memory instruction of the
// per-cell kernels.  Each cell's arithmetic is the per-cell kernels' own, so the vectors
// they write are bit-identical; only the order in which dot-product terms are summed differs.
struct BoxVec {
    Bbox b;
    int g0, G, J;          // groups g0 .. g0 + G - 1 of each of the box's J x K rows
    unsigned int n;        // G J K
    FastDiv dG, dJ;
};
inline BoxVec boxvec(Bbox b) {
    BoxVec v;
    v.b = b;
    v.g0 = b.i0 / 4;
    v.G = b.i1 / 4 - v.g0 + 1;
    v.J = b.j1 - b.j0 + 1;
    const unsigned long long n = (unsigned long long)v.G * v.J * (b.k1 - b.k0 + 1);
    if (n >= (1ull << 31)) throw std::runtime_error("Error: pressure box exceeds 2^31 cells.\n");
    v.n = (unsigned int)n;
    v.dG = fastdiv((unsigned int)v.G);
    v.dJ = fastdiv((unsigned int)v.J);
    return v;
}
// first cell (i, j, k) of group t
__device__ inline void vec_group(const BoxVec &v, unsigned int t, int &i, int &j, int &k) {
    const unsigned int row = v.dG.div(t), kk = v.dJ.div(row);
    i = 4 * (v.g0 + (int)(t - row * (unsigned int)v.G));
    j = v.b.j0 + (int)(row - kk * (unsigned int)v.J);
    k = v.b.k0 + (int)kk;
}
__device__ inline float4 ld4(const float *p) { return *reinterpret_cast<const float4 *>(p); }
__device__ inline void st4(float *p, const float (&a)[4]) {
    *reinterpret_cast<float4 *>(p) = make_float4(a[0], a[1], a[2], a[3]);
}
__device__ inline void unpack(const float4 &v, float (&a)[4]) { a[0] = v.x; a[1] = v.y; a[2] = v.z; a[3] = v.w; }
// stores the lanes of group (i, ...) that lie inside [i0, i1]
__device__ inline void st_lanes(float *p, const float (&a)[4], int i, int i0, int i1) {
    if (i >= i0 && i + 3 <= i1) { st4(p, a); return; }
#pragma unroll
    for (int l = 0; l < 4; l++)
        if (i + l >= i0 && i + l <= i1) p[l] = a[l];
}

// Sum of products a_hi x + a_lo x over the seven stencil terms.  The operator is carried as
// hi + lo floats (hi = its FP32 rounding, lo = the FP32 rounding of the remainder), the
// products a_hi x are split exactly with fmaf and summed with TwoSum, so the row sum keeps
// about 48 bits: the FP32 iteration then sees the FP64 operator.  With the operator rounded
// to FP32 the Krylov recurrence needed 118 iterations where the FP64 solver needs 105; with
// the split operator it needs 104 (256^3 dam break), for 16 more bytes per cell.
struct RowSum {
    float hi = 0.0f, lo = 0.0f;
    __device__ void add(float ah, float x) {   // hi + lo += ah x, the product split exactly
        const float p = ah * x, e = fmaf(ah, x, -p);
        const float t = hi + p, bp = t - hi;
        const float err = (hi - (t - bp)) + (p - bp);
        hi = t;
        lo += err + e;
    }
    __device__ void add(float ah, float al, float x) { add(ah, x); lo += al * x; }
    __device__ float value() const { return hi + lo; }
};

template <bool SPLIT>
__global__ void __launch_bounds__(RB) k_spmv_dot_v4(Dims d, BoxVec v, OpView<float> A, OpView<float> Al,
                                                    const float *__restrict__ s, float *__restrict__ z,
                                                    double *partials, unsigned int *counter, PcgScalars *sc,
                                                    int float_scalars) {
    if (sc->done) return;
    const size_t sl = (size_t)d.ni * d.nj;
    DotAcc<float> acc;
    for (unsigned int t = blockIdx.x * blockDim.x + threadIdx.x; t < v.n; t += gridDim.x * blockDim.x) {
        int i, j, k;
        vec_group(v, t, i, j, k);
        const size_t c = flat3(i, j, k, d.ni, d.nj);
        const bool zm = k > v.b.k0, ym = j > v.b.j0, yp = j < v.b.j1, zp = k < v.b.k1;
        const bool xm = i - 1 >= v.b.i0, xp = i + 4 <= v.b.i1;
        // the stencil's seven s values per lane (zero outside the box, as the per-cell kernel)
        float szm[4] = {0, 0, 0, 0}, sym[4] = {0, 0, 0, 0}, syp[4] = {0, 0, 0, 0}, szp[4] = {0, 0, 0, 0}, s4[4];
        float sxm[4], sxp[4];
        if (zm) unpack(ld4(s + c - sl), szm);
        if (ym) unpack(ld4(s + c - d.ni), sym);
        unpack(ld4(s + c), s4);
        if (yp) unpack(ld4(s + c + d.ni), syp);
        if (zp) unpack(ld4(s + c + sl), szp);
        {
            const float sxl = xm ? s[c - 1] : 0.0f, sxr = xp ? s[c + 4] : 0.0f;
#pragma unroll
            for (int l = 0; l < 4; l++) {
                const int ii = i + l;
                sxm[l] = ii - 1 >= v.b.i0 ? (l == 0 ? sxl : s4[l > 0 ? l - 1 : 0]) : 0.0f;
                sxp[l] = ii + 1 <= v.b.i1 ? (l == 3 ? sxr : s4[l < 3 ? l + 1 : 3]) : 0.0f;
            }
        }
        float res[4];
        RowSum q[4];
        {   // the operator's FP32 part, in the per-cell kernel's term order
            float azm[4] = {0, 0, 0, 0}, aym[4] = {0, 0, 0, 0}, ax4[4], dg4[4], ay4[4], az4[4];
            if (zm) unpack(ld4(A.az + c - sl), azm);
            if (ym) unpack(ld4(A.ay + c - d.ni), aym);
            unpack(ld4(A.ax + c), ax4); unpack(ld4(A.diag + c), dg4); unpack(ld4(A.ay + c), ay4);
            unpack(ld4(A.az + c), az4);
            const float axl = xm ? A.ax[c - 1] : 0.0f;
#pragma unroll
            for (int l = 0; l < 4; l++) {
                const float axm_l = i + l - 1 >= v.b.i0 ? (l == 0 ? axl : ax4[l > 0 ? l - 1 : 0]) : 0.0f;
                if (SPLIT) {
                    q[l].add(azm[l], szm[l]); q[l].add(aym[l], sym[l]); q[l].add(axm_l, sxm[l]);
                    q[l].add(dg4[l], s4[l]); q[l].add(ax4[l], sxp[l]); q[l].add(ay4[l], syp[l]);
                    q[l].add(az4[l], szp[l]);
                } else {
                    float r = 0;
                    r += azm[l] * szm[l];
                    r += aym[l] * sym[l];
                    r += axm_l * sxm[l];
                    r += dg4[l] * s4[l];
                    r += ax4[l] * sxp[l];
                    r += ay4[l] * syp[l];
                    r += az4[l] * szp[l];
                    res[l] = r;
                }
            }
        }
        if (SPLIT) {   // the remainder lo, added to the low words of the row sums
            // (loaded after the FP32 part is consumed, keeping fewer values live at once)
            asm volatile("" ::: "memory");
            float lzm[4] = {0, 0, 0, 0}, lym[4] = {0, 0, 0, 0}, lx4[4], ldg[4], ly4[4], lz4[4];
            if (zm) unpack(ld4(Al.az + c - sl), lzm);
            if (ym) unpack(ld4(Al.ay + c - d.ni), lym);
            unpack(ld4(Al.ax + c), lx4); unpack(ld4(Al.diag + c), ldg); unpack(ld4(Al.ay + c), ly4);
            unpack(ld4(Al.az + c), lz4);
            const float lxl = xm ? Al.ax[c - 1] : 0.0f;
#pragma unroll
            for (int l = 0; l < 4; l++) {
                const float lxm_l = i + l - 1 >= v.b.i0 ? (l == 0 ? lxl : lx4[l > 0 ? l - 1 : 0]) : 0.0f;
                q[l].lo += lzm[l] * szm[l] + lym[l] * sym[l] + lxm_l * sxm[l] + ldg[l] * s4[l] + lx4[l] * sxp[l] +
                           ly4[l] * syp[l] + lz4[l] * szp[l];
                res[l] = q[l].value();
            }
        }
#pragma unroll
        for (int l = 0; l < 4; l++)
            if (i + l >= v.b.i0 && i + l <= v.b.i1) acc.add(s4[l], res[l]);
        st_lanes(z + c, res, i, v.b.i0, v.b.i1);
    }
    grid_sum(acc.value(), partials, counter, [&](double tot) {
        sc->sz = tot;
        sc->alpha = sc->rho / tot;
        sc->alpha_used = step_scalar(sc->alpha, float_scalars);
    });
}

__global__ void __launch_bounds__(RB) k_update_xr_v4(Dims d, BoxVec v, const float *__restrict__ s,
                                                     const float *__restrict__ z, float *__restrict__ x,
                                                     float *__restrict__ r, double *partials, unsigned int *counter,
                                                     PcgScalars *sc) {
    if (sc->done) return;
    const float a = (float)sc->alpha_used, na = (float)(-sc->alpha_used);
    MaxAcc<float> m;
    for (unsigned int t = blockIdx.x * blockDim.x + threadIdx.x; t < v.n; t += gridDim.x * blockDim.x) {
        int i, j, k;
        vec_group(v, t, i, j, k);
        const size_t c = flat3(i, j, k, d.ni, d.nj);
        float x4[4], s4[4], r4[4], z4[4];
        unpack(ld4(x + c), x4); unpack(ld4(s + c), s4); unpack(ld4(r + c), r4); unpack(ld4(z + c), z4);
#pragma unroll
        for (int l = 0; l < 4; l++) {
            x4[l] += a * s4[l];
            const float rr = r4[l] + na * z4[l];
            r4[l] = rr;
            if (i + l >= v.b.i0 && i + l <= v.b.i1) m.add(rr < 0.0f ? -rr : rr);
        }
        st_lanes(x + c, x4, i, v.b.i0, v.b.i1);
        st_lanes(r + c, r4, i, v.b.i0, v.b.i1);
    }
    grid_max(m.value(), partials, counter, [&](double tot) {
        sc->resid = tot;
        sc->iters += 1;
        if (!sc->reliable) {
            if (tot <= sc->tol) sc->done = 1;
        } else {
            sc->rmax = fmax(sc->rmax, tot);
            if (tot <= sc->tol || tot <= sc->delta * sc->rmax) sc->update = 1;
        }
    });
}

__global__ void __launch_bounds__(RB) k_dot_zr_v4(Dims d, BoxVec v, const float *__restrict__ z,
                                                  const float *__restrict__ r, double *partials, unsigned int *counter,
                                                  PcgScalars *sc, int first, int float_scalars) {
    if (sc->done) return;
    DotAcc<float> acc;
    for (unsigned int t = blockIdx.x * blockDim.x + threadIdx.x; t < v.n; t += gridDim.x * blockDim.x) {
        int i, j, k;
        vec_group(v, t, i, j, k);
        const size_t c = flat3(i, j, k, d.ni, d.nj);
        float z4[4], r4[4];
        unpack(ld4(z + c), z4); unpack(ld4(r + c), r4);
#pragma unroll
        for (int l = 0; l < 4; l++)
            if (i + l >= v.b.i0 && i + l <= v.b.i1) acc.add(z4[l], r4[l]);
    }
    grid_sum(acc.value(), partials, counter, [&](double tot) {
        if (first) {
            sc->rho = tot;
        } else {
            sc->beta = tot / sc->rho;
            sc->beta_used = step_scalar(sc->beta, float_scalars);
            sc->rho = tot;
        }
    });
}

__global__ void __launch_bounds__(RB) k_update_s_v4(Dims d, BoxVec v, const float *__restrict__ z,
                                                    float *__restrict__ s, PcgScalars *sc, int first) {
    if (sc->done) return;
    const float b = first ? 0.0f : (float)sc->beta_used;
    for (unsigned int t = blockIdx.x * blockDim.x + threadIdx.x; t < v.n; t += gridDim.x * blockDim.x) {
        int i, j, k;
        vec_group(v, t, i, j, k);
        const size_t c = flat3(i, j, k, d.ni, d.nj);
        float z4[4], s4[4];
        unpack(ld4(z + c), z4); unpack(ld4(s + c), s4);
#pragma unroll
        for (int l = 0; l < 4; l++) s4[l] = first ? z4[l] : z4[l] + b * s4[l];
        st_lanes(s + c, s4, i, v.b.i0, v.b.i1);
    }
}

// the group kernels apply to FP32 vectors on grids whose rows start 16-byte aligned
template <typename T> inline bool use_v4(Dims d) { return std::is_same<T, float>::value && d.ni % 4 == 0; }
static unsigned int vec_grid(const BoxVec &v) { return grid_for(v.n, RB, MAX_RED_BLOCKS); }

// ---- host launchers ----
static unsigned int red_grid(const BoxIt2 &bx) {
    const unsigned int n = bx.n;
    return grid_for(n, RB, MAX_RED_BLOCKS);
}

template <typename T>
void pcg_init(Dims d, Bbox bb, const T *b, PcgVecs<T> v, cudaStream_t st) {
    BoxIt2 bx = boxit2(bb);
    k_pcg_init<T><<<red_grid(bx), RB, 0, st>>>(d, bx, b, v.x, v.r, v.s, v.z);
}

template <typename T>
void pcg_spmv_dot(Dims d, Bbox bb, OpView<T> A, PcgVecs<T> v, PcgWork w, int float_scalars, cudaStream_t st) {
    if constexpr (std::is_same<T, float>::value) {
        if (use_v4<T>(d)) {
            const BoxVec bv = boxvec(bb);
            k_spmv_dot_v4<false><<<vec_grid(bv), RB, 0, st>>>(d, bv, A, A, v.s, v.z, w.partials, w.counter, w.sc,
                                                              float_scalars);
            return;
        }
    }
    BoxIt2 bx = boxit2(bb);
    k_spmv_dot<T><<<red_grid(bx), RB, 0, st>>>(d, bx, A, v.s, v.z, w.partials, w.counter, w.sc, float_scalars);
}

// the same split-operator row sum per cell, for rows that are not 16-byte aligned
__global__ void __launch_bounds__(RB) k_spmv_dot_split(Dims d, BoxIt2 bx, OpView<float> A, OpView<float> Al,
                                                       const float *__restrict__ s, float *__restrict__ z,
                                                       double *partials, unsigned int *counter, PcgScalars *sc) {
    if (sc->done) return;
    const unsigned int n = bx.n;
    const size_t sl = (size_t)d.ni * d.nj;
    DotAcc<float> acc;
    for (unsigned int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int i, j, k;
        box_cell(bx, t, i, j, k);
        size_t c = flat3(i, j, k, d.ni, d.nj);
        RowSum q;
        q.add(nb(bx, A.az, c - sl, i, j, k - 1), nb(bx, Al.az, c - sl, i, j, k - 1), nb(bx, s, c - sl, i, j, k - 1));
        q.add(nb(bx, A.ay, c - d.ni, i, j - 1, k), nb(bx, Al.ay, c - d.ni, i, j - 1, k), nb(bx, s, c - d.ni, i, j - 1, k));
        q.add(nb(bx, A.ax, c - 1, i - 1, j, k), nb(bx, Al.ax, c - 1, i - 1, j, k), nb(bx, s, c - 1, i - 1, j, k));
        q.add(A.diag[c], Al.diag[c], s[c]);
        q.add(A.ax[c], Al.ax[c], nb(bx, s, c + 1, i + 1, j, k));
        q.add(A.ay[c], Al.ay[c], nb(bx, s, c + d.ni, i, j + 1, k));
        q.add(A.az[c], Al.az[c], nb(bx, s, c + sl, i, j, k + 1));
        const float res = q.value();
        z[c] = res;
        acc.add(s[c], res);
    }
    grid_sum(acc.value(), partials, counter, [&](double tot) {
        sc->sz = tot;
        sc->alpha = sc->rho / tot;
        sc->alpha_used = sc->alpha;   // FP64 step length (the mixed solver does not truncate it)
    });
}

void pcg_spmv_dot_split(Dims d, Bbox bb, OpView<float> A, OpView<float> Alo, PcgVecs<float> v, PcgWork w,
                        cudaStream_t st) {
    if (use_v4<float>(d)) {
        const BoxVec bv = boxvec(bb);
        k_spmv_dot_v4<true><<<vec_grid(bv), RB, 0, st>>>(d, bv, A, Alo, v.s, v.z, w.partials, w.counter, w.sc, 0);
        return;
    }
    BoxIt2 bx = boxit2(bb);
    k_spmv_dot_split<<<red_grid(bx), RB, 0, st>>>(d, bx, A, Alo, v.s, v.z, w.partials, w.counter, w.sc);
}

template <typename T>
void pcg_update_xr(Dims d, Bbox bb, PcgVecs<T> v, PcgWork w, cudaStream_t st) {
    if constexpr (std::is_same<T, float>::value) {
        if (use_v4<T>(d)) {
            const BoxVec bv = boxvec(bb);
            k_update_xr_v4<<<vec_grid(bv), RB, 0, st>>>(d, bv, v.s, v.z, v.x, v.r, w.partials, w.counter, w.sc);
            return;
        }
    }
    BoxIt2 bx = boxit2(bb);
    k_update_xr<T><<<red_grid(bx), RB, 0, st>>>(d, bx, v.s, v.z, v.x, v.r, w.partials, w.counter, w.sc);
}

template <typename T>
void pcg_precondition_fwd(Dims d, Bbox bb, FactorView<T> F, const T *r, T *z, cudaStream_t st) {
    BoxIt2 bx = boxit2(bb);
    int levels = bx.I + bx.J + bx.K - 2;
    unsigned int g = grid_for((size_t)bx.I * bx.J, 128, 152u * 8u);
    for (int l = 0; l < levels; l++) k_fwd_level<T><<<g, 128, 0, st>>>(d, bx, l, F, r, z);
}

template <typename T>
void pcg_precondition_bwd(Dims d, Bbox bb, FactorView<T> F, T *z, cudaStream_t st) {
    BoxIt2 bx = boxit2(bb);
    int levels = bx.I + bx.J + bx.K - 2;
    unsigned int g = grid_for((size_t)bx.I * bx.J, 128, 152u * 8u);
    for (int l = levels - 1; l >= 0; l--) k_bwd_level<T><<<g, 128, 0, st>>>(d, bx, l, F, z);
}

template <typename T>
void pcg_precondition(Dims d, Bbox bb, FactorView<T> F, const T *r, T *z, cudaStream_t st) {
    pcg_precondition_fwd<T>(d, bb, F, r, z, st);
    pcg_precondition_bwd<T>(d, bb, F, z, st);
}

template <typename T>
void pcg_dot_zr(Dims d, Bbox bb, PcgVecs<T> v, PcgWork w, int first, int float_scalars, cudaStream_t st) {
    if constexpr (std::is_same<T, float>::value) {
        if (use_v4<T>(d)) {
            const BoxVec bv = boxvec(bb);
            k_dot_zr_v4<<<vec_grid(bv), RB, 0, st>>>(d, bv, v.z, v.r, w.partials, w.counter, w.sc, first, float_scalars);
            return;
        }
    }
    BoxIt2 bx = boxit2(bb);
    k_dot_zr<T><<<red_grid(bx), RB, 0, st>>>(d, bx, v.z, v.r, w.partials, w.counter, w.sc, first, float_scalars);
}

template <typename T>
void pcg_update_s(Dims d, Bbox bb, PcgVecs<T> v, PcgWork w, int first, cudaStream_t st) {
    if constexpr (std::is_same<T, float>::value) {
        if (use_v4<T>(d)) {
            const BoxVec bv = boxvec(bb);
            k_update_s_v4<<<vec_grid(bv), RB, 0, st>>>(d, bv, v.z, v.s, w.sc, first);
            return;
        }
    }
    BoxIt2 bx = boxit2(bb);
    k_update_s<T><<<red_grid(bx), RB, 0, st>>>(d, bx, v.z, v.s, w.sc, first);
}


// pressure grid (float) <- x over the box; the caller zeroes the grid first
template <typename T>
__global__ void k_store_pressure(Dims d, BoxIt2 bx, const T *__restrict__ x, float *pr) {
    const unsigned int n = bx.n;
    for (unsigned int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int i, j, k;
        box_cell(bx, t, i, j, k);
        size_t c = flat3(i, j, k, d.ni, d.nj);
        pr[c] = (float)x[c];
    }
}

// K14: FP64 true residual r = b - A x (A in FP64), |r|_inf, and its FP32 copy for the
// next inner solve of the mixed-precision refinement.
__global__ void __launch_bounds__(RB) k_true_residual(Dims d, BoxIt2 bx, OpView<double> A, const double *__restrict__ b,
                                                      const double *__restrict__ x, double *r, float *rf,
                                                      double *partials, unsigned int *counter, PcgScalars *sc) {
    const unsigned int n = bx.n;
    size_t sl = (size_t)d.ni * d.nj;
    double m = 0.0;
    for (unsigned int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int i, j, k;
        box_cell(bx, t, i, j, k);
        size_t c = flat3(i, j, k, d.ni, d.nj);
        double res = 0;
        res += nb(bx, A.az, c - sl, i, j, k - 1) * nb(bx, x, c - sl, i, j, k - 1);
        res += nb(bx, A.ay, c - d.ni, i, j - 1, k) * nb(bx, x, c - d.ni, i, j - 1, k);
        res += nb(bx, A.ax, c - 1, i - 1, j, k) * nb(bx, x, c - 1, i - 1, j, k);
        res += A.diag[c] * x[c];
        res += A.ax[c] * nb(bx, x, c + 1, i + 1, j, k);
        res += A.ay[c] * nb(bx, x, c + d.ni, i, j + 1, k);
        res += A.az[c] * nb(bx, x, c + sl, i, j, k + 1);
        double rr = b[c] - res;
        r[c] = rr;
        rf[c] = (float)rr;
        m = fmax(m, fabs(rr));
    }
    grid_max(m, partials, counter, [&](double tot) {
        sc->resid = tot;
        sc->rmax = tot;
    });
}

// Reliable update, part 1: x64 += x32, x32 = 0 (only while an update is requested)
__global__ void k_reliable_fold(Dims d, BoxIt2 bx, float *x32, double *x64, const PcgScalars *sc) {
    if (sc->done || !sc->update) return;
    const unsigned int n = bx.n;
    for (unsigned int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int i, j, k;
        box_cell(bx, t, i, j, k);
        size_t c = flat3(i, j, k, d.ni, d.nj);
        x64[c] += (double)x32[c];
        x32[c] = 0.0f;
    }
}

// Reliable update, part 2: r64 = b - A64 x64, r32 = (float) r64, |r64|_inf; ends the update
__global__ void __launch_bounds__(RB) k_reliable_residual(Dims d, BoxIt2 bx, OpView<double> A,
                                                          const double *__restrict__ b, const double *__restrict__ x,
                                                          double *r, float *rf, double *partials,
                                                          unsigned int *counter, PcgScalars *sc) {
    if (sc->done || !sc->update) return;
    const unsigned int n = bx.n;
    size_t sl = (size_t)d.ni * d.nj;
    double m = 0.0;
    for (unsigned int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int i, j, k;
        box_cell(bx, t, i, j, k);
        size_t c = flat3(i, j, k, d.ni, d.nj);
        double res = 0;
        res += nb(bx, A.az, c - sl, i, j, k - 1) * nb(bx, x, c - sl, i, j, k - 1);
        res += nb(bx, A.ay, c - d.ni, i, j - 1, k) * nb(bx, x, c - d.ni, i, j - 1, k);
        res += nb(bx, A.ax, c - 1, i - 1, j, k) * nb(bx, x, c - 1, i - 1, j, k);
        res += A.diag[c] * x[c];
        res += A.ax[c] * nb(bx, x, c + 1, i + 1, j, k);
        res += A.ay[c] * nb(bx, x, c + d.ni, i, j + 1, k);
        res += A.az[c] * nb(bx, x, c + sl, i, j, k + 1);
        double rr = b[c] - res;
        r[c] = rr;
        rf[c] = (float)rr;
        m = fmax(m, fabs(rr));
    }
    grid_max(m, partials, counter, [&](double tot) {
        sc->resid = tot;
        sc->rmax = tot;
        sc->update = 0;
        sc->updates += 1;
        if (tot <= sc->target) sc->done = 1;
    });
}

// x64 += (double) correction
__global__ void k_refine(Dims d, BoxIt2 bx, const float *__restrict__ dxf, double *x) {
    const unsigned int n = bx.n;
    for (unsigned int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int i, j, k;
        box_cell(bx, t, i, j, k);
        size_t c = flat3(i, j, k, d.ni, d.nj);
        x[c] += (double)dxf[c];
    }
}

// x64 = 0 over the box
__global__ void k_zero_box(Dims d, BoxIt2 bx, double *x) {
    const unsigned int n = bx.n;
    for (unsigned int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int i, j, k;
        box_cell(bx, t, i, j, k);
        x[flat3(i, j, k, d.ni, d.nj)] = 0.0;
    }
}

template <typename T>
void pcg_store_pressure(Dims d, Bbox bb, const T *x, float *pressure, cudaStream_t st) {
    BoxIt2 bx = boxit2(bb);
    k_store_pressure<T><<<red_grid(bx), RB, 0, st>>>(d, bx, x, pressure);
}

void pcg_true_residual(Dims d, Bbox bb, OpView<double> A, const double *b, const double *x, double *r, float *rf,
                       PcgWork w, cudaStream_t st) {
    BoxIt2 bx = boxit2(bb);
    k_true_residual<<<red_grid(bx), RB, 0, st>>>(d, bx, A, b, x, r, rf, w.partials, w.counter, w.sc);
}

void pcg_refine(Dims d, Bbox bb, const float *corr, double *x, cudaStream_t st) {
    BoxIt2 bx = boxit2(bb);
    k_refine<<<red_grid(bx), RB, 0, st>>>(d, bx, corr, x);
}

void pcg_reliable_update(Dims d, Bbox bb, OpView<double> A, const double *b, double *x64, float *x32, double *r64,
                         float *r32, PcgWork w, cudaStream_t st) {
    BoxIt2 bx = boxit2(bb);
    k_reliable_fold<<<red_grid(bx), RB, 0, st>>>(d, bx, x32, x64, w.sc);
    k_reliable_residual<<<red_grid(bx), RB, 0, st>>>(d, bx, A, b, x64, r64, r32, w.partials, w.counter, w.sc);
}

// x = the previous substep's pressure (scaled), zero outside the pressure cells
__global__ void k_warm_start(Dims d, BoxIt2 bx, const float *__restrict__ prev, const unsigned char *__restrict__ fluid,
                             double scale, double *x, const float *__restrict__ prev2, double scale2) {
    const unsigned int n = bx.n;
    for (unsigned int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        int i, j, k;
        box_cell(bx, t, i, j, k);
        const size_t c = flat3(i, j, k, d.ni, d.nj);
        double v = (double)prev[c] * scale;
        if (prev2) v += (double)prev2[c] * scale2;
        x[c] = fluid[c] ? v : 0.0;
    }
}

void pcg_warm_start(Dims d, Bbox bb, const float *prev, const unsigned char *fluid, double scale, double *x,
                    cudaStream_t st, const float *prev2, double scale2) {
    BoxIt2 bx = boxit2(bb);
    k_warm_start<<<red_grid(bx), RB, 0, st>>>(d, bx, prev, fluid, scale, x, prev2, scale2);
}

void pcg_zero(Dims d, Bbox bb, double *x, cudaStream_t st) {
    BoxIt2 bx = boxit2(bb);
    k_zero_box<<<red_grid(bx), RB, 0, st>>>(d, bx, x);
}

#define FFGPU_PCG_INST(T)                                                                                     \
    template void pcg_init<T>(Dims, Bbox, const T *, PcgVecs<T>, cudaStream_t);                               \
    template void pcg_spmv_dot<T>(Dims, Bbox, OpView<T>, PcgVecs<T>, PcgWork, int, cudaStream_t);           \
    template void pcg_update_xr<T>(Dims, Bbox, PcgVecs<T>, PcgWork, cudaStream_t);                          \
    template void pcg_precondition<T>(Dims, Bbox, FactorView<T>, const T *, T *, cudaStream_t);             \
    template void pcg_precondition_fwd<T>(Dims, Bbox, FactorView<T>, const T *, T *, cudaStream_t);         \
    template void pcg_precondition_bwd<T>(Dims, Bbox, FactorView<T>, T *, cudaStream_t);                    \
    template void pcg_dot_zr<T>(Dims, Bbox, PcgVecs<T>, PcgWork, int, int, cudaStream_t);                   \
    template void pcg_update_s<T>(Dims, Bbox, PcgVecs<T>, PcgWork, int, cudaStream_t);                      \
    template void pcg_store_pressure<T>(Dims, Bbox, const T *, float *, cudaStream_t);
FFGPU_PCG_INST(double)
FFGPU_PCG_INST(float)

}  // namespace ffgpu
