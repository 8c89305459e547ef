// The mixed-precision solve in a copy of the pressure box with its axes reordered.
//
// The MIC(0) wavefront (mic_wavefront.cu) sweeps the box's slowest axis plane by plane, with
// 16 x 16-cell tiles over the other two; its critical path is about K + 7 (A - 1) + 7 (B - 1)
// steps for K planes and A x B tiles.  On a box whose slowest axis is its longest (the 256^3 dam
// break's is 90 x 128 x 254 cells) the chain is shorter when the shortest axis is swept instead:
// ~258 against ~352 steps.  The mixed solve therefore copies its operator, factor and right-hand
// side into a box-sized grid whose axes are the box's in a chosen order (new axis a = old axis
// perm[a]), runs unchanged on it, and copies the solution back.  A coupling or factor entry along
// new axis a is the old one along perm[a]: A'(c', c' + e_a) = A(c, c + e_perm[a]).  The rows'
// arithmetic is the same (the SpMV sums its seven terms in the new axes' order); the FP64 solver
// keeps the grid's own order, in which its SpMV sums as the reference does.
#include "kernels.h"
#include "pcg.h"

namespace ffgpu {
namespace {

struct PermIt {
    Bbox b;
    int I, J, K;       // box extents (old axes)
    int perm[3];       // new axis a <- old axis perm[a]
    Dims dp;           // permuted grid (row length padded to a multiple of 4)
    __device__ size_t to_new(int li, int lj, int lk) const {
        const int l[3] = {li, lj, lk};
        return flat3(l[perm[0]], l[perm[1]], l[perm[2]], dp.ni, dp.nj);
    }
};

PermIt permit(Bbox bb, AxisMap m, Dims dp) {
    PermIt p;
    p.b = bb;
    p.I = bb.i1 - bb.i0 + 1; p.J = bb.j1 - bb.j0 + 1; p.K = bb.k1 - bb.k0 + 1;
    for (int a = 0; a < 3; a++) p.perm[a] = m.perm[a];
    p.dp = dp;
    return p;
}

__global__ void k_permute_system(Dims d, PermIt P, PressureSystem sys, PermutedSystem out) {
    const size_t n = (size_t)P.I * P.J * P.K;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        const int li = (int)(t % P.I), lj = (int)((t / P.I) % P.J), lk = (int)(t / ((size_t)P.I * P.J));
        const size_t c = flat3(P.b.i0 + li, P.b.j0 + lj, P.b.k0 + lk, d.ni, d.nj);
        const size_t q = P.to_new(li, lj, lk);
        const double a[3] = {sys.ax[c], sys.ay[c], sys.az[c]};
        const double l[3] = {sys.lx[c], sys.ly[c], sys.lz[c]};
        const double dg = sys.diag[c];
        const double na[3] = {a[P.perm[0]], a[P.perm[1]], a[P.perm[2]]};
        out.diag[q] = dg; out.ax[q] = na[0]; out.ay[q] = na[1]; out.az[q] = na[2];
        const float dh = (float)dg, xh = (float)na[0], yh = (float)na[1], zh = (float)na[2];
        out.diag32[q] = dh; out.ax32[q] = xh; out.ay32[q] = yh; out.az32[q] = zh;
        out.diag32lo[q] = (float)(dg - (double)dh); out.ax32lo[q] = (float)(na[0] - (double)xh);
        out.ay32lo[q] = (float)(na[1] - (double)yh); out.az32lo[q] = (float)(na[2] - (double)zh);
        out.inv32[q] = (float)sys.inv[c];
        out.lx32[q] = (float)l[P.perm[0]]; out.ly32[q] = (float)l[P.perm[1]]; out.lz32[q] = (float)l[P.perm[2]];
    }
}

template <typename T>
__global__ void k_permute_box(Dims d, PermIt P, const T *__restrict__ src, T *__restrict__ dst, int back) {
    const size_t n = (size_t)P.I * P.J * P.K;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        const int li = (int)(t % P.I), lj = (int)((t / P.I) % P.J), lk = (int)(t / ((size_t)P.I * P.J));
        const size_t c = flat3(P.b.i0 + li, P.b.j0 + lj, P.b.k0 + lk, d.ni, d.nj);
        const size_t q = P.to_new(li, lj, lk);
        if (back) dst[c] = src[q];
        else dst[q] = src[c];
    }
}

// The system copy as 32 x 32 tiles of the plane of old x and old axis P.perm[0] (the copy's x), one
// plane of the third axis per blockIdx.z: read along old x, written along the copy's x through a
// shared-memory transpose, so both sides move whole lines (with perm[0] != 0 the one-cell-per-thread
// kernel above writes every value to a separate line, and its twelve outputs do not fit in L2).
// Blocks of 32 x 8 threads.
constexpr int PT = 32, PR = 8;

struct PermTile {
    int l[3];   // old box coordinates of this thread's cell in the load phase
    int w[3];   // and in the store phase
    bool lin, win;
};
__device__ inline PermTile perm_tile(const PermIt &P, int r) {
    const int p0 = P.perm[0], o = 3 - p0;   // p0 is 1 or 2; o the remaining old axis
    const int ext[3] = {P.I, P.J, P.K};
    const int x0 = blockIdx.x * PT, a0 = blockIdx.y * PT;
    PermTile t;
    t.l[0] = x0 + threadIdx.x; t.l[p0] = a0 + threadIdx.y + PR * r; t.l[o] = blockIdx.z;
    t.w[0] = x0 + threadIdx.y + PR * r; t.w[p0] = a0 + threadIdx.x; t.w[o] = blockIdx.z;
    t.lin = t.l[0] < ext[0] && t.l[p0] < ext[p0];
    t.win = t.w[0] < ext[0] && t.w[p0] < ext[p0];
    return t;
}
__device__ inline size_t old_cell(const Dims &d, const PermIt &P, const int *l) {
    return flat3(P.b.i0 + l[0], P.b.j0 + l[1], P.b.k0 + l[2], d.ni, d.nj);
}

__global__ void __launch_bounds__(PT * PR) k_permute_system_t(Dims d, PermIt P, PressureSystem sys, PermutedSystem out) {
    __shared__ double tile[PT][PT + 1];
    int inv[3];   // new axis of each old axis
    for (int a = 0; a < 3; a++) inv[P.perm[a]] = a;
    const double *src[8] = {sys.diag, sys.ax, sys.ay, sys.az, sys.inv, sys.lx, sys.ly, sys.lz};
    double *a64[3] = {out.ax, out.ay, out.az};
    float *a32[3] = {out.ax32, out.ay32, out.az32}, *a32lo[3] = {out.ax32lo, out.ay32lo, out.az32lo};
    float *l32[3] = {out.lx32, out.ly32, out.lz32};
    for (int m = 0; m < 8; m++) {
#pragma unroll
        for (int r = 0; r < PT / PR; r++) {
            const PermTile t = perm_tile(P, r);
            if (t.lin) tile[threadIdx.y + PR * r][threadIdx.x] = src[m][old_cell(d, P, t.l)];
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < PT / PR; r++) {
            const PermTile t = perm_tile(P, r);
            if (!t.win) continue;
            const double v = tile[threadIdx.x][threadIdx.y + PR * r];
            const size_t q = P.to_new(t.w[0], t.w[1], t.w[2]);
            if (m == 0) {
                const float h = (float)v;
                out.diag[q] = v; out.diag32[q] = h; out.diag32lo[q] = (float)(v - (double)h);
            } else if (m < 4) {   // coupling along old axis m - 1: the copy's axis inv[m - 1]
                const int n = inv[m - 1];
                const float h = (float)v;
                a64[n][q] = v; a32[n][q] = h; a32lo[n][q] = (float)(v - (double)h);
            } else if (m == 4) {
                out.inv32[q] = (float)v;
            } else {
                l32[inv[m - 5]][q] = (float)v;
            }
        }
        __syncthreads();
    }
}

dim3 perm_tiles(const PermIt &P) {
    const int ext[3] = {P.I, P.J, P.K};
    const int p0 = P.perm[0], o = 3 - p0;
    return dim3((unsigned)((ext[0] + PT - 1) / PT), (unsigned)((ext[p0] + PT - 1) / PT), (unsigned)ext[o]);
}

}  // namespace

AxisMap choose_axis_map(Bbox bb, Dims &dp, Bbox &pbox) {
    const int e[3] = {bb.i1 - bb.i0 + 1, bb.j1 - bb.j0 + 1, bb.k1 - bb.k0 + 1};
    AxisMap m{{0, 1, 2}};
    // sweep the shortest axis when it is under 4/5 of the slowest one; the slowest axis takes the
    // shortest one's place, the third keeps its own
    const int shortest = e[0] <= e[1] ? (e[0] <= e[2] ? 0 : 2) : (e[1] <= e[2] ? 1 : 2);
    if (shortest != 2 && 5 * e[shortest] < 4 * e[2]) {
        if (shortest == 0) m = AxisMap{{2, 1, 0}};   // x' = z, y' = y, z' = x
        else m = AxisMap{{0, 2, 1}};                 // x' = x, y' = z, z' = y
    }
    const int ne[3] = {e[m.perm[0]], e[m.perm[1]], e[m.perm[2]]};
    dp = Dims{(ne[0] + 3) / 4 * 4, ne[1], ne[2]};
    pbox = Bbox{0, 0, 0, ne[0] - 1, ne[1] - 1, ne[2] - 1};
    return m;
}

void launch_permute_system(Dims d, Bbox bb, AxisMap m, Dims dp, PressureSystem sys, PermutedSystem out,
                           cudaStream_t st) {
    const PermIt P = permit(bb, m, dp);
    const size_t n = (size_t)P.I * P.J * P.K;
    if (n == 0) return;
    if (P.perm[0] != 0) k_permute_system_t<<<perm_tiles(P), dim3(PT, PR), 0, st>>>(d, P, sys, out);
    else k_permute_system<<<grid_for(n, 256), 256, 0, st>>>(d, P, sys, out);
    FFGPU_CUDA(cudaGetLastError());
}

template <typename T>
void launch_permute_box(Dims d, Bbox bb, AxisMap m, Dims dp, const T *src, T *dst, int back, cudaStream_t st) {
    const PermIt P = permit(bb, m, dp);
    const size_t n = (size_t)P.I * P.J * P.K;
    if (n == 0) return;
    // one box-sized vector fits in L2, which absorbs the scattered side: the one-cell-per-thread
    // kernel measured faster here (24 against 45 us at 256^3) than the tiled transpose
    k_permute_box<T><<<grid_for(n, 256), 256, 0, st>>>(d, P, src, dst, back);
    FFGPU_CUDA(cudaGetLastError());
}

template void launch_permute_box<double>(Dims, Bbox, AxisMap, Dims, const double *, double *, int, cudaStream_t);
template void launch_permute_box<float>(Dims, Bbox, AxisMap, Dims, const float *, float *, int, cudaStream_t);

}  // namespace ffgpu
