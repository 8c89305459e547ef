// K1-K3: counting sort of marker particles by cell.  Gives per-cell particle ranges
// (cell_start) and a stable permutation (particles of one cell in increasing particle
// index), so every later gather is deterministic.  The cell index is the reference's
// positionToGridIndex: floor(p * (1/dx)) in double (grid3d.h:55-60).
#include "common.cuh"
#include "kernels.h"

namespace ffgpu {

size_t scan_scratch_ints(size_t n) { return (n + SCAN_TILE - 1) / SCAN_TILE + 1; }

constexpr int SCAN_BLOCK = 256;
constexpr int SCAN_ITEMS = SCAN_TILE / SCAN_BLOCK;   // 16

__global__ void __launch_bounds__(SCAN_BLOCK) k_tile_sums(const int *__restrict__ in, size_t n, int *sums) {
    size_t base = (size_t)blockIdx.x * SCAN_TILE;
    int s = 0;
    for (int q = 0; q < SCAN_ITEMS; q++) {
        size_t t = base + (size_t)q * SCAN_BLOCK + threadIdx.x;
        if (t < n) s += in[t];
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    __shared__ int ws[SCAN_BLOCK / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < SCAN_BLOCK / 32; w++) t += ws[w];
        sums[blockIdx.x] = t;
    }
}

// Exclusive scan of the tile sums in one block (sequential per thread chunk).
__global__ void k_scan_sums(int *sums, int nt) {
    __shared__ int part[1024];
    int per = (nt + blockDim.x - 1) / blockDim.x;
    int b0 = threadIdx.x * per, b1 = min(b0 + per, nt);
    int s = 0;
    for (int b = b0; b < b1; b++) s += sums[b];
    part[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int t = 0; t < (int)blockDim.x; t++) { int v = part[t]; part[t] = run; run += v; }
        sums[nt] = run;
    }
    __syncthreads();
    int run = part[threadIdx.x];
    for (int b = b0; b < b1; b++) { int v = sums[b]; sums[b] = run; run += v; }
}

__device__ inline int warp_excl_scan(int v, int &total) {
    int lane = threadIdx.x & 31;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    total = __shfl_sync(0xffffffffu, x, 31);
    return x - v;
}

__global__ void __launch_bounds__(SCAN_BLOCK) k_tile_scan(const int *__restrict__ in, int *out, size_t n,
                                                          const int *__restrict__ sums) {
    __shared__ int tile[SCAN_TILE];
    __shared__ int wsum[SCAN_BLOCK / 32];
    size_t base = (size_t)blockIdx.x * SCAN_TILE;
    for (int q = 0; q < SCAN_ITEMS; q++) {
        int l = q * SCAN_BLOCK + threadIdx.x;
        size_t t = base + l;
        tile[l] = t < n ? in[t] : 0;
    }
    __syncthreads();
    int loc[SCAN_ITEMS];
    int s = 0;
    for (int q = 0; q < SCAN_ITEMS; q++) { loc[q] = s; s += tile[threadIdx.x * SCAN_ITEMS + q]; }
    int wt;
    int ex = warp_excl_scan(s, wt);
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = wt;
    __syncthreads();
    int woff = 0;
    for (int w = 0; w < (int)(threadIdx.x >> 5); w++) woff += wsum[w];
    int off = sums[blockIdx.x] + woff + ex;
    __syncthreads();
    for (int q = 0; q < SCAN_ITEMS; q++) tile[threadIdx.x * SCAN_ITEMS + q] = off + loc[q];
    __syncthreads();
    for (int q = 0; q < SCAN_ITEMS; q++) {
        int l = q * SCAN_BLOCK + threadIdx.x;
        size_t t = base + l;
        if (t < n) out[t] = tile[l];
    }
}

__global__ void k_write_total(int *out, size_t n, const int *sums, int nt) { out[n] = sums[nt]; }

void launch_exclusive_scan(const int *in, int *out, size_t n, int *scratch, cudaStream_t st) {
    int nt = (int)((n + SCAN_TILE - 1) / SCAN_TILE);
    if (nt == 0) {
        FFGPU_CUDA(cudaMemsetAsync(out, 0, sizeof(int), st));
        return;
    }
    k_tile_sums<<<nt, SCAN_BLOCK, 0, st>>>(in, n, scratch);
    k_scan_sums<<<1, 1024, 0, st>>>(scratch, nt);
    k_tile_scan<<<nt, SCAN_BLOCK, 0, st>>>(in, out, n, scratch);
    k_write_total<<<1, 1, 0, st>>>(out, n, scratch, nt);
}

// Cell keys: floor(x / dx) in double (Grid3d::positionToGridIndex, grid3d.h:55-60), or with
// float_keys the float floor(x * (float)(1 / dx)) that FP32 MAC sampling uses.
__global__ void k_cell_keys(Dims d, double dx, int np, const float *__restrict__ px, const float *__restrict__ py,
                            const float *__restrict__ pz, int *key, int *rank, int *count, int float_keys) {
    const double inv = 1.0 / dx;
    const float invf = (float)inv;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        int i, j, k;
        if (float_keys) {
            i = (int)floorf(px[p] * invf); j = (int)floorf(py[p] * invf); k = (int)floorf(pz[p] * invf);
        } else {
            i = floor_fd(px[p], inv, invf); j = floor_fd(py[p], inv, invf); k = floor_fd(pz[p], inv, invf);
        }
        i = min(max(i, 0), d.ni - 1); j = min(max(j, 0), d.nj - 1); k = min(max(k, 0), d.nk - 1);
        int c = (int)flat3(i, j, k, d.ni, d.nj);
        key[p] = c;
        rank[p] = atomicAdd(&count[c], 1);
    }
}

void launch_cell_keys(Dims d, double dx, int np, const float *px, const float *py, const float *pz,
                      int *key, int *rank, int *count, cudaStream_t st, bool float_keys) {
    if (np == 0) return;
    k_cell_keys<<<grid_for(np, 256), 256, 0, st>>>(d, dx, np, px, py, pz, key, rank, count, float_keys ? 1 : 0);
}

__global__ void k_scatter_sorted(int np, const int *__restrict__ key, const int *__restrict__ rank,
                                 const int *__restrict__ cell_start, int *sorted_idx) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x)
        sorted_idx[cell_start[key[p]] + rank[p]] = p;
}

void launch_scatter_sorted(int np, const int *key, const int *rank, const int *cell_start, int *sorted_idx,
                           cudaStream_t st) {
    if (np == 0) return;
    k_scatter_sorted<<<grid_for(np, 256), 256, 0, st>>>(np, key, rank, cell_start, sorted_idx);
}

// Restores particle-index order inside each cell (atomic ranks are unordered).
__global__ void k_sort_within_cells(size_t nc, const int *__restrict__ cell_start, int *idx) {
    for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < nc; c += (size_t)gridDim.x * blockDim.x) {
        int a = cell_start[c], b = cell_start[c + 1];
        for (int x = a + 1; x < b; x++) {
            int v = idx[x];
            int y = x - 1;
            while (y >= a && idx[y] > v) { idx[y + 1] = idx[y]; y--; }
            idx[y + 1] = v;
        }
    }
}

void launch_sort_within_cells(size_t ncells, const int *cell_start, int *sorted_idx, cudaStream_t st) {
    k_sort_within_cells<<<grid_for(ncells, 256), 256, 0, st>>>(ncells, cell_start, sorted_idx);
}

constexpr int MAX_GATHER_ATTRS = 16;
struct PtrPack { const float *src[MAX_GATHER_ATTRS]; float *dst[MAX_GATHER_ATTRS]; };

__global__ void k_gather(int np, const int *__restrict__ idx, PtrPack pk, int nattr) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        int s = idx[p];
        for (int a = 0; a < nattr; a++) pk.dst[a][p] = pk.src[a][s];
    }
}

void launch_gather_particles(int np, const int *sorted_idx, const float *const *src, float *const *dst, int nattr,
                             cudaStream_t st) {
    if (nattr < 0 || nattr > MAX_GATHER_ATTRS) throw std::invalid_argument("Error: too many particle attributes to gather.\n");
    if (np == 0) return;
    PtrPack pk;
    for (int a = 0; a < nattr; a++) { pk.src[a] = src[a]; pk.dst[a] = dst[a]; }
    k_gather<<<grid_for(np, 256), 256, 0, st>>>(np, sorted_idx, pk, nattr);
}

}  // namespace ffgpu
