// FFP3 fluid-particle output of the marker particles, on the GPU:
//   FluidSimulation::_classifyFluidParticleTypesThread (fluidsimulation.cpp:9511-9552): boundary
//     particles in the cells within 2 + boundary width cells of a grid side, else surface where the
//     surface level set sampled at p - dx/2 is >= -surface width dx, else interior (a NaN sample
//     leaves the particle out);
//   FluidSimulation::_generateFluidParticleDataFFP3 (fluidsimulation.cpp:9554-9676): particles with
//     id < id limit and an enabled type grouped by type (surface, boundary, interior), then id, then
//     particle order; per type and id the header holds the end of the id's run within the type;
//   FluidSimulation::_generateFluidParticleFFP3FileData (fluidsimulation.h:2036-2068): 4 uint32
//     (the three type counts and the id limit), 3 uint32 per id, then the grouped records.
// The grouping is a stable sort of the particles by key = type * id limit + id: the particles with
// a key are compacted in order, then two stable counting-sort passes on 9-bit digits (keys stay
// below 2^18); each pass splits the list into chunks, one warp per chunk counts and later places
// its chunk's elements in order.  The records are then gathered in sorted order.
#include <climits>
#include <cstdint>
#include <stdexcept>

#include "common.cuh"
#include "ffp3.h"
#include "kernels.h"
#include "tension.cuh"

namespace ffgpu {
namespace {

constexpr int RADIX_BITS = 9, RADIX = 1 << RADIX_BITS;
constexpr int CHUNK = 2048;          // elements per warp in a counting-sort pass
constexpr int SORT_WARPS = 4;        // warps per block (each owns RADIX counters in shared memory)

// type and key of every particle: 0 surface, 1 boundary, 2 interior, 3 unset; key -1 when the
// particle is not written (unset, its type's output off, or id >= id limit)
// The surface test (float)sample_centred(surface, ...) >= c, c = -surface width: 0 surface, 2 interior,
// 3 neither (a NaN sample).  The trilinear sample is first formed in float; its distance from the
// double one stays below 3e-5 of the largest corner (weights off by at most ~1e-6 each, eight terms),
// so whenever the float sample clears c by that bound plus a 2^-20 relative margin (more than the
// final rounding to float) the double evaluation gives the same answer and is skipped.
__device__ inline int surface_side(const float *__restrict__ g, Dims d, double dx, float px, float py, float pz,
                                   float c) {
    const float sh = (float)(0.5 * dx);
    const float x = px - sh, y = py - sh, z = pz - sh;
    const double inv = 1.0 / dx;
    const float invf = (float)inv;
    const int i = floor_fd(x, inv, invf), j = floor_fd(y, inv, invf), k = floor_fd(z, inv, invf);
    const float gx = (float)((double)(float)i * dx), gy = (float)((double)(float)j * dx), gz = (float)((double)(float)k * dx);
    const float ix = (x - gx) * invf, iy = (y - gy) * invf, iz = (z - gz) * invf;
    auto G = [&](int a, int b, int e) -> float {
        return (a >= 0 && b >= 0 && e >= 0 && a < d.ni && b < d.nj && e < d.nk) ? g[flat3(a, b, e, d.ni, d.nj)] : 0.0f;
    };
    const float p0 = G(i, j, k), p1 = G(i + 1, j, k), p2 = G(i, j + 1, k), p3 = G(i, j, k + 1), p4 = G(i + 1, j, k + 1),
                p5 = G(i, j + 1, k + 1), p6 = G(i + 1, j + 1, k), p7 = G(i + 1, j + 1, k + 1);
    const float ux = 1.0f - ix, uy = 1.0f - iy, uz = 1.0f - iz;
    const float s = p0 * ux * uy * uz + p1 * ix * uy * uz + p2 * ux * iy * uz + p3 * ux * uy * iz + p4 * ix * uy * iz +
                    p5 * ux * iy * iz + p6 * ix * iy * uz + p7 * ix * iy * iz;
    const float mx = fmaxf(fmaxf(fmaxf(fabsf(p0), fabsf(p1)), fmaxf(fabsf(p2), fabsf(p3))),
                           fmaxf(fmaxf(fabsf(p4), fabsf(p5)), fmaxf(fabsf(p6), fabsf(p7))));
    const float bound = 3e-5f * mx + 1e-30f, margin = fabsf(c) * 9.6e-7f + 1e-30f;
    if (s - bound >= c + margin) return 0;
    if (s + bound < c - margin) return 2;
    const float e = (float)sample_centred(g, d, dx, px, py, pz);   // the reference's double arithmetic
    return e >= c ? 0 : (e < c ? 2 : 3);
}

__global__ void k_ffp3_classify(Dims d, double dx, int bw, float sw, const float *__restrict__ surface, int np,
                                const float *__restrict__ px, const float *__restrict__ py,
                                const float *__restrict__ pz, const unsigned int *__restrict__ ids, int id_limit,
                                int enabled, unsigned char *type, int *key, int *flag) {
    const double inv = 1.0 / dx;
    const float invf = (float)inv;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        const float x = px[p], y = py[p], z = pz[p];
        const int i = floor_fd(x, inv, invf), j = floor_fd(y, inv, invf), k = floor_fd(z, inv, invf);
        const bool in = i >= 0 && j >= 0 && k >= 0 && i < d.ni && j < d.nj && k < d.nk;
        const bool inner = i >= bw && j >= bw && k >= bw && i < d.ni - bw && j < d.nj - bw && k < d.nk - bw;
        int t;
        if (in && !inner) {
            t = 1;
        } else {
            t = surface_side(surface, d, dx, x, y, z, -sw);
        }
        type[p] = (unsigned char)t;
        const int id = (int)ids[p];
        const int kk = (t < 3 && ((enabled >> t) & 1) && id < id_limit) ? t * id_limit + id : -1;
        key[p] = kk;
        flag[p] = kk >= 0 ? 1 : 0;
    }
}

// key_start[k] = the first sorted position of key k (entries were INT_MAX); a key that does not occur
// keeps INT_MAX until the suffix minimum below gives it the next key's start
__global__ void k_ffp3_run_starts(int total, int nkeys, const int *__restrict__ skey, int *key_start) {
    if (blockIdx.x == 0 && threadIdx.x == 0) key_start[nkeys] = total;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += gridDim.x * blockDim.x) {
        const int k = skey[q];
        if (q == 0 || skey[q - 1] != k) key_start[k] = q;
    }
}

// a[q] = min(a[q], a[q + 1], ..., a[n - 1]), one block: chunk minima, their suffix minima, then each chunk
__global__ void __launch_bounds__(1024) k_suffix_min(int n, int *a) {
    __shared__ int cm[1024];
    const int t = threadIdx.x, C = (n + 1023) / 1024;
    const int lo = min(n, t * C), hi = min(n, lo + C);
    int m = INT_MAX;
    for (int q = hi - 1; q >= lo; q--) m = min(m, a[q]);
    cm[t] = m;
    __syncthreads();
    if (t == 0) {
        int r = INT_MAX;
        for (int u = 1023; u >= 0; u--) { r = min(r, cm[u]); cm[u] = r; }
    }
    __syncthreads();
    int carry = t + 1 < 1024 ? cm[t + 1] : INT_MAX;
    for (int q = hi - 1; q >= lo; q--) { carry = min(carry, a[q]); a[q] = carry; }
}

// the particles with a key, in order: (key, particle)
__global__ void k_ffp3_compact(int np, const int *__restrict__ key, const int *__restrict__ off, int *okey, int *oidx) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        const int k = key[p];
        if (k >= 0) {
            okey[off[p]] = k;
            oidx[off[p]] = p;
        }
    }
}

// counting-sort pass, step 1: per chunk, the count of each digit (counts[digit * nchunks + chunk])
__global__ void __launch_bounds__(32 * SORT_WARPS) k_radix_count(int n, int nchunks, int shift,
                                                                 const int *__restrict__ key, int *counts) {
    __shared__ int h[SORT_WARPS][RADIX];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int chunk = blockIdx.x * SORT_WARPS + w;
    for (int b = lane; b < RADIX; b += 32) h[w][b] = 0;
    __syncwarp();
    if (chunk < nchunks) {
        const int a = chunk * CHUNK, e = min(n, a + CHUNK);
        for (int q = a + lane; q < e; q += 32) atomicAdd(&h[w][(key[q] >> shift) & (RADIX - 1)], 1);
        __syncwarp();
        for (int b = lane; b < RADIX; b += 32) counts[(size_t)b * nchunks + chunk] = h[w][b];
    }
}

// step 3 (after the exclusive scan of the counts): each chunk's elements placed in order
__global__ void __launch_bounds__(32 * SORT_WARPS) k_radix_scatter(int n, int nchunks, int shift,
                                                                   const int *__restrict__ key,
                                                                   const int *__restrict__ idx,
                                                                   const int *__restrict__ offsets, int *okey,
                                                                   int *oidx) {
    __shared__ int cur[SORT_WARPS][RADIX];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int chunk = blockIdx.x * SORT_WARPS + w;
    if (chunk >= nchunks) return;   // warp-uniform; no block barrier follows
    for (int b = lane; b < RADIX; b += 32) cur[w][b] = offsets[(size_t)b * nchunks + chunk];
    __syncwarp();
    const int a = chunk * CHUNK, e = min(n, a + CHUNK);
    const unsigned lt = (1u << lane) - 1u;
    for (int q0 = a; q0 < e; q0 += 32) {
        const int q = q0 + lane;
        const bool live = q < e;
        const int k = live ? key[q] : -1;
        const int dg = live ? (k >> shift) & (RADIX - 1) : RADIX;   // RADIX: no digit
        const unsigned same = __match_any_sync(0xffffffffu, dg);
        const int leader = __ffs(same) - 1;
        int base = 0;
        if (live && lane == leader) {
            base = cur[w][dg];
            cur[w][dg] = base + __popc(same);
        }
        base = __shfl_sync(0xffffffffu, base, leader);
        __syncwarp();
        if (live) {
            const int at = base + __popc(same & lt);
            okey[at] = k;
            oidx[at] = idx[q];
        }
    }
}

// header: per id (3 uint32: the run ends within the surface, boundary, interior groups), after the
// 4 leading uint32 (the type counts and the id limit)
__global__ void k_ffp3_header(int id_limit, const int *__restrict__ key_start, unsigned int *head) {
    const int total = key_start[3 * id_limit];
    const int off[3] = {key_start[0], key_start[id_limit], key_start[2 * id_limit]};
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        head[0] = (unsigned int)(off[1] - off[0]);
        head[1] = (unsigned int)(off[2] - off[1]);
        head[2] = (unsigned int)(total - off[2]);
        head[3] = (unsigned int)id_limit;
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < id_limit; i += gridDim.x * blockDim.x)
        for (int t = 0; t < 3; t++) head[4 + 3 * (size_t)i + t] = (unsigned int)(key_start[t * id_limit + i + 1] - off[t]);
}

// the records in sorted order: positions and velocities (xyz float), speeds, ids (uint16)
__global__ void k_ffp3_records(int total, const int *__restrict__ sidx, const float *__restrict__ px,
                               const float *__restrict__ py, const float *__restrict__ pz, const float *__restrict__ vx,
                               const float *__restrict__ vy, const float *__restrict__ vz,
                               const unsigned int *__restrict__ ids, float *pos, uint16_t *id, float *vel, float *speed) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += gridDim.x * blockDim.x) {
        const int p = sidx[q];
        pos[3 * (size_t)q] = px[p]; pos[3 * (size_t)q + 1] = py[p]; pos[3 * (size_t)q + 2] = pz[p];
        id[q] = (uint16_t)ids[p];
        const float a = vx[p], b = vy[p], c = vz[p];
        if (vel) { vel[3 * (size_t)q] = a; vel[3 * (size_t)q + 1] = b; vel[3 * (size_t)q + 2] = c; }
        if (speed) speed[q] = sqrtf(a * a + b * b + c * c);   // vmath::vec3::length
    }
}

}  // namespace

Ffp3Counts launch_ffp3(Dims d, double dx, const float *surface, int np, const float *px, const float *py,
                       const float *pz, const float *vx, const float *vy, const float *vz, const unsigned int *ids,
                       const Ffp3Params &prm, Ffp3Work &w, cudaStream_t st, unsigned long long &launches) {
    const int L = prm.id_limit;
    if (L < 0 || L > 65536) throw std::domain_error("Error: fluid particle id limit out of range.\n");
    const int nkeys = 3 * L;
    w.type.reserve((size_t)std::max(np, 1));
    w.key.reserve((size_t)std::max(np, 1));
    w.flag.reserve((size_t)np + 1);
    w.off.reserve((size_t)np + 1);
    w.keys[0].reserve((size_t)std::max(np, 1)); w.keys[1].reserve((size_t)std::max(np, 1));
    w.idx[0].reserve((size_t)std::max(np, 1)); w.idx[1].reserve((size_t)std::max(np, 1));
    w.key_start.reserve((size_t)nkeys + 1);
    const size_t nmax = std::max((size_t)np + 1, (size_t)nkeys + 1);
    const int nchunks_max = std::max(1, (np + CHUNK - 1) / CHUNK);
    w.counts.reserve((size_t)RADIX * nchunks_max + 1);
    w.coff.reserve((size_t)RADIX * nchunks_max + 1);
    w.scan_tmp.reserve(scan_scratch_ints(std::max(nmax, (size_t)RADIX * nchunks_max + 1)) + 64);
    const float sw = (float)(prm.surface_width_cells * dx);
    if (np > 0)
        k_ffp3_classify<<<grid_for(np, 256), 256, 0, st>>>(d, dx, 2 + prm.boundary_width, sw, surface, np, px, py, pz,
                                                           ids, L, prm.enabled, w.type, w.key, w.flag);
    launch_exclusive_scan(w.flag, w.off, (size_t)np, w.scan_tmp, st);
    int total = 0;
    FFGPU_CUDA(cudaMemcpyAsync(&total, w.off.p + np, sizeof(int), cudaMemcpyDeviceToHost, st));
    FFGPU_CUDA(cudaStreamSynchronize(st));
    launches += 3;
    // stable sort of the keyed particles by key (two 9-bit digits; keys < 3 * 65536 < 2^18)
    int cur = 0;
    if (total > 0) {
        k_ffp3_compact<<<grid_for(np, 256), 256, 0, st>>>(np, w.key, w.off, w.keys[0], w.idx[0]);
        launches++;
        const int nchunks = (total + CHUNK - 1) / CHUNK;
        const unsigned blocks = (unsigned)((nchunks + SORT_WARPS - 1) / SORT_WARPS);
        for (int pass = 0; pass < 2; pass++) {
            const int shift = pass * RADIX_BITS;
            k_radix_count<<<blocks, 32 * SORT_WARPS, 0, st>>>(total, nchunks, shift, w.keys[cur], w.counts);
            launch_exclusive_scan(w.counts, w.coff, (size_t)RADIX * nchunks, w.scan_tmp, st);
            k_radix_scatter<<<blocks, 32 * SORT_WARPS, 0, st>>>(total, nchunks, shift, w.keys[cur], w.idx[cur], w.coff,
                                                                 w.keys[1 - cur], w.idx[1 - cur]);
            cur = 1 - cur;
            launches += 3;
        }
    }
    // each key's first sorted position (the exclusive scan of the key counts): run starts, the end
    // (key 3L) at total, then the suffix minimum fills the keys that do not occur
    FFGPU_CUDA(cudaMemsetAsync(w.key_start.p, 0x7f, (size_t)nkeys * sizeof(int), st));   // 0x7f7f7f7f: above any start
    k_ffp3_run_starts<<<grid_for((size_t)std::max(total, 1), 256), 256, 0, st>>>(total, nkeys, w.keys[cur], w.key_start);
    k_suffix_min<<<1, 1024, 0, st>>>(nkeys + 1, w.key_start);
    launches += 2;
    const size_t head = (4 + 3 * (size_t)L) * sizeof(unsigned int);
    Ffp3Counts c;
    c.total = total;
    c.bytes[0] = head + 12 * (size_t)total;
    c.bytes[1] = head + 2 * (size_t)total;
    c.bytes[2] = prm.velocity ? head + 12 * (size_t)total : 0;
    c.bytes[3] = prm.speed ? head + 4 * (size_t)total : 0;
    for (int a = 0; a < 4; a++) w.out[a].reserve(std::max<size_t>(c.bytes[a], 16));
    unsigned int *h0 = reinterpret_cast<unsigned int *>(w.out[0].p);
    k_ffp3_header<<<grid_for((size_t)std::max(L, 1), 256), 256, 0, st>>>(L, w.key_start, h0);
    for (int a = 1; a < 4; a++)
        if (c.bytes[a]) FFGPU_CUDA(cudaMemcpyAsync(w.out[a].p, h0, head, cudaMemcpyDeviceToDevice, st));
    launches++;
    if (total > 0) {
        float *pos = reinterpret_cast<float *>(w.out[0].p + head);
        uint16_t *id = reinterpret_cast<uint16_t *>(w.out[1].p + head);
        float *vel = prm.velocity ? reinterpret_cast<float *>(w.out[2].p + head) : nullptr;
        float *speed = prm.speed ? reinterpret_cast<float *>(w.out[3].p + head) : nullptr;
        k_ffp3_records<<<grid_for(total, 256), 256, 0, st>>>(total, w.idx[cur], px, py, pz, vx, vy, vz, ids, pos, id,
                                                             vel, speed);
        launches++;
    }
    unsigned int h[3] = {0, 0, 0};
    FFGPU_CUDA(cudaMemcpyAsync(h, h0, sizeof(h), cudaMemcpyDeviceToHost, st));
    FFGPU_CUDA(cudaStreamSynchronize(st));
    c.surface = (int)h[0]; c.boundary = (int)h[1]; c.interior = (int)h[2];
    return c;
}

}  // namespace ffgpu
