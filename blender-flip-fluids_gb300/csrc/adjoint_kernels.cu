// Adjoint (transposed) kernels of one substep, for gradients of a particle-velocity loss
// with respect to the particle velocities at the start of the substep.  With particle
// positions, cell classification, transfer weights and solid weights held fixed, the
// substep v0 -> v1 is affine:
//   v1 = a I(C E2 P (E1 S v0 + g dt)) + b (v0 + I(C E2 P (...)) - I(C E1 S v0))
// (S: P2G, E1/E2: extrapolations, P: pressure projection, C: solid constraint, I: G2P
// sampling, a = PIC ratio, b = 1 - a).  Each kernel below applies the transpose of one of
// those maps; every one is a deterministic gather (no float atomics).  The projection's
// transpose contains A^-1, applied by a second PCG solve on the same symmetric operator
// with the same MIC(0) factor as the forward solve.
#include "common.cuh"
#include "kernels.h"
#include "adjoint.h"

namespace ffgpu {

// ---- G2P^T: per face, gather trilinear weights x dL/dv1 of the particles sampling it ----
__global__ void k_g2p_transpose(Dims d, float dxf, float inv, float hdx, double ddx, int comp,
                                const int *__restrict__ cell_start, const int *__restrict__ sidx,
                                const float *__restrict__ spx, const float *__restrict__ spy,
                                const float *__restrict__ spz, const float *__restrict__ g1, float scale_cur,
                                float scale_saved, float *gcur, float *gsaved) {
    const int fw = d.ni + (comp == 0), fh = d.nj + (comp == 1), fd = d.nk + (comp == 2);
    const size_t nf = (size_t)fw * fh * fd;
    for (size_t f = blockIdx.x * (size_t)blockDim.x + threadIdx.x; f < nf; f += (size_t)gridDim.x * blockDim.x) {
        int fi = (int)(f % fw), fj = (int)((f / fw) % fh), fk = (int)(f / ((size_t)fw * fh));
        int i0 = max(fi - 1, 0), i1 = min(comp == 0 ? fi : fi + 1, d.ni - 1);
        int j0 = max(fj - 1, 0), j1 = min(comp == 1 ? fj : fj + 1, d.nj - 1);
        int k0 = max(fk - 1, 0), k1 = min(comp == 2 ? fk : fk + 1, d.nk - 1);
        float acc = 0.0f;
        for (int ck = k0; ck <= k1; ck++)
            for (int cj = j0; cj <= j1; cj++) {
                size_t base = flat3(0, cj, ck, d.ni, d.nj);
                for (int q = cell_start[base + i0]; q < cell_start[base + i1 + 1]; q++) {
                    float x = spx[q], y = spy[q], z = spz[q];
                    double X = x, Y = y, Z = z;
                    if (!(X >= 0 && Y >= 0 && Z >= 0 && X < ddx * d.ni && Y < ddx * d.nj && Z < ddx * d.nk)) continue;
                    if (comp != 0) x = x - hdx;
                    if (comp != 1) y = y - hdx;
                    if (comp != 2) z = z - hdx;
                    int bi = (int)floorf(x * inv), bj = (int)floorf(y * inv), bk = (int)floorf(z * inv);
                    int di = fi - bi, dj = fj - bj, dk = fk - bk;
                    if (di < 0 || di > 1 || dj < 0 || dj > 1 || dk < 0 || dk > 1) continue;
                    float tx = fmaf(-(float)bi, dxf, x) * inv, ty = fmaf(-(float)bj, dxf, y) * inv,
                          tz = fmaf(-(float)bk, dxf, z) * inv;
                    float wgt = (di ? tx : 1.0f - tx) * (dj ? ty : 1.0f - ty) * (dk ? tz : 1.0f - tz);
                    acc += wgt * g1[sidx[q]];
                }
            }
        gcur[f] = scale_cur * acc;
        gsaved[f] = scale_saved * acc;
    }
}

// ---- extrapolation^T for recorded layer L (reverse order), out of place ----
__device__ inline bool done_at(const unsigned char *valid0, const unsigned char *layer_of, size_t t, int i, int j,
                               int k, int w, int h, int dd, int L) {
    bool border = i == 0 || j == 0 || k == 0 || i == w - 1 || j == h - 1 || k == dd - 1;
    return border || valid0[t] || layer_of[t] < L;
}

__global__ void k_extrap_transpose(int w, int h, int dd, int L, const unsigned char *__restrict__ valid0,
                                   const unsigned char *__restrict__ layer_of, const float *__restrict__ gin,
                                   float *gout) {
    size_t n = (size_t)w * h * dd, sl = (size_t)w * h;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        int i = (int)(t % w), j = (int)((t / w) % h), k = (int)(t / sl);
        if (layer_of[t] == L) { gout[t] = 0.0f; continue; }   // its input value was overwritten
        float v = gin[t];
        if (done_at(valid0, layer_of, t, i, j, k, w, h, dd, L)) {
            const int oi[6] = {1, -1, 0, 0, 0, 0}, oj[6] = {0, 0, 1, -1, 0, 0}, ok[6] = {0, 0, 0, 0, 1, -1};
            for (int q = 0; q < 6; q++) {
                int a = i + oi[q], b = j + oj[q], c = k + ok[q];
                if (a < 0 || b < 0 || c < 0 || a >= w || b >= h || c >= dd) continue;
                size_t u = flat3(a, b, c, w, h);
                if (layer_of[u] != L) continue;
                // u was extrapolated at layer L from its done neighbours (never on the border)
                int cnt = 0;
                for (int r = 0; r < 6; r++) {
                    size_t m = flat3(a + oi[r], b + oj[r], c + ok[r], w, h);
                    if (done_at(valid0, layer_of, m, a + oi[r], b + oj[r], c + ok[r], w, h, dd, L)) cnt++;
                }
                v += gin[u] / (float)cnt;
            }
        }
        gout[t] = v;
    }
}

// ---- projection^T, part 1: faces (pass-through / zero) and the pressure gradient ----
// Face classification exactly as the forward (pressuresolver.cpp:1047-1205).
struct FaceInfo { int active; int untouched; size_t c1, c2; bool f1, f2; double d1, d2; };

__device__ inline FaceInfo face_info(Dims d, int comp, size_t q, const float *phi, const float *wg) {
    FaceInfo fi;
    int fw = d.ni + (comp == 0), fh = d.nj + (comp == 1);
    int i = (int)(q % fw), j = (int)((q / fw) % fh), k = (int)(q / ((size_t)fw * fh));
    int ax = comp == 0 ? i : (comp == 1 ? j : k);
    int na = comp == 0 ? d.ni : (comp == 1 ? d.nj : d.nk);
    fi.active = 0; fi.untouched = 0; fi.c1 = fi.c2 = 0; fi.f1 = fi.f2 = false; fi.d1 = fi.d2 = 0.0;
    if (ax == 0 || ax == na - 1) { fi.untouched = 1; return fi; }
    int i1 = i - (comp == 0), j1 = j - (comp == 1), k1 = k - (comp == 2);
    bool in2 = ax < na;
    fi.c1 = flat3(i1, j1, k1, d.ni, d.nj);
    fi.c2 = in2 ? flat3(i, j, k, d.ni, d.nj) : fi.c1;
    fi.f1 = phi[fi.c1] < 0.0f;
    fi.f2 = in2 && phi[fi.c2] < 0.0f;
    if (!(wg[q] > 0 && (fi.f1 || fi.f2))) return fi;
    fi.active = 1;
    const float eps = 1e-6f;
    // u_p = u_b - factor * (p2~ - p1~);  d(p2~ - p1~)/dp1 -> d1, /dp2 -> d2
    if (fi.f1 && fi.f2) { fi.d1 = -1.0; fi.d2 = 1.0; }
    else if (fi.f1) {
        float phi1 = phi[fi.c1], phi2 = in2 ? phi[fi.c2] : 1.0f;
        float th = phi2 / (phi1 + eps);
        th = (float)fmin(fmax((double)th, -25.0), 25.0);
        fi.d1 = (double)th - 1.0;
    } else {
        float phi1 = phi[fi.c1], phi2 = phi[fi.c2];
        float th = phi1 / (phi2 + eps);
        th = (float)fmin(fmax((double)th, -25.0), 25.0);
        fi.d2 = 1.0 - (double)th;
    }
    return fi;
}

// g_b_in (per face): gradient w.r.t. the field before projection, except the divergence
// term added later; gp (per cell): -G^T g_up on pressure cells.
__global__ void k_proj_faces_transpose(Dims d, int comp, const float *__restrict__ phi, const float *__restrict__ wg,
                                       const float *__restrict__ gup, float *gub) {
    size_t nf = d.faces(comp);
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < nf; q += (size_t)gridDim.x * blockDim.x) {
        FaceInfo fi = face_info(d, comp, q, phi, wg);
        gub[q] = (fi.active || fi.untouched) ? gup[q] : 0.0f;
    }
}

__global__ void k_proj_pressure_grad(Dims d, Bbox bb, double factor, const float *__restrict__ phi,
                                     const float *__restrict__ wu, const float *__restrict__ wv,
                                     const float *__restrict__ ww, const float *__restrict__ gu,
                                     const float *__restrict__ gv, const float *__restrict__ gw,
                                     const unsigned char *__restrict__ fluid, double *gp) {
    int I = bb.i1 - bb.i0 + 1, J = bb.j1 - bb.j0 + 1, K = bb.k1 - bb.k0 + 1;
    size_t n = (size_t)I * J * K;
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        int i = bb.i0 + (int)(t % I), j = bb.j0 + (int)((t / I) % J), k = bb.k0 + (int)(t / ((size_t)I * J));
        size_t c = flat3(i, j, k, d.ni, d.nj);
        if (!fluid[c]) { gp[c] = 0.0; continue; }
        double acc = 0.0;
        // the 6 faces of cell c: lower faces have c as their upper cell (d2), upper faces as lower (d1)
        const float *wgs[3] = {wu, wv, ww};
        const float *gs[3] = {gu, gv, gw};
        for (int comp = 0; comp < 3; comp++) {
            int fw = d.ni + (comp == 0), fh = d.nj + (comp == 1);
            size_t lo = flat3(i, j, k, fw, fh);
            size_t hi = flat3(i + (comp == 0), j + (comp == 1), k + (comp == 2), fw, fh);
            FaceInfo a = face_info(d, comp, lo, phi, wgs[comp]);
            if (a.active) acc += a.d2 * (double)gs[comp][lo];
            FaceInfo b = face_info(d, comp, hi, phi, wgs[comp]);
            if (b.active) acc += b.d1 * (double)gs[comp][hi];
        }
        gp[c] = -factor * acc;
    }
}

// gub += D^T gb: b_c = -(1/dx) (w_r u_r - w_l u_l + ...), on pressure cells
__global__ void k_div_transpose(Dims d, int comp, double inv_dx, const float *__restrict__ wg,
                                const unsigned char *__restrict__ fluid, const double *__restrict__ gb, float *gub) {
    int fw = d.ni + (comp == 0), fh = d.nj + (comp == 1), fd = d.nk + (comp == 2);
    size_t nf = (size_t)fw * fh * fd;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < nf; q += (size_t)gridDim.x * blockDim.x) {
        int i = (int)(q % fw), j = (int)((q / fw) % fh), k = (int)(q / ((size_t)fw * fh));
        int ax = comp == 0 ? i : (comp == 1 ? j : k);
        int na = comp == 0 ? d.ni : (comp == 1 ? d.nj : d.nk);
        double acc = 0.0;
        if (ax > 0) {   // lower cell: this face is its upper (right) face
            size_t c1 = flat3(i - (comp == 0), j - (comp == 1), k - (comp == 2), d.ni, d.nj);
            if (fluid[c1]) acc += -inv_dx * (double)wg[q] * gb[c1];
        }
        if (ax < na) {  // upper cell: this face is its lower (left) face
            size_t c2 = flat3(i, j, k, d.ni, d.nj);
            if (fluid[c2]) acc += inv_dx * (double)wg[q] * gb[c2];
        }
        gub[q] += (float)acc;
    }
}

// ---- P2G^T: per particle, gather w_pf / W_f x g_f over the faces within the kernel radius ----
__global__ void k_p2g_transpose(Dims d, double dx, float r, int comp, int np, const int *__restrict__ sidx,
                                const float *__restrict__ spx, const float *__restrict__ spy,
                                const float *__restrict__ spz, const float *__restrict__ wsum,
                                const float *__restrict__ g, float *gv0) {
    const int CW = 10;
    const int fw = d.ni + (comp == 0), fh = d.nj + (comp == 1), fd = d.nk + (comp == 2);
    const float hdx = (float)(0.5 * dx);
    const float ofx = comp == 0 ? 0.0f : hdx, ofy = comp == 1 ? 0.0f : hdx, ofz = comp == 2 ? 0.0f : hdx;
    const double chunkdx = dx * CW;
    const float rsq = r * r;
    const float coef1 = (4.0f / 9.0f) * (1.0f / (r * r * r * r * r * r));
    const float coef2 = (17.0f / 9.0f) * (1.0f / (r * r * r * r));
    const float coef3 = (22.0f / 9.0f) * (1.0f / (r * r));
    const float eps = 1e-6f;
    const double inv = 1.0 / dx;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < np; q += gridDim.x * blockDim.x) {
        float x = spx[q] - ofx, y = spy[q] - ofy, z = spz[q] - ofz;
        int a0 = (int)floor((x - r) * inv), a1 = (int)floor((x + r) * inv) + 1;
        int b0 = (int)floor((y - r) * inv), b1 = (int)floor((y + r) * inv) + 1;
        int c0 = (int)floor((z - r) * inv), c1 = (int)floor((z + r) * inv) + 1;
        float acc = 0.0f;
        for (int fk = max(c0, 0); fk <= min(c1, fd - 1); fk++)
            for (int fj = max(b0, 0); fj <= min(b1, fh - 1); fj++)
                for (int fi = max(a0, 0); fi <= min(a1, fw - 1); fi++) {
                    int A = fi / CW, B = fj / CW, C = fk / CW;
                    float bx = (float)((double)(float)A * chunkdx), by = (float)((double)(float)B * chunkdx),
                          bz = (float)((double)(float)C * chunkdx);
                    float gx = (float)((double)(float)(fi - CW * A) * dx), gy = (float)((double)(float)(fj - CW * B) * dx),
                          gz = (float)((double)(float)(fk - CW * C) * dx);
                    float vx = gx - (x - bx), vy = gy - (y - by), vz = gz - (z - bz);
                    float d2 = vx * vx + vy * vy + vz * vz;
                    if (!(d2 < rsq)) continue;
                    float wgt = 1.0f - coef1 * d2 * d2 * d2 + coef2 * d2 * d2 - coef3 * d2;
                    size_t f = flat3(fi, fj, fk, fw, fh);
                    float W = wsum[f];
                    acc += (W > eps ? wgt / W : wgt) * g[f];
                }
        gv0[sidx[q]] += acc;
    }
}

// ---- loss: L = mean over particles with y > ymin of vy^2; writes dL/dv1 (SoA) ----
__global__ void k_loss_grad_vy2(int np, double ymin, const float *__restrict__ py, const float *__restrict__ vy,
                                float inv_count, float *gx, float *gy, float *gz) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
        gx[p] = 0.0f; gz[p] = 0.0f;
        gy[p] = (double)py[p] > ymin ? 2.0f * vy[p] * inv_count : 0.0f;
    }
}

__global__ void k_count_above(int np, double ymin, const float *__restrict__ py, int *count) {
    int c = 0;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) c += (double)py[p] > ymin;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(count, c);
}

__global__ void k_scale_add(size_t n, const float *__restrict__ a, float s, float *out) {
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
        out[t] = s * a[t];
}

__global__ void k_add_inplace(size_t n, const float *__restrict__ a, float *out) {
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
        out[t] += a[t];
}

// ---- launchers ----
void adj_g2p_transpose(Dims d, double dx, int comp, const int *cell_start, const int *sidx, const float *spx,
                       const float *spy, const float *spz, const float *g1, float scale_cur, float scale_saved,
                       float *gcur, float *gsaved, cudaStream_t st) {
    size_t nf = d.faces(comp);
    k_g2p_transpose<<<grid_for(nf, 256, 152u * 64u), 256, 0, st>>>(d, (float)dx, (float)(1.0 / dx), (float)(0.5 * dx),
                                                                   dx, comp, cell_start, sidx, spx, spy, spz, g1,
                                                                   scale_cur, scale_saved, gcur, gsaved);
}

void adj_extrapolate_transpose(int w, int h, int dd, int layers, const unsigned char *valid0,
                               const unsigned char *layer_of, float *g, float *tmp, cudaStream_t st) {
    size_t n = (size_t)w * h * dd;
    unsigned int grid = grid_for(n, 256, 152u * 32u);
    float *a = g, *b = tmp;
    for (int L = layers - 1; L >= 0; L--) {
        k_extrap_transpose<<<grid, 256, 0, st>>>(w, h, dd, L, valid0, layer_of, a, b);
        float *t = a; a = b; b = t;
    }
    if (a != g) FFGPU_CUDA(cudaMemcpyAsync(g, a, n * 4, cudaMemcpyDeviceToDevice, st));
}

void adj_projection_faces(Dims d, int comp, const float *phi, const float *wg, const float *gup, float *gub,
                          cudaStream_t st) {
    size_t nf = d.faces(comp);
    k_proj_faces_transpose<<<grid_for(nf, 256), 256, 0, st>>>(d, comp, phi, wg, gup, gub);
}

void adj_pressure_grad(Dims d, Bbox bb, double dx, double dt, const float *phi, const float *wu, const float *wv,
                       const float *ww, const float *gu, const float *gv, const float *gw, const unsigned char *fluid,
                       double *gp, cudaStream_t st) {
    size_t n = (size_t)(bb.i1 - bb.i0 + 1) * (bb.j1 - bb.j0 + 1) * (bb.k1 - bb.k0 + 1);
    k_proj_pressure_grad<<<grid_for(n, 256), 256, 0, st>>>(d, bb, (double)(float)(dt / dx), phi, wu, wv, ww, gu, gv,
                                                           gw, fluid, gp);
}

void adj_div_transpose(Dims d, int comp, double dx, const float *wg, const unsigned char *fluid, const double *gb,
                       float *gub, cudaStream_t st) {
    size_t nf = d.faces(comp);
    k_div_transpose<<<grid_for(nf, 256), 256, 0, st>>>(d, comp, 1.0 / dx, wg, fluid, gb, gub);
}

void adj_p2g_transpose(Dims d, double dx, double radius, int comp, int np, const int *sidx, const float *spx,
                       const float *spy, const float *spz, const float *wsum, const float *g, float *gv0,
                       cudaStream_t st) {
    if (np == 0) return;
    k_p2g_transpose<<<grid_for(np, 256), 256, 0, st>>>(d, dx, (float)radius, comp, np, sidx, spx, spy, spz, wsum, g,
                                                       gv0);
}

int adj_loss_grad_vy2(int np, double ymin, const float *py, const float *vy, float *gx, float *gy, float *gz,
                      int *count_dev, int *count_host, cudaStream_t st) {
    FFGPU_CUDA(cudaMemsetAsync(count_dev, 0, sizeof(int), st));
    if (np) k_count_above<<<grid_for(np, 256), 256, 0, st>>>(np, ymin, py, count_dev);
    FFGPU_CUDA(cudaMemcpyAsync(count_host, count_dev, sizeof(int), cudaMemcpyDeviceToHost, st));
    FFGPU_CUDA(cudaStreamSynchronize(st));
    int m = *count_host;
    if (np) k_loss_grad_vy2<<<grid_for(np, 256), 256, 0, st>>>(np, ymin, py, vy, m > 0 ? 1.0f / (float)m : 0.0f, gx, gy, gz);
    return m;
}

void adj_scale(size_t n, const float *a, float s, float *out, cudaStream_t st) {
    k_scale_add<<<grid_for(n, 256), 256, 0, st>>>(n, a, s, out);
}

void adj_add(size_t n, const float *a, float *out, cudaStream_t st) {
    k_add_inplace<<<grid_for(n, 256), 256, 0, st>>>(n, a, out);
}

}  // namespace ffgpu
