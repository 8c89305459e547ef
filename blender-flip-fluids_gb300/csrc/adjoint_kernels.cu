// Adjoint (transposed) kernels of one substep, for gradients of a loss on the particle
// state (x1, v1) after the substep with respect to the state (x0, v0) before it.  The
// discrete structure is held fixed at the recorded forward pass: liquid level set and cell
// classification, valid flags, extrapolation layers, solid weights, the cells the sample
// points fall in, and which particles the collision handling moved.  With it fixed,
//   ue = E1 S(x0) v0,  uc = C E2 P (ue + g dt),  us = C ue
//   v1 = a I(x0) uc + b (v0 + I(x0) uc - I(x0) us)
//   x1 = x0 + h3 (2 k1 + 3 k2 + 4 k3),  k1 = uc(x0), k2 = uc(x0 + h1 k1), k3 = uc(x0 + h2 k2)
// (S: P2G, E1/E2: extrapolations, P: pressure projection, C: solid constraint, I: G2P
// sampling, a = PIC ratio, b = 1 - a).  The map is affine in v0 and smooth in x0 inside
// the fixed structure.  Each kernel below applies the transpose of one piece; every one is a
// deterministic gather (no float atomics).  The projection's transpose contains A^-1,
// applied by a second PCG solve on the same symmetric operator with the same MIC(0) factor
// as the forward solve.
#include <algorithm>

#include "common.cuh"
#include "kernels.h"
#include "mac_sample.cuh"
#include "adjoint.h"

namespace ffgpu {

// ---- RK3 advection^T and the position part of G2P^T, per particle (cell-sorted order q) ----
// Forward (k_advect, k_g2p): k1 = u(x), p2 = x + h1 k1, k2 = u(p2), p3 = x + h2 k2,
// k3 = u(p3), x' = x + h3 (2 k1 + 3 k2 + 4 k3); v' = a u(x) + b (v + u(x) - s(x)).
// From gx' (may be null: zero) and gv' (particle order) this writes
//   gx = gx' + J(x)^T (gk1 + (a+b) gv') + J(p2)^T gk2 + J(p3)^T gk3 - b Js(x)^T gv'
// in particle order, with gk3 = 4 h3 gx', gk2 = 3 h3 gx' + h2 J(p3)^T gk3,
// gk1 = 2 h3 gx' + h1 J(p2)^T gk2; and, in sorted order, the weights of the transposed
// sampling at x (wc = gk1 + (a+b) gv' on the current field, ws = -b gv' on the saved field)
// and the stage points p2, p3 with their weights gk2, gk3 (pt2/pt3: x, y, z, gx, gy, gz).
// A particle whose position the collision handling changed passes gx' through unchanged
// and nothing into the field (gk1 = gk2 = gk3 = 0).
__global__ void k_advect_transpose(MacDev cur, MacDev sav, float a, float b, float h1, float h2, float h3, int np,
                                   size_t cap, const int *__restrict__ sidx, const float *__restrict__ spx,
                                   const float *__restrict__ spy, const float *__restrict__ spz,
                                   const float *__restrict__ gx1, const float *__restrict__ gy1,
                                   const float *__restrict__ gz1, const float *__restrict__ gvx,
                                   const float *__restrict__ gvy, const float *__restrict__ gvz,
                                   const unsigned char *__restrict__ collided, float *gx0, float *gy0, float *gz0,
                                   float *wc, float *ws, float *pt2, float *pt3) {
    const float ab = a + b;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < np; q += gridDim.x * blockDim.x) {
        const int p = sidx[q];
        const float x = spx[q], y = spy[q], z = spz[q];
        const float vx = gvx[p], vy = gvy[p], vz = gvz[p];
        float ox = 0.0f, oy = 0.0f, oz = 0.0f;
        if (gx1) { ox = gx1[p]; oy = gy1[p]; oz = gz1[p]; }
        const bool moving = !collided[p] && (ox != 0.0f || oy != 0.0f || oz != 0.0f);
        // stage points exactly as the forward computes them
        float k1x, k1y, k1z, k2x, k2y, k2z;
        sample_mac(cur, x, y, z, k1x, k1y, k1z);
        const float p2x = x + h1 * k1x, p2y = y + h1 * k1y, p2z = z + h1 * k1z;
        sample_mac(cur, p2x, p2y, p2z, k2x, k2y, k2z);
        const float p3x = x + h2 * k2x, p3y = y + h2 * k2y, p3z = z + h2 * k2z;
        float k3gx = 0.0f, k3gy = 0.0f, k3gz = 0.0f, k2gx = 0.0f, k2gy = 0.0f, k2gz = 0.0f;
        float k1gx = 0.0f, k1gy = 0.0f, k1gz = 0.0f;
        float j3x = 0.0f, j3y = 0.0f, j3z = 0.0f, j2x = 0.0f, j2y = 0.0f, j2z = 0.0f;
        if (moving) {
            const float c3 = 4.0f * h3, c2 = 3.0f * h3, c1 = 2.0f * h3;
            k3gx = c3 * ox; k3gy = c3 * oy; k3gz = c3 * oz;
            sample_mac_jt(cur, p3x, p3y, p3z, k3gx, k3gy, k3gz, j3x, j3y, j3z);
            k2gx = c2 * ox + h2 * j3x; k2gy = c2 * oy + h2 * j3y; k2gz = c2 * oz + h2 * j3z;
            sample_mac_jt(cur, p2x, p2y, p2z, k2gx, k2gy, k2gz, j2x, j2y, j2z);
            k1gx = c1 * ox + h1 * j2x; k1gy = c1 * oy + h1 * j2y; k1gz = c1 * oz + h1 * j2z;
        }
        const float wcx = k1gx + ab * vx, wcy = k1gy + ab * vy, wcz = k1gz + ab * vz;
        float j1x, j1y, j1z, jsx, jsy, jsz;
        sample_mac_jt(cur, x, y, z, wcx, wcy, wcz, j1x, j1y, j1z);
        sample_mac_jt(sav, x, y, z, -b * vx, -b * vy, -b * vz, jsx, jsy, jsz);
        gx0[p] = ox + j1x + j2x + j3x + jsx;
        gy0[p] = oy + j1y + j2y + j3y + jsy;
        gz0[p] = oz + j1z + j2z + j3z + jsz;
        // a point outside the grid samples zero: its transposed-sampling weights are zero
        const float in1 = mac_inside(cur, x, y, z) ? 1.0f : 0.0f;
        const float in2 = mac_inside(cur, p2x, p2y, p2z) ? 1.0f : 0.0f;
        const float in3 = mac_inside(cur, p3x, p3y, p3z) ? 1.0f : 0.0f;
        wc[q] = in1 * wcx; wc[cap + q] = in1 * wcy; wc[2 * cap + q] = in1 * wcz;
        ws[q] = in1 * (-b * vx); ws[cap + q] = in1 * (-b * vy); ws[2 * cap + q] = in1 * (-b * vz);
        pt2[q] = p2x; pt2[cap + q] = p2y; pt2[2 * cap + q] = p2z;
        pt2[3 * cap + q] = in2 * k2gx; pt2[4 * cap + q] = in2 * k2gy; pt2[5 * cap + q] = in2 * k2gz;
        pt3[q] = p3x; pt3[cap + q] = p3y; pt3[2 * cap + q] = p3z;
        pt3[3 * cap + q] = in3 * k3gx; pt3[4 * cap + q] = in3 * k3gy; pt3[5 * cap + q] = in3 * k3gz;
    }
}

// ---- transposed MAC sampling: per face, gather trilinear weight x per-point weight over the
// cell-sorted points that sample it (G2P^T and the RK3 stages).  Points outside the grid carry
// zero weights.  Points keyed by the float floor the sampling uses (widen = 0) lie in the
// face's two base cells along its own axis; points keyed by the double-precision floor of the
// particle sort (widen = 1) can differ from the sampling's float floor by one cell at a cell
// boundary, so that axis scans one more cell on each side. ----
__global__ void k_sample_transpose(Dims d, float dxf, float inv, float hdx, int comp, GridDecode dec, int widen,
                                   const int *__restrict__ cell_start, const float *__restrict__ qx,
                                   const float *__restrict__ qy, const float *__restrict__ qz,
                                   const float *__restrict__ wa, const float *__restrict__ wb, float *ga, float *gb,
                                   int accumulate) {
    const unsigned int nf = (unsigned int)d.faces(comp);
    for (unsigned int f = blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += gridDim.x * blockDim.x) {
        int fi, fj, fk;
        dec(f, fi, fj, fk);
        int i0 = max(fi - 1 - (comp == 0 ? widen : 0), 0), i1 = min(fi + (comp == 0 ? widen : 1), d.ni - 1);
        int j0 = max(fj - 1 - (comp == 1 ? widen : 0), 0), j1 = min(fj + (comp == 1 ? widen : 1), d.nj - 1);
        int k0 = max(fk - 1 - (comp == 2 ? widen : 0), 0), k1 = min(fk + (comp == 2 ? widen : 1), d.nk - 1);
        float acc = 0.0f, accb = 0.0f;
        for (int ck = k0; ck <= k1; ck++)
            for (int cj = j0; cj <= j1; cj++) {
                size_t base = flat3(0, cj, ck, d.ni, d.nj);
                for (int q = cell_start[base + i0]; q < cell_start[base + i1 + 1]; q++) {
                    float x = qx[q], y = qy[q], z = qz[q];
                    if (comp != 0) x = x - hdx;
                    if (comp != 1) y = y - hdx;
                    if (comp != 2) z = z - hdx;
                    int bi = (int)floorf(x * inv), bj = (int)floorf(y * inv), bk = (int)floorf(z * inv);
                    int di = fi - bi, dj = fj - bj, dk = fk - bk;
                    if (di < 0 || di > 1 || dj < 0 || dj > 1 || dk < 0 || dk > 1) continue;
                    float tx = fmaf(-(float)bi, dxf, x) * inv, ty = fmaf(-(float)bj, dxf, y) * inv,
                          tz = fmaf(-(float)bk, dxf, z) * inv;
                    float wgt = (di ? tx : 1.0f - tx) * (dj ? ty : 1.0f - ty) * (dk ? tz : 1.0f - tz);
                    acc += wgt * wa[q];
                    if (wb) accb += wgt * wb[q];
                }
            }
        if (accumulate) ga[f] += acc;
        else ga[f] = acc;
        if (wb) gb[f] = accb;
    }
}

// ---- extrapolation^T for recorded layer L (reverse order), out of place ----
// layer_of holds the forward's record per face: layer (low 5 bits, layers <= 31) and the
// number of done neighbours the value was averaged over minus one (high 3 bits); 0xFF = not
// extrapolated.  A face extrapolated at layer L hands g / count to each neighbour that was
// done at L (border, valid, or extrapolated at an earlier layer) and keeps nothing itself.
__global__ void k_extrap_transpose(int w, int h, int dd, GridDecode dec, int L, const unsigned char *__restrict__ valid0,
                                   const unsigned char *__restrict__ layer_of, const float *__restrict__ gin,
                                   float *gout) {
    const unsigned int n = (unsigned int)w * h * dd;
    const size_t sl = (size_t)w * h;
    for (unsigned int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const unsigned char rec = layer_of[t];
        if ((rec & 31) == L) { gout[t] = 0.0f; continue; }   // its input value was overwritten
        float v = gin[t];
        int i, j, k;
        dec(t, i, j, k);
        const bool border = i == 0 || j == 0 || k == 0 || i == w - 1 || j == h - 1 || k == dd - 1;
        if (border || valid0[t] || (rec & 31) < L) {
            const bool has[6] = {i + 1 < w, i > 0, j + 1 < h, j > 0, k + 1 < dd, k > 0};
            const long long off[6] = {1, -1, w, -(long long)w, (long long)sl, -(long long)sl};
            for (int q = 0; q < 6; q++) {
                if (!has[q]) continue;
                const size_t u = (size_t)((long long)t + off[q]);
                const unsigned char ru = layer_of[u];
                if ((ru & 31) == L) v += gin[u] / (float)((ru >> 5) + 1);
            }
        }
        gout[t] = v;
    }
}

// ---- projection^T, part 1: faces (pass-through / zero) and the pressure gradient ----
// Face classification exactly as the forward (pressuresolver.cpp:1047-1205).
struct FaceInfo { int active; int untouched; size_t c1, c2; bool f1, f2; double d1, d2; };

__device__ inline FaceInfo face_info(Dims d, int comp, int i, int j, int k, size_t q, const float *phi,
                                     const float *wg) {
    FaceInfo fi;
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
__global__ void k_proj_faces_transpose(Dims d, int comp, GridDecode dec, const float *__restrict__ phi,
                                       const float *__restrict__ wg, const float *__restrict__ gup, float *gub) {
    const unsigned int nf = (unsigned int)d.faces(comp);
    for (unsigned int q = blockIdx.x * blockDim.x + threadIdx.x; q < nf; q += gridDim.x * blockDim.x) {
        int i, j, k;
        dec(q, i, j, k);
        FaceInfo fi = face_info(d, comp, i, j, k, q, phi, wg);
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
            FaceInfo a = face_info(d, comp, i, j, k, lo, phi, wgs[comp]);
            if (a.active) acc += a.d2 * (double)gs[comp][lo];
            FaceInfo b = face_info(d, comp, i + (comp == 0), j + (comp == 1), k + (comp == 2), hi, phi, wgs[comp]);
            if (b.active) acc += b.d1 * (double)gs[comp][hi];
        }
        gp[c] = -factor * acc;
    }
}

// gub += D^T gb: b_c = -(1/dx) (w_r u_r - w_l u_l + ...), on pressure cells
__global__ void k_div_transpose(Dims d, int comp, GridDecode dec, double inv_dx, const float *__restrict__ wg,
                                const unsigned char *__restrict__ fluid, const double *__restrict__ gb, float *gub) {
    const unsigned int nf = (unsigned int)d.faces(comp);
    for (unsigned int q = blockIdx.x * blockDim.x + threadIdx.x; q < nf; q += gridDim.x * blockDim.x) {
        int i, j, k;
        dec(q, i, j, k);
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

// ---- P2G^T: per particle, gather over the faces within the kernel radius ----
// The transfer u_f = sum_p w_pf v_p / W_f (valid faces; otherwise the unnormalised sum) gives
//   dL/dv_p += sum_f g_f w_pf / W_f                               (invalid faces: g_f w_pf)
//   dL/dx_p += sum_f g_f (v_p - u_f) / W_f * dw_pf/dx_p           (invalid faces: g_f v_p dw_pf/dx_p)
// with w = (1 - s)^2 (1 - 4 s / 9), s = |x_f - x_p|^2 / r^2 (the reference's polynomial
// 1 - (4/9) s^3 + (17/9) s^2 - (22/9) s, factored), so dw/ds = -(2/9)(1 - s)(11 - 6 s) and
// dw/dx_p = (4/9)(1 - s)(11 - 6 s)(x_f - x_p) / r^2.
// W_f and u_f are the recorded sums in the same factored form, so faces whose weight sum is
// barely above the validity threshold keep their relative precision.  gx0 may be null.  The
// block-frame face coordinates (velocityadvector.cpp:492-496, double products rounded to
// float) depend on one face index each; they are tabulated per CTA in shared memory.
__global__ void k_p2g_transpose(Dims d, double dx, float r, int comp, int np, const int *__restrict__ sidx,
                                const float *__restrict__ spx, const float *__restrict__ spy,
                                const float *__restrict__ spz, const float *__restrict__ svel,
                                const float *__restrict__ wsum, const float *__restrict__ ufield,
                                const unsigned char *__restrict__ valid, const float *__restrict__ g, float *gv0,
                                float *gx0, float *gy0, float *gz0) {
    extern __shared__ float tab[];   // [nt]: block origin of face index t, [nt + t]: its offset in the block
    const int CW = 10;
    const int fw = d.ni + (comp == 0), fh = d.nj + (comp == 1), fd = d.nk + (comp == 2);
    const int nt = max(fw, max(fh, fd));
    const float hdx = (float)(0.5 * dx);
    const float ofx = comp == 0 ? 0.0f : hdx, ofy = comp == 1 ? 0.0f : hdx, ofz = comp == 2 ? 0.0f : hdx;
    const double chunkdx = dx * CW;
    const float rsq = r * r, inv_rsq = 1.0f / rsq;
    const double inv = 1.0 / dx;
    const float invf = (float)inv;
    for (int t = threadIdx.x; t < nt; t += blockDim.x) {
        const int A = t / CW;
        tab[t] = (float)((double)(float)A * chunkdx);
        tab[nt + t] = (float)((double)(float)(t - CW * A) * dx);
    }
    __syncthreads();
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < np; q += gridDim.x * blockDim.x) {
        float x = spx[q] - ofx, y = spy[q] - ofy, z = spz[q] - ofz;
        const float vp = svel[q];
        const int a0 = floor_fd(x - r, inv, invf), a1 = floor_fd(x + r, inv, invf) + 1;
        const int b0 = floor_fd(y - r, inv, invf), b1 = floor_fd(y + r, inv, invf) + 1;
        const int c0 = floor_fd(z - r, inv, invf), c1 = floor_fd(z + r, inv, invf) + 1;
        float acc = 0.0f, ax = 0.0f, ay = 0.0f, az = 0.0f;
        for (int fk = max(c0, 0); fk <= min(c1, fd - 1); fk++)
            for (int fj = max(b0, 0); fj <= min(b1, fh - 1); fj++)
                for (int fi = max(a0, 0); fi <= min(a1, fw - 1); fi++) {
                    const float vx = tab[nt + fi] - (x - tab[fi]), vy = tab[nt + fj] - (y - tab[fj]),
                                vz = tab[nt + fk] - (z - tab[fk]);
                    float d2 = vx * vx + vy * vy + vz * vz;
                    if (!(d2 < rsq)) continue;
                    const float sq = d2 * inv_rsq, om = 1.0f - sq;
                    const float wgt = om * om * (1.0f - (4.0f / 9.0f) * sq);
                    size_t f = flat3(fi, fj, fk, fw, fh);
                    const float gf = g[f];
                    const bool ok = valid[f] != 0;
                    const float W = ok ? wsum[f] : 1.0f;
                    acc += wgt / W * gf;
                    const float cf = (4.0f / 9.0f) * om * (11.0f - 6.0f * sq) * inv_rsq * gf *
                                     (ok ? (vp - ufield[f]) / W : vp);
                    ax += cf * vx; ay += cf * vy; az += cf * vz;
                }
        const int p = sidx[q];
        gv0[p] += acc;
        if (gx0) { gx0[p] += ax; gy0[p] += ay; gz0[p] += az; }
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
void adj_advect_transpose(Dims d, double dx, float a, float b, double dt, int np, size_t cap, const int *sidx,
                          const float *spx, const float *spy, const float *spz, const float *const gx1[3],
                          const float *const gv1[3], const unsigned char *collided, float *const gx0[3], float *wc,
                          float *ws, float *pt2, float *pt3, MacView cur, MacView saved, cudaStream_t st) {
    if (np == 0) return;
    const float h1 = (float)(0.5 * dt), h2 = (float)(0.75 * dt), h3 = (float)(dt / 9.0f);
    k_advect_transpose<<<grid_for(np, 128, 152u * 32u), 128, 0, st>>>(
        make_mac(d, dx, cur), make_mac(d, dx, saved), a, b, h1, h2, h3, np, cap, sidx, spx, spy, spz,
        gx1 ? gx1[0] : nullptr, gx1 ? gx1[1] : nullptr, gx1 ? gx1[2] : nullptr, gv1[0], gv1[1], gv1[2], collided,
        gx0[0], gx0[1], gx0[2], wc, ws, pt2, pt3);
}

void adj_sample_transpose(Dims d, double dx, int comp, bool float_keys, const int *cell_start, const float *qx,
                          const float *qy, const float *qz, const float *wa, const float *wb, float *ga, float *gb,
                          bool accumulate, cudaStream_t st) {
    size_t nf = d.faces(comp);
    const GridDecode dec = grid_decode(d.ni + (comp == 0), d.nj + (comp == 1), d.nk + (comp == 2));
    k_sample_transpose<<<grid_for(nf, 256, 152u * 64u), 256, 0, st>>>(d, (float)dx, (float)(1.0 / dx), (float)(0.5 * dx),
                                                                      comp, dec, float_keys ? 0 : 1, cell_start, qx, qy,
                                                                      qz, wa, wb, ga, gb, accumulate ? 1 : 0);
}

void adj_extrapolate_transpose(int w, int h, int dd, int layers, const unsigned char *valid0,
                               const unsigned char *layer_of, float *g, float *tmp, cudaStream_t st) {
    size_t n = (size_t)w * h * dd;
    unsigned int grid = grid_for(n, 256, 152u * 32u);
    const GridDecode dec = grid_decode(w, h, dd);
    float *a = g, *b = tmp;
    for (int L = layers - 1; L >= 0; L--) {
        k_extrap_transpose<<<grid, 256, 0, st>>>(w, h, dd, dec, L, valid0, layer_of, a, b);
        float *t = a; a = b; b = t;
    }
    if (a != g) FFGPU_CUDA(cudaMemcpyAsync(g, a, n * 4, cudaMemcpyDeviceToDevice, st));
}

void adj_projection_faces(Dims d, int comp, const float *phi, const float *wg, const float *gup, float *gub,
                          cudaStream_t st) {
    size_t nf = d.faces(comp);
    const GridDecode dec = grid_decode(d.ni + (comp == 0), d.nj + (comp == 1), d.nk + (comp == 2));
    k_proj_faces_transpose<<<grid_for(nf, 256), 256, 0, st>>>(d, comp, dec, phi, wg, gup, gub);
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
    const GridDecode dec = grid_decode(d.ni + (comp == 0), d.nj + (comp == 1), d.nk + (comp == 2));
    k_div_transpose<<<grid_for(nf, 256), 256, 0, st>>>(d, comp, dec, 1.0 / dx, wg, fluid, gb, gub);
}

void adj_p2g_transpose(Dims d, double dx, double radius, int comp, int np, const int *sidx, const float *spx,
                       const float *spy, const float *spz, const float *svel, const float *wsum, const float *ufield,
                       const unsigned char *valid, const float *g, float *gv0, float *const gx0[3], cudaStream_t st) {
    if (np == 0) return;
    const int nt = std::max(d.ni, std::max(d.nj, d.nk)) + 1;
    k_p2g_transpose<<<grid_for(np, 256), 256, 2 * nt * sizeof(float), st>>>(
        d, dx, (float)radius, comp, np, sidx, spx, spy, spz, svel, wsum, ufield, valid, g, gv0, gx0 ? gx0[0] : nullptr,
        gx0 ? gx0[1] : nullptr, gx0 ? gx0[2] : nullptr);
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

__global__ void k_fill(size_t n, float v, float *out) {
    for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
        out[t] = v;
}

void adj_fill(size_t n, float v, float *out, cudaStream_t st) {
    if (n) k_fill<<<grid_for(n, 256), 256, 0, st>>>(n, v, out);
}

}  // namespace ffgpu
