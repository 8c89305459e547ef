// Adjoint kernels (adjoint_kernels.cu).
#pragma once
#include "kernels.h"

namespace ffgpu {

// RK3 advection^T plus the position part of G2P^T (per particle, cell-sorted order); gx1 may be
// null (zero).  wc/ws: 3 x cap, pt2/pt3: 6 x cap floats, component-major.
void adj_advect_transpose(Dims d, double dx, float a, float b, double dt, int np, size_t cap, const int *sidx,
                          const float *spx, const float *spy, const float *spz, const float *const gx1[3],
                          const float *const gv1[3], const unsigned char *collided, float *const gx0[3], float *wc,
                          float *ws, float *pt2, float *pt3, MacView cur, MacView saved, cudaStream_t st);
// transposed trilinear sampling of one component at cell-sorted points with weights wa (into
// ga, accumulated or overwritten) and optionally wb (into gb, overwritten); float_keys: the
// points were sorted with the sampling's float cell floor (otherwise the double one)
void adj_sample_transpose(Dims d, double dx, int comp, bool float_keys, const int *cell_start, const float *qx,
                          const float *qy, const float *qz, const float *wa, const float *wb, float *ga, float *gb,
                          bool accumulate, cudaStream_t st);
void adj_extrapolate_transpose(int w, int h, int dd, int layers, const unsigned char *valid0,
                               const unsigned char *layer_of, float *g, float *tmp, cudaStream_t st);
void adj_projection_faces(Dims d, int comp, const float *phi, const float *wg, const float *gup, float *gub,
                          cudaStream_t st);
void adj_pressure_grad(Dims d, Bbox bb, double dx, double dt, const float *phi, const float *wu, const float *wv,
                       const float *ww, const float *gu, const float *gv, const float *gw, const unsigned char *fluid,
                       double *gp, cudaStream_t st);
void adj_div_transpose(Dims d, int comp, double dx, const float *wg, const unsigned char *fluid, const double *gb,
                       float *gub, cudaStream_t st);
// P2G^T for one component: dL/dv0 (+=) and, when gx0 is not null, dL/dx0 (+=); wsum / ufield are
// the recorded accurate weight sums and transfer outputs, valid the recorded valid flags
void adj_p2g_transpose(Dims d, double dx, double radius, int comp, int np, const int *sidx, const float *spx,
                       const float *spy, const float *spz, const float *svel, const float *wsum, const float *ufield,
                       const unsigned char *valid, const float *g, float *gv0, float *const gx0[3], cudaStream_t st);
int adj_loss_grad_vy2(int np, double ymin, const float *py, const float *vy, float *gx, float *gy, float *gz,
                      int *count_dev, int *count_host, cudaStream_t st);
void adj_scale(size_t n, const float *a, float s, float *out, cudaStream_t st);
void adj_add(size_t n, const float *a, float *out, cudaStream_t st);
void adj_fill(size_t n, float v, float *out, cudaStream_t st);

}  // namespace ffgpu
