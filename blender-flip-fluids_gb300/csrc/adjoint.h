// Adjoint kernels (adjoint_kernels.cu).
#pragma once
#include "kernels.h"

namespace ffgpu {

void adj_g2p_transpose(Dims d, double dx, int comp, const int *cell_start, const int *sidx, const float *spx,
                       const float *spy, const float *spz, const float *g1, float scale_cur, float scale_saved,
                       float *gcur, float *gsaved, cudaStream_t st);
void adj_extrapolate_transpose(int w, int h, int dd, int layers, const unsigned char *valid0,
                               const unsigned char *layer_of, float *g, float *tmp, cudaStream_t st);
void adj_projection_faces(Dims d, int comp, const float *phi, const float *wg, const float *gup, float *gub,
                          cudaStream_t st);
void adj_pressure_grad(Dims d, Bbox bb, double dx, double dt, const float *phi, const float *wu, const float *wv,
                       const float *ww, const float *gu, const float *gv, const float *gw, const unsigned char *fluid,
                       double *gp, cudaStream_t st);
void adj_div_transpose(Dims d, int comp, double dx, const float *wg, const unsigned char *fluid, const double *gb,
                       float *gub, cudaStream_t st);
void adj_p2g_transpose(Dims d, double dx, double radius, int comp, int np, const int *sidx, const float *spx,
                       const float *spy, const float *spz, const float *wsum, const float *g, float *gv0,
                       cudaStream_t st);
int adj_loss_grad_vy2(int np, double ymin, const float *py, const float *vy, float *gx, float *gy, float *gz,
                      int *count_dev, int *count_host, cudaStream_t st);
void adj_scale(size_t n, const float *a, float s, float *out, cudaStream_t st);
void adj_add(size_t n, const float *a, float *out, cudaStream_t st);

}  // namespace ffgpu
