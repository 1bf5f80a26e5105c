// Receiver-side kernels (internal).
#pragma once

#include "common.cuh"
#include "internal.h"

namespace ac3d {

void launch_far_field(const DevGeometry& G, int prec, const double4* recv, int L, double k, const cd* x, cd* y,
                      DevBuf& scratch, cudaStream_t s);
void launch_far_field_t(const DevGeometry& G, int prec, const double4* recv, int L, double k, const cd* vf, cd* out,
                        cudaStream_t s);
void launch_accum_abs(const cd* y, int L, double* yt, cudaStream_t s);
void launch_compute_u(const double* yt, int L, double* u, double* coef, cudaStream_t s);
void launch_vf(const double* u, const cd* y, int L, cd* vf, cudaStream_t s);
void launch_listener_aca(const DevGeometry& G, int prec, const void* pts, int L, double k, double eps, int maxk,
                         void* pool, long long pool_cap, unsigned long long* used, long long* term_off, int* rank,
                         int* status, const int4* block, const int* order, cudaStream_t s);

void launch_lr_apply(int prec, const void* pool, const long long* toff, const int* rank, int iter_lim, int L, int ne,
                     const cd* x, int trans, cd* t, cd* out, cudaStream_t s);

// Shape-derivative terms of the adjoint gradient (adjoint.cu).
struct AdjointArgs {
  int prec;
  double k;
  int npairs;            // incidences (element, corner) over all differentiable points
  const int* pair_elem;  // [npairs]
  const int* pair_corner;
  int ntouch;            // distinct elements appearing in pairs
  const int* touch_elem; // [ntouch]
  const int* pair_touch; // [npairs] index into touch_elem
  const double4* recv;
  int L;
  const cd* vf;          // [L]
  const cd* x;           // [Ne]
  const cd* lmb;         // [Ne]
  int rhs_kind;          // 0 point source, 1 plane wave
  double rhs_v[3];
  const int* h_off;      // [HH + 1] CSR over pairs
  int HH;
  double* grad;          // [HH] accumulated (+=)
};
void launch_adjoint_terms(const DevGeometry& G, const AdjointArgs& a, DevBuf& scratch, cudaStream_t s);

}  // namespace ac3d
