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
// The receiver ACA in double-float arithmetic (the mixed path's default assembly): pts_df holds L
// double-float points (8 floats each: x, y, z as hi/lo pairs, two pad); the terms end up in the
// pool as complex FP64.
void launch_listener_aca_df(const DevGeometry& G, const void* pts_df, int L, double k, double eps, int maxk,
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

// The same terms for up to kAdjMaxRhs plane-wave incidence directions of one frequency at once:
// every shape-derivative entry is evaluated once and applied to every direction's x, lambda and
// vf. grad[h] += sum_r w[r] (A_r - B_r + C_r).
constexpr int kAdjMaxRhs = 16;
struct AdjointMultiArgs {
  int prec;
  double k;
  int npairs;
  const int* pair_elem;
  const int* pair_corner;
  int ntouch;
  const int* touch_elem;
  const int* pair_touch;
  const double4* recv;
  int L;
  int nr;                          // directions in this batch (<= kAdjMaxRhs)
  const cd* vf;                    // nr x L, direction-major
  const cd* x;                     // nr x Ne, direction-major
  const cd* lmb;                   // nr x Ne, direction-major
  double dir[kAdjMaxRhs][3];       // plane-wave directions (unit)
  double w[kAdjMaxRhs];            // weights of the directions' terms
  const int* h_off;
  int HH;
  double* grad;
};
void launch_adjoint_terms_multi(const DevGeometry& G, const AdjointMultiArgs& a, DevBuf& scratch, cudaStream_t s);

}  // namespace ac3d
