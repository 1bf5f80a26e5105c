// Device-resident BiCGSTAB interface (internal).
#pragma once

#include "internal.h"

namespace ac3d {

// Solver scalars, kept on the device for the whole solve.
struct KState {
  double rho_re, rho_im, rho_old_re, rho_old_im;
  double rho_new_re, rho_new_im;   // rho of the running iteration (committed at its end)
  double alpha_new_re, alpha_new_im;
  double alpha_re, alpha_im, omega_re, omega_im;
  double beta_re, beta_im;
  double bnorm2, rnorm2, tol2, rhat2;
  int iter, maxit;
  int done;      // 0 running, 1 converged, 2 iteration limit, 3 breakdown (rhat . v == 0)
  int restart;   // this iteration restarts with rhat = r
  int restarts;
  int pad;
  double rsum[5];   // fixed-order totals of the latest residual partials: (rhat, r), -, -, |r|^2
  unsigned ticket;  // CTA completion counter of kf_xr (zero between launches)
  int pad2;
};

// Device vectors of one solve (complex, FP32 or FP64 according to the solve).
struct KrylovBufs {
  int n = 0;
  void *b = nullptr, *x = nullptr, *r = nullptr, *rhat = nullptr, *p = nullptr, *v = nullptr, *s = nullptr,
       *t = nullptr;
  double* partials = nullptr;  // (nleaf + vector grid) x 5: per-leaf matvec partials, then vector partials
  int nparts_r = 0;            // number of partials feeding the rho step (vector grid)
  int nleaf = 0;
  double* red5 = nullptr;      // fixed-order totals of the latest matvec's dot partials
  void *p32 = nullptr, *s32 = nullptr;  // FP32 shadows of p and s (FP64 vectors on FP32 storage)
  KState* state = nullptr;
};

void krylov_enqueue_init(const KrylovBufs& B, int vec64, double tol, int maxit, cudaStream_t s);
void krylov_enqueue_iterations(const KrylovBufs& B, const DevPartition& DP, const DevHMat& H, bool transposed,
                               int vec64, int count, cudaStream_t s);
int krylov_vec_grid(int n);

void launch_matvec_ex(const DevPartition& DP, const DevHMat& H, bool transposed, int vec64, const void* x, void* y,
                      const void* b_minus, const MatvecEpilogue& ep, const int* done, cudaStream_t s,
                      const void* x32 = nullptr, bool pdl = false);
void launch_to32(int n, const void* a, void* b, cudaStream_t s);
void launch_add32(int n, void* x, const void* d, cudaStream_t s);
void launch_add64(int n, void* x, const void* d, cudaStream_t s);
void launch_copy64(int n, const void* a, void* b, cudaStream_t s);
void launch_zero64(int n, void* b, cudaStream_t s);
void launch_negate64(int n, void* a, cudaStream_t s);
int launch_norm2_64(int n, const void* a, double* partials, cudaStream_t s);
void launch_reduce5(const double* partials, int n, double* out, cudaStream_t s);

}  // namespace ac3d
