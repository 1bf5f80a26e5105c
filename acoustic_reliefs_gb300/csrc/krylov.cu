// Device-resident BiCGSTAB (van der Vorst 1992), the solver the reference runs through
// Eigen::BiCGSTAB with an identity preconditioner and zero initial guess (adjoint.cpp:92-95,
// 190-209; acoustics3d.cpp:266-269). Stop rule: |r|^2 <= tol^2 |b|^2 on the recursively updated
// residual, checked before every iteration; at most `maxit` iterations.
//
// All scalars live in a device struct; dot products are FP64 and reduced in a fixed order
// (per-CTA partials, then one CTA), so a solve is bit-reproducible. Every kernel returns at once
// when the state says the solve has finished, which lets the host replay a captured graph of a
// fixed number of iterations until the flag is set.
#include "common.cuh"
#include "internal.h"
#include "krylov.h"
#include "launch.cuh"

namespace ac3d {

namespace {
constexpr int kVecThreads = 256;
constexpr int kVecWarps = kVecThreads / 32;
}  // namespace

__device__ __forceinline__ void block_sums(double* d, int nd, double (*sd)[5]) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int i = 0; i < nd; i++) d[i] = warp_sum(d[i]);
  if (lane == 0)
    for (int i = 0; i < nd; i++) sd[w][i] = d[i];
  __syncthreads();
}

__device__ __forceinline__ void write_partials(double* d, double* partials) {
  __shared__ double sd[kVecWarps][5];
  block_sums(d, 5, sd);
  if (threadIdx.x < 5) {
    double s = 0;
    for (int w = 0; w < kVecWarps; w++) s += sd[w][threadIdx.x];
    partials[(size_t)blockIdx.x * 5 + threadIdx.x] = s;
  }
}

// Fixed-order reduction of `n` partial 5-vectors by one CTA; result in out[5] (all threads).
__device__ __forceinline__ void reduce_partials(const double* partials, int n, double* out) {
  __shared__ double sd[kVecWarps][5];
  double d[5] = {0, 0, 0, 0, 0};
  for (int i = threadIdx.x; i < n; i += blockDim.x)
    for (int c = 0; c < 5; c++) d[c] += __ldcg(&partials[(size_t)i * 5 + c]);  // written by other CTAs
  block_sums(d, 5, sd);
  for (int c = 0; c < 5; c++) {
    double s = 0;
    for (int w = 0; w < kVecWarps; w++) s += sd[w][c];
    out[c] = s;
  }
  __syncthreads();
}

template <typename VT>
__global__ void __launch_bounds__(kVecThreads) k_init(int n, const cplx<VT>* __restrict__ b, cplx<VT>* x,
                                                      cplx<VT>* r, cplx<VT>* rhat, cplx<VT>* p, cplx<VT>* v,
                                                      double* partials) {
  double d[5] = {0, 0, 0, 0, 0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    cplx<VT> bi = b[i];
    x[i] = cplx<VT>();
    r[i] = bi;
    rhat[i] = bi;
    p[i] = cplx<VT>();
    v[i] = cplx<VT>();
    double a2 = (double)bi.re * bi.re + (double)bi.im * bi.im;
    d[0] += a2;
    d[4] += a2;
  }
  write_partials(d, partials);
}

__global__ void k_scalar_init(KState* st, const double* partials, int n, double tol, int maxit) {
  double s[5];
  reduce_partials(partials, n, s);
  if (threadIdx.x == 0) {
    st->bnorm2 = s[4];
    st->rnorm2 = s[4];
    st->rhat2 = s[4];
    st->tol2 = tol * tol * s[4];
    st->rho_re = st->alpha_re = st->omega_re = 1.0;
    st->rho_im = st->alpha_im = st->omega_im = 0.0;
    st->rho_old_re = 1.0;
    st->rho_old_im = 0.0;
    st->beta_re = st->beta_im = 0.0;
    st->iter = 0;
    st->maxit = maxit;
    st->done = s[4] == 0.0 ? 1 : 0;
    st->restart = 0;
    st->restarts = 0;
    for (int c = 0; c < 5; c++) st->rsum[c] = s[c];
    st->ticket = 0u;
  }
}

__device__ __forceinline__ void cdivd(double ar, double ai, double br, double bi, double& cr, double& ci) {
  double s = fabs(br) + fabs(bi);
  double xr = br / s, xi = bi / s, yr = ar / s, yi = ai / s;
  double d = xr * xr + xi * xi;
  cr = (yr * xr + yi * xi) / d;
  ci = (yi * xr - yr * xi) / d;
}










// ------------------------------------------------------------------------------------------
// Fused iteration: every CTA of a vector kernel reduces the partials itself (same order, same
// result in every CTA) instead of a separate single-CTA scalar kernel; CTA 0 commits the state,
// only into fields that no other CTA of the same kernel reads.
// ------------------------------------------------------------------------------------------
struct RhoStep {
  bool stop;      // converged or out of iterations: nothing more to do
  bool restart;
  double rho_re, rho_im, beta_re, beta_im, rr;
  int done;
};

__device__ __forceinline__ RhoStep rho_step(const KState* st, const double* s) {
  RhoStep o{};
  o.rr = s[4];
  o.done = 0;
  if (!(o.rr > st->tol2)) {
    o.stop = true;
    o.done = 1;
    return o;
  }
  if (st->iter >= st->maxit) {
    o.stop = true;
    o.done = 2;
    return o;
  }
  o.rho_re = s[0];
  o.rho_im = s[1];
  if (o.rho_re * o.rho_re + o.rho_im * o.rho_im <= 1e-24 * st->rhat2 * o.rr) {
    o.restart = true;
    o.rho_re = o.rr;
    o.rho_im = 0.0;
    return o;
  }
  double q1r, q1i, q2r, q2i;
  cdivd(o.rho_re, o.rho_im, st->rho_re, st->rho_im, q1r, q1i);
  cdivd(st->alpha_re, st->alpha_im, st->omega_re, st->omega_im, q2r, q2i);
  o.beta_re = q1r * q2r - q1i * q2i;
  o.beta_im = q1r * q2i + q1i * q2r;
  return o;
}

// start of an iteration: convergence test, rho, beta; p = r + beta (p - omega v)
template <typename VT>
__global__ void __launch_bounds__(kVecThreads) kf_p(KState* st, const double* partials, int nparts, int n,
                                                    const cplx<VT>* __restrict__ r, cplx<VT>* p, cplx<VT>* v,
                                                    cplx<VT>* rhat, cf* p32) {
  grid_dep_wait();  // programmatic launch: the preceding kernel has completed past this point
  grid_dep_launch();
  if (st->done) return;
  // the scalars once per CTA (FP64 division is slow): every CTA gets the same values
  __shared__ RhoStep so;
  if (threadIdx.x == 0) so = rho_step(st, st->rsum);
  __syncthreads();
  const RhoStep o = so;
  (void)partials;
  (void)nparts;
  if (o.stop) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      st->rnorm2 = o.rr;
      st->done = o.done;
    }
    return;
  }
  const VT br = (VT)o.beta_re, bi = (VT)o.beta_im;
  const VT wr = (VT)(o.restart ? 1.0 : st->omega_re), wi = (VT)(o.restart ? 0.0 : st->omega_im);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const cplx<VT> ri = r[i];
    cplx<VT> pn;
    if (o.restart) {
      rhat[i] = ri;
      pn = ri;
      v[i] = cplx<VT>();
    } else {
      const cplx<VT> pi = p[i], vi = v[i];
      const VT tr = pi.re - (wr * vi.re - wi * vi.im);
      const VT ti = pi.im - (wr * vi.im + wi * vi.re);
      pn = cplx<VT>(ri.re + br * tr - bi * ti, ri.im + br * ti + bi * tr);
    }
    p[i] = pn;
    if (p32) p32[i] = cf((float)pn.re, (float)pn.im);  // matvec input of the FP32-storage solve
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    st->rnorm2 = o.rr;
    st->rho_new_re = o.rho_re;
    st->rho_new_im = o.rho_im;
    st->restart = o.restart ? 1 : 0;  // rhat2 is committed by kf_xr (other CTAs here read it)
    if (o.restart) st->restarts++;
  }
}

// alpha = rho / (rhat, v); s = r - alpha v
template <typename VT>
__global__ void __launch_bounds__(kVecThreads) kf_s(KState* st, const double* red5, int n,
                                                    const cplx<VT>* __restrict__ r, const cplx<VT>* __restrict__ v,
                                                    cplx<VT>* s, cf* s32) {
  grid_dep_wait();  // programmatic launch: the preceding kernel has completed past this point
  grid_dep_launch();
  if (st->done) return;
  __shared__ double sa[3];
  if (threadIdx.x == 0) {
    const double d0 = red5[0], d1 = red5[1];
    sa[2] = (d0 == 0.0 && d1 == 0.0) ? 1.0 : 0.0;
    if (sa[2] == 0.0) cdivd(st->rho_new_re, st->rho_new_im, d0, d1, sa[0], sa[1]);
  }
  __syncthreads();
  if (sa[2] != 0.0) {
    if (blockIdx.x == 0 && threadIdx.x == 0) st->done = 3;
    return;
  }
  const double ar = sa[0], ai = sa[1];
  const VT a_r = (VT)ar, a_i = (VT)ai;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const cplx<VT> ri = r[i], vi = v[i];
    const cplx<VT> si(ri.re - (a_r * vi.re - a_i * vi.im), ri.im - (a_r * vi.im + a_i * vi.re));
    s[i] = si;
    if (s32) s32[i] = cf((float)si.re, (float)si.im);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    st->alpha_new_re = ar;
    st->alpha_new_im = ai;
  }
}

// omega = (t, s) / (t, t); x += alpha p + omega s; r = s - omega t; partials (rhat, r), |r|^2
template <typename VT>
__global__ void __launch_bounds__(kVecThreads) kf_xr(KState* st, const double* red5, int n, cplx<VT>* x,
                                                     const cplx<VT>* __restrict__ p, const cplx<VT>* __restrict__ s,
                                                     cplx<VT>* r, const cplx<VT>* __restrict__ t,
                                                     const cplx<VT>* __restrict__ rhat, double* out_partials) {
  grid_dep_wait();  // programmatic launch: the preceding kernel has completed past this point
  grid_dep_launch();
  if (st->done) return;
  __shared__ double sw[2];
  __shared__ bool s_last;
  if (threadIdx.x == 0) {
    const double d2 = red5[2], d3 = red5[3], d4 = red5[4];
    sw[0] = d4 > 0.0 ? d2 / d4 : 0.0;
    sw[1] = d4 > 0.0 ? d3 / d4 : 0.0;
  }
  __syncthreads();
  const double wr_d = sw[0], wi_d = sw[1];
  const double ar_d = st->alpha_new_re, ai_d = st->alpha_new_im;
  const VT ar = (VT)ar_d, ai = (VT)ai_d, wr = (VT)wr_d, wi = (VT)wi_d;
  double d[5] = {0, 0, 0, 0, 0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const cplx<VT> pi = p[i], si = s[i], ti = t[i], hi = rhat[i];
    cplx<VT> xi = x[i];
    xi.re += (ar * pi.re - ai * pi.im) + (wr * si.re - wi * si.im);
    xi.im += (ar * pi.im + ai * pi.re) + (wr * si.im + wi * si.re);
    x[i] = xi;
    const cplx<VT> ri(si.re - (wr * ti.re - wi * ti.im), si.im - (wr * ti.im + wi * ti.re));
    r[i] = ri;
    d[0] += (double)hi.re * ri.re + (double)hi.im * ri.im;
    d[1] += (double)hi.re * ri.im - (double)hi.im * ri.re;
    d[4] += (double)ri.re * ri.re + (double)ri.im * ri.im;
  }
  write_partials(d, out_partials);
  // the last CTA to finish reduces the partials in fixed order for the next kf_p
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(&st->ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (s_last) {
    __threadfence();
    double tot[5];
    reduce_partials(out_partials, gridDim.x, tot);
    if (threadIdx.x == 0) {
      for (int c = 0; c < 5; c++) st->rsum[c] = tot[c];
      st->ticket = 0u;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    st->rho_old_re = st->rho_re;
    st->rho_old_im = st->rho_im;
    st->rho_re = st->rho_new_re;
    st->rho_im = st->rho_new_im;
    st->alpha_re = ar_d;
    st->alpha_im = ai_d;
    st->omega_re = wr_d;
    st->omega_im = wi_d;
    if (st->restart) st->rhat2 = st->rnorm2;
    st->iter++;
  }
}

// ------------------------------------------------------------------------------------------
// Refinement helpers (mixed precision): FP64 residual -> FP32 right-hand side, x64 += d32.
// ------------------------------------------------------------------------------------------
__global__ void k_to32(int n, const cd* __restrict__ a, cf* b) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    b[i] = cf((float)a[i].re, (float)a[i].im);
}
__global__ void k_add64(int n, cd* x, const cd* __restrict__ d) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    x[i].re += d[i].re;
    x[i].im += d[i].im;
  }
}
__global__ void k_add32(int n, cd* x, const cf* __restrict__ d) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    x[i].re += (double)d[i].re;
    x[i].im += (double)d[i].im;
  }
}
__global__ void k_copy64(int n, const cd* __restrict__ a, cd* b) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) b[i] = a[i];
}
__global__ void k_zero64(int n, cd* b) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) b[i] = cd();
}
__global__ void k_negate64(int n, cd* a) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    a[i].re = -a[i].re;
    a[i].im = -a[i].im;
  }
}
__global__ void __launch_bounds__(kVecThreads) k_norm2_64(int n, const cd* __restrict__ a, double* partials) {
  double d[5] = {0, 0, 0, 0, 0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    d[4] += a[i].re * a[i].re + a[i].im * a[i].im;
  write_partials(d, partials);
}
__global__ void k_reduce5(const double* partials, int n, double* out) {
  double s[5];
  reduce_partials(partials, n, s);
  if (threadIdx.x < 5) out[threadIdx.x] = s[threadIdx.x];
}

// ------------------------------------------------------------------------------------------
// Host side
// ------------------------------------------------------------------------------------------
static int vec_grid(int n) {
  int g = (n + kVecThreads - 1) / kVecThreads;
  return g < 1 ? 1 : (g > 1184 ? 1184 : g);
}

// vec64: 0 FP32 vectors; 1 FP64 vectors and FP64 matvec arithmetic (FP64 storage); 2 FP64 vectors,
// FP32 storage and FP32 matvec arithmetic on FP32 shadow copies of p and s (B.p32, B.s32)
// All launches but the first of a captured chunk are programmatic dependents of the kernel
// before them (launch.cuh): each kernel's set-up overlaps the end of the previous one.
#ifndef AC3D_PDL
#define AC3D_PDL 1
#endif
constexpr bool kPdl = AC3D_PDL != 0;


template <typename VT>
static void enqueue_iteration(const KrylovBufs& B, const DevPartition& DP, const DevHMat& H, bool tr, int vec64,
                              bool first, cudaStream_t s) {
  const int n = B.n, G = vec_grid(n);
  cf* p32 = vec64 == 2 ? (cf*)B.p32 : nullptr;
  cf* s32 = vec64 == 2 ? (cf*)B.s32 : nullptr;
  KState* st = B.state;
  // partials: xr / init write slots [0, G) of rpart; the matvec gathers write the per-leaf slots
  double* rpart = B.partials + (size_t)DP.nleaf * 5;
  launch_k(kPdl && !first, kf_p<VT>, dim3(G), dim3(kVecThreads), 0, s, st, (const double*)rpart, G, n, (const cplx<VT>*)B.r,
           (cplx<VT>*)B.p, (cplx<VT>*)B.v, (cplx<VT>*)B.rhat, p32);
  MatvecEpilogue e1;
  e1.dot_a = B.rhat;
  e1.partials = B.partials;
  e1.red5 = B.red5;
  launch_matvec_ex(DP, H, tr, vec64, B.p, B.v, nullptr, e1, &st->done, s, p32, kPdl);
  launch_k(kPdl, kf_s<VT>, dim3(G), dim3(kVecThreads), 0, s, st, (const double*)B.red5, n, (const cplx<VT>*)B.r,
           (const cplx<VT>*)B.v, (cplx<VT>*)B.s, s32);
  MatvecEpilogue e2;
  e2.dot_b = B.s;
  e2.partials = B.partials;
  e2.red5 = B.red5;
  launch_matvec_ex(DP, H, tr, vec64, B.s, B.t, nullptr, e2, &st->done, s, s32, kPdl);
  launch_k(kPdl, kf_xr<VT>, dim3(G), dim3(kVecThreads), 0, s, st, (const double*)B.red5, n, (cplx<VT>*)B.x,
           (const cplx<VT>*)B.p, (const cplx<VT>*)B.s, (cplx<VT>*)B.r, (const cplx<VT>*)B.t, (const cplx<VT>*)B.rhat,
           rpart);
}

void krylov_enqueue_init(const KrylovBufs& B, int vec64, double tol, int maxit, cudaStream_t s) {
  const int n = B.n, G = vec_grid(n);
  double* rpart = B.partials + (size_t)B.nleaf * 5;
  note_launch();
  if (vec64)
    k_init<double><<<G, kVecThreads, 0, s>>>(n, (const cd*)B.b, (cd*)B.x, (cd*)B.r, (cd*)B.rhat, (cd*)B.p,
                                             (cd*)B.v, rpart);
  else
    k_init<float><<<G, kVecThreads, 0, s>>>(n, (const cf*)B.b, (cf*)B.x, (cf*)B.r, (cf*)B.rhat, (cf*)B.p,
                                            (cf*)B.v, rpart);
  note_launch();
  k_scalar_init<<<1, kVecThreads, 0, s>>>(B.state, rpart, G, tol, maxit);
  AC3D_CUDA(cudaGetLastError());
}

void krylov_enqueue_iterations(const KrylovBufs& B, const DevPartition& DP, const DevHMat& H, bool tr, int vec64,
                               int count, cudaStream_t s) {
  for (int i = 0; i < count; i++) {
    if (vec64)
      enqueue_iteration<double>(B, DP, H, tr, vec64, i == 0, s);
    else
      enqueue_iteration<float>(B, DP, H, tr, 0, i == 0, s);
  }
}

int krylov_vec_grid(int n) { return vec_grid(n); }

void launch_to32(int n, const void* a, void* b, cudaStream_t s) {
  note_launch();
  k_to32<<<vec_grid(n), kVecThreads, 0, s>>>(n, (const cd*)a, (cf*)b);
  AC3D_CUDA(cudaGetLastError());
}
void launch_add32(int n, void* x, const void* d, cudaStream_t s) {
  note_launch();
  k_add32<<<vec_grid(n), kVecThreads, 0, s>>>(n, (cd*)x, (const cf*)d);
  AC3D_CUDA(cudaGetLastError());
}
void launch_add64(int n, void* x, const void* d, cudaStream_t s) {
  note_launch();
  k_add64<<<vec_grid(n), kVecThreads, 0, s>>>(n, (cd*)x, (const cd*)d);
  AC3D_CUDA(cudaGetLastError());
}
void launch_copy64(int n, const void* a, void* b, cudaStream_t s) {
  note_launch();
  k_copy64<<<vec_grid(n), kVecThreads, 0, s>>>(n, (const cd*)a, (cd*)b);
  AC3D_CUDA(cudaGetLastError());
}
void launch_zero64(int n, void* b, cudaStream_t s) {
  note_launch();
  k_zero64<<<vec_grid(n), kVecThreads, 0, s>>>(n, (cd*)b);
  AC3D_CUDA(cudaGetLastError());
}
void launch_negate64(int n, void* a, cudaStream_t s) {
  note_launch();
  k_negate64<<<vec_grid(n), kVecThreads, 0, s>>>(n, (cd*)a);
  AC3D_CUDA(cudaGetLastError());
}
int launch_norm2_64(int n, const void* a, double* partials, cudaStream_t s) {
  note_launch();
  k_norm2_64<<<vec_grid(n), kVecThreads, 0, s>>>(n, (const cd*)a, partials);
  AC3D_CUDA(cudaGetLastError());
  return vec_grid(n);
}
void launch_reduce5(const double* partials, int n, double* out, cudaStream_t s) {
  note_launch();
  k_reduce5<<<1, kVecThreads, 0, s>>>(partials, n, out);
  AC3D_CUDA(cudaGetLastError());
}

}  // namespace ac3d
