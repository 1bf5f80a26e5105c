// Far field at the receivers and the diffusion coefficient.
//
// The reference approximates the receiver matrix Q (L x Ne, Q_lj = M(receiver l, element j)) by
// ACA (compute_ACA_listener, aca.cpp:84-134) and applies y = U (V x) (adjoint.cpp:101-102) and
// adj_b = V^T (U^T vf) (adjoint.cpp:198). Here Q is evaluated exactly, on the fly, with every
// entry recomputed inside the product (L x Ne x 6 kernel evaluations, never stored): this is the
// GPU-native choice, and it differs from the reference's ACA product only by the ACA error.
// The ACA route is available too (launch_listener_aca in assemble.cu).
//
// compute_u (adjoint.cpp:388-397) and the adjoint seed vf = u conj(y)/|y| (adjoint.cpp:145) are
// small single-CTA kernels.
#include "common.cuh"
#include "internal.h"
#include "listener.h"

namespace ac3d {

namespace {
constexpr int kFFThreads = 256;
constexpr int kFFWarps = kFFThreads / 32;
constexpr int kFFRecv = 4;  // receivers per CTA in the forward product
}  // namespace

template <typename R>
GeoView<R> geo_view(const DevGeometry& G);

// partial[l * S + split] = sum over elements j of this split of Q_lj x_j
template <typename R>
__global__ void __launch_bounds__(kFFThreads) far_kernel(GeoView<R> G, const double4* __restrict__ recv, int L,
                                                         R k, const cd* __restrict__ x, cd* partial, int S) {
  __shared__ double sd[kFFWarps][2 * kFFRecv];
  const int l0 = blockIdx.x * kFFRecv;
  const int split = blockIdx.y;
  const int ne = G.ne;
  const int per = (ne + S - 1) / S;
  const int j0 = split * per, j1 = min(ne, j0 + per);
  double4 P[kFFRecv];
  for (int a = 0; a < kFFRecv; a++) P[a] = recv[min(l0 + a, L - 1)];
  R ar[kFFRecv], ai[kFFRecv];
  for (int a = 0; a < kFFRecv; a++) ar[a] = ai[a] = 0;
  for (int j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
    const double4 va = G.va[j];
    const ElemGeo<R> g = G.eg[j];
    const cd xj = x[j];
    const R xr = (R)xj.re, xi = (R)xj.im;
#pragma unroll
    for (int a = 0; a < kFFRecv; a++) {
      cplx<R> q = entry_from_d<R>(k, (R)(P[a].x - va.x), (R)(P[a].y - va.y), (R)(P[a].z - va.z), g);
      ar[a] += q.re * xr - q.im * xi;
      ai[a] += q.re * xi + q.im * xr;
    }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int a = 0; a < kFFRecv; a++) {
    double vr = warp_sum((double)ar[a]), vi = warp_sum((double)ai[a]);
    if (lane == 0) {
      sd[w][2 * a] = vr;
      sd[w][2 * a + 1] = vi;
    }
  }
  __syncthreads();
  if (threadIdx.x < 2 * kFFRecv) {
    const int a = threadIdx.x >> 1;
    if (l0 + a < L) {
      double s = 0;
      for (int ww = 0; ww < kFFWarps; ww++) s += sd[ww][threadIdx.x];
      ((double*)partial)[((size_t)(l0 + a) * S + split) * 2 + (threadIdx.x & 1)] = s;
    }
  }
}

__global__ void far_reduce_kernel(const cd* __restrict__ partial, int L, int S, cd* y) {
  int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= L) return;
  double sr = 0, si = 0;
  for (int s = 0; s < S; s++) {
    sr += partial[(size_t)l * S + s].re;
    si += partial[(size_t)l * S + s].im;
  }
  y[l] = cd(sr, si);
}

// out_j = sum_l Q_lj vf_l  (plain transpose), receivers staged through shared memory
template <typename R>
__global__ void __launch_bounds__(kFFThreads) far_t_kernel(GeoView<R> G, const double4* __restrict__ recv, int L, R k,
                                                           const cd* __restrict__ vf, cd* out) {
  __shared__ double4 sp[kFFThreads];
  __shared__ cd sv[kFFThreads];
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const bool ok = j < G.ne;
  double4 va = make_double4(0, 0, 0, 0);
  ElemGeo<R> g;
  if (ok) {
    va = G.va[j];
    g = G.eg[j];
  }
  double sr = 0, si = 0;
  for (int base = 0; base < L; base += kFFThreads) {
    const int cnt = min(kFFThreads, L - base);
    __syncthreads();
    if (threadIdx.x < cnt) {
      sp[threadIdx.x] = recv[base + threadIdx.x];
      sv[threadIdx.x] = vf[base + threadIdx.x];
    }
    __syncthreads();
    if (ok) {
      R ar = 0, ai = 0;
      for (int a = 0; a < cnt; a++) {
        const double4 P = sp[a];
        cplx<R> q = entry_from_d<R>(k, (R)(P.x - va.x), (R)(P.y - va.y), (R)(P.z - va.z), g);
        const R vr = (R)sv[a].re, vi = (R)sv[a].im;
        ar += q.re * vr - q.im * vi;
        ai += q.re * vi + q.im * vr;
      }
      sr += ar;
      si += ai;
    }
  }
  if (ok) out[j] = cd(sr, si);
}

void launch_far_field(const DevGeometry& G, int prec, const double4* recv, int L, double k, const cd* x, cd* y,
                      DevBuf& scratch, cudaStream_t s) {
  const int S = std::max(1, std::min(64, (G.ne + 2047) / 2048));
  scratch.ensure((size_t)L * S * sizeof(cd), s);
  dim3 grid((L + kFFRecv - 1) / kFFRecv, S);
  note_launch();
  if (prec == PREC_FP64)
    far_kernel<double><<<grid, kFFThreads, 0, s>>>(geo_view<double>(G), recv, L, k, x, scratch.as<cd>(), S);
  else
    far_kernel<float><<<grid, kFFThreads, 0, s>>>(geo_view<float>(G), recv, L, (float)k, x, scratch.as<cd>(), S);
  AC3D_CUDA(cudaGetLastError());
  note_launch();
  far_reduce_kernel<<<(L + 127) / 128, 128, 0, s>>>(scratch.as<cd>(), L, S, y);
  AC3D_CUDA(cudaGetLastError());
}

void launch_far_field_t(const DevGeometry& G, int prec, const double4* recv, int L, double k, const cd* vf, cd* out,
                        cudaStream_t s) {
  const int nb = (G.ne + kFFThreads - 1) / kFFThreads;
  note_launch();
  if (prec == PREC_FP64)
    far_t_kernel<double><<<nb, kFFThreads, 0, s>>>(geo_view<double>(G), recv, L, k, vf, out);
  else
    far_t_kernel<float><<<nb, kFFThreads, 0, s>>>(geo_view<float>(G), recv, L, (float)k, vf, out);
  AC3D_CUDA(cudaGetLastError());
}

// yt += |y| (one frequency of a band)
__global__ void accum_abs_kernel(const cd* __restrict__ y, int L, double* yt) {
  int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l < L) yt[l] += sqrt(y[l].re * y[l].re + y[l].im * y[l].im);
}

// c and u = dc/dyt from yt (compute_u, adjoint.cpp:388-397). out: c at coef[0].
__global__ void compute_u_kernel(const double* __restrict__ yt, int L, double* u, double* coef) {
  __shared__ double s1[32], s2[32];
  double a = 0, b = 0;
  for (int l = threadIdx.x; l < L; l += blockDim.x) {
    double v = yt[l] * yt[l];
    a += v;
    b += v * v;
  }
  a = warp_sum(a);
  b = warp_sum(b);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) {
    s1[w] = a;
    s2[w] = b;
  }
  __syncthreads();
  double Ls = 0, Lsq = 0;
  for (int i = 0; i < (int)(blockDim.x >> 5); i++) {
    Ls += s1[i];
    Lsq += s2[i];
  }
  const double sq = Ls * Ls;
  if (threadIdx.x == 0) coef[0] = (sq - Lsq) / ((L - 1) * Lsq);
  if (u)
    for (int l = threadIdx.x; l < L; l += blockDim.x) {
      double v = yt[l] * yt[l];
      u[l] = 4 * (Ls * Lsq - v * sq) / ((L - 1) * Lsq * Lsq) * yt[l];
    }
}

// vf = u conj(y) / |y| (adjoint.cpp:145)
__global__ void vf_kernel(const double* __restrict__ u, const cd* __restrict__ y, int L, cd* vf) {
  int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= L) return;
  double a = sqrt(y[l].re * y[l].re + y[l].im * y[l].im);
  vf[l] = cd(u[l] * y[l].re / a, -u[l] * y[l].im / a);
}

// Low-rank receiver matrix Q ~ U V from the receiver ACA (terms u_q | v_q in a pool):
//   forward   y = U (V x)        (adjoint.cpp:101-102)
//   transpose out = V^T (U^T vf) (adjoint.cpp:198)
// Phase A: one warp per term, t_q = v_q . x (or u_q . vf); phase B: one thread per output entry.
template <typename R>
__global__ void lr_dot_kernel(const cplx<R>* __restrict__ pool, const long long* __restrict__ toff,
                              const int* __restrict__ rank, int L, int ne, const cd* __restrict__ x, int trans,
                              cd* t) {
  const int lane = threadIdx.x & 31;
  const int q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (q >= *rank) return;
  const cplx<R>* vec = pool + toff[q] + (trans ? 0 : L);
  const int len = trans ? L : ne;
  double ar = 0, ai = 0;
  for (int i = lane; i < len; i += 32) {
    const cplx<R> a = vec[i];
    const cd b = x[i];
    ar += (double)a.re * b.re - (double)a.im * b.im;
    ai += (double)a.re * b.im + (double)a.im * b.re;
  }
  ar = warp_sum(ar);
  ai = warp_sum(ai);
  if (lane == 0) t[q] = cd(ar, ai);
}

template <typename R>
__global__ void lr_expand_kernel(const cplx<R>* __restrict__ pool, const long long* __restrict__ toff,
                                 const int* __restrict__ rank, int L, int ne, const cd* __restrict__ t, int trans,
                                 cd* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int len = trans ? ne : L;
  if (i >= len) return;
  const int off = trans ? L : 0;
  const int r = *rank;
  double ar = 0, ai = 0;
  for (int q = 0; q < r; q++) {
    const cplx<R> a = pool[toff[q] + off + i];
    const cd b = t[q];
    ar += (double)a.re * b.re - (double)a.im * b.im;
    ai += (double)a.re * b.im + (double)a.im * b.re;
  }
  out[i] = cd(ar, ai);
}

void launch_lr_apply(int prec, const void* pool, const long long* toff, const int* rank, int iter_lim, int L, int ne,
                     const cd* x, int trans, cd* t, cd* out, cudaStream_t s) {
  const int nb = std::max(1, (iter_lim * 32 + 255) / 256);
  const int len = trans ? ne : L;
  if (prec == PREC_FP64) {
    note_launch();
    lr_dot_kernel<double><<<nb, 256, 0, s>>>((const cd*)pool, toff, rank, L, ne, x, trans, t);
    note_launch();
    lr_expand_kernel<double><<<(len + 255) / 256, 256, 0, s>>>((const cd*)pool, toff, rank, L, ne, t, trans, out);
  } else {
    note_launch();
    lr_dot_kernel<float><<<nb, 256, 0, s>>>((const cf*)pool, toff, rank, L, ne, x, trans, t);
    note_launch();
    lr_expand_kernel<float><<<(len + 255) / 256, 256, 0, s>>>((const cf*)pool, toff, rank, L, ne, t, trans, out);
  }
  AC3D_CUDA(cudaGetLastError());
}

void launch_accum_abs(const cd* y, int L, double* yt, cudaStream_t s) {
  note_launch();
  accum_abs_kernel<<<(L + 255) / 256, 256, 0, s>>>(y, L, yt);
  AC3D_CUDA(cudaGetLastError());
}
void launch_compute_u(const double* yt, int L, double* u, double* coef, cudaStream_t s) {
  note_launch();
  compute_u_kernel<<<1, 1024, 0, s>>>(yt, L, u, coef);
  AC3D_CUDA(cudaGetLastError());
}
void launch_vf(const double* u, const cd* y, int L, cd* vf, cudaStream_t s) {
  note_launch();
  vf_kernel<<<(L + 255) / 256, 256, 0, s>>>(u, y, L, vf);
  AC3D_CUDA(cudaGetLastError());
}

}  // namespace ac3d
