// Shape-derivative terms of the adjoint gradient (compute_der_A/B/C, adjoint.cpp:244-386).
//
// For every differentiable vertex h and each incidence (element i, corner o) of h:
//   A = Re( x_i sum_l vf_l dQ_li/dq_{o,y} )                     (receivers as targets)
//   B = Re( lmb_i sum_j x_j dM_ij/dp_y ) + Re( x_i sum_j lmb_j dM_ji/dq_{o,y} )
//   C = -Re( db_i/dp_y lmb_i )
// and dc/dh += A - B + C (adjoint.cpp:231). B is a dense all-pairs sweep over every element j
// exactly as in the reference (it does not use the H-matrix). The first sum of B depends only on
// the element i, so it is computed once per distinct element instead of once per incidence.
// All sweeps are tiled (8 targets per CTA, element range split across CTAs) with per-thread
// sums in the kernel precision and FP64 block/split reductions in a fixed order.
#include "common.cuh"
#include "internal.h"
#include "listener.h"

namespace ac3d {

namespace {
constexpr int kAdjThreads = 256;
constexpr int kAdjWarps = kAdjThreads / 32;
constexpr int kTile = 8;
}  // namespace

template <typename R>
GeoView<R> geo_view(const DevGeometry& G);

// A: one warp per incidence, lanes over receivers.
template <typename R>
__global__ void __launch_bounds__(kAdjThreads) derA_kernel(GeoView<R> G, AdjointArgs a, double* outA) {
  const int lane = threadIdx.x & 31;
  const int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (t >= a.npairs) return;
  const int j = a.pair_elem[t], o = a.pair_corner[t];
  const double4 va = G.va[j];
  const ElemGeo<R> g = G.eg[j];
  R sr = 0, si = 0;
  for (int l = lane; l < a.L; l += 32) {
    const double4 P = a.recv[l];
    cplx<R> d = dM_source<R>((R)a.k, (R)(P.x - va.x), (R)(P.y - va.y), (R)(P.z - va.z), g, o);
    const R vr = (R)a.vf[l].re, vi = (R)a.vf[l].im;
    sr += d.re * vr - d.im * vi;
    si += d.re * vi + d.im * vr;
  }
  double r = warp_sum((double)sr), i = warp_sum((double)si);
  if (lane == 0) {
    const cd xj = a.x[j];
    outA[t] = r * xj.re - i * xj.im;
  }
}

// s1[touch * S + split] = sum_{j in split} x_j dM(c_i, tri_j)/dp_y, i = touch_elem[touch]
template <typename R>
__global__ void __launch_bounds__(kAdjThreads) derB_s1_kernel(GeoView<R> G, AdjointArgs a, cd* part, int S) {
  __shared__ double sd[kAdjWarps][2 * kTile];
  const int t0 = blockIdx.x * kTile, split = blockIdx.y;
  const int per = (G.ne + S - 1) / S;
  const int j0 = split * per, j1 = min(G.ne, j0 + per);
  double4 C[kTile];
  for (int p = 0; p < kTile; p++) C[p] = G.cen[a.touch_elem[min(t0 + p, a.ntouch - 1)]];
  R ar[kTile], ai[kTile];
  for (int p = 0; p < kTile; p++) ar[p] = ai[p] = 0;
  const R k = (R)a.k;
  for (int j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
    const double4 va = G.va[j];
    const ElemGeo<R> g = G.eg[j];
    const R xr = (R)a.x[j].re, xi = (R)a.x[j].im;
#pragma unroll 2
    for (int p = 0; p < kTile; p++) {
      cplx<R> d = dM_target<R>(k, (R)(C[p].x - va.x), (R)(C[p].y - va.y), (R)(C[p].z - va.z), g);
      ar[p] += d.re * xr - d.im * xi;
      ai[p] += d.re * xi + d.im * xr;
    }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int p = 0; p < kTile; p++) {
    double vr = warp_sum((double)ar[p]), vi = warp_sum((double)ai[p]);
    if (lane == 0) {
      sd[w][2 * p] = vr;
      sd[w][2 * p + 1] = vi;
    }
  }
  __syncthreads();
  if (threadIdx.x < 2 * kTile) {
    const int p = threadIdx.x >> 1;
    if (t0 + p < a.ntouch) {
      double s = 0;
      for (int ww = 0; ww < kAdjWarps; ww++) s += sd[ww][threadIdx.x];
      double* dst = (double*)&part[(size_t)(t0 + p) * S + split];
      dst[threadIdx.x & 1] = s;
    }
  }
}

// s2[pair * S + split] = sum_{j in split} lmb_j dM(c_j, tri_i)/dq_{o,y}
template <typename R>
__global__ void __launch_bounds__(kAdjThreads) derB_s2_kernel(GeoView<R> G, AdjointArgs a, cd* part, int S) {
  __shared__ double sd[kAdjWarps][2 * kTile];
  const int t0 = blockIdx.x * kTile, split = blockIdx.y;
  const int per = (G.ne + S - 1) / S;
  const int j0 = split * per, j1 = min(G.ne, j0 + per);
  double4 A[kTile];
  ElemGeo<R> Eg[kTile];
  int O[kTile];
  for (int p = 0; p < kTile; p++) {
    const int t = min(t0 + p, a.npairs - 1);
    const int i = a.pair_elem[t];
    A[p] = G.va[i];
    Eg[p] = G.eg[i];
    O[p] = a.pair_corner[t];
  }
  R ar[kTile], ai[kTile];
  for (int p = 0; p < kTile; p++) ar[p] = ai[p] = 0;
  const R k = (R)a.k;
  for (int j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
    const double4 c = G.cen[j];
    const R lr = (R)a.lmb[j].re, li = (R)a.lmb[j].im;
#pragma unroll 2
    for (int p = 0; p < kTile; p++) {
      cplx<R> d = dM_source<R>(k, (R)(c.x - A[p].x), (R)(c.y - A[p].y), (R)(c.z - A[p].z), Eg[p], O[p]);
      ar[p] += d.re * lr - d.im * li;
      ai[p] += d.re * li + d.im * lr;
    }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int p = 0; p < kTile; p++) {
    double vr = warp_sum((double)ar[p]), vi = warp_sum((double)ai[p]);
    if (lane == 0) {
      sd[w][2 * p] = vr;
      sd[w][2 * p + 1] = vi;
    }
  }
  __syncthreads();
  if (threadIdx.x < 2 * kTile) {
    const int p = threadIdx.x >> 1;
    if (t0 + p < a.npairs) {
      double s = 0;
      for (int ww = 0; ww < kAdjWarps; ww++) s += sd[ww][threadIdx.x];
      double* dst = (double*)&part[(size_t)(t0 + p) * S + split];
      dst[threadIdx.x & 1] = s;
    }
  }
}

// Per incidence: A - B + C; per vertex h: sum over its incidences in CSR order.
__global__ void adj_combine_kernel(AdjointArgs a, const double4* __restrict__ cen, const double* __restrict__ outA,
                                   const cd* __restrict__ s1, const cd* __restrict__ s2, int S1, int S2) {
  const int h = blockIdx.x * blockDim.x + threadIdx.x;
  if (h >= a.HH) return;
  double acc = 0;
  for (int t = a.h_off[h]; t < a.h_off[h + 1]; t++) {
    const int i = a.pair_elem[t];
    const int ti = a.pair_touch[t];
    double s1r = 0, s1i = 0, s2r = 0, s2i = 0;
    for (int s = 0; s < S1; s++) {
      s1r += s1[(size_t)ti * S1 + s].re;
      s1i += s1[(size_t)ti * S1 + s].im;
    }
    for (int s = 0; s < S2; s++) {
      s2r += s2[(size_t)t * S2 + s].re;
      s2i += s2[(size_t)t * S2 + s].im;
    }
    const cd li = a.lmb[i], xi = a.x[i];
    const double B = (s1r * li.re - s1i * li.im) + (s2r * xi.re - s2i * xi.im);
    // C: -Re(db_i/dp_y lmb_i)
    const double4 c = cen[i];
    double dbr, dbi;
    if (a.rhs_kind == 0) {
      const double dx = c.x - a.rhs_v[0], dy = c.y - a.rhs_v[1], dz = c.z - a.rhs_v[2];
      const double R = sqrt(dx * dx + dy * dy + dz * dz);
      double sn, cs;
      sincos(a.k * R, &sn, &cs);
      // e^{-ikR}(-ikR - 1) / (4 pi R^2) * dy / (3R)
      const double f = dy / (3.0 * R) / (4.0 * kPi * R * R);
      const double kr = a.k * R;
      // (cs - i sn)(-1 - i kr) = (-cs - kr sn) + i (sn - kr cs)
      dbr = f * (-cs - kr * sn);
      dbi = f * (sn - kr * cs);
    } else {
      const double ph = a.k * (a.rhs_v[0] * c.x + a.rhs_v[1] * c.y + a.rhs_v[2] * c.z);
      double sn, cs;
      sincos(ph, &sn, &cs);
      // -ik d_y/3 (cs - i sn) = (-k d_y/3) sn + i (-k d_y / 3) cs
      const double f = -a.k * a.rhs_v[1] / 3.0;
      dbr = f * sn;
      dbi = f * cs;
    }
    const double C = -(dbr * li.re - dbi * li.im);
    acc += outA[t] - B + C;
  }
  a.grad[h] += acc;
}

template <typename R>
static void adjoint_t(const DevGeometry& G, const AdjointArgs& a, DevBuf& scratch, cudaStream_t s) {
  int dev = 0, sms = 0;
  AC3D_CUDA(cudaGetDevice(&dev));
  AC3D_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int tiles1 = (a.ntouch + kTile - 1) / kTile, tiles2 = (a.npairs + kTile - 1) / kTile;
  auto pick = [&](int tiles) { return std::max(1, std::min(256, (sms * 8 + tiles - 1) / std::max(1, tiles))); };
  const int S1 = pick(tiles1), S2 = pick(tiles2);
  size_t bytesA = (size_t)a.npairs * sizeof(double);
  size_t bytes1 = (size_t)a.ntouch * S1 * sizeof(cd);
  size_t bytes2 = (size_t)a.npairs * S2 * sizeof(cd);
  scratch.ensure(bytesA + bytes1 + bytes2 + 64, s);
  double* outA = scratch.as<double>();
  cd* s1 = (cd*)((char*)scratch.p + ((bytesA + 15) / 16) * 16);
  cd* s2 = s1 + (size_t)a.ntouch * S1;
  GeoView<R> gv = geo_view<R>(G);
  note_launch();
  derA_kernel<R><<<(a.npairs * 32 + kAdjThreads - 1) / kAdjThreads, kAdjThreads, 0, s>>>(gv, a, outA);
  AC3D_CUDA(cudaGetLastError());
  note_launch();
  derB_s1_kernel<R><<<dim3(tiles1, S1), kAdjThreads, 0, s>>>(gv, a, s1, S1);
  AC3D_CUDA(cudaGetLastError());
  note_launch();
  derB_s2_kernel<R><<<dim3(tiles2, S2), kAdjThreads, 0, s>>>(gv, a, s2, S2);
  AC3D_CUDA(cudaGetLastError());
  note_launch();
  adj_combine_kernel<<<(a.HH + 127) / 128, 128, 0, s>>>(a, G.cen.as<double4>(), outA, s1, s2, S1, S2);
  AC3D_CUDA(cudaGetLastError());
}

void launch_adjoint_terms(const DevGeometry& G, const AdjointArgs& a, DevBuf& scratch, cudaStream_t s) {
  if (a.npairs == 0 || a.HH == 0) return;
  if (a.prec == PREC_FP64)
    adjoint_t<double>(G, a, scratch, s);
  else
    adjoint_t<float>(G, a, scratch, s);
}

}  // namespace ac3d
