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

// ------------------------------------------------------------------------------------------
// Several plane-wave directions of one frequency at once (up to NR per launch). The shape
// derivatives of M and of the receiver matrix depend only on the geometry and k, so each
// derivative entry is evaluated once and multiplied into every direction's vectors; per
// (target, direction) the sums are reduced in the same fixed order as the single-direction path.
// ------------------------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ cplx<R> ld_c(const cd* p) {
  const cd v = *p;
  return {(R)v.re, (R)v.im};
}

template <typename R, int NR>
__global__ void __launch_bounds__(kAdjThreads) derA_multi_kernel(GeoView<R> G, AdjointMultiArgs a, double* outA) {
  const int lane = threadIdx.x & 31;
  const int t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (t >= a.npairs) return;
  const int j = a.pair_elem[t], o = a.pair_corner[t];
  const double4 va = G.va[j];
  const ElemGeo<R> g = G.eg[j];
  R sr[NR], si[NR];
#pragma unroll
  for (int r = 0; r < NR; r++) sr[r] = si[r] = 0;
  for (int l = lane; l < a.L; l += 32) {
    const double4 P = a.recv[l];
    const cplx<R> d = dM_source<R>((R)a.k, (R)(P.x - va.x), (R)(P.y - va.y), (R)(P.z - va.z), g, o);
#pragma unroll
    for (int r = 0; r < NR; r++)
      if (r < a.nr) {
        const cplx<R> v = ld_c<R>(a.vf + (size_t)r * a.L + l);
        sr[r] += d.re * v.re - d.im * v.im;
        si[r] += d.re * v.im + d.im * v.re;
      }
  }
#pragma unroll
  for (int r = 0; r < NR; r++) {
    const double vr = warp_sum((double)sr[r]), vi = warp_sum((double)si[r]);
    if (lane == 0 && r < a.nr) {
      const cd xj = a.x[(size_t)r * G.ne + j];
      outA[(size_t)t * NR + r] = vr * xj.re - vi * xj.im;
    }
  }
}

// der_B's sweeps for every direction as tiled products: a CTA takes kBT targets; per tile of kBJ
// elements every derivative entry (target, element) is evaluated once into shared memory, the
// tile's kBJ x NR vector values are staged beside it, and each thread accumulates two (target,
// direction) sums over the tile in element order. Partials per element split, summed in split
// order by the combine kernel.
namespace {
constexpr int kBT = 32;  // targets per CTA
template <typename R>
constexpr int bj() { return sizeof(R) == 4 ? 64 : 32; }  // elements per tile (FP64 tiles are half as long)
}  // namespace

// s1[(i, r)] = sum_j x_r[j] dM(c_i, tri_j)/dp_y over the touched elements i (kind 0), or
// s2[(pair, r)] = sum_j lmb_r[j] dM(c_j, tri_i)/dq_{o,y} over the incidences (i, o) (kind 1)
template <typename R, int NR, int KIND>
__global__ void __launch_bounds__(kAdjThreads) derB_tiled_kernel(GeoView<R> G, AdjointMultiArgs a, cd* part, int S) {
  static_assert(kBT * NR == 2 * kAdjThreads, "two (target, direction) sums per thread");
  constexpr int kBJ = bj<R>();
  __shared__ cplx<R> Dt[kBT][kBJ + 1];
  __shared__ cplx<R> Vt[kBJ][NR];
  __shared__ double4 Tp[kBT];     // target point (kind 0: centroid of i) or vertex a of i (kind 1)
  __shared__ ElemGeo<R> Tg[kBT];  // kind 1: geometry of i
  __shared__ int To[kBT];         // kind 1: corner o
  const int ntarget = KIND == 0 ? a.ntouch : a.npairs;
  const int t0 = blockIdx.x * kBT, split = blockIdx.y;
  const int per = (G.ne + S - 1) / S;
  const int j0 = split * per, j1 = min(G.ne, j0 + per);
  const cd* vec = KIND == 0 ? a.x : a.lmb;
  for (int p = threadIdx.x; p < kBT; p += blockDim.x) {
    const int t = min(t0 + p, ntarget - 1);
    if (KIND == 0) {
      Tp[p] = G.cen[a.touch_elem[t]];
    } else {
      const int i = a.pair_elem[t];
      Tp[p] = G.va[i];
      Tg[p] = G.eg[i];
      To[p] = a.pair_corner[t];
    }
  }
  const int p_acc = threadIdx.x / (NR / 2), r_acc = 2 * (threadIdx.x % (NR / 2));
  R ar0 = 0, ai0 = 0, ar1 = 0, ai1 = 0;
  const R k = (R)a.k;
  for (int jt = j0; jt < j1; jt += kBJ) {
    __syncthreads();  // the previous tile is consumed (and the targets are staged)
    for (int e = threadIdx.x; e < kBT * kBJ; e += blockDim.x) {
      const int p = e / kBJ, jj = e - p * kBJ, j = jt + jj;
      cplx<R> d;
      if (j < j1) {
        if (KIND == 0) {
          const double4 va = G.va[j];
          const ElemGeo<R> g = G.eg[j];
          d = dM_target<R>(k, (R)(Tp[p].x - va.x), (R)(Tp[p].y - va.y), (R)(Tp[p].z - va.z), g);
        } else {
          const double4 c = G.cen[j];
          d = dM_source<R>(k, (R)(c.x - Tp[p].x), (R)(c.y - Tp[p].y), (R)(c.z - Tp[p].z), Tg[p], To[p]);
        }
      }
      Dt[p][jj] = d;
    }
    for (int e = threadIdx.x; e < kBJ * NR; e += blockDim.x) {
      const int jj = e / NR, r = e - jj * NR, j = jt + jj;
      Vt[jj][r] = (j < j1 && r < a.nr) ? ld_c<R>(vec + (size_t)r * G.ne + j) : cplx<R>();
    }
    __syncthreads();
    const int nj = min(kBJ, j1 - jt);
    for (int jj = 0; jj < nj; jj++) {
      const cplx<R> d = Dt[p_acc][jj], v0 = Vt[jj][r_acc], v1 = Vt[jj][r_acc + 1];
      ar0 += d.re * v0.re - d.im * v0.im;
      ai0 += d.re * v0.im + d.im * v0.re;
      ar1 += d.re * v1.re - d.im * v1.im;
      ai1 += d.re * v1.im + d.im * v1.re;
    }
  }
  if (t0 + p_acc < ntarget) {
    cd* dst = part + ((size_t)(t0 + p_acc) * NR + r_acc) * S + split;
    dst[0] = cd((double)ar0, (double)ai0);
    dst[S] = cd((double)ar1, (double)ai1);
  }
}

// Per vertex h: sum over its incidences (CSR order), then over the directions, of
// w_r (A_r - B_r + C_r), with C_r of the plane wave e^{-ik d_r.x} (sphere.h:22-26 along d_r).
template <int NR>
__global__ void adj_combine_multi_kernel(AdjointMultiArgs a, const double4* __restrict__ cen,
                                         const double* __restrict__ outA, const cd* __restrict__ s1,
                                         const cd* __restrict__ s2, int S1, int S2, int ne) {
  const int h = blockIdx.x * blockDim.x + threadIdx.x;
  if (h >= a.HH) return;
  double acc = 0;
  for (int t = a.h_off[h]; t < a.h_off[h + 1]; t++) {
    const int i = a.pair_elem[t];
    const int ti = a.pair_touch[t];
    const double4 c = cen[i];
    for (int r = 0; r < a.nr; r++) {
      double s1r = 0, s1i = 0, s2r = 0, s2i = 0;
      for (int s = 0; s < S1; s++) {
        const cd v = s1[((size_t)ti * NR + r) * S1 + s];
        s1r += v.re;
        s1i += v.im;
      }
      for (int s = 0; s < S2; s++) {
        const cd v = s2[((size_t)t * NR + r) * S2 + s];
        s2r += v.re;
        s2i += v.im;
      }
      const cd li = a.lmb[(size_t)r * ne + i], xi = a.x[(size_t)r * ne + i];
      const double B = (s1r * li.re - s1i * li.im) + (s2r * xi.re - s2i * xi.im);
      const double ph = a.k * (a.dir[r][0] * c.x + a.dir[r][1] * c.y + a.dir[r][2] * c.z);
      double sn, cs;
      sincos(ph, &sn, &cs);
      const double f = -a.k * a.dir[r][1] / 3.0;
      const double C = -(f * sn * li.re - f * cs * li.im);
      acc += a.w[r] * (outA[(size_t)t * NR + r] - B + C);
    }
  }
  a.grad[h] += acc;
}

template <typename R, int NR>
static void adjoint_multi_t(const DevGeometry& G, const AdjointMultiArgs& a, DevBuf& scratch, cudaStream_t s) {
  const int sms = device_sm_count();
  const int tiles1 = (a.ntouch + kBT - 1) / kBT, tiles2 = (a.npairs + kBT - 1) / kBT;
  auto pick = [&](int tiles) { return std::max(1, std::min(256, (sms * 8 + tiles - 1) / std::max(1, tiles))); };
  const int S1 = pick(tiles1), S2 = pick(tiles2);
  const size_t bytesA = ((size_t)a.npairs * NR * sizeof(double) + 15) / 16 * 16;
  const size_t bytes1 = (size_t)a.ntouch * NR * S1 * sizeof(cd);
  const size_t bytes2 = (size_t)a.npairs * NR * S2 * sizeof(cd);
  scratch.ensure(bytesA + bytes1 + bytes2 + 64, s);
  double* outA = scratch.as<double>();
  cd* s1 = (cd*)((char*)scratch.p + bytesA);
  cd* s2 = s1 + (size_t)a.ntouch * NR * S1;
  GeoView<R> gv = geo_view<R>(G);
  note_launch();
  derA_multi_kernel<R, NR><<<(a.npairs * 32 + kAdjThreads - 1) / kAdjThreads, kAdjThreads, 0, s>>>(gv, a, outA);
  AC3D_CUDA(cudaGetLastError());
  note_launch();
  derB_tiled_kernel<R, NR, 0><<<dim3(tiles1, S1), kAdjThreads, 0, s>>>(gv, a, s1, S1);
  AC3D_CUDA(cudaGetLastError());
  note_launch();
  derB_tiled_kernel<R, NR, 1><<<dim3(tiles2, S2), kAdjThreads, 0, s>>>(gv, a, s2, S2);
  AC3D_CUDA(cudaGetLastError());
  note_launch();
  adj_combine_multi_kernel<NR><<<(a.HH + 127) / 128, 128, 0, s>>>(a, G.cen.as<double4>(), outA, s1, s2, S1, S2, G.ne);
  AC3D_CUDA(cudaGetLastError());
}

void launch_adjoint_terms_multi(const DevGeometry& G, const AdjointMultiArgs& a, DevBuf& scratch, cudaStream_t s) {
  if (a.npairs == 0 || a.HH == 0 || a.nr <= 0) return;
  if (a.nr > kAdjMaxRhs) throw Error(3, "internal: too many directions in one adjoint batch");
  if (a.prec == PREC_FP64)
    adjoint_multi_t<double, kAdjMaxRhs>(G, a, scratch, s);
  else
    adjoint_multi_t<float, kAdjMaxRhs>(G, a, scratch, s);
}

void launch_adjoint_terms(const DevGeometry& G, const AdjointArgs& a, DevBuf& scratch, cudaStream_t s) {
  if (a.npairs == 0 || a.HH == 0) return;
  if (a.prec == PREC_FP64)
    adjoint_t<double>(G, a, scratch, s);
  else
    adjoint_t<float>(G, a, scratch, s);
}

}  // namespace ac3d
