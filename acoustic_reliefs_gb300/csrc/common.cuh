// Shared device helpers for the acoustics3d GB300 kernels: complex type, quadrature rule,
// the double-layer collocation entry M(p, element) and its shape derivatives.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace ac3d {

constexpr double kPi = 3.14159265358979323846;

template <typename R>
struct alignas(2 * sizeof(R)) cplx {
  R re, im;
  __host__ __device__ cplx() : re(0), im(0) {}
  __host__ __device__ cplx(R r, R i) : re(r), im(i) {}
  template <typename S>
  __host__ __device__ explicit cplx(const cplx<S>& o) : re((R)o.re), im((R)o.im) {}
};
typedef cplx<float> cf;
typedef cplx<double> cd;

template <typename R>
__host__ __device__ __forceinline__ cplx<R> operator+(cplx<R> a, cplx<R> b) { return {a.re + b.re, a.im + b.im}; }
template <typename R>
__host__ __device__ __forceinline__ cplx<R> operator-(cplx<R> a, cplx<R> b) { return {a.re - b.re, a.im - b.im}; }
template <typename R>
__host__ __device__ __forceinline__ cplx<R> operator*(cplx<R> a, cplx<R> b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <typename R>
__host__ __device__ __forceinline__ cplx<R> operator*(R s, cplx<R> a) { return {s * a.re, s * a.im}; }
// acc += a * b
template <typename R>
__host__ __device__ __forceinline__ void cfma(cplx<R>& acc, cplx<R> a, cplx<R> b) {
  acc.re = fma(a.re, b.re, acc.re);
  acc.re = fma(-a.im, b.im, acc.re);
  acc.im = fma(a.re, b.im, acc.im);
  acc.im = fma(a.im, b.re, acc.im);
}
// acc -= a * b
template <typename R>
__host__ __device__ __forceinline__ void cfms(cplx<R>& acc, cplx<R> a, cplx<R> b) {
  acc.re = fma(-a.re, b.re, acc.re);
  acc.re = fma(a.im, b.im, acc.re);
  acc.im = fma(-a.re, b.im, acc.im);
  acc.im = fma(-a.im, b.re, acc.im);
}
template <typename R>
__host__ __device__ __forceinline__ R abs2(cplx<R> a) { return a.re * a.re + a.im * a.im; }
template <typename R>
__host__ __device__ __forceinline__ cplx<R> conj(cplx<R> a) { return {a.re, -a.im}; }
// a / b, scaled to avoid overflow in |b|^2
template <typename R>
__host__ __device__ __forceinline__ cplx<R> cdiv(cplx<R> a, cplx<R> b) {
  R s = fabs(b.re) + fabs(b.im);
  R br = b.re / s, bi = b.im / s;
  R ar = a.re / s, ai = a.im / s;
  R d = br * br + bi * bi;
  return {(ar * br + ai * bi) / d, (ai * br - ar * bi) / d};
}

__device__ __forceinline__ void sincos_(float x, float* s, float* c) { sincosf(x, s, c); }
__device__ __forceinline__ void sincos_(double x, double* s, double* c) { sincos(x, s, c); }

// Strang-Fix / Dunavant 6-point rule on the reference triangle: weight, m, n with the point
// a + m (b - a) + n (c - a). Same table and order as the reference (constants.h:39-46).
__host__ __device__ __forceinline__ constexpr double quad_w(int q) {
  return q < 3 ? 0.223381589678011 : 0.109951743655322;
}
__host__ __device__ __forceinline__ constexpr double quad_m(int q) {
  return q == 0 ? 0.445948490915965 : q == 1 ? 0.445948490915965 : q == 2 ? 0.108103018168070
       : q == 3 ? 0.091576213509771 : q == 4 ? 0.091576213509771 : 0.816847572980459;
}
__host__ __device__ __forceinline__ constexpr double quad_n(int q) {
  return q == 0 ? 0.108103018168070 : q == 1 ? 0.445948490915965 : q == 2 ? 0.445948490915965
       : q == 3 ? 0.816847572980459 : q == 4 ? 0.091576213509771 : 0.091576213509771;
}

// Per-element geometry in precision R: edge vectors ab = b - a, ac = c - a and the unnormalised
// normal n = ab x ac (|n| = twice the area), as in compute_intermediates (helpers.cpp:16-32).
template <typename R>
struct ElemGeo {
  R ab[3];
  R ac[3];
  R n[3];
};

struct Vec3d {
  double x, y, z;
};

// Geometry views handed to kernels. Positions are kept in FP64 so that differences between
// nearby points can be formed without cancellation before rounding to R.
template <typename R>
struct GeoView {
  const double4* cen;     // element centroids (collocation points), FP64
  const double4* va;      // vertex a of each element, FP64
  const ElemGeo<R>* eg;   // edge vectors and normal in R
  const float4* cen32;    // FP32 centroids (far-field rows)
  const float4* va32;     // FP32 vertex a (far-field columns)
  int ne;
};

// Double-layer kernel summed over the 6-point rule for a source element given the displacement
// d = p - a (collocation point minus the element's vertex a):
//   M = 1/2 sum_q w_q e^{-ikr}(1 + ikr) (r.n) / (4 pi r^3),   r = d - m ab - n ac,
// which is dGdr(k, r) (-(r.n)/r) of integrate.h:11-19 summed as in integrate.cpp:5-14.
template <typename R>
__device__ __forceinline__ cplx<R> entry_from_d(R k, R dx, R dy, R dz, const ElemGeo<R>& g) {
  R acc_re = 0, acc_im = 0;
#pragma unroll
  for (int q = 0; q < 6; q++) {
    const R m = (R)quad_m(q), n = (R)quad_n(q), w = (R)quad_w(q);
    R rx = dx - m * g.ab[0] - n * g.ac[0];
    R ry = dy - m * g.ab[1] - n * g.ac[1];
    R rz = dz - m * g.ab[2] - n * g.ac[2];
    R r2 = rx * rx + ry * ry + rz * rz;
    R r = sqrt(r2);
    R rinv = R(1) / r;
    R s = rx * g.n[0] + ry * g.n[1] + rz * g.n[2];
    R kr = k * r;
    R sn, cs;
    sincos_(kr, &sn, &cs);
    // e^{-ikr}(1 + ikr) = (cs + kr sn) + i (kr cs - sn)
    R f = w * s * rinv * rinv * rinv;
    acc_re += f * (cs + kr * sn);
    acc_im += f * (kr * cs - sn);
  }
  const R scale = (R)(0.5 / (4.0 * kPi));
  return {acc_re * scale, acc_im * scale};
}

// Near-field entry: displacement formed in FP64 (no cancellation for adjacent panels).
template <typename R>
__device__ __forceinline__ cplx<R> entry_near(R k, const GeoView<R>& G, double4 p, int e) {
  double4 a = G.va[e];
  ElemGeo<R> g = G.eg[e];
  return entry_from_d<R>(k, (R)(p.x - a.x), (R)(p.y - a.y), (R)(p.z - a.z), g);
}

// Far-field entry (admissible blocks, receivers): FP32 positions suffice for R = float because
// the points are separated by at least the cluster radii; FP64 positions for R = double.
template <typename R>
struct FarPt;
template <>
struct FarPt<float> {
  static __device__ __forceinline__ float4 cen(const GeoView<float>& G, int i) { return G.cen32[i]; }
  static __device__ __forceinline__ float4 va(const GeoView<float>& G, int e) { return G.va32[e]; }
};
template <>
struct FarPt<double> {
  static __device__ __forceinline__ double4 cen(const GeoView<double>& G, int i) { return G.cen[i]; }
  static __device__ __forceinline__ double4 va(const GeoView<double>& G, int e) { return G.va[e]; }
};

template <typename R, typename P4>
__device__ __forceinline__ cplx<R> entry_far(R k, const GeoView<R>& G, P4 p, int e) {
  auto a = FarPt<R>::va(G, e);
  ElemGeo<R> g = G.eg[e];
  return entry_from_d<R>(k, (R)(p.x - a.x), (R)(p.y - a.y), (R)(p.z - a.z), g);
}

// ------------------------------------------------------------------------------------------
// Shape derivatives (chain rule; the reference evaluates equivalent generated closed forms,
// derivatives.cpp:5-177). With K = F(r) s, F = e^{-ikr}(1 + ikr)/(4 pi r^3), s = r.n:
//   F'(r) = e^{-ikr} (k^2 r^2 - 3 (1 + ikr)) / (4 pi r^4).
// Target vertex y-shift moves the centroid by 1/3:  dK = F' (r_y / (3 r)) s + F n_y / 3.
// Source vertex o y-shift with barycentric weight l_o: dr = -l_o y_hat, dn = y_hat x w_o,
// w_a = b - c, w_b = c - a, w_c = a - b:  dK = F' (-l_o r_y / r) s + F (-l_o n_y + r_x w_z - r_z w_x).
// ------------------------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ void FdF(R k, R r, R& Fre, R& Fim, R& dFre, R& dFim) {
  R sn, cs;
  sincos_(k * r, &sn, &cs);
  R kr = k * r;
  R rinv = R(1) / r;
  R r3 = rinv * rinv * rinv;
  // e^{-ikr}(1 + ikr) = (cs + kr sn) + i (kr cs - sn)
  Fre = (cs + kr * sn) * r3;
  Fim = (kr * cs - sn) * r3;
  // e^{-ikr}(k^2 r^2 - 3 - 3ikr) = cs (k2r2 - 3) - 3 kr sn + i (-(k2r2-3) sn - 3 kr cs)
  R a = kr * kr - R(3);
  R r4 = r3 * rinv;
  dFre = (cs * a - R(3) * kr * sn) * r4;
  dFim = (-sn * a - R(3) * kr * cs) * r4;
}

// dM(p, element)/d(target vertex y) from the displacement d = p - a.
template <typename R>
__device__ __forceinline__ cplx<R> dM_target(R k, R dx, R dy, R dz, const ElemGeo<R>& g) {
  R are = 0, aim = 0;
#pragma unroll
  for (int q = 0; q < 6; q++) {
    const R m = (R)quad_m(q), n = (R)quad_n(q), w = (R)quad_w(q);
    R rx = dx - m * g.ab[0] - n * g.ac[0];
    R ry = dy - m * g.ab[1] - n * g.ac[1];
    R rz = dz - m * g.ab[2] - n * g.ac[2];
    R r = sqrt(rx * rx + ry * ry + rz * rz);
    R Fre, Fim, dFre, dFim;
    FdF<R>(k, r, Fre, Fim, dFre, dFim);
    R s = rx * g.n[0] + ry * g.n[1] + rz * g.n[2];
    R c1 = w * ry * s / (R(3) * r);
    R c2 = w * g.n[1] / R(3);
    are += c1 * dFre + c2 * Fre;
    aim += c1 * dFim + c2 * Fim;
  }
  const R scale = (R)(0.5 / (4.0 * kPi));
  return {are * scale, aim * scale};
}

// dM(p, element)/d(source vertex o y) from d = p - a. w = (wx, wz) of the o-th edge vector.
template <typename R>
__device__ __forceinline__ cplx<R> dM_source(R k, R dx, R dy, R dz, const ElemGeo<R>& g, int o) {
  // w_a = b - c = ab - ac, w_b = c - a = ac, w_c = a - b = -ab
  R wx = o == 0 ? g.ab[0] - g.ac[0] : (o == 1 ? g.ac[0] : -g.ab[0]);
  R wz = o == 0 ? g.ab[2] - g.ac[2] : (o == 1 ? g.ac[2] : -g.ab[2]);
  R are = 0, aim = 0;
#pragma unroll
  for (int q = 0; q < 6; q++) {
    const R m = (R)quad_m(q), n = (R)quad_n(q), w = (R)quad_w(q);
    R lam = o == 0 ? R(1) - m - n : (o == 1 ? m : n);
    R rx = dx - m * g.ab[0] - n * g.ac[0];
    R ry = dy - m * g.ab[1] - n * g.ac[1];
    R rz = dz - m * g.ab[2] - n * g.ac[2];
    R r = sqrt(rx * rx + ry * ry + rz * rz);
    R Fre, Fim, dFre, dFim;
    FdF<R>(k, r, Fre, Fim, dFre, dFim);
    R s = rx * g.n[0] + ry * g.n[1] + rz * g.n[2];
    R c1 = -w * lam * ry * s / r;
    R c2 = w * (-lam * g.n[1] + rx * wz - rz * wx);
    are += c1 * dFre + c2 * Fre;
    aim += c1 * dFim + c2 * Fim;
  }
  const R scale = (R)(0.5 / (4.0 * kPi));
  return {are * scale, aim * scale};
}

// ------------------------------------------------------------------------------------------
// Reductions
// ------------------------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

}  // namespace ac3d
