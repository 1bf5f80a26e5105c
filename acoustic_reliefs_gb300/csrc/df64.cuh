// Double-float arithmetic (an unevaluated sum hi + lo of two FP32 numbers, about 47 bits) for
// the FP64-accurate entry evaluation and ACA recursion of the mixed-precision path. Everything
// runs on the FP32 pipes: GB300's FP64 rate is a small fraction of its FP32 rate.
//
// Error-free transformations: TwoSum (Knuth, TAOCP vol. 2, 4.2.2), FastTwoSum (Dekker 1971),
// TwoProd with a fused multiply-add. The add is the "sloppy" double-float add of Hida, Li and
// Bailey (QD library report, 2001): its error is bounded by about 2^-47 (|a| + |b|), which is what
// the ACA residuals need (their accuracy is measured against the size of the block's entries,
// not of the cancelled result). Square root and reciprocal take one Newton step in double-float
// from the correctly rounded FP32 value. sin/cos use a table of e^{i 2 pi j / 256} and short
// Taylor polynomials on the remaining |s| <= pi / 256.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

namespace ac3d {

struct df64 {
  float hi, lo;
};

__host__ __device__ __forceinline__ df64 df_make(float h, float l) { return {h, l}; }

__host__ __device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
__host__ __device__ __forceinline__ void fast_two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  e = b - (s - a);
}
__host__ __device__ __forceinline__ void two_prod(float a, float b, float& p, float& e) {
  p = a * b;
  e = fmaf(a, b, -p);
}

// Nearest double-float of an FP64 value (lo carries the next 24 bits).
__host__ __device__ __forceinline__ df64 df_from_double(double x) {
  const float h = (float)x;
  return {h, (float)(x - (double)h)};
}
__host__ __device__ __forceinline__ double df_to_double(df64 a) { return (double)a.hi + (double)a.lo; }

__host__ __device__ __forceinline__ df64 df_neg(df64 a) { return {-a.hi, -a.lo}; }

__host__ __device__ __forceinline__ df64 operator+(df64 a, df64 b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  e += a.lo + b.lo;
  fast_two_sum(s, e, s, e);
  return {s, e};
}
__host__ __device__ __forceinline__ df64 operator-(df64 a, df64 b) { return a + df_neg(b); }
__host__ __device__ __forceinline__ df64 operator-(df64 a) { return df_neg(a); }
__host__ __device__ __forceinline__ df64 operator*(df64 a, df64 b) {
  float p, e;
  two_prod(a.hi, b.hi, p, e);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  fast_two_sum(p, e, p, e);
  return {p, e};
}
__host__ __device__ __forceinline__ df64 df_mul_f(df64 a, float b) {
  float p, e;
  two_prod(a.hi, b, p, e);
  e = fmaf(a.lo, b, e);
  fast_two_sum(p, e, p, e);
  return {p, e};
}
// a + float b
__host__ __device__ __forceinline__ df64 df_add_f(df64 a, float b) {
  float s, e;
  two_sum(a.hi, b, s, e);
  e += a.lo;
  fast_two_sum(s, e, s, e);
  return {s, e};
}
// a * b + c with one normalisation
__host__ __device__ __forceinline__ df64 df_fma(df64 a, df64 b, df64 c) {
  float p, e;
  two_prod(a.hi, b.hi, p, e);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  float s, t;
  two_sum(p, c.hi, s, t);
  t += e + c.lo;
  fast_two_sum(s, t, s, t);
  return {s, t};
}
__host__ __device__ __forceinline__ df64 df_sqr(df64 a) {
  float p, e;
  two_prod(a.hi, a.hi, p, e);
  e = fmaf(2.0f * a.hi, a.lo, e);
  fast_two_sum(p, e, p, e);
  return {p, e};
}
// x0^2 + x1^2 + x2^2 with one normalisation: the leading squares exactly (TwoProd), their sum by
// TwoSum, the cross terms 2 hi lo and all error terms summed in FP32. Error about 2^-47 of the
// sum, as with three double-float squares and two additions, in fewer operations. (A signed dot
// product summed this way loses accuracy under cancellation; r.n keeps the multiply-add chain.)
__host__ __device__ __forceinline__ df64 df_norm2_3(df64 x0, df64 x1, df64 x2) {
  float p0, e0, p1, e1, p2, e2;
  two_prod(x0.hi, x0.hi, p0, e0);
  two_prod(x1.hi, x1.hi, p1, e1);
  two_prod(x2.hi, x2.hi, p2, e2);
  float s, t0, t1;
  two_sum(p0, p1, s, t0);
  two_sum(s, p2, s, t1);
  const float c = fmaf(x0.hi, x0.lo, fmaf(x1.hi, x1.lo, x2.hi * x2.lo));
  float lo = ((e0 + e1) + (e2 + t0)) + fmaf(2.0f, c, t1);
  fast_two_sum(s, lo, s, lo);
  return {s, lo};
}
// t + (a b - c d) with one normalisation, for |a b|, |c d| well below |t| (the rotation of a table
// entry t by a small angle): products exact, their difference by TwoSum, the rest in FP32.
__host__ __device__ __forceinline__ df64 df_add_prod_diff(df64 t, df64 a, df64 b, df64 c, df64 d) {
  float p, pe, q, qe;
  two_prod(a.hi, b.hi, p, pe);
  two_prod(c.hi, d.hi, q, qe);
  float dd, de;
  two_sum(p, -q, dd, de);
  float lo = (pe - qe) + de + fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, -fmaf(c.hi, d.lo, c.lo * d.hi)));
  float h, he;
  two_sum(t.hi, dd, h, he);
  lo = (lo + he) + t.lo;
  fast_two_sum(h, lo, h, lo);
  return {h, lo};
}

// Multiplication by a power of two is exact.
__host__ __device__ __forceinline__ df64 df_ldexp(df64 a, float pow2) { return {a.hi * pow2, a.lo * pow2}; }

__host__ __device__ __forceinline__ df64& operator+=(df64& a, df64 b) { return a = a + b; }
__host__ __device__ __forceinline__ df64& operator-=(df64& a, df64 b) { return a = a - b; }

// Ordering of normalised double-floats (|lo| <= ulp(hi) / 2): by hi, then by lo.
__host__ __device__ __forceinline__ bool operator>(df64 a, df64 b) { return a.hi > b.hi || (a.hi == b.hi && a.lo > b.lo); }
__host__ __device__ __forceinline__ bool operator==(df64 a, df64 b) { return a.hi == b.hi && a.lo == b.lo; }
__host__ __device__ __forceinline__ bool df_is_zero(df64 a) { return a.hi == 0.0f; }

// sqrt(x), x > 0: s0 = correctly rounded FP32 root, then s0 + (x - s0^2) / (2 s0) with the
// residual formed exactly (Sterbenz: x.hi - s0^2 has no rounding error).
__host__ __device__ __forceinline__ df64 df_sqrt(df64 x) {
  const float s0 = sqrtf(x.hi);
  float p, e;
  two_prod(s0, s0, p, e);
  const float d = ((x.hi - p) - e) + x.lo;
  const float c = d * (0.5f * (1.0f / s0));  // = d * (0.5f / s0) bit for bit, a reciprocal not a division
  float h, l;
  fast_two_sum(s0, c, h, l);
  return {h, l};
}

// 1 / x: y0 = correctly rounded FP32 reciprocal, then y0 + y0 (1 - x y0).
__host__ __device__ __forceinline__ df64 df_rcp(df64 x) {
  const float y0 = 1.0f / x.hi;
  float p, e;
  two_prod(x.hi, y0, p, e);
  const float h = ((1.0f - p) - e) - x.lo * y0;
  float r, l;
  fast_two_sum(y0, y0 * h, r, l);
  return {r, l};
}

// ------------------------------------------------------------------------------------------
// cos / sin of a double-float angle t >= 0 (t below about 2^14 rad).
// t = j (2 pi / 256) + s with |s| <= pi / 256; table entry j (mod 256) holds cos and sin of
// j 2 pi / 256 as double-floats {cos.hi, cos.lo, sin.hi, sin.lo}. On |s| <= 0.0123:
//   cos s = 1 + c',  c' = -s^2/2 + s^4/24 - s^6/720   (s^8/8! < 1e-19)
//   sin s = s + s',  s' = -s^3/6 + s^5/120            (s^7/7! < 1e-17)
// The leading s^2/2 is a double-float square; the smaller terms are FP32 (their relative error
// times their size is below 1e-14). Then e^{it} = T_j + T_j (c' + i sin s).
// ------------------------------------------------------------------------------------------
constexpr int kDfTab = 256;
constexpr double kDfStep = 6.283185307179586476925286766559 / kDfTab;

__host__ __device__ __forceinline__ void df_sincos(df64 t, const float4* __restrict__ tab, df64& c, df64& s) {
  // the step 2 pi / 256 as three floats (about 72 bits)
  const float step0 = (float)kDfStep;
  const float step1 = (float)(kDfStep - (double)step0);
  const float step2 = (float)(kDfStep - (double)step0 - (double)step1);
  const float inv_step = (float)(1.0 / kDfStep);
  const float jf = rintf(t.hi * inv_step);
  // s = t - jf (step0 + step1 + step2): both products exact (p0 + e0, p1 + e1), t.hi - p0
  // exact (Sterbenz), the small terms summed as double-floats
  float p0, e0, p1, e1;
  two_prod(jf, step0, p0, e0);
  two_prod(jf, step1, p1, e1);
  df64 r{t.hi - p0, 0.0f};
  r = df_add_f(r, t.lo);
  r = df_add_f(r, -e0);
  r = df_add_f(r, -p1);
  r.lo -= e1 + jf * step2;
  float sh, sl;
  fast_two_sum(r.hi, r.lo, sh, sl);
  const df64 sv{sh, sl};
  const df64 s2 = df_sqr(sv);
  const float z = s2.hi;
  // c' = -s2/2 + z^2/24 - z^3/720 ; s' = -s z/6 + s z^2/120
  const float c_small = z * z * (1.0f / 24.0f - z * (1.0f / 720.0f));
  const df64 cp = df_add_f(df_ldexp(df_neg(s2), 0.5f), c_small);
  const float s_small = -sh * z * (1.0f / 6.0f - z * (1.0f / 120.0f));
  const df64 sn = df_add_f(sv, s_small);
  const float4 T = tab[((int)jf) & (kDfTab - 1)];
  const df64 tc{T.x, T.y}, ts{T.z, T.w};
  // cos t = Tc + (Tc c' - Ts sin s), sin t = Ts + (Ts c' + Tc sin s)
  c = df_add_prod_diff(tc, tc, cp, ts, sn);
  s = df_add_prod_diff(ts, ts, cp, df_neg(tc), sn);
}

// ------------------------------------------------------------------------------------------
// Complex double-float
// ------------------------------------------------------------------------------------------
struct cdf {
  df64 re, im;
};

__host__ __device__ __forceinline__ cdf operator+(cdf a, cdf b) { return {a.re + b.re, a.im + b.im}; }
__host__ __device__ __forceinline__ cdf operator-(cdf a, cdf b) { return {a.re - b.re, a.im - b.im}; }
__host__ __device__ __forceinline__ cdf operator*(cdf a, cdf b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
// acc -= a * b
__host__ __device__ __forceinline__ void cdf_fms(cdf& acc, cdf a, cdf b) {
  acc.re = df_fma(df_neg(a.re), b.re, acc.re);
  acc.re = df_fma(a.im, b.im, acc.re);
  acc.im = df_fma(df_neg(a.re), b.im, acc.im);
  acc.im = df_fma(df_neg(a.im), b.re, acc.im);
}
__host__ __device__ __forceinline__ df64 cdf_abs2(cdf a) { return df_sqr(a.re) + df_sqr(a.im); }
// Division by a pivot d with a power-of-two rescaling: FP32 has a far narrower exponent range
// than FP64, and |d|^2 of a small pivot would underflow. With sc = 2^-e bringing max(|Re d|,
// |Im d|) into [0.5, 1) (clamped to the normal range), a / d = (a sc) conj(w) / |w|^2, w = d sc;
// the scalings are exact.
struct CdfDivisor {
  cdf inv;  // conj(w) / |w|^2
  float sc;
};
__host__ __device__ __forceinline__ CdfDivisor cdf_divisor(cdf d) {
  const float a = fmaxf(fabsf(d.re.hi), fabsf(d.im.hi));
  int e = 0;
  frexpf(a, &e);
  e = e < -126 ? -126 : (e > 126 ? 126 : e);
  const float sc = ldexpf(1.0f, -e);
  const cdf w{df_ldexp(d.re, sc), df_ldexp(d.im, sc)};
  const df64 r = df_rcp(cdf_abs2(w));
  return {{w.re * r, df_neg(w.im * r)}, sc};
}
__host__ __device__ __forceinline__ cdf cdf_divide(cdf a, const CdfDivisor& D) {
  const cdf as{df_ldexp(a.re, D.sc), df_ldexp(a.im, D.sc)};
  return as * D.inv;
}

}  // namespace ac3d
