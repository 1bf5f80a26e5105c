// Double-float (about 47-bit) evaluation of the collocation entry M(p, element) for the
// mixed-precision path's near-field blocks and ACA rows and columns. The entries agree with the
// FP64 path's to about 1e-13 relative, so ACA picks the FP64 path's pivots and ranks, and only
// the stored factors are rounded to FP32.
//
// Per element the six quadrature points y_q = a + m_q (b - a) + n_q (c - a) are formed in FP64
// and kept as double-floats with the unnormalised normal n = (b - a) x (c - a); per collocation
// point the centroid is kept as a double-float. The entry is
//   M = 1/2 sum_q w_q e^{-ikr}(1 + ikr) (r.n) / (4 pi r^3),  r = p - y_q,
// the dGdr(k, r) (-(r.n)/r) of integrate.h:11-19 summed over the rule of integrate.cpp:5-14.
#pragma once

#include "common.cuh"
#include "df64.cuh"

namespace ac3d {

struct alignas(16) DfPt {
  df64 x, y, z;
  float pad[2];
};

struct alignas(16) DfElem {
  df64 yq[6][3];
  df64 n[3];
  float pad[2];
};
static_assert(sizeof(DfElem) == 176, "DfElem layout");
static_assert(sizeof(DfPt) == 32, "DfPt layout");

__host__ __device__ __forceinline__ cdf entry_df(df64 k, const DfPt* __restrict__ pp, const DfElem* __restrict__ ge,
                                        const float4* __restrict__ tab) {
  const DfPt p = *pp;
  const df64 nx = ge->n[0], ny = ge->n[1], nz = ge->n[2];
  df64 are{0.f, 0.f}, aim{0.f, 0.f};
#pragma unroll 1
  for (int q = 0; q < 6; q++) {
    const df64 rx = p.x - ge->yq[q][0];
    const df64 ry = p.y - ge->yq[q][1];
    const df64 rz = p.z - ge->yq[q][2];
    const df64 r2 = df_norm2_3(rx, ry, rz);
    const df64 r = df_sqrt(r2);
    const df64 rinv = df_rcp(r);
    const df64 s = df_fma(rz, nz, df_fma(ry, ny, rx * nx));
    const df64 kr = k * r;
    df64 cs, sn;
    df_sincos(kr, tab, cs, sn);
    const df64 w = q < 3 ? df_from_double(quad_w(0)) : df_from_double(quad_w(3));
    const df64 f = (s * (rinv * df_sqr(rinv))) * w;
    // e^{-ikr}(1 + ikr) = (cs + kr sn) + i (kr cs - sn)
    are = df_fma(f, df_fma(kr, sn, cs), are);
    aim = df_fma(f, df_fma(kr, cs, df_neg(sn)), aim);
  }
  const df64 scale = df_from_double(0.5 / (4.0 * kPi));
  return {are * scale, aim * scale};
}

}  // namespace ac3d
