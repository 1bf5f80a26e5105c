// Element geometry and incident-field kernels.
//
// geometry: centroids and unnormalised normals N = (b - a) x (c - a) from vertex positions and
// tree-ordered connectivity (compute_intermediates, helpers.cpp:16-32), written in FP64 and
// rounded copies for the FP32 path.
// rhs: point source e^{-ikr}/(4 pi r) (compute_G_r, helpers.cpp:46-50) or plane wave e^{-ik d.c}
// (sphere_test::compute_b, sphere.h:22-26 with d = +x).
#include "common.cuh"
#include "entry_df.cuh"
#include "internal.h"

namespace ac3d {

__global__ void geometry_kernel(const double* __restrict__ P, const int* __restrict__ E, int ne, double4* cen,
                                double4* va, float4* cen32, float4* va32, ElemGeo<float>* eg32,
                                ElemGeo<double>* eg64, DfPt* cen_df, DfElem* el_df) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  int ia = E[3 * e], ib = E[3 * e + 1], ic = E[3 * e + 2];
  double a[3], b[3], c[3];
  for (int d = 0; d < 3; d++) {
    a[d] = P[3 * ia + d];
    b[d] = P[3 * ib + d];
    c[d] = P[3 * ic + d];
  }
  double cx = __dadd_rn(__dadd_rn(a[0], b[0]), c[0]) / 3;
  double cy = __dadd_rn(__dadd_rn(a[1], b[1]), c[1]) / 3;
  double cz = __dadd_rn(__dadd_rn(a[2], b[2]), c[2]) / 3;
  double ab[3], ac[3];
  for (int d = 0; d < 3; d++) {
    ab[d] = b[d] - a[d];
    ac[d] = c[d] - a[d];
  }
  double n0 = __dsub_rn(__dmul_rn(ac[2], ab[1]), __dmul_rn(ac[1], ab[2]));
  double n1 = __dsub_rn(__dmul_rn(ac[0], ab[2]), __dmul_rn(ac[2], ab[0]));
  double n2 = __dsub_rn(__dmul_rn(ac[1], ab[0]), __dmul_rn(ac[0], ab[1]));
  cen[e] = make_double4(cx, cy, cz, 0.0);
  va[e] = make_double4(a[0], a[1], a[2], 0.0);
  cen32[e] = make_float4((float)cx, (float)cy, (float)cz, 0.f);
  va32[e] = make_float4((float)a[0], (float)a[1], (float)a[2], 0.f);
  ElemGeo<double> g;
  ElemGeo<float> f;
  for (int d = 0; d < 3; d++) {
    g.ab[d] = ab[d];
    g.ac[d] = ac[d];
    f.ab[d] = (float)ab[d];
    f.ac[d] = (float)ac[d];
  }
  g.n[0] = n0;
  g.n[1] = n1;
  g.n[2] = n2;
  f.n[0] = (float)n0;
  f.n[1] = (float)n1;
  f.n[2] = (float)n2;
  eg64[e] = g;
  eg32[e] = f;
  // double-float copies: centroid, quadrature points a + m (b - a) + n (c - a) formed in FP64
  DfPt pd;
  pd.x = df_from_double(cx);
  pd.y = df_from_double(cy);
  pd.z = df_from_double(cz);
  pd.pad[0] = pd.pad[1] = 0.f;
  cen_df[e] = pd;
  DfElem ed;
  for (int q = 0; q < 6; q++)
    for (int d = 0; d < 3; d++) ed.yq[q][d] = df_from_double(fma(quad_n(q), ac[d], fma(quad_m(q), ab[d], a[d])));
  ed.n[0] = df_from_double(n0);
  ed.n[1] = df_from_double(n1);
  ed.n[2] = df_from_double(n2);
  ed.pad[0] = ed.pad[1] = 0.f;
  el_df[e] = ed;
}

// cos / sin of j 2 pi / 256 in FP64, stored as double-floats (the table of df_sincos)
__global__ void df_table_kernel(float4* tab) {
  const int j = threadIdx.x;
  if (j >= kDfTab) return;
  double sn, cs;
  sincos(j * kDfStep, &sn, &cs);
  const df64 c = df_from_double(cs), s = df_from_double(sn);
  tab[j] = make_float4(c.hi, c.lo, s.hi, s.lo);
}

void launch_geometry(DevGeometry& G, cudaStream_t s) {
  size_t ne = (size_t)G.ne;
  G.cen.ensure(ne * sizeof(double4), s);
  G.va.ensure(ne * sizeof(double4), s);
  G.cen32.ensure(ne * sizeof(float4), s);
  G.va32.ensure(ne * sizeof(float4), s);
  G.eg32.ensure(ne * sizeof(ElemGeo<float>), s);
  G.eg64.ensure(ne * sizeof(ElemGeo<double>), s);
  G.cen_df.ensure(ne * sizeof(DfPt), s);
  G.el_df.ensure(ne * sizeof(DfElem), s);
  if (G.df_tab.bytes == 0) {
    G.df_tab.alloc(kDfTab * sizeof(float4), s);
    note_launch();
    df_table_kernel<<<1, kDfTab, 0, s>>>(G.df_tab.as<float4>());
    AC3D_CUDA(cudaGetLastError());
  }
  int T = 256;
  note_launch();
  geometry_kernel<<<(G.ne + T - 1) / T, T, 0, s>>>(G.P.as<double>(), G.E.as<int>(), G.ne, G.cen.as<double4>(),
                                                   G.va.as<double4>(), G.cen32.as<float4>(), G.va32.as<float4>(),
                                                   G.eg32.as<ElemGeo<float>>(), G.eg64.as<ElemGeo<double>>(),
                                                   G.cen_df.as<DfPt>(), G.el_df.as<DfElem>());
  AC3D_CUDA(cudaGetLastError());
}

// The incident field is always formed in FP64 (it is the refinement right-hand side).
template <typename V>
__global__ void rhs_kernel(const double4* __restrict__ cen, int ne, double k, int kind, double vx, double vy,
                           double vz, cplx<V>* out) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  double4 c = cen[e];
  double re, im;
  if (kind == 0) {
    double dx = c.x - vx, dy = c.y - vy, dz = c.z - vz;
    double r = sqrt(dx * dx + dy * dy + dz * dz);
    double sn, cs;
    sincos(k * r, &sn, &cs);
    double f = 1.0 / (4.0 * kPi * r);
    re = cs * f;
    im = -sn * f;
  } else {
    double ph = k * (vx * c.x + vy * c.y + vz * c.z);
    double sn, cs;
    sincos(ph, &sn, &cs);
    re = cs;
    im = -sn;
  }
  out[e] = cplx<V>((V)re, (V)im);
}

void launch_rhs(const DevGeometry& G, int vec64, double k, int kind, const double* v3, void* out, cudaStream_t s) {
  int T = 256;
  int nb = (G.ne + T - 1) / T;
  note_launch();
  if (vec64)
    rhs_kernel<double><<<nb, T, 0, s>>>(G.cen.as<double4>(), G.ne, k, kind, v3[0], v3[1], v3[2], (cd*)out);
  else
    rhs_kernel<float><<<nb, T, 0, s>>>(G.cen.as<double4>(), G.ne, k, kind, v3[0], v3[1], v3[2], (cf*)out);
  AC3D_CUDA(cudaGetLastError());
}

__global__ void pack_points_kernel(const double* __restrict__ p, int n, double4* out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = make_double4(p[3 * i], p[3 * i + 1], p[3 * i + 2], 0.0);
}

void launch_pack_points(const double* p, int n, void* out, cudaStream_t s) {
  note_launch();
  pack_points_kernel<<<(n + 255) / 256, 256, 0, s>>>(p, n, (double4*)out);
  AC3D_CUDA(cudaGetLastError());
}

}  // namespace ac3d
