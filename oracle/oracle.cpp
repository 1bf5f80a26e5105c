// FP64 CPU oracle for the acoustics3d BEM hot path.
//
// TEST INFRASTRUCTURE ONLY. This file restates, in plain C++17 + OpenMP with no Eigen, the
// algorithm of the reference's `acoustics3d_cpp` library so that the GPU product can be checked
// against it. Only the tests, the smoke check and the CPU-baseline leg of the benchmark load it;
// the product never does.
//
// Parity status: the reference itself cannot be compiled (its Eigen submodule is empty and no
// Eigen headers exist), so this restatement is pinned only by the analytic rigid-sphere Mie
// series known answer (misc/analytic_sphere.py:13-26) and by its own dense-versus-H-matrix
// cross-check; bit-level agreement with the reference binary is unpinned.
//
// Every function cites the reference file:line it follows (paths relative to the reference
// project root). Floating-point contraction is disabled in the build so that x86 and Arm hosts
// produce identical numbers.

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

typedef std::complex<double> cd;
const double kPi = 3.14159265358979323846;         // constants.h:12
const double kSpeedOfSound = 344.0;                 // constants.h:13

// Strang-Fix / Dunavant 6-point triangle rule (weight, m, n), as tabulated in constants.h:39-46.
const double kQuad[6][3] = {
    {0.223381589678011, 0.445948490915965, 0.108103018168070},
    {0.223381589678011, 0.445948490915965, 0.445948490915965},
    {0.223381589678011, 0.108103018168070, 0.445948490915965},
    {0.109951743655322, 0.091576213509771, 0.816847572980459},
    {0.109951743655322, 0.091576213509771, 0.091576213509771},
    {0.109951743655322, 0.816847572980459, 0.091576213509771},
};

struct V3 {
  double x, y, z;
};
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline double norm(V3 a) { return std::sqrt(dot(a, a)); }

// ---------------------------------------------------------------------------------------------
// Geometry (helpers.cpp:7-32)
// ---------------------------------------------------------------------------------------------
struct Geometry {
  int V = 0, Ne = 0;
  std::vector<double> P;  // V x 3
  std::vector<int> E;     // Ne x 3 (tree order)
  std::vector<double> C;  // Ne x 3 centroids
  std::vector<double> N;  // Ne x 3 unnormalised normals (b-a) x (c-a), |N| = 2 area
  V3 p(int v) const { return {P[3 * v], P[3 * v + 1], P[3 * v + 2]}; }
  V3 c(int e) const { return {C[3 * e], C[3 * e + 1], C[3 * e + 2]}; }
  V3 n(int e) const { return {N[3 * e], N[3 * e + 1], N[3 * e + 2]}; }
  V3 vert(int e, int o) const { return p(E[3 * e + o]); }
};

// compute_centers (helpers.cpp:7-14): (a + b + c) / 3 evaluated left to right.
void centers(const double* P, const int* E, int Ne, std::vector<double>& C) {
  C.assign(3 * (size_t)Ne, 0.0);
  for (int e = 0; e < Ne; e++)
    for (int d = 0; d < 3; d++)
      C[3 * e + d] = (P[3 * E[3 * e] + d] + P[3 * E[3 * e + 1] + d] + P[3 * E[3 * e + 2] + d]) / 3;
}

// compute_intermediates (helpers.cpp:16-32): centroids and N = ab x ac.
void intermediates(Geometry& g) {
  centers(g.P.data(), g.E.data(), g.Ne, g.C);
  g.N.assign(3 * (size_t)g.Ne, 0.0);
  for (int e = 0; e < g.Ne; e++) {
    V3 a = g.vert(e, 0), b = g.vert(e, 1), c = g.vert(e, 2);
    V3 ab = sub(b, a), ac = sub(c, a);
    g.N[3 * e + 0] = ac.z * ab.y - ac.y * ab.z;
    g.N[3 * e + 1] = ac.x * ab.z - ac.z * ab.x;
    g.N[3 * e + 2] = ac.y * ab.x - ac.x * ab.y;
  }
}

// ---------------------------------------------------------------------------------------------
// Kernel and collocation entry (integrate.h:11-19, integrate.cpp:5-14)
// ---------------------------------------------------------------------------------------------
inline cd dGdr(double k, double r) {
  const cd I(0.0, 1.0);
  return std::exp(-I * k * r) * (-I * k * r - 1.0) / (4 * kPi * r * r);
}

inline cd kernel(double k, V3 p, V3 pt, V3 nrm) {
  V3 rv = sub(p, pt);
  double rn = norm(rv);
  return dGdr(k, rn) * (-dot(rv, nrm) / rn);
}

// M(p, element e): half the 6-point sum of the double-layer kernel over element e.
cd entry(double k, V3 p, const Geometry& g, int e) {
  V3 qa = g.vert(e, 0), qb = g.vert(e, 1), qc = g.vert(e, 2), qn = g.n(e);
  V3 ab = sub(qb, qa), ac = sub(qc, qa);
  cd res = 0;
  for (int i = 0; i < 6; i++) {
    double m = kQuad[i][1], n = kQuad[i][2];
    V3 pt = {qa.x + m * ab.x + n * ac.x, qa.y + m * ab.y + n * ac.y, qa.z + m * ab.z + n * ac.z};
    res += kQuad[i][0] * kernel(k, p, pt, qn);
  }
  return res * 0.5;
}

// ---------------------------------------------------------------------------------------------
// Cluster tree and dual-tree traversal (clustertree.cpp:49-137)
// ---------------------------------------------------------------------------------------------
struct Node {
  double c[3];
  double r;
  int s, e;
  bool leaf = true;
  int left = -1, right = -1;
};

struct Tree {
  std::vector<Node> nodes;
  std::vector<int> order;  // reordering: position -> original element
  int leaf_size;

  // build_tree (clustertree.cpp:60-101): centre = mean, radius = max distance, split on the
  // longest bounding-box axis at the mean with `<` going left. Sums run in index order.
  int build(int start, const std::vector<int>& idx, const std::vector<double>& C) {
    if (idx.empty()) return -1;
    Node nd;
    int n = (int)idx.size();
    double sum[3] = {0, 0, 0};
    for (int i : idx)
      for (int d = 0; d < 3; d++) sum[d] += C[3 * i + d];
    for (int d = 0; d < 3; d++) nd.c[d] = sum[d] / n;
    double rmax = 0;
    for (int i : idx) {
      V3 dv = {C[3 * i] - nd.c[0], C[3 * i + 1] - nd.c[1], C[3 * i + 2] - nd.c[2]};
      rmax = std::max(rmax, norm(dv));
    }
    nd.r = rmax;
    nd.s = start;
    nd.e = start + n;
    int id = (int)nodes.size();
    nodes.push_back(nd);
    if (n <= leaf_size) {
      for (int i = 0; i < n; i++) order[start + i] = idx[i];
      return id;
    }
    double lo[3], hi[3];
    for (int d = 0; d < 3; d++) lo[d] = hi[d] = C[3 * idx[0] + d];
    for (int i : idx)
      for (int d = 0; d < 3; d++) {
        lo[d] = std::min(lo[d], C[3 * i + d]);
        hi[d] = std::max(hi[d], C[3 * i + d]);
      }
    int dim = 0;
    double best = hi[0] - lo[0];
    for (int d = 1; d < 3; d++)
      if (hi[d] - lo[d] > best) {
        best = hi[d] - lo[d];
        dim = d;
      }
    double gamma = nodes[id].c[dim];
    std::vector<int> L, R;
    for (int i : idx) (C[3 * i + dim] < gamma ? L : R).push_back(i);
    if (L.empty() || R.empty()) {  // degenerate split (coincident centroids): keep as a leaf
      for (int i = 0; i < n; i++) order[start + i] = idx[i];
      return id;
    }
    nodes[id].leaf = false;
    int l = build(start, L, C);
    int r = build(start + (int)L.size(), R, C);
    nodes[id].left = l;
    nodes[id].right = r;
    return id;
  }

  // dual_tree_traversal (clustertree.cpp:110-137); blocks are (rs, re, cs, ce).
  void traverse(int s, int t, double factor, std::vector<int>& direct, std::vector<int>& approx) const {
    const Node& S = nodes[s];
    const Node& T = nodes[t];
    V3 dv = {S.c[0] - T.c[0], S.c[1] - T.c[1], S.c[2] - T.c[2]};
    double dist = norm(dv);
    if (dist > factor * (S.r + T.r)) {
      approx.insert(approx.end(), {S.s, S.e, T.s, T.e});
    } else if (S.leaf && T.leaf) {
      direct.insert(direct.end(), {S.s, S.e, T.s, T.e});
    } else {
      bool split_src = T.leaf || ((S.e - S.s) > (T.e - T.s));
      if (split_src) {
        traverse(S.left, t, factor, direct, approx);
        traverse(S.right, t, factor, direct, approx);
      } else {
        traverse(s, T.left, factor, direct, approx);
        traverse(s, T.right, factor, direct, approx);
      }
    }
  }
};

struct Mesh {
  Geometry g;
  std::vector<int> order;
  std::vector<int> direct, approx;  // 4 ints per block
  std::vector<double> node_c, node_r;
  std::vector<int> node_range, node_child;
  bool tree_ok = true;
};

// ---------------------------------------------------------------------------------------------
// ACA with partial pivoting (aca.cpp:9-82 and :84-134)
// ---------------------------------------------------------------------------------------------

// argmax_abs (aca.cpp:25-36): first index of the largest |v|^2; -1 start so index 0 wins ties.
int argmax_abs(const std::vector<cd>& v) {
  int best = 0;
  double mv = -1;
  for (int i = 0; i < (int)v.size(); i++) {
    double a = std::norm(v[i]);
    if (a > mv) {
      mv = a;
      best = i;
    }
  }
  return best;
}

// argmax_abs_masked (aca.cpp:9-23): as above over indices not yet used as row pivots.
int argmax_abs_masked(const std::vector<cd>& v, const std::vector<char>& used) {
  int best = 0;
  double mv = -1;
  for (int i = 0; i < (int)v.size(); i++) {
    if (used[i]) continue;
    double a = std::norm(v[i]);
    if (a > mv) {
      mv = a;
      best = i;
    }
  }
  return best;
}

struct LowRank {
  int m = 0, n = 0, r = 0;
  std::vector<cd> U;  // column-major m x r
  std::vector<cd> V;  // row-major r x n
};

// compute_ACA_block / compute_ACA_listener. Rows are the collocation points `rowpts` (element
// centroids for boundary blocks, receivers for the listener matrix), columns are elements.
// `zero_guard` selects the boundary-block variant that keeps v unscaled when v_j == 0
// (aca.cpp:56-60); the listener variant divides unconditionally (aca.cpp:104).
LowRank aca(double k, const std::vector<V3>& rowpts, int rs, int re, const Geometry& g, int cs, int ce,
            double eps, int maxk, bool zero_guard) {
  LowRank lr;
  int M = re - rs, N = ce - cs;
  lr.m = M;
  lr.n = N;
  int iter_lim = std::min(maxk, std::min(M - 1, N - 1));
  if (iter_lim < 0) iter_lim = 0;
  std::vector<cd> U((size_t)M * iter_lim, 0.0), V((size_t)iter_lim * N, 0.0);
  std::vector<char> used(M, 0);
  used[0] = 1;
  int i = 0, iter = 0;
  double err = 0;
  std::vector<cd> v(N), u(M);
  while (iter < iter_lim) {
    for (int c = 0; c < N; c++) {
      cd acc = 0;
      for (int q = 0; q < iter; q++) acc += U[(size_t)q * M + i] * V[(size_t)q * N + c];
      v[c] = entry(k, rowpts[rs + i], g, cs + c) - acc;
    }
    int j = argmax_abs(v);
    cd vj = v[j];
    for (int c = 0; c < N; c++) V[(size_t)iter * N + c] = (zero_guard && vj == 0.0) ? v[c] : v[c] / vj;
    for (int r = 0; r < M; r++) {
      cd acc = 0;
      for (int q = 0; q < iter; q++) acc += U[(size_t)q * M + r] * V[(size_t)q * N + j];
      u[r] = entry(k, rowpts[rs + r], g, cs + j) - acc;
      U[(size_t)iter * M + r] = u[r];
    }
    double vn = 0, un = 0;
    for (int c = 0; c < N; c++) vn += std::norm(V[(size_t)iter * N + c]);
    for (int r = 0; r < M; r++) un += std::norm(u[r]);
    double dots = 0;
    for (int q = 0; q < iter; q++) {
      cd ud = 0, vd = 0;
      for (int r = 0; r < M; r++) ud += u[r] * U[(size_t)q * M + r];
      for (int c = 0; c < N; c++) vd += V[(size_t)iter * N + c] * V[(size_t)q * N + c];
      dots += std::abs(ud) * std::abs(vd);
    }
    err += un * vn + 2 * dots;
    if (std::sqrt(un * vn / err) <= eps) break;
    i = argmax_abs_masked(u, used);
    used[i] = 1;
    iter++;
  }
  lr.r = iter;
  lr.U.assign(U.begin(), U.begin() + (size_t)M * iter);
  lr.V.assign(V.begin(), V.begin() + (size_t)iter * N);
  return lr;
}

// ---------------------------------------------------------------------------------------------
// H-matrix (hmatrix.cpp:10-85, hmatrix.h:84-139)
// ---------------------------------------------------------------------------------------------
struct HMat {
  const Mesh* mesh;
  int Ne;
  double k;
  std::vector<std::vector<cd>> D;  // column-major near blocks
  std::vector<LowRank> A;
};

HMat* assemble(const Mesh* ms, double k, double aca_tol) {
  HMat* h = new HMat;
  h->mesh = ms;
  h->Ne = ms->g.Ne;
  h->k = k;
  const Geometry& g = ms->g;
  std::vector<V3> cpts(g.Ne);
  for (int e = 0; e < g.Ne; e++) cpts[e] = g.c(e);
  int nd = (int)ms->direct.size() / 4, na = (int)ms->approx.size() / 4;
  h->D.resize(nd);
  h->A.resize(na);
#pragma omp parallel for schedule(dynamic, 4)
  for (int b = 0; b < nd; b++) {
    int rs = ms->direct[4 * b], re = ms->direct[4 * b + 1], cs = ms->direct[4 * b + 2], ce = ms->direct[4 * b + 3];
    int m = re - rs, n = ce - cs;
    std::vector<cd>& blk = h->D[b];
    blk.resize((size_t)m * n);
    for (int c = 0; c < n; c++)
      for (int r = 0; r < m; r++) blk[(size_t)c * m + r] = entry(k, cpts[rs + r], g, cs + c);
  }
#pragma omp parallel for schedule(dynamic, 1)
  for (int b = 0; b < na; b++) {
    int rs = ms->approx[4 * b], re = ms->approx[4 * b + 1], cs = ms->approx[4 * b + 2], ce = ms->approx[4 * b + 3];
    h->A[b] = aca(k, cpts, rs, re, g, cs, ce, aca_tol, 100 /* APPROX_ACA_MAX_K, constants.h:16 */, true);
  }
  return h;
}

// y = (K - I/2) x or its plain (non-conjugate) transpose, blocks summed in traversal order.
void hmatvec(const HMat* h, const cd* x, cd* y, bool transposed) {
  const Mesh* ms = h->mesh;
  int Ne = h->Ne;
  for (int i = 0; i < Ne; i++) y[i] = -0.5 * x[i];
  int nd = (int)h->D.size(), na = (int)h->A.size();
  for (int b = 0; b < nd; b++) {
    int rs = ms->direct[4 * b], re = ms->direct[4 * b + 1], cs = ms->direct[4 * b + 2], ce = ms->direct[4 * b + 3];
    int m = re - rs, n = ce - cs;
    const std::vector<cd>& blk = h->D[b];
    if (!transposed) {
      for (int r = 0; r < m; r++) {
        cd acc = 0;
        for (int c = 0; c < n; c++) acc += blk[(size_t)c * m + r] * x[cs + c];
        y[rs + r] += acc;
      }
    } else {
      for (int c = 0; c < n; c++) {
        cd acc = 0;
        for (int r = 0; r < m; r++) acc += blk[(size_t)c * m + r] * x[rs + r];
        y[cs + c] += acc;
      }
    }
  }
  std::vector<cd> t;
  for (int b = 0; b < na; b++) {
    int rs = ms->approx[4 * b], cs = ms->approx[4 * b + 2];
    const LowRank& lr = h->A[b];
    t.assign(lr.r, 0.0);
    if (!transposed) {
      for (int q = 0; q < lr.r; q++)
        for (int c = 0; c < lr.n; c++) t[q] += lr.V[(size_t)q * lr.n + c] * x[cs + c];
      for (int r = 0; r < lr.m; r++) {
        cd acc = 0;
        for (int q = 0; q < lr.r; q++) acc += lr.U[(size_t)q * lr.m + r] * t[q];
        y[rs + r] += acc;
      }
    } else {
      for (int q = 0; q < lr.r; q++)
        for (int r = 0; r < lr.m; r++) t[q] += lr.U[(size_t)q * lr.m + r] * x[rs + r];
      for (int c = 0; c < lr.n; c++) {
        cd acc = 0;
        for (int q = 0; q < lr.r; q++) acc += lr.V[(size_t)q * lr.n + c] * t[q];
        y[cs + c] += acc;
      }
    }
  }
}

// ---------------------------------------------------------------------------------------------
// BiCGSTAB: van der Vorst (1992), zero initial guess, stop when ||r|| <= tol ||b|| on the
// recursively updated residual, no preconditioner. This is how the reference configures
// Eigen::BiCGSTAB (adjoint.cpp:92-95); Eigen's own source is not available here.
// ---------------------------------------------------------------------------------------------
inline cd cdot(const std::vector<cd>& a, const std::vector<cd>& b) {  // sum conj(a) b
  cd s = 0;
  for (size_t i = 0; i < a.size(); i++) s += std::conj(a[i]) * b[i];
  return s;
}
inline double nrm2(const std::vector<cd>& a) {
  double s = 0;
  for (const cd& v : a) s += std::norm(v);
  return s;
}

int bicgstab(const HMat* h, const cd* b, cd* xout, double tol, int maxit, bool transposed, double* err_out) {
  int n = h->Ne;
  std::vector<cd> x(n, 0.0), r(b, b + n), rhat(b, b + n), p(n, 0.0), v(n, 0.0), s(n), t(n);
  double bn2 = nrm2(r);
  if (bn2 == 0) {
    std::fill(xout, xout + n, cd(0));
    if (err_out) *err_out = 0;
    return 0;
  }
  double tol2 = tol * tol * bn2;
  cd rho = 1, alpha = 1, omega = 1;
  int it = 0;
  while (nrm2(r) > tol2 && it < maxit) {
    cd rho_old = rho;
    rho = cdot(rhat, r);
    if (std::abs(rho) < 1e-300 * nrm2(rhat) || std::abs(rho) == 0.0) {  // breakdown: fresh shadow residual
      rhat = r;
      rho = cdot(rhat, r);
      std::fill(p.begin(), p.end(), cd(0));
      std::fill(v.begin(), v.end(), cd(0));
      rho_old = alpha = omega = 1;
    }
    cd beta = (rho / rho_old) * (alpha / omega);
    for (int i = 0; i < n; i++) p[i] = r[i] + beta * (p[i] - omega * v[i]);
    hmatvec(h, p.data(), v.data(), transposed);
    alpha = rho / cdot(rhat, v);
    for (int i = 0; i < n; i++) s[i] = r[i] - alpha * v[i];
    hmatvec(h, s.data(), t.data(), transposed);
    double tt = nrm2(t);
    omega = tt > 0 ? cdot(t, s) / tt : cd(0);
    for (int i = 0; i < n; i++) {
      x[i] += alpha * p[i] + omega * s[i];
      r[i] = s[i] - omega * t[i];
    }
    it++;
  }
  std::copy(x.begin(), x.end(), xout);
  if (err_out) *err_out = std::sqrt(nrm2(r) / bn2);
  return it;
}

// ---------------------------------------------------------------------------------------------
// Shape derivatives of M with respect to vertex y-coordinates. The reference evaluates
// code-generated closed forms (derivatives.cpp:5-177); these are the same derivatives written
// from the chain rule: K = F(r) s with F(r) = e^{-ikr}(1+ikr)/(4 pi r^3), s = (p - y).N, and
// F'(r) = e^{-ikr}(k^2 r^2 - 3(1+ikr))/(4 pi r^4).
// ---------------------------------------------------------------------------------------------
inline void FdF(double k, double r, cd& F, cd& dF) {
  const cd I(0.0, 1.0);
  cd e = std::exp(-I * k * r);
  double r2 = r * r;
  F = e * (1.0 + I * k * r) / (4 * kPi * r2 * r);
  dF = e * (k * k * r2 - 3.0 * (1.0 + I * k * r)) / (4 * kPi * r2 * r2);
}

// dM(p, tri q)/d p_y where p is the centroid of a target triangle and one of its vertices moves
// (dMij_dpy, derivatives.cpp:147-153): the centroid moves by 1/3.
cd dM_dtarget_y(double k, V3 p, V3 qa, V3 qb, V3 qc) {
  V3 ab = sub(qb, qa), ac = sub(qc, qa);
  V3 N = {ac.z * ab.y - ac.y * ab.z, ac.x * ab.z - ac.z * ab.x, ac.y * ab.x - ac.x * ab.y};
  cd res = 0;
  for (int i = 0; i < 6; i++) {
    double m = kQuad[i][1], n = kQuad[i][2];
    V3 pt = {qa.x + m * ab.x + n * ac.x, qa.y + m * ab.y + n * ac.y, qa.z + m * ab.z + n * ac.z};
    V3 rv = sub(p, pt);
    double r = norm(rv);
    cd F, dF;
    FdF(k, r, F, dF);
    double s = dot(rv, N);
    res += kQuad[i][0] * (dF * (rv.y / (3.0 * r)) * s + F * (N.y / 3.0));
  }
  return 0.5 * res;
}

// dM(p, tri q)/d q_{o,y} for source-vertex o (dMij_dq{1,2,3}y, derivatives.cpp:155-177).
cd dM_dsource_y(double k, V3 p, V3 qa, V3 qb, V3 qc, int o) {
  V3 ab = sub(qb, qa), ac = sub(qc, qa);
  V3 N = {ac.z * ab.y - ac.y * ab.z, ac.x * ab.z - ac.z * ab.x, ac.y * ab.x - ac.x * ab.y};
  V3 w = o == 0 ? sub(qb, qc) : (o == 1 ? sub(qc, qa) : sub(qa, qb));  // dN/dq_{o,y} = y_hat x w
  cd res = 0;
  for (int i = 0; i < 6; i++) {
    double m = kQuad[i][1], n = kQuad[i][2];
    double lam = o == 0 ? 1.0 - m - n : (o == 1 ? m : n);
    V3 pt = {qa.x + m * ab.x + n * ac.x, qa.y + m * ab.y + n * ac.y, qa.z + m * ab.z + n * ac.z};
    V3 rv = sub(p, pt);
    double r = norm(rv);
    cd F, dF;
    FdF(k, r, F, dF);
    double s = dot(rv, N);
    double ds = -lam * N.y + rv.x * w.z - rv.z * w.x;
    res += kQuad[i][0] * (dF * (-lam * rv.y / r) * s + F * ds);
  }
  return 0.5 * res;
}

// d b_i / d p_y for the point-source right-hand side b = e^{-ikR}/(4 pi R) (dbi_dpy,
// derivatives.cpp:133-145), or for a plane wave b = e^{-ik d.c}.
cd db_dy(double k, V3 c, const double* src, int kind) {
  const cd I(0.0, 1.0);
  if (kind == 0) {
    V3 d = {c.x - src[0], c.y - src[1], c.z - src[2]};
    double R = norm(d);
    return std::exp(-I * k * R) * (-I * k * R - 1.0) / (4 * kPi * R * R) * (d.y / (3.0 * R));
  }
  double ph = k * (src[0] * c.x + src[1] * c.y + src[2] * c.z);
  return -I * k * (src[1] / 3.0) * std::exp(-I * ph);
}

}  // namespace

// =============================================================================================
// C interface used by the Python test wrapper (ctypes). Complex vectors are interleaved doubles.
// =============================================================================================
extern "C" {

double orc_wavenumber(double f) { return 2 * kPi * f / kSpeedOfSound; }  // helpers.h:8

int orc_num_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

// DiffBEM::set_mesh (acoustics3d.cpp:36-67): tree on centroids, Es permuted by tree order,
// block lists from the dual traversal. Ps is never permuted.
void* orc_mesh_new(const double* Ps, int V, const int* Es, int Ne, int leaf, double factor) {
  Mesh* ms = new Mesh;
  std::vector<double> C;
  centers(Ps, Es, Ne, C);
  Tree tr;
  tr.leaf_size = leaf;
  tr.order.assign(Ne, 0);
  std::vector<int> idx(Ne);
  std::iota(idx.begin(), idx.end(), 0);
  tr.build(0, idx, C);
  ms->order = tr.order;
  ms->g.V = V;
  ms->g.Ne = Ne;
  ms->g.P.assign(Ps, Ps + 3 * (size_t)V);
  ms->g.E.resize(3 * (size_t)Ne);
  for (int i = 0; i < Ne; i++)
    for (int d = 0; d < 3; d++) ms->g.E[3 * i + d] = Es[3 * tr.order[i] + d];
  intermediates(ms->g);
  // ClusterTree::check (clustertree.cpp:33-47) on the reordered centroids
  for (const Node& nd : tr.nodes)
    for (int i = nd.s; i < nd.e; i++) {
      V3 dv = {ms->g.C[3 * i] - nd.c[0], ms->g.C[3 * i + 1] - nd.c[1], ms->g.C[3 * i + 2] - nd.c[2]};
      if (!(norm(dv) <= nd.r + 1e-6)) ms->tree_ok = false;
    }
  tr.traverse(0, 0, factor, ms->direct, ms->approx);
  for (const Node& nd : tr.nodes) {
    ms->node_c.insert(ms->node_c.end(), {nd.c[0], nd.c[1], nd.c[2]});
    ms->node_r.push_back(nd.r);
    ms->node_range.insert(ms->node_range.end(), {nd.s, nd.e});
    ms->node_child.insert(ms->node_child.end(), {nd.left, nd.right});
  }
  return ms;
}

void orc_mesh_free(void* m) { delete (Mesh*)m; }
int orc_mesh_tree_ok(void* m) { return ((Mesh*)m)->tree_ok ? 1 : 0; }
void orc_mesh_counts(void* m, int* nd, int* na, int* nnodes) {
  Mesh* ms = (Mesh*)m;
  *nd = (int)ms->direct.size() / 4;
  *na = (int)ms->approx.size() / 4;
  *nnodes = (int)ms->node_r.size();
}
void orc_mesh_get(void* m, int* order, int* Es, int* direct, int* approx) {
  Mesh* ms = (Mesh*)m;
  std::copy(ms->order.begin(), ms->order.end(), order);
  std::copy(ms->g.E.begin(), ms->g.E.end(), Es);
  std::copy(ms->direct.begin(), ms->direct.end(), direct);
  std::copy(ms->approx.begin(), ms->approx.end(), approx);
}
void orc_mesh_nodes(void* m, double* c, double* r, int* range, int* child) {
  Mesh* ms = (Mesh*)m;
  std::copy(ms->node_c.begin(), ms->node_c.end(), c);
  std::copy(ms->node_r.begin(), ms->node_r.end(), r);
  std::copy(ms->node_range.begin(), ms->node_range.end(), range);
  std::copy(ms->node_child.begin(), ms->node_child.end(), child);
}
// Replace vertex positions (height updates keep the block partition, acoustics3d.cpp:139-146).
void orc_mesh_set_points(void* m, const double* Ps) {
  Mesh* ms = (Mesh*)m;
  ms->g.P.assign(Ps, Ps + 3 * (size_t)ms->g.V);
  intermediates(ms->g);
}
void orc_mesh_geometry(void* m, double* C, double* N) {
  Mesh* ms = (Mesh*)m;
  std::copy(ms->g.C.begin(), ms->g.C.end(), C);
  std::copy(ms->g.N.begin(), ms->g.N.end(), N);
}

// compute_G_r (helpers.cpp:46-50) for kind 0 (point source at src), or a plane wave
// e^{-ik d.c} along unit direction d = src for kind 1 (sphere.h:22-26 uses d = +x).
void orc_rhs(void* m, double k, const double* src, int kind, double* out) {
  Mesh* ms = (Mesh*)m;
  const cd I(0.0, 1.0);
  for (int e = 0; e < ms->g.Ne; e++) {
    V3 c = ms->g.c(e);
    cd v;
    if (kind == 0) {
      V3 d = {c.x - src[0], c.y - src[1], c.z - src[2]};
      double r = norm(d);
      v = std::exp(-I * k * r) / (4 * kPi * r);
    } else {
      v = std::exp(-I * k * (src[0] * c.x + src[1] * c.y + src[2] * c.z));
    }
    out[2 * e] = v.real();
    out[2 * e + 1] = v.imag();
  }
}

// Single entries M(p_i, element j) in tree order, i and j given as index lists.
void orc_entries(void* m, double k, int n, const int* rows, const int* cols, double* out) {
  Mesh* ms = (Mesh*)m;
#pragma omp parallel for
  for (int t = 0; t < n; t++) {
    cd v = entry(k, ms->g.c(rows[t]), ms->g, cols[t]);
    out[2 * t] = v.real();
    out[2 * t + 1] = v.imag();
  }
}

// Dense boundary matrix (integrate.cpp:32-44) including the -I/2 jump, row-major Ne x Ne.
void orc_dense_boundary(void* m, double k, double* out) {
  Mesh* ms = (Mesh*)m;
  int Ne = ms->g.Ne;
#pragma omp parallel for
  for (int i = 0; i < Ne; i++)
    for (int j = 0; j < Ne; j++) {
      cd v = entry(k, ms->g.c(i), ms->g, j);
      if (i == j) v -= 0.5;
      out[2 * ((size_t)i * Ne + j)] = v.real();
      out[2 * ((size_t)i * Ne + j) + 1] = v.imag();
    }
}

// Dense listener matrix (integrate.cpp:46-57), row-major L x Ne.
void orc_dense_listener(void* m, double k, const double* Ls, int L, double* out) {
  Mesh* ms = (Mesh*)m;
  int Ne = ms->g.Ne;
#pragma omp parallel for
  for (int l = 0; l < L; l++)
    for (int j = 0; j < Ne; j++) {
      cd v = entry(k, V3{Ls[3 * l], Ls[3 * l + 1], Ls[3 * l + 2]}, ms->g, j);
      out[2 * ((size_t)l * Ne + j)] = v.real();
      out[2 * ((size_t)l * Ne + j) + 1] = v.imag();
    }
}

void* orc_hmat_new(void* m, double k, double aca_tol) { return assemble((Mesh*)m, k, aca_tol); }
void orc_hmat_free(void* h) { delete (HMat*)h; }
void orc_hmat_ranks(void* h, int* ranks) {
  HMat* hm = (HMat*)h;
  for (size_t b = 0; b < hm->A.size(); b++) ranks[b] = hm->A[b].r;
}
// Low-rank factors of approx block b: U column-major (m x r), V row-major (r x n).
void orc_hmat_block_factors(void* h, int b, double* U, double* V) {
  HMat* hm = (HMat*)h;
  const LowRank& lr = hm->A[b];
  std::memcpy(U, lr.U.data(), lr.U.size() * sizeof(cd));
  std::memcpy(V, lr.V.data(), lr.V.size() * sizeof(cd));
}
void orc_hmat_matvec(void* h, const double* x, double* y, int transposed) {
  hmatvec((HMat*)h, (const cd*)x, (cd*)y, transposed != 0);
}
int orc_bicgstab(void* h, const double* b, double* x, double tol, int maxit, int transposed, double* err) {
  return bicgstab((HMat*)h, (const cd*)b, (cd*)x, tol, maxit, transposed != 0, err);
}

// Listener matrix Q (L x Ne) by ACA (compute_ACA_listener, aca.cpp:84-134; Q_ACA_MAX_K = 5000).
void* orc_listener_new(void* m, double k, const double* Ls, int L, double tol) {
  Mesh* ms = (Mesh*)m;
  std::vector<V3> pts(L);
  for (int l = 0; l < L; l++) pts[l] = {Ls[3 * l], Ls[3 * l + 1], Ls[3 * l + 2]};
  LowRank* lr = new LowRank(aca(k, pts, 0, L, ms->g, 0, ms->g.Ne, tol, 5000, false));
  return lr;
}
void orc_listener_free(void* q) { delete (LowRank*)q; }
int orc_listener_rank(void* q) { return ((LowRank*)q)->r; }
// y = U (V x) (adjoint.cpp:101-102), or out = V^T (U^T v) (adjoint.cpp:198).
void orc_listener_apply(void* q, const double* xin, double* yout, int transposed) {
  LowRank* lr = (LowRank*)q;
  const cd* x = (const cd*)xin;
  cd* y = (cd*)yout;
  std::vector<cd> t(lr->r, 0.0);
  if (!transposed) {
    for (int a = 0; a < lr->r; a++)
      for (int c = 0; c < lr->n; c++) t[a] += lr->V[(size_t)a * lr->n + c] * x[c];
    for (int r = 0; r < lr->m; r++) {
      cd acc = 0;
      for (int a = 0; a < lr->r; a++) acc += lr->U[(size_t)a * lr->m + r] * t[a];
      y[r] = acc;
    }
  } else {
    for (int a = 0; a < lr->r; a++)
      for (int r = 0; r < lr->m; r++) t[a] += lr->U[(size_t)a * lr->m + r] * x[r];
    for (int c = 0; c < lr->n; c++) {
      cd acc = 0;
      for (int a = 0; a < lr->r; a++) acc += lr->V[(size_t)a * lr->n + c] * t[a];
      y[c] = acc;
    }
  }
}

// compute_u (adjoint.cpp:388-397): returns c, writes u (L reals).
double orc_compute_u(int L, const double* yt, double* u) {
  double Ls = 0, Lsq = 0;
  for (int l = 0; l < L; l++) {
    double v = yt[l] * yt[l];
    Ls += v;
    Lsq += v * v;
  }
  double sq = Ls * Ls;
  double c = (sq - Lsq) / ((L - 1) * Lsq);
  for (int l = 0; l < L; l++) {
    double v = yt[l] * yt[l];
    u[l] = 4 * (Ls * Lsq - v * sq) / ((L - 1) * Lsq * Lsq) * yt[l];
  }
  return c;
}

// Incidence lists (set_diff_points, acoustics3d.cpp:69-101) in CSR form: for differentiable
// point h, pairs (element, corner) in offsets[h]..offsets[h+1].

// compute_der_A (adjoint.cpp:244-289).
void orc_der_A(void* m, double k, const double* Ls, int L, int HH, const int* off, const int* pairs,
               const double* vf, const double* x, double* out) {
  Mesh* ms = (Mesh*)m;
  const cd* VF = (const cd*)vf;
  const cd* X = (const cd*)x;
#pragma omp parallel for schedule(dynamic, 8)
  for (int h = 0; h < HH; h++) {
    double acc = 0;
    for (int t = off[h]; t < off[h + 1]; t++) {
      int j = pairs[2 * t], o = pairs[2 * t + 1];
      V3 q1 = ms->g.vert(j, 0), q2 = ms->g.vert(j, 1), q3 = ms->g.vert(j, 2);
      cd res = 0;
      for (int l = 0; l < L; l++)
        res += VF[l] * dM_dsource_y(k, V3{Ls[3 * l], Ls[3 * l + 1], Ls[3 * l + 2]}, q1, q2, q3, o);
      acc += (res * X[j]).real();
    }
    out[h] = acc;
  }
}

// compute_der_B (adjoint.cpp:291-352): dense all-pairs sum.
void orc_der_B(void* m, double k, int HH, const int* off, const int* pairs, const double* lmb,
               const double* x, double* out) {
  Mesh* ms = (Mesh*)m;
  const cd* LM = (const cd*)lmb;
  const cd* X = (const cd*)x;
  int Ne = ms->g.Ne;
  int npairs = off[HH];
  std::vector<double> per(npairs);
#pragma omp parallel for schedule(dynamic, 4)
  for (int t = 0; t < npairs; t++) {
    int i = pairs[2 * t], o = pairs[2 * t + 1];
    V3 ci = ms->g.c(i);
    V3 p1 = ms->g.vert(i, 0), p2 = ms->g.vert(i, 1), p3 = ms->g.vert(i, 2);
    cd s1 = 0, s2 = 0;
    for (int j = 0; j < Ne; j++) {
      V3 q1 = ms->g.vert(j, 0), q2 = ms->g.vert(j, 1), q3 = ms->g.vert(j, 2);
      s1 += X[j] * dM_dtarget_y(k, ci, q1, q2, q3);
      s2 += LM[j] * dM_dsource_y(k, ms->g.c(j), p1, p2, p3, o);
    }
    per[t] = (s1 * LM[i]).real() + (s2 * X[i]).real();
  }
  for (int h = 0; h < HH; h++) {
    double acc = 0;
    for (int t = off[h]; t < off[h + 1]; t++) acc += per[t];
    out[h] = acc;
  }
}

// compute_der_C (adjoint.cpp:354-386): out[h] = -sum Re(db_i/dp_y lambda_i).
void orc_der_C(void* m, double k, const double* src, int kind, int HH, const int* off, const int* pairs,
               const double* lmb, double* out) {
  Mesh* ms = (Mesh*)m;
  const cd* LM = (const cd*)lmb;
  for (int h = 0; h < HH; h++) {
    double acc = 0;
    for (int t = off[h]; t < off[h + 1]; t++) {
      int i = pairs[2 * t];
      acc -= (db_dy(k, ms->g.c(i), src, kind) * LM[i]).real();
    }
    out[h] = acc;
  }
}

// Pointwise derivative helpers exposed for finite-difference tests.
void orc_dM_dtarget_y(double k, const double* p, const double* q, double* out) {
  cd v = dM_dtarget_y(k, V3{p[0], p[1], p[2]}, V3{q[0], q[1], q[2]}, V3{q[3], q[4], q[5]}, V3{q[6], q[7], q[8]});
  out[0] = v.real();
  out[1] = v.imag();
}
void orc_dM_dsource_y(double k, const double* p, const double* q, int o, double* out) {
  cd v = dM_dsource_y(k, V3{p[0], p[1], p[2]}, V3{q[0], q[1], q[2]}, V3{q[3], q[4], q[5]}, V3{q[6], q[7], q[8]}, o);
  out[0] = v.real();
  out[1] = v.imag();
}
void orc_entry_pt(double k, const double* p, const double* q, double* out) {
  Geometry g;
  g.V = 3;
  g.Ne = 1;
  g.P.assign(q, q + 9);
  g.E = {0, 1, 2};
  intermediates(g);
  cd v = entry(k, V3{p[0], p[1], p[2]}, g, 0);
  out[0] = v.real();
  out[1] = v.imag();
}

}  // extern "C"
