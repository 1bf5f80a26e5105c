// Device-resident GMRES (Saad and Schultz 1986): Arnoldi with classical Gram-Schmidt and Givens
// rotations, one cycle of at most m iterations per call. An option beside the reference's
// BiCGSTAB (Eigen::BiCGSTAB at adjoint.cpp:92-95 and acoustics3d.cpp:266-269): it solves the same
// system to the same relative residual with one matvec per iteration instead of two. Restarts are
// the caller's refinement loop: when the basis fills before the tolerance is met, the caller forms
// the true residual and runs another cycle on it.
//
// Storage: the basis vectors are kept unnormalised, V_k stored with its scale s_k = 1 / |V_k|, so
// that the vector the update pass writes is the next matvec's input without a normalisation pass:
//   W = A V_j;  h_kj = s_k s_j (V_k^H W);  V_{j+1} = s_j W - sum_k (h_kj s_k) V_k;
//   h_{j+1,j} = |V_{j+1}|,  s_{j+1} = 1 / h_{j+1,j}.
// Per iteration: the matvec (into W), then the Gram-Schmidt kernel and the Givens step (rotation
// of the new Hessenberg column, residual estimate |g_{j+1}|, stop test). FP32 cycles need a second
// Gram-Schmidt pass (one loses orthogonality over long cycles); they run it delayed by one
// iteration (k_gm_dcgs, below), with the basis stored normalised. FP64 cycles take one classical
// pass (k_gm_fused). When a batch cannot have all its CTAs resident at once, separate dot and
// update kernels with last-CTA reductions (two classical passes for FP32) run instead. Vectors and
// their arithmetic, the dots and the norms are in the solve's vector type (FP32 for the
// mixed-precision inner solve, FP64 for the FP64 solve); the Hessenberg matrix, the rotations and
// the scalars are FP64. No atomics touch floating-point sums, so a solve is bit-reproducible.
//
// Batches: the kernels take the cycle as the grid's y index, so nrb independent cycles (one per
// right-hand side of a block solve) run together and share each block matvec; their inputs and
// outputs are element-major block vectors (stride nrb).
//
// The Givens step (norm, rotation of the new column, residual estimate, stop test) is serial work
// of one CTA, about 10 us per iteration on the 20k relief. Where the fused cooperative kernel runs,
// it goes either to a kernel of its own on a forked graph branch (k_gm_rotate), overlapping the
// next matvec, which needs only V_{j+1}, and joined before the next Gram-Schmidt kernel; or, in
// a request server's slots, to one extra CTA of the fused kernel that starts it while the element
// CTAs run the last update. Either way the arithmetic and its order are the same, so the results
// are bitwise the same.
#include <algorithm>
#include <mutex>

#include "common.cuh"
#include "df64.cuh"
#include "gmres.h"
#include "internal.h"
#include "krylov.h"
#include "launch.cuh"
#include "multi.h"

namespace ac3d {

namespace {
constexpr int kGmThreads = 256;
constexpr int kGmWarps = kGmThreads / 32;
constexpr int kSliceMax = 1024;  // elements per CTA of the dot and update passes
constexpr int kGmMaxRestart = 600;  // longest cycle (ac3d_set_krylov accepts up to 600)

struct Dc {  // complex FP64 scalar arithmetic of the small dense part
  double re, im;
};
__device__ __forceinline__ Dc dc(double r, double i) { return Dc{r, i}; }
__device__ __forceinline__ Dc operator*(Dc a, Dc b) { return Dc{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__device__ __forceinline__ Dc operator+(Dc a, Dc b) { return Dc{a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ Dc operator-(Dc a, Dc b) { return Dc{a.re - b.re, a.im - b.im}; }
__device__ __forceinline__ Dc conjd(Dc a) { return Dc{a.re, -a.im}; }
__device__ __forceinline__ double abs2(Dc a) { return a.re * a.re + a.im * a.im; }
}  // namespace

// FP64 arrays of a cycle, after the state struct (offsets in doubles).
struct GmLayout {
  int m, G;
  __host__ __device__ size_t s() const { return 0; }                                     // m + 1
  __host__ __device__ size_t hcol() const { return (size_t)m + 1; }                      // 2 (m + 1)
  __host__ __device__ size_t coef() const { return hcol() + 2 * ((size_t)m + 1); }       // 2 (m + 1)
  __host__ __device__ size_t g() const { return coef() + 2 * ((size_t)m + 1); }          // 2 (m + 1)
  __host__ __device__ size_t cs() const { return g() + 2 * ((size_t)m + 1); }            // 2 m
  __host__ __device__ size_t sn() const { return cs() + 2 * (size_t)m; }                 // 2 m
  __host__ __device__ size_t R() const { return sn() + 2 * (size_t)m; }                  // 2 m m
  __host__ __device__ size_t part() const { return R() + 2 * (size_t)m * m; }            // 2 (m + 1) G
  __host__ __device__ size_t npart() const { return part() + 2 * ((size_t)m + 1) * G; }  // G
  __host__ __device__ size_t part2() const { return npart() + (size_t)G; }               // 2 (m + 1) G
  __host__ __device__ size_t h2() const { return part2() + 2 * ((size_t)m + 1) * G; }     // 2 (m + 1)
  __host__ __device__ size_t abpart() const { return h2() + 2 * ((size_t)m + 1); }      // 3 G
  __host__ __device__ size_t ab() const { return abpart() + 3 * (size_t)G; }             // 4
  __host__ __device__ size_t total() const { return ab() + 4; }
};

// Column r = blockIdx.y of a batch: its state, scalars and basis.
struct GmCols {
  GState* st;
  GMulti* gm;
  double* gd;
  size_t gds;  // doubles per column
  size_t Vs;   // basis elements per column
  int vs;      // element stride of the block vectors
};

// Ends the cycle of this column with `code` (once) and counts it towards the batch's completion
// (the batch is the grid's y extent).
__device__ __forceinline__ void gm_mark_done(GState* st, GMulti* gm, int code) {
  if (st->done || !code) return;
  st->done = code;
  __threadfence();
  if (atomicAdd(&gm->ndone, 1) == (int)gridDim.y - 1) gm->done_all = 1;
}

// Contiguous element range of this CTA.
__device__ __forceinline__ void gm_range(int n, int& lo, int& hi) {
  const int per = (n + (int)gridDim.x - 1) / (int)gridDim.x;
  lo = min(n, (int)blockIdx.x * per);
  hi = min(n, lo + per);
}

// Last-CTA election after this CTA's partial results are written.
__device__ __forceinline__ bool gm_last_cta(unsigned* ticket) {
  __shared__ bool s_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (s_last) __threadfence();
  return s_last;
}

// Fixed-order sum of a run of G per-CTA partials by one warp: lanes take every 32nd partial, then
// a fixed xor tree. The sums are in the vector type: GB300's FP64 pipe is a small fraction of its
// FP32 rate, so bulk FP64 arithmetic would dominate these latency-bound passes.
template <typename VT>
__device__ __forceinline__ double warp_sum_run(const double* p, int G, int lane, int stride = 1) {
  VT a = 0;
  for (int c = lane; c < G; c += 32) a += (VT)__ldcg(&p[(size_t)c * stride]);
  return (double)warp_sum(a);
}

// sqrt(x) and 1 / x of an FP64 scalar through double-float arithmetic on the FP32 pipes (about 47
// bits): on this GPU FP64 square roots and divisions are long dependent sequences, and these sit on
// the serial tail of every iteration. Outside FP32's comfortable range, or for 0, negative and
// non-finite values, the FP64 operation.
__device__ __forceinline__ double gm_sqrt(double x) {
  if (x > 1e-30 && x < 1e30) return df_to_double(df_sqrt(df_from_double(x)));
  return sqrt(x);
}
__device__ __forceinline__ double gm_rcp(double x) {
  const double a = fabs(x);
  if (a > 1e-30 && a < 1e30) return df_to_double(df_rcp(df_from_double(x)));
  return 1.0 / x;
}

// The new Hessenberg column h (j + 1 entries in gd, h_{j+1} = nrm) by one CTA: rotate it by the
// earlier Givens rotations, form the new rotation, update the residual estimate |g_{j+1}| and
// decide whether the cycle goes on (the final step of an iteration). Shared memory: 4 j + 3
// entries of 16 bytes (dynamic).
__device__ __noinline__ void gm_rotate(GmCols C, GState* st, double* gd, GmLayout L, int m, int j, double nrm) {
  // Rotate the new column h (j + 2 entries) by the earlier rotations: with x_0 = h_0,
  //   r_i = c_i x_i + s_i h_{i+1},  x_{i+1} = conj(c_i) h_{i+1} - conj(s_i) x_i  (i < j).
  // The recurrence is a composition of affine maps x -> M_i x + N_i (M_i = -conj(s_i), N_i =
  // conj(c_i) h_{i+1}), so it runs as a parallel inclusive scan of the maps, composing later after
  // earlier, (M2, N2) o (M1, N1) = (M2 M1, M2 N1 + N2), and then x_{i+1} = M_i x_0 + N_i. The scan
  // is in double-float complex arithmetic on the FP32 pipes: a chain of dependent FP64 operations
  // runs at a small fraction of that rate on this GPU.
  extern __shared__ __align__(16) unsigned char gsm[];
  Dc* hs = reinterpret_cast<Dc*>(gsm);      // h: j + 2 entries (the coefficients are no longer needed)
  Dc* xs = hs + (j + 2);                    // x_i: j + 1 entries
  cdf* sm = reinterpret_cast<cdf*>(xs + (j + 1));  // M_i: j entries
  cdf* sn = sm + j;                                // N_i: j entries
  __syncthreads();
  // the column was completed by other CTAs before this CTA's ticket or barrier (read past L1)
  for (int k = threadIdx.x; k <= j; k += blockDim.x)
    hs[k] = dc(__ldcg(&gd[L.hcol() + 2 * k]), __ldcg(&gd[L.hcol() + 2 * k + 1]));
  __syncthreads();
  if (threadIdx.x == 0) hs[j + 1] = dc(nrm, 0.0);
  for (int i = threadIdx.x; i < j; i += blockDim.x) {
    const Dc c = dc(gd[L.cs() + 2 * i], gd[L.cs() + 2 * i + 1]);
    const Dc t = conjd(c) * hs[i + 1];
    sn[i] = cdf{df_from_double(t.re), df_from_double(t.im)};
    sm[i] = cdf{df_from_double(-gd[L.sn() + 2 * i]), df_from_double(gd[L.sn() + 2 * i + 1])};
  }
  __syncthreads();
  constexpr int kPer = (kGmMaxRestart + kGmThreads - 1) / kGmThreads;  // scan entries per thread
  for (int d = 1; d < j; d <<= 1) {
    cdf nm[kPer], nn[kPer];
#pragma unroll
    for (int u = 0; u < kPer; u++) {
      const int i = threadIdx.x + u * kGmThreads;
      if (i < j) {
        nm[u] = sm[i];
        nn[u] = sn[i];
        if (i >= d) {
          const cdf m1 = sm[i - d], n1 = sn[i - d];
          nn[u] = nm[u] * n1 + nn[u];
          nm[u] = nm[u] * m1;
        }
      }
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < kPer; u++) {
      const int i = threadIdx.x + u * kGmThreads;
      if (i < j) {
        sm[i] = nm[u];
        sn[i] = nn[u];
      }
    }
    __syncthreads();
  }
  {
    const cdf x0{df_from_double(hs[0].re), df_from_double(hs[0].im)};
    if (threadIdx.x == 0) xs[0] = hs[0];
    for (int i = threadIdx.x; i < j; i += blockDim.x) {
      const cdf x = sm[i] * x0 + sn[i];
      xs[i + 1] = dc(df_to_double(x.re), df_to_double(x.im));
    }
  }
  __syncthreads();
  double* R = gd + L.R() + 2 * (size_t)j * m;  // column j: rows 0..j
  for (int i = threadIdx.x; i < j; i += blockDim.x) {
    const Dc c = dc(gd[L.cs() + 2 * i], gd[L.cs() + 2 * i + 1]);
    const Dc s = dc(gd[L.sn() + 2 * i], gd[L.sn() + 2 * i + 1]);
    const Dc rv = c * xs[i] + s * hs[i + 1];
    R[2 * i] = rv.re;
    R[2 * i + 1] = rv.im;
  }
  if (threadIdx.x == 0) {
    const Dc a0 = xs[j], b0 = hs[j + 1];
    const double d = gm_sqrt(abs2(a0) + abs2(b0));
    Dc c = dc(1.0, 0.0), s = dc(0.0, 0.0);
    if (d > 0.0) {
      const double id = gm_rcp(d);
      c = dc(a0.re * id, -a0.im * id);  // conj(a) / d
      s = dc(b0.re * id, -b0.im * id);  // conj(b) / d
    }
    R[2 * j] = d;
    R[2 * j + 1] = 0.0;
    gd[L.cs() + 2 * j] = c.re;
    gd[L.cs() + 2 * j + 1] = c.im;
    gd[L.sn() + 2 * j] = s.re;
    gd[L.sn() + 2 * j + 1] = s.im;
    const Dc gj = dc(gd[L.g() + 2 * j], gd[L.g() + 2 * j + 1]);
    const Dc g1 = dc(0.0, 0.0) - conjd(s) * gj;
    const Dc g0 = c * gj;
    gd[L.g() + 2 * j] = g0.re;
    gd[L.g() + 2 * j + 1] = g0.im;
    gd[L.g() + 2 * (j + 1)] = g1.re;
    gd[L.g() + 2 * (j + 1) + 1] = g1.im;
    const double res = gm_sqrt(abs2(g1));
    gd[L.s() + j + 1] = nrm > 0.0 ? gm_rcp(nrm) : 0.0;
    st->resid = res;
    st->j = j + 1;
    st->ticket = 0u;
    int code = 0;
    if (!isfinite(res) || !isfinite(d) || d == 0.0)
      code = (d == 0.0 && isfinite(res) && res <= st->tol_abs) ? 1 : 3;
    else if (res <= st->tol_abs || nrm == 0.0)
      code = 1;
    else if (j + 1 >= m)
      code = 2;
    gm_mark_done(st, C.gm, code);
  }
}

// V_0 = b (rounded to VT), q = V_0, s_0 = 1 / |V_0|, g = (|V_0|, 0, ...).
template <typename VT, typename BT>
__global__ void __launch_bounds__(kGmThreads) k_gm_init(GmCols C, int m, int n, const cplx<BT>* __restrict__ b,
                                                        cplx<VT>* V, cplx<VT>* q, double tol,
                                                        const double* __restrict__ tolv) {
  const int r = blockIdx.y, vs = C.vs;
  GState* st = C.st + r;
  double* gd = C.gd + r * C.gds;
  V += r * C.Vs;
  b += r;
  q += r;
  const GmLayout L{m, (int)gridDim.x};
  int lo, hi;
  gm_range(n, lo, hi);
  VT a = 0;
  for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    const cplx<BT> bi = b[(size_t)i * vs];
    const cplx<VT> v((VT)bi.re, (VT)bi.im);
    V[i] = v;
    q[(size_t)i * vs] = v;
    a = fma(v.re, v.re, fma(v.im, v.im, a));
  }
  __shared__ VT sw[kGmWarps];
  a = warp_sum(a);
  if ((threadIdx.x & 31) == 0) sw[threadIdx.x >> 5] = a;
  __syncthreads();
  if (threadIdx.x == 0) {
    VT t = 0;
    for (int w = 0; w < kGmWarps; w++) t += sw[w];
    gd[L.npart() + blockIdx.x] = (double)t;
  }
  if (!gm_last_cta(&st->ticket)) return;
  if (threadIdx.x < 32) {
    const double b2 = warp_sum_run<VT>(gd + L.npart(), L.G, threadIdx.x);
    if (threadIdx.x == 0) {
      const double beta = sqrt(b2);
      st->j = 0;
      st->m = m;
      st->beta = beta;
      st->tol_abs = (tolv ? tolv[r] : tol) * beta;
      st->resid = beta;
      gd[L.s()] = beta > 0.0 ? 1.0 / beta : 0.0;
      gd[L.g()] = beta;
      gd[L.g() + 1] = 0.0;
      st->ticket = 0u;
      // a zero right-hand side has the zero solution; a non-finite one cannot be solved
      gm_mark_done(st, C.gm, beta > 0.0 && isfinite(beta) ? 0 : (beta == 0.0 ? 1 : 3));
    }
  }
}

// Per-CTA partial dots conj(V_k) . X over the CTA's elements (X staged in shared memory as xsm,
// len elements from lo) for k = 0..j, each warp four vectors at a time.
template <typename VT>
__device__ __forceinline__ void gs_dot_partials(const cplx<VT>* __restrict__ V, const cplx<VT>* xsm, int len,
                                                int lo, int n, int j, const GmLayout& L, double* gd) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int kb = 4 * warp; kb <= j; kb += 4 * kGmWarps) {
    VT ar[4] = {0, 0, 0, 0}, ai[4] = {0, 0, 0, 0};
    // four elements per lane per step: sixteen loads in flight before their products, which keep
    // the element order t, t + 32, t + 64, t + 96
    for (int t0 = 0; t0 < len; t0 += 128) {
      cplx<VT> v[4][4];
#pragma unroll
      for (int e = 0; e < 4; e++) {
        const int t = t0 + 32 * e + lane;
#pragma unroll
        for (int u = 0; u < 4; u++)
          v[e][u] = (t < len && kb + u <= j) ? V[(size_t)(kb + u) * n + lo + t] : cplx<VT>();
      }
#pragma unroll
      for (int e = 0; e < 4; e++) {
        const int t = t0 + 32 * e + lane;
        const cplx<VT> x = t < len ? xsm[t] : cplx<VT>();
#pragma unroll
        for (int u = 0; u < 4; u++) {  // conj(v) x
          ar[u] = fma(v[e][u].re, x.re, ar[u]);
          ar[u] = fma(v[e][u].im, x.im, ar[u]);
          ai[u] = fma(v[e][u].re, x.im, ai[u]);
          ai[u] = fma(-v[e][u].im, x.re, ai[u]);
        }
      }
    }
#pragma unroll
    for (int u = 0; u < 4; u++) {
      ar[u] = warp_sum(ar[u]);
      ai[u] = warp_sum(ai[u]);
    }
    if (lane == 0)
#pragma unroll
      for (int u = 0; u < 4; u++)
        if (kb + u <= j) {
          gd[L.part() + ((size_t)(kb + u) * L.G + blockIdx.x) * 2] = (double)ar[u];
          gd[L.part() + ((size_t)(kb + u) * L.G + blockIdx.x) * 2 + 1] = (double)ai[u];
        }
  }
}

// The last CTA's part of a dot pass: sums the partials in CTA order into h_k = s_k sx V_k^H X
// (sx = s_j on the first pass, 1 on the second), sets (first pass) or adds to (second pass) the
// Hessenberg column, writes the update coefficients h_k s_k and resets the ticket.
template <typename VT>
__device__ __forceinline__ void gs_dot_tail(GState* st, double* gd, const GmLayout& L, int j, int second) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const double sx = second ? 1.0 : gd[L.s() + j];
  for (int kb = 4 * warp; kb <= j; kb += 4 * kGmWarps) {
    VT a[8];
#pragma unroll
    for (int u = 0; u < 8; u++) a[u] = 0;
    // two partials per lane per step (sixteen loads in flight), summed in CTA order per lane
    for (int c0 = lane; c0 < L.G; c0 += 64) {
      double w[2][8];
#pragma unroll
      for (int e = 0; e < 2; e++) {
        const int c = c0 + 32 * e;
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const bool ok = c < L.G && kb + u <= j;
          w[e][2 * u] = ok ? __ldcg(&gd[L.part() + ((size_t)(kb + u) * L.G + c) * 2]) : 0.0;
          w[e][2 * u + 1] = ok ? __ldcg(&gd[L.part() + ((size_t)(kb + u) * L.G + c) * 2 + 1]) : 0.0;
        }
      }
#pragma unroll
      for (int e = 0; e < 2; e++)
#pragma unroll
        for (int u = 0; u < 8; u++) a[u] += (VT)w[e][u];
    }
#pragma unroll
    for (int u = 0; u < 8; u++) a[u] = warp_sum(a[u]);
    if (lane < 4 && kb + lane <= j) {
      const int k = kb + lane;
      double hr = 0, hi2 = 0;
#pragma unroll
      for (int u = 0; u < 4; u++)
        if (u == lane) {
          hr = (double)a[2 * u];
          hi2 = (double)a[2 * u + 1];
        }
      const double sk = gd[L.s() + k];
      hr *= sk * sx;
      hi2 *= sk * sx;
      if (second) {
        gd[L.hcol() + 2 * k] += hr;
        gd[L.hcol() + 2 * k + 1] += hi2;
      } else {
        gd[L.hcol() + 2 * k] = hr;
        gd[L.hcol() + 2 * k + 1] = hi2;
      }
      gd[L.coef() + 2 * k] = hr * sk;
      gd[L.coef() + 2 * k + 1] = hi2 * sk;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) st->ticket = 0u;
}

// One Gram-Schmidt pass, dots: h_k = s_k sx V_k^H X for k = 0..j, X the matvec output (sx = s_j,
// first pass) or the first pass's result (sx = 1, second pass). Per-CTA partials over the CTA's
// elements; the last CTA sums them in CTA order, sets (first pass) or adds to (second pass) the
// Hessenberg column and writes the update coefficients h_k s_k.
template <typename VT>
__global__ void __launch_bounds__(kGmThreads) k_gm_dots(GmCols C, int m, int n, const cplx<VT>* __restrict__ V,
                                                        const cplx<VT>* __restrict__ X, int second) {
  grid_dep_wait();  // X comes from the kernel just before
  grid_dep_launch();
  const int r = blockIdx.y;
  GState* st = C.st + r;
  if (st->done) return;
  double* gd = C.gd + r * C.gds;
  V += r * C.Vs;
  // X: the matvec output (block vectors) on the first pass, the first pass's result (one column
  // of n) on the second
  const int xstr = second ? 1 : C.vs;
  X += second ? (size_t)r * n : (size_t)r;
  const GmLayout L{m, (int)gridDim.x};
  const int j = st->j;
  int lo, hi;
  gm_range(n, lo, hi);
  __shared__ cplx<VT> xsm[kSliceMax];
  for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) xsm[i - lo] = X[(size_t)i * xstr];
  __syncthreads();
  gs_dot_partials<VT>(V, xsm, hi - lo, lo, n, j, L, gd);
  if (!gm_last_cta(&st->ticket)) return;
  gs_dot_tail<VT>(st, gd, L, j, second);
}

// One Gram-Schmidt pass, update: U = sx X - sum_k coef_k V_k (sx = s_j on the first pass, 1 on
// the second). Not final: U goes to Y (the second pass's input). Final: U is V_{j+1} (also into q,
// the next matvec's input), with |U|^2 partials; the last CTA rotates the new Hessenberg column,
// updates the residual estimate and decides whether the cycle goes on.
template <typename VT>
__global__ void __launch_bounds__(kGmThreads) k_gm_update(GmCols C, int m, int n, cplx<VT>* V,
                                                          const cplx<VT>* __restrict__ X, cplx<VT>* Y, cplx<VT>* q,
                                                          int second, int final_pass) {
  grid_dep_wait();  // the coefficients come from the dot pass just before
  grid_dep_launch();
  const int r = blockIdx.y;
  GState* st = C.st + r;
  if (st->done) return;
  double* gd = C.gd + r * C.gds;
  V += r * C.Vs;
  // X: the matvec output (block vectors, first pass) or this column's first-pass result; Y: this
  // column's first-pass result; q: the next matvec's input (block vectors)
  const int xstr = second ? 1 : C.vs;
  X += second ? (size_t)r * n : (size_t)r;
  Y += (size_t)r * n;
  q += r;
  const GmLayout L{m, (int)gridDim.x};
  const int j = st->j;
  extern __shared__ __align__(16) unsigned char gsm[];
  cplx<VT>* coef = reinterpret_cast<cplx<VT>*>(gsm);  // j + 1 coefficients
  for (int k = threadIdx.x; k <= j; k += blockDim.x)
    coef[k] = cplx<VT>((VT)gd[L.coef() + 2 * k], (VT)gd[L.coef() + 2 * k + 1]);
  __syncthreads();
  const VT sx = second ? VT(1) : (VT)gd[L.s() + j];
  int lo, hi;
  gm_range(n, lo, hi);
  cplx<VT>* out = final_pass ? V + (size_t)(j + 1) * n : Y;
  __shared__ cplx<VT> us[kSliceMax];  // U of this CTA's elements (not final: the second pass's dots)
  VT a = 0;
  for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    const cplx<VT> x = X[(size_t)i * xstr];
    VT ur = sx * x.re, ui = sx * x.im;
    const cplx<VT>* Vi = V + i;
    int k = 0;
    // sixteen loads in flight before their products; the products keep the order k = 0, 1, ...
    for (; k + 16 <= j + 1; k += 16) {
      cplx<VT> v[16];
#pragma unroll
      for (int u = 0; u < 16; u++) v[u] = Vi[(size_t)(k + u) * n];
#pragma unroll
      for (int u = 0; u < 16; u++) {
        const cplx<VT> c = coef[k + u];
        ur = fma(-c.re, v[u].re, ur);
        ur = fma(c.im, v[u].im, ur);
        ui = fma(-c.re, v[u].im, ui);
        ui = fma(-c.im, v[u].re, ui);
      }
    }
    for (; k <= j; k++) {
      const cplx<VT> v = Vi[(size_t)k * n];
      const cplx<VT> c = coef[k];
      ur = fma(-c.re, v.re, ur);
      ur = fma(c.im, v.im, ur);
      ui = fma(-c.re, v.im, ui);
      ui = fma(-c.im, v.re, ui);
    }
    const cplx<VT> u(ur, ui);
    out[i] = u;
    if (final_pass) {
      q[(size_t)i * C.vs] = u;
      a = fma(ur, ur, fma(ui, ui, a));
    } else {
      us[i - lo] = u;
    }
  }
  if (!final_pass) {
    // the second pass's dots of U, from shared memory, with the same partials and tail as a dot
    // pass (one kernel boundary fewer per iteration)
    __syncthreads();
    gs_dot_partials<VT>(V, us, hi - lo, lo, n, j, L, gd);
    if (gm_last_cta(&st->ticket)) gs_dot_tail<VT>(st, gd, L, j, 1);
    return;
  }
  __shared__ VT sw[kGmWarps];
  a = warp_sum(a);
  if ((threadIdx.x & 31) == 0) sw[threadIdx.x >> 5] = a;
  __syncthreads();
  if (threadIdx.x == 0) {
    VT t = 0;
    for (int w = 0; w < kGmWarps; w++) t += sw[w];
    gd[L.npart() + blockIdx.x] = (double)t;
  }
  if (!gm_last_cta(&st->ticket)) return;
  __shared__ double nrm_s;
  __syncthreads();
  if (threadIdx.x < 32) {
    const double u2 = warp_sum_run<VT>(gd + L.npart(), L.G, threadIdx.x);
    if (threadIdx.x == 0) nrm_s = gm_sqrt(u2);
  }
  __syncthreads();
  gm_rotate(C, st, gd, L, m, j, nrm_s);
}

// ------------------------------------------------------------------------------------------
// Fused Gram-Schmidt iteration: one cooperative launch in place of the dot and update passes.
// All CTAs of the batch are resident (cooperative launch), and the phases are separated by grid
// barriers instead of kernel boundaries and last-CTA reductions:
//   1  dots: per-CTA partials of V_k^H X over the CTA's elements (k <= j);
//   2  reduce: CTA c sums the partials of k = c, c + G, ... in CTA order into h_k (Hessenberg
//      column) and the update coefficients h_k s_k;
//   3  update: U = s_j X - sum_k coef_k V_k over the CTA's elements; with two passes U goes to
//      W2 with the second pass's partials (and |U|^2 partials), then
//   4  reduce as in 2 (h_k added to the column, |h_k|^2 kept), and
//   5  the second update into V_{j+1}; |V_{j+1}|^2 = |U|^2 - sum_k |h_k|^2 (the second pass
//      removes only a rounding-sized part of U); with one pass phase 3 writes V_{j+1} and its
//      |.|^2 partials directly.
// CTA 0 of each cycle then rotates the new column and updates the residual estimate, as the
// final update pass does. Sums run in fixed orders, so results do not depend on timing. A cycle
// that has ended passes the barriers without work.
// ------------------------------------------------------------------------------------------
constexpr uint32_t kBarSpin = 1u << 22;  // polls (with a short sleep) before a barrier gives up

// Grid-wide barrier over all CTAs of a cooperative launch (every CTA calls it the same number of
// times). One 64-bit arrival counter that is never reset during a cycle: arrival ticket t belongs
// to barrier instance t / total (no CTA arrives at the next instance before all have arrived at
// this one), which is complete when the counter reaches (t / total + 1) total. One atomic per CTA
// and a poll, instead of a count reset and a generation bump after the last arrival. Returns
// false on every thread if this CTA's wait gave up (recorded in bar_fail).
__device__ __forceinline__ bool gm_grid_barrier(GMulti* gm, unsigned total) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();  // this CTA's writes before its arrival
    const unsigned long long t = atomicAdd(&gm->bar, 1ull);
    const unsigned long long target = (t / total + 1) * (unsigned long long)total;
    volatile unsigned long long* c = &gm->bar;
    int ok = 1;
    uint32_t it = 0;
    while (*c < target) {
      if (++it > kBarSpin) {
        ok = 0;
        atomicExch(&gm->bar_fail, 1);
        break;
      }
      __nanosleep(20);
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Elements per lane per round of loads in gf_dot_partials: with FP32 vectors one round covers a
// CTA's slice of a 20k-element vector over 152 CTAs (135 elements). (The FP32 fused kernel runs at
// 3 CTAs per SM, 80 registers, without spills.)
template <typename VT>
struct GfDotRound {
  static constexpr int E = sizeof(VT) == 4 ? 5 : 4;
};

// Per-CTA partial dots conj(V_k) . X over elements [lo, hi) (X from global memory with stride
// xs), k = 0..j, into part[(k G + c) 2]; same ordering as gs_dot_partials: each lane takes the
// elements lane, lane + 32, ... in that order, whatever the round width.
template <typename VT>
__device__ __forceinline__ void gf_dot_partials(const cplx<VT>* __restrict__ V, const cplx<VT>* X, int xs, int lo,
                                                int len, int n, int j, double* part, int G) {
  constexpr int kGfE = GfDotRound<VT>::E;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int kb = 4 * warp; kb <= j; kb += 4 * kGmWarps) {
    VT ar[4] = {0, 0, 0, 0}, ai[4] = {0, 0, 0, 0};
    for (int t0 = 0; t0 < len; t0 += 32 * kGfE) {
      cplx<VT> v[kGfE][4], x[kGfE];
#pragma unroll
      for (int e = 0; e < kGfE; e++) {
        const int t = t0 + 32 * e + lane;
        x[e] = t < len ? X[(size_t)(lo + t) * xs] : cplx<VT>();
#pragma unroll
        for (int u = 0; u < 4; u++)
          v[e][u] = (t < len && kb + u <= j) ? V[(size_t)(kb + u) * n + lo + t] : cplx<VT>();
      }
#pragma unroll
      for (int e = 0; e < kGfE; e++)
#pragma unroll
        for (int u = 0; u < 4; u++) {  // conj(v) x
          ar[u] = fma(v[e][u].re, x[e].re, ar[u]);
          ar[u] = fma(v[e][u].im, x[e].im, ar[u]);
          ai[u] = fma(v[e][u].re, x[e].im, ai[u]);
          ai[u] = fma(-v[e][u].im, x[e].re, ai[u]);
        }
    }
#pragma unroll
    for (int u = 0; u < 4; u++) {
      ar[u] = warp_sum(ar[u]);
      ai[u] = warp_sum(ai[u]);
    }
    if (lane == 0)
#pragma unroll
      for (int u = 0; u < 4; u++)
        if (kb + u <= j) {
          part[((size_t)(kb + u) * G + blockIdx.x) * 2] = (double)ar[u];
          part[((size_t)(kb + u) * G + blockIdx.x) * 2 + 1] = (double)ai[u];
        }
  }
}

// Phase 2 / 4: this CTA's coefficients k = c, c + G, ... <= j (a warp each): h_k = s_k sx times
// the sum of the partials in CTA order; the Hessenberg column gets h_k (set, or added on the
// second pass), the update coefficient h_k s_k goes to coef, and on the second pass h_k to h2.
template <typename VT>
__device__ __forceinline__ void gf_reduce(double* gd, const GmLayout& L, const double* part, int G, int j, double sx,
                                          int second) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k = blockIdx.x + warp * G; k <= j; k += kGmWarps * G) {
    VT ar = 0, ai = 0;
    for (int c = lane; c < G; c += 32) {
      ar += (VT)__ldcg(&part[((size_t)k * G + c) * 2]);
      ai += (VT)__ldcg(&part[((size_t)k * G + c) * 2 + 1]);
    }
    ar = warp_sum(ar);
    ai = warp_sum(ai);
    if (lane == 0) {
      const double sk = gd[L.s() + k];
      const double hr = (double)ar * sk * sx, hi2 = (double)ai * sk * sx;
      if (second) {
        gd[L.hcol() + 2 * k] += hr;
        gd[L.hcol() + 2 * k + 1] += hi2;
        gd[L.h2() + 2 * k] = hr;
        gd[L.h2() + 2 * k + 1] = hi2;
      } else {
        gd[L.hcol() + 2 * k] = hr;
        gd[L.hcol() + 2 * k + 1] = hi2;
      }
      gd[L.coef() + 2 * k] = hr * sk;
      gd[L.coef() + 2 * k + 1] = hi2 * sk;
    }
  }
}

// Basis vectors per round of loads in gf_update (16). With FP32 vectors the last round is partial
// (loads and products beyond j skipped), so a thread waits for ceil((j + 1) / 16) rounds, not for
// a remainder one vector at a time; with FP64 vectors the remainder goes one vector at a time. The
// products keep the order k = 0, 1, ... either way.
constexpr int kGfChunk = 16;

// U = sx X - sum_k coef_k V_k over [lo, hi), written to out (and to q, stride qs, if q); returns
// this thread's |U|^2.
template <typename VT>
__device__ __forceinline__ VT gf_update(const cplx<VT>* __restrict__ V, const cplx<VT>* X, int xs, VT sx,
                                        const cplx<VT>* coef, int lo, int hi, int n, int j, cplx<VT>* out,
                                        cplx<VT>* q, int qs) {
  constexpr int KC = kGfChunk;
  constexpr bool partial_rounds = sizeof(VT) == 4;
  VT a = 0;
  for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    const cplx<VT> x = X[(size_t)i * xs];
    VT ur = sx * x.re, ui = sx * x.im;
    const cplx<VT>* Vi = V + i;
    int k = 0;
    if constexpr (partial_rounds) {
      for (; k <= j; k += KC) {
        cplx<VT> v[KC];
#pragma unroll
        for (int u = 0; u < KC; u++) v[u] = k + u <= j ? Vi[(size_t)(k + u) * n] : cplx<VT>();
#pragma unroll
        for (int u = 0; u < KC; u++) {
          if (k + u > j) break;
          const cplx<VT> c = coef[k + u];
          ur = fma(-c.re, v[u].re, ur);
          ur = fma(c.im, v[u].im, ur);
          ui = fma(-c.re, v[u].im, ui);
          ui = fma(-c.im, v[u].re, ui);
        }
      }
    } else {
      for (; k + KC <= j + 1; k += KC) {
        cplx<VT> v[KC];
#pragma unroll
        for (int u = 0; u < KC; u++) v[u] = Vi[(size_t)(k + u) * n];
#pragma unroll
        for (int u = 0; u < KC; u++) {
          const cplx<VT> c = coef[k + u];
          ur = fma(-c.re, v[u].re, ur);
          ur = fma(c.im, v[u].im, ur);
          ui = fma(-c.re, v[u].im, ui);
          ui = fma(-c.im, v[u].re, ui);
        }
      }
      for (; k <= j; k++) {
        const cplx<VT> v = Vi[(size_t)k * n];
        const cplx<VT> c = coef[k];
        ur = fma(-c.re, v.re, ur);
        ur = fma(c.im, v.im, ur);
        ui = fma(-c.re, v.im, ui);
        ui = fma(-c.im, v.re, ui);
      }
    }
    const cplx<VT> u(ur, ui);
    out[i] = u;
    if (q) q[(size_t)i * qs] = u;
    a = fma(ur, ur, fma(ui, ui, a));
  }
  return a;
}

// Sum of a CTA's per-thread values in warp order, written to dst by thread 0.
template <typename VT>
__device__ __forceinline__ void gf_cta_sum(VT a, double* dst) {
  __shared__ VT sw[kGmWarps];
  a = warp_sum(a);
  if ((threadIdx.x & 31) == 0) sw[threadIdx.x >> 5] = a;
  __syncthreads();
  if (threadIdx.x == 0) {
    VT t = 0;
    for (int w = 0; w < kGmWarps; w++) t += sw[w];
    *dst = (double)t;
  }
}

// |V_{j+1}| from the |U|^2 partials of G CTAs (two passes: minus the second pass's sum_k |h2_k|^2,
// k in order), then the Givens step of gm_rotate; one CTA.
template <typename VT>
__device__ __forceinline__ void gf_norm_rotate(GmCols C, GState* st, double* gd, const GmLayout& L, int m, int j,
                                               int G, int reorth) {
  __shared__ double nrm_s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double u2 = warp_sum_run<VT>(gd + L.npart(), G, threadIdx.x);
    if (reorth) {
      double s2 = 0;
      for (int k = threadIdx.x; k <= j; k += 32) {
        const double hr = __ldcg(&gd[L.h2() + 2 * k]), hi2 = __ldcg(&gd[L.h2() + 2 * k + 1]);
        s2 += hr * hr + hi2 * hi2;
      }
      s2 = warp_sum(s2);
      u2 = fmax(u2 - s2, 0.0);
    }
    if (threadIdx.x == 0) nrm_s = gm_sqrt(u2);
  }
  __syncthreads();
  gm_rotate(C, st, gd, L, m, j, nrm_s);
}

template <typename VT>
__global__ void __launch_bounds__(kGmThreads, sizeof(VT) == 4 ? 3 : 2) k_gm_fused(GmCols C, int m, int n, int LG, cplx<VT>* V,
                                                         const cplx<VT>* __restrict__ W, cplx<VT>* W2, cplx<VT>* q,
                                                         int reorth, int givens) {
  // givens: where the Givens step runs. 0: CTA 0 after its last update; 1: k_gm_rotate after this
  // kernel (the caller forks it); 2: one CTA more than the element CTAs (the last), right after
  // the last grid barrier, while the others run the last update.
  if (*(volatile const int*)&C.gm->done_all) return;  // as in k_gm_dcgs
  const int r = blockIdx.y, G = (int)gridDim.x - (givens == 2 ? 1 : 0);
  const bool rot_cta = givens == 2 && (int)blockIdx.x == G;
  // with the Givens step forked, the next matvec may start streaming its matrix during the last
  // update (it reads V_{j+1} only after this kernel has completed). Not with the Givens CTA: inside
  // a request server the early matvec CTAs would hold SM room that other requests' kernels need.
  const bool early = givens == 1;
  const unsigned total = gridDim.x * gridDim.y;
  GState* st = C.st + r;
  double* gd = C.gd + r * C.gds;
  V += r * C.Vs;
  const cplx<VT>* X = W + r;  // the matvec output (block vectors)
  W2 += (size_t)r * n;
  q += r;
  const GmLayout L{m, LG};
  const bool run = st->done == 0;  // changed only by the Givens step, after the last barrier
  const bool work = run && !rot_cta;  // element work of this CTA
  const int j = st->j;
  int lo, hi;
  {  // contiguous element range of this CTA among the G element CTAs (none for the Givens CTA)
    const int per = (n + G - 1) / G;
    lo = min(n, (int)blockIdx.x * per);
    hi = min(n, lo + per);
  }
  extern __shared__ __align__(16) unsigned char gsm[];
  cplx<VT>* coef = reinterpret_cast<cplx<VT>*>(gsm);
  const double sj = work ? gd[L.s() + j] : 0.0;
  bool ok = true;
  auto load_coef = [&]() {
    for (int k = threadIdx.x; k <= j; k += blockDim.x)
      coef[k] = cplx<VT>((VT)__ldcg(&gd[L.coef() + 2 * k]), (VT)__ldcg(&gd[L.coef() + 2 * k + 1]));
    __syncthreads();
  };
  // 1, 2: first-pass dots and their reduction
  if (work) gf_dot_partials<VT>(V, X, C.vs, lo, hi - lo, n, j, gd + L.part(), G);
  ok = gm_grid_barrier(C.gm, total) && ok;
  if (work && ok) gf_reduce<VT>(gd, L, gd + L.part(), G, j, sj, 0);
  ok = gm_grid_barrier(C.gm, total) && ok;
  if (work && ok) load_coef();
  VT a = 0;
  if (reorth) {
    // 3: U into W2, second-pass dots of U and |U|^2
    if (work && ok) {
      a = gf_update<VT>(V, X, C.vs, (VT)sj, coef, lo, hi, n, j, W2, nullptr, 0);
      __syncthreads();  // W2 of this CTA's elements is complete
      gf_dot_partials<VT>(V, W2, 1, lo, hi - lo, n, j, gd + L.part2(), G);
    }
    if (work && ok) gf_cta_sum<VT>(a, gd + L.npart() + blockIdx.x);
    ok = gm_grid_barrier(C.gm, total) && ok;
    // 4: second-pass coefficients
    if (work && ok) gf_reduce<VT>(gd, L, gd + L.part2(), G, j, 1.0, 1);
    ok = gm_grid_barrier(C.gm, total) && ok;
    if (early) grid_dep_launch();
    // 5: V_{j+1} = U - sum_k coef_k V_k
    if (work && ok) {
      load_coef();
      gf_update<VT>(V, W2, 1, (VT)1, coef, lo, hi, n, j, V + (size_t)(j + 1) * n, q, C.vs);
    }
  } else {
    if (early) grid_dep_launch();
    // 3: V_{j+1} with its |.|^2 partials
    if (work && ok) {
      a = gf_update<VT>(V, X, C.vs, (VT)sj, coef, lo, hi, n, j, V + (size_t)(j + 1) * n, q, C.vs);
      gf_cta_sum<VT>(a, gd + L.npart() + blockIdx.x);
    }
    // givens 1: k_gm_rotate reads the |.|^2 partials after this kernel has completed
    if (givens != 1) ok = gm_grid_barrier(C.gm, total) && ok;
  }
  if (!run || (int)blockIdx.x != (givens == 2 ? G : 0)) return;
  if (!ok) {
    if (threadIdx.x == 0) gm_mark_done(st, C.gm, 3);
    return;
  }
  if (givens == 1) return;
  // the new column's norm, its rotation and the residual estimate
  gf_norm_rotate<VT>(C, st, gd, L, m, j, G, reorth);
}

// Givens step of a fused iteration on its own (the fused kernel launched with givens = 1), one CTA
// per cycle, after the fused kernel has completed: the same norm, rotation, residual estimate and
// stop test as the fused kernel's CTA 0 would run, from the partials it left (G of them). A cycle
// that has ended (or whose fused kernel gave up at a barrier) is left alone.
template <typename VT>
__global__ void __launch_bounds__(kGmThreads) k_gm_rotate(GmCols C, int m, int LG, int G, int reorth) {
  GState* st = C.st + blockIdx.y;
  if (st->done) return;
  double* gd = C.gd + blockIdx.y * C.gds;
  gf_norm_rotate<VT>(C, st, gd, GmLayout{m, LG}, m, st->j, G, reorth);
}

// ------------------------------------------------------------------------------------------
// Gram-Schmidt with delayed reorthogonalisation (FP32 cycles): one reduction per iteration.
// After Bielich, Langou, Thomas, Swirydowicz, Yamazaki and Boman, "Low-synch Gram-Schmidt with
// delayed reorthogonalization for Krylov solvers" (Parallel Computing, 2022), in this form:
// the matvec input of iteration j is u_j, the first-pass result of iteration j - 1 (not yet
// reorthogonalised, not normalised), with A q_{j-1} = Q_j h_{j-1} + u_j. With w = A u_j, one
// pass over the basis gives the dots a = Q_j^H u_j, b = Q_j^H w, alpha = |u_j|^2 and
// beta = u_j^H w. Then
//   rho = sqrt(alpha - |a|^2),  q_j = (u_j - Q_j a) / rho          (the lagged second pass),
//   column j - 1 of H: h_{j-1} + a, subdiagonal rho                   (finished now),
//   gamma = (beta - a^H b) / rho^2,
//   u_{j+1} = (w - gamma u_j - Q_j (b - gamma a)) / rho               (= A q_j - Q_{j+1} h_j),
//   first-pass column j: h_kj = b_k / rho (k < j), h_jj = gamma - a_{j-1}.
// (The exact first-pass column is (b - H a) / rho; the H a term is of the size of the lost
// orthogonality times |H| and is left out.) Both vectors come out of one more pass over the basis,
// so an iteration reads the basis twice and has two grid barriers, against three or four passes
// and four barriers with two classical passes. The basis vectors q_k are stored normalised
// (s_k = 1). The Givens step of column j - 1 runs after the reduction; the cycle's stop test
// therefore sees column j - 1 during iteration j, and the iteration that finds convergence has
// already run its matvec. A cycle that fills its basis ends after the reduction of iteration m,
// which finishes column m - 1.
// ------------------------------------------------------------------------------------------

// Elements per lane per round of loads in gd_dot_partials (two dot products per basis load).
constexpr int kGdE = 2;

// Per-CTA partial dots a_k = conj(V_k) . U and b_k = conj(V_k) . X (k < j) over [lo, lo + len)
// of the block vectors U and X (stride xs), into pa / pb[(k G + c) 2]; each lane takes the
// elements lane, lane + 32, ... in that order.
template <typename VT>
__device__ __forceinline__ void gd_dot_partials(const cplx<VT>* __restrict__ V, const cplx<VT>* U,
                                                const cplx<VT>* X, int xs, int lo, int len, int n, int j,
                                                double* pa, double* pb, int G) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int kb = 4 * warp; kb < j; kb += 4 * kGmWarps) {
    VT ar[4] = {0, 0, 0, 0}, ai[4] = {0, 0, 0, 0}, br[4] = {0, 0, 0, 0}, bi[4] = {0, 0, 0, 0};
    for (int t0 = 0; t0 < len; t0 += 32 * kGdE) {
      cplx<VT> v[kGdE][4], u[kGdE], x[kGdE];
#pragma unroll
      for (int e = 0; e < kGdE; e++) {
        const int t = t0 + 32 * e + lane;
        u[e] = t < len ? U[(size_t)(lo + t) * xs] : cplx<VT>();
        x[e] = t < len ? X[(size_t)(lo + t) * xs] : cplx<VT>();
#pragma unroll
        for (int q = 0; q < 4; q++)
          v[e][q] = (t < len && kb + q < j) ? V[(size_t)(kb + q) * n + lo + t] : cplx<VT>();
      }
#pragma unroll
      for (int e = 0; e < kGdE; e++)
#pragma unroll
        for (int q = 0; q < 4; q++) {  // conj(v) u and conj(v) x
          ar[q] = fma(v[e][q].re, u[e].re, ar[q]);
          ar[q] = fma(v[e][q].im, u[e].im, ar[q]);
          ai[q] = fma(v[e][q].re, u[e].im, ai[q]);
          ai[q] = fma(-v[e][q].im, u[e].re, ai[q]);
          br[q] = fma(v[e][q].re, x[e].re, br[q]);
          br[q] = fma(v[e][q].im, x[e].im, br[q]);
          bi[q] = fma(v[e][q].re, x[e].im, bi[q]);
          bi[q] = fma(-v[e][q].im, x[e].re, bi[q]);
        }
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
      ar[q] = warp_sum(ar[q]);
      ai[q] = warp_sum(ai[q]);
      br[q] = warp_sum(br[q]);
      bi[q] = warp_sum(bi[q]);
    }
    if (lane == 0)
#pragma unroll
      for (int q = 0; q < 4; q++)
        if (kb + q < j) {
          const size_t o = ((size_t)(kb + q) * G + blockIdx.x) * 2;
          pa[o] = (double)ar[q];
          pa[o + 1] = (double)ai[q];
          pb[o] = (double)br[q];
          pb[o + 1] = (double)bi[q];
        }
  }
}

// Reduction of iteration j: slots 0..j-1 are a_k, j..2j-1 are b_k, 2j is (alpha, beta); this CTA
// sums the slots c, c + G, ... (a warp each) over the G per-CTA partials in CTA order.
template <typename VT>
__device__ __forceinline__ void gd_reduce(double* gd, const GmLayout& L, int G, int j) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int sl = blockIdx.x + warp * G; sl <= 2 * j; sl += kGmWarps * G) {
    if (sl == 2 * j) {
      VT al = 0, br = 0, bi = 0;
      for (int c = lane; c < G; c += 32) {
        al += (VT)__ldcg(&gd[L.abpart() + 3 * c]);
        br += (VT)__ldcg(&gd[L.abpart() + 3 * c + 1]);
        bi += (VT)__ldcg(&gd[L.abpart() + 3 * c + 2]);
      }
      al = warp_sum(al);
      br = warp_sum(br);
      bi = warp_sum(bi);
      if (lane == 0) {
        gd[L.ab()] = (double)al;
        gd[L.ab() + 1] = (double)br;
        gd[L.ab() + 2] = (double)bi;
      }
      continue;
    }
    const bool isb = sl >= j;
    const int k = isb ? sl - j : sl;
    const double* part = gd + (isb ? L.part2() : L.part());
    VT sr = 0, si = 0;
    for (int c = lane; c < G; c += 32) {
      sr += (VT)__ldcg(&part[((size_t)k * G + c) * 2]);
      si += (VT)__ldcg(&part[((size_t)k * G + c) * 2 + 1]);
    }
    sr = warp_sum(sr);
    si = warp_sum(si);
    if (lane == 0) {
      double* dst = gd + (isb ? L.h2() : L.coef()) + 2 * k;
      dst[0] = (double)sr;
      dst[1] = (double)si;
    }
  }
}

// rho^2 = alpha - |a|^2 and gamma = (beta - a^H b) / rho^2 from the reduced values, by the first
// warp of the CTA (lanes over k, a fixed xor tree: every CTA gets the same bits); into sh[0..2] =
// (rho^2, gamma.re, gamma.im).
__device__ __forceinline__ void gd_scalars(const double* gd, const GmLayout& L, int j, double* sh) {
  if (threadIdx.x >= 32) return;
  const int lane = threadIdx.x;
  double aa = 0, abr = 0, abi = 0;
  for (int k = lane; k < j; k += 32) {
    const double ar = __ldcg(&gd[L.coef() + 2 * k]), ai = __ldcg(&gd[L.coef() + 2 * k + 1]);
    const double br = __ldcg(&gd[L.h2() + 2 * k]), bi = __ldcg(&gd[L.h2() + 2 * k + 1]);
    aa += ar * ar + ai * ai;
    abr += ar * br + ai * bi;  // conj(a) b
    abi += ar * bi - ai * br;
  }
  aa = warp_sum(aa);
  abr = warp_sum(abr);
  abi = warp_sum(abi);
  if (lane == 0) {
    const double al = __ldcg(&gd[L.ab()]), br = __ldcg(&gd[L.ab() + 1]), bi = __ldcg(&gd[L.ab() + 2]);
    const double r2 = al - aa;
    const double ir2 = r2 > 0.0 ? gm_rcp(r2) : 0.0;
    sh[0] = r2;
    sh[1] = (br - abr) * ir2;
    sh[2] = (bi - abi) * ir2;
  }
}

// The Givens step of iteration j (one CTA per cycle): column j - 1 finished (h_{j-1} + a,
// subdiagonal rho) and rotated as gm_rotate does, then the first-pass column j stored for the
// next iteration. Iteration 0 only sets g_0 = rho and the first-pass column 0.
template <typename VT>
__device__ __forceinline__ void gd_givens(GmCols C, GState* st, double* gd, const GmLayout& L, int m, int j) {
  __shared__ double sh[3];
  __shared__ int s_go;
  gd_scalars(gd, L, j, sh);
  __syncthreads();
  const double r2 = sh[0];
  const double rho = r2 > 0.0 ? gm_sqrt(r2) : 0.0;
  const double gr = sh[1], gi = sh[2];
  if (j > 0) {
    for (int k = threadIdx.x; k < j; k += blockDim.x) {
      gd[L.hcol() + 2 * k] += __ldcg(&gd[L.coef() + 2 * k]);
      gd[L.hcol() + 2 * k + 1] += __ldcg(&gd[L.coef() + 2 * k + 1]);
    }
    __syncthreads();
    gm_rotate(C, st, gd, L, m, j - 1, rho);  // st->j = j; its done test
    __syncthreads();
    if (threadIdx.x == 0) {
      gd[L.s() + j] = 1.0;  // q_j is stored normalised
      s_go = *(volatile int*)&st->done == 0 && j < m;
    }
  } else if (threadIdx.x == 0) {
    gd[L.g()] = rho;
    gd[L.g() + 1] = 0.0;
    gd[L.s()] = 1.0;
    st->resid = rho;
    s_go = rho > 0.0 && isfinite(rho);
    if (!s_go) gm_mark_done(st, C.gm, rho == 0.0 ? 1 : 3);
  }
  __syncthreads();
  if (!s_go) return;
  // first-pass column j: b_k / rho, then gamma - a_{j-1}
  const double ir = gm_rcp(rho);
  for (int k = threadIdx.x; k < j; k += blockDim.x) {
    gd[L.hcol() + 2 * k] = __ldcg(&gd[L.h2() + 2 * k]) * ir;
    gd[L.hcol() + 2 * k + 1] = __ldcg(&gd[L.h2() + 2 * k + 1]) * ir;
  }
  if (threadIdx.x == 0) {
    const double ar = j > 0 ? __ldcg(&gd[L.coef() + 2 * (j - 1)]) : 0.0;
    const double ai = j > 0 ? __ldcg(&gd[L.coef() + 2 * (j - 1) + 1]) : 0.0;
    gd[L.hcol() + 2 * j] = gr - ar;
    gd[L.hcol() + 2 * j + 1] = gi - ai;
    st->j = j + 1;
  }
}

// Phase 3 of k_gm_dcgs over this CTA's elements [lo, hi).
template <typename VT>
__device__ __forceinline__ void gd_update(const double* gd, const GmLayout& L, int m, int n, int j, cplx<VT>* V,
                                          const cplx<VT>* X, cplx<VT>* U, int vs, int lo, int hi) {
  extern __shared__ __align__(16) unsigned char gsm[];
  __shared__ double sh[3];
  gd_scalars(gd, L, j, sh);
  __syncthreads();
  const double r2 = sh[0];
  const double irho = r2 > 0.0 ? gm_rcp(gm_sqrt(r2)) : 0.0;
  const double gr = sh[1], gi = sh[2];
  cplx<VT>* ca = reinterpret_cast<cplx<VT>*>(gsm);
  cplx<VT>* cb = ca + (m + 1);
  for (int k = threadIdx.x; k < j; k += blockDim.x) {
    const double ar = __ldcg(&gd[L.coef() + 2 * k]), ai = __ldcg(&gd[L.coef() + 2 * k + 1]);
    const double br = __ldcg(&gd[L.h2() + 2 * k]), bi = __ldcg(&gd[L.h2() + 2 * k + 1]);
    ca[k] = cplx<VT>((VT)ar, (VT)ai);
    cb[k] = cplx<VT>((VT)(br - (gr * ar - gi * ai)), (VT)(bi - (gr * ai + gi * ar)));
  }
  __syncthreads();
  const VT ir = (VT)irho, g_re = (VT)gr, g_im = (VT)gi;
  cplx<VT>* Vj = V + (size_t)j * n;
  for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    const cplx<VT> u = U[(size_t)i * vs], x = X[(size_t)i * vs];
    VT pr = u.re, pi = u.im;  // u - Q a
    VT qr = fma(-g_re, u.re, fma(g_im, u.im, x.re)), qi = fma(-g_re, u.im, fma(-g_im, u.re, x.im));  // w - gamma u
    const cplx<VT>* Vi = V + i;
    for (int k = 0; k < j; k += kGfChunk) {
      cplx<VT> v[kGfChunk];
#pragma unroll
      for (int q = 0; q < kGfChunk; q++) v[q] = k + q < j ? Vi[(size_t)(k + q) * n] : cplx<VT>();
#pragma unroll
      for (int q = 0; q < kGfChunk; q++) {
        if (k + q >= j) break;
        const cplx<VT> a = ca[k + q], b = cb[k + q];
        pr = fma(-a.re, v[q].re, pr);
        pr = fma(a.im, v[q].im, pr);
        pi = fma(-a.re, v[q].im, pi);
        pi = fma(-a.im, v[q].re, pi);
        qr = fma(-b.re, v[q].re, qr);
        qr = fma(b.im, v[q].im, qr);
        qi = fma(-b.re, v[q].im, qi);
        qi = fma(-b.im, v[q].re, qi);
      }
    }
    Vj[i] = cplx<VT>(pr * ir, pi * ir);
    U[(size_t)i * vs] = cplx<VT>(qr * ir, qi * ir);
  }
}

// One iteration with delayed reorthogonalisation (cooperative launch; FP32 cycles). U: the matvec
// input u_j (block vectors; it receives u_{j+1}), W: w = A u_j. givens as in k_gm_fused (1: the
// caller forks k_gm_dgivens; 2: the extra last CTA of each cycle).
template <typename VT>
__global__ void __launch_bounds__(kGmThreads, 3) k_gm_dcgs(GmCols C, int m, int n, int LG, cplx<VT>* V,
                                                           const cplx<VT>* __restrict__ W, cplx<VT>* U, int givens) {
  // every cycle of the batch has ended (set by a Givens step of an earlier kernel, so all CTAs read
  // the same value): the iterations left in a captured chunk pass without their barriers
  if (*(volatile const int*)&C.gm->done_all) return;
  const int r = blockIdx.y, G = (int)gridDim.x - (givens == 2 ? 1 : 0);
  const bool giv_cta = givens == 2 && (int)blockIdx.x == G;
  const unsigned total = gridDim.x * gridDim.y;
  GState* st = C.st + r;
  double* gd = C.gd + r * C.gds;
  V += r * C.Vs;
  const cplx<VT>* X = W + r;
  U += r;
  const GmLayout L{m, LG};
  const bool run = st->done == 0;  // changed only by the Givens step, after the reduction
  const bool work = run && !giv_cta;
  const int j = st->j;
  int lo, hi;
  {
    const int per = (n + G - 1) / G;
    lo = min(n, (int)blockIdx.x * per);
    hi = min(n, lo + per);
  }
  bool ok = true;
  // 1: dots of the basis against u_j and w; |u_j|^2 and u_j^H w
  if (work) {
    gd_dot_partials<VT>(V, U, X, C.vs, lo, hi - lo, n, j, gd + L.part(), gd + L.part2(), G);
    VT al = 0, br = 0, bi = 0;
    for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
      const cplx<VT> u = U[(size_t)i * C.vs], x = X[(size_t)i * C.vs];
      al = fma(u.re, u.re, fma(u.im, u.im, al));
      br = fma(u.re, x.re, fma(u.im, x.im, br));
      bi = fma(u.re, x.im, fma(-u.im, x.re, bi));
    }
    __shared__ VT sw[3][kGmWarps];
    al = warp_sum(al);
    br = warp_sum(br);
    bi = warp_sum(bi);
    if ((threadIdx.x & 31) == 0) {
      sw[0][threadIdx.x >> 5] = al;
      sw[1][threadIdx.x >> 5] = br;
      sw[2][threadIdx.x >> 5] = bi;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
      VT t = 0;
      for (int w = 0; w < kGmWarps; w++) t += sw[threadIdx.x][w];
      gd[L.abpart() + 3 * blockIdx.x + threadIdx.x] = (double)t;
    }
  }
  ok = gm_grid_barrier(C.gm, total) && ok;
  // 2: the sums
  if (work && ok) gd_reduce<VT>(gd, L, G, j);
  ok = gm_grid_barrier(C.gm, total) && ok;
  if (givens == 1) grid_dep_launch();  // the next matvec reads u_{j+1} only after this kernel
  if (!run) return;
  if (!ok) {
    if (blockIdx.x == 0 && threadIdx.x == 0) gm_mark_done(st, C.gm, 3);
    return;
  }
  if (giv_cta) {
    gd_givens<VT>(C, st, gd, L, m, j);
    return;
  }
  // 3 (not after a full basis: iteration m only finishes column m - 1):
  // q_j = (u - Q a) / rho into V_j, u_{j+1} = (w - gamma u - Q (b - gamma a)) / rho into U
  if (j < m) gd_update<VT>(gd, L, m, n, j, V, X, U, C.vs, lo, hi);
  if (givens == 0 && blockIdx.x == 0) {
    __syncthreads();
    gd_givens<VT>(C, st, gd, L, m, j);
  }
}

// The Givens step of a delayed-reorthogonalisation iteration on its own (k_gm_dcgs launched with
// givens = 1), one CTA per cycle, after that kernel has completed.
template <typename VT>
__global__ void __launch_bounds__(kGmThreads) k_gm_dgivens(GmCols C, int m, int LG) {
  GState* st = C.st + blockIdx.y;
  if (st->done) return;
  double* gd = C.gd + blockIdx.y * C.gds;
  gd_givens<VT>(C, st, gd, GmLayout{m, LG}, m, st->j);
}

// y = R^{-1} g over the completed columns, then coef_k = y_k s_k (one CTA).
__global__ void __launch_bounds__(kGmThreads) k_gm_solve(GmCols C, int m, int G) {
  const GmLayout L{m, G};
  const GState* st = C.st + blockIdx.y;
  double* gd = C.gd + blockIdx.y * C.gds;
  const int jj = st->done == 3 ? 0 : st->j;  // a failed cycle adds nothing
  extern __shared__ __align__(16) unsigned char gsm[];
  Dc* gs = reinterpret_cast<Dc*>(gsm);  // jj entries
  for (int k = threadIdx.x; k < jj; k += blockDim.x) gs[k] = dc(gd[L.g() + 2 * k], gd[L.g() + 2 * k + 1]);
  __shared__ Dc yk;
  __syncthreads();
  for (int k = jj - 1; k >= 0; k--) {
    const double* Rk = gd + L.R() + 2 * (size_t)k * m;  // column k
    if (threadIdx.x == 0) {
      const double id = gm_rcp(Rk[2 * k]);  // the diagonal is real and positive
      yk = dc(gs[k].re * id, gs[k].im * id);
      const double sk = gd[L.s() + k];
      gd[L.coef() + 2 * k] = yk.re * sk;
      gd[L.coef() + 2 * k + 1] = yk.im * sk;
    }
    __syncthreads();
    const Dc y = yk;
    for (int l = threadIdx.x; l < k; l += blockDim.x) gs[l] = gs[l] - dc(Rk[2 * l], Rk[2 * l + 1]) * y;
    __syncthreads();
  }
}

// x = sum_k coef_k V_k over the completed columns (complex FP64 vector, or FP32 block vectors).
template <typename VT, typename XT>
__global__ void __launch_bounds__(kGmThreads) k_gm_x(GmCols C, int m, int n, const cplx<VT>* __restrict__ V,
                                                     cplx<XT>* x) {
  const GmLayout L{m, 1};
  const int r = blockIdx.y;
  const GState* st = C.st + r;
  const double* gd = C.gd + r * C.gds;
  V += r * C.Vs;
  x += r;
  const int jj = st->done == 3 ? 0 : st->j;
  extern __shared__ __align__(16) unsigned char gsm[];
  cplx<VT>* coef = reinterpret_cast<cplx<VT>*>(gsm);
  for (int k = threadIdx.x; k < jj; k += blockDim.x)
    coef[k] = cplx<VT>((VT)gd[L.coef() + 2 * k], (VT)gd[L.coef() + 2 * k + 1]);
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    VT ar = 0, ai = 0;
    const cplx<VT>* Vi = V + i;
#pragma unroll 4
    for (int k = 0; k < jj; k++) {
      const cplx<VT> v = Vi[(size_t)k * n];
      const cplx<VT> c = coef[k];
      ar = fma(c.re, v.re, ar);
      ar = fma(-c.im, v.im, ar);
      ai = fma(c.re, v.im, ai);
      ai = fma(c.im, v.re, ai);
    }
    x[(size_t)i * C.vs] = cplx<XT>((XT)ar, (XT)ai);
  }
}

// ------------------------------------------------------------------------------------------
// Host side
// ------------------------------------------------------------------------------------------
int gmres_grid(int n) {
  return std::max(device_sm_count(), (n + kSliceMax - 1) / kSliceMax);
}

size_t gmres_scalar_doubles(int m, int n) {
  return GmLayout{m, gmres_grid(n)}.total();
}

static GmCols cols(const GmresBufs& B) {
  return GmCols{B.state, B.gm, B.gd, B.gds, B.Vs, B.vs};
}

void gmres_enqueue_init(const GmresBufs& B, double tol, cudaStream_t s) {
  const dim3 grid(gmres_grid(B.n), B.nrb);
  const GmCols C = cols(B);
  note_launch();
  if (B.vec64)
    k_gm_init<double, double><<<grid, kGmThreads, 0, s>>>(C, B.m, B.n, (const cd*)B.b, (cplx<double>*)B.V,
                                                          (cplx<double>*)B.q, tol, B.tolv);
  else if (B.b32)
    k_gm_init<float, float><<<grid, kGmThreads, 0, s>>>(C, B.m, B.n, (const cf*)B.b, (cplx<float>*)B.V,
                                                        (cplx<float>*)B.q, tol, B.tolv);
  else
    k_gm_init<float, double><<<grid, kGmThreads, 0, s>>>(C, B.m, B.n, (const cd*)B.b, (cplx<float>*)B.V,
                                                         (cplx<float>*)B.q, tol, B.tolv);
  AC3D_CUDA(cudaGetLastError());
}

size_t gmres_update_smem(int m) {
  // the update pass keeps j + 1 coefficients, then 4 j + 3 complex FP64 values of the rotation
  return std::max(sizeof(cplx<double>) * ((size_t)m + 1), sizeof(double) * 2 * (4 * (size_t)m + 3));
}

// The Gram-Schmidt passes of one iteration, after the matvec into B.W. Returns true if the
// Givens step was left to k_gm_rotate (a fused kernel with B.rot_stream set).
template <typename VT>
static bool enqueue_gs(const GmresBufs& B, cudaStream_t s) {
  const dim3 grid(gmres_grid(B.n), B.nrb);
  const size_t smem = gmres_update_smem(B.m);
  // FP32 cycles with two passes: delayed reorthogonalisation (k_gm_dcgs)
  constexpr bool fp32 = sizeof(VT) == 4;
  const bool dcgs = fp32 && B.reorth;
  // with the static arrays, long cycles pass the 48 KB that needs no opt-in
  static std::once_flag once;
  static int fused_per_sm = 0, dcgs_per_sm = 0;  // resident CTAs per SM of the cooperative kernels
  std::call_once(once, [] {
    const int sm = (int)gmres_update_smem(kGmMaxRestart);
    AC3D_CUDA(cudaFuncSetAttribute(k_gm_update<VT>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    AC3D_CUDA(cudaFuncSetAttribute(k_gm_fused<VT>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    AC3D_CUDA(cudaFuncSetAttribute(k_gm_rotate<VT>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
    AC3D_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fused_per_sm, k_gm_fused<VT>, kGmThreads, sm));
    if constexpr (fp32) {
      AC3D_CUDA(cudaFuncSetAttribute(k_gm_dcgs<VT>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
      AC3D_CUDA(cudaFuncSetAttribute(k_gm_dgivens<VT>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
      AC3D_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&dcgs_per_sm, k_gm_dcgs<VT>, kGmThreads, sm));
    }
  });
  if (B.m > kGmMaxRestart) throw Error(3, "internal: GMRES cycle longer than the update pass supports");
  // one cooperative launch when every cycle of the batch can have a CTA resident at once
  const int LG = gmres_grid(B.n);
  const int cap = (dcgs ? dcgs_per_sm : fused_per_sm) * device_sm_count();
  const int Gc = std::min(LG, cap / std::max(B.nrb, 1));
  if (Gc >= 1 && (dcgs || !B.reorth || B.W2)) {
    const GmCols C = cols(B);
    // the Givens step: forked (rot_stream), else on one more CTA per cycle when it fits
    const int givens = B.rot_stream ? 1 : ((Gc + 1) * B.nrb <= cap ? 2 : 0);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(Gc + (givens == 2 ? 1 : 0), B.nrb);
    cfg.blockDim = dim3(kGmThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    note_launch();
    if constexpr (fp32) {
      if (dcgs)
        AC3D_CUDA(cudaLaunchKernelEx(&cfg, k_gm_dcgs<VT>, C, B.m, B.n, LG, (cplx<VT>*)B.V, (const cplx<VT>*)B.W,
                                     (cplx<VT>*)B.q, givens));
    }
    if (!dcgs)
      AC3D_CUDA(cudaLaunchKernelEx(&cfg, k_gm_fused<VT>, C, B.m, B.n, LG, (cplx<VT>*)B.V, (const cplx<VT>*)B.W,
                                   (cplx<VT>*)B.W2, (cplx<VT>*)B.q, B.reorth, givens));
    if (givens != 1) return false;
    // the Givens step on the branch: it waits for this kernel, and the next Gram-Schmidt kernel
    // waits for it (the caller joins the branch back)
    AC3D_CUDA(cudaEventRecord(B.ev_gs, s));
    AC3D_CUDA(cudaStreamWaitEvent(B.rot_stream, B.ev_gs, 0));
    static int prio_high = [] {
      int lo = 0, hi = 0;
      AC3D_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
      return hi;
    }();
    cudaLaunchConfig_t rc = {};
    rc.gridDim = dim3(1, B.nrb);
    rc.blockDim = dim3(kGmThreads);
    rc.dynamicSmemBytes = smem;
    rc.stream = B.rot_stream;
    cudaLaunchAttribute rattr[1];
    rattr[0].id = cudaLaunchAttributePriority;  // ahead of the matvec's waiting CTAs
    rattr[0].val.priority = prio_high;
    rc.attrs = rattr;
    rc.numAttrs = 1;
    note_launch();
    if constexpr (fp32) {
      if (dcgs) AC3D_CUDA(cudaLaunchKernelEx(&rc, k_gm_dgivens<VT>, C, B.m, LG));
    }
    if (!dcgs) AC3D_CUDA(cudaLaunchKernelEx(&rc, k_gm_rotate<VT>, C, B.m, LG, Gc, B.reorth));
    AC3D_CUDA(cudaEventRecord(B.ev_rot, B.rot_stream));
    return true;
  }
  const GmCols C = cols(B);
  launch_k(true, k_gm_dots<VT>, grid, dim3(kGmThreads), 0, s, C, B.m, B.n, (const cplx<VT>*)B.V,
           (const cplx<VT>*)B.W, 0);
  if (B.reorth) {
    // first pass into W2, with the second pass's dots of W2
    launch_k(true, k_gm_update<VT>, grid, dim3(kGmThreads), smem, s, C, B.m, B.n, (cplx<VT>*)B.V,
             (const cplx<VT>*)B.W, (cplx<VT>*)B.W2, (cplx<VT>*)B.q, 0, 0);
    launch_k(true, k_gm_update<VT>, grid, dim3(kGmThreads), smem, s, C, B.m, B.n, (cplx<VT>*)B.V,
             (const cplx<VT>*)B.W2, (cplx<VT>*)B.W2, (cplx<VT>*)B.q, 1, 1);
  } else {
    launch_k(true, k_gm_update<VT>, grid, dim3(kGmThreads), smem, s, C, B.m, B.n, (cplx<VT>*)B.V,
             (const cplx<VT>*)B.W, (cplx<VT>*)B.W2, (cplx<VT>*)B.q, 0, 1);
  }
  return false;
}

// Waits on stream s for the Givens branch of the previous iteration, if it forked one.
static void join_rotation(const GmresBufs& B, bool forked, cudaStream_t s) {
  if (forked) AC3D_CUDA(cudaStreamWaitEvent(s, B.ev_rot, 0));
}

void gmres_enqueue_iterations(const GmresBufs& B, const DevPartition& DP, const DevHMat& H, bool tr, int count,
                              cudaStream_t s) {
  bool forked = false;
  for (int i = 0; i < count; i++) {
    MatvecEpilogue ep;  // no fused dots
    launch_matvec_ex(DP, H, tr, B.vec64, B.q, B.W, nullptr, ep, &B.gm->done_all, s, nullptr, i > 0);
    join_rotation(B, forked, s);
    forked = B.vec64 ? enqueue_gs<double>(B, s) : enqueue_gs<float>(B, s);
  }
  join_rotation(B, forked, s);
}

void gmres_enqueue_iterations_block(const GmresBufs& B, const MultiBufs& MB, const DevPartition& DP,
                                    const DevHMat& H, int count, cudaStream_t s) {
  bool forked = false;
  for (int i = 0; i < count; i++) {
    launch_mmatvec(DP, H, MB, B.q, B.W, nullptr, nullptr, &B.gm->done_all, s);
    join_rotation(B, forked, s);
    forked = enqueue_gs<float>(B, s);
  }
  join_rotation(B, forked, s);
}

void gmres_enqueue_finish(const GmresBufs& B, void* x, cudaStream_t s) {
  const int G = gmres_grid(B.n);
  const GmCols C = cols(B);
  note_launch();
  k_gm_solve<<<dim3(1, B.nrb), kGmThreads, sizeof(double) * 2 * (size_t)B.m, s>>>(C, B.m, G);
  AC3D_CUDA(cudaGetLastError());
  const dim3 gx(std::max(1, std::min((B.n + kGmThreads - 1) / kGmThreads, 4 * device_sm_count())), B.nrb);
  note_launch();
  if (B.vec64)
    k_gm_x<double, double><<<gx, kGmThreads, sizeof(cplx<double>) * (size_t)B.m, s>>>(
        C, B.m, B.n, (const cplx<double>*)B.V, (cplx<double>*)x);
  else if (B.b32)
    k_gm_x<float, float><<<gx, kGmThreads, sizeof(cplx<float>) * (size_t)B.m, s>>>(
        C, B.m, B.n, (const cplx<float>*)B.V, (cplx<float>*)x);
  else
    k_gm_x<float, double><<<gx, kGmThreads, sizeof(cplx<float>) * (size_t)B.m, s>>>(
        C, B.m, B.n, (const cplx<float>*)B.V, (cplx<double>*)x);
  AC3D_CUDA(cudaGetLastError());
}

}  // namespace ac3d
