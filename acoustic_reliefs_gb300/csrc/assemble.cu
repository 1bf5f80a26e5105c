// H-matrix assembly on the GPU: near-field quadrature and partially pivoted ACA.
//
// Near field (compute_block, integrate.cpp:87-100; hmatrix.cpp:20-44): one CTA per dense block,
// one thread per entry, 6-point rule, displacement formed in FP64. Storage is column-major per
// block (entry (r, c) at c * m + r), blocks packed back to back.
//
// ACA (compute_ACA_block, aca.cpp:38-82, with argmax rules aca.cpp:9-36): one CTA per admissible
// block. The sequence of the reference is kept exactly: first row pivot 0; v = row - U(i,:) V;
// column pivot j = first index of max |v|^2; V row = v / v_j (v itself when v_j == 0 and the zero
// guard is on); u = column - U V(:, j); err += |u|^2 |v|^2 + 2 sum_q |u^T U_q| |v V_q^T| (plain,
// non-conjugated products); stop when sqrt(|u|^2 |v|^2 / err) <= eps, dropping the converging
// term; next row pivot = first max of |u|^2 over rows not used yet. Each rank-1 term (u | v) is
// bump-allocated from one pool with an atomic counter, so storage is proportional to the actual
// ranks; the pool offset of term q of block b is term_off[b * maxk + q].
#include "common.cuh"
#include "internal.h"
#include "listener.h"

#include <algorithm>

namespace ac3d {

namespace {
constexpr int kAcaThreads = 256;
constexpr int kAcaWarps = kAcaThreads / 32;
}  // namespace

template <typename R>
__global__ void __launch_bounds__(256) near_kernel(GeoView<R> G, const int4* __restrict__ blocks,
                                                   const long long* __restrict__ near_off, R k, cplx<R>* out) {
  const int b = blockIdx.x;
  const int4 q = blocks[b];
  const int m = q.y - q.x, n = q.w - q.z;
  cplx<R>* dst = out + near_off[b];
  const int mn = m * n;
  for (int t = threadIdx.x; t < mn; t += blockDim.x) {
    int c = t / m, r = t - c * m;
    dst[t] = entry_near<R>(k, G, G.cen[q.x + r], q.z + c);
  }
}

// Block-wide argmax of (value, index): larger value wins, smaller index on ties. Threads start
// from (-1, 0) and skip NaN values, which reproduces a sequential scan with a strict `>` from -1.
template <typename R>
__device__ __forceinline__ void block_argmax(R& val, int& idx, R* sv, int* si) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    R ov = __shfl_xor_sync(0xffffffffu, val, o);
    int oi = __shfl_xor_sync(0xffffffffu, idx, o);
    if (ov > val || (ov == val && oi < idx)) {
      val = ov;
      idx = oi;
    }
  }
  if (lane == 0) {
    sv[w] = val;
    si[w] = idx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    R bv = sv[0];
    int bi = si[0];
    for (int i = 1; i < kAcaWarps; i++)
      if (sv[i] > bv || (sv[i] == bv && si[i] < bi)) {
        bv = sv[i];
        bi = si[i];
      }
    sv[0] = bv;
    si[0] = bi;
  }
  __syncthreads();
  val = sv[0];
  idx = si[0];
  __syncthreads();
}

__device__ __forceinline__ double block_sum(double v, double* sd) {
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sd[w] = v;
  __syncthreads();
  double s = 0;
  if (threadIdx.x == 0) {
    for (int i = 0; i < kAcaWarps; i++) s += sd[i];
    sd[0] = s;
  }
  __syncthreads();
  s = sd[0];
  __syncthreads();
  return s;
}

template <typename R, typename P4>
struct AcaArgs {
  GeoView<R> G;
  const int4* blocks;
  const int* order;
  const P4* rowpts;
  R k;
  double eps;
  int maxk;
  int zero_guard;
  int iter_cap;
  cplx<R>* pool;
  long long pool_cap;
  unsigned long long* pool_used;
  long long* term_off;
  int* rank;
  int* status;
  int* passes;  // per block: rows (and columns) evaluated, or null
};

template <typename R, typename P4>
__global__ void __launch_bounds__(kAcaThreads) aca_kernel(AcaArgs<R, P4> A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ R s_rv[kAcaWarps];
  __shared__ int s_ri[kAcaWarps];
  __shared__ double s_d[kAcaWarps];
  __shared__ long long s_base;
  __shared__ int s_flag;

  const int b = A.order[blockIdx.x];
  const int4 q = A.blocks[b];
  const int rs = q.x, cs = q.z, m = q.y - q.x, n = q.w - q.z;
  int iter_lim = min(A.maxk, min(m - 1, n - 1));
  if (iter_lim < 0) iter_lim = 0;
  if (iter_lim > A.iter_cap) iter_lim = A.iter_cap;  // host guarantees iter_cap >= every iter_lim

  cplx<R>* uq = (cplx<R>*)smem_raw;
  cplx<R>* vq = uq + A.iter_cap;
  long long* toff = (long long*)(vq + A.iter_cap);
  unsigned* used = (unsigned*)(toff + A.iter_cap);

  const int tid = threadIdx.x, T = blockDim.x, lane = tid & 31, warp = tid >> 5;

  // Exactly-zero blocks: every source element lies in one axis-aligned plane x_d = v (edge
  // vectors have an exact zero d-component) that also holds every target point exactly. Then
  // r_d = 0 and the normal has no other component, each quadrature term is exactly 0, and the
  // iteration below would produce only zero terms, none of which is stored. Checked on the
  // current geometry, so height updates are honoured.
  if (A.zero_guard && iter_lim > 0) {
    int zero_axes = 0;
    for (int d = 0; d < 3; d++) {
      const double v = d == 0 ? A.G.va[cs].x : (d == 1 ? A.G.va[cs].y : A.G.va[cs].z);
      int ok = 1;
      for (int j = tid; j < n && ok; j += T) {
        const double4 a = A.G.va[cs + j];
        const ElemGeo<R> g = A.G.eg[cs + j];
        const double ad = d == 0 ? a.x : (d == 1 ? a.y : a.z);
        ok = ad == v && g.ab[d] == R(0) && g.ac[d] == R(0);
      }
      for (int i = tid; i < m && ok; i += T) {
        const double4 p = A.G.cen[rs + i];
        ok = (d == 0 ? p.x : (d == 1 ? p.y : p.z)) == v;
      }
      if (__syncthreads_and(ok)) zero_axes++;
    }
    if (zero_axes) {
      if (tid == 0) {
        A.rank[b] = 0;
        if (A.passes) A.passes[b] = 0;
      }
      return;
    }
  }

  for (int w = tid; w < (m + 31) / 32; w += T) used[w] = 0;
  __syncthreads();
  if (tid == 0) used[0] = 1u;
  double err = 0;  // meaningful in thread 0
  int i = 0, iter = 0;
  int nst = 0;           // stored (nonzero) terms; a term with u == 0 or v == 0 is exactly zero in
                         // every later residual, cross term and product, so it is not stored
  bool need_alloc = true;
  int npass = 0;  // loop passes that evaluated a row and a column
  __syncthreads();

  while (iter < iter_lim) {
    // --- storage of the current term (a slot is reused after a zero term) -------------------
    if (need_alloc) {
      if (tid == 0) {
        unsigned long long need = (unsigned long long)(m + n);
        unsigned long long base = atomicAdd(A.pool_used, need);
        s_flag = (base + need > (unsigned long long)A.pool_cap) ? 1 : 0;
        s_base = (long long)base;
        if (s_flag) atomicOr(A.status, 1);
      }
      __syncthreads();
      if (s_flag) break;
      need_alloc = false;
    }
    npass++;
    cplx<R>* unew = A.pool + s_base;
    cplx<R>* vnew = unew + m;
    for (int p = tid; p < nst; p += T) uq[p] = A.pool[toff[p] + i];
    __syncthreads();

    // --- row residual v = M(i, :) - U(i, :) V ---------------------------------------------
    const P4 pi = A.rowpts[rs + i];
    R best = R(-1);
    int bidx = 0;
    for (int c = tid; c < n; c += T) {
      cplx<R> v = entry_far<R>(A.k, A.G, pi, cs + c);
      for (int p = 0; p < nst; p++) cfms(v, uq[p], A.pool[toff[p] + m + c]);
      vnew[c] = v;
      R a = abs2(v);
      if (a > best) {
        best = a;
        bidx = c;
      }
    }
    block_argmax<R>(best, bidx, s_rv, s_ri);
    const int j = bidx;
    const cplx<R> vj = vnew[j];
    for (int p = tid; p < nst; p += T) vq[p] = A.pool[toff[p] + m + j];
    __syncthreads();
    const bool keep = A.zero_guard && vj.re == R(0) && vj.im == R(0);
    double vn = 0;
    for (int c = tid; c < n; c += T) {
      cplx<R> v = vnew[c];
      if (!keep) v = cdiv(v, vj);
      vnew[c] = v;
      vn += (double)v.re * (double)v.re + (double)v.im * (double)v.im;
    }

    // --- column residual u = M(:, j) - U V(:, j) ------------------------------------------
    double un = 0;
    for (int r = tid; r < m; r += T) {
      cplx<R> u = entry_far<R>(A.k, A.G, A.rowpts[rs + r], cs + j);
      for (int p = 0; p < nst; p++) cfms(u, A.pool[toff[p] + r], vq[p]);
      unew[r] = u;
      un += (double)u.re * (double)u.re + (double)u.im * (double)u.im;
    }
    __syncthreads();

    // --- cross terms sum_q |u^T U_q| |v V_q^T| (one warp per earlier stored term) -----------
    double dots = 0;
    for (int p = warp; p < nst; p += kAcaWarps) {
      const cplx<R>* Up = A.pool + toff[p];
      const cplx<R>* Vp = Up + m;
      cplx<R> ud(0, 0), vd(0, 0);
      for (int r = lane; r < m; r += 32) cfma(ud, unew[r], Up[r]);
      for (int c = lane; c < n; c += 32) cfma(vd, vnew[c], Vp[c]);
      double udr = warp_sum((double)ud.re), udi = warp_sum((double)ud.im);
      double vdr = warp_sum((double)vd.re), vdi = warp_sum((double)vd.im);
      if (lane == 0) dots += sqrt(udr * udr + udi * udi) * sqrt(vdr * vdr + vdi * vdi);
    }
    un = block_sum(un, s_d);
    vn = block_sum(vn, s_d);
    dots = block_sum(dots, s_d);
    if (tid == 0) {
      err += un * vn + 2 * dots;
      s_flag = (sqrt(un * vn / err) <= A.eps) ? 1 : 0;
    }
    __syncthreads();
    if (s_flag) break;
    const bool zero_term = (un == 0.0) || (vn == 0.0);

    // --- next row pivot: first max |u|^2 over unused rows --------------------------------
    best = R(-1);
    bidx = 0;
    for (int r = tid; r < m; r += T) {
      if ((used[r >> 5] >> (r & 31)) & 1u) continue;
      R a = abs2(unew[r]);
      if (a > best) {
        best = a;
        bidx = r;
      }
    }
    block_argmax<R>(best, bidx, s_rv, s_ri);
    i = bidx;
    if (tid == 0) {
      used[i >> 5] |= 1u << (i & 31);
      if (!zero_term) {
        toff[nst] = s_base;
        A.term_off[(long long)b * A.maxk + nst] = s_base;
      }
    }
    if (!zero_term) {
      nst++;
      need_alloc = true;
    }
    iter++;
    __syncthreads();
  }
  if (tid == 0) {
    A.rank[b] = nst;
    if (A.passes) A.passes[b] = npass;
  }
}

// ------------------------------------------------------------------------------------------
// Warp-per-block ACA for blocks of at most 32 LPL rows and columns: the same sequence as
// aca_kernel (pivot rules, stop rule, dropped converging term, zero terms not stored, exactly-zero
// blocks skipped) with warp shuffles in place of block barriers. Lane l owns rows and columns
// l + 32 k (k < LPL) and keeps the current term's u and v there in registers; the earlier terms
// are read from the pool four at a time. Norms and cross terms are summed in the storage type R
// (the FP64 path is unchanged); the error estimate is accumulated in FP64.
// ------------------------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ void warp_argmax(R& val, int& idx) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    R ov = __shfl_xor_sync(0xffffffffu, val, o);
    int oi = __shfl_xor_sync(0xffffffffu, idx, o);
    if (ov > val || (ov == val && oi < idx)) {
      val = ov;
      idx = oi;
    }
  }
}

// One out-of-line copy of the far-field entry for the warp kernel: its rows-per-lane loops are
// unrolled, and inlining the 6-point evaluation (with sincos) at every unrolled site made the code
// outgrow the instruction cache.
template <typename R, typename P4>
__device__ __noinline__ cplx<R> entry_far_call(R k, const GeoView<R>* G, P4 p, int e) {
  return entry_far<R>(k, *G, p, e);
}

template <typename R>
__device__ __forceinline__ R warp_sum_r(R v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// acc -= sum_{p < nst} coef[p] * pool[toff[p] + off]: loads issued four at a time
template <typename R>
__device__ __forceinline__ void sub_terms(cplx<R>& acc, const cplx<R>* coef, const cplx<R>* __restrict__ pool,
                                          const long long* toff, long long off, int nst) {
  int p = 0;
  for (; p + 4 <= nst; p += 4) {
    const cplx<R> a0 = pool[toff[p] + off], a1 = pool[toff[p + 1] + off];
    const cplx<R> a2 = pool[toff[p + 2] + off], a3 = pool[toff[p + 3] + off];
    cfms(acc, coef[p], a0);
    cfms(acc, coef[p + 1], a1);
    cfms(acc, coef[p + 2], a2);
    cfms(acc, coef[p + 3], a3);
  }
  for (; p < nst; p++) cfms(acc, coef[p], pool[toff[p] + off]);
}

// Blocks of 129-256 rows (8 rows per lane) are few (less than one wave at 4 CTAs per SM), so
// that variant takes the registers of 2 CTAs per SM and keeps its u / v rows unspilled.
template <typename R, typename P4, int LPL>
__global__ void __launch_bounds__(256, sizeof(R) == 4 ? (LPL == 8 ? 2 : 4) : 1)
    aca_warp_kernel(AcaArgs<R, P4> A, int nblocks) {
  __shared__ __align__(16) unsigned char s_raw[8 * kWarpAcaTerms * (2 * sizeof(cplx<R>) + sizeof(long long))];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int bi = blockIdx.x * 8 + warp;
  if (bi >= nblocks) return;
  cplx<R>* uq = reinterpret_cast<cplx<R>*>(s_raw) + warp * kWarpAcaTerms;
  cplx<R>* vq = reinterpret_cast<cplx<R>*>(s_raw) + (8 + warp) * kWarpAcaTerms;
  long long* toff = reinterpret_cast<long long*>(s_raw + 16 * kWarpAcaTerms * sizeof(cplx<R>)) + warp * kWarpAcaTerms;
  const int b = A.order[bi];
  const int4 q = A.blocks[b];
  const int rs = q.x, cs = q.z, m = q.y - q.x, n = q.w - q.z;
  int iter_lim = min(A.maxk, min(m - 1, n - 1));
  if (iter_lim < 0) iter_lim = 0;
  if (iter_lim > kWarpAcaTerms) iter_lim = kWarpAcaTerms;  // the host routes only blocks that fit

  if (A.zero_guard && iter_lim > 0) {  // exactly-zero block (see aca_kernel)
    bool zero = false;
    for (int d = 0; d < 3 && !zero; d++) {
      const double4 a0 = A.G.va[cs];
      const double v = d == 0 ? a0.x : (d == 1 ? a0.y : a0.z);
      bool ok = true;
      for (int j = lane; j < n; j += 32) {
        const double4 a = A.G.va[cs + j];
        const ElemGeo<R> g = A.G.eg[cs + j];
        ok = ok && (d == 0 ? a.x : (d == 1 ? a.y : a.z)) == v && g.ab[d] == R(0) && g.ac[d] == R(0);
      }
      for (int i = lane; i < m; i += 32) {
        const double4 p = A.G.cen[rs + i];
        ok = ok && (d == 0 ? p.x : (d == 1 ? p.y : p.z)) == v;
      }
      zero = __all_sync(0xffffffffu, ok);
    }
    if (zero) {
      if (lane == 0) {
        A.rank[b] = 0;
        if (A.passes) A.passes[b] = 0;
      }
      return;
    }
  }

  unsigned used_l = lane == 0 ? 1u : 0u;  // bit k: row lane + 32 k is used (row 0 first)
  double err = 0;
  int i = 0, iter = 0, nst = 0, npass = 0;
  bool need_alloc = true;
  long long base = 0;
  cplx<R> u_l[LPL], v_l[LPL];
  while (iter < iter_lim) {
    if (need_alloc) {
      unsigned long long bb = 0;
      int ovf = 0;
      if (lane == 0) {
        const unsigned long long need = (unsigned long long)(m + n);
        bb = atomicAdd(A.pool_used, need);
        ovf = bb + need > (unsigned long long)A.pool_cap;
        if (ovf) atomicOr(A.status, 1);
      }
      ovf = __shfl_sync(0xffffffffu, ovf, 0);
      if (ovf) break;
      base = (long long)__shfl_sync(0xffffffffu, bb, 0);
      need_alloc = false;
    }
    npass++;
    cplx<R>* unew = A.pool + base;
    cplx<R>* vnew = unew + m;
    for (int p = lane; p < nst; p += 32) uq[p] = A.pool[toff[p] + i];
    __syncwarp();
    // row residual and column pivot
    const P4 pi = A.rowpts[rs + i];
    R best = R(-1);
    int bidx = 0;
#pragma unroll
    for (int k = 0; k < LPL; k++) {
      const int c = lane + 32 * k;
      if (c < n) {
        cplx<R> v = entry_far_call<R, P4>(A.k, &A.G, pi, cs + c);
        sub_terms(v, uq, A.pool, toff, (long long)m + c, nst);
        v_l[k] = v;
        const R a = abs2(v);
        if (a > best) {
          best = a;
          bidx = c;
        }
      }
    }
    warp_argmax<R>(best, bidx);
    const int j = bidx;
    cplx<R> mine = v_l[0];
#pragma unroll
    for (int k = 1; k < LPL; k++)
      if (k == (j >> 5)) mine = v_l[k];
    const cplx<R> vj(__shfl_sync(0xffffffffu, mine.re, j & 31), __shfl_sync(0xffffffffu, mine.im, j & 31));
    for (int p = lane; p < nst; p += 32) vq[p] = A.pool[toff[p] + m + j];
    __syncwarp();
    const bool keep = A.zero_guard && vj.re == R(0) && vj.im == R(0);
    R vn = 0;
#pragma unroll
    for (int k = 0; k < LPL; k++) {
      const int c = lane + 32 * k;
      if (c < n) {
        cplx<R> v = v_l[k];
        if (!keep) v = cdiv(v, vj);
        v_l[k] = v;
        vnew[c] = v;
        vn += abs2(v);
      }
    }
    // column residual
    R un = 0;
#pragma unroll
    for (int k = 0; k < LPL; k++) {
      const int r = lane + 32 * k;
      if (r < m) {
        cplx<R> u = entry_far_call<R, P4>(A.k, &A.G, A.rowpts[rs + r], cs + j);
        sub_terms(u, vq, A.pool, toff, (long long)r, nst);
        u_l[k] = u;
        unew[r] = u;
        un += abs2(u);
      }
    }
    // cross terms sum_q |u^T U_q| |v V_q^T|
    R dots = 0;
    for (int p = 0; p < nst; p++) {
      const cplx<R>* Up = A.pool + toff[p];
      const cplx<R>* Vp = Up + m;
      cplx<R> ud(0, 0), vd(0, 0);
#pragma unroll
      for (int k = 0; k < LPL; k++) {
        const int r = lane + 32 * k;
        if (r < m) cfma(ud, u_l[k], Up[r]);
        if (r < n) cfma(vd, v_l[k], Vp[r]);
      }
      const R udr = warp_sum_r(ud.re), udi = warp_sum_r(ud.im);
      const R vdr = warp_sum_r(vd.re), vdi = warp_sum_r(vd.im);
      dots += sqrt(udr * udr + udi * udi) * sqrt(vdr * vdr + vdi * vdi);
    }
    const double unt = (double)warp_sum_r(un), vnt = (double)warp_sum_r(vn);
    err += unt * vnt + 2 * (double)dots;
    if (sqrt(unt * vnt / err) <= A.eps) break;
    const bool zero_term = (unt == 0.0) || (vnt == 0.0);
    // next row pivot over unused rows
    best = R(-1);
    bidx = 0;
#pragma unroll
    for (int k = 0; k < LPL; k++) {
      const int r = lane + 32 * k;
      if (r < m && !((used_l >> k) & 1u)) {
        const R a = abs2(u_l[k]);
        if (a > best) {
          best = a;
          bidx = r;
        }
      }
    }
    warp_argmax<R>(best, bidx);
    i = bidx;
    if (lane == (i & 31)) used_l |= 1u << (i >> 5);
    if (!zero_term) {
      if (lane == 0) {
        toff[nst] = base;
        A.term_off[(long long)b * A.maxk + nst] = base;
      }
      nst++;
      need_alloc = true;
    }
    iter++;
    __syncwarp();
  }
  if (lane == 0) {
    A.rank[b] = nst;
    if (A.passes) A.passes[b] = npass;
  }
}

__global__ void rank_scan_kernel(const int* __restrict__ rank, int na, int* t_off) {
  __shared__ int sums[1024];
  const int tid = threadIdx.x;
  const int chunk = (na + 1023) / 1024;
  const int s = min(na, tid * chunk), e = min(na, s + chunk);
  int acc = 0;
  for (int i = s; i < e; i++) acc += rank[i];
  sums[tid] = acc;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    int v = tid >= o ? sums[tid - o] : 0;
    __syncthreads();
    sums[tid] += v;
    __syncthreads();
  }
  int base = tid ? sums[tid - 1] : 0;
  for (int i = s; i < e; i++) {
    t_off[i] = base;
    base += rank[i];
  }
  if (tid == 1023) t_off[na] = sums[1023];
}

template <typename R>
GeoView<R> geo_view(const DevGeometry& G);
template <>
GeoView<float> geo_view<float>(const DevGeometry& G) {
  return {G.cen.as<double4>(), G.va.as<double4>(), G.eg32.as<ElemGeo<float>>(), G.cen32.as<float4>(),
          G.va32.as<float4>(), G.ne};
}
template <>
GeoView<double> geo_view<double>(const DevGeometry& G) {
  return {G.cen.as<double4>(), G.va.as<double4>(), G.eg64.as<ElemGeo<double>>(), G.cen32.as<float4>(),
          G.va32.as<float4>(), G.ne};
}

void launch_near_assembly(const DevGeometry& G, const DevPartition& DP, DevHMat& H, cudaStream_t s) {
  if (DP.nd == 0) return;
  note_launch();
  if (H.prec == PREC_FP64)
    near_kernel<double><<<DP.nd, 256, 0, s>>>(geo_view<double>(G), DP.blocks_d.as<int4>(),
                                              DP.near_off.as<long long>(), H.k, H.near.as<cd>());
  else
    near_kernel<float><<<DP.nd, 256, 0, s>>>(geo_view<float>(G), DP.blocks_d.as<int4>(),
                                             DP.near_off.as<long long>(), (float)H.k, H.near.as<cf>());
  AC3D_CUDA(cudaGetLastError());
}

template <typename R, typename P4, int LPL>
static void aca_launch_warp(const AcaArgs<R, P4>& a, int nblocks, cudaStream_t s) {
  if (nblocks <= 0) return;
  note_launch();
  aca_warp_kernel<R, P4, LPL><<<(nblocks + 7) / 8, 256, 0, s>>>(a, nblocks);
  AC3D_CUDA(cudaGetLastError());
}

// aca_order = [CTA blocks | warp blocks up to 256 | up to 128 | up to 64], counts in DP.aca_split
template <typename R, typename P4>
static void aca_launch_all(AcaArgs<R, P4> a, const DevPartition& DP, int max_rows, cudaStream_t s,
                           cudaStream_t s_small) {
  // two streams with about equal work: the CTA blocks then the blocks up to 128 on s, the blocks
  // up to 256 then those up to 64 on s_small
  const int* order = DP.aca_order.as<int>();
  const int o1 = DP.aca_split[0], o2 = o1 + DP.aca_split[1], o3 = o2 + DP.aca_split[2];
  if (DP.aca_split[0] > 0) aca_launch_t(a, DP.aca_split[0], max_rows, s);
  a.order = order + o1;
  aca_launch_warp<R, P4, 8>(a, DP.aca_split[1], s_small);
  a.order = order + o2;
  aca_launch_warp<R, P4, 4>(a, DP.aca_split[2], s);
  a.order = order + o3;
  aca_launch_warp<R, P4, 2>(a, DP.aca_split[3], s_small);
}

template <typename R, typename P4>
static void aca_launch_t(const AcaArgs<R, P4>& a, int nblocks, int max_rows, cudaStream_t s) {
  size_t smem = (size_t)a.iter_cap * (2 * sizeof(cplx<R>) + sizeof(long long)) + (size_t)((max_rows + 31) / 32) * 4;
  if (smem > 48 * 1024) {
    if (smem > 227 * 1024) throw Error(4, "ACA block too large for shared memory");
    AC3D_CUDA(cudaFuncSetAttribute(aca_kernel<R, P4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  }
  note_launch();
  aca_kernel<R, P4><<<nblocks, kAcaThreads, smem, s>>>(a);
  AC3D_CUDA(cudaGetLastError());
}

void launch_aca(const DevGeometry& G, const DevPartition& DP, DevHMat& H, double eps, int max_rows, cudaStream_t s,
                cudaStream_t s_small) {
  if (DP.na == 0) return;
  int iter_cap = H.maxk;
  if (H.prec == PREC_FP64) {
    AcaArgs<double, double4> a{geo_view<double>(G), DP.blocks_a.as<int4>(), DP.aca_order.as<int>(),
                               G.cen.as<double4>(), H.k, eps, H.maxk, 1, iter_cap, H.pool.as<cd>(),
                               H.pool_cap, H.pool_used.as<unsigned long long>(), H.term_off.as<long long>(),
                               H.rank.as<int>(), (int*)(H.pool_used.as<unsigned long long>() + 1),
                               H.passes.as<int>()};
    aca_launch_all(a, DP, max_rows, s, s_small);
  } else {
    AcaArgs<float, float4> a{geo_view<float>(G), DP.blocks_a.as<int4>(), DP.aca_order.as<int>(),
                             G.cen32.as<float4>(), (float)H.k, eps, H.maxk, 1, iter_cap, H.pool.as<cf>(),
                             H.pool_cap, H.pool_used.as<unsigned long long>(), H.term_off.as<long long>(),
                             H.rank.as<int>(), (int*)(H.pool_used.as<unsigned long long>() + 1),
                             H.passes.as<int>()};
    aca_launch_all(a, DP, max_rows, s, s_small);
  }
}

// Flat list of stored terms for the matvec: task t -> (block, pool offset of the term).
__global__ void task_map_kernel(const int* __restrict__ rank, const int* __restrict__ t_off,
                                const long long* __restrict__ term_off, int na, int maxk, int* task_b,
                                long long* task_off) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= na) return;
  const int r = rank[b], o = t_off[b];
  for (int q = 0; q < r; q++) {
    task_b[o + q] = b;
    task_off[o + q] = term_off[(long long)b * maxk + q];
  }
}

void launch_rank_scan(const DevPartition& DP, DevHMat& H, cudaStream_t s) {
  note_launch();
  rank_scan_kernel<<<1, 1024, 0, s>>>(H.rank.as<int>(), DP.na, H.t_off.as<int>());
  AC3D_CUDA(cudaGetLastError());
  note_launch();
  task_map_kernel<<<(DP.na + 255) / 256, 256, 0, s>>>(H.rank.as<int>(), H.t_off.as<int>(), H.term_off.as<long long>(),
                                                       DP.na, H.maxk, H.task_b.as<int>(), H.task_off.as<long long>());
  AC3D_CUDA(cudaGetLastError());
}

// ------------------------------------------------------------------------------------------
// Listener ACA (compute_ACA_listener, aca.cpp:84-134): one block of L receivers x Ne elements,
// maxk 5000, no zero guard. Rows are receiver points.
// ------------------------------------------------------------------------------------------
void launch_listener_aca(const DevGeometry& G, int prec, const void* pts, int L, double k, double eps, int maxk,
                         void* pool, long long pool_cap, unsigned long long* used, long long* term_off, int* rank,
                         int* status, const int4* block, const int* order, cudaStream_t s) {
  int iter_lim = std::min(maxk, std::min(L - 1, G.ne - 1));
  if (iter_lim < 1) iter_lim = 1;
  if (prec == PREC_FP64) {
    AcaArgs<double, double4> a{geo_view<double>(G), block, order, (const double4*)pts, k, eps, maxk, 0, iter_lim,
                               (cd*)pool, pool_cap, used, term_off, rank, status, nullptr};
    aca_launch_t(a, 1, L, s);
  } else {
    AcaArgs<float, float4> a{geo_view<float>(G), block, order, (const float4*)pts, (float)k, eps, maxk, 0,
                             iter_lim, (cf*)pool, pool_cap, used, term_off, rank, status, nullptr};
    aca_launch_t(a, 1, L, s);
  }
}

}  // namespace ac3d
