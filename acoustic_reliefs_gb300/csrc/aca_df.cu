// Mixed-precision assembly with FP64-accurate entries: near-field entries, and the admissible
// blocks' rows and columns with the ACA recursion, evaluated in double-float arithmetic (about 47
// bits, on the FP32 pipes); everything is stored in complex FP32. Near-field entries of nearly
// coplanar neighbours cancel in r.n, so FP32 evaluation from FP64 displacements is not enough
// there (5.6e-5 instead of 1.3e-5 from the FP64 path on a 5280-triangle relief at 3.5 kHz).
//
// The ACA sequence is the reference's (compute_ACA_block, aca.cpp:38-82, argmax rules
// aca.cpp:9-36) exactly as the FP32 / FP64 kernels of assemble.cu run it: first row pivot 0;
// v = row - U(i,:) V; column pivot j = first index of max |v|^2; V row = v / v_j (v itself when
// v_j == 0); u = column - U V(:, j); err += |u|^2 |v|^2 + 2 sum_q |u^T U_q| |v V_q^T|; stop when
// sqrt(|u|^2 |v|^2 / err) <= eps, dropping the converging term; next row pivot = first max of
// |u|^2 over unused rows. Entries, residuals, the pivot magnitudes and the norms are double-float,
// so the pivots and ranks are the FP64 path's (the two differ only where two candidates agree to
// about 1e-12); the cross terms of the error estimate are FP32 sums of the leading parts (they
// only scale err). The estimate, the norms and the stopping test are double-float too (the FP64
// pipes of GB300 are too slow to hold them), the test as |u|^2 |v|^2 <= eps^2 err. The terms live in a double-float pool while the recursion needs them; packing
// rounds them to the FP32 per-leaf segments the matvec streams.
#include "common.cuh"
#include "df64.cuh"
#include "entry_df.cuh"
#include "internal.h"

namespace ac3d {

namespace {
constexpr int kDfThreads = 256;
constexpr int kDfWarps = kDfThreads / 32;
}  // namespace

struct AcaDfArgs {
  const double4* cen;          // FP64 centroids and vertices: the exactly-zero block test
  const double4* va;
  const ElemGeo<double>* eg;
  const DfPt* pts;             // double-float centroids (rows)
  const DfElem* el;            // double-float quadrature points and normals (columns)
  const float4* tab;           // df_sincos table in global memory (copied to shared memory)
  const int4* blocks;
  const int* order;
  df64 k;
  double eps;
  df64 eps2;       // eps^2 as a double-float (the stopping test)
  int maxk;
  int iter_cap;
  cdf* pool;
  long long pool_cap;
  unsigned long long* pool_used;
  long long* term_off;
  int* rank;
  int* status;
  int* passes;     // per block: rows (and columns) evaluated, or null
  int zero_guard;  // boundary blocks: v kept when v_j == 0 and exactly-zero blocks skipped
};

// One out-of-line copy of the entry (its loops are not unrolled into the callers' unrolled
// rows-per-lane loops; see entry_far_call in assemble.cu).
__device__ __noinline__ cdf entry_df_call(df64 k, const DfPt* p, const DfElem* e, const float4* tab) {
  return entry_df(k, p, e, tab);
}

__device__ __forceinline__ void load_table(const float4* __restrict__ g, float4* s) {
  for (int i = threadIdx.x; i < kDfTab; i += blockDim.x) s[i] = g[i];
  __syncthreads();
}

// Exactly-zero block (all source elements in one axis-aligned plane that holds every target
// point, judged on the FP64 geometry; see aca_kernel): evaluated by the `count` threads
// t0, t0 + step, ... of a warp or CTA; `all` reduces the verdict over them.
template <typename All>
__device__ __forceinline__ bool zero_block(const AcaDfArgs& A, int rs, int m, int cs, int n, int t0, int step,
                                           All all) {
  for (int d = 0; d < 3; d++) {
    const double4 a0 = A.va[cs];
    const double v = d == 0 ? a0.x : (d == 1 ? a0.y : a0.z);
    bool ok = true;
    for (int j = t0; j < n && ok; j += step) {
      const double4 a = A.va[cs + j];
      const ElemGeo<double> g = A.eg[cs + j];
      ok = (d == 0 ? a.x : (d == 1 ? a.y : a.z)) == v && g.ab[d] == 0.0 && g.ac[d] == 0.0;
    }
    for (int i = t0; i < m && ok; i += step) {
      const double4 p = A.cen[rs + i];
      ok = (d == 0 ? p.x : (d == 1 ? p.y : p.z)) == v;
    }
    if (all(ok)) return true;
  }
  return false;
}

__device__ __forceinline__ df64 shfl_df(df64 v, int src) {
  return {__shfl_sync(0xffffffffu, v.hi, src), __shfl_sync(0xffffffffu, v.lo, src)};
}

// Sum over the warp by butterfly; every lane ends with the same value (the double-float add is
// commutative bit for bit: TwoSum's error term is exact).
__device__ __forceinline__ df64 warp_sum_df(df64 v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = v + df64{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
  return v;
}

// a * b of two FP32 values, exactly, as a double-float
__device__ __forceinline__ df64 df_prod_ff(float a, float b) {
  float p, e;
  two_prod(a, b, p, e);
  return {p, e};
}

// The ACA stopping test of the FP64 path, sqrt(|u|^2 |v|^2 / err) <= eps, as uv <= eps^2 err
// without a square root or a division; with err = 0 (then uv = 0) the FP64 test sees 0 / 0 and
// does not stop, and neither does this one.
__device__ __forceinline__ bool aca_converged(df64 uv, df64 err, df64 eps2) {
  return !df_is_zero(err) && !(uv > eps2 * err);
}

// (value, index) argmax over the warp: larger value wins, smaller index on ties
__device__ __forceinline__ void warp_argmax_df(df64& val, int& idx) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const df64 ov{__shfl_xor_sync(0xffffffffu, val.hi, o), __shfl_xor_sync(0xffffffffu, val.lo, o)};
    const int oi = __shfl_xor_sync(0xffffffffu, idx, o);
    if (ov > val || (ov == val && oi < idx)) {
      val = ov;
      idx = oi;
    }
  }
}

// acc -= sum_{p < nst} coef[p] * pool[toff[p] + off], two loads in flight
__device__ __forceinline__ void sub_terms_df(cdf& acc, const cdf* coef, const cdf* __restrict__ pool,
                                             const long long* toff, long long off, int nst) {
  int p = 0;
  for (; p + 2 <= nst; p += 2) {
    const cdf a0 = pool[toff[p] + off], a1 = pool[toff[p + 1] + off];
    cdf_fms(acc, coef[p], a0);
    cdf_fms(acc, coef[p + 1], a1);
  }
  if (p < nst) cdf_fms(acc, coef[p], pool[toff[p] + off]);
}

// FP32 complex product of the leading parts: acc += a b
__device__ __forceinline__ void lead_fma(float& re, float& im, const cdf& a, const cdf& b) {
  re = fmaf(a.re.hi, b.re.hi, re);
  re = fmaf(-a.im.hi, b.im.hi, re);
  im = fmaf(a.re.hi, b.im.hi, im);
  im = fmaf(a.im.hi, b.re.hi, im);
}

// ------------------------------------------------------------------------------------------
// Warp per block (sides up to 32 LPL): lane l owns rows / columns l + 32 k, the current u and v
// stay in registers, earlier terms are read from the pool.
// ------------------------------------------------------------------------------------------
template <int LPL>
__global__ void __launch_bounds__(256, LPL == 8 ? 1 : 2) aca_df_warp_kernel(AcaDfArgs A, int nblocks) {
  __shared__ float4 s_tab[kDfTab];
  __shared__ __align__(16) unsigned char s_raw[8 * kWarpAcaTerms * (2 * sizeof(cdf) + sizeof(long long))];
  load_table(A.tab, s_tab);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int bi = blockIdx.x * 8 + warp;
  if (bi >= nblocks) return;
  cdf* uq = reinterpret_cast<cdf*>(s_raw) + warp * kWarpAcaTerms;
  cdf* vq = reinterpret_cast<cdf*>(s_raw) + (8 + warp) * kWarpAcaTerms;
  long long* toff = reinterpret_cast<long long*>(s_raw + 16 * kWarpAcaTerms * sizeof(cdf)) + warp * kWarpAcaTerms;
  const int b = A.order[bi];
  const int4 q = A.blocks[b];
  const int rs = q.x, cs = q.z, m = q.y - q.x, n = q.w - q.z;
  int iter_lim = min(A.maxk, min(m - 1, n - 1));
  if (iter_lim < 0) iter_lim = 0;
  if (iter_lim > kWarpAcaTerms) iter_lim = kWarpAcaTerms;  // the host routes only blocks that fit

  if (iter_lim > 0 &&
      zero_block(A, rs, m, cs, n, lane, 32, [](bool ok) { return __all_sync(0xffffffffu, ok) != 0; })) {
    if (lane == 0) {
      A.rank[b] = 0;
      if (A.passes) A.passes[b] = 0;
    }
    return;
  }

  unsigned used_l = lane == 0 ? 1u : 0u;  // bit k: row lane + 32 k is used (row 0 first)
  df64 err{0.0f, 0.0f};
  int i = 0, iter = 0, nst = 0, npass = 0;
  bool need_alloc = true;
  long long base = 0;
  cdf u_l[LPL], v_l[LPL];
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
    cdf* unew = A.pool + base;
    cdf* vnew = unew + m;
    for (int p = lane; p < nst; p += 32) uq[p] = A.pool[toff[p] + i];
    __syncwarp();
    // row residual and column pivot
    const DfPt* pi = A.pts + rs + i;
    df64 best{-1.0f, 0.0f};
    int bidx = 0;
#pragma unroll
    for (int kk = 0; kk < LPL; kk++) {
      const int c = lane + 32 * kk;
      if (c < n) {
        cdf v = entry_df_call(A.k, pi, A.el + cs + c, s_tab);
        sub_terms_df(v, uq, A.pool, toff, (long long)m + c, nst);
        v_l[kk] = v;
        const df64 a = cdf_abs2(v);
        if (a > best) {
          best = a;
          bidx = c;
        }
      }
    }
    warp_argmax_df(best, bidx);
    const int j = bidx;
    cdf mine = v_l[0];
#pragma unroll
    for (int kk = 1; kk < LPL; kk++)
      if (kk == (j >> 5)) mine = v_l[kk];
    const cdf vj{shfl_df(mine.re, j & 31), shfl_df(mine.im, j & 31)};
    for (int p = lane; p < nst; p += 32) vq[p] = A.pool[toff[p] + m + j];
    __syncwarp();
    const bool keep = df_is_zero(vj.re) && df_is_zero(vj.im);
    const CdfDivisor dv = keep ? CdfDivisor{cdf{}, 1.0f} : cdf_divisor(vj);
    df64 vn{0.0f, 0.0f};
#pragma unroll
    for (int kk = 0; kk < LPL; kk++) {
      const int c = lane + 32 * kk;
      if (c < n) {
        cdf v = v_l[kk];
        if (!keep) v = cdf_divide(v, dv);
        v_l[kk] = v;
        vnew[c] = v;
        vn += cdf_abs2(v);
      }
    }
    // column residual
    df64 un{0.0f, 0.0f};
#pragma unroll
    for (int kk = 0; kk < LPL; kk++) {
      const int r = lane + 32 * kk;
      if (r < m) {
        cdf u = entry_df_call(A.k, A.pts + rs + r, A.el + cs + j, s_tab);
        sub_terms_df(u, vq, A.pool, toff, (long long)r, nst);
        u_l[kk] = u;
        unew[r] = u;
        un += cdf_abs2(u);
      }
    }
    // cross terms sum_q |u^T U_q| |v V_q^T| (FP32 on the leading parts, exact products summed as
    // double-floats: all on the FP32 pipes)
    df64 dots{0.0f, 0.0f};
    for (int p = 0; p < nst; p++) {
      const cdf* Up = A.pool + toff[p];
      const cdf* Vp = Up + m;
      float udr = 0.f, udi = 0.f, vdr = 0.f, vdi = 0.f;
#pragma unroll
      for (int kk = 0; kk < LPL; kk++) {
        const int r = lane + 32 * kk;
        if (r < m) lead_fma(udr, udi, u_l[kk], Up[r]);
        if (r < n) lead_fma(vdr, vdi, v_l[kk], Vp[r]);
      }
      udr = warp_sum(udr);
      udi = warp_sum(udi);
      vdr = warp_sum(vdr);
      vdi = warp_sum(vdi);
      dots += df_prod_ff(sqrtf(udr * udr + udi * udi), sqrtf(vdr * vdr + vdi * vdi));
    }
    const df64 unt = warp_sum_df(un), vnt = warp_sum_df(vn);
    const df64 uv = unt * vnt;
    err += uv + df_ldexp(dots, 2.0f);
    if (aca_converged(uv, err, A.eps2)) break;
    const bool zero_term = df_is_zero(unt) || df_is_zero(vnt);
    // next row pivot over unused rows
    best = df64{-1.0f, 0.0f};
    bidx = 0;
#pragma unroll
    for (int kk = 0; kk < LPL; kk++) {
      const int r = lane + 32 * kk;
      if (r < m && !((used_l >> kk) & 1u)) {
        const df64 a = cdf_abs2(u_l[kk]);
        if (a > best) {
          best = a;
          bidx = r;
        }
      }
    }
    warp_argmax_df(best, bidx);
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

// ------------------------------------------------------------------------------------------
// One CTA per block (blocks with a side above 256).
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ void block_argmax_df(df64& val, int& idx, df64* sv, int* si) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  warp_argmax_df(val, idx);
  if (lane == 0) {
    sv[w] = val;
    si[w] = idx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    df64 bv = sv[0];
    int bi = si[0];
    for (int k = 1; k < kDfWarps; k++)
      if (sv[k] > bv || (sv[k] == bv && si[k] < bi)) {
        bv = sv[k];
        bi = si[k];
      }
    sv[0] = bv;
    si[0] = bi;
  }
  __syncthreads();
  val = sv[0];
  idx = si[0];
  __syncthreads();
}

// Sum over the CTA: warp sums, then the warps' sums in order by thread 0; every thread gets it.
__device__ __forceinline__ df64 block_sum_df(df64 v, df64* sd) {
  v = warp_sum_df(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sd[w] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    df64 s = sd[0];
    for (int k = 1; k < kDfWarps; k++) s += sd[k];
    sd[0] = s;
  }
  __syncthreads();
  v = sd[0];
  __syncthreads();
  return v;
}

__global__ void __launch_bounds__(kDfThreads) aca_df_kernel(AcaDfArgs A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ float4 s_tab[kDfTab];
  __shared__ df64 s_rv[kDfWarps];
  __shared__ int s_ri[kDfWarps];
  __shared__ df64 s_d[kDfWarps];
  __shared__ long long s_base;
  __shared__ int s_flag;
  load_table(A.tab, s_tab);

  const int b = A.order[blockIdx.x];
  const int4 q = A.blocks[b];
  const int rs = q.x, cs = q.z, m = q.y - q.x, n = q.w - q.z;
  int iter_lim = min(A.maxk, min(m - 1, n - 1));
  if (iter_lim < 0) iter_lim = 0;
  if (iter_lim > A.iter_cap) iter_lim = A.iter_cap;  // host guarantees iter_cap >= every iter_lim

  cdf* uq = reinterpret_cast<cdf*>(smem_raw);
  cdf* vq = uq + A.iter_cap;
  long long* toff = reinterpret_cast<long long*>(vq + A.iter_cap);
  unsigned* used = reinterpret_cast<unsigned*>(toff + A.iter_cap);
  const int tid = threadIdx.x, T = blockDim.x, lane = tid & 31, warp = tid >> 5;

  if (A.zero_guard && iter_lim > 0 &&
      zero_block(A, rs, m, cs, n, tid, T, [](bool ok) { return __syncthreads_and(ok) != 0; })) {
    if (tid == 0) {
      A.rank[b] = 0;
      if (A.passes) A.passes[b] = 0;
    }
    return;
  }

  for (int w = tid; w < (m + 31) / 32; w += T) used[w] = 0;
  __syncthreads();
  if (tid == 0) used[0] = 1u;
  df64 err{0.0f, 0.0f};  // meaningful in thread 0
  int i = 0, iter = 0, nst = 0, npass = 0;
  bool need_alloc = true;
  __syncthreads();

  while (iter < iter_lim) {
    if (need_alloc) {
      if (tid == 0) {
        const unsigned long long need = (unsigned long long)(m + n);
        const unsigned long long bb = atomicAdd(A.pool_used, need);
        s_flag = (bb + need > (unsigned long long)A.pool_cap) ? 1 : 0;
        s_base = (long long)bb;
        if (s_flag) atomicOr(A.status, 1);
      }
      __syncthreads();
      if (s_flag) break;
      need_alloc = false;
    }
    npass++;
    cdf* unew = A.pool + s_base;
    cdf* vnew = unew + m;
    for (int p = tid; p < nst; p += T) uq[p] = A.pool[toff[p] + i];
    __syncthreads();

    // row residual v = M(i, :) - U(i, :) V
    const DfPt* pi = A.pts + rs + i;
    df64 best{-1.0f, 0.0f};
    int bidx = 0;
    for (int c = tid; c < n; c += T) {
      cdf v = entry_df_call(A.k, pi, A.el + cs + c, s_tab);
      sub_terms_df(v, uq, A.pool, toff, (long long)m + c, nst);
      vnew[c] = v;
      const df64 a = cdf_abs2(v);
      if (a > best) {
        best = a;
        bidx = c;
      }
    }
    block_argmax_df(best, bidx, s_rv, s_ri);
    const int j = bidx;
    const cdf vj = vnew[j];
    for (int p = tid; p < nst; p += T) vq[p] = A.pool[toff[p] + m + j];
    __syncthreads();
    const bool keep = A.zero_guard && df_is_zero(vj.re) && df_is_zero(vj.im);
    const CdfDivisor dv = keep ? CdfDivisor{cdf{}, 1.0f} : cdf_divisor(vj);
    df64 vn{0.0f, 0.0f};
    for (int c = tid; c < n; c += T) {
      cdf v = vnew[c];
      if (!keep) v = cdf_divide(v, dv);
      vnew[c] = v;
      vn += cdf_abs2(v);
    }

    // column residual u = M(:, j) - U V(:, j)
    df64 un{0.0f, 0.0f};
    for (int r = tid; r < m; r += T) {
      cdf u = entry_df_call(A.k, A.pts + rs + r, A.el + cs + j, s_tab);
      sub_terms_df(u, vq, A.pool, toff, (long long)r, nst);
      unew[r] = u;
      un += cdf_abs2(u);
    }
    __syncthreads();

    // cross terms (one warp per earlier stored term, FP32 on the leading parts, exact products
    // summed as double-floats)
    df64 dots{0.0f, 0.0f};
    for (int p = warp; p < nst; p += kDfWarps) {
      const cdf* Up = A.pool + toff[p];
      const cdf* Vp = Up + m;
      float udr = 0.f, udi = 0.f, vdr = 0.f, vdi = 0.f;
      for (int r = lane; r < m; r += 32) lead_fma(udr, udi, unew[r], Up[r]);
      for (int c = lane; c < n; c += 32) lead_fma(vdr, vdi, vnew[c], Vp[c]);
      udr = warp_sum(udr);
      udi = warp_sum(udi);
      vdr = warp_sum(vdr);
      vdi = warp_sum(vdi);
      if (lane == 0) dots += df_prod_ff(sqrtf(udr * udr + udi * udi), sqrtf(vdr * vdr + vdi * vdi));
    }
    const df64 unt = block_sum_df(un, s_d);
    const df64 vnt = block_sum_df(vn, s_d);
    dots = block_sum_df(lane == 0 ? dots : df64{0.0f, 0.0f}, s_d);
    if (tid == 0) {
      const df64 uv = unt * vnt;
      err += uv + df_ldexp(dots, 2.0f);
      s_flag = aca_converged(uv, err, A.eps2) ? 1 : 0;
    }
    __syncthreads();
    if (s_flag) break;
    const bool zero_term = df_is_zero(unt) || df_is_zero(vnt);

    // next row pivot: first max |u|^2 over unused rows
    best = df64{-1.0f, 0.0f};
    bidx = 0;
    for (int r = tid; r < m; r += T) {
      if ((used[r >> 5] >> (r & 31)) & 1u) continue;
      const df64 a = cdf_abs2(unew[r]);
      if (a > best) {
        best = a;
        bidx = r;
      }
    }
    block_argmax_df(best, bidx, s_rv, s_ri);
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
// Near field: one CTA per block, one thread per entry, rounded to complex FP32.
// ------------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) near_df_kernel(const DfPt* __restrict__ pts, const DfElem* __restrict__ el,
                                                      const float4* __restrict__ tab, const int4* __restrict__ blocks,
                                                      const long long* __restrict__ near_off, df64 k, cf* out) {
  __shared__ float4 s_tab[kDfTab];
  load_table(tab, s_tab);
  const int b = blockIdx.x;
  const int4 q = blocks[b];
  const int m = q.y - q.x, n = q.w - q.z;
  cf* dst = out + near_off[b];
  const int mn = m * n;
  for (int t = threadIdx.x; t < mn; t += blockDim.x) {
    const int c = t / m, r = t - c * m;
    const cdf v = entry_df(k, pts + q.x + r, el + q.z + c, s_tab);
    dst[t] = cf(v.re.hi, v.im.hi);
  }
}

void launch_near_assembly_df(const DevGeometry& G, const DevPartition& DP, DevHMat& H, cudaStream_t s) {
  if (DP.nd == 0) return;
  note_launch();
  near_df_kernel<<<DP.nd, 256, 0, s>>>(G.cen_df.as<DfPt>(), G.el_df.as<DfElem>(), G.df_tab.as<float4>(),
                                       DP.blocks_d.as<int4>(), DP.near_off.as<long long>(), df_from_double(H.k),
                                       H.near.as<cf>());
  AC3D_CUDA(cudaGetLastError());
}

template <int LPL>
static void aca_df_launch_warp(const AcaDfArgs& a, int nblocks, cudaStream_t s) {
  if (nblocks <= 0) return;
  note_launch();
  aca_df_warp_kernel<LPL><<<(nblocks + 7) / 8, 256, 0, s>>>(a, nblocks);
  AC3D_CUDA(cudaGetLastError());
}

void launch_aca_df(const DevGeometry& G, const DevPartition& DP, DevHMat& H, double eps, int max_rows, cudaStream_t s,
                   cudaStream_t s_small) {
  if (DP.na == 0) return;
  AcaDfArgs a{G.cen.as<double4>(), G.va.as<double4>(), G.eg64.as<ElemGeo<double>>(), G.cen_df.as<DfPt>(),
              G.el_df.as<DfElem>(), G.df_tab.as<float4>(), DP.blocks_a.as<int4>(), DP.aca_order.as<int>(),
              df_from_double(H.k), eps, df_from_double(eps * eps), H.maxk, H.maxk, H.pool.as<cdf>(), H.pool_cap,
              H.pool_used.as<unsigned long long>(), H.term_off.as<long long>(), H.rank.as<int>(),
              (int*)(H.pool_used.as<unsigned long long>() + 1), H.passes.as<int>(), 1};
  // same grouping and stream split as launch_aca: CTA blocks, then warp blocks up to 256 / 128 / 64
  const int* order = DP.aca_order.as<int>();
  const int o1 = DP.aca_split[0], o2 = o1 + DP.aca_split[1], o3 = o2 + DP.aca_split[2];
  if (DP.aca_split[0] > 0) {
    const size_t smem = (size_t)a.iter_cap * (2 * sizeof(cdf) + sizeof(long long)) + (size_t)((max_rows + 31) / 32) * 4;
    if (smem > 48 * 1024) {
      if (smem > 200 * 1024) throw Error(4, "ACA block too large for shared memory");
      AC3D_CUDA(cudaFuncSetAttribute(aca_df_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    }
    note_launch();
    aca_df_kernel<<<DP.aca_split[0], kDfThreads, smem, s>>>(a);
    AC3D_CUDA(cudaGetLastError());
  }
  a.order = order + o1;
  aca_df_launch_warp<8>(a, DP.aca_split[1], s_small);
  a.order = order + o2;
  aca_df_launch_warp<4>(a, DP.aca_split[2], s);
  a.order = order + o3;
  aca_df_launch_warp<2>(a, DP.aca_split[3], s_small);
}

// Receiver ACA (compute_ACA_listener, aca.cpp:84-134: one block of L receivers x Ne elements, no
// zero guard) in double-float, then the terms converted in place to complex FP64 (same size).
__global__ void cdf_to_cd_kernel(cdf* pool, const unsigned long long* used) {
  const unsigned long long n = *used;
  for (unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x) {
    const cdf v = pool[i];
    reinterpret_cast<cd*>(pool)[i] = cd(df_to_double(v.re), df_to_double(v.im));
  }
}

void launch_listener_aca_df(const DevGeometry& G, const void* pts_df, int L, double k, double eps, int maxk,
                            void* pool, long long pool_cap, unsigned long long* used, long long* term_off, int* rank,
                            int* status, const int4* block, const int* order, cudaStream_t s) {
  int iter_lim = std::min(maxk, std::min(L - 1, G.ne - 1));
  if (iter_lim < 1) iter_lim = 1;
  AcaDfArgs a{G.cen.as<double4>(), G.va.as<double4>(), G.eg64.as<ElemGeo<double>>(), (const DfPt*)pts_df,
              G.el_df.as<DfElem>(), G.df_tab.as<float4>(), block, order, df_from_double(k), eps,
              df_from_double(eps * eps), maxk, iter_lim,
              (cdf*)pool, pool_cap, used, term_off, rank, status, nullptr, 0};
  const size_t smem = (size_t)iter_lim * (2 * sizeof(cdf) + sizeof(long long)) + (size_t)((L + 31) / 32) * 4;
  if (smem > 200 * 1024) throw Error(4, "receiver ACA too large for shared memory (at most about 5000 receivers)");
  if (smem > 48 * 1024)
    AC3D_CUDA(cudaFuncSetAttribute(aca_df_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  note_launch();
  aca_df_kernel<<<1, kDfThreads, smem, s>>>(a);
  AC3D_CUDA(cudaGetLastError());
  note_launch();
  cdf_to_cd_kernel<<<4 * device_sm_count(), 256, 0, s>>>((cdf*)pool, used);
  AC3D_CUDA(cudaGetLastError());
}

}  // namespace ac3d
