// H-matrix matvec y = op(K - I/2) x (generic_product_impl::scaleAndAddTo, hmatrix.h:84-139),
// op = identity or the plain (non-conjugate) transpose.
//
// The matrix is held as per-leaf segments (R x K column-major, R = leaf size):
//   near segment of a row leaf   : its dense blocks side by side, columns indexing x;
//   U segment of a row leaf      : rows of the leaf of every admissible block above it, one column
//                                  per rank-1 term;
//   V segment of a column leaf   : columns of the leaf of every admissible block beside it.
// Forward:    p = per-column dots of the V segments with x   (dot pass, one CTA per leaf)
//             t[b, q] = sum over the column leaves of b of p (reduce, fixed leaf order)
//             y = -x/2 + near x + U t                         (gather pass, one CTA per leaf)
// Transpose:  the same with U and V swapped, plus the dense blocks read column-wise.
// Both passes stream their segments through shared memory with bulk async copies, so the bytes
// in flight are set by the copy ring, not by how many loads a warp can issue. No atomics; every
// sum has a fixed order, so results are bit-reproducible.
#include <algorithm>
#include <atomic>
#include <mutex>
#include <type_traits>

#include "common.cuh"
#include "internal.h"
#include "launch.cuh"
#include "segstream.cuh"

namespace ac3d {

namespace {
constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
}  // namespace

// Double-float: the unevaluated sum hi + lo of two FP32 numbers, about 48 significant bits, used
// for the FP64-vector residual of iterative refinement so that it runs on the FP32 pipes (GB300's
// FP64 rate is a small fraction of its FP32 rate). Error-free transformations: two_sum (Knuth),
// two_prod by FMA (the double-double arithmetic of Dekker 1971, Hida-Li-Bailey 2001). The _rn
// intrinsics keep the compiler from contracting the exact splits into FMAs.
struct df32 {
  float hi, lo;
  __host__ __device__ df32(float h = 0.f, float l = 0.f) : hi(h), lo(l) {}
};

__device__ __forceinline__ df32 df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return df32(s, e);
}
__device__ __forceinline__ df32 df_fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return df32(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ df32 df_add(df32 x, df32 y) {
  const df32 s = df_two_sum(x.hi, y.hi);
  return df_fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo)));
}
// acc + a z for a float a: the product's rounding error and a z.lo go to the low word, which is
// renormalised when accumulators are combined (df_add).
__device__ __forceinline__ void df_mac(df32& acc, float a, df32 z) {
  const float p = __fmul_rn(a, z.hi);
  const float pe = __fmaf_rn(a, z.lo, __fmaf_rn(a, z.hi, -p));
  const df32 s = df_two_sum(acc.hi, p);
  acc = df32(s.hi, __fadd_rn(acc.lo, __fadd_rn(s.lo, pe)));
}

// Accumulator arithmetic of the matvec passes: plain FP32 / FP64, or double-float.
template <typename AT, typename MT>
__device__ __forceinline__ void acc_mac(AT& ar, AT& ai, const cplx<MT>& a, const AT& zr, const AT& zi) {
  ar = fma((AT)a.re, zr, ar);
  ar = fma(-(AT)a.im, zi, ar);
  ai = fma((AT)a.re, zi, ai);
  ai = fma((AT)a.im, zr, ai);
}
__device__ __forceinline__ void acc_mac(df32& ar, df32& ai, const cplx<float>& a, const df32& zr, const df32& zi) {
  df_mac(ar, a.re, zr);
  df_mac(ar, -a.im, zi);
  df_mac(ai, a.re, zi);
  df_mac(ai, a.im, zr);
}
template <typename AT>
__device__ __forceinline__ AT acc_add(AT a, AT b) { return a + b; }
__device__ __forceinline__ df32 acc_add(df32 a, df32 b) { return df_add(a, b); }
template <typename AT>
__device__ __forceinline__ AT acc_shfl_xor(AT v, int o) { return __shfl_xor_sync(0xffffffffu, v, o); }
__device__ __forceinline__ df32 acc_shfl_xor(df32 v, int o) {
  return df32(__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o));
}
template <typename VT, typename AT>
__device__ __forceinline__ VT acc_to(AT v) { return (VT)v; }
template <>
__device__ __forceinline__ double acc_to<double, df32>(df32 v) { return (double)v.hi + (double)v.lo; }

// x (FP64) -> double-float multipliers
__global__ void to_df_kernel(int n, const cd* __restrict__ x, cplx<df32>* out) {
  grid_dep_wait();
  grid_dep_launch();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const cd v = x[i];
  const float rh = __double2float_rn(v.re), ih = __double2float_rn(v.im);
  out[i] = cplx<df32>(df32(rh, __double2float_rn(v.re - (double)rh)), df32(ih, __double2float_rn(v.im - (double)ih)));
}

// Lanes per column and rows per lane of the dot pass for leaves of up to 32 RPL rows: a group of G
// lanes shares one column, lane g summing rows g, g + G, g + 2G, ..., so one warp instruction
// covers 32 / G columns and the cross-lane sum takes log2(G) shuffle levels.
template <int RPL>
struct DotShape {
  static constexpr int G = RPL <= 2 ? 8 : RPL == 4 ? 16 : 32;
  static constexpr int RPG = 32 * RPL / G;
};

// Dot pass: p[kptr[leaf] + k] = sum_rows S[k][row] x[leaf rows] for every column k of the leaf's
// low-rank segment (region B).
template <typename MT, typename AT, int RPL>
__global__ void __launch_bounds__(kThreads, 4) seg_dot_kernel(SegView V, const cplx<MT>* __restrict__ lrseg,
                                                           const cplx<AT>* __restrict__ xm, cplx<AT>* __restrict__ p,
                                                           const int* __restrict__ done) {
  constexpr int G = DotShape<RPL>::G, RPG = DotShape<RPL>::RPG;
  constexpr int CPW = 32 / G;             // columns per warp step
  constexpr int STEP = kWarps * CPW;      // columns per CTA step
  extern __shared__ __align__(128) unsigned char dsmem[];
  auto stage = reinterpret_cast<unsigned char(*)[kStageBytes]>(dsmem);
  __shared__ __align__(8) uint64_t full[kStages];
  // the segments and the partition are not written by any kernel of a solve: the first stages
  // stream in before the wait for the preceding kernel (which writes x and the done flag)
  const int leaf = V.order[blockIdx.x];
  const int ls = V.leaf_start[leaf], R = V.leaf_start[leaf + 1] - ls;
  const int k0 = V.b_kptr[leaf], K = V.b_kptr[leaf + 1] - k0;
  // a set done flag stays set for the rest of the solve, so reading it before the wait can only
  // miss a flag that is being set (checked again after the wait)
  if (K == 0 || (done && *(volatile const int*)done)) {
    grid_dep_wait();
    grid_dep_launch();
    return;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane % G, slot = lane / G;
  AT xr[RPG], xi[RPG];
  init_ring(full);
  cplx<AT>* out = p + k0;
  auto after_prefetch = [&]() -> bool {
    grid_dep_wait();
    grid_dep_launch();
    if (done && *done) return false;
#pragma unroll
    for (int t = 0; t < RPG; t++) {
      const int row = g + G * t;
      const cplx<AT> v = row < R ? xm[ls + row] : cplx<AT>();
      xr[t] = v.re;
      xi[t] = v.im;
    }
    return true;
  };
  stream_leaf<MT>(stage, full, R, nullptr, 0, lrseg + V.b_seg[leaf], K, V.err, after_prefetch,
                  [&](const cplx<MT>* S, int, int c0, int ncols, int, int, int) {
                    // two columns per lane in flight: j and j + STEP
                    for (int jb = warp * CPW; jb < ncols; jb += 2 * STEP) {
                      AT a[4];
#pragma unroll
                      for (int u = 0; u < 2; u++) {
                        const int j = jb + slot + u * STEP;
                        AT ar = 0, ai = 0;
                        if (j < ncols) {
                          const cplx<MT>* col = S + j * R;
#pragma unroll
                          for (int t = 0; t < RPG; t++) {
                            const int row = g + G * t;
                            if (row < R) acc_mac(ar, ai, col[row], xr[t], xi[t]);
                          }
                        }
                        a[2 * u] = ar;
                        a[2 * u + 1] = ai;
                      }
#pragma unroll
                      for (int o = G / 2; o > 0; o >>= 1)
#pragma unroll
                        for (int u = 0; u < 4; u++) a[u] = acc_add(a[u], acc_shfl_xor(a[u], o));
                      if (g == 0) {
                        const int j = jb + slot;
                        if (j < ncols) out[c0 + j] = cplx<AT>(a[0], a[1]);
                        if (j + STEP < ncols) out[c0 + j + STEP] = cplx<AT>(a[2], a[3]);
                      }
                    }
                  });
}

// t[task] = sum over the leaf entries of the task's block of p[kpos[e] + q], in leaf order
// (kpos is stored block-major, so a block's entries are consecutive).
template <typename AT>
__global__ void __launch_bounds__(256) seg_reduce_kernel(const int* __restrict__ task_b,
                                                         const int* __restrict__ t_off, int ntask_cap,
                                                         const int* __restrict__ t_total,
                                                         const int* __restrict__ ent_ptr,
                                                         const int* __restrict__ kpos,
                                                         const cplx<AT>* __restrict__ p, cplx<AT>* __restrict__ t,
                                                         const int* __restrict__ done) {
  grid_dep_wait();
  grid_dep_launch();
  if (done && *done) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ntask_cap || i >= *t_total) return;
  const int b = task_b[i];
  const int q = i - t_off[b];
  const int e0 = ent_ptr[b], e1 = ent_ptr[b + 1];
  AT sr = 0, si = 0;
  int e = e0;
  // batches of 16: every load of a batch is issued before its first add (a block spans up to a
  // few hundred leaves); the adds keep the entry order, so any batching gives the same sums
  for (; e + 15 < e1; e += 16) {
    int kk[16];
#pragma unroll
    for (int u = 0; u < 16; u++) kk[u] = kpos[e + u];
    cplx<AT> v[16];
#pragma unroll
    for (int u = 0; u < 16; u++) v[u] = p[kk[u] + q];
#pragma unroll
    for (int u = 0; u < 16; u++) {
      sr = acc_add(sr, v[u].re);
      si = acc_add(si, v[u].im);
    }
  }
  for (; e + 3 < e1; e += 4) {
    const int k0 = kpos[e], k1 = kpos[e + 1], k2 = kpos[e + 2], k3 = kpos[e + 3];
    const cplx<AT> v0 = p[k0 + q], v1 = p[k1 + q], v2 = p[k2 + q], v3 = p[k3 + q];
    sr = acc_add(sr, v0.re);
    si = acc_add(si, v0.im);
    sr = acc_add(sr, v1.re);
    si = acc_add(si, v1.im);
    sr = acc_add(sr, v2.re);
    si = acc_add(si, v2.im);
    sr = acc_add(sr, v3.re);
    si = acc_add(si, v3.im);
  }
  for (; e < e1; e++) {
    const cplx<AT> v = p[kpos[e] + q];
    sr = acc_add(sr, v.re);
    si = acc_add(si, v.im);
  }
  t[i] = cplx<AT>(sr, si);
}

// Gather pass: y[leaf rows] = -x/2 + S_A x[a_idx] + S_B t[b_idx] (+ transposed dense blocks), or
// b - that; optional fused FP64 dot partials (conj(a).y, conj(y).b, |y|^2) per leaf.
//
// Warp-specialised: kWarps consumer warps compute, one producer warp feeds the copy ring. For
// each chunk (at most kPCols columns) the producer waits until the consumers have released the
// stage (its "empty" mbarrier, one arrival per consumer warp), issues the chunk's bulk copy, then
// gathers its column multipliers (x[idx] or t[idx]) into the stage's multiplier buffer with
// cp.async; the stage's "full" mbarrier expects the copy's bytes and one arrival per producer
// lane. A padding column (index -1) is zero in the segment, so it gathers any valid multiplier
// (element 0). The compute uses the dot pass's layout: G lanes per column, each lane summing RPG
// rows, 32 / G columns per warp step.
constexpr int kGatherThreads = kThreads + 32;
#ifndef AC3D_GATHER_MIN_CTAS
#define AC3D_GATHER_MIN_CTAS 4
#endif

// The grid is persistent: the CTAs that fit on the device at once (P) take the row leaves in the
// order V.order (decreasing work), CTA k the leaves k, 2P - 1 - k, 2P + k, ... (a serpentine over
// the sorted list). The producer goes on to the next leaf's chunks as soon as it has issued the
// current leaf's last one (it loads the next leaf's geometry while it streams the current one),
// so an SM slot never waits for an empty ring between leaves. Every stage carries its leaf slot,
// column count and first / last flags; the consumer warps finish a leaf (row sums, epilogue, dot
// partials) when they consume its last chunk, synchronising among themselves on an mbarrier
// while the producer keeps streaming. A leaf's row sums have a fixed order (each warp's columns
// in chunk order, then the warps in order), and the last CTA to finish reduces the per-leaf dot
// partials in fixed order, so results are reproducible. Against one CTA per leaf this takes 104
// instead of 101 us for back-to-back matvecs without overlap, but 6.7% less time per BiCGSTAB
// iteration inside the solve and 3% more served solves/s over the relief sweep.
constexpr int kPCols = 128;                  // multiplier columns per stage (chunks are capped at it)
constexpr int kPProdCols = kPCols / 32;      // per producer lane
constexpr int kLeafSlots = kStages + 1;      // leaves whose chunks can be in the ring at once

struct StageMeta {
  int slot, ncols, first, last;  // slot < 0: no more leaves
};

// Barrier of the consumer warps only (the producer keeps streaming): every consumer thread arrives
// on an mbarrier (release) and waits for the phase (acquire), with the bounded wait, so a failed
// pipeline cannot leave threads blocked. Returns false if the phase did not complete.
__device__ __forceinline__ bool consumer_sync(uint64_t* bar, uint32_t& phase) {
  mbar_arrive(bar);
  const bool ok = mbar_wait_bounded(bar, phase);
  phase ^= 1u;
  return ok;
}

template <typename MT, typename VT, typename AT, bool TRANS, int RPL>
__global__ void __launch_bounds__(kGatherThreads, AC3D_GATHER_MIN_CTAS) seg_gather_persist_kernel(
    SegView V, int nleaf, const cplx<MT>* __restrict__ near, const cplx<MT>* __restrict__ lrseg,
    const cplx<AT>* __restrict__ t, const cplx<VT>* __restrict__ x, const cplx<AT>* __restrict__ xm,
    cplx<VT>* __restrict__ y, const cplx<VT>* __restrict__ bminus, const cplx<VT>* __restrict__ dot_a,
    const cplx<VT>* __restrict__ dot_b, double* partials, double* red5, unsigned* ticket,
    const int* __restrict__ done) {
  constexpr int G = DotShape<RPL>::G, RPG = DotShape<RPL>::RPG;
  constexpr int CPW = 32 / G;
  constexpr int STEP = kWarps * CPW;
  constexpr int RMAX = 32 * RPL;
  extern __shared__ __align__(128) unsigned char dsmem[];
  auto stage = reinterpret_cast<unsigned char(*)[kStageBytes]>(dsmem);
  __shared__ __align__(8) uint64_t full[kStages];
  __shared__ __align__(8) uint64_t empty[kStages];
  __shared__ __align__(8) uint64_t cbar;  // consumer barrier, kThreads arrivals per phase
  __shared__ __align__(16) unsigned char zraw[kStages * kPCols * sizeof(cplx<AT>)];
  auto zbuf = reinterpret_cast<cplx<AT>(*)[kPCols]>(zraw);
  __shared__ __align__(16) unsigned char praw[kWarps * RMAX * sizeof(cplx<AT>)];
  cplx<AT>* part = reinterpret_cast<cplx<AT>*>(praw);
  __shared__ StageMeta meta[kStages];
  __shared__ int slot_leaf[kLeafSlots], slot_ls[kLeafSlots], slot_R[kLeafSlots];
  __shared__ double sdot[kWarps][5];
  __shared__ int s_fail;
  __shared__ bool s_last;
  grid_dep_launch();  // as in the one-CTA-per-leaf pass
  if (done && *done) {
    grid_dep_wait();
    return;
  }
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int P = gridDim.x, kc = blockIdx.x;
  // geometry of the n-th leaf of this CTA in the serpentine (leaf -1: none left)
  struct LeafGeo {
    int leaf, ls, R, a_cols, b_cols, a_k, b_k;
    long long a_seg, b_seg;
  };
  auto leaf_geo = [&](int n) -> LeafGeo {
    LeafGeo o{-1, 0, 0, 0, 0, 0, 0, 0, 0};
    const long long li = (long long)n * P + ((n & 1) ? P - 1 - kc : kc);
    if (li >= nleaf) return o;
    o.leaf = V.order[li];
    o.ls = V.leaf_start[o.leaf];
    o.R = V.leaf_start[o.leaf + 1] - o.ls;
    if (!TRANS) {
      o.a_k = V.a_kptr[o.leaf];
      o.a_cols = V.a_kptr[o.leaf + 1] - o.a_k;
      o.a_seg = V.a_seg[o.leaf];
    }
    o.b_k = V.b_kptr[o.leaf];
    o.b_cols = V.b_kptr[o.leaf + 1] - o.b_k;
    o.b_seg = V.b_seg[o.leaf];
    return o;
  };
  if (tid == 0) {
    for (int st = 0; st < kStages; st++) {
      mbar_init(&full[st], 1 + 32);
      mbar_init(&empty[st], kWarps);
    }
    mbar_init(&cbar, kThreads);
    s_fail = 0;
    fence_barrier_init();
  }
  __syncthreads();

  if (warp == kWarps) {
    // ---- producer warp: every leaf's chunks in order, with no gap between leaves
    bool waited = false, failed = false;
    long long seq = 0;  // stage sequence number
    LeafGeo nxt = leaf_geo(0);
    for (int n = 0; !failed; n++) {
      const LeafGeo cur = nxt;
      if (cur.leaf >= 0) nxt = leaf_geo(n + 1);  // in flight while this leaf streams
      const int leaf = cur.leaf, ls = cur.ls, R = cur.R, a_cols = cur.a_cols, b_cols = cur.b_cols;
      const int cpc = leaf >= 0 ? min(kPCols, max(2, (int)(kStageBytes / sizeof(cplx<MT>)) / R & ~1)) : 2;
      const int na = (a_cols + cpc - 1) / cpc, nb = (b_cols + cpc - 1) / cpc;
      const int nch = leaf >= 0 ? max(na + nb, 1) : 1;  // a leaf with no columns still gets one stage
      if (lane == 0 && leaf >= 0) {
        slot_leaf[n % kLeafSlots] = leaf;
        slot_ls[n % kLeafSlots] = ls;
        slot_R[n % kLeafSlots] = R;
      }
      for (int c = 0; c < nch; c++, seq++) {
        const int s = (int)(seq % kStages);
        if (seq >= kStages) {
          const bool got =
              __all_sync(0xffffffffu, mbar_wait_bounded(&empty[s], (uint32_t)(seq / kStages - 1) & 1u));
          if (!got) {
            if (lane == 0) atomicExch(&s_fail, 1);
            failed = true;
            break;
          }
        }
        // chunk geometry
        int ncols = 0;
        const cplx<MT>* src = nullptr;
        const int* idx = nullptr;
        const cplx<AT>* z = nullptr;
        if (leaf >= 0 && c < na) {
          const int c0 = c * cpc;
          ncols = min(cpc, a_cols - c0);
          src = near + cur.a_seg + (long long)c0 * R;
          idx = V.a_idx + cur.a_k + c0;
          z = xm;
        } else if (leaf >= 0 && c < na + nb) {
          const int c0 = (c - na) * cpc;
          ncols = min(cpc, b_cols - c0);
          src = lrseg + cur.b_seg + (long long)c0 * R;
          idx = V.b_idx + cur.b_k + c0;
          z = t;
        }
        if (lane == 0) {
          meta[s] = StageMeta{leaf >= 0 ? n % kLeafSlots : -1, ncols, c == 0, c == nch - 1};
          const uint32_t bytes = (uint32_t)(ncols * R * sizeof(cplx<MT>));
          fence_proxy_async();
          mbar_expect_tx(&full[s], bytes);  // zero bytes: a plain arrival
          if (bytes) bulk_copy_g2s(stage[s], src, bytes, &full[s]);
        }
        if (ncols > 0 && c >= na && !waited) {  // t comes from the preceding kernel
          grid_dep_wait();
          waited = true;
        }
#pragma unroll
        for (int u = 0; u < kPProdCols; u++) {
          const int col = lane + 32 * u;
          if (col < ncols) cp_async_elem<sizeof(cplx<AT>)>(&zbuf[s][col], z + max(idx[col], 0));
        }
        cp_async_arrive_noinc(&full[s]);
      }
      if (leaf < 0) break;  // the end marker went out
    }
    if (!waited) grid_dep_wait();
    cp_async_wait_all();
    if (lane == 0)
      for (long long cc = max(0LL, seq - kStages); cc < seq; cc++)
        mbar_wait_bounded(&full[cc % kStages], (uint32_t)(cc / kStages) & 1u);
  } else {
    // ---- consumer warps
    const int g = lane % G, slot = lane / G;
    AT ar[RPG], ai[RPG];
#pragma unroll
    for (int q = 0; q < RPG; q++) ar[q] = ai[q] = 0;
    int leaf = -1, ls = 0, R = 0;
    uint32_t cphase = 0;
    bool cok = true;
    for (long long seq = 0;; seq++) {
      const int s = (int)(seq % kStages);
      const bool got = __all_sync(0xffffffffu, mbar_wait_bounded(&full[s], (uint32_t)(seq / kStages) & 1u));
      if (!got) {
        if (lane == 0) atomicExch(&s_fail, 1);
        break;
      }
      const StageMeta mt = meta[s];
      if (mt.slot < 0) {
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]);
        break;
      }
      if (mt.first) {
        leaf = slot_leaf[mt.slot];
        ls = slot_ls[mt.slot];
        R = slot_R[mt.slot];
      }
      const int ncols = mt.ncols;
      const cplx<MT>* S = (const cplx<MT>*)stage[s];
      const cplx<AT>* Z = zbuf[s];
      for (int jb = warp * CPW; jb < ncols; jb += 2 * STEP) {
#pragma unroll
        for (int u = 0; u < 2; u++) {
          const int j = jb + slot + u * STEP;
          if (j < ncols) {
            const cplx<AT> zz = Z[j];
            const cplx<MT>* col = S + j * R;
#pragma unroll
            for (int q = 0; q < RPG; q++) {
              const int row = g + G * q;
              if (row < R) acc_mac(ar[q], ai[q], col[row], zz.re, zz.im);
            }
          }
        }
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[s]);
      if (!mt.last) continue;
      // ---- the leaf is complete: its row sums and epilogue
#pragma unroll
      for (int o = G; o < 32; o <<= 1)
#pragma unroll
        for (int q = 0; q < RPG; q++) {
          ar[q] = acc_add(ar[q], acc_shfl_xor(ar[q], o));
          ai[q] = acc_add(ai[q], acc_shfl_xor(ai[q], o));
        }
      if (slot == 0) {
#pragma unroll
        for (int q = 0; q < RPG; q++) {
          const int row = g + G * q;
          if (row < R) part[warp * R + row] = cplx<AT>(ar[q], ai[q]);
        }
      }
#pragma unroll
      for (int q = 0; q < RPG; q++) ar[q] = ai[q] = 0;
      __syncwarp();
      if (TRANS) {
        AT tr[RPL], ti[RPL];
#pragma unroll
        for (int jr = 0; jr < RPL; jr++) tr[jr] = ti[jr] = 0;
        for (int it = V.trn_ptr[leaf] + warp; it < V.trn_ptr[leaf + 1]; it += kWarps) {
          const int b = V.trn[it];
          const int4 blk = V.blocks_d[b];
          const int m = blk.y - blk.x;
          const cplx<AT>* xs = xm + blk.x;
#pragma unroll
          for (int jr = 0; jr < RPL; jr++) {
            const int col = lane + 32 * jr;
            if (col < R) {
              const cplx<MT>* Dc = near + V.near_off[b] + (long long)col * m;
              for (int r = 0; r < m; r++) {
                const cplx<AT> zz = xs[r];
                acc_mac(tr[jr], ti[jr], Dc[r], zz.re, zz.im);
              }
            }
          }
        }
#pragma unroll
        for (int jr = 0; jr < RPL; jr++) {
          const int col = lane + 32 * jr;
          if (col < R) {
            cplx<AT>& pc = part[warp * R + col];
            pc = cplx<AT>(acc_add(pc.re, tr[jr]), acc_add(pc.im, ti[jr]));
          }
        }
      }
      if (!(cok = consumer_sync(&cbar, cphase))) break;
      double d[5] = {0, 0, 0, 0, 0};
      if (tid < R) {
        const int r = tid;
        AT sr = 0, si = 0;
        for (int w = 0; w < kWarps; w++) {
          sr = acc_add(sr, part[w * R + r].re);
          si = acc_add(si, part[w * R + r].im);
        }
        const cplx<VT> xv = x[ls + r];
        VT yr = acc_to<VT>(sr) - VT(0.5) * xv.re;
        VT yi = acc_to<VT>(si) - VT(0.5) * xv.im;
        if (bminus) {
          const cplx<VT> bv = bminus[ls + r];
          yr = bv.re - yr;
          yi = bv.im - yi;
        }
        const cplx<VT> o(yr, yi);
        y[ls + r] = o;
        const double oyr = (double)o.re, oyi = (double)o.im;
        if (dot_a) {
          const cplx<VT> a = dot_a[ls + r];
          d[0] += (double)a.re * oyr + (double)a.im * oyi;
          d[1] += (double)a.re * oyi - (double)a.im * oyr;
        }
        if (dot_b) {
          const cplx<VT> bb = dot_b[ls + r];
          d[2] += oyr * (double)bb.re + oyi * (double)bb.im;
          d[3] += oyr * (double)bb.im - oyi * (double)bb.re;
        }
        d[4] += oyr * oyr + oyi * oyi;
      }
      if (partials) {
        for (int i = 0; i < 5; i++) d[i] = warp_sum(d[i]);
        if (lane == 0)
          for (int i = 0; i < 5; i++) sdot[warp][i] = d[i];
        if (!(cok = consumer_sync(&cbar, cphase))) break;
        if (tid < 5) {
          double sum = 0;
          for (int w = 0; w < kWarps; w++) sum += sdot[w][tid];
          partials[(size_t)leaf * 5 + tid] = sum;
        }
      }
      if (!(cok = consumer_sync(&cbar, cphase))) break;  // part and sdot are free for the next leaf
    }
    if (!cok && lane == 0) atomicExch(&s_fail, 1);
  }
  __syncthreads();
  if (s_fail && tid == 0) atomicExch(V.err, 1);
  if (partials && red5) {
    // the last CTA to finish reduces all leaves' partials in fixed order into red5
    __threadfence();
    __syncthreads();
    if (tid == 0) s_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    __syncthreads();
    if (s_last) {
      __threadfence();
      const bool consumer = warp < kWarps;
      double acc[5] = {0, 0, 0, 0, 0};
      if (consumer)
        for (int l = tid; l < nleaf; l += kThreads)
          for (int i = 0; i < 5; i++) acc[i] += __ldcg(&partials[(size_t)l * 5 + i]);
      for (int i = 0; i < 5; i++) acc[i] = warp_sum(acc[i]);
      __syncthreads();
      if (lane == 0 && consumer)
        for (int i = 0; i < 5; i++) sdot[warp][i] = acc[i];
      __syncthreads();
      if (tid < 5) {
        double sum = 0;
        for (int w = 0; w < kWarps; w++) sum += sdot[w][tid];
        red5[tid] = sum;
      }
      if (tid == 0) *ticket = 0u;
    }
  }
}

static std::atomic<int> g_sms{0};
int device_sm_count() {
  int n = g_sms.load();
  if (!n) {
    int dev = 0;
    AC3D_CUDA(cudaGetDevice(&dev));
    AC3D_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
    g_sms.store(n);
  }
  return n;
}

constexpr size_t kRingBytes = (size_t)kStages * kStageBytes;

template <typename MT, typename VT, typename AT, int RPL>
static void set_smem_attrs_rpl() {
  AC3D_CUDA(cudaFuncSetAttribute(seg_dot_kernel<MT, AT, RPL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kRingBytes));
  // the largest shared-memory carveout, so that four CTAs of the ring size fit on an SM
  AC3D_CUDA(cudaFuncSetAttribute(seg_dot_kernel<MT, AT, RPL>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 100));
  for (auto kern : {seg_gather_persist_kernel<MT, VT, AT, false, RPL>, seg_gather_persist_kernel<MT, VT, AT, true, RPL>}) {
    AC3D_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
    AC3D_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kRingBytes));
  }
}

template <typename MT, typename VT, typename AT>
static void set_smem_attrs() {
  set_smem_attrs_rpl<MT, VT, AT, 1>();
  set_smem_attrs_rpl<MT, VT, AT, 2>();
  set_smem_attrs_rpl<MT, VT, AT, 4>();
  set_smem_attrs_rpl<MT, VT, AT, 8>();
}

void prepare_matvec_kernels() {
  // once per process (one device per process); contexts on other threads wait for the first call
  static std::once_flag once;
  std::call_once(once, [] {
    set_smem_attrs<float, float, float>();
    set_smem_attrs<float, double, df32>();
    set_smem_attrs<float, double, float>();
    set_smem_attrs<double, double, double>();
  });
}

template <typename MT, typename VT, typename AT, int RPL>
static void mv_t(const DevPartition& DP, const DevHMat& H, bool tr, const void* x, void* y, const void* bminus,
                 const MatvecEpilogue& ep, const int* done, void* tvec, cudaStream_t s, const void* x32, bool pdl) {
  SegView v;
  v.leaf_start = DP.leaf_start.as<int>();
  v.a_seg = DP.near_seg.as<long long>();
  v.a_kptr = DP.didx_ptr.as<int>();
  v.a_idx = DP.didx.as<int>();
  v.blocks_d = DP.blocks_d.as<int4>();
  v.near_off = DP.near_off.as<long long>();
  v.trn_ptr = DP.tr_near_ptr.as<int>();
  v.trn = DP.tr_near.as<int>();
  v.err = H.err.as<int>();
  const cplx<MT>* useg = H.useg.as<cplx<MT>>();
  const cplx<MT>* vseg = H.vseg.as<cplx<MT>>();
  cplx<AT>* t = (cplx<AT>*)tvec;
  cplx<AT>* p = H.pbuf.as<cplx<AT>>();
  // column multipliers taken from x in the accumulator type: x itself, its FP32 shadow x32 (FP64
  // vectors on FP32 arithmetic) or its double-float copy
  const cplx<AT>* xm = x32 ? (const cplx<AT>*)x32 : (const cplx<AT>*)x;
  if constexpr (std::is_same<AT, df32>::value) {
    launch_k(pdl, to_df_kernel, dim3((DP.ne + 255) / 256), dim3(256), 0, s, DP.ne, (const cd*)x,
             H.xdf.as<cplx<df32>>());
    xm = H.xdf.as<cplx<df32>>();
  }
  if (DP.na > 0) {
    // dot pass over the segments on the input side: V by column leaf (forward), U by row leaf
    SegView d = v;
    d.b_seg = tr ? H.seg_f.as<long long>() : H.seg_t.as<long long>();
    d.b_kptr = tr ? H.kseg_f.as<int>() : H.kseg_t.as<int>();
    d.order = tr ? H.order_rows.as<int>() : H.order_cols.as<int>();
    launch_k(pdl, seg_dot_kernel<MT, AT, RPL>, dim3(DP.nleaf), dim3(kThreads), kRingBytes, s, d,
             tr ? useg : vseg, xm, p, done);
    launch_k(pdl, seg_reduce_kernel<AT>, dim3((int)((H.task_cap + 255) / 256)), dim3(256), 0, s,
             H.task_b.as<int>(), H.t_off.as<int>(), (int)H.task_cap, H.t_off.as<int>() + DP.na,
             tr ? DP.blk_fw_ptr.as<int>() : DP.blk_tr_ptr.as<int>(), tr ? H.kpos_f.as<int>() : H.kpos_t.as<int>(),
             p, t, done);
  }
  v.b_seg = tr ? H.seg_t.as<long long>() : H.seg_f.as<long long>();
  v.b_kptr = tr ? H.kseg_t.as<int>() : H.kseg_f.as<int>();
  v.b_idx = tr ? H.vidx.as<int>() : H.uidx.as<int>();
  v.order = tr ? H.order_cols.as<int>() : H.order_rows.as<int>();
  const cplx<AT>* tc = t;
  // the gather reads x and the done flag before its wait, which needs the dot and reduce passes
  // between it and the kernel that wrote them; without low-rank blocks it is an ordinary launch
  // one resident wave: as many CTAs as fit on the device at once (each takes a share of the leaves)
  auto kern = tr ? seg_gather_persist_kernel<MT, VT, AT, true, RPL> : seg_gather_persist_kernel<MT, VT, AT, false, RPL>;
  static std::atomic<int> per_sm[2] = {{0}, {0}};
  int nb = per_sm[tr].load();
  if (!nb) {
    AC3D_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, kGatherThreads, kRingBytes));
    nb = std::max(nb, 1);
    per_sm[tr].store(nb);
  }
  const int P = std::min(DP.nleaf, nb * device_sm_count());
  launch_k(pdl && DP.na > 0, kern, dim3(P), dim3(kGatherThreads), kRingBytes, s, v, DP.nleaf,
           (const cplx<MT>*)H.near.as<cplx<MT>>(),
           tr ? vseg : useg, tc, (const cplx<VT>*)x, xm, (cplx<VT>*)y, (const cplx<VT>*)bminus,
           (const cplx<VT>*)ep.dot_a, (const cplx<VT>*)ep.dot_b, ep.partials, ep.red5, H.ticket.as<unsigned>(), done);

}

template <typename MT, typename VT, typename AT>
static void mv_rpl(const DevPartition& DP, const DevHMat& H, bool tr, const void* x, void* y, const void* bminus,
                   const MatvecEpilogue& ep, const int* done, void* tvec, cudaStream_t s, const void* x32,
                   bool pdl) {
  const int rpl = (DP.max_leaf + 31) / 32;
  if (rpl <= 1)
    mv_t<MT, VT, AT, 1>(DP, H, tr, x, y, bminus, ep, done, tvec, s, x32, pdl);
  else if (rpl <= 2)
    mv_t<MT, VT, AT, 2>(DP, H, tr, x, y, bminus, ep, done, tvec, s, x32, pdl);
  else if (rpl <= 4)
    mv_t<MT, VT, AT, 4>(DP, H, tr, x, y, bminus, ep, done, tvec, s, x32, pdl);
  else
    mv_t<MT, VT, AT, 8>(DP, H, tr, x, y, bminus, ep, done, tvec, s, x32, pdl);
}

// vec64: 0 FP32 vectors; 1 FP64 vectors (FP64 storage: FP64 arithmetic; FP32 storage: the
// double-float residual); 2 FP64 vectors on FP32 storage with FP32 arithmetic, the multipliers
// taken from the FP32 shadow x32 of x. pdl: launch the passes as programmatic dependents (the
// kernel before the first pass then must follow the same protocol, see launch.cuh).
void launch_matvec_ex(const DevPartition& DP, const DevHMat& H, bool transposed, int vec64, const void* x, void* y,
                      const void* b_minus, const MatvecEpilogue& ep, const int* done, cudaStream_t s,
                      const void* x32, bool pdl) {
  if (H.prec == PREC_FP64) {
    if (!vec64) throw Error(3, "internal: FP64 H-matrix needs FP64 vectors");
    mv_rpl<double, double, double>(DP, H, transposed, x, y, b_minus, ep, done, H.tvec64.p, s, nullptr, pdl);
  } else if (vec64 == 2) {
    if (!x32) throw Error(3, "internal: FP32 shadow of the matvec input missing");
    mv_rpl<float, double, float>(DP, H, transposed, x, y, b_minus, ep, done, H.tvec.p, s, x32, pdl);
  } else if (vec64) {
    // FP32 H-matrix with FP64 vectors (refinement residuals): double-float arithmetic
    mv_rpl<float, double, df32>(DP, H, transposed, x, y, b_minus, ep, done, H.tvec64.p, s, nullptr, pdl);
  } else {
    mv_rpl<float, float, float>(DP, H, transposed, x, y, b_minus, ep, done, H.tvec.p, s, nullptr, pdl);
  }
}

void launch_matvec(const DevPartition& DP, const DevHMat& H, int ne, bool transposed, int vec64, const void* x,
                   void* y, const void* b_minus, const MatvecEpilogue& ep, cudaStream_t s) {
  (void)ne;
  launch_matvec_ex(DP, H, transposed, vec64, x, y, b_minus, ep, nullptr, s, nullptr, false);
}

int matvec_grid(const DevPartition& DP, bool) { return DP.nleaf; }

}  // namespace ac3d
