// Block (multi-right-hand-side) H-matrix matvec and block BiCGSTAB.
//
// Up to 16 right-hand sides of one frequency (incidence directions) share one H-matrix. Block
// vectors hold nrb complex FP32 values per element, element-major (Ne x nrb), so every matrix
// byte streamed from HBM serves nrb products. The passes follow the single-vector matvec
// (matvec.cu) over the same per-leaf segments and copy ring: dot pass over the V segments,
// per-term reduce, gather pass over the near and U segments. The plain transpose (adjoint solves,
// hmatrix.h:95-115) runs the same passes with the roles swapped: dot pass over the U segments of
// the row leaves, reduce over the blocks' row-leaf entries, gather over the V segments of the
// column leaves and a transposed copy of the near field laid out by column leaf.
//
// Block BiCGSTAB: nrb independent BiCGSTAB recurrences (van der Vorst 1992) sharing the matvecs,
// with per-column scalars, FP64 dot products reduced in fixed order, and per-column convergence;
// a column that has converged (or broken down) is frozen while the others continue.
#include <algorithm>
#include <mutex>

#include "common.cuh"
#include "internal.h"
#include "multi.h"
#include "segstream.cuh"
#include "tcgen05.cuh"

namespace ac3d {

namespace {
constexpr int kMT = 256;          // threads per CTA
constexpr int kMW = kMT / 32;     // warps per CTA
constexpr int kMPieces = 512;     // gather: multiplier values per chunk (columns x nrb)
constexpr int kGroup = 32;        // CTAs per first-level reduction group
}  // namespace

// Fixed-order two-level reduction of per-CTA partial vectors (part[blockIdx.x][NV]): the last CTA
// of each group of 32 sums its group into gpart, the last group to finish sums the group totals
// into out[NV]. tickets: one counter per group plus one, zero between launches (reset here).
template <int NV>
__device__ __forceinline__ void grid_reduce(const double* part, double* gpart, unsigned* tickets, double* out) {
  __shared__ bool s_last;
  const int g = blockIdx.x / kGroup, ng = (gridDim.x + kGroup - 1) / kGroup;
  const int gsize = min(kGroup, (int)gridDim.x - g * kGroup);
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(&tickets[g], 1u) == (unsigned)(gsize - 1);
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  for (int v = threadIdx.x; v < NV; v += blockDim.x) {
    double a = 0;
#pragma unroll 8
    for (int i = 0; i < gsize; i++) a += __ldcg(&part[(size_t)(g * kGroup + i) * NV + v]);
    gpart[(size_t)g * NV + v] = a;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    tickets[g] = 0u;
    s_last = atomicAdd(&tickets[ng], 1u) == (unsigned)(ng - 1);
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  for (int v = threadIdx.x; v < NV; v += blockDim.x) {
    double a = 0;
#pragma unroll 8
    for (int i = 0; i < ng; i++) a += __ldcg(&gpart[(size_t)i * NV + v]);
    out[v] = a;
  }
  if (threadIdx.x == 0) tickets[ng] = 0u;
}

// Sums d[c] (c < 5) over the threads of the CTA that share a column j = tid % NRB and writes the
// CTA's partials part[blockIdx.x][c][j].
template <int NRB>
__device__ __forceinline__ void cta_partials(double d[5], double* part) {
  __shared__ double sred[kMW][5][NRB];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < 5; c++)
#pragma unroll
    for (int o = NRB; o < 32; o <<= 1) d[c] += __shfl_xor_sync(0xffffffffu, d[c], o);
  if (lane < NRB)
    for (int c = 0; c < 5; c++) sred[warp][c][lane] = d[c];
  __syncthreads();
  for (int v = threadIdx.x; v < 5 * NRB; v += blockDim.x) {
    double a = 0;
    for (int w = 0; w < kMW; w++) a += sred[w][v / NRB][v % NRB];
    part[(size_t)blockIdx.x * 5 * NRB + v] = a;
  }
}

// ------------------------------------------------------------------------------------------
// Matvec passes
// ------------------------------------------------------------------------------------------
// Dot pass: P[k][j] = sum_rows V[row][k] X[row][j]. Lane (j = lane % NRB, h = lane / NRB) holds
// X[row][j] for rows h, h + H, ... (H = 32 / NRB); one warp per segment column.
template <int NRB, int RPL>
__global__ void __launch_bounds__(kMT) mseg_dot_kernel(SegView V, const cf* __restrict__ seg,
                                                       const cf* __restrict__ X, cf* __restrict__ P,
                                                       const int* __restrict__ done) {
  constexpr int H = 32 / NRB;
  constexpr int RPH = (32 * RPL + H - 1) / H;
  extern __shared__ __align__(128) unsigned char dsmem[];
  auto stage = reinterpret_cast<unsigned char(*)[kStageBytes]>(dsmem);
  __shared__ __align__(8) uint64_t full[kStages];
  if (done && *done) return;
  const int leaf = V.order[blockIdx.x];
  const int ls = V.leaf_start[leaf], R = V.leaf_start[leaf + 1] - ls;
  const int k0 = V.b_kptr[leaf], K = V.b_kptr[leaf + 1] - k0;
  if (K == 0) return;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int j = lane % NRB, h = lane / NRB;
  float xr[RPH], xi[RPH];
#pragma unroll
  for (int t = 0; t < RPH; t++) {
    const int row = h + H * t;
    const cf v = row < R ? X[(size_t)(ls + row) * NRB + j] : cf();
    xr[t] = v.re;
    xi[t] = v.im;
  }
  init_ring(full);
  cf* out = P + (size_t)k0 * NRB;
  stream_leaf<float>(stage, full, R, nullptr, 0, seg + V.b_seg[leaf], K, V.err,
                     [&](const cf* S, int, int c0, int ncols, int, int, int) {
                       for (int c = warp; c < ncols; c += kMW) {
                         const cf* col = S + c * R;
                         float ar0 = 0, ai0 = 0, ar1 = 0, ai1 = 0;  // two chains for ILP
#pragma unroll
                         for (int t = 0; t < RPH; t++) {
                           const int row = h + H * t;
                           if (row < R) {
                             const cf v = col[row];
                             float& ar = (t & 1) ? ar1 : ar0;
                             float& ai = (t & 1) ? ai1 : ai0;
                             ar = fmaf(v.re, xr[t], ar);
                             ar = fmaf(-v.im, xi[t], ar);
                             ai = fmaf(v.re, xi[t], ai);
                             ai = fmaf(v.im, xr[t], ai);
                           }
                         }
                         float ar = ar0 + ar1, ai = ai0 + ai1;
#pragma unroll
                         for (int o = NRB; o < 32; o <<= 1) {
                           ar += __shfl_xor_sync(0xffffffffu, ar, o);
                           ai += __shfl_xor_sync(0xffffffffu, ai, o);
                         }
                         if (h == 0) out[(size_t)(c0 + c) * NRB + j] = cf(ar, ai);
                       }
                     });
}

// ------------------------------------------------------------------------------------------
// Dot pass on the tensor cores (tcgen05; nrb = 8 or 16, leaves of at most 32 rows). For a leaf
// with R rows and K segment columns, P (K x nrb complex) = S^T X_leaf is the real product
// D (K x 2 nrb) = A (K x 2R) B (2R x 2 nrb), where row k of A is segment column k (re, im
// interleaved, 2R floats) and B interleaves X by row: row 2r = (Xr_r | Xi_r), row 2r + 1 =
// (-Xi_r | Xr_r); columns 0..nrb-1 of D are Re P, nrb..2nrb-1 Im P. Operands are TF32 with every
// FP32 value split as hi + lo, and the product hi hi + hi lo + lo hi takes two MMAs per K step:
// A_hi [B_hi | B_lo] (N = 4 nrb; the two halves are summed when D is read back) and A_lo B_hi
// accumulated onto the first half. Tiles of 128 segment columns (M = 128), K = 2R rounded up to
// 8 (Kd), FP32 accumulation in tensor memory.
//
// The segments are split once per H-matrix (tc_split_kernel) into their hi and lo parts, stored
// tile by tile in the canonical K-major layout the MMA reads: 8-row x 16-byte core matrices,
// adjacent along K, 8-row groups Kd / 4 core matrices apart; a tile's lo part follows its hi
// part, and only the leaf's last tile is shorter than 128 rows (rounded up to 8). The pass is
// then a pipeline without repacking, in three warp roles: warp 0 bulk-copies tile pairs into a
// ring of stages, warp 1 issues the MMAs of each landed tile into one of two accumulators, and
// warps 4..7 (tensor-memory lanes 0..127) read finished accumulators back into P. The roles meet
// only on mbarriers; every wait is bounded, and a role that gives up records the failure so the
// others stop at their next wait.
// ------------------------------------------------------------------------------------------
constexpr int kTcM = 128;
constexpr int kTcKmax = 64;  // 2R for leaves of up to 32 rows
constexpr int kTcStages = 3;
constexpr size_t kTcStageBytes = 2ull * kTcM * kTcKmax * sizeof(float);  // largest tile pair

__host__ __device__ constexpr int tc_tile_off(int row, int kq, int kq_n) {
  return (row >> 3) * (kq_n * 128) + kq * 128 + (row & 7) * 16;
}

// B operand: 4 nrb rows (hi parts, then lo parts) of up to kTcKmax values
template <int NRB>
__host__ __device__ constexpr size_t tc_b_bytes() {
  return (size_t)(4 * NRB) * kTcKmax * sizeof(float);
}

template <int NRB>
constexpr size_t tc_dot_smem() {
  return tc_b_bytes<NRB>() + (size_t)kTcStages * kTcStageBytes;
}

// Bytes of a leaf's split segment: hi and lo parts of ceil8(K) rows of Kd floats.
__host__ __device__ constexpr long long tc_leaf_bytes(int R, int K) {
  return 8ll * ((2 * R + 7) & ~7) * ((K + 7) & ~7);
}

// One CTA per leaf: the leaf's segment (R x K column-major complex) into split TF32 tiles.
__global__ void tc_split_kernel(const cf* __restrict__ seg, const long long* __restrict__ seg_off,
                                const int* __restrict__ kseg, const int* __restrict__ leaf_start,
                                const long long* __restrict__ tc_off, unsigned char* __restrict__ tc) {
  const int l = blockIdx.x;
  const int R = leaf_start[l + 1] - leaf_start[l], K = kseg[l + 1] - kseg[l];
  const int Kd = (2 * R + 7) & ~7, kq_n = Kd / 4;
  const float* S = reinterpret_cast<const float*>(seg + seg_off[l]);
  unsigned char* dst = tc + tc_off[l];
  for (int t = 0; t * kTcM < K; t++) {
    const int rows = min(kTcM, K - t * kTcM), g8 = (rows + 7) & ~7;
    unsigned char* hi_base = dst + (size_t)t * 2 * kTcM * Kd * sizeof(float);
    unsigned char* lo_base = hi_base + (size_t)g8 * Kd * sizeof(float);
    for (int e = threadIdx.x; e < g8 * kq_n; e += blockDim.x) {
      const int rr = e % g8, kq = e / g8;
      const int k = t * kTcM + rr;
      float v[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int kk = 4 * kq + q;
        v[q] = rr < rows && kk < 2 * R ? S[(size_t)k * 2 * R + kk] : 0.f;
      }
      float4 hi, lo;
      split_tf32(v[0], hi.x, lo.x);
      split_tf32(v[1], hi.y, lo.y);
      split_tf32(v[2], hi.z, lo.z);
      split_tf32(v[3], hi.w, lo.w);
      const int o = tc_tile_off(rr, kq, kq_n);
      *reinterpret_cast<float4*>(hi_base + o) = hi;
      *reinterpret_cast<float4*>(lo_base + o) = lo;
    }
  }
}

template <int NRB>
__global__ void __launch_bounds__(kMT, 1) mseg_dot_tc_kernel(SegView V, const unsigned char* __restrict__ tcs,
                                                             const long long* __restrict__ tc_off,
                                                             const cf* __restrict__ X, cf* __restrict__ P,
                                                             const int* __restrict__ done) {
  constexpr int N = 2 * NRB;  // columns of D
  constexpr int NT = 2 * N;   // accumulator columns in tensor memory (hi | lo halves)
  static_assert(NT == 32 || NT == 64, "nrb 8 or 16");
  extern __shared__ __align__(128) unsigned char dsmem[];
  unsigned char* Bt = dsmem;
  unsigned char* ring = dsmem + tc_b_bytes<NRB>();
  __shared__ __align__(8) uint64_t full[kTcStages], empty[kTcStages], accf[2], acce[2];
  __shared__ uint32_t s_tmem;
  __shared__ int s_fail, s_issued, s_consumed;
  if (done && *done) return;
  const int leaf = V.order[blockIdx.x];
  const int ls = V.leaf_start[leaf], R = V.leaf_start[leaf + 1] - ls;
  const int k0 = V.b_kptr[leaf], K = V.b_kptr[leaf + 1] - k0;
  if (K == 0 || R > kTcKmax / 2) return;  // the host launches this pass only for leaves of <= 32 rows
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int Kd = (2 * R + 7) & ~7, kq_n = Kd / 4;
  const int ntiles = (K + kTcM - 1) / kTcM;
  const unsigned char* src = tcs + tc_off[leaf];
  // B operand, 2N x Kd K-major: rows n < N the hi parts, N + n the lo parts
  for (int e = tid; e < N * kq_n; e += blockDim.x) {
    const int n = e % N, kq = e / N, jj = n % NRB;
    float v[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int kk = 4 * kq + q;
      v[q] = 0.f;
      if (kk < 2 * R) {
        const cf x = X[(size_t)(ls + (kk >> 1)) * NRB + jj];
        v[q] = n < NRB ? ((kk & 1) ? -x.im : x.re) : ((kk & 1) ? x.re : x.im);
      }
    }
    float4 hi, lo;
    split_tf32(v[0], hi.x, lo.x);
    split_tf32(v[1], hi.y, lo.y);
    split_tf32(v[2], hi.z, lo.z);
    split_tf32(v[3], hi.w, lo.w);
    *reinterpret_cast<float4*>(Bt + tc_tile_off(n, kq, kq_n)) = hi;
    *reinterpret_cast<float4*>(Bt + tc_tile_off(N + n, kq, kq_n)) = lo;
  }
  if (tid == 0) {
    for (int s = 0; s < kTcStages; s++) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; b++) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], 128);
    }
    s_fail = 0;
    s_issued = 0;
    s_consumed = 0;
    fence_barrier_init();
  }
  if (warp == 0) {
    tmem_alloc(&s_tmem, 2 * NT);
    tmem_relinquish();
  }
  fence_proxy_async();  // the B stores become visible to the tensor core
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = s_tmem;
  const uint32_t sbo = (uint32_t)(kq_n * 128);
  volatile int* fail = &s_fail;
  auto give_up = [&]() {
    *fail = 1;
    atomicExch(V.err, 1);
  };
  if (warp == 0) {
    if (lane == 0) {  // producer
      int t = 0;
      for (; t < ntiles && !*fail; t++) {
        const int s = t % kTcStages;
        if (t >= kTcStages && !mbar_wait_bounded(&empty[s], (uint32_t)(t / kTcStages - 1) & 1u)) {
          give_up();
          break;
        }
        const int rows = min(kTcM, K - t * kTcM), g8 = (rows + 7) & ~7;
        const uint32_t bytes = 8u * (uint32_t)(g8 * Kd);
        mbar_expect_tx(&full[s], bytes);
        bulk_copy_g2s(ring + (size_t)s * kTcStageBytes, src + (size_t)t * 2 * kTcM * Kd * sizeof(float), bytes,
                      &full[s]);
      }
      s_issued = t;
    }
  } else if (warp == 1) {
    if (lane == 0) {  // MMA issuer
      const uint32_t idw = umma_idesc_tf32(kTcM, NT), idn = umma_idesc_tf32(kTcM, N);
      int t = 0;
      for (; t < ntiles && !*fail; t++) {
        const int s = t % kTcStages, b = t & 1;
        if (!mbar_wait_bounded(&full[s], (uint32_t)(t / kTcStages) & 1u) ||
            (t >= 2 && !mbar_wait_bounded(&acce[b], (uint32_t)((t >> 1) - 1) & 1u))) {
          give_up();
          break;
        }
        tc_fence_after();
        const int rows = min(kTcM, K - t * kTcM), g8 = (rows + 7) & ~7;
        const unsigned char* Ah = ring + (size_t)s * kTcStageBytes;
        const unsigned char* Al = Ah + (size_t)4 * g8 * Kd;
        const uint32_t d = tmem + (uint32_t)(b * NT);
        for (int ks = 0; ks < Kd / 8; ks++) {
          const uint32_t o = (uint32_t)ks * 256u;
          const uint64_t bd = umma_smem_desc(Bt + o, 128, sbo);
          umma_tf32(d, umma_smem_desc(Ah + o, 128, sbo), bd, idw, ks > 0 ? 1u : 0u);
          umma_tf32(d, umma_smem_desc(Al + o, 128, sbo), bd, idn, 1u);
        }
        umma_commit(&empty[s]);
        umma_commit(&accf[b]);
      }
      s_consumed = t;
    }
  } else if (warp >= 4) {  // accumulator read-back: warp 4 + w reads tensor-memory lanes 32 w ..
    const int ew = warp - 4;
    cf* out = P + (size_t)k0 * NRB;
    for (int t = 0; t < ntiles; t++) {
      const int b = t & 1;
      int got = 1;
      if (lane == 0) got = !*fail && mbar_wait_bounded(&accf[b], (uint32_t)(t >> 1) & 1u);
      if (!__shfl_sync(0xffffffffu, got, 0)) {
        if (lane == 0 && !*fail) give_up();
        break;
      }
      tc_fence_after();
      const uint32_t ta = tmem + ((uint32_t)(ew * 32) << 16) + (uint32_t)(b * NT);
      float v[64];
      tmem_ld32(ta, *reinterpret_cast<float(*)[32]>(v));
      if constexpr (NT == 64) tmem_ld32(ta + 32, *reinterpret_cast<float(*)[32]>(v + 32));
      const int row = ew * 32 + lane, rows = min(kTcM, K - t * kTcM);
      if (row < rows) {
        float4* o = reinterpret_cast<float4*>(out + (size_t)(t * kTcM + row) * NRB);
#pragma unroll
        for (int j = 0; j < NRB; j += 2)
          o[j / 2] = make_float4(v[j] + v[N + j], v[NRB + j] + v[N + NRB + j], v[j + 1] + v[N + j + 1],
                                 v[NRB + j + 1] + v[N + NRB + j + 1]);
      }
      tc_fence_before();
      mbar_arrive(&acce[b]);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (tid == 0 && s_fail) {
    // after a failure: let the copies that were issued but not consumed land before the CTA exits
    for (int t = s_consumed; t < s_issued; t++)
      mbar_wait_bounded(&full[t % kTcStages], (uint32_t)(t / kTcStages) & 1u);
  }
  __syncthreads();
  tc_fence_after();
  if (warp == 0) tmem_dealloc(tmem, 2 * NT);
}

// T[task][j] = sum over the task's block entries of P[kpos[e] + q][j], in leaf order.
template <int NRB>
__global__ void __launch_bounds__(256) mseg_reduce_kernel(const int* __restrict__ task_b,
                                                          const int* __restrict__ t_off, int ntask_cap,
                                                          const int* __restrict__ t_total,
                                                          const int* __restrict__ ent_ptr,
                                                          const int* __restrict__ kpos, const cf* __restrict__ P,
                                                          cf* __restrict__ T, const int* __restrict__ done) {
  if (done && *done) return;
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int task = (int)(i / NRB), j = (int)(i % NRB);
  if (task >= ntask_cap || task >= *t_total) return;
  const int b = task_b[task];
  const int q = task - t_off[b];
  float sr = 0, si = 0;
  const int e1 = ent_ptr[b + 1];
  int e = ent_ptr[b];
  for (; e + 3 < e1; e += 4) {  // four independent loads in flight, summed in entry order
    const int k0 = kpos[e], k1 = kpos[e + 1], k2 = kpos[e + 2], k3 = kpos[e + 3];
    const cf v0 = P[(size_t)(k0 + q) * NRB + j], v1 = P[(size_t)(k1 + q) * NRB + j];
    const cf v2 = P[(size_t)(k2 + q) * NRB + j], v3 = P[(size_t)(k3 + q) * NRB + j];
    sr += v0.re;
    si += v0.im;
    sr += v1.re;
    si += v1.im;
    sr += v2.re;
    si += v2.im;
    sr += v3.re;
    si += v3.im;
  }
  for (; e < e1; e++) {
    const cf v = P[(size_t)(kpos[e] + q) * NRB + j];
    sr += v.re;
    si += v.im;
  }
  T[(size_t)task * NRB + j] = cf(sr, si);
}

// Gather pass: Y[rows][j] = -X/2 + near X[idx] + U T[idx], with per-column dot partials. Lane l
// owns rows l + 32 q of the leaf and accumulates all NRB right-hand sides of them; warp w takes the
// chunk columns w, w + 8, ..., so each segment element read from shared memory feeds 4 NRB FMAs
// against the column's multiplier row (read as broadcast 16-byte loads). The warps' partial tiles
// are summed once per leaf in fixed order. With every chunk's bulk copy each thread gathers (at
// most) one 16-byte piece of a column's multiplier row (two of its nrb values) by cp.async into
// the stage's multiplier buffer; the stage's mbarrier expects the copy bytes and one arrival per
// thread, as in the single-vector gather pass.
template <int NRB, int RPL>
__global__ void __launch_bounds__(kMT) mseg_gather_kernel(SegView V, const cf* __restrict__ near,
                                                          const cf* __restrict__ lrseg, const cf* __restrict__ T,
                                                          const cf* __restrict__ X, cf* __restrict__ Y,
                                                          const cf* __restrict__ dot_a, const cf* __restrict__ dot_b,
                                                          double* part, double* gpart, unsigned* tickets,
                                                          double* red, const int* __restrict__ done) {
  constexpr int CMAX = kMPieces / NRB;        // columns per chunk at most
  constexpr int PPC = NRB / 2;                // 16-byte pieces per multiplier row
  extern __shared__ __align__(128) unsigned char dsmem[];
  auto stage = reinterpret_cast<unsigned char(*)[kStageBytes]>(dsmem);
  __shared__ __align__(8) uint64_t full[kStages];
  __shared__ __align__(16) unsigned char zraw[kStages * kMPieces * sizeof(cf)];
  auto zbuf = reinterpret_cast<cf(*)[kMPieces]>(zraw);
  if (done && *done) return;
  const int leaf = V.order[blockIdx.x];
  const int ls = V.leaf_start[leaf], R = V.leaf_start[leaf + 1] - ls;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  const int a_cols = V.a_kptr[leaf + 1] - V.a_kptr[leaf];
  const int* a_idx = V.a_idx + V.a_kptr[leaf];
  const int b_cols = V.b_kptr[leaf + 1] - V.b_kptr[leaf];
  const int* b_idx = V.b_idx + V.b_kptr[leaf];
  const cf* a_ptr = near + V.a_seg[leaf];
  const cf* b_ptr = lrseg + V.b_seg[leaf];
  const int cpc = min(CMAX, max(2, (int)(kStageBytes / sizeof(cf)) / R & ~1));
  const int na = (a_cols + cpc - 1) / cpc, nb = (b_cols + cpc - 1) / cpc;
  const int nch = na + nb;
  struct Chunk {
    const cf* src;
    const int* idx;
    const cf* z;
    int ncols;
  };
  auto chunk = [&](int c) {
    Chunk k;
    if (c < na) {
      const int c0 = c * cpc;
      k.ncols = min(cpc, a_cols - c0);
      k.src = a_ptr + (long long)c0 * R;
      k.idx = a_idx + c0;
      k.z = X;
    } else {
      const int c0 = (c - na) * cpc;
      k.ncols = min(cpc, b_cols - c0);
      k.src = b_ptr + (long long)c0 * R;
      k.idx = b_idx + c0;
      k.z = T;
    }
    return k;
  };
  // this thread's piece: column tid / PPC, values 2 (tid % PPC) and 2 (tid % PPC) + 1
  const int pcol = tid / PPC, ppos = 2 * (tid % PPC);
  auto col_index = [&](int c) {
    if (c >= nch) return -1;
    const Chunk k = chunk(c);
    return pcol < k.ncols ? k.idx[pcol] : -1;
  };
  auto issue = [&](int c, int s, int zi) {
    const Chunk k = chunk(c);
    if (pcol < k.ncols) {
      cf* dst = &zbuf[s][pcol * NRB + ppos];
      if (zi >= 0) {
        cp_async_elem<16>(dst, k.z + (size_t)zi * NRB + ppos);
      } else {
        dst[0] = cf();
        dst[1] = cf();
      }
    }
    cp_async_arrive_noinc(&full[s]);
    if (tid == 0) {
      const uint32_t bytes = (uint32_t)(k.ncols * R * sizeof(cf));
      mbar_expect_tx(&full[s], bytes);
      bulk_copy_g2s(stage[s], k.src, bytes, &full[s]);
    }
  };

  if (tid == 0) {
    for (int st = 0; st < kStages; st++) mbar_init(&full[st], 1 + kMT);
    fence_barrier_init();
  }
  __syncthreads();
  {
    int zi[kStages];
#pragma unroll
    for (int c = 0; c < kStages; c++) zi[c] = col_index(c);
#pragma unroll
    for (int c = 0; c < kStages; c++)
      if (c < nch) issue(c, c, zi[c]);
  }
  int next_zi = col_index(kStages);

  float ar[RPL][NRB], ai[RPL][NRB];
#pragma unroll
  for (int q = 0; q < RPL; q++)
#pragma unroll
    for (int jj = 0; jj < NRB; jj++) ar[q][jj] = ai[q][jj] = 0.f;
  bool ok = true;
  int c = 0;
  for (; c < nch; c++) {
    const int s = c % kStages;
    if (!cta_wait(&full[s], (uint32_t)(c / kStages) & 1u)) {
      ok = false;
      break;
    }
    const int ncols = chunk(c).ncols;
    const cf* S = (const cf*)stage[s];
    const cf* Z = zbuf[s];
    for (int cc = warp; cc < ncols; cc += kMW) {
      const cf* col = S + cc * R;
      cf u[RPL];
#pragma unroll
      for (int q = 0; q < RPL; q++) {
        const int row = lane + 32 * q;
        u[q] = row < R ? col[row] : cf();
      }
      const float4* z4 = reinterpret_cast<const float4*>(Z + cc * NRB);
#pragma unroll
      for (int jj = 0; jj < NRB / 2; jj++) {
        const float4 zz = z4[jj];  // multipliers 2 jj and 2 jj + 1
#pragma unroll
        for (int q = 0; q < RPL; q++) {
          ar[q][2 * jj] = fmaf(u[q].re, zz.x, ar[q][2 * jj]);
          ar[q][2 * jj] = fmaf(-u[q].im, zz.y, ar[q][2 * jj]);
          ai[q][2 * jj] = fmaf(u[q].re, zz.y, ai[q][2 * jj]);
          ai[q][2 * jj] = fmaf(u[q].im, zz.x, ai[q][2 * jj]);
          ar[q][2 * jj + 1] = fmaf(u[q].re, zz.z, ar[q][2 * jj + 1]);
          ar[q][2 * jj + 1] = fmaf(-u[q].im, zz.w, ar[q][2 * jj + 1]);
          ai[q][2 * jj + 1] = fmaf(u[q].re, zz.w, ai[q][2 * jj + 1]);
          ai[q][2 * jj + 1] = fmaf(u[q].im, zz.z, ai[q][2 * jj + 1]);
        }
      }
    }
    __syncthreads();  // stage s and its multipliers are consumed
    if (c + kStages < nch) {
      fence_proxy_async();
      const int zi = next_zi;
      next_zi = col_index(c + kStages + 1);
      issue(c + kStages, s, zi);
    }
  }
  if (!ok) {
    if (tid == 0) {
      atomicExch(V.err, 1);
      for (int cc = c; cc < min(nch, c + kStages); cc++)
        mbar_wait_bounded(&full[cc % kStages], (uint32_t)(cc / kStages) & 1u);
    }
    cp_async_wait_all();
    __syncthreads();
  }
  // sum the warps' tiles in fixed order through four slots in the ring memory (all stages are
  // consumed): slot w = warp w + warp w + 4, then slot 0 + 1 + 2 + 3
  cf* tile = (cf*)stage;
  const int tsz = R * NRB;
  __syncthreads();
  for (int round = 0; round < 2; round++) {
    if ((warp >> 2) == round) {
      cf* dst = tile + (warp & 3) * tsz;
#pragma unroll
      for (int q = 0; q < RPL; q++) {
        const int row = lane + 32 * q;
        if (row < R) {
#pragma unroll
          for (int jj = 0; jj < NRB; jj++) {
            cf v(ar[q][jj], ai[q][jj]);
            if (round) v = cf(dst[row * NRB + jj].re + v.re, dst[row * NRB + jj].im + v.im);
            dst[row * NRB + jj] = v;
          }
        }
      }
    }
    __syncthreads();
  }
  double d[5] = {0, 0, 0, 0, 0};
  for (int i = tid; i < tsz; i += kMT) {  // column j = tid % NRB for every i of this thread
    const int row = i / NRB;
    {
      const cf t0 = tile[i], t1 = tile[tsz + i], t2 = tile[2 * tsz + i], t3 = tile[3 * tsz + i];
      const float sr = ((t0.re + t1.re) + t2.re) + t3.re, si = ((t0.im + t1.im) + t2.im) + t3.im;
      const size_t e = (size_t)(ls + row) * NRB + i % NRB;
      const cf xv = X[e];
      const cf o(sr - 0.5f * xv.re, si - 0.5f * xv.im);
      Y[e] = o;
      const double oyr = o.re, oyi = o.im;
      if (dot_a) {
        const cf a = dot_a[e];
        d[0] += (double)a.re * oyr + (double)a.im * oyi;
        d[1] += (double)a.re * oyi - (double)a.im * oyr;
      }
      if (dot_b) {
        const cf bb = dot_b[e];
        d[2] += oyr * (double)bb.re + oyi * (double)bb.im;
        d[3] += oyr * (double)bb.im - oyi * (double)bb.re;
      }
      d[4] += oyr * oyr + oyi * oyi;
    }
  }
  if (part) {
    cta_partials<NRB>(d, part);
    grid_reduce<5 * NRB>(part, gpart, tickets, red);
  }
}

// ------------------------------------------------------------------------------------------
// Block BiCGSTAB vector steps (element-major block vectors, column j = index % NRB)
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ void cdiv64(double ar, double ai, double br, double bi, double& cr, double& ci) {
  const double s = fabs(br) + fabs(bi);
  const double xr = br / s, xi = bi / s, yr = ar / s, yi = ai / s;
  const double d = xr * xr + xi * xi;
  cr = (yr * xr + yi * xi) / d;
  ci = (yi * xr - yr * xi) / d;
}

template <int NRB>
__global__ void __launch_bounds__(kMT) mk_init(int n, const cf* __restrict__ b, cf* x, cf* r, cf* rhat, cf* p,
                                               cf* v, double* part) {
  double d[5] = {0, 0, 0, 0, 0};
  const long long m = (long long)n * NRB;
  for (long long i = (long long)blockIdx.x * kMT + threadIdx.x; i < m; i += (long long)gridDim.x * kMT) {
    const cf bi = b[i];
    x[i] = cf();
    r[i] = bi;
    rhat[i] = bi;
    p[i] = cf();
    v[i] = cf();
    d[4] += (double)bi.re * bi.re + (double)bi.im * bi.im;
  }
  cta_partials<NRB>(d, part);
}

template <int NRB>
__global__ void mk_scalar_init(KStateM* st, const double* __restrict__ part, int nparts,
                               const double* __restrict__ tol, int maxit, double* rtot) {
  const int j = threadIdx.x;
  if (j == 0) {
    st->iter = 0;
    st->maxit = maxit;
    st->nrb = NRB;
    st->ticket = 0u;
  }
  if (j < NRB) {
    double s = 0;
    for (int i = 0; i < nparts; i++) s += part[(size_t)i * 5 * NRB + 4 * NRB + j];
    KCol& k = st->col[j];
    k.bnorm2 = k.rnorm2 = k.rhat2 = s;
    k.tol2 = tol[j] * tol[j] * s;
    k.rho_re = k.alpha_re = k.omega_re = 1.0;
    k.rho_im = k.alpha_im = k.omega_im = 0.0;
    k.rho_new_re = 1.0;
    k.rho_new_im = 0.0;
    for (int c = 0; c < 5; c++) rtot[c * NRB + j] = 0.0;
    rtot[0 * NRB + j] = s;  // (rhat, r) = |b|^2 at the start
    rtot[4 * NRB + j] = s;
    k.done = s == 0.0 ? 1 : 0;
    k.restart = 0;
    k.restarts = 0;
  }
  __syncthreads();
  if (j == 0) {
    int all = 1;
    for (int c = 0; c < NRB; c++) all &= st->col[c].done != 0;
    st->done_all = all;
  }
}

// Per-column scalars shared by the CTAs of one vector kernel (computed by threads 0..NRB-1).
struct MScal {
  double a_re, a_im, b_re, b_im;
  int active, restart;
};

// start of an iteration: per-column convergence test, rho, beta; p = r + beta (p - omega v)
template <int NRB>
__global__ void __launch_bounds__(kMT) mkf_p(KStateM* st, const double* __restrict__ rtot, int n,
                                             const cf* __restrict__ r, cf* p, cf* v, cf* rhat) {
  __shared__ MScal sc[NRB];
  __shared__ int s_any;
  if (st->done_all) return;
  const int t = threadIdx.x;
  if (t == 0) s_any = 0;
  __syncthreads();
  if (t < NRB) {
    const KCol& k = st->col[t];
    MScal o{0, 0, 0, 0, 0, 0};
    int stop_code = 0;
    if (k.done == 0) {
      const double rr = rtot[4 * NRB + t];
      if (!(rr > k.tol2)) {
        stop_code = 1;
      } else if (st->iter >= st->maxit) {
        stop_code = 2;
      } else {
        double rho_re = rtot[0 * NRB + t], rho_im = rtot[1 * NRB + t];
        o.active = 1;
        if (rho_re * rho_re + rho_im * rho_im <= 1e-24 * k.rhat2 * rr) {
          o.restart = 1;
          rho_re = rr;
          rho_im = 0.0;
        } else {
          double q1r, q1i, q2r, q2i;
          cdiv64(rho_re, rho_im, k.rho_re, k.rho_im, q1r, q1i);
          cdiv64(k.alpha_re, k.alpha_im, k.omega_re, k.omega_im, q2r, q2i);
          o.b_re = q1r * q2r - q1i * q2i;
          o.b_im = q1r * q2i + q1i * q2r;
          o.a_re = k.omega_re;  // omega for the p update
          o.a_im = k.omega_im;
        }
        if (blockIdx.x == 0) {
          KCol& kw = st->col[t];
          kw.rnorm2 = rr;
          kw.rho_new_re = rho_re;
          kw.rho_new_im = rho_im;
          kw.restart = o.restart;
          if (o.restart) kw.restarts++;
        }
      }
      if (stop_code && blockIdx.x == 0) {
        st->col[t].rnorm2 = rr;
        st->col[t].done = stop_code;
      }
    }
    sc[t] = o;
    if (o.active) atomicOr(&s_any, 1);
  }
  __syncthreads();
  if (!s_any) {
    if (blockIdx.x == 0 && t == 0) st->done_all = 1;
    return;
  }
  const long long m = (long long)n * NRB;
  for (long long i = (long long)blockIdx.x * kMT + t; i < m; i += (long long)gridDim.x * kMT) {
    const MScal& o = sc[i % NRB];
    if (!o.active) continue;
    const cf ri = r[i];
    if (o.restart) {
      rhat[i] = ri;
      p[i] = ri;
      v[i] = cf();
    } else {
      const float br = (float)o.b_re, bi = (float)o.b_im, wr = (float)o.a_re, wi = (float)o.a_im;
      const cf pi = p[i], vi = v[i];
      const float tr = pi.re - (wr * vi.re - wi * vi.im);
      const float ti = pi.im - (wr * vi.im + wi * vi.re);
      p[i] = cf(ri.re + br * tr - bi * ti, ri.im + br * ti + bi * tr);
    }
  }
}

// alpha = rho / (rhat, v); s = r - alpha v
template <int NRB>
__global__ void __launch_bounds__(kMT) mkf_s(KStateM* st, const double* __restrict__ red, int n,
                                             const cf* __restrict__ r, const cf* __restrict__ v, cf* s) {
  __shared__ MScal sc[NRB];
  if (st->done_all) return;
  const int t = threadIdx.x;
  if (t < NRB) {
    MScal o{0, 0, 0, 0, 0, 0};
    const KCol& k = st->col[t];
    if (k.done == 0) {
      const double d0 = red[0 * NRB + t], d1 = red[1 * NRB + t];
      if (d0 == 0.0 && d1 == 0.0) {
        if (blockIdx.x == 0) st->col[t].done = 3;
      } else {
        cdiv64(k.rho_new_re, k.rho_new_im, d0, d1, o.a_re, o.a_im);
        o.active = 1;
        if (blockIdx.x == 0) {
          st->col[t].alpha_re = o.a_re;  // the alpha of this iteration (alpha of the last one is
          st->col[t].alpha_im = o.a_im;  // no longer needed: beta was formed in mkf_p)
        }
      }
    }
    sc[t] = o;
  }
  __syncthreads();
  const long long m = (long long)n * NRB;
  for (long long i = (long long)blockIdx.x * kMT + t; i < m; i += (long long)gridDim.x * kMT) {
    const MScal& o = sc[i % NRB];
    if (!o.active) continue;
    const float ar = (float)o.a_re, ai = (float)o.a_im;
    const cf ri = r[i], vi = v[i];
    s[i] = cf(ri.re - (ar * vi.re - ai * vi.im), ri.im - (ar * vi.im + ai * vi.re));
  }
}

// omega = (t, s) / (t, t); x += alpha p + omega s; r = s - omega t; per-column residual partials
template <int NRB>
__global__ void __launch_bounds__(kMT) mkf_xr(KStateM* st, const double* __restrict__ red, int n, cf* x,
                                              const cf* __restrict__ p, const cf* __restrict__ s, cf* r,
                                              const cf* __restrict__ tv, const cf* __restrict__ rhat, double* part,
                                              double* gpart, unsigned* tickets, double* rtot) {
  __shared__ MScal sc[NRB];
  if (st->done_all) return;
  const int t = threadIdx.x;
  if (t < NRB) {
    MScal o{0, 0, 0, 0, 0, 0};
    const KCol& k = st->col[t];
    if (k.done == 0) {
      const double d2 = red[2 * NRB + t], d3 = red[3 * NRB + t], d4 = red[4 * NRB + t];
      o.b_re = d4 > 0.0 ? d2 / d4 : 0.0;  // omega
      o.b_im = d4 > 0.0 ? d3 / d4 : 0.0;
      o.a_re = k.alpha_re;
      o.a_im = k.alpha_im;
      o.active = 1;
    }
    sc[t] = o;
  }
  __syncthreads();
  double d[5] = {0, 0, 0, 0, 0};
  const long long m = (long long)n * NRB;
  for (long long i = (long long)blockIdx.x * kMT + t; i < m; i += (long long)gridDim.x * kMT) {
    const MScal& o = sc[i % NRB];
    if (!o.active) continue;
    const float ar = (float)o.a_re, ai = (float)o.a_im, wr = (float)o.b_re, wi = (float)o.b_im;
    const cf pi = p[i], si = s[i], ti = tv[i], hi = rhat[i];
    cf xi = x[i];
    xi.re += (ar * pi.re - ai * pi.im) + (wr * si.re - wi * si.im);
    xi.im += (ar * pi.im + ai * pi.re) + (wr * si.im + wi * si.re);
    x[i] = xi;
    const cf ri(si.re - (wr * ti.re - wi * ti.im), si.im - (wr * ti.im + wi * ti.re));
    r[i] = ri;
    d[0] += (double)hi.re * ri.re + (double)hi.im * ri.im;
    d[1] += (double)hi.re * ri.im - (double)hi.im * ri.re;
    d[4] += (double)ri.re * ri.re + (double)ri.im * ri.im;
  }
  cta_partials<NRB>(d, part);
  // commit this iteration's scalars before the reduction (only CTA 0 writes them)
  if (blockIdx.x == 0 && t < NRB && sc[t].active) {
    KCol& k = st->col[t];
    k.rho_re = k.rho_new_re;
    k.rho_im = k.rho_new_im;
    k.omega_re = sc[t].b_re;
    k.omega_im = sc[t].b_im;
    if (k.restart) k.rhat2 = k.rnorm2;
  }
  if (blockIdx.x == 0 && t == 0) st->iter++;
  // the residual totals for the next mkf_p (frozen columns contribute zeros and are not read)
  grid_reduce<5 * NRB>(part, gpart, tickets, rtot);
}

__global__ void block_get_kernel(int n, int nrb, int j, const cd* __restrict__ block, cd* col) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) col[i] = block[(size_t)i * nrb + j];
}
__global__ void block_set_kernel(int n, int nrb, int j, const cd* __restrict__ col, cd* block) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) block[(size_t)i * nrb + j] = col[i];
}

// ------------------------------------------------------------------------------------------
// Host side
// ------------------------------------------------------------------------------------------
int multi_vec_grid(int n, int nrb) {
  const long long g = ((long long)n * nrb + kMT - 1) / kMT;
  return (int)std::max<long long>(1, std::min<long long>(g, 1184));
}

constexpr size_t kMRing = (size_t)kStages * kStageBytes;

template <int NRB>
static void set_tc_attrs() {
  AC3D_CUDA(cudaFuncSetAttribute(mseg_dot_tc_kernel<NRB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)tc_dot_smem<NRB>()));
}

template <int NRB, int RPL>
static void set_multi_attrs() {
  AC3D_CUDA(cudaFuncSetAttribute(mseg_dot_kernel<NRB, RPL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMRing));
  AC3D_CUDA(cudaFuncSetAttribute(mseg_gather_kernel<NRB, RPL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)kMRing));
  AC3D_CUDA(cudaFuncSetAttribute(mseg_dot_kernel<NRB, RPL>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  AC3D_CUDA(cudaFuncSetAttribute(mseg_gather_kernel<NRB, RPL>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
}

void prepare_multi_kernels() {
  static std::once_flag once;
  std::call_once(once, [] {
    set_multi_attrs<4, 1>();
    set_multi_attrs<4, 2>();
    set_multi_attrs<8, 1>();
    set_multi_attrs<8, 2>();
    set_multi_attrs<16, 1>();
    set_multi_attrs<16, 2>();
    set_tc_attrs<8>();
    set_tc_attrs<16>();
  });
}

template <int NRB, int RPL>
static void mmv_t(const DevPartition& DP, const DevHMat& H, const MultiBufs& B, const void* x, void* y,
                  const void* dot_a, const void* dot_b, const int* done, cudaStream_t s) {
  const bool tr = B.tr;
  if (tr && !H.nearT.p) throw Error(3, "internal: transposed near field not built");
  SegView v{};
  v.leaf_start = DP.leaf_start.as<int>();
  v.a_seg = tr ? DP.near_seg_t.as<long long>() : DP.near_seg.as<long long>();
  v.a_kptr = tr ? DP.didx_t_ptr.as<int>() : DP.didx_ptr.as<int>();
  v.a_idx = tr ? DP.didx_t.as<int>() : DP.didx.as<int>();
  v.err = H.err.as<int>();
  cf* P = (cf*)B.pbuf;
  cf* T = (cf*)B.tbuf;
  if (DP.na > 0) {
    // dot pass: V segments of the column leaves (forward) or U segments of the row leaves (A^T)
    SegView d = v;
    d.b_seg = tr ? H.seg_f.as<long long>() : H.seg_t.as<long long>();
    d.b_kptr = tr ? H.kseg_f.as<int>() : H.kseg_t.as<int>();
    d.order = tr ? H.order_rows.as<int>() : H.order_cols.as<int>();
    note_launch();
    bool launched = false;
    if constexpr (NRB >= 8 && RPL == 1) {
      const DevBuf& tcs = tr ? H.tcseg_f : H.tcseg_t;
      if (B.tc && tcs.p) {
        mseg_dot_tc_kernel<NRB><<<DP.nleaf, kMT, tc_dot_smem<NRB>(), s>>>(
            d, tcs.as<unsigned char>(), (tr ? H.tcoff_f : H.tcoff_t).as<long long>(), (const cf*)x, P, done);
        launched = true;
      }
    }
    if (!launched)
      mseg_dot_kernel<NRB, RPL><<<DP.nleaf, kMT, kMRing, s>>>(d, tr ? H.useg.as<cf>() : H.vseg.as<cf>(),
                                                               (const cf*)x, P, done);
    AC3D_CUDA(cudaGetLastError());
    note_launch();
    const long long thr = H.task_cap * NRB;
    mseg_reduce_kernel<NRB><<<(int)((thr + 255) / 256), 256, 0, s>>>(
        H.task_b.as<int>(), H.t_off.as<int>(), (int)H.task_cap, H.t_off.as<int>() + DP.na,
        tr ? DP.blk_fw_ptr.as<int>() : DP.blk_tr_ptr.as<int>(), tr ? H.kpos_f.as<int>() : H.kpos_t.as<int>(), P,
        T, done);
    AC3D_CUDA(cudaGetLastError());
  }
  v.b_seg = tr ? H.seg_t.as<long long>() : H.seg_f.as<long long>();
  v.b_kptr = tr ? H.kseg_t.as<int>() : H.kseg_f.as<int>();
  v.b_idx = tr ? H.vidx.as<int>() : H.uidx.as<int>();
  v.order = tr ? H.order_cols.as<int>() : H.order_rows.as<int>();
  const bool dots = dot_a || dot_b;
  note_launch();
  const cf* g_near = tr ? H.nearT.as<cf>() : H.near.as<cf>();
  const cf* g_lr = tr ? H.vseg.as<cf>() : H.useg.as<cf>();
  double* g_part = dots ? B.partials : nullptr;
  double* g_gpart = B.partials + (size_t)std::max(DP.nleaf, 1184) * 5 * NRB;
  mseg_gather_kernel<NRB, RPL><<<DP.nleaf, kMT, kMRing, s>>>(v, g_near, g_lr, T, (const cf*)x, (cf*)y,
                                                              (const cf*)dot_a, (const cf*)dot_b, g_part, g_gpart,
                                                              B.ticket, B.red, done);
  if (DP.nleaf > 1024 * kGroup) throw Error(1, "block solves support at most 32768 leaf clusters");
  AC3D_CUDA(cudaGetLastError());
}

template <int NRB>
static void mmv_rpl(const DevPartition& DP, const DevHMat& H, const MultiBufs& B, const void* x, void* y,
                    const void* dot_a, const void* dot_b, const int* done, cudaStream_t s) {
  if (DP.max_leaf <= 32)
    mmv_t<NRB, 1>(DP, H, B, x, y, dot_a, dot_b, done, s);
  else if (DP.max_leaf <= 64)
    mmv_t<NRB, 2>(DP, H, B, x, y, dot_a, dot_b, done, s);
  else
    throw Error(1, "block solves need leaf clusters of at most 64 elements");
}

// One CTA per near block: block b (m x n, column-major at near_off[b]) transposed to n x m
// column-major at near_off_t[b]. Padding columns of the transposed segments stay zero.
__global__ void near_transpose_kernel(const int4* __restrict__ blocks, const long long* __restrict__ off,
                                      const long long* __restrict__ off_t, const cf* __restrict__ near, cf* nearT) {
  const int b = blockIdx.x;
  const int4 q = blocks[b];
  const int m = q.y - q.x, n = q.w - q.z;
  const cf* src = near + off[b];
  cf* dst = nearT + off_t[b];
  for (int t = threadIdx.x; t < m * n; t += blockDim.x) {
    const int r = t / n, c = t - r * n;
    dst[t] = src[c * m + r];
  }
}

void ensure_near_transposed(const DevPartition& DP, DevHMat& H, cudaStream_t s) {
  if (H.nearT.p) return;
  if (H.prec == PREC_FP64) throw Error(3, "internal: block matvec needs FP32 storage");
  const size_t bytes = (size_t)std::max<int64_t>(DP.near_total_t, 2) * sizeof(cf);
  H.nearT.alloc(bytes, s);
  AC3D_CUDA(cudaMemsetAsync(H.nearT.p, 0, bytes, s));
  if (DP.nd == 0) return;
  note_launch();
  near_transpose_kernel<<<DP.nd, 256, 0, s>>>(DP.blocks_d.as<int4>(), DP.near_off.as<long long>(),
                                              DP.near_off_t.as<long long>(), H.near.as<cf>(), H.nearT.as<cf>());
  AC3D_CUDA(cudaGetLastError());
}

void build_tc_segments(const DevPartition& DP, DevHMat& H, bool tr, const std::vector<long long>& off,
                       cudaStream_t s) {
  DevBuf& tcs = tr ? H.tcseg_f : H.tcseg_t;
  DevBuf& tco = tr ? H.tcoff_f : H.tcoff_t;
  if (tcs.p) return;
  if (H.prec == PREC_FP64) throw Error(3, "internal: block matvec needs FP32 storage");
  if ((int)off.size() != DP.nleaf + 1) throw Error(3, "internal: split segment offsets");
  tco.alloc(off.size() * sizeof(long long), s);
  // pageable source: the copy is staged before the call returns, so off may go away after it
  AC3D_CUDA(cudaMemcpyAsync(tco.p, off.data(), off.size() * sizeof(long long), cudaMemcpyHostToDevice, s));
  tcs.alloc((size_t)std::max<long long>(off.back(), 16), s);
  if (DP.nleaf == 0) return;
  note_launch();
  tc_split_kernel<<<DP.nleaf, 256, 0, s>>>(tr ? H.useg.as<cf>() : H.vseg.as<cf>(),
                                          (tr ? H.seg_f : H.seg_t).as<long long>(),
                                          (tr ? H.kseg_f : H.kseg_t).as<int>(), DP.leaf_start.as<int>(),
                                          tco.as<long long>(), tcs.as<unsigned char>());
  AC3D_CUDA(cudaGetLastError());
}

long long tc_segment_bytes(int R, int K) { return tc_leaf_bytes(R, K); }


void launch_mmatvec(const DevPartition& DP, const DevHMat& H, const MultiBufs& B, const void* x, void* y,
                    const void* dot_a, const void* dot_b, const int* done, cudaStream_t s) {
  if (H.prec == PREC_FP64) throw Error(3, "internal: block matvec needs FP32 storage");
  switch (B.nrb) {
    case 4: mmv_rpl<4>(DP, H, B, x, y, dot_a, dot_b, done, s); break;
    case 8: mmv_rpl<8>(DP, H, B, x, y, dot_a, dot_b, done, s); break;
    case 16: mmv_rpl<16>(DP, H, B, x, y, dot_a, dot_b, done, s); break;
    default: throw Error(3, "internal: block width must be 4, 8 or 16");
  }
}

// Partial buffers: matvec partials (max(nleaf, 1184) CTAs) then its group totals (1024 groups);
// vector partials (1184 CTAs), their group totals (64 groups), then the residual totals. Tickets:
// 1024 for the matvec groups, then 64 for the vector groups.
static double* vtotals(const MultiBufs& B, int nrb) {
  return B.vpartials + (size_t)(1184 + 64) * 5 * nrb;
}

template <int NRB>
static void mk_init_t(const MultiBufs& B, int maxit, cudaStream_t s) {
  const int G = multi_vec_grid(B.n, NRB);
  note_launch();
  mk_init<NRB><<<G, kMT, 0, s>>>(B.n, (const cf*)B.b, (cf*)B.x, (cf*)B.r, (cf*)B.rhat, (cf*)B.p, (cf*)B.v,
                                 B.vpartials);
  AC3D_CUDA(cudaGetLastError());
  note_launch();
  mk_scalar_init<NRB><<<1, 32, 0, s>>>(B.state, B.vpartials, G, B.tol, maxit, vtotals(B, NRB));
  AC3D_CUDA(cudaGetLastError());
}

void mkrylov_enqueue_init(const MultiBufs& B, int maxit, cudaStream_t s) {
  switch (B.nrb) {
    case 4: mk_init_t<4>(B, maxit, s); break;
    case 8: mk_init_t<8>(B, maxit, s); break;
    default: mk_init_t<16>(B, maxit, s); break;
  }
}

template <int NRB>
static void mk_iter_t(const MultiBufs& B, const DevPartition& DP, const DevHMat& H, cudaStream_t s) {
  const int n = B.n, G = multi_vec_grid(n, NRB);
  KStateM* st = B.state;
  const int* done = &st->done_all;
  double* vpart = B.vpartials;
  double* vgpart = B.vpartials + (size_t)1184 * 5 * NRB;
  double* vtot = vtotals(B, NRB);
  unsigned* vtick = B.ticket + 1024;
  note_launch();
  mkf_p<NRB><<<G, kMT, 0, s>>>(st, vtot, n, (const cf*)B.r, (cf*)B.p, (cf*)B.v, (cf*)B.rhat);
  launch_mmatvec(DP, H, B, B.p, B.v, B.rhat, nullptr, done, s);
  note_launch();
  mkf_s<NRB><<<G, kMT, 0, s>>>(st, B.red, n, (const cf*)B.r, (const cf*)B.v, (cf*)B.s);
  launch_mmatvec(DP, H, B, B.s, B.t, nullptr, B.s, done, s);
  note_launch();
  mkf_xr<NRB><<<G, kMT, 0, s>>>(st, B.red, n, (cf*)B.x, (const cf*)B.p, (const cf*)B.s, (cf*)B.r,
                                (const cf*)B.t, (const cf*)B.rhat, vpart, vgpart, vtick, vtot);
  AC3D_CUDA(cudaGetLastError());
}

void mkrylov_enqueue_iterations(const MultiBufs& B, const DevPartition& DP, const DevHMat& H, int count,
                                cudaStream_t s) {
  for (int i = 0; i < count; i++) {
    switch (B.nrb) {
      case 4: mk_iter_t<4>(B, DP, H, s); break;
      case 8: mk_iter_t<8>(B, DP, H, s); break;
      default: mk_iter_t<16>(B, DP, H, s); break;
    }
  }
}

void launch_block_get(int n, int nrb, int j, const void* block, void* col, cudaStream_t s) {
  note_launch();
  block_get_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, nrb, j, (const cd*)block, (cd*)col);
  AC3D_CUDA(cudaGetLastError());
}
void launch_block_set(int n, int nrb, int j, const void* col, void* block, cudaStream_t s) {
  note_launch();
  block_set_kernel<<<(n + 255) / 256, 256, 0, s>>>(n, nrb, j, (const cd*)col, (cd*)block);
  AC3D_CUDA(cudaGetLastError());
}

}  // namespace ac3d
