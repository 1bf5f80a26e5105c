// Repacking of the ACA pool into the per-leaf segments the matvec streams.
//
// ACA writes every rank-1 term (u | v) into its own pool slot, in the order blocks finish. The
// matvec streams, per leaf cluster, one contiguous R x K column-major segment:
//   U segment of row leaf L    : u_{b,q}[rows of L] for every admissible block b whose rows
//                                contain L (list fw_lr), q < rank(b);
//   V segment of column leaf L : v_{b,q}[columns of L] for every b whose columns contain L (tr_lr).
// K is padded to an even count so that every segment starts and ends on a 16-byte boundary (the
// bulk-copy rule); padding columns are zero with index -1. For each list entry e (leaf, block)
// kpos[e] is the segment column of the block's first term, which the reduce step of the matvec
// uses to sum a term's per-leaf partial dots. Offsets are prefix sums over the ranks computed on
// the device in a fixed order, so packing is deterministic. The pool itself is not needed after.
#include "common.cuh"
#include "df64.cuh"
#include "internal.h"

namespace ac3d {

// Per leaf: K = sum of the ranks of its list, padded to even, into kseg[l] (a warp per leaf, the
// ranks summed by lanes; integer sums, so the order does not matter).
__global__ void leaf_k_kernel(const int* __restrict__ rank, const int* __restrict__ ptr,
                              const int* __restrict__ items, int nleaf, int* kseg) {
  const int l = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (l >= nleaf) return;
  int K = 0;
  for (int it = ptr[l] + lane; it < ptr[l + 1]; it += 32) K += rank[items[it]];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) K += __shfl_xor_sync(0xffffffffu, K, o);
  if (lane == 0) kseg[l] = K + (K & 1);
}

// kseg[l] (holding K of leaf l) becomes the prefix of K, seg[l] the prefix of R K (one CTA).
__global__ void leaf_scan_kernel(const int* __restrict__ leaf_start, int nleaf, int* kseg, long long* seg) {
  __shared__ long long sk[1024], ss[1024];
  const int tid = threadIdx.x;
  const int chunk = (nleaf + 1023) / 1024;
  const int s = min(nleaf, tid * chunk), e = min(nleaf, s + chunk);
  long long ak = 0, as = 0;
  for (int l = s; l < e; l++) {
    const int K = kseg[l];
    ak += K;
    as += (long long)K * (leaf_start[l + 1] - leaf_start[l]);
  }
  sk[tid] = ak;
  ss[tid] = as;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    long long vk = tid >= o ? sk[tid - o] : 0, vs = tid >= o ? ss[tid - o] : 0;
    __syncthreads();
    sk[tid] += vk;
    ss[tid] += vs;
    __syncthreads();
  }
  long long bk = tid ? sk[tid - 1] : 0, bs = tid ? ss[tid - 1] : 0;
  for (int l = s; l < e; l++) {
    const int K = kseg[l];  // this thread's own leaf, read before it is overwritten
    kseg[l] = (int)bk;
    seg[l] = bs;
    bk += K;
    bs += (long long)K * (leaf_start[l + 1] - leaf_start[l]);
  }
  if (tid == 1023) {
    kseg[nleaf] = (int)sk[1023];
    seg[nleaf] = ss[1023];
  }
}

// Stored value of a pool entry: the entry itself, or the FP32 rounding (the leading part) of a
// double-float term of the mixed-precision assembly.
template <typename R>
__device__ __forceinline__ cplx<R> seg_value(const cplx<R>& v) { return v; }
__device__ __forceinline__ cf seg_value(const cdf& v) { return cf(v.re.hi, v.im.hi); }

constexpr int kPackThreads = 256;
constexpr int kPackChunk = 512;  // list entries per round of a leaf's scan

// One CTA per leaf: the first segment column of every listed block (an exclusive scan of the ranks
// in list order, a chunk of the list at a time), then a warp per list entry copies the leaf's
// slice of the block's terms (lanes over the leaf's rows, four terms per round of loads) and
// writes the segment column indices (phase-1 output positions t_off[b] + q) and the entry's first
// column. The list entries' metadata loads and copies run in parallel across the warps; the
// output is the same as copying the list in order.
template <typename P, typename R>
__global__ void __launch_bounds__(kPackThreads) pack_segments_kernel(
    const P* __restrict__ pool, const long long* __restrict__ task_off, const int* __restrict__ t_off,
    const int* __restrict__ rank, const int4* __restrict__ blocks, const int* __restrict__ leaf_start,
    const int* __restrict__ ptr, const int* __restrict__ items, int cols, const int* __restrict__ kseg,
    const long long* __restrict__ seg, cplx<R>* S, int* sidx, const int* __restrict__ pos, int* kpos) {
  __shared__ int sb[kPackChunk], sr[kPackChunk], sbase[kPackChunk];
  __shared__ int wsum[kPackThreads / 32];
  __shared__ int s_total;
  const int l = blockIdx.x;
  const int ls = leaf_start[l], Rn = leaf_start[l + 1] - ls;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  cplx<R>* dst = S + seg[l];
  int* idx = sidx + kseg[l];
  const int it0 = ptr[l], nit = ptr[l + 1] - it0;
  int base = 0;  // segment columns of the entries before this chunk
  for (int c0 = 0; c0 < nit; c0 += kPackChunk) {
    const int cn = min(kPackChunk, nit - c0);
    for (int i = threadIdx.x; i < kPackChunk; i += kPackThreads) {
      const int b = i < cn ? items[it0 + c0 + i] : 0;
      sb[i] = b;
      sr[i] = i < cn ? rank[b] : 0;
    }
    __syncthreads();
    // exclusive scan of sr: each thread two consecutive entries, warp scan, then the warp totals
    const int a0 = sr[2 * threadIdx.x], a1 = sr[2 * threadIdx.x + 1];
    int v = a0 + a1;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int t = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += t;
    }
    if (lane == 31) wsum[warp] = v;
    __syncthreads();
    int wb = 0;
    for (int w = 0; w < warp; w++) wb += wsum[w];
    const int excl = base + wb + v - (a0 + a1);
    sbase[2 * threadIdx.x] = excl;
    sbase[2 * threadIdx.x + 1] = excl + a0;
    if (threadIdx.x == kPackThreads - 1) s_total = wb + v;
    __syncthreads();
    for (int i = warp; i < cn; i += kPackThreads / 32) {
      const int b = sb[i], r = sr[i], kb = sbase[i];
      const int4 q4 = blocks[b];
      const int off = cols ? (q4.y - q4.x) + (ls - q4.z) : (ls - q4.x);
      const long long* to = task_off + t_off[b];
      for (int q0 = 0; q0 < r; q0 += 4) {  // four terms per round of loads
        long long src[4];
#pragma unroll
        for (int u = 0; u < 4; u++) src[u] = q0 + u < r ? to[q0 + u] + off : -1;
        for (int row = lane; row < Rn; row += 32) {
          P val[4];
#pragma unroll
          for (int u = 0; u < 4; u++) val[u] = pool[(src[u] >= 0 ? src[u] : src[0]) + row];
#pragma unroll
          for (int u = 0; u < 4; u++)
            if (src[u] >= 0) dst[(long long)(kb + q0 + u) * Rn + row] = seg_value(val[u]);
        }
      }
      for (int q = lane; q < r; q += 32) idx[kb + q] = t_off[b] + q;
      if (lane == 0) kpos[pos[it0 + c0 + i]] = kseg[l] + kb;  // block-major order
    }
    base += s_total;
    __syncthreads();  // the chunk's arrays are free
  }
  if (base & 1) {  // padding column
    for (int row = threadIdx.x; row < Rn; row += kPackThreads) dst[(long long)base * Rn + row] = cplx<R>();
    if (threadIdx.x == 0) idx[base] = -1;
  }
}

template <typename P, typename R>
static void pack_side(const DevPartition& DP, DevHMat& H, bool cols, cudaStream_t s) {
  const int* ptr = cols ? DP.tr_lr_ptr.as<int>() : DP.fw_lr_ptr.as<int>();
  const int* items = cols ? DP.tr_lr.as<int>() : DP.fw_lr.as<int>();
  DevBuf& kseg = cols ? H.kseg_t : H.kseg_f;
  DevBuf& seg = cols ? H.seg_t : H.seg_f;
  DevBuf& S = cols ? H.vseg : H.useg;
  DevBuf& idx = cols ? H.vidx : H.uidx;
  DevBuf& kpos = cols ? H.kpos_t : H.kpos_f;
  note_launch();
  leaf_k_kernel<<<(DP.nleaf + 7) / 8, 256, 0, s>>>(H.rank.as<int>(), ptr, items, DP.nleaf, kseg.as<int>());
  AC3D_CUDA(cudaGetLastError());
  note_launch();
  leaf_scan_kernel<<<1, 1024, 0, s>>>(DP.leaf_start.as<int>(), DP.nleaf, kseg.as<int>(), seg.as<long long>());
  AC3D_CUDA(cudaGetLastError());
  note_launch();
  pack_segments_kernel<P, R><<<DP.nleaf, kPackThreads, 0, s>>>(H.pool.as<P>(), H.task_off.as<long long>(),
                                                   H.t_off.as<int>(), H.rank.as<int>(), DP.blocks_a.as<int4>(),
                                                   DP.leaf_start.as<int>(), ptr, items, cols ? 1 : 0, kseg.as<int>(),
                                                   seg.as<long long>(), S.as<cplx<R>>(), idx.as<int>(),
                                                   cols ? DP.tr_pos.as<int>() : DP.fw_pos.as<int>(), kpos.as<int>());
  AC3D_CUDA(cudaGetLastError());
}

void launch_pack(const DevPartition& DP, DevHMat& H, bool cols, cudaStream_t s) {
  if (DP.na == 0) return;
  if (H.prec == PREC_FP64)
    pack_side<cd, double>(DP, H, cols, s);
  else if (H.pool_df)
    pack_side<cdf, float>(DP, H, cols, s);
  else
    pack_side<cf, float>(DP, H, cols, s);
}

}  // namespace ac3d
