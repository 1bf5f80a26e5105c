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

// Per leaf: K = sum of ranks of its list, padded to even; kseg = prefix of K, seg = prefix of R K.
__global__ void leaf_scan_kernel(const int* __restrict__ rank, const int* __restrict__ leaf_start,
                                 const int* __restrict__ ptr, const int* __restrict__ items, int nleaf, int* kseg,
                                 long long* seg) {
  __shared__ long long sk[1024], ss[1024];
  const int tid = threadIdx.x;
  const int chunk = (nleaf + 1023) / 1024;
  const int s = min(nleaf, tid * chunk), e = min(nleaf, s + chunk);
  auto kleaf = [&](int l) {
    int K = 0;
    for (int it = ptr[l]; it < ptr[l + 1]; it++) K += rank[items[it]];
    return K + (K & 1);
  };
  long long ak = 0, as = 0;
  for (int l = s; l < e; l++) {
    const int K = kleaf(l);
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
    kseg[l] = (int)bk;
    seg[l] = bs;
    const int K = kleaf(l);
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

// One CTA per leaf: copy the leaf's slices of every listed block's terms, write the segment
// column indices (phase-1 output positions t_off[b] + q) and the first column of each entry.
template <typename P, typename R>
__global__ void pack_segments_kernel(const P* __restrict__ pool, const long long* __restrict__ task_off,
                                     const int* __restrict__ t_off, const int* __restrict__ rank,
                                     const int4* __restrict__ blocks, const int* __restrict__ leaf_start,
                                     const int* __restrict__ ptr, const int* __restrict__ items, int cols,
                                     const int* __restrict__ kseg, const long long* __restrict__ seg, cplx<R>* S,
                                     int* sidx, const int* __restrict__ pos, int* kpos) {
  const int l = blockIdx.x;
  const int ls = leaf_start[l], Rn = leaf_start[l + 1] - ls;
  cplx<R>* dst = S + seg[l];
  int* idx = sidx + kseg[l];
  int kbase = 0;
  for (int it = ptr[l]; it < ptr[l + 1]; it++) {
    const int b = items[it];
    const int r = rank[b];
    const int4 q4 = blocks[b];
    const int off = cols ? (q4.y - q4.x) + (ls - q4.z) : (ls - q4.x);
    const long long* to = task_off + t_off[b];
    for (int e = threadIdx.x; e < r * Rn; e += blockDim.x) {
      const int q = e / Rn, row = e - q * Rn;
      dst[(long long)(kbase + q) * Rn + row] = seg_value(pool[to[q] + off + row]);
    }
    for (int q = threadIdx.x; q < r; q += blockDim.x) idx[kbase + q] = t_off[b] + q;
    if (threadIdx.x == 0) kpos[pos[it]] = kseg[l] + kbase;  // block-major order
    kbase += r;
  }
  if (kbase & 1) {  // padding column
    for (int row = threadIdx.x; row < Rn; row += blockDim.x) dst[(long long)kbase * Rn + row] = cplx<R>();
    if (threadIdx.x == 0) idx[kbase] = -1;
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
  leaf_scan_kernel<<<1, 1024, 0, s>>>(H.rank.as<int>(), DP.leaf_start.as<int>(), ptr, items, DP.nleaf,
                                      kseg.as<int>(), seg.as<long long>());
  AC3D_CUDA(cudaGetLastError());
  note_launch();
  pack_segments_kernel<P, R><<<DP.nleaf, 256, 0, s>>>(H.pool.as<P>(), H.task_off.as<long long>(),
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
