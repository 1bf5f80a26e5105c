// H-matrix matvec y = op(K - I/2) x (generic_product_impl::scaleAndAddTo, hmatrix.h:84-139),
// op = identity or the plain (non-conjugate) transpose.
//
// Two kernels, no atomics, fixed summation order:
//   phase 1: one warp per rank-1 term (b, q): t[b, q] = v_{b,q} . x[cols(b)]  (forward) or
//            u_{b,q} . x[rows(b)] (transpose). Term vectors are contiguous in the pool.
//   gather : one CTA per leaf cluster. Forward: rows of the leaf accumulate their near blocks
//            (column-major, lane = row, coalesced) and the leaf's slice of every admissible block
//            covering it (u_{b,q}[slice] t[b,q]); transpose: columns of the leaf accumulate the
//            transposed near blocks and slices v_{b,q}[slice] t[b,q]. Then y = -x/2 + sum, or
//            y = b - (that) for refinement residuals, with optional fused FP64 dot partials.
#include "common.cuh"
#include "internal.h"

namespace ac3d {

namespace {
constexpr int kGatherThreads = 256;
constexpr int kGatherWarps = kGatherThreads / 32;
}  // namespace

struct MvView {
  const int4* blocks_a;
  const int4* blocks_d;
  const int* rank;
  const int* t_off;
  const long long* term_off;
  const long long* near_off;
  const int* task_b;
  const long long* task_off;
  const int* leaf_start;
  const int* near_ptr;
  const int* near_items;
  const int* lr_ptr;
  const int* lr_items;
  int na, nleaf, maxk;
};

// acc (ar, ai) += a * x with the product formed in the accumulator precision
template <typename AT, typename A, typename X>
__device__ __forceinline__ void cmac(AT& ar, AT& ai, const A& a, const X& x) {
  ar = fma((AT)a.re, (AT)x.re, ar);
  ar = fma(-(AT)a.im, (AT)x.im, ar);
  ai = fma((AT)a.re, (AT)x.im, ai);
  ai = fma((AT)a.im, (AT)x.re, ai);
}

template <typename MT, typename VT, typename AT>
__global__ void __launch_bounds__(256) mv_phase1(MvView V, const cplx<MT>* __restrict__ pool,
                                                 const cplx<VT>* __restrict__ x, cplx<AT>* __restrict__ tvec,
                                                 int transposed, const int* __restrict__ done) {
  if (done && *done) return;
  const int total = V.t_off[V.na];
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int task = gw; task < total; task += nw) {
    const int b = V.task_b[task];
    const cplx<MT>* vec = pool + V.task_off[task];
    const int4 blk = V.blocks_a[b];
    const int m = blk.y - blk.x, n = blk.w - blk.z;
    const cplx<VT>* xs;
    int len;
    if (!transposed) {
      vec += m;
      xs = x + blk.z;
      len = n;
    } else {
      xs = x + blk.x;
      len = m;
    }
    AT ar = 0, ai = 0, br = 0, bi = 0;
    int i = lane;
    for (; i + 96 < len; i += 128) {
      cplx<MT> a0 = vec[i], a1 = vec[i + 32], a2 = vec[i + 64], a3 = vec[i + 96];
      cplx<VT> x0 = xs[i], x1 = xs[i + 32], x2 = xs[i + 64], x3 = xs[i + 96];
      cmac<AT>(ar, ai, a0, x0);
      cmac<AT>(br, bi, a1, x1);
      cmac<AT>(ar, ai, a2, x2);
      cmac<AT>(br, bi, a3, x3);
    }
    for (; i < len; i += 32) cmac<AT>(ar, ai, vec[i], xs[i]);
    ar = warp_sum(ar + br);
    ai = warp_sum(ai + bi);
    if (lane == 0) tvec[task] = cplx<AT>(ar, ai);
  }
}

template <typename MT, typename VT, typename AT, bool TRANS>
__global__ void __launch_bounds__(kGatherThreads) mv_gather(MvView V, const cplx<MT>* __restrict__ near,
                                                            const cplx<MT>* __restrict__ pool,
                                                            const cplx<AT>* __restrict__ tvec,
                                                            const cplx<VT>* __restrict__ x, cplx<VT>* __restrict__ y,
                                                            const cplx<VT>* __restrict__ bminus,
                                                            const cplx<VT>* __restrict__ dot_a,
                                                            const cplx<VT>* __restrict__ dot_b, double* partials,
                                                            const int* __restrict__ done) {
  __shared__ cplx<AT> part[kGatherWarps][32 * kGatherWarps];
  __shared__ double sdot[kGatherWarps][5];
  if (done && *done) return;
  const int leaf = blockIdx.x;
  const int ls = V.leaf_start[leaf], le = V.leaf_start[leaf + 1];
  const int R = le - ls;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nrw = (R + 31) >> 5;           // warps needed to cover the leaf's rows
  const int groups = kGatherWarps / nrw;   // independent groups splitting the work list
  const int g = warp / nrw;
  const int row = (warp - g * nrw) * 32 + lane;
  const bool active = g < groups && row < R;

  AT accr = 0, acci = 0;
  if (g < groups) {
    // dense near blocks
    for (int it = V.near_ptr[leaf] + g; it < V.near_ptr[leaf + 1]; it += groups) {
      const int b = V.near_items[it];
      const int4 blk = V.blocks_d[b];
      const cplx<MT>* D = near + V.near_off[b];
      if (!TRANS) {
        const int n = blk.w - blk.z;
        const cplx<VT>* xs = x + blk.z;
        if (active) {
          int c = 0;
          AT br = 0, bi = 0;
          const cplx<MT>* Dr = D + row;
          for (; c + 3 < n; c += 4) {
            cplx<MT> d0 = Dr[(size_t)c * R], d1 = Dr[(size_t)(c + 1) * R], d2 = Dr[(size_t)(c + 2) * R],
                     d3 = Dr[(size_t)(c + 3) * R];
            cmac<AT>(accr, acci, d0, xs[c]);
            cmac<AT>(br, bi, d1, xs[c + 1]);
            cmac<AT>(accr, acci, d2, xs[c + 2]);
            cmac<AT>(br, bi, d3, xs[c + 3]);
          }
          for (; c < n; c++) cmac<AT>(accr, acci, Dr[(size_t)c * R], xs[c]);
          accr += br;
          acci += bi;
        }
      } else {
        const int m = blk.y - blk.x;
        const cplx<VT>* xs = x + blk.x;
        if (active) {
          const cplx<MT>* Dc = D + (size_t)row * m;  // column `row` of the block
          for (int r = 0; r < m; r++) {
            cplx<MT> d0 = Dc[r];
            cplx<VT> x0 = xs[r];
            accr = fma((AT)d0.re, (AT)x0.re, accr);
            accr = fma(-(AT)d0.im, (AT)x0.im, accr);
            acci = fma((AT)d0.re, (AT)x0.im, acci);
            acci = fma((AT)d0.im, (AT)x0.re, acci);
          }
        }
      }
    }
    // low-rank slices
    for (int it = V.lr_ptr[leaf] + g; it < V.lr_ptr[leaf + 1]; it += groups) {
      const int b = V.lr_items[it];
      const int4 blk = V.blocks_a[b];
      const int rk = V.rank[b];
      const cplx<AT>* tb = tvec + V.t_off[b];
      const int off = TRANS ? (blk.y - blk.x) + (ls - blk.z) : (ls - blk.x);
      if (active) {
        const long long* tob = V.task_off + V.t_off[b];
        const cplx<MT>* base = pool + off + row;
        int q = 0;
        AT br = 0, bi = 0;
        for (; q + 3 < rk; q += 4) {
          const long long o0 = tob[q], o1 = tob[q + 1], o2 = tob[q + 2], o3 = tob[q + 3];
          cplx<MT> u0 = base[o0], u1 = base[o1], u2 = base[o2], u3 = base[o3];
          cmac<AT>(accr, acci, u0, tb[q]);
          cmac<AT>(br, bi, u1, tb[q + 1]);
          cmac<AT>(accr, acci, u2, tb[q + 2]);
          cmac<AT>(br, bi, u3, tb[q + 3]);
        }
        for (; q < rk; q++) cmac<AT>(accr, acci, base[tob[q]], tb[q]);
        accr += br;
        acci += bi;
      }
    }
    part[g][row] = cplx<AT>(accr, acci);
  }
  __syncthreads();

  // combine groups in fixed order and apply the -x/2 jump term
  double d[5] = {0, 0, 0, 0, 0};
  if (threadIdx.x < R) {
    const int r = threadIdx.x;
    AT sr = 0, si = 0;
    for (int gg = 0; gg < groups; gg++) {
      sr += part[gg][r].re;
      si += part[gg][r].im;
    }
    cplx<VT> xv = x[ls + r];
    AT yr = sr - AT(0.5) * (AT)xv.re;
    AT yi = si - AT(0.5) * (AT)xv.im;
    if (bminus) {
      cplx<VT> bv = bminus[ls + r];
      yr = (AT)bv.re - yr;
      yi = (AT)bv.im - yi;
    }
    cplx<VT> out((VT)yr, (VT)yi);
    y[ls + r] = out;
    const double oyr = (double)out.re, oyi = (double)out.im;
    if (dot_a) {  // conj(a) . y
      cplx<VT> a = dot_a[ls + r];
      d[0] = (double)a.re * oyr + (double)a.im * oyi;
      d[1] = (double)a.re * oyi - (double)a.im * oyr;
    }
    if (dot_b) {  // conj(y) . b
      cplx<VT> bb = dot_b[ls + r];
      d[2] = oyr * (double)bb.re + oyi * (double)bb.im;
      d[3] = oyr * (double)bb.im - oyi * (double)bb.re;
    }
    d[4] = oyr * oyr + oyi * oyi;
  }
  if (partials) {
    for (int i = 0; i < 5; i++) d[i] = warp_sum(d[i]);
    if (lane == 0)
      for (int i = 0; i < 5; i++) sdot[warp][i] = d[i];
    __syncthreads();
    if (threadIdx.x < 5) {
      double s = 0;
      for (int w = 0; w < kGatherWarps; w++) s += sdot[w][threadIdx.x];
      partials[(size_t)leaf * 5 + threadIdx.x] = s;
    }
  }
}

static MvView mv_view(const DevPartition& DP, const DevHMat& H, bool tr) {
  MvView v;
  v.blocks_a = DP.blocks_a.as<int4>();
  v.blocks_d = DP.blocks_d.as<int4>();
  v.rank = H.rank.as<int>();
  v.t_off = H.t_off.as<int>();
  v.term_off = H.term_off.as<long long>();
  v.near_off = DP.near_off.as<long long>();
  v.task_b = H.task_b.as<int>();
  v.task_off = H.task_off.as<long long>();
  v.leaf_start = DP.leaf_start.as<int>();
  v.near_ptr = tr ? DP.tr_near_ptr.as<int>() : DP.fw_near_ptr.as<int>();
  v.near_items = tr ? DP.tr_near.as<int>() : DP.fw_near.as<int>();
  v.lr_ptr = tr ? DP.tr_lr_ptr.as<int>() : DP.fw_lr_ptr.as<int>();
  v.lr_items = tr ? DP.tr_lr.as<int>() : DP.fw_lr.as<int>();
  v.na = DP.na;
  v.nleaf = DP.nleaf;
  v.maxk = H.maxk;
  return v;
}

static int g_sms = 0;
int device_sm_count() {
  if (!g_sms) {
    int dev = 0;
    AC3D_CUDA(cudaGetDevice(&dev));
    AC3D_CUDA(cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev));
  }
  return g_sms;
}

template <typename MT, typename VT, typename AT>
static void mv_t(const DevPartition& DP, const DevHMat& H, bool tr, const void* x, void* y, const void* bminus,
                 const MatvecEpilogue& ep, const int* done, void* tvec, cudaStream_t s) {
  MvView v = mv_view(DP, H, tr);
  if (DP.na > 0) {
    note_launch();
    mv_phase1<MT, VT, AT><<<device_sm_count() * 4, 256, 0, s>>>(v, H.pool.as<cplx<MT>>(), (const cplx<VT>*)x,
                                                        (cplx<AT>*)tvec, tr ? 1 : 0, done);
    AC3D_CUDA(cudaGetLastError());
  }
  note_launch();
  if (tr)
    mv_gather<MT, VT, AT, true><<<DP.nleaf, kGatherThreads, 0, s>>>(
        v, H.near.as<cplx<MT>>(), H.pool.as<cplx<MT>>(), (const cplx<AT>*)tvec, (const cplx<VT>*)x, (cplx<VT>*)y,
        (const cplx<VT>*)bminus, (const cplx<VT>*)ep.dot_a, (const cplx<VT>*)ep.dot_b, ep.partials, done);
  else
    mv_gather<MT, VT, AT, false><<<DP.nleaf, kGatherThreads, 0, s>>>(
        v, H.near.as<cplx<MT>>(), H.pool.as<cplx<MT>>(), (const cplx<AT>*)tvec, (const cplx<VT>*)x, (cplx<VT>*)y,
        (const cplx<VT>*)bminus, (const cplx<VT>*)ep.dot_a, (const cplx<VT>*)ep.dot_b, ep.partials, done);
  AC3D_CUDA(cudaGetLastError());
}

void launch_matvec_ex(const DevPartition& DP, const DevHMat& H, bool transposed, int vec64, const void* x, void* y,
                      const void* b_minus, const MatvecEpilogue& ep, const int* done, cudaStream_t s) {
  if (H.prec == PREC_FP64) {
    if (!vec64) throw Error(3, "internal: FP64 H-matrix needs FP64 vectors");
    mv_t<double, double, double>(DP, H, transposed, x, y, b_minus, ep, done, H.tvec64.p, s);
  } else if (vec64) {
    mv_t<float, double, double>(DP, H, transposed, x, y, b_minus, ep, done, H.tvec64.p, s);
  } else {
    mv_t<float, float, float>(DP, H, transposed, x, y, b_minus, ep, done, H.tvec.p, s);
  }
}

void launch_matvec(const DevPartition& DP, const DevHMat& H, int ne, bool transposed, int vec64, const void* x,
                   void* y, const void* b_minus, const MatvecEpilogue& ep, cudaStream_t s) {
  (void)ne;
  launch_matvec_ex(DP, H, transposed, vec64, x, y, b_minus, ep, nullptr, s);
}

int matvec_grid(const DevPartition& DP, bool) { return DP.nleaf; }

}  // namespace ac3d
