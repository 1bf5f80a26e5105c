// Bulk-async streaming of contiguous segments through shared memory (sm_90+ PTX: mbarrier and
// cp.async.bulk). One thread issues copies of whole column chunks of an R x K column-major
// segment into a ring of stages; all warps consume the stages in order. Every wait is bounded:
// after kSpinLimit polls the kernel records an error code and stops using the pipeline.
#pragma once

#include <stdint.h>

#include "common.cuh"

namespace ac3d {

// Ring shape (stages x bytes); the defaults were chosen by measurement on GB300.
#ifndef AC3D_RING_STAGES
#define AC3D_RING_STAGES 3
#endif
#ifndef AC3D_STAGE_BYTES
#define AC3D_STAGE_BYTES 16384
#endif
constexpr int kStages = AC3D_RING_STAGES;
constexpr int kStageBytes = AC3D_STAGE_BYTES;  // bytes per stage (multiple of 16)
constexpr uint32_t kSpinLimit = 1u << 26; // polls before a wait is declared failed

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// dst (shared) and src (global) 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// Plain arrival (release semantics at CTA scope) on an mbarrier.
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Per-thread asynchronous gather of one 8- or 16-byte element into shared memory (src aligned to
// its size). Completion is reported to an mbarrier by cp_async_arrive_noinc.
template <int BYTES>
__device__ __forceinline__ void cp_async_elem(void* dst, const void* src) {
  static_assert(BYTES == 8 || BYTES == 16, "8 or 16 bytes");
  if constexpr (BYTES == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
  else
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}

// One arrival on the mbarrier once every cp.async this thread issued before has landed (the
// arrival counts against the barrier's expected count: no increment).
__device__ __forceinline__ void cp_async_arrive_noinc(uint64_t* bar) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Bounded wait on a phase of an mbarrier; false if it did not complete within kSpinLimit polls.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  for (uint32_t i = 0; i < kSpinLimit; i++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// CTA-wide bounded wait: thread 0 polls the mbarrier while the other threads wait at the CTA
// barrier, which costs them no issue slots; every thread gets the same verdict. The barrier
// orders what the completed phase covers (bulk copies, cp.async arrivals, MMA completion) before
// every thread's later accesses.
__device__ __forceinline__ bool cta_wait(uint64_t* bar, uint32_t parity) {
  bool got = true;
  if (threadIdx.x == 0) got = mbar_wait_bounded(bar, parity);
  return !__syncthreads_or(!got);
}

// ------------------------------------------------------------------------------------------
// Per-leaf segment views and the copy ring shared by the matvec passes
// ------------------------------------------------------------------------------------------
struct SegView {
  const int* leaf_start;
  const int* order;  // CTA -> leaf, leaves by decreasing work
  // region A: near segments (forward gather only)
  const long long* a_seg;
  const int* a_kptr;
  const int* a_idx;
  // region B: low-rank segments
  const long long* b_seg;
  const int* b_kptr;
  const int* b_idx;
  // transposed dense blocks
  const int4* blocks_d;
  const long long* near_off;
  const int* trn_ptr;
  const int* trn;
  int* err;
};

// Iterates the chunks of the (up to two) regions of one leaf through the copy ring and calls
// fn(stage_ptr, region, first_column, columns, next_region, next_first_column, next_columns) for
// each chunk, all threads together (next_columns = 0 after the last chunk), so that the callback
// can prefetch what the next chunk needs while it computes this one. pre() runs on all threads
// once the first stages are in flight and before any is consumed; it returns the same value on
// every thread, false to stop (the copies in flight land before the return).
template <typename MT, typename P, typename F>
__device__ __forceinline__ bool stream_leaf(unsigned char (*stage)[kStageBytes], uint64_t* full, int R,
                                            const cplx<MT>* a_ptr, int a_cols, const cplx<MT>* b_ptr, int b_cols,
                                            int* err, P&& pre, F&& fn) {
  const int cpc = max(2, (int)(kStageBytes / sizeof(cplx<MT>)) / R & ~1);  // columns per chunk, even
  const int na = (a_cols + cpc - 1) / cpc, nb = (b_cols + cpc - 1) / cpc;
  const int nch = na + nb;
  auto chunk = [&](int c, const cplx<MT>*& src, int& region, int& c0, int& ncols) {
    if (c < na) {
      region = 0;
      c0 = c * cpc;
      ncols = min(cpc, a_cols - c0);
      src = a_ptr + (long long)c0 * R;
    } else {
      region = 1;
      c0 = (c - na) * cpc;
      ncols = min(cpc, b_cols - c0);
      src = b_ptr + (long long)c0 * R;
    }
  };
  if (threadIdx.x == 0) {
    for (int c = 0; c < min(nch, kStages); c++) {
      const cplx<MT>* src;
      int region, c0, ncols;
      chunk(c, src, region, c0, ncols);
      const uint32_t bytes = (uint32_t)(ncols * R * sizeof(cplx<MT>));
      mbar_expect_tx(&full[c], bytes);
      bulk_copy_g2s(stage[c], src, bytes, &full[c]);
    }
  }
  if (!pre()) {
    if (threadIdx.x == 0)
      for (int c = 0; c < min(nch, kStages); c++) mbar_wait_bounded(&full[c], 0u);
    __syncthreads();
    return true;
  }
  bool ok = true;
  int c = 0;
  for (; c < nch; c++) {
    const int s = c % kStages;
    const uint32_t parity = (uint32_t)(c / kStages) & 1u;
    if (!cta_wait(&full[s], parity)) {
      ok = false;
      break;
    }
    const cplx<MT>* src;
    int region, c0, ncols;
    chunk(c, src, region, c0, ncols);
    int nregion = 0, nc0 = 0, nncols = 0;
    if (c + 1 < nch) {
      const cplx<MT>* nsrc;
      chunk(c + 1, nsrc, nregion, nc0, nncols);
    }
    fn((const cplx<MT>*)stage[s], region, c0, ncols, nregion, nc0, nncols);
    __syncthreads();  // every warp is done with stage s
    if (threadIdx.x == 0 && c + kStages < nch) {
      fence_proxy_async();
      const cplx<MT>* src2;
      int region2, c02, ncols2;
      chunk(c + kStages, src2, region2, c02, ncols2);
      const uint32_t bytes = (uint32_t)(ncols2 * R * sizeof(cplx<MT>));
      mbar_expect_tx(&full[s], bytes);
      bulk_copy_g2s(stage[s], src2, bytes, &full[s]);
    }
  }
  if (!ok) {
    // record the failure and let the copies already issued land before the CTA exits
    if (threadIdx.x == 0) {
      atomicExch(err, 1);
      for (int cc = c; cc < min(nch, c + kStages); cc++)
        mbar_wait_bounded(&full[cc % kStages], (uint32_t)(cc / kStages) & 1u);
    }
    __syncthreads();
  }
  return ok;
}

template <typename MT, typename F>
__device__ __forceinline__ bool stream_leaf(unsigned char (*stage)[kStageBytes], uint64_t* full, int R,
                                            const cplx<MT>* a_ptr, int a_cols, const cplx<MT>* b_ptr, int b_cols,
                                            int* err, F&& fn) {
  return stream_leaf<MT>(stage, full, R, a_ptr, a_cols, b_ptr, b_cols, err, [] { return true; }, fn);
}

__device__ __forceinline__ void init_ring(uint64_t* full) {
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; s++) mbar_init(&full[s], 1);
    fence_barrier_init();
  }
  __syncthreads();
}

}  // namespace ac3d
