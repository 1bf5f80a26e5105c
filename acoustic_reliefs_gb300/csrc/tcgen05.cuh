// Blackwell 5th-generation tensor-core primitives (sm_100 family PTX: tcgen05.*), used by the
// block matvec. One thread of a CTA issues tcgen05.mma with both operands in shared memory and the
// FP32 accumulator in tensor memory (TMEM); tcgen05.commit reports completion on an mbarrier, and
// warps read the accumulator back with tcgen05.ld. Operands are TF32 (K-major, no swizzle); a
// value x is split as x = hi + lo with hi = tf32(x), lo = tf32(x - hi), and a product is formed as
// hi_a hi_b + hi_a lo_b + lo_a hi_b (three MMAs), which keeps FP32-level accuracy.
#pragma once

#include <stdint.h>

#include "segstream.cuh"

namespace ac3d {

// Canonical K-major layout without swizzle: 8-row x 16-byte core matrices (8 rows x 4 TF32).
// Within a core matrix row r is at r * 16 bytes; core matrices along K are `lbo` bytes apart and
// 8-row groups `sbo` bytes apart.
__device__ __forceinline__ uint64_t umma_smem_desc(const void* base, uint32_t lbo, uint32_t sbo) {
  const uint32_t a = smem_u32(base);
  uint64_t d = 0;
  d |= (uint64_t)((a >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version for sm_100
  // base offset 0, relative LBO mode, layout type 0 (no swizzle)
  return d;
}

// Instruction descriptor of tcgen05.mma.kind::tf32: D FP32, A and B TF32, both K-major, M x N.
__host__ __device__ constexpr uint32_t umma_idesc_tf32(int M, int N) {
  return (1u << 4)                       // D format: F32
         | (2u << 7)                     // A format: TF32
         | (2u << 10)                    // B format: TF32
         | ((uint32_t)(N >> 3) << 17)    // N / 8
         | ((uint32_t)(M >> 4) << 24);   // M / 16
}

__device__ __forceinline__ uint32_t to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// x = hi + lo, both TF32 values (as floats)
__device__ __forceinline__ void split_tf32(float x, float& hi, float& lo) {
  hi = __uint_as_float(to_tf32(x));
  lo = __uint_as_float(to_tf32(x - hi));
}

// TMEM allocation of `ncols` columns (power of two, 32..512) by one whole warp; the address is
// written to shared memory at `dst`.
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
               "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// D[tmem] (+)= A[smem] B[smem]; accumulate = 0 overwrites D.
__device__ __forceinline__ void umma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "setp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n"
      "}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Arrive once on the mbarrier when every MMA this thread issued before has completed.
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

// 32 consecutive accumulator columns of this thread's TMEM lane (warp w of a warpgroup reads
// lanes 32 w .. 32 w + 31; taddr carries the lane in bits 16..31 and the column in 0..15).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// Offset in floats of element (row, k) in a K-major, no-swizzle tile with `kdim` K values
// (a multiple of 4): core matrix (row / 8, k / 4) of 128 bytes; core matrices along K are
// adjacent (128 bytes apart), 8-row groups kdim / 4 core matrices apart.
__device__ __forceinline__ int kmajor_off(int row, int k, int kdim) {
  return ((row >> 3) * (kdim >> 2) + (k >> 2)) * 32 + (row & 7) * 4 + (k & 3);
}

}  // namespace ac3d
