// Self-check of the tensor-core product used by the block matvec: one CTA forms
// D (128 x 32) = A (128 x K) B^T (B: 32 x K) with tcgen05.mma (TF32 operands split in three
// products, FP32 accumulator in TMEM), in the operand layouts the block gather pass uses.
#include <cuda_runtime.h>

#include "../../include/ac3d.h"
#include "internal.h"
#include "tcgen05.cuh"

namespace ac3d {

__global__ void __launch_bounds__(128) tc_selftest_kernel(const float* __restrict__ A, const float* __restrict__ B,
                                                          int K, float* __restrict__ D, int* err) {
  extern __shared__ __align__(1024) unsigned char sm[];
  float* Ah = reinterpret_cast<float*>(sm);
  float* Al = Ah + 128 * K;
  float* Bh = Al + 128 * K;
  float* Bl = Bh + 32 * K;
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t s_tmem;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int i = tid; i < 128 * K; i += blockDim.x) {
    const int row = i / K, k = i - row * K;
    float hi, lo;
    split_tf32(A[i], hi, lo);
    Ah[kmajor_off(row, k, K)] = hi;
    Al[kmajor_off(row, k, K)] = lo;
  }
  for (int i = tid; i < 32 * K; i += blockDim.x) {
    const int n = i / K, k = i - n * K;
    float hi, lo;
    split_tf32(B[i], hi, lo);
    Bh[kmajor_off(n, k, K)] = hi;
    Bl[kmajor_off(n, k, K)] = lo;
  }
  if (tid == 0) {
    mbar_init(&bar, 1);
    fence_barrier_init();
  }
  if (warp == 0) {
    tmem_alloc(&s_tmem, 32);
    tmem_relinquish();
  }
  fence_proxy_async();  // the operand stores become visible to the tensor core (async proxy)
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = s_tmem;
  if (tid == 0) {
    const uint32_t idesc = umma_idesc_tf32(128, 32);
    const uint32_t sbo = (uint32_t)(K / 4) * 128u;
    for (int ks = 0; ks < K / 8; ks++) {  // K = 8 per instruction: two core matrices, 256 bytes
      const uint64_t ah = umma_smem_desc(Ah + ks * 64, 128, sbo), al = umma_smem_desc(Al + ks * 64, 128, sbo);
      const uint64_t bh = umma_smem_desc(Bh + ks * 64, 128, sbo), bl = umma_smem_desc(Bl + ks * 64, 128, sbo);
      umma_tf32(tmem, ah, bh, idesc, ks > 0 ? 1u : 0u);
      umma_tf32(tmem, ah, bl, idesc, 1u);
      umma_tf32(tmem, al, bh, idesc, 1u);
    }
    umma_commit(&bar);
  }
  const bool ok = mbar_wait_bounded(&bar, 0);
  if (!ok && tid == 0) atomicExch(err, 1);
  tc_fence_after();
  float v[32];
  tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16), v);
  for (int c = 0; c < 32; c++) D[(warp * 32 + lane) * 32 + c] = v[c];
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, 32);
}

}  // namespace ac3d

extern "C" int ac3d_tensor_selftest(const float* A, const float* B, int K, float* D) {
  using namespace ac3d;
  if (!A || !B || !D || K < 8 || K > 128 || (K % 8) != 0) return AC3D_ERR_ARG;
  float *dA = nullptr, *dB = nullptr, *dD = nullptr;
  int* derr = nullptr;
  int herr = 0;
  const size_t smem = (size_t)(2 * 128 + 2 * 32) * K * sizeof(float);
  cudaError_t e = cudaSuccess;
  auto step = [&](cudaError_t r) {
    if (e == cudaSuccess) e = r;
  };
  step(cudaMalloc(&dA, 128 * (size_t)K * sizeof(float)));
  step(cudaMalloc(&dB, 32 * (size_t)K * sizeof(float)));
  step(cudaMalloc(&dD, 128 * 32 * sizeof(float)));
  step(cudaMalloc(&derr, sizeof(int)));
  if (e == cudaSuccess) {
    step(cudaMemcpy(dA, A, 128 * (size_t)K * sizeof(float), cudaMemcpyHostToDevice));
    step(cudaMemcpy(dB, B, 32 * (size_t)K * sizeof(float), cudaMemcpyHostToDevice));
    step(cudaMemset(derr, 0, sizeof(int)));
    step(cudaFuncSetAttribute(tc_selftest_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  }
  if (e == cudaSuccess) {
    note_launch();
    tc_selftest_kernel<<<1, 128, smem>>>(dA, dB, K, dD, derr);
    step(cudaGetLastError());
    step(cudaDeviceSynchronize());
    step(cudaMemcpy(D, dD, 128 * 32 * sizeof(float), cudaMemcpyDeviceToHost));
    step(cudaMemcpy(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost));
  }
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dD);
  cudaFree(derr);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return AC3D_ERR_CUDA;
  }
  return herr ? AC3D_ERR_CUDA : AC3D_OK;
}
