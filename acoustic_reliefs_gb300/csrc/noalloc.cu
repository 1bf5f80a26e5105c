// Receiver far field without any device allocation.
//
// Some callers cannot allocate device memory at the moment they need a result: an audio engine's
// real-time processing callback, a renderer's frame loop, or a host application whose own
// allocator already owns the device memory. A device allocation can block, synchronise the device
// or fail under memory pressure, so such callers need an entry point that only uses memory they
// pass in plus memory reserved when the library was loaded.
//
// ac3d_far_field_noalloc computes the scattered pressure at receivers from a given surface
// solution, y_l = sum_j M(receiver l, element j) x_j (the receiver product of the solver, FP64),
// like the far-field step of ac3d_pressures, but reads the mesh directly from the caller's
// device arrays and keeps its per-split partial sums in the file-scope array below instead of a
// buffer it would otherwise allocate. The array is fixed at kScratch complex entries (1 MiB) and
// every GPU that loads the library holds it until the process exits.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <mutex>

#include "../../include/ac3d.h"
#include "common.cuh"
#include "internal.h"

namespace ac3d {

namespace {
constexpr int kScratch = 65536;  // complex FP64 partial sums: receivers x element splits
constexpr int kNaThreads = 256;
constexpr int kNaRecv = 4;       // receivers per CTA
constexpr int kMaxDevices = 64;
}  // namespace

// Shared by every call on a device; each call overwrites the slots it uses before reading them.
// (double2: a device variable needs a type without constructors; it is read as complex pairs.)
static __device__ __align__(256) double2 g_far_scratch[kScratch];

// partial[l * S + split] = sum over elements j of the split of M(L_l, j) x_j, geometry read from
// vertex positions P (nv x 3) and connectivity E (ne x 3); elements with an index outside [0, nv)
// are skipped.
__global__ void __launch_bounds__(kNaThreads) far_noalloc_kernel(const double* __restrict__ P, int nv,
                                                                 const int* __restrict__ E, int ne,
                                                                 const double* __restrict__ Ls, int L, double k,
                                                                 const cd* __restrict__ x, cd* partial, int S) {
  __shared__ double sd[kNaThreads / 32][2 * kNaRecv];
  const int l0 = blockIdx.x * kNaRecv, split = blockIdx.y;
  const int per = (ne + S - 1) / S;
  const int j0 = split * per, j1 = min(ne, j0 + per);
  double px[kNaRecv], py[kNaRecv], pz[kNaRecv];
  for (int a = 0; a < kNaRecv; a++) {
    const int l = min(l0 + a, L - 1);
    px[a] = Ls[3 * l];
    py[a] = Ls[3 * l + 1];
    pz[a] = Ls[3 * l + 2];
  }
  double ar[kNaRecv], ai[kNaRecv];
  for (int a = 0; a < kNaRecv; a++) ar[a] = ai[a] = 0;
  for (int j = j0 + threadIdx.x; j < j1; j += blockDim.x) {
    const int ia = E[3 * j], ib = E[3 * j + 1], ic = E[3 * j + 2];
    if ((unsigned)ia >= (unsigned)nv || (unsigned)ib >= (unsigned)nv || (unsigned)ic >= (unsigned)nv) continue;
    ElemGeo<double> g;
    double a3[3];
    for (int d = 0; d < 3; d++) {
      a3[d] = P[3 * ia + d];
      g.ab[d] = P[3 * ib + d] - a3[d];
      g.ac[d] = P[3 * ic + d] - a3[d];
    }
    g.n[0] = g.ac[2] * g.ab[1] - g.ac[1] * g.ab[2];
    g.n[1] = g.ac[0] * g.ab[2] - g.ac[2] * g.ab[0];
    g.n[2] = g.ac[1] * g.ab[0] - g.ac[0] * g.ab[1];
    const cd xj = x[j];
#pragma unroll
    for (int a = 0; a < kNaRecv; a++) {
      const cd q = entry_from_d<double>(k, px[a] - a3[0], py[a] - a3[1], pz[a] - a3[2], g);
      ar[a] += q.re * xj.re - q.im * xj.im;
      ai[a] += q.re * xj.im + q.im * xj.re;
    }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int a = 0; a < kNaRecv; a++) {
    const double vr = warp_sum(ar[a]), vi = warp_sum(ai[a]);
    if (lane == 0) {
      sd[w][2 * a] = vr;
      sd[w][2 * a + 1] = vi;
    }
  }
  __syncthreads();
  if (threadIdx.x < 2 * kNaRecv) {
    const int a = threadIdx.x >> 1;
    if (l0 + a < L) {
      double s = 0;
      for (int ww = 0; ww < kNaThreads / 32; ww++) s += sd[ww][threadIdx.x];
      ((double*)partial)[((size_t)(l0 + a) * S + split) * 2 + (threadIdx.x & 1)] = s;
    }
  }
}

__global__ void far_noalloc_reduce(const cd* __restrict__ partial, int L, int S, cd* y) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= L) return;
  double sr = 0, si = 0;
  for (int s = 0; s < S; s++) {
    sr += partial[(size_t)l * S + s].re;
    si += partial[(size_t)l * S + s].im;
  }
  y[l] = cd(sr, si);
}

// Device address of g_far_scratch for each device, looked up once with that device current.
// The lookup also loads this file's kernels on that device (CUDA loads modules lazily, and
// loading reserves the array), so after it the entry point itself allocates nothing. The address
// belongs to the device's primary context: it is not valid across a cudaDeviceReset.
static cd* scratch_address(int dev) {
  static std::mutex mu;
  static cd* addr[kMaxDevices] = {nullptr};
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_far_scratch);
    if (e != cudaSuccess) {
      cudaGetLastError();  // clears the error this lookup set
      return nullptr;
    }
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, far_noalloc_kernel) != cudaSuccess ||
        cudaFuncGetAttributes(&fa, far_noalloc_reduce) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    addr[dev] = (cd*)p;
  }
  return addr[dev];
}

// Resolves the scratch address on the current device ahead of the first far-field call.
void noalloc_prepare() {
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < kMaxDevices)
    scratch_address(dev);
  else
    cudaGetLastError();
}

}  // namespace ac3d

extern "C" int ac3d_far_field_noalloc(const double* Ps_dev, int V, const int32_t* Es_dev, int Ne, const double* x_dev,
                                      double k, const double* Ls_dev, int L, double* y_dev, void* stream) {
  using namespace ac3d;
  if (!Ps_dev || !Es_dev || !x_dev || !Ls_dev || !y_dev || V < 3 || Ne < 1 || L < 1 || !(k > 0)) return AC3D_ERR_ARG;
  // split the elements so that about 2048 go to one CTA, capped by the scratch capacity
  int S = std::max(1, std::min(64, (Ne + 2047) / 2048));
  if ((long long)L * S > kScratch) S = kScratch / L;
  if (S < 1) {
    std::fprintf(stderr,
                 "ac3d_far_field_noalloc: %d receivers exceed the fixed scratch capacity of %d entries\n", L,
                 kScratch);
    return AC3D_ERR_RESOURCE;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return AC3D_ERR_CUDA;
  }
  cd* scratch = scratch_address(dev);
  if (!scratch) return AC3D_ERR_CUDA;
  cudaStream_t s = (cudaStream_t)stream;
  // each launch's own status: a pending error of unrelated earlier work is neither reported nor
  // cleared here; the error state a failed launch sets is cleared
  const cd* xc = (const cd*)x_dev;
  void* a1[] = {(void*)&Ps_dev, (void*)&V, (void*)&Es_dev, (void*)&Ne, (void*)&Ls_dev, (void*)&L, (void*)&k,
                (void*)&xc, (void*)&scratch, (void*)&S};
  note_launch();
  if (cudaLaunchKernel((const void*)far_noalloc_kernel, dim3((L + kNaRecv - 1) / kNaRecv, S), dim3(kNaThreads), a1,
                       0, s) != cudaSuccess) {
    cudaGetLastError();
    return AC3D_ERR_CUDA;
  }
  cd* yc = (cd*)y_dev;
  void* a2[] = {(void*)&scratch, (void*)&L, (void*)&S, (void*)&yc};
  note_launch();
  if (cudaLaunchKernel((const void*)far_noalloc_reduce, dim3((L + 127) / 128), dim3(128), a2, 0, s) != cudaSuccess) {
    cudaGetLastError();
    return AC3D_ERR_CUDA;
  }
  return AC3D_OK;
}
