// Kernel launches with optional programmatic dependent launch (PDL, sm_90+).
//
// A kernel launched with pdl = true may be scheduled while the preceding kernel of the stream is
// still running. Such a kernel calls grid_dep_wait() before it reads anything the preceding
// kernel writes and before it writes anything that kernel reads or writes; work before the wait
// is limited to shared memory and to data that no kernel of the sequence writes (or, where the
// launch sequence guarantees it, data written two or more kernels earlier). Every kernel of
// a PDL sequence calls grid_dep_wait() and only then grid_dep_launch(), so that once a kernel
// starts, the kernel two places before it has completed and its writes are visible.
// For a kernel launched without the attribute both calls are no-ops.
#pragma once

#include <utility>

#include "common.cuh"
#include "internal.h"

namespace ac3d {

__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_dep_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KArgs, typename... Args>
void launch_k(bool pdl, void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
              Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  if (pdl) {
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
  }
  note_launch();
  AC3D_CUDA(cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...));
}

}  // namespace ac3d
