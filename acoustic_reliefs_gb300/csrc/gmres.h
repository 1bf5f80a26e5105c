// Device-resident GMRES interface (internal).
#pragma once

#include <cstddef>

#include "internal.h"

namespace ac3d {

// Scalars of one GMRES cycle, kept on the device.
struct GState {
  int j;       // basis vectors 0..j exist; iterations done in this cycle
  int m;       // basis capacity: at most m iterations per cycle
  int done;    // 0 running, 1 converged, 2 basis full, 3 breakdown (non-finite values)
  int pad;
  double tol_abs;   // stop when the least-squares residual estimate falls to this
  double beta;      // norm of the right-hand side of the cycle
  double resid;     // latest least-squares residual estimate |g_j|
  unsigned ticket;  // last-CTA ticket of the reducing passes (zero between launches)
  int pad2;
};

// Completion of a batch of cycles (one per right-hand side): done_all becomes 1 when every cycle
// of the batch has ended. The matvec passes read it to skip their work after the last one.
struct GMulti {
  int ndone;     // cycles that have ended
  int done_all;
  unsigned long long bar;  // arrivals at the grid barriers of the Gram-Schmidt kernels (zero at init)
  int bar_fail;            // a grid barrier gave up waiting
  int pad[3];
};
static_assert(offsetof(GMulti, bar) % 8 == 0, "64-bit atomics need an aligned arrival counter");
static_assert(sizeof(GState) % 8 == 0, "GMulti follows the cycles' states in one allocation");

// Device buffers of one cycle, or of a batch of nrb independent cycles that share their matvecs
// (column r: state st + r, scalars gd + r gds, basis V + r Vs elements; the matvec input q and
// output W, the right-hand side b and the solution are block vectors with element stride vs). vec64: 0 complex FP32 vectors (FP32 H-matrix and arithmetic),
// 1 complex FP64 vectors (FP64 H-matrix).
struct GmresBufs {
  int n = 0, m = 0, vec64 = 0;
  int nrb = 1, vs = 1;   // cycles in the batch; element stride of the block vectors
  size_t gds = 0, Vs = 0;
  GMulti* gm = nullptr;
  const double* tolv = nullptr;  // per-cycle relative tolerances (batch), else the scalar one
  int b32 = 0;           // 1: the right-hand side and the solution are complex FP32 (batch)
  void* b = nullptr;   // right-hand side, complex FP64 (n), or FP32 block vectors (b32)
  void* V = nullptr;   // basis, (m + 1) x n vectors of the vector type
  void* q = nullptr;   // the next matvec's input (n)
  void* W = nullptr;   // the matvec's output (n)
  void* W2 = nullptr;  // the first Gram-Schmidt pass's result (n per cycle), when there are two
  int reorth = 0;      // 1: two classical Gram-Schmidt passes (FP32 vectors; the second one delayed by an
                       // iteration in the cooperative kernel)
  double* gd = nullptr;  // gmres_scalar_doubles(m, n) doubles
  GState* state = nullptr;
  // Branch for the Givens step (rotation of the new Hessenberg column, residual estimate, stop
  // test): when rot_stream is set, the iterations enqueued on a stream fork it after each
  // cooperative Gram-Schmidt kernel, so that it runs beside the next matvec (which needs only the
  // new input vector) and joins before the next Gram-Schmidt kernel (which needs j and the
  // Hessenberg column the Givens step leaves).
  cudaStream_t rot_stream = nullptr;
  cudaEvent_t ev_gs = nullptr, ev_rot = nullptr;
};

int gmres_grid(int n);
size_t gmres_scalar_doubles(int m, int n);
size_t gmres_update_smem(int m);
void gmres_enqueue_init(const GmresBufs& B, double tol, cudaStream_t s);
void gmres_enqueue_iterations(const GmresBufs& B, const DevPartition& DP, const DevHMat& H, bool transposed,
                              int count, cudaStream_t s);
// x = the cycle's solution: the least-squares coefficients applied to the basis (complex FP64,
// n; or the FP32 block vectors of a batch)
void gmres_enqueue_finish(const GmresBufs& B, void* x, cudaStream_t s);
struct MultiBufs;
// A batch's iterations: one block matvec of all the cycles' inputs (the block solver's passes and
// buffers in MB), then every cycle's Gram-Schmidt passes.
void gmres_enqueue_iterations_block(const GmresBufs& B, const MultiBufs& MB, const DevPartition& DP,
                                    const DevHMat& H, int count, cudaStream_t s);

}  // namespace ac3d
