// Block (multi-right-hand-side) matvec and block BiCGSTAB interface (internal).
#pragma once

#include "internal.h"

namespace ac3d {

constexpr int kMaxRhs = 16;  // right-hand sides per block solve

// Scalars of one column of the block BiCGSTAB.
struct KCol {
  double rho_re, rho_im, rho_new_re, rho_new_im;
  double alpha_re, alpha_im, omega_re, omega_im;
  double bnorm2, rnorm2, tol2, rhat2;
  int done;        // 0 running, 1 converged, 2 iteration limit, 3 breakdown
  int restart, restarts, pad;
};

// Block solver state. The first 16 bytes are what the host polls.
struct KStateM {
  int iter, maxit, done_all, nrb;
  unsigned ticket;
  int pad[3];
  KCol col[kMaxRhs];
};

// Block vectors: nrb complex FP32 values per element, element-major (Ne x nrb).
struct MultiBufs {
  int n = 0, nrb = 0;
  bool tr = false;             // plain transpose A^T (adjoint solves) instead of A
  bool tc = true;              // dot pass on the tensor cores (nrb 8 or 16, leaves of <= 32 rows)
  void *b = nullptr, *x = nullptr, *r = nullptr, *rhat = nullptr, *p = nullptr, *v = nullptr, *s = nullptr,
       *t = nullptr;
  double* partials = nullptr;  // (max(nleaf, 1184) + 1024) x 5 x nrb: matvec partials, group totals
  double* vpartials = nullptr; // (1184 + 64 + 1) x 5 x nrb: vector partials, group totals, totals
  double* red = nullptr;       // 5 x nrb: totals of the latest matvec's dot partials
  unsigned* ticket = nullptr;  // 1024 + 64 reduction tickets (zero between launches)
  void* pbuf = nullptr;        // per-column partial dots of the dot pass (K x nrb)
  void* tbuf = nullptr;        // per-term intermediate (terms x nrb)
  const double* tol = nullptr; // nrb relative tolerances
  KStateM* state = nullptr;
};

int multi_vec_grid(int n, int nrb);
void prepare_multi_kernels();
// y = A x (or A^T x with B.tr) for block vectors; optional dot partials per column (dot_a:
// conj(a).y, dot_b: conj(y).b and |y|^2), reduced in fixed order into red (5 x nrb). FP32 storage
// only. The transposed orientation streams the same per-leaf segments with the roles of U and V
// swapped and a transposed copy of the near field (ensure_near_transposed).
void launch_mmatvec(const DevPartition& DP, const DevHMat& H, const MultiBufs& B, const void* x, void* y,
                    const void* dot_a, const void* dot_b, const int* done, cudaStream_t s);
// Builds H.nearT, the near blocks transposed into the segment layout of A^T (once per H-matrix).
void ensure_near_transposed(const DevPartition& DP, DevHMat& H, cudaStream_t s);
// Builds the TF32 hi / lo split of the dot-pass segments (V by column leaf for A, U by row leaf
// for A^T with tr) that the tensor-core dot pass streams (once per H-matrix and orientation).
// off: nleaf + 1 byte offsets, off[l + 1] - off[l] = tc_segment_bytes(R_l, K_l).
void build_tc_segments(const DevPartition& DP, DevHMat& H, bool tr, const std::vector<long long>& off,
                       cudaStream_t s);
long long tc_segment_bytes(int R, int K);
void mkrylov_enqueue_init(const MultiBufs& B, int maxit, cudaStream_t s);
void mkrylov_enqueue_iterations(const MultiBufs& B, const DevPartition& DP, const DevHMat& H, int count,
                                cudaStream_t s);
// column j of an element-major block (Ne x nrb, complex FP64) to / from a contiguous vector
void launch_block_get(int n, int nrb, int j, const void* block, void* col, cudaStream_t s);
void launch_block_set(int n, int nrb, int j, const void* col, void* block, cudaStream_t s);

}  // namespace ac3d
