// Host state of one solver context (the C-ABI's ac3d_ctx) and the orchestration steps that the
// request server (serve.cpp) shares with the single-context entry points (api.cpp).
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/ac3d.h"
#include "common.cuh"
#include "internal.h"
#include "gmres.h"
#include "krylov.h"

struct ac3d_ctx {
  // constructor parameters (DiffBEM, acoustics3d.cpp:22-34)
  int cluster_size = 64;
  double radius_factor = 1.5;
  std::vector<double> bands{1000};
  int n_freqs = 1;
  double aca_tol = 1e-3, q_tol = 1e-3, solver_tol = 1e-3;
  double src[3] = {0, 100, 0};
  int src_kind = AC3D_INCIDENT_POINT;
  double listener_radius = 50, listener_ds = 5;
  bool recompute = false;
  // extensions
  int prec = AC3D_PREC_MIXED;
  int assembly = AC3D_ASSEMBLY_DF;  // arithmetic of the mixed-precision assembly
  bool block_tc = true;             // block matvec dot pass on the tensor cores
  int listener_mode = AC3D_LISTENER_DENSE;
  int maxit = 0;           // 0: twice the number of unknowns
  double inner_tol = 1e-6; // floor of the relative tolerance of each FP32 inner solve
  int max_outer = 10;
  int chunk = 8;           // BiCGSTAB iterations per captured graph launch
  int krylov = AC3D_KRYLOV_BICGSTAB;  // inner solver of the single right-hand-side solves
  int gm_restart = 300;    // GMRES basis size: iterations per cycle before a restart
  int gm_chunk = 16;       // GMRES iterations per captured graph launch
  int maxk = 100;          // APPROX_ACA_MAX_K (constants.h:16)
  bool actual = false;     // use_actual: the coefficient / gradient calls run on the exact operator

  cudaStream_t stream = nullptr;
  cudaStream_t side = nullptr;                 // concurrent assembly work (low priority)
  cudaStream_t asm_s = nullptr;                // assembly kernels (low priority; stream is high)
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_join_asm = nullptr;
  cudaStream_t rot = nullptr;                  // GMRES Givens steps beside the next matvec (high)
  cudaEvent_t ev_gs = nullptr, ev_rot = nullptr;
  // Run the Givens step of each GMRES iteration as its own kernel beside the next matvec (on
  // `rot`). A request server's slots keep it inside the Gram-Schmidt kernel: there the other
  // slots' kernels fill the GPU, and a separate one-CTA kernel waits for a free CTA slot (behind
  // long assembly CTAs) on the solve's critical path.
  bool givens_branch = true;
  std::string err;
  ac3d_stats stats{};

  // mesh (shared with a server's other slots when the context serves requests)
  bool mesh_set = false, diff_set = false;
  std::shared_ptr<ac3d::MeshState> m = std::make_shared<ac3d::MeshState>();
  // use_actual: the same tree with every leaf pair a dense block (built on first use from the
  // set_mesh inputs, so that the element order is the H-matrix state's)
  std::shared_ptr<ac3d::MeshState> m_dense;
  std::vector<double> Ps_in;
  std::vector<int32_t> Es_in;
  std::vector<double> Ls;   // receivers for value/gradient
  ac3d::DevBuf Ls_dev;
  // differentiable points
  std::vector<int> diff_pts;
  std::unordered_map<int, int> Hs;
  std::vector<int> h_off, pair_elem, pair_corner, pair_touch, touch;
  ac3d::DevBuf d_h_off, d_pair_elem, d_pair_corner, d_pair_touch, d_touch;

  // work buffers
  ac3d::DevBuf kv, partials, kstate, red, b64, x64, r64, ff_scratch, adj_scratch, tmp_recv;
  ac3d::DevBuf kv32;  // FP32 shadows of the Krylov p and s of the mixed-precision inner solve
  ac3d::DevBuf gm;    // GMRES basis, matvec input / output, scalars and state
  std::unique_ptr<ac3d::DevHMat> last_H;  // H-matrix of the latest forward solve (matvec timing)
  ac3d::KState* h_state = nullptr;  // pinned
  ac3d::GState* h_gstate = nullptr;  // pinned, two slots
  double* h_red = nullptr;    // pinned

  ~ac3d_ctx() {
    if (h_state) cudaFreeHost(h_state);
    if (h_gstate) cudaFreeHost(h_gstate);
    if (h_red) cudaFreeHost(h_red);
  }
};

namespace ac3d {

struct ListenerLR;

// Non-convergence message naming the context's Krylov method.
std::string not_converged_message(const ac3d_ctx* c);
double wavenumber(double f);  // k = 2 pi f / c, c = 344 m/s (helpers.h:8, constants.h:13)
// Tree, partition and geometry of a mesh, device arrays on stream s (synchronised on return).
std::shared_ptr<MeshState> build_mesh_state(const double* Ps, int V, const int32_t* Es, int Ne, int cluster_size,
                                            double radius_factor, int maxk, cudaStream_t s);
void ensure_work(ac3d_ctx* c);
void reset_stats(ac3d_ctx* c);
void upload_receivers(ac3d_ctx* c, const double* L, int n, DevBuf& dst);
// One frequency on the context's mesh: assemble, solve, receivers (x_out: Ne, y_out: L complex
// FP64 device vectors). Returns the H-matrix if `keep`.
std::unique_ptr<DevHMat> forward_one(ac3d_ctx* c, double f, const double4* recv, const double* Lh, int L, cd* x_out,
                                     cd* y_out, bool keep, std::unique_ptr<ListenerLR>* q_keep = nullptr);

}  // namespace ac3d
