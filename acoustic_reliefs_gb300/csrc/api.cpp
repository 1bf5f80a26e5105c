// Host orchestration and the C-ABI of libac3d.so.
//
// Mirrors the reference binding DiffBEM (acoustics3d_cpp/src/acoustics3d.cpp:22-351) and its
// driver bem3d::gradient (acoustics3d_cpp/src/adjoint.cpp:24-242): set_mesh builds the tree and
// partition once; every evaluation updates vertex heights, assembles one H-matrix per frequency
// on the GPU, solves with the device-resident BiCGSTAB, evaluates the receivers, forms the
// diffusion coefficient and, for the gradient, runs the adjoint solve and shape derivatives.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/ac3d.h"
#include "context.h"
#include "internal.h"
#include "gmres.h"
#include "krylov.h"
#include "listener.h"
#include "multi.h"

namespace ac3d {

std::atomic<long long> g_kernel_launches{0};
thread_local long long t_kernel_launches = 0;

void cuda_check(cudaError_t e, const char* what, const char* file, int line) {
  if (e != cudaSuccess) {
    throw Error(AC3D_ERR_CUDA, std::string(cudaGetErrorName(e)) + ": " + cudaGetErrorString(e) + " (" + what +
                                   " at " + file + ":" + std::to_string(line) + ")");
  }
}

void DevBuf::alloc(size_t n, cudaStream_t stream) {
  release();
  s = stream;
  if (n == 0) n = 16;
  cudaError_t e = cudaMallocAsync(&p, n, s);
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    throw Error(AC3D_ERR_RESOURCE, "device allocation of " + std::to_string(n) + " bytes failed");
  }
  AC3D_CUDA(e);
  bytes = n;
}

void DevBuf::release() {
  if (p) cudaFreeAsync(p, s);
  p = nullptr;
  bytes = 0;
}

template <typename T>
static void upload(DevBuf& d, const std::vector<T>& h, cudaStream_t s) {
  d.alloc(std::max<size_t>(h.size(), 1) * sizeof(T), s);
  if (!h.empty()) AC3D_CUDA(cudaMemcpyAsync(d.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s));
}

double wavenumber(double f) { return 2 * kPiHost * f / 344.0; }  // helpers.h:8, constants.h:13

// get_frequencies (helpers.cpp:67-83)
static std::vector<double> frequencies(double band, int n) {
  if (n == 1) return {band};
  double bw = std::pow(2.0, 1.0 / 6.0);
  double lo = std::log(band / bw), hi = std::log(band * bw);
  double d = (hi - lo) / (n - 1.0);
  std::vector<double> f;
  for (int i = 0; i < n; i++) f.push_back(std::exp(lo + i * d));
  return f;
}

// compute_listener_pts + spherical_to_cartesian (helpers.cpp:34-65)
static std::vector<double> hemisphere(double radius, double ds) {
  std::vector<double> el{0}, az{0};
  for (double e = ds; e < 91; e += ds)
    for (double a = 0; a < 360; a += ds) {
      el.push_back(e);
      az.push_back(a);
    }
  std::vector<double> L;
  for (size_t i = 0; i < el.size(); i++) {
    double th = el[i] * kPiHost / 180.0, ph = az[i] * kPiHost / 180.0;
    L.push_back(radius * std::sin(th) * std::cos(ph));
    L.push_back(radius * std::cos(th));
    L.push_back(-radius * std::sin(th) * std::sin(ph));
  }
  return L;
}

struct GpuTimer {
  cudaEvent_t a = nullptr, b = nullptr;
  cudaStream_t s;
  explicit GpuTimer(cudaStream_t st) : s(st) {
    AC3D_CUDA(cudaEventCreate(&a));
    AC3D_CUDA(cudaEventCreate(&b));
    AC3D_CUDA(cudaEventRecord(a, s));
  }
  double stop() {
    AC3D_CUDA(cudaEventRecord(b, s));
    AC3D_CUDA(cudaEventSynchronize(b));
    float ms = 0;
    AC3D_CUDA(cudaEventElapsedTime(&ms, a, b));
    return ms;
  }
  ~GpuTimer() {
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
  }
};

// A captured chunk of solver iterations as an executable graph. If enqueueing throws during the
// capture, the capture is ended and its graph discarded, so the stream is usable again; the
// executable graph is destroyed on every exit path after the stream has drained (an error may be
// thrown while a launch is in flight).
struct CapturedGraph {
  cudaStream_t s;
  cudaGraphExec_t exec = nullptr;
  long long nodes = 0;  // kernels per launch
  // host milliseconds spent capturing and instantiating are added to *ms_host
  template <typename F>
  CapturedGraph(cudaStream_t st, double* ms_host, F&& enqueue) : s(st) {
    const auto t0 = std::chrono::steady_clock::now();
    struct Add {
      double* acc;
      std::chrono::steady_clock::time_point t0;
      ~Add() { *acc += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count(); }
    } add{ms_host, t0};
    const long long before = t_kernel_launches;
    AC3D_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    try {
      enqueue();
    } catch (...) {
      cudaGraph_t g = nullptr;
      if (cudaStreamEndCapture(s, &g) == cudaSuccess && g) cudaGraphDestroy(g);
      cudaGetLastError();
      unnote_launches(t_kernel_launches - before);
      throw;
    }
    cudaGraph_t graph = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(s, &graph);
    nodes = t_kernel_launches - before;
    unnote_launches(nodes);  // captured, not launched
    AC3D_CUDA(ec);
    const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) exec = nullptr;
    AC3D_CUDA(ei);
  }
  CapturedGraph(const CapturedGraph&) = delete;
  CapturedGraph& operator=(const CapturedGraph&) = delete;
  void launch() {
    AC3D_CUDA(cudaGraphLaunch(exec, s));
    note_launch(nodes);
  }
  ~CapturedGraph() {
    if (exec) {
      cudaStreamSynchronize(s);
      cudaGraphExecDestroy(exec);
    }
  }
};

// An event destroyed on every exit path.
struct ScopedEvent {
  cudaEvent_t e = nullptr;
  ScopedEvent() { AC3D_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming)); }
  ScopedEvent(const ScopedEvent&) = delete;
  ScopedEvent& operator=(const ScopedEvent&) = delete;
  ~ScopedEvent() {
    if (e) cudaEventDestroy(e);
  }
};

struct GraphCache {
  cudaGraphExec_t exec = nullptr;
  const void* key_h = nullptr;
  const void* key_x = nullptr;
  bool tr = false;
  int vec64 = 0;
  ~GraphCache() {
    if (exec) cudaGraphExecDestroy(exec);
  }
};

}  // namespace ac3d

using namespace ac3d;


namespace ac3d {

std::string not_converged_message(const ac3d_ctx* c) {
  return c->krylov == AC3D_KRYLOV_GMRES ? "GMRES (restarted by the refinement loop) did not reach solver_tol"
                                        : "BiCGSTAB did not reach solver_tol";
}

void require_mesh(ac3d_ctx* c) {
  if (!c->mesh_set) throw Error(AC3D_ERR_STATE, "No mesh set. Set one using set_mesh or precompute.");
}

// ------------------------------------------------------------------------------------------
// Assembly
// ------------------------------------------------------------------------------------------
std::unique_ptr<DevHMat> assemble(ac3d_ctx* c, double k, int prec) {
  cudaStream_t s = c->stream;
  auto H = std::make_unique<DevHMat>();
  H->prec = prec;
  H->pool_df = prec != PREC_FP64 && c->assembly == AC3D_ASSEMBLY_DF;
  H->k = k;
  H->maxk = c->maxk;
  const size_t cs = prec == PREC_FP64 ? sizeof(cd) : sizeof(cf);
  const size_t pool_es = prec == PREC_FP64 || H->pool_df ? 16 : sizeof(cf);  // cd or cdf terms
  H->near.alloc((size_t)std::max<int64_t>(c->m->P.near_total, 2) * cs, s);
  if (prec != PREC_FP64) H->xdf.alloc((size_t)c->m->Ne * sizeof(cd), s);
  AC3D_CUDA(cudaMemsetAsync(H->near.p, 0, (size_t)std::max<int64_t>(c->m->P.near_total, 2) * cs, s));
  // near field and ACA kernels on the low-priority assembly streams; every buffer is allocated
  // and freed on s, which waits for them before it reads their results
  cudaStream_t as = c->asm_s;
  AC3D_CUDA(cudaEventRecord(c->ev_fork, s));
  AC3D_CUDA(cudaStreamWaitEvent(as, c->ev_fork, 0));
  // On every way out (an exception included), s waits for the assembly streams before anything
  // frees H's buffers on s (destroyed before H: declared after it).
  struct JoinAssembly {
    ac3d_ctx* c;
    ~JoinAssembly() {
      cudaEventRecord(c->ev_join_asm, c->asm_s);
      cudaStreamWaitEvent(c->stream, c->ev_join_asm, 0);
      cudaEventRecord(c->ev_join, c->side);
      cudaStreamWaitEvent(c->stream, c->ev_join, 0);
    }
  } join_assembly{c};
  if (H->pool_df)
    launch_near_assembly_df(c->m->G, c->m->DP, *H, as);
  else
    launch_near_assembly(c->m->G, c->m->DP, *H, as);
  H->err.alloc(16, s);
  AC3D_CUDA(cudaMemsetAsync(H->err.p, 0, 16, s));
  H->ticket.alloc(16, s);
  AC3D_CUDA(cudaMemsetAsync(H->ticket.p, 0, 16, s));

  const int na = c->m->DP.na;
  H->rank.alloc((size_t)std::max(na, 1) * sizeof(int), s);
  H->passes.alloc((size_t)std::max(na, 1) * sizeof(int), s);
  H->t_off.alloc((size_t)(na + 1) * sizeof(int), s);
  AC3D_CUDA(cudaMemsetAsync(H->rank.p, 0, (size_t)std::max(na, 1) * sizeof(int), s));
  if (na > 0) {
    H->term_off.alloc((size_t)na * c->maxk * sizeof(long long), s);
    H->pool_used.alloc(16, s);
    int64_t cap = c->m->pool_hint[prec];
    if (cap <= 0) cap = std::min<int64_t>(c->m->worst_pool, 16 * c->m->sum_mn);
    cap = std::max<int64_t>(cap, 1024);
    for (int attempt = 0;; attempt++) {
      H->pool.alloc((size_t)cap * pool_es, s);
      H->pool_cap = cap;
      AC3D_CUDA(cudaMemsetAsync(H->pool_used.p, 0, 16, s));
      // the ACA groups on the two assembly streams (the first after the near field)
      AC3D_CUDA(cudaEventRecord(c->ev_fork, s));
      AC3D_CUDA(cudaStreamWaitEvent(as, c->ev_fork, 0));
      AC3D_CUDA(cudaStreamWaitEvent(c->side, c->ev_fork, 0));
      if (H->pool_df)
        launch_aca_df(c->m->G, c->m->DP, *H, c->aca_tol, c->m->P.max_rows, as, c->side);
      else
        launch_aca(c->m->G, c->m->DP, *H, c->aca_tol, c->m->P.max_rows, as, c->side);
      AC3D_CUDA(cudaEventRecord(c->ev_join, c->side));
      AC3D_CUDA(cudaEventRecord(c->ev_join_asm, as));
      AC3D_CUDA(cudaStreamWaitEvent(s, c->ev_join, 0));
      AC3D_CUDA(cudaStreamWaitEvent(s, c->ev_join_asm, 0));
      unsigned long long hu[2];
      AC3D_CUDA(cudaMemcpyAsync(hu, H->pool_used.p, 16, cudaMemcpyDeviceToHost, s));
      AC3D_CUDA(cudaStreamSynchronize(s));
      int status = (int)(hu[1] & 0xffffffffu);
      if (!(status & 1)) {
        H->pool_used_host = (int64_t)hu[0];
        break;
      }
      if (cap >= c->m->worst_pool || attempt > 8) throw Error(AC3D_ERR_INTERNAL, "ACA pool overflow at worst-case size");
      cap = std::min<int64_t>(c->m->worst_pool, std::max<int64_t>(cap * 2, (int64_t)hu[0]));
    }
    c->m->pool_hint[prec] = std::min<int64_t>(c->m->worst_pool, H->pool_used_host + H->pool_used_host / 8 + 4096);
    const size_t tcap = (size_t)std::max<int64_t>(c->m->P.aca_term_cap, 1);
    H->task_cap = (int64_t)tcap;
    H->task_b.alloc(tcap * sizeof(int), s);
    H->task_off.alloc(tcap * sizeof(long long), s);
    launch_rank_scan(c->m->DP, *H, s);
    H->tvec.alloc(tcap * (prec == PREC_FP64 ? sizeof(cd) : sizeof(cf)), s);
    H->tvec64.alloc(tcap * sizeof(cd), s);
    H->ranks_host.resize(na);
    std::vector<int> passes(na);
    AC3D_CUDA(cudaMemcpyAsync(H->ranks_host.data(), H->rank.p, na * sizeof(int), cudaMemcpyDeviceToHost, s));
    AC3D_CUDA(cudaMemcpyAsync(passes.data(), H->passes.p, na * sizeof(int), cudaMemcpyDeviceToHost, s));
    AC3D_CUDA(cudaStreamSynchronize(s));
    int64_t lr = 0, ev = 0;
    int mx = 0;
    double sr = 0;
    for (int b = 0; b < na; b++) {
      int r = H->ranks_host[b];
      const int* q = &c->m->P.approx[4 * b];
      lr += (int64_t)r * ((q[1] - q[0]) + (q[3] - q[2]));
      ev += (int64_t)passes[b] * ((q[1] - q[0]) + (q[3] - q[2]));
      mx = std::max(mx, r);
      sr += r;
    }
    H->lr_entries = lr;
    H->aca_evaluated = ev;
    c->stats.lr_entries = lr;
    c->stats.aca_entries_evaluated = ev;
    // per-leaf segments (U by row leaf, V by column leaf), then the pool is released
    int64_t sum_rn = 0, kf = 0, kt = 0;
    for (int b = 0; b < na; b++) sum_rn += (int64_t)H->ranks_host[b] * (c->m->P.approx[4 * b + 3] - c->m->P.approx[4 * b + 2]);
    const int nleaf = c->m->DP.nleaf;
    int64_t segf = 0, segt = 0;
    for (int l = 0; l < nleaf; l++) {
      const int Rl = c->m->P.leaf_start[l + 1] - c->m->P.leaf_start[l];
      int K = 0;
      for (int it = c->m->P.fw_lr_ptr[l]; it < c->m->P.fw_lr_ptr[l + 1]; it++) K += H->ranks_host[c->m->P.fw_lr[it]];
      K += K & 1;
      kf += K;
      segf += (int64_t)K * Rl;
      K = 0;
      for (int it = c->m->P.tr_lr_ptr[l]; it < c->m->P.tr_lr_ptr[l + 1]; it++) K += H->ranks_host[c->m->P.tr_lr[it]];
      K += K & 1;
      kt += K;
      segt += (int64_t)K * Rl;
    }
    H->kseg_f.alloc((size_t)(nleaf + 1) * sizeof(int), s);
    H->kseg_t.alloc((size_t)(nleaf + 1) * sizeof(int), s);
    H->seg_f.alloc((size_t)(nleaf + 1) * sizeof(long long), s);
    H->seg_t.alloc((size_t)(nleaf + 1) * sizeof(long long), s);
    H->useg.alloc((size_t)std::max<int64_t>(segf, 2) * cs, s);
    H->vseg.alloc((size_t)std::max<int64_t>(segt, 2) * cs, s);
    H->uidx.alloc((size_t)std::max<int64_t>(kf, 1) * sizeof(int), s);
    H->vidx.alloc((size_t)std::max<int64_t>(kt, 1) * sizeof(int), s);
    H->kpos_f.alloc((size_t)std::max<size_t>(c->m->P.fw_lr.size(), 1) * sizeof(int), s);
    H->kpos_t.alloc((size_t)std::max<size_t>(c->m->P.tr_lr.size(), 1) * sizeof(int), s);
    H->pbuf.alloc((size_t)std::max<int64_t>(std::max(kf, kt), 1) * sizeof(cd), s);
    // leaves by decreasing streamed bytes: row leaves (near + U columns) for the forward gather and
    // the transposed dot, column leaves (V columns; + transposed near) for the forward dot and the
    // transposed gather. The hardware dispatches CTAs in index order, so this is
    // longest-first list scheduling.
    {
      std::vector<int64_t> wr(nleaf), wc(nleaf);
      std::vector<int> ord(nleaf);
      for (int l = 0; l < nleaf; l++) {
        const int Rl = c->m->P.leaf_start[l + 1] - c->m->P.leaf_start[l];
        int64_t kr = c->m->P.didx_ptr[l + 1] - c->m->P.didx_ptr[l], kc = 0;
        for (int it = c->m->P.fw_lr_ptr[l]; it < c->m->P.fw_lr_ptr[l + 1]; it++) kr += H->ranks_host[c->m->P.fw_lr[it]];
        for (int it = c->m->P.tr_lr_ptr[l]; it < c->m->P.tr_lr_ptr[l + 1]; it++) kc += H->ranks_host[c->m->P.tr_lr[it]];
        for (int it = c->m->P.tr_near_ptr[l]; it < c->m->P.tr_near_ptr[l + 1]; it++) {
          const int* q = &c->m->P.direct[4 * c->m->P.tr_near[it]];
          kc += q[1] - q[0];
        }
        wr[l] = kr * Rl;
        wc[l] = kc * Rl;
      }
      auto sorted = [&](const std::vector<int64_t>& w) {
        for (int l = 0; l < nleaf; l++) ord[l] = l;
        std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return w[a] > w[b]; });
        return ord;
      };
      upload(H->order_rows, sorted(wr), s);
      upload(H->order_cols, sorted(wc), s);
    }
    launch_pack(c->m->DP, *H, false, s);
    launch_pack(c->m->DP, *H, true, s);
    H->pool.release();
    H->term_off.release();
    (void)sum_rn;
    c->stats.max_rank = mx;
    c->stats.mean_rank = sr / na;
  } else {
    // no admissible blocks: only the near field ran on the assembly stream
    AC3D_CUDA(cudaEventRecord(c->ev_join_asm, as));
    AC3D_CUDA(cudaStreamWaitEvent(s, c->ev_join_asm, 0));
    AC3D_CUDA(cudaMemsetAsync(H->t_off.p, 0, sizeof(int), s));
    H->tvec.alloc(16, s);
    H->tvec64.alloc(16, s);
    for (DevBuf* kb : {&H->kseg_f, &H->kseg_t}) {
      kb->alloc((size_t)(c->m->DP.nleaf + 1) * sizeof(int), s);
      AC3D_CUDA(cudaMemsetAsync(kb->p, 0, (size_t)(c->m->DP.nleaf + 1) * sizeof(int), s));
    }
    for (DevBuf* sb : {&H->seg_f, &H->seg_t}) {
      sb->alloc((size_t)(c->m->DP.nleaf + 1) * sizeof(long long), s);
      AC3D_CUDA(cudaMemsetAsync(sb->p, 0, (size_t)(c->m->DP.nleaf + 1) * sizeof(long long), s));
    }
    H->useg.alloc(32, s);
    H->vseg.alloc(32, s);
    H->uidx.alloc(16, s);
    H->vidx.alloc(16, s);
    std::vector<int> ord(c->m->DP.nleaf);
    for (int l = 0; l < c->m->DP.nleaf; l++) ord[l] = l;
    upload(H->order_rows, ord, s);
    upload(H->order_cols, ord, s);
  }
  c->stats.near_entries = c->m->P.near_total;
  c->stats.hmat_bytes = (long long)H->bytes();
  return H;
}

// ------------------------------------------------------------------------------------------
// Solve op(A) x = b (b, x FP64 device vectors of length Ne)
// ------------------------------------------------------------------------------------------
struct SolveCache {
  std::vector<std::unique_ptr<GraphCache>> graphs;
};

void ensure_work(ac3d_ctx* c) {
  cudaStream_t s = c->stream;
  const size_t n = (size_t)c->m->Ne;
  c->kv.ensure(8 * n * sizeof(cd), s);
  c->kv32.ensure(2 * n * sizeof(cf), s);
  const int G = krylov_vec_grid(c->m->Ne);
  c->partials.ensure((size_t)(c->m->DP.nleaf + G) * 5 * sizeof(double) + 64, s);
  c->kstate.ensure(sizeof(KState), s);
  c->red.ensure(16 * sizeof(double), s);
  c->b64.ensure(n * sizeof(cd), s);
  c->x64.ensure(n * sizeof(cd), s);
  c->r64.ensure(n * sizeof(cd), s);
  if (!c->h_state) AC3D_CUDA(cudaMallocHost(&c->h_state, 2 * sizeof(KState)));
  (void)device_sm_count();  // query outside any stream capture
  prepare_matvec_kernels();
  if (!c->h_red) AC3D_CUDA(cudaMallocHost(&c->h_red, 8 * sizeof(double)));
}

KrylovBufs bufs(ac3d_ctx* c, int vec64) {
  KrylovBufs B;
  B.n = c->m->Ne;
  const size_t es = vec64 ? sizeof(cd) : sizeof(cf);
  char* base = (char*)c->kv.p;
  void** slots[8] = {&B.b, &B.x, &B.r, &B.rhat, &B.p, &B.v, &B.s, &B.t};
  for (int i = 0; i < 8; i++) *slots[i] = base + (size_t)i * c->m->Ne * es;
  if (vec64 == 2) {
    B.p32 = c->kv32.p;
    B.s32 = (char*)c->kv32.p + (size_t)c->m->Ne * sizeof(cf);
  }
  B.partials = c->partials.as<double>();
  B.nparts_r = krylov_vec_grid(c->m->Ne);
  B.nleaf = c->m->DP.nleaf;
  B.red5 = c->red.as<double>() + 8;
  B.state = c->kstate.as<KState>();
  return B;
}

// Runs BiCGSTAB on the prepared buffers (B.b filled). Returns iterations; done flag in *done.
int run_krylov(ac3d_ctx* c, const DevHMat& H, const KrylovBufs& B, bool tr, int vec64, double tol, int* done) {
  cudaStream_t s = c->stream;
  const int maxit = c->maxit > 0 ? c->maxit : 2 * c->m->Ne;
  krylov_enqueue_init(B, vec64, tol, maxit, s);
  // capture one chunk of iterations as a graph and replay it until the state reports completion
  CapturedGraph g(s, &c->stats.ms_graph, [&] { krylov_enqueue_iterations(B, c->m->DP, H, tr, vec64, c->chunk, s); });
  int launched = 0;
  const int max_launch = maxit / c->chunk + 2;
  // keep one chunk in flight while the host reads the previous state
  g.launch();
  AC3D_CUDA(cudaMemcpyAsync(&c->h_state[0], B.state, sizeof(KState), cudaMemcpyDeviceToHost, s));
  launched++;
  ScopedEvent sev;
  cudaEvent_t ev = sev.e;
  AC3D_CUDA(cudaEventRecord(ev, s));
  KState st{};
  while (true) {
    bool more = launched < max_launch;
    if (more) {
      g.launch();
      AC3D_CUDA(cudaMemcpyAsync(&c->h_state[launched & 1], B.state, sizeof(KState), cudaMemcpyDeviceToHost, s));
    }
    AC3D_CUDA(cudaEventSynchronize(ev));
    st = c->h_state[(launched - 1) & 1];
    if (st.done || !more) break;
    launched++;
    AC3D_CUDA(cudaEventRecord(ev, s));
  }
  AC3D_CUDA(cudaStreamSynchronize(s));
  st = c->h_state[(launched - 1) & 1];
  if (launched < max_launch) {
    // the extra chunk in flight was a no-op; reread the final state
    AC3D_CUDA(cudaMemcpy(&st, B.state, sizeof(KState), cudaMemcpyDeviceToHost));
  } else {
    AC3D_CUDA(cudaMemcpy(&st, B.state, sizeof(KState), cudaMemcpyDeviceToHost));
  }
  *done = st.done;
  c->stats.matvecs += 2 * st.iter;
  return st.iter;
}

// GMRES buffers of this context, carved from one allocation: nrb cycles (a batch shares its
// matvecs; the block vectors q, W and b belong to the caller then) in the H-matrix's precision.
GmresBufs gmres_bufs(ac3d_ctx* c, const DevHMat& H, const void* b, int nrb = 1) {
  GmresBufs G;
  G.n = c->m->Ne;
  G.m = std::max(1, std::min(c->gm_restart, G.n));
  G.vec64 = H.prec == PREC_FP64 ? 1 : 0;
  G.nrb = nrb;
  G.vs = nrb;
  const size_t es = G.vec64 ? sizeof(cd) : sizeof(cf);
  auto up = [](size_t v) { return (v + 255) & ~(size_t)255; };
  G.Vs = ((size_t)G.m + 1) * G.n;
  G.gds = (gmres_scalar_doubles(G.m, G.n) + 1) & ~(size_t)1;
  const size_t vb = up(G.Vs * es * nrb), nb = up((size_t)G.n * es);
  const size_t gb = up(G.gds * nrb * sizeof(double)), sb = up(nrb * sizeof(GState) + sizeof(GMulti));
  const size_t vecs = nrb == 1 ? 3 * nb : 0;  // single: q, W, W2 here; a batch uses the caller's
  c->gm.ensure(vb + vecs + gb + sb, c->stream);
  char* p = (char*)c->gm.p;
  G.V = p;
  if (nrb == 1) {
    G.q = p + vb;
    G.W = p + vb + nb;
    G.W2 = p + vb + 2 * nb;
  }
  G.gd = (double*)(p + vb + vecs);
  G.state = (GState*)(p + vb + vecs + gb);
  G.gm = (GMulti*)(G.state + nrb);
  G.b = (void*)b;
  // FP32 classical Gram-Schmidt loses orthogonality over long cycles: two passes keep the FP32
  // cycle converging like the FP64 one
  G.reorth = G.vec64 ? 0 : 1;
  G.rot_stream = c->givens_branch ? c->rot : nullptr;
  G.ev_gs = c->ev_gs;
  G.ev_rot = c->ev_rot;
  if (!c->h_gstate) AC3D_CUDA(cudaMallocHost(&c->h_gstate, 2 * sizeof(GState)));
  return G;
}

// Zero states (their tickets start at zero; each reducing pass leaves them at zero) and batch
// completion count; no host wait, so the host captures the cycle's graph while the device runs
// the assembly.
void gmres_reset(const GmresBufs& G, cudaStream_t s) {
  AC3D_CUDA(cudaMemsetAsync(G.state, 0, G.nrb * sizeof(GState) + sizeof(GMulti), s));
}

// One GMRES cycle on op(A) d = b (complex FP64 device vectors): at most gm_restart iterations, in
// the H-matrix's precision. Returns the iterations; the state's done code in *done.
int run_gmres(ac3d_ctx* c, const DevHMat& H, const cd* b, cd* d, bool tr, double tol, int* done) {
  cudaStream_t s = c->stream;
  GmresBufs G = gmres_bufs(c, H, b);
  gmres_reset(G, s);
  gmres_enqueue_init(G, tol, s);
  CapturedGraph g(s, &c->stats.ms_graph, [&] { gmres_enqueue_iterations(G, c->m->DP, H, tr, c->gm_chunk, s); });
  // keep one chunk in flight while the host reads the state after the previous one
  const int max_launch = (G.m + c->gm_chunk - 1) / c->gm_chunk + 1;
  int launched = 0;
  g.launch();
  AC3D_CUDA(cudaMemcpyAsync(&c->h_gstate[0], G.state, sizeof(GState), cudaMemcpyDeviceToHost, s));
  launched++;
  ScopedEvent sev;
  cudaEvent_t ev = sev.e;
  AC3D_CUDA(cudaEventRecord(ev, s));
  while (true) {
    const bool more = launched < max_launch;
    if (more) {
      g.launch();
      AC3D_CUDA(cudaMemcpyAsync(&c->h_gstate[launched & 1], G.state, sizeof(GState), cudaMemcpyDeviceToHost, s));
    }
    AC3D_CUDA(cudaEventSynchronize(ev));
    const GState st = c->h_gstate[(launched - 1) & 1];
    if (st.done || !more) break;
    launched++;
    AC3D_CUDA(cudaEventRecord(ev, s));
  }
  gmres_enqueue_finish(G, d, s);
  GState st{};
  GMulti gm{};
  AC3D_CUDA(cudaMemcpyAsync(&c->h_gstate[0], G.state, sizeof(GState), cudaMemcpyDeviceToHost, s));
  AC3D_CUDA(cudaMemcpyAsync(&gm, G.gm, sizeof(GMulti), cudaMemcpyDeviceToHost, s));
  AC3D_CUDA(cudaStreamSynchronize(s));
  if (gm.bar_fail) throw Error(AC3D_ERR_CUDA, "GMRES Gram-Schmidt grid barrier timed out (bounded wait)");
  st = c->h_gstate[0];
  *done = st.done;
  c->stats.matvecs += st.j;
  return st.j;
}

double reduce_norm2_residual(ac3d_ctx* c, const DevHMat& H, bool tr, const cd* b, const cd* x, cd* r) {
  cudaStream_t s = c->stream;
  MatvecEpilogue ep;
  ep.partials = c->partials.as<double>();
  launch_matvec(c->m->DP, H, c->m->Ne, tr, 1, x, r, b, ep, s);
  launch_reduce5(c->partials.as<double>(), c->m->DP.nleaf, c->red.as<double>(), s);
  AC3D_CUDA(cudaMemcpyAsync(c->h_red, c->red.p, 5 * sizeof(double), cudaMemcpyDeviceToHost, s));
  AC3D_CUDA(cudaStreamSynchronize(s));
  c->stats.matvecs++;
  return c->h_red[4];
}

// x = op(A)^{-1} b to relative residual solver_tol (FP64 b, x on device).
void check_pipeline(ac3d_ctx* c, const DevHMat& H) {
  int e = 0;
  AC3D_CUDA(cudaMemcpyAsync(&e, H.err.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  AC3D_CUDA(cudaStreamSynchronize(c->stream));
  if (e) throw Error(AC3D_ERR_CUDA, "matvec copy pipeline timed out (bounded mbarrier wait)");
}

void solve_impl(ac3d_ctx* c, DevHMat& H, const cd* b, cd* x, bool tr);

void solve(ac3d_ctx* c, DevHMat& H, const cd* b, cd* x, bool tr) {
  solve_impl(c, H, b, x, tr);
  check_pipeline(c, H);
}

// GMRES cycles inside the refinement loop: x = 0, then d = op(A)^{-1} r by one cycle, x += d and
// r = b - op(A) x in FP64 (double-float arithmetic on an FP32 H-matrix) until |r| <= tol |b|. A
// cycle runs in the H-matrix's precision; an FP32 cycle stops at inner_tol (or 0.3 of what is
// still needed), an FP64 one at half of what is needed.
void solve_gmres(ac3d_ctx* c, DevHMat& H, const cd* b, cd* x, bool tr) {
  cudaStream_t s = c->stream;
  const int n = c->m->Ne;
  const double tol = c->solver_tol;
  const bool fp64 = H.prec == PREC_FP64;
  KrylovBufs B = bufs(c, 1);  // B.x holds each cycle's correction
  launch_zero64(n, x, s);
  launch_copy64(n, b, c->r64.p, s);
  const int nb = launch_norm2_64(n, b, c->partials.as<double>(), s);
  launch_reduce5(c->partials.as<double>(), nb, c->red.as<double>(), s);
  AC3D_CUDA(cudaMemcpyAsync(&c->h_red[5], c->red.as<double>() + 4, sizeof(double), cudaMemcpyDeviceToHost, s));
  double bn2 = 0.0, rn2 = 0.0;
  int outer = 0, done = 0;
  while (outer < c->max_outer) {
    const double need = outer == 0 ? tol : tol * std::sqrt(bn2 / rn2);
    const double tin = fp64 ? 0.5 * need : std::max(c->inner_tol, 0.3 * need);
    const int it = run_gmres(c, H, c->r64.as<cd>(), (cd*)B.x, tr, tin, &done);  // ends synchronised
    if (outer == 0) bn2 = c->h_red[5];
    c->stats.iterations += it;
    launch_add64(n, x, B.x, s);
    rn2 = reduce_norm2_residual(c, H, tr, b, x, c->r64.as<cd>());
    outer++;
    if (rn2 <= tol * tol * bn2) break;
    if (done == 3) break;  // non-finite values: no further cycle can help
  }
  c->stats.outer_steps += outer;
  c->stats.rel_residual = bn2 > 0 ? std::sqrt(rn2 / bn2) : 0.0;
  if (rn2 > tol * tol * bn2) c->stats.converged = 0;
}

void solve_impl(ac3d_ctx* c, DevHMat& H, const cd* b, cd* x, bool tr) {
  cudaStream_t s = c->stream;
  ensure_work(c);
  const int n = c->m->Ne;
  const double tol = c->solver_tol;
  int done = 0;
  if (c->krylov == AC3D_KRYLOV_GMRES) {
    solve_gmres(c, H, b, x, tr);
    return;
  }
  if (H.prec == PREC_FP64) {
    KrylovBufs B = bufs(c, 1);
    launch_copy64(n, b, B.b, s);
    int it = run_krylov(c, H, B, tr, 1, tol, &done);
    launch_copy64(n, B.x, x, s);
    c->stats.iterations += it;
    c->stats.outer_steps += 1;
    // final true residual, FP64
    double rn2 = reduce_norm2_residual(c, H, tr, b, x, c->r64.as<cd>());
    int np = launch_norm2_64(n, b, c->partials.as<double>(), s);
    launch_reduce5(c->partials.as<double>(), np, c->red.as<double>(), s);
    AC3D_CUDA(cudaMemcpyAsync(c->h_red, c->red.p, 5 * sizeof(double), cudaMemcpyDeviceToHost, s));
    AC3D_CUDA(cudaStreamSynchronize(s));
    double b2 = c->h_red[4];
    c->stats.rel_residual = b2 > 0 ? std::sqrt(rn2 / b2) : 0.0;
    if (done != 1) c->stats.converged = 0;
    return;
  }
  // mixed precision: inner BiCGSTAB with FP64 vectors and scalars on the FP32 H-matrix (FP32
  // matvec arithmetic on FP32 shadows of p and s), inside FP64 iterative refinement
  KrylovBufs B = bufs(c, 2);
  launch_zero64(n, x, s);
  // x = 0: the first residual is b itself. |b|^2 is read back without a wait (the first inner
  // tolerance does not depend on it), so the host captures the inner solve's graph while the
  // device still runs the assembly.
  launch_copy64(n, b, c->r64.p, s);
  const int nb = launch_norm2_64(n, b, c->partials.as<double>(), s);
  launch_reduce5(c->partials.as<double>(), nb, c->red.as<double>(), s);
  AC3D_CUDA(cudaMemcpyAsync(&c->h_red[5], c->red.as<double>() + 4, sizeof(double), cudaMemcpyDeviceToHost, s));
  double bn2 = 0.0, rn2 = 0.0;
  int outer = 0;
  while (outer < c->max_outer) {
    launch_copy64(n, c->r64.p, B.b, s);
    const double need = outer == 0 ? tol : tol * std::sqrt(bn2 / rn2);
    const double tin = std::max(c->inner_tol, 0.3 * need);
    int it = run_krylov(c, H, B, tr, 2, tin, &done);  // ends with the stream synchronised
    if (outer == 0) bn2 = c->h_red[5];
    c->stats.iterations += it;
    launch_add64(n, x, B.x, s);
    rn2 = reduce_norm2_residual(c, H, tr, b, x, c->r64.as<cd>());
    outer++;
    if (rn2 <= tol * tol * bn2) break;
    if (done == 3 && it == 0) break;
  }
  c->stats.outer_steps += outer;
  c->stats.rel_residual = bn2 > 0 ? std::sqrt(rn2 / bn2) : 0.0;
  if (rn2 > tol * tol * bn2) c->stats.converged = 0;
}

// ------------------------------------------------------------------------------------------
// Block solve: up to 16 right-hand sides of one H-matrix (FP32 storage), FP32 block BiCGSTAB
// inside per-column FP64 iterative refinement. b64 / x64: element-major Ne x nrb complex FP64.
// ------------------------------------------------------------------------------------------
struct BlockWork {
  DevBuf kv, parts, vparts, red, tick, pbuf, tbuf, tolb, state, r64, xcol, bcol, rcol, zcol;
};

int run_block_krylov(ac3d_ctx* c, const DevHMat& H, const MultiBufs& B, std::vector<int>& done) {
  cudaStream_t s = c->stream;
  const int maxit = c->maxit > 0 ? c->maxit : 2 * B.n;
  mkrylov_enqueue_init(B, maxit, s);
  {
    CapturedGraph g(s, &c->stats.ms_graph, [&] { mkrylov_enqueue_iterations(B, c->m->DP, H, c->chunk, s); });
    int head[4] = {0, 0, 0, 0};  // iter, maxit, done_all, nrb
    const int max_launch = maxit / c->chunk + 2;
    for (int launched = 0; launched < max_launch; launched++) {
      g.launch();
      AC3D_CUDA(cudaMemcpyAsync(head, B.state, sizeof(head), cudaMemcpyDeviceToHost, s));
      AC3D_CUDA(cudaStreamSynchronize(s));
      if (head[2]) break;
    }
  }
  KStateM st;
  AC3D_CUDA(cudaMemcpy(&st, B.state, sizeof(KStateM), cudaMemcpyDeviceToHost));
  done.assign(B.nrb, 0);
  for (int j = 0; j < B.nrb; j++) done[j] = st.col[j].done;
  c->stats.matvecs += 2 * st.iter;
  return st.iter;
}

// One batch of GMRES cycles, one per column of the FP32 block right-hand side B.b (element-major,
// tolerances B.tol): every iteration is one block matvec of all the columns' inputs, then each
// column's Gram-Schmidt passes. Writes the FP32 block solution B.x; per-column done codes in
// `done`. Returns the iterations of the longest cycle.
int run_block_gmres(ac3d_ctx* c, const DevHMat& H, const MultiBufs& B, std::vector<int>& done) {
  cudaStream_t s = c->stream;
  GmresBufs G = gmres_bufs(c, H, B.b, B.nrb);
  G.b32 = 1;
  G.tolv = B.tol;
  G.q = B.p;   // block vectors of the block solver, free during a GMRES batch
  G.W = B.v;
  G.W2 = B.s;  // nrb columns of n
  gmres_reset(G, s);
  gmres_enqueue_init(G, 1.0, s);
  {
    CapturedGraph g(s, &c->stats.ms_graph, [&] { gmres_enqueue_iterations_block(G, B, c->m->DP, H, c->gm_chunk, s); });
    const int max_launch = (G.m + c->gm_chunk - 1) / c->gm_chunk + 1;
    GMulti gm{};
    for (int launched = 0; launched < max_launch; launched++) {
      g.launch();
      AC3D_CUDA(cudaMemcpyAsync(&gm, G.gm, sizeof(GMulti), cudaMemcpyDeviceToHost, s));
      AC3D_CUDA(cudaStreamSynchronize(s));
      if (gm.done_all) break;
    }
  }
  gmres_enqueue_finish(G, B.x, s);
  std::vector<GState> st(G.nrb);
  GMulti gmf{};
  AC3D_CUDA(cudaMemcpyAsync(st.data(), G.state, G.nrb * sizeof(GState), cudaMemcpyDeviceToHost, s));
  AC3D_CUDA(cudaMemcpyAsync(&gmf, G.gm, sizeof(GMulti), cudaMemcpyDeviceToHost, s));
  AC3D_CUDA(cudaStreamSynchronize(s));
  if (gmf.bar_fail) throw Error(AC3D_ERR_CUDA, "GMRES Gram-Schmidt grid barrier timed out (bounded wait)");
  done.assign(G.nrb, 0);
  int iters = 0;
  for (int j = 0; j < G.nrb; j++) {
    done[j] = st[j].done;
    iters = std::max(iters, st[j].j);
  }
  c->stats.matvecs += iters;
  return iters;
}

// |b - A x|^2 of one column (contiguous FP64 vectors) with the double-float residual matvec
double column_residual2(ac3d_ctx* c, const DevHMat& H, bool tr, const cd* b, const cd* x, cd* r) {
  return reduce_norm2_residual(c, H, tr, b, x, r);
}

double column_norm2(ac3d_ctx* c, const cd* v) {
  cudaStream_t s = c->stream;
  const int np = launch_norm2_64(c->m->Ne, v, c->partials.as<double>(), s);
  launch_reduce5(c->partials.as<double>(), np, c->red.as<double>(), s);
  AC3D_CUDA(cudaMemcpyAsync(c->h_red, c->red.p, 5 * sizeof(double), cudaMemcpyDeviceToHost, s));
  AC3D_CUDA(cudaStreamSynchronize(s));
  return c->h_red[4];
}

// Block vectors and reduction buffers of one block solve (or block matvec timing) in W.
MultiBufs block_bufs(ac3d_ctx* c, DevHMat& H, int nrb, BlockWork& W, bool tr) {
  cudaStream_t s = c->stream;
  ensure_work(c);
  prepare_multi_kernels();
  if (tr) ensure_near_transposed(c->m->DP, H, s);
  const int n = c->m->Ne, nleaf = c->m->DP.nleaf;
  if (c->block_tc && nrb >= 8 && c->m->DP.max_leaf <= 32 && !(tr ? H.tcseg_f.p : H.tcseg_t.p)) {
    // byte offsets of the split dot-pass segments: V by column leaf (A), U by row leaf (A^T)
    const Partition& P = c->m->P;
    const std::vector<int>& ptr = tr ? P.fw_lr_ptr : P.tr_lr_ptr;
    const std::vector<int>& items = tr ? P.fw_lr : P.tr_lr;
    std::vector<long long> off(nleaf + 1, 0);
    for (int l = 0; l < nleaf; l++) {
      int K = 0;
      for (int it = ptr[l]; it < ptr[l + 1]; it++) K += H.ranks_host[items[it]];
      K += K & 1;
      off[l + 1] = off[l] + tc_segment_bytes(P.leaf_start[l + 1] - P.leaf_start[l], K);
    }
    build_tc_segments(c->m->DP, H, tr, off, s);
    c->stats.hmat_bytes = (long long)H.bytes();  // the split segments are part of the H-matrix's footprint
  }
  const size_t blk32 = (size_t)n * nrb * sizeof(cf);
  W.kv.ensure(8 * blk32, s);
  MultiBufs B;
  B.n = n;
  B.nrb = nrb;
  B.tr = tr;
  B.tc = c->block_tc;
  void** slots[8] = {&B.b, &B.x, &B.r, &B.rhat, &B.p, &B.v, &B.s, &B.t};
  for (int i = 0; i < 8; i++) *slots[i] = (char*)W.kv.p + (size_t)i * blk32;
  W.parts.ensure((size_t)(std::max(nleaf, 1184) + 1024) * 5 * nrb * sizeof(double), s);
  W.vparts.ensure((size_t)(1184 + 64 + 1) * 5 * nrb * sizeof(double), s);
  W.red.ensure((size_t)5 * nrb * sizeof(double), s);
  if (!W.tick.p) {
    W.tick.alloc((1024 + 64) * sizeof(unsigned), s);
    AC3D_CUDA(cudaMemsetAsync(W.tick.p, 0, (1024 + 64) * sizeof(unsigned), s));
  }
  W.pbuf.ensure(std::max<size_t>(H.pbuf.bytes / sizeof(cd), 1) * nrb * sizeof(cf), s);
  W.tbuf.ensure((size_t)std::max<int64_t>(H.task_cap, 1) * nrb * sizeof(cf), s);
  W.tolb.ensure((size_t)nrb * sizeof(double), s);
  W.state.ensure(sizeof(KStateM), s);
  B.partials = W.parts.as<double>();
  B.vpartials = W.vparts.as<double>();
  B.red = W.red.as<double>();
  B.ticket = W.tick.as<unsigned>();
  B.pbuf = W.pbuf.p;
  B.tbuf = W.tbuf.p;
  B.tol = W.tolb.as<double>();
  B.state = W.state.as<KStateM>();
  return B;
}

void solve_block(ac3d_ctx* c, DevHMat& H, int nrb, int nr, const cd* b64, cd* x64, BlockWork& W, bool tr = false) {
  cudaStream_t s = c->stream;
  MultiBufs B = block_bufs(c, H, nrb, W, tr);
  const int n = c->m->Ne;
  W.r64.ensure((size_t)n * nrb * sizeof(cd), s);
  for (DevBuf* b : {&W.xcol, &W.bcol, &W.rcol, &W.zcol}) b->ensure((size_t)n * sizeof(cd), s);
  AC3D_CUDA(cudaMemsetAsync(W.zcol.p, 0, (size_t)n * sizeof(cd), s));

  const double tol = c->solver_tol;
  AC3D_CUDA(cudaMemsetAsync(x64, 0, (size_t)n * nrb * sizeof(cd), s));
  AC3D_CUDA(cudaMemcpyAsync(W.r64.p, b64, (size_t)n * nrb * sizeof(cd), cudaMemcpyDeviceToDevice, s));
  std::vector<double> bn2(nrb, 0.0), rn2(nrb, 0.0);
  for (int j = 0; j < nr; j++) {
    launch_block_get(n, nrb, j, b64, W.bcol.p, s);
    bn2[j] = rn2[j] = column_norm2(c, W.bcol.as<cd>());
  }
  int outer = 0, iters = 0;
  std::vector<int> done;
  std::vector<double> tin(nrb, 1.0);
  while (outer < c->max_outer) {
    bool any = false;
    for (int j = 0; j < nrb; j++) {
      const bool act = j < nr && rn2[j] > tol * tol * bn2[j];
      if (act) {
        any = true;
        tin[j] = std::max(c->inner_tol, 0.3 * tol * std::sqrt(bn2[j] / rn2[j]));
      } else {
        tin[j] = 1.0;
        launch_block_set(n, nrb, j, W.zcol.p, W.r64.p, s);  // converged or padding: zero right-hand side
      }
    }
    if (!any) break;
    AC3D_CUDA(cudaMemcpyAsync(W.tolb.p, tin.data(), nrb * sizeof(double), cudaMemcpyHostToDevice, s));
    launch_to32(n * nrb, W.r64.p, B.b, s);
    iters += c->krylov == AC3D_KRYLOV_GMRES ? run_block_gmres(c, H, B, done) : run_block_krylov(c, H, B, done);
    launch_add32(n * nrb, x64, B.x, s);
    for (int j = 0; j < nr; j++) {
      if (!(rn2[j] > tol * tol * bn2[j])) continue;
      launch_block_get(n, nrb, j, x64, W.xcol.p, s);
      launch_block_get(n, nrb, j, b64, W.bcol.p, s);
      rn2[j] = column_residual2(c, H, tr, W.bcol.as<cd>(), W.xcol.as<cd>(), W.rcol.as<cd>());
      launch_block_set(n, nrb, j, W.rcol.p, W.r64.p, s);
    }
    outer++;
  }
  check_pipeline(c, H);
  c->stats.iterations += iters;
  c->stats.outer_steps += outer;
  double worst = 0;
  for (int j = 0; j < nr; j++) {
    const double rr = bn2[j] > 0 ? std::sqrt(rn2[j] / bn2[j]) : 0.0;
    worst = std::max(worst, rr);
    if (rn2[j] > tol * tol * bn2[j]) c->stats.converged = 0;
  }
  c->stats.rel_residual = std::max(c->stats.rel_residual, worst);
  c->stats.solves += nr;
}

// ------------------------------------------------------------------------------------------
// Geometry / mesh
// ------------------------------------------------------------------------------------------
void upload_points(MeshState& m, const std::vector<double>& Ps, cudaStream_t s) {
  m.G.P.ensure(Ps.size() * sizeof(double), s);
  AC3D_CUDA(cudaMemcpyAsync(m.G.P.p, Ps.data(), Ps.size() * sizeof(double), cudaMemcpyHostToDevice, s));
  launch_geometry(m.G, s);
}

void ensure_base_geometry(ac3d_ctx* c) {
  if (!c->m->geom_base) {
    upload_points(*c->m, c->m->Ps0, c->stream);
    c->m->geom_base = true;
  }
}

std::vector<double> heights_to_points(ac3d_ctx* c, const double* x) {
  std::vector<double> Ps = c->m->Ps0;
  if (x)
    for (const auto& kv : c->Hs) Ps[3 * (size_t)kv.first + 1] = x[kv.second] + c->m->Ps0[3 * (size_t)kv.first + 1];
  return Ps;
}

void upload_receivers(ac3d_ctx* c, const double* L, int n, DevBuf& dst) {
  std::vector<double> v(4 * (size_t)n);
  for (int i = 0; i < n; i++) {
    v[4 * i] = L[3 * i];
    v[4 * i + 1] = L[3 * i + 1];
    v[4 * i + 2] = L[3 * i + 2];
    v[4 * i + 3] = 0;
  }
  upload(dst, v, c->stream);
}

// Receiver matrix by ACA (reference mode, compute_ACA_listener, aca.cpp:84-134).
struct ListenerLR {
  DevBuf pool, toff, rank, used, blk, ord, pts, t;
  int L = 0, iter_lim = 0;
  int prec = PREC_MIXED;  // precision of the stored terms (the apply's arithmetic)
};

std::unique_ptr<ListenerLR> listener_lr(ac3d_ctx* c, double k, const double* Lh, int L) {
  cudaStream_t s = c->stream;
  auto Q = std::make_unique<ListenerLR>();
  Q->L = L;
  const int maxk = 5000;  // Q_ACA_MAX_K (constants.h:17)
  Q->iter_lim = std::max(1, std::min(maxk, std::min(L - 1, c->m->Ne - 1)));
  // mixed precision with the double-float assembly: receiver ACA in double-float, terms in FP64
  const bool df = c->prec != PREC_FP64 && c->assembly == AC3D_ASSEMBLY_DF;
  Q->prec = df ? PREC_FP64 : c->prec;
  const size_t cs = Q->prec == PREC_FP64 ? sizeof(cd) : sizeof(cf);
  const long long cap = (long long)Q->iter_lim * (L + c->m->Ne);
  Q->pool.alloc((size_t)cap * cs, s);
  Q->toff.alloc((size_t)Q->iter_lim * sizeof(long long), s);
  Q->rank.alloc(sizeof(int), s);
  Q->used.alloc(16, s);
  Q->t.alloc((size_t)Q->iter_lim * sizeof(cd), s);
  AC3D_CUDA(cudaMemsetAsync(Q->used.p, 0, 16, s));
  upload(Q->blk, std::vector<int>{0, L, 0, c->m->Ne}, s);
  upload(Q->ord, std::vector<int>{0}, s);
  if (df) {
    std::vector<float> v(8 * (size_t)L, 0.f);
    for (int i = 0; i < L; i++)
      for (int d = 0; d < 3; d++) {
        const float hi = (float)Lh[3 * i + d];
        v[8 * i + 2 * d] = hi;
        v[8 * i + 2 * d + 1] = (float)(Lh[3 * i + d] - (double)hi);
      }
    upload(Q->pts, v, s);
    launch_listener_aca_df(c->m->G, Q->pts.p, L, k, c->q_tol, maxk, Q->pool.p, cap, Q->used.as<unsigned long long>(),
                           Q->toff.as<long long>(), Q->rank.as<int>(), (int*)(Q->used.as<unsigned long long>() + 1),
                           Q->blk.as<int4>(), Q->ord.as<int>(), s);
    return Q;
  }
  if (c->prec == PREC_FP64) {
    std::vector<double> v(4 * (size_t)L);
    for (int i = 0; i < L; i++)
      for (int d = 0; d < 3; d++) v[4 * i + d] = Lh[3 * i + d];
    upload(Q->pts, v, s);
  } else {
    std::vector<float> v(4 * (size_t)L, 0.f);
    for (int i = 0; i < L; i++)
      for (int d = 0; d < 3; d++) v[4 * i + d] = (float)Lh[3 * i + d];
    upload(Q->pts, v, s);
  }
  launch_listener_aca(c->m->G, c->prec, Q->pts.p, L, k, c->q_tol, maxk, Q->pool.p, cap,
                      Q->used.as<unsigned long long>(), Q->toff.as<long long>(), Q->rank.as<int>(),
                      (int*)(Q->used.as<unsigned long long>() + 1), Q->blk.as<int4>(), Q->ord.as<int>(), s);
  return Q;
}

void listener_apply(ac3d_ctx* c, const ListenerLR& Q, const cd* in, cd* out, bool trans) {
  launch_lr_apply(Q.prec, Q.pool.p, Q.toff.as<long long>(), Q.rank.as<int>(), Q.iter_lim, Q.L, c->m->Ne, in,
                  trans ? 1 : 0, Q.t.as<cd>(), out, c->stream);
}

// One frequency: assemble, solve -b, receivers. Keeps H if `keep`.
std::unique_ptr<DevHMat> forward_one(ac3d_ctx* c, double f, const double4* recv, const double* Lh, int L, cd* x_out,
                                     cd* y_out, bool keep, std::unique_ptr<ListenerLR>* q_keep) {
  cudaStream_t s = c->stream;
  const double k = wavenumber(f);
  GpuTimer ta(s);
  auto H = assemble(c, k, c->prec);
  c->stats.ms_assemble += ta.stop();
  ensure_work(c);
  // b = -incident field (the system is (K - I/2) x = -b, adjoint.cpp:95)
  GpuTimer ts(s);
  launch_rhs(c->m->G, 1, k, c->src_kind, c->src, c->b64.p, s);
  launch_negate64(c->m->Ne, c->b64.p, s);
  solve(c, *H, c->b64.as<cd>(), x_out, false);
  c->stats.solves++;
  c->stats.ms_solve += ts.stop();
  if (y_out) {
    GpuTimer tl(s);
    if (c->listener_mode == AC3D_LISTENER_ACA) {
      auto Q = listener_lr(c, k, Lh, L);
      listener_apply(c, *Q, x_out, y_out, false);
      if (q_keep) *q_keep = std::move(Q);
    } else {
      launch_far_field(c->m->G, c->prec, recv, L, k, x_out, y_out, c->ff_scratch, s);
    }
    c->stats.ms_listener += tl.stop();
  }
  if (!keep) H.reset();
  return H;
}

// bem3d::gradient (adjoint.cpp:24-242) for one band at the geometry currently on the device.
double band_eval(ac3d_ctx* c, double band, bool forward_only, double* grad_dev) {
  cudaStream_t s = c->stream;
  const int L = (int)c->Ls.size() / 3;
  const int n = c->m->Ne;
  auto freqs = frequencies(band, c->n_freqs);
  const int F = (int)freqs.size();
  DevBuf xs, ys, yt, u, coef, vf, adjb, lmb;
  xs.alloc((size_t)F * n * sizeof(cd), s);
  ys.alloc((size_t)F * L * sizeof(cd), s);
  yt.alloc((size_t)L * sizeof(double), s);
  u.alloc((size_t)L * sizeof(double), s);
  coef.alloc(16, s);
  AC3D_CUDA(cudaMemsetAsync(yt.p, 0, (size_t)L * sizeof(double), s));
  std::vector<std::unique_ptr<DevHMat>> saved(F);
  std::vector<std::unique_ptr<ListenerLR>> savedQ(F);
  const bool keep = !forward_only && !c->recompute;
  for (int fi = 0; fi < F; fi++) {
    cd* xf = xs.as<cd>() + (size_t)fi * n;
    cd* yf = ys.as<cd>() + (size_t)fi * L;
    saved[fi] = forward_one(c, freqs[fi], c->Ls_dev.as<double4>(), c->Ls.data(), L, xf, yf, keep,
                            keep ? &savedQ[fi] : nullptr);
    launch_accum_abs(yf, L, yt.as<double>(), s);
  }
  launch_compute_u(yt.as<double>(), L, u.as<double>(), coef.as<double>(), s);
  double cval = 0;
  AC3D_CUDA(cudaMemcpyAsync(&cval, coef.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  AC3D_CUDA(cudaStreamSynchronize(s));
  if (forward_only) return cval;

  GpuTimer tadj(s);
  vf.alloc((size_t)L * sizeof(cd), s);
  adjb.alloc((size_t)n * sizeof(cd), s);
  lmb.alloc((size_t)n * sizeof(cd), s);
  for (int fi = 0; fi < F; fi++) {
    const double k = wavenumber(freqs[fi]);
    cd* xf = xs.as<cd>() + (size_t)fi * n;
    cd* yf = ys.as<cd>() + (size_t)fi * L;
    launch_vf(u.as<double>(), yf, L, vf.as<cd>(), s);
    if (c->listener_mode == AC3D_LISTENER_ACA) {
      std::unique_ptr<ListenerLR> Q = std::move(savedQ[fi]);
      if (!Q) Q = listener_lr(c, k, c->Ls.data(), L);  // recompute (adjoint.cpp:177-178)
      listener_apply(c, *Q, vf.as<cd>(), adjb.as<cd>(), true);
    } else {
      launch_far_field_t(c->m->G, c->prec, c->Ls_dev.as<double4>(), L, k, vf.as<cd>(), adjb.as<cd>(), s);
    }
    std::unique_ptr<DevHMat> H = std::move(saved[fi]);
    if (!H) H = assemble(c, k, c->prec);  // recompute_matrices (adjoint.cpp:173-195)
    solve(c, *H, adjb.as<cd>(), lmb.as<cd>(), true);
    c->stats.solves++;
    H.reset();
    AdjointArgs a{};
    a.prec = c->prec;
    a.k = k;
    a.npairs = (int)c->pair_elem.size();
    a.pair_elem = c->d_pair_elem.as<int>();
    a.pair_corner = c->d_pair_corner.as<int>();
    a.ntouch = (int)c->touch.size();
    a.touch_elem = c->d_touch.as<int>();
    a.pair_touch = c->d_pair_touch.as<int>();
    a.recv = c->Ls_dev.as<double4>();
    a.L = L;
    a.vf = vf.as<cd>();
    a.x = xf;
    a.lmb = lmb.as<cd>();
    a.rhs_kind = c->src_kind;
    for (int d = 0; d < 3; d++) a.rhs_v[d] = c->src[d];
    a.h_off = c->d_h_off.as<int>();
    a.HH = (int)c->h_off.size() - 1;
    a.grad = grad_dev;
    launch_adjoint_terms(c->m->G, a, c->adj_scratch, s);
  }
  AC3D_CUDA(cudaStreamSynchronize(s));
  c->stats.ms_adjoint += tadj.stop();
  return cval;
}

// Loss 1 - mean_{f, d} c(f, d) over the frequencies and plane-wave directions d, c(f, d) the
// diffusion coefficient of the context's receivers for the one frequency f (compute_u,
// adjoint.cpp:388-397, of |y|); grad_dev (HH) += d loss / d heights. Per frequency one H-matrix
// serves every direction: forward block solves, per-direction receivers and adjoint right-hand
// sides, transposed block solves, then the shape-derivative terms of all directions in batches
// that share each derivative evaluation (adjoint.cpp:24-242 per direction, with the sign and
// weight of the mean). coefs receives c(f, d), frequency-major.
double multi_eval(ac3d_ctx* c, const std::vector<double>& freqs, const std::vector<double>& dirs, double* grad_dev,
                  std::vector<double>& coefs) {
  cudaStream_t s = c->stream;
  const int L = (int)c->Ls.size() / 3;
  const int n = c->m->Ne;
  const int F = (int)freqs.size(), D = (int)dirs.size() / 3;
  const bool fp64 = c->prec == AC3D_PREC_FP64;
  const double wgt = -1.0 / ((double)F * D);
  DevBuf X, LMB, Y, VF, ADJ, yt, u, coef, b64, x64;
  X.alloc((size_t)D * n * sizeof(cd), s);
  LMB.alloc((size_t)D * n * sizeof(cd), s);
  ADJ.alloc((size_t)D * n * sizeof(cd), s);
  Y.alloc((size_t)D * L * sizeof(cd), s);
  VF.alloc((size_t)D * L * sizeof(cd), s);
  yt.alloc((size_t)L * sizeof(double), s);
  u.alloc((size_t)L * sizeof(double), s);
  coef.alloc((size_t)F * D * sizeof(double), s);
  ensure_work(c);
  BlockWork W;
  // op(A) Z = B for the D columns of B (direction-major, n each), in batches of kMaxRhs
  auto solve_all = [&](const cd* Bm, cd* Z, DevHMat& H, bool tr) {
    for (int start = 0; start < D; start += kMaxRhs) {
      const int nr = std::min(kMaxRhs, D - start);
      if (fp64) {  // FP64 storage: one right-hand side at a time through the FP64 solver
        for (int j = 0; j < nr; j++) {
          solve(c, H, Bm + (size_t)(start + j) * n, Z + (size_t)(start + j) * n, tr);
          c->stats.solves++;
        }
        continue;
      }
      const int nrb = nr <= 4 ? 4 : nr <= 8 ? 8 : 16;
      b64.ensure((size_t)n * nrb * sizeof(cd), s);
      x64.ensure((size_t)n * nrb * sizeof(cd), s);
      AC3D_CUDA(cudaMemsetAsync(b64.p, 0, (size_t)n * nrb * sizeof(cd), s));
      for (int j = 0; j < nr; j++) launch_block_set(n, nrb, j, Bm + (size_t)(start + j) * n, b64.p, s);
      solve_block(c, H, nrb, nr, b64.as<cd>(), x64.as<cd>(), W, tr);
      for (int j = 0; j < nr; j++) launch_block_get(n, nrb, j, x64.p, Z + (size_t)(start + j) * n, s);
    }
  };
  for (int fi = 0; fi < F; fi++) {
    const double k = wavenumber(freqs[fi]);
    GpuTimer ta(s);
    auto H = assemble(c, k, c->prec);
    c->stats.ms_assemble += ta.stop();
    // forward: b = -incident field (adjoint.cpp:95), one column per direction
    GpuTimer ts(s);
    for (int d = 0; d < D; d++) {
      launch_rhs(c->m->G, 1, k, AC3D_INCIDENT_PLANE, &dirs[3 * d], ADJ.as<cd>() + (size_t)d * n, s);
      launch_negate64(n, ADJ.as<cd>() + (size_t)d * n, s);
    }
    solve_all(ADJ.as<cd>(), X.as<cd>(), *H, false);
    c->stats.ms_solve += ts.stop();
    // receivers, coefficient and adjoint right-hand side of each direction (adjoint.cpp:101-178)
    GpuTimer tadj(s);
    std::unique_ptr<ListenerLR> Q;
    if (c->listener_mode == AC3D_LISTENER_ACA) Q = listener_lr(c, k, c->Ls.data(), L);
    for (int d = 0; d < D; d++) {
      cd* xd = X.as<cd>() + (size_t)d * n;
      cd* yd = Y.as<cd>() + (size_t)d * L;
      cd* vfd = VF.as<cd>() + (size_t)d * L;
      if (Q)
        listener_apply(c, *Q, xd, yd, false);
      else
        launch_far_field(c->m->G, c->prec, c->Ls_dev.as<double4>(), L, k, xd, yd, c->ff_scratch, s);
      AC3D_CUDA(cudaMemsetAsync(yt.p, 0, (size_t)L * sizeof(double), s));
      launch_accum_abs(yd, L, yt.as<double>(), s);
      launch_compute_u(yt.as<double>(), L, u.as<double>(), coef.as<double>() + (size_t)fi * D + d, s);
      launch_vf(u.as<double>(), yd, L, vfd, s);
      if (Q)
        listener_apply(c, *Q, vfd, ADJ.as<cd>() + (size_t)d * n, true);
      else
        launch_far_field_t(c->m->G, c->prec, c->Ls_dev.as<double4>(), L, k, vfd, ADJ.as<cd>() + (size_t)d * n, s);
    }
    solve_all(ADJ.as<cd>(), LMB.as<cd>(), *H, true);
    H.reset();
    // shape-derivative terms, all directions of a batch per derivative evaluation
    const int batch = kAdjMaxRhs;
    for (int start = 0; start < D; start += batch) {
      AdjointMultiArgs a{};
      a.prec = c->prec;
      a.k = k;
      a.npairs = (int)c->pair_elem.size();
      a.pair_elem = c->d_pair_elem.as<int>();
      a.pair_corner = c->d_pair_corner.as<int>();
      a.ntouch = (int)c->touch.size();
      a.touch_elem = c->d_touch.as<int>();
      a.pair_touch = c->d_pair_touch.as<int>();
      a.recv = c->Ls_dev.as<double4>();
      a.L = L;
      a.nr = std::min(batch, D - start);
      a.vf = VF.as<cd>() + (size_t)start * L;
      a.x = X.as<cd>() + (size_t)start * n;
      a.lmb = LMB.as<cd>() + (size_t)start * n;
      for (int r = 0; r < a.nr; r++) {
        for (int q = 0; q < 3; q++) a.dir[r][q] = dirs[3 * (start + r) + q];
        a.w[r] = wgt;
      }
      a.h_off = c->d_h_off.as<int>();
      a.HH = (int)c->h_off.size() - 1;
      a.grad = grad_dev;
      launch_adjoint_terms_multi(c->m->G, a, c->adj_scratch, s);
    }
    AC3D_CUDA(cudaStreamSynchronize(s));
    c->stats.ms_adjoint += tadj.stop();
  }
  coefs.assign((size_t)F * D, 0.0);
  AC3D_CUDA(cudaMemcpyAsync(coefs.data(), coef.p, (size_t)F * D * sizeof(double), cudaMemcpyDeviceToHost, s));
  AC3D_CUDA(cudaStreamSynchronize(s));
  double mean = 0;
  for (double v : coefs) mean += v;
  return 1.0 - mean / ((double)F * D);
}

void reset_stats(ac3d_ctx* c) {
  ac3d_stats z{};
  z.n_elements = c->m->Ne;
  z.n_direct = c->m->DP.nd;
  z.n_approx = c->m->DP.na;
  z.n_leaves = c->m->DP.nleaf;
  z.converged = 1;
  c->stats = z;
}

template <typename F>
int guard(ac3d_ctx* c, F&& f) {
  if (!c) return AC3D_ERR_ARG;
  try {
    c->err.clear();
    auto t0 = std::chrono::steady_clock::now();
    const long long l0 = t_kernel_launches;
    f();
    c->stats.ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    c->stats.kernel_launches = t_kernel_launches - l0;
    return AC3D_OK;
  } catch (const Error& e) {
    c->err = e.what();
    if (e.code == AC3D_ERR_CUDA) cudaGetLastError();
    return e.code;
  } catch (const std::exception& e) {
    c->err = e.what();
    return AC3D_ERR_INTERNAL;
  }
}


// Tree, partition and geometry of a mesh (DiffBEM::set_mesh, acoustics3d.cpp:36-67), built with
// its device arrays on stream s (synchronised before returning).
std::shared_ptr<MeshState> build_mesh_state(const double* Ps, int V, const int32_t* Es, int Ne, int cluster_size,
                                            double radius_factor, int maxk, cudaStream_t s) {
  for (int i = 0; i < 3 * Ne; i++)
    if (Es[i] < 0 || Es[i] >= V) {
      throw Error(AC3D_ERR_ARG, "element index out of range");
    }
  for (int i = 0; i < 3 * V; i++)
    if (!std::isfinite(Ps[i])) {
      throw Error(AC3D_ERR_ARG, "non-finite vertex coordinate");
    }
  auto ms = std::make_shared<MeshState>();
  MeshState* mp = ms.get();
  {
    mp->V = V;
    mp->Ne = Ne;
    mp->Ps0.assign(Ps, Ps + 3 * (size_t)V);
    // centroids in the input order (compute_centers, helpers.cpp:7-14)
    std::vector<double> C(3 * (size_t)Ne);
    for (int e = 0; e < Ne; e++)
      for (int d = 0; d < 3; d++)
        C[3 * e + d] = (Ps[3 * Es[3 * e] + d] + Ps[3 * Es[3 * e + 1] + d] + Ps[3 * Es[3 * e + 2] + d]) / 3;
    build_partition(C.data(), Ne, cluster_size, radius_factor, mp->P);
    if (mp->P.max_leaf > 256) throw Error(AC3D_ERR_ARG, "leaf clusters above 256 elements are not supported");
    mp->Es.resize(3 * (size_t)Ne);
    for (int i = 0; i < Ne; i++)
      for (int d = 0; d < 3; d++) mp->Es[3 * i + d] = Es[3 * mp->P.order[i] + d];
    build_leaf_lists(mp->P, maxk);
    // ClusterTree::check (clustertree.cpp:33-47) on the reordered centroids
    for (int e = 0; e < Ne; e++)
      for (int d = 0; d < 3; d++)
        C[3 * e + d] =
            (Ps[3 * mp->Es[3 * e] + d] + Ps[3 * mp->Es[3 * e + 1] + d] + Ps[3 * mp->Es[3 * e + 2] + d]) / 3;
    mp->P.tree_ok = true;
    for (const TreeNode& nd : mp->P.nodes)
      for (int i = nd.s; i < nd.e; i++) {
        double dx = C[3 * i] - nd.c[0], dy = C[3 * i + 1] - nd.c[1], dz = C[3 * i + 2] - nd.c[2];
        if (!(std::sqrt(dx * dx + dy * dy + dz * dz) <= nd.r + 1e-6)) mp->P.tree_ok = false;
      }
    // device partition
    DevPartition& DP = mp->DP;
    DP.ne = Ne;
    DP.nleaf = (int)mp->P.leaf_start.size() - 1;
    DP.nd = (int)mp->P.direct.size() / 4;
    DP.na = (int)mp->P.approx.size() / 4;
    DP.max_leaf = mp->P.max_leaf;
    upload(DP.blocks_d, mp->P.direct, s);
    upload(DP.blocks_a, mp->P.approx, s);
    upload(DP.leaf_start, mp->P.leaf_start, s);
    upload(DP.fw_near_ptr, mp->P.fw_near_ptr, s);
    upload(DP.fw_near, mp->P.fw_near, s);
    upload(DP.fw_lr_ptr, mp->P.fw_lr_ptr, s);
    upload(DP.fw_lr, mp->P.fw_lr, s);
    upload(DP.tr_near_ptr, mp->P.tr_near_ptr, s);
    upload(DP.tr_near, mp->P.tr_near, s);
    upload(DP.tr_lr_ptr, mp->P.tr_lr_ptr, s);
    upload(DP.tr_lr, mp->P.tr_lr, s);
    std::vector<long long> no(mp->P.near_off.begin(), mp->P.near_off.end());
    upload(DP.near_off, no, s);
    {
      // blocks for the CTA kernel first, then the warp kernels by largest side (256, 128, 64), each
      // group by decreasing m + n (longest first)
      std::vector<int> grp[4];
      for (int b : mp->P.aca_order) {
        const int* q = &mp->P.approx[4 * b];
        const int side = std::max(q[1] - q[0], q[3] - q[2]);
        const int g = (side > kWarpAcaMaxDim || maxk > kWarpAcaTerms) ? 0 : side > 128 ? 1 : side > 64 ? 2 : 3;
        grp[g].push_back(b);
      }
      std::vector<int> all;
      for (int g = 0; g < 4; g++) {
        DP.aca_split[g] = (int)grp[g].size();
        all.insert(all.end(), grp[g].begin(), grp[g].end());
      }
      upload(DP.aca_order, all, s);
    }
    upload(DP.near_seg, std::vector<long long>(mp->P.near_seg.begin(), mp->P.near_seg.end()), s);
    upload(DP.near_off_t, std::vector<long long>(mp->P.near_off_t.begin(), mp->P.near_off_t.end()), s);
    upload(DP.near_seg_t, std::vector<long long>(mp->P.near_seg_t.begin(), mp->P.near_seg_t.end()), s);
    upload(DP.didx_t_ptr, mp->P.didx_t_ptr, s);
    upload(DP.didx_t, mp->P.didx_t, s);
    DP.near_total_t = mp->P.near_total_t;
    upload(DP.didx_ptr, mp->P.didx_ptr, s);
    upload(DP.didx, mp->P.didx, s);
    upload(DP.blk_fw_ptr, mp->P.blk_fw_ptr, s);
    upload(DP.blk_fw, mp->P.blk_fw, s);
    upload(DP.blk_tr_ptr, mp->P.blk_tr_ptr, s);
    upload(DP.blk_tr, mp->P.blk_tr, s);
    upload(DP.fw_pos, mp->P.fw_pos, s);
    upload(DP.tr_pos, mp->P.tr_pos, s);
    mp->sum_mn = 0;
    mp->worst_pool = 0;
    for (int b = 0; b < DP.na; b++) {
      const int* q = &mp->P.approx[4 * b];
      int m = q[1] - q[0], n = q[3] - q[2];
      mp->sum_mn += m + n;
      mp->worst_pool += (int64_t)std::max(0, std::min(maxk, std::min(m - 1, n - 1))) * (m + n);
    }
    mp->pool_hint[0] = mp->pool_hint[1] = 0;
    // geometry
    mp->G.ne = Ne;
    mp->G.nv = V;
    upload(mp->G.E, mp->Es, s);
    upload_points(*mp, mp->Ps0, s);
    mp->geom_base = true;
    AC3D_CUDA(cudaStreamSynchronize(s));
  }
  return ms;
}

}  // namespace ac3d

// ============================================================================================
// C-ABI
// ============================================================================================
extern "C" {

const char* ac3d_version(void) { return "acoustic_reliefs_gb300 0.1 (sm_103a)"; }

int ac3d_create(ac3d_ctx** out, int cluster_size, double radius_factor, const double* freq_bands, int n_bands,
                int n_freqs, double approx_aca_tol, double q_aca_tol, double solver_tol, const double* src_pt,
                double listener_radius, double listener_ds, int recompute_matrices) {
  if (!out) return AC3D_ERR_ARG;
  *out = nullptr;
  if (cluster_size < 1 || cluster_size > 256 || n_freqs < 1 || n_bands < 0 || (n_bands > 0 && !freq_bands) ||
      listener_ds <= 0 || !(solver_tol > 0) || !(approx_aca_tol >= 0))
    return AC3D_ERR_ARG;
  ac3d_ctx* c = new ac3d_ctx;
  c->cluster_size = cluster_size;
  c->radius_factor = radius_factor;
  c->bands.assign(freq_bands, freq_bands + n_bands);
  c->n_freqs = n_freqs;
  c->aca_tol = approx_aca_tol;
  c->q_tol = q_aca_tol;
  c->solver_tol = solver_tol;
  if (src_pt)
    for (int d = 0; d < 3; d++) c->src[d] = src_pt[d];
  c->listener_radius = listener_radius;
  c->listener_ds = listener_ds;
  c->recompute = recompute_matrices != 0;
  c->Ls = hemisphere(listener_radius, listener_ds);
  int rc = guard(c, [&] {
    // The context's stream at the highest priority, the assembly kernels on two streams at the
    // lowest: when several contexts share the GPU (the request server), the latency-bound solve
    // kernels of one request take SMs as they free up ahead of the compute-bound ACA blocks of
    // another. Within one context the streams are ordered by events as before.
    int prio_low = 0, prio_high = 0;
    AC3D_CUDA(cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high));
    AC3D_CUDA(cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, prio_high));
    AC3D_CUDA(cudaStreamCreateWithPriority(&c->side, cudaStreamNonBlocking, prio_low));
    AC3D_CUDA(cudaStreamCreateWithPriority(&c->asm_s, cudaStreamNonBlocking, prio_low));
    AC3D_CUDA(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
    AC3D_CUDA(cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming));
    AC3D_CUDA(cudaEventCreateWithFlags(&c->ev_join_asm, cudaEventDisableTiming));
    AC3D_CUDA(cudaStreamCreateWithPriority(&c->rot, cudaStreamNonBlocking, prio_high));
    AC3D_CUDA(cudaEventCreateWithFlags(&c->ev_gs, cudaEventDisableTiming));
    AC3D_CUDA(cudaEventCreateWithFlags(&c->ev_rot, cudaEventDisableTiming));
    int dev = 0;
    AC3D_CUDA(cudaGetDevice(&dev));
    cudaMemPool_t pool;
    AC3D_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
    uint64_t thr = UINT64_MAX;
    AC3D_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
    noalloc_prepare();  // ac3d_far_field_noalloc then allocates nothing on this device
    upload_receivers(c, c->Ls.data(), (int)c->Ls.size() / 3, c->Ls_dev);
    AC3D_CUDA(cudaStreamSynchronize(c->stream));
  });
  if (rc != AC3D_OK) {
    delete c;
    return rc;
  }
  *out = c;
  return AC3D_OK;
}

void ac3d_destroy(ac3d_ctx* c) {
  if (!c) return;
  cudaStream_t s = c->stream;
  if (s) cudaStreamSynchronize(s);
  // every device buffer is released on the context stream, so all of them go before the stream
  c->last_H.reset();
  DevBuf* bufs[] = {&c->kv, &c->kv32, &c->partials, &c->kstate, &c->red, &c->b64, &c->x64, &c->r64, &c->ff_scratch,
                    &c->adj_scratch, &c->tmp_recv, &c->Ls_dev, &c->d_h_off, &c->d_pair_elem, &c->d_pair_corner,
                    &c->d_pair_touch, &c->d_touch, &c->gm};
  for (DevBuf* b : bufs) b->release();
  c->m.reset();  // a mesh shared with other contexts stays alive until its last user goes
  c->m_dense.reset();
  for (cudaStream_t* st : {&c->side, &c->asm_s, &c->rot})
    if (*st) {
      cudaStreamSynchronize(*st);
      cudaStreamDestroy(*st);
      *st = nullptr;
    }
  if (c->ev_fork) cudaEventDestroy(c->ev_fork);
  if (c->ev_join) cudaEventDestroy(c->ev_join);
  if (c->ev_join_asm) cudaEventDestroy(c->ev_join_asm);
  if (c->ev_gs) cudaEventDestroy(c->ev_gs);
  if (c->ev_rot) cudaEventDestroy(c->ev_rot);
  if (s) {
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    c->stream = nullptr;
  }
  delete c;
}

int ac3d_select_device(int device) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) {
    cudaGetLastError();
    return AC3D_ERR_ARG;
  }
  return cudaSetDevice(device) == cudaSuccess ? AC3D_OK : AC3D_ERR_CUDA;
}

const char* ac3d_last_error(const ac3d_ctx* c) { return c ? c->err.c_str() : "null context"; }

int ac3d_set_precision(ac3d_ctx* c, int p) {
  if (!c || (p != AC3D_PREC_MIXED && p != AC3D_PREC_FP64)) return AC3D_ERR_ARG;
  c->prec = p;
  return AC3D_OK;
}

int ac3d_set_incident(ac3d_ctx* c, int kind, const double* v) {
  if (!c || !v || (kind != AC3D_INCIDENT_POINT && kind != AC3D_INCIDENT_PLANE)) return AC3D_ERR_ARG;
  c->src_kind = kind;
  double nrm = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  for (int d = 0; d < 3; d++) c->src[d] = kind == AC3D_INCIDENT_PLANE ? v[d] / nrm : v[d];
  return AC3D_OK;
}

int ac3d_set_listener_mode(ac3d_ctx* c, int mode) {
  if (!c || (mode != AC3D_LISTENER_DENSE && mode != AC3D_LISTENER_ACA)) return AC3D_ERR_ARG;
  c->listener_mode = mode;
  return AC3D_OK;
}

int ac3d_set_solver(ac3d_ctx* c, int max_iterations, double inner_tol, int max_outer) {
  if (!c || max_iterations < 0 || !(inner_tol > 0 && inner_tol < 1) || max_outer < 1) return AC3D_ERR_ARG;
  c->maxit = max_iterations;
  c->inner_tol = inner_tol;
  c->max_outer = max_outer;
  return AC3D_OK;
}

int ac3d_set_assembly(ac3d_ctx* c, int mode) {
  if (!c || (mode != AC3D_ASSEMBLY_DF && mode != AC3D_ASSEMBLY_FP32)) return AC3D_ERR_ARG;
  c->assembly = mode;
  return AC3D_OK;
}

int ac3d_set_tensor_cores(ac3d_ctx* c, int on) {
  if (!c) return AC3D_ERR_ARG;
  c->block_tc = on != 0;
  return AC3D_OK;
}

int ac3d_set_krylov(ac3d_ctx* c, int method, int restart) {
  if (!c || (method != AC3D_KRYLOV_BICGSTAB && method != AC3D_KRYLOV_GMRES) || restart < 0 || restart > 600)
    return AC3D_ERR_ARG;
  c->krylov = method;
  c->gm_restart = restart > 0 ? restart : 300;
  return AC3D_OK;
}

int ac3d_set_listeners(ac3d_ctx* c, const double* Ls, int L) {
  if (!c || !Ls || L < 2) return AC3D_ERR_ARG;
  return guard(c, [&] {
    c->Ls.assign(Ls, Ls + 3 * (size_t)L);
    upload_receivers(c, Ls, L, c->Ls_dev);
    AC3D_CUDA(cudaStreamSynchronize(c->stream));
  });
}

int ac3d_set_mesh(ac3d_ctx* c, const double* Ps, int V, const int32_t* Es, int Ne, int32_t* Es_out) {
  if (!c || !Ps || !Es || V < 3 || Ne < 1) return AC3D_ERR_ARG;
  return guard(c, [&] {
    c->mesh_set = false;
    c->diff_set = false;
    c->m_dense.reset();
    c->Ps_in.assign(Ps, Ps + 3 * (size_t)V);
    c->Es_in.assign(Es, Es + 3 * (size_t)Ne);
    std::shared_ptr<MeshState> m = build_mesh_state(Ps, V, Es, Ne, c->cluster_size, c->radius_factor, c->maxk,
                                                    c->stream);
    c->m = std::move(m);
    c->mesh_set = true;
    reset_stats(c);
    if (Es_out) std::memcpy(Es_out, c->m->Es.data(), c->m->Es.size() * sizeof(int32_t));
  });
}

int ac3d_set_diff_points(ac3d_ctx* c, const int32_t* pts, int HH) {
  if (!c || (HH > 0 && !pts) || HH < 0) return AC3D_ERR_ARG;
  return guard(c, [&] {
    require_mesh(c);
    cudaStream_t s = c->stream;
    c->Hs.clear();
    c->diff_pts.assign(pts, pts + HH);
    int h = 0;
    for (int i = 0; i < HH; i++) {
      if (pts[i] < 0 || pts[i] >= c->m->V) throw Error(AC3D_ERR_ARG, "differentiable point index out of range");
      c->Hs[pts[i]] = h++;  // later duplicates overwrite, as std::unordered_map::operator[] does
    }
    // incidence lists (acoustics3d.cpp:79-98): for each element j, corners 0..2
    std::vector<std::vector<std::pair<int, int>>> lists(HH);
    for (int j = 0; j < c->m->Ne; j++)
      for (int o = 0; o < 3; o++) {
        auto it = c->Hs.find(c->m->Es[3 * j + o]);
        if (it != c->Hs.end()) lists[it->second].push_back({j, o});
      }
    c->h_off.assign(HH + 1, 0);
    c->pair_elem.clear();
    c->pair_corner.clear();
    for (int i = 0; i < HH; i++) {
      for (auto& pr : lists[i]) {
        c->pair_elem.push_back(pr.first);
        c->pair_corner.push_back(pr.second);
      }
      c->h_off[i + 1] = (int)c->pair_elem.size();
    }
    std::vector<int> tid(c->m->Ne, -1);
    c->touch.clear();
    c->pair_touch.resize(c->pair_elem.size());
    for (size_t t = 0; t < c->pair_elem.size(); t++) {
      int e = c->pair_elem[t];
      if (tid[e] < 0) {
        tid[e] = (int)c->touch.size();
        c->touch.push_back(e);
      }
      c->pair_touch[t] = tid[e];
    }
    upload(c->d_h_off, c->h_off, s);
    upload(c->d_pair_elem, c->pair_elem, s);
    upload(c->d_pair_corner, c->pair_corner, s);
    upload(c->d_pair_touch, c->pair_touch, s);
    upload(c->d_touch, c->touch, s);
    AC3D_CUDA(cudaStreamSynchronize(s));
    c->diff_set = true;
  });
}

int ac3d_set_band(ac3d_ctx* c, double fb) {
  if (!c) return AC3D_ERR_ARG;
  c->bands.assign(1, fb);
  return AC3D_OK;
}

int ac3d_set_bands(ac3d_ctx* c, const double* fb, int n) {
  if (!c || n < 1 || !fb) return AC3D_ERR_ARG;
  c->bands.assign(fb, fb + n);
  return AC3D_OK;
}

int ac3d_num_listeners(const ac3d_ctx* c, int* L) {
  if (!c || !L) return AC3D_ERR_ARG;
  *L = (int)c->Ls.size() / 3;
  return AC3D_OK;
}

int ac3d_get_listeners(const ac3d_ctx* c, double* out) {
  if (!c || !out) return AC3D_ERR_ARG;
  std::memcpy(out, c->Ls.data(), c->Ls.size() * sizeof(double));
  return AC3D_OK;
}

int ac3d_set_points(ac3d_ctx* c, const double* Ps) {
  if (!c || !Ps) return AC3D_ERR_ARG;
  return guard(c, [&] {
    require_mesh(c);
    c->m->Ps0.assign(Ps, Ps + 3 * (size_t)c->m->V);
    upload_points(*c->m, c->m->Ps0, c->stream);
    c->m->geom_base = true;
  });
}

int ac3d_pressures(ac3d_ctx* c, double f, const double* Ls, int L, double* out) {
  if (!c || !out || !(f > 0) || (Ls && L < 1)) return AC3D_ERR_ARG;
  return guard(c, [&] {
    require_mesh(c);
    reset_stats(c);
    cudaStream_t s = c->stream;
    ensure_base_geometry(c);
    const double4* recv = c->Ls_dev.as<double4>();
    const double* Lh = c->Ls.data();
    int nL = (int)c->Ls.size() / 3;
    if (Ls) {
      Lh = Ls;
      upload_receivers(c, Ls, L, c->tmp_recv);
      recv = c->tmp_recv.as<double4>();
      nL = L;
    }
    ensure_work(c);
    DevBuf y;
    y.alloc((size_t)nL * sizeof(cd), s);
    c->last_H.reset();
    c->last_H = forward_one(c, f, recv, Lh, nL, c->x64.as<cd>(), y.as<cd>(), true);
    AC3D_CUDA(cudaMemcpyAsync(out, y.p, (size_t)nL * sizeof(cd), cudaMemcpyDeviceToHost, s));
    AC3D_CUDA(cudaStreamSynchronize(s));
    if (!c->stats.converged) throw Error(AC3D_ERR_NOT_CONVERGED, not_converged_message(c));
  });
}

int ac3d_pressures_dev(ac3d_ctx* c, double f, const double* Ls_dev, int L, double* out_dev, void* stream) {
  if (!c || !out_dev || !(f > 0) || (Ls_dev && L < 1)) return AC3D_ERR_ARG;
  return guard(c, [&] {
    require_mesh(c);
    if (c->listener_mode == AC3D_LISTENER_ACA && Ls_dev)
      throw Error(AC3D_ERR_ARG, "receiver ACA mode needs host receivers (use ac3d_pressures)");
    reset_stats(c);
    cudaStream_t us = (cudaStream_t)stream;
    cudaStream_t s = c->stream;
    cudaEvent_t ev;
    AC3D_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    AC3D_CUDA(cudaEventRecord(ev, us));
    AC3D_CUDA(cudaStreamWaitEvent(s, ev, 0));
    ensure_base_geometry(c);
    const double4* recv = c->Ls_dev.as<double4>();
    int nL = (int)c->Ls.size() / 3;
    if (Ls_dev) {
      c->tmp_recv.ensure((size_t)L * sizeof(double4), s);
      launch_pack_points(Ls_dev, L, c->tmp_recv.p, s);
      recv = c->tmp_recv.as<double4>();
      nL = L;
    }
    ensure_work(c);
    c->last_H.reset();
    c->last_H = forward_one(c, f, recv, c->Ls.data(), nL, c->x64.as<cd>(), (cd*)out_dev, true);
    AC3D_CUDA(cudaEventRecord(ev, s));
    AC3D_CUDA(cudaStreamWaitEvent(us, ev, 0));
    AC3D_CUDA(cudaEventDestroy(ev));
    if (!c->stats.converged) throw Error(AC3D_ERR_NOT_CONVERGED, not_converged_message(c));
  });
}

int ac3d_solve_multi(ac3d_ctx* c, double f, int kind, const double* vecs, int nrhs, const double* Ls, int L,
                     double* p_out, double* x_out) {
  if (!c || !vecs || nrhs < 1 || !(f > 0) || (kind != AC3D_INCIDENT_POINT && kind != AC3D_INCIDENT_PLANE) ||
      (Ls && L < 1))
    return AC3D_ERR_ARG;
  return guard(c, [&] {
    require_mesh(c);
    if (c->listener_mode == AC3D_LISTENER_ACA && p_out)
      throw Error(AC3D_ERR_ARG, "block solves evaluate receivers exactly (listener mode 'dense')");
    reset_stats(c);
    cudaStream_t s = c->stream;
    ensure_base_geometry(c);
    const double k = wavenumber(f);
    const int n = c->m->Ne;
    GpuTimer ta(s);
    auto H = assemble(c, k, c->prec);
    c->stats.ms_assemble += ta.stop();
    ensure_work(c);
    const double4* recv = c->Ls_dev.as<double4>();
    int nL = (int)c->Ls.size() / 3;
    if (Ls) {
      upload_receivers(c, Ls, L, c->tmp_recv);
      recv = c->tmp_recv.as<double4>();
      nL = L;
    }
    DevBuf ycol, b64, x64;
    ycol.alloc((size_t)nL * sizeof(cd), s);
    BlockWork W;
    GpuTimer ts(s);
    for (int start = 0; start < nrhs; start += kMaxRhs) {
      const int nr = std::min(kMaxRhs, nrhs - start);
      const int nrb = nr <= 4 ? 4 : nr <= 8 ? 8 : 16;
      b64.ensure((size_t)n * nrb * sizeof(cd), s);
      x64.ensure((size_t)n * nrb * sizeof(cd), s);
      AC3D_CUDA(cudaMemsetAsync(b64.p, 0, (size_t)n * nrb * sizeof(cd), s));
      for (int j = 0; j < nr; j++) {
        double v[3];
        const double* w = vecs + 3 * (size_t)(start + j);
        const double nrm = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
        if (kind == AC3D_INCIDENT_PLANE && !(nrm > 0)) throw Error(AC3D_ERR_ARG, "zero plane-wave direction");
        for (int d = 0; d < 3; d++) v[d] = kind == AC3D_INCIDENT_PLANE ? w[d] / nrm : w[d];
        // b = -incident field (adjoint.cpp:95)
        launch_rhs(c->m->G, 1, k, kind, v, c->b64.p, s);
        launch_negate64(n, c->b64.p, s);
        launch_block_set(n, nrb, j, c->b64.p, b64.p, s);
      }
      if (c->prec == AC3D_PREC_FP64) {
        // FP64 storage: one right-hand side at a time through the FP64 solver
        for (int j = 0; j < nr; j++) {
          launch_block_get(n, nrb, j, b64.p, c->b64.p, s);
          solve(c, *H, c->b64.as<cd>(), c->x64.as<cd>(), false);
          c->stats.solves++;
          launch_block_set(n, nrb, j, c->x64.p, x64.p, s);
        }
      } else {
        solve_block(c, *H, nrb, nr, b64.as<cd>(), x64.as<cd>(), W);
      }
      for (int j = 0; j < nr; j++) {
        launch_block_get(n, nrb, j, x64.p, c->x64.p, s);
        if (x_out)
          AC3D_CUDA(cudaMemcpyAsync(x_out + 2 * (size_t)n * (start + j), c->x64.p, (size_t)n * sizeof(cd),
                                    cudaMemcpyDeviceToHost, s));
        if (p_out) {
          launch_far_field(c->m->G, c->prec, recv, nL, k, c->x64.as<cd>(), ycol.as<cd>(), c->ff_scratch, s);
          AC3D_CUDA(cudaMemcpyAsync(p_out + 2 * (size_t)nL * (start + j), ycol.p, (size_t)nL * sizeof(cd),
                                    cudaMemcpyDeviceToHost, s));
        }
        AC3D_CUDA(cudaStreamSynchronize(s));
      }
    }
    c->stats.ms_solve += ts.stop();
    c->last_H = std::move(H);
    if (!c->stats.converged) throw Error(AC3D_ERR_NOT_CONVERGED, not_converged_message(c));
  });
}

int ac3d_surface_values(ac3d_ctx* c, double f, double* out) {
  if (!c || !out || !(f > 0)) return AC3D_ERR_ARG;
  return guard(c, [&] {
    require_mesh(c);
    reset_stats(c);
    cudaStream_t s = c->stream;
    ensure_base_geometry(c);
    ensure_work(c);
    c->last_H.reset();
    c->last_H = forward_one(c, f, nullptr, nullptr, 0, c->x64.as<cd>(), nullptr, true);
    AC3D_CUDA(cudaMemcpyAsync(out, c->x64.p, (size_t)c->m->Ne * sizeof(cd), cudaMemcpyDeviceToHost, s));
    AC3D_CUDA(cudaStreamSynchronize(s));
    if (!c->stats.converged) throw Error(AC3D_ERR_NOT_CONVERGED, not_converged_message(c));
  });
}

// use_actual (adjoint.cpp:33-83,148-170): the reference builds the dense boundary and receiver
// matrices and solves by QR. Here the coefficient / gradient calls run, for their duration, on
// the same tree with every leaf pair a dense block, in FP64, with the exact receiver product and
// BiCGSTAB to 1e-12 in place of the direct solve (pvals and surface_vals, as in the reference,
// keep the H-matrix).
constexpr double kActualTol = 1e-12;
constexpr double kDenseFactor = 1e300;  // no pair of clusters is admissible

int ac3d_set_actual(ac3d_ctx* c, int on) {
  if (!c) return AC3D_ERR_ARG;
  c->actual = on != 0;
  return AC3D_OK;
}

struct ActualScope {
  ac3d_ctx* c;
  bool on;
  std::shared_ptr<MeshState> m;
  int prec = 0, listener = 0;
  double tol = 0;
  explicit ActualScope(ac3d_ctx* cc) : c(cc), on(cc->actual && cc->mesh_set) {
    if (!on) return;
    if (!c->m_dense) {
      auto d = build_mesh_state(c->Ps_in.data(), c->m->V, c->Es_in.data(), c->m->Ne, c->cluster_size, kDenseFactor,
                                c->maxk, c->stream);
      if (d->Es != c->m->Es) throw Error(AC3D_ERR_STATE, "internal: dense partition has another element order");
      c->m_dense = std::move(d);
    }
    if (c->m_dense->Ps0 != c->m->Ps0) {  // follow set_points
      c->m_dense->Ps0 = c->m->Ps0;
      c->m_dense->geom_base = false;
    }
    m = c->m;
    prec = c->prec;
    listener = c->listener_mode;
    tol = c->solver_tol;
    c->m = c->m_dense;
    c->prec = AC3D_PREC_FP64;
    c->listener_mode = AC3D_LISTENER_DENSE;
    c->solver_tol = std::min(tol, kActualTol);
  }
  ~ActualScope() {
    if (!on) return;
    c->m = m;
    c->prec = prec;
    c->listener_mode = listener;
    c->solver_tol = tol;
  }
};

int ac3d_band_value(ac3d_ctx* c, double fb, double* cv) {
  if (!c || !cv) return AC3D_ERR_ARG;
  return guard(c, [&] {
    require_mesh(c);
    ActualScope as(c);
    reset_stats(c);
    ensure_base_geometry(c);
    *cv = band_eval(c, fb, true, nullptr);
  });
}

int ac3d_values(ac3d_ctx* c, double* out) {
  if (!c || !out) return AC3D_ERR_ARG;
  return guard(c, [&] {
    require_mesh(c);
    ActualScope as(c);
    reset_stats(c);
    ensure_base_geometry(c);
    for (size_t b = 0; b < c->bands.size(); b++) out[b] = band_eval(c, c->bands[b], true, nullptr);
  });
}

int ac3d_value(ac3d_ctx* c, const double* x, double* cv) {
  if (!c || !cv) return AC3D_ERR_ARG;
  return guard(c, [&] {
    require_mesh(c);
    ActualScope as(c);
    reset_stats(c);
    upload_points(*c->m, heights_to_points(c, x), c->stream);
    c->m->geom_base = x == nullptr;
    double acc = 0;
    for (double fb : c->bands) acc += band_eval(c, fb, true, nullptr);
    *cv = acc / (double)c->bands.size();
  });
}

int ac3d_gradient(ac3d_ctx* c, const double* x, double* cv, double* grad) {
  if (!c || !x || !cv || !grad) return AC3D_ERR_ARG;
  return guard(c, [&] {
    require_mesh(c);
    if (!c->diff_set)
      throw Error(AC3D_ERR_STATE, "No differentiable points set. Set them using set_diff_pts or precompute.");
    ActualScope as(c);
    reset_stats(c);
    cudaStream_t s = c->stream;
    upload_points(*c->m, heights_to_points(c, x), c->stream);
    c->m->geom_base = false;
    const int HH = (int)c->h_off.size() - 1;
    DevBuf g;
    g.alloc((size_t)std::max(HH, 1) * sizeof(double), s);
    AC3D_CUDA(cudaMemsetAsync(g.p, 0, (size_t)std::max(HH, 1) * sizeof(double), s));
    double acc = 0;
    for (double fb : c->bands) acc += band_eval(c, fb, false, g.as<double>());
    AC3D_CUDA(cudaMemcpyAsync(grad, g.p, (size_t)HH * sizeof(double), cudaMemcpyDeviceToHost, s));
    AC3D_CUDA(cudaStreamSynchronize(s));
    *cv = acc;
  });
}

int ac3d_gradient_multi(ac3d_ctx* c, const double* x, const double* freqs, int nf, const double* dirs, int nd,
                        double* loss, double* grad, double* coefs) {
  if (!c || !freqs || nf < 1 || !dirs || nd < 1 || !loss || !grad) return AC3D_ERR_ARG;
  for (int i = 0; i < nf; i++)
    if (!(freqs[i] > 0)) return AC3D_ERR_ARG;
  return guard(c, [&] {
    require_mesh(c);
    if (!c->diff_set)
      throw Error(AC3D_ERR_STATE, "No differentiable points set. Set them using set_diff_pts or precompute.");
    if (c->actual) throw Error(AC3D_ERR_ARG, "multi-direction gradients run on the H-matrix (use_actual off)");
    std::vector<double> dv(3 * (size_t)nd);
    for (int d = 0; d < nd; d++) {
      const double* w = dirs + 3 * (size_t)d;
      const double nrm = std::sqrt(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
      if (!(nrm > 0)) throw Error(AC3D_ERR_ARG, "zero plane-wave direction");
      for (int q = 0; q < 3; q++) dv[3 * (size_t)d + q] = w[q] / nrm;
    }
    reset_stats(c);
    cudaStream_t s = c->stream;
    upload_points(*c->m, heights_to_points(c, x), s);
    c->m->geom_base = false;
    const int HH = (int)c->h_off.size() - 1;
    DevBuf g;
    g.alloc((size_t)std::max(HH, 1) * sizeof(double), s);
    AC3D_CUDA(cudaMemsetAsync(g.p, 0, (size_t)std::max(HH, 1) * sizeof(double), s));
    std::vector<double> cf;
    *loss = multi_eval(c, std::vector<double>(freqs, freqs + nf), dv, g.as<double>(), cf);
    AC3D_CUDA(cudaMemcpyAsync(grad, g.p, (size_t)HH * sizeof(double), cudaMemcpyDeviceToHost, s));
    AC3D_CUDA(cudaStreamSynchronize(s));
    if (coefs) std::copy(cf.begin(), cf.end(), coefs);
    if (!c->stats.converged) throw Error(AC3D_ERR_NOT_CONVERGED, not_converged_message(c));
  });
}

int ac3d_value_dev(ac3d_ctx* c, const double* x_dev, double* c_dev, void* stream) {
  if (!c || !c_dev) return AC3D_ERR_ARG;
  return guard(c, [&] {
    require_mesh(c);
    ActualScope as(c);
    cudaStream_t us = (cudaStream_t)stream;
    cudaStream_t s = c->stream;
    cudaEvent_t ev;
    AC3D_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    AC3D_CUDA(cudaEventRecord(ev, us));
    AC3D_CUDA(cudaStreamWaitEvent(s, ev, 0));
    std::vector<double> x;
    if (x_dev) {
      const int HH = (int)c->diff_pts.size();
      x.resize(HH);
      AC3D_CUDA(cudaMemcpyAsync(x.data(), x_dev, HH * sizeof(double), cudaMemcpyDeviceToHost, s));
      AC3D_CUDA(cudaStreamSynchronize(s));
    }
    reset_stats(c);
    upload_points(*c->m, heights_to_points(c, x_dev ? x.data() : nullptr), c->stream);
    c->m->geom_base = x_dev == nullptr;
    double acc = 0;
    for (double fb : c->bands) acc += band_eval(c, fb, true, nullptr);
    acc /= (double)c->bands.size();
    AC3D_CUDA(cudaMemcpyAsync(c_dev, &acc, sizeof(double), cudaMemcpyHostToDevice, s));
    AC3D_CUDA(cudaEventRecord(ev, s));
    AC3D_CUDA(cudaStreamWaitEvent(us, ev, 0));
    AC3D_CUDA(cudaStreamSynchronize(s));
    AC3D_CUDA(cudaEventDestroy(ev));
  });
}

int ac3d_gradient_dev(ac3d_ctx* c, const double* x_dev, double* c_dev, double* g_dev, void* stream) {
  if (!c || !x_dev || !c_dev || !g_dev) return AC3D_ERR_ARG;
  return guard(c, [&] {
    require_mesh(c);
    if (!c->diff_set)
      throw Error(AC3D_ERR_STATE, "No differentiable points set. Set them using set_diff_pts or precompute.");
    ActualScope as(c);
    cudaStream_t us = (cudaStream_t)stream;
    cudaStream_t s = c->stream;
    cudaEvent_t ev;
    AC3D_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    AC3D_CUDA(cudaEventRecord(ev, us));
    AC3D_CUDA(cudaStreamWaitEvent(s, ev, 0));
    const int HH = (int)c->h_off.size() - 1;
    std::vector<double> x(HH);
    AC3D_CUDA(cudaMemcpyAsync(x.data(), x_dev, HH * sizeof(double), cudaMemcpyDeviceToHost, s));
    AC3D_CUDA(cudaStreamSynchronize(s));
    reset_stats(c);
    upload_points(*c->m, heights_to_points(c, x.data()), c->stream);
    c->m->geom_base = false;
    AC3D_CUDA(cudaMemsetAsync(g_dev, 0, (size_t)HH * sizeof(double), s));
    double acc = 0;
    for (double fb : c->bands) acc += band_eval(c, fb, false, g_dev);
    AC3D_CUDA(cudaMemcpyAsync(c_dev, &acc, sizeof(double), cudaMemcpyHostToDevice, s));
    AC3D_CUDA(cudaEventRecord(ev, s));
    AC3D_CUDA(cudaStreamWaitEvent(us, ev, 0));
    AC3D_CUDA(cudaStreamSynchronize(s));
    AC3D_CUDA(cudaEventDestroy(ev));
  });
}

int ac3d_sphere(const double* Ps, int V, const int32_t* Es, int Ne, double freq, int LL, double lrad, int precision,
                int actual, double* out) {
  if (!Ps || !Es || !out || LL < 1) return AC3D_ERR_ARG;
  const double band = freq;
  const double src[3] = {1.0, 0.0, 0.0};
  ac3d_ctx* c = nullptr;
  // sphere.h:32,43,51: leaf 128, factor 1.5, tolerances 1e-10. actual (sphere.h:65-69, dense QR):
  // every leaf pair a dense block, FP64, BiCGSTAB to 1e-12
  int rc = actual ? ac3d_create(&c, 128, kDenseFactor, &band, 1, 1, 1e-10, 1e-10, kActualTol, src, 1.0, 5.0, 0)
                  : ac3d_create(&c, 128, 1.5, &band, 1, 1, 1e-10, 1e-10, 1e-10, src, 1.0, 5.0, 0);
  if (actual) precision = AC3D_PREC_FP64;
  if (rc) return rc;
  std::vector<int32_t> Eo(3 * (size_t)Ne);
  std::vector<double> L(3 * (size_t)LL, 0.0);
  for (int l = 0; l < LL; l++) {  // sphere.h:58-63
    double th = (double)l / (double)LL * 2 * kPiHost;
    L[3 * l] = lrad * std::cos(th);
    L[3 * l + 2] = -lrad * std::sin(th);
  }
  if (!(rc = ac3d_set_precision(c, precision)) && !(rc = ac3d_set_incident(c, AC3D_INCIDENT_PLANE, src)) &&
      !(rc = ac3d_set_mesh(c, Ps, V, Es, Ne, Eo.data())))
    rc = ac3d_pressures(c, freq, L.data(), LL, out);
  ac3d_destroy(c);
  return rc;
}

struct ac3d_partition {
  ac3d::Partition P;
};

int ac3d_partition_build(const double* Ps, int V, const int32_t* Es, int Ne, int cluster_size, double radius_factor,
                         ac3d_partition** out) {
  if (!Ps || !Es || !out || V < 3 || Ne < 1 || cluster_size < 1) return AC3D_ERR_ARG;
  for (int i = 0; i < 3 * Ne; i++)
    if (Es[i] < 0 || Es[i] >= V) return AC3D_ERR_ARG;
  try {
    auto* p = new ac3d_partition;
    std::vector<double> C(3 * (size_t)Ne);
    for (int e = 0; e < Ne; e++)
      for (int d = 0; d < 3; d++)
        C[3 * e + d] = (Ps[3 * Es[3 * e] + d] + Ps[3 * Es[3 * e + 1] + d] + Ps[3 * Es[3 * e + 2] + d]) / 3;
    build_partition(C.data(), Ne, cluster_size, radius_factor, p->P);
    // ClusterTree::check on the reordered centroids
    std::vector<double> Cr(3 * (size_t)Ne);
    for (int i = 0; i < Ne; i++)
      for (int d = 0; d < 3; d++) Cr[3 * i + d] = C[3 * p->P.order[i] + d];
    for (const TreeNode& nd : p->P.nodes)
      for (int i = nd.s; i < nd.e; i++) {
        double dx = Cr[3 * i] - nd.c[0], dy = Cr[3 * i + 1] - nd.c[1], dz = Cr[3 * i + 2] - nd.c[2];
        if (!(std::sqrt(dx * dx + dy * dy + dz * dz) <= nd.r + 1e-6)) p->P.tree_ok = false;
      }
    *out = p;
    return AC3D_OK;
  } catch (...) {
    return AC3D_ERR_INTERNAL;
  }
}

int ac3d_partition_counts(const ac3d_partition* p, int* nd, int* na, int* nl, int* ok) {
  if (!p) return AC3D_ERR_ARG;
  if (nd) *nd = (int)p->P.direct.size() / 4;
  if (na) *na = (int)p->P.approx.size() / 4;
  if (nl) *nl = (int)p->P.leaf_start.size() - 1;
  if (ok) *ok = p->P.tree_ok ? 1 : 0;
  return AC3D_OK;
}

int ac3d_partition_get(const ac3d_partition* p, int32_t* order, int32_t* direct, int32_t* approx, int32_t* leaves) {
  if (!p) return AC3D_ERR_ARG;
  if (order) std::copy(p->P.order.begin(), p->P.order.end(), order);
  if (direct) std::copy(p->P.direct.begin(), p->P.direct.end(), direct);
  if (approx) std::copy(p->P.approx.begin(), p->P.approx.end(), approx);
  if (leaves) std::copy(p->P.leaf_start.begin(), p->P.leaf_start.end(), leaves);
  return AC3D_OK;
}

void ac3d_partition_free(ac3d_partition* p) { delete p; }

int ac3d_matvec_timing(ac3d_ctx* c, int iters, int transposed, double* ms, long long* bytes) {
  if (!c || iters < 1 || !ms || !bytes) return AC3D_ERR_ARG;
  return guard(c, [&] {
    if (!c->last_H) throw Error(AC3D_ERR_STATE, "no H-matrix: call ac3d_pressures first");
    cudaStream_t s = c->stream;
    const DevHMat& H = *c->last_H;
    ensure_work(c);
    // the variant the solve runs: FP64 vectors on the FP64 H-matrix; on the FP32 H-matrix FP32
    // vectors (GMRES) or FP64 vectors with their FP32 shadows (BiCGSTAB), FP32 arithmetic
    const int vec64 = H.prec == PREC_FP64 ? 1 : (c->krylov == AC3D_KRYLOV_GMRES ? 0 : 2);
    KrylovBufs B = bufs(c, vec64);
    // x = the last solution, y = scratch
    if (vec64 == 0)
      launch_to32(c->m->Ne, c->x64.p, B.p, s);
    else
      launch_copy64(c->m->Ne, c->x64.p, B.p, s);
    if (vec64 == 2) launch_to32(c->m->Ne, c->x64.p, B.p32, s);
    MatvecEpilogue ep;
    // back-to-back matvecs launched as the solve launches them: every pass after the first a
    // programmatic dependent of the one before (x is not written, so each pass may start early)
    auto one = [&](bool pdl) {
      launch_matvec_ex(c->m->DP, H, transposed != 0, vec64, B.p, B.v, nullptr, ep, nullptr, s, B.p32, pdl);
    };
    one(false);  // warm-up
    cudaEvent_t e0, e1;
    AC3D_CUDA(cudaEventCreate(&e0));
    AC3D_CUDA(cudaEventCreate(&e1));
    AC3D_CUDA(cudaEventRecord(e0, s));
    for (int i = 0; i < iters; i++) one(i > 0);
    AC3D_CUDA(cudaEventRecord(e1, s));
    AC3D_CUDA(cudaEventSynchronize(e1));
    float t = 0;
    AC3D_CUDA(cudaEventElapsedTime(&t, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = t / iters;
    // stored entries once; x read and y written once (FP32 or FP64); the FP32 shadow read once
    const long long es = H.prec == PREC_FP64 ? 16 : 8;
    *bytes = (c->m->P.near_total + H.lr_entries) * es + c->m->Ne * (vec64 == 0 ? 16LL : 32LL + (vec64 == 2 ? 8 : 0));
  });
}

int ac3d_block_matvec_timing(ac3d_ctx* c, int nrb, int iters, int transposed, double* ms, long long* bytes) {
  if (!c || !ms || !bytes || iters < 1 || (nrb != 4 && nrb != 8 && nrb != 16)) return AC3D_ERR_ARG;
  return guard(c, [&] {
    if (!c->last_H) throw Error(AC3D_ERR_STATE, "no H-matrix: call ac3d_pressures or ac3d_solve_multi first");
    DevHMat& H = *c->last_H;
    if (H.prec == PREC_FP64) throw Error(AC3D_ERR_ARG, "block matvecs need the mixed-precision (FP32) H-matrix");
    cudaStream_t s = c->stream;
    BlockWork W;
    MultiBufs B = block_bufs(c, H, nrb, W, transposed != 0);
    const size_t blk32 = (size_t)c->m->Ne * nrb * sizeof(cf);
    AC3D_CUDA(cudaMemsetAsync(B.x, 0x3c, blk32, s));  // FP32 values near 0.01
    for (int i = 0; i < 3; i++) launch_mmatvec(c->m->DP, H, B, B.x, B.v, nullptr, nullptr, nullptr, s);
    cudaEvent_t e0, e1;
    AC3D_CUDA(cudaEventCreate(&e0));
    AC3D_CUDA(cudaEventCreate(&e1));
    AC3D_CUDA(cudaEventRecord(e0, s));
    for (int i = 0; i < iters; i++) launch_mmatvec(c->m->DP, H, B, B.x, B.v, nullptr, nullptr, nullptr, s);
    AC3D_CUDA(cudaEventRecord(e1, s));
    AC3D_CUDA(cudaEventSynchronize(e1));
    float t = 0;
    AC3D_CUDA(cudaEventElapsedTime(&t, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    check_pipeline(c, H);
    *ms = t / iters;
    // every stored matrix entry once (complex FP32), the block input read and the output written
    *bytes = 8 * (long long)(c->m->P.near_total + H.lr_entries) + 2 * (long long)blk32;
  });
}

int ac3d_get_ranks(ac3d_ctx* c, int32_t* ranks, int n) {
  if (!c || !ranks || n < 0) return AC3D_ERR_ARG;
  return guard(c, [&] {
    if (!c->last_H) throw Error(AC3D_ERR_STATE, "no H-matrix: call ac3d_pressures or ac3d_surface_values first");
    const std::vector<int>& r = c->last_H->ranks_host;
    if (n != (int)r.size())
      throw Error(AC3D_ERR_ARG, "expected " + std::to_string(r.size()) + " admissible blocks, got " + std::to_string(n));
    std::copy(r.begin(), r.end(), ranks);
  });
}

long long ac3d_kernel_launches(void) { return g_kernel_launches.load(); }

int ac3d_get_stats(const ac3d_ctx* c, ac3d_stats* out) {
  if (!c || !out) return AC3D_ERR_ARG;
  *out = c->stats;
  return AC3D_OK;
}

}  // extern "C"
