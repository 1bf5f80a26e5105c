// Request server: continuous batching of forward solves on one GPU.
//
// Registered meshes (tree, partition, geometry: MeshState) stay on the device and are shared
// read-only by `slots` solver contexts. Each slot owns a CUDA stream pair, its Krylov work buffers
// and a host thread; a slot takes the next admissible request from the queue as soon as its
// previous one finishes, so requests that arrive while others run start without waiting for a
// batch boundary, and the kernels of all running requests overlap on the GPU. Admission is by
// device bytes: a request starts only if its footprint estimate fits in the budget that the
// running requests leave. A request's result is computed by the same kernels in the same fixed
// summation order whether it runs alone or beside others.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/ac3d.h"
#include "context.h"
#include "internal.h"

namespace ac3d {
namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
  return std::chrono::duration<double, std::milli>(b - a).count();
}

struct MeshEntry {
  std::shared_ptr<MeshState> m;
  int cluster_size = 32;
  double radius_factor = 2.0, aca_tol = 1e-4, solver_tol = 1e-6;
  double lr_per_k = 0;  // largest observed (stored low-rank entries) / wavenumber, per precision
};

struct Request {
  long long id = 0;
  int mesh = 0;
  double f = 0;
  int kind = AC3D_INCIDENT_PLANE;
  double v[3] = {0, 0, 0};
  std::vector<double> Ls;
  int state = AC3D_REQ_QUEUED;
  int bypassed = 0;
  std::vector<double> out;
  ac3d_request_info info{};
  Clock::time_point t_submit, t_start, t_end;
};

// Wavenumber below which the low-rank estimate is not scaled down further.
constexpr double kFloorK = 2 * 3.14159265358979323846 * 250.0 / 344.0;

}  // namespace
}  // namespace ac3d

using namespace ac3d;

struct ac3d_server {
  int device = 0;
  int prec = AC3D_PREC_MIXED;
  int assembly = AC3D_ASSEMBLY_DF;
  int krylov = AC3D_KRYLOV_BICGSTAB, gm_restart = 300;
  int64_t budget = 0, in_use = 0;
  int running = 0;
  cudaStream_t stream = nullptr;  // mesh uploads
  std::vector<std::unique_ptr<MeshEntry>> meshes;
  std::vector<ac3d_ctx*> slots;
  std::vector<std::thread> workers;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request*> queue;
  std::unordered_map<long long, std::unique_ptr<Request>> reqs;
  long long next_id = 1;
  bool stop = false;
  std::string err;
};

namespace ac3d {
namespace {

// Device bytes a request may hold at its peak (assembly: near field, ACA pool and packed segments
// coexist), from the partition and what earlier requests on the mesh needed.
int64_t footprint(const ac3d_server* S, const MeshEntry& me, double f, int L) {
  const MeshState& m = *me.m;
  const int64_t es = S->prec == AC3D_PREC_FP64 ? 16 : 8;
  const double k = std::max(wavenumber(f), kFloorK);
  int64_t lr = me.lr_per_k > 0 ? (int64_t)(me.lr_per_k * k * 1.25) : 12 * m.sum_mn;
  lr = std::min<int64_t>(std::max<int64_t>(lr, 1), std::max<int64_t>(m.worst_pool, 1));
  const int64_t pool = std::max<int64_t>(m.pool_hint[S->prec == AC3D_PREC_FP64 ? 1 : 0].load(), lr);
  // ACA pool terms: complex FP64, or double-float for the mixed path's default assembly
  const int64_t pool_es = S->prec == AC3D_PREC_FP64 || S->assembly == AC3D_ASSEMBLY_DF ? 16 : 8;
  const int64_t H = (m.P.near_total + lr) * es + pool * pool_es + (int64_t)m.P.aca_term_cap * 48;
  int64_t work = (int64_t)m.Ne * 176 + (int64_t)(m.DP.nleaf + 64) * 40 + (int64_t)L * 64 * 16 + (1 << 20);
  if (S->krylov == AC3D_KRYLOV_GMRES) {
    const int mm = std::min(S->gm_restart, m.Ne);
    work += ((int64_t)mm + 4) * m.Ne * (es == 16 ? 16 : 8) +
            (int64_t)gmres_scalar_doubles(mm, m.Ne) * 8 + 4096;
  }
  return H + work;
}

int admit_index(const ac3d_server* S) {
  const int n = (int)S->queue.size();
  std::vector<long long> fp(n);
  std::vector<int> by(n);
  for (int i = 0; i < n; i++) {
    fp[i] = S->queue[i]->info.footprint_bytes;
    by[i] = S->queue[i]->bypassed;
  }
  return ac3d_admit_next(fp.data(), by.data(), n, S->budget, S->in_use, S->running);
}

// `me` was looked up under the server lock: add_mesh may grow the mesh list meanwhile, but an
// entry itself never moves.
void run_request(ac3d_server* S, ac3d_ctx* c, Request* r, MeshEntry& me) {
  c->m = me.m;
  c->mesh_set = true;
  c->prec = S->prec;
  c->assembly = S->assembly;
  c->aca_tol = me.aca_tol;
  c->solver_tol = me.solver_tol;
  c->cluster_size = me.cluster_size;
  c->radius_factor = me.radius_factor;
  c->src_kind = r->kind;
  const double nrm = std::sqrt(r->v[0] * r->v[0] + r->v[1] * r->v[1] + r->v[2] * r->v[2]);
  for (int d = 0; d < 3; d++) c->src[d] = r->kind == AC3D_INCIDENT_PLANE ? r->v[d] / nrm : r->v[d];
  reset_stats(c);
  cudaStream_t s = c->stream;
  const int L = (int)r->Ls.size() / 3;
  upload_receivers(c, r->Ls.data(), L, c->tmp_recv);
  ensure_work(c);
  DevBuf y;
  y.alloc((size_t)L * sizeof(cd), s);
  forward_one(c, r->f, c->tmp_recv.as<double4>(), r->Ls.data(), L, c->x64.as<cd>(), y.as<cd>(), false);
  r->out.resize(2 * (size_t)L);
  AC3D_CUDA(cudaMemcpyAsync(r->out.data(), y.p, (size_t)L * sizeof(cd), cudaMemcpyDeviceToHost, s));
  AC3D_CUDA(cudaStreamSynchronize(s));
  y.release();
  const ac3d_stats& st = c->stats;
  r->info.hmat_bytes = st.hmat_bytes;
  r->info.lr_entries = st.lr_entries;
  r->info.near_entries = st.near_entries;
  r->info.iterations = st.iterations;
  r->info.outer_steps = st.outer_steps;
  r->info.rel_residual = st.rel_residual;
  r->info.ms_assemble = st.ms_assemble;
  r->info.ms_solve = st.ms_solve;
  r->info.ms_listener = st.ms_listener;
  r->info.ms_graph = st.ms_graph;
  r->info.aca_entries_evaluated = st.aca_entries_evaluated;
  if (!st.converged) throw Error(AC3D_ERR_NOT_CONVERGED, not_converged_message(c));
}

void worker(ac3d_server* S, int slot) {
  cudaSetDevice(S->device);
  ac3d_ctx* c = S->slots[slot];
  std::unique_lock<std::mutex> lk(S->mu);
  while (true) {
    int idx = -1;
    S->cv_work.wait(lk, [&] {
      if (S->stop && S->queue.empty()) return true;
      idx = admit_index(S);
      return idx >= 0;
    });
    if (idx < 0) break;  // stopping with an empty queue
    Request* r = S->queue[idx];
    for (int j = 0; j < idx; j++) S->queue[j]->bypassed++;
    S->queue.erase(S->queue.begin() + idx);
    r->state = AC3D_REQ_RUNNING;
    r->t_start = Clock::now();
    r->info.slot = slot;
    S->in_use += r->info.footprint_bytes;
    S->running++;
    c->krylov = S->krylov;
    c->gm_restart = S->gm_restart;
    MeshEntry* me = S->meshes[r->mesh].get();
    lk.unlock();

    int rc = AC3D_OK;
    std::string msg;
    try {
      run_request(S, c, r, *me);
    } catch (const Error& e) {
      rc = e.code;
      msg = e.what();
      if (e.code == AC3D_ERR_CUDA) cudaGetLastError();
    } catch (const std::exception& e) {
      rc = AC3D_ERR_INTERNAL;
      msg = e.what();
    }
    c->m.reset();
    c->mesh_set = false;

    lk.lock();
    r->t_end = Clock::now();
    S->in_use -= r->info.footprint_bytes;
    S->running--;
    if (rc == AC3D_OK) {
      me->lr_per_k = std::max(me->lr_per_k, (double)r->info.lr_entries / std::max(wavenumber(r->f), kFloorK));
    } else {
      S->err = msg;
    }
    r->info.status = rc;
    r->info.queue_ms = ms_between(r->t_submit, r->t_start);
    r->info.run_ms = ms_between(r->t_start, r->t_end);
    r->info.latency_ms = ms_between(r->t_submit, r->t_end);
    r->state = rc == AC3D_OK ? AC3D_REQ_DONE : AC3D_REQ_FAILED;
    S->cv_done.notify_all();
    S->cv_work.notify_all();
  }
}

template <typename F>
int sguard(ac3d_server* S, F&& f) {
  if (!S) return AC3D_ERR_ARG;
  try {
    f();
    return AC3D_OK;
  } catch (const Error& e) {
    std::lock_guard<std::mutex> lk(S->mu);
    S->err = e.what();
    if (e.code == AC3D_ERR_CUDA) cudaGetLastError();
    return e.code;
  } catch (const std::exception& e) {
    std::lock_guard<std::mutex> lk(S->mu);
    S->err = e.what();
    return AC3D_ERR_INTERNAL;
  }
}

}  // namespace
}  // namespace ac3d

extern "C" {

int ac3d_admit_next(const long long* footprints, const int* bypassed, int n_queued, long long budget,
                    long long in_use, int n_running) {
  if (n_queued <= 0 || !footprints) return -1;
  for (int i = 0; i < n_queued; i++) {
    if (footprints[i] <= budget - in_use || (n_running == 0 && i == 0)) return i;
    if (bypassed && bypassed[i] >= AC3D_SERVE_MAX_BYPASS) return -1;  // it must go next
  }
  return -1;
}

int ac3d_server_create(ac3d_server** out, int slots, int precision, long long hbm_budget_bytes) {
  if (!out || slots < 1 || slots > 64 || (precision != AC3D_PREC_MIXED && precision != AC3D_PREC_FP64))
    return AC3D_ERR_ARG;
  *out = nullptr;
  auto* S = new ac3d_server;
  S->prec = precision;
  int rc = sguard(S, [&] {
    AC3D_CUDA(cudaGetDevice(&S->device));
    AC3D_CUDA(cudaStreamCreateWithFlags(&S->stream, cudaStreamNonBlocking));
    size_t fr = 0, tot = 0;
    AC3D_CUDA(cudaMemGetInfo(&fr, &tot));
    S->budget = hbm_budget_bytes > 0 ? hbm_budget_bytes : (int64_t)(0.85 * (double)fr);
    const double band = 1000.0, src[3] = {0, 100, 0};
    for (int i = 0; i < slots; i++) {
      ac3d_ctx* c = nullptr;
      int r = ac3d_create(&c, 32, 2.0, &band, 1, 1, 1e-4, 1e-4, 1e-6, src, 50.0, 5.0, 0);
      if (r != AC3D_OK) throw Error(r, "cannot create a slot context");
      c->prec = precision;
      c->givens_branch = false;
      S->slots.push_back(c);
    }
    for (int i = 0; i < slots; i++) S->workers.emplace_back(worker, S, i);
  });
  if (rc != AC3D_OK) {
    ac3d_server_destroy(S);
    return rc;
  }
  *out = S;
  return AC3D_OK;
}

void ac3d_server_destroy(ac3d_server* S) {
  if (!S) return;
  {
    std::unique_lock<std::mutex> lk(S->mu);
    S->stop = true;
    S->cv_work.notify_all();
  }
  for (auto& t : S->workers) t.join();
  for (ac3d_ctx* c : S->slots) ac3d_destroy(c);
  S->meshes.clear();  // device arrays were allocated on S->stream
  if (S->stream) {
    cudaStreamSynchronize(S->stream);
    cudaStreamDestroy(S->stream);
  }
  delete S;
}

const char* ac3d_server_last_error(const ac3d_server* S) { return S ? S->err.c_str() : "null server"; }

int ac3d_server_set_krylov(ac3d_server* S, int method, int restart) {
  if (!S || (method != AC3D_KRYLOV_BICGSTAB && method != AC3D_KRYLOV_GMRES) || restart < 0 || restart > 600)
    return AC3D_ERR_ARG;
  std::lock_guard<std::mutex> lk(S->mu);
  S->krylov = method;
  S->gm_restart = restart > 0 ? restart : 300;
  return AC3D_OK;
}

int ac3d_server_set_assembly(ac3d_server* S, int mode) {
  if (!S || (mode != AC3D_ASSEMBLY_DF && mode != AC3D_ASSEMBLY_FP32)) return AC3D_ERR_ARG;
  std::lock_guard<std::mutex> lk(S->mu);
  S->assembly = mode;
  return AC3D_OK;
}

int ac3d_server_add_mesh(ac3d_server* S, const double* Ps, int V, const int32_t* Es, int Ne, int cluster_size,
                         double radius_factor, double aca_tol, double solver_tol, int32_t* Es_out, int* mesh_id) {
  if (!S || !Ps || !Es || V < 3 || Ne < 1 || !mesh_id || cluster_size < 1 || cluster_size > 256 ||
      !(solver_tol > 0) || !(aca_tol >= 0))
    return AC3D_ERR_ARG;
  return sguard(S, [&] {
    auto me = std::make_unique<MeshEntry>();
    me->m = build_mesh_state(Ps, V, Es, Ne, cluster_size, radius_factor, 100, S->stream);
    me->cluster_size = cluster_size;
    me->radius_factor = radius_factor;
    me->aca_tol = aca_tol;
    me->solver_tol = solver_tol;
    if (Es_out) std::memcpy(Es_out, me->m->Es.data(), me->m->Es.size() * sizeof(int32_t));
    std::lock_guard<std::mutex> lk(S->mu);
    *mesh_id = (int)S->meshes.size();
    S->meshes.push_back(std::move(me));
  });
}

int ac3d_server_submit(ac3d_server* S, int mesh_id, double frequency, int kind, const double* v, const double* Ls,
                       int L, long long* request) {
  if (!S || !request || !v || !Ls || L < 1 || !(frequency > 0) ||
      (kind != AC3D_INCIDENT_POINT && kind != AC3D_INCIDENT_PLANE))
    return AC3D_ERR_ARG;
  if (kind == AC3D_INCIDENT_PLANE && !(v[0] * v[0] + v[1] * v[1] + v[2] * v[2] > 0)) return AC3D_ERR_ARG;
  auto r = std::make_unique<Request>();
  r->f = frequency;
  r->kind = kind;
  for (int d = 0; d < 3; d++) r->v[d] = v[d];
  r->Ls.assign(Ls, Ls + 3 * (size_t)L);
  std::lock_guard<std::mutex> lk(S->mu);
  if (mesh_id < 0 || mesh_id >= (int)S->meshes.size()) {
    S->err = "unknown mesh id";
    return AC3D_ERR_ARG;
  }
  if (S->stop) {
    S->err = "server is shutting down";
    return AC3D_ERR_STATE;
  }
  r->mesh = mesh_id;
  r->info.footprint_bytes = footprint(S, *S->meshes[mesh_id], frequency, L);
  if (r->info.footprint_bytes > S->budget) {
    S->err = "request needs an estimated " + std::to_string(r->info.footprint_bytes) +
             " device bytes, more than the server budget of " + std::to_string(S->budget);
    return AC3D_ERR_RESOURCE;
  }
  r->id = S->next_id++;
  r->t_submit = Clock::now();
  *request = r->id;
  S->queue.push_back(r.get());
  S->reqs[r->id] = std::move(r);
  S->cv_work.notify_one();
  return AC3D_OK;
}

int ac3d_server_poll(ac3d_server* S, long long request, int* state) {
  if (!S || !state) return AC3D_ERR_ARG;
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->reqs.find(request);
  if (it == S->reqs.end()) return AC3D_ERR_ARG;
  *state = it->second->state;
  return AC3D_OK;
}

int ac3d_server_wait(ac3d_server* S, long long request, double* out, ac3d_request_info* info) {
  if (!S) return AC3D_ERR_ARG;
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->reqs.find(request);
  if (it == S->reqs.end()) return AC3D_ERR_ARG;
  Request* r = it->second.get();
  S->cv_done.wait(lk, [&] { return r->state == AC3D_REQ_DONE || r->state == AC3D_REQ_FAILED; });
  if (out && !r->out.empty()) std::memcpy(out, r->out.data(), r->out.size() * sizeof(double));
  if (info) *info = r->info;
  const int rc = r->info.status;
  S->reqs.erase(it);
  return rc;
}

}  // extern "C"
