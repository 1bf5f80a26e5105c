// Heightmap texture <-> differentiable-vertex heights on the device: the bilinear lookup eval_uv
// (acoustics_opt.py:23-33) and its transpose, the texture gradient of acoustic_gradient
// (acoustics_opt.py:44-57).
//
// The texel indices and weights depend only on the uvs and the texture size, so they are computed
// once on the host, with the reference's arithmetic (numpy modf, negative fractions wrapped to
// 1 + f, indices clamped at the far edges, weights as the products (1 - vf)(1 - uf), ...). The
// lookup then sums w0 t0 + w1 t1 + w2 t2 + w3 t3 left to right, and the transpose gathers, per
// texel, the contributions w g[i] in the order the reference's loop adds them (vertex by vertex,
// corners in the order 00, 01, 10, 11) from a texel-major list: both are bitwise the NumPy
// results, and the transpose needs no atomics.
#include <algorithm>
#include <cmath>
#include <vector>

#include "ac3d.h"
#include "internal.h"

struct ac3d_texmap {
  int n = 0, H = 0, W = 0;
  ac3d::DevBuf idx;   // n x 4 flat texel indices (int4)
  ac3d::DevBuf wts;   // n x 4 weights (double)
  ac3d::DevBuf ptr;   // H W + 1 offsets of each texel's contributions
  ac3d::DevBuf cvert; // contribution -> vertex
  ac3d::DevBuf cwt;   // contribution -> weight
};

namespace ac3d {
namespace {

constexpr int kTexThreads = 256;

__global__ void tex_sample_kernel(int n, const int4* __restrict__ idx, const double4* __restrict__ w,
                                  const double* __restrict__ tex, double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int4 k = idx[i];
  const double4 c = w[i];
  double s = __dmul_rn(c.x, tex[k.x]);
  s = __dadd_rn(s, __dmul_rn(c.y, tex[k.y]));
  s = __dadd_rn(s, __dmul_rn(c.z, tex[k.z]));
  s = __dadd_rn(s, __dmul_rn(c.w, tex[k.w]));
  out[i] = s;
}

__global__ void tex_scatter_kernel(int ntex, const int* __restrict__ ptr, const int* __restrict__ cv,
                                   const double* __restrict__ cw, const double* __restrict__ g,
                                   double* __restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntex) return;
  double s = 0.0;
  for (int e = ptr[t]; e < ptr[t + 1]; e++) s = __dadd_rn(s, __dmul_rn(cw[e], g[cv[e]]));
  out[t] = s;
}

}  // namespace
}  // namespace ac3d

using namespace ac3d;

extern "C" {

int ac3d_texmap_create(ac3d_texmap** out, const double* uvs, int n, int H, int W) {
  if (!out || !uvs || n < 1 || H < 1 || W < 1 || (long long)H * W > 0x7fffffffLL) return AC3D_ERR_ARG;
  *out = nullptr;
  auto* m = new ac3d_texmap;
  m->n = n;
  m->H = H;
  m->W = W;
  try {
    std::vector<int> idx(4 * (size_t)n);
    std::vector<double> wts(4 * (size_t)n);
    for (int i = 0; i < n; i++) {
      // eval_uv, acoustics_opt.py:25-33
      double ui_d, vi_d;
      double uf = std::modf(uvs[2 * i] * W - 0.5, &ui_d);
      double vf = std::modf(uvs[2 * i + 1] * H - 0.5, &vi_d);
      if (uf < 0) uf = 1 + uf;
      if (vf < 0) vf = 1 + vf;
      if (!(std::fabs(ui_d) < 2e9) || !(std::fabs(vi_d) < 2e9)) throw Error(AC3D_ERR_ARG, "uv out of range");
      const int ui = std::max((int)ui_d, 0), vi = std::max((int)vi_d, 0);
      const int ui1 = std::min(ui + 1, W - 1), vi1 = std::min(vi + 1, H - 1);
      if (ui >= W || vi >= H) throw Error(AC3D_ERR_ARG, "uv outside the texture");
      const int k[4] = {vi * W + ui, vi * W + ui1, vi1 * W + ui, vi1 * W + ui1};
      const double w[4] = {(1 - vf) * (1 - uf), (1 - vf) * uf, vf * (1 - uf), vf * uf};
      for (int c = 0; c < 4; c++) {
        idx[4 * (size_t)i + c] = k[c];
        wts[4 * (size_t)i + c] = w[c];
      }
    }
    // texel-major contribution lists in (vertex, corner) order (acoustics_opt.py:52-56)
    const int ntex = H * W;
    std::vector<int> ptr(ntex + 1, 0), cv(4 * (size_t)n);
    std::vector<double> cw(4 * (size_t)n);
    for (size_t e = 0; e < idx.size(); e++) ptr[idx[e] + 1]++;
    for (int t = 0; t < ntex; t++) ptr[t + 1] += ptr[t];
    std::vector<int> fill(ptr.begin(), ptr.end() - 1);
    for (int i = 0; i < n; i++)
      for (int c = 0; c < 4; c++) {
        const size_t e = 4 * (size_t)i + c;
        const int p = fill[idx[e]]++;
        cv[p] = i;
        cw[p] = wts[e];
      }
    cudaStream_t s = 0;
    m->idx.alloc(idx.size() * sizeof(int), s);
    m->wts.alloc(wts.size() * sizeof(double), s);
    m->ptr.alloc(ptr.size() * sizeof(int), s);
    m->cvert.alloc(cv.size() * sizeof(int), s);
    m->cwt.alloc(cw.size() * sizeof(double), s);
    AC3D_CUDA(cudaMemcpy(m->idx.p, idx.data(), idx.size() * sizeof(int), cudaMemcpyHostToDevice));
    AC3D_CUDA(cudaMemcpy(m->wts.p, wts.data(), wts.size() * sizeof(double), cudaMemcpyHostToDevice));
    AC3D_CUDA(cudaMemcpy(m->ptr.p, ptr.data(), ptr.size() * sizeof(int), cudaMemcpyHostToDevice));
    AC3D_CUDA(cudaMemcpy(m->cvert.p, cv.data(), cv.size() * sizeof(int), cudaMemcpyHostToDevice));
    AC3D_CUDA(cudaMemcpy(m->cwt.p, cw.data(), cw.size() * sizeof(double), cudaMemcpyHostToDevice));
  } catch (const Error& e) {
    delete m;
    return e.code;
  } catch (...) {
    delete m;
    return AC3D_ERR_INTERNAL;
  }
  *out = m;
  return AC3D_OK;
}

void ac3d_texmap_destroy(ac3d_texmap* m) {
  if (!m) return;
  cudaDeviceSynchronize();
  for (DevBuf* b : {&m->idx, &m->wts, &m->ptr, &m->cvert, &m->cwt}) b->release();
  delete m;
}

int ac3d_texmap_sample_dev(const ac3d_texmap* m, const double* tex_dev, double* heights_dev, void* stream) {
  if (!m || !tex_dev || !heights_dev) return AC3D_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  note_launch();
  tex_sample_kernel<<<(m->n + kTexThreads - 1) / kTexThreads, kTexThreads, 0, s>>>(
      m->n, m->idx.as<int4>(), m->wts.as<double4>(), tex_dev, heights_dev);
  return cudaGetLastError() == cudaSuccess ? AC3D_OK : AC3D_ERR_CUDA;
}

int ac3d_texmap_scatter_dev(const ac3d_texmap* m, const double* grad_dev, double* tex_grad_dev, void* stream) {
  if (!m || !grad_dev || !tex_grad_dev) return AC3D_ERR_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int ntex = m->H * m->W;
  note_launch();
  tex_scatter_kernel<<<(ntex + kTexThreads - 1) / kTexThreads, kTexThreads, 0, s>>>(
      ntex, m->ptr.as<int>(), m->cvert.as<int>(), m->cwt.as<double>(), grad_dev, tex_grad_dev);
  return cudaGetLastError() == cudaSuccess ? AC3D_OK : AC3D_ERR_CUDA;
}

}  // extern "C"
