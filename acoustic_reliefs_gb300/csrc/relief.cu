// Relief meshes generated on the device: the box base of generate_base_mesh
// (pyoptim/mesher.py:87-149: six unwelded structured face grids, quads split in two), the 1 -> 4
// midpoint subdivision of the top face (face_subdivision, mesher.py:153-231) and the top vertices
// with their texture uvs (acoustics_opt.py:182-210; rect_points_to_uv, pyoptim/diffmesh.py:248).
// The output is bitwise the host generator's (acoustic_reliefs_gb300/meshes.py): vertices are formed
// with the same FP64 operations in the same order (no contraction), and midpoint vertices get
// their ids in the order their edges first occur (face by face, edges (1,2), (2,3), (1,3)), which
// is the insertion order of the host's edge dictionary.
//
// Per subdivision level: every subdivided face's three edges go into an open-addressing hash table
// keyed by the vertex pair, each keeping the smallest (face position, slot) rank that holds it; the
// ranks that own their edge are numbered by a fixed-order scan, which gives the midpoint ids; each
// face then writes its children (1 to 4, by which of its edges were split) at the scanned offset.
#include <cuda_runtime.h>

#include <vector>

#include "../../include/ac3d.h"
#include "internal.h"

namespace ac3d {

namespace {

constexpr unsigned long long kEmpty = ~0ull;

__device__ __forceinline__ unsigned long long edge_key(int a, int b) {
  const int lo = min(a, b), hi = max(a, b);
  return ((unsigned long long)(unsigned)lo << 32) | (unsigned)hi;
}

__device__ __forceinline__ unsigned hash64(unsigned long long k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  k *= 0xc4ceb9fe1a85ec53ull;
  k ^= k >> 33;
  return (unsigned)k;
}

// slot of key (inserted if absent); table size is a power of two above twice the keys
__device__ int table_slot(unsigned long long* keys, unsigned mask, unsigned long long k, bool insert) {
  unsigned h = hash64(k) & mask;
  for (unsigned probe = 0; probe <= mask; probe++) {
    const unsigned long long cur = keys[h];
    if (cur == k) return (int)h;
    if (cur == kEmpty) {
      if (!insert) return -1;
      const unsigned long long prev = atomicCAS(&keys[h], kEmpty, k);
      if (prev == kEmpty || prev == k) return (int)h;
    }
    h = (h + 1) & mask;
  }
  return -1;
}

// One face grid (generate_base_mesh's `grid`): vertices start + i u + j v for j <= nv, i <= nu;
// quads (j, i) split into (a, c, d), (a, d, b) (sign > 0) or (a, d, c), (a, b, d).
struct Grid {
  double start[3], u[3], v[3];
  int nu, nv, sign, vbase, fbase;
};

__global__ void grid_vertices_kernel(Grid g, double* P) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (g.nu + 1) * (g.nv + 1)) return;
  const int j = t / (g.nu + 1), i = t - j * (g.nu + 1);
  for (int d = 0; d < 3; d++)
    P[3 * (size_t)(g.vbase + t) + d] = __dadd_rn(__dadd_rn(g.start[d], __dmul_rn((double)i, g.u[d])),
                                                 __dmul_rn((double)j, g.v[d]));
}

__global__ void grid_faces_kernel(Grid g, int* E) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.nu * g.nv) return;
  const int j = t / g.nu, i = t - j * g.nu;
  const int a = g.vbase + j * (g.nu + 1) + i, b = a + 1, c = a + g.nu + 1, d = c + 1;
  int* f = E + 3 * (size_t)(g.fbase + 2 * t);
  if (g.sign > 0) {
    f[0] = a, f[1] = c, f[2] = d;
    f[3] = a, f[4] = d, f[5] = b;
  } else {
    f[0] = a, f[1] = d, f[2] = c;
    f[3] = a, f[4] = b, f[5] = d;
  }
}

// edges of the subdivided faces: keys in, smallest rank per key
__global__ void edge_insert_kernel(const int* E, const int* faces, int T, unsigned long long* keys, int* minrank,
                                   unsigned mask, int* err) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= 3 * T) return;
  const int t = r / 3, e = r - 3 * t;
  const int* f = E + 3 * (size_t)faces[t];
  const int a = e == 0 ? f[0] : (e == 1 ? f[1] : f[0]);
  const int b = e == 0 ? f[1] : (e == 1 ? f[2] : f[2]);
  const int s = table_slot(keys, mask, edge_key(a, b), true);
  if (s < 0) {
    atomicExch(err, 1);
    return;
  }
  atomicMin(&minrank[s], r);
}

// owner[r] = 1 if rank r is the first occurrence of its edge
__global__ void edge_owner_kernel(const int* E, const int* faces, int T, const unsigned long long* keys,
                                  const int* minrank, unsigned mask, int* owner) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= 3 * T) return;
  const int t = r / 3, e = r - 3 * t;
  const int* f = E + 3 * (size_t)faces[t];
  const int a = e == 0 ? f[0] : (e == 1 ? f[1] : f[0]);
  const int b = e == 0 ? f[1] : (e == 1 ? f[2] : f[2]);
  const int s = table_slot(const_cast<unsigned long long*>(keys), mask, edge_key(a, b), false);
  owner[r] = (s >= 0 && minrank[s] == r) ? 1 : 0;
}

// Exclusive scan of n ints into out (out[n] = total) by one CTA of 1024 threads, in a fixed order.
__global__ void scan_kernel(const int* in, int n, int* out) {
  __shared__ int sums[1024];
  const int tid = threadIdx.x;
  const int chunk = (n + 1023) / 1024;
  const int s = min(n, tid * chunk), e = min(n, s + chunk);
  int acc = 0;
  for (int i = s; i < e; i++) acc += in[i];
  sums[tid] = acc;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    const int v = tid >= o ? sums[tid - o] : 0;
    __syncthreads();
    sums[tid] += v;
    __syncthreads();
  }
  int base = tid ? sums[tid - 1] : 0;
  for (int i = s; i < e; i++) {
    out[i] = base;
    base += in[i];
  }
  if (tid == 1023) out[n] = sums[1023];
}

// midpoint vertex of every owned edge: (P[a] + P[b]) / 2 at V + scan[r]
__global__ void midpoint_kernel(const int* E, const int* faces, int T, const int* owner, const int* scan, int V,
                                double* P) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= 3 * T || !owner[r]) return;
  const int t = r / 3, e = r - 3 * t;
  const int* f = E + 3 * (size_t)faces[t];
  const int a = e == 0 ? f[0] : (e == 1 ? f[1] : f[0]);
  const int b = e == 0 ? f[1] : (e == 1 ? f[2] : f[2]);
  const size_t m = (size_t)V + scan[r];
  for (int d = 0; d < 3; d++) P[3 * m + d] = __dadd_rn(P[3 * (size_t)a + d], P[3 * (size_t)b + d]) / 2.0;
}

// midpoint id of edge (a, b), or -1 if the edge was not split
__device__ __forceinline__ int mid_of(int a, int b, const unsigned long long* keys, const int* minrank,
                                      unsigned mask, const int* scan, int V) {
  const int s = table_slot(const_cast<unsigned long long*>(keys), mask, edge_key(a, b), false);
  return s < 0 ? -1 : V + scan[minrank[s]];
}

// children per face: 1 + number of split edges (face_subdivision's seven cases)
__global__ void child_count_kernel(const int* E, int F, const unsigned long long* keys, const int* minrank,
                                   unsigned mask, const int* scan, int V, int* cnt) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= F) return;
  const int i1 = E[3 * (size_t)f], i2 = E[3 * (size_t)f + 1], i3 = E[3 * (size_t)f + 2];
  const int n = (mid_of(i1, i2, keys, minrank, mask, scan, V) >= 0) + (mid_of(i2, i3, keys, minrank, mask, scan, V) >= 0) +
                (mid_of(i1, i3, keys, minrank, mask, scan, V) >= 0);
  cnt[f] = 1 + n;
}

__global__ void child_faces_kernel(const int* E, int F, const unsigned long long* keys, const int* minrank,
                                   unsigned mask, const int* scan, int V, const int* off, const int* sub, int* E2,
                                   int* faces2, const int* foff) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= F) return;
  const int i1 = E[3 * (size_t)f], i2 = E[3 * (size_t)f + 1], i3 = E[3 * (size_t)f + 2];
  const int i4 = mid_of(i1, i2, keys, minrank, mask, scan, V);
  const int i5 = mid_of(i2, i3, keys, minrank, mask, scan, V);
  const int i6 = mid_of(i1, i3, keys, minrank, mask, scan, V);
  int* o = E2 + 3 * (size_t)off[f];
  int n = 0;
  auto put = [&](int a, int b, int c) {
    o[3 * n] = a, o[3 * n + 1] = b, o[3 * n + 2] = c;
    n++;
  };
  if (i4 >= 0 && i5 < 0 && i6 < 0) {
    put(i4, i2, i3), put(i1, i4, i3);
  } else if (i5 >= 0 && i4 < 0 && i6 < 0) {
    put(i1, i2, i5), put(i1, i5, i3);
  } else if (i6 >= 0 && i4 < 0 && i5 < 0) {
    put(i1, i2, i6), put(i2, i3, i6);
  } else if (i4 < 0 && i5 >= 0 && i6 >= 0) {
    put(i1, i2, i6), put(i2, i5, i6), put(i5, i3, i6);
  } else if (i5 < 0 && i4 >= 0 && i6 >= 0) {
    put(i1, i4, i6), put(i2, i6, i4), put(i2, i3, i6);
  } else if (i6 < 0 && i4 >= 0 && i5 >= 0) {
    put(i1, i4, i3), put(i3, i4, i5), put(i4, i2, i5);
  } else if (i4 >= 0 && i5 >= 0 && i6 >= 0) {
    put(i1, i4, i6), put(i4, i2, i5), put(i6, i5, i3), put(i4, i5, i6);
  } else {
    put(i1, i2, i3);
  }
  if (sub[f])  // the next level subdivides this face's four children
    for (int c = 0; c < 4; c++) faces2[foff[f] + c] = off[f] + c;
}

__global__ void mark_kernel(const int* faces, int T, int* sub) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < T) sub[faces[t]] = 1;
}

__global__ void times4_kernel(const int* sub, int F, int* four) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f < F) four[f] = 4 * sub[f];
}

// Largest y and the x, z extents (exact, by a fixed single-CTA reduction).
__global__ void extent_kernel(const double* P, int V, double* ext) {
  __shared__ double s[6][256];
  double v[6] = {-INFINITY, INFINITY, -INFINITY, INFINITY, -INFINITY, INFINITY};  // max/min x, y, z
  for (int i = threadIdx.x; i < V; i += blockDim.x)
    for (int d = 0; d < 3; d++) {
      const double x = P[3 * (size_t)i + d];
      v[2 * d] = fmax(v[2 * d], x);
      v[2 * d + 1] = fmin(v[2 * d + 1], x);
    }
  for (int q = 0; q < 6; q++) s[q][threadIdx.x] = v[q];
  __syncthreads();
  if (threadIdx.x < 6) {
    double r = s[threadIdx.x][0];
    for (int t = 1; t < (int)blockDim.x; t++)
      r = (threadIdx.x & 1) ? fmin(r, s[threadIdx.x][t]) : fmax(r, s[threadIdx.x][t]);
    ext[threadIdx.x] = r;
  }
}

// numpy isclose(y, ymax) with rtol 1e-5, atol 1e-8
__global__ void top_flag_kernel(const double* P, int V, const double* ext, int* flag) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V) return;
  const double y = P[3 * (size_t)i + 1], ym = ext[2];
  flag[i] = fabs(y - ym) <= __dadd_rn(1e-8, __dmul_rn(1e-5, fabs(ym))) ? 1 : 0;
}

// top ids in vertex order and their uvs: (x - min) / (max - min) * (0.9999 - 0.0001) + 0.0001
__global__ void top_uv_kernel(const double* P, int V, const int* flag, const int* pos, const double* ext, int* top,
                              double* uv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= V || !flag[i]) return;
  const int t = pos[i];
  top[t] = i;
  const double span = 0.9999 - 0.0001;
  const double x = P[3 * (size_t)i], z = P[3 * (size_t)i + 2];
  uv[2 * (size_t)t] = __dadd_rn(__dmul_rn(__ddiv_rn(__dsub_rn(x, ext[1]), __dsub_rn(ext[0], ext[1])), span), 0.0001);
  uv[2 * (size_t)t + 1] =
      __dadd_rn(__dmul_rn(__ddiv_rn(__dsub_rn(z, ext[5]), __dsub_rn(ext[4], ext[5])), span), 0.0001);
}

int blocks(long long n) { return (int)((n + 255) / 256); }

}  // namespace

}  // namespace ac3d

extern "C" int ac3d_relief_sizes(int nx, int ny, int nz, int subdiv_top, int* V, int* F) {
  if (!V || !F || nx < 1 || ny < 1 || nz < 1 || subdiv_top < 0 || subdiv_top > 6) return AC3D_ERR_ARG;
  long long v = 2LL * (nx + 1) * (ny + 1) + 2LL * (nx + 1) * (nz + 1) + 2LL * (ny + 1) * (nz + 1);
  // each level adds the top face's edge midpoints: a (n+1) x (n'+1) grid of triangles has
  // 3 n n' + n + n' edges
  long long a = nx, c = nz;
  for (int s = 0; s < subdiv_top; s++) {
    v += 3 * a * c + a + c;
    a *= 2;
    c *= 2;
  }
  const long long f = 4LL * nx * ny + 4LL * ny * nz + 2LL * nx * nz * (1 + (1LL << (2 * subdiv_top)));
  if (v > 2000000000LL || f > 2000000000LL) return AC3D_ERR_ARG;
  *V = (int)v;
  *F = (int)f;
  return AC3D_OK;
}

extern "C" int ac3d_relief_dev(double w, double b, double h, int nx, int ny, int nz, int subdiv_top, double* Ps_dev,
                               int32_t* Es_dev, int32_t* top_dev, double* uvs_dev, int* n_top, void* stream) {
  using namespace ac3d;
  int V = 0, F = 0;
  if (!Ps_dev || !Es_dev || !top_dev || !uvs_dev || !n_top || !(w > 0) || !(b > 0) || !(h > 0))
    return AC3D_ERR_ARG;
  int rc = ac3d_relief_sizes(nx, ny, nz, subdiv_top, &V, &F);
  if (rc != AC3D_OK) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  try {
    // base box (generate_base_mesh): six grids in the host generator's order
    const double dx = w / nx, dy = h / ny, dz = b / nz;
    const Grid gs[6] = {
        {{-w / 2, 0, -b / 2}, {dx, 0, 0}, {0, dy, 0}, nx, ny, 1, 0, 0},
        {{-w / 2, 0, b / 2}, {dx, 0, 0}, {0, dy, 0}, nx, ny, -1, 0, 0},
        {{-w / 2, h, -b / 2}, {dx, 0, 0}, {0, 0, dz}, nx, nz, 1, 0, 0},
        {{-w / 2, 0, -b / 2}, {dx, 0, 0}, {0, 0, dz}, nx, nz, -1, 0, 0},
        {{-w / 2, 0, -b / 2}, {0, dy, 0}, {0, 0, dz}, ny, nz, 1, 0, 0},
        {{w / 2, 0, -b / 2}, {0, dy, 0}, {0, 0, dz}, ny, nz, -1, 0, 0},
    };
    int vb = 0, fb = 0, Vc = 0, Fc = 0, top_fbase = 0;
    for (int k = 0; k < 6; k++) {
      Grid g = gs[k];
      g.vbase = vb;
      g.fbase = fb;
      if (k == 2) top_fbase = fb;
      note_launch();
      grid_vertices_kernel<<<blocks((long long)(g.nu + 1) * (g.nv + 1)), 256, 0, s>>>(g, Ps_dev);
      note_launch();
      grid_faces_kernel<<<blocks((long long)g.nu * g.nv), 256, 0, s>>>(g, Es_dev);
      vb += (g.nu + 1) * (g.nv + 1);
      fb += 2 * g.nu * g.nv;
    }
    AC3D_CUDA(cudaGetLastError());
    Vc = vb;
    Fc = fb;
    // subdivision levels; the first level's faces are the top grid's triangles (every vertex at
    // y = h, and no other face has three top vertices)
    int T = 2 * nx * nz;
    DevBuf faces, faces2, sub, keys, minrank, owner, scanb, cnt, off, Etmp, four, foff, err, ext, flag, pos;
    {
      std::vector<int> f0(T);
      for (int t = 0; t < T; t++) f0[t] = top_fbase + t;
      faces.alloc((size_t)T * sizeof(int), s);
      AC3D_CUDA(cudaMemcpyAsync(faces.p, f0.data(), (size_t)T * sizeof(int), cudaMemcpyHostToDevice, s));
      AC3D_CUDA(cudaStreamSynchronize(s));
    }
    err.alloc(sizeof(int), s);
    AC3D_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), s));
    for (int level = 0; level < subdiv_top; level++) {
      unsigned size = 1;
      while (size < 4u * 3u * (unsigned)T) size <<= 1;
      const unsigned mask = size - 1;
      keys.ensure((size_t)size * sizeof(unsigned long long), s);
      minrank.ensure((size_t)size * sizeof(int), s);
      AC3D_CUDA(cudaMemsetAsync(keys.p, 0xff, (size_t)size * sizeof(unsigned long long), s));
      AC3D_CUDA(cudaMemsetAsync(minrank.p, 0x7f, (size_t)size * sizeof(int), s));
      owner.ensure((size_t)3 * T * sizeof(int), s);
      scanb.ensure(((size_t)3 * T + 1) * sizeof(int), s);
      note_launch();
      edge_insert_kernel<<<blocks(3LL * T), 256, 0, s>>>(Es_dev, faces.as<int>(), T, keys.as<unsigned long long>(),
                                                         minrank.as<int>(), mask, err.as<int>());
      note_launch();
      edge_owner_kernel<<<blocks(3LL * T), 256, 0, s>>>(Es_dev, faces.as<int>(), T, keys.as<unsigned long long>(),
                                                        minrank.as<int>(), mask, owner.as<int>());
      note_launch();
      scan_kernel<<<1, 1024, 0, s>>>(owner.as<int>(), 3 * T, scanb.as<int>());
      note_launch();
      midpoint_kernel<<<blocks(3LL * T), 256, 0, s>>>(Es_dev, faces.as<int>(), T, owner.as<int>(), scanb.as<int>(),
                                                      Vc, Ps_dev);
      int nmid = 0;
      AC3D_CUDA(cudaMemcpyAsync(&nmid, scanb.as<int>() + 3 * T, sizeof(int), cudaMemcpyDeviceToHost, s));
      // faces: children counts, offsets, children; the subdivided faces' children are next
      sub.ensure((size_t)Fc * sizeof(int), s);
      AC3D_CUDA(cudaMemsetAsync(sub.p, 0, (size_t)Fc * sizeof(int), s));
      note_launch();
      mark_kernel<<<blocks(T), 256, 0, s>>>(faces.as<int>(), T, sub.as<int>());
      cnt.ensure((size_t)Fc * sizeof(int), s);
      off.ensure(((size_t)Fc + 1) * sizeof(int), s);
      four.ensure((size_t)Fc * sizeof(int), s);
      foff.ensure(((size_t)Fc + 1) * sizeof(int), s);
      note_launch();
      child_count_kernel<<<blocks(Fc), 256, 0, s>>>(Es_dev, Fc, keys.as<unsigned long long>(), minrank.as<int>(), mask,
                                                    scanb.as<int>(), Vc, cnt.as<int>());
      note_launch();
      scan_kernel<<<1, 1024, 0, s>>>(cnt.as<int>(), Fc, off.as<int>());
      note_launch();
      times4_kernel<<<blocks(Fc), 256, 0, s>>>(sub.as<int>(), Fc, four.as<int>());
      note_launch();
      scan_kernel<<<1, 1024, 0, s>>>(four.as<int>(), Fc, foff.as<int>());
      int F2 = 0;
      AC3D_CUDA(cudaMemcpyAsync(&F2, off.as<int>() + Fc, sizeof(int), cudaMemcpyDeviceToHost, s));
      AC3D_CUDA(cudaStreamSynchronize(s));
      Etmp.ensure((size_t)3 * F2 * sizeof(int), s);
      faces2.ensure((size_t)4 * T * sizeof(int), s);
      note_launch();
      child_faces_kernel<<<blocks(Fc), 256, 0, s>>>(Es_dev, Fc, keys.as<unsigned long long>(), minrank.as<int>(), mask,
                                                    scanb.as<int>(), Vc, off.as<int>(), sub.as<int>(), Etmp.as<int>(),
                                                    faces2.as<int>(), foff.as<int>());
      AC3D_CUDA(cudaGetLastError());
      AC3D_CUDA(cudaMemcpyAsync(Es_dev, Etmp.p, (size_t)3 * F2 * sizeof(int), cudaMemcpyDeviceToDevice, s));
      std::swap(faces, faces2);
      Vc += nmid;
      Fc = F2;
      T *= 4;
    }
    int herr = 0;
    AC3D_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    AC3D_CUDA(cudaStreamSynchronize(s));
    if (herr || Vc != V || Fc != F) throw Error(AC3D_ERR_INTERNAL, "relief generation: unexpected mesh size");
    // top vertices (isclose(y, max y)) and their uvs over the bounding box
    ext.alloc(6 * sizeof(double), s);
    flag.alloc((size_t)V * sizeof(int), s);
    pos.alloc(((size_t)V + 1) * sizeof(int), s);
    note_launch();
    extent_kernel<<<1, 256, 0, s>>>(Ps_dev, V, ext.as<double>());
    note_launch();
    top_flag_kernel<<<blocks(V), 256, 0, s>>>(Ps_dev, V, ext.as<double>(), flag.as<int>());
    note_launch();
    scan_kernel<<<1, 1024, 0, s>>>(flag.as<int>(), V, pos.as<int>());
    note_launch();
    top_uv_kernel<<<blocks(V), 256, 0, s>>>(Ps_dev, V, flag.as<int>(), pos.as<int>(), ext.as<double>(), top_dev,
                                            uvs_dev);
    AC3D_CUDA(cudaGetLastError());
    AC3D_CUDA(cudaMemcpyAsync(n_top, pos.as<int>() + V, sizeof(int), cudaMemcpyDeviceToHost, s));
    AC3D_CUDA(cudaStreamSynchronize(s));
  } catch (const Error& e) {
    cudaGetLastError();
    return e.code;
  }
  return AC3D_OK;
}
