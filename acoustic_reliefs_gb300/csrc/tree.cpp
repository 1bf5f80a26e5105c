// Cluster tree, block partition and per-leaf work lists (host side).
//
// Semantics follow the reference ClusterTree (clustertree.cpp:49-137): a binary tree over
// element centroids; each node stores the mean of its centroids (summed in index order) and the
// largest distance to it; a node with more than `leaf_size` elements splits on the longest
// bounding-box axis at the mean, `<` going left, and leaf order defines the element permutation.
// Blocks come from the dual traversal: admissible when dist > factor (r_s + r_t), dense when both
// are leaves, otherwise the larger cluster (the source when the target is a leaf) is split.
//
// The GPU-side data layout is built here: near blocks get contiguous column-major storage, and
// every leaf gets the lists of blocks it must gather for y = A x (rows) and y = A^T x (columns),
// so the matvec needs no atomics and sums in a fixed order.
#include <algorithm>
#include <cmath>
#include <numeric>

#include "internal.h"

namespace ac3d {

namespace {

struct Builder {
  const double* C;
  int leaf_size;
  Partition* P;
  std::vector<int> scratch;

  int build(int start, int* idx, int n) {
    TreeNode nd;
    double sum[3] = {0, 0, 0};
    for (int t = 0; t < n; t++)
      for (int d = 0; d < 3; d++) sum[d] += C[3 * idx[t] + d];
    for (int d = 0; d < 3; d++) nd.c[d] = sum[d] / n;
    double rmax = 0;
    for (int t = 0; t < n; t++) {
      const double* c = C + 3 * idx[t];
      double dx = c[0] - nd.c[0], dy = c[1] - nd.c[1], dz = c[2] - nd.c[2];
      rmax = std::max(rmax, std::sqrt(dx * dx + dy * dy + dz * dz));
    }
    nd.r = rmax;
    nd.s = start;
    nd.e = start + n;
    nd.left = nd.right = -1;
    nd.leaf = true;
    int id = (int)P->nodes.size();
    P->nodes.push_back(nd);
    if (n <= leaf_size) {
      for (int t = 0; t < n; t++) P->order[start + t] = idx[t];
      return id;
    }
    double lo[3], hi[3];
    for (int d = 0; d < 3; d++) lo[d] = hi[d] = C[3 * idx[0] + d];
    for (int t = 0; t < n; t++)
      for (int d = 0; d < 3; d++) {
        double v = C[3 * idx[t] + d];
        lo[d] = std::min(lo[d], v);
        hi[d] = std::max(hi[d], v);
      }
    int dim = 0;
    for (int d = 1; d < 3; d++)
      if (hi[d] - lo[d] > hi[dim] - lo[dim]) dim = d;
    const double gamma = P->nodes[id].c[dim];
    // stable partition: left keeps index order, right keeps index order
    int nl = 0;
    scratch.resize(std::max<size_t>(scratch.size(), (size_t)n));
    int nr = 0;
    for (int t = 0; t < n; t++) {
      int i = idx[t];
      if (C[3 * i + dim] < gamma)
        idx[nl++] = i;
      else
        scratch[nr++] = i;
    }
    std::copy(scratch.begin(), scratch.begin() + nr, idx + nl);
    if (nl == 0 || nr == 0) {  // all centroids coincide along the split: keep as a leaf
      for (int t = 0; t < n; t++) P->order[start + t] = idx[t];
      return id;
    }
    P->nodes[id].leaf = false;
    int l = build(start, idx, nl);
    int r = build(start + nl, idx + nl, nr);
    P->nodes[id].left = l;
    P->nodes[id].right = r;
    return id;
  }
};

void traverse(const Partition& P, int s, int t, double factor, std::vector<int>& direct, std::vector<int>& approx) {
  const TreeNode& S = P.nodes[s];
  const TreeNode& T = P.nodes[t];
  double dx = S.c[0] - T.c[0], dy = S.c[1] - T.c[1], dz = S.c[2] - T.c[2];
  double dist = std::sqrt(dx * dx + dy * dy + dz * dz);
  if (dist > factor * (S.r + T.r)) {
    approx.insert(approx.end(), {S.s, S.e, T.s, T.e});
  } else if (S.leaf && T.leaf) {
    direct.insert(direct.end(), {S.s, S.e, T.s, T.e});
  } else {
    bool split_src = T.leaf || ((S.e - S.s) > (T.e - T.s));
    if (split_src) {
      traverse(P, S.left, t, factor, direct, approx);
      traverse(P, S.right, t, factor, direct, approx);
    } else {
      traverse(P, s, T.left, factor, direct, approx);
      traverse(P, s, T.right, factor, direct, approx);
    }
  }
}

}  // namespace

void build_partition(const double* C, int ne, int leaf_size, double factor, Partition& P) {
  if (ne <= 0) throw Error(2, "mesh has no elements");
  if (leaf_size < 1) throw Error(2, "cluster_size must be >= 1");
  P = Partition();
  P.ne = ne;
  P.order.assign(ne, 0);
  std::vector<int> idx(ne);
  std::iota(idx.begin(), idx.end(), 0);
  Builder b{C, leaf_size, &P, {}};
  b.build(0, idx.data(), ne);
  traverse(P, 0, 0, factor, P.direct, P.approx);
  // leaves in position order
  for (const TreeNode& nd : P.nodes)
    if (nd.leaf) P.leaf_start.push_back(nd.s);
  std::sort(P.leaf_start.begin(), P.leaf_start.end());
  P.leaf_start.push_back(ne);
  P.max_leaf = 0;
  for (size_t l = 0; l + 1 < P.leaf_start.size(); l++)
    P.max_leaf = std::max(P.max_leaf, P.leaf_start[l + 1] - P.leaf_start[l]);
}

void build_leaf_lists(Partition& P, int maxk) {
  int nleaf = (int)P.leaf_start.size() - 1;
  std::vector<int> leaf_of(P.ne);
  for (int l = 0; l < nleaf; l++)
    for (int i = P.leaf_start[l]; i < P.leaf_start[l + 1]; i++) leaf_of[i] = l;
  int nd = (int)P.direct.size() / 4, na = (int)P.approx.size() / 4;

  auto csr = [&](std::vector<std::vector<int>>& lists, std::vector<int>& ptr, std::vector<int>& items) {
    ptr.assign(nleaf + 1, 0);
    for (int l = 0; l < nleaf; l++) ptr[l + 1] = ptr[l] + (int)lists[l].size();
    items.clear();
    items.reserve(ptr[nleaf]);
    for (int l = 0; l < nleaf; l++) items.insert(items.end(), lists[l].begin(), lists[l].end());
  };
  std::vector<std::vector<int>> fn(nleaf), fl(nleaf), tn(nleaf), tl(nleaf);
  for (int b = 0; b < nd; b++) {
    const int* q = &P.direct[4 * b];
    if (P.leaf_start[leaf_of[q[0]]] != q[0] || P.leaf_start[leaf_of[q[2]]] != q[2])
      throw Error(3, "internal: near block not aligned to leaves");
    fn[leaf_of[q[0]]].push_back(b);
    tn[leaf_of[q[2]]].push_back(b);
  }
  for (int l = 0; l < nleaf; l++) {
    std::stable_sort(fn[l].begin(), fn[l].end(), [&](int a, int c) { return P.direct[4 * a + 2] < P.direct[4 * c + 2]; });
    std::stable_sort(tn[l].begin(), tn[l].end(), [&](int a, int c) { return P.direct[4 * a] < P.direct[4 * c]; });
  }
  P.max_rows = 0;
  P.aca_term_cap = 0;
  for (int b = 0; b < na; b++) {
    const int* q = &P.approx[4 * b];
    for (int l = leaf_of[q[0]]; l < nleaf && P.leaf_start[l] < q[1]; l++) fl[l].push_back(b);
    for (int l = leaf_of[q[2]]; l < nleaf && P.leaf_start[l] < q[3]; l++) tl[l].push_back(b);
    int m = q[1] - q[0], n = q[3] - q[2];
    P.max_rows = std::max(P.max_rows, m);
    P.aca_term_cap += std::max(0, std::min(maxk, std::min(m - 1, n - 1)));
  }
  // The low-rank blocks of a leaf's lists ordered by cluster (the blocks' row cluster for the
  // U side, column cluster for the V side), then by block: the blocks that share a cluster occupy
  // one run of consecutive segment columns in every leaf of that cluster, in the same order, so a
  // pass can accumulate a cluster's terms over its leaves.
  for (int l = 0; l < nleaf; l++) {
    std::stable_sort(fl[l].begin(), fl[l].end(), [&](int a, int c) {
      const int* qa = &P.approx[4 * a];
      const int* qc = &P.approx[4 * c];
      return qa[0] != qc[0] ? qa[0] < qc[0] : qa[1] != qc[1] ? qa[1] < qc[1] : a < c;
    });
    std::stable_sort(tl[l].begin(), tl[l].end(), [&](int a, int c) {
      const int* qa = &P.approx[4 * a];
      const int* qc = &P.approx[4 * c];
      return qa[2] != qc[2] ? qa[2] < qc[2] : qa[3] != qc[3] ? qa[3] < qc[3] : a < c;
    });
  }
  csr(fn, P.fw_near_ptr, P.fw_near);
  // near storage in forward leaf order: each leaf's blocks form one R x NC column-major segment
  P.near_off.assign(nd, 0);
  P.near_seg.assign(nleaf + 1, 0);
  P.didx_ptr.assign(nleaf + 1, 0);
  P.didx.clear();
  int64_t off = 0;
  for (int l = 0; l < nleaf; l++) {
    P.near_seg[l] = off;
    for (int it = P.fw_near_ptr[l]; it < P.fw_near_ptr[l + 1]; it++) {
      const int b = P.fw_near[it];
      const int* q = &P.direct[4 * b];
      P.near_off[b] = off;
      off += (int64_t)(q[1] - q[0]) * (q[3] - q[2]);
      for (int c = q[2]; c < q[3]; c++) P.didx.push_back(c);
    }
    // pad to an even column count: segments start and end on 16-byte boundaries (bulk copies)
    if ((P.didx.size() - P.didx_ptr[l]) & 1) {
      P.didx.push_back(-1);
      off += P.leaf_start[l + 1] - P.leaf_start[l];
    }
    P.didx_ptr[l + 1] = (int)P.didx.size();
  }
  P.near_seg[nleaf] = off;
  P.near_total = off;
  // near storage of the transpose (block adjoint solves): the blocks whose columns are leaf l,
  // each transposed to (its columns) x (its rows) column-major, in row order, form leaf l's
  // segment; its columns are the blocks' rows
  P.near_off_t.assign(nd, 0);
  P.near_seg_t.assign(nleaf + 1, 0);
  P.didx_t_ptr.assign(nleaf + 1, 0);
  P.didx_t.clear();
  off = 0;
  for (int l = 0; l < nleaf; l++) {
    P.near_seg_t[l] = off;
    for (int b : tn[l]) {
      const int* q = &P.direct[4 * b];
      P.near_off_t[b] = off;
      off += (int64_t)(q[1] - q[0]) * (q[3] - q[2]);
      for (int r = q[0]; r < q[1]; r++) P.didx_t.push_back(r);
    }
    if ((P.didx_t.size() - P.didx_t_ptr[l]) & 1) {
      P.didx_t.push_back(-1);
      off += P.leaf_start[l + 1] - P.leaf_start[l];
    }
    P.didx_t_ptr[l + 1] = (int)P.didx_t.size();
  }
  P.near_seg_t[nleaf] = off;
  P.near_total_t = off;
  csr(fl, P.fw_lr_ptr, P.fw_lr);
  csr(tn, P.tr_near_ptr, P.tr_near);
  csr(tl, P.tr_lr_ptr, P.tr_lr);

  P.iter_lim.assign(na, 0);
  for (int b = 0; b < na; b++) {
    const int* q = &P.approx[4 * b];
    P.iter_lim[b] = std::max(0, std::min(maxk, std::min(q[1] - q[0] - 1, q[3] - q[2] - 1)));
  }
  // block -> its entries in the leaf lists, in leaf order
  auto inv = [&](const std::vector<int>& items, std::vector<int>& bptr, std::vector<int>& bl, std::vector<int>& pos) {
    bptr.assign(na + 1, 0);
    for (int b : items) bptr[b + 1]++;
    for (int b = 0; b < na; b++) bptr[b + 1] += bptr[b];
    bl.assign(items.size(), 0);
    pos.assign(items.size(), 0);
    std::vector<int> fill(bptr.begin(), bptr.end() - 1);
    for (size_t e = 0; e < items.size(); e++) {
      pos[e] = fill[items[e]];
      bl[fill[items[e]]++] = (int)e;
    }
  };
  inv(P.fw_lr, P.blk_fw_ptr, P.blk_fw, P.fw_pos);
  inv(P.tr_lr, P.blk_tr_ptr, P.blk_tr, P.tr_pos);

  P.aca_order.resize(na);
  std::iota(P.aca_order.begin(), P.aca_order.end(), 0);
  std::stable_sort(P.aca_order.begin(), P.aca_order.end(), [&](int a, int c) {
    int sa = P.approx[4 * a + 1] - P.approx[4 * a] + P.approx[4 * a + 3] - P.approx[4 * a + 2];
    int sc = P.approx[4 * c + 1] - P.approx[4 * c] + P.approx[4 * c + 3] - P.approx[4 * c + 2];
    return sa > sc;
  });
}

}  // namespace ac3d
