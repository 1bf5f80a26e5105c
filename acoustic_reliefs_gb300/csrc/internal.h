// Internal declarations shared by the host orchestration (api.cpp, tree.cpp) and the CUDA
// translation units. Nothing here is part of the public C-ABI (include/ac3d.h).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <stdexcept>
#include <string>
#include <vector>

namespace ac3d {

constexpr double kPiHost = 3.14159265358979323846;

// Kernels launched by this library: process-wide, and by the calling thread (so that a context's
// counts and the captured-node accounting of its graphs are not mixed with other threads');
// graph replays add their captured node count.
extern std::atomic<long long> g_kernel_launches;
extern thread_local long long t_kernel_launches;
inline void note_launch(long long n = 1) {
  g_kernel_launches.fetch_add(n, std::memory_order_relaxed);
  t_kernel_launches += n;
}
// A stream capture's launches were counted by note_launch but are graph nodes, not launches.
inline void unnote_launches(long long n) {
  g_kernel_launches.fetch_sub(n, std::memory_order_relaxed);
  t_kernel_launches -= n;
}

// ------------------------------------------------------------------------------------------
// Errors: host code throws; the C-ABI converts to status codes + a per-context message.
// ------------------------------------------------------------------------------------------
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

void cuda_check(cudaError_t e, const char* what, const char* file, int line);
#define AC3D_CUDA(x) ::ac3d::cuda_check((x), #x, __FILE__, __LINE__)

// ------------------------------------------------------------------------------------------
// Device buffer (stream-ordered allocation on the owning context's stream).
// ------------------------------------------------------------------------------------------
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaStream_t s = nullptr;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept { *this = std::move(o); }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      release();
      p = o.p;
      bytes = o.bytes;
      s = o.s;
      o.p = nullptr;
      o.bytes = 0;
    }
    return *this;
  }
  ~DevBuf() { release(); }
  void alloc(size_t n, cudaStream_t stream);
  void ensure(size_t n, cudaStream_t stream) {
    if (n > bytes) alloc(n, stream);
  }
  void release();
  template <typename T>
  T* as() const { return (T*)p; }
};

// ------------------------------------------------------------------------------------------
// Cluster tree and block partition (host; ClusterTree, clustertree.cpp:49-137)
// ------------------------------------------------------------------------------------------
struct TreeNode {
  double c[3];
  double r;
  int s, e;
  int left, right;
  bool leaf;
};

struct Partition {
  int ne = 0;
  std::vector<int> order;              // tree position -> original element index
  std::vector<TreeNode> nodes;
  std::vector<int> direct;             // 4 ints per near block (rs, re, cs, ce)
  std::vector<int> approx;             // 4 ints per admissible block
  std::vector<int> leaf_start;         // leaf ranges, ascending (nleaf + 1 entries)
  // Per-leaf work lists (CSR), forward (row leaves) and transposed (column leaves).
  std::vector<int> fw_near_ptr, fw_near;   // near blocks whose rows are the leaf
  std::vector<int> fw_lr_ptr, fw_lr;       // admissible blocks whose rows contain the leaf
  std::vector<int> tr_near_ptr, tr_near;   // near blocks whose columns are the leaf
  std::vector<int> tr_lr_ptr, tr_lr;       // admissible blocks whose columns contain the leaf
  std::vector<int64_t> near_off;       // element offset of each near block (column-major storage);
                                       // blocks of one row leaf are consecutive, so a leaf's near data is
                                       // one R x NC column-major segment
  int64_t near_total = 0;
  std::vector<int64_t> near_seg;       // per leaf: element offset of its near segment
  std::vector<int> didx_ptr, didx;     // per leaf: global column index of every near-segment column
  // the same for the transposed near field (segments of A^T by leaf; columns = global rows)
  std::vector<int64_t> near_off_t, near_seg_t;
  std::vector<int> didx_t_ptr, didx_t;
  int64_t near_total_t = 0;
  // per admissible block: its entries in the fw_lr / tr_lr lists (one per row / column leaf),
  // in leaf order; the matvec sums a term's per-leaf partial dots over these
  std::vector<int> blk_fw_ptr, blk_fw, blk_tr_ptr, blk_tr;
  std::vector<int> fw_pos, tr_pos;     // list entry -> its position in the block-major lists
  std::vector<int> iter_lim;           // per admissible block: min(maxk, m - 1, n - 1)
  std::vector<int> aca_order;          // admissible blocks by decreasing m + n
  int max_rows = 0;                    // largest admissible block row count
  int64_t aca_term_cap = 0;            // sum over blocks of min(maxk, m-1, n-1)
  int max_leaf = 0;
  bool tree_ok = true;
};

void build_partition(const double* C, int ne, int leaf_size, double factor, Partition& P);
void build_leaf_lists(Partition& P, int maxk);

// ------------------------------------------------------------------------------------------
// Device views
// ------------------------------------------------------------------------------------------
struct DevPartition {
  int ne = 0;  // elements
  int nleaf = 0, nd = 0, na = 0;
  // aca_order is split into blocks for the CTA ACA kernel, then warp-per-block ACA for blocks of
  // at most 256, 128 and 64 rows and columns; aca_split holds the four counts
  int aca_split[4] = {0, 0, 0, 0};
  int max_leaf = 0;
  DevBuf near_seg, didx_ptr, didx;
  DevBuf near_off_t, near_seg_t, didx_t_ptr, didx_t;  // transposed near layout (block adjoint)
  int64_t near_total_t = 0;
  DevBuf blk_fw_ptr, blk_fw, blk_tr_ptr, blk_tr;
  DevBuf fw_pos, tr_pos;
  DevBuf blocks_d, blocks_a;            // int4
  DevBuf leaf_start;                    // int (nleaf + 1)
  DevBuf fw_near_ptr, fw_near, fw_lr_ptr, fw_lr;
  DevBuf tr_near_ptr, tr_near, tr_lr_ptr, tr_lr;
  DevBuf near_off;                      // int64
  DevBuf aca_order;                     // int
};

// Element geometry on device (recomputed from vertex positions for every height update).
struct DevGeometry {
  int ne = 0, nv = 0;
  DevBuf P;          // double (nv x 3)
  DevBuf E;          // int (ne x 3), tree order
  DevBuf cen, va;    // double4
  DevBuf cen32, va32;  // float4
  DevBuf eg32;       // ElemGeo<float>
  DevBuf eg64;       // ElemGeo<double>
  DevBuf cen_df;     // DfPt: centroids as double-floats (mixed-precision entry evaluation)
  DevBuf el_df;      // DfElem: quadrature points and normal as double-floats
  DevBuf df_tab;     // float4 [256]: cos / sin of j 2 pi / 256 as double-floats
};

// One mesh: positions, elements in tree order, block partition (host and device) and element
// geometry. Read-only while solves run on it, so several contexts (a server's slots) share one.
struct MeshState {
  int V = 0, Ne = 0;
  std::vector<double> Ps0;  // base positions (V x 3)
  std::vector<int> Es;      // elements in tree order (Ne x 3)
  Partition P;
  DevPartition DP;
  DevGeometry G;
  int64_t sum_mn = 0;      // sum over admissible blocks of m + n
  int64_t worst_pool = 0;  // ACA pool entries if every block reached its iteration limit
  std::atomic<int64_t> pool_hint[2];  // per storage precision: pool size the last assembly needed
  bool geom_base = false;  // G holds Ps0 (no heights applied)
  MeshState() {
    pool_hint[0] = 0;
    pool_hint[1] = 0;
  }
};

enum Precision { PREC_MIXED = 0, PREC_FP64 = 1 };

// Warp-per-block ACA: largest block side and largest number of iterations it handles.
constexpr int kWarpAcaMaxDim = 256;
constexpr int kWarpAcaTerms = 128;

// An assembled H-matrix of (K - I/2) at one wavenumber.
struct DevHMat {
  int prec = PREC_MIXED;  // storage: complex FP32 (mixed) or complex FP64
  bool pool_df = false;   // mixed storage assembled in double-float: the ACA pool holds cdf terms
  double k = 0;
  int maxk = 100;
  DevBuf near;            // complex storage of all near blocks
  DevBuf nearT;           // transposed near field (FP32; built on the first transposed block matvec)
  DevBuf tcseg_f, tcseg_t;  // TF32 hi / lo split of the U / V segments (tensor-core block dot pass)
  DevBuf tcoff_f, tcoff_t;  // int64 [nleaf + 1]: byte offsets into tcseg_f / tcseg_t
  DevBuf pool;            // rank-1 terms (u | v) of all admissible blocks
  DevBuf term_off;        // int64 [na * maxk] offset of each term in the pool
  DevBuf rank;            // int [na]
  DevBuf passes;          // int [na]: ACA loop passes (rows and columns evaluated) per block
  DevBuf t_off;           // int [na + 1] prefix of ranks
  DevBuf task_b;          // int [sum ranks] block of each stored term
  DevBuf task_off;        // int64 [sum ranks] pool offset of each stored term
  // per-leaf segments packed from the pool after ACA (the pool is released afterwards)
  DevBuf kseg_f, kseg_t;  // int [nleaf + 1]: prefix of (even-padded) segment columns per row / column leaf
  DevBuf seg_f, seg_t;    // int64 [nleaf + 1]: element prefix of the U / V segments
  DevBuf useg, vseg;      // R x K column-major slices of U (row leaves) / V (column leaves)
  DevBuf uidx, vidx;      // int: phase-1 output index of every segment column (-1: padding)
  DevBuf kpos_f, kpos_t;  // int: first segment column of every list entry, block-major order
  DevBuf order_rows, order_cols;  // int [nleaf]: leaves by decreasing streamed bytes (gather / dot)
  DevBuf pbuf;            // per-column partial dots of the dot pass
  DevBuf err;             // int: set by a kernel whose copy pipeline timed out
  DevBuf ticket;          // unsigned: gather-pass completion ticket (zero between launches)
  int64_t task_cap = 0;   // upper bound of the number of stored terms
  DevBuf tvec;            // intermediate V x per term (complex, vector precision)
  DevBuf tvec64;          // FP64 / double-float intermediate for refinement residuals
  DevBuf xdf;             // double-float copy of the residual matvec input (FP32 storage only)
  DevBuf pool_used;       // unsigned long long
  int64_t pool_cap = 0;
  int64_t pool_used_host = 0;
  std::vector<int> ranks_host;
  int64_t lr_entries = 0; // sum r (m + n)
  int64_t aca_evaluated = 0;  // entries ACA evaluated: sum passes (m + n)
  size_t bytes() const {
    return near.bytes + nearT.bytes + tcseg_f.bytes + tcseg_t.bytes + tcoff_f.bytes + tcoff_t.bytes + pool.bytes + term_off.bytes + rank.bytes + t_off.bytes + task_b.bytes + task_off.bytes +
           tvec.bytes + tvec64.bytes + useg.bytes + vseg.bytes + uidx.bytes + vidx.bytes + kpos_f.bytes +
           kpos_t.bytes + pbuf.bytes + kseg_f.bytes + kseg_t.bytes + seg_f.bytes + seg_t.bytes + xdf.bytes;
  }
};

// ------------------------------------------------------------------------------------------
// Kernel launchers (implemented in the .cu files)
// ------------------------------------------------------------------------------------------
void launch_geometry(DevGeometry& G, cudaStream_t s);
void launch_pack_points(const double* p, int n, void* out, cudaStream_t s);
void launch_rhs(const DevGeometry& G, int prec_vec64, double k, int kind, const double* v3, void* out, cudaStream_t s);

void launch_near_assembly(const DevGeometry& G, const DevPartition& DP, DevHMat& H, cudaStream_t s);
// Large blocks run on s, small blocks (one warp each) on s_small, which may be another stream.
void launch_aca(const DevGeometry& G, const DevPartition& DP, DevHMat& H, double eps, int max_rows, cudaStream_t s,
                cudaStream_t s_small);
// Mixed-precision assembly with double-float entries and ACA recursion (FP64-accurate entries,
// pivots and ranks; FP32 storage): near field into H.near (cf), ACA terms into H.pool (cdf).
void launch_near_assembly_df(const DevGeometry& G, const DevPartition& DP, DevHMat& H, cudaStream_t s);
void launch_aca_df(const DevGeometry& G, const DevPartition& DP, DevHMat& H, double eps, int max_rows, cudaStream_t s,
                   cudaStream_t s_small);
void launch_rank_scan(const DevPartition& DP, DevHMat& H, cudaStream_t s);
// Packs the pool into the U segments (row leaves, cols = false) or V segments (column leaves).
void launch_pack(const DevPartition& DP, DevHMat& H, bool cols, cudaStream_t s);

// Matvec y = op(A) x with op = identity or plain transpose. vec: 0 = complex FP32 vectors,
// 1 = complex FP64 vectors. residual: y = b - op(A) x instead (b given).
struct MatvecEpilogue {
  // optional fused dot products over the produced vector y (FP64 partials per CTA)
  const void* dot_a = nullptr;  // if set: partial sum conj(dot_a) . y
  const void* dot_b = nullptr;  // if set: partial sum conj(y) . dot_b  (and |y|^2)
  double* partials = nullptr;   // per-CTA partials [grid x 5]
  double* red5 = nullptr;       // if set: the fixed-order total of the partials (last CTA writes it)
};
void launch_matvec(const DevPartition& DP, const DevHMat& H, int ne, bool transposed, int vec64,
                   const void* x, void* y, const void* b_minus, const MatvecEpilogue& ep, cudaStream_t s);
int matvec_grid(const DevPartition& DP, bool transposed);
int device_sm_count();
// Looks up the allocation-free far field's fixed scratch on the current device (noalloc.cu), so
// that its first call there loads nothing.
void noalloc_prepare();
// Sets the shared-memory limits of the matvec kernels (call outside stream capture).
void prepare_matvec_kernels();

}  // namespace ac3d
