/* C-ABI of libac3d.so: the GB300 BEM hot path behind the reference's `acoustics3d` binding.
 *
 * Each entry point replaces one method of the reference binding class DiffBEM
 * (acoustics3d_cpp/src/acoustics3d.cpp, bound at :353-383) or the free function `sphere`
 * (acoustics3d_cpp/include/sphere.h:28-85); the citation is given beside each declaration.
 * Arguments are plain pointers and sizes. Vertex positions are (V, 3) float64 row-major,
 * connectivity (Ne, 3) int32 row-major, complex outputs interleaved float64 (re, im).
 *
 * Every function returns AC3D_OK (0) or an error code; ac3d_last_error() gives the message.
 * Where the reference printed to std::cerr and returned a sentinel (acoustics3d.cpp:110-113,
 * 133-136, 200-207, 241-243), these return AC3D_ERR_STATE. A context owns one CUDA stream and
 * is not reentrant; use one context per host thread.
 */
#ifndef AC3D_H
#define AC3D_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AC3D_OK 0
#define AC3D_ERR_ARG 1        /* invalid argument */
#define AC3D_ERR_STATE 2      /* mesh / differentiable points not set */
#define AC3D_ERR_INTERNAL 3
#define AC3D_ERR_RESOURCE 4   /* device memory or shared-memory limits */
#define AC3D_ERR_CUDA 5
#define AC3D_ERR_NOT_CONVERGED 6 /* solver hit its iteration limit (results still written) */

#define AC3D_PREC_MIXED 0     /* complex FP32 blocks, FP64 dots and iterative refinement */
#define AC3D_PREC_FP64 1      /* everything complex FP64 */

#define AC3D_INCIDENT_POINT 0 /* point source e^{-ikr}/(4 pi r) at the given point */
#define AC3D_INCIDENT_PLANE 1 /* plane wave e^{-ik d.x} along the given unit vector */

#define AC3D_KRYLOV_BICGSTAB 0 /* the reference's solver (Eigen::BiCGSTAB, adjoint.cpp:92-95) */
#define AC3D_KRYLOV_GMRES 1    /* GMRES: one matvec per iteration, restarted by the refinement loop */

#define AC3D_ASSEMBLY_DF 0    /* mixed precision: entries and ACA in double-float (FP64-accurate
                                 pivots and ranks), stored in FP32 (default) */
#define AC3D_ASSEMBLY_FP32 1  /* mixed precision: entries and ACA in FP32 */

#define AC3D_LISTENER_DENSE 0 /* receiver matrix evaluated exactly on the fly */
#define AC3D_LISTENER_ACA 1   /* receiver matrix by ACA with Q_ACA_tol, as the reference */

typedef struct ac3d_ctx ac3d_ctx;

/* Statistics of the most recent call. */
typedef struct ac3d_stats {
  int n_elements, n_direct, n_approx, n_leaves;
  long long near_entries, lr_entries; /* stored complex entries */
  double mean_rank;
  int max_rank;
  long long hmat_bytes;     /* device bytes of the last H-matrix (including the split segments of
                               tensor-core block matvecs once they are built) */
  int solves;               /* linear solves in the call */
  int iterations;           /* Krylov iterations, summed over solves and refinement steps */
  int outer_steps;          /* refinement steps (mixed precision) summed over solves */
  int matvecs;
  double rel_residual;      /* final |b - A x| / |b| of the last solve (FP64) */
  int converged;            /* 1 if every solve met solver_tol */
  double ms_assemble, ms_solve, ms_listener, ms_adjoint, ms_total;
  long long kernel_launches; /* kernels this library launched in the call (graph nodes counted) */
  long long aca_entries_evaluated; /* matrix entries ACA evaluated (rows and columns of every pass,
                                      6 kernel evaluations each) in the last assembly */
  double ms_graph;          /* host milliseconds spent capturing and instantiating solver graphs */
} ac3d_stats;

/* DiffBEM(cluster_size, radius_factor, freq_bands, n_freqs, approx_ACA_tol, Q_ACA_tol,
 *         solver_tol, src_pt, listener_radius, listener_ds, recompute_matrices)
 * -- acoustics3d.cpp:22-34 (constructor), defaults at :355-357. */
int ac3d_create(ac3d_ctx** ctx, int cluster_size, double radius_factor, const double* freq_bands, int n_bands,
                int n_freqs, double approx_aca_tol, double q_aca_tol, double solver_tol, const double* src_pt,
                double listener_radius, double listener_ds, int recompute_matrices);
void ac3d_destroy(ac3d_ctx* ctx);
/* Selects the CUDA device used by contexts created afterwards on the calling host thread
 * (the library carries its own CUDA runtime, so another runtime's current device does not
 * carry over). No reference counterpart: the reference is CPU-only. */
int ac3d_select_device(int device);
const char* ac3d_last_error(const ac3d_ctx* ctx);

/* Options with no reference counterpart (the reference is FP64, point source, ACA receivers). */
int ac3d_set_precision(ac3d_ctx* ctx, int precision);
int ac3d_set_incident(ac3d_ctx* ctx, int kind, const double* v3);
int ac3d_set_listener_mode(ac3d_ctx* ctx, int mode);
int ac3d_set_solver(ac3d_ctx* ctx, int max_iterations, double inner_tol, int max_outer);
/* Krylov method of the single right-hand-side solves (forward, adjoint, exact operator):
 * AC3D_KRYLOV_BICGSTAB (default, as the reference) or AC3D_KRYLOV_GMRES with a basis of `restart`
 * vectors (1..600; 0: 300). GMRES stops on the same relative residual; each cycle of at most
 * `restart` iterations is followed by a true-residual check of the refinement loop, which starts
 * the next cycle if needed (at most max_outer cycles; max_iterations applies to BiCGSTAB only).
 * Block solves (ac3d_solve_multi) then run one GMRES cycle per direction, the cycles sharing each
 * block matvec, instead of block BiCGSTAB. No reference counterpart. */
int ac3d_set_krylov(ac3d_ctx* ctx, int method, int restart);
/* Arithmetic of the mixed-precision assembly (no effect on AC3D_PREC_FP64): AC3D_ASSEMBLY_DF
 * (default) evaluates near-field entries, the admissible blocks' rows and columns, and runs ACA
 * (compute_ACA_block, aca.cpp:38-82; receivers aca.cpp:84-134) in double-float arithmetic on the
 * FP32 pipes, so the low-rank blocks have the FP64 path's pivots and ranks and every stored entry
 * differs from the FP64 path's only by its FP32 rounding; AC3D_ASSEMBLY_FP32 evaluates in FP32
 * (faster; pivots and ranks may differ from the FP64 path's where candidates are within FP32
 * rounding of each other). No reference counterpart. */
int ac3d_set_assembly(ac3d_ctx* ctx, int mode);
/* Block matvecs of 8 or 16 right-hand sides (ac3d_solve_multi, ac3d_gradient_multi) form their
 * dot pass S^T X on the tensor cores (tcgen05.mma, TF32 operands split so that three products
 * keep FP32 accuracy, FP32 accumulation) when on (default) and leaves have at most 32 elements;
 * off: FP32 CUDA cores. The first such matvec of an H-matrix stores the split segments it
 * streams (about twice the low-rank V or U storage). No reference counterpart. */
int ac3d_set_tensor_cores(ac3d_ctx* ctx, int on);
/* Replace the receivers used by value / values / band_value / gradient (default: the
 * hemisphere of compute_listener_pts, helpers.cpp:52-65). */
int ac3d_set_listeners(ac3d_ctx* ctx, const double* Ls, int L);

/* set_mesh(Ps, Es) -> (Ps, Es reordered) -- acoustics3d.cpp:36-67. Es_out (Ne x 3) receives the
 * tree-ordered connectivity; Ps is not permuted. */
int ac3d_set_mesh(ac3d_ctx* ctx, const double* Ps, int V, const int32_t* Es, int Ne, int32_t* Es_out);
/* set_diff_points(diff_pts) -- acoustics3d.cpp:69-101. */
int ac3d_set_diff_points(ac3d_ctx* ctx, const int32_t* diff_pts, int HH);
/* set_band(freq_band) -- acoustics3d.cpp:348-351; ac3d_set_bands replaces the whole list. */
int ac3d_set_band(ac3d_ctx* ctx, double freq_band);
int ac3d_set_bands(ac3d_ctx* ctx, const double* freq_bands, int n_bands);

/* get_listeners() -- acoustics3d.cpp:317-319. */
int ac3d_num_listeners(const ac3d_ctx* ctx, int* L);
int ac3d_get_listeners(const ac3d_ctx* ctx, double* Ls_out);
/* Replace all vertex positions (same topology; the block partition of set_mesh is kept, as the
 * reference keeps it across height updates, acoustics3d.cpp:139-146). */
int ac3d_set_points(ac3d_ctx* ctx, const double* Ps);

/* pvals(frequency[, listeners]) -- acoustics3d.cpp:236-280. Ls may be NULL (context receivers);
 * out receives L complex pressures. */
int ac3d_pressures(ac3d_ctx* ctx, double frequency, const double* Ls, int L, double* out);
/* Same as ac3d_pressures with receivers (L x 3 float64) and output (L complex) in device memory,
 * ordered after `stream` (a cudaStream_t), which waits for completion. Ls_dev may be NULL
 * (context receivers). No host copies of inputs or outputs. */
int ac3d_pressures_dev(ac3d_ctx* ctx, double frequency, const double* Ls_dev, int L, double* out_dev, void* stream);
/* Forward solves of nrhs incident fields at one frequency against one H-matrix: block BiCGSTAB
 * (or, with ac3d_set_krylov GMRES, one GMRES cycle per right-hand side sharing each block matvec)
 * over up to 16 right-hand sides at a time (more run in batches of 16), each matrix byte read once
 * per matvec for the whole block. kind: AC3D_INCIDENT_*; vecs: nrhs x 3 (plane-wave directions or
 * point-source positions). p_out (nrhs x L complex) receives the pressures at the receivers Ls
 * (L x 3; NULL: the context's receivers), x_out (nrhs x Ne complex, tree order) the surface
 * solutions; either may be NULL. No reference counterpart: the reference solves one right-hand
 * side at a time (bem3d::gradient, adjoint.cpp:92-95; DiffBEM::pvals, acoustics3d.cpp:236-280). */
int ac3d_solve_multi(ac3d_ctx* ctx, double frequency, int kind, const double* vecs, int nrhs, const double* Ls, int L,
                     double* p_out, double* x_out);
/* surface_vals(frequency) -- acoustics3d.cpp:282-315; out receives Ne complex values. */
int ac3d_surface_values(ac3d_ctx* ctx, double frequency, double* out);
/* band_value(freq_band) -- acoustics3d.cpp:162-176. */
int ac3d_band_value(ac3d_ctx* ctx, double freq_band, double* c);
/* values() -- acoustics3d.cpp:178-197; out receives one coefficient per band. */
int ac3d_values(ac3d_ctx* ctx, double* out);
/* value() / value(x) -- acoustics3d.cpp:109-160: mean over bands; x (HH heights) may be NULL. */
int ac3d_value(ac3d_ctx* ctx, const double* x, double* c);
/* gradient(x) -> (c, dc/dx) -- acoustics3d.cpp:199-234: c and gradient summed over bands. */
int ac3d_gradient(ac3d_ctx* ctx, const double* x, double* c, double* grad);
/* Same as ac3d_value / ac3d_gradient with x, c and grad in device memory; the work is ordered
 * after `stream` (a cudaStream_t) and `stream` waits for its completion. */
int ac3d_value_dev(ac3d_ctx* ctx, const double* x_dev, double* c_dev, void* stream);
int ac3d_gradient_dev(ac3d_ctx* ctx, const double* x_dev, double* c_dev, double* grad_dev, void* stream);
/* Multi-incidence objective: loss = 1 - mean over the nf frequencies and nd plane-wave directions
 * (nd x 3, normalised here) of the diffusion coefficient of the context's receivers for that one
 * frequency and direction (compute_u, adjoint.cpp:388-397, on one |y|), with heights x (HH);
 * grad (HH) receives d loss / dx, coefs (nf x nd, frequency-major, may be NULL) the coefficients.
 * The gradient is the reference's adjoint (adjoint.cpp:24-242) per frequency and direction; here
 * the directions of a frequency share one H-matrix, forward and transposed block solves and every
 * shape-derivative evaluation. No reference counterpart as one call (the reference's objective has
 * one point source). */
int ac3d_gradient_multi(ac3d_ctx* ctx, const double* x, const double* freqs, int nf, const double* dirs, int nd,
                        double* loss, double* grad, double* coefs);

/* sphere(sphere_mesh, freq, LL, lrad, actual) -- sphere.h:28-85, with the mesh passed as
 * arrays instead of an OBJ path: leaf 128, factor 1.5, ACA and solver tolerance 1e-10, plane
 * wave e^{-ikx}, LL receivers on a circle of radius lrad in the xz plane. actual != 0 replaces the
 * reference's dense QR solve (sphere.h:65-69) by the exact operator (every leaf pair a dense
 * block, FP64) solved to 1e-12 by the context's Krylov method (BiCGSTAB by default). */
int ac3d_sphere(const double* Ps, int V, const int32_t* Es, int Ne, double freq, int LL, double lrad, int precision,
                int actual, double* out);
/* use_actual attribute (acoustics3d.h:49; adjoint.cpp:33-83,148-170): when on, band_value,
 * values, value and gradient (and their _dev forms) run on the exact operator -- the same tree
 * with every leaf pair a dense block, FP64, exact receiver product, solved to 1e-12 (BiCGSTAB by
 * default) in place of the reference's dense QR solve. pvals and surface_vals keep the H-matrix, as in the reference. */
int ac3d_set_actual(ac3d_ctx* ctx, int on);

/* read_obj / write_obj -- read_obj.cpp:8-63. ac3d_read_obj reads "v" and triangle "f" records
 * (vertex index of "a", "a/b", "a//c", "a/b/c"; negative indices relative to the vertices read so
 * far) and skips "vn", "vt", "vp", comments and grouping / material records, where the reference
 * rejects files that have them. With Ps and Es NULL it only sets *V and *Ne; otherwise it fills
 * Ps (V x 3) and Es (Ne x 3, 0-based) when V_cap and Ne_cap hold the mesh (else
 * AC3D_ERR_RESOURCE). Faces that are not triangles and indices out of range are AC3D_ERR_ARG.
 * ac3d_write_obj writes full-precision vertices (a write / read round trip is exact) and 1-based
 * faces. No context: ac3d_obj_last_error() gives the calling thread's last message. */
int ac3d_read_obj(const char* path, double* Ps, int V_cap, int32_t* Es, int Ne_cap, int* V, int* Ne);
int ac3d_write_obj(const char* path, const double* Ps, int V, const int32_t* Es, int Ne);
const char* ac3d_obj_last_error(void);

/* Heightmap texture -> differentiable-vertex heights and back (eval_uv, acoustics_opt.py:23-33,
 * and the texture gradient of acoustic_gradient, acoustics_opt.py:44-57). A texmap holds, on the
 * current device, the bilinear texel indices and weights of n uv points (n x 2, (0, 0) at the
 * top-left texel's corner) on an H x W texture, and the transposed (texel-major) lists.
 * ac3d_texmap_sample_dev: heights (n) from the texture (H x W row-major), both FP64 device arrays;
 * ac3d_texmap_scatter_dev: texture gradient (H x W) from per-point gradients (n). Both are
 * ordered on `stream` (a cudaStream_t) and give the reference's NumPy results bitwise. */
typedef struct ac3d_texmap ac3d_texmap;
int ac3d_texmap_create(ac3d_texmap** out, const double* uvs, int n, int H, int W);
void ac3d_texmap_destroy(ac3d_texmap* map);
int ac3d_texmap_sample_dev(const ac3d_texmap* map, const double* tex_dev, double* heights_dev, void* stream);
int ac3d_texmap_scatter_dev(const ac3d_texmap* map, const double* grad_dev, double* tex_grad_dev, void* stream);

/* Kernels this library has launched in the process so far, from every context, server slot and
 * thread (a graph replay counts its kernel nodes). No reference counterpart. */
long long ac3d_kernel_launches(void);

int ac3d_get_stats(const ac3d_ctx* ctx, ac3d_stats* out);
/* Times `iters` back-to-back H-matrix matvecs (y = op(A) x, inner-solve precision) on the
 * H-matrix of the most recent ac3d_pressures / ac3d_surface_values call, with CUDA events on the
 * context stream, in the variant the context's solver runs, launched as in the solve (programmatic
 * dependent launches). Outputs the mean milliseconds per matvec and the algorithmic bytes per
 * matvec: stored matrix entries x entry size + reading x and writing y (32 Ne for FP64 vectors,
 * + 8 Ne for the FP32 shadow of x the mixed BiCGSTAB reads; 16 Ne for the FP32 vectors of the
 * mixed GMRES). No reference counterpart. */
int ac3d_matvec_timing(ac3d_ctx* ctx, int iters, int transposed, double* ms_per_matvec, long long* bytes);
/* ACA ranks (stored terms, after the dropped converging term; aca.cpp:78-79) of every admissible
 * block of the H-matrix of the most recent ac3d_pressures / ac3d_surface_values call, in the
 * order of ac3d_partition_get's approx list; n must equal that count (stats n_approx). No
 * reference counterpart (the reference keeps them inside HMatrix, hmatrix.h:27-71). */
int ac3d_get_ranks(ac3d_ctx* ctx, int32_t* ranks, int n);
/* Times the block matvec of nrb (4, 8 or 16) right-hand sides (A, or its plain transpose with
 * transposed != 0) on the FP32 H-matrix of the most recent solve, as the block solvers launch it,
 * with CUDA events on the context stream. Outputs the mean milliseconds per block matvec and its
 * algorithmic bytes: stored entries x 8 + the block input and output (8 Ne nrb each). No reference
 * counterpart. */
int ac3d_block_matvec_timing(ac3d_ctx* ctx, int nrb, int iters, int transposed, double* ms, long long* bytes);

/* Receiver far field y_l = sum_j M(receiver l, element j) x_j (FP64), with every argument in
 * device memory: Ps_dev (V x 3 float64), Es_dev (Ne x 3 int32, the connectivity x is ordered by,
 * e.g. the Es returned by ac3d_set_mesh), x_dev (Ne complex), Ls_dev (L x 3 float64), y_dev (L
 * complex); k = 2 pi f / 344. It allocates no device memory: for callers that cannot allocate
 * at that point (a real-time audio callback, a frame loop, a host whose allocator owns the device
 * memory). Its scratch is a fixed 65536-entry (1 MiB) array reserved on every GPU that loads the
 * library; L above 65536 is rejected with AC3D_ERR_RESOURCE. It runs on this library's current
 * device, which is not another CUDA runtime's (torch's) current device: select it with
 * ac3d_select_device on the calling thread. The array's address is looked up once per device,
 * which also loads the entry point's kernels there (CUDA loads modules lazily, and loading
 * reserves the array): ac3d_create does this for its device, and otherwise the first call does
 * it and may allocate, so make that first call before any stream capture and outside the
 * allocation-free section. The address is not valid across a cudaDeviceReset of the device. All
 * calls share the array: calls that overlap on the GPU (different streams) race. Work is ordered
 * on `stream` (a cudaStream_t); the call does not wait for it. A launch failure returns
 * AC3D_ERR_CUDA; errors pending from earlier unrelated work are left alone. Elements whose
 * indices fall outside [0, V) are skipped. No counterpart in the reference (its far field is a host ACA
 * product, aca.cpp:84-134 with adjoint.cpp:101-102). */
int ac3d_far_field_noalloc(const double* Ps_dev, int V, const int32_t* Es_dev, int Ne, const double* x_dev, double k,
                           const double* Ls_dev, int L, double* y_dev, void* stream);

/* Relief mesh generated on the device (generate_base_mesh + face_subdivision,
 * pyoptim/mesher.py:87-231; top vertices and uvs as acoustics_opt.py:182-210): a w x h x b box of
 * six unwelded structured face grids (nx x ny, nx x nz, ny x nz quads, two triangles each), the
 * top face (y = h) subdivided subdiv_top times 1 -> 4. ac3d_relief_sizes gives the vertex and
 * triangle counts; ac3d_relief_dev writes Ps_dev (V x 3 float64), Es_dev (F x 3 int32), the top
 * vertex ids top_dev and their uvs uvs_dev (n_top x 2 float64; both sized for up to V entries), on
 * `stream`, and waits for it. Bitwise the host generator's output. Heights from a heightmap are then
 * the texture lookup of ac3d_texmap_sample_dev at these uvs. */
int ac3d_relief_sizes(int nx, int ny, int nz, int subdiv_top, int* V, int* F);
int ac3d_relief_dev(double w, double b, double h, int nx, int ny, int nz, int subdiv_top, double* Ps_dev,
                    int32_t* Es_dev, int32_t* top_dev, double* uvs_dev, int* n_top, void* stream);

/* Host-only cluster tree and block partition (ClusterTree, clustertree.cpp:49-137, as used by
 * set_mesh, acoustics3d.cpp:43-58). No GPU work: for inspection and tests. */
typedef struct ac3d_partition ac3d_partition;
int ac3d_partition_build(const double* Ps, int V, const int32_t* Es, int Ne, int cluster_size, double radius_factor,
                         ac3d_partition** out);
/* counts: n_direct, n_approx, n_leaves, tree_ok (1 if every centroid lies inside its node radius) */
int ac3d_partition_counts(const ac3d_partition* p, int* n_direct, int* n_approx, int* n_leaves, int* tree_ok);
/* order (Ne): tree position -> input element; direct (4 n_direct), approx (4 n_approx): blocks
 * (row start, row end, column start, column end) in traversal order; leaves (n_leaves + 1). */
int ac3d_partition_get(const ac3d_partition* p, int32_t* order, int32_t* direct, int32_t* approx, int32_t* leaves);
void ac3d_partition_free(ac3d_partition* p);
/* Library version string. */
const char* ac3d_version(void);
/* Self-check of the tensor-core product of the block matvec: D (128 x 32) = A (128 x K) B^T with
 * B (32 x K), all row-major FP32 host arrays, K a multiple of 8 up to 128, formed by one CTA with
 * tcgen05.mma (TF32 operands split in three products, FP32 accumulation in tensor memory). No
 * reference counterpart. */
int ac3d_tensor_selftest(const float* A, const float* B, int K, float* D);

/* ---------------------------------------------------------------------------------------------
 * Request server. No reference counterpart: the reference solves one frequency at a time inside
 * DiffBEM (bem3d::gradient's frequency loop, adjoint.cpp:46-104). A server keeps registered
 * meshes (tree, partition, geometry) on the device and runs `slots` solver contexts, each on its
 * own CUDA stream and host thread, so the kernels of up to `slots` requests overlap on the GPU.
 * A queued request is admitted when a slot is free and its estimated device footprint fits in
 * what the admitted requests leave of the byte budget (first in, first out; a request that does
 * not fit may be overtaken by later ones that do, at most AC3D_SERVE_MAX_BYPASS times). Each
 * request's result does not depend on what runs beside it: every sum has a fixed order.
 * ------------------------------------------------------------------------------------------- */
typedef struct ac3d_server ac3d_server;

#define AC3D_REQ_QUEUED 0
#define AC3D_REQ_RUNNING 1
#define AC3D_REQ_DONE 2
#define AC3D_REQ_FAILED 3
#define AC3D_SERVE_MAX_BYPASS 8

typedef struct ac3d_request_info {
  int status;                  /* AC3D_OK or the error code of the request */
  int slot;                    /* slot that ran it */
  double queue_ms;             /* submit -> admitted */
  double run_ms;               /* admitted -> result on the host */
  double latency_ms;           /* submit -> result on the host */
  long long footprint_bytes;   /* admission estimate */
  long long hmat_bytes;        /* device bytes of the assembled H-matrix */
  long long lr_entries, near_entries;
  int iterations, outer_steps; /* Krylov iterations; refinement steps */
  double rel_residual;         /* final FP64 |b - A x| / |b| */
  double ms_assemble, ms_solve, ms_listener; /* device time of the phases */
  double ms_graph;             /* host time capturing and instantiating solver graphs (within run_ms) */
  long long aca_entries_evaluated; /* matrix entries the ACA of this request evaluated */
} ac3d_request_info;

/* precision: AC3D_PREC_*; hbm_budget_bytes <= 0 takes 85% of the device memory free at creation. */
int ac3d_server_create(ac3d_server** out, int slots, int precision, long long hbm_budget_bytes);
/* Waits for every submitted request, then releases the slots, meshes and streams. */
void ac3d_server_destroy(ac3d_server* srv);
/* Krylov method of the requests that start after the call (ac3d_set_krylov semantics). No
 * reference counterpart. */
int ac3d_server_set_krylov(ac3d_server* srv, int method, int restart);
/* Mixed-precision assembly arithmetic of the requests that start after the call
 * (ac3d_set_assembly semantics). No reference counterpart. */
int ac3d_server_set_assembly(ac3d_server* srv, int mode);
const char* ac3d_server_last_error(const ac3d_server* srv);
/* Registers a mesh (set_mesh semantics: Es_out, if given, receives the tree-ordered connectivity
 * the results refer to) with its H-matrix and solver parameters. */
int ac3d_server_add_mesh(ac3d_server* srv, const double* Ps, int V, const int32_t* Es, int Ne, int cluster_size,
                         double radius_factor, double aca_tol, double solver_tol, int32_t* Es_out, int* mesh_id);
/* Queues a forward solve at `frequency` with incident field `incident_kind` / `incident_vec`
 * (AC3D_INCIDENT_*) and pressures at the L receivers Ls (L x 3, copied). Fails with
 * AC3D_ERR_RESOURCE if the request's footprint estimate exceeds the whole budget. */
int ac3d_server_submit(ac3d_server* srv, int mesh_id, double frequency, int incident_kind, const double* incident_vec,
                       const double* Ls, int L, long long* request);
/* state: AC3D_REQ_* */
int ac3d_server_poll(ac3d_server* srv, long long request, int* state);
/* Blocks until the request finishes, copies its L complex pressures (2L doubles) into out and its
 * record into info (either may be NULL), and forgets the request. Returns the request's status. */
int ac3d_server_wait(ac3d_server* srv, long long request, double* out, ac3d_request_info* info);
/* Admission rule of the server as a pure function (no GPU): given the footprints of the queued
 * requests in arrival order, how often each was overtaken, the budget and the bytes in use,
 * returns the queue index to admit next, or -1 if none may start now. */
int ac3d_admit_next(const long long* footprints, const int* bypassed, int n_queued, long long budget,
                    long long in_use, int n_running);

#ifdef __cplusplus
}
#endif

#endif /* AC3D_H */
