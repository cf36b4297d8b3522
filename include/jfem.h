/* jfem.h — C ABI of libjfem_cuda.so, the sm_103a elasticity hot path.
 *
 * Plain C types only: host pointers unless a name says "device".  All calls are
 * synchronous on return (work runs on a context-owned CUDA stream).  A context is
 * not thread-safe; use one per host thread.  Status: 0 OK, >0 soft outcome,
 * <0 error (message in jfem_last_error).
 *
 * The entry points replace these reference interfaces (JuliaFEM.jl):
 *   backend plugin   initialize_backend(::GPU, physics, time)   ext/JuliaFEMCUDAExt.jl:867-869
 *                    solve_backend!(data, physics; tol, ...)     ext/JuliaFEMCUDAExt.jl:886-916
 *                    (declared src/backend/abstract.jl:228,241, dispatched :195-200)
 *   legacy assembly  assemble!(assembly, ::Problem{Elasticity}, elements, time)
 *                    src/problems_elasticity.jl:65-81 (element kernel :203-451,
 *                    surface loads :454-502) filling assembly.K / assembly.f
 *                    (src/assembly/problems.jl:14-40) and the COO→CSC of
 *                    src/solvers.jl:57-93.
 */
#ifndef JFEM_H
#define JFEM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define JFEM_OK                0
#define JFEM_NOT_CONVERGED     1   /* like the @warn of ext/JuliaFEMCUDAExt.jl:630 */
#define JFEM_STALL             2   /* learned preconditioner stalled; fell back to Jacobi */
#define JFEM_ERR_INVALID      -1   /* bad argument / call order (error() in the reference) */
#define JFEM_ERR_CUDA         -2
#define JFEM_ERR_OOM          -3   /* device or host memory (or host threads) exhausted */
#define JFEM_ERR_NEG_JACOBIAN -4   /* detJ <= 0 in an element */
#define JFEM_ERR_NAN          -5   /* NaN/Inf, or J <= 0 in the Neo-Hookean law */
#define JFEM_ERR_TIMEOUT      -6   /* a bounded device loop ran out of its budget */
#define JFEM_ERR_TOO_LARGE    -7   /* jfem_apply_noalloc: mesh needs more than its fixed scratch */

/* Every entry point returns one of these codes; no C++ exception crosses this
 * interface.  A jfem_set_mesh that fails after its argument checks leaves the
 * context without a mesh (later calls answer JFEM_ERR_INVALID until a mesh is
 * set); a failed jfem_set_traction / jfem_set_surface_load leaves it without a
 * surface load; a failed jfem_batch_add leaves the batch as it was. */

/* Size of the fixed device array jfem_apply_noalloc works in (every GPU that
 * loads the library holds it until the process exits). */
#define JFEM_NOALLOC_SCRATCH_BYTES (64u << 20)

/* element, face and material codes */
#define JFEM_TET4   4
#define JFEM_TET10 10
#define JFEM_HEX8   8
#define JFEM_TRI3   3
#define JFEM_TRI6   6
#define JFEM_QUAD4  4
#define JFEM_LINEAR_ELASTIC 0
#define JFEM_NEO_HOOKEAN    1

/* solve methods and precisions */
#define JFEM_PCG_JACOBI   0
#define JFEM_FCG_LEARNED  1
#define JFEM_NEWTON       2
#define JFEM_FCG_TWO_LEVEL 3  /* flexible CG, Jacobi + the coarse space of jfem_set_coarse_space */
#define JFEM_FP64         0   /* FP64 apply throughout */
#define JFEM_MIXED        1   /* FP32 apply, FP64 vectors/dots/residual + refinement */

/* jfem_apply flags */
#define JFEM_APPLY_FP32   1   /* FP32 element arithmetic (default FP64) */
#define JFEM_APPLY_MASKED 2   /* zero prescribed DOFs of input and output */

typedef struct jfem_ctx jfem_ctx;

/* Keyword arguments of solve!(physics; tol, max_iter, newton_tol, max_newton,
 * max_cg_per_newton) (src/backend/abstract.jl:181-188) and the Eisenstat–Walker
 * parameters of ext/JuliaFEMCUDAExt.jl:685-694.
 * Tolerances: by default tol is a relative FP64 residual ‖f − K u‖ / ‖f − K u₀‖
 * over the free DOFs (u₀ = prescribed values, free part zero) and Newton stops
 * when ‖R_free‖ ≤ newton_tol·‖f_int‖.  The reference tests absolute norms
 * instead — CG ‖r‖ < tol (src/backend/cpu.jl:230,244, ext/JuliaFEMCUDAExt.jl:567,620),
 * Newton ‖R‖ < newton_tol (ext/JuliaFEMCUDAExt.jl:754,779) — which tol_absolute = 1
 * selects, so solve!(tol = 1e-6) keeps its meaning through this ABI. */
typedef struct jfem_solve_opts {
  int method;             /* JFEM_PCG_JACOBI, JFEM_FCG_LEARNED, JFEM_NEWTON */
  int precision;          /* JFEM_FP64 or JFEM_MIXED */
  double tol;
  int max_iter;
  double newton_tol;
  int max_newton;
  int max_cg_per_newton;
  int n_load_steps;       /* Newton: prescribed values and loads ramped over steps */
  double forcing_power;
  double forcing_max;
  double time_budget_s;   /* 0 = none; else JFEM_ERR_TIMEOUT when exceeded (checked every 16
                             CG iterations); u then receives the best iterate found so far
                             (the last accepted Newton state for JFEM_NEWTON) and stats the
                             counts up to that point */
  double refine_drop;     /* JFEM_MIXED: FP64 residual each time ‖r‖ drops by this factor (0 → 0.3
                             for JFEM_PCG_JACOBI, 0.01 for the flexible-CG methods) */
  int tol_absolute;       /* 0: relative tests (default); 1: the reference's absolute ‖r‖ and ‖R‖ */
} jfem_solve_opts;

#define JFEM_HISTORY_MAX 256
/* Fields of ElasticitySolution (src/backend/abstract.jl:138-151). */
typedef struct jfem_stats {
  int status;
  int newton_iterations;
  int cg_iterations;
  int refinements;        /* FP64 true-residual evaluations */
  int fallbacks;          /* learned FCG → Jacobi-PCG switches */
  double residual;        /* final relative FP64 residual */
  double solve_time_s;
  int history_len;
  double history[3 * JFEM_HISTORY_MAX];   /* (cg_iters, ‖R‖, η) per Newton iteration */
} jfem_stats;

/* Fill opts with the reference defaults (tol 1e-6, max_iter 1000, newton_tol 1e-6,
 * max_newton 20, max_cg_per_newton 50, forcing 0.5 / 0.9). */
void jfem_default_opts(jfem_solve_opts* opts);
const char* jfem_version(void);

/* context lifetime (replaces CUDA.jl device/array management of
 * ext/JuliaFEMCUDAExt.jl:86-217) */
int jfem_create(jfem_ctx** out, int device_ordinal);
int jfem_destroy(jfem_ctx* ctx);
const char* jfem_last_error(const jfem_ctx* ctx);

/* Model definition — the host packing of initialize_gpu_data!
 * (ext/JuliaFEMCUDAExt.jl:86-217): coordinates, connectivity, materials,
 * Dirichlet masks and the surface-traction table.
 *   X     3 × n_nodes column-major (x,y,z of node 1, then node 2, …)
 *   conn  n_en × n_elem column-major, node numbers starting at index_base
 * The node→element adjacency and the sparsity pattern are built on the device. */
int jfem_set_mesh(jfem_ctx* ctx, int elem_type, int64_t n_nodes, const double* X,
                  int64_t n_elem, const int64_t* conn, int index_base);
/* E, nu: n_elem values when per_element, else 1 (problems_elasticity.jl:310-311). */
int jfem_set_material(jfem_ctx* ctx, int model, const double* E, const double* nu,
                      int per_element);
/* Elasticity properties finite_strain / geometric_stiffness (problems_elasticity.jl:36-46). */
int jfem_set_formulation(jfem_ctx* ctx, int finite_strain, int geometric_stiffness);
/* Prescribed DOFs (global DOF = 3(node-base)+comp+base) and their values
 * (src/problems_dirichlet.jl:60-89, src/solvers.jl:196-210).  values may be NULL (zero). */
int jfem_set_dirichlet(jfem_ctx* ctx, int64_t n, const int64_t* dofs, const double* values,
                       int index_base);
/* Surface traction: face_conn n_fn × n_faces column-major, t 3 × n_faces
 * (problems_elasticity.jl:454-502, consistent integration). */
int jfem_set_traction(jfem_ctx* ctx, int face_type, int64_t n_faces, const int64_t* face_conn,
                      const double* t, int index_base);
/* Surface loads: traction t (3 × n_faces, may be NULL) and pressure p (n_faces, may
 * be NULL; positive towards the surface, f += w·(−p)·n·N with n the normalised
 * ∂X/∂ξ₁ × ∂X/∂ξ₂ of the face, problems_elasticity.jl:486-493).  Replaces the
 * previous face table. */
int jfem_set_surface_load(jfem_ctx* ctx, int face_type, int64_t n_faces, const int64_t* face_conn,
                          const double* t, const double* p, int index_base);
/* Current displacement state u (3 n_nodes) for finite-strain assembly / tangent. */
int jfem_set_state(jfem_ctx* ctx, const double* u);

/* FP64 assembly of the global K (CSC, structural pattern of sparse.jl:121-132 +
 * sparse(): full 3×3 node blocks, explicit zeros kept) and of f = f_ext − f_int
 * (problems_elasticity.jl:433).  Call with colptr == NULL to get nnz in *nnz_inout;
 * then with arrays of n+1, nnz, nnz entries.  f (3 n_nodes) may be NULL. */
int jfem_assemble_csc(jfem_ctx* ctx, int index_base, int64_t* nnz_inout, int64_t* colptr,
                      int64_t* rowval, double* nzval, double* f);

/* Matrix-free y = K v (tangent at the current state for finite strain); the
 * pure operator (does not subtract f_ext, unlike ext/JuliaFEMCUDAExt.jl:442-478). */
int jfem_apply(jfem_ctx* ctx, const double* v, double* y, int flags);
/* Same with device pointers (3 n_nodes doubles each). */
int jfem_apply_device(jfem_ctx* ctx, const double* v_device, double* y_device, int flags);

/* Internal force f_int(u) at the current state (FP64), host or device output. */
int jfem_internal_force(jfem_ctx* ctx, double* f_int);

/* solve_backend! (ext/JuliaFEMCUDAExt.jl:886-916): load vector, Dirichlet values,
 * PCG / learned FCG / Newton–Krylov per opts.  u (3 n_nodes) receives the
 * displacement.  stats may be NULL. */
int jfem_solve(jfem_ctx* ctx, const jfem_solve_opts* opts, double* u, jfem_stats* stats);
/* Same with u left in device memory (u_device: 3 n_nodes doubles). */
int jfem_solve_device(jfem_ctx* ctx, const jfem_solve_opts* opts, double* u_device,
                      jfem_stats* stats);

/* Matrix-free FP64 y = K v for a linear-elastic mesh held entirely in device
 * memory, without allocating any device memory.  No counterpart in the
 * reference: it exists for callers that cannot call cudaMalloc — a host
 * application that owns the device memory through its own arena or pool (an
 * embedding simulation, a Julia CUDA memory pool), or a latency-critical loop
 * where an allocation could stall the device.  Inputs and outputs are the
 * caller's device buffers: X (3 × n_nodes), conn (n_en × n_elem column-major,
 * numbers from index_base), E and nu (one per element), v and y (3 n_nodes).
 * Working storage is one fixed array of JFEM_NOALLOC_SCRATCH_BYTES per device;
 * meshes that need more return JFEM_ERR_TOO_LARGE (roughly 200k Tet10,
 * 280k Hex8 or 500k Tet4 elements).  All calls share that array, so calls that
 * overlap on the GPU race and must be serialised by the caller.  The first call
 * on a device resolves the array's address for that device; make it before any
 * stream capture.  Runs on `stream` (a cudaStream_t, NULL = legacy default) and
 * returns after the stream has finished the work (it synchronises that
 * stream).  Status as elsewhere: JFEM_ERR_INVALID for node numbers outside
 * [index_base, index_base + n_nodes) or a material with E ≤ 0 or ν outside
 * (−1, 1/2) — such elements are skipped, never read out of bounds —,
 * JFEM_ERR_NEG_JACOBIAN, JFEM_ERR_CUDA when a launch or the stream fails. */
int jfem_apply_noalloc(int elem_type, int64_t n_nodes, const double* X_device, int64_t n_elem,
                       const int64_t* conn_device, int index_base, const double* E_device,
                       const double* nu_device, const double* v_device, double* y_device,
                       void* stream);

/* ------------------------------------------------------------------------
 * Learned preconditioner for flexible CG (method JFEM_FCG_LEARNED).  No
 * counterpart in the reference (its solvers are unpreconditioned CG,
 * src/backend/cpu.jl:221-254, ext/JuliaFEMCUDAExt.jl:531-577).
 *
 * Network N: linear message passing on the mesh node graph (nodes i ~ j when
 * they share an element), 3 layers of width JFEM_MPNN_WIDTH, no activation and
 * no biases, BF16 weights with FP32 accumulation:
 *   h0 = y (3 channels per node),   a_l,i = mean of h_l over the neighbours of i,
 *   h_{l+1} = Ws_l h_l + Wn_l a_l   (3 → 32 → 32 → 32),   N(y) = mask ⊙ Wo h3.
 * Preconditioner, symmetric positive definite for any weights (flexible CG
 * then keeps PCG's convergence):
 *   y = mask ⊙ D^{-1/2} r,   z = D^{-1/2} (y + Nᵀ N y),   D = diag K,
 * with Nᵀ the network's backward-data pass.  With all weights zero it is
 * Jacobi.  Training loss of a pair (r, e), r = K e, averaged over the pairs:
 *   ℓ = 1 − (zᵀ K e)² / ((zᵀ K z)(eᵀ K e)) = 1 − cos²_K(z, e)
 * (the share of e's energy left after one optimally scaled step along z; K z
 * from the FP32 apply).  The weights belong to the context and survive
 * jfem_set_mesh; training pairs do not.
 * Weight layout (row-major [out][in]): Ws1 32×3, Wn1 32×3, Ws2, Wn2, Ws3, Wn3
 * 32×32, Wo 3×32. */
#define JFEM_MPNN_WIDTH  32
#define JFEM_MPNN_PARAMS 4384
/* Seeded random weights: uniform in ±0.5·sqrt(6 / (fan_in + fan_out)) per layer. */
int jfem_mpnn_init(jfem_ctx* ctx, uint64_t seed);
/* JFEM_MPNN_PARAMS float values, rounded to BF16 on the way in. */
int jfem_mpnn_set_weights(jfem_ctx* ctx, const float* w);
int jfem_mpnn_get_weights(jfem_ctx* ctx, float* w);
/* Solve the current system (FP64 Jacobi-PCG to tol) and append up to max_pairs
 * (residual, error) pairs taken from its own iterates x_k (k = 0, 16, 32, 64, …):
 * e = x* − x_k, r = K e.  Returns the number of pairs held, or < 0. */
int jfem_mpnn_collect(jfem_ctx* ctx, int max_pairs, double tol);
int jfem_mpnn_clear(jfem_ctx* ctx);
/* Adam on the held pairs, mini-batches of `batch` pairs in a seeded shuffled
 * order, minimising the mean of ℓ above.  losses[epochs] (may be NULL)
 * receives the mean loss of each epoch. */
int jfem_mpnn_train(jfem_ctx* ctx, int epochs, int batch, double lr, uint64_t seed, double* losses);
/* Loss ℓ and its gradient (JFEM_MPNN_PARAMS) for one pair (r, e) given on the
 * host, through the training kernels — for gradient checks. */
int jfem_mpnn_loss_grad(jfem_ctx* ctx, const double* r, const double* e, double* loss, float* grad);
/* z = D^{-1/2}(y + NᵀN y), y = mask ⊙ D^{-1/2} r, for a host residual r
 * (3 n_nodes), through the inference kernels. */
int jfem_mpnn_precondition(jfem_ctx* ctx, const double* r, double* z);

/* ------------------------------------------------------------------------
 * Two-level preconditioner (methods JFEM_FCG_TWO_LEVEL and JFEM_FCG_LEARNED):
 *   z = S r + P A_c⁻¹ Pᵀ r,   A_c = Pᵀ K P,
 * S the smoother (D⁻¹, or the learned network above), P the rigid-body modes
 * (3 translations, 3 rotations about the centroid) of node aggregates — the
 * nodes binned into a structured grid of equal boxes over the bounding box —
 * zero on prescribed DOFs.  A_c is assembled on the device (double-float, from
 * the FP64 geometry records) from the elements that straddle aggregates or
 * hold prescribed DOFs, inverted (Gauss–Jordan, a pivot below 1e-12 of its
 * diagonal drops that mode) and applied in FP32.  No counterpart in the
 * reference, whose GPU solver design note recommends a multigrid-type coarse
 * correction with point smoothers
 * (docs/src/book/design/gpu_solver_strategy_expert_validated.md:114-156) but
 * ships unpreconditioned CG.  A_c is the coarse projection of the small-strain
 * stiffness; with finite strain it is the coarse level of the Newton tangent
 * solves (JFEM_NEWTON solves each tangent system by this flexible CG whenever
 * a coarse space is enabled, else by Jacobi-PCG).
 * coarse_dofs: 0 = no coarse space (JFEM_FCG_LEARNED is then one-level),
 * < 0 = automatic (about one coarse DOF per 1,000 DOFs, within [192, 2304];
 * the default), > 0 = about that many, at most JFEM_COARSE_MAX_DOFS (the
 * binning never exceeds it).  Kept across jfem_set_mesh. */
#define JFEM_COARSE_MAX_DOFS 4096
int jfem_set_coarse_space(jfem_ctx* ctx, int coarse_dofs);
/* Builds the coarse space for the current mesh, mask and material if needed
 * and reports its size: aggregates, coarse DOFs (6 per aggregate), elements
 * evaluated for A_c, and the device time of the last A_c set-up (assembly and
 * inversion, ms).  Each output may be NULL. */
int jfem_coarse_info(jfem_ctx* ctx, int* n_aggregates, int* n_coarse_dofs, int64_t* n_elements,
                     double* setup_ms);
/* A_c (n_coarse_dofs², row-major, rows 6a..6a+5 = aggregate a: x, y, z
 * translation, rotation about x, y, z) and the aggregate of each node
 * (n_nodes); either may be NULL.  For parity tests. */
int jfem_coarse_matrix(jfem_ctx* ctx, double* Ac, int* node_aggregate);
/* z = D⁻¹ r + P A_c⁻¹ Pᵀ r for a host residual r (3 n_nodes): the two-level
 * preconditioner with the Jacobi smoother, through the solver's kernels. */
int jfem_coarse_precondition(jfem_ctx* ctx, const double* r, double* z);

/* ------------------------------------------------------------------------
 * Batched solves: many small independent linear-elastic Tet4 problems solved
 * by Jacobi-PCG to an FP64 relative residual in one persistent, graph-captured
 * launch (one CTA per instance at a time, instances taken largest first).  No
 * counterpart in the reference, which runs one solve! per problem
 * (src/solvers.jl:273-344).  Instances: mesh (X 3 × n_nodes, conn 4 × n_elem,
 * numbers from index_base), E and nu, prescribed DOFs (value zero) and a
 * constant traction t (3 × n_faces) on Tri3 faces (face_conn 3 × n_faces),
 * integrated consistently (problems_elasticity.jl:454-502).  jfem_batch_add
 * returns the instance number (≥ 0) or an error. */
typedef struct jfem_batch jfem_batch;
int jfem_batch_create(jfem_batch** out, int device_ordinal);
int jfem_batch_destroy(jfem_batch* batch);
const char* jfem_batch_last_error(const jfem_batch* batch);
int jfem_batch_add(jfem_batch* batch, int64_t n_nodes, const double* X, int64_t n_elem, const int64_t* conn,
                   int index_base, double E, double nu, int64_t n_fixed, const int64_t* fixed_dofs,
                   int64_t n_faces, const int64_t* face_conn, const double* t);
/* Solve every instance to tol.  block_size 0 = autotune (block size, CTAs per
 * SM, and whether the largest instances run on thread-block clusters of 2, 4
 * or 8 CTAs, each cluster solving one instance; every candidate timed on the
 * whole batch, fastest kept), else 128/256/512/1024 with one CTA per instance.
 * Outputs (each may be NULL): u (3 × total nodes, instances in order),
 * per-instance iterations, status (0 / JFEM_NOT_CONVERGED), final relative
 * residual and latency (seconds from the instance's start to its end on the
 * GPU); solve_s = the launch's CUDA-event time. */
int jfem_batch_solve(jfem_batch* batch, double tol, int max_iter, int block_size, double* u, int* iterations,
                     int* status, double* residual, double* latency_s, double* solve_s);
/* Launch configuration of the last solve (the autotuner's choice when it ran):
 * the single-CTA launch, and the cluster launch of the largest instances
 * (cluster_size 1 and n_clustered 0 when there is none). */
int jfem_batch_config(const jfem_batch* batch, int* block_size, int* grid);
/* Where the autotuned configuration of the last block_size-0 solve came from:
 * 0 none yet, 1 timed by this batch object, 2 the autotuner cache.  The cache
 * is keyed by GPU name, element type and the batch shape (instance count,
 * largest and mean instance DOFs, each rounded up to a power of two); it lives
 * for the process and, when the environment variable JFEM_AUTOTUNE_CACHE names
 * a file, is read from and written to that file (JSON, one entry per line). */
int jfem_batch_tune_source(const jfem_batch* batch);
int jfem_batch_cluster_config(const jfem_batch* batch, int* cluster_size, int* n_clustered, int* cluster_block);
/* Fix the configuration jfem_batch_solve uses when its block_size is 0 (instead
 * of the autotuner): single-CTA block size, cluster size (1, 2, 4, 8), the
 * number of largest instances solved on clusters and their block size (256 or
 * 512).  block_size 0 returns to the autotuner. */
int jfem_batch_set_config(jfem_batch* batch, int block_size, int cluster_size, int n_clustered, int cluster_block);

/* Nodal strain or stress by a least-squares fit (postprocess!(problem, time,
 * Val{:strain} / Val{:stress}) with lsq_fit, src/problems_elasticity.jl:521-594):
 * the integration-point field of the displacement u (3 n_nodes, host) —
 * small strain ε = sym ∇u or σ = λ tr(ε) I + 2μ ε, order 11, 22, 33, 12, 23, 13,
 * tensor shear — projected onto the nodal shape functions.  The mass-matrix
 * system is solved in FP64 by Jacobi-PCG on its six columns to the relative
 * residual tol (the reference factorises it).  nodal: 6 × n_nodes (host). */
#define JFEM_FIELD_STRAIN 0
#define JFEM_FIELD_STRESS 1
int jfem_recover_field(jfem_ctx* ctx, const double* u, int field, double tol, int max_iter, double* nodal,
                       int* iterations);

/* Reverse Cuthill–McKee renumbering of the mesh's node graph (nodes sharing an
 * element), as symrcm in src/graph/graph_ordering.jl:21-98: search from node
 * `start`, neighbours in increasing-degree order, reversed.  perm[k] (n_nodes,
 * numbers from index_base) is the old node placed at new position k.  The
 * bandwidths 2·max|v−w|+1 before and after (graph_ordering.jl:21-29) may be
 * NULL.  Host code; needs no device. */
int jfem_rcm(int64_t n_nodes, int64_t n_elem, int nodes_per_elem, const int64_t* conn, int index_base,
             int64_t start, int64_t* perm, int64_t* bandwidth_before, int64_t* bandwidth_after);

/* Kernels launched by the library on this context since its creation. */
int64_t jfem_kernel_launches(const jfem_ctx* ctx);
/* Event-timed duration (ms) of the last matrix-free apply launch sequence. */
double jfem_last_apply_ms(const jfem_ctx* ctx);
/* The context's CUDA stream (cudaStream_t), for event timing and interop. */
void* jfem_stream(const jfem_ctx* ctx);
/* Runs the apply (flags as jfem_apply) reps times on device-resident vectors
 * and returns the mean CUDA-event duration of the element kernel and of the node
 * gather kernel (ms), each measured on the context stream.  No counterpart in the
 * reference (measurement hook). */
int jfem_time_apply(jfem_ctx* ctx, int flags, int reps, double* ms_element, double* ms_gather);
/* Runs the FP64 assembly of K's values and f_int (the integration-point kernel
 * and the CSC scatter of jfem_assemble_csc, without the pattern and without
 * the download) reps times into device scratch and returns the mean CUDA-event
 * duration of each kernel (ms) and the number of stored entries.  No
 * counterpart in the reference (measurement hook). */
int jfem_time_assembly(jfem_ctx* ctx, int reps, double* ms_qpoint, double* ms_scatter, int64_t* nnz);

#ifdef __cplusplus
}
#endif
#endif /* JFEM_H */
