// jfem_common.cuh — shared declarations of libjfem_cuda.so (sm_103a).
//
// Device data layout (one context = one mesh on one GPU):
//   X64   [N][3]  f64    node coordinates (FP64 parity path)
//   X32   [N]     float4 node coordinates (FP32 apply; .w unused)
//   conn  [n_en][E] i32  structure-of-arrays connectivity (coalesced per local node)
//   adj_ptr[N+1], adj[E*n_en]  node → (element<<4 | local) lists, ascending element
//   nb_ptr[N+1],  nbr[nb]      node → sorted neighbour nodes (3×3 block pattern)
//   slot[E*n_en*n_en] u16      for adjacency entry t of node J and local node b of
//                              that element: position of conn[b] in nbr(J)
//   lam/mu [E] f64 + f32       per-element Lamé constants
//   mask  [N] u8               bit c set: DOF 3n+c prescribed
//   ye32/ye64 [n_en*3][E]      per-element apply results (SoA), gathered per node
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <exception>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/jfem.h"

#define JFEM_MAX_NEIGHBOURS 512   // unique neighbour nodes per node (pattern build)
#define JFEM_RED_BLOCKS 1216      // fixed reduction grid: 152 SMs x 8 → deterministic sums
#define JFEM_RED_THREADS 256
// Reduction partials (doubles) of the solvers: [0, 4G) the PCG/FCG dot products;
// then the flexible-CG β terms: Σ D⁻¹r·q_old per reduction block, Σ
// D^{-1/2}(y + v)·q_old per block of the network's last neighbour pass (its grid
// is capped at JFEM_RED_BLOCKS), and Ec·Pᵀq_old per coarse-solve block
// (≤ 4,096 rows / 8 per block).
#define JFEM_PART_T1 (4 * JFEM_RED_BLOCKS)
#define JFEM_PART_T1N (5 * JFEM_RED_BLOCKS)
#define JFEM_PART_T2 (6 * JFEM_RED_BLOCKS)
#define JFEM_PART_SIZE (JFEM_PART_T2 + 512)
#define JFEM_TILE 256             // elements per tile of the shared-memory apply
#define JFEM_TILE_CTAS 3          // resident CTAs per SM the small-strain tile kernel is compiled for

namespace jfem {

// ---------------------------------------------------------------------------
// Element traits.  Shape-function derivatives at the integration points are
// constexpr so that, in fully unrolled loops, the compiler folds the table into
// immediates (zero entries vanish).  Rules: Tet4 GLTET1, Tet10 GLTET4, Hex8
// GLHEX8 (src/elements/integrate.jl:19,27-28; src/quadrature/gltet.jl:7-25,
// src/quadrature/glquad.jl:6-40); derivatives from
// src/basis/lagrange_generated.jl:229-311.
// ---------------------------------------------------------------------------
template <int ET> struct Elem;
template <> struct Elem<JFEM_TET4> { static constexpr int NN = 4, NQ = 1; };
template <> struct Elem<JFEM_TET10> { static constexpr int NN = 10, NQ = 4; };
template <> struct Elem<JFEM_HEX8> { static constexpr int NN = 8, NQ = 8; };

// (5 ± 3√5)/20 and (5 − √5)/20, the GLTET4 abscissae; 1/√3 for Gauss–Legendre 2.
#define JFEM_TET4A 0.58541019662496845446
#define JFEM_TET4B 0.13819660112501051518
#define JFEM_GL2 0.5773502691896258

__host__ __device__ constexpr double qp_coord(int et, int q, int d) {
  if (et == JFEM_TET4) return 0.25;
  if (et == JFEM_TET10) return (q == d) ? JFEM_TET4A : JFEM_TET4B;   // (a,b,b),(b,a,b),(b,b,a),(b,b,b)
  // Hex8: q = i + 2j + 4k, first coordinate fastest
  return ((q >> d) & 1) ? JFEM_GL2 : -JFEM_GL2;
}

__host__ __device__ constexpr double qp_weight(int et, int q) {
  return et == JFEM_TET4 ? 1.0 / 6.0 : et == JFEM_TET10 ? 1.0 / 24.0 : 1.0;
}

__host__ __device__ constexpr double hex_sign(int i, int d) {
  // node order (-1,-1,-1),(1,-1,-1),(1,1,-1),(-1,1,-1),(-1,-1,1),(1,-1,1),(1,1,1),(-1,1,1)
  return d == 0 ? ((i == 1 || i == 2 || i == 5 || i == 6) ? 1.0 : -1.0)
       : d == 1 ? ((i == 2 || i == 3 || i == 6 || i == 7) ? 1.0 : -1.0)
                : (i >= 4 ? 1.0 : -1.0);
}

// ∂N_i/∂ξ_d at integration point q.
__host__ __device__ constexpr double dshape(int et, int q, int i, int d) {
  if (et == JFEM_TET4) {
    return i == 0 ? -1.0 : (i - 1 == d ? 1.0 : 0.0);
  }
  if (et == JFEM_TET10) {
    const double u = qp_coord(et, q, 0), v = qp_coord(et, q, 1), w = qp_coord(et, q, 2);
    switch (i) {
      case 0: return -3.0 + 4.0 * u + 4.0 * v + 4.0 * w;
      case 1: return d == 0 ? -1.0 + 4.0 * u : 0.0;
      case 2: return d == 1 ? -1.0 + 4.0 * v : 0.0;
      case 3: return d == 2 ? -1.0 + 4.0 * w : 0.0;
      case 4: return d == 0 ? 4.0 - 8.0 * u - 4.0 * v - 4.0 * w : -4.0 * u;
      case 5: return d == 0 ? 4.0 * v : d == 1 ? 4.0 * u : 0.0;
      case 6: return d == 1 ? 4.0 - 8.0 * v - 4.0 * u - 4.0 * w : -4.0 * v;
      case 7: return d == 2 ? 4.0 - 8.0 * w - 4.0 * u - 4.0 * v : -4.0 * w;
      case 8: return d == 0 ? 4.0 * w : d == 1 ? 0.0 : 4.0 * u;
      default: return d == 0 ? 0.0 : d == 1 ? 4.0 * w : 4.0 * v;
    }
  }
  // Hex8 trilinear
  const double x0 = qp_coord(et, q, 0), x1 = qp_coord(et, q, 1), x2 = qp_coord(et, q, 2);
  const double f0 = 1.0 + hex_sign(i, 0) * x0, f1 = 1.0 + hex_sign(i, 1) * x1,
               f2 = 1.0 + hex_sign(i, 2) * x2;
  return d == 0 ? 0.125 * hex_sign(i, 0) * f1 * f2
       : d == 1 ? 0.125 * f0 * hex_sign(i, 1) * f2
                : 0.125 * f0 * f1 * hex_sign(i, 2);
}

// Surface rules: Tri3 GLTRI1, Tri6 GLTRI3, Quad4 GLQUAD4 (integrate.jl:15,23-24).
__host__ __device__ inline int face_nodes(int ft) { return ft == JFEM_TRI3 ? 3 : ft == JFEM_TRI6 ? 6 : 4; }
__host__ __device__ inline int face_nq(int ft) { return ft == JFEM_TRI3 ? 1 : ft == JFEM_TRI6 ? 3 : 4; }

// ---------------------------------------------------------------------------
// small dense helpers (Real = float or double)
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ R det3(const R J[3][3]) {
  return J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
         J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
         J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
}

// adjugate: adj = det · J⁻¹
template <typename R>
__device__ __forceinline__ void adj3(const R J[3][3], R A[3][3]) {
  A[0][0] = J[1][1] * J[2][2] - J[1][2] * J[2][1];
  A[0][1] = J[0][2] * J[2][1] - J[0][1] * J[2][2];
  A[0][2] = J[0][1] * J[1][2] - J[0][2] * J[1][1];
  A[1][0] = J[1][2] * J[2][0] - J[1][0] * J[2][2];
  A[1][1] = J[0][0] * J[2][2] - J[0][2] * J[2][0];
  A[1][2] = J[0][2] * J[1][0] - J[0][0] * J[1][2];
  A[2][0] = J[1][0] * J[2][1] - J[1][1] * J[2][0];
  A[2][1] = J[0][1] * J[2][0] - J[0][0] * J[2][1];
  A[2][2] = J[0][0] * J[1][1] - J[0][1] * J[1][0];
}

// Block-wide deterministic sum (fixed tree order).  blockDim.x ≤ 1024, multiple of 32.
template <typename T>
__device__ __forceinline__ T block_sum(T v, T* sh /* ≥ 32 entries */) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  const int nw = blockDim.x >> 5;
  T r = (threadIdx.x < nw) ? sh[threadIdx.x] : T(0);
  if (w == 0)
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
  __syncthreads();
  if (threadIdx.x == 0) sh[0] = r;
  __syncthreads();
  r = sh[0];
  __syncthreads();
  return r;
}

// Sum of n partials in a fixed order (every thread returns the same value).
__device__ __forceinline__ double reduce_partials(const double* __restrict__ part, int n, double* sh) {
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += part[i];
  return block_sum(s, sh);
}

// Device error flag: first error wins.
__device__ __forceinline__ void raise_error(int* flag, int code) { atomicCAS(flag, 0, code); }

// ---------------------------------------------------------------------------
// bulk asynchronous copies global → shared (cp.async.bulk, completion counted
// in bytes on a shared-memory mbarrier).  Addresses 16-byte aligned, sizes a
// multiple of 16 bytes.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
// Orders this thread's earlier generic-proxy shared-memory accesses before
// later async-proxy (bulk copy) writes to the same memory.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned done;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
// Wait for the phase of the given parity with a bounded number of polls;
// false (and JFEM_ERR_TIMEOUT raised) when the budget runs out.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity, int* err) {
  for (unsigned k = 0; k < (1u << 20); ++k)
    if (mbar_try_wait(bar, parity)) return true;
  raise_error(err, JFEM_ERR_TIMEOUT);
  return false;
}

// Prolongation of the two-level preconditioner at DOF (i, c): (P Ec)_ic =
// t_a + (ω_a × d_i)_c with (t_a, ω_a) = Ec[6a .. 6a+5], a the aggregate of node
// i and d_i = X_i − c_a (jfem_coarse.cu).  The caller applies the Dirichlet mask.
__device__ __forceinline__ float coarse_prolong_v(const float* e, float4 d, int c) {
  return c == 0 ? e[0] + e[4] * d.z - e[5] * d.y : c == 1 ? e[1] + e[5] * d.x - e[3] * d.z : e[2] + e[3] * d.y - e[4] * d.x;
}
__device__ __forceinline__ float coarse_prolong(const int* __restrict__ node_agg, const float4* __restrict__ d32,
                                                const float* __restrict__ Ec, int64_t i, int c) {
  return coarse_prolong_v(Ec + 6 * node_agg[i], d32[i], c);
}

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
struct SolverScalars {
  double rz[2];      // r·z by iteration parity
  double rr[2];      // r·r by iteration parity
  double bb;         // ‖b_free‖²
  double tol2;       // tol² · bb — stop threshold on r·r
  int done[2];       // stop flag by iteration parity
  int iters;
  int max_iters;
  // mixed (double-float) solver: one slot, scalars formed by the last block
  // of the launch that completes the reduction
  double alpha, beta;
  float2 alpha_df, beta_df;
  unsigned arrive[4];   // last-block counters (return to 0 after every use)
  // flexible CG with the learned preconditioner
  double pAp;           // p·Ap of the last apply (denominator of the next β)
  int restart;          // next direction is z itself (β = 0)
};

// Learned preconditioner weights (jfem_mpnn.cu): owned by the context, kept
// across meshes.  Flat layout of JFEM_MPNN_PARAMS values, row-major [out][in].
#define MP_W 32
#define MP_W1S 0
#define MP_W1N (MP_W1S + MP_W * 3)
#define MP_W2S (MP_W1N + MP_W * 3)
#define MP_W2N (MP_W2S + MP_W * MP_W)
#define MP_W3S (MP_W2N + MP_W * MP_W)
#define MP_W3N (MP_W3S + MP_W * MP_W)
#define MP_WO (MP_W3N + MP_W * MP_W)
#define MP_P (MP_WO + 3 * MP_W)
static_assert(MP_P == JFEM_MPNN_PARAMS, "parameter layout");
// Per-sample activation buffers of the network ([B][N][C] each).  Two forward
// passes are kept while training (pass 0 on y, pass 1 on the loss gradient ĝ).
struct MpBufs {
  float *a1[2] = {nullptr, nullptr}, *h1[2] = {nullptr, nullptr}, *a2[2] = {nullptr, nullptr},
        *h2[2] = {nullptr, nullptr}, *a3[2] = {nullptr, nullptr}, *h3[2] = {nullptr, nullptr};
  float *dA = nullptr, *dB = nullptr, *gn = nullptr;          // 32 channels
  float *y = nullptr, *u = nullptr, *v = nullptr, *ghat = nullptr, *w = nullptr, *t3a = nullptr,
        *t3b = nullptr, *kz = nullptr;                          // 3 channels
};

struct MpnnState {
  float* w32 = nullptr;          // FP32 master weights (Adam state lives beside them)
  __nv_bfloat16* wbf = nullptr;  // BF16 weights used by every forward pass
  float* m = nullptr;
  float* v = nullptr;
  float* g = nullptr;            // last gradient
  int64_t step = 0;
  bool ready = false;
  // Inference form of the (linear) network: N = Σ_{k=0..3} C_k ⊗ A^k with A the
  // neighbour mean and C_k the 3×3 sums of the layer products (Wo·X3·X2·X1,
  // X_l ∈ {Ws_l, Wn_l}, k of them Wn).  Formed in FP64 from the BF16 weights
  // whenever they change; FP32 on the device.
  float* poly = nullptr;         // C_0..C_3 row-major, 36 values
  bool poly_fresh = false;
};

struct Ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  int64_t launches = 0;
  double last_apply_ms = 0.0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;

  // mesh
  int et = 0, nn = 0;
  int64_t N = 0, E = 0;
  double* X64 = nullptr;
  float4* X32 = nullptr;
  int* conn = nullptr;
  int* adj_ptr = nullptr;
  unsigned* adj = nullptr;
  int* nb_ptr = nullptr;
  int* nbr = nullptr;
  uint16_t* slot = nullptr;
  int64_t n_blocks = 0;   // 3×3 blocks in the pattern
  int dmax = 0;           // max neighbours of a node
  int amax = 0;           // max elements of a node

  // material / formulation
  int model = JFEM_LINEAR_ELASTIC;
  int finite = 0, geom = 0;
  double* lam64 = nullptr;
  double* mu64 = nullptr;
  float* lam32 = nullptr;
  float* mu32 = nullptr;
  bool have_material = false;

  // Dirichlet
  uint8_t* mask = nullptr;
  double* gvals = nullptr;   // prescribed values (3N, zero on free DOFs)
  int64_t n_fixed = 0;
  int64_t n_fixed_nonzero = 0;

  // traction
  int ft = 0, nfn = 0;
  int64_t F = 0;
  int* fconn = nullptr;
  double* ftrac = nullptr;    // [F][4]: traction (3) and pressure
  int* fadj_ptr = nullptr;
  unsigned* fadj = nullptr;
  double* f_ext = nullptr;
  bool f_ext_dirty = true;

  // state (finite strain)
  double* u_state = nullptr;
  bool have_state = false;

  // operator geometry (FP64-prepared; see jfem_apply.cu)
  bool geo_ready = false;
  bool geo_affine = true;
  double* geo64 = nullptr;
  float* geo32 = nullptr;

  // element tiles of the shared-memory FP32 apply (jfem_tiles.cu)
  int64_t ntiles = 0, Epad = 0, n_bnodes = 0, n_bslots = 0;
  int tile_Lmax = 0;
  int* tperm = nullptr;         // [Epad] tile position → element (−1 padding)
  uint16_t* tconn = nullptr;    // [n_en][Epad] tile-local node of each element node
  int* tnode_ptr = nullptr;     // [ntiles+1]
  int* tnodes = nullptr;        // [Σ L] each tile's nodes in ascending global order (the staging order)
  uint16_t* tloc = nullptr;     // [Σ L] local index (gather order: element slots descending) of each
  uint16_t* tadj_ptr = nullptr; // per tile: L+1 offsets into the tile's adjacency block
  uint16_t* tadj = nullptr;     // [ntiles][T·n_en] local node · T + local element (an element-vector slot)
  int* tout = nullptr;          // per tile node: its global node when interior, −1 − (bpart position) when shared
  int* bnodes = nullptr;        // nodes shared by several tiles
  int* bptr = nullptr;          // [n_bnodes+1] runs of bpart per shared node
  float4* bpart = nullptr;      // [n_bslots] tile partial sums (x, y, z, unused), grouped by node, ascending tile
  float* geoT32 = nullptr;      // geometry records in tile order
  float* nhstate = nullptr;     // [16·n_q][Epad] Neo-Hookean point state at u_state (F, C⁻¹ sym, μ − λ ln J), tile order
  uint64_t state_version = 1;   // bumped whenever u_state, the material, the formulation or the geometry change
  uint64_t diag_state_version = 0, diag_mask_gen = 0;   // what c->dinv was computed for (0: never)
  uint64_t nhstate_version = 0; // state_version nhstate was computed at

  // scratch
  float* ye32 = nullptr;
  double* ye64 = nullptr;
  double* qd = nullptr;       // FP64 per-integration-point data for assembly
  size_t qd_bytes = 0;
  int* d_err = nullptr;

  // solver
  double *x = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *Ap = nullptr,
         *dinv = nullptr, *b = nullptr, *tmp = nullptr, *tmp2 = nullptr, *xbest = nullptr;
  float2* p2 = nullptr;       // p as double-float (hi, lo): the mixed solver's direction, the FP32 apply input
  float2 *xd = nullptr, *rd = nullptr;   // mixed solver: x and r as double-float
  float* Apf = nullptr;       // FP32 apply output
  float* dinvf = nullptr;     // Jacobi inverse diagonal (FP32: an exact SPD preconditioner in its own right)
  double* part = nullptr;     // reduction partials (4 × JFEM_RED_BLOCKS)
  SolverScalars* sc = nullptr;
  SolverScalars* sc_host = nullptr;   // pinned mirror
  double* norms = nullptr;            // 2 doubles
  double* norms_host = nullptr;       // pinned mirror
  cudaGraphExec_t pcg_graph = nullptr;
  int pcg_graph_key = -1;
  int64_t chunk_launches = 0;

  // learned preconditioner: weights (kept across meshes) and, per mesh, the
  // training pairs [pairs][N][3] (x, t, d), activations for B samples, FCG z
  MpnnState* mp = nullptr;
  float *mp_x = nullptr, *mp_t = nullptr, *mp_d = nullptr, *mp_den = nullptr;
  float* mp_c = nullptr;      // [pairs][N][3] coarse term Q r̃ of each pair (pairs collected two-level)
  int mp_coarse = -1;         // pairs collected with (1) or without (0) the coarse space; −1 none held
  int64_t mp_pairs = 0, mp_cap = 0;
  MpBufs mb;                  // activations and scratch for m_actB samples (one arena)
  float* marena = nullptr;
  float* mgpart = nullptr;    // weight-gradient block partials
  double* mdots = nullptr;    // loss dot-product partials of a training batch
  float* mcoef = nullptr;     // per-pair loss-gradient coefficients
  int64_t m_actB = 0, m_gpart_cap = 0;
  float4* mi = nullptr;       // network inference vectors, 7 × [N] float4: y, A y, A² y, u, h, g, v
  float* invdeg = nullptr;    // 1 / (neighbours of each node), the mean-aggregation weights

  // two-level preconditioner: Galerkin coarse space of rigid-body modes on node
  // aggregates (jfem_coarse.cu).  Structure per (mesh, Dirichlet mask); values
  // per geometry generation (material and coordinates).
  int coarse_target = -1;       // requested coarse DOFs: 0 off, < 0 automatic (kept across meshes)
  uint64_t geo_gen = 1;         // bumped by every geometry invalidation
  uint64_t mask_gen = 1;        // bumped by every jfem_set_dirichlet
  uint64_t coarse_geo_gen = 0, coarse_mask_gen = 0;   // generations the coarse data was built for
  int coarse_built_target = 0;
  int nagg = 0, nc = 0, nc_pad = 0;   // aggregates, coarse DOFs (6 per aggregate), padded to 32
  int nb_bins[3] = {0, 0, 0};
  int* agg_ptr = nullptr;       // [nagg+1] nodes of each aggregate (CSR, ascending node)
  int* agg_nodes = nullptr;     // [N]
  int* node_agg = nullptr;      // [N] aggregate of each node
  float4* node_d32 = nullptr;   // [N] X_i − centroid of its aggregate (FP32; w unused)
  float2* node_ddf = nullptr;   // [N][3] the same in double-float (coarse matrix)
  int64_t n_celem = 0;          // elements whose A_c contribution is not zero
  int* celem = nullptr;         // [n_celem] element ids, ascending
  int* celem_aggs = nullptr;    // [n_celem][10] distinct aggregates of the element, ascending, −1 padded
  int64_t* celem_off = nullptr; // [n_celem] first contribution block of the element (A_e² blocks)
  int64_t n_contrib = 0;
  float2* contrib = nullptr;    // [n_contrib][36] 6×6 element blocks of A_c (double-float)
  int64_t n_cblk = 0;           // nonzero 6×6 blocks of A_c
  int* cblk_ab = nullptr;       // [n_cblk][2] (row aggregate, column aggregate)
  int* cblk_ptr = nullptr;      // [n_cblk+1] into cblk_src
  int64_t* cblk_src = nullptr;  // contribution blocks of each A_c block, ascending element
  float2* Ac = nullptr;         // [nc_pad][nc_pad] A_c, inverted in place (double-float)
  double* Ac_diag = nullptr;    // [nc_pad] diagonal of A_c before the inversion
  float2* gj_buf = nullptr;     // Gauss–Jordan panels: P (32×32), row panel, old column panel
  float* Ainv32 = nullptr;      // [nc_pad][nc_pad] A_c⁻¹ rounded to FP32 (the per-iteration coarse solve)
  int n_chunks = 0;             // restriction chunks (≤ 1,024 nodes of one aggregate each)
  int* chunk_begin = nullptr;   // [n_chunks+1] into agg_nodes
  int* agg_chunk_ptr = nullptr; // [nagg+1] the chunks of each aggregate (contiguous)
  float* cpart = nullptr;       // [n_chunks][12] chunk partials of Pᵀ r and Pᵀ q_old
  int* chunk_agg = nullptr;     // [n_chunks] aggregate of each restriction chunk
  unsigned* agg_cnt = nullptr;  // [nagg] chunks of the aggregate finished in this restriction (back to 0)
  float* RQ = nullptr;          // [2][nc_pad] Pᵀr, Pᵀq_old (zero beyond nc)
  float* Ec = nullptr;          // [nc_pad] coarse correction A_c⁻¹ Pᵀ r
  double coarse_setup_ms = 0.0; // last coarse value setup (CUDA events)

  std::vector<void*> owned;   // everything cudaMalloc'ed for this mesh
};

// error helpers (host)
int set_err(Ctx* c, int code, const std::string& msg);
int cuda_check(Ctx* c, cudaError_t e, const char* what);
int sync_and_check(Ctx* c, const char* what);
template <typename T>
int dalloc(Ctx* c, T** p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  c->owned.reserve(c->owned.size() + 1);   // may throw, before anything is allocated
  cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
  if (e != cudaSuccess) {
    *p = nullptr;
    return set_err(c, JFEM_ERR_OOM, std::string("cudaMalloc failed: ") + cudaGetErrorString(e));
  }
  c->owned.push_back((void*)*p);
  return 0;
}
void dfree(Ctx* c, void* p);
void free_mesh(Ctx* c);

// Runs task(k) for k in [0, ntasks), each on its own host thread.  An exception
// in a task is carried to the calling thread (the first one, after every thread
// has been joined), and a thread that cannot be started runs its task on the
// calling thread instead.
template <class F>
void host_tasks(int64_t ntasks, F task) {
  std::exception_ptr first;
  std::mutex mu;
  auto run = [&](int64_t k) {
    try {
      task(k);
    } catch (...) {
      std::lock_guard<std::mutex> lk(mu);
      if (!first) first = std::current_exception();
    }
  };
  std::vector<std::thread> th;
  th.reserve((size_t)ntasks);
  for (int64_t k = 0; k < ntasks; ++k) {
    bool started = false;
    try {
      th.emplace_back(run, k);
      started = true;
    } catch (...) {
    }
    if (!started) run(k);
  }
  for (auto& x : th) x.join();
  if (first) std::rethrow_exception(first);
}

// Runs body(i0, i1) over contiguous ranges of [0, n) on up to 16 host threads
// (at least 16 items each); callers make every range's work independent, so
// results do not depend on the split.
template <class F>
void host_parallel(int64_t n, F body) {
  const int64_t hw = std::max<int64_t>(1, std::min<int64_t>(16, (int64_t)std::thread::hardware_concurrency()));
  const int64_t nt = std::min<int64_t>(hw, std::max<int64_t>(1, n / 16));
  if (nt <= 1) {
    body((int64_t)0, n);
    return;
  }
  host_tasks(nt, [&](int64_t k) { body(n * k / nt, n * (k + 1) / nt); });
}

inline int grid_for(int64_t n, int threads, int64_t cap = 152LL * 64) {
  int64_t g = (n + threads - 1) / threads;
  if (g < 1) g = 1;
  if (g > cap) g = cap;
  return (int)g;
}

// ---------------------------------------------------------------------------
// host-side launchers (one TU each)
// ---------------------------------------------------------------------------
// jfem_mesh.cu
int mesh_setup(Ctx* c, int et, int64_t N, const double* X, int64_t E, const int64_t* conn, int base);
int faces_setup(Ctx* c, int ft, int64_t F, const int64_t* fconn, const double* t, const double* p, int base);
// jfem_tiles.cu
int tiles_build(Ctx* c, const double* X, const int64_t* conn, int base);
int exclusive_scan_i32(Ctx* c, const int* in, int* out, int64_t n, int64_t* total);
// jfem_assemble.cu
int assemble_csc_device(Ctx* c, int base, int64_t* colptr_d, int64_t* rowval_d, double* nzval_d,
                        double* f_d);
int traction_device(Ctx* c, double* f_d);
int jacobi_diag_device(Ctx* c, double* dinv_d);
// jfem_apply.cu
int geometry_prepare(Ctx* c);
int geometry_invalidate(Ctx* c);
void enqueue_apply(Ctx* c, const double* v, double* y, bool fp32, bool masked, bool mask_in, double* part,
                   const int* stop, const float2* v2);
void enqueue_split(Ctx* c, const double* v, float2* v2);
bool apply_is_tiled(const Ctx* c);
// Neo-Hookean tangent applies read the point state cached for the current u
// (nh_state_prepare; off the captured graphs) instead of recomputing it.
inline bool nh_cache_ready(const Ctx* c) { return c->nhstate && c->nhstate_version == c->state_version; }
int nh_state_prepare(Ctx* c);
void enqueue_apply_tiled(Ctx* c, const float2* v2, float* y, bool masked, double* part, const int* stop,
                         SolverScalars* sc = nullptr);
void enqueue_internal_force(Ctx* c, double* f);
int apply_device(Ctx* c, const double* v, double* y, bool fp32, bool masked, double* partial_pAp);
void prepare_geo_tet4_affine(int64_t E, const int* conn, const double* X, const double* lam, const double* mu,
                             double* g64, float* g32, cudaStream_t stream);
int internal_force_device(Ctx* c, double* f_d);
int time_apply(Ctx* c, bool fp32, bool masked, int reps, double* ms_elem, double* ms_gather);
int time_assembly(Ctx* c, int reps, double* ms_qpoint, double* ms_scatter);
// jfem_mpnn.cu
int mpnn_ensure(Ctx* c);
int mpnn_init(Ctx* c, uint64_t seed);
int mpnn_set_weights(Ctx* c, const float* w);
int mpnn_get_weights(Ctx* c, float* w);
int mpnn_collect(Ctx* c, int max_pairs, double tol);
int mpnn_train(Ctx* c, int epochs, int batch, double lr, uint64_t seed, double* losses);
int mpnn_loss_grad(Ctx* c, const double* r, const double* e, double* loss, float* grad);
int mpnn_precondition(Ctx* c, const double* r, double* z);
int mpnn_ensure_act(Ctx* c, int64_t B);
int mpnn_refresh_poly(Ctx* c);
int mpnn_ensure_infer(Ctx* c);                             // the float4 inference vectors
// v = NᵀN y for one sample (y, v: [N] float4).  With t1part, the last pass also
// leaves block partials of Σ D^{-1/2}(y + v)·q_old (flexible CG's β) and
// returns the number of blocks.
int enqueue_mpnn_spd(Ctx* c, const float4* y, float4* v, const float* dinvf = nullptr, const float* qold = nullptr,
                     double* t1part = nullptr, SolverScalars* sc = nullptr, const double* t2 = nullptr, int n2 = 0);
// jfem_coarse.cu
int coarse_prepare(Ctx* c);   // structure and values for the current mesh, mask and geometry
int coarse_info(Ctx* c, int* n_agg, int* n_coarse, int64_t* n_elem_listed, double* setup_ms);
int coarse_matrix(Ctx* c, double* Ac_h, int* node_agg_h);
int coarse_precondition(Ctx* c, const double* r_h, double* z_h);
// Ec = A_c⁻¹ Pᵀ r; with qold, also the block partials of Ec·Pᵀ q_old into t2part
void enqueue_coarse_restrict_solve(Ctx* c, const float2* r, const int* stop, const float* qold = nullptr,
                                   double* t2part = nullptr, SolverScalars* sc = nullptr, const double* t1 = nullptr,
                                   int n1 = 0);
int coarse_gemv_blocks(const Ctx* c);
// jfem_recovery.cu
int recover_field(Ctx* c, const double* u_h, int field, double tol, int max_iter, double* nodal_h, int* iters_out);
// jfem_solver.cu
int pcg_fp64_snapshots(Ctx* c, const double* f, double tol, int max_iter, double* snaps, int max_snaps,
                       int* n_snaps, int* snap_iters, int* iters_out, double* relres_out);
void enqueue_axpy(Ctx* c, int64_t n, double a, const double* x, double* y);
int solve_device(Ctx* c, const jfem_solve_opts* o, double* u_d, jfem_stats* st);

}  // namespace jfem

#include "jfem_df.cuh"

namespace jfem {

// Flexible CG's β = (Σ t1 + Σ t2) / p·q_old (0 on restart), each partial list
// summed in index order (FP64) as k_fcg_beta sums them — run by the last block
// of the launch that writes the final partials (after arrive_last), so β needs
// no launch of its own.  sh: ≥ 32 doubles of shared memory.
__device__ __forceinline__ void fcg_beta_last_block(SolverScalars* sc, const double* t1, int n1, const double* t2,
                                                    int n2, double* sh) {
  const double a = reduce_partials_cg(t1, n1, sh);
  const double b = t2 ? reduce_partials_cg(t2, n2, sh) : 0.0;
  if (threadIdx.x == 0) {
    const double beta = sc->restart ? 0.0 : (a + b) / sc->pAp;
    sc->beta = beta;
    sc->beta_df = df_from_double(beta);
    sc->restart = 0;
  }
}

}  // namespace jfem

struct jfem_ctx {
  jfem::Ctx c;
};
