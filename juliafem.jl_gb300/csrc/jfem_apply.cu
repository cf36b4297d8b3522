// jfem_apply.cu — matrix-free K·v / tangent apply and internal force.
//
// Reference: the two-phase Tet4 operator of ext/JuliaFEMCUDAExt.jl:222-361,442-478
// (stress per Gauss point, then an atomic-free node gather) and the nodal matvec
// of src/nodal_assembly_structures.jl:197-212.  Here the stress never leaves
// registers: phase 1 is one thread per element computing y_e = K_e v_e for every
// integration point and writing the element vector (SoA, coalesced); phase 2 is
// one thread per node summing the element vectors of that node in ascending
// element order (deterministic, no atomics) and optionally a p·Ap partial sum.
//
// Geometry is prepared once per mesh/material in FP64 and stored as FP32 (and
// FP64 for the residual path): for affine elements (every Tet4, straight-sided
// Tet10, parallelepiped Hex8) J is constant, so one record per element holds
// J⁻¹ (9) and λ·detJ, μ·detJ (2); otherwise a record per integration point holds
// J⁻¹ (9) and detJ, plus λ, μ per element.  Computing J from FP32 coordinates
// would lose |X|/h·2⁻²⁴ relative accuracy (≈2e-5 on a 20-long beam with h = 0.05).
//
// Per integration point with reference derivatives dN (compile-time constants):
//   Gv[c][a] = Σ_i v_i[c] dN_i[a],  ∇v[c][d] = Σ_a Gv[c][a] J⁻¹[d][a]
//   flux P (σ, or the tangent δP = F δS + ∇v S),  Q[c][a] = w detJ Σ_d P[c][d] J⁻¹[d][a]
//   y_i[c] += Σ_a Q[c][a] dN_i[a]
#include "jfem_common.cuh"
#include "jfem_df.cuh"

namespace jfem {

void launch_apply_tet4(Ctx* c, bool fp32, int mode, const double* v, const float2* v2, bool mask_in, const int* stop);
void launch_apply_tet10(Ctx* c, bool fp32, int mode, const double* v, const float2* v2, bool mask_in, const int* stop);
void launch_apply_hex8(Ctx* c, bool fp32, int mode, const double* v, const float2* v2, bool mask_in, const int* stop);
void launch_tile_tet4(Ctx* c, const float2* v2, float* y, bool masked, double* part, const int* stop);
void launch_tile_tet10(Ctx* c, const float2* v2, float* y, bool masked, double* part, const int* stop);
void launch_tile_hex8(Ctx* c, const float2* v2, float* y, bool masked, double* part, const int* stop);
void nh_state_tet4(Ctx* c);
void nh_state_tet10(Ctx* c);
void nh_state_hex8(Ctx* c);

// ---------------------------------------------------------------------------
// geometry preparation (FP64)
// ---------------------------------------------------------------------------
template <int ET>
__global__ void k_affine_check(int64_t E, const int* __restrict__ conn, const double* __restrict__ X,
                               int* __restrict__ nonaffine, int* err) {
  constexpr int NN = Elem<ET>::NN, NQ = Elem<ET>::NQ;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
    double J0[3][3];
    for (int q = 0; q < NQ; ++q) {
      double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
      for (int i = 0; i < NN; ++i) {
        const int64_t n = conn[(int64_t)i * E + e];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int b = 0; b < 3; ++b) J[a][b] += dshape(ET, q, i, a) * X[3 * n + b];
      }
      if (!(det3(J) > 0.0)) raise_error(err, JFEM_ERR_NEG_JACOBIAN);
      if (q == 0) {
        for (int a = 0; a < 3; ++a)
          for (int b = 0; b < 3; ++b) J0[a][b] = J[a][b];
      } else {
        double sc = 0.0, df = 0.0;
        for (int a = 0; a < 3; ++a)
          for (int b = 0; b < 3; ++b) {
            sc = fmax(sc, fabs(J0[a][b]));
            df = fmax(df, fabs(J[a][b] - J0[a][b]));
          }
        if (df > 1e-12 * sc) atomicExch(nonaffine, 1);
      }
    }
  }
}

// Records (SoA, stride E):
//   affine:     k = 0..8 J⁻¹ (row-major [d][a]), 9 λ·detJ, 10 μ·detJ           → 11
//   non-affine: k = 10q + 0..8 J⁻¹, 10q + 9 detJ; then 10NQ: λ, 10NQ+1: μ      → 10NQ+2
template <int ET>
__global__ void k_prepare_geo(int64_t E, const int* __restrict__ conn, const double* __restrict__ X,
                              const double* __restrict__ lam, const double* __restrict__ mu, int affine,
                              double* __restrict__ g64, float* __restrict__ g32) {
  constexpr int NN = Elem<ET>::NN, NQ = Elem<ET>::NQ;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
    const int nq = affine ? 1 : NQ;
    for (int q = 0; q < nq; ++q) {
      double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
      for (int i = 0; i < NN; ++i) {
        const int64_t n = conn[(int64_t)i * E + e];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int b = 0; b < 3; ++b) J[a][b] += dshape(ET, q, i, a) * X[3 * n + b];
      }
      const double det = det3(J);
      double A[3][3];
      adj3(J, A);
      const double id = 1.0 / det;
      // J⁻¹[d][a] with ∂N/∂X_d = Σ_a J⁻¹[d][a] ∂N/∂ξ_a
      double rec[10];
      for (int d = 0; d < 3; ++d)
        for (int a = 0; a < 3; ++a) rec[3 * d + a] = A[d][a] * id;
      if (affine) {
        for (int k = 0; k < 9; ++k) {
          g64[(int64_t)k * E + e] = rec[k];
          g32[(int64_t)k * E + e] = (float)rec[k];
        }
        const double ld = lam[e] * det, md = mu[e] * det;
        g64[(int64_t)9 * E + e] = ld;
        g64[(int64_t)10 * E + e] = md;
        g32[(int64_t)9 * E + e] = (float)ld;
        g32[(int64_t)10 * E + e] = (float)md;
      } else {
        rec[9] = det;
        for (int k = 0; k < 10; ++k) {
          g64[(int64_t)(10 * q + k) * E + e] = rec[k];
          g32[(int64_t)(10 * q + k) * E + e] = (float)rec[k];
        }
      }
    }
    if (!affine) {
      g64[(int64_t)(10 * NQ) * E + e] = lam[e];
      g64[(int64_t)(10 * NQ + 1) * E + e] = mu[e];
      g32[(int64_t)(10 * NQ) * E + e] = (float)lam[e];
      g32[(int64_t)(10 * NQ + 1) * E + e] = (float)mu[e];
    }
  }
}

// Affine Tet4 records for a concatenated batch of meshes (jfem_batch.cu).
void prepare_geo_tet4_affine(int64_t E, const int* conn, const double* X, const double* lam, const double* mu,
                             double* g64, float* g32, cudaStream_t stream) {
  k_prepare_geo<JFEM_TET4><<<grid_for(E, 128), 128, 0, stream>>>(E, conn, X, lam, mu, 1, g64, g32);
}

// ---------------------------------------------------------------------------
// phase 2: node gather (ascending element order), masking and optional v·y partials.
// One thread per node (GATHER_GL = 1; with GL > 1 lanes split a node's entries
// and combine in a fixed butterfly — measured slower on the Tet10 beam).
// ---------------------------------------------------------------------------
#define GATHER_GL 1
template <typename R, bool DOT>
__global__ void __launch_bounds__(JFEM_RED_THREADS) k_gather(int64_t N, int64_t E, const int* __restrict__ ptr,
                                                             const unsigned* __restrict__ adj,
                                                             const R* __restrict__ ye,
                                                             const uint8_t* __restrict__ mask, int masked,
                                                             const double* __restrict__ v,
                                                             double* __restrict__ y, double* __restrict__ part,
                                                             const int* __restrict__ stop) {
  constexpr int GL = GATHER_GL, NPW = 32 / GL;
  __shared__ double sh[32];
  if (stop && *stop) return;
  const int lane = threadIdx.x & 31;
  const int sub = lane & (GL - 1);
  const int grp = lane / GL;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  double dot = 0.0;
  for (int64_t jb = warp * NPW; jb < N; jb += nwarps * NPW) {   // warp-uniform trip count
    const int64_t j = jb + grp;
    const bool act = j < N;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    if (act) {
      const int t1 = __ldg(ptr + j + 1);
      for (int t = __ldg(ptr + j) + sub; t < t1; t += GL) {
        const unsigned pk = __ldg(adj + t);
        const int64_t e = pk >> 4;
        const int a = (int)(pk & 15u);
        s0 += (double)__ldg(ye + (int64_t)(3 * a + 0) * E + e);
        s1 += (double)__ldg(ye + (int64_t)(3 * a + 1) * E + e);
        s2 += (double)__ldg(ye + (int64_t)(3 * a + 2) * E + e);
      }
    }
#pragma unroll
    for (int o = GL / 2; o > 0; o >>= 1) {
      s0 += __shfl_xor_sync(0xffffffffu, s0, o);
      s1 += __shfl_xor_sync(0xffffffffu, s1, o);
      s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    if (act && sub == 0) {
      if (masked) {
        const uint8_t m = __ldg(mask + j);
        if (m & 1) s0 = 0.0;
        if (m & 2) s1 = 0.0;
        if (m & 4) s2 = 0.0;
      }
      y[3 * j] = s0;
      y[3 * j + 1] = s1;
      y[3 * j + 2] = s2;
      if (DOT) dot += v[3 * j] * s0 + v[3 * j + 1] * s1 + v[3 * j + 2] * s2;
    }
  }
  if (DOT) {
    const double b = block_sum(dot, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = b;
  }
}

// Split v into FP32 (hi, lo) pairs: hi = fl32(v), lo = fl32(v − hi).
__global__ void k_split(int64_t n, const double* __restrict__ v, float2* __restrict__ v2) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double x = v[i];
    const float hi = (float)x;
    v2[i] = make_float2(hi, (float)(x - (double)hi));
  }
}

// Boundary nodes of the tiled apply: sum the tile partials in ascending tile
// order into y (FP32); optional v·y partials (double-float products, v the
// split input) into part[3G + blockIdx.x].  With sc (mixed PCG), the last block
// to finish forms p·Ap = Σ part[0..G) + Σ part[3G..4G) in FP64, in index order,
// and α = r·z / p·Ap for the update kernel.  Launched with G = JFEM_RED_BLOCKS
// blocks.  Each thread takes BND_ROUNDS nodes (k, k + stride, …) and issues
// their loads in two waves (node and run offsets; then the first BND_UNROLL
// partials of each run, the mask byte and v), so a thread waits for about two
// memory latencies; runs longer than BND_UNROLL (nodes shared by more tiles)
// finish in a loop.
constexpr int BND_ROUNDS = 1;
constexpr int BND_UNROLL = 4;

__global__ void __launch_bounds__(JFEM_RED_THREADS, 4) k_tile_boundary(int64_t nb, const int* __restrict__ bnodes,
                                                                    const int* __restrict__ bptr,
                                                                    const float4* __restrict__ bpart,
                                                                    const uint8_t* __restrict__ mask, int masked,
                                                                    const float2* __restrict__ vdot,
                                                                    float* __restrict__ y, double* __restrict__ part,
                                                                    SolverScalars* __restrict__ sc,
                                                                    const int* __restrict__ stop) {
  __shared__ double sh[32];
  if (stop && *stop) return;
  float2 dot = make_float2(0.f, 0.f);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t k0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k0 < nb; k0 += BND_ROUNDS * stride) {
    int g[BND_ROUNDS], i0[BND_ROUNDS], i1[BND_ROUNDS];
#pragma unroll
    for (int r = 0; r < BND_ROUNDS; ++r) {   // wave 1
      const int64_t k = k0 + r * stride;
      g[r] = 0;
      i0[r] = i1[r] = 0;
      if (k < nb) {
        g[r] = __ldg(bnodes + k);
        i0[r] = __ldg(bptr + k);
        i1[r] = __ldg(bptr + k + 1);
      }
    }
    float4 q[BND_ROUNDS][BND_UNROLL];
    unsigned m[BND_ROUNDS];
    float2 vv[BND_ROUNDS][3];
#pragma unroll
    for (int r = 0; r < BND_ROUNDS; ++r) {   // wave 2
      const int64_t k = k0 + r * stride;
#pragma unroll
      for (int u = 0; u < BND_UNROLL; ++u)
        q[r][u] = i0[r] + u < i1[r] ? __ldcs(bpart + i0[r] + u) : make_float4(0.f, 0.f, 0.f, 0.f);   // read once
      m[r] = (k < nb && masked) ? (unsigned)__ldg(mask + g[r]) : 0u;
      if (part && k < nb) {
#pragma unroll
        for (int c = 0; c < 3; ++c) vv[r][c] = __ldg(vdot + 3 * (int64_t)g[r] + c);
      }
    }
#pragma unroll
    for (int r = 0; r < BND_ROUNDS; ++r) {
      const int64_t k = k0 + r * stride;
      if (k >= nb) continue;
      float s0 = 0.f, s1 = 0.f, s2 = 0.f;
#pragma unroll
      for (int u = 0; u < BND_UNROLL; ++u) {   // ascending tile order, as the loop below continues it
        s0 += q[r][u].x;
        s1 += q[r][u].y;
        s2 += q[r][u].z;
      }
      for (int i = i0[r] + BND_UNROLL; i < i1[r]; ++i) {
        const float4 t = __ldcs(bpart + i);
        s0 += t.x;
        s1 += t.y;
        s2 += t.z;
      }
      if (m[r] & 1) s0 = 0.f;
      if (m[r] & 2) s1 = 0.f;
      if (m[r] & 4) s2 = 0.f;
      const int64_t gg = g[r];
      y[3 * gg] = s0;
      y[3 * gg + 1] = s1;
      y[3 * gg + 2] = s2;
      if (part) {
        dot = df_add_abs(dot, df_add_abs(df_dot_term(vv[r][0], s0),
                                         df_add_abs(df_dot_term(vv[r][1], s1), df_dot_term(vv[r][2], s2))));
      }
    }
  }
  if (part) {
    const double b = block_sum_df(dot, sh);
    if (threadIdx.x == 0) part[3 * JFEM_RED_BLOCKS + blockIdx.x] = b;
    if (sc && arrive_last(&sc->arrive[0])) {
      const double2 ab = reduce_partials2_cg(part, part + 3 * JFEM_RED_BLOCKS, JFEM_RED_BLOCKS, sh);
      const double pAp = ab.x + ab.y;
      if (threadIdx.x == 0) {
        const double a = sc->rz[0] / pAp;
        sc->pAp = pAp;
        sc->alpha = a;
        sc->alpha_df = df_from_double(a);
        sc->arrive[0] = 0;
      }
    }
  }
}

// y (FP64) = y32 (FP32), for callers of the FP32 apply that want doubles
__global__ void k_widen(int64_t n, const float* __restrict__ a, double* __restrict__ b) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (double)a[i];
}

// geometry records to tile order (padding zero)
__global__ void k_permute_records(int rec, int64_t E, int64_t Epad, const int* __restrict__ perm,
                                  const float* __restrict__ src, float* __restrict__ dst) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (int64_t)rec * Epad;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(i / Epad);
    const int64_t p = i - (int64_t)k * Epad;
    const int e = perm[p];
    dst[i] = e >= 0 ? src[(int64_t)k * E + e] : 0.f;
  }
}

void enqueue_split(Ctx* c, const double* v, float2* v2) {
  k_split<<<grid_for(3 * c->N, 256), 256, 0, c->stream>>>(3 * c->N, v, v2);
  c->launches += 1;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
int geometry_invalidate(Ctx* c) {
  if (c->pcg_graph) {   // captured launches hold the geometry pointers
    cudaGraphExecDestroy(c->pcg_graph);
    c->pcg_graph = nullptr;
    c->pcg_graph_key = -1;
  }
  if (c->geo64) { dfree(c, c->geo64); c->geo64 = nullptr; }
  if (c->geo32) { dfree(c, c->geo32); c->geo32 = nullptr; }
  if (c->geoT32) { dfree(c, c->geoT32); c->geoT32 = nullptr; }
  c->geo_ready = false;
  ++c->state_version;
  ++c->geo_gen;
  return 0;
}

template <int ET>
static int prepare_et(Ctx* c) {
  constexpr int NQ = Elem<ET>::NQ;
  int* flag = nullptr;
  if (cudaMalloc(&flag, sizeof(int)) != cudaSuccess) return set_err(c, JFEM_ERR_OOM, "geometry flag");
  cudaMemsetAsync(flag, 0, sizeof(int), c->stream);
  cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream);
  k_affine_check<ET><<<grid_for(c->E, 128), 128, 0, c->stream>>>(c->E, c->conn, c->X64, flag, c->d_err);
  int h_flag = 0, h_err = 0;
  cudaMemcpyAsync(&h_flag, flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  cudaMemcpyAsync(&h_err, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  int rc = sync_and_check(c, "affine check");
  cudaFree(flag);
  c->launches += 1;
  if (rc) return rc;
  if (h_err) return set_err(c, JFEM_ERR_NEG_JACOBIAN, "element with non-positive Jacobian determinant");
  c->geo_affine = (h_flag == 0);
  const int64_t rec = c->geo_affine ? 11 : (10 * NQ + 2);
  if ((rc = dalloc(c, &c->geo64, rec * c->E))) return rc;
  if ((rc = dalloc(c, &c->geo32, rec * c->E))) return rc;
  k_prepare_geo<ET><<<grid_for(c->E, 128), 128, 0, c->stream>>>(c->E, c->conn, c->X64, c->lam64, c->mu64,
                                                                c->geo_affine ? 1 : 0, c->geo64, c->geo32);
  c->launches += 1;
  if (c->ntiles > 0) {
    if ((rc = dalloc(c, &c->geoT32, rec * c->Epad))) return rc;
    k_permute_records<<<grid_for(rec * c->Epad, 256), 256, 0, c->stream>>>((int)rec, c->E, c->Epad, c->tperm,
                                                                          c->geo32, c->geoT32);
    c->launches += 1;
  }
  rc = sync_and_check(c, "geometry");
  if (!rc) c->geo_ready = true;
  return rc;
}

int geometry_prepare(Ctx* c) {
  if (c->geo_ready) return 0;
  if (!c->have_material) return set_err(c, JFEM_ERR_INVALID, "jfem_set_material must come first");
  switch (c->et) {
    case JFEM_TET4: return prepare_et<JFEM_TET4>(c);
    case JFEM_TET10: return prepare_et<JFEM_TET10>(c);
    default: return prepare_et<JFEM_HEX8>(c);
  }
}

static void launch_elements(Ctx* c, bool fp32, int mode, const double* v, const float2* v2, bool mask_in,
                            const int* stop) {
  switch (c->et) {
    case JFEM_TET4: launch_apply_tet4(c, fp32, mode, v, v2, mask_in, stop); break;
    case JFEM_TET10: launch_apply_tet10(c, fp32, mode, v, v2, mask_in, stop); break;
    default: launch_apply_hex8(c, fp32, mode, v, v2, mask_in, stop); break;
  }
}

static void launch_gather(Ctx* c, bool fp32, bool masked, const double* v, double* y, double* part, const int* stop) {
  const unsigned gb = part ? JFEM_RED_BLOCKS : grid_for(c->N * GATHER_GL, JFEM_RED_THREADS);
  if (fp32) {
    if (part) k_gather<float, true><<<gb, JFEM_RED_THREADS, 0, c->stream>>>(c->N, c->E, c->adj_ptr, c->adj, c->ye32, c->mask, masked, v, y, part, stop);
    else k_gather<float, false><<<gb, JFEM_RED_THREADS, 0, c->stream>>>(c->N, c->E, c->adj_ptr, c->adj, c->ye32, c->mask, masked, v, y, part, stop);
  } else {
    if (part) k_gather<double, true><<<gb, JFEM_RED_THREADS, 0, c->stream>>>(c->N, c->E, c->adj_ptr, c->adj, c->ye64, c->mask, masked, v, y, part, stop);
    else k_gather<double, false><<<gb, JFEM_RED_THREADS, 0, c->stream>>>(c->N, c->E, c->adj_ptr, c->adj, c->ye64, c->mask, masked, v, y, part, stop);
  }
  c->launches += 1;
}

// Enqueue (no sync): y = K v (masked rows zero when masked), partial v·y sums
// into part[0..JFEM_RED_BLOCKS) when part != nullptr.
// FP32 with a split input and a built tiling → the tiled apply (interior
// partials in part[0..G), boundary partials in part[3G..4G)); otherwise the
// two-phase apply (partials in part[0..G)).
bool apply_is_tiled(const Ctx* c) { return c->geoT32 && c->ntiles > 0; }

// Point state of the Neo-Hookean tangent at the current u_state (enqueued, no
// sync); later tiled tangent applies read it until u, the material, the
// formulation or the geometry change (state_version).
int nh_state_prepare(Ctx* c) {
  if (!c->finite || c->model != JFEM_NEO_HOOKEAN) return 0;
  int rc = geometry_prepare(c);
  if (rc) return rc;
  if (!apply_is_tiled(c)) return 0;
  if (nh_cache_ready(c)) return 0;
  if (!c->nhstate) {
    const int nq = c->et == JFEM_TET4 ? Elem<JFEM_TET4>::NQ : c->et == JFEM_TET10 ? Elem<JFEM_TET10>::NQ
                                                                                    : Elem<JFEM_HEX8>::NQ;
    if ((rc = dalloc(c, &c->nhstate, (size_t)16 * nq * c->Epad))) return rc;
  }
  switch (c->et) {
    case JFEM_TET4: nh_state_tet4(c); break;
    case JFEM_TET10: nh_state_tet10(c); break;
    default: nh_state_hex8(c); break;
  }
  c->nhstate_version = c->state_version;
  return 0;
}

static void launch_tiles(Ctx* c, const float2* v2, float* y, bool masked, double* part, const int* stop) {
  switch (c->et) {
    case JFEM_TET4: launch_tile_tet4(c, v2, y, masked, part, stop); break;
    case JFEM_TET10: launch_tile_tet10(c, v2, y, masked, part, stop); break;
    default: launch_tile_hex8(c, v2, y, masked, part, stop); break;
  }
}

static void launch_tile_boundary(Ctx* c, const float2* vdot, float* y, bool masked, double* part, const int* stop,
                                 SolverScalars* sc = nullptr) {
  k_tile_boundary<<<JFEM_RED_BLOCKS, JFEM_RED_THREADS, 0, c->stream>>>(
      c->n_bnodes, c->bnodes, c->bptr, c->bpart, c->mask, masked ? 1 : 0, vdot, y, part, sc, stop);
  c->launches += 1;
}

// Tiled FP32 apply of the split input v2: tile pass + boundary pass, y FP32;
// v·y partials (double-float products) into part[0..G) and part[3G..4G).
// With sc (mixed PCG): the boundary pass also forms α (see k_tile_boundary).
void enqueue_apply_tiled(Ctx* c, const float2* v2, float* y, bool masked, double* part, const int* stop,
                         SolverScalars* sc) {
  launch_tiles(c, v2, y, masked, part, stop);
  launch_tile_boundary(c, v2, y, masked, part, stop, sc);
}

void enqueue_apply(Ctx* c, const double* v, double* y, bool fp32, bool masked, bool mask_in, double* part,
                   const int* stop, const float2* v2) {
  launch_elements(c, fp32, 0, v, fp32 ? v2 : nullptr, mask_in, stop);
  launch_gather(c, fp32, masked, v, y, part, stop);
}

int apply_device(Ctx* c, const double* v, double* y, bool fp32, bool masked, double* part) {
  int rc = geometry_prepare(c);
  if (rc) return rc;
  cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream);
  cudaEventRecord(c->ev0, c->stream);
  if (fp32 && apply_is_tiled(c)) {
    enqueue_split(c, v, c->p2);
    enqueue_apply_tiled(c, c->p2, c->Apf, masked, part, nullptr);
    k_widen<<<grid_for(3 * c->N, 256), 256, 0, c->stream>>>(3 * c->N, c->Apf, y);
    c->launches += 1;
  } else {
    if (fp32) enqueue_split(c, v, c->p2);
    enqueue_apply(c, v, y, fp32, masked, masked, part, nullptr, fp32 ? c->p2 : nullptr);
  }
  cudaEventRecord(c->ev1, c->stream);
  int h_err = 0;
  cudaMemcpyAsync(&h_err, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  rc = sync_and_check(c, "apply");
  if (rc) return rc;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, c->ev0, c->ev1);
  c->last_apply_ms = ms;
  if (h_err) return set_err(c, h_err, "invalid material state in apply (det C <= 0 or NaN)");
  return 0;
}

// Enqueue f_int(u) (FP64) into f (no sync).  Linear small strain: K u.
void enqueue_internal_force(Ctx* c, double* f) {
  if (!c->finite) launch_elements(c, false, 0, c->u_state, nullptr, false, nullptr);
  else launch_elements(c, false, 1, nullptr, nullptr, false, nullptr);
  launch_gather(c, false, false, nullptr, f, nullptr, nullptr);
}

int internal_force_device(Ctx* c, double* f) {
  int rc = geometry_prepare(c);
  if (rc) return rc;
  cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream);
  enqueue_internal_force(c, f);
  int h_err = 0;
  cudaMemcpyAsync(&h_err, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  rc = sync_and_check(c, "internal force");
  if (rc) return rc;
  if (h_err) return set_err(c, h_err, "invalid material state (det C <= 0 or NaN)");
  return 0;
}

}  // namespace jfem

namespace jfem {

__global__ void k_fill_pattern(int64_t n, double* __restrict__ v) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    v[i] = 1.0 + 1e-3 * (double)(i % 97);
}

// Event-timed element and gather kernels of the apply, reps times on ctx vectors.
int time_apply(Ctx* c, bool fp32, bool masked, int reps, double* ms_elem, double* ms_gather) {
  int rc = geometry_prepare(c);
  if (rc) return rc;
  if (reps <= 0) return set_err(c, JFEM_ERR_INVALID, "reps must be positive");
  k_fill_pattern<<<grid_for(3 * c->N, 256), 256, 0, c->stream>>>(3 * c->N, c->tmp);
  if (fp32) enqueue_split(c, c->tmp, c->p2);
  cudaEvent_t e0, e1, e2;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventCreate(&e2);
  double se = 0.0, sg = 0.0;
  for (int r = 0; r < reps; ++r) {
    cudaEventRecord(e0, c->stream);
    if (fp32 && apply_is_tiled(c)) {
      launch_tiles(c, c->p2, c->Apf, masked, c->part, nullptr);
      cudaEventRecord(e1, c->stream);
      launch_tile_boundary(c, c->p2, c->Apf, masked, c->part, nullptr);
    } else {
      launch_elements(c, fp32, 0, c->tmp, fp32 ? c->p2 : nullptr, masked, nullptr);
      cudaEventRecord(e1, c->stream);
      launch_gather(c, fp32, masked, c->tmp, c->tmp2, c->part, nullptr);
    }
    cudaEventRecord(e2, c->stream);
    cudaEventSynchronize(e2);
    float a = 0.f, b = 0.f;
    cudaEventElapsedTime(&a, e0, e1);
    cudaEventElapsedTime(&b, e1, e2);
    se += a;
    sg += b;
  }
  rc = sync_and_check(c, "timed apply");
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(e2);
  if (rc) return rc;
  *ms_elem = se / reps;
  *ms_gather = sg / reps;
  return 0;
}

}  // namespace jfem
