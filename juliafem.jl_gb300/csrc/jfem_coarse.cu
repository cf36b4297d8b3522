// jfem_coarse.cu — the coarse level of the two-level preconditioner used by
// flexible CG (methods JFEM_FCG_TWO_LEVEL and JFEM_FCG_LEARNED):
//
//   z = S r + P A_c⁻¹ Pᵀ r,      A_c = Pᵀ K P,
//
// S the fine-level smoother (Jacobi D⁻¹, or the learned SPD network), P the
// rigid-body modes of node aggregates: the nodes are binned into a structured
// grid of boxes over the mesh's bounding box, and each aggregate a contributes
// six columns — three translations and three rotations about its centroid c_a,
// (P_a)_i = m_i ⊙ (t + ω × (X_i − c_a)), m_i zero on prescribed DOFs.  Both terms
// are symmetric positive (semi)definite, so z = M r with M SPD and flexible CG
// keeps PCG's convergence.  The reference ships only unpreconditioned CG
// (src/backend/cpu.jl:221-254, ext/JuliaFEMCUDAExt.jl:531-577); its GPU solver
// design note names a multigrid-type coarse correction with GPU-friendly
// point smoothers as the preconditioner to build
// (docs/src/book/design/gpu_solver_strategy_expert_validated.md:114-156).  An
// aggregation coarse space of rigid-body modes is that coarse level in its
// algebraic form: it needs no mesh hierarchy and removes the low-energy
// bending modes that set Jacobi-PCG's iteration count on slender parts.
//
// Set-up, per (mesh, Dirichlet mask) on the host: the aggregation, node
// offsets X_i − c_a, and the list of elements whose A_c contribution is not
// zero — an element whose nodes all lie in one aggregate with no prescribed DOF
// moves rigidly under every mode of that aggregate, so K_e P_e = 0 there.
// Per geometry generation (material, coordinates) on the device, in
// double-float (48-bit, on the FP32 pipe — GB300's FP64 pipe is far slower; the
// physical gradients come from the FP64 geometry records):
//   k_coarse_elem    one warp per listed element: the strain of each mode at
//                    each integration point and the 6×6 blocks
//                    Σ_q w_q (λ tr ε_a tr ε_b + 2μ ε_a : ε_b) for every pair
//                    of the element's aggregates;
//   k_coarse_reduce  each A_c block summed over its elements in ascending
//                    element order (deterministic, no atomics);
//   k_gj_*           blocked Gauss–Jordan inversion of the dense SPD A_c
//                    (diagonal pivots, 32×32 blocks; a pivot below 1e-12 of
//                    its original diagonal drops that mode);
// the inverse is rounded to FP32 for the per-iteration coarse solve.
// Per CG iteration: k_coarse_restrict (one CTA per chunk of an aggregate's
// nodes: partial force and moment resultants of r about c_a; the aggregate's
// last chunk to finish sums its chunks in chunk order into Pᵀ r), k_coarse_gemv
// (Ec = A_c⁻¹ Pᵀ r, one warp per row); the prolongation P Ec is fused into the
// kernel that forms z.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "jfem_common.cuh"
#include "jfem_df.cuh"

namespace jfem {

#define CG_MAXN 10   // node slots per element in celem_aggs (Tet10 has the most nodes)

// ---------------------------------------------------------------------------
// A_c contributions (double-float on the FP32 pipe: GB300's FP64 pipe runs at a
// small fraction of its FP32 rate; the physical gradients start from the FP64
// geometry records and every product after them is double-float, 48-bit)
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 df_sub(float2 a, float2 b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ float2 df_zero() { return make_float2(0.f, 0.f); }

// component c of mode k at offset d (translations, then e_x × d, e_y × d, e_z × d)
__device__ __forceinline__ float2 mode_component(int k, int c, const float2 d[3]) {
  switch (k) {
    case 0: return make_float2(c == 0 ? 1.f : 0.f, 0.f);
    case 1: return make_float2(c == 1 ? 1.f : 0.f, 0.f);
    case 2: return make_float2(c == 2 ? 1.f : 0.f, 0.f);
    case 3: return c == 0 ? df_zero() : c == 1 ? df_neg(d[2]) : d[1];
    case 4: return c == 0 ? d[2] : c == 1 ? df_zero() : df_neg(d[0]);
    default: return c == 0 ? df_neg(d[1]) : c == 1 ? d[0] : df_zero();
  }
}

template <int ET>
__global__ void __launch_bounds__(64) k_coarse_elem(int64_t n_celem, const int* __restrict__ celem,
                                                    const int* __restrict__ celem_aggs,
                                                    const int64_t* __restrict__ celem_off, int64_t E,
                                                    const int* __restrict__ conn, const uint8_t* __restrict__ mask,
                                                    const int* __restrict__ node_agg,
                                                    const float2* __restrict__ node_d,
                                                    const double* __restrict__ geo, int affine,
                                                    float2* __restrict__ contrib) {
  constexpr int NN = Elem<ET>::NN, NQ = Elem<ET>::NQ, NC = 6 * NN;
  __shared__ float2 s_d[2][NN][3];
  __shared__ int s_al[2][NN];
  __shared__ unsigned s_m[2][NN];
  __shared__ float2 s_gN[2][NQ][NN][3];
  __shared__ float2 s_S[2][NQ][NC][6];
  __shared__ float2 s_lw[2][NQ], s_mw[2][NQ];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int64_t k = (int64_t)blockIdx.x * 2 + w; k < n_celem; k += (int64_t)gridDim.x * 2) {
    const int64_t e = celem[k];
    const int* al = celem_aggs + k * CG_MAXN;
    int A = 0;
    while (A < NN && al[A] >= 0) ++A;
    if (lane < NN) {
      const int n = conn[(int64_t)lane * E + e];
      const int a = node_agg[n];
      int la = 0;
      while (la < A - 1 && al[la] != a) ++la;
      s_al[w][lane] = la;
      s_m[w][lane] = mask[n];
#pragma unroll
      for (int b = 0; b < 3; ++b) s_d[w][lane][b] = node_d[3 * (int64_t)n + b];
    }
    // physical gradients ∇N_i(q) = J⁻ᵀ dN_i(q) (FP64 from the records, then rounded
    // to double-float) and the weights w_q λ detJ, w_q μ detJ
    for (int t = lane; t < NQ * NN; t += 32) {
      const int q = t / NN, i = t % NN;
      const int64_t base = affine ? 0 : 10 * q;
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        double s = 0.0;
#pragma unroll
        for (int a = 0; a < 3; ++a) s += geo[(base + 3 * d + a) * E + e] * dshape(ET, q, i, a);
        s_gN[w][q][i][d] = df_from_double(s);
      }
    }
    if (lane < NQ) {
      const int q = lane;
      const double wq = qp_weight(ET, q);
      double lw, mw;
      if (affine) {
        lw = wq * geo[9 * E + e];
        mw = wq * geo[10 * E + e];
      } else {
        const double det = geo[(int64_t)(10 * q + 9) * E + e];
        lw = wq * det * geo[(int64_t)(10 * NQ) * E + e];
        mw = wq * det * geo[(int64_t)(10 * NQ + 1) * E + e];
      }
      s_lw[w][q] = df_from_double(lw);
      s_mw[w][q] = df_from_double(2.0 * mw);   // 2μ, the factor of ε:ε
    }
    __syncwarp();
    // strain (xx, yy, zz, xy, yz, xz) of every mode column (aggregate α, mode k) at every q
    const int ncol = 6 * A;
    for (int t = lane; t < NQ * ncol; t += 32) {
      const int q = t / ncol, col = t % ncol, alpha = col / 6, km = col % 6;
      float2 G[3][3];
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int d = 0; d < 3; ++d) G[c][d] = df_zero();
      for (int i = 0; i < NN; ++i) {
        if (s_al[w][i] != alpha) continue;
        const unsigned m = s_m[w][i];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          if ((m >> c) & 1u) continue;
          const float2 vc = mode_component(km, c, s_d[w][i]);
          if (km < 3) {   // a translation: vc is 0 or 1
            if (vc.x != 0.f)
#pragma unroll
              for (int d = 0; d < 3; ++d) G[c][d] = df_add(G[c][d], s_gN[w][q][i][d]);
          } else {
#pragma unroll
            for (int d = 0; d < 3; ++d) G[c][d] = df_add(G[c][d], df_mul(vc, s_gN[w][q][i][d]));
          }
        }
      }
      float2* S = s_S[w][q][col];
      const float2 half = make_float2(0.5f, 0.f);
      S[0] = G[0][0];
      S[1] = G[1][1];
      S[2] = G[2][2];
      S[3] = df_mul(half, df_add(G[0][1], G[1][0]));
      S[4] = df_mul(half, df_add(G[1][2], G[2][1]));
      S[5] = df_mul(half, df_add(G[0][2], G[2][0]));
    }
    __syncwarp();
    // blocks (α, β): entry (k, l) = Σ_q λ_q tr ε_αk tr ε_βl + 2μ_q ε_αk : ε_βl, formed once
    // per unordered column pair and written to both (α, β)[k][l] and (β, α)[l][k], so
    // the assembled A_c is exactly symmetric
    const int64_t off = celem_off[k];
    for (int t = lane; t < ncol * ncol; t += 32) {
      const int ca = t / ncol, cb = t % ncol;
      if (cb < ca) continue;
      float2 s = df_zero();
#pragma unroll
      for (int q = 0; q < NQ; ++q) {
        const float2* a = s_S[w][q][ca];
        const float2* b = s_S[w][q][cb];
        const float2 tra = df_add(df_add(a[0], a[1]), a[2]), trb = df_add(df_add(b[0], b[1]), b[2]);
        const float2 dd = df_add(df_add(df_mul(a[0], b[0]), df_mul(a[1], b[1])), df_mul(a[2], b[2]));
        const float2 od = df_add(df_add(df_mul(a[3], b[3]), df_mul(a[4], b[4])), df_mul(a[5], b[5]));
        s = df_add(s, df_mul(s_lw[w][q], df_mul(tra, trb)));
        s = df_add(s, df_mul(s_mw[w][q], df_add(dd, df_add(od, od))));
      }
      const int alpha = ca / 6, beta = cb / 6;
      contrib[(off + alpha * A + beta) * 36 + 6 * (ca % 6) + (cb % 6)] = s;
      if (ca != cb) contrib[(off + beta * A + alpha) * 36 + 6 * (cb % 6) + (ca % 6)] = s;
    }
    __syncwarp();
  }
}

// A_c block (a, b) = Σ of its element blocks, ascending element order (double-float)
__global__ void k_coarse_reduce(int64_t n_cblk, const int* __restrict__ cblk_ab, const int* __restrict__ cblk_ptr,
                                const int64_t* __restrict__ cblk_src, const float2* __restrict__ contrib, int ld,
                                float2* __restrict__ Ac) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n_cblk * 36;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = t / 36;
    const int ent = (int)(t % 36);
    float2 s = df_zero();
    for (int p = cblk_ptr[b]; p < cblk_ptr[b + 1]; ++p) s = df_add(s, contrib[cblk_src[p] * 36 + ent]);
    const int ra = cblk_ab[2 * b], cb = cblk_ab[2 * b + 1];
    Ac[(int64_t)(6 * ra + ent / 6) * ld + 6 * cb + ent % 6] = s;
  }
}

__global__ void k_diag_copy(int n, int ld, const float2* __restrict__ A, double* __restrict__ d) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    d[i] = df_to_double(A[(int64_t)i * ld + i]);
}

__global__ void k_round_f32(int64_t n, const float2* __restrict__ a, float* __restrict__ b) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = __fadd_rn(a[i].x, a[i].y);
}

// ---------------------------------------------------------------------------
// blocked Gauss–Jordan inversion (double-float, in place; A symmetric positive
// definite).  Per pivot block K with P = A_KK⁻¹:  A_IJ −= A_IK P A_KJ,
// A_KJ ← P A_KJ,  A_IK ← −A_IK P,  A_KK ← P  (I, J ≠ K).  After the last block A
// holds A⁻¹.  Each pivot's reciprocal is formed in FP64 by one thread.
// ---------------------------------------------------------------------------
#define GJ_B 32

__global__ void __launch_bounds__(1024) k_gj_pivot(const float2* __restrict__ A, int ld, int K0,
                                                   const double* __restrict__ diag0, float2* __restrict__ P) {
  __shared__ float2 B[GJ_B][GJ_B + 1];
  __shared__ float2 prow[GJ_B], pcol[GJ_B];
  __shared__ float2 pinv;
  const int i = threadIdx.y, j = threadIdx.x;
  B[i][j] = A[(int64_t)(K0 + i) * ld + K0 + j];
  __syncthreads();
  for (int k = 0; k < GJ_B; ++k) {
    if (i == 0 && j == 0) {
      const double piv = df_to_double(B[k][k]), d0 = diag0[K0 + k];
      pinv = (d0 > 0.0 && piv > 1e-12 * d0) ? df_from_double(1.0 / piv) : df_zero();   // else: drop this mode
    }
    if (i == 0) prow[j] = B[k][j];
    if (j == 0) pcol[i] = B[i][k];
    __syncthreads();
    const float2 p = pinv;
    float2 v = B[i][j];
    if (i != k && j != k) v = df_sub(v, df_mul(df_mul(pcol[i], prow[j]), p));
    else if (i == k && j != k) v = df_mul(prow[j], p);
    else if (i != k) v = df_neg(df_mul(pcol[i], p));
    else v = p;
    B[i][j] = v;
    __syncthreads();
  }
  P[i * GJ_B + j] = B[i][j];
}

// row panel Brow[:, J] = P A_KJ and a copy of the old column panel Ccol[J, :] = A_JK
__global__ void __launch_bounds__(256) k_gj_panel(const float2* __restrict__ A, int ld, int Kb,
                                                  const float2* __restrict__ P, float2* __restrict__ Brow,
                                                  float2* __restrict__ Ccol) {
  __shared__ float2 sP[GJ_B][GJ_B + 1], sA[GJ_B][GJ_B + 1];
  const int J = blockIdx.x;
  if (J == Kb) return;
  const int K0 = Kb * GJ_B, J0 = J * GJ_B;
  for (int t = threadIdx.x; t < GJ_B * GJ_B; t += blockDim.x) {
    const int r = t / GJ_B, q = t % GJ_B;
    sP[r][q] = P[t];
    sA[r][q] = A[(int64_t)(K0 + r) * ld + J0 + q];
    Ccol[(int64_t)(J0 + r) * GJ_B + q] = A[(int64_t)(J0 + r) * ld + K0 + q];
  }
  __syncthreads();
  for (int t = threadIdx.x; t < GJ_B * GJ_B; t += blockDim.x) {
    const int r = t / GJ_B, q = t % GJ_B;
    float2 s = df_zero();
#pragma unroll 8
    for (int k = 0; k < GJ_B; ++k) s = df_add(s, df_mul(sP[r][k], sA[k][q]));
    Brow[(int64_t)r * ld + J0 + q] = s;
  }
}

// every block of A; each CTA writes only its own block and reads only the panels
__global__ void __launch_bounds__(256) k_gj_update(float2* __restrict__ A, int ld, int Kb,
                                                   const float2* __restrict__ P, const float2* __restrict__ Brow,
                                                   const float2* __restrict__ Ccol) {
  __shared__ float2 sC[GJ_B][GJ_B + 1], sB[GJ_B][GJ_B + 1];
  const int I = blockIdx.y, J = blockIdx.x;
  const int I0 = I * GJ_B, J0 = J * GJ_B;
  if (I == Kb && J == Kb) {
    for (int t = threadIdx.x; t < GJ_B * GJ_B; t += blockDim.x)
      A[(int64_t)(I0 + t / GJ_B) * ld + J0 + t % GJ_B] = P[t];
    return;
  }
  if (I == Kb) {
    for (int t = threadIdx.x; t < GJ_B * GJ_B; t += blockDim.x)
      A[(int64_t)(I0 + t / GJ_B) * ld + J0 + t % GJ_B] = Brow[(int64_t)(t / GJ_B) * ld + J0 + t % GJ_B];
    return;
  }
  for (int t = threadIdx.x; t < GJ_B * GJ_B; t += blockDim.x) {
    const int r = t / GJ_B, q = t % GJ_B;
    sC[r][q] = Ccol[(int64_t)(I0 + r) * GJ_B + q];
    sB[r][q] = (J == Kb) ? P[t] : Brow[(int64_t)r * ld + J0 + q];
  }
  __syncthreads();
  for (int t = threadIdx.x; t < GJ_B * GJ_B; t += blockDim.x) {
    const int r = t / GJ_B, q = t % GJ_B;
    float2 s = df_zero();
#pragma unroll 8
    for (int k = 0; k < GJ_B; ++k) s = df_add(s, df_mul(sC[r][k], sB[k][q]));
    float2* a = A + (int64_t)(I0 + r) * ld + J0 + q;
    *a = (J == Kb) ? df_neg(s) : df_sub(*a, s);
  }
}

// ---------------------------------------------------------------------------
// per-iteration kernels
// ---------------------------------------------------------------------------

// Restriction Pᵀ r: for aggregate a, Σ_{i ∈ a} φ_k(d_i) · r_i — force (k < 3) and
// moment (k ≥ 3) resultants of r about the centroid (r is zero on prescribed
// DOFs) — and, when qold is given, the same for flexible CG's previous q (FP32).
// Each aggregate's node list is cut into chunks of at most CR_CHUNK nodes, one
// CTA per chunk (FP32 per thread and warp, FP64 across warps, fixed order); the
// chunk partials go to cpart[chunk][12] (r: 0..5, q_old: 6..11) and the coarse
// solve sums them.
#define CR_CHUNK 1024
__device__ __forceinline__ void add_resultants(float s[6], float4 d, float fx, float fy, float fz) {
  s[0] += fx;
  s[1] += fy;
  s[2] += fz;
  s[3] = fmaf(d.y, fz, fmaf(-d.z, fy, s[3]));
  s[4] = fmaf(d.z, fx, fmaf(-d.x, fz, s[4]));
  s[5] = fmaf(d.x, fy, fmaf(-d.y, fx, s[5]));
}

__global__ void __launch_bounds__(256) k_coarse_restrict(int n_chunks, const int* __restrict__ chunk_begin,
                                                         const int* __restrict__ agg_nodes,
                                                         const float4* __restrict__ d32,
                                                         const float2* __restrict__ r,
                                                         const float* __restrict__ qold, const int* __restrict__ stop,
                                                         const int* __restrict__ chunk_agg,
                                                         const int* __restrict__ agg_chunk_ptr,
                                                         unsigned* __restrict__ agg_cnt, int ld,
                                                         float* __restrict__ cpart, float* __restrict__ RQ) {
  __shared__ float sh[8][12];
  __shared__ int last;
  if (stop && *stop) return;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int ch = blockIdx.x;
  const int nk = qold ? 12 : 6;
  float s[12] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  // a chunk is at most CR_CHUNK = 4 · 256 nodes: every thread issues its four node
  // indices, then all their loads, before it adds anything (the loads overlap)
  const int t0 = chunk_begin[ch] + threadIdx.x, t1 = chunk_begin[ch + 1];
  int64_t idx[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) idx[u] = t0 + 256 * u < t1 ? (int64_t)agg_nodes[t0 + 256 * u] : -1;
  float2 rv[4][3];
  float4 dv[4];
  float qv[4][3];
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    if (idx[u] < 0) continue;
    const int64_t i = idx[u];
    rv[u][0] = r[3 * i];
    rv[u][1] = r[3 * i + 1];
    rv[u][2] = r[3 * i + 2];
    dv[u] = d32[i];
    if (qold) {
      qv[u][0] = qold[3 * i];
      qv[u][1] = qold[3 * i + 1];
      qv[u][2] = qold[3 * i + 2];
    }
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    if (idx[u] < 0) continue;
    add_resultants(s, dv[u], rv[u][0].x + rv[u][0].y, rv[u][1].x + rv[u][1].y, rv[u][2].x + rv[u][2].y);
    if (qold) add_resultants(s + 6, dv[u], qv[u][0], qv[u][1], qv[u][2]);
  }
  // FP32 warp trees, then the block's warps in order (FP32: the coarse level
  // is an FP32 preconditioner component; GB300's FP64 pipe would be the
  // kernel's bottleneck)
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    if (k < nk) {   // nk is the same for the whole block
      float v = s[k];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      if (lane == 0) sh[wid][k] = v;
    }
  }
  __syncthreads();
  if (threadIdx.x < nk) {
    float v = 0.f;
    for (int q = 0; q < nw; ++q) v += sh[q][threadIdx.x];
    cpart[12 * ch + threadIdx.x] = v;
    __threadfence();
  }
  __syncthreads();
  // the aggregate's last chunk to finish sums its chunks' partials in chunk
  // order into Pᵀr (RQ[0..ld)) and Pᵀq_old (RQ[ld..2ld)); nothing waits
  const int a = chunk_agg[ch];
  const int c0 = agg_chunk_ptr[a], c1 = agg_chunk_ptr[a + 1];
  if (threadIdx.x == 0) last = atomicAdd(agg_cnt + a, 1u) == (unsigned)(c1 - c0 - 1) ? 1 : 0;
  __syncthreads();
  if (!last) return;
  __threadfence();
  if (threadIdx.x < nk) {
    float v = 0.f;
    for (int q = c0; q < c1; ++q) v += __ldcg(cpart + 12 * q + threadIdx.x);
    const int k = threadIdx.x % 6, half = threadIdx.x / 6;
    RQ[half * ld + 6 * a + k] = v;
  }
  if (threadIdx.x == 0) agg_cnt[a] = 0;
}

// Ec = A_c⁻¹ Pᵀ r, one warp per row: Pᵀr (and Pᵀq_old with t2part) staged in
// shared memory from the restriction's per-aggregate sums, then each lane
// issues its contiguous float4 loads of the row of A_c⁻¹ (FP32) in batches of
// CG_GEMV_BATCH before it adds (fixed lane order and shuffle tree).  With
// t2part, also the products Ec_row·(Pᵀq_old)_row, summed over the block's rows
// in warp order, into t2part[block]; with sc, β (fcg_beta_last_block).
#define CG_GEMV_MAX JFEM_COARSE_MAX_DOFS
#define CG_GEMV_BATCH 12
__global__ void __launch_bounds__(256) k_coarse_gemv(int nc, int ld, const float* __restrict__ Ainv,
                                                     const float* __restrict__ RQ, const int* __restrict__ stop,
                                                     float* __restrict__ Ec, double* __restrict__ t2part,
                                                     SolverScalars* __restrict__ sc, const double* __restrict__ t1,
                                                     int n1) {
  __shared__ __align__(16) float R[CG_GEMV_MAX];
  __shared__ float Q[CG_GEMV_MAX];
  __shared__ double sh[32];
  if (stop && *stop) return;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int t0 = threadIdx.x; t0 < ld; t0 += 8 * blockDim.x) {   // ld ≤ 4096: at most two rounds
    float a[8], b[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int t = t0 + u * blockDim.x;
      a[u] = t < ld ? __ldcg(RQ + t) : 0.f;
      b[u] = (t2part && t < ld) ? __ldcg(RQ + ld + t) : 0.f;
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int t = t0 + u * blockDim.x;
      if (t < ld) {
        R[t] = a[u];
        Q[t] = b[u];
      }
    }
  }
  __syncthreads();
  const int row = blockIdx.x * (blockDim.x >> 5) + wid;
  double prod = 0.0;
  if (row < nc) {
    const float4* a = reinterpret_cast<const float4*>(Ainv + (int64_t)row * ld);
    const float4* x = reinterpret_cast<const float4*>(R);
    const int n4 = ld / 4;
    float s = 0.f;
    for (int j0 = lane; j0 < n4; j0 += 32 * CG_GEMV_BATCH) {
      float4 av[CG_GEMV_BATCH];
#pragma unroll
      for (int b = 0; b < CG_GEMV_BATCH; ++b) {
        const int j = j0 + 32 * b;
        av[b] = j < n4 ? __ldg(a + j) : make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int b = 0; b < CG_GEMV_BATCH; ++b) {
        const int j = j0 + 32 * b;
        const float4 xv = j < n4 ? x[j] : make_float4(0.f, 0.f, 0.f, 0.f);
        s = fmaf(av[b].x, xv.x, s);
        s = fmaf(av[b].y, xv.y, s);
        s = fmaf(av[b].z, xv.z, s);
        s = fmaf(av[b].w, xv.w, s);
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) Ec[row] = s;
    prod = (double)s * (double)Q[row];
  }
  if (!t2part) return;
  if (lane == 0) sh[wid] = prod;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += sh[q];
    t2part[blockIdx.x] = t;
  }
  // with sc: the last block forms flexible CG's β from the smoother's t1
  // partials (written by an earlier launch) and this launch's t2 partials
  if (sc && arrive_last(&sc->arrive[2])) {
    fcg_beta_last_block(sc, t1, n1, t2part, (int)gridDim.x, sh);
    if (threadIdx.x == 0) sc->arrive[2] = 0;
  }
}

// z = D⁻¹ r + P Ec (FP64 out): the two-level preconditioner with the Jacobi smoother
// for a host-given residual (jfem_coarse_precondition)
__global__ void k_coarse_jacobi_out(int64_t N, const double* __restrict__ r, const double* __restrict__ dinv,
                                    const uint8_t* __restrict__ mask, const int* __restrict__ node_agg,
                                    const float4* __restrict__ d32, const float* __restrict__ Ec,
                                    double* __restrict__ z) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < 3 * N; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = q / 3;
    const int c = (int)(q % 3);
    if ((mask[i] >> c) & 1) {
      z[q] = 0.0;
      continue;
    }
    z[q] = dinv[q] * r[q] + (double)coarse_prolong(node_agg, d32, Ec, i, c);
  }
}

__global__ void k_to_df(int64_t n, const double* __restrict__ a, float2* __restrict__ b) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float hi = (float)a[i];
    b[i] = make_float2(hi, (float)(a[i] - (double)hi));
  }
}

// ---------------------------------------------------------------------------
// host: structure (aggregation, element lists, block pattern)
// ---------------------------------------------------------------------------
// Coarse DOFs when none are requested: about one per 1,000 fine DOFs, within
// [192, 2304] — enough aggregates to carry the bending modes of slender parts
// (on the 2M-DOF Tet10 cantilever: 1,728 coarse DOFs after rounding the bins,
// 261 two-level iterations, against 287 with 1,458, 392 with 552 and 207 with
// 3,936), few enough that the set-up (the dense inverse is cubic in the coarse
// size: 12 ms here, 69 ms at 3,936) stays a small share of a solve.
static int auto_coarse_dofs(int64_t n_dofs) {
  const int64_t v = n_dofs / 1000;
  return (int)std::min<int64_t>(2304, std::max<int64_t>(192, v));
}

static int coarse_build(Ctx* c, int target_nc) {
  const int64_t N = c->N, E = c->E;
  const int nn = c->nn;
  std::vector<double> X((size_t)(3 * N));
  std::vector<int> conn((size_t)(nn * E));
  std::vector<uint8_t> mask((size_t)N);
  cudaMemcpyAsync(X.data(), c->X64, 3 * N * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  cudaMemcpyAsync(conn.data(), c->conn, (size_t)nn * E * sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  cudaMemcpyAsync(mask.data(), c->mask, N, cudaMemcpyDeviceToHost, c->stream);
  int rc = sync_and_check(c, "coarse set-up download");
  if (rc) return rc;
  // bins over the bounding box: about target_nc / 6 boxes of equal edge H
  double lo[3], hi[3], ext[3];
  for (int d = 0; d < 3; ++d) {
    lo[d] = hi[d] = X[d];
  }
  for (int64_t i = 0; i < N; ++i)
    for (int d = 0; d < 3; ++d) {
      lo[d] = std::min(lo[d], X[3 * i + d]);
      hi[d] = std::max(hi[d], X[3 * i + d]);
    }
  const double emax = std::max(hi[0] - lo[0], std::max(hi[1] - lo[1], hi[2] - lo[2]));
  if (!(emax > 0.0)) return set_err(c, JFEM_ERR_INVALID, "coarse space: the mesh has no extent");
  for (int d = 0; d < 3; ++d) ext[d] = std::max(hi[d] - lo[d], 1e-9 * emax);
  const int n_target = std::max(1, target_nc / 6);
  double H = std::cbrt(ext[0] * ext[1] * ext[2] / n_target);
  int nb[3];
  for (;;) {   // rounding each axis can overshoot the target; stay within JFEM_COARSE_MAX_DOFS
    for (int d = 0; d < 3; ++d) nb[d] = (int)std::max<long>(1, std::lround(ext[d] / H));
    if (6LL * nb[0] * nb[1] * nb[2] <= JFEM_COARSE_MAX_DOFS) break;
    H *= 1.05;
  }
  const int64_t ncell = (int64_t)nb[0] * nb[1] * nb[2];
  std::vector<int64_t> cell((size_t)N);
  std::vector<int> cell_id((size_t)ncell, -1);
  host_parallel(N, [&](int64_t i0, int64_t i1) {
    for (int64_t i = i0; i < i1; ++i) {
      int64_t cidx = 0;
      for (int d = 2; d >= 0; --d) {
        const int64_t b = std::min<int64_t>(nb[d] - 1, (int64_t)std::floor((X[3 * i + d] - lo[d]) / ext[d] * nb[d]));
        cidx = cidx * nb[d] + std::max<int64_t>(0, b);
      }
      cell[(size_t)i] = cidx;
    }
  });
  for (int64_t i = 0; i < N; ++i) cell_id[(size_t)cell[(size_t)i]] = 0;
  int nagg = 0;
  for (int64_t k = 0; k < ncell; ++k)
    if (cell_id[(size_t)k] == 0) cell_id[(size_t)k] = nagg++;
  const int nc = 6 * nagg, nc_pad = (nc + GJ_B - 1) / GJ_B * GJ_B;
  std::vector<int> node_agg((size_t)N), agg_ptr((size_t)nagg + 1, 0), agg_nodes((size_t)N);
  host_parallel(N, [&](int64_t i0, int64_t i1) {
    for (int64_t i = i0; i < i1; ++i) node_agg[(size_t)i] = cell_id[(size_t)cell[(size_t)i]];
  });
  for (int64_t i = 0; i < N; ++i) ++agg_ptr[(size_t)node_agg[(size_t)i] + 1];   // few counters: serial
  for (int a = 0; a < nagg; ++a) agg_ptr[(size_t)a + 1] += agg_ptr[(size_t)a];
  {
    std::vector<int> cur(agg_ptr.begin(), agg_ptr.end() - 1);
    for (int64_t i = 0; i < N; ++i) agg_nodes[(size_t)cur[(size_t)node_agg[(size_t)i]]++] = (int)i;
  }
  // restriction chunks: each aggregate's node list cut into pieces of ≤ CR_CHUNK
  std::vector<int> chunk_begin, agg_chunk_ptr(1, 0), chunk_agg;
  for (int a = 0; a < nagg; ++a) {
    for (int t = agg_ptr[(size_t)a]; t < agg_ptr[(size_t)a + 1]; t += CR_CHUNK) {
      chunk_begin.push_back(t);
      chunk_agg.push_back(a);
    }
    agg_chunk_ptr.push_back((int)chunk_begin.size());
  }
  const int n_chunks = (int)chunk_begin.size();
  chunk_begin.push_back((int)N);
  std::vector<double> cen((size_t)3 * nagg, 0.0);
  host_parallel(nagg, [&](int64_t a0, int64_t a1) {
    for (int64_t a = a0; a < a1; ++a) {
      double s[3] = {0, 0, 0};
      for (int t = agg_ptr[(size_t)a]; t < agg_ptr[(size_t)a + 1]; ++t)
        for (int d = 0; d < 3; ++d) s[d] += X[3 * (size_t)agg_nodes[(size_t)t] + d];
      const double cnt = (double)(agg_ptr[(size_t)a + 1] - agg_ptr[(size_t)a]);
      for (int d = 0; d < 3; ++d) cen[3 * (size_t)a + d] = s[d] / cnt;
    }
  });
  std::vector<float2> ddf((size_t)(3 * N));
  std::vector<float4> d32((size_t)N);
  host_parallel(N, [&](int64_t i0, int64_t i1) {
    for (int64_t i = i0; i < i1; ++i) {
      const int a = node_agg[(size_t)i];
      double dv[3];
      for (int d = 0; d < 3; ++d) {
        dv[d] = X[3 * (size_t)i + d] - cen[3 * (size_t)a + d];
        ddf[3 * (size_t)i + d] = df_from_double(dv[d]);
      }
      d32[(size_t)i] = make_float4((float)dv[0], (float)dv[1], (float)dv[2], 0.f);
    }
  });
  // elements with a nonzero contribution, their aggregates and contribution blocks
  // (each element's sorted aggregates on host threads into a scratch array,
  // then compacted in ascending element order)
  std::vector<int> celem, celem_aggs;
  std::vector<int64_t> celem_off;
  int64_t n_contrib = 0;
  {
    std::vector<int> eag((size_t)E * CG_MAXN);
    std::vector<int8_t> eA((size_t)E);
    host_parallel(E, [&](int64_t e0, int64_t e1) {
      for (int64_t e = e0; e < e1; ++e) {
        int* ag = &eag[(size_t)e * CG_MAXN];
        int A = 0;
        bool masked = false;
        for (int i = 0; i < nn; ++i) {
          const int n = conn[(size_t)i * E + e];
          masked = masked || mask[(size_t)n] != 0;
          const int a = node_agg[(size_t)n];
          bool seen = false;
          for (int q = 0; q < A; ++q) seen = seen || ag[q] == a;
          if (!seen) ag[A++] = a;
        }
        std::sort(ag, ag + A);
        eA[(size_t)e] = (int8_t)((A < 2 && !masked) ? 0 : A);
      }
    });
    for (int64_t e = 0; e < E; ++e) {
      const int A = eA[(size_t)e];
      if (A == 0) continue;
      celem.push_back((int)e);
      for (int q = 0; q < CG_MAXN; ++q) celem_aggs.push_back(q < A ? eag[(size_t)e * CG_MAXN + q] : -1);
      celem_off.push_back(n_contrib);
      n_contrib += (int64_t)A * A;
    }
  }
  const int64_t n_celem = (int64_t)celem.size();
  if (n_contrib >= (1LL << 31)) return set_err(c, JFEM_ERR_TOO_LARGE, "coarse space: too many element blocks");
  // A_c block pattern: (a, b) keys; sources in ascending element order
  std::vector<int> cnt((size_t)nagg * nagg, 0);
  for (int64_t k = 0; k < n_celem; ++k) {
    const int* ag = &celem_aggs[(size_t)k * CG_MAXN];
    for (int x = 0; x < CG_MAXN && ag[x] >= 0; ++x)
      for (int y = 0; y < CG_MAXN && ag[y] >= 0; ++y) ++cnt[(size_t)ag[x] * nagg + ag[y]];
  }
  std::vector<int> key_blk((size_t)nagg * nagg, -1), cblk_ab, cblk_ptr(1, 0);
  for (int64_t key = 0; key < (int64_t)nagg * nagg; ++key)
    if (cnt[(size_t)key]) {
      key_blk[(size_t)key] = (int)(cblk_ab.size() / 2);
      cblk_ab.push_back((int)(key / nagg));
      cblk_ab.push_back((int)(key % nagg));
      cblk_ptr.push_back(cblk_ptr.back() + cnt[(size_t)key]);
    }
  const int64_t n_cblk = (int64_t)cblk_ab.size() / 2;
  std::vector<int64_t> cblk_src((size_t)cblk_ptr.back());
  {
    std::vector<int> cur(cblk_ptr.begin(), cblk_ptr.end() - 1);
    for (int64_t k = 0; k < n_celem; ++k) {
      const int* ag = &celem_aggs[(size_t)k * CG_MAXN];
      int A = 0;
      while (A < CG_MAXN && ag[A] >= 0) ++A;
      for (int x = 0; x < A; ++x)
        for (int y = 0; y < A; ++y) {
          const int b = key_blk[(size_t)ag[x] * nagg + ag[y]];
          cblk_src[(size_t)cur[(size_t)b]++] = celem_off[(size_t)k] + (int64_t)x * A + y;
        }
    }
  }
  // device arrays (owned by the mesh; any previous set is released first)
  if (c->pcg_graph) {   // captured launches hold the old coarse pointers
    cudaGraphExecDestroy(c->pcg_graph);
    c->pcg_graph = nullptr;
    c->pcg_graph_key = -1;
  }
  // Until the last step below succeeds the context holds no coarse space
  // (built target −1, released arrays null): a failure here makes the next
  // coarse_prepare build it again instead of reading a partial set.
  c->coarse_built_target = -1;
  c->coarse_geo_gen = 0;
  auto release = [&](auto*& p) {
    dfree(c, p);
    p = nullptr;
  };
  release(c->agg_ptr); release(c->agg_nodes); release(c->node_agg); release(c->node_d32); release(c->node_ddf);
  release(c->celem); release(c->celem_aggs); release(c->celem_off); release(c->contrib); release(c->cblk_ab);
  release(c->cblk_ptr); release(c->cblk_src); release(c->Ac); release(c->Ac_diag); release(c->gj_buf);
  release(c->Ainv32); release(c->Ec); release(c->chunk_begin); release(c->agg_chunk_ptr); release(c->cpart);
  release(c->chunk_agg); release(c->agg_cnt); release(c->RQ);
  c->nagg = nagg;
  c->nc = nc;
  c->nc_pad = nc_pad;
  for (int d = 0; d < 3; ++d) c->nb_bins[d] = nb[d];
  c->n_celem = n_celem;
  c->n_contrib = n_contrib;
  c->n_cblk = n_cblk;
  c->n_chunks = n_chunks;
  if ((rc = dalloc(c, &c->agg_ptr, (size_t)nagg + 1)) || (rc = dalloc(c, &c->agg_nodes, (size_t)N)) ||
      (rc = dalloc(c, &c->node_agg, (size_t)N)) || (rc = dalloc(c, &c->node_d32, (size_t)N)) ||
      (rc = dalloc(c, &c->node_ddf, (size_t)(3 * N))) || (rc = dalloc(c, &c->celem, (size_t)n_celem)) ||
      (rc = dalloc(c, &c->celem_aggs, (size_t)n_celem * CG_MAXN)) ||
      (rc = dalloc(c, &c->celem_off, (size_t)n_celem)) || (rc = dalloc(c, &c->contrib, (size_t)n_contrib * 36)) ||
      (rc = dalloc(c, &c->cblk_ab, (size_t)(2 * n_cblk))) || (rc = dalloc(c, &c->cblk_ptr, (size_t)n_cblk + 1)) ||
      (rc = dalloc(c, &c->cblk_src, cblk_src.size())) || (rc = dalloc(c, &c->Ac, (size_t)nc_pad * nc_pad)) ||
      (rc = dalloc(c, &c->Ac_diag, (size_t)nc_pad)) || (rc = dalloc(c, &c->chunk_begin, (size_t)n_chunks + 1)) ||
      (rc = dalloc(c, &c->agg_chunk_ptr, (size_t)nagg + 1)) ||
      (rc = dalloc(c, &c->cpart, (size_t)12 * n_chunks)) || (rc = dalloc(c, &c->chunk_agg, (size_t)n_chunks)) ||
      (rc = dalloc(c, &c->agg_cnt, (size_t)nagg)) || (rc = dalloc(c, &c->RQ, (size_t)2 * nc_pad)) ||
      (rc = dalloc(c, &c->gj_buf, (size_t)GJ_B * GJ_B + 2 * (size_t)GJ_B * nc_pad)) ||
      (rc = dalloc(c, &c->Ainv32, (size_t)nc_pad * nc_pad)) || (rc = dalloc(c, &c->Ec, (size_t)nc_pad)))
    return rc;
  auto up = [&](void* dst, const void* src, size_t bytes) {
    if (bytes) cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream);
  };
  up(c->agg_ptr, agg_ptr.data(), agg_ptr.size() * sizeof(int));
  up(c->agg_nodes, agg_nodes.data(), agg_nodes.size() * sizeof(int));
  up(c->node_agg, node_agg.data(), node_agg.size() * sizeof(int));
  up(c->node_d32, d32.data(), d32.size() * sizeof(float4));
  up(c->node_ddf, ddf.data(), ddf.size() * sizeof(float2));
  up(c->celem, celem.data(), celem.size() * sizeof(int));
  up(c->celem_aggs, celem_aggs.data(), celem_aggs.size() * sizeof(int));
  up(c->celem_off, celem_off.data(), celem_off.size() * sizeof(int64_t));
  up(c->cblk_ab, cblk_ab.data(), cblk_ab.size() * sizeof(int));
  up(c->cblk_ptr, cblk_ptr.data(), cblk_ptr.size() * sizeof(int));
  up(c->cblk_src, cblk_src.data(), cblk_src.size() * sizeof(int64_t));
  up(c->chunk_begin, chunk_begin.data(), chunk_begin.size() * sizeof(int));
  up(c->agg_chunk_ptr, agg_chunk_ptr.data(), agg_chunk_ptr.size() * sizeof(int));
  up(c->chunk_agg, chunk_agg.data(), chunk_agg.size() * sizeof(int));
  cudaMemsetAsync(c->agg_cnt, 0, (size_t)nagg * sizeof(unsigned), c->stream);
  cudaMemsetAsync(c->RQ, 0, (size_t)2 * nc_pad * sizeof(float), c->stream);
  cudaMemsetAsync(c->Ec, 0, (size_t)nc_pad * sizeof(float), c->stream);
  if ((rc = sync_and_check(c, "coarse set-up upload"))) return rc;
  c->coarse_mask_gen = c->mask_gen;
  c->coarse_built_target = target_nc;
  c->coarse_geo_gen = 0;   // values follow
  return 0;
}

// ---------------------------------------------------------------------------
// host: values (A_c and its inverse)
// ---------------------------------------------------------------------------
template <int ET>
static void launch_coarse_elem(Ctx* c) {
  const unsigned g = (unsigned)std::max<int64_t>(1, std::min<int64_t>((c->n_celem + 1) / 2, 152LL * 64));
  k_coarse_elem<ET><<<g, 64, 0, c->stream>>>(c->n_celem, c->celem, c->celem_aggs, c->celem_off, c->E, c->conn,
                                             c->mask, c->node_agg, c->node_ddf, c->geo64, c->geo_affine ? 1 : 0,
                                             c->contrib);
}

// A_c (not inverted) into c->Ac
static int coarse_assemble(Ctx* c) {
  if (c->n_celem > 0) {
    switch (c->et) {
      case JFEM_TET4: launch_coarse_elem<JFEM_TET4>(c); break;
      case JFEM_TET10: launch_coarse_elem<JFEM_TET10>(c); break;
      default: launch_coarse_elem<JFEM_HEX8>(c); break;
    }
    c->launches += 1;
  }
  cudaMemsetAsync(c->Ac, 0, (size_t)c->nc_pad * c->nc_pad * sizeof(float2), c->stream);
  if (c->n_cblk > 0) {
    k_coarse_reduce<<<grid_for(c->n_cblk * 36, 256), 256, 0, c->stream>>>(c->n_cblk, c->cblk_ab, c->cblk_ptr,
                                                                          c->cblk_src, c->contrib, c->nc_pad, c->Ac);
    c->launches += 1;
  }
  return 0;
}

// A_c is always the coarse projection of the small-strain stiffness (λ, μ of
// the material records, reference configuration); for finite strain it is the
// coarse level of the tangent systems' preconditioner, an SPD approximation of
// the tangent's own coarse operator (flexible CG needs no more).
static int coarse_values(Ctx* c) {
  int rc = geometry_prepare(c);
  if (rc) return rc;
  cudaEventRecord(c->ev0, c->stream);
  coarse_assemble(c);
  const int n = c->nc_pad, nbk = n / GJ_B;
  k_diag_copy<<<grid_for(n, 256), 256, 0, c->stream>>>(n, n, c->Ac, c->Ac_diag);
  c->launches += 1;
  float2* P = c->gj_buf;
  float2* Brow = P + GJ_B * GJ_B;
  float2* Ccol = Brow + (size_t)GJ_B * n;
  for (int kb = 0; kb < nbk; ++kb) {
    k_gj_pivot<<<1, dim3(GJ_B, GJ_B), 0, c->stream>>>(c->Ac, n, kb * GJ_B, c->Ac_diag, P);
    k_gj_panel<<<nbk, 256, 0, c->stream>>>(c->Ac, n, kb, P, Brow, Ccol);
    k_gj_update<<<dim3(nbk, nbk), 256, 0, c->stream>>>(c->Ac, n, kb, P, Brow, Ccol);
    c->launches += 3;
  }
  k_round_f32<<<grid_for((int64_t)n * n, 256), 256, 0, c->stream>>>((int64_t)n * n, c->Ac, c->Ainv32);
  c->launches += 1;
  cudaEventRecord(c->ev1, c->stream);
  if ((rc = sync_and_check(c, "coarse matrix"))) return rc;
  float ms = 0.f;
  cudaEventElapsedTime(&ms, c->ev0, c->ev1);
  c->coarse_setup_ms = ms;
  c->coarse_geo_gen = c->geo_gen;
  return 0;
}

static int coarse_target_dofs(const Ctx* c) {
  return c->coarse_target > 0 ? c->coarse_target : auto_coarse_dofs(3 * c->N);
}

int coarse_prepare(Ctx* c) {
  if (c->N == 0) return set_err(c, JFEM_ERR_INVALID, "jfem_set_mesh must come first");
  int rc = geometry_prepare(c);
  if (rc) return rc;
  const int target = coarse_target_dofs(c);
  if (!c->node_agg || c->coarse_mask_gen != c->mask_gen || c->coarse_built_target != target) {
    if ((rc = coarse_build(c, target))) return rc;
  }
  if (c->coarse_geo_gen != c->geo_gen) {
    if ((rc = coarse_values(c))) return rc;
  }
  return 0;
}

int coarse_gemv_blocks(const Ctx* c) { return (c->nc + 7) / 8; }

void enqueue_coarse_restrict_solve(Ctx* c, const float2* r, const int* stop, const float* qold, double* t2part,
                                   SolverScalars* sc, const double* t1, int n1) {
  k_coarse_restrict<<<c->n_chunks, 256, 0, c->stream>>>(c->n_chunks, c->chunk_begin, c->agg_nodes, c->node_d32, r,
                                                        t2part ? qold : nullptr, stop, c->chunk_agg,
                                                        c->agg_chunk_ptr, c->agg_cnt, c->nc_pad, c->cpart, c->RQ);
  k_coarse_gemv<<<coarse_gemv_blocks(c), 256, 0, c->stream>>>(c->nc, c->nc_pad, c->Ainv32, c->RQ, stop, c->Ec,
                                                              t2part, sc, t1, n1);
  c->launches += 2;
}

int coarse_info(Ctx* c, int* n_agg, int* n_coarse, int64_t* n_elem_listed, double* setup_ms) {
  int rc = coarse_prepare(c);
  if (rc) return rc;
  if (n_agg) *n_agg = c->nagg;
  if (n_coarse) *n_coarse = c->nc;
  if (n_elem_listed) *n_elem_listed = c->n_celem;
  if (setup_ms) *setup_ms = c->coarse_setup_ms;
  return 0;
}

int coarse_matrix(Ctx* c, double* Ac_h, int* node_agg_h) {
  int rc = coarse_prepare(c);
  if (rc) return rc;
  if (node_agg_h) cudaMemcpyAsync(node_agg_h, c->node_agg, c->N * sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  std::vector<float2> tmp;
  if (Ac_h) {
    coarse_assemble(c);   // overwrites the inverse: recomputed by the next coarse_prepare
    c->coarse_geo_gen = 0;
    tmp.resize((size_t)c->nc * c->nc);
    cudaMemcpy2DAsync(tmp.data(), (size_t)c->nc * sizeof(float2), c->Ac, (size_t)c->nc_pad * sizeof(float2),
                      (size_t)c->nc * sizeof(float2), (size_t)c->nc, cudaMemcpyDeviceToHost, c->stream);
  }
  const int rc2 = sync_and_check(c, "coarse matrix download");
  if (rc2) return rc2;
  for (size_t k = 0; k < tmp.size(); ++k) Ac_h[k] = df_to_double(tmp[k]);
  return 0;
}

int coarse_precondition(Ctx* c, const double* r_h, double* z_h) {
  int rc = coarse_prepare(c);
  if (rc) return rc;
  if ((rc = jacobi_diag_device(c, c->dinv))) return rc;
  const int64_t n3 = 3 * c->N;
  cudaMemcpyAsync(c->tmp, r_h, n3 * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  k_to_df<<<grid_for(n3, 256), 256, 0, c->stream>>>(n3, c->tmp, c->rd);
  enqueue_coarse_restrict_solve(c, c->rd, nullptr);
  k_coarse_jacobi_out<<<grid_for(n3, 256), 256, 0, c->stream>>>(c->N, c->tmp, c->dinv, c->mask, c->node_agg,
                                                                 c->node_d32, c->Ec, c->tmp2);
  c->launches += 2;
  cudaMemcpyAsync(z_h, c->tmp2, n3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  return sync_and_check(c, "two-level preconditioner");
}

}  // namespace jfem
