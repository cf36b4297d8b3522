// jfem_apply_kernels.cuh — element kernels of the matrix-free apply (see
// jfem_apply.cu for the design); included by one translation unit per element
// type so the instantiations compile in parallel.
#pragma once
#include "jfem_common.cuh"
#include "jfem_df.cuh"

namespace jfem {

// KIN_NHC: Neo-Hookean tangent from the cached point state (F, C⁻¹, μ − λ ln J)
enum Kin { KIN_SMALL = 0, KIN_SVK = 1, KIN_NH = 2, KIN_NHC = 3 };
__host__ __device__ constexpr bool kin_needs_u(int kin) { return kin == KIN_SVK || kin == KIN_NH; }

// ---------------------------------------------------------------------------
// constitutive flux at one integration point
// ---------------------------------------------------------------------------
// Linear small strain: P = λ tr(ε) I + 2μ ε with ε = sym(∇v).
template <typename R>
__device__ __forceinline__ void flux_small(const R gv[3][3], R lam, R mu, R P[3][3]) {
  const R tr = gv[0][0] + gv[1][1] + gv[2][2];
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int d = 0; d < 3; ++d) P[c][d] = mu * (gv[c][d] + gv[d][c]) + (c == d ? lam * tr : R(0));
}

// Finite-strain tangent: δP = F δS + [geom] ∇v S, δE = sym(Fᵀ∇v).
// SVK: S = λ tr(E) I + 2μ E, δS = λ tr(δE) I + 2μ δE.
// Neo-Hookean: S = μ(I − C⁻¹) + λ lnJ C⁻¹, δS = λ tr(C⁻¹δE) C⁻¹ + 2(μ − λ lnJ) C⁻¹ δE C⁻¹.
// Returns false when det C ≤ 0.
template <typename R, int KIN, bool GEOM>
__device__ __forceinline__ bool flux_tangent(const R gu[3][3], const R gv[3][3], R lam, R mu, R P[3][3]) {
  R F[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) F[i][j] = gu[i][j] + (i == j ? R(1) : R(0));
  // C = FᵀF, δE = sym(Fᵀ ∇v)
  R C[3][3], dE[3][3], FtG[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      C[i][j] = F[0][i] * F[0][j] + F[1][i] * F[1][j] + F[2][i] * F[2][j];
      FtG[i][j] = F[0][i] * gv[0][j] + F[1][i] * gv[1][j] + F[2][i] * gv[2][j];
    }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) dE[i][j] = R(0.5) * (FtG[i][j] + FtG[j][i]);
  R S[3][3], dS[3][3];
  bool ok = true;
  if (KIN == KIN_SVK) {
    const R trE = R(0.5) * (C[0][0] + C[1][1] + C[2][2] - R(3));
    const R trdE = dE[0][0] + dE[1][1] + dE[2][2];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const R Eij = R(0.5) * (C[i][j] - (i == j ? R(1) : R(0)));
        S[i][j] = R(2) * mu * Eij + (i == j ? lam * trE : R(0));
        dS[i][j] = R(2) * mu * dE[i][j] + (i == j ? lam * trdE : R(0));
      }
  } else {
    const R detC = det3(C);
    ok = detC > R(0);
    R Ci[3][3];
    adj3(C, Ci);
    const R id = R(1) / detC;
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) Ci[i][j] *= id;
    const R lnJ = R(0.5) * log(detC);
    const R cc = mu - lam * lnJ;
    R CidE[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) CidE[i][j] = Ci[i][0] * dE[0][j] + Ci[i][1] * dE[1][j] + Ci[i][2] * dE[2][j];
    const R tr = CidE[0][0] + CidE[1][1] + CidE[2][2];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        S[i][j] = mu * ((i == j ? R(1) : R(0)) - Ci[i][j]) + lam * lnJ * Ci[i][j];
        const R CdC = CidE[i][0] * Ci[0][j] + CidE[i][1] * Ci[1][j] + CidE[i][2] * Ci[2][j];
        dS[i][j] = lam * tr * Ci[i][j] + R(2) * cc * CdC;
      }
  }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      R s = F[i][0] * dS[0][j] + F[i][1] * dS[1][j] + F[i][2] * dS[2][j];
      if (GEOM) s += gv[i][0] * S[0][j] + gv[i][1] * S[1][j] + gv[i][2] * S[2][j];
      P[i][j] = s;
    }
  return ok;
}

// Neo-Hookean tangent action from the cached state of point q (16 values per
// point: F row-major, C⁻¹ as 00 11 22 01 12 02, cc = μ − λ ln J; the same
// scaling as the record's λ, μ):  S = μ I − cc C⁻¹,
// δS = λ (C⁻¹:δE) C⁻¹ + 2 cc C⁻¹ δE C⁻¹,  δP = F δS (+ ∇v S with GEOM).
template <typename R, bool GEOM, class ST>
__device__ __forceinline__ void flux_tangent_cached(const ST& st, int q, const R gv[3][3], R lam, R mu,
                                                    R P[3][3]) {
  R F[3][3], Ci[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) F[i][j] = st(16 * q + 3 * i + j);
  Ci[0][0] = st(16 * q + 9);
  Ci[1][1] = st(16 * q + 10);
  Ci[2][2] = st(16 * q + 11);
  Ci[0][1] = Ci[1][0] = st(16 * q + 12);
  Ci[1][2] = Ci[2][1] = st(16 * q + 13);
  Ci[0][2] = Ci[2][0] = st(16 * q + 14);
  const R cc = st(16 * q + 15);
  R FtG[3][3], dE[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) FtG[i][j] = F[0][i] * gv[0][j] + F[1][i] * gv[1][j] + F[2][i] * gv[2][j];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) dE[i][j] = R(0.5) * (FtG[i][j] + FtG[j][i]);
  R CidE[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) CidE[i][j] = Ci[i][0] * dE[0][j] + Ci[i][1] * dE[1][j] + Ci[i][2] * dE[2][j];
  const R tr = CidE[0][0] + CidE[1][1] + CidE[2][2];
  R S[3][3], dS[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      S[i][j] = (i == j ? mu : R(0)) - cc * Ci[i][j];
      const R CdC = CidE[i][0] * Ci[0][j] + CidE[i][1] * Ci[1][j] + CidE[i][2] * Ci[2][j];
      dS[i][j] = lam * tr * Ci[i][j] + R(2) * cc * CdC;
    }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      R v = F[i][0] * dS[0][j] + F[i][1] * dS[1][j] + F[i][2] * dS[2][j];
      if (GEOM) v += gv[i][0] * S[0][j] + gv[i][1] * S[1][j] + gv[i][2] * S[2][j];
      P[i][j] = v;
    }
}

// First Piola stress P = F S at state u (finite) — internal force flux.
template <typename R, int KIN>
__device__ __forceinline__ bool flux_pk1(const R gu[3][3], R lam, R mu, R P[3][3]) {
  R F[3][3], C[3][3], S[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) F[i][j] = gu[i][j] + (i == j ? R(1) : R(0));
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) C[i][j] = F[0][i] * F[0][j] + F[1][i] * F[1][j] + F[2][i] * F[2][j];
  bool ok = true;
  if (KIN == KIN_SVK) {
    const R trE = R(0.5) * (C[0][0] + C[1][1] + C[2][2] - R(3));
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) S[i][j] = mu * (C[i][j] - (i == j ? R(1) : R(0))) + (i == j ? lam * trE : R(0));
  } else {
    const R detC = det3(C);
    ok = detC > R(0);
    R Ci[3][3];
    adj3(C, Ci);
    const R id = R(1) / detC;
    const R lnJ = R(0.5) * log(detC);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) S[i][j] = mu * ((i == j ? R(1) : R(0)) - Ci[i][j] * id) + lam * lnJ * Ci[i][j] * id;
  }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) P[i][j] = F[i][0] * S[0][j] + F[i][1] * S[1][j] + F[i][2] * S[2][j];
  return ok;
}

// ---------------------------------------------------------------------------
// reference derivatives used by the apply: for i ≥ 1 the constexpr table
// rounded to R; node 0 gets −Σ_{i≥1}, so the discrete gradient of a constant
// field is exactly zero in R arithmetic and the operator stays symmetric.
// ---------------------------------------------------------------------------
template <typename R>
__host__ __device__ constexpr R dnr(int et, int q, int i, int a) {
  if (i > 0) return (R)dshape(et, q, i, a);
  R s = R(0);
  const int nn = et == JFEM_TET4 ? 4 : et == JFEM_TET10 ? 10 : 8;
  for (int j = 1; j < nn; ++j) s += (R)dshape(et, q, j, a);
  return -s;
}

// Geometry record sources for element_op: record k of the element, either read
// from the SoA array in HBM or from values already loaded into registers.
template <typename R>
struct GeoGlobal {
  const R* p;
  int64_t stride;
  __device__ __forceinline__ R operator()(int k) const { return __ldg(p + (int64_t)k * stride); }
};
template <typename R>
struct GeoRegs {
  const R* r;
  __device__ __forceinline__ R operator()(int k) const { return r[k]; }
};

// ---------------------------------------------------------------------------
// Element operator from element-local differences.
//   dv[i] = v_i − v_0, du[i] = u_i − u_0 (i ≥ 1; index 0 unused).
//   geo: record source (GeoGlobal / GeoRegs), record k = geo(k).
//   MODE 0: y = K v (linear) / K_T(u) v (finite); MODE 1: y = f_int(u).
// Returns false when the material state is invalid (det C ≤ 0).
// ---------------------------------------------------------------------------
struct NoState {
  __device__ __forceinline__ float operator()(int) const { return 0.f; }
};

template <int ET, typename R, bool AFFINE, int KIN, bool GEOM, int MODE, class GEO, class ST = NoState>
__device__ __forceinline__ bool element_op(const R (&dv)[Elem<ET>::NN][3], const R (&du)[Elem<ET>::NN][3],
                                           const GEO& geo, R (&y)[Elem<ET>::NN][3], const ST& st = ST()) {
  constexpr int NN = Elem<ET>::NN, NQ = Elem<ET>::NQ;
  constexpr bool NEED_U = kin_needs_u(KIN);
  constexpr bool NEED_V = (MODE == 0);
#pragma unroll
  for (int i = 0; i < NN; ++i) y[i][0] = y[i][1] = y[i][2] = R(0);
  R iJ[9], lam, mu, det = R(1);
  if (AFFINE) {
#pragma unroll
    for (int k = 0; k < 9; ++k) iJ[k] = geo(k);
    lam = geo(9);
    mu = geo(10);
  } else {
    lam = geo(10 * NQ);
    mu = geo(10 * NQ + 1);
  }
  bool ok = true;
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    if (!AFFINE) {
#pragma unroll
      for (int k = 0; k < 9; ++k) iJ[k] = geo(10 * q + k);
      det = geo(10 * q + 9);
    }
    R gv[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, gu[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    if (NEED_V) {
      R G[3][3];
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          R s = R(0);
#pragma unroll
          for (int i = 1; i < NN; ++i) {
            const R dn = dnr<R>(ET, q, i, a);
            if (dn != R(0)) s += dv[i][c] * dn;
          }
          G[c][a] = s;
        }
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int d = 0; d < 3; ++d) gv[c][d] = G[c][0] * iJ[3 * d] + G[c][1] * iJ[3 * d + 1] + G[c][2] * iJ[3 * d + 2];
    }
    if (NEED_U) {
      R G[3][3];
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          R s = R(0);
#pragma unroll
          for (int i = 1; i < NN; ++i) {
            const R dn = dnr<R>(ET, q, i, a);
            if (dn != R(0)) s += du[i][c] * dn;
          }
          G[c][a] = s;
        }
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int d = 0; d < 3; ++d) gu[c][d] = G[c][0] * iJ[3 * d] + G[c][1] * iJ[3 * d + 1] + G[c][2] * iJ[3 * d + 2];
    }
    R P[3][3];
    if (MODE == 1) {
      ok &= flux_pk1<R, KIN>(gu, lam, mu, P);
    } else if (KIN == KIN_SMALL) {
      flux_small<R>(gv, lam, mu, P);
    } else if (KIN == KIN_NHC) {
      flux_tangent_cached<R, GEOM>(st, q, gv, lam, mu, P);
    } else {
      ok &= flux_tangent<R, KIN, GEOM>(gu, gv, lam, mu, P);
    }
    // Q[c][a] = w·detJ Σ_d P[c][d] J⁻¹[d][a]   (affine records carry detJ inside λ, μ)
    const R wq = (R)qp_weight(ET, q) * det;
    R Q[3][3];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int a = 0; a < 3; ++a) Q[c][a] = wq * (P[c][0] * iJ[a] + P[c][1] * iJ[3 + a] + P[c][2] * iJ[6 + a]);
#pragma unroll
    for (int i = 0; i < NN; ++i)
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const R dn = dnr<R>(ET, q, i, a);
        if (dn != R(0)) {
          y[i][0] += Q[0][a] * dn;
          y[i][1] += Q[1][a] * dn;
          y[i][2] += Q[2][a] * dn;
        }
      }
  }
  return ok;
}

// ---------------------------------------------------------------------------
// two-phase apply, phase 1: one thread per element, element vectors to HBM
//   SPLIT:  v given as FP32 (hi, lo) pairs per DOF (v ≈ hi + lo).  Gradients
//           use element-local differences v_i − v_0 = (hi_i − hi_0) + (lo_i − lo_0):
//           for a smooth field the hi difference is exact (Sterbenz), so ∇v
//           keeps FP32 accuracy relative to ∇v itself instead of losing
//           |v|/(h|∇v|) — the cancellation that otherwise limits how far an
//           FP32 operator can drive the FP64 residual.
// ---------------------------------------------------------------------------
template <int ET, typename R, bool AFFINE, int KIN, bool GEOM, int MODE, bool SPLIT>
__global__ void __launch_bounds__(128) k_apply_elem(int64_t E, const int* __restrict__ conn,
                                                    const R* __restrict__ geo, const double* __restrict__ v,
                                                    const float2* __restrict__ v2,
                                                    const double* __restrict__ u,
                                                    const uint8_t* __restrict__ mask, R* __restrict__ ye,
                                                    int* err, const int* __restrict__ stop,
                                                    int mask_in) {
  constexpr int NN = Elem<ET>::NN;
  if (stop && *stop) return;
  constexpr bool NEED_U = kin_needs_u(KIN);
  constexpr bool NEED_V = (MODE == 0);
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
    int nodes[NN];
#pragma unroll
    for (int i = 0; i < NN; ++i) nodes[i] = __ldg(conn + (int64_t)i * E + e);
    R dv[NN][3], du[NN][3];
    R h0[3] = {0, 0, 0}, l0[3] = {0, 0, 0}, u0[3] = {0, 0, 0};
#pragma unroll
    for (int i = 0; i < NN; ++i) {
      const int64_t n = nodes[i];
      uint8_t m = 0;
      if (NEED_V && mask_in) m = __ldg(mask + n);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        if (NEED_V) {
          R hi, lo = R(0);
          if (SPLIT) {
            const float2 t = __ldg(v2 + 3 * n + c);
            hi = t.x;
            lo = t.y;
          } else {
            hi = (R)__ldg(v + 3 * n + c);
          }
          if ((m >> c) & 1) { hi = R(0); lo = R(0); }
          if (i == 0) { h0[c] = hi; l0[c] = lo; }
          else dv[i][c] = SPLIT ? (hi - h0[c]) + (lo - l0[c]) : hi - h0[c];
        }
        if (NEED_U) {
          const R uv = (R)__ldg(u + 3 * n + c);
          if (i == 0) u0[c] = uv;
          else du[i][c] = uv - u0[c];
        }
      }
    }
    R y[NN][3];
    const bool ok = element_op<ET, R, AFFINE, KIN, GEOM, MODE>(dv, du, GeoGlobal<R>{geo + e, E}, y);
    if (!ok) raise_error(err, JFEM_ERR_NAN);
#pragma unroll
    for (int i = 0; i < NN; ++i)
#pragma unroll
      for (int c = 0; c < 3; ++c) ye[(int64_t)(3 * i + c) * E + e] = y[i][c];
  }
}

// ---------------------------------------------------------------------------
// tiled FP32 apply (see jfem_tiles.cu).  One CTA of JFEM_TILE threads per tile
// (persistent over tiles); dynamic shared memory, in this order:
//   yxy  [NN][T]     float2 x, y components of the element vectors of the tile
//   yz   [NN][T]     f32    their z components
//     (before the element pass the same bytes hold the staged element data:
//      sconn [NN][T] u16 local connectivity, srec [11][T] f32 affine records)
//   sadj [T·NN]      u16    the tile's node → slot (local node · T + element) lists
//   sptr [Lmax+1]    u16    end offsets into sadj (bits 0-12) and the node's
//                           Dirichlet mask (bits 13-15; entry j+1 is node j's)
//   vs   [3·Lmax]    float2 (hi, lo) of the tile's nodes (masked DOFs zero)
//   us   [3·Lmax]    f32    state u of the tile's nodes (finite strain only)
//   stout [Lmax]     i32    output word of each local node (tout)
// The loads of one tile are issued in two waves, so a tile waits for about
// three global-memory latencies instead of one per node round:
//   header   n0, L                                   (tnode_ptr)
//   (nodes are staged in ascending global order — tnodes, coalesced — into
//    their local slots tloc; the local order, by element slots descending,
//    gives the gather's warps nodes of similar loop length)
//   wave 1   bulk async copies (cp.async.bulk, one mbarrier, issued by the
//            lanes of warp 0): the adjacency block, the NN connectivity rows
//            and the 11 affine record rows of the tile (all 16-byte aligned:
//            rows of T elements of a tile-padded [k][Epad] array);
//            per node: global index, local slot
//   wave 2   per node (depends on wave 1): adjacency end offset, mask byte,
//            v (hi, lo) and u
// The node gather then reads each node's output word (tout, staged with the
// node: the global node when interior, −1 − slot when shared), sums its element slots from shared
// memory and writes y (interior) or bpart[slot] (shared).  Optional v·y
// partial over interior nodes (double-float, v = hi + lo as staged) into
// part[blockIdx.x] (FP64).
// ---------------------------------------------------------------------------
__host__ __device__ constexpr int tile_sptr_len(int Lmax) { return (Lmax + 8) & ~7; }

// bytes of the element-vector region (also holds the staged element data)
template <int NN, bool AFFINE>
__host__ __device__ constexpr size_t tile_elem_region_bytes() {
  constexpr size_t yb = (size_t)NN * JFEM_TILE * (sizeof(float2) + sizeof(float));
  constexpr size_t sb = (size_t)NN * JFEM_TILE * sizeof(uint16_t) + (AFFINE ? (size_t)11 * JFEM_TILE * sizeof(float) : 0);
  return ((yb > sb ? yb : sb) + 15) & ~(size_t)15;
}

template <int NN, bool NEED_U, bool AFFINE>
__host__ __device__ constexpr size_t tile_smem_bytes(int Lmax) {
  return tile_elem_region_bytes<NN, AFFINE>() + (size_t)JFEM_TILE * NN * sizeof(uint16_t) +
         (size_t)tile_sptr_len(Lmax) * sizeof(uint16_t) + (size_t)3 * Lmax * sizeof(float2) +
         (NEED_U ? (size_t)3 * Lmax * sizeof(float) : 0) + (size_t)Lmax * sizeof(int);
}

// node rounds per thread covered by the unrolled waves (tiles of JFEM_TILE
// Morton-ordered elements hold ≈ 0.4, 1.3 and 2.6 nodes per element for Tet4,
// Hex8 and Tet10); nodes beyond are staged by a plain loop
template <int ET>
__host__ __device__ constexpr int tile_node_rounds() {
  return ET == JFEM_TET4 ? 1 : ET == JFEM_HEX8 ? 2 : 3;
}
constexpr int TILE_PTR_BITS = 13;   // sadj offsets < 2^13 (T·NN ≤ 2560)
static_assert(JFEM_TILE * 10 < (1 << TILE_PTR_BITS), "tile adjacency offsets must fit 13 bits");

template <int ET, bool AFFINE, int KIN, bool GEOM>
__global__ void __launch_bounds__(JFEM_TILE, KIN == KIN_SMALL ? JFEM_TILE_CTAS : (KIN == KIN_NHC ? 2 : 1)) k_tile_apply(
    int64_t ntiles, int64_t E, int64_t Epad, const int* __restrict__ tnode_ptr, const int* __restrict__ tnodes,
    const uint16_t* __restrict__ tloc, const uint16_t* __restrict__ tconn, const float* __restrict__ geo, const uint16_t* __restrict__ tadj_ptr,
    const uint16_t* __restrict__ tadj, const int* __restrict__ tout,
    const float2* __restrict__ v2, const double* __restrict__ u,
    const uint8_t* __restrict__ mask, int masked, int Lmax, float* __restrict__ y, float4* __restrict__ bpart,
    double* __restrict__ part, const float* __restrict__ nhs, int* err, const int* __restrict__ stop) {
  constexpr int NN = Elem<ET>::NN;
  constexpr int T = JFEM_TILE;
  constexpr int NADJ = T * NN;   // adjacency entries per tile; NADJ·2 bytes is a multiple of 16
  constexpr int NR = tile_node_rounds<ET>();
  constexpr unsigned PMASK = (1u << TILE_PTR_BITS) - 1;
  constexpr bool NEED_U = kin_needs_u(KIN);
  constexpr int NCOPY = 1 + NN + (AFFINE ? 11 : 0);   // bulk copies per tile
  constexpr unsigned TILE_BYTES = (unsigned)((NADJ + NN * T) * sizeof(uint16_t) + (AFFINE ? 11 * T * sizeof(float) : 0));
  static_assert(NCOPY <= 32, "one bulk copy per lane of warp 0");
  static_assert((T * sizeof(uint16_t)) % 16 == 0 && (T * sizeof(float)) % 16 == 0, "bulk copy rows: 16-byte multiples");
  static_assert((NN * T * sizeof(uint16_t)) % 16 == 0, "srec must start 16-byte aligned");
  extern __shared__ float4 smem_f4[];
  float2* yxy = reinterpret_cast<float2*>(smem_f4);
  float* yz = reinterpret_cast<float*>(yxy + NN * T);
  uint16_t* sconn = reinterpret_cast<uint16_t*>(smem_f4);
  float* srec = reinterpret_cast<float*>(sconn + NN * T);
  uint16_t* sadj = reinterpret_cast<uint16_t*>(reinterpret_cast<char*>(smem_f4) + tile_elem_region_bytes<NN, AFFINE>());
  uint16_t* sptr = sadj + NADJ;
  float2* vs = reinterpret_cast<float2*>(sptr + tile_sptr_len(Lmax));
  float* us = reinterpret_cast<float*>(vs + 3 * Lmax);
  int* stout = reinterpret_cast<int*>(us + (NEED_U ? 3 * Lmax : 0));   // output word per local node
  __shared__ double sh[32];
  __shared__ uint64_t tile_bar;
  if (stop && *stop) return;
  const int tid = threadIdx.x;
  if (tid == 0) mbar_init(&tile_bar, 1);
  __syncthreads();
  float2 dot = make_float2(0.f, 0.f);
  bool ok = true;
  unsigned phase = 0;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x, phase ^= 1u) {
    if (tid < 32) {   // wave 1, bulk part (the previous tile's readers passed the loop-end barrier)
      if (tid == 0) mbar_expect_tx(&tile_bar, TILE_BYTES);
      __syncwarp();
      if (tid < NCOPY) {
        fence_proxy_async_smem();
        if (tid == 0) {
          bulk_copy_g2s(sadj, tadj + t * (int64_t)NADJ, NADJ * sizeof(uint16_t), &tile_bar);
        } else if (tid <= NN) {
          const int a = tid - 1;
          bulk_copy_g2s(sconn + a * T, tconn + (int64_t)a * Epad + t * T, T * sizeof(uint16_t), &tile_bar);
        } else {
          const int k = tid - 1 - NN;
          bulk_copy_g2s(srec + k * T, geo + (int64_t)k * Epad + t * T, T * sizeof(float), &tile_bar);
        }
      }
    }
    const int n0 = __ldg(tnode_ptr + t);
    const int L = __ldg(tnode_ptr + t + 1) - n0;
    const int64_t e = t * T + tid;
    const bool valid = e < E;
    {   // node staging in ascending global order (coalesced), each node written
        // to its local slot jl (the gather order); wave 1: global index, slot
      int gn[NR], jl[NR];
#pragma unroll
      for (int r = 0; r < NR; ++r) {
        const int k = tid + r * T;
        gn[r] = 0;
        jl[r] = 0;
        if (k < L) {
          gn[r] = __ldg(tnodes + n0 + k);
          jl[r] = __ldg(tloc + n0 + k);
        }
      }
      // wave 2: adjacency end offset, output word, mask, v (hi, lo), u
      unsigned mk[NR], pe[NR];
      int ow[NR];
      float2 h[NR][3];
      float uu[NR][3];
#pragma unroll
      for (int r = 0; r < NR; ++r) {
        const int k = tid + r * T;
        mk[r] = 0;
        pe[r] = 0;
        ow[r] = 0;
        if (k < L) {
          const int64_t g = gn[r];
          pe[r] = __ldg(tadj_ptr + n0 + t + jl[r] + 1);
          ow[r] = __ldg(tout + n0 + jl[r]);
          mk[r] = masked ? (unsigned)__ldg(mask + g) : 0u;
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            h[r][c] = __ldg(v2 + 3 * g + c);
            if (NEED_U) uu[r][c] = (float)__ldg(u + 3 * g + c);
          }
        }
      }
#pragma unroll
      for (int r = 0; r < NR; ++r) {
        const int k = tid + r * T;
        if (k < L) {
          const int j = jl[r];
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            vs[3 * j + c] = ((mk[r] >> c) & 1) ? make_float2(0.f, 0.f) : h[r][c];
            if (NEED_U) us[3 * j + c] = uu[r][c];
          }
          sptr[j + 1] = (uint16_t)(pe[r] | (mk[r] << TILE_PTR_BITS));
          stout[j] = ow[r];
        }
      }
      if (tid == 0) sptr[0] = 0;
      for (int k = tid + NR * T; k < L; k += T) {   // tiles with more nodes than the unrolled rounds
        const int64_t g = __ldg(tnodes + n0 + k);
        const int j = __ldg(tloc + n0 + k);
        const unsigned m = masked ? (unsigned)__ldg(mask + g) : 0u;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const float2 hv = __ldg(v2 + 3 * g + c);
          vs[3 * j + c] = ((m >> c) & 1) ? make_float2(0.f, 0.f) : hv;
          if (NEED_U) us[3 * j + c] = (float)__ldg(u + 3 * g + c);
        }
        sptr[j + 1] = (uint16_t)(__ldg(tadj_ptr + n0 + t + j + 1) | (m << TILE_PTR_BITS));
        stout[j] = __ldg(tout + n0 + j);
      }
    }
    const bool have_tile = mbar_wait_bounded(&tile_bar, phase, err);
    if (__syncthreads_or(!have_tile)) break;   // a bulk copy never completed: error raised, stop
    int li[NN];
    float rec[11];
    if (valid) {
#pragma unroll
      for (int a = 0; a < NN; ++a) li[a] = sconn[a * T + tid];
      if constexpr (AFFINE) {
#pragma unroll
        for (int k = 0; k < 11; ++k) rec[k] = srec[k * T + tid];
      }
    }
    __syncthreads();   // the element vectors below overwrite the staged element data
    if (valid) {
      float dv[NN][3], du[NN][3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float2 h0 = vs[3 * li[0] + c];
        const float u0 = NEED_U ? us[3 * li[0] + c] : 0.f;
#pragma unroll
        for (int i = 1; i < NN; ++i) {
          const float2 h = vs[3 * li[i] + c];
          dv[i][c] = (h.x - h0.x) + (h.y - h0.y);
          if (NEED_U) du[i][c] = us[3 * li[i] + c] - u0;
        }
      }
      float yl[NN][3];
      if constexpr (KIN == KIN_NHC) {   // point state cached in tile order: [16·n_q][Epad]
        const GeoGlobal<float> st{nhs + e, Epad};
        if constexpr (AFFINE) ok &= element_op<ET, float, true, KIN, GEOM, 0>(dv, du, GeoRegs<float>{rec}, yl, st);
        else ok &= element_op<ET, float, false, KIN, GEOM, 0>(dv, du, GeoGlobal<float>{geo + e, Epad}, yl, st);
      } else if constexpr (AFFINE) {
        ok &= element_op<ET, float, true, KIN, GEOM, 0>(dv, du, GeoRegs<float>{rec}, yl);
      } else {
        ok &= element_op<ET, float, false, KIN, GEOM, 0>(dv, du, GeoGlobal<float>{geo + e, Epad}, yl);
      }
#pragma unroll
      for (int a = 0; a < NN; ++a) {
        yxy[a * T + tid] = make_float2(yl[a][0], yl[a][1]);
        yz[a * T + tid] = yl[a][2];
      }
    }
    __syncthreads();
    {   // node gather: four slots per step (their indices, then their element
        // vectors, then the adds in slot order: the sum's order is unchanged)
      auto gather = [&](int j, int o) {
        const unsigned w1 = sptr[j + 1];
        const int k1 = (int)(w1 & PMASK);
        float s0 = 0.f, s1 = 0.f, s2 = 0.f;
        int k = (int)(sptr[j] & PMASK);
        for (; k + 4 <= k1; k += 4) {
          int sl[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) sl[u] = sadj[k + u];
          float2 q[4];
          float z[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            q[u] = yxy[sl[u]];
            z[u] = yz[sl[u]];
          }
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            s0 += q[u].x;
            s1 += q[u].y;
            s2 += z[u];
          }
        }
        for (; k < k1; ++k) {
          const int sl = sadj[k];
          const float2 q = yxy[sl];
          s0 += q.x;
          s1 += q.y;
          s2 += yz[sl];
        }
        if (o >= 0) {
          const unsigned m = w1 >> TILE_PTR_BITS;
          if (m & 1) s0 = 0.f;
          if (m & 2) s1 = 0.f;
          if (m & 4) s2 = 0.f;
          const int64_t g = o;
          y[3 * g] = s0;
          y[3 * g + 1] = s1;
          y[3 * g + 2] = s2;
          if (part) {   // v·y in double-float from the staged (masked) v
            dot = df_add_abs(dot, df_add_abs(df_dot_term(vs[3 * j], s0),
                                             df_add_abs(df_dot_term(vs[3 * j + 1], s1), df_dot_term(vs[3 * j + 2], s2))));
          }
        } else {   // shared node: partial sum; the boundary pass applies the mask
          bpart[-1 - o] = make_float4(s0, s1, s2, 0.f);
        }
      };
#pragma unroll
      for (int r = 0; r < NR; ++r) {
        const int j = tid + r * T;
        if (j < L) gather(j, stout[j]);
      }
      for (int j = tid + NR * T; j < L; j += T) gather(j, stout[j]);
    }
    __syncthreads();
  }
  if (!ok) raise_error(err, JFEM_ERR_NAN);
  if (part) {
    const double b = block_sum_df(dot, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = b;
  }
}

// ---------------------------------------------------------------------------
// launch helpers, instantiated once per element type (jfem_apply_<type>.cu)
// ---------------------------------------------------------------------------
template <int ET, typename R, bool AFFINE, int KIN, bool GEOM, int MODE>
static void launch_elem(Ctx* c, const R* geo, const double* v, const float2* v2, R* ye, const int* stop,
                        bool mask_in) {
  const unsigned g = grid_for(c->E, 128, 1LL << 30);
  if (v2 && MODE == 0)
    k_apply_elem<ET, R, AFFINE, KIN, GEOM, MODE, true><<<g, 128, 0, c->stream>>>(
        c->E, c->conn, geo, v, v2, c->u_state, c->mask, ye, c->d_err, stop, mask_in ? 1 : 0);
  else
    k_apply_elem<ET, R, AFFINE, KIN, GEOM, MODE, false><<<g, 128, 0, c->stream>>>(
        c->E, c->conn, geo, v, nullptr, c->u_state, c->mask, ye, c->d_err, stop, mask_in ? 1 : 0);
  c->launches += 1;
}

template <int ET, typename R, bool AFFINE, int MODE>
static void dispatch_kin(Ctx* c, const R* geo, const double* v, const float2* v2, R* ye, bool mask_in,
                         const int* stop) {
  const int kin = (!c->finite && MODE == 0) ? KIN_SMALL : (c->model == JFEM_NEO_HOOKEAN ? KIN_NH : KIN_SVK);
  if (MODE == 0 && kin == KIN_SMALL) {
    launch_elem<ET, R, AFFINE, KIN_SMALL, false, 0>(c, geo, v, v2, ye, stop, mask_in);
  } else if (kin == KIN_SVK) {
    if (MODE == 1) launch_elem<ET, R, AFFINE, KIN_SVK, false, 1>(c, geo, v, nullptr, ye, stop, false);
    else if (c->geom) launch_elem<ET, R, AFFINE, KIN_SVK, true, 0>(c, geo, v, v2, ye, stop, mask_in);
    else launch_elem<ET, R, AFFINE, KIN_SVK, false, 0>(c, geo, v, v2, ye, stop, mask_in);
  } else if (kin == KIN_NH) {
    if (MODE == 1) launch_elem<ET, R, AFFINE, KIN_NH, false, 1>(c, geo, v, nullptr, ye, stop, false);
    else if (c->geom) launch_elem<ET, R, AFFINE, KIN_NH, true, 0>(c, geo, v, v2, ye, stop, mask_in);
    else launch_elem<ET, R, AFFINE, KIN_NH, false, 0>(c, geo, v, v2, ye, stop, mask_in);
  }
}

template <int ET, bool AFFINE, int KIN, bool GEOM>
static void launch_tile_k(Ctx* c, const float2* v2, float* y, bool masked, double* part, const int* stop) {
  constexpr int NN = Elem<ET>::NN;
  const size_t sm = tile_smem_bytes<NN, kin_needs_u(KIN), AFFINE>(c->tile_Lmax);
  auto kern = k_tile_apply<ET, AFFINE, KIN, GEOM>;
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  const unsigned g = JFEM_RED_BLOCKS;   // CTAs take tiles b, b + g, …
  kern<<<g, JFEM_TILE, sm, c->stream>>>(
      c->ntiles, c->E, c->Epad, c->tnode_ptr, c->tnodes, c->tloc, c->tconn, c->geoT32, c->tadj_ptr, c->tadj, c->tout,
      v2, c->u_state, c->mask, masked ? 1 : 0, c->tile_Lmax, y, c->bpart, part, c->nhstate, c->d_err, stop);
  c->launches += 1;
}

// Tiled FP32 element + in-tile gather launch (the boundary sum is a separate kernel).
template <int ET>
void launch_tile_et(Ctx* c, const float2* v2, float* y, bool masked, double* part, const int* stop) {
  int kin = !c->finite ? KIN_SMALL : (c->model == JFEM_NEO_HOOKEAN ? KIN_NH : KIN_SVK);
  if (kin == KIN_NH && nh_cache_ready(c)) {
    if (c->geo_affine) {
      if (c->geom) launch_tile_k<ET, true, KIN_NHC, true>(c, v2, y, masked, part, stop);
      else launch_tile_k<ET, true, KIN_NHC, false>(c, v2, y, masked, part, stop);
    } else {
      if (c->geom) launch_tile_k<ET, false, KIN_NHC, true>(c, v2, y, masked, part, stop);
      else launch_tile_k<ET, false, KIN_NHC, false>(c, v2, y, masked, part, stop);
    }
    return;
  }
  if (c->geo_affine) {
    if (kin == KIN_SMALL) launch_tile_k<ET, true, KIN_SMALL, false>(c, v2, y, masked, part, stop);
    else if (kin == KIN_SVK) {
      if (c->geom) launch_tile_k<ET, true, KIN_SVK, true>(c, v2, y, masked, part, stop);
      else launch_tile_k<ET, true, KIN_SVK, false>(c, v2, y, masked, part, stop);
    } else {
      if (c->geom) launch_tile_k<ET, true, KIN_NH, true>(c, v2, y, masked, part, stop);
      else launch_tile_k<ET, true, KIN_NH, false>(c, v2, y, masked, part, stop);
    }
  } else {
    if (kin == KIN_SMALL) launch_tile_k<ET, false, KIN_SMALL, false>(c, v2, y, masked, part, stop);
    else if (kin == KIN_SVK) {
      if (c->geom) launch_tile_k<ET, false, KIN_SVK, true>(c, v2, y, masked, part, stop);
      else launch_tile_k<ET, false, KIN_SVK, false>(c, v2, y, masked, part, stop);
    } else {
      if (c->geom) launch_tile_k<ET, false, KIN_NH, true>(c, v2, y, masked, part, stop);
      else launch_tile_k<ET, false, KIN_NH, false>(c, v2, y, masked, part, stop);
    }
  }
}

// Neo-Hookean point state at u (tile order, one thread per tile position):
// ∇u from the FP32 state differences exactly as the tangent apply forms it,
// F = I + ∇u, C = FᵀF, C⁻¹, cc = μ − λ ln J with the record's λ, μ.
template <int ET, bool AFFINE>
__global__ void __launch_bounds__(128) k_nh_state(int64_t E, int64_t Epad, const int* __restrict__ perm,
                                                  const int* __restrict__ conn, const double* __restrict__ u,
                                                  const float* __restrict__ geo, float* __restrict__ st,
                                                  int* err) {
  constexpr int NN = Elem<ET>::NN, NQ = Elem<ET>::NQ;
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < E; p += (int64_t)gridDim.x * blockDim.x) {
    const int e = perm[p];   // positions below E hold elements
    float u0[3], du[NN][3];
    const int64_t g0 = conn[e];
#pragma unroll
    for (int c = 0; c < 3; ++c) u0[c] = (float)u[3 * g0 + c];
#pragma unroll
    for (int i = 1; i < NN; ++i) {
      const int64_t g = conn[(int64_t)i * E + e];
#pragma unroll
      for (int c = 0; c < 3; ++c) du[i][c] = (float)u[3 * g + c] - u0[c];
    }
    const GeoGlobal<float> rec{geo + p, Epad};
    float iJ[9], lam, mu;
    if (AFFINE) {
#pragma unroll
      for (int k = 0; k < 9; ++k) iJ[k] = rec(k);
      lam = rec(9);
      mu = rec(10);
    } else {
      lam = rec(10 * NQ);
      mu = rec(10 * NQ + 1);
    }
    bool ok = true;
#pragma unroll 1
    for (int q = 0; q < NQ; ++q) {
      if (!AFFINE) {
#pragma unroll
        for (int k = 0; k < 9; ++k) iJ[k] = rec(10 * q + k);
      }
      float G[3][3], F[3][3];
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          float s = 0.f;
#pragma unroll
          for (int i = 1; i < NN; ++i) {
            const float dn = dnr<float>(ET, q, i, a);
            if (dn != 0.f) s += du[i][c] * dn;
          }
          G[c][a] = s;
        }
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int d = 0; d < 3; ++d)
          F[c][d] = (G[c][0] * iJ[3 * d] + G[c][1] * iJ[3 * d + 1] + G[c][2] * iJ[3 * d + 2]) + (c == d ? 1.f : 0.f);
      float C[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) C[i][j] = F[0][i] * F[0][j] + F[1][i] * F[1][j] + F[2][i] * F[2][j];
      const float detC = det3(C);
      ok &= detC > 0.f;
      float Ci[3][3];
      adj3(C, Ci);
      const float id = 1.f / detC;
      const float lnJ = 0.5f * logf(detC);
      float* o = st + p;
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) o[(int64_t)(16 * q + 3 * i + j) * Epad] = F[i][j];
      o[(int64_t)(16 * q + 9) * Epad] = Ci[0][0] * id;
      o[(int64_t)(16 * q + 10) * Epad] = Ci[1][1] * id;
      o[(int64_t)(16 * q + 11) * Epad] = Ci[2][2] * id;
      o[(int64_t)(16 * q + 12) * Epad] = Ci[0][1] * id;
      o[(int64_t)(16 * q + 13) * Epad] = Ci[1][2] * id;
      o[(int64_t)(16 * q + 14) * Epad] = Ci[0][2] * id;
      o[(int64_t)(16 * q + 15) * Epad] = mu - lam * lnJ;
    }
    if (!ok) raise_error(err, JFEM_ERR_NAN);
  }
}

template <int ET>
void nh_state_et(Ctx* c) {
  const unsigned g = grid_for(c->E, 128);
  if (c->geo_affine)
    k_nh_state<ET, true><<<g, 128, 0, c->stream>>>(c->E, c->Epad, c->tperm, c->conn, c->u_state, c->geoT32,
                                                   c->nhstate, c->d_err);
  else
    k_nh_state<ET, false><<<g, 128, 0, c->stream>>>(c->E, c->Epad, c->tperm, c->conn, c->u_state, c->geoT32,
                                                    c->nhstate, c->d_err);
  c->launches += 1;
}

// FP32 element pass (mode 0 only).  v2: split copy of v, see k_apply_elem.
template <int ET>
void launch_apply_f32_et(Ctx* c, const double* v, const float2* v2, bool mask_in, const int* stop) {
  if (c->geo_affine) dispatch_kin<ET, float, true, 0>(c, c->geo32, v, v2, c->ye32, mask_in, stop);
  else dispatch_kin<ET, float, false, 0>(c, c->geo32, v, v2, c->ye32, mask_in, stop);
}

// FP64 element pass.  mode 0: y = K v (tangent for finite strain); mode 1: f_int(u).
template <int ET>
void launch_apply_f64_et(Ctx* c, int mode, const double* v, bool mask_in, const int* stop) {
  if (mode == 0) {
    if (c->geo_affine) dispatch_kin<ET, double, true, 0>(c, c->geo64, v, nullptr, c->ye64, mask_in, stop);
    else dispatch_kin<ET, double, false, 0>(c, c->geo64, v, nullptr, c->ye64, mask_in, stop);
  } else {
    if (c->geo_affine) dispatch_kin<ET, double, true, 1>(c, c->geo64, v, nullptr, c->ye64, false, stop);
    else dispatch_kin<ET, double, false, 1>(c, c->geo64, v, nullptr, c->ye64, false, stop);
  }
}

// Both passes in one translation unit (the cheap Tet4 instantiations).  The
// Tet10 and Hex8 passes are compiled in separate translation units
// (jfem_apply_<type>_f32.cu, jfem_apply_<type>_f64.cu) so the build runs them
// in parallel.
template <int ET>
void launch_apply_et(Ctx* c, bool fp32, int mode, const double* v, const float2* v2, bool mask_in,
                     const int* stop) {
  if (fp32) launch_apply_f32_et<ET>(c, v, v2, mask_in, stop);
  else launch_apply_f64_et<ET>(c, mode, v, mask_in, stop);
}

}  // namespace jfem
