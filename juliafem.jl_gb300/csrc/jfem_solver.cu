// jfem_solver.cu — Jacobi-PCG (FP64 vectors and dots, FP32 or FP64 apply, FP64
// true-residual "reliable updates" = iterative refinement) and inexact
// Newton–Krylov with load stepping for finite strain.
//
// Reference loops: CG of src/backend/cpu.jl:221-254 and
// ext/JuliaFEMCUDAExt.jl:531-577 (there with a device→host sync per dot and an
// allocation per operator call); Newton–Krylov with Eisenstat–Walker forcing
// ext/JuliaFEMCUDAExt.jl:685-854 (η = min(forcing_max, ‖R‖^forcing_power),
// :723-724,819-820); legacy Newton src/solvers.jl:575-620.
//
// Two device loops, both four launches per iteration:
//
// FP64 (precision JFEM_FP64): element apply, node gather (+ p·Ap partials),
// update 1 (x, r, z, r·z and r·r partials), update 2 (p and the scalars), all
// in double.  Scalars and the stop flag live in two slots selected by
// iteration parity: iteration k reads slot s and only block 0 of its last
// launch writes slot 1−s, so no launch reads what it writes.
//
// Mixed (JFEM_MIXED): GB300 runs FP64 at ~1/64 of its FP32 rate, so the
// recursion runs in double-float (jfem_df.cuh, 48-bit significand) on the FP32
// pipe, with x, r, p stored as float2 pairs in HBM: tiled FP32 apply of p
// (v·y partials in double-float), boundary pass whose last block forms
// α = r·z / p·Ap in FP64, update 1 (δx += αp, r −= αAp, r·z and r·r) whose
// last block forms β and the stop flag, update 2 (p = D⁻¹r + βp).  z is never
// stored.  x itself stays FP64: δx, the correction since the last refinement,
// is folded into it at every refinement.  The true residual f − K x, its norm
// and the stopping test stay FP64.
//
// Reductions are fixed-shape block partials summed in a fixed order, so every
// run gives bit-identical iterates.  Chunks of PCG_CHUNK (even) iterations are
// captured once into a CUDA graph; the host reads the scalars between chunks
// only.  After convergence every launch returns at entry, so overshoot inside a
// chunk costs nothing.
#include <chrono>
#include <cmath>

#include "jfem_common.cuh"
#include "jfem_df.cuh"

namespace jfem {

#define PCG_CHUNK 16
#define G_ JFEM_RED_BLOCKS
// part layout: [0,G) p·Ap, [G,2G) r·z, [2G,3G) r·r, [3G,4G) residual norms

__global__ void __launch_bounds__(JFEM_RED_THREADS) k_pcg_update1(int64_t n, const SolverScalars* __restrict__ sc,
                                                                  int slot, double* __restrict__ x,
                                                                  double* __restrict__ r, double* __restrict__ z,
                                                                  const double* __restrict__ p,
                                                                  const double* __restrict__ Ap,
                                                                  const double* __restrict__ dinv,
                                                                  double* __restrict__ part, int tiled) {
  __shared__ double sh[32];
  if (sc->done[slot]) return;
  // p·Ap partials: part[0..G) (+ part[3G..4G) from the tile-boundary kernel)
  const double pAp = reduce_partials(part, G_, sh) + (tiled ? reduce_partials(part + 3 * G_, G_, sh) : 0.0);
  const double alpha = sc->rz[slot] / pAp;
  double rz = 0.0, rr = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] += alpha * p[i];
    const double ri = r[i] - alpha * Ap[i];
    r[i] = ri;
    const double zi = dinv[i] * ri;
    z[i] = zi;
    rz += ri * zi;
    rr += ri * ri;
  }
  rz = block_sum(rz, sh);
  rr = block_sum(rr, sh);
  if (threadIdx.x == 0) {
    part[G_ + blockIdx.x] = rz;
    part[2 * G_ + blockIdx.x] = rr;
  }
}

__global__ void __launch_bounds__(JFEM_RED_THREADS) k_pcg_update2(int64_t n, SolverScalars* __restrict__ sc, int slot,
                                                                  double* __restrict__ p, const double* __restrict__ z,
                                                                  const double* __restrict__ part,
                                                                  float2* __restrict__ p2) {
  __shared__ double sh[32];
  const bool lead = blockIdx.x == 0 && threadIdx.x == 0;
  if (sc->done[slot]) {
    if (lead) {   // carry the final state into the other slot
      sc->done[1 - slot] = 1;
      sc->rz[1 - slot] = sc->rz[slot];
      sc->rr[1 - slot] = sc->rr[slot];
    }
    return;
  }
  const double rz_new = reduce_partials(part + G_, G_, sh);
  const double rr_new = reduce_partials(part + 2 * G_, G_, sh);
  const double beta = rz_new / sc->rz[slot];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double pi = z[i] + beta * p[i];
    p[i] = pi;
    if (p2) {   // FP32 (hi, lo) split for the FP32 apply
      const float hi = (float)pi;
      p2[i] = make_float2(hi, (float)(pi - (double)hi));
    }
  }
  if (lead) {
    const int it = sc->iters + 1;
    sc->iters = it;
    sc->rz[1 - slot] = rz_new;
    sc->rr[1 - slot] = rr_new;
    sc->done[1 - slot] = (rr_new <= sc->tol2 || it >= sc->max_iters || !(rr_new == rr_new)) ? 1 : 0;
  }
}

// r = (f − y) on free DOFs, 0 on prescribed (y may be null = 0); ‖r‖² partials
// → part[3G..4G); when fn2 is set also ‖y‖² over all DOFs → part[0..G).
// fn2 = 1: also ‖y‖² over all DOFs → part[0..G); fn2 = 2: also ‖r_new − r_old‖²
// (drift of the recursive residual) → part[0..G).
__global__ void __launch_bounds__(JFEM_RED_THREADS) k_residual(int64_t N, const double* __restrict__ f, double fs,
                                                               const double* __restrict__ y,
                                                               const uint8_t* __restrict__ mask,
                                                               double* __restrict__ r, int fn2,
                                                               double* __restrict__ part) {
  __shared__ double sh[32];
  double rr = 0.0, yy = 0.0;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < N; j += (int64_t)gridDim.x * blockDim.x) {
    const uint8_t m = mask[j];
    for (int c = 0; c < 3; ++c) {
      const double yv = y ? y[3 * j + c] : 0.0;
      const double v = ((m >> c) & 1) ? 0.0 : fs * f[3 * j + c] - yv;
      if (fn2 == 2) {
        const double d = v - r[3 * j + c];
        yy += d * d;
      } else {
        yy += yv * yv;
      }
      r[3 * j + c] = v;
      rr += v * v;
    }
  }
  rr = block_sum(rr, sh);
  if (threadIdx.x == 0) part[3 * G_ + blockIdx.x] = rr;
  if (fn2) {
    yy = block_sum(yy, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = yy;
  }
}

// z = dinv r (and p = z on restart); r·z → part[G..2G), r·r → part[2G..3G)
__global__ void __launch_bounds__(JFEM_RED_THREADS) k_precond(int64_t n, const double* __restrict__ r,
                                                              const double* __restrict__ dinv, double* __restrict__ z,
                                                              double* __restrict__ p, int restart,
                                                              double* __restrict__ part, float2* __restrict__ p2) {
  __shared__ double sh[32];
  double rz = 0.0, rr = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double ri = r[i];
    const double zi = dinv[i] * ri;
    z[i] = zi;
    if (restart) {
      p[i] = zi;
      if (p2) {
        const float hi = (float)zi;
        p2[i] = make_float2(hi, (float)(zi - (double)hi));
      }
    }
    rz += ri * zi;
    rr += ri * ri;
  }
  rz = block_sum(rz, sh);
  rr = block_sum(rr, sh);
  if (threadIdx.x == 0) {
    part[G_ + blockIdx.x] = rz;
    part[2 * G_ + blockIdx.x] = rr;
  }
}

// ---------------------------------------------------------------------------
// mixed solver (double-float vectors)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(JFEM_RED_THREADS) k_dfcg_update1(int64_t n, SolverScalars* __restrict__ sc,
                                                                   float2* __restrict__ x, float2* __restrict__ r,
                                                                   const float2* __restrict__ p,
                                                                   const float* __restrict__ Ap,
                                                                   const float* __restrict__ dinv,
                                                                   double* __restrict__ part) {
  __shared__ double sh[32];
  if (sc->done[0]) return;
  const float2 a = sc->alpha_df, na = df_neg(a);
  float2 rz = make_float2(0.f, 0.f), rr = make_float2(0.f, 0.f);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] = df_add_abs(x[i], df_mul(a, p[i]));
    const float2 ri = df_add(r[i], df_mul_f(na, Ap[i]));
    r[i] = ri;
    rz = df_add_abs(rz, df_mul(ri, df_mul_f(ri, dinv[i])));
    rr = df_add_abs(rr, df_mul(ri, ri));
  }
  const double2 zr = block_sum2_df(rz, rr, sh);
  if (threadIdx.x == 0) {
    part[G_ + blockIdx.x] = zr.x;
    part[2 * G_ + blockIdx.x] = zr.y;
  }
  if (arrive_last(&sc->arrive[1])) {
    const double2 t = reduce_partials2_cg(part + G_, part + 2 * G_, G_, sh);
    const double rz_new = t.x, rr_new = t.y;
    if (threadIdx.x == 0) {
      const double beta = rz_new / sc->rz[0];
      sc->beta = beta;
      sc->beta_df = df_from_double(beta);
      sc->rz[0] = rz_new;
      sc->rr[0] = rr_new;
      const int it = sc->iters + 1;
      sc->iters = it;
      sc->done[0] = (rr_new <= sc->tol2 || it >= sc->max_iters || !(rr_new == rr_new)) ? 1 : 0;
      sc->arrive[1] = 0;
    }
  }
}

__global__ void __launch_bounds__(JFEM_RED_THREADS) k_dfcg_update2(int64_t n, const SolverScalars* __restrict__ sc,
                                                                   float2* __restrict__ p,
                                                                   const float2* __restrict__ r,
                                                                   const float* __restrict__ dinv) {
  if (sc->done[0]) return;
  const float2 b = sc->beta_df;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = df_add_abs(df_mul_f(r[i], dinv[i]), df_mul(b, p[i]));
}

// r·z → part[G..2G), r·r → part[2G..3G) from the double-float r; p = D⁻¹r on restart
__global__ void __launch_bounds__(JFEM_RED_THREADS) k_dfcg_precond(int64_t n, const float2* __restrict__ r,
                                                                   const float* __restrict__ dinv,
                                                                   float2* __restrict__ p, int restart,
                                                                   double* __restrict__ part) {
  __shared__ double sh[32];
  float2 rz = make_float2(0.f, 0.f), rr = make_float2(0.f, 0.f);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 ri = r[i];
    const float2 zi = df_mul_f(ri, dinv[i]);
    if (restart) p[i] = zi;
    rz = df_add_abs(rz, df_mul(ri, zi));
    rr = df_add_abs(rr, df_mul(ri, ri));
  }
  const double rzb = block_sum_df(rz, sh);
  const double rrb = block_sum_df(rr, sh);
  if (threadIdx.x == 0) {
    part[G_ + blockIdx.x] = rzb;
    part[2 * G_ + blockIdx.x] = rrb;
  }
}

__global__ void k_df_from_double(int64_t n, const double* __restrict__ a, float2* __restrict__ b) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = df_from_double(a[i]);
}

// x (FP64) += δx (double-float); δx ← 0.  The mixed solver accumulates the
// correction since the last refinement in double-float and folds it into the
// FP64 iterate at every refinement, so x keeps FP64 precision (a 48-bit x would
// floor the true residual at ≈2⁻⁴⁸‖K‖‖x‖, above 1e-8 on slender cantilevers).
__global__ void k_df_absorb(int64_t n, float2* __restrict__ dx, double* __restrict__ x) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] += df_to_double(dx[i]);
    dx[i] = make_float2(0.f, 0.f);
  }
}

__global__ void k_df_to_double(int64_t n, const float2* __restrict__ a, double* __restrict__ b) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = df_to_double(a[i]);
}

__global__ void k_narrow(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

// slot 0 ← (r·z, r·r) of k_precond; optionally bb ← r·r and tol2 = tol² bb
__global__ void k_scalars_reset(SolverScalars* __restrict__ sc, const double* __restrict__ part, int set_bb,
                                double tol, int max_iters, int reset_iters) {
  __shared__ double sh[32];
  const double rz = reduce_partials(part + G_, G_, sh);
  const double rr = reduce_partials(part + 2 * G_, G_, sh);
  if (threadIdx.x == 0) {
    sc->rz[0] = rz;
    sc->rr[0] = rr;
    if (set_bb) {
      sc->bb = rr;
      sc->tol2 = tol * tol * rr;
    }
    if (reset_iters) sc->iters = 0;
    sc->max_iters = max_iters;
    sc->done[0] = (rr <= sc->tol2 || sc->iters >= max_iters) ? 1 : 0;
    sc->done[1] = 0;
    for (int k = 0; k < 4; ++k) sc->arrive[k] = 0;
  }
}

// out[0] = Σ part[3G..4G), out[1] = Σ part[0..G)
__global__ void k_sum_norms(const double* __restrict__ part, double* __restrict__ out) {
  __shared__ double sh[32];
  const double a = reduce_partials(part + 3 * G_, G_, sh);
  const double b = reduce_partials(part, G_, sh);
  if (threadIdx.x == 0) {
    out[0] = a;
    out[1] = b;
  }
}

// u += du on free DOFs; prescribed DOFs set to frac·g when assign_fixed
__global__ void k_update_state(int64_t N, double* __restrict__ u, const double* __restrict__ du,
                               const double* __restrict__ gvals, double frac, int assign_fixed,
                               const uint8_t* __restrict__ mask) {
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < N; j += (int64_t)gridDim.x * blockDim.x) {
    const uint8_t m = mask[j];
    for (int c = 0; c < 3; ++c) {
      if ((m >> c) & 1) {
        if (assign_fixed) u[3 * j + c] = frac * gvals[3 * j + c];
      } else {
        u[3 * j + c] += du[3 * j + c];
      }
    }
  }
}

// dg = frac·g − u on prescribed DOFs (the incremental Dirichlet value of
// src/problems_dirichlet.jl:60-89), 0 elsewhere; ‖dg‖² → part[3G..4G)
__global__ void __launch_bounds__(JFEM_RED_THREADS) k_bc_increment(int64_t N, const double* __restrict__ gvals,
                                                                   double frac, const double* __restrict__ u,
                                                                   const uint8_t* __restrict__ mask,
                                                                   double* __restrict__ dg, double* __restrict__ part) {
  __shared__ double sh[32];
  double s = 0.0;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < N; j += (int64_t)gridDim.x * blockDim.x) {
    const uint8_t m = mask[j];
    for (int c = 0; c < 3; ++c) {
      const double v = ((m >> c) & 1) ? frac * gvals[3 * j + c] - u[3 * j + c] : 0.0;
      dg[3 * j + c] = v;
      s += v * v;
    }
  }
  s = block_sum(s, sh);
  if (threadIdx.x == 0) part[3 * G_ + blockIdx.x] = s;
}

__global__ void k_sub_free(int64_t n, double* __restrict__ a, const double* __restrict__ b) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    a[i] -= b[i];   // b is masked (zero on prescribed rows)
}

__global__ void k_axpy(int64_t n, double a, const double* __restrict__ x, double* __restrict__ y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] += a * x[i];
}

void enqueue_axpy(Ctx* c, int64_t n, double a, const double* x, double* y) {
  k_axpy<<<grid_for(n, 256), 256, 0, c->stream>>>(n, a, x, y);
  c->launches += 1;
}

// ---------------------------------------------------------------------------
// flexible CG (Notay's FCG with one stored direction) for the learned
// preconditioner, double-float vectors like the mixed PCG:
//   z = B(r);  β = z·q_old / p_old·q_old (0 on restart);  p = z − βp;
//   q = K p;  α = p·r / p·q;  δx += αp;  r −= αq
// With a fixed SPD preconditioner this is PCG; with the network (nonlinear in
// r) the explicit orthogonalisation against the previous direction keeps the
// recursion consistent; the learned preconditioner is symmetric positive
// definite, for which FCG is PCG.  part regions: [0,G) tile p·q, [3G,4G)
// boundary p·q, [G,2G) r·r, [2G,3G) p·r, and the β terms of JFEM_PART_*.
// ---------------------------------------------------------------------------
// y = mask ⊙ D^{-1/2} r (FP32), the network input, one float4 per node
__global__ void __launch_bounds__(256) k_fcg_input(int64_t N, const float2* __restrict__ r,
                                                   const float* __restrict__ dinv, const uint8_t* __restrict__ mask,
                                                   const SolverScalars* __restrict__ sc, float4* __restrict__ y) {
  if (sc->done[0]) return;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    const uint8_t m = mask[i];
    float v[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float2 rq = r[3 * i + c];
      v[c] = ((m >> c) & 1) ? 0.f : sqrtf(dinv[3 * i + c]) * (rq.x + rq.y);
    }
    y[i] = make_float4(v[0], v[1], v[2], 0.f);
  }
}

// β = z·q_old / p_old·q_old (0 on restart) from its two parts, formed before z
// exists: Σ S(r)·q_old (the smoother's part; partials from the update kernel for
// Jacobi, from the network's last pass otherwise) and Ec·Pᵀq_old (the coarse
// part; partials from the coarse solve), each summed in a fixed order.
__global__ void __launch_bounds__(JFEM_RED_THREADS) k_fcg_beta(SolverScalars* __restrict__ sc,
                                                               const double* __restrict__ t1, int n1,
                                                               const double* __restrict__ t2, int n2) {
  __shared__ double sh[32];
  if (sc->done[0]) return;
  const double a = reduce_partials_cg(t1, n1, sh);
  const double b = t2 ? reduce_partials_cg(t2, n2, sh) : 0.0;
  if (threadIdx.x == 0) {
    const double beta = sc->restart ? 0.0 : (a + b) / sc->pAp;
    sc->beta = beta;
    sc->beta_df = df_from_double(beta);
    sc->restart = 0;
  }
}

// p = z − βp with z formed on the fly, node by node: z = D^{-1/2}(y + NᵀN y)
// (NN; y, v = NᵀN y given) or D⁻¹r (Jacobi), plus the coarse correction P Ec
// when COARSE, zero on prescribed DOFs (D⁻¹ is zero there).  p·r partials →
// the last block leaves p·r for α.
template <bool NN, bool COARSE>
__global__ void __launch_bounds__(JFEM_RED_THREADS, 4) k_fcg_zp(int64_t N, const float4* __restrict__ y,
                                                             const float4* __restrict__ v,
                                                             const float* __restrict__ dinv,
                                                             const uint8_t* __restrict__ mask,
                                                             const int* __restrict__ node_agg,
                                                             const float4* __restrict__ d32,
                                                             const float* __restrict__ Ec, float2* __restrict__ p,
                                                             const float2* __restrict__ r,
                                                             SolverScalars* __restrict__ sc, double* __restrict__ part) {
  __shared__ double sh[32];
  if (sc->done[0]) return;
  const float2 nb = df_neg(sc->beta_df);
  const bool keep = sc->beta != 0.0;
  float2 dot = make_float2(0.f, 0.f);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  // ND nodes per thread and round (two with the Jacobi smoother; the
  // network's variant needs the registers for its own vectors): every load
  // (and the coarse aggregate's Ec after its index) is issued before any
  // arithmetic
  constexpr int ND = NN ? 1 : 2;
  for (int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i0 < N; i0 += ND * stride) {
    int64_t ii[ND];
    bool val[ND];
#pragma unroll
    for (int n = 0; n < ND; ++n) {
      ii[n] = i0 + n * stride;
      val[n] = ii[n] < N;
    }
    float2 rq[ND][3], po[ND][3];
    float dv[ND][3];
    float4 y4[ND], v4[ND], dd[ND];
    int ag[ND];
    uint8_t m[ND];
#pragma unroll
    for (int n = 0; n < ND; ++n) {
      const int64_t i = val[n] ? ii[n] : i0;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        rq[n][c] = r[3 * i + c];
        po[n][c] = keep ? p[3 * i + c] : make_float2(0.f, 0.f);
        dv[n][c] = dinv[3 * i + c];
      }
      if (NN) {
        y4[n] = y[i];
        v4[n] = v[i];
      }
      if (COARSE) {
        m[n] = mask[i];
        ag[n] = node_agg[i];
        dd[n] = d32[i];
      }
    }
    float ec[ND][6];
    if (COARSE) {
#pragma unroll
      for (int n = 0; n < ND; ++n)
#pragma unroll
        for (int k = 0; k < 6; ++k) ec[n][k] = Ec[6 * ag[n] + k];
    }
#pragma unroll
    for (int n = 0; n < ND; ++n) {
      if (!val[n]) continue;
      const int64_t i = ii[n];
      float zc[3];
      if (NN) {
        zc[0] = sqrtf(dv[n][0]) * (y4[n].x + v4[n].x);
        zc[1] = sqrtf(dv[n][1]) * (y4[n].y + v4[n].y);
        zc[2] = sqrtf(dv[n][2]) * (y4[n].z + v4[n].z);
      } else {
#pragma unroll
        for (int c = 0; c < 3; ++c) zc[c] = dv[n][c] * (rq[n][c].x + rq[n][c].y);
      }
      if (COARSE) {   // P Ec at the node: e_a + θ_a × d
#pragma unroll
        for (int c = 0; c < 3; ++c)
          if (!((m[n] >> c) & 1)) zc[c] += coarse_prolong_v(ec[n], dd[n], c);
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        float2 pi = make_float2(zc[c], 0.f);
        if (keep) pi = df_add_abs(pi, df_mul(nb, po[n][c]));
        p[3 * i + c] = pi;
        dot = df_add_abs(dot, df_mul(pi, rq[n][c]));
      }
    }
  }
  const double b = block_sum_df(dot, sh);
  if (threadIdx.x == 0) part[2 * G_ + blockIdx.x] = b;
  if (arrive_last(&sc->arrive[3])) {
    const double pr = reduce_partials_cg(part + 2 * G_, G_, sh);
    if (threadIdx.x == 0) {
      sc->rz[0] = pr;
      sc->arrive[3] = 0;
    }
  }
}

// x += αp, r −= αq; r·r partials → the last block updates the scalars and the
// stop flag.  T1 (Jacobi smoother): also Σ D⁻¹r·q partials for the next β.
// ynext (the network): the next iteration's input D^{-1/2} r per node (float4
// x, y, z; zero on prescribed DOFs, where D⁻¹ is zero), formed here while r is
// in registers.
template <bool T1>
__global__ void __launch_bounds__(JFEM_RED_THREADS) k_fcg_update(int64_t n, SolverScalars* __restrict__ sc,
                                                                 float2* __restrict__ x, float2* __restrict__ r,
                                                                 const float2* __restrict__ p,
                                                                 const float* __restrict__ q,
                                                                 const float* __restrict__ dinv,
                                                                 float* __restrict__ ynext,
                                                                 double* __restrict__ part) {
  __shared__ double sh[32];
  if (sc->done[0]) return;
  const float2 a = sc->alpha_df, na = df_neg(a);
  float2 rr = make_float2(0.f, 0.f), t1 = make_float2(0.f, 0.f);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] = df_add_abs(x[i], df_mul(a, p[i]));
    const float qi = q[i];
    const float2 ri = df_add(r[i], df_mul_f(na, qi));
    r[i] = ri;
    rr = df_add_abs(rr, df_mul(ri, ri));
    if (T1) t1 = df_add_abs(t1, df_two_prod(dinv[i] * (ri.x + ri.y), qi));
    if (ynext) {
      const int64_t node = i / 3;
      ynext[4 * node + (i - 3 * node)] = sqrtf(dinv[i]) * (ri.x + ri.y);
    }
  }
  const double2 bs = block_sum2_df(rr, t1, sh);
  if (threadIdx.x == 0) {
    part[G_ + blockIdx.x] = bs.x;
    if (T1) part[JFEM_PART_T1 + blockIdx.x] = bs.y;
  }
  if (arrive_last(&sc->arrive[1])) {
    const double rr_new = reduce_partials_cg(part + G_, G_, sh);
    if (threadIdx.x == 0) {
      sc->rr[0] = rr_new;
      sc->rz[0] = rr_new;   // reported in place of r·z (positive while the solve is healthy)
      const int it = sc->iters + 1;
      sc->iters = it;
      sc->done[0] = (rr_new <= sc->tol2 || it >= sc->max_iters || !(rr_new == rr_new)) ? 1 : 0;
      sc->arrive[1] = 0;
    }
  }
}

// r·r → part[G..2G) for a (re)start, and Σ D⁻¹r·q_old partials (the Jacobi β term
// for a kept direction)
__global__ void __launch_bounds__(JFEM_RED_THREADS) k_fcg_norms(int64_t n, const float2* __restrict__ r,
                                                                const float* __restrict__ dinv,
                                                                const float* __restrict__ qold,
                                                                double* __restrict__ part) {
  __shared__ double sh[32];
  float2 rr = make_float2(0.f, 0.f), t1 = make_float2(0.f, 0.f);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float2 ri = r[i];
    rr = df_add_abs(rr, df_mul(ri, ri));
    t1 = df_add_abs(t1, df_two_prod(dinv[i] * (ri.x + ri.y), qold[i]));
  }
  const double2 bs = block_sum2_df(rr, t1, sh);
  if (threadIdx.x == 0) {
    part[G_ + blockIdx.x] = bs.x;
    part[JFEM_PART_T1 + blockIdx.x] = bs.y;
  }
}

__global__ void k_fcg_reset(SolverScalars* __restrict__ sc, const double* __restrict__ part, int set_bb, double tol,
                            int max_iters, int reset_iters, int restart) {
  __shared__ double sh[32];
  const double rr = reduce_partials(part + G_, G_, sh);
  if (threadIdx.x == 0) {
    sc->rz[0] = rr;
    sc->rr[0] = rr;
    if (set_bb) {
      sc->bb = rr;
      sc->tol2 = tol * tol * rr;
    }
    if (reset_iters) sc->iters = 0;
    sc->max_iters = max_iters;
    sc->restart = restart;
    sc->done[0] = (rr <= sc->tol2 || sc->iters >= max_iters) ? 1 : 0;
    sc->done[1] = 0;
    for (int k = 0; k < 4; ++k) sc->arrive[k] = 0;
  }
}

// ---------------------------------------------------------------------------
// host orchestration
// ---------------------------------------------------------------------------
static double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

static int read_scalars(Ctx* c) {
  cudaMemcpyAsync(c->sc_host, c->sc, sizeof(SolverScalars), cudaMemcpyDeviceToHost, c->stream);
  return sync_and_check(c, "solver scalars");
}

static int read_norms(Ctx* c, double* a, double* b) {
  k_sum_norms<<<1, JFEM_RED_THREADS, 0, c->stream>>>(c->part, c->norms);
  c->launches += 1;
  cudaMemcpyAsync(c->norms_host, c->norms, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  int rc = sync_and_check(c, "norms");
  if (rc) return rc;
  *a = c->norms_host[0];
  if (b) *b = c->norms_host[1];
  return 0;
}

// r ← f − K x (FP64 apply, prescribed rows zero); returns ‖r‖² and, when
// drift2 is given, ‖r_new − r_old‖² (distance from the recursive residual).
static int true_residual(Ctx* c, const double* f, const double* xv, double* r, double* rr_out,
                         double* drift2 = nullptr) {
  enqueue_apply(c, xv, c->tmp, false, true, false, nullptr, nullptr, nullptr);
  k_residual<<<G_, JFEM_RED_THREADS, 0, c->stream>>>(c->N, f, 1.0, c->tmp, c->mask, r, drift2 ? 2 : 0, c->part);
  c->launches += 1;
  return read_norms(c, rr_out, drift2);
}

// One flexible-CG iteration: [coarse: restriction of r and q_old, coarse solve]
// [network: input, 6 neighbour passes] β; p = z − βp (z formed in place);
// q = K p (tiled apply, α); x, r update.
static void enqueue_fcg_iteration(Ctx* c, bool nn, bool coarse) {
  const int64_t n = 3 * c->N;
  double* t2 = coarse ? c->part + JFEM_PART_T2 : nullptr;
  // β is formed by the last block of the launch that writes the last of its
  // partials: the network's last pass (nn), else the coarse solve (coarse),
  // else its own launch
  if (coarse)
    enqueue_coarse_restrict_solve(c, c->rd, &c->sc->done[0], c->Apf, t2, nn ? nullptr : c->sc,
                                  c->part + JFEM_PART_T1, G_);
  const int n2 = coarse ? coarse_gemv_blocks(c) : 0;
  const int* na = coarse ? c->node_agg : nullptr;
  const float4* d32 = coarse ? c->node_d32 : nullptr;
  const float* Ec = coarse ? c->Ec : nullptr;
  float4* y = c->mi;
  float4* v = c->mi ? c->mi + 6 * c->N : nullptr;
  if (nn) {
    // y (the network's input) was formed by the previous update, or after the
    // last (re)start
    enqueue_mpnn_spd(c, y, v, c->dinvf, c->Apf, c->part + JFEM_PART_T1N, c->sc, t2, n2);
    if (coarse)
      k_fcg_zp<true, true><<<G_, JFEM_RED_THREADS, 0, c->stream>>>(c->N, y, v, c->dinvf, c->mask, na, d32, Ec, c->p2,
                                                                   c->rd, c->sc, c->part);
    else
      k_fcg_zp<true, false><<<G_, JFEM_RED_THREADS, 0, c->stream>>>(c->N, y, v, c->dinvf, c->mask, na, d32, Ec, c->p2,
                                                                    c->rd, c->sc, c->part);
  } else {
    if (!coarse) k_fcg_beta<<<1, JFEM_RED_THREADS, 0, c->stream>>>(c->sc, c->part + JFEM_PART_T1, G_, t2, n2);
    if (coarse)
      k_fcg_zp<false, true><<<G_, JFEM_RED_THREADS, 0, c->stream>>>(c->N, nullptr, nullptr, c->dinvf, c->mask, na, d32,
                                                                    Ec, c->p2, c->rd, c->sc, c->part);
    else
      k_fcg_zp<false, false><<<G_, JFEM_RED_THREADS, 0, c->stream>>>(c->N, nullptr, nullptr, c->dinvf, c->mask, na,
                                                                     d32, Ec, c->p2, c->rd, c->sc, c->part);
  }
  c->launches += nn ? 1 : (coarse ? 1 : 2);
  enqueue_apply_tiled(c, c->p2, c->Apf, true, c->part, &c->sc->done[0], c->sc);
  if (nn)
    k_fcg_update<false><<<G_, JFEM_RED_THREADS, 0, c->stream>>>(n, c->sc, c->xd, c->rd, c->p2, c->Apf, c->dinvf,
                                                                reinterpret_cast<float*>(y), c->part);
  else
    k_fcg_update<true><<<G_, JFEM_RED_THREADS, 0, c->stream>>>(n, c->sc, c->xd, c->rd, c->p2, c->Apf, c->dinvf,
                                                               nullptr, c->part);
  c->launches += 1;
}

static void enqueue_iteration(Ctx* c, bool fp32, int slot) {
  const int64_t n = 3 * c->N;
  if (fp32) {   // mixed: double-float vectors, tiled FP32 apply
    enqueue_apply_tiled(c, c->p2, c->Apf, true, c->part, &c->sc->done[0], c->sc);
    k_dfcg_update1<<<G_, JFEM_RED_THREADS, 0, c->stream>>>(n, c->sc, c->xd, c->rd, c->p2, c->Apf, c->dinvf,
                                                          c->part);
    k_dfcg_update2<<<G_, JFEM_RED_THREADS, 0, c->stream>>>(n, c->sc, c->p2, c->rd, c->dinvf);
    c->launches += 2;
    return;
  }
  enqueue_apply(c, c->p, c->Ap, false, true, false, c->part, &c->sc->done[slot], nullptr);
  k_pcg_update1<<<G_, JFEM_RED_THREADS, 0, c->stream>>>(n, c->sc, slot, c->x, c->r, c->z, c->p, c->Ap,
                                                       c->dinv, c->part, 0);
  k_pcg_update2<<<G_, JFEM_RED_THREADS, 0, c->stream>>>(n, c->sc, slot, c->p, c->z, c->part, nullptr);
  c->launches += 2;
}

// kind: 0 FP64 PCG, 1 mixed PCG, 2 FCG Jacobi, 3 FCG learned, 4 FCG Jacobi + coarse,
// 5 FCG learned + coarse
static int graph_key(Ctx* c, int kind) {
  return kind | (c->finite << 3) | (c->model << 4) | (c->geom << 5) | ((c->geo_affine ? 1 : 0) << 6) |
         (c->et << 7) | ((c->geoT32 ? 1 : 0) << 12) | ((nh_cache_ready(c) ? 1 : 0) << 13);
}

static int build_graph(Ctx* c, int kind) {
  const int key = graph_key(c, kind);
  if (c->pcg_graph && c->pcg_graph_key == key) return 0;
  if (c->pcg_graph) {
    cudaGraphExecDestroy(c->pcg_graph);
    c->pcg_graph = nullptr;
  }
  cudaGraph_t g = nullptr;
  const int64_t l0 = c->launches;
  cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda_check(c, e, "begin capture");
  for (int k = 0; k < PCG_CHUNK; ++k) {
    if (kind >= 2) enqueue_fcg_iteration(c, kind == 3 || kind == 5, kind >= 4);
    else enqueue_iteration(c, kind == 1, kind == 1 ? 0 : (k & 1));
  }
  e = cudaStreamEndCapture(c->stream, &g);
  if (e != cudaSuccess) return cuda_check(c, e, "end capture");
  e = cudaGraphInstantiate(&c->pcg_graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_check(c, e, "graph instantiate");
  c->pcg_graph_key = key;
  c->chunk_launches = c->launches - l0;
  c->launches = l0;   // counted when the graph runs
  return 0;
}

struct PcgResult {
  int iters = 0;
  int refinements = 0;
  double relres = 0.0;
  int status = 0;
  int fallbacks = 0;
};

// FP64 iterates captured at iteration counts first, 2·first, 4·first, … (after
// the graph chunk that reaches them), for training-pair collection.
struct PcgSnap {
  double* buf = nullptr;   // [max][3N]
  int max = 0, count = 0, next = 16;
  int* iters = nullptr;
};

// PCG on the masked operator for K x = f over the free DOFs; x holds the
// initial guess (prescribed entries fixed).  tol is relative to ‖f_free − K x₀‖
// (the relative residual when the free part of x₀ is zero).
//
// The stopping test always uses the true FP64 residual f − K x.  A "refinement"
// replaces the recursive residual by the true one.  When the two differ by less
// than 10 % the search direction is kept (a reliable update: CG keeps its
// convergence speed); otherwise the direction restarts (p = z), because with an
// FP32 operator the recursion can drift from the FP64 residual by about
// ε₃₂·‖K‖‖x‖ and continuing an old direction after a large replacement
// diverges, while restarting is defect correction with CG inner solves.
// Refinements happen at recursive convergence and, when `reliable`, each time
// the recursive residual norm has dropped by `drop` since the last true one.  When two refinements in a row gain less than 2× the solve has
// reached the attainable accuracy of the arithmetic: the best iterate is kept
// and JFEM_NOT_CONVERGED returned.
static int pcg(Ctx* c, const double* f, bool fp32, double tol, int max_iter, double time_budget, double t_start,
               bool reliable, bool x_zero, PcgResult* res, double drop = 1e-2, PcgSnap* snap = nullptr,
               bool tol_abs = false) {
  int rc = 0;
  double rr0 = 0.0;
  const int64_t n = 3 * c->N;
  const unsigned gv = grid_for(n, 256);
  if (fp32 && !apply_is_tiled(c)) return set_err(c, JFEM_ERR_INVALID, "mixed solve needs the tiled apply");
  if (x_zero) {
    k_residual<<<G_, JFEM_RED_THREADS, 0, c->stream>>>(c->N, f, 1.0, nullptr, c->mask, c->r, 0, c->part);
    c->launches += 1;
    if ((rc = read_norms(c, &rr0, nullptr))) return rc;
  } else if ((rc = true_residual(c, f, c->x, c->r, &rr0))) {
    return rc;
  }
  if (tol_abs && rr0 > 0.0) tol /= std::sqrt(rr0);   // ‖r‖ ≤ tol as the reference's CG tests it
  if (fp32) {   // double-float state: δx, r, p; FP32 Jacobi diagonal
    k_narrow<<<gv, 256, 0, c->stream>>>(n, c->dinv, c->dinvf);
    cudaMemsetAsync(c->xd, 0, n * sizeof(float2), c->stream);   // correction δx since the last refinement
    k_df_from_double<<<gv, 256, 0, c->stream>>>(n, c->r, c->rd);
    k_dfcg_precond<<<G_, JFEM_RED_THREADS, 0, c->stream>>>(n, c->rd, c->dinvf, c->p2, 1, c->part);
    c->launches += 4;
  } else {
    k_precond<<<G_, JFEM_RED_THREADS, 0, c->stream>>>(n, c->r, c->dinv, c->z, c->p, 1, c->part, nullptr);
    c->launches += 1;
  }
  k_scalars_reset<<<1, JFEM_RED_THREADS, 0, c->stream>>>(c->sc, c->part, 1, tol, max_iter, 1);
  c->launches += 1;
  if ((rc = read_scalars(c))) return rc;
  const double bb = c->sc_host->bb;
  res->iters = 0;
  res->refinements = 0;
  res->relres = 0.0;
  res->status = 0;
  if (!(bb > 0.0)) return 0;
  if ((rc = build_graph(c, fp32 ? 1 : 0))) return rc;
  const double ru = fp32 ? drop * drop : 0.0;
  const double goal = tol * tol * bb;
  double rr_true_last = rr0, rr_best = rr0;
  cudaMemcpyAsync(c->xbest, c->x, 3 * c->N * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
  int refinements = 0, stalls = 0;
  for (;;) {
    if (!c->sc_host->done[0]) {
      cudaError_t e = cudaGraphLaunch(c->pcg_graph, c->stream);
      if (e != cudaSuccess) return cuda_check(c, e, "graph launch");
      c->launches += c->chunk_launches;
      if ((rc = read_scalars(c))) return rc;
      if (snap && !fp32 && snap->count < snap->max && c->sc_host->iters >= snap->next && !c->sc_host->done[0]) {
        cudaMemcpyAsync(snap->buf + (int64_t)snap->count * 3 * c->N, c->x, 3 * c->N * sizeof(double),
                        cudaMemcpyDeviceToDevice, c->stream);
        snap->iters[snap->count++] = c->sc_host->iters;
        snap->next *= 2;
      }
    }
    const SolverScalars& s = *c->sc_host;
    const double rr = s.rr[0];
    const int iters = s.iters;
    const bool at_cap = iters >= max_iter;
    const bool bad = !(rr == rr) || !(s.rz[0] > 0.0) || rr > 1e30 * bb;
    const bool check = s.done[0] || bad || (reliable && rr < ru * rr_true_last);
    if (check) {
      double rr_t = 0.0, drift2 = 0.0;
      if (fp32) {   // x += δx (FP64); FP64 copy of the recursive r for the drift
        k_df_absorb<<<gv, 256, 0, c->stream>>>(n, c->xd, c->x);
        k_df_to_double<<<gv, 256, 0, c->stream>>>(n, c->rd, c->r);
        c->launches += 2;
      }
      if ((rc = true_residual(c, f, c->x, c->r, &rr_t, &drift2))) return rc;
      ++refinements;
      const bool finite = rr_t == rr_t && rr_t < 1e300;
      if (finite && rr_t < rr_best) {
        rr_best = rr_t;
        cudaMemcpyAsync(c->xbest, c->x, 3 * c->N * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
      }
      stalls = (finite && rr_t < 0.25 * rr_true_last) ? 0 : stalls + 1;
      const bool converged = finite && rr_t <= goal;
      if (converged || at_cap || stalls >= 2 || !finite) {
        if (!converged) {   // return the best iterate found
          cudaMemcpyAsync(c->x, c->xbest, 3 * c->N * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
          if ((rc = sync_and_check(c, "best iterate"))) return rc;
        }
        res->iters = iters;
        res->refinements = refinements;
        res->relres = std::sqrt((converged ? rr_t : rr_best) / bb);
        res->status = converged ? 0 : JFEM_NOT_CONVERGED;
        return 0;
      }
      rr_true_last = rr_t;
      if (!finite) {   // restart from the best iterate
        cudaMemcpyAsync(c->x, c->xbest, 3 * c->N * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
        if ((rc = true_residual(c, f, c->x, c->r, &rr_t))) return rc;
        rr_true_last = rr_t;
        if (fp32) cudaMemsetAsync(c->xd, 0, n * sizeof(float2), c->stream);
      }
      // refinement: r ← true residual; keep p when the drift is small, else restart
      const int restart = (finite && drift2 < 0.01 * rr_t) ? 0 : 1;
      if (fp32) {
        k_df_from_double<<<gv, 256, 0, c->stream>>>(n, c->r, c->rd);
        k_dfcg_precond<<<G_, JFEM_RED_THREADS, 0, c->stream>>>(n, c->rd, c->dinvf, c->p2, restart, c->part);
        c->launches += 2;
      } else {
        k_precond<<<G_, JFEM_RED_THREADS, 0, c->stream>>>(n, c->r, c->dinv, c->z, c->p, restart, c->part, nullptr);
        c->launches += 1;
      }
      k_scalars_reset<<<1, JFEM_RED_THREADS, 0, c->stream>>>(c->sc, c->part, 0, tol, max_iter, 0);
      c->launches += 1;
      if ((rc = read_scalars(c))) return rc;
    }
    if (time_budget > 0.0 && now_s() - t_start > time_budget) {
      // hand back the better (true FP64 residual) of the current and the best iterate
      if (fp32) {
        k_df_absorb<<<gv, 256, 0, c->stream>>>(n, c->xd, c->x);
        c->launches += 1;
      }
      double rr_t = 0.0;
      if ((rc = true_residual(c, f, c->x, c->r, &rr_t))) return rc;
      if (rr_t == rr_t && rr_t < rr_best) rr_best = rr_t;
      else cudaMemcpyAsync(c->x, c->xbest, 3 * c->N * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
      res->iters = iters;
      res->refinements = refinements;
      res->relres = std::sqrt(rr_best / bb);
      res->status = JFEM_ERR_TIMEOUT;
      return set_err(c, JFEM_ERR_TIMEOUT, "solve exceeded its time budget");
    }
  }
}

// Flexible CG with the learned preconditioner (nn) or Jacobi, mixed precision
// (double-float vectors, FP32 tiled apply, the FP64 true residual decides).
// Refinements as in pcg() (the direction is kept when the recursive and true
// residuals agree to 10 %).  When the learned preconditioner stalls (two
// refinements without a 4× gain in the true residual, or no 10 % progress of
// the recursive residual norm over `window` iterations — generous, since CG
// residual norms are not monotone) the solve continues with Jacobi from the
// best iterate (res->fallbacks = 1).
// reliable = false (Newton's inner solves, whose caller judges every step by
// its own FP64 residual): no FP64 true residual, neither on the way nor at
// the end — the recursive residual decides, as in pcg without reliable updates.
static int fcg(Ctx* c, const double* f, bool nn, bool coarse, double tol, int max_iter, double time_budget,
               double t_start, bool x_zero, PcgResult* res, double drop, bool tol_abs = false, bool reliable = true) {
  int rc = 0;
  double rr0 = 0.0;
  const int64_t n = 3 * c->N;
  const unsigned gv = grid_for(n, 256);
  if (!apply_is_tiled(c)) return set_err(c, JFEM_ERR_INVALID, "flexible CG needs the tiled apply");
  if (nn && (!c->mp || !c->mp->ready)) return set_err(c, JFEM_ERR_INVALID, "no network weights (jfem_mpnn_init)");
  if (nn && (rc = mpnn_ensure_infer(c))) return rc;
  if (nn && (rc = mpnn_refresh_poly(c))) return rc;
  if (coarse && (rc = coarse_prepare(c))) return rc;
  const auto kind_of = [&]() { return (nn ? 3 : 2) + (coarse ? 2 : 0); };
  if (x_zero) {
    k_residual<<<G_, JFEM_RED_THREADS, 0, c->stream>>>(c->N, f, 1.0, nullptr, c->mask, c->r, 0, c->part);
    c->launches += 1;
    if ((rc = read_norms(c, &rr0, nullptr))) return rc;
  } else if ((rc = true_residual(c, f, c->x, c->r, &rr0))) {
    return rc;
  }
  if (tol_abs && rr0 > 0.0) tol /= std::sqrt(rr0);
  k_narrow<<<gv, 256, 0, c->stream>>>(n, c->dinv, c->dinvf);
  cudaMemsetAsync(c->xd, 0, n * sizeof(float2), c->stream);
  cudaMemsetAsync(c->Apf, 0, n * sizeof(float), c->stream);
  k_df_from_double<<<gv, 256, 0, c->stream>>>(n, c->r, c->rd);
  k_fcg_norms<<<G_, JFEM_RED_THREADS, 0, c->stream>>>(n, c->rd, c->dinvf, c->Apf, c->part);
  k_fcg_reset<<<1, JFEM_RED_THREADS, 0, c->stream>>>(c->sc, c->part, 1, tol, max_iter, 1, 1);
  c->launches += 4;
  if (nn) {   // the network's first input; later ones come from the update kernel
    k_fcg_input<<<grid_for(c->N, 256), 256, 0, c->stream>>>(c->N, c->rd, c->dinvf, c->mask, c->sc, c->mi);
    c->launches += 1;
  }
  if ((rc = read_scalars(c))) return rc;
  const double bb = c->sc_host->bb;
  *res = PcgResult();
  if (!(bb > 0.0)) return 0;
  if ((rc = build_graph(c, kind_of()))) return rc;
  const double ru = drop * drop;
  const double goal = tol * tol * bb;
  const int window = 4096;
  double rr_true_last = rr0, rr_best = rr0, rr_rec_best = rr0;
  int rec_best_it = 0;
  cudaMemcpyAsync(c->xbest, c->x, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
  int refinements = 0, stalls = 0, fallbacks = 0;
  for (;;) {
    if (!c->sc_host->done[0]) {
      cudaError_t e = cudaGraphLaunch(c->pcg_graph, c->stream);
      if (e != cudaSuccess) return cuda_check(c, e, "graph launch");
      c->launches += c->chunk_launches;
      if ((rc = read_scalars(c))) return rc;
    }
    const SolverScalars& s = *c->sc_host;
    const double rr = s.rr[0];
    const int iters = s.iters;
    const bool at_cap = iters >= max_iter;
    const bool bad = !(rr == rr) || rr > 1e30 * bb;
    if (rr < 0.9 * rr_rec_best) {
      rr_rec_best = rr;
      rec_best_it = iters;
    }
    const bool stagnant = nn && iters - rec_best_it >= window;
    if (!reliable && s.done[0] && !bad) {   // the recursive residual decides
      k_df_absorb<<<gv, 256, 0, c->stream>>>(n, c->xd, c->x);
      c->launches += 1;
      if ((rc = sync_and_check(c, "flexible CG result"))) return rc;
      res->iters = iters;
      res->refinements = refinements;
      res->fallbacks = fallbacks;
      res->relres = std::sqrt(rr / bb);
      res->status = rr <= goal ? (fallbacks ? JFEM_STALL : 0) : JFEM_NOT_CONVERGED;
      return 0;
    }
    const bool check = s.done[0] || bad || (reliable && rr < ru * rr_true_last) || stagnant;
    if (check) {
      double rr_t = 0.0, drift2 = 0.0;
      k_df_absorb<<<gv, 256, 0, c->stream>>>(n, c->xd, c->x);
      k_df_to_double<<<gv, 256, 0, c->stream>>>(n, c->rd, c->r);
      c->launches += 2;
      if ((rc = true_residual(c, f, c->x, c->r, &rr_t, &drift2))) return rc;
      ++refinements;
      const bool finite = rr_t == rr_t && rr_t < 1e300;
      if (finite && rr_t < rr_best) {
        rr_best = rr_t;
        cudaMemcpyAsync(c->xbest, c->x, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
      }
      stalls = (finite && rr_t < 0.25 * rr_true_last && !stagnant) ? 0 : stalls + 1;
      const bool converged = finite && rr_t <= goal;
      bool switch_jacobi = false;
      if (!converged && !at_cap && (stalls >= 2 || !finite) && nn) {   // learned preconditioner stalled
        switch_jacobi = true;   // continue as plain Jacobi-PCG
        nn = false;
        coarse = false;
        fallbacks = 1;
        stalls = 0;
      }
      if (converged || at_cap || (!switch_jacobi && (stalls >= 2 || !finite))) {
        if (!converged) {
          cudaMemcpyAsync(c->x, c->xbest, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
          if ((rc = sync_and_check(c, "best iterate"))) return rc;
        }
        res->iters = iters;
        res->refinements = refinements;
        res->fallbacks = fallbacks;
        res->relres = std::sqrt((converged ? rr_t : rr_best) / bb);
        res->status = converged ? (fallbacks ? JFEM_STALL : 0) : JFEM_NOT_CONVERGED;
        return 0;
      }
      rr_true_last = rr_t;
      if (!finite || switch_jacobi) {   // continue from the best iterate
        cudaMemcpyAsync(c->x, c->xbest, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
        if ((rc = true_residual(c, f, c->x, c->r, &rr_t))) return rc;
        rr_true_last = rr_t;
      }
      if (switch_jacobi && (rc = build_graph(c, kind_of()))) return rc;
      rr_rec_best = rr_t;
      rec_best_it = iters;
      const int restart = (!finite || switch_jacobi || !(drift2 < 0.01 * rr_t)) ? 1 : 0;
      k_df_from_double<<<gv, 256, 0, c->stream>>>(n, c->r, c->rd);
      k_fcg_norms<<<G_, JFEM_RED_THREADS, 0, c->stream>>>(n, c->rd, c->dinvf, c->Apf, c->part);
      k_fcg_reset<<<1, JFEM_RED_THREADS, 0, c->stream>>>(c->sc, c->part, 0, tol, max_iter, 0, restart);
      c->launches += 3;
      if (nn) {   // the network's input from the refreshed residual
        k_fcg_input<<<grid_for(c->N, 256), 256, 0, c->stream>>>(c->N, c->rd, c->dinvf, c->mask, c->sc, c->mi);
        c->launches += 1;
      }
      if ((rc = read_scalars(c))) return rc;
    }
    if (time_budget > 0.0 && now_s() - t_start > time_budget) {
      // hand back the better (true FP64 residual) of the current and the best iterate
      k_df_absorb<<<gv, 256, 0, c->stream>>>(n, c->xd, c->x);
      c->launches += 1;
      double rr_t = 0.0;
      if ((rc = true_residual(c, f, c->x, c->r, &rr_t))) return rc;
      if (rr_t == rr_t && rr_t < rr_best) rr_best = rr_t;
      else cudaMemcpyAsync(c->x, c->xbest, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
      res->iters = iters;
      res->refinements = refinements;
      res->fallbacks = fallbacks;
      res->relres = std::sqrt(rr_best / bb);
      res->status = JFEM_ERR_TIMEOUT;
      return set_err(c, JFEM_ERR_TIMEOUT, "solve exceeded its time budget");
    }
  }
}

static int prepare_rhs(Ctx* c) {
  if (c->f_ext_dirty) {
    int rc = traction_device(c, c->f_ext);
    if (rc) return rc;
    c->f_ext_dirty = false;
  }
  return 0;
}

static void fill_stats(jfem_stats* st, int status, int newton, int cg, int refin, double res, double t) {
  if (!st) return;
  st->status = status;
  st->newton_iterations = newton;
  st->cg_iterations = cg;
  st->refinements = refin;
  st->residual = res;
  st->solve_time_s = t;
}

// Linear solve K u = f_ext with prescribed values eliminated (solvers.jl:192-216).
static int solve_linear(Ctx* c, const jfem_solve_opts* o, double* u_d, jfem_stats* st) {
  const double t0 = now_s();
  int rc = 0;
  if ((rc = geometry_prepare(c))) return rc;
  if ((rc = prepare_rhs(c))) return rc;
  if ((rc = jacobi_diag_device(c, c->dinv))) return rc;
  cudaMemcpyAsync(c->x, c->gvals, 3 * c->N * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
  const bool fp32 = o->precision == JFEM_MIXED;
  PcgResult pr;
  // FP64 true residual each time ‖r‖ drops by `drop`: 0.3 for Jacobi-PCG's long runs; the
  // flexible-CG methods converge in a few hundred iterations, over which an FP32 apply's
  // drift stays far below the residual, so every 100× suffices there
  const bool flexible = o->method == JFEM_FCG_LEARNED || o->method == JFEM_FCG_TWO_LEVEL;
  const double drop = o->refine_drop > 0.0 ? o->refine_drop : (flexible ? 0.01 : 0.3);
  const bool tol_abs = o->tol_absolute != 0;
  if (o->method == JFEM_FCG_LEARNED || o->method == JFEM_FCG_TWO_LEVEL) {
    const bool nn = o->method == JFEM_FCG_LEARNED;
    const bool coarse = !nn || c->coarse_target != 0;
    rc = fcg(c, c->f_ext, nn, coarse, o->tol, o->max_iter, o->time_budget_s, t0, c->n_fixed_nonzero == 0, &pr,
             drop, tol_abs);
  } else
    rc = pcg(c, c->f_ext, fp32, o->tol, o->max_iter, o->time_budget_s, t0, true, c->n_fixed_nonzero == 0, &pr,
             drop, nullptr, tol_abs);
  if (rc && rc != JFEM_ERR_TIMEOUT) return rc;
  // on JFEM_ERR_TIMEOUT x holds the best iterate found before the budget ran out
  const int rc_solve = rc;
  cudaMemcpyAsync(u_d, c->x, 3 * c->N * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
  if ((rc = sync_and_check(c, "solution copy"))) return rc;
  fill_stats(st, rc_solve ? rc_solve : pr.status, 1, pr.iters, pr.refinements, pr.relres, now_s() - t0);
  if (st) {
    st->history_len = 0;
    st->fallbacks = pr.fallbacks;
  }
  return rc_solve ? rc_solve : pr.status;
}

// FP64 Jacobi-PCG of the current system from x = prescribed values to tol,
// keeping iterates at 16, 32, 64, … iterations (training-pair collection).
// Leaves x* in c->x, D⁻¹ in c->dinv.
int pcg_fp64_snapshots(Ctx* c, const double* f, double tol, int max_iter, double* snaps, int max_snaps,
                       int* n_snaps, int* snap_iters, int* iters_out, double* relres_out) {
  int rc = 0;
  if ((rc = geometry_prepare(c))) return rc;
  if ((rc = prepare_rhs(c))) return rc;
  if ((rc = jacobi_diag_device(c, c->dinv))) return rc;
  cudaMemcpyAsync(c->x, c->gvals, 3 * c->N * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
  PcgSnap sn;
  sn.buf = snaps;
  sn.max = max_snaps;
  sn.iters = snap_iters;
  PcgResult pr;
  rc = pcg(c, f == c->f_ext ? c->f_ext : f, false, tol, max_iter, 0.0, now_s(), false, c->n_fixed_nonzero == 0,
           &pr, 1e-2, &sn);
  if (rc) return rc;
  *n_snaps = sn.count;
  *iters_out = pr.iters;
  *relres_out = pr.relres;
  return sync_and_check(c, "snapshots");
}

// A Newton solve that ran out of its time budget hands back the last accepted
// Newton state (u after the last completed Newton update).
static void newton_timeout_state(Ctx* c, double* u_d, jfem_stats* st, int newton, int cg, int refin, double rel,
                                 double t0) {
  cudaMemcpyAsync(u_d, c->u_state, 3 * c->N * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
  cudaStreamSynchronize(c->stream);
  fill_stats(st, JFEM_ERR_TIMEOUT, newton, cg, refin, rel, now_s() - t0);
}

// Inexact Newton–Krylov with load stepping.  Step s of S applies s/S of the
// traction and of the prescribed values; the first iteration of a step carries
// the increment of the prescribed DOFs.  Converged when ‖R_free‖ ≤
// newton_tol·‖f_int‖ (FP64; f_int over all DOFs, reactions included), or, with
// opts.tol_absolute, when ‖R_free‖ ≤ newton_tol as in the reference.
static int solve_newton(Ctx* c, const jfem_solve_opts* o, double* u_d, jfem_stats* st) {
  const double t0 = now_s();
  int rc = 0;
  if ((rc = geometry_prepare(c))) return rc;
  if ((rc = prepare_rhs(c))) return rc;
  const int64_t n = 3 * c->N;
  if (!c->have_state) {
    cudaMemsetAsync(c->u_state, 0, n * sizeof(double), c->stream);
    c->have_state = true;
    ++c->state_version;
  }
  const int steps = o->n_load_steps > 0 ? o->n_load_steps : 1;
  const bool fp32 = o->precision == JFEM_MIXED;
  int total_cg = 0, total_newton = 0, refin = 0, hist = 0, status = 0;
  double last_rel = 0.0;
  double* dg = c->tmp2;
  if (st) st->history_len = 0;
  for (int s = 1; s <= steps; ++s) {
    const double frac = (double)s / steps;
    bool converged = false;
    for (int k = 1; k <= o->max_newton + 1; ++k) {
      const bool first = (k == 1);
      // R = frac f_ext − f_int(u) on free DOFs
      enqueue_internal_force(c, c->Ap);
      k_residual<<<G_, JFEM_RED_THREADS, 0, c->stream>>>(c->N, c->f_ext, frac, c->Ap, c->mask, c->b, 1, c->part);
      c->launches += 1;
      double rr = 0.0, ff = 0.0;
      if ((rc = read_norms(c, &rr, &ff))) return rc;
      const double rn = std::sqrt(rr);
      double scale = std::sqrt(ff);
      if (!(scale > 0.0)) scale = 1.0;
      if (!(rn == rn)) return set_err(c, JFEM_ERR_NAN, "NaN in the Newton residual");
      last_rel = rn / scale;
      // increment of the prescribed values: carried by the first iteration of the step
      double dgg = 0.0;
      if (first) {
        k_bc_increment<<<G_, JFEM_RED_THREADS, 0, c->stream>>>(c->N, c->gvals, frac, c->u_state, c->mask, dg, c->part);
        c->launches += 1;
        if ((rc = read_norms(c, &dgg, nullptr))) return rc;
      }
      // relative test by default; with tol_absolute the reference's ‖R‖ < newton_tol
      // (ext/JuliaFEMCUDAExt.jl:754,779)
      const double newton_goal = o->tol_absolute ? o->newton_tol : o->newton_tol * scale;
      if ((!first || dgg == 0.0) && rn <= newton_goal) {
        converged = true;
        break;
      }
      if (k > o->max_newton) break;
      // tangent Jacobi diagonal at u, rhs b = R − K_T dg
      if ((rc = jacobi_diag_device(c, c->dinv))) return rc;
      if (dgg > 0.0) {
        enqueue_apply(c, dg, c->tmp, fp32, true, false, nullptr, nullptr, nullptr);
        k_sub_free<<<G_, JFEM_RED_THREADS, 0, c->stream>>>(n, c->b, c->tmp);
        c->launches += 1;
      }
      double eta = std::pow(last_rel, o->forcing_power);
      // An iteration that only carries a prescribed-value increment (‖R‖ = 0)
      // has no residual to scale the forcing term by; solve it to 1e-2 instead
      // of to the floor (Newton corrects the rest in the next iteration).
      if (first && dgg > 0.0 && !(rn > 0.0)) eta = 1e-2;
      if (eta > o->forcing_max) eta = o->forcing_max;
      if (eta < 1e-12) eta = 1e-12;
      cudaMemsetAsync(c->x, 0, n * sizeof(double), c->stream);
      if (fp32 && (rc = nh_state_prepare(c))) return rc;   // tangent point state at u for this Newton step
      PcgResult pr;
      // With a coarse space (the default) the tangent system is solved by the
      // two-level flexible CG: the tangent through the tiled apply, the
      // linear-elastic coarse matrix PᵀKP as the coarse level (an SPD
      // approximation of the tangent's; flexible CG needs no more).  Without
      // one (jfem_set_coarse_space(ctx, 0)): Jacobi-PCG.
      const bool two_level = fp32 && c->coarse_target != 0 && apply_is_tiled(c);
      rc = two_level ? fcg(c, c->b, false, true, eta, o->max_cg_per_newton, o->time_budget_s, t0, true, &pr, 0.01,
                           false, false)
                     : pcg(c, c->b, fp32, eta, o->max_cg_per_newton, o->time_budget_s, t0, false, true, &pr);
      if (rc) {
        if (rc == JFEM_ERR_TIMEOUT) newton_timeout_state(c, u_d, st, total_newton, total_cg + pr.iters, refin, last_rel, t0);
        return rc;
      }
      total_cg += pr.iters;
      refin += pr.refinements;
      ++total_newton;
      k_update_state<<<G_, JFEM_RED_THREADS, 0, c->stream>>>(c->N, c->u_state, c->x, c->gvals, frac, first ? 1 : 0,
                                                            c->mask);
      c->launches += 1;
      ++c->state_version;
      if (st && hist < JFEM_HISTORY_MAX) {
        st->history[3 * hist] = pr.iters;
        st->history[3 * hist + 1] = rn;
        st->history[3 * hist + 2] = eta;
        st->history_len = ++hist;
      }
      if (o->time_budget_s > 0.0 && now_s() - t0 > o->time_budget_s) {
        newton_timeout_state(c, u_d, st, total_newton, total_cg, refin, last_rel, t0);
        return set_err(c, JFEM_ERR_TIMEOUT, "solve exceeded its time budget");
      }
    }
    if (!converged) status = JFEM_NOT_CONVERGED;
  }
  cudaMemcpyAsync(u_d, c->u_state, n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
  if ((rc = sync_and_check(c, "solution copy"))) return rc;
  fill_stats(st, status, total_newton, total_cg, refin, last_rel, now_s() - t0);
  return status;
}

int solve_device(Ctx* c, const jfem_solve_opts* o, double* u_d, jfem_stats* st) {
  if (c->N == 0) return set_err(c, JFEM_ERR_INVALID, "jfem_set_mesh must come first");
  if (!c->have_material) return set_err(c, JFEM_ERR_INVALID, "jfem_set_material must come first");
  if (!o) return set_err(c, JFEM_ERR_INVALID, "opts is NULL");
  if (!(o->tol > 0.0) || o->max_iter <= 0) return set_err(c, JFEM_ERR_INVALID, "tol must be > 0 and max_iter > 0");
  if (o->method == JFEM_NEWTON && (o->max_newton <= 0 || o->max_cg_per_newton <= 0 || !(o->newton_tol > 0.0)))
    return set_err(c, JFEM_ERR_INVALID, "Newton options must be positive");
  switch (o->method) {
    case JFEM_PCG_JACOBI:
    case JFEM_FCG_LEARNED:
    case JFEM_FCG_TWO_LEVEL: return solve_linear(c, o, u_d, st);
    case JFEM_NEWTON: return solve_newton(c, o, u_d, st);
    default: return set_err(c, JFEM_ERR_INVALID, "unknown solve method");
  }
}

}  // namespace jfem
