// jfem_mpnn.cu — learned preconditioner: a message-passing network on the mesh
// node graph, its forward, adjoint and gradient kernels, Adam, training-pair
// collection from the solver's own iterates, and the ABI around them.  No
// counterpart in the reference (its CG is unpreconditioned:
// src/backend/cpu.jl:221-254, ext/JuliaFEMCUDAExt.jl:531-577); the semantics
// are those of oracle/mpnn_oracle.py.
//
// Graph: node i's neighbours are the nodes that share an element with it — the
// 3×3-block sparsity pattern (nb_ptr, nbr) without i itself.  N is linear
// message passing, 3 layers of width 32:
//   a_i = (1/deg_i) Σ_{j~i} h_j,   h'_i = Ws h_i + Wn a_i     (3 → 32 → 32 → 32)
//   N(y)_i = mask_i ⊙ (Wo h3_i)                               (32 → 3)
// and the preconditioner is z = D^{-1/2}(y + NᵀN y), y = mask ⊙ D^{-1/2} r:
// symmetric positive definite for any weights, so flexible CG keeps PCG's
// convergence (a non-symmetric or nonlinear learned map loses the Krylov
// acceleration).  Nᵀ is the network's backward-data pass.  Weights are BF16
// (converted to FP32 in shared memory), activations and accumulation FP32.
// Training loss per pair (scaled units, r̃ = D^{1/2} y = K t):
//   ℓ = 1 − (zᵀr̃)² / ((zᵀKz)(tᵀr̃)) = 1 − cos²_K(z, t)
// with K z from the tiled FP32 apply, one apply per pair per step.  Rows are (sample, node) pairs, row-major [B][N][C]; one
// thread per row.  Every reduction (weight gradients, loss) is a fixed-shape
// block partial followed by an in-order sum: training is bit-reproducible.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>
#include <vector>

#include "jfem_common.cuh"
#include "jfem_df.cuh"

namespace jfem {

#define MP_THREADS 128
#define MP_DOT_BLOCKS 32   // blocks per pair of the loss dot products

__device__ __forceinline__ bool dof_free(const uint8_t* mask, int64_t i, int c) { return !((mask[i] >> c) & 1); }

// ---------------------------------------------------------------------------
// forward
// ---------------------------------------------------------------------------
template <int CIN>
__device__ __forceinline__ void load_row(const float* __restrict__ p, float (&h)[CIN]) {
  if constexpr (CIN % 4 == 0) {
    const float4* q = reinterpret_cast<const float4*>(p);
#pragma unroll
    for (int c = 0; c < CIN / 4; ++c) {
      const float4 v = __ldg(q + c);
      h[4 * c] = v.x;
      h[4 * c + 1] = v.y;
      h[4 * c + 2] = v.z;
      h[4 * c + 3] = v.w;
    }
  } else {
#pragma unroll
    for (int c = 0; c < CIN; ++c) h[c] = __ldg(p + c);
  }
}

template <int C>
__device__ __forceinline__ void store_row(float* __restrict__ p, const float (&h)[C]) {
  if constexpr (C % 4 == 0) {
    float4* q = reinterpret_cast<float4*>(p);
#pragma unroll
    for (int c = 0; c < C / 4; ++c) q[c] = make_float4(h[4 * c], h[4 * c + 1], h[4 * c + 2], h[4 * c + 3]);
  } else {
#pragma unroll
    for (int c = 0; c < C; ++c) p[c] = h[c];
  }
}

// mean over the neighbours j ≠ i of rows j of sample block hb
template <int CIN>
__device__ __forceinline__ void neighbour_mean(const float* __restrict__ hb, const int* __restrict__ nb_ptr,
                                               const int* __restrict__ nbr, int64_t i, float (&a)[CIN]) {
#pragma unroll
  for (int c = 0; c < CIN; ++c) a[c] = 0.f;
  const int j0 = __ldg(nb_ptr + i), j1 = __ldg(nb_ptr + i + 1);
  for (int jj = j0; jj < j1; ++jj) {
    const int64_t j = __ldg(nbr + jj);
    if (j == i) continue;
    float hj[CIN];
    load_row<CIN>(hb + j * CIN, hj);
#pragma unroll
    for (int c = 0; c < CIN; ++c) a[c] += hj[c];
  }
  const int deg = j1 - j0 - 1;
  const float id = deg > 0 ? 1.f / (float)deg : 0.f;
#pragma unroll
  for (int c = 0; c < CIN; ++c) a[c] *= id;
}

__device__ __forceinline__ float inv_degree(const int* __restrict__ nb_ptr, int64_t i) {
  const int deg = __ldg(nb_ptr + i + 1) - __ldg(nb_ptr + i) - 1;
  return deg > 0 ? 1.f / (float)deg : 0.f;
}

// One layer over B samples: hout = Ws h + Wn agg(h).  agg (may be null) keeps
// the neighbour means for the weight gradient.
template <int CIN>
__global__ void __launch_bounds__(MP_THREADS) k_mp_layer(int64_t rows, int64_t N, const int* __restrict__ nb_ptr,
                                                         const int* __restrict__ nbr, const float* __restrict__ hin,
                                                         const __nv_bfloat16* __restrict__ Ws,
                                                         const __nv_bfloat16* __restrict__ Wn,
                                                         float* __restrict__ agg, float* __restrict__ hout) {
  __shared__ float ws[MP_W * CIN], wn[MP_W * CIN];
  for (int k = threadIdx.x; k < MP_W * CIN; k += blockDim.x) {
    ws[k] = __bfloat162float(Ws[k]);
    wn[k] = __bfloat162float(Wn[k]);
  }
  __syncthreads();
  for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < rows;
       row += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = row / N, i = row - b * N;
    const float* hb = hin + b * N * CIN;
    float h[CIN], a[CIN];
    load_row<CIN>(hb + i * CIN, h);
    neighbour_mean<CIN>(hb, nb_ptr, nbr, i, a);
    if (agg) store_row<CIN>(agg + row * CIN, a);
    float out[MP_W];
#pragma unroll
    for (int k = 0; k < MP_W; ++k) {
      float s = 0.f;
#pragma unroll
      for (int c = 0; c < CIN; ++c) s = fmaf(ws[k * CIN + c], h[c], fmaf(wn[k * CIN + c], a[c], s));
      out[k] = s;
    }
    store_row<MP_W>(hout + row * MP_W, out);
  }
}

// u = mask ⊙ Wo h3
__global__ void __launch_bounds__(MP_THREADS) k_mp_out(int64_t rows, int64_t N, const float* __restrict__ h3,
                                                       const __nv_bfloat16* __restrict__ Wo,
                                                       const uint8_t* __restrict__ mask, float* __restrict__ u) {
  __shared__ float wo[3 * MP_W];
  for (int k = threadIdx.x; k < 3 * MP_W; k += blockDim.x) wo[k] = __bfloat162float(Wo[k]);
  __syncthreads();
  for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < rows;
       row += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = row % N;
    float h[MP_W];
    load_row<MP_W>(h3 + row * MP_W, h);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      float s = 0.f;
#pragma unroll
      for (int c = 0; c < MP_W; ++c) s = fmaf(wo[k * MP_W + c], h[c], s);
      u[row * 3 + k] = dof_free(mask, i, k) ? s : 0.f;
    }
  }
}

// Block partial of Σ_rows u ⊗ v (KU × KV) from rows staged in shared memory.
template <int KU, int KV>
__device__ __forceinline__ void outer_partial(const float* su, const float* sv, int nrows, float* __restrict__ out) {
  for (int e = threadIdx.x; e < KU * KV; e += blockDim.x) {
    const int k = e / KV, c = e - (e / KV) * KV;
    float s = 0.f;
    for (int r = 0; r < nrows; ++r) s = fmaf(su[r * KU + k], sv[r * KV + c], s);
    out[e] = s;
  }
}

// Output layer backward: dh3 = Woᵀ (mask ⊙ dout); gradient partial of Wo
// (3 × 32) per block when gpart is set.  One row per thread, grid =
// ceil(rows / MP_THREADS) when gpart is set.
__global__ void __launch_bounds__(MP_THREADS) k_mp_bwd_out(int64_t rows, int64_t N, const float* __restrict__ dout,
                                                           const float* __restrict__ h3,
                                                           const __nv_bfloat16* __restrict__ Wo,
                                                           const uint8_t* __restrict__ mask, float* __restrict__ dh3,
                                                           float* __restrict__ gpart) {
  __shared__ float wo[3 * MP_W];
  __shared__ float su[MP_THREADS * 3];
  __shared__ float sv[MP_THREADS * MP_W];
  for (int k = threadIdx.x; k < 3 * MP_W; k += blockDim.x) wo[k] = __bfloat162float(Wo[k]);
  __syncthreads();
  const int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int r = threadIdx.x;
  float g[3] = {0.f, 0.f, 0.f};
  if (row < rows) {
    const int64_t i = row % N;
#pragma unroll
    for (int k = 0; k < 3; ++k) g[k] = dof_free(mask, i, k) ? dout[row * 3 + k] : 0.f;
    float dh[MP_W];
#pragma unroll
    for (int c = 0; c < MP_W; ++c) dh[c] = g[0] * wo[c] + g[1] * wo[MP_W + c] + g[2] * wo[2 * MP_W + c];
    store_row<MP_W>(dh3 + row * MP_W, dh);
  }
  if (!gpart) return;
  float h[MP_W];
  if (row < rows) load_row<MP_W>(h3 + row * MP_W, h);
#pragma unroll
  for (int k = 0; k < 3; ++k) su[r * 3 + k] = g[k];
#pragma unroll
  for (int c = 0; c < MP_W; ++c) sv[r * MP_W + c] = row < rows ? h[c] : 0.f;
  __syncthreads();
  outer_partial<3, MP_W>(su, sv, MP_THREADS, gpart + (int64_t)blockIdx.x * (3 * MP_W));
}

// Hidden layer backward (linear): with dout = ∂/∂hout, the self part of
// ∂/∂hin (Wsᵀ dout → dh_self) and gn = Wnᵀ dout / deg for the neighbour part
// (when NEED_DH); gradient partials of Ws, Wn (Σ dout ⊗ hin, Σ dout ⊗ agg) per
// block when gpart is set.  Dynamic shared memory when gpart is set:
// MP_THREADS × (MP_W + 2·CIN) floats.
template <int CIN, bool NEED_DH>
__global__ void __launch_bounds__(MP_THREADS) k_mp_bwd_layer(int64_t rows, int64_t N, const int* __restrict__ nb_ptr,
                                                             const float* __restrict__ dout,
                                                             const float* __restrict__ hin,
                                                             const float* __restrict__ agg,
                                                             const __nv_bfloat16* __restrict__ Ws,
                                                             const __nv_bfloat16* __restrict__ Wn,
                                                             float* __restrict__ dh_self, float* __restrict__ gn,
                                                             float* __restrict__ gpart) {
  __shared__ float ws[MP_W * CIN], wn[MP_W * CIN];
  extern __shared__ float4 mp_dyn[];
  for (int k = threadIdx.x; k < MP_W * CIN; k += blockDim.x) {
    ws[k] = __bfloat162float(Ws[k]);
    wn[k] = __bfloat162float(Wn[k]);
  }
  __syncthreads();
  const int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int r = threadIdx.x;
  float dp[MP_W];
#pragma unroll
  for (int k = 0; k < MP_W; ++k) dp[k] = 0.f;
  if (row < rows) {
    load_row<MP_W>(dout + row * MP_W, dp);
    if (NEED_DH) {
      const float id = inv_degree(nb_ptr, row % N);
      float ds[CIN], g[CIN];
#pragma unroll
      for (int c = 0; c < CIN; ++c) {
        float s1 = 0.f, s2 = 0.f;
#pragma unroll
        for (int k = 0; k < MP_W; ++k) {
          s1 = fmaf(ws[k * CIN + c], dp[k], s1);
          s2 = fmaf(wn[k * CIN + c], dp[k], s2);
        }
        ds[c] = s1;
        g[c] = s2 * id;
      }
      store_row<CIN>(dh_self + row * CIN, ds);
      store_row<CIN>(gn + row * CIN, g);
    }
  }
  if (!gpart) return;
  float* su = reinterpret_cast<float*>(mp_dyn);
  float* sh_ = su + MP_THREADS * MP_W;
  float* sa = sh_ + MP_THREADS * CIN;
  float h[CIN], a[CIN];
#pragma unroll
  for (int c = 0; c < CIN; ++c) h[c] = a[c] = 0.f;
  if (row < rows) {
    load_row<CIN>(hin + row * CIN, h);
    load_row<CIN>(agg + row * CIN, a);
  }
#pragma unroll
  for (int k = 0; k < MP_W; ++k) su[r * MP_W + k] = dp[k];
#pragma unroll
  for (int c = 0; c < CIN; ++c) {
    sh_[r * CIN + c] = h[c];
    sa[r * CIN + c] = a[c];
  }
  __syncthreads();
  float* gp = gpart + (int64_t)blockIdx.x * (2 * MP_W * CIN);
  outer_partial<MP_W, CIN>(su, sh_, MP_THREADS, gp);
  outer_partial<MP_W, CIN>(su, sa, MP_THREADS, gp + MP_W * CIN);
}

// dh_i = dh_self_i + Σ_{k~i} gn_k  (the transpose of the neighbour mean)
template <int C>
__global__ void __launch_bounds__(MP_THREADS) k_mp_bwd_agg(int64_t rows, int64_t N, const int* __restrict__ nb_ptr,
                                                           const int* __restrict__ nbr,
                                                           const float* __restrict__ dh_self,
                                                           const float* __restrict__ gn, float* __restrict__ dh) {
  for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < rows;
       row += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = row / N, i = row - b * N;
    const float* gb = gn + b * N * C;
    float s[C];
    load_row<C>(dh_self + row * C, s);
    const int j0 = __ldg(nb_ptr + i), j1 = __ldg(nb_ptr + i + 1);
    for (int jj = j0; jj < j1; ++jj) {
      const int64_t j = __ldg(nbr + jj);
      if (j == i) continue;
      float g[C];
      load_row<C>(gb + j * C, g);
#pragma unroll
      for (int c = 0; c < C; ++c) s[c] += g[c];
    }
    store_row<C>(dh + row * C, s);
  }
}

// grad[e] (+)= Σ_blocks gpart[blk][e] in block order (FP64 accumulation)
__global__ void k_mp_grad_reduce(int nblk, int width, const float* __restrict__ gpart, float* __restrict__ grad,
                                 int accumulate) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < width; e += gridDim.x * blockDim.x) {
    double s = accumulate ? (double)grad[e] : 0.0;
    for (int k = 0; k < nblk; ++k) s += (double)gpart[(int64_t)k * width + e];
    grad[e] = (float)s;
  }
}

__global__ void k_mp_adam(int n, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                          float* __restrict__ v, __nv_bfloat16* __restrict__ wbf, float lr, float b1, float b2,
                          float eps, float c1, float c2) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const float gk = g[k];
    const float mk = b1 * m[k] + (1.f - b1) * gk;
    const float vk = b2 * v[k] + (1.f - b2) * gk * gk;
    m[k] = mk;
    v[k] = vk;
    const float wk = w[k] - lr * (mk / c1) / (sqrtf(vk / c2) + eps);
    w[k] = wk;
    wbf[k] = __float2bfloat16_rn(wk);
  }
}

__global__ void k_mp_to_bf16(int n, float* __restrict__ w, __nv_bfloat16* __restrict__ wbf) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const __nv_bfloat16 b = __float2bfloat16_rn(w[k]);
    wbf[k] = b;
    w[k] = __bfloat162float(b);
  }
}

// ---------------------------------------------------------------------------
// loss (energy-norm cosine) and its gradient with respect to z
// ---------------------------------------------------------------------------
// z = mask ⊙ (y + v) / sq (+ cq, the pair's coarse term, when given) of one pair
// as the double-float input of the tiled apply
__global__ void k_mp_zsplit(int64_t n3, const float* __restrict__ y, const float* __restrict__ v,
                            const float* __restrict__ sq, const float* __restrict__ cq, float2* __restrict__ p2) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n3; q += (int64_t)gridDim.x * blockDim.x)
    p2[q] = make_float2(sq[q] > 0.f ? (y[q] + v[q]) / sq[q] + (cq ? cq[q] : 0.f) : 0.f, 0.f);
}

// per pair b = blockIdx.y: partials of a_b = zᵀr̃ = Σ (y + v) y (+ Σ cq sq y) and
// q_b = zᵀKz into dots[(b·gridDim.x + blockIdx.x)·2 + {0, 1}]
__global__ void __launch_bounds__(256) k_mp_cos_dots(int64_t n3, const float* __restrict__ y,
                                                     const float* __restrict__ v, const float* __restrict__ sq,
                                                     const float* __restrict__ cq, const float* __restrict__ kz,
                                                     double* __restrict__ dots) {
  __shared__ double sh[32];
  const int64_t b = blockIdx.y;
  const float* yb = y + b * n3;
  const float* vb = v + b * n3;
  const float* sb = sq + b * n3;
  const float* cb = cq ? cq + b * n3 : nullptr;
  const float* kb = kz + b * n3;
  double a = 0.0, q = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n3; i += (int64_t)gridDim.x * blockDim.x) {
    const double yv = (double)yb[i] + (double)vb[i];
    const double ci = (cb && sb[i] > 0.f) ? (double)cb[i] : 0.0;
    a += yv * (double)yb[i] + ci * (double)sb[i] * (double)yb[i];
    q += (sb[i] > 0.f ? (double)((yb[i] + vb[i]) / sb[i]) + ci : 0.0) * (double)kb[i];
  }
  a = block_sum(a, sh);
  q = block_sum(q, sh);
  if (threadIdx.x == 0) {
    dots[(b * gridDim.x + blockIdx.x) * 2] = a;
    dots[(b * gridDim.x + blockIdx.x) * 2 + 1] = q;
  }
}

// per pair: ℓ_b, and ∂ℓ/∂z = c1 r̃ + c2 Kz with c1 = −2a/(q den), c2 = 2a²/(q² den)
// (× scale) into coef[2b], coef[2b+1]; Σ scale·ℓ_b → dots[2·B·nbx] (one thread,
// pair order)
__global__ void k_mp_cos_coef(int B, int nbx, double* __restrict__ dots, const float* __restrict__ den, float scale,
                              float* __restrict__ coef) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double L = 0.0;
  for (int b = 0; b < B; ++b) {
    double a = 0.0, q = 0.0;
    for (int k = 0; k < nbx; ++k) {
      a += dots[((int64_t)b * nbx + k) * 2];
      q += dots[((int64_t)b * nbx + k) * 2 + 1];
    }
    const double dn = (double)den[b];
    const bool ok = q > 0.0 && dn > 0.0;
    L += ok ? 1.0 - a * a / (q * dn) : 1.0;
    coef[2 * b] = ok ? (float)(-2.0 * a / (q * dn) * scale) : 0.f;
    coef[2 * b + 1] = ok ? (float)(2.0 * a * a / (q * q * dn) * scale) : 0.f;
  }
  dots[(int64_t)2 * B * nbx] = L * (double)scale;
}

// ĝ = D^{-1/2} ∂ℓ/∂z = mask ⊙ (c1 y + c2 Kz / sq)   (r̃ / sq = y)
__global__ void __launch_bounds__(MP_THREADS) k_mp_cos_ghat(int64_t rows, int64_t N, const float* __restrict__ y,
                                                            const float* __restrict__ sq,
                                                            const float* __restrict__ kz,
                                                            const float* __restrict__ coef,
                                                            const uint8_t* __restrict__ mask,
                                                            float* __restrict__ ghat) {
  for (int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; row < rows;
       row += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = row / N, i = row - b * N;
    const float c1 = coef[2 * b], c2 = coef[2 * b + 1];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int64_t q = row * 3 + k;
      ghat[q] = (dof_free(mask, i, k) && sq[q] > 0.f) ? c1 * y[q] + c2 * kz[q] / sq[q] : 0.f;
    }
  }
}

// ---------------------------------------------------------------------------
// training pairs
// ---------------------------------------------------------------------------
// v = D^{-1/2} r on free DOFs; Σ v² partials → part[blockIdx.x]
__global__ void __launch_bounds__(256) k_mp_sample_norm(int64_t N, const double* __restrict__ r,
                                                        const double* __restrict__ dinv,
                                                        const uint8_t* __restrict__ mask, double* __restrict__ part) {
  __shared__ double sh[32];
  double s = 0.0;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < 3 * N; q += (int64_t)gridDim.x * blockDim.x) {
    const double v = dof_free(mask, q / 3, (int)(q % 3)) ? sqrt(dinv[q]) * r[q] : 0.0;
    s += v * v;
  }
  s = block_sum(s, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// y = D^{-1/2} r / s, t = e / s, sq = D^{1/2} (free DOFs; zero elsewhere);
// partials of tᵀr̃ = Σ t sq y (= ‖t‖²_K)
__global__ void __launch_bounds__(256) k_mp_make_sample(int64_t N, const double* __restrict__ r,
                                                        const double* __restrict__ e, const double* __restrict__ dinv,
                                                        const uint8_t* __restrict__ mask, double inv_s,
                                                        float* __restrict__ y, float* __restrict__ t,
                                                        float* __restrict__ sq, double* __restrict__ part) {
  __shared__ double sh[32];
  double s = 0.0;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < 3 * N; q += (int64_t)gridDim.x * blockDim.x) {
    const bool fr = dof_free(mask, q / 3, (int)(q % 3)) && dinv[q] > 0.0;
    const double isq = fr ? sqrt(dinv[q]) : 0.0;
    const double sqq = fr ? 1.0 / isq : 0.0;
    const double tq = fr ? e[q] * inv_s : 0.0;
    const double yq = isq * r[q] * inv_s;
    y[q] = (float)yq;
    t[q] = (float)tq;
    sq[q] = (float)sqq;
    s += tq * sqq * yq;
  }
  s = block_sum(s, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void k_mp_sub(int64_t n, const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ c) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    c[i] = a[i] - b[i];
}

// y = mask ⊙ D^{-1/2} r (FP64 r, for the host-facing preconditioner), one float4 per node
__global__ void k_mp_input_d(int64_t N, const double* __restrict__ r, const double* __restrict__ dinv,
                             const uint8_t* __restrict__ mask, float4* __restrict__ y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    float v[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) v[c] = dof_free(mask, i, c) ? (float)(sqrt(dinv[3 * i + c]) * r[3 * i + c]) : 0.f;
    y[i] = make_float4(v[0], v[1], v[2], 0.f);
  }
}

// z = D^{-1/2} (y + v) (FP64 out)
__global__ void k_mp_precond_out(int64_t N, const float4* __restrict__ y, const float4* __restrict__ v,
                                 const double* __restrict__ dinv, const uint8_t* __restrict__ mask,
                                 double* __restrict__ z) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < 3 * N; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = q / 3;
    const int c = (int)(q % 3);
    const float yq = reinterpret_cast<const float*>(y)[4 * i + c], vq = reinterpret_cast<const float*>(v)[4 * i + c];
    z[q] = dof_free(mask, i, c) ? sqrt(dinv[q]) * ((double)yq + (double)vq) : 0.0;
  }
}

// ---------------------------------------------------------------------------
// inference in polynomial form (3 channels): N y = mask ⊙ Σ_k C_k A^k y and
// Nᵀ u = Σ_k (Aᵀ)^k C_kᵀ u by Horner's rule.  A y_i = invdeg_i Σ_{j~i} y_j;
// Aᵀ g_i = Σ_{j~i} invdeg_j g_j (the node graph is symmetric).
// ---------------------------------------------------------------------------
__global__ void k_mp_invdeg(int64_t N, const int* __restrict__ nb_ptr, float* __restrict__ invdeg) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
    const int deg = nb_ptr[i + 1] - nb_ptr[i] - 1;
    invdeg[i] = deg > 0 ? 1.f / (float)deg : 0.f;
  }
}

__device__ __forceinline__ void mat3_acc(const float* __restrict__ C, bool transpose, const float (&x)[3],
                                         float (&y)[3]) {
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) y[a] = fmaf(transpose ? C[3 * b + a] : C[3 * a + b], x[b], y[a]);
}

// The neighbour sums of the inference kernels: an 8-lane group per node strides
// over the node's row of the graph, each lane taking MP_UNROLL neighbours per
// round — their index loads first, then their 16-byte gathers (mostly L2), so the
// loads overlap instead of forming a chain — and reduces by a fixed xor-shuffle
// tree, so every run gives the same bits.  The group's lanes share the node, so the group mask
// is uniform wherever the loop condition is.  Vectors are one float4 per node;
// the inputs of the adjoint steps carry the neighbour weight 1/deg_j in .w.
#define MP_GL 8
__device__ __forceinline__ unsigned group_mask() {
  return ((1u << MP_GL) - 1u) << (threadIdx.x & (32 - MP_GL));
}

#define MP_UNROLL 4   // neighbours per lane and round: index loads, then gathers, then sums

// float4 held by lane `src` of the 8-lane group, to every lane of the group
__device__ __forceinline__ float4 group_bcast4(float4 v, int src) {
  const unsigned gm = group_mask();
  return make_float4(__shfl_sync(gm, v.x, src, MP_GL), __shfl_sync(gm, v.y, src, MP_GL),
                     __shfl_sync(gm, v.z, src, MP_GL), __shfl_sync(gm, v.w, src, MP_GL));
}
template <bool WEIGHTED>
__device__ __forceinline__ void group_neighbour_sum(const int* __restrict__ nb_ptr, const int* __restrict__ nbr,
                                                    const float4* __restrict__ in, int64_t i, int g, float s[3]) {
  s[0] = s[1] = s[2] = 0.f;
  const int j0 = __ldg(nb_ptr + i), j1 = __ldg(nb_ptr + i + 1);
  for (int base = j0 + g; base < j1; base += MP_GL * MP_UNROLL) {
    int64_t j[MP_UNROLL];
#pragma unroll
    for (int u = 0; u < MP_UNROLL; ++u) {
      const int jj = base + MP_GL * u;
      j[u] = jj < j1 ? (int64_t)__ldg(nbr + jj) : i;   // i itself stands for "no neighbour"
    }
    float4 v[MP_UNROLL];
#pragma unroll
    for (int u = 0; u < MP_UNROLL; ++u) v[u] = j[u] != i ? __ldg(in + j[u]) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int u = 0; u < MP_UNROLL; ++u) {
      const float w = WEIGHTED ? v[u].w : 1.f;
      s[0] = fmaf(w, v[u].x, s[0]);
      s[1] = fmaf(w, v[u].y, s[1]);
      s[2] = fmaf(w, v[u].z, s[2]);
    }
  }
  const unsigned gm = group_mask();
#pragma unroll
  for (int o = MP_GL / 2; o > 0; o >>= 1) {
    s[0] += __shfl_xor_sync(gm, s[0], o, MP_GL);
    s[1] += __shfl_xor_sync(gm, s[1], o, MP_GL);
    s[2] += __shfl_xor_sync(gm, s[2], o, MP_GL);
  }
}

// a = A in (neighbour mean); LAST: also u = mask ⊙ Σ_k C_k A^k y (with y, a1 = A y,
// in = A² y, a = A³ y) and h = C_3ᵀ u, the first Horner term of the adjoint
template <bool LAST>
__global__ void __launch_bounds__(256) k_mp_poly_fwd(int64_t N, const int* __restrict__ nb_ptr,
                                                     const int* __restrict__ nbr, const float* __restrict__ invdeg,
                                                     const float4* __restrict__ in, const float4* __restrict__ y,
                                                     const float4* __restrict__ a1, const float* __restrict__ poly,
                                                     const uint8_t* __restrict__ mask, float4* __restrict__ out,
                                                     float4* __restrict__ h) {
  __shared__ float C[36];
  if (threadIdx.x < 36) C[threadIdx.x] = poly[threadIdx.x];
  __syncthreads();
  const int g = threadIdx.x & (MP_GL - 1);
  const int64_t g0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / MP_GL;
  const int64_t gs = (int64_t)gridDim.x * blockDim.x / MP_GL;
  for (int64_t i = g0; i < N; i += gs) {
    // the epilogue's operands, one per lane, loaded before the neighbour sum so
    // their latency overlaps it: lane 0 1/deg and the mask, lanes 1-3 y, A y, A² y
    float4 pre = make_float4(0.f, 0.f, 0.f, 0.f);
    if (g == 0) pre = make_float4(__ldg(invdeg + i), LAST ? __int_as_float((int)mask[i]) : 0.f, 0.f, 0.f);
    if (LAST) {
      if (g == 1) pre = y[i];
      else if (g == 2) pre = a1[i];
      else if (g == 3) pre = in[i];
    }
    float s[3];
    group_neighbour_sum<false>(nb_ptr, nbr, in, i, g, s);
    float4 y4, a14, a24;
    if (LAST) {
      y4 = group_bcast4(pre, 1);
      a14 = group_bcast4(pre, 2);
      a24 = group_bcast4(pre, 3);
    }
    if (g != 0) continue;
    const float id = pre.x;
    float a[3] = {s[0] * id, s[1] * id, s[2] * id};
    if (!LAST) {
      out[i] = make_float4(a[0], a[1], a[2], 0.f);
    } else {
      const float yv[3] = {y4.x, y4.y, y4.z};
      const float a1v[3] = {a14.x, a14.y, a14.z};
      const float a2v[3] = {a24.x, a24.y, a24.z};
      float u[3] = {0.f, 0.f, 0.f};
      mat3_acc(C, false, yv, u);
      mat3_acc(C + 9, false, a1v, u);
      mat3_acc(C + 18, false, a2v, u);
      mat3_acc(C + 27, false, a, u);
      const unsigned m = (unsigned)__float_as_int(pre.y);
#pragma unroll
      for (int k = 0; k < 3; ++k) u[k] = ((m >> k) & 1) ? 0.f : u[k];
      float hv[3] = {0.f, 0.f, 0.f};
      mat3_acc(C + 27, true, u, hv);
      out[i] = make_float4(u[0], u[1], u[2], 0.f);
      h[i] = make_float4(hv[0], hv[1], hv[2], id);
    }
  }
}

// Horner step of the adjoint: out = C_kᵀ u + Aᵀ g (g.w = 1/deg); out.w = 1/deg_i
// for the next step.  FCG (the last step, out = v = NᵀN y): also block partials
// of Σ D^{-1/2}(y + v)·q_old, flexible CG's β term of the smoother, into
// t1part[block] (fixed order), and with sc flexible CG's β in the last block.
template <bool FCG>
__global__ void __launch_bounds__(256) k_mp_poly_adj(int64_t N, const int* __restrict__ nb_ptr,
                                                     const int* __restrict__ nbr, const float* __restrict__ invdeg,
                                                     const float4* __restrict__ g, const float4* __restrict__ u,
                                                     const float* __restrict__ poly, int k, float4* __restrict__ out,
                                                     const float4* __restrict__ y, const float* __restrict__ dinvf,
                                                     const float* __restrict__ qold, double* __restrict__ t1part,
                                                     SolverScalars* __restrict__ sc, const double* __restrict__ t2,
                                                     int n2) {
  __shared__ float C[9];
  __shared__ double sh[32];
  if (threadIdx.x < 9) C[threadIdx.x] = poly[9 * k + threadIdx.x];
  __syncthreads();
  const int gl = threadIdx.x & (MP_GL - 1);
  const int64_t g0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / MP_GL;
  const int64_t gs = (int64_t)gridDim.x * blockDim.x / MP_GL;
  float2 t1 = make_float2(0.f, 0.f);
  for (int64_t i = g0; i < N; i += gs) {
    // lane 0 loads u and 1/deg before the neighbour sum (their latency overlaps
    // it); the β term's operands follow the sum (loaded earlier, they queue in
    // front of the neighbour gathers on the L1 this pass saturates)
    float4 u4 = make_float4(0.f, 0.f, 0.f, 0.f);
    float idg = 0.f;
    if (gl == 0) {
      u4 = u[i];
      idg = __ldg(invdeg + i);
    }
    float s[3];
    group_neighbour_sum<true>(nb_ptr, nbr, g, i, gl, s);   // every lane of the group holds the sum
    if (!FCG) {
      if (gl != 0) continue;
      const float uv[3] = {u4.x, u4.y, u4.z};
      mat3_acc(C, true, uv, s);
      out[i] = make_float4(s[0], s[1], s[2], idg);
      continue;
    }
    // last step: out_c = s_c + (C_kᵀ u)_c and the β term's component c on lane c
    // (lanes 0-2; lane 3 writes .w), the same fmaf order as a whole-vector
    // product; on one lane the β term's loads and double-float sums made this
    // pass 22 µs slower than a plain step on the 2M-DOF beam, on three 18 µs
    const unsigned gm = group_mask();
    const float u0 = __shfl_sync(gm, u4.x, 0, MP_GL), u1 = __shfl_sync(gm, u4.y, 0, MP_GL),
                u2 = __shfl_sync(gm, u4.z, 0, MP_GL), id = __shfl_sync(gm, idg, 0, MP_GL);
    if (gl > 3) continue;
    const int c = gl < 3 ? gl : 0;
    const float sc_ = gl == 0 ? s[0] : gl == 1 ? s[1] : s[2];
    const float oc = fmaf(C[6 + c], u2, fmaf(C[3 + c], u1, fmaf(C[c], u0, sc_)));
    float* outw = reinterpret_cast<float*>(out + i);
    if (gl == 3) {
      outw[3] = id;
      continue;
    }
    outw[gl] = oc;
    const float yc = reinterpret_cast<const float*>(y)[4 * i + gl];
    t1 = df_add_abs(t1, df_two_prod(sqrtf(dinvf[3 * i + gl]) * (yc + oc), qold[3 * i + gl]));
  }
  if (FCG) {
    const double b = block_sum_df(t1, sh);
    if (threadIdx.x == 0) t1part[blockIdx.x] = b;
    // with sc: the last block forms flexible CG's β (t2: the coarse level's
    // partials from an earlier launch, or none)
    if (sc && arrive_last(&sc->arrive[2])) {
      fcg_beta_last_block(sc, t1part, (int)gridDim.x, t2, n2, sh);
      if (threadIdx.x == 0) sc->arrive[2] = 0;
    }
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

int mpnn_ensure(Ctx* c) {
  if (c->mp && c->mp->ready) return 0;
  if (!c->mp) c->mp = new MpnnState();
  MpnnState* m = c->mp;
  if (!m->w32) {
    if (cudaMalloc(&m->w32, MP_P * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&m->wbf, MP_P * sizeof(__nv_bfloat16)) != cudaSuccess ||
        cudaMalloc(&m->m, MP_P * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&m->v, MP_P * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&m->g, MP_P * sizeof(float)) != cudaSuccess ||
        cudaMalloc(&m->poly, 36 * sizeof(float)) != cudaSuccess)
      return set_err(c, JFEM_ERR_OOM, "network weights");
  }
  return 0;
}

static int upload_weights(Ctx* c, const float* w) {
  MpnnState* m = c->mp;
  cudaMemcpyAsync(m->w32, w, MP_P * sizeof(float), cudaMemcpyHostToDevice, c->stream);
  k_mp_to_bf16<<<grid_for(MP_P, 256), 256, 0, c->stream>>>(MP_P, m->w32, m->wbf);
  cudaMemsetAsync(m->m, 0, MP_P * sizeof(float), c->stream);
  cudaMemsetAsync(m->v, 0, MP_P * sizeof(float), c->stream);
  c->launches += 1;
  m->step = 0;
  m->poly_fresh = false;
  int rc = sync_and_check(c, "network weights");
  if (!rc) m->ready = true;
  return rc;
}

int mpnn_init(Ctx* c, uint64_t seed) {
  int rc = mpnn_ensure(c);
  if (rc) return rc;
  std::vector<float> w(MP_P);
  const int shapes[7][2] = {{MP_W, 3}, {MP_W, 3}, {MP_W, MP_W}, {MP_W, MP_W}, {MP_W, MP_W}, {MP_W, MP_W}, {3, MP_W}};
  uint64_t st = seed;
  int k = 0;
  for (int s = 0; s < 7; ++s) {
    const double lim = 0.5 * std::sqrt(6.0 / (shapes[s][0] + shapes[s][1]));
    for (int q = 0; q < shapes[s][0] * shapes[s][1]; ++q) {
      const double u = (double)(splitmix(st) >> 11) * (1.0 / 9007199254740992.0);
      w[(size_t)k++] = (float)((2.0 * u - 1.0) * lim);
    }
  }
  return upload_weights(c, w.data());
}

int mpnn_set_weights(Ctx* c, const float* w) {
  int rc = mpnn_ensure(c);
  if (rc) return rc;
  return upload_weights(c, w);
}

int mpnn_get_weights(Ctx* c, float* w) {
  if (!c->mp || !c->mp->ready) return set_err(c, JFEM_ERR_INVALID, "no network weights (jfem_mpnn_init first)");
  cudaMemcpyAsync(w, c->mp->w32, MP_P * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
  return sync_and_check(c, "network weights download");
}

// One arena for B samples: two forward passes (a1 3, h1 32, a2 32, h2 32, a3 32,
// h3 32 channels each), scratch dA, dB, gn (32) and y, u, v, ĝ, w, t3a, t3b, Kz (3).
// Every buffer starts on a 256-byte boundary (the 32-channel rows are read and
// written as float4).
int mpnn_ensure_act(Ctx* c, int64_t B) {
  if (c->m_actB >= B) return 0;
  if (c->pcg_graph) {   // a captured solve graph holds the old buffer addresses
    cudaStreamSynchronize(c->stream);
    cudaGraphExecDestroy(c->pcg_graph);
    c->pcg_graph = nullptr;
    c->pcg_graph_key = -1;
  }
  if (c->marena) dfree(c, c->marena);
  c->marena = nullptr;
  const int64_t r = B * c->N;
  auto padded = [&](int64_t ch) { return (r * ch + 63) / 64 * 64; };
  const int64_t per_pass = padded(3) + 5 * padded(MP_W);
  const int64_t total = 2 * per_pass + 3 * padded(MP_W) + 8 * padded(3);
  int rc = dalloc(c, &c->marena, (size_t)total);
  if (rc) return rc;
  float* p = c->marena;
  auto take = [&](int64_t ch) {
    float* q = p;
    p += padded(ch);
    return q;
  };
  MpBufs& b = c->mb;
  for (int k = 0; k < 2; ++k) {
    b.a1[k] = take(3);
    b.h1[k] = take(MP_W);
    b.a2[k] = take(MP_W);
    b.h2[k] = take(MP_W);
    b.a3[k] = take(MP_W);
    b.h3[k] = take(MP_W);
  }
  b.dA = take(MP_W);
  b.dB = take(MP_W);
  b.gn = take(MP_W);
  b.y = take(3);
  b.u = take(3);
  b.v = take(3);
  b.ghat = take(3);
  b.w = take(3);
  b.t3a = take(3);
  b.t3b = take(3);
  b.kz = take(3);
  if (c->mdots) dfree(c, c->mdots);
  if (c->mcoef) dfree(c, c->mcoef);
  rc = dalloc(c, &c->mdots, (size_t)2 * B * MP_DOT_BLOCKS + 1);
  if (!rc) rc = dalloc(c, &c->mcoef, (size_t)2 * B);
  if (rc) return rc;
  c->m_actB = B;
  return 0;
}

static int ensure_gpart(Ctx* c, int64_t nblk) {
  const int64_t need = nblk * (2 * MP_W * MP_W);
  if (c->m_gpart_cap >= need) return 0;
  if (c->mgpart) dfree(c, c->mgpart);
  int rc = dalloc(c, &c->mgpart, (size_t)need);
  if (rc) return rc;
  c->m_gpart_cap = need;
  return 0;
}

// u = N(h0) for B samples; pass k keeps its aggregates (for weight gradients)
// when keep is set.
static void enqueue_forward(Ctx* c, int64_t B, const float* h0, int k, bool keep, float* u) {
  const MpnnState* m = c->mp;
  const MpBufs& b = c->mb;
  const int64_t rows = B * c->N;
  const unsigned g = grid_for(rows, MP_THREADS);
  k_mp_layer<3><<<g, MP_THREADS, 0, c->stream>>>(rows, c->N, c->nb_ptr, c->nbr, h0, m->wbf + MP_W1S,
                                                 m->wbf + MP_W1N, keep ? b.a1[k] : nullptr, b.h1[k]);
  k_mp_layer<MP_W><<<g, MP_THREADS, 0, c->stream>>>(rows, c->N, c->nb_ptr, c->nbr, b.h1[k], m->wbf + MP_W2S,
                                                    m->wbf + MP_W2N, keep ? b.a2[k] : nullptr, b.h2[k]);
  k_mp_layer<MP_W><<<g, MP_THREADS, 0, c->stream>>>(rows, c->N, c->nb_ptr, c->nbr, b.h2[k], m->wbf + MP_W3S,
                                                    m->wbf + MP_W3N, keep ? b.a3[k] : nullptr, b.h3[k]);
  k_mp_out<<<g, MP_THREADS, 0, c->stream>>>(rows, c->N, b.h3[k], m->wbf + MP_WO, c->mask, u);
  c->launches += 4;
}

// Backward through N for B samples with output gradient dout (3 channels).
// With grad (weight gradients of ⟨dout, N(h0)⟩ from the kept pass k, written or
// accumulated into mp->g) and/or din (the input gradient Nᵀ dout).
static void enqueue_backward(Ctx* c, int64_t B, const float* dout, int k, const float* h0, bool grad, bool accumulate,
                             float* din) {
  const MpnnState* m = c->mp;
  const MpBufs& b = c->mb;
  const int64_t rows = B * c->N;
  const unsigned gs = grid_for(rows, MP_THREADS);
  const unsigned nblk = (unsigned)((rows + MP_THREADS - 1) / MP_THREADS);
  float* gp = grad ? c->mgpart : nullptr;
  const int acc = accumulate ? 1 : 0;
  const size_t sm32 = grad ? (size_t)MP_THREADS * (MP_W + 2 * MP_W) * sizeof(float) : 0;
  const size_t sm3 = grad ? (size_t)MP_THREADS * (MP_W + 2 * 3) * sizeof(float) : 0;
  k_mp_bwd_out<<<nblk, MP_THREADS, 0, c->stream>>>(rows, c->N, dout, b.h3[k], m->wbf + MP_WO, c->mask, b.dA, gp);
  if (grad) k_mp_grad_reduce<<<1, 128, 0, c->stream>>>((int)nblk, 3 * MP_W, c->mgpart, m->g + MP_WO, acc);
  // layer 3 (input h2), layer 2 (input h1): dA → dB (self), gn → dA (Σ)
  const float* hin[2] = {b.h2[k], b.h1[k]};
  const float* aggs[2] = {b.a3[k], b.a2[k]};
  const int offs[2] = {MP_W3S, MP_W2S};
  for (int l = 0; l < 2; ++l) {
    k_mp_bwd_layer<MP_W, true><<<nblk, MP_THREADS, sm32, c->stream>>>(
        rows, c->N, c->nb_ptr, b.dA, hin[l], aggs[l], m->wbf + offs[l], m->wbf + offs[l] + MP_W * MP_W, b.dB, b.gn,
        gp);
    if (grad)
      k_mp_grad_reduce<<<16, 128, 0, c->stream>>>((int)nblk, 2 * MP_W * MP_W, c->mgpart, m->g + offs[l], acc);
    k_mp_bwd_agg<MP_W><<<gs, MP_THREADS, 0, c->stream>>>(rows, c->N, c->nb_ptr, c->nbr, b.dB, b.gn, b.dA);
  }
  // layer 1 (input h0, 3 channels)
  if (din) {
    k_mp_bwd_layer<3, true><<<nblk, MP_THREADS, sm3, c->stream>>>(rows, c->N, c->nb_ptr, b.dA, h0, b.a1[k],
                                                                  m->wbf + MP_W1S, m->wbf + MP_W1N, b.t3a, b.t3b, gp);
    k_mp_bwd_agg<3><<<gs, MP_THREADS, 0, c->stream>>>(rows, c->N, c->nb_ptr, c->nbr, b.t3a, b.t3b, din);
  } else {
    k_mp_bwd_layer<3, false><<<nblk, MP_THREADS, sm3, c->stream>>>(rows, c->N, c->nb_ptr, b.dA, h0, b.a1[k],
                                                                   m->wbf + MP_W1S, m->wbf + MP_W1N, nullptr, nullptr,
                                                                   gp);
  }
  if (grad) k_mp_grad_reduce<<<2, 128, 0, c->stream>>>((int)nblk, 2 * MP_W * 3, c->mgpart, m->g + MP_W1S, acc);
  c->launches += 8 + (grad ? 4 : 0) + (din ? 1 : 0);
}

static void set_bwd_smem() {
  static bool done = false;
  if (done) return;
  cudaFuncSetAttribute(k_mp_bwd_layer<MP_W, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)(MP_THREADS * (MP_W + 2 * MP_W) * sizeof(float)));
  done = true;
}

// C_0..C_3 of the polynomial form from the current (BF16-valued) weights, FP64
// on the host; also the per-node mean weights of the mesh.
int mpnn_refresh_poly(Ctx* c) {
  MpnnState* m = c->mp;
  if (!c->invdeg) {
    int rc = dalloc(c, &c->invdeg, (size_t)c->N);
    if (rc) return rc;
    k_mp_invdeg<<<grid_for(c->N, 256), 256, 0, c->stream>>>(c->N, c->nb_ptr, c->invdeg);
    c->launches += 1;
  }
  if (m->poly_fresh) return sync_and_check(c, "aggregation weights");
  std::vector<float> w(MP_P);
  cudaMemcpyAsync(w.data(), m->w32, MP_P * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
  int rc = sync_and_check(c, "network weights");
  if (rc) return rc;
  auto W = [&](int off, int rows, int cols, int r, int col) { return (double)w[(size_t)(off + r * cols + col)]; };
  double C[4][3][3] = {};
  for (int path = 0; path < 8; ++path) {   // bit l set: layer l+1 uses Wn
    // T = X1 (32×3), then X2·T, X3·T, Wo·T
    double T[MP_W][3], U[MP_W][3];
    const int o1 = (path & 1) ? MP_W1N : MP_W1S;
    for (int a = 0; a < MP_W; ++a)
      for (int b = 0; b < 3; ++b) T[a][b] = W(o1, MP_W, 3, a, b);
    const int offs[2] = {(path & 2) ? MP_W2N : MP_W2S, (path & 4) ? MP_W3N : MP_W3S};
    for (int l = 0; l < 2; ++l) {
      for (int a = 0; a < MP_W; ++a)
        for (int b = 0; b < 3; ++b) {
          double s2 = 0.0;
          for (int q = 0; q < MP_W; ++q) s2 += W(offs[l], MP_W, MP_W, a, q) * T[q][b];
          U[a][b] = s2;
        }
      std::memcpy(T, U, sizeof(T));
    }
    const int k = ((path >> 0) & 1) + ((path >> 1) & 1) + ((path >> 2) & 1);
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) {
        double s2 = 0.0;
        for (int q = 0; q < MP_W; ++q) s2 += W(MP_WO, 3, MP_W, a, q) * T[q][b];
        C[k][a][b] += s2;
      }
  }
  float cf[36];
  for (int k = 0; k < 4; ++k)
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) cf[9 * k + 3 * a + b] = (float)C[k][a][b];
  cudaMemcpyAsync(m->poly, cf, sizeof(cf), cudaMemcpyHostToDevice, c->stream);
  rc = sync_and_check(c, "aggregation polynomial");
  if (!rc) m->poly_fresh = true;
  return rc;
}

// v = NᵀN y for one sample in polynomial form (mpnn_refresh_poly first):
// a1 = A y, a2 = A a1, u = mask ⊙ Σ C_k A^k y, then Horner for Nᵀ u.  Uses the
// float4 inference vectors (mpnn_ensure_infer first).
int mpnn_ensure_infer(Ctx* c) {
  if (c->mi) return 0;
  if (c->pcg_graph) {   // a captured solve graph may hold older buffer addresses
    cudaStreamSynchronize(c->stream);
    cudaGraphExecDestroy(c->pcg_graph);
    c->pcg_graph = nullptr;
    c->pcg_graph_key = -1;
  }
  int rc = dalloc(c, &c->mi, (size_t)7 * c->N);
  if (rc) return rc;
  cudaMemsetAsync(c->mi, 0, (size_t)7 * c->N * sizeof(float4), c->stream);
  return 0;
}

int enqueue_mpnn_spd(Ctx* c, const float4* y, float4* v, const float* dinvf, const float* qold, double* t1part,
                     SolverScalars* sc, const double* t2, int n2) {
  const float* P = c->mp->poly;
  // a resident grid (8 CTAs of 256 per SM) striding over the nodes; its block
  // partials are what flexible CG's β sums
  const unsigned g = grid_for(c->N * MP_GL, 256, JFEM_RED_BLOCKS);
  float4 *a1 = c->mi + c->N, *a2 = c->mi + 2 * c->N, *u = c->mi + 3 * c->N, *h = c->mi + 4 * c->N,
         *g2 = c->mi + 5 * c->N;
  k_mp_poly_fwd<false><<<g, 256, 0, c->stream>>>(c->N, c->nb_ptr, c->nbr, c->invdeg, y, nullptr, nullptr, P, c->mask,
                                                  a1, nullptr);
  k_mp_poly_fwd<false><<<g, 256, 0, c->stream>>>(c->N, c->nb_ptr, c->nbr, c->invdeg, a1, nullptr, nullptr, P,
                                                  c->mask, a2, nullptr);
  k_mp_poly_fwd<true><<<g, 256, 0, c->stream>>>(c->N, c->nb_ptr, c->nbr, c->invdeg, a2, y, a1, P, c->mask, u, h);
  // h = C3ᵀu;  g2 = C2ᵀu + Aᵀh;  h = C1ᵀu + Aᵀg2;  v = C0ᵀu + Aᵀh
  k_mp_poly_adj<false><<<g, 256, 0, c->stream>>>(c->N, c->nb_ptr, c->nbr, c->invdeg, h, u, P, 2, g2, nullptr, nullptr,
                                                  nullptr, nullptr, nullptr, nullptr, 0);
  k_mp_poly_adj<false><<<g, 256, 0, c->stream>>>(c->N, c->nb_ptr, c->nbr, c->invdeg, g2, u, P, 1, h, nullptr, nullptr,
                                                  nullptr, nullptr, nullptr, nullptr, 0);
  if (t1part)
    k_mp_poly_adj<true><<<g, 256, 0, c->stream>>>(c->N, c->nb_ptr, c->nbr, c->invdeg, h, u, P, 0, v, y, dinvf, qold,
                                                   t1part, sc, t2, n2);
  else
    k_mp_poly_adj<false><<<g, 256, 0, c->stream>>>(c->N, c->nb_ptr, c->nbr, c->invdeg, h, u, P, 0, v, nullptr,
                                                    nullptr, nullptr, nullptr, nullptr, nullptr, 0);
  c->launches += 6;
  return (int)g;
}

// forward, loss and gradient for B pairs (y, sq [B][N][3], den [B]); the
// gradient of scale·Σ_b ℓ_b lands in mp->g, the loss in *loss_out (if set).
static int train_step(Ctx* c, int64_t B, const float* y, const float* sq, const float* cq, const float* den,
                      float scale, double* loss_out) {
  const int64_t N = c->N, rows = B * N, n3 = 3 * N;
  const int64_t nblk = (rows + MP_THREADS - 1) / MP_THREADS;
  int rc = ensure_gpart(c, nblk);
  if (rc) return rc;
  set_bwd_smem();
  MpBufs& b = c->mb;
  const unsigned gs = grid_for(rows, MP_THREADS);
  // u = N y (pass 0 kept), v = Nᵀ u
  enqueue_forward(c, B, y, 0, true, b.u);
  enqueue_backward(c, B, b.u, 0, y, false, false, b.v);
  // K z per pair, z = (y + v)/sq (FP32 tiled apply)
  for (int64_t k = 0; k < B; ++k) {
    k_mp_zsplit<<<grid_for(n3, 256), 256, 0, c->stream>>>(n3, y + k * n3, b.v + k * n3, sq + k * n3,
                                                          cq ? cq + k * n3 : nullptr, c->p2);
    enqueue_apply_tiled(c, c->p2, c->Apf, true, nullptr, nullptr, nullptr);
    cudaMemcpyAsync(b.kz + k * n3, c->Apf, n3 * sizeof(float), cudaMemcpyDeviceToDevice, c->stream);
    c->launches += 1;
  }
  k_mp_cos_dots<<<dim3(MP_DOT_BLOCKS, (unsigned)B), 256, 0, c->stream>>>(n3, y, b.v, sq, cq, b.kz, c->mdots);
  k_mp_cos_coef<<<1, 32, 0, c->stream>>>((int)B, MP_DOT_BLOCKS, c->mdots, den, scale, c->mcoef);
  k_mp_cos_ghat<<<gs, MP_THREADS, 0, c->stream>>>(rows, N, y, sq, b.kz, c->mcoef, c->mask, b.ghat);
  c->launches += 3;
  // ∂ℓ/∂W = ∂⟨N ĝ, N y⟩/∂W: backward of pass 0 with N ĝ, of pass 1 (on ĝ) with u
  enqueue_forward(c, B, b.ghat, 1, true, b.w);
  enqueue_backward(c, B, b.w, 0, y, true, false, nullptr);
  enqueue_backward(c, B, b.u, 1, b.ghat, true, true, nullptr);
  if (loss_out) {
    double L = 0.0;
    cudaMemcpyAsync(&L, c->mdots + 2 * B * MP_DOT_BLOCKS, sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if ((rc = sync_and_check(c, "training loss"))) return rc;
    *loss_out = L;
  }
  return 0;
}

static double sum_partials_host(Ctx* c, int n) {
  std::vector<double> h((size_t)n);
  cudaMemcpyAsync(h.data(), c->part, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  if (sync_and_check(c, "partials")) return NAN;
  double s = 0.0;
  for (double v : h) s += v;
  return s;
}

// coarse term of a training pair: cq = mask ⊙ P Ec (Ec = A_c⁻¹ Pᵀ r̃ for the
// pair's scaled residual r̃)
__global__ void k_mp_coarse_term(int64_t N, const int* __restrict__ node_agg, const float4* __restrict__ d32,
                                 const float* __restrict__ Ec, const uint8_t* __restrict__ mask,
                                 const double* __restrict__ dinv, float* __restrict__ cq) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < 3 * N; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = q / 3;
    const int k = (int)(q % 3);
    cq[q] = (dof_free(mask, i, k) && dinv[q] > 0.0) ? coarse_prolong(node_agg, d32, Ec, i, k) : 0.f;
  }
}

// r̃ = r / s as double-float (the restriction's input)
__global__ void k_mp_scaled_df(int64_t n, const double* __restrict__ r, double inv_s, float2* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double v = r[i] * inv_s;
    const float hi = (float)v;
    out[i] = make_float2(hi, (float)(v - (double)hi));
  }
}

// Append (y, t, sq, den) — and, for a two-level context, the coarse term cq —
// for one pair (r, e) (device, FP64).
static int append_pair(Ctx* c, const double* r, const double* e) {
  const int64_t n3 = 3 * c->N;
  const bool coarse = c->mp_coarse == 1;
  if (c->mp_pairs >= c->mp_cap || (coarse && !c->mp_c)) {   // grow geometrically
    const int64_t cap = std::max<int64_t>(16, c->mp_pairs >= c->mp_cap ? 2 * c->mp_cap : c->mp_cap);
    float *x = nullptr, *t = nullptr, *d = nullptr, *den = nullptr, *cc = nullptr;
    int rc = dalloc(c, &x, (size_t)cap * n3);
    if (!rc) rc = dalloc(c, &t, (size_t)cap * n3);
    if (!rc) rc = dalloc(c, &d, (size_t)cap * n3);
    if (!rc) rc = dalloc(c, &den, (size_t)cap);
    if (!rc && coarse) rc = dalloc(c, &cc, (size_t)cap * n3);
    if (rc) return rc;
    if (c->mp_pairs) {
      cudaMemcpyAsync(x, c->mp_x, c->mp_pairs * n3 * sizeof(float), cudaMemcpyDeviceToDevice, c->stream);
      cudaMemcpyAsync(t, c->mp_t, c->mp_pairs * n3 * sizeof(float), cudaMemcpyDeviceToDevice, c->stream);
      cudaMemcpyAsync(d, c->mp_d, c->mp_pairs * n3 * sizeof(float), cudaMemcpyDeviceToDevice, c->stream);
      cudaMemcpyAsync(den, c->mp_den, c->mp_pairs * sizeof(float), cudaMemcpyDeviceToDevice, c->stream);
      if (coarse && c->mp_c)
        cudaMemcpyAsync(cc, c->mp_c, c->mp_pairs * n3 * sizeof(float), cudaMemcpyDeviceToDevice, c->stream);
      cudaStreamSynchronize(c->stream);
    }
    if (c->mp_x) {
      dfree(c, c->mp_x);
      dfree(c, c->mp_t);
      dfree(c, c->mp_d);
      dfree(c, c->mp_den);
    }
    if (c->mp_c) dfree(c, c->mp_c);
    c->mp_x = x;
    c->mp_t = t;
    c->mp_d = d;
    c->mp_den = den;
    c->mp_c = cc;
    c->mp_cap = cap;
  }
  k_mp_sample_norm<<<JFEM_RED_BLOCKS, 256, 0, c->stream>>>(c->N, r, c->dinv, c->mask, c->part);
  c->launches += 1;
  const double nf = (double)(n3 - c->n_fixed);
  const double ss = sum_partials_host(c, JFEM_RED_BLOCKS);
  if (!(ss > 0.0) || !(nf > 0.0)) return 0;   // nothing to learn from a zero residual
  const double s = std::sqrt(ss / nf);
  const int64_t k = c->mp_pairs;
  k_mp_make_sample<<<JFEM_RED_BLOCKS, 256, 0, c->stream>>>(c->N, r, e, c->dinv, c->mask, 1.0 / s, c->mp_x + k * n3,
                                                           c->mp_t + k * n3, c->mp_d + k * n3, c->part);
  c->launches += 1;
  const double den = sum_partials_host(c, JFEM_RED_BLOCKS);
  if (!(den > 0.0)) return 0;
  if (coarse) {   // cq = Q r̃ with the current system's coarse operator
    k_mp_scaled_df<<<grid_for(n3, 256), 256, 0, c->stream>>>(n3, r, 1.0 / s, c->rd);
    enqueue_coarse_restrict_solve(c, c->rd, nullptr);
    k_mp_coarse_term<<<grid_for(n3, 256), 256, 0, c->stream>>>(c->N, c->node_agg, c->node_d32, c->Ec, c->mask,
                                                                c->dinv, c->mp_c + k * n3);
    c->launches += 2;
  }
  const float denf = (float)den;
  cudaMemcpyAsync(c->mp_den + k, &denf, sizeof(float), cudaMemcpyHostToDevice, c->stream);
  int rc = sync_and_check(c, "training pair");
  if (rc) return rc;
  c->mp_pairs += 1;
  return 0;
}

// Pairs carry the coarse term when the context's coarse space is on; pairs of
// both kinds are never mixed.
static int pairs_coarse_state(Ctx* c) {
  const int want = c->coarse_target != 0 ? 1 : 0;
  if (c->mp_pairs > 0 && c->mp_coarse != want)
    return set_err(c, JFEM_ERR_INVALID,
                   "training pairs were collected with another coarse-space setting (jfem_mpnn_clear first)");
  c->mp_coarse = want;
  if (want) return coarse_prepare(c);
  return 0;
}

int mpnn_collect(Ctx* c, int max_pairs, double tol) {
  if (max_pairs <= 0) return set_err(c, JFEM_ERR_INVALID, "max_pairs must be positive");
  int rc = geometry_prepare(c);
  if (rc) return rc;
  if ((rc = pairs_coarse_state(c))) return rc;
  const int64_t n3 = 3 * c->N;
  const int max_snaps = max_pairs - 1;   // plus the x = 0 pair
  std::vector<int> snap_iters((size_t)std::max(1, max_snaps));
  double* snaps = nullptr;
  if (max_snaps > 0 && cudaMalloc(&snaps, (size_t)max_snaps * n3 * sizeof(double)) != cudaSuccess)
    return set_err(c, JFEM_ERR_OOM, "iterate snapshots");
  int n_snaps = 0, iters = 0;
  double relres = 0.0;
  rc = pcg_fp64_snapshots(c, c->f_ext, tol, 100000, snaps, max_snaps, &n_snaps, snap_iters.data(), &iters, &relres);
  if (!rc) {
    // c->x = x*; pairs e_k = x* − x_k (x_0 = prescribed values only), r_k = K e_k (masked)
    double* e = c->b;
    for (int k = -1; k < n_snaps && !rc; ++k) {
      if (k < 0) k_mp_sub<<<grid_for(n3, 256), 256, 0, c->stream>>>(n3, c->x, c->gvals, e);
      else k_mp_sub<<<grid_for(n3, 256), 256, 0, c->stream>>>(n3, c->x, snaps + (int64_t)k * n3, e);
      c->launches += 1;
      enqueue_apply(c, e, c->tmp, false, true, true, nullptr, nullptr, nullptr);
      rc = append_pair(c, c->tmp, e);
    }
  }
  if (snaps) cudaFree(snaps);
  return rc ? rc : (int)c->mp_pairs;
}

int mpnn_train(Ctx* c, int epochs, int batch, double lr, uint64_t seed, double* losses) {
  if (!c->mp || !c->mp->ready) return set_err(c, JFEM_ERR_INVALID, "no network weights (jfem_mpnn_init first)");
  if (c->mp_pairs <= 0) return set_err(c, JFEM_ERR_INVALID, "no training pairs (jfem_mpnn_collect first)");
  if (epochs <= 0 || batch <= 0 || !(lr > 0.0)) return set_err(c, JFEM_ERR_INVALID, "epochs, batch, lr must be positive");
  const int64_t B = std::min<int64_t>(batch, c->mp_pairs);
  int rc = geometry_prepare(c);
  if (rc) return rc;
  if ((rc = mpnn_ensure_act(c, B))) return rc;
  MpnnState* m = c->mp;
  const int64_t nb = (c->mp_pairs + B - 1) / B;
  std::vector<int64_t> order((size_t)nb);
  uint64_t st = seed;
  for (int ep = 0; ep < epochs; ++ep) {
    std::iota(order.begin(), order.end(), 0);
    for (int64_t k = nb - 1; k > 0; --k) std::swap(order[(size_t)k], order[(size_t)(splitmix(st) % (uint64_t)(k + 1))]);
    double ep_loss = 0.0;
    for (int64_t q = 0; q < nb; ++q) {
      const int64_t s0 = order[(size_t)q] * B;
      const int64_t Bq = std::min<int64_t>(B, c->mp_pairs - s0);
      const int64_t off = s0 * 3 * c->N;
      double lq = 0.0;
      rc = train_step(c, Bq, c->mp_x + off, c->mp_d + off, c->mp_coarse == 1 ? c->mp_c + off : nullptr, c->mp_den + s0,
                      1.f / (float)Bq, losses ? &lq : nullptr);
      if (rc) return rc;
      m->step += 1;
      const float c1 = 1.f - std::pow(0.9f, (float)m->step), c2 = 1.f - std::pow(0.999f, (float)m->step);
      k_mp_adam<<<grid_for(MP_P, 256), 256, 0, c->stream>>>(MP_P, m->w32, m->g, m->m, m->v, m->wbf, (float)lr, 0.9f,
                                                            0.999f, 1e-8f, c1, c2);
      c->launches += 1;
      if (losses) ep_loss += lq * (double)Bq;
    }
    if (losses) losses[ep] = ep_loss / (double)c->mp_pairs;
  }
  m->poly_fresh = false;
  return sync_and_check(c, "training");
}

int mpnn_loss_grad(Ctx* c, const double* r_h, const double* e_h, double* loss, float* grad) {
  if (!c->mp || !c->mp->ready) return set_err(c, JFEM_ERR_INVALID, "no network weights (jfem_mpnn_init first)");
  int rc = geometry_prepare(c);
  if (rc) return rc;
  if ((rc = jacobi_diag_device(c, c->dinv))) return rc;
  if ((rc = mpnn_ensure_act(c, 1))) return rc;
  const int64_t n3 = 3 * c->N;
  cudaMemcpyAsync(c->tmp, r_h, n3 * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(c->b, e_h, n3 * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  const int64_t keep = c->mp_pairs;   // the pair goes to slot `keep` and is dropped again below
  const int keep_state = c->mp_coarse;
  if ((rc = pairs_coarse_state(c))) return rc;
  if ((rc = append_pair(c, c->tmp, c->b))) return rc;
  if (c->mp_pairs == keep) return set_err(c, JFEM_ERR_INVALID, "zero residual or error");
  const int64_t off = keep * n3;
  double L = 0.0;
  rc = train_step(c, 1, c->mp_x + off, c->mp_d + off, c->mp_coarse == 1 ? c->mp_c + off : nullptr, c->mp_den + keep, 1.f,
                  &L);
  c->mp_pairs = keep;
  if (keep == 0) c->mp_coarse = keep_state;
  if (rc) return rc;
  cudaMemcpyAsync(grad, c->mp->g, MP_P * sizeof(float), cudaMemcpyDeviceToHost, c->stream);
  if ((rc = sync_and_check(c, "gradient"))) return rc;
  *loss = L;
  return 0;
}

int mpnn_precondition(Ctx* c, const double* r_h, double* z_h) {
  if (!c->mp || !c->mp->ready) return set_err(c, JFEM_ERR_INVALID, "no network weights (jfem_mpnn_init first)");
  int rc = geometry_prepare(c);
  if (rc) return rc;
  if ((rc = jacobi_diag_device(c, c->dinv))) return rc;
  if ((rc = mpnn_ensure_infer(c))) return rc;
  if ((rc = mpnn_refresh_poly(c))) return rc;
  const int64_t n3 = 3 * c->N;
  float4* y = c->mi;
  float4* v = c->mi + 6 * c->N;
  cudaMemcpyAsync(c->tmp, r_h, n3 * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  k_mp_input_d<<<grid_for(c->N, 256), 256, 0, c->stream>>>(c->N, c->tmp, c->dinv, c->mask, y);
  enqueue_mpnn_spd(c, y, v);
  k_mp_precond_out<<<grid_for(n3, 256), 256, 0, c->stream>>>(c->N, y, v, c->dinv, c->mask, c->tmp2);
  c->launches += 2;
  cudaMemcpyAsync(z_h, c->tmp2, n3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  return sync_and_check(c, "preconditioner");
}

}  // namespace jfem
