// jfem_batch.cu — many small independent linear-elastic Tet4 solves in one
// CUDA-graph-captured solve of persistent launches.
//
// The reference solves one problem per solve! call (src/solvers.jl:273-344,
// ext/JuliaFEMCUDAExt.jl:867-916); a batch of uneven systems there is a loop
// of host round trips.  Here every instance is an independent Jacobi-PCG solve
// owned by one team: a single CTA, or for the largest instances a thread-block
// cluster of 2, 4 or 8 CTAs that share the instance's loops and exchange their
// block sums through distributed shared memory.  Persistent grids of teams take
// instances from device counters in decreasing-size order (longest first), so
// uneven sizes balance across SMs; the cluster launch and the single-CTA launch
// are parallel branches of the graph, and no team ever waits for another.  Per
// instance:
//   * FP32 matrix-free apply (element pass over the instance's elements into a
//     per-element scratch, team barrier, node gather in ascending element
//     order: deterministic) with the same element operator as the main apply;
//   * double-float vectors (jfem_df.cuh) for r, p and the correction δx, an
//     FP64 iterate x, FP64 true residual f − K x (FP64 element apply) at
//     recursive convergence and every time the residual drops by 0.3, as the
//     single-mesh mixed solver does;
//   * fixed-order reductions (block, then cluster rank order), so results are
//     bit-reproducible for a given configuration.
// Per-instance latency comes from %globaltimer around each instance.  Block
// size, CTAs per SM, cluster size and the share of instances on clusters are
// chosen by an autotuner (timed solves of the whole batch, fastest kept).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <numeric>
#include <string>
#include <vector>

#include "jfem_apply_kernels.cuh"
#include "jfem_abi_guard.h"
#include "jfem_tune.h"

namespace jfem {

struct BatchDev {
  int n_inst = 0;
  int64_t N = 0, E = 0;             // totals
  const int64_t* node_off = nullptr;   // [n_inst+1]
  const int64_t* elem_off = nullptr;   // [n_inst+1]
  const int* order = nullptr;          // instances, largest first
  const int* conn = nullptr;           // [4][E] SoA, global node numbers
  const float* g32 = nullptr;          // [11][E] affine records (FP32)
  const double* g64 = nullptr;         // [11][E] (FP64)
  const int* adj_ptr = nullptr;        // [N+1] node → (element << 2 | local), ascending element
  const int* adj = nullptr;
  const uint8_t* mask = nullptr;       // [N]
  const double* f = nullptr;           // [3N]
  double tol = 1e-8;
  int max_iter = 100000;
  double drop = 0.3;
  // scratch / outputs
  float* ye32 = nullptr;               // [E][12]
  double* ye64 = nullptr;              // [E][12]
  double* x = nullptr;                 // [3N] FP64 iterate (the solution)
  double* dinv = nullptr;              // [3N]
  float* dinvf = nullptr;
  float2* dx = nullptr;                // [3N] correction since the last refinement
  float2* r = nullptr;
  float2* p = nullptr;
  float* Ap = nullptr;
  double* r64 = nullptr;
  int* next = nullptr;                 // [2] work counters of the two launches (zeroed before every solve)
  int* iters = nullptr;                // [n_inst]
  int* status = nullptr;
  double* relres = nullptr;
  unsigned long long* t_ns = nullptr;
};

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ bool dfree3(const uint8_t* mask, int64_t node, int c) { return !((mask[node] >> c) & 1); }

// The CTAs that solve one instance: one CTA (C = 1), or the C CTAs of a thread-
// block cluster.  Loops over the instance's elements, nodes and DOFs are
// strided over all C·blockDim threads; sync() is a block barrier (C = 1) or a
// cluster barrier with release/acquire order (global writes before it are
// visible to every CTA of the cluster after it); sum() adds one value per CTA
// in rank order through distributed shared memory, so every CTA gets the same,
// deterministic total.  Nothing spins: cluster barriers are hardware barriers.
__device__ __forceinline__ int cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return (int)r;
}
template <typename T>
__device__ __forceinline__ T dsmem_load(const T* p, int rank);
template <>
__device__ __forceinline__ double dsmem_load<double>(const double* p, int rank) {
  unsigned ra;
  double v;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(smem_u32(p)), "r"(rank));
  asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(v) : "r"(ra) : "memory");
  return v;
}
template <>
__device__ __forceinline__ int dsmem_load<int>(const int* p, int rank) {
  unsigned ra;
  int v;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(ra) : "r"(smem_u32(p)), "r"(rank));
  asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(v) : "r"(ra) : "memory");
  return v;
}

template <int C>
struct Team {
  int rank = 0;
  double* xch = nullptr;   // __shared__ double[2]: this CTA's published partial, double-buffered
  int par = 0;
  __device__ __forceinline__ int64_t tid() const { return (int64_t)rank * blockDim.x + threadIdx.x; }
  __device__ __forceinline__ int64_t nthr() const { return (int64_t)C * blockDim.x; }
  __device__ __forceinline__ void sync() const {
    if constexpr (C == 1) {
      __syncthreads();
    } else {
      __threadfence();
      __syncwarp();   // the .aligned barrier wants converged warps (callers may follow a thread-0 branch)
      asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
    }
  }
  // v: this CTA's value (the same in all its threads) → Σ over the team's CTAs
  __device__ __forceinline__ double sum(double v) {
    if constexpr (C == 1) {
      return v;
    } else {
      if (threadIdx.x == 0) xch[par] = v;
      sync();
      double s = 0.0;
#pragma unroll
      for (int r = 0; r < C; ++r) s += dsmem_load(xch + par, r);
      par ^= 1;   // the next sum writes the other slot: every CTA has read this one before passing that sum's barrier
      return s;
    }
  }
};

// y = K v over the instance's elements (FP32: v double-float; FP64: v double)
// into ye, then the node gather into out (masked).  Returns Σ v·out over the
// instance (double-float products for FP32) when want_dot.
template <bool FP32, int C>
__device__ double batch_apply(const BatchDev& a, Team<C>& tm, int64_t n0, int64_t n1, int64_t e0, int64_t e1,
                              const float2* v2, const double* v64, float* out32, double* out64, bool want_dot,
                              double* sh) {
  constexpr int ET = JFEM_TET4;
  for (int64_t e = e0 + tm.tid(); e < e1; e += tm.nthr()) {
    int nd[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) nd[i] = __ldg(a.conn + (int64_t)i * a.E + e);
    if (FP32) {
      float dv[4][3], du[4][3], y[4][3];
      float2 h0[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) h0[c] = dfree3(a.mask, nd[0], c) ? v2[3 * (int64_t)nd[0] + c] : make_float2(0.f, 0.f);
#pragma unroll
      for (int i = 1; i < 4; ++i)
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const float2 h = dfree3(a.mask, nd[i], c) ? v2[3 * (int64_t)nd[i] + c] : make_float2(0.f, 0.f);
          dv[i][c] = (h.x - h0[c].x) + (h.y - h0[c].y);
        }
      element_op<ET, float, true, KIN_SMALL, false, 0>(dv, du, GeoGlobal<float>{a.g32 + e, a.E}, y);
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int c = 0; c < 3; ++c) a.ye32[e * 12 + 3 * i + c] = y[i][c];
    } else {
      double dv[4][3], du[4][3], y[4][3];
      double v0[3];
#pragma unroll
      for (int c = 0; c < 3; ++c) v0[c] = dfree3(a.mask, nd[0], c) ? v64[3 * (int64_t)nd[0] + c] : 0.0;
#pragma unroll
      for (int i = 1; i < 4; ++i)
#pragma unroll
        for (int c = 0; c < 3; ++c) dv[i][c] = (dfree3(a.mask, nd[i], c) ? v64[3 * (int64_t)nd[i] + c] : 0.0) - v0[c];
      element_op<ET, double, true, KIN_SMALL, false, 0>(dv, du, GeoGlobal<double>{a.g64 + e, a.E}, y);
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int c = 0; c < 3; ++c) a.ye64[e * 12 + 3 * i + c] = y[i][c];
    }
  }
  tm.sync();
  float2 dot = make_float2(0.f, 0.f);
  double dot64 = 0.0;
  for (int64_t j = n0 + tm.tid(); j < n1; j += tm.nthr()) {
    const int k1 = __ldg(a.adj_ptr + j + 1);
    if (FP32) {
      float s[3] = {0.f, 0.f, 0.f};
      for (int k = __ldg(a.adj_ptr + j); k < k1; ++k) {
        const int pk = __ldg(a.adj + k);
        const float* ye = a.ye32 + (int64_t)(pk >> 2) * 12 + 3 * (pk & 3);
        s[0] += ye[0];
        s[1] += ye[1];
        s[2] += ye[2];
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float sc = dfree3(a.mask, j, c) ? s[c] : 0.f;
        out32[3 * j + c] = sc;
        if (want_dot) dot = df_add(dot, df_mul_f(v2[3 * j + c], sc));
      }
    } else {
      double s[3] = {0.0, 0.0, 0.0};
      for (int k = __ldg(a.adj_ptr + j); k < k1; ++k) {
        const int pk = __ldg(a.adj + k);
        const double* ye = a.ye64 + (int64_t)(pk >> 2) * 12 + 3 * (pk & 3);
        s[0] += ye[0];
        s[1] += ye[1];
        s[2] += ye[2];
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const double sc = dfree3(a.mask, j, c) ? s[c] : 0.0;
        out64[3 * j + c] = sc;
        if (want_dot) dot64 += v64[3 * j + c] * sc;
      }
    }
  }
  double res = 0.0;
  if (want_dot) res = tm.sum(FP32 ? block_sum_df(dot, sh) : block_sum(dot64, sh));
  tm.sync();
  return res;
}

// Jacobi diagonal: per element the (i, c) diagonal of K_e for small strain,
// w(μ(|g_i|² + g_ic²) + λ g_ic²) with g_i = ∇N_i, then a node gather.
template <int C>
__device__ void batch_diag(const BatchDev& a, Team<C>& tm, int64_t n0, int64_t n1, int64_t e0, int64_t e1) {
  constexpr int ET = JFEM_TET4;
  const double w = qp_weight(ET, 0);
  for (int64_t e = e0 + tm.tid(); e < e1; e += tm.nthr()) {
    double iJ[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) iJ[k] = a.g64[(int64_t)k * a.E + e];
    const double lam = a.g64[(int64_t)9 * a.E + e], mu = a.g64[(int64_t)10 * a.E + e];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      double g[3];
#pragma unroll
      for (int d = 0; d < 3; ++d)
        g[d] = iJ[3 * d] * dshape(ET, 0, i, 0) + iJ[3 * d + 1] * dshape(ET, 0, i, 1) + iJ[3 * d + 2] * dshape(ET, 0, i, 2);
      const double gg = g[0] * g[0] + g[1] * g[1] + g[2] * g[2];
#pragma unroll
      for (int c = 0; c < 3; ++c) a.ye64[e * 12 + 3 * i + c] = w * (mu * (gg + g[c] * g[c]) + lam * g[c] * g[c]);
    }
  }
  tm.sync();
  for (int64_t j = n0 + tm.tid(); j < n1; j += tm.nthr()) {
    double s[3] = {0.0, 0.0, 0.0};
    const int k1 = __ldg(a.adj_ptr + j + 1);
    for (int k = __ldg(a.adj_ptr + j); k < k1; ++k) {
      const int pk = __ldg(a.adj + k);
      const double* ye = a.ye64 + (int64_t)(pk >> 2) * 12 + 3 * (pk & 3);
      s[0] += ye[0];
      s[1] += ye[1];
      s[2] += ye[2];
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const double d = (dfree3(a.mask, j, c) && s[c] > 0.0) ? 1.0 / s[c] : 0.0;
      a.dinv[3 * j + c] = d;
      a.dinvf[3 * j + c] = (float)d;
    }
  }
  tm.sync();
}

// r_rec → FP64 true residual: x += δx, r64 = f − K x (masked); returns
// (‖r64‖², ‖r64 − r_rec‖²) and replaces r by r64 (double-float).
template <int C>
__device__ void batch_refine(const BatchDev& a, Team<C>& tm, int64_t n0, int64_t n1, int64_t e0, int64_t e1,
                             double* sh, double* rr_t, double* drift2) {
  for (int64_t q = 3 * n0 + tm.tid(); q < 3 * n1; q += tm.nthr()) {
    a.x[q] += df_to_double(a.dx[q]);
    a.dx[q] = make_float2(0.f, 0.f);
  }
  tm.sync();
  batch_apply<false>(a, tm, n0, n1, e0, e1, nullptr, a.x, nullptr, a.r64, false, sh);
  double s1 = 0.0, s2 = 0.0;
  for (int64_t q = 3 * n0 + tm.tid(); q < 3 * n1; q += tm.nthr()) {
    const bool fr = dfree3(a.mask, q / 3, (int)(q % 3));
    const double v = fr ? a.f[q] - a.r64[q] : 0.0;
    const double d = v - df_to_double(a.r[q]);
    s1 += v * v;
    s2 += d * d;
    a.r[q] = df_from_double(v);
  }
  *rr_t = tm.sum(block_sum(s1, sh));
  *drift2 = tm.sum(block_sum(s2, sh));
}

// z = D⁻¹ r (double-float), optionally p = z; returns r·z
template <int C>
__device__ double batch_precond(const BatchDev& a, Team<C>& tm, int64_t n0, int64_t n1, bool restart, double* sh) {
  float2 rz = make_float2(0.f, 0.f);
  for (int64_t q = 3 * n0 + tm.tid(); q < 3 * n1; q += tm.nthr()) {
    const float2 rq = a.r[q];
    const float2 zq = df_mul_f(rq, a.dinvf[q]);
    if (restart) a.p[q] = zq;
    rz = df_add(rz, df_mul(rq, zq));
  }
  return tm.sum(block_sum_df(rz, sh));
}

template <int C>
__device__ void batch_solve_instance(const BatchDev& a, Team<C>& tm, int inst, double* sh) {
  const int64_t n0 = a.node_off[inst], n1 = a.node_off[inst + 1];
  const int64_t e0 = a.elem_off[inst], e1 = a.elem_off[inst + 1];
  batch_diag(a, tm, n0, n1, e0, e1);
  // x = 0 (the batch's prescribed values are zero), r = f on the free DOFs
  double s = 0.0;
  for (int64_t q = 3 * n0 + tm.tid(); q < 3 * n1; q += tm.nthr()) {
    const double v = dfree3(a.mask, q / 3, (int)(q % 3)) ? a.f[q] : 0.0;
    a.x[q] = 0.0;
    a.dx[q] = make_float2(0.f, 0.f);
    a.r[q] = df_from_double(v);
    s += v * v;
  }
  const double bb = tm.sum(block_sum(s, sh));
  int it = 0, status = 0;
  double relres = 0.0;
  if (bb > 0.0) {
    const double goal = a.tol * a.tol * bb;
    double rr_true_last = bb, rr_best = bb;
    double rz = batch_precond(a, tm, n0, n1, true, sh);
    int stalls = 0;
    status = JFEM_NOT_CONVERGED;
    relres = 1.0;
    for (;;) {
      const double pAp = batch_apply<true>(a, tm, n0, n1, e0, e1, a.p, nullptr, a.Ap, nullptr, true, sh);
      const double alpha = rz / pAp;
      const float2 al = df_from_double(alpha), nal = df_neg(al);
      float2 rzn = make_float2(0.f, 0.f), rrn = make_float2(0.f, 0.f);
      for (int64_t q = 3 * n0 + tm.tid(); q < 3 * n1; q += tm.nthr()) {
        a.dx[q] = df_add_abs(a.dx[q], df_mul(al, a.p[q]));
        const float2 rq = df_add(a.r[q], df_mul_f(nal, a.Ap[q]));
        a.r[q] = rq;
        rzn = df_add(rzn, df_mul(rq, df_mul_f(rq, a.dinvf[q])));
        rrn = df_add(rrn, df_mul(rq, rq));
      }
      const double rz_new = tm.sum(block_sum_df(rzn, sh));
      const double rr = tm.sum(block_sum_df(rrn, sh));
      ++it;
      // next direction first: a refinement keeps it (p·r = r·z holds for it)
      const float2 be = df_from_double(rz_new / rz);
      for (int64_t q = 3 * n0 + tm.tid(); q < 3 * n1; q += tm.nthr())
        a.p[q] = df_add(df_mul_f(a.r[q], a.dinvf[q]), df_mul(be, a.p[q]));
      rz = rz_new;
      tm.sync();
      const bool bad = !(rr == rr) || !(pAp > 0.0);
      if (rr <= goal || rr < a.drop * a.drop * rr_true_last || it >= a.max_iter || bad) {
        double rr_t = 0.0, drift2 = 0.0;
        batch_refine(a, tm, n0, n1, e0, e1, sh, &rr_t, &drift2);
        const bool finite = rr_t == rr_t && rr_t < 1e300;
        if (finite && rr_t < rr_best) rr_best = rr_t;
        stalls = (finite && rr_t < 0.25 * rr_true_last) ? 0 : stalls + 1;
        if (finite && rr_t <= goal) {
          status = 0;
          relres = sqrt(rr_t / bb);
          break;
        }
        if (it >= a.max_iter || stalls >= 2 || !finite) {
          relres = sqrt(rr_best / bb);
          break;
        }
        rr_true_last = rr_t;
        rz = batch_precond(a, tm, n0, n1, !(drift2 < 0.01 * rr_t), sh);
      }
    }
  }
  if (tm.rank == 0 && threadIdx.x == 0) {
    a.iters[inst] = it;
    a.status[inst] = status;
    a.relres[inst] = bb > 0.0 ? relres : 0.0;
  }
}

// Persistent solver over the instances order[k_begin..k_end): a team (one CTA,
// or one cluster of C CTAs) takes the next position from the counter and
// solves that instance.
template <int BS, int C>
__global__ void __launch_bounds__(BS) k_batch_pcg(BatchDev a, int* __restrict__ next, int k_begin, int k_end) {
  __shared__ double sh[32];
  __shared__ double xch[2];
  __shared__ int s_k;
  Team<C> tm;
  tm.xch = xch;
  if constexpr (C > 1) tm.rank = cluster_rank();
  for (;;) {
    tm.sync();
    if (tm.rank == 0 && threadIdx.x == 0) s_k = k_begin + atomicAdd(next, 1);
    tm.sync();
    int k;
    if constexpr (C == 1) {
      k = s_k;
    } else {
      k = dsmem_load(&s_k, 0);
      tm.sync();   // every CTA has read rank 0's s_k before it is written again
    }
    if (k >= k_end) break;
    const int inst = a.order[k];
    const unsigned long long t0 = global_ns();
    batch_solve_instance(a, tm, inst, sh);
    tm.sync();
    if (tm.rank == 0 && threadIdx.x == 0) a.t_ns[inst] = global_ns() - t0;
  }
  tm.sync();   // no CTA leaves while another may still read its shared memory
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct BatchHost {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t side = nullptr;             // second branch of the captured solve
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  std::string err;
  // instances (host, FP64)
  std::vector<double> X;           // [N][3]
  std::vector<int> conn;           // [E][4] global node numbers
  std::vector<double> lam, mu;     // [E]
  std::vector<uint8_t> mask;       // [N]
  std::vector<double> f;           // [3N]
  std::vector<int64_t> node_off{0}, elem_off{0};
  bool uploaded = false;
  BatchDev d;
  std::vector<void*> owned;
  cudaGraphExec_t graph = nullptr;
  struct Config {
    int bs = 0, grid = 0;        // single-CTA launch over order[n_large..n_inst)
    int cluster = 1, bs_c = 0;   // cluster launch over order[0..n_large), C CTAs per instance
    int grid_c = 0, n_large = 0;
    int per_sm = 1, frac = 0, per_sm_c = 1;   // how grid, n_large, grid_c were derived (autotuner cache)
    bool operator==(const Config& o) const {
      return bs == o.bs && grid == o.grid && cluster == o.cluster && bs_c == o.bs_c && grid_c == o.grid_c &&
             n_large == o.n_large;
    }
  };
  Config graph_cfg, tuned;
  Config forced;                 // set by jfem_batch_set_config (bs 0: none)
  double tuned_ms = 0.0;
  int tune_source = 0;           // 0 none, 1 autotuned in this object, 2 from the autotuner cache
  int64_t launches = 0;
};

static int bset_err(BatchHost* b, int code, const std::string& m) {
  b->err = m;
  return code;
}

template <typename T>
static int bupload(BatchHost* b, T** dst, const std::vector<T>& src, size_t count = 0) {
  const size_t n = std::max<size_t>(count ? count : src.size(), 1);
  if (cudaMalloc((void**)dst, n * sizeof(T)) != cudaSuccess) return bset_err(b, JFEM_ERR_OOM, "batch buffers");
  b->owned.push_back(*dst);
  if (!src.empty()) cudaMemcpyAsync(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice, b->stream);
  return 0;
}

static void bfree_device(BatchHost* b) {
  cudaStreamSynchronize(b->stream);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
  for (void* p : b->owned) cudaFree(p);
  b->owned.clear();
  b->uploaded = false;
  b->tuned = BatchHost::Config();
}

static int batch_upload(BatchHost* b) {
  if (b->uploaded) return 0;
  bfree_device(b);
  const int n_inst = (int)b->node_off.size() - 1;
  const int64_t N = b->node_off.back(), E = b->elem_off.back();
  if (n_inst <= 0 || N == 0 || E == 0) return bset_err(b, JFEM_ERR_INVALID, "empty batch");
  BatchDev& d = b->d;
  d = BatchDev();
  d.n_inst = n_inst;
  d.N = N;
  d.E = E;
  // adjacency (node → element << 2 | local), ascending element
  std::vector<int> cnt((size_t)N + 1, 0), adj((size_t)E * 4);
  for (int64_t e = 0; e < E; ++e)
    for (int i = 0; i < 4; ++i) cnt[(size_t)b->conn[(size_t)e * 4 + i] + 1]++;
  for (int64_t j = 0; j < N; ++j) cnt[(size_t)j + 1] += cnt[(size_t)j];
  std::vector<int> cur(cnt.begin(), cnt.end() - 1);
  for (int64_t e = 0; e < E; ++e)
    for (int i = 0; i < 4; ++i) {
      const int j = b->conn[(size_t)e * 4 + i];
      adj[(size_t)cur[(size_t)j]++] = (int)((e << 2) | i);
    }
  std::vector<int> soa((size_t)E * 4);
  for (int64_t e = 0; e < E; ++e)
    for (int i = 0; i < 4; ++i) soa[(size_t)i * E + e] = b->conn[(size_t)e * 4 + i];
  std::vector<int> order((size_t)n_inst);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    return (b->elem_off[(size_t)x + 1] - b->elem_off[(size_t)x]) > (b->elem_off[(size_t)y + 1] - b->elem_off[(size_t)y]);
  });
  int rc = 0;
  int64_t *no = nullptr, *eo = nullptr;
  int *ord = nullptr, *cn = nullptr, *ap = nullptr, *aj = nullptr;
  uint8_t* mk = nullptr;
  double *Xd = nullptr, *fd = nullptr, *ld = nullptr, *md = nullptr;
  if ((rc = bupload(b, &no, b->node_off)) || (rc = bupload(b, &eo, b->elem_off)) || (rc = bupload(b, &ord, order)) ||
      (rc = bupload(b, &cn, soa)) || (rc = bupload(b, &ap, cnt)) || (rc = bupload(b, &aj, adj)) ||
      (rc = bupload(b, &mk, b->mask)) || (rc = bupload(b, &Xd, b->X)) || (rc = bupload(b, &fd, b->f)) ||
      (rc = bupload(b, &ld, b->lam)) || (rc = bupload(b, &md, b->mu)))
    return rc;
  d.node_off = no;
  d.elem_off = eo;
  d.order = ord;
  d.conn = cn;
  d.adj_ptr = ap;
  d.adj = aj;
  d.mask = mk;
  d.f = fd;
  std::vector<float> ef;
  std::vector<double> edb;
  std::vector<float2> ef2;
  std::vector<int> ei;
  std::vector<unsigned long long> eu;
  float *g32 = nullptr, *ye32 = nullptr, *dinvf = nullptr, *Ap = nullptr;
  double *g64 = nullptr, *ye64 = nullptr, *x = nullptr, *dinv = nullptr, *r64 = nullptr, *relres = nullptr;
  float2 *dx = nullptr, *r = nullptr, *p = nullptr;
  int *next = nullptr, *iters = nullptr, *status = nullptr;
  unsigned long long* tns = nullptr;
  if ((rc = bupload(b, &g32, ef, (size_t)11 * E)) || (rc = bupload(b, &g64, edb, (size_t)11 * E)) ||
      (rc = bupload(b, &ye32, ef, (size_t)12 * E)) || (rc = bupload(b, &ye64, edb, (size_t)12 * E)) ||
      (rc = bupload(b, &x, edb, (size_t)3 * N)) || (rc = bupload(b, &dinv, edb, (size_t)3 * N)) ||
      (rc = bupload(b, &dinvf, ef, (size_t)3 * N)) || (rc = bupload(b, &dx, ef2, (size_t)3 * N)) ||
      (rc = bupload(b, &r, ef2, (size_t)3 * N)) || (rc = bupload(b, &p, ef2, (size_t)3 * N)) ||
      (rc = bupload(b, &Ap, ef, (size_t)3 * N)) || (rc = bupload(b, &r64, edb, (size_t)3 * N)) ||
      (rc = bupload(b, &next, ei, 2)) || (rc = bupload(b, &iters, ei, (size_t)n_inst)) ||
      (rc = bupload(b, &status, ei, (size_t)n_inst)) || (rc = bupload(b, &relres, edb, (size_t)n_inst)) ||
      (rc = bupload(b, &tns, eu, (size_t)n_inst)))
    return rc;
  d.g32 = g32;
  d.g64 = g64;
  d.ye32 = ye32;
  d.ye64 = ye64;
  d.x = x;
  d.dinv = dinv;
  d.dinvf = dinvf;
  d.dx = dx;
  d.r = r;
  d.p = p;
  d.Ap = Ap;
  d.r64 = r64;
  d.next = next;
  d.iters = iters;
  d.status = status;
  d.relres = relres;
  d.t_ns = tns;
  // geometry records (FP64 prepared, FP32 copy) with the single-mesh kernel
  prepare_geo_tet4_affine(E, cn, Xd, ld, md, g64, g32, b->stream);
  cudaError_t e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return bset_err(b, JFEM_ERR_CUDA, std::string("batch upload: ") + cudaGetErrorString(e));
  b->uploaded = true;
  return 0;
}

template <int BS>
static void launch_single(BatchHost* b, cudaStream_t st, int grid, int k0, int k1) {
  k_batch_pcg<BS, 1><<<grid, BS, 0, st>>>(b->d, b->d.next + 1, k0, k1);
}

template <int BS, int C>
static cudaError_t launch_cluster(BatchHost* b, int grid, int k0, int k1) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(BS);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = b->stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = C;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_batch_pcg<BS, C>, b->d, b->d.next, k0, k1);
}

// Clusters of C CTAs of BS threads the device can hold at once (0: the shape
// cannot be scheduled, so the autotuner skips it).
template <int BS, int C>
static int max_clusters(BatchHost* b, int grid) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(BS);
  cfg.stream = b->stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = C;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, k_batch_pcg<BS, C>, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

static int max_clusters_for(BatchHost* b, int bs, int C, int grid) {
  if (bs == 256) return C == 2 ? max_clusters<256, 2>(b, grid) : C == 4 ? max_clusters<256, 4>(b, grid) : max_clusters<256, 8>(b, grid);
  return C == 2 ? max_clusters<512, 2>(b, grid) : C == 4 ? max_clusters<512, 4>(b, grid) : max_clusters<512, 8>(b, grid);
}

template <int BS>
static cudaError_t launch_cluster_c(BatchHost* b, int C, int grid, int k0, int k1) {
  switch (C) {
    case 2: return launch_cluster<BS, 2>(b, grid, k0, k1);
    case 4: return launch_cluster<BS, 4>(b, grid, k0, k1);
    default: return launch_cluster<BS, 8>(b, grid, k0, k1);
  }
}

// The largest n_large instances (the order is largest first) on clusters and
// the rest on single CTAs, as two branches of the captured graph that run at
// the same time (the side stream forks from and joins back into the main one;
// the two kernels share no data and take work from separate counters).
static int enqueue_batch(BatchHost* b, const BatchHost::Config& cf) {
  cudaMemsetAsync(b->d.next, 0, 2 * sizeof(int), b->stream);
  const bool both = cf.n_large > 0 && cf.n_large < b->d.n_inst;
  cudaStream_t st_single = both ? b->side : b->stream;
  if (both) {
    cudaEventRecord(b->ev_fork, b->stream);
    cudaStreamWaitEvent(b->side, b->ev_fork, 0);
  }
  if (cf.n_large > 0) {
    const cudaError_t e = cf.bs_c == 256 ? launch_cluster_c<256>(b, cf.cluster, cf.grid_c, 0, cf.n_large)
                                         : launch_cluster_c<512>(b, cf.cluster, cf.grid_c, 0, cf.n_large);
    if (e != cudaSuccess) {
      if (both) {   // close the fork so the capture (if any) ends cleanly
        cudaEventRecord(b->ev_join, b->side);
        cudaStreamWaitEvent(b->stream, b->ev_join, 0);
      }
      return bset_err(b, JFEM_ERR_CUDA, std::string("cluster launch: ") + cudaGetErrorString(e));
    }
    b->launches += 1;
  }
  if (cf.n_large < b->d.n_inst) {
    switch (cf.bs) {
      case 128: launch_single<128>(b, st_single, cf.grid, cf.n_large, b->d.n_inst); break;
      case 256: launch_single<256>(b, st_single, cf.grid, cf.n_large, b->d.n_inst); break;
      case 512: launch_single<512>(b, st_single, cf.grid, cf.n_large, b->d.n_inst); break;
      default: launch_single<1024>(b, st_single, cf.grid, cf.n_large, b->d.n_inst); break;
    }
    b->launches += 1;
  }
  if (both) {
    cudaEventRecord(b->ev_join, b->side);
    cudaStreamWaitEvent(b->stream, b->ev_join, 0);
  }
  return 0;
}

static int batch_graph(BatchHost* b, const BatchHost::Config& cf) {
  if (b->graph && b->graph_cfg == cf) return 0;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return bset_err(b, JFEM_ERR_CUDA, "batch capture");
  const int64_t l0 = b->launches;
  const int rc = enqueue_batch(b, cf);
  b->launches = l0;
  e = cudaStreamEndCapture(b->stream, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return bset_err(b, JFEM_ERR_CUDA, "batch capture end");
  e = cudaGraphInstantiate(&b->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return bset_err(b, JFEM_ERR_CUDA, "batch graph instantiate");
  b->graph_cfg = cf;
  return 0;
}

static int batch_run(BatchHost* b, const BatchHost::Config& cf, float* ms) {
  int rc = batch_graph(b, cf);
  if (rc) return rc;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, b->stream);
  cudaError_t e = cudaGraphLaunch(b->graph, b->stream);
  b->launches += (cf.n_large > 0) + (cf.n_large < b->d.n_inst);
  cudaEventRecord(e1, b->stream);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  if (e == cudaSuccess) e = cudaGetLastError();
  float t = 0.f;
  cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess) return bset_err(b, JFEM_ERR_CUDA, std::string("batch solve: ") + cudaGetErrorString(e));
  *ms = t;
  return 0;
}

static int sm_count(int device) {
  int n = 0;
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device);
  return n > 0 ? n : 1;
}

// ---------------------------------------------------------------------------
// autotuner cache: the configuration chosen for a (GPU, element type, batch
// shape) is kept for the process and, when JFEM_AUTOTUNE_CACHE names a file,
// in that file (JSON object, one entry per line) for later processes; entries
// read back are launched only when tune_entry_valid accepts them.  The
// batch shape is bucketed to powers of two: instance count, largest and mean
// instance DOFs.  Entries hold the configuration in relative form (CTAs per SM,
// fraction on clusters), re-derived for the batch at hand.
// ---------------------------------------------------------------------------
static std::mutex g_tune_mu;
static std::map<std::string, TuneEntry> g_tune;
static bool g_tune_loaded = false;

static int pow2_bucket(int64_t v) {
  int k = 0;
  while ((1LL << k) < v && k < 62) ++k;
  return k;
}

static std::string tune_key(const BatchHost* b) {
  cudaDeviceProp prop;
  std::string name = cudaGetDeviceProperties(&prop, b->device) == cudaSuccess ? prop.name : "unknown";
  for (char& ch : name)
    if (ch == '"' || ch == '\\' || ch == '\n') ch = '_';
  const int n = b->d.n_inst;
  int64_t mx = 0, tot = 0;
  for (int k = 0; k < n; ++k) {
    const int64_t dofs = 3 * (b->node_off[(size_t)k + 1] - b->node_off[(size_t)k]);
    mx = std::max(mx, dofs);
    tot += dofs;
  }
  char buf[256];
  std::snprintf(buf, sizeof buf, "%s|tet4|n%d|max%d|mean%d", name.c_str(), pow2_bucket(n), pow2_bucket(mx),
                pow2_bucket(n ? tot / n : 0));
  return buf;
}

static void tune_cache_load_locked() {
  if (g_tune_loaded) return;
  g_tune_loaded = true;
  const char* path = std::getenv("JFEM_AUTOTUNE_CACHE");
  if (!path || !*path) return;
  FILE* fp = std::fopen(path, "r");
  if (!fp) return;
  char line[1024];
  while (std::fgets(line, sizeof line, fp)) {
    char key[512];
    TuneEntry e;
    if (std::sscanf(line, " \"%511[^\"]\": {\"bs\": %d, \"per_sm\": %d, \"cluster\": %d, \"bs_c\": %d, "
                          "\"frac\": %d, \"per_sm_c\": %d, \"ms\": %lf}",
                    key, &e.bs, &e.per_sm, &e.cluster, &e.bs_c, &e.frac, &e.per_sm_c, &e.ms) == 8 &&
        tune_entry_valid(e))
      g_tune[key] = e;
  }
  std::fclose(fp);
}

static void tune_cache_store_locked() {
  const char* path = std::getenv("JFEM_AUTOTUNE_CACHE");
  if (!path || !*path) return;
  const std::string tmp = std::string(path) + ".tmp";
  FILE* fp = std::fopen(tmp.c_str(), "w");
  if (!fp) return;
  std::fprintf(fp, "{\n");
  size_t k = 0;
  for (const auto& kv : g_tune) {
    const TuneEntry& e = kv.second;
    std::fprintf(fp, "  \"%s\": {\"bs\": %d, \"per_sm\": %d, \"cluster\": %d, \"bs_c\": %d, \"frac\": %d, "
                     "\"per_sm_c\": %d, \"ms\": %.6f}%s\n",
                 kv.first.c_str(), e.bs, e.per_sm, e.cluster, e.bs_c, e.frac, e.per_sm_c, e.ms,
                 ++k < g_tune.size() ? "," : "");
  }
  std::fprintf(fp, "}\n");
  std::fclose(fp);
  std::rename(tmp.c_str(), path);
}

// Times the whole batch for every candidate configuration and keeps the
// fastest (ties to the earlier, simpler one): single-CTA teams for all
// instances at block sizes 128–1024 and 1/2/4 CTAs per SM; then the largest
// 1/8, 1/4 or 1/2 of the instances on clusters of 2, 4 or 8 CTAs (block 256 or
// 512, one or two cluster CTAs per SM) running beside the rest on single CTAs
// of the best size above.  A configuration cached for the same GPU and batch
// shape is taken instead when its cluster shape can be scheduled here.
static int batch_autotune(BatchHost* b) {
  if (b->tuned.bs) return 0;
  const int sms = sm_count(b->device);
  const int n = b->d.n_inst;
  const std::string key = tune_key(b);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    tune_cache_load_locked();
    auto it = g_tune.find(key);
    if (it != g_tune.end()) {
      const TuneEntry& e = it->second;
      BatchHost::Config cf;
      cf.bs = e.bs;
      cf.per_sm = e.per_sm;
      cf.grid = std::min(n, sms * e.per_sm);
      const int nl = e.frac > 0 ? n / e.frac : 0;
      if (e.cluster > 1 && nl >= 1) {
        cf.cluster = e.cluster;
        cf.bs_c = e.bs_c;
        cf.frac = e.frac;
        cf.per_sm_c = e.per_sm_c;
        cf.n_large = nl;
        cf.grid_c = std::min(nl, e.per_sm_c * sms / e.cluster) * e.cluster;
      }
      if (cf.bs && (cf.n_large == 0 || max_clusters_for(b, cf.bs_c, cf.cluster, cf.grid_c) >= 1)) {
        b->tuned = cf;
        b->tuned_ms = e.ms;
        b->tune_source = 2;
        return 0;
      }
    }
  }
  float best = 1e30f;
  auto try_cfg = [&](const BatchHost::Config& cf) -> int {
    float ms = 0.f;
    const int rc = batch_run(b, cf, &ms);
    if (rc) return rc;
    if (ms < best) {
      best = ms;
      b->tuned = cf;
    }
    return 0;
  };
  for (int bs : {128, 256, 512, 1024})
    for (int k : {1, 2, 4}) {
      if (bs * k > 2048) continue;
      BatchHost::Config cf;
      cf.bs = bs;
      cf.per_sm = k;
      cf.grid = std::min(n, sms * k);
      if (int rc = try_cfg(cf)) return rc;
    }
  const BatchHost::Config single = b->tuned;
  for (int frac : {8, 4, 2})
    for (int C : {2, 4, 8})
      for (int bs_c : {256, 512})
        for (int per_sm : {1, 2}) {
          const int nl = n / frac;
          if (nl < 1 || sms < C) continue;
          BatchHost::Config cf = single;
          cf.cluster = C;
          cf.bs_c = bs_c;
          cf.n_large = nl;
          cf.frac = frac;
          cf.per_sm_c = per_sm;
          cf.grid_c = std::min(nl, per_sm * sms / C) * C;
          if (max_clusters_for(b, bs_c, C, cf.grid_c) < 1) continue;   // shape not schedulable here
          if (try_cfg(cf)) {   // a cluster shape the launch refused: keep the configurations that ran
            cudaGetLastError();
            b->err.clear();
          }
        }
  b->tuned_ms = best;
  b->tune_source = 1;
  {
    const BatchHost::Config& t = b->tuned;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune[key] = TuneEntry{t.bs, t.per_sm, t.n_large > 0 ? t.cluster : 1, t.n_large > 0 ? t.bs_c : 0,
                            t.n_large > 0 ? t.frac : 0, t.n_large > 0 ? t.per_sm_c : 1, (double)best};
    tune_cache_store_locked();
  }
  return 0;
}

}  // namespace jfem

using jfem::BatchHost;

struct jfem_batch {
  BatchHost b;
};

extern "C" {

int jfem_batch_create(jfem_batch** out, int device) {
  ABI_TRY
  if (!out) return JFEM_ERR_INVALID;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return JFEM_ERR_CUDA;
  if (device < 0 || device >= ndev) return JFEM_ERR_INVALID;
  if (cudaSetDevice(device) != cudaSuccess) return JFEM_ERR_CUDA;
  jfem_batch* h = new (std::nothrow) jfem_batch();
  if (!h) return JFEM_ERR_OOM;
  h->b.device = device;
  if (cudaStreamCreateWithFlags(&h->b.stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&h->b.side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->b.ev_fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->b.ev_join, cudaEventDisableTiming) != cudaSuccess) {
    if (h->b.stream) cudaStreamDestroy(h->b.stream);
    if (h->b.side) cudaStreamDestroy(h->b.side);
    if (h->b.ev_fork) cudaEventDestroy(h->b.ev_fork);
    if (h->b.ev_join) cudaEventDestroy(h->b.ev_join);
    delete h;
    return JFEM_ERR_CUDA;
  }
  *out = h;
  return JFEM_OK;
  ABI_CATCH(nullptr)
}

int jfem_batch_destroy(jfem_batch* h) {
  ABI_TRY
  if (!h) return JFEM_OK;
  cudaSetDevice(h->b.device);
  jfem::bfree_device(&h->b);
  if (h->b.stream) cudaStreamDestroy(h->b.stream);
  if (h->b.side) cudaStreamDestroy(h->b.side);
  if (h->b.ev_fork) cudaEventDestroy(h->b.ev_fork);
  if (h->b.ev_join) cudaEventDestroy(h->b.ev_join);
  delete h;
  return JFEM_OK;
  ABI_CATCH(nullptr)
}

const char* jfem_batch_last_error(const jfem_batch* h) { return h ? h->b.err.c_str() : "null batch"; }

int jfem_batch_add(jfem_batch* h, int64_t n_nodes, const double* X, int64_t n_elem, const int64_t* conn,
                   int index_base, double E, double nu, int64_t n_fixed, const int64_t* fixed_dofs,
                   int64_t n_faces, const int64_t* face_conn, const double* t) {
  ABI_TRY
  if (!h) return JFEM_ERR_INVALID;
  BatchHost* b = &h->b;
  if (n_nodes <= 0 || n_elem <= 0 || !X || !conn) return jfem::bset_err(b, JFEM_ERR_INVALID, "empty instance");
  if (!(E > 0.0) || !(nu > -1.0 && nu < 0.5)) return jfem::bset_err(b, JFEM_ERR_INVALID, "invalid material");
  if ((n_fixed > 0 && !fixed_dofs) || (n_faces > 0 && (!face_conn || !t)))
    return jfem::bset_err(b, JFEM_ERR_INVALID, "NULL array");
  const int64_t N0 = b->node_off.back(), E0 = b->elem_off.back();
  if (N0 + n_nodes > INT32_MAX / 2 || (E0 + n_elem) * 4 > INT32_MAX)
    return jfem::bset_err(b, JFEM_ERR_INVALID, "batch too large for 32-bit indices");
  for (int64_t k = 0; k < 4 * n_elem; ++k) {
    const int64_t v = conn[k] - index_base;
    if (v < 0 || v >= n_nodes) return jfem::bset_err(b, JFEM_ERR_INVALID, "connectivity out of range");
  }
  for (int64_t e = 0; e < n_elem; ++e) {   // det J = det[X1−X0; X2−X0; X3−X0] > 0
    double J[3][3];
    const int64_t n0 = conn[4 * e] - index_base;
    for (int a = 0; a < 3; ++a)
      for (int d = 0; d < 3; ++d) J[a][d] = X[3 * (conn[4 * e + a + 1] - index_base) + d] - X[3 * n0 + d];
    const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                       J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                       J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    if (!(det > 0.0)) return jfem::bset_err(b, JFEM_ERR_NEG_JACOBIAN, "element with non-positive Jacobian determinant");
  }
  for (int64_t k = 0; k < n_fixed; ++k) {
    const int64_t v = fixed_dofs[k] - index_base;
    if (v < 0 || v >= 3 * n_nodes) return jfem::bset_err(b, JFEM_ERR_INVALID, "fixed DOF out of range");
  }
  for (int64_t k = 0; k < 3 * n_faces; ++k) {
    const int64_t v = face_conn[k] - index_base;
    if (v < 0 || v >= n_nodes) return jfem::bset_err(b, JFEM_ERR_INVALID, "face connectivity out of range");
  }
  // The instance is appended to the batch's host arrays; if an append runs out
  // of memory they are cut back to their previous lengths, so the batch never
  // holds half an instance.
  const size_t nX = b->X.size(), nconn = b->conn.size(), nlam = b->lam.size(), nmu = b->mu.size(),
               nmask = b->mask.size(), nf = b->f.size(), nnode = b->node_off.size(), nelem = b->elem_off.size();
  try {
    b->X.insert(b->X.end(), X, X + 3 * n_nodes);
    for (int64_t k = 0; k < 4 * n_elem; ++k) b->conn.push_back((int)(N0 + conn[k] - index_base));
    const double lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu)), mu = E / (2.0 * (1.0 + nu));
    b->lam.insert(b->lam.end(), (size_t)n_elem, lam);
    b->mu.insert(b->mu.end(), (size_t)n_elem, mu);
    std::vector<uint8_t> mk((size_t)n_nodes, 0);
    for (int64_t k = 0; k < n_fixed; ++k) {
      const int64_t v = fixed_dofs[k] - index_base;
      mk[(size_t)(v / 3)] |= (uint8_t)(1u << (v % 3));
    }
    b->mask.insert(b->mask.end(), mk.begin(), mk.end());
    // consistent load of a constant traction on Tri3 faces: area/3 per node
    // (src/problems_elasticity.jl:454-502 with the 1-point rule, exact here)
    std::vector<double> f((size_t)3 * n_nodes, 0.0);
    for (int64_t k = 0; k < n_faces; ++k) {
      int64_t nd[3];
      for (int i = 0; i < 3; ++i) nd[i] = face_conn[3 * k + i] - index_base;
      double u[3], v[3];
      for (int d = 0; d < 3; ++d) {
        u[d] = X[3 * nd[1] + d] - X[3 * nd[0] + d];
        v[d] = X[3 * nd[2] + d] - X[3 * nd[0] + d];
      }
      const double cx = u[1] * v[2] - u[2] * v[1], cy = u[2] * v[0] - u[0] * v[2], cz = u[0] * v[1] - u[1] * v[0];
      const double area = 0.5 * std::sqrt(cx * cx + cy * cy + cz * cz);
      for (int i = 0; i < 3; ++i)
        for (int d = 0; d < 3; ++d) f[(size_t)(3 * nd[i] + d)] += area / 3.0 * t[3 * k + d];
    }
    b->f.insert(b->f.end(), f.begin(), f.end());
    b->node_off.push_back(N0 + n_nodes);
    b->elem_off.push_back(E0 + n_elem);
  } catch (...) {
    b->X.resize(nX);
    b->conn.resize(nconn);
    b->lam.resize(nlam);
    b->mu.resize(nmu);
    b->mask.resize(nmask);
    b->f.resize(nf);
    b->node_off.resize(nnode);
    b->elem_off.resize(nelem);
    throw;
  }
  b->uploaded = false;
  return (int)(b->node_off.size() - 2);
  ABI_CATCH(h ? &h->b.err : nullptr)
}

int jfem_batch_solve(jfem_batch* h, double tol, int max_iter, int block_size, double* u, int* iterations,
                     int* status, double* residual, double* latency_s, double* solve_s) {
  ABI_TRY
  if (!h) return JFEM_ERR_INVALID;
  BatchHost* b = &h->b;
  if (cudaSetDevice(b->device) != cudaSuccess) return jfem::bset_err(b, JFEM_ERR_CUDA, "cudaSetDevice");
  if (!(tol > 0.0) || max_iter <= 0) return jfem::bset_err(b, JFEM_ERR_INVALID, "tol and max_iter must be positive");
  if (block_size != 0 && block_size != 128 && block_size != 256 && block_size != 512 && block_size != 1024)
    return jfem::bset_err(b, JFEM_ERR_INVALID, "block_size must be 0 (autotune), 128, 256, 512 or 1024");
  int rc = jfem::batch_upload(b);
  if (rc) return rc;
  if (b->d.tol != tol || b->d.max_iter != max_iter) {   // the captured launch holds these by value
    b->d.tol = tol;
    b->d.max_iter = max_iter;
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    b->tuned = BatchHost::Config();
  }
  BatchHost::Config cf;
  const int sms = jfem::sm_count(b->device);
  if (block_size == 0 && b->forced.bs) {
    cf = b->forced;
    cf.n_large = std::min(cf.n_large, b->d.n_inst);
    cf.grid = std::min(std::max(b->d.n_inst - cf.n_large, 1), sms * std::max(1, 1024 / cf.bs));
    if (cf.n_large > 0) {
      cf.grid_c = std::min(cf.n_large, std::max(sms / cf.cluster, 1)) * cf.cluster;
      if (jfem::max_clusters_for(b, cf.bs_c, cf.cluster, cf.grid_c) < 1)
        return jfem::bset_err(b, JFEM_ERR_INVALID, "cluster shape cannot be scheduled on this device");
    }
  } else if (block_size == 0) {
    if ((rc = jfem::batch_autotune(b))) return rc;
    cf = b->tuned;
  } else {
    cf.bs = block_size;
    cf.grid = std::min(b->d.n_inst, jfem::sm_count(b->device) * std::max(1, 1024 / block_size));
  }
  float ms = 0.f;
  if ((rc = jfem::batch_run(b, cf, &ms))) return rc;
  const int n = b->d.n_inst;
  std::vector<unsigned long long> tns((size_t)n);
  if (u) cudaMemcpyAsync(u, b->d.x, 3 * b->d.N * sizeof(double), cudaMemcpyDeviceToHost, b->stream);
  if (iterations) cudaMemcpyAsync(iterations, b->d.iters, n * sizeof(int), cudaMemcpyDeviceToHost, b->stream);
  if (status) cudaMemcpyAsync(status, b->d.status, n * sizeof(int), cudaMemcpyDeviceToHost, b->stream);
  if (residual) cudaMemcpyAsync(residual, b->d.relres, n * sizeof(double), cudaMemcpyDeviceToHost, b->stream);
  cudaMemcpyAsync(tns.data(), b->d.t_ns, n * sizeof(unsigned long long), cudaMemcpyDeviceToHost, b->stream);
  cudaError_t e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return jfem::bset_err(b, JFEM_ERR_CUDA, std::string("batch download: ") + cudaGetErrorString(e));
  if (latency_s)
    for (int k = 0; k < n; ++k) latency_s[k] = (double)tns[(size_t)k] * 1e-9;
  if (solve_s) *solve_s = ms * 1e-3;
  return JFEM_OK;
  ABI_CATCH(h ? &h->b.err : nullptr)
}

int jfem_batch_tune_source(const jfem_batch* h) { return h ? h->b.tune_source : JFEM_ERR_INVALID; }

int jfem_batch_config(const jfem_batch* h, int* block_size, int* grid) {
  if (!h) return JFEM_ERR_INVALID;
  const BatchHost::Config& cf = h->b.graph_cfg;
  if (block_size) *block_size = cf.bs;
  if (grid) *grid = cf.grid;
  return JFEM_OK;
}

int jfem_batch_set_config(jfem_batch* h, int block_size, int cluster_size, int n_clustered, int cluster_block) {
  ABI_TRY
  if (!h) return JFEM_ERR_INVALID;
  BatchHost* b = &h->b;
  if (block_size == 0) {
    b->forced = BatchHost::Config();
    return JFEM_OK;
  }
  if (block_size != 128 && block_size != 256 && block_size != 512 && block_size != 1024)
    return jfem::bset_err(b, JFEM_ERR_INVALID, "block_size must be 0 (autotune), 128, 256, 512 or 1024");
  if (cluster_size != 1 && cluster_size != 2 && cluster_size != 4 && cluster_size != 8)
    return jfem::bset_err(b, JFEM_ERR_INVALID, "cluster_size must be 1, 2, 4 or 8");
  if (n_clustered < 0 || (cluster_size > 1 && cluster_block != 256 && cluster_block != 512))
    return jfem::bset_err(b, JFEM_ERR_INVALID, "n_clustered must be >= 0 and cluster_block 256 or 512");
  BatchHost::Config cf;
  cf.bs = block_size;
  cf.cluster = cluster_size;
  cf.n_large = cluster_size > 1 ? n_clustered : 0;
  cf.bs_c = cluster_size > 1 ? cluster_block : 0;
  b->forced = cf;
  return JFEM_OK;
  ABI_CATCH(h ? &h->b.err : nullptr)
}

int jfem_batch_cluster_config(const jfem_batch* h, int* cluster_size, int* n_clustered, int* cluster_block) {
  if (!h) return JFEM_ERR_INVALID;
  const BatchHost::Config& cf = h->b.graph_cfg;
  if (cluster_size) *cluster_size = cf.n_large > 0 ? cf.cluster : 1;
  if (n_clustered) *n_clustered = cf.n_large;
  if (cluster_block) *cluster_block = cf.n_large > 0 ? cf.bs_c : 0;
  return JFEM_OK;
}

}  // extern "C"
