// jfem_noalloc.cu — jfem_apply_noalloc: the matrix-free FP64 apply y = K v for a
// linear-elastic mesh given entirely in device memory, with all of its working
// storage in one fixed, file-scope device array instead of cudaMalloc.
//
// Who needs it: code that drives this library from inside a host application
// that owns the device memory and may not allocate behind its back — a solver
// embedded in a simulation whose memory arena is reserved up front, a Julia
// session whose CUDA memory pool accounts for every byte, a latency-critical
// time-step loop where cudaMalloc/cudaFree can stall the device.  Those callers
// already hold their inputs and outputs in device memory; this entry point needs
// nothing else.
//
// Working storage: g_noalloc_scratch, JFEM_NOALLOC_SCRATCH_BYTES (64 MiB), held
// by every GPU that loads the library until the process exits.  Per call it
// holds the node → element adjacency (rebuilt each call, counts cleared first)
// and the per-element results.  All calls share it and it keeps the previous
// call's contents, so calls that overlap on the GPU (different streams or
// threads without ordering) race; serialise them.  The first call on a device
// resolves the array's device address for that device (cudaGetSymbolAddress);
// make that first call before any stream capture.  Meshes needing more than the
// array holds are rejected with JFEM_ERR_TOO_LARGE.
#include <cstring>
#include <mutex>

#include "jfem_common.cuh"
#include "jfem_abi_guard.h"

namespace jfem {

static __device__ __align__(256) unsigned char g_noalloc_scratch[JFEM_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
void* g_addr[kMaxDevices] = {nullptr};
std::mutex g_addr_mu;

inline size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

struct Layout {
  size_t cnt, cursor, ptr, adj, ye, err, total;
};

Layout layout(int64_t N, int64_t E, int nn) {
  Layout L;
  size_t o = 0;
  L.err = o;    o += align256(sizeof(int));
  L.cnt = o;    o += align256((size_t)(N + 1) * sizeof(int));
  L.cursor = o; o += align256((size_t)N * sizeof(int));
  L.ptr = o;    o += align256((size_t)(N + 1) * sizeof(int));
  L.adj = o;    o += align256((size_t)E * nn * sizeof(unsigned));
  L.ye = o;     o += align256((size_t)E * nn * 3 * sizeof(double));
  L.total = o;
  return L;
}

__global__ void k_na_zero(int* __restrict__ a, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    a[i] = 0;
}

__global__ void k_na_count(const int64_t* __restrict__ conn, int64_t E, int nn, int64_t N, int base,
                           int* __restrict__ cnt, int* __restrict__ err) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < E * nn; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t v = conn[t] - base;
    if (v < 0 || v >= N) {
      atomicCAS(err, 0, JFEM_ERR_INVALID);
      continue;
    }
    atomicAdd(&cnt[v], 1);
  }
}

// single-block exclusive scan of cnt[0..n) into ptr[0..n], ptr[n] = total
__global__ void k_na_scan(const int* __restrict__ cnt, int* __restrict__ ptr, int64_t n) {
  __shared__ long long sh[32];
  __shared__ long long carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int64_t b0 = 0; b0 < n; b0 += blockDim.x) {
    const int64_t i = b0 + threadIdx.x;
    const long long v = i < n ? cnt[i] : 0;
    long long s = v;
    for (int o = 1; o < 32; o <<= 1) {
      const long long t = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += t;
    }
    if (lane == 31) sh[w] = s;
    __syncthreads();
    if (w == 0) {
      long long ws = lane < nw ? sh[lane] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        const long long t = __shfl_up_sync(0xffffffffu, ws, o);
        if (lane >= o) ws += t;
      }
      if (lane < nw) sh[lane] = ws;
    }
    __syncthreads();
    const long long incl = s + (w > 0 ? sh[w - 1] : 0) + carry;
    if (i < n) ptr[i] = (int)(incl - v);
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) ptr[n] = (int)carry;
}

__global__ void k_na_fill(const int64_t* __restrict__ conn, int64_t E, int nn, int64_t N, int base,
                          const int* __restrict__ ptr, int* __restrict__ cursor, unsigned* __restrict__ adj) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < E * nn; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t v = conn[t] - base;
    if (v < 0 || v >= N) continue;
    const int64_t e = t / nn;
    const int a = (int)(t - e * nn);
    adj[ptr[v] + atomicAdd(&cursor[v], 1)] = ((unsigned)e << 4) | (unsigned)a;
  }
}

__global__ void k_na_sort(const int* __restrict__ ptr, unsigned* __restrict__ adj, int64_t N) {
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < N; j += (int64_t)gridDim.x * blockDim.x) {
    const int s = ptr[j], e = ptr[j + 1];
    for (int i = s + 1; i < e; ++i) {
      const unsigned key = adj[i];
      int k = i - 1;
      while (k >= s && adj[k] > key) {
        adj[k + 1] = adj[k];
        --k;
      }
      adj[k + 1] = key;
    }
  }
}

// FP64 element kernel, geometry evaluated per integration point from X.  An
// element whose node numbers fall outside [0, N) or whose material is not
// admissible (E > 0, −1 < ν < 1/2; NaN fails both) is not evaluated: it raises
// JFEM_ERR_INVALID and writes zeros, so no load ever leaves X's or v's bounds.
template <int ET>
__global__ void __launch_bounds__(128) k_na_elem(int64_t E, int64_t N, const int64_t* __restrict__ conn, int base,
                                                 const double* __restrict__ X, const double* __restrict__ Em,
                                                 const double* __restrict__ num, const double* __restrict__ v,
                                                 double* __restrict__ ye, int* __restrict__ err) {
  constexpr int NN = Elem<ET>::NN, NQ = Elem<ET>::NQ;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
    int64_t nodes[NN];
    bool in_range = true;
#pragma unroll
    for (int i = 0; i < NN; ++i) {
      nodes[i] = conn[e * NN + i] - base;
      in_range = in_range && nodes[i] >= 0 && nodes[i] < N;
    }
    const double Ee = Em[e], ne = num[e];
    if (!in_range || !(Ee > 0.0) || !(ne > -1.0 && ne < 0.5)) {
      raise_error(err, JFEM_ERR_INVALID);
#pragma unroll
      for (int i = 0; i < NN; ++i)
#pragma unroll
        for (int c = 0; c < 3; ++c) ye[(int64_t)(3 * i + c) * E + e] = 0.0;
      continue;
    }
    const double lam = Ee * ne / ((1.0 + ne) * (1.0 - 2.0 * ne));
    const double mu = Ee / (2.0 * (1.0 + ne));
    double y[NN][3];
#pragma unroll
    for (int i = 0; i < NN; ++i) y[i][0] = y[i][1] = y[i][2] = 0.0;
    for (int q = 0; q < NQ; ++q) {
      double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
      double G[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
      for (int i = 0; i < NN; ++i) {
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          const double dn = dshape(ET, q, i, a);
#pragma unroll
          for (int b = 0; b < 3; ++b) {
            J[a][b] += dn * X[3 * nodes[i] + b];
            G[b][a] += v[3 * nodes[i] + b] * dn;
          }
        }
      }
      const double det = det3(J);
      if (!(det > 0.0)) {
        atomicCAS(err, 0, JFEM_ERR_NEG_JACOBIAN);
        break;
      }
      double A[3][3];
      adj3(J, A);
      const double id = 1.0 / det;
      double gv[3][3];
      for (int c = 0; c < 3; ++c)
        for (int d = 0; d < 3; ++d) gv[c][d] = (G[c][0] * A[d][0] + G[c][1] * A[d][1] + G[c][2] * A[d][2]) * id;
      const double tr = gv[0][0] + gv[1][1] + gv[2][2];
      double Q[3][3];
      const double w = qp_weight(ET, q);   // w·detJ·J⁻¹ = w·adj(J)
      for (int c = 0; c < 3; ++c) {
        double P[3];
        for (int d = 0; d < 3; ++d) P[d] = mu * (gv[c][d] + gv[d][c]) + (c == d ? lam * tr : 0.0);
        for (int a = 0; a < 3; ++a) Q[c][a] = w * (P[0] * A[0][a] + P[1] * A[1][a] + P[2] * A[2][a]);
      }
#pragma unroll
      for (int i = 0; i < NN; ++i)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          const double dn = dshape(ET, q, i, a);
          y[i][0] += Q[0][a] * dn;
          y[i][1] += Q[1][a] * dn;
          y[i][2] += Q[2][a] * dn;
        }
    }
#pragma unroll
    for (int i = 0; i < NN; ++i)
#pragma unroll
      for (int c = 0; c < 3; ++c) ye[(int64_t)(3 * i + c) * E + e] = y[i][c];
  }
}

__global__ void k_na_gather(int64_t N, int64_t E, int nn, const int* __restrict__ ptr, const unsigned* __restrict__ adj,
                            const double* __restrict__ ye, double* __restrict__ y) {
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < N; j += (int64_t)gridDim.x * blockDim.x) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int t = ptr[j]; t < ptr[j + 1]; ++t) {
      const int64_t e = adj[t] >> 4;
      const int a = (int)(adj[t] & 15u);
      if (e >= E || a >= nn) continue;   // k_na_fill writes only e < E, a < nn; checked all the same
      s0 += ye[(int64_t)(3 * a) * E + e];
      s1 += ye[(int64_t)(3 * a + 1) * E + e];
      s2 += ye[(int64_t)(3 * a + 2) * E + e];
    }
    y[3 * j] = s0;
    y[3 * j + 1] = s1;
    y[3 * j + 2] = s2;
  }
}

// Device address of g_noalloc_scratch on the current device (resolved once per device).
int scratch_address(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return JFEM_ERR_CUDA;
  std::lock_guard<std::mutex> lk(g_addr_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return JFEM_ERR_CUDA;
    g_addr[dev] = p;
  }
  *out = g_addr[dev];
  return 0;
}

}  // namespace
}  // namespace jfem

extern "C" int jfem_apply_noalloc(int elem_type, int64_t n_nodes, const double* X, int64_t n_elem,
                                  const int64_t* conn, int index_base, const double* E, const double* nu,
                                  const double* v, double* y, void* stream) {
  ABI_TRY
  using namespace jfem;
  if (!(elem_type == JFEM_TET4 || elem_type == JFEM_TET10 || elem_type == JFEM_HEX8)) return JFEM_ERR_INVALID;
  if (n_nodes <= 0 || n_elem <= 0 || !X || !conn || !E || !nu || !v || !y) return JFEM_ERR_INVALID;
  if (index_base != 0 && index_base != 1) return JFEM_ERR_INVALID;
  const int nn = elem_type == JFEM_TET4 ? 4 : elem_type == JFEM_TET10 ? 10 : 8;
  if (n_elem >= (1LL << 28) || n_nodes >= (1LL << 30)) return JFEM_ERR_TOO_LARGE;
  const Layout L = layout(n_nodes, n_elem, nn);
  if (L.total > (size_t)JFEM_NOALLOC_SCRATCH_BYTES) return JFEM_ERR_TOO_LARGE;
  void* base = nullptr;
  if (scratch_address(&base)) return JFEM_ERR_CUDA;
  unsigned char* s = (unsigned char*)base;
  int* err = (int*)(s + L.err);
  int* cnt = (int*)(s + L.cnt);
  int* cursor = (int*)(s + L.cursor);
  int* ptr = (int*)(s + L.ptr);
  unsigned* adj = (unsigned*)(s + L.adj);
  double* ye = (double*)(s + L.ye);
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t N = n_nodes, Ne = n_elem;
  // Each launch's own status (cudaLaunchKernelEx), so an error the caller left
  // behind on this thread is neither reported nor cleared here.
  cudaError_t launch_err = cudaSuccess;
  auto launch = [&](auto kernel, unsigned grid, unsigned block, auto... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.stream = st;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, kernel, args...);
    if (launch_err == cudaSuccess) launch_err = e;
  };
  // clear what must start at zero: the error flag, the counts and the fill cursors
  launch(k_na_zero, 1, 32, err, (int64_t)1);
  launch(k_na_zero, grid_for(N + 1, 256), 256, cnt, N + 1);
  launch(k_na_zero, grid_for(N, 256), 256, cursor, N);
  launch(k_na_count, grid_for(Ne * nn, 256), 256, conn, Ne, nn, N, index_base, cnt, err);
  launch(k_na_scan, 1, 1024, (const int*)cnt, ptr, N);
  launch(k_na_fill, grid_for(Ne * nn, 256), 256, conn, Ne, nn, N, index_base, (const int*)ptr, cursor, adj);
  launch(k_na_sort, grid_for(N, 128), 128, (const int*)ptr, adj, N);
  const unsigned ge = grid_for(Ne, 128, 1LL << 30);
  switch (elem_type) {
    case JFEM_TET4: launch(k_na_elem<JFEM_TET4>, ge, 128, Ne, N, conn, index_base, X, E, nu, v, ye, err); break;
    case JFEM_TET10: launch(k_na_elem<JFEM_TET10>, ge, 128, Ne, N, conn, index_base, X, E, nu, v, ye, err); break;
    default: launch(k_na_elem<JFEM_HEX8>, ge, 128, Ne, N, conn, index_base, X, E, nu, v, ye, err); break;
  }
  launch(k_na_gather, grid_for(N, 256), 256, N, Ne, nn, (const int*)ptr, (const unsigned*)adj, (const double*)ye, y);
  int h_err = 0;
  const cudaError_t ce = launch_err == cudaSuccess
                             ? cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost, st)
                             : launch_err;
  const cudaError_t se = cudaStreamSynchronize(st);   // the work launched above has ended either way
  if (ce != cudaSuccess || se != cudaSuccess) return JFEM_ERR_CUDA;
  return h_err;
  ABI_CATCH(nullptr)
}
