// jfem_mesh.cu — device-side mesh preparation: connectivity conversion, the
// node → element adjacency (the reference's NodeToElementsMap,
// src/nodal_assembly_structures.jl:69-87, and the CSR node→elements list of
// ext/JuliaFEMCUDAExt.jl:180-193) and the 3×3-block sparsity pattern of the
// global matrix (the structural pattern produced by the COO push of
// src/sparse/sparse.jl:121-132 followed by sparse()).
//
// Everything here is deterministic: counts use atomics (order-free), lists are
// sorted after filling, and pattern rows are sorted unique node numbers.
#include "jfem_common.cuh"

namespace jfem {

// ---------------------------------------------------------------------------
// scan (exclusive, int32 in → int32 out, int64 total); three phases
// ---------------------------------------------------------------------------
#define SCAN_T 512
#define SCAN_ITEMS 4
#define SCAN_TILE (SCAN_T * SCAN_ITEMS)

__global__ void k_scan_tiles(const int* __restrict__ in, int* __restrict__ out,
                             long long* __restrict__ tile_sum, int64_t n) {
  __shared__ long long sh[SCAN_T / 32];
  const int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)threadIdx.x * SCAN_ITEMS;
  long long v[SCAN_ITEMS];
  long long loc = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    v[k] = (base + k < n) ? (long long)in[base + k] : 0;
    loc += v[k];
  }
  // warp inclusive scan of loc
  long long s = loc;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    long long t = __shfl_up_sync(0xffffffffu, s, o);
    if (lane >= o) s += t;
  }
  if (lane == 31) sh[w] = s;
  __syncthreads();
  if (w == 0) {
    long long ws = (lane < SCAN_T / 32) ? sh[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      long long t = __shfl_up_sync(0xffffffffu, ws, o);
      if (lane >= o) ws += t;
    }
    if (lane < SCAN_T / 32) sh[lane] = ws;
  }
  __syncthreads();
  long long excl = s - loc + (w > 0 ? sh[w - 1] : 0);
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    if (base + k < n) out[base + k] = (int)excl;   // tile-local; fixed up below
    excl += v[k];
  }
  if (threadIdx.x == SCAN_T - 1) tile_sum[blockIdx.x] = excl;
}

__global__ void k_scan_sums(long long* __restrict__ tile_sum, int ntiles, long long* total) {
  // single block: sequential chunks of blockDim, carried prefix
  __shared__ long long sh[32];
  __shared__ long long carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int b0 = 0; b0 < ntiles; b0 += blockDim.x) {
    const int i = b0 + threadIdx.x;
    long long v = (i < ntiles) ? tile_sum[i] : 0;
    long long s = v;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 1; o < 32; o <<= 1) {
      long long t = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += t;
    }
    if (lane == 31) sh[w] = s;
    __syncthreads();
    if (w == 0) {
      const int nw = blockDim.x >> 5;
      long long ws = (lane < nw) ? sh[lane] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        long long t = __shfl_up_sync(0xffffffffu, ws, o);
        if (lane >= o) ws += t;
      }
      if (lane < nw) sh[lane] = ws;
    }
    __syncthreads();
    const long long incl = s + (w > 0 ? sh[w - 1] : 0) + carry;
    if (i < ntiles) tile_sum[i] = incl - v;   // exclusive
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = incl;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void k_scan_add(int* __restrict__ out, const long long* __restrict__ tile_sum, int64_t n,
                           int* overflow) {
  const int64_t i = (int64_t)blockIdx.x * SCAN_TILE + threadIdx.x;
  const long long off = tile_sum[blockIdx.x];
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; ++k) {
    const int64_t j = i + (int64_t)k * SCAN_T;
    if (j < n) {
      const long long v = (long long)out[j] + off;
      if (v > 0x7fffffffLL) atomicExch(overflow, 1);
      out[j] = (int)v;
    }
  }
}

int exclusive_scan_i32(Ctx* c, const int* in, int* out, int64_t n, int64_t* total) {
  const int64_t ntiles = (n + SCAN_TILE - 1) / SCAN_TILE;
  long long* ts = nullptr;
  long long* tot = nullptr;
  int* ovf = nullptr;
  if (cudaMalloc(&ts, (ntiles + 1) * sizeof(long long)) != cudaSuccess ||
      cudaMalloc(&tot, sizeof(long long)) != cudaSuccess || cudaMalloc(&ovf, sizeof(int)) != cudaSuccess) {
    cudaFree(ts); cudaFree(tot); cudaFree(ovf);
    return set_err(c, JFEM_ERR_OOM, "scan scratch allocation failed");
  }
  cudaMemsetAsync(ovf, 0, sizeof(int), c->stream);
  if (ntiles > 0) {
    k_scan_tiles<<<(unsigned)ntiles, SCAN_T, 0, c->stream>>>(in, out, ts, n);
    k_scan_sums<<<1, 1024, 0, c->stream>>>(ts, (int)ntiles, tot);
    k_scan_add<<<(unsigned)ntiles, SCAN_T, 0, c->stream>>>(out, ts, n, ovf);
    c->launches += 3;
  } else {
    cudaMemsetAsync(tot, 0, sizeof(long long), c->stream);
  }
  long long h_tot = 0;
  int h_ovf = 0;
  cudaMemcpyAsync(&h_tot, tot, sizeof(long long), cudaMemcpyDeviceToHost, c->stream);
  cudaMemcpyAsync(&h_ovf, ovf, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  int rc = sync_and_check(c, "scan");
  cudaFree(ts);
  cudaFree(tot);
  cudaFree(ovf);
  if (rc) return rc;
  if (h_ovf || h_tot > 0x7fffffffLL) return set_err(c, JFEM_ERR_INVALID, "index range exceeds int32");
  *total = h_tot;
  return 0;
}

// ---------------------------------------------------------------------------
// connectivity / coordinates
// ---------------------------------------------------------------------------
__global__ void k_conn_soa(const int64_t* __restrict__ conn64, int* __restrict__ conn, int64_t E, int nn,
                           int64_t N, int base, int* err) {
  const int64_t total = E * nn;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = t / nn;
    const int a = (int)(t - e * nn);
    const int64_t v = conn64[t] - base;
    if (v < 0 || v >= N) {
      raise_error(err, JFEM_ERR_INVALID);
      conn[(int64_t)a * E + e] = 0;
    } else {
      conn[(int64_t)a * E + e] = (int)v;
    }
  }
}

__global__ void k_coords32(const double* __restrict__ X, float4* __restrict__ X32, int64_t N) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x)
    X32[i] = make_float4((float)X[3 * i], (float)X[3 * i + 1], (float)X[3 * i + 2], 0.f);
}

// ---------------------------------------------------------------------------
// adjacency (node → (item << 4 | local)), generic over elements and faces
// ---------------------------------------------------------------------------
__global__ void k_adj_count(const int* __restrict__ conn, int64_t M, int nper, int* __restrict__ cnt) {
  const int64_t total = M * nper;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&cnt[conn[t]], 1);   // conn SoA: t = a*M + e
}

__global__ void k_adj_fill(const int* __restrict__ conn, int64_t M, int nper, const int* __restrict__ ptr,
                           int* __restrict__ cursor, unsigned* __restrict__ adj) {
  const int64_t total = M * nper;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int a = (int)(t / M);
    const int64_t e = t - (int64_t)a * M;
    const int node = conn[t];
    const int pos = ptr[node] + atomicAdd(&cursor[node], 1);
    adj[pos] = ((unsigned)e << 4) | (unsigned)a;
  }
}

__global__ void k_adj_sort(const int* __restrict__ ptr, unsigned* __restrict__ adj, int64_t N,
                           int* __restrict__ amax) {
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
    atomicMax(amax, e - s);
  }
}

// Neighbour lists.  FILL = false: count unique neighbours; true: write them and
// the slot map.
template <bool FILL>
__global__ void __launch_bounds__(128) k_neighbours(const int* __restrict__ conn, int64_t E, int nn,
                                                    const int* __restrict__ adj_ptr,
                                                    const unsigned* __restrict__ adj, int64_t N,
                                                    int* __restrict__ nb_cnt, const int* __restrict__ nb_ptr,
                                                    int* __restrict__ nbr, uint16_t* __restrict__ slot,
                                                    int* __restrict__ dmax, int* err) {
  int list[JFEM_MAX_NEIGHBOURS];
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < N; j += (int64_t)gridDim.x * blockDim.x) {
    int cnt = 0;
    bool over = false;
    const int s = adj_ptr[j], t1 = adj_ptr[j + 1];
    for (int t = s; t < t1 && !over; ++t) {
      const int64_t e = adj[t] >> 4;
      for (int b = 0; b < nn; ++b) {
        const int v = conn[(int64_t)b * E + e];
        // binary search in sorted list[0, cnt)
        int lo = 0, hi = cnt;
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (list[mid] < v) lo = mid + 1; else hi = mid;
        }
        if (lo < cnt && list[lo] == v) continue;
        if (cnt >= JFEM_MAX_NEIGHBOURS) { over = true; break; }
        for (int k = cnt; k > lo; --k) list[k] = list[k - 1];
        list[lo] = v;
        ++cnt;
      }
    }
    if (over) {
      raise_error(err, JFEM_ERR_INVALID);
      if (!FILL) nb_cnt[j] = 0;
      continue;
    }
    if (!FILL) {
      nb_cnt[j] = cnt;
      atomicMax(dmax, cnt);
    } else {
      const int p0 = nb_ptr[j];
      for (int k = 0; k < cnt; ++k) nbr[p0 + k] = list[k];
      for (int t = s; t < t1; ++t) {
        const int64_t e = adj[t] >> 4;
        for (int b = 0; b < nn; ++b) {
          const int v = conn[(int64_t)b * E + e];
          int lo = 0, hi = cnt;
          while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (list[mid] < v) lo = mid + 1; else hi = mid;
          }
          slot[(int64_t)t * nn + b] = (uint16_t)lo;
        }
      }
    }
  }
}

static int build_adjacency(Ctx* c, const int* conn, int64_t M, int nper, int** ptr_out,
                           unsigned** adj_out, int* amax_out) {
  const int64_t N = c->N;
  int* cnt = nullptr;
  int* cursor = nullptr;
  int* amax = nullptr;
  int rc = 0;
  if ((rc = dalloc(c, ptr_out, N + 1))) return rc;
  if ((rc = dalloc(c, adj_out, M * nper))) return rc;
  if (cudaMalloc(&cnt, (N + 1) * sizeof(int)) != cudaSuccess || cudaMalloc(&cursor, N * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&amax, sizeof(int)) != cudaSuccess) {
    cudaFree(cnt); cudaFree(cursor); cudaFree(amax);
    return set_err(c, JFEM_ERR_OOM, "adjacency scratch allocation failed");
  }
  cudaMemsetAsync(cnt, 0, (N + 1) * sizeof(int), c->stream);
  cudaMemsetAsync(cursor, 0, N * sizeof(int), c->stream);
  cudaMemsetAsync(amax, 0, sizeof(int), c->stream);
  const int T = 256;
  k_adj_count<<<grid_for(M * nper, T), T, 0, c->stream>>>(conn, M, nper, cnt);
  c->launches += 1;
  int64_t total = 0;
  rc = exclusive_scan_i32(c, cnt, *ptr_out, N + 1, &total);
  if (!rc) {
    k_adj_fill<<<grid_for(M * nper, T), T, 0, c->stream>>>(conn, M, nper, *ptr_out, cursor, *adj_out);
    k_adj_sort<<<grid_for(N, 128), 128, 0, c->stream>>>(*ptr_out, *adj_out, N, amax);
    c->launches += 2;
    cudaMemcpyAsync(amax_out, amax, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    rc = sync_and_check(c, "adjacency");
  }
  cudaFree(cnt);
  cudaFree(cursor);
  cudaFree(amax);
  return rc;
}

static int mesh_build(Ctx* c, int et, int nn, int64_t N, const double* X, int64_t E, const int64_t* conn_h,
                      int base);

int mesh_setup(Ctx* c, int et, int64_t N, const double* X, int64_t E, const int64_t* conn_h, int base) {
  if (!(et == JFEM_TET4 || et == JFEM_TET10 || et == JFEM_HEX8))
    return set_err(c, JFEM_ERR_INVALID, "unsupported element type (4=Tet4, 10=Tet10, 8=Hex8)");
  if (N <= 0 || E <= 0 || !X || !conn_h) return set_err(c, JFEM_ERR_INVALID, "empty mesh");
  if (base != 0 && base != 1) return set_err(c, JFEM_ERR_INVALID, "index_base must be 0 or 1");
  const int nn = et == JFEM_TET4 ? 4 : et == JFEM_TET10 ? 10 : 8;
  if (N > 0x7fffffffLL / 3 || E >= (1LL << 28) || E * nn > 0x7fffffffLL)
    return set_err(c, JFEM_ERR_INVALID, "mesh too large for 32-bit device indices");
  // A failure past this point (a bad node number found on the device, device or
  // host memory exhausted) leaves the context without a mesh, never with a
  // partial one that later calls would read.
  free_mesh(c);
  int rc = 0;
  try {
    rc = mesh_build(c, et, nn, N, X, E, conn_h, base);
  } catch (...) {
    free_mesh(c);
    throw;
  }
  if (rc) free_mesh(c);
  return rc;
}

static int mesh_build(Ctx* c, int et, int nn, int64_t N, const double* X, int64_t E, const int64_t* conn_h,
                      int base) {
  c->et = et;
  c->nn = nn;
  c->N = N;
  c->E = E;
  int rc = 0;
  if ((rc = dalloc(c, &c->d_err, 1))) return rc;
  cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream);
  if ((rc = dalloc(c, &c->X64, 3 * N))) return rc;
  if ((rc = dalloc(c, &c->X32, N))) return rc;
  if ((rc = dalloc(c, &c->conn, E * nn))) return rc;
  int64_t* conn64 = nullptr;
  if (cudaMalloc(&conn64, E * nn * sizeof(int64_t)) != cudaSuccess)
    return set_err(c, JFEM_ERR_OOM, "connectivity upload buffer");
  cudaMemcpyAsync(c->X64, X, 3 * N * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(conn64, conn_h, E * nn * sizeof(int64_t), cudaMemcpyHostToDevice, c->stream);
  k_conn_soa<<<grid_for(E * nn, 256), 256, 0, c->stream>>>(conn64, c->conn, E, nn, N, base, c->d_err);
  k_coords32<<<grid_for(N, 256), 256, 0, c->stream>>>(c->X64, c->X32, N);
  c->launches += 2;
  int h_err = 0;
  cudaMemcpyAsync(&h_err, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  rc = sync_and_check(c, "connectivity upload");
  cudaFree(conn64);
  if (rc) return rc;
  if (h_err) return set_err(c, JFEM_ERR_INVALID, "connectivity refers to a node outside 1..n_nodes");

  if ((rc = build_adjacency(c, c->conn, E, nn, &c->adj_ptr, &c->adj, &c->amax))) return rc;

  // neighbour pattern
  int* nb_cnt = nullptr;
  int* dmax = nullptr;
  if (cudaMalloc(&nb_cnt, (N + 1) * sizeof(int)) != cudaSuccess || cudaMalloc(&dmax, sizeof(int)) != cudaSuccess) {
    cudaFree(nb_cnt); cudaFree(dmax);
    return set_err(c, JFEM_ERR_OOM, "pattern scratch allocation failed");
  }
  cudaMemsetAsync(nb_cnt, 0, (N + 1) * sizeof(int), c->stream);
  cudaMemsetAsync(dmax, 0, sizeof(int), c->stream);
  const int TB = 128;
  k_neighbours<false><<<grid_for(N, TB), TB, 0, c->stream>>>(c->conn, E, nn, c->adj_ptr, c->adj, N, nb_cnt,
                                                             nullptr, nullptr, nullptr, dmax, c->d_err);
  c->launches += 1;
  if ((rc = dalloc(c, &c->nb_ptr, N + 1))) { cudaFree(nb_cnt); cudaFree(dmax); return rc; }
  int64_t nb_total = 0;
  rc = exclusive_scan_i32(c, nb_cnt, c->nb_ptr, N + 1, &nb_total);
  if (!rc) rc = dalloc(c, &c->nbr, nb_total);
  if (!rc) rc = dalloc(c, &c->slot, E * nn * nn);
  if (!rc) {
    k_neighbours<true><<<grid_for(N, TB), TB, 0, c->stream>>>(c->conn, E, nn, c->adj_ptr, c->adj, N, nullptr,
                                                              c->nb_ptr, c->nbr, c->slot, dmax, c->d_err);
    c->launches += 1;
    cudaMemcpyAsync(&c->dmax, dmax, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(&h_err, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    rc = sync_and_check(c, "pattern");
  }
  cudaFree(nb_cnt);
  cudaFree(dmax);
  if (rc) return rc;
  if (h_err) return set_err(c, JFEM_ERR_INVALID, "a node has more than 512 neighbours");
  c->n_blocks = nb_total;

  if ((rc = tiles_build(c, X, conn_h, base))) return rc;

  // per-mesh scratch and solver vectors
  const int64_t n = 3 * N;
  if ((rc = dalloc(c, &c->ye32, E * nn * 3))) return rc;
  if ((rc = dalloc(c, &c->ye64, E * nn * 3))) return rc;
  if ((rc = dalloc(c, &c->mask, N))) return rc;
  if ((rc = dalloc(c, &c->gvals, n))) return rc;
  if ((rc = dalloc(c, &c->f_ext, n))) return rc;
  if ((rc = dalloc(c, &c->u_state, n))) return rc;
  double** vecs[] = {&c->x, &c->r, &c->z, &c->p, &c->Ap, &c->dinv, &c->b, &c->tmp, &c->tmp2, &c->xbest};
  for (double** v : vecs)
    if ((rc = dalloc(c, v, n))) return rc;
  if ((rc = dalloc(c, &c->p2, n))) return rc;
  if ((rc = dalloc(c, &c->xd, n))) return rc;
  if ((rc = dalloc(c, &c->rd, n))) return rc;
  if ((rc = dalloc(c, &c->Apf, n))) return rc;
  if ((rc = dalloc(c, &c->dinvf, n))) return rc;
  if ((rc = dalloc(c, &c->part, JFEM_PART_SIZE))) return rc;
  if ((rc = dalloc(c, &c->sc, 1))) return rc;
  if ((rc = dalloc(c, &c->norms, 2))) return rc;
  cudaMemsetAsync(c->mask, 0, N, c->stream);
  cudaMemsetAsync(c->sc, 0, sizeof(SolverScalars), c->stream);
  cudaMemsetAsync(c->Apf, 0, n * sizeof(float), c->stream);
  cudaMemsetAsync(c->gvals, 0, n * sizeof(double), c->stream);
  cudaMemsetAsync(c->f_ext, 0, n * sizeof(double), c->stream);
  cudaMemsetAsync(c->u_state, 0, n * sizeof(double), c->stream);
  c->n_fixed = 0;
  c->F = 0;
  c->f_ext_dirty = true;
  c->have_state = false;
  c->have_material = false;
  return sync_and_check(c, "mesh scratch");
}

// ---------------------------------------------------------------------------
// faces (surface traction table)
// ---------------------------------------------------------------------------
static void faces_clear(Ctx* c);
static int faces_build(Ctx* c, int64_t F, const int64_t* fconn_h, const double* t_h, const double* p_h, int base);

int faces_setup(Ctx* c, int ft, int64_t F, const int64_t* fconn_h, const double* t_h, const double* p_h,
                int base) {
  if (c->N == 0) return set_err(c, JFEM_ERR_INVALID, "jfem_set_mesh must come first");
  if (!(ft == JFEM_TRI3 || ft == JFEM_TRI6 || ft == JFEM_QUAD4))
    return set_err(c, JFEM_ERR_INVALID, "unsupported face type (3=Tri3, 6=Tri6, 4=Quad4)");
  if (F < 0 || (F > 0 && (!fconn_h || (!t_h && !p_h)))) return set_err(c, JFEM_ERR_INVALID, "bad surface-load arrays");
  if (F >= (1LL << 28)) return set_err(c, JFEM_ERR_INVALID, "too many faces");
  // The previous table is dropped first; a failure past this point leaves the
  // context with no surface load rather than a table later calls would read
  // half-built.
  faces_clear(c);
  c->ft = ft;
  c->nfn = face_nodes(ft);
  if (F == 0) return 0;
  int rc = 0;
  try {
    rc = faces_build(c, F, fconn_h, t_h, p_h, base);
  } catch (...) {
    faces_clear(c);
    throw;
  }
  if (rc) faces_clear(c);
  return rc;
}

static void faces_clear(Ctx* c) {
  if (c->fconn) { dfree(c, c->fconn); c->fconn = nullptr; }
  if (c->ftrac) { dfree(c, c->ftrac); c->ftrac = nullptr; }
  if (c->fadj_ptr) { dfree(c, c->fadj_ptr); c->fadj_ptr = nullptr; }
  if (c->fadj) { dfree(c, c->fadj); c->fadj = nullptr; }
  c->F = 0;
  c->f_ext_dirty = true;
}

static int faces_build(Ctx* c, int64_t F, const int64_t* fconn_h, const double* t_h, const double* p_h, int base) {
  c->F = F;
  int rc = 0;
  if ((rc = dalloc(c, &c->fconn, F * c->nfn))) return rc;
  if ((rc = dalloc(c, &c->ftrac, 4 * F))) return rc;
  {
    // face load records (t1, t2, t3, p): traction and pressure (positive towards the surface)
    std::vector<double> rec(4 * F, 0.0);
    for (int64_t f = 0; f < F; ++f) {
      if (t_h)
        for (int k = 0; k < 3; ++k) rec[4 * f + k] = t_h[3 * f + k];
      if (p_h) rec[4 * f + 3] = p_h[f];
    }
    cudaMemcpyAsync(c->ftrac, rec.data(), 4 * F * sizeof(double), cudaMemcpyHostToDevice, c->stream);
    if ((rc = sync_and_check(c, "surface-load upload"))) return rc;
  }
  int64_t* tmp = nullptr;
  if (cudaMalloc(&tmp, F * c->nfn * sizeof(int64_t)) != cudaSuccess) return set_err(c, JFEM_ERR_OOM, "face upload");
  cudaMemsetAsync(c->d_err, 0, sizeof(int), c->stream);
  cudaMemcpyAsync(tmp, fconn_h, F * c->nfn * sizeof(int64_t), cudaMemcpyHostToDevice, c->stream);
  k_conn_soa<<<grid_for(F * c->nfn, 256), 256, 0, c->stream>>>(tmp, c->fconn, F, c->nfn, c->N, base, c->d_err);
  c->launches += 1;
  int h_err = 0;
  cudaMemcpyAsync(&h_err, c->d_err, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  rc = sync_and_check(c, "face upload");
  cudaFree(tmp);
  if (rc) return rc;
  if (h_err) return set_err(c, JFEM_ERR_INVALID, "face connectivity refers to a node outside the mesh");
  int famax = 0;
  return build_adjacency(c, c->fconn, F, c->nfn, &c->fadj_ptr, &c->fadj, &famax);
}

}  // namespace jfem
