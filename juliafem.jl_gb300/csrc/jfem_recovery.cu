// jfem_recovery.cu — nodal strain / stress recovery by a least-squares fit.
//
// Restates lsq_fit with get_strain_vector / get_stress_vector of
// src/problems_elasticity.jl:521-583: the integration-point field f (small
// strain ε = sym ∇u, or σ = λ tr(ε) I + 2μ ε, order 11, 22, 33, 12, 23, 13 with
// tensor shear components) is projected onto the nodal shape functions,
//   A x = b,  A = Σ_e Σ_q w detJ N Nᵀ,  b = Σ_e Σ_q w detJ N fᵀ   (6 columns).
// The reference factorises A (ldlt); A is a well-conditioned mass matrix, so
// here it is applied matrix-free and solved by Jacobi-PCG on the six columns at
// once, in FP64, to a relative residual `tol` per column.  Element passes write
// per-element contributions, node gathers sum them in ascending element order
// (deterministic, no atomics), as in the stiffness apply.
//
// Not replicated: the reference integrates A with the element's own rule, which
// is singular for simplices (Tet4 GLTET1: rank 1 per element; Tet10 GLTET4: rank
// 4 on 10 nodes).  The fit here uses rules exact for N·Nᵀ — GLTET4 for Tet4,
// GLTET15 for Tet10 (the points and weights of src/quadrature/gltet.jl:46-63),
// GLHEX8 for Hex8 — with J evaluated from the coordinates at each point.
#include <cmath>
#include <vector>

#include "jfem_common.cuh"

namespace jfem {

// recovery rule: exact for N·Nᵀ
__host__ __device__ constexpr int rec_nq(int et) { return et == JFEM_TET4 ? 4 : et == JFEM_TET10 ? 15 : 8; }

__host__ __device__ constexpr double rec_coord(int et, int q, int d) {
  if (et == JFEM_TET4) return qp_coord(JFEM_TET10, q, d);   // GLTET4
  if (et == JFEM_HEX8) return qp_coord(JFEM_HEX8, q, d);    // GLHEX8
  // GLTET15: centre, two classes of 4 (b, b, c) points, one class of 6 (d, d, f) points
  const double a = 0.25, b1 = 0.3197936278296299, c1 = 0.040619116511110234, b2 = 0.09197107805272303,
               c2 = 0.724086765841831, dd = 0.05635083268962915, ff = 0.4436491673103708;
  if (q == 0) return a;
  if (q <= 8) {
    const double b = q <= 4 ? b1 : b2, c = q <= 4 ? c1 : c2;
    const int k = (q - 1) % 4;              // (b,b,b), (b,b,c), (b,c,b), (c,b,b)
    return (k == 0) ? b : ((k == 1 && d == 2) || (k == 2 && d == 1) || (k == 3 && d == 0)) ? c : b;
  }
  const int k = q - 9;                      // (d,d,f), (d,f,d), (f,d,d), (d,f,f), (f,d,f), (f,f,d)
  const bool fpos[6][3] = {{false, false, true}, {false, true, false}, {true, false, false},
                           {false, true, true},  {true, false, true},  {true, true, false}};
  return fpos[k][d] ? ff : dd;
}

__host__ __device__ constexpr double rec_weight(int et, int q) {
  if (et == JFEM_TET4) return 1.0 / 24.0;
  if (et == JFEM_HEX8) return 1.0;
  return q == 0 ? 0.019753086419753086 : q <= 4 ? 0.011511367871045397 : q <= 8 ? 0.01198951396316977
                                                                                  : 0.008818342151675485;
}

// N_i and ∂N_i/∂ξ_a at a reference point (u, v, w)
__host__ __device__ constexpr double shape_at(int et, double u, double v, double w, int i) {
  if (et == JFEM_TET4) return i == 0 ? 1.0 - u - v - w : i == 1 ? u : i == 2 ? v : w;
  if (et == JFEM_TET10) {
    const double L[4] = {1.0 - u - v - w, u, v, w};
    const int ea[6] = {0, 1, 2, 0, 1, 2}, eb[6] = {1, 2, 0, 3, 3, 3};
    return i < 4 ? L[i] * (2.0 * L[i] - 1.0) : 4.0 * L[ea[i - 4]] * L[eb[i - 4]];
  }
  return 0.125 * (1.0 + hex_sign(i, 0) * u) * (1.0 + hex_sign(i, 1) * v) * (1.0 + hex_sign(i, 2) * w);
}

__host__ __device__ constexpr double dshape_at(int et, double u, double v, double w, int i, int a) {
  if (et == JFEM_TET4) return i == 0 ? -1.0 : (i - 1 == a ? 1.0 : 0.0);
  if (et == JFEM_TET10) {
    const double L[4] = {1.0 - u - v - w, u, v, w};
    const double dL[4][3] = {{-1.0, -1.0, -1.0}, {1.0, 0.0, 0.0}, {0.0, 1.0, 0.0}, {0.0, 0.0, 1.0}};
    const int ea[6] = {0, 1, 2, 0, 1, 2}, eb[6] = {1, 2, 0, 3, 3, 3};
    if (i < 4) return (4.0 * L[i] - 1.0) * dL[i][a];
    const int p = ea[i - 4], r = eb[i - 4];
    return 4.0 * (dL[p][a] * L[r] + L[p] * dL[r][a]);
  }
  const double x[3] = {u, v, w};
  double f = 0.125 * hex_sign(i, a);
  for (int d = 0; d < 3; ++d)
    if (d != a) f *= 1.0 + hex_sign(i, d) * x[d];
  return f;
}

// per element and recovery point: J from the coordinates, b_e[i][k] = Σ_q w detJ N_i f_k,
// the mass diagonal Σ_q w detJ N_i², and w detJ kept per point for the mass apply
template <int ET>
__global__ void k_rec_rhs(int64_t E, const int* __restrict__ conn, const double* __restrict__ X,
                          const double* __restrict__ lam, const double* __restrict__ mu,
                          const double* __restrict__ u, int field, double* __restrict__ yb,
                          double* __restrict__ yd, double* __restrict__ wdet) {
  constexpr int NN = Elem<ET>::NN, NQ = rec_nq(ET);
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
    double ue[NN][3], xe[NN][3];
#pragma unroll
    for (int i = 0; i < NN; ++i) {
      const int64_t n = conn[(int64_t)i * E + e];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        ue[i][c] = u[3 * n + c];
        xe[i][c] = X[3 * n + c];
      }
    }
    double b[NN][6], d[NN];
#pragma unroll
    for (int i = 0; i < NN; ++i) {
      d[i] = 0.0;
#pragma unroll
      for (int k = 0; k < 6; ++k) b[i][k] = 0.0;
    }
    const double la = lam[e], m = mu[e];
    for (int q = 0; q < NQ; ++q) {
      const double qu = rec_coord(ET, q, 0), qv = rec_coord(ET, q, 1), qw = rec_coord(ET, q, 2);
      double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
      for (int i = 0; i < NN; ++i)
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          const double dn = dshape_at(ET, qu, qv, qw, i, a);
#pragma unroll
          for (int c = 0; c < 3; ++c) J[a][c] += dn * xe[i][c];
        }
      double A[3][3];
      adj3(J, A);
      const double detJ = det3(J), id = 1.0 / detJ;
      double gu[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
      for (int i = 0; i < NN; ++i) {
        double g[3];
#pragma unroll
        for (int dd = 0; dd < 3; ++dd)
          g[dd] = id * (A[dd][0] * dshape_at(ET, qu, qv, qw, i, 0) + A[dd][1] * dshape_at(ET, qu, qv, qw, i, 1) +
                        A[dd][2] * dshape_at(ET, qu, qv, qw, i, 2));
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
          for (int dd = 0; dd < 3; ++dd) gu[c][dd] += ue[i][c] * g[dd];
      }
      double t[3][3];
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int c = 0; c < 3; ++c) t[a][c] = 0.5 * (gu[a][c] + gu[c][a]);
      if (field == JFEM_FIELD_STRESS) {
        const double tr = t[0][0] + t[1][1] + t[2][2];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int c = 0; c < 3; ++c) t[a][c] = 2.0 * m * t[a][c] + (a == c ? la * tr : 0.0);
      }
      const double f[6] = {t[0][0], t[1][1], t[2][2], t[0][1], t[1][2], t[0][2]};
      const double w = rec_weight(ET, q) * detJ;
      wdet[(int64_t)q * E + e] = w;
#pragma unroll
      for (int i = 0; i < NN; ++i) {
        const double ni = shape_at(ET, qu, qv, qw, i);
        d[i] += w * ni * ni;
#pragma unroll
        for (int k = 0; k < 6; ++k) b[i][k] += w * ni * f[k];
      }
    }
#pragma unroll
    for (int i = 0; i < NN; ++i) {
      yd[(int64_t)i * E + e] = d[i];
#pragma unroll
      for (int k = 0; k < 6; ++k) yb[((int64_t)i * 6 + k) * E + e] = b[i][k];
    }
  }
}

// per element: y_e[i][k] = Σ_q w detJ N_i Σ_j N_j v_j[k]  (A applied to six columns)
template <int ET>
__global__ void k_rec_mass(int64_t E, const int* __restrict__ conn, const double* __restrict__ wdet,
                           const double* __restrict__ v, double* __restrict__ yb) {
  constexpr int NN = Elem<ET>::NN, NQ = rec_nq(ET);
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x) {
    double ve[NN][6], y[NN][6];
#pragma unroll
    for (int i = 0; i < NN; ++i) {
      const int64_t n = conn[(int64_t)i * E + e];
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        ve[i][k] = v[6 * n + k];
        y[i][k] = 0.0;
      }
    }
    for (int q = 0; q < NQ; ++q) {
      const double qu = rec_coord(ET, q, 0), qv = rec_coord(ET, q, 1), qw = rec_coord(ET, q, 2);
      const double w = wdet[(int64_t)q * E + e];
      double s[6] = {0, 0, 0, 0, 0, 0};
#pragma unroll
      for (int j = 0; j < NN; ++j)
#pragma unroll
        for (int k = 0; k < 6; ++k) s[k] += shape_at(ET, qu, qv, qw, j) * ve[j][k];
#pragma unroll
      for (int i = 0; i < NN; ++i)
#pragma unroll
        for (int k = 0; k < 6; ++k) y[i][k] += w * shape_at(ET, qu, qv, qw, i) * s[k];
    }
#pragma unroll
    for (int i = 0; i < NN; ++i)
#pragma unroll
      for (int k = 0; k < 6; ++k) yb[((int64_t)i * 6 + k) * E + e] = y[i][k];
  }
}

// out[node][k] = Σ over the node's (element, local) entries, ascending element (C columns)
template <int C>
__global__ void k_rec_gather(int64_t N, int64_t E, const int* __restrict__ adj_ptr, const unsigned* __restrict__ adj,
                             const double* __restrict__ ye, double* __restrict__ out) {
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < N; j += (int64_t)gridDim.x * blockDim.x) {
    double s[C];
#pragma unroll
    for (int k = 0; k < C; ++k) s[k] = 0.0;
    for (int t = adj_ptr[j]; t < adj_ptr[j + 1]; ++t) {
      const unsigned pk = adj[t];
      const int64_t e = pk >> 4;
      const int a = pk & 15;
#pragma unroll
      for (int k = 0; k < C; ++k) s[k] += ye[((int64_t)a * C + k) * E + e];
    }
#pragma unroll
    for (int k = 0; k < C; ++k) out[C * j + k] = s[k];
  }
}

// Six-column PCG steps.  dots[k·G + b]: block partials of column k.
__global__ void __launch_bounds__(256) k_rec_dots(int64_t N, const double* __restrict__ a,
                                                  const double* __restrict__ b, double* __restrict__ part) {
  __shared__ double sh[32];
  double s[6] = {0, 0, 0, 0, 0, 0};
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < N; j += (int64_t)gridDim.x * blockDim.x)
#pragma unroll
    for (int k = 0; k < 6; ++k) s[k] += a[6 * j + k] * b[6 * j + k];
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    const double v = block_sum(s[k], sh);
    if (threadIdx.x == 0) part[(int64_t)k * gridDim.x + blockIdx.x] = v;
  }
}

// mode 0: x = b/d, r = b − y (y = A x), z = r/d, p = z
// mode 1: x += α p, r −= α q, z = r/d   (α per column)
// mode 2: p = z + β p                    (β per column)
__global__ void k_rec_axpy(int64_t N, int mode, const double* __restrict__ coef, const double* __restrict__ d,
                           const double* __restrict__ b, const double* __restrict__ y, double* __restrict__ x,
                           double* __restrict__ r, double* __restrict__ z, double* __restrict__ p) {
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < N; j += (int64_t)gridDim.x * blockDim.x) {
    const double id = d[j] > 0.0 ? 1.0 / d[j] : 0.0;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const int64_t q = 6 * j + k;
      if (mode == 0) {
        r[q] = b[q] - y[q];
        z[q] = r[q] * id;
        p[q] = z[q];
      } else if (mode == 1) {
        x[q] += coef[k] * p[q];
        r[q] -= coef[k] * y[q];
        z[q] = r[q] * id;
      } else {
        p[q] = z[q] + coef[k] * p[q];
      }
    }
  }
}

__global__ void k_rec_init(int64_t N, const double* __restrict__ d, const double* __restrict__ b,
                           double* __restrict__ x) {
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < N; j += (int64_t)gridDim.x * blockDim.x) {
    const double id = d[j] > 0.0 ? 1.0 / d[j] : 0.0;
#pragma unroll
    for (int k = 0; k < 6; ++k) x[6 * j + k] = b[6 * j + k] * id;
  }
}

template <int ET>
static void rec_launch_rhs(Ctx* c, const double* u, int field, double* yb, double* yd, double* wdet) {
  k_rec_rhs<ET><<<grid_for(c->E, 128), 128, 0, c->stream>>>(c->E, c->conn, c->X64, c->lam64, c->mu64, u, field, yb,
                                                           yd, wdet);
}
template <int ET>
static void rec_launch_mass(Ctx* c, const double* wdet, const double* v, double* yb) {
  k_rec_mass<ET><<<grid_for(c->E, 128), 128, 0, c->stream>>>(c->E, c->conn, wdet, v, yb);
}

static void rec_mass(Ctx* c, const double* wdet, const double* v, double* ye, double* out) {
  switch (c->et) {
    case JFEM_TET4: rec_launch_mass<JFEM_TET4>(c, wdet, v, ye); break;
    case JFEM_TET10: rec_launch_mass<JFEM_TET10>(c, wdet, v, ye); break;
    default: rec_launch_mass<JFEM_HEX8>(c, wdet, v, ye); break;
  }
  k_rec_gather<6><<<grid_for(c->N, 256), 256, 0, c->stream>>>(c->N, c->E, c->adj_ptr, c->adj, ye, out);
  c->launches += 2;
}

static int rec_dots(Ctx* c, const double* a, const double* b, double out[6]) {
  const int G = JFEM_RED_BLOCKS;
  k_rec_dots<<<G, 256, 0, c->stream>>>(c->N, a, b, c->part);   // c->part: six columns of G partials here
  c->launches += 1;
  std::vector<double> h((size_t)6 * G);
  cudaMemcpyAsync(h.data(), c->part, 6 * G * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  const int rc = sync_and_check(c, "recovery dots");
  if (rc) return rc;
  for (int k = 0; k < 6; ++k) {
    double s = 0.0;
    for (int q = 0; q < G; ++q) s += h[(size_t)k * G + q];
    out[k] = s;
  }
  return 0;
}

int recover_field(Ctx* c, const double* u_h, int field, double tol, int max_iter, double* nodal_h, int* iters_out) {
  int rc = geometry_prepare(c);
  if (rc) return rc;
  const int64_t N = c->N, E = c->E, nn = c->nn;
  double *u = nullptr, *ye = nullptr, *yd = nullptr, *wdet = nullptr, *d = nullptr, *b = nullptr, *x = nullptr, *r = nullptr,
         *z = nullptr, *p = nullptr, *q = nullptr, *coef = nullptr, *part6 = nullptr;
  std::vector<void*> tmp;
  auto alloc = [&](double** ptr, size_t count) {
    if (cudaMalloc((void**)ptr, count * sizeof(double)) != cudaSuccess) return false;
    tmp.push_back(*ptr);
    return true;
  };
  auto cleanup = [&]() {
    cudaStreamSynchronize(c->stream);
    for (void* t : tmp) cudaFree(t);
  };
  if (!alloc(&u, 3 * N) || !alloc(&ye, (size_t)6 * nn * E) || !alloc(&yd, (size_t)nn * E) ||
      !alloc(&wdet, (size_t)15 * E) || !alloc(&d, N) ||
      !alloc(&b, 6 * N) || !alloc(&x, 6 * N) || !alloc(&r, 6 * N) || !alloc(&z, 6 * N) || !alloc(&p, 6 * N) ||
      !alloc(&q, 6 * N) || !alloc(&coef, 6) || !alloc(&part6, (size_t)6 * JFEM_RED_BLOCKS)) {
    cleanup();
    return set_err(c, JFEM_ERR_OOM, "recovery buffers");
  }
  double* part_saved = c->part;
  c->part = part6;   // six columns of block partials
  cudaMemcpyAsync(u, u_h, 3 * N * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  switch (c->et) {
    case JFEM_TET4: rec_launch_rhs<JFEM_TET4>(c, u, field, ye, yd, wdet); break;
    case JFEM_TET10: rec_launch_rhs<JFEM_TET10>(c, u, field, ye, yd, wdet); break;
    default: rec_launch_rhs<JFEM_HEX8>(c, u, field, ye, yd, wdet); break;
  }
  k_rec_gather<6><<<grid_for(N, 256), 256, 0, c->stream>>>(N, E, c->adj_ptr, c->adj, ye, b);
  k_rec_gather<1><<<grid_for(N, 256), 256, 0, c->stream>>>(N, E, c->adj_ptr, c->adj, yd, d);
  k_rec_init<<<grid_for(N, 256), 256, 0, c->stream>>>(N, d, b, x);
  c->launches += 4;
  rec_mass(c, wdet, x, ye, q);
  k_rec_axpy<<<grid_for(N, 256), 256, 0, c->stream>>>(N, 0, nullptr, d, b, q, x, r, z, p);
  c->launches += 1;
  double bb[6], rz[6], rr[6];
  int it = 0;
  if ((rc = rec_dots(c, b, b, bb)) || (rc = rec_dots(c, r, z, rz))) {
    c->part = part_saved;
    cleanup();
    return rc;
  }
  for (; it < max_iter; ++it) {
    if ((rc = rec_dots(c, r, r, rr))) break;
    bool done = true;
    for (int k = 0; k < 6; ++k) done = done && rr[k] <= tol * tol * bb[k];
    if (done) break;
    rec_mass(c, wdet, p, ye, q);
    double pq[6], al[6];
    if ((rc = rec_dots(c, p, q, pq))) break;
    for (int k = 0; k < 6; ++k) al[k] = (pq[k] > 0.0 && rz[k] > 0.0) ? rz[k] / pq[k] : 0.0;
    cudaMemcpyAsync(coef, al, sizeof(al), cudaMemcpyHostToDevice, c->stream);
    k_rec_axpy<<<grid_for(N, 256), 256, 0, c->stream>>>(N, 1, coef, d, b, q, x, r, z, p);
    double rzn[6], be[6];
    if ((rc = rec_dots(c, r, z, rzn))) break;
    for (int k = 0; k < 6; ++k) {
      be[k] = rz[k] > 0.0 ? rzn[k] / rz[k] : 0.0;
      rz[k] = rzn[k];
    }
    cudaMemcpyAsync(coef, be, sizeof(be), cudaMemcpyHostToDevice, c->stream);
    k_rec_axpy<<<grid_for(N, 256), 256, 0, c->stream>>>(N, 2, coef, d, b, q, x, r, z, p);
    c->launches += 2;
  }
  c->part = part_saved;
  if (!rc) {
    cudaMemcpyAsync(nodal_h, x, 6 * N * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    rc = sync_and_check(c, "recovery download");
  }
  cleanup();
  if (rc) return rc;
  if (iters_out) *iters_out = it;
  return it >= max_iter ? JFEM_NOT_CONVERGED : 0;
}

}  // namespace jfem
