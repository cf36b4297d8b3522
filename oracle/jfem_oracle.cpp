// jfem_oracle.cpp — CPU FP64 restatement of JuliaFEM's 3D elasticity hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle that the GPU library is
// checked against; nothing in the product links or calls it.  Only tests/,
// __graft_entry__.smoke() and bench.py's cpu_baseline / --impl reference legs
// use it.
//
// Parity status: the reference (Julia, mid-refactor) cannot be executed here
// and its own tests hold no golden vectors for this path, so K-entry parity is
// "parity unpinned" by the reference.  The restatement is pinned instead by
// (i) the reference fixture test/testdata/cube_tet4.inp run as a patch test
// with its analytic homogeneous solution, (ii) closed forms (Tet4 K = V BᵀDB,
// rigid-body null space, beam theory), and (iii) an independent numpy
// restatement (oracle/np_oracle.py) agreeing to ~1e-13.
//
// What it follows (reference file:line):
//   shape functions     src/basis/lagrange_generated.jl:229-311 (Tet4/Tet10/Hex8),
//                       :88-160 (Tri3/Tri6/Quad4)
//   quadrature          src/quadrature/gltet.jl:7-25, glquad.jl:6-40, quaddata.jl:3-4,
//                       gltri.jl:6-30; default rules src/elements/integrate.jl:11-31
//   Jacobian/gradients  src/basis/math.jl:47-53,185-205 (J = Σ dN⊗X, ∇N = J⁻¹·dN)
//   element kernel      src/problems_elasticity.jl:203-451 (B-matrix form, Voigt
//                       order 11,22,33,12,23,13 with engineering shear :189-197,
//                       Hooke D :313-317, Km :370-375, Kg :378-404, f_int :407-409)
//   Neo-Hookean         src/materials/neo_hookean.jl:129-143,205-231 (S = 2∂ψ/∂C,
//                       𝔻 = 4∂²ψ/∂C², written in closed form)
//   surface traction    src/problems_elasticity.jl:454-502
//   COO + sparse()      src/sparse/sparse.jl:121-132,53 (all entries pushed, zeros kept,
//                       duplicates summed in push order)
//   in-place CSC add    src/sparse/sparsematrixcsc.jl:69-98 (fixed pattern)
//   DOF map             src/assembly/problems.jl:466-478 (gdof = 3(node-1)+j)
//   Dirichlet           src/solvers.jl:192-216 (elimination of prescribed DOFs)
//   CG                  src/backend/cpu.jl:221-254 (+ Jacobi preconditioner and a
//                       relative tolerance)
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#include <numeric>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef int64_t i64;

namespace {

enum { TET4 = 4, TET10 = 10, HEX8 = 8 };
enum { TRI3 = 3, TRI6 = 6, QUAD4 = 4 };
enum { LINEAR = 0, NEOHOOKE = 1 };

int n_nodes_of(int et) { return et == TET4 ? 4 : et == TET10 ? 10 : et == HEX8 ? 8 : -1; }

struct Rule {
  int nq = 0;
  double xi[64][3];
  double w[64];
};

// GLTET1 (gltet.jl:7-11), GLTET4 (gltet.jl:17-25), GLHEX8 (glquad.jl tensor product
// of quaddata.jl:3-4; CartesianIndices order: first coordinate varies fastest).
Rule volume_rule(int et) {
  Rule r;
  if (et == TET4) {
    r.nq = 1;
    r.xi[0][0] = r.xi[0][1] = r.xi[0][2] = 0.25;
    r.w[0] = 1.0 / 6.0;
  } else if (et == TET10) {
    const double a = (5.0 + 3.0 * std::sqrt(5.0)) / 20.0;
    const double b = (5.0 - std::sqrt(5.0)) / 20.0;
    const double pts[4][3] = {{a, b, b}, {b, a, b}, {b, b, a}, {b, b, b}};
    r.nq = 4;
    for (int q = 0; q < 4; ++q) {
      for (int d = 0; d < 3; ++d) r.xi[q][d] = pts[q][d];
      r.w[q] = 1.0 / 24.0;
    }
  } else if (et == HEX8) {
    const double p[2] = {-0.5773502691896258, 0.5773502691896258};
    r.nq = 8;
    int q = 0;
    for (int k = 0; k < 2; ++k)
      for (int j = 0; j < 2; ++j)
        for (int i = 0; i < 2; ++i) {
          r.xi[q][0] = p[i];
          r.xi[q][1] = p[j];
          r.xi[q][2] = p[k];
          r.w[q] = 1.0;
          ++q;
        }
  }
  return r;
}

// Surface rules: Tri3 → GLTRI1, Tri6 → GLTRI3, Quad4 → GLQUAD4 (integrate.jl:15,23-24).
Rule surface_rule(int ft) {
  Rule r;
  if (ft == TRI3) {
    r.nq = 1;
    r.xi[0][0] = r.xi[0][1] = 1.0 / 3.0;
    r.w[0] = 0.5;
  } else if (ft == TRI6) {
    const double pts[3][2] = {{2.0 / 3.0, 1.0 / 6.0}, {1.0 / 6.0, 2.0 / 3.0}, {1.0 / 6.0, 1.0 / 6.0}};
    r.nq = 3;
    for (int q = 0; q < 3; ++q) {
      r.xi[q][0] = pts[q][0];
      r.xi[q][1] = pts[q][1];
      r.w[q] = 1.0 / 6.0;
    }
  } else if (ft == QUAD4) {
    const double p[2] = {-0.5773502691896258, 0.5773502691896258};
    r.nq = 4;
    int q = 0;
    for (int j = 0; j < 2; ++j)
      for (int i = 0; i < 2; ++i) {
        r.xi[q][0] = p[i];
        r.xi[q][1] = p[j];
        r.w[q] = 1.0;
        ++q;
      }
  }
  return r;
}

// Volume basis N(ξ) and ∂N/∂ξ (lagrange_generated.jl:229-311).
void volume_basis(int et, const double* xi, double* N, double (*dN)[3]) {
  const double u = xi[0], v = xi[1], w = xi[2];
  if (et == TET4) {
    N[0] = 1 - u - v - w; N[1] = u; N[2] = v; N[3] = w;
    const double d[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int i = 0; i < 4; ++i) for (int k = 0; k < 3; ++k) dN[i][k] = d[i][k];
  } else if (et == TET10) {
    N[0] = 1 - 3 * u - 3 * v - 3 * w + 2 * u * u + 2 * v * v + 2 * w * w + 4 * u * v + 4 * u * w + 4 * v * w;
    N[1] = -u + 2 * u * u;
    N[2] = -v + 2 * v * v;
    N[3] = -w + 2 * w * w;
    N[4] = 4 * u - 4 * u * u - 4 * u * v - 4 * u * w;
    N[5] = 4 * u * v;
    N[6] = 4 * v - 4 * v * v - 4 * u * v - 4 * v * w;
    N[7] = 4 * w - 4 * w * w - 4 * u * w - 4 * v * w;
    N[8] = 4 * u * w;
    N[9] = 4 * v * w;
    const double d[10][3] = {
        {-3 + 4 * u + 4 * v + 4 * w, -3 + 4 * v + 4 * u + 4 * w, -3 + 4 * w + 4 * u + 4 * v},
        {-1 + 4 * u, 0, 0},
        {0, -1 + 4 * v, 0},
        {0, 0, -1 + 4 * w},
        {4 - 8 * u - 4 * v - 4 * w, -4 * u, -4 * u},
        {4 * v, 4 * u, 0},
        {-4 * v, 4 - 8 * v - 4 * u - 4 * w, -4 * v},
        {-4 * w, -4 * w, 4 - 8 * w - 4 * u - 4 * v},
        {4 * w, 0, 4 * u},
        {0, 4 * w, 4 * v}};
    for (int i = 0; i < 10; ++i) for (int k = 0; k < 3; ++k) dN[i][k] = d[i][k];
  } else if (et == HEX8) {
    const double s[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                            {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
    for (int i = 0; i < 8; ++i) {
      const double a = 1 + s[i][0] * u, b = 1 + s[i][1] * v, c = 1 + s[i][2] * w;
      N[i] = 0.125 * a * b * c;
      dN[i][0] = 0.125 * s[i][0] * b * c;
      dN[i][1] = 0.125 * a * s[i][1] * c;
      dN[i][2] = 0.125 * a * b * s[i][2];
    }
  }
}

int surface_nodes_of(int ft) { return ft == TRI3 ? 3 : ft == TRI6 ? 6 : ft == QUAD4 ? 4 : -1; }

// Surface basis (lagrange_generated.jl:88-160).
void surface_basis(int ft, const double* xi, double* N, double (*dN)[2]) {
  const double u = xi[0], v = xi[1];
  if (ft == TRI3) {
    N[0] = 1 - u - v; N[1] = u; N[2] = v;
    dN[0][0] = -1; dN[0][1] = -1; dN[1][0] = 1; dN[1][1] = 0; dN[2][0] = 0; dN[2][1] = 1;
  } else if (ft == TRI6) {
    N[0] = 1 - 3 * u - 3 * v + 2 * u * u + 4 * u * v + 2 * v * v;
    N[1] = -u + 2 * u * u;
    N[2] = -v + 2 * v * v;
    N[3] = 4 * u - 4 * u * u - 4 * u * v;
    N[4] = 4 * u * v;
    N[5] = 4 * v - 4 * u * v - 4 * v * v;
    const double d[6][2] = {{-3 + 4 * u + 4 * v, -3 + 4 * u + 4 * v}, {-1 + 4 * u, 0}, {0, -1 + 4 * v},
                            {4 - 8 * u - 4 * v, -4 * u}, {4 * v, 4 * u}, {-4 * v, 4 - 4 * u - 8 * v}};
    for (int i = 0; i < 6; ++i) { dN[i][0] = d[i][0]; dN[i][1] = d[i][1]; }
  } else if (ft == QUAD4) {
    const double s[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
    for (int i = 0; i < 4; ++i) {
      N[i] = 0.25 * (1 + s[i][0] * u) * (1 + s[i][1] * v);
      dN[i][0] = 0.25 * s[i][0] * (1 + s[i][1] * v);
      dN[i][1] = 0.25 * (1 + s[i][0] * u) * s[i][1];
    }
  }
}

double det3(const double J[3][3]) {
  return J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
         J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
         J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
}

void inv3(const double A[3][3], double det, double B[3][3]) {
  const double id = 1.0 / det;
  B[0][0] = (A[1][1] * A[2][2] - A[1][2] * A[2][1]) * id;
  B[0][1] = (A[0][2] * A[2][1] - A[0][1] * A[2][2]) * id;
  B[0][2] = (A[0][1] * A[1][2] - A[0][2] * A[1][1]) * id;
  B[1][0] = (A[1][2] * A[2][0] - A[1][0] * A[2][2]) * id;
  B[1][1] = (A[0][0] * A[2][2] - A[0][2] * A[2][0]) * id;
  B[1][2] = (A[0][2] * A[1][0] - A[0][0] * A[1][2]) * id;
  B[2][0] = (A[1][0] * A[2][1] - A[1][1] * A[2][0]) * id;
  B[2][1] = (A[0][1] * A[2][0] - A[0][0] * A[2][1]) * id;
  B[2][2] = (A[0][0] * A[1][1] - A[0][1] * A[1][0]) * id;
}

// Voigt index pairs in the reference order 11, 22, 33, 12, 23, 13.
const int VI[6] = {0, 1, 2, 0, 1, 0};
const int VJ[6] = {0, 1, 2, 1, 2, 2};

// Hooke matrix D (problems_elasticity.jl:313-317).
void hooke(double E, double nu, double D[6][6]) {
  const double la = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
  const double mu = E / (2.0 * (1.0 + nu));
  for (int i = 0; i < 6; ++i) for (int j = 0; j < 6; ++j) D[i][j] = 0.0;
  D[0][0] = D[1][1] = D[2][2] = 2 * mu + la;
  D[3][3] = D[4][4] = D[5][5] = mu;
  D[0][1] = D[1][0] = D[1][2] = D[2][1] = D[0][2] = D[2][0] = la;
}

// Compressible Neo-Hookean, ψ = μ/2(I₁−3) − μ ln J + λ/2 ln²J (neo_hookean.jl:129-143).
// S = μ(I − C⁻¹) + λ lnJ C⁻¹ ;  𝔻ᵢⱼₖₗ = λ C⁻¹ᵢⱼC⁻¹ₖₗ + (μ − λ lnJ)(C⁻¹ᵢₖC⁻¹ⱼₗ + C⁻¹ᵢₗC⁻¹ⱼₖ).
// Returns false when J ≤ 0 (neo_hookean.jl:137 throws DomainError there).
bool neo_hookean(double E, double nu, const double C[3][3], double S[6], double D[6][6]) {
  const double la = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
  const double mu = E / (2.0 * (1.0 + nu));
  const double detC = det3(C);
  if (!(detC > 0.0)) return false;
  const double lnJ = 0.5 * std::log(detC);
  double Ci[3][3];
  inv3(C, detC, Ci);
  for (int I = 0; I < 6; ++I) {
    const int i = VI[I], j = VJ[I];
    S[I] = mu * ((i == j ? 1.0 : 0.0) - Ci[i][j]) + la * lnJ * Ci[i][j];
  }
  const double c = mu - la * lnJ;
  for (int I = 0; I < 6; ++I)
    for (int K = 0; K < 6; ++K) {
      const int i = VI[I], j = VJ[I], k = VI[K], l = VJ[K];
      D[I][K] = la * Ci[i][j] * Ci[k][l] + c * (Ci[i][k] * Ci[j][l] + Ci[i][l] * Ci[j][k]);
    }
  return true;
}

// One volume element (problems_elasticity.jl:203-451).  Xe, ue node-major (n_en×3).
// Ke column-major (3n_en)², fint (3n_en).  Returns 0, or -4 (non-positive detJ),
// -5 (J ≤ 0 in the Neo-Hookean law).
int element_kernel(int et, int model, int finite, int geom, const double* Xe, const double* ue,
                   double E, double nu, double* Ke, double* fint) {
  const int nn = n_nodes_of(et);
  const int nd = 3 * nn;
  const Rule rule = volume_rule(et);
  std::fill(Ke, Ke + nd * nd, 0.0);
  std::fill(fint, fint + nd, 0.0);
  std::vector<double> BL(6 * nd), BNL(9 * nd);
  double N[10], dN[10][3], grad[10][3];
  for (int q = 0; q < rule.nq; ++q) {
    volume_basis(et, rule.xi[q], N, dN);
    double J[3][3] = {{0}};
    for (int i = 0; i < nn; ++i)
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) J[a][b] += dN[i][a] * Xe[3 * i + b];
    const double detJ = det3(J);
    if (!(detJ > 0.0)) return -4;
    double iJ[3][3];
    inv3(J, detJ, iJ);
    for (int i = 0; i < nn; ++i)
      for (int a = 0; a < 3; ++a) {
        double s = 0.0;
        for (int b = 0; b < 3; ++b) s += iJ[a][b] * dN[i][b];
        grad[i][a] = s;
      }
    const double w = rule.w[q] * detJ;
    // ∇u (grad!): gradu[i][j] = Σ_k u_k[i] ∂N_k/∂X_j
    double gu[3][3] = {{0}};
    if (ue)
      for (int k = 0; k < nn; ++k)
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) gu[i][j] += ue[3 * k + i] * grad[k][j];
    double F[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    double eps[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        if (finite) {
          double gtg = 0.0;
          for (int k = 0; k < 3; ++k) gtg += gu[k][i] * gu[k][j];
          eps[i][j] = 0.5 * (gu[i][j] + gu[j][i] + gtg);
          F[i][j] += gu[i][j];
        } else {
          eps[i][j] = 0.5 * (gu[i][j] + gu[j][i]);
        }
      }
    double ev[6];
    for (int I = 0; I < 6; ++I) ev[I] = (I < 3 ? 1.0 : 2.0) * eps[VI[I]][VJ[I]];
    // BL (problems_elasticity.jl:269-302)
    std::fill(BL.begin(), BL.end(), 0.0);
    for (int i = 0; i < nn; ++i) {
      double* c0 = &BL[6 * (3 * i + 0)];
      double* c1 = &BL[6 * (3 * i + 1)];
      double* c2 = &BL[6 * (3 * i + 2)];
      const double* g = grad[i];
      if (finite) {
        // row r of BL for column 3i+k: column-major storage BL[6*col + row]
        for (int k = 0; k < 3; ++k) {
          double* c = &BL[6 * (3 * i + k)];
          c[0] = F[k][0] * g[0];
          c[1] = F[k][1] * g[1];
          c[2] = F[k][2] * g[2];
          c[3] = F[k][0] * g[1] + F[k][1] * g[0];
          c[4] = F[k][1] * g[2] + F[k][2] * g[1];
          c[5] = F[k][2] * g[0] + F[k][0] * g[2];
        }
      } else {
        c0[0] = g[0];
        c1[1] = g[1];
        c2[2] = g[2];
        c0[3] = g[1];
        c1[3] = g[0];
        c1[4] = g[2];
        c2[4] = g[1];
        c0[5] = g[2];
        c2[5] = g[0];
      }
    }
    double D[6][6], sv[6];
    if (model == NEOHOOKE) {
      double C[3][3];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) C[i][j] = 2.0 * eps[i][j] + (i == j ? 1.0 : 0.0);
      if (!neo_hookean(E, nu, C, sv, D)) return -5;
    } else {
      hooke(E, nu, D);
      for (int I = 0; I < 6; ++I) {
        double s = 0.0;
        for (int K = 0; K < 6; ++K) s += D[I][K] * ev[K];
        sv[I] = s;
      }
    }
    // Km += w BLᵀ D BL   (problems_elasticity.jl:370-375)
    std::vector<double> BtD(nd * 6);
    for (int c = 0; c < nd; ++c)
      for (int K = 0; K < 6; ++K) {
        double s = 0.0;
        for (int I = 0; I < 6; ++I) s += BL[6 * c + I] * D[I][K];
        BtD[6 * c + K] = s;
      }
    for (int cj = 0; cj < nd; ++cj)
      for (int ci = 0; ci < nd; ++ci) {
        double s = 0.0;
        for (int K = 0; K < 6; ++K) s += BtD[6 * ci + K] * BL[6 * cj + K];
        Ke[cj * nd + ci] += w * s;
      }
    // Kg += w BNLᵀ S3 BNL  (problems_elasticity.jl:378-404)
    if (geom) {
      double S[3][3];
      for (int I = 0; I < 6; ++I) { S[VI[I]][VJ[I]] = sv[I]; S[VJ[I]][VI[I]] = sv[I]; }
      for (int a = 0; a < nn; ++a)
        for (int b = 0; b < nn; ++b) {
          double s = 0.0;
          for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) s += grad[a][i] * S[i][j] * grad[b][j];
          for (int k = 0; k < 3; ++k) Ke[(3 * b + k) * nd + (3 * a + k)] += w * s;
        }
    }
    // f_int += w BLᵀ σ  (problems_elasticity.jl:407-409)
    for (int c = 0; c < nd; ++c) {
      double s = 0.0;
      for (int I = 0; I < 6; ++I) s += BL[6 * c + I] * sv[I];
      fint[c] += w * s;
    }
  }
  return 0;
}

void gather_element(int nn, const i64* conn, i64 e, const double* X, const double* u, double* Xe,
                    double* ue) {
  for (int a = 0; a < nn; ++a) {
    const i64 n = conn[e * nn + a];
    for (int k = 0; k < 3; ++k) {
      Xe[3 * a + k] = X[3 * n + k];
      if (u) ue[3 * a + k] = u[3 * n + k];
    }
  }
}

int nthreads_req = 0;

}  // namespace

extern "C" {

// Number of OpenMP threads used by the parallel loops (0 = library default).
void orc_set_threads(int n) {
  nthreads_req = n;
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#endif
}

int orc_get_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// Single element (problems_elasticity.jl:203-451).  Ke column-major (3n_en)².
int orc_element(int et, int model, int finite, int geom, const double* Xe, const double* ue,
                double E, double nu, double* Ke, double* fint) {
  if (n_nodes_of(et) < 0) return -1;
  return element_kernel(et, model, finite, geom, Xe, ue, E, nu, Ke, fint);
}

// Global assembly by COO push (sparse.jl:121-132) and sparse() (sparse.jl:53):
// every (3n_en)² entry of every element is pushed in element order, column-major
// within the element; sparse() sorts by (column,row) and sums duplicates in push
// order; numerical zeros stay structural.  conn is element-major, 0-based.
// Call once with colptr == NULL to get nnz, then again with arrays of that size.
// fint receives Σ_e f_int (length 3N).  per_element: E/nu arrays have n_elem
// entries (else 1).  Returns 0 or a negative error.
int orc_assemble_coo(int et, int model, int finite, int geom, i64 n_nodes, const double* X,
                     i64 n_elem, const i64* conn, const double* E, const double* nu,
                     int per_element, const double* u, i64* nnz_inout, i64* colptr, i64* rowval,
                     double* nzval, double* fint) {
  const int nn = n_nodes_of(et);
  if (nn < 0) return -1;
  const int nd = 3 * nn;
  const i64 n = 3 * n_nodes;
  const i64 ntrip = n_elem * nd * nd;
  std::vector<i64> I(ntrip), Jc(ntrip);
  std::vector<double> V(ntrip);
  std::vector<double> fe_all((size_t)n_elem * nd);
  int err = 0;
#pragma omp parallel for schedule(static) reduction(min : err)
  for (i64 e = 0; e < n_elem; ++e) {
    double Xe[30], ue[30], Ke[900];
    gather_element(nn, conn, e, X, u, Xe, ue);
    const double Ee = per_element ? E[e] : E[0];
    const double ne = per_element ? nu[e] : nu[0];
    const int rc = element_kernel(et, model, finite, geom, Xe, u ? ue : nullptr, Ee, ne, Ke,
                                  &fe_all[(size_t)e * nd]);
    if (rc < err) err = rc;
    i64 gd[30];
    for (int a = 0; a < nn; ++a)
      for (int k = 0; k < 3; ++k) gd[3 * a + k] = 3 * conn[e * nn + a] + k;
    i64 t = e * nd * nd;
    for (int j = 0; j < nd; ++j)
      for (int i = 0; i < nd; ++i, ++t) {
        I[t] = gd[i];
        Jc[t] = gd[j];
        V[t] = Ke[j * nd + i];
      }
  }
  if (err) return err;
  if (fint) {
    std::fill(fint, fint + n, 0.0);
    for (i64 e = 0; e < n_elem; ++e)
      for (int a = 0; a < nn; ++a)
        for (int k = 0; k < 3; ++k) fint[3 * conn[e * nn + a] + k] += fe_all[(size_t)e * nd + 3 * a + k];
  }
  // Stable counting sort by row, then stable counting sort by column, gives
  // (column,row) order with push order preserved among duplicates.
  std::vector<i64> cnt(n + 1, 0), ord(ntrip), ord2(ntrip);
  for (i64 t = 0; t < ntrip; ++t) cnt[I[t] + 1]++;
  for (i64 r = 0; r < n; ++r) cnt[r + 1] += cnt[r];
  for (i64 t = 0; t < ntrip; ++t) ord[cnt[I[t]]++] = t;
  std::fill(cnt.begin(), cnt.end(), 0);
  for (i64 t = 0; t < ntrip; ++t) cnt[Jc[t] + 1]++;
  for (i64 c = 0; c < n; ++c) cnt[c + 1] += cnt[c];
  for (i64 s = 0; s < ntrip; ++s) {
    const i64 t = ord[s];
    ord2[cnt[Jc[t]]++] = t;
  }
  // ord2 is sorted by (col,row) but the row-sort permuted push order among equal
  // (row,col); restore push order inside each run by sorting the run indices.
  i64 nnz = 0;
  std::vector<i64> cp(n + 1, 0);
  i64 s = 0;
  while (s < ntrip) {
    i64 r = s;
    const i64 t0 = ord2[s];
    while (r < ntrip && I[ord2[r]] == I[t0] && Jc[ord2[r]] == Jc[t0]) ++r;
    std::sort(ord2.begin() + s, ord2.begin() + r);
    ++nnz;
    cp[Jc[t0] + 1]++;
    s = r;
  }
  if (!colptr) {
    *nnz_inout = nnz;
    return 0;
  }
  if (*nnz_inout < nnz) return -1;
  *nnz_inout = nnz;
  for (i64 c = 0; c < n; ++c) cp[c + 1] += cp[c];
  for (i64 c = 0; c <= n; ++c) colptr[c] = cp[c];
  i64 k = 0;
  s = 0;
  while (s < ntrip) {
    i64 r = s;
    const i64 t0 = ord2[s];
    double acc = 0.0;
    while (r < ntrip && I[ord2[r]] == I[t0] && Jc[ord2[r]] == Jc[t0]) {
      acc += V[ord2[r]];
      ++r;
    }
    rowval[k] = I[t0];
    nzval[k] = acc;
    ++k;
    s = r;
  }
  return 0;
}

// Structural pattern of the global matrix from node adjacency: every pair of
// nodes sharing an element couples with a full 3×3 block (the same pattern the
// COO push of sparse.jl:121-132 produces).  Two-phase like orc_assemble_coo.
int orc_pattern(int et, i64 n_nodes, i64 n_elem, const i64* conn, i64* nnz_inout, i64* colptr,
                i64* rowval) {
  const int nn = n_nodes_of(et);
  if (nn < 0) return -1;
  std::vector<std::vector<i64>> nb(n_nodes);
  for (i64 e = 0; e < n_elem; ++e)
    for (int a = 0; a < nn; ++a)
      for (int b = 0; b < nn; ++b) nb[conn[e * nn + a]].push_back(conn[e * nn + b]);
  i64 nnz = 0;
  for (i64 j = 0; j < n_nodes; ++j) {
    std::sort(nb[j].begin(), nb[j].end());
    nb[j].erase(std::unique(nb[j].begin(), nb[j].end()), nb[j].end());
    nnz += 9 * (i64)nb[j].size();
  }
  if (!colptr) {
    *nnz_inout = nnz;
    return 0;
  }
  if (*nnz_inout < nnz) return -1;
  *nnz_inout = nnz;
  i64 k = 0;
  colptr[0] = 0;
  for (i64 j = 0; j < n_nodes; ++j)
    for (int dj = 0; dj < 3; ++dj) {
      for (i64 i : nb[j])
        for (int di = 0; di < 3; ++di) rowval[k++] = 3 * i + di;
      colptr[3 * j + dj + 1] = k;
    }
  return 0;
}

// In-place add of all element matrices into a fixed CSC pattern
// (sparsematrixcsc.jl:69-98: error when a row is missing).  nzval and fint are
// zeroed first.  Elements are integrated in parallel; the adds run per column
// in ascending element order, so results do not depend on the thread count.
int orc_assemble_pattern(int et, int model, int finite, int geom, i64 n_nodes, const double* X,
                         i64 n_elem, const i64* conn, const double* E, const double* nu,
                         int per_element, const double* u, const i64* colptr, const i64* rowval,
                         double* nzval, double* fint) {
  const int nn = n_nodes_of(et);
  if (nn < 0) return -1;
  const int nd = 3 * nn;
  const i64 n = 3 * n_nodes;
  std::vector<double> Ke_all((size_t)n_elem * nd * nd), fe_all((size_t)n_elem * nd);
  int err = 0;
#pragma omp parallel for schedule(static) reduction(min : err)
  for (i64 e = 0; e < n_elem; ++e) {
    double Xe[30], ue[30];
    gather_element(nn, conn, e, X, u, Xe, ue);
    const double Ee = per_element ? E[e] : E[0];
    const double ne = per_element ? nu[e] : nu[0];
    const int rc = element_kernel(et, model, finite, geom, Xe, u ? ue : nullptr, Ee, ne,
                                  &Ke_all[(size_t)e * nd * nd], &fe_all[(size_t)e * nd]);
    if (rc < err) err = rc;
  }
  if (err) return err;
  // node → (element, local) lists in ascending element order
  std::vector<i64> cnt(n_nodes + 1, 0);
  for (i64 e = 0; e < n_elem; ++e)
    for (int a = 0; a < nn; ++a) cnt[conn[e * nn + a] + 1]++;
  for (i64 j = 0; j < n_nodes; ++j) cnt[j + 1] += cnt[j];
  std::vector<i64> adj(cnt[n_nodes]);
  {
    std::vector<i64> cur(cnt.begin(), cnt.end() - 1);
    for (i64 e = 0; e < n_elem; ++e)
      for (int a = 0; a < nn; ++a) adj[cur[conn[e * nn + a]]++] = e * nn + a;
  }
  int missing = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(max : missing)
  for (i64 j = 0; j < n_nodes; ++j) {
    for (int dj = 0; dj < 3; ++dj) {
      const i64 c = 3 * j + dj;
      const i64 c0 = colptr[c], c1 = colptr[c + 1];
      for (i64 k = c0; k < c1; ++k) nzval[k] = 0.0;
      for (i64 t = cnt[j]; t < cnt[j + 1]; ++t) {
        const i64 e = adj[t] / nn;
        const int a = (int)(adj[t] % nn);
        const double* Ke = &Ke_all[(size_t)e * nd * nd];
        for (int b = 0; b < nn; ++b)
          for (int di = 0; di < 3; ++di) {
            const i64 r = 3 * conn[e * nn + b] + di;
            const i64* p = std::lower_bound(rowval + c0, rowval + c1, r);
            if (p == rowval + c1 || *p != r) {
              missing = 1;
              continue;
            }
            nzval[p - rowval] += Ke[(3 * a + dj) * nd + 3 * b + di];
          }
      }
    }
  }
  if (missing) return -1;
  if (fint) {
    for (i64 j = 0; j < n_nodes; ++j)
      for (int k = 0; k < 3; ++k) {
        double s = 0.0;
        for (i64 t = cnt[j]; t < cnt[j + 1]; ++t) s += fe_all[(size_t)(adj[t] / nn) * nd + 3 * (adj[t] % nn) + k];
        fint[3 * j + k] = s;
      }
  }
  (void)n;
  return 0;
}

// Consistent surface traction (problems_elasticity.jl:454-502): for each face and
// surface integration point, f += w·‖∂X/∂ξ₁ × ∂X/∂ξ₂‖·t ⊗ N.  t is 3 per face.
// f (length 3N) is accumulated into (not zeroed).
int orc_traction(int ft, i64 n_faces, const i64* fconn, const double* X, const double* t,
                 double* f) {
  const int nf = surface_nodes_of(ft);
  if (nf < 0) return -1;
  const Rule rule = surface_rule(ft);
  for (i64 s = 0; s < n_faces; ++s) {
    double fe[18] = {0};
    for (int q = 0; q < rule.nq; ++q) {
      double N[6], dN[6][2];
      surface_basis(ft, rule.xi[q], N, dN);
      double J[2][3] = {{0}};
      for (int i = 0; i < nf; ++i)
        for (int a = 0; a < 2; ++a)
          for (int b = 0; b < 3; ++b) J[a][b] += dN[i][a] * X[3 * fconn[s * nf + i] + b];
      const double cx = J[0][1] * J[1][2] - J[0][2] * J[1][1];
      const double cy = J[0][2] * J[1][0] - J[0][0] * J[1][2];
      const double cz = J[0][0] * J[1][1] - J[0][1] * J[1][0];
      const double w = rule.w[q] * std::sqrt(cx * cx + cy * cy + cz * cz);
      for (int i = 0; i < nf; ++i)
        for (int k = 0; k < 3; ++k) fe[3 * i + k] += w * t[3 * s + k] * N[i];
    }
    for (int i = 0; i < nf; ++i)
      for (int k = 0; k < 3; ++k) f[3 * fconn[s * nf + i] + k] += fe[3 * i + k];
  }
  return 0;
}

// Surface pressure (problems_elasticity.jl:486-493): for each face and surface
// integration point, n = (∂X/∂ξ₁ × ∂X/∂ξ₂)/‖·‖ and, positive pressure acting
// towards the surface, f += w·‖∂X/∂ξ₁ × ∂X/∂ξ₂‖·(−p)·n ⊗ N.  p is one value per
// face.  f (length 3N) is accumulated into (not zeroed).
int orc_pressure(int ft, i64 n_faces, const i64* fconn, const double* X, const double* p, double* f) {
  const int nf = surface_nodes_of(ft);
  if (nf < 0) return -1;
  const Rule rule = surface_rule(ft);
  for (i64 s = 0; s < n_faces; ++s) {
    double fe[18] = {0};
    for (int q = 0; q < rule.nq; ++q) {
      double N[6], dN[6][2];
      surface_basis(ft, rule.xi[q], N, dN);
      double J[2][3] = {{0}};
      for (int i = 0; i < nf; ++i)
        for (int a = 0; a < 2; ++a)
          for (int b = 0; b < 3; ++b) J[a][b] += dN[i][a] * X[3 * fconn[s * nf + i] + b];
      const double c[3] = {J[0][1] * J[1][2] - J[0][2] * J[1][1], J[0][2] * J[1][0] - J[0][0] * J[1][2],
                           J[0][0] * J[1][1] - J[0][1] * J[1][0]};
      const double a = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
      const double w = rule.w[q] * a;
      for (int i = 0; i < nf; ++i)
        for (int k = 0; k < 3; ++k) fe[3 * i + k] += w * (-p[s]) * (c[k] / a) * N[i];
    }
    for (int i = 0; i < nf; ++i)
      for (int k = 0; k < 3; ++k) f[3 * fconn[s * nf + i] + k] += fe[3 * i + k];
  }
  return 0;
}

// y = A x for a CSC matrix (column-oriented SpMV, element_assembly_structures.jl:307-309).
void orc_csc_spmv(i64 n, const i64* colptr, const i64* rowval, const double* nzval,
                  const double* x, double* y) {
  std::fill(y, y + n, 0.0);
  for (i64 c = 0; c < n; ++c) {
    const double xc = x[c];
    for (i64 k = colptr[c]; k < colptr[c + 1]; ++k) y[rowval[k]] += nzval[k] * xc;
  }
}

// Jacobi-preconditioned CG on the system with prescribed DOFs eliminated
// (solvers.jl:192-216 elimination; CG loop backend/cpu.jl:221-254).
// fixed[i] != 0 marks prescribed DOFs whose values are taken from x on entry;
// free DOFs start from x as given.  Stops when ‖r_I‖ ≤ tol·‖b_I − K_IB x_B‖.
// Matrix is CSC and symmetric; the SpMV is row-parallel over the CSC arrays
// read as CSR (valid by symmetry) so it can use threads.
int orc_pcg(i64 n, const i64* colptr, const i64* rowval, const double* nzval, const double* b,
            const unsigned char* fixed, double tol, int maxit, double* x, int* iters,
            double* relres) {
  std::vector<double> r(n), z(n), p(n), Ap(n), dinv(n, 0.0), xb(n, 0.0);
  for (i64 c = 0; c < n; ++c) {
    if (fixed[c]) xb[c] = x[c];
    for (i64 k = colptr[c]; k < colptr[c + 1]; ++k)
      if (rowval[k] == c && !fixed[c]) dinv[c] = 1.0 / nzval[k];
  }
  auto spmv_sym = [&](const std::vector<double>& v, std::vector<double>& y) {
#pragma omp parallel for schedule(static)
    for (i64 i = 0; i < n; ++i) {
      double s = 0.0;
      for (i64 k = colptr[i]; k < colptr[i + 1]; ++k) s += nzval[k] * v[rowval[k]];
      y[i] = s;
    }
  };
  // b' = b − K x_B on free rows
  spmv_sym(xb, Ap);
  double bn = 0.0;
  for (i64 i = 0; i < n; ++i) {
    if (fixed[i]) { r[i] = 0.0; continue; }
    r[i] = b[i] - Ap[i];
    bn += r[i] * r[i];
  }
  bn = std::sqrt(bn);
  // initial guess on free DOFs
  std::vector<double> x0(n);
  for (i64 i = 0; i < n; ++i) x0[i] = fixed[i] ? 0.0 : x[i];
  spmv_sym(x0, Ap);
  for (i64 i = 0; i < n; ++i) if (!fixed[i]) r[i] -= Ap[i];
  std::vector<double> xx(x0);
  double rz = 0.0, rn = 0.0;
  for (i64 i = 0; i < n; ++i) {
    z[i] = dinv[i] * r[i];
    p[i] = z[i];
    rz += r[i] * z[i];
    rn += r[i] * r[i];
  }
  if (bn == 0.0) bn = 1.0;
  int it = 0;
  while (std::sqrt(rn) > tol * bn && it < maxit) {
    spmv_sym(p, Ap);
    double pAp = 0.0;
    for (i64 i = 0; i < n; ++i) {
      if (fixed[i]) Ap[i] = 0.0;
      pAp += p[i] * Ap[i];
    }
    const double alpha = rz / pAp;
    double rz2 = 0.0;
    rn = 0.0;
    for (i64 i = 0; i < n; ++i) {
      xx[i] += alpha * p[i];
      r[i] -= alpha * Ap[i];
      z[i] = dinv[i] * r[i];
      rz2 += r[i] * z[i];
      rn += r[i] * r[i];
    }
    const double beta = rz2 / rz;
    rz = rz2;
    for (i64 i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    ++it;
  }
  for (i64 i = 0; i < n; ++i) x[i] = fixed[i] ? xb[i] : xx[i];
  if (iters) *iters = it;
  if (relres) *relres = std::sqrt(rn) / bn;
  return it < maxit || std::sqrt(rn) <= tol * bn ? 0 : 1;
}

// Matrix-free y = K(u) v summed element by element in FP64 (the operator the GPU
// apply computes).  For finite strain the tangent at state u is used.  y zeroed.
int orc_apply(int et, int model, int finite, int geom, i64 n_nodes, const double* X, i64 n_elem,
              const i64* conn, const double* E, const double* nu, int per_element,
              const double* u, const double* v, double* y) {
  const int nn = n_nodes_of(et);
  if (nn < 0) return -1;
  const int nd = 3 * nn;
  std::vector<double> ye_all((size_t)n_elem * nd);
  int err = 0;
#pragma omp parallel for schedule(static) reduction(min : err)
  for (i64 e = 0; e < n_elem; ++e) {
    double Xe[30], ue[30], ve[30], Ke[900], fe[30];
    gather_element(nn, conn, e, X, u, Xe, ue);
    for (int a = 0; a < nn; ++a)
      for (int k = 0; k < 3; ++k) ve[3 * a + k] = v[3 * conn[e * nn + a] + k];
    const double Ee = per_element ? E[e] : E[0];
    const double ne = per_element ? nu[e] : nu[0];
    const int rc = element_kernel(et, model, finite, geom, Xe, u ? ue : nullptr, Ee, ne, Ke, fe);
    if (rc < err) err = rc;
    for (int i = 0; i < nd; ++i) {
      double s = 0.0;
      for (int j = 0; j < nd; ++j) s += Ke[j * nd + i] * ve[j];
      ye_all[(size_t)e * nd + i] = s;
    }
  }
  if (err) return err;
  std::fill(y, y + 3 * n_nodes, 0.0);
  for (i64 e = 0; e < n_elem; ++e)
    for (int i = 0; i < nd; ++i) y[3 * conn[e * nn + i / 3] + i % 3] += ye_all[(size_t)e * nd + i];
  return 0;
}

}  // extern "C"
