// jfem_abi.cu — extern "C" entry points of libjfem_cuda.so (declared in
// include/jfem.h, which names the reference interface each one replaces).
#include <cstdio>
#include <cstring>
#include <new>
#include <utility>

#include "jfem_common.cuh"
#include "jfem_abi_guard.h"

namespace jfem {

int set_err(Ctx* c, int code, const std::string& msg) {
  c->err = msg;
  return code;
}

int cuda_check(Ctx* c, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return 0;
  return set_err(c, e == cudaErrorMemoryAllocation ? JFEM_ERR_OOM : JFEM_ERR_CUDA,
                 std::string(what) + ": " + cudaGetErrorString(e));
}

int sync_and_check(Ctx* c, const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_check(c, e, what);
  e = cudaStreamSynchronize(c->stream);
  return cuda_check(c, e, what);
}

void dfree(Ctx* c, void* p) {
  if (!p) return;
  for (size_t i = 0; i < c->owned.size(); ++i)
    if (c->owned[i] == p) {
      c->owned[i] = c->owned.back();
      c->owned.pop_back();
      break;
    }
  cudaFree(p);
}

void free_mesh(Ctx* c) {
  cudaStreamSynchronize(c->stream);
  if (c->pcg_graph) {
    cudaGraphExecDestroy(c->pcg_graph);
    c->pcg_graph = nullptr;
    c->pcg_graph_key = -1;
  }
  for (void* p : c->owned) cudaFree(p);
  c->owned.clear();
  Ctx fresh;
  // keep device, stream, events, pinned mirrors, counters
  fresh.device = c->device;
  fresh.stream = c->stream;
  fresh.ev0 = c->ev0;
  fresh.ev1 = c->ev1;
  fresh.sc_host = c->sc_host;
  fresh.norms_host = c->norms_host;
  fresh.mp = c->mp;
  fresh.coarse_target = c->coarse_target;
  fresh.geo_gen = c->geo_gen + 1;
  fresh.mask_gen = c->mask_gen + 1;
  fresh.launches = c->launches;
  fresh.err = std::move(c->err);
  *c = std::move(fresh);   // moves only: nothing here allocates, so this cannot throw
}

}  // namespace jfem

using jfem::Ctx;

static int enter(jfem_ctx* h) {
  if (!h) return JFEM_ERR_INVALID;
  const cudaError_t e = cudaSetDevice(h->c.device);
  if (e != cudaSuccess) return jfem::cuda_check(&h->c, e, "cudaSetDevice");
  return 0;
}

#define ENTER(h)                 \
  do {                           \
    const int _rc = enter(h);    \
    if (_rc) return _rc;         \
  } while (0)

extern "C" {

const char* jfem_version(void) { return "jfem-gb300 0.1 (sm_103a)"; }

void jfem_default_opts(jfem_solve_opts* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->method = JFEM_PCG_JACOBI;
  o->precision = JFEM_MIXED;
  o->tol = 1e-6;
  o->max_iter = 1000;
  o->newton_tol = 1e-6;
  o->max_newton = 20;
  o->max_cg_per_newton = 50;
  o->n_load_steps = 1;
  o->forcing_power = 0.5;
  o->forcing_max = 0.9;
  o->time_budget_s = 0.0;
}

int jfem_create(jfem_ctx** out, int device_ordinal) {
  ABI_TRY
  if (!out) return JFEM_ERR_INVALID;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return JFEM_ERR_CUDA;
  if (device_ordinal < 0 || device_ordinal >= ndev) return JFEM_ERR_INVALID;
  if (cudaSetDevice(device_ordinal) != cudaSuccess) return JFEM_ERR_CUDA;
  jfem_ctx* h = new (std::nothrow) jfem_ctx();
  if (!h) return JFEM_ERR_OOM;
  Ctx* c = &h->c;
  c->device = device_ordinal;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess ||
      cudaMallocHost(&c->sc_host, sizeof(jfem::SolverScalars)) != cudaSuccess ||
      cudaMallocHost(&c->norms_host, 2 * sizeof(double)) != cudaSuccess) {
    delete h;
    return JFEM_ERR_CUDA;
  }
  *out = h;
  return JFEM_OK;
  ABI_CATCH(nullptr)
}

int jfem_destroy(jfem_ctx* h) {
  ABI_TRY
  if (!h) return JFEM_OK;
  cudaSetDevice(h->c.device);
  Ctx* c = &h->c;
  jfem::free_mesh(c);
  if (c->mp) {
    cudaFree(c->mp->w32);
    cudaFree(c->mp->wbf);
    cudaFree(c->mp->m);
    cudaFree(c->mp->v);
    cudaFree(c->mp->g);
    cudaFree(c->mp->poly);
    delete c->mp;
    c->mp = nullptr;
  }
  if (c->sc_host) cudaFreeHost(c->sc_host);
  if (c->norms_host) cudaFreeHost(c->norms_host);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete h;
  return JFEM_OK;
  ABI_CATCH(nullptr)
}

const char* jfem_last_error(const jfem_ctx* h) { return h ? h->c.err.c_str() : "null context"; }

int64_t jfem_kernel_launches(const jfem_ctx* h) { return h ? h->c.launches : 0; }

double jfem_last_apply_ms(const jfem_ctx* h) { return h ? h->c.last_apply_ms : 0.0; }

void* jfem_stream(const jfem_ctx* h) { return h ? (void*)h->c.stream : nullptr; }

int jfem_time_apply(jfem_ctx* h, int flags, int reps, double* ms_element, double* ms_gather) {
  ABI_TRY
  ENTER(h);
  Ctx* c = &h->c;
  if (c->N == 0 || !c->have_material) return jfem::set_err(c, JFEM_ERR_INVALID, "mesh and material must be set");
  if (!ms_element || !ms_gather) return jfem::set_err(c, JFEM_ERR_INVALID, "NULL output");
  return jfem::time_apply(c, (flags & JFEM_APPLY_FP32) != 0, (flags & JFEM_APPLY_MASKED) != 0, reps, ms_element,
                          ms_gather);
  ABI_CATCH(h ? &h->c.err : nullptr)
}

int jfem_time_assembly(jfem_ctx* h, int reps, double* ms_qpoint, double* ms_scatter, int64_t* nnz) {
  ABI_TRY
  ENTER(h);
  Ctx* c = &h->c;
  if (c->N == 0 || !c->have_material) return jfem::set_err(c, JFEM_ERR_INVALID, "mesh and material must be set");
  if (!ms_qpoint || !ms_scatter || !nnz) return jfem::set_err(c, JFEM_ERR_INVALID, "NULL output");
  *nnz = 9 * c->n_blocks;
  return jfem::time_assembly(c, reps, ms_qpoint, ms_scatter);
  ABI_CATCH(h ? &h->c.err : nullptr)
}

int jfem_set_mesh(jfem_ctx* h, int elem_type, int64_t n_nodes, const double* X, int64_t n_elem, const int64_t* conn,
                  int index_base) {
  ABI_TRY
  ENTER(h);
  Ctx* c = &h->c;
  c->err.clear();
  return jfem::mesh_setup(c, elem_type, n_nodes, X, n_elem, conn, index_base);
  ABI_CATCH(h ? &h->c.err : nullptr)
}

int jfem_set_material(jfem_ctx* h, int model, const double* E, const double* nu, int per_element) {
  ABI_TRY
  ENTER(h);
  Ctx* c = &h->c;
  if (c->N == 0) return jfem::set_err(c, JFEM_ERR_INVALID, "jfem_set_mesh must come first");
  if (model != JFEM_LINEAR_ELASTIC && model != JFEM_NEO_HOOKEAN)
    return jfem::set_err(c, JFEM_ERR_INVALID, "unknown material model");
  if (!E || !nu) return jfem::set_err(c, JFEM_ERR_INVALID, "E and nu are required");
  const int64_t ne = per_element ? c->E : 1;
  std::vector<double> lam(c->E), mu(c->E);
  for (int64_t e = 0; e < c->E; ++e) {
    const double Ee = E[per_element ? e : 0], ne_ = nu[per_element ? e : 0];
    if (!(Ee > 0.0) || !(ne_ > -1.0 && ne_ < 0.5))
      return jfem::set_err(c, JFEM_ERR_INVALID, "material needs E > 0 and -1 < nu < 0.5");
    lam[e] = Ee * ne_ / ((1.0 + ne_) * (1.0 - 2.0 * ne_));
    mu[e] = Ee / (2.0 * (1.0 + ne_));
  }
  (void)ne;
  int rc = 0;
  if (!c->lam64) {
    if ((rc = jfem::dalloc(c, &c->lam64, c->E))) return rc;
    if ((rc = jfem::dalloc(c, &c->mu64, c->E))) return rc;
  }
  cudaMemcpyAsync(c->lam64, lam.data(), c->E * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(c->mu64, mu.data(), c->E * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  if ((rc = jfem::sync_and_check(c, "material upload"))) return rc;
  c->model = model;
  c->have_material = true;
  jfem::geometry_invalidate(c);
  return JFEM_OK;
  ABI_CATCH(h ? &h->c.err : nullptr)
}

int jfem_set_formulation(jfem_ctx* h, int finite_strain, int geometric_stiffness) {
  ABI_TRY
  ENTER(h);
  Ctx* c = &h->c;
  c->finite = finite_strain ? 1 : 0;
  c->geom = geometric_stiffness ? 1 : 0;
  ++c->state_version;
  return JFEM_OK;
  ABI_CATCH(h ? &h->c.err : nullptr)
}

int jfem_set_dirichlet(jfem_ctx* h, int64_t n, const int64_t* dofs, const double* values, int index_base) {
  ABI_TRY
  ENTER(h);
  Ctx* c = &h->c;
  if (c->N == 0) return jfem::set_err(c, JFEM_ERR_INVALID, "jfem_set_mesh must come first");
  if (n < 0 || (n > 0 && !dofs)) return jfem::set_err(c, JFEM_ERR_INVALID, "bad Dirichlet arrays");
  std::vector<uint8_t> mask(c->N, 0);
  std::vector<double> g(3 * c->N, 0.0);
  int64_t nz = 0;
  for (int64_t i = 0; i < n; ++i) {
    const int64_t d = dofs[i] - index_base;
    if (d < 0 || d >= 3 * c->N) return jfem::set_err(c, JFEM_ERR_INVALID, "Dirichlet DOF out of range");
    mask[d / 3] |= (uint8_t)(1u << (d % 3));
    const double v = values ? values[i] : 0.0;
    g[d] = v;
    if (v != 0.0) ++nz;
  }
  cudaMemcpyAsync(c->mask, mask.data(), c->N, cudaMemcpyHostToDevice, c->stream);
  cudaMemcpyAsync(c->gvals, g.data(), 3 * c->N * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  c->n_fixed = n;
  c->n_fixed_nonzero = nz;
  ++c->mask_gen;
  return jfem::sync_and_check(c, "Dirichlet upload");
  ABI_CATCH(h ? &h->c.err : nullptr)
}

int jfem_set_traction(jfem_ctx* h, int face_type, int64_t n_faces, const int64_t* face_conn, const double* t,
                      int index_base) {
  ABI_TRY
  ENTER(h);
  if (n_faces > 0 && !t) return jfem::set_err(&h->c, JFEM_ERR_INVALID, "traction array is NULL");
  return jfem::faces_setup(&h->c, face_type, n_faces, face_conn, t, nullptr, index_base);
  ABI_CATCH(h ? &h->c.err : nullptr)
}

int jfem_set_surface_load(jfem_ctx* h, int face_type, int64_t n_faces, const int64_t* face_conn, const double* t,
                          const double* p, int index_base) {
  ABI_TRY
  ENTER(h);
  return jfem::faces_setup(&h->c, face_type, n_faces, face_conn, t, p, index_base);
  ABI_CATCH(h ? &h->c.err : nullptr)
}

int jfem_set_state(jfem_ctx* h, const double* u) {
  ABI_TRY
  ENTER(h);
  Ctx* c = &h->c;
  if (c->N == 0) return jfem::set_err(c, JFEM_ERR_INVALID, "jfem_set_mesh must come first");
  if (!u) {
    cudaMemsetAsync(c->u_state, 0, 3 * c->N * sizeof(double), c->stream);
    c->have_state = false;
  } else {
    cudaMemcpyAsync(c->u_state, u, 3 * c->N * sizeof(double), cudaMemcpyHostToDevice, c->stream);
    c->have_state = true;
  }
  ++c->state_version;
  return jfem::sync_and_check(c, "state upload");
  ABI_CATCH(h ? &h->c.err : nullptr)
}

int jfem_assemble_csc(jfem_ctx* h, int index_base, int64_t* nnz_inout, int64_t* colptr, int64_t* rowval,
                      double* nzval, double* f) {
  ABI_TRY
  ENTER(h);
  Ctx* c = &h->c;
  if (c->N == 0) return jfem::set_err(c, JFEM_ERR_INVALID, "jfem_set_mesh must come first");
  if (!c->have_material) return jfem::set_err(c, JFEM_ERR_INVALID, "jfem_set_material must come first");
  if (!nnz_inout) return jfem::set_err(c, JFEM_ERR_INVALID, "nnz_inout is NULL");
  const int64_t nnz = 9 * c->n_blocks;
  const int64_t n = 3 * c->N;
  if (!colptr && !rowval && !nzval && !f) {
    *nnz_inout = nnz;
    return JFEM_OK;
  }
  if (*nnz_inout < nnz && (rowval || nzval)) return jfem::set_err(c, JFEM_ERR_INVALID, "nnz_inout too small");
  *nnz_inout = nnz;
  int64_t *d_cp = nullptr, *d_rv = nullptr;
  double *d_nz = nullptr, *d_f = nullptr;
  int rc = 0;
  auto cleanup = [&]() {
    cudaFree(d_cp);
    cudaFree(d_rv);
    cudaFree(d_nz);
    cudaFree(d_f);
  };
  if ((colptr && cudaMalloc(&d_cp, (n + 1) * sizeof(int64_t)) != cudaSuccess) ||
      (rowval && cudaMalloc(&d_rv, nnz * sizeof(int64_t)) != cudaSuccess) ||
      (nzval && cudaMalloc(&d_nz, nnz * sizeof(double)) != cudaSuccess) ||
      (f && cudaMalloc(&d_f, n * sizeof(double)) != cudaSuccess)) {
    cleanup();
    return jfem::set_err(c, JFEM_ERR_OOM, "assembly output buffers");
  }
  double* d_fint = nullptr;
  if (f && cudaMalloc(&d_fint, n * sizeof(double)) != cudaSuccess) {
    cleanup();
    return jfem::set_err(c, JFEM_ERR_OOM, "assembly output buffers");
  }
  rc = jfem::assemble_csc_device(c, index_base, d_cp, d_rv, d_nz, d_fint);
  if (!rc && f) rc = jfem::traction_device(c, d_f);
  if (!rc && f) {
    // f = f_ext − f_int (problems_elasticity.jl:433)
    jfem::enqueue_axpy(c, n, -1.0, d_fint, d_f);
  }
  if (!rc) {
    if (colptr) cudaMemcpyAsync(colptr, d_cp, (n + 1) * sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream);
    if (rowval) cudaMemcpyAsync(rowval, d_rv, nnz * sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream);
    if (nzval) cudaMemcpyAsync(nzval, d_nz, nnz * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (f) cudaMemcpyAsync(f, d_f, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    rc = jfem::sync_and_check(c, "assembly download");
  }
  cudaFree(d_fint);
  cleanup();
  return rc;
  ABI_CATCH(h ? &h->c.err : nullptr)
}

int jfem_apply_device(jfem_ctx* h, const double* v, double* y, int flags) {
  ABI_TRY
  ENTER(h);
  Ctx* c = &h->c;
  if (c->N == 0 || !c->have_material) return jfem::set_err(c, JFEM_ERR_INVALID, "mesh and material must be set");
  if (!v || !y) return jfem::set_err(c, JFEM_ERR_INVALID, "NULL vector");
  return jfem::apply_device(c, v, y, (flags & JFEM_APPLY_FP32) != 0, (flags & JFEM_APPLY_MASKED) != 0, nullptr);
  ABI_CATCH(h ? &h->c.err : nullptr)
}

int jfem_apply(jfem_ctx* h, const double* v, double* y, int flags) {
  ABI_TRY
  ENTER(h);
  Ctx* c = &h->c;
  if (c->N == 0 || !c->have_material) return jfem::set_err(c, JFEM_ERR_INVALID, "mesh and material must be set");
  if (!v || !y) return jfem::set_err(c, JFEM_ERR_INVALID, "NULL vector");
  const int64_t n = 3 * c->N;
  cudaMemcpyAsync(c->tmp, v, n * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  int rc = jfem::apply_device(c, c->tmp, c->tmp2, (flags & JFEM_APPLY_FP32) != 0, (flags & JFEM_APPLY_MASKED) != 0,
                              nullptr);
  if (rc) return rc;
  cudaMemcpyAsync(y, c->tmp2, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  return jfem::sync_and_check(c, "apply download");
  ABI_CATCH(h ? &h->c.err : nullptr)
}

int jfem_internal_force(jfem_ctx* h, double* f_int) {
  ABI_TRY
  ENTER(h);
  Ctx* c = &h->c;
  if (c->N == 0 || !c->have_material) return jfem::set_err(c, JFEM_ERR_INVALID, "mesh and material must be set");
  if (!f_int) return jfem::set_err(c, JFEM_ERR_INVALID, "NULL output");
  int rc = jfem::internal_force_device(c, c->tmp2);
  if (rc) return rc;
  cudaMemcpyAsync(f_int, c->tmp2, 3 * c->N * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  return jfem::sync_and_check(c, "internal force download");
  ABI_CATCH(h ? &h->c.err : nullptr)
}

int jfem_solve_device(jfem_ctx* h, const jfem_solve_opts* opts, double* u_device, jfem_stats* stats) {
  ABI_TRY
  ENTER(h);
  Ctx* c = &h->c;
  if (!u_device) return jfem::set_err(c, JFEM_ERR_INVALID, "NULL output");
  if (stats) std::memset(stats, 0, sizeof(*stats));
  const int rc = jfem::solve_device(c, opts, u_device, stats);
  if (stats && rc < 0) stats->status = rc;
  return rc;
  ABI_CATCH(h ? &h->c.err : nullptr)
}

int jfem_solve(jfem_ctx* h, const jfem_solve_opts* opts, double* u, jfem_stats* stats) {
  ABI_TRY
  ENTER(h);
  Ctx* c = &h->c;
  if (!u) return jfem::set_err(c, JFEM_ERR_INVALID, "NULL output");
  if (c->N == 0) return jfem::set_err(c, JFEM_ERR_INVALID, "jfem_set_mesh must come first");
  double* d_u = nullptr;
  if (cudaMalloc(&d_u, 3 * c->N * sizeof(double)) != cudaSuccess)
    return jfem::set_err(c, JFEM_ERR_OOM, "solution buffer");
  if (stats) std::memset(stats, 0, sizeof(*stats));
  int rc = jfem::solve_device(c, opts, d_u, stats);
  if (rc >= 0 || rc == JFEM_ERR_TIMEOUT) {   // on a timeout u receives the best iterate so far
    cudaMemcpyAsync(u, d_u, 3 * c->N * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    const int rc2 = jfem::sync_and_check(c, "solution download");
    if (rc2) rc = rc2;
  }
  if (stats && rc < 0) stats->status = rc;
  if (rc == JFEM_ERR_TIMEOUT) jfem::set_err(c, JFEM_ERR_TIMEOUT, "solve exceeded its time budget");
  cudaFree(d_u);
  return rc;
  ABI_CATCH(h ? &h->c.err : nullptr)
}

int jfem_recover_field(jfem_ctx* h, const double* u, int field, double tol, int max_iter, double* nodal,
                       int* iterations) {
  ABI_TRY
  ENTER(h);
  Ctx* c = &h->c;
  if (c->N == 0 || !c->have_material) return jfem::set_err(c, JFEM_ERR_INVALID, "mesh and material must be set");
  if (!u || !nodal) return jfem::set_err(c, JFEM_ERR_INVALID, "NULL array");
  if (field != JFEM_FIELD_STRAIN && field != JFEM_FIELD_STRESS)
    return jfem::set_err(c, JFEM_ERR_INVALID, "field must be JFEM_FIELD_STRAIN or JFEM_FIELD_STRESS");
  if (!(tol > 0.0) || max_iter <= 0) return jfem::set_err(c, JFEM_ERR_INVALID, "tol and max_iter must be positive");
  return jfem::recover_field(c, u, field, tol, max_iter, nodal, iterations);
  ABI_CATCH(h ? &h->c.err : nullptr)
}

int jfem_set_coarse_space(jfem_ctx* h, int coarse_dofs) {
  ABI_TRY
  ENTER(h);
  if (coarse_dofs > JFEM_COARSE_MAX_DOFS)
    return jfem::set_err(&h->c, JFEM_ERR_INVALID, "coarse_dofs above JFEM_COARSE_MAX_DOFS");
  h->c.coarse_target = coarse_dofs < 0 ? -1 : coarse_dofs;
  return JFEM_OK;
  ABI_CATCH(h ? &h->c.err : nullptr)
}

int jfem_coarse_info(jfem_ctx* h, int* n_aggregates, int* n_coarse_dofs, int64_t* n_elements, double* setup_ms) {
  ABI_TRY
  ENTER(h);
  Ctx* c = &h->c;
  if (c->N == 0 || !c->have_material) return jfem::set_err(c, JFEM_ERR_INVALID, "mesh and material must be set");
  return jfem::coarse_info(c, n_aggregates, n_coarse_dofs, n_elements, setup_ms);
  ABI_CATCH(h ? &h->c.err : nullptr)
}

int jfem_coarse_matrix(jfem_ctx* h, double* Ac, int* node_aggregate) {
  ABI_TRY
  ENTER(h);
  Ctx* c = &h->c;
  if (c->N == 0 || !c->have_material) return jfem::set_err(c, JFEM_ERR_INVALID, "mesh and material must be set");
  return jfem::coarse_matrix(c, Ac, node_aggregate);
  ABI_CATCH(h ? &h->c.err : nullptr)
}

int jfem_coarse_precondition(jfem_ctx* h, const double* r, double* z) {
  ABI_TRY
  ENTER(h);
  Ctx* c = &h->c;
  if (c->N == 0 || !c->have_material) return jfem::set_err(c, JFEM_ERR_INVALID, "mesh and material must be set");
  if (!r || !z) return jfem::set_err(c, JFEM_ERR_INVALID, "NULL array");
  return jfem::coarse_precondition(c, r, z);
  ABI_CATCH(h ? &h->c.err : nullptr)
}

int jfem_mpnn_init(jfem_ctx* h, uint64_t seed) {
  ABI_TRY
  ENTER(h);
  return jfem::mpnn_init(&h->c, seed);
  ABI_CATCH(h ? &h->c.err : nullptr)
}

int jfem_mpnn_set_weights(jfem_ctx* h, const float* w) {
  ABI_TRY
  ENTER(h);
  if (!w) return jfem::set_err(&h->c, JFEM_ERR_INVALID, "NULL weights");
  return jfem::mpnn_set_weights(&h->c, w);
  ABI_CATCH(h ? &h->c.err : nullptr)
}

int jfem_mpnn_get_weights(jfem_ctx* h, float* w) {
  ABI_TRY
  ENTER(h);
  if (!w) return jfem::set_err(&h->c, JFEM_ERR_INVALID, "NULL weights");
  return jfem::mpnn_get_weights(&h->c, w);
  ABI_CATCH(h ? &h->c.err : nullptr)
}

int jfem_mpnn_collect(jfem_ctx* h, int max_pairs, double tol) {
  ABI_TRY
  ENTER(h);
  Ctx* c = &h->c;
  if (c->N == 0 || !c->have_material) return jfem::set_err(c, JFEM_ERR_INVALID, "mesh and material must be set");
  if (!(tol > 0.0)) return jfem::set_err(c, JFEM_ERR_INVALID, "tol must be positive");
  return jfem::mpnn_collect(c, max_pairs, tol);
  ABI_CATCH(h ? &h->c.err : nullptr)
}

int jfem_mpnn_clear(jfem_ctx* h) {
  ABI_TRY
  ENTER(h);
  h->c.mp_pairs = 0;
  h->c.mp_coarse = -1;
  return JFEM_OK;
  ABI_CATCH(h ? &h->c.err : nullptr)
}

int jfem_mpnn_train(jfem_ctx* h, int epochs, int batch, double lr, uint64_t seed, double* losses) {
  ABI_TRY
  ENTER(h);
  return jfem::mpnn_train(&h->c, epochs, batch, lr, seed, losses);
  ABI_CATCH(h ? &h->c.err : nullptr)
}

int jfem_mpnn_loss_grad(jfem_ctx* h, const double* r, const double* e, double* loss, float* grad) {
  ABI_TRY
  ENTER(h);
  Ctx* c = &h->c;
  if (c->N == 0 || !c->have_material) return jfem::set_err(c, JFEM_ERR_INVALID, "mesh and material must be set");
  if (!r || !e || !loss || !grad) return jfem::set_err(c, JFEM_ERR_INVALID, "NULL argument");
  return jfem::mpnn_loss_grad(c, r, e, loss, grad);
  ABI_CATCH(h ? &h->c.err : nullptr)
}

int jfem_mpnn_precondition(jfem_ctx* h, const double* r, double* z) {
  ABI_TRY
  ENTER(h);
  Ctx* c = &h->c;
  if (c->N == 0 || !c->have_material) return jfem::set_err(c, JFEM_ERR_INVALID, "mesh and material must be set");
  if (!r || !z) return jfem::set_err(c, JFEM_ERR_INVALID, "NULL vector");
  return jfem::mpnn_precondition(c, r, z);
  ABI_CATCH(h ? &h->c.err : nullptr)
}

}  // extern "C"
