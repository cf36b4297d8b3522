"""Two-level preconditioner (jfem_coarse.cu) through the C ABI against the
numpy/scipy restatement in oracle/coarse_oracle.py: the aggregation, the double-float
coarse matrix A_c = Pᵀ K P (≤ 1e-12 relative; K from the oracle's FP64
assembly), the preconditioner z = D⁻¹r + P A_c⁻¹ Pᵀ r applied by the solver's
kernels (FP32 coarse solve), and flexible CG with it: the displacement of the
oracle's direct solve, and the iteration count of the oracle's FP64 two-level
PCG on the same aggregation."""
import numpy as np
import pytest
import scipy.sparse as sp

import coarse_oracle as co
from conftest import rel_err

pytestmark = pytest.mark.gpu


def _oracle_K(orc, et, X, conn, E, nu):
    cp, rv, nz, _ = orc.assemble_coo(et, X, conn, E, nu)
    n = 3 * X.shape[0]
    return sp.csc_matrix((nz, rv, cp), shape=(n, n)).tocsr(), (cp, rv, nz)


@pytest.mark.parametrize("et,dims,distort", [(10, (12, 3, 3), 0.0), (10, (8, 3, 2), 0.02), (8, (10, 4, 3), 0.02),
                                             (4, (12, 4, 4), 0.0)])
def test_coarse_matrix_matches_oracle(jfem, orc, gpu_ctx_factory, et, dims, distort):
    """Aggregation bit-identical; A_c within 1e-12 of the oracle's Pᵀ K P on
    clamped boxes with per-element E (affine and, distorted, per-point geometry)."""
    w = jfem.workloads.cantilever(et, *dims, 4.0, 1.0, 1.0)
    m = w.mesh
    g = np.random.default_rng(et + 7)
    X = m.X + distort * g.standard_normal(m.X.shape) * (4.0 / dims[0])
    E = g.uniform(80e3, 300e3, m.n_elem)
    with gpu_ctx_factory() as ctx:
        ctx.set_mesh(et, X, m.conn)
        ctx.set_material(E, 0.3)
        ctx.set_dirichlet(w.fixed_dofs)
        ctx.set_coarse_space(96)
        na_gpu, nc_gpu, n_listed, _ = ctx.coarse_info()
        Ac_gpu, agg_gpu = ctx.coarse_matrix()
    agg, na, nb = co.aggregates(X, 96)
    assert na == na_gpu and nc_gpu == 6 * na and 0 < n_listed <= m.n_elem
    assert np.array_equal(agg_gpu, agg)
    K, _ = _oracle_K(orc, et, X, m.conn, E, 0.3)
    P = co.prolongation(X, agg, na, w.fixed_mask())
    Ac = co.coarse_matrix(K, P)
    assert rel_err(Ac_gpu, Ac) <= 1e-12
    assert np.array_equal(Ac_gpu, Ac_gpu.T)          # element blocks mirrored exactly


def test_coarse_preconditioner_matches_oracle(jfem, orc, gpu_ctx_factory):
    """z = D⁻¹r + P A_c⁻¹ Pᵀ r for random residuals: the solver's FP32
    restriction, coarse solve and prolongation against the oracle in FP64."""
    w = jfem.workloads.cantilever(10, 20, 3, 3, 5.0, 1.0, 1.0)
    m = w.mesh
    g = np.random.default_rng(3)
    fixed = w.fixed_mask().astype(bool)
    with gpu_ctx_factory(w) as ctx:
        ctx.set_coarse_space(-1)
        K, _ = _oracle_K(orc, 10, m.X, m.conn, w.E, w.nu)
        agg, na, _ = co.aggregates(m.X, co.auto_coarse_dofs(m.n_dofs))
        M = co.two_level(K, co.prolongation(m.X, agg, na, w.fixed_mask()), w.fixed_mask())
        for _ in range(2):
            r = g.standard_normal(m.n_dofs)
            r[fixed] = 0.0
            z = ctx.coarse_precondition(r)
            assert rel_err(z, M(r)) <= 2e-5
            assert np.all(z[fixed] == 0.0)


@pytest.mark.parametrize("et,dims", [(10, (40, 4, 4)), (4, (40, 6, 6))])
def test_two_level_fcg_solve(jfem, orc, gpu_ctx_factory, et, dims):
    """Flexible CG with the two-level preconditioner to 1e-10: u within 1e-8 of
    the oracle's direct solve; at least 8× fewer iterations than Jacobi-PCG;
    no more than 25 % (+5) above the oracle's FP64 two-level PCG on the same
    aggregation (the GPU applies the coarse level in FP32)."""
    w = jfem.workloads.cantilever(et, *dims, 10.0, 1.0, 1.0)
    m = w.mesh
    abi = jfem._abi
    with gpu_ctx_factory(w) as ctx:
        _, st_j, rc_j = ctx.solve(method=abi.PCG_JACOBI, precision=abi.MIXED, tol=1e-10, max_iter=200000)
        u, st, rc = ctx.solve(method=abi.FCG_TWO_LEVEL, precision=abi.MIXED, tol=1e-10, max_iter=200000)
        na, nc, _, setup_ms = ctx.coarse_info()
    assert rc_j == 0 and rc == 0 and st.residual <= 1e-10 and setup_ms > 0.0
    K, (cp, rv, nz) = _oracle_K(orc, et, m.X, m.conn, w.E, w.nu)
    f = orc.traction(w.face_type, w.faces, m.X, w.traction)
    uo = orc.direct_solve(cp, rv, nz, f, w.fixed_mask().astype(bool))
    assert rel_err(u, uo) <= 1e-8
    assert st.cg_iterations * 8 <= st_j.cg_iterations, (st_j.cg_iterations, st.cg_iterations)
    agg, na_o, _ = co.aggregates(m.X, co.auto_coarse_dofs(m.n_dofs))
    assert na_o == na
    _, it_o = co.pcg(K, f, w.fixed_mask(), co.two_level(K, co.prolongation(m.X, agg, na, w.fixed_mask()),
                                                         w.fixed_mask()), tol=1e-10)
    assert st.cg_iterations <= 1.25 * it_o + 5, (st.cg_iterations, it_o)


def test_coarse_space_follows_material_and_mask(jfem, gpu_ctx_factory):
    """A new material or Dirichlet set rebuilds the coarse level (the solve
    stays converged and matches a fresh context); coarse_dofs 0 leaves the
    learned method one-level, and the two-level method still uses the
    automatic size."""
    w = jfem.workloads.cantilever(10, 20, 2, 2, 5.0, 1.0, 1.0)
    abi = jfem._abi
    E2 = np.random.default_rng(9).uniform(50e3, 300e3, w.mesh.n_elem)
    with gpu_ctx_factory(w) as ctx:
        u1, st1, _ = ctx.solve(method=abi.FCG_TWO_LEVEL, precision=abi.MIXED, tol=1e-10, max_iter=100000)
        ctx.set_material(E2, 0.3)
        u2, st2, rc2 = ctx.solve(method=abi.FCG_TWO_LEVEL, precision=abi.MIXED, tol=1e-10, max_iter=100000)
        ctx.set_coarse_space(0)
        u3, st3, rc3 = ctx.solve(method=abi.FCG_TWO_LEVEL, precision=abi.MIXED, tol=1e-10, max_iter=100000)
    with gpu_ctx_factory(w) as fresh:
        fresh.set_material(E2, 0.3)
        u4, st4, _ = fresh.solve(method=abi.FCG_TWO_LEVEL, precision=abi.MIXED, tol=1e-10, max_iter=100000)
    assert rc2 == 0 and rc3 == 0 and st2.residual <= 1e-10
    assert np.array_equal(u2, u4) and st2.cg_iterations == st4.cg_iterations   # deterministic rebuild
    assert rel_err(u3, u2) <= 1e-8
    assert not np.array_equal(u1, u2)
