"""Nodal strain / stress recovery on the GPU (jfem_recover_field) against the
numpy restatement of the reference's least-squares fit."""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("et,dims", [(10, (8, 2, 2)), (4, (10, 3, 3)), (8, (6, 3, 2))])
def test_recovery_matches_oracle(jfem, npo, et, dims):
    w = jfem.workloads.cantilever(et, *dims, 4.0, 1.0, 1.0)
    m = w.mesh
    E = np.random.default_rng(et).uniform(100e3, 300e3, m.n_elem)
    with jfem.Context(0) as ctx:
        ctx.set_mesh(m.elem_type, m.X, m.conn)
        ctx.set_material(E, 0.3)
        ctx.set_dirichlet(w.fixed_dofs)
        ctx.set_traction(w.face_type, w.faces, w.traction)
        u, st, rc = ctx.solve(method=0, precision=0, tol=1e-10, max_iter=100000)
        assert rc == 0
        for field in (0, 1):
            got = ctx.recover_field(u, field, tol=1e-13)
            ref = npo.lsq_fit(et, m.X, m.conn, E, 0.3, u, field)
            assert rel_err(got, ref) <= 1e-9


def test_recovery_patch_test_fixture(jfem):
    """The reference's cube_tet4.inp patch test: uniform stress (0, 0, −1) at every node."""
    from conftest import GOLDEN
    d = np.load(GOLDEN / "cube_tet4.npz")
    with jfem.Context(0) as ctx:
        ctx.set_mesh(4, d["X"], d["conn"])
        ctx.set_material(float(d["E"]), float(d["nu"]))
        s = ctx.recover_field(d["u_exact"], 1, tol=1e-14)
    ref = np.zeros(6)
    ref[2] = -1.0
    assert np.abs(s - ref).max() <= 1e-10
