"""The coarse-space oracle (oracle/coarse_oracle.py) pinned by exact properties:
global rigid-body motions built from the aggregate modes lie in the null space
of A_c = Pᵀ K P for an unconstrained mesh; A_c is symmetric positive definite
once the cantilever is clamped; and the two-level preconditioner it defines
cuts the Jacobi-PCG iterations of a slender Tet10 cantilever by an order of
magnitude while converging to the same displacement."""
import numpy as np
import pytest
import scipy.sparse as sp

import coarse_oracle as co


def _K(orc, w):
    m = w.mesh
    cp, rv, nz, _ = orc.assemble_coo(m.elem_type, m.X, m.conn, w.E, w.nu)
    return sp.csc_matrix((nz, rv, cp), shape=(m.n_dofs, m.n_dofs)).tocsr()


@pytest.mark.parametrize("et", [4, 10, 8])
def test_global_rigid_motions_are_in_the_null_space(jfem, orc, et):
    m = jfem.mesh.box_mesh(et, 6, 3, 3, 3.0, 1.0, 1.0)
    cp, rv, nz, _ = orc.assemble_coo(et, m.X, m.conn, 210e3, 0.3)
    K = sp.csc_matrix((nz, rv, cp), shape=(m.n_dofs, m.n_dofs))
    agg, na, nb = co.aggregates(m.X, 96)
    assert na == np.prod(nb) and na >= 8
    P = co.prolongation(m.X, agg, na, np.zeros(m.n_dofs, np.uint8))
    Ac = co.coarse_matrix(K, P)
    scale = np.abs(Ac).max()
    cen = np.zeros((na, 3))
    np.add.at(cen, agg, m.X)
    cen /= np.bincount(agg)[:, None]
    for k in range(3):
        g = np.zeros(6 * na)
        g[k::6] = 1.0                                            # the same translation everywhere
        assert np.abs(Ac @ g).max() <= 1e-10 * scale
        om = np.eye(3)[k]                                        # rotation ω = e_k about the origin
        g = np.zeros(6 * na)
        g[0::6], g[1::6], g[2::6] = np.cross(om, cen).T
        g[3 + k::6] = 1.0
        assert np.abs(Ac @ g).max() <= 1e-10 * scale * max(1.0, np.abs(g).max())


def test_two_level_cuts_cantilever_iterations(jfem, orc):
    w = jfem.workloads.cantilever(10, 40, 4, 4, 10.0, 1.0, 1.0)
    m = w.mesh
    K = _K(orc, w)
    f = orc.traction(w.face_type, w.faces, m.X, w.traction)
    fixed = w.fixed_mask()
    agg, na, nb = co.aggregates(m.X, co.auto_coarse_dofs(m.n_dofs))
    P = co.prolongation(m.X, agg, na, fixed)
    Ac = co.coarse_matrix(K, P)
    assert np.allclose(Ac, Ac.T, rtol=0, atol=1e-12 * np.abs(Ac).max())
    assert np.linalg.eigvalsh(Ac).min() > 0.0
    free = fixed.reshape(-1) == 0
    dinv = np.where(free, 1.0 / K.diagonal(), 0.0)
    x1, it_j = co.pcg(K, f, fixed, lambda r: dinv * r)
    x2, it_2 = co.pcg(K, f, fixed, co.two_level(K, P, fixed))
    assert it_2 * 8 <= it_j, (it_j, it_2)
    assert np.linalg.norm(x2 - x1) <= 1e-6 * np.linalg.norm(x1)
