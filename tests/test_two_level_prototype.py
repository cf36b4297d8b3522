"""Numerical experiment behind the design note on the learned preconditioner
(not part of the library): a Galerkin coarse space of rigid-body modes on node
aggregates, added to Jacobi, cuts the PCG iterations of a slender Tet10
cantilever by more than an order of magnitude.  CPU only: K assembled by the
oracle, CG in numpy/scipy."""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def _pcg(K, b, free, M, tol=1e-8, maxit=20000):
    x = np.zeros_like(b)
    r = b * free
    z = M(r)
    p = z.copy()
    rz = r @ z
    bb = np.sqrt(r @ r)
    for it in range(1, maxit + 1):
        q = (K @ (p * free)) * free
        a = rz / (p @ q)
        x += a * p
        r -= a * q
        if np.sqrt(r @ r) <= tol * bb:
            return x, it
        z = M(r)
        rzn = r @ z
        p = z + (rzn / rz) * p
        rz = rzn
    return x, maxit


def _rigid_body_coarse_space(X, free, box):
    """Columns: 3 translations and 3 small rotations about the centroid of every
    aggregate (nodes binned into boxes of edge `box`); prescribed rows zeroed."""
    X = X.reshape(-1, 3)
    n_nodes = X.shape[0]
    cell = np.floor((X - X.min(0)) / box + 1e-9).astype(np.int64)
    dims = cell.max(0) + 1
    _, agg = np.unique(cell[:, 0] + dims[0] * (cell[:, 1] + dims[1] * cell[:, 2]), return_inverse=True)
    n_agg = int(agg.max()) + 1
    cen = np.zeros((n_agg, 3))
    np.add.at(cen, agg, X)
    cen /= np.bincount(agg)[:, None]
    d = X - cen[agg]
    nodes = np.arange(n_nodes)
    rows, cols, vals = [], [], []
    for c in range(3):
        rows.append(3 * nodes + c)
        cols.append(6 * agg + c)
        vals.append(np.ones(n_nodes))
    rotations = [((1, -d[:, 2]), (2, d[:, 1])), ((0, d[:, 2]), (2, -d[:, 0])), ((0, -d[:, 1]), (1, d[:, 0]))]
    for k, comps in enumerate(rotations):
        for c, v in comps:
            rows.append(3 * nodes + c)
            cols.append(6 * agg + 3 + k)
            vals.append(v)
    P = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(3 * n_nodes, 6 * n_agg))
    P = (sp.diags(free.astype(float)) @ P).tocsc()
    P.eliminate_zeros()
    live = np.diff(P.indptr) > 0          # aggregates entirely on the clamped face carry no mode
    return P[:, live]


def test_rigid_body_coarse_space_cuts_pcg_iterations(jfem, orc):
    w = jfem.workloads.cantilever(10, 40, 4, 4, 10.0, 1.0, 1.0)
    m = w.mesh
    cp, rv, nz, _ = orc.assemble_coo(10, m.X, m.conn, w.E, w.nu)
    n = m.n_dofs
    K = sp.csc_matrix((nz, rv, cp), shape=(n, n))
    f = orc.traction(w.face_type, w.faces, m.X, w.traction)
    free = ~w.fixed_mask().astype(bool)
    fr = free.astype(float)
    dinv = np.where(free, 1.0 / K.diagonal(), 0.0)
    x1, it_jacobi = _pcg(K, f, fr, lambda r: dinv * r)
    P = _rigid_body_coarse_space(m.X, free, 0.5)
    Kc = (P.T @ (sp.diags(fr) @ K @ sp.diags(fr)) @ P).tocsc()
    lu = spla.splu(Kc)
    x2, it_two_level = _pcg(K, f, fr, lambda r: dinv * r + P @ lu.solve(P.T @ r))
    assert it_two_level * 10 <= it_jacobi, (it_jacobi, it_two_level)     # measured: 1,463 vs 91
    assert np.linalg.norm(x2 - x1) <= 1e-6 * np.linalg.norm(x1)
