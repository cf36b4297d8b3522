"""The oracle itself: pinned against the reference fixture (patch test), closed
forms, and the independent numpy restatement; checked against the committed
golden vectors so it cannot drift."""
import hashlib

import numpy as np
import pytest

from conftest import GOLDEN, rel_err


def _hash(cp, rv):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(cp, dtype=np.int64).tobytes())
    h.update(np.ascontiguousarray(rv, dtype=np.int64).tobytes())
    return h.hexdigest()


@pytest.mark.parametrize("et,dims", [(4, (4, 2, 3)), (10, (3, 2, 2)), (8, (3, 3, 2))])
@pytest.mark.parametrize("model,finite", [(0, False), (0, True), (1, True)])
def test_cpp_matches_numpy_restatement(jfem, orc, npo, et, dims, model, finite):
    m = jfem.mesh.box_mesh(et, *dims, Lx=1.5, Ly=1.0, Lz=0.7)
    g = np.random.default_rng(1)
    u = 0.02 * g.standard_normal(m.n_dofs) if finite else None
    E = g.uniform(100e3, 300e3, m.n_elem)
    cp, rv, nz, fi = orc.assemble_coo(et, m.X, m.conn, E, 0.3, u=u, model=model, finite=finite, geom=finite)
    K, f2 = npo.assemble(et, m.X, m.conn, E, 0.3, u=u, model=model, finite=finite)
    assert np.array_equal(K.indptr, cp) and np.array_equal(K.indices, rv)
    assert rel_err(nz, K.data) < 1e-13
    if finite:
        assert rel_err(fi, f2) < 1e-12


def test_pattern_paths_agree(jfem, orc):
    m = jfem.mesh.box_mesh(10, 3, 2, 2)
    cp, rv, nz, fi = orc.assemble_coo(10, m.X, m.conn, 210e3, 0.3)
    cp2, rv2 = orc.pattern(10, m.n_nodes, m.conn)
    assert np.array_equal(cp, cp2) and np.array_equal(rv, rv2)
    nz2, _ = orc.assemble_pattern(10, m.X, m.conn, 210e3, 0.3, cp2, rv2)
    assert np.array_equal(nz, nz2)   # same ascending-element summation order


@pytest.mark.parametrize("et", [4, 10, 8])
def test_rigid_modes_and_symmetry(jfem, orc, et):
    m = jfem.mesh.box_mesh(et, 3, 2, 2, 2.0, 1.0, 1.0)
    cp, rv, nz, _ = orc.assemble_coo(et, m.X, m.conn, 210e3, 0.3)
    K = orc.to_scipy(cp, rv, nz).toarray()
    X = m.X
    modes = [np.tile(e, m.n_nodes) for e in np.eye(3)]
    modes += [np.stack([-X[:, 1], X[:, 0], 0 * X[:, 0]], 1).ravel(),
              np.stack([0 * X[:, 0], -X[:, 2], X[:, 1]], 1).ravel(),
              np.stack([X[:, 2], 0 * X[:, 0], -X[:, 0]], 1).ravel()]
    for r in modes:
        assert np.abs(K @ r).max() < 1e-10 * np.abs(K).max() * np.abs(r).max()
    assert np.abs(K - K.T).max() < 1e-12 * np.abs(K).max()
    ev = np.linalg.eigvalsh(K)
    assert (ev > -1e-8 * ev.max()).all() and (ev > 1e-8 * ev.max()).sum() == K.shape[0] - 6


def test_tet4_closed_form(orc):
    # K = V BᵀDB for a single Tet4 (constant strain)
    X = np.array([[0.1, 0.0, 0.0], [1.2, 0.1, 0.0], [0.2, 0.9, 0.1], [0.0, 0.2, 1.1]])
    E, nu = 210e3, 0.3
    Ke, _ = orc.element(4, X, E, nu)
    A = np.vstack([np.ones(4), X.T]).T
    V = np.linalg.det(A) / 6.0
    C = np.linalg.inv(A)            # rows 1..3 are ∂N/∂x
    g = C[1:, :].T                  # (4,3)
    B = np.zeros((6, 12))
    for a in range(4):
        gx, gy, gz = g[a]
        B[:, 3 * a:3 * a + 3] = [[gx, 0, 0], [0, gy, 0], [0, 0, gz], [gy, gx, 0], [0, gz, gy], [gz, 0, gx]]
    la = E * nu / ((1 + nu) * (1 - 2 * nu))
    mu = E / (2 * (1 + nu))
    D = np.zeros((6, 6))
    D[:3, :3] = la
    D[np.arange(3), np.arange(3)] = la + 2 * mu
    D[np.arange(3, 6), np.arange(3, 6)] = mu
    assert rel_err(Ke, V * B.T @ D @ B) < 1e-14


def test_patch_test_reference_fixture(orc):
    """test/testdata/cube_tet4.inp: symmetry planes + unit pressure → linear field."""
    d = np.load(GOLDEN / "cube_tet4.npz")
    X, conn, faces = d["X"], d["conn"], d["faces"]
    cp, rv, nz, _ = orc.assemble_coo(4, X, conn, float(d["E"]), float(d["nu"]))
    T = np.cross(X[faces[:, 1]] - X[faces[:, 0]], X[faces[:, 2]] - X[faces[:, 0]])
    t = -d["p"][:, None] * T / np.linalg.norm(T, axis=1)[:, None]
    f = orc.traction(3, faces, X, t)
    fixed = np.zeros(3 * len(X), bool)
    fixed[d["dofs"]] = True
    u = orc.direct_solve(cp, rv, nz, f, fixed)
    assert np.abs(u - d["u_exact"]).max() < 1e-12 * np.abs(d["u_exact"]).max()


@pytest.mark.parametrize("name", ["tet4_cantilever", "tet10_cantilever_small"])
def test_oracle_against_golden(jfem, orc, name):
    d = np.load(GOLDEN / f"{name}.npz")
    wl = jfem.workloads
    w = wl.cfg_tet4_cantilever() if name == "tet4_cantilever" else \
        wl.cantilever(10, 40, 4, 4, 4.0, 0.4, 0.4)
    m = w.mesh
    cp, rv, nz, _ = orc.assemble_coo(m.elem_type, m.X, m.conn, w.E, w.nu)
    assert _hash(cp, rv) == str(d["pattern_sha256"]) and nz.size == int(d["nnz"])
    assert rel_err(nz[d["sample_idx"]], d["sample_val"]) < 1e-13
    assert rel_err(orc.spmv(cp, rv, nz, d["w"]), d["Kw"]) < 1e-13
    f = orc.traction(w.face_type, w.faces, m.X, w.traction)
    assert rel_err(f, d["f"]) < 1e-14
    u, it, rr, st = orc.pcg(cp, rv, nz, f, w.fixed_mask(), tol=1e-12, maxit=200000)
    assert st == 0 and rel_err(u, d["u"]) < 1e-8


def test_cantilever_beam_theory(jfem, orc):
    """Tet10 cantilever tip deflection within 3% of Timoshenko beam theory."""
    d = np.load(GOLDEN / "tet10_cantilever_small.npz")
    w = jfem.workloads.cantilever(10, 40, 4, 4, 4.0, 0.4, 0.4)
    L, b, E, nu = 4.0, 0.4, 210e3, 0.3
    P = b * b * 1.0
    I = b ** 4 / 12
    G = E / (2 * (1 + nu))
    delta = P * L ** 3 / (3 * E * I) + P * L / (5 / 6 * G * b * b)
    tip = w.mesh.nodes_where(0, L)
    uz = d["u"].reshape(-1, 3)[tip, 2].mean()
    assert abs(-uz / delta - 1) < 0.03


def test_newton_oracle_golden(jfem, orc):
    d = np.load(GOLDEN / "hex8_neohookean_small.npz")
    w = jfem.workloads.cube_compression(n=4, steps=5, top_uz=-0.1)
    assert np.allclose(w.E, d["E"], rtol=0, atol=0)
    m = w.mesh
    u, its = orc.newton(8, m.X, m.conn, w.E, w.nu, w.fixed_mask().astype(bool), w.prescribed(),
                        n_steps=5, tol=1e-10, max_newton=25, model=1)
    assert rel_err(u, d["u"]) < 1e-9
    assert max(its) <= 8


@pytest.mark.parametrize("et", [4, 10, 8])
def test_lsq_fit_reproduces_a_uniform_field(jfem, npo, et):
    """The least-squares nodal fit (problems_elasticity.jl:554-583) of a linear
    displacement field returns its constant strain and stress at every node."""
    m = jfem.mesh.box_mesh(et, 3, 2, 2, 1.5, 1.0, 0.8)
    Gd = np.array([[1e-3, 2e-4, -3e-4], [5e-4, -2e-3, 1e-4], [0.0, 3e-4, 1.5e-3]])
    u = (m.X @ Gd.T).reshape(-1)
    eps = 0.5 * (Gd + Gd.T)
    la, mu = npo.lame(210e3, 0.3)
    sig = la * np.trace(eps) * np.eye(3) + 2 * mu * eps
    for field, t in ((0, eps), (1, sig)):
        x = npo.lsq_fit(et, m.X, m.conn, 210e3, 0.3, u, field)
        ref = np.array([t[0, 0], t[1, 1], t[2, 2], t[0, 1], t[1, 2], t[0, 2]])
        assert np.abs(x - ref).max() <= 1e-10 * np.abs(ref).max()


def _box_surface(jfem, et, dims, seed, amp=0.03):
    """All six faces of a distorted box mesh (curved Tri6 / warped Quad4)."""
    m = jfem.mesh.box_mesh(et, *dims, 1.4, 1.0, 0.8)
    X = m.X + amp * np.random.default_rng(seed).standard_normal(m.X.shape)
    flip = {3: [0, 2, 1], 6: [0, 2, 1, 5, 4, 3], 4: [0, 3, 2, 1]}   # reversed orientation, same face
    ft, faces = None, []
    for axis in range(3):
        for side in range(2):
            ft, fc = m.face(axis, side)
            P = m.X[fc]                                  # orient every side outward
            nrm = np.cross(P[:, 1] - P[:, 0], P[:, 2] - P[:, 0]).sum(0)
            if (nrm[axis] > 0) != (side == 1):
                fc = fc[:, flip[ft]]
            faces.append(fc)
    return m, X, ft, np.concatenate(faces)


@pytest.mark.parametrize("et", [4, 10, 8])
def test_surface_loads_cpp_matches_numpy(jfem, orc, npo, et):
    """Consistent traction and pressure (problems_elasticity.jl:454-502) for
    Tri3, Tri6 and Quad4 faces: the C++ oracle against the numpy restatement on
    non-planar faces with per-face values; a uniform pressure on the closed
    surface of a box has zero resultant; on one flat face it gives −p·A·n."""
    m, X, ft, faces = _box_surface(jfem, et, (3, 2, 2), seed=et)
    g = np.random.default_rng(10 + et)
    t = g.standard_normal((faces.shape[0], 3))
    p = g.uniform(0.5, 2.0, faces.shape[0])
    assert rel_err(orc.traction(ft, faces, X, t), npo.traction(ft, faces, X, t)) <= 1e-13
    assert rel_err(orc.pressure(ft, faces, X, p), npo.traction(ft, faces, X, np.zeros(3), p=p)) <= 1e-13
    # a closed (distorted) surface under uniform pressure: no net force
    fp = orc.pressure(ft, faces, X, 1.0)
    assert np.abs(fp.reshape(-1, 3).sum(0)).max() <= 1e-12 * np.abs(fp).max()
    # flat x = 1.4 face of the undistorted box: resultant −p·A·n (A = 1.0·0.8,
    # n = ±e_x by the face's orientation)
    ft1, f1 = m.face(0, 1)
    P = m.X[f1]
    n = np.sign(np.cross(P[:, 1] - P[:, 0], P[:, 2] - P[:, 0]).sum(0)[0])
    r = orc.pressure(ft1, f1, m.X, 2.5).reshape(-1, 3).sum(0)
    assert np.allclose(r, [-2.5 * 0.8 * n, 0.0, 0.0], rtol=0, atol=1e-12)
