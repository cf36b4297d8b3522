"""The numpy restatement of the learned preconditioner's network (oracle/mpnn_oracle.py),
pinned by central finite differences and by its symmetry properties, on CPU."""
import numpy as np

import mpnn_oracle as mo


def graph_from_conn(n_nodes, conn):
    nn = conn.shape[1]
    a = np.repeat(conn, nn, axis=1).ravel()
    b = np.tile(conn, (1, nn)).ravel()
    key = np.unique(a.astype(np.int64) * n_nodes + b)
    rows, cols = key // n_nodes, key % n_nodes
    ptr = np.zeros(n_nodes + 1, dtype=np.int64)
    np.cumsum(np.bincount(rows, minlength=n_nodes), out=ptr[1:])
    return mo.node_graph(ptr, cols)


def small_case(jfem, seed=3):
    """A Tet10 box with a random SPD stand-in for K on the node graph's 3×3 blocks."""
    m = jfem.mesh.box_mesh(10, 3, 2, 2, 3.0, 1.0, 1.0)
    g = graph_from_conn(m.n_nodes, m.conn.reshape(m.n_elem, -1))
    rng = np.random.default_rng(seed)
    mask3 = np.ones((m.n_nodes, 3))
    mask3[m.nodes_where(0, 0.0)] = 0.0
    n = 3 * m.n_nodes
    ptr, idx, rows = g
    w = rng.uniform(0.1, 1.0, rows.size)
    Kn = np.zeros((m.n_nodes, m.n_nodes))
    Kn[rows, idx] = -w
    Kn = 0.5 * (Kn + Kn.T)
    Kn[np.arange(m.n_nodes), np.arange(m.n_nodes)] = -Kn.sum(1) + 0.05
    K = np.kron(Kn, np.eye(3)) + 0.01 * np.eye(n)
    f = mask3.reshape(-1)
    K = K * f[:, None] * f[None, :]

    def kmul(v):
        return (K @ v.reshape(-1)).reshape(-1, 3)

    t = rng.standard_normal((m.n_nodes, 3)) * mask3
    sq = np.sqrt(np.diag(K)).reshape(-1, 3)
    y = (kmul(t) / np.where(sq > 0, sq, 1.0)) * mask3     # D^{-1/2} K t
    return g, mask3, y, t, sq, kmul


def test_gradient_matches_finite_differences(jfem):
    g, mask3, y, t, sq, kmul = small_case(jfem)
    p = mo.init_params(11)
    L, grad = mo.loss_and_grad(p, y, t, sq, g, mask3, kmul)
    assert 0.0 <= L <= 1.0
    rng = np.random.default_rng(0)
    for k in rng.choice(mo.N_PARAMS, 40, replace=False):
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        fd = (mo.loss(pp, y, t, sq, g, mask3, kmul) - mo.loss(pm, y, t, sq, g, mask3, kmul)) / (2 * h)
        assert abs(fd - grad[k]) <= 1e-6 * max(1.0, abs(fd)) + 1e-9, (k, fd, grad[k])


def test_adjoint_and_spd(jfem):
    """Nᵀ is the adjoint of N, and the preconditioner is symmetric positive definite."""
    g, mask3, y, _, sq, _ = small_case(jfem)
    p = mo.init_params(5)
    rng = np.random.default_rng(2)
    a = rng.standard_normal(y.shape) * mask3
    b = rng.standard_normal(y.shape) * mask3
    Na, _ = mo.forward(p, a, g, mask3)
    assert np.all(Na[mask3 == 0] == 0.0)
    assert abs(np.sum(Na * b) - np.sum(a * mo.adjoint(p, b, g, mask3))) <= 1e-12 * np.abs(Na).sum() * np.abs(b).max()
    dinv = np.where(sq > 0, 1.0 / np.where(sq > 0, sq, 1.0) ** 2, 0.0).reshape(-1)
    za = mo.precondition(p, a.reshape(-1), dinv, g, mask3)
    zb = mo.precondition(p, b.reshape(-1), dinv, g, mask3)
    assert abs(za @ b.reshape(-1) - zb @ a.reshape(-1)) <= 1e-10 * np.abs(za).max() * np.abs(b).sum()
    assert za @ a.reshape(-1) > 0.0


def test_bf16_rounding():
    w = np.array([1.0, 1.0 + 2.0 ** -9, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -9, -3.14159, 1e-3], dtype=np.float32)
    r = mo.bf16_round(w)
    # 7 stored mantissa bits: 1 + 2^-8 is a tie and rounds to the even neighbour 1.0
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 and r[3] == np.float32(1.0 + 2.0 ** -7)
    assert np.all(np.abs(r - w) <= np.abs(w) * 2.0 ** -8)
    assert np.all(mo.bf16_round(r) == r)
