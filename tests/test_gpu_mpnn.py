"""Learned preconditioner on the GPU, through the C ABI: gradients and the
preconditioner against the numpy oracle (oracle/mpnn_oracle.py), flexible CG
against Jacobi-PCG, training on solver-generated pairs, and the Jacobi fallback."""
import numpy as np
import pytest
import scipy.sparse as sp

import mpnn_oracle as mo
from conftest import rel_err
from test_mpnn_oracle import graph_from_conn

pytestmark = pytest.mark.gpu


def _setup(ctx, w, mesh=True):
    m = w.mesh
    if mesh:
        ctx.set_mesh(m.elem_type, m.X, m.conn)
    ctx.set_material(w.E, w.nu)
    if mesh:
        ctx.set_dirichlet(w.fixed_dofs, w.fixed_values)
    ctx.set_traction(w.face_type, w.faces, w.traction)


def _small(jfem):
    return jfem.workloads.learned_family(1, seed_item=900, nx=6, ny=2, nz=2, L=3.0)[0]


def _oracle_operator(orc, w):
    m = w.mesh
    cp, rv, nz, _ = orc.assemble_coo(10, m.X, m.conn, w.E, w.nu)
    K = sp.csc_matrix((nz, rv, cp), shape=(m.n_dofs, m.n_dofs))
    mask = w.fixed_mask().astype(bool)
    fm = (~mask).astype(np.float64)

    def kmul(v):
        return ((K @ (v.reshape(-1) * fm)) * fm).reshape(-1, 3)
    return K, mask, kmul


@pytest.mark.parametrize("coarse", [False, True])
def test_gradient_and_loss_match_oracle(jfem, orc, coarse):
    """One training pair through the GPU forward / adjoint / backward kernels
    (FP32, BF16 weights) against the FP64 oracle, same BF16 weights; with the
    coarse space on, z carries the coarse term Q r̃ (oracle: coarse_oracle's
    FP64 Q; GPU: the solver's FP32 coarse level)."""
    import coarse_oracle as co
    w = _small(jfem)
    m = w.mesh
    K, mask, kmul = _oracle_operator(orc, w)
    with jfem.Context(0) as ctx:
        _setup(ctx, w)
        ctx.set_coarse_space(-1 if coarse else 0)
        ctx.mpnn_init(7)
        p = ctx.mpnn_get_weights().astype(np.float64)
        assert np.array_equal(p, mo.bf16_round(p.astype(np.float32)))
        e = np.random.default_rng(1).standard_normal(m.n_dofs)
        e[mask] = 0.0
        r = ctx.apply(e, fp32=False, masked=True)
        L, g = ctx.mpnn_loss_grad(r, e)
    diag = K.diagonal()
    dinv = np.where(mask, 0.0, 1.0 / diag)
    v = np.sqrt(dinv) * r
    s = np.sqrt(np.sum(v * v) / np.sum(~mask))
    f32 = lambda a: a.astype(np.float32).astype(np.float64).reshape(-1, 3)
    y, t = f32(v / s), f32(np.where(mask, 0.0, e) / s)
    sq = f32(np.where(mask, 0.0, np.sqrt(diag)))
    G = graph_from_conn(m.n_nodes, m.conn.reshape(m.n_elem, -1))
    mask3 = (~mask).reshape(-1, 3).astype(np.float64)
    c = None
    if coarse:
        agg, na, _ = co.aggregates(m.X, co.auto_coarse_dofs(m.n_dofs))
        P = co.prolongation(m.X, agg, na, w.fixed_mask())
        c = co.two_level(K, P, w.fixed_mask())(r / s) - dinv * (r / s)     # Q r̃ alone
        c = c.reshape(-1, 3)
    Lo, go = mo.loss_and_grad(p, y, t, sq, G, mask3, kmul, c=c)
    tol_l, tol_g = (2e-5, 2e-4) if coarse else (1e-5, 1e-4)       # FP32 coarse level on the GPU
    assert abs(L - Lo) <= tol_l * abs(Lo)
    assert np.abs(g - go).max() <= tol_g * np.abs(go).max()      # FP32 sums over ~1e3 rows


def test_preconditioner_matches_oracle_and_is_spd(jfem, orc):
    w = _small(jfem)
    m = w.mesh
    K, mask, _ = _oracle_operator(orc, w)
    G = graph_from_conn(m.n_nodes, m.conn.reshape(m.n_elem, -1))
    mask3 = (~mask).reshape(-1, 3).astype(np.float64)
    rng = np.random.default_rng(4)
    a, b = rng.standard_normal(m.n_dofs), rng.standard_normal(m.n_dofs)
    with jfem.Context(0) as ctx:
        _setup(ctx, w)
        ctx.mpnn_init(11)
        p = ctx.mpnn_get_weights().astype(np.float64)
        za, zb = ctx.mpnn_precondition(a), ctx.mpnn_precondition(b)
    dinv = np.where(mask, 0.0, 1.0 / K.diagonal())
    zo = mo.precondition(p, a, dinv, G, mask3)
    assert rel_err(za, zo) <= 1e-5
    assert abs(za @ b - zb @ a) <= 1e-5 * abs(za @ b) + 1e-12
    assert za @ a > 0.0 and np.all(za[mask] == 0.0)


def test_fcg_with_zero_network_is_jacobi_pcg(jfem):
    """With Nᵀ N = 0 the preconditioner is Jacobi and flexible CG is PCG in
    exact arithmetic; in finite precision the two β formulas (z·q_old / p·q vs
    r·z ratios) give different iteration counts, the same solution.  The system
    is homogeneous and small (a few hundred iterations): on the heterogeneous
    40×4×4 family members (σ_log 0.5, ~3,000 Jacobi iterations) both counts move
    by 15–30 % with the summation order alone — loss of orthogonality, not the
    method — so they cannot test this identity."""
    w = jfem.workloads.learned_family(1, seed_item=901, nx=12, ny=3, nz=3, L=4.0, sigma_log=0.0)[0]
    with jfem.Context(0) as ctx:
        _setup(ctx, w)
        ctx.set_coarse_space(0)                  # one-level: the learned method without a coarse space
        ctx.mpnn_set_weights(np.zeros(jfem._abi.MPNN_PARAMS, np.float32))
        u1, s1, rc1 = ctx.solve(method=jfem._abi.PCG_JACOBI, precision=1, tol=1e-8, max_iter=100000)
        u2, s2, rc2 = ctx.solve(method=jfem._abi.FCG_LEARNED, precision=1, tol=1e-8, max_iter=100000)
    assert rc1 == 0 and rc2 == 0 and s2.residual <= 1e-8
    assert abs(s2.cg_iterations - s1.cg_iterations) <= 0.25 * s1.cg_iterations
    assert rel_err(u2, u1) <= 1e-6


def test_trained_network_reduces_iterations_on_unseen_systems(jfem):
    """One-level (coarse space off): train on pairs the solver generates for 32
    systems of the Tet10 family (per-element lognormal E, random surface-patch
    tractions), then solve 3 unseen systems: learned FCG reaches the FP64
    relative residual 1e-8 in fewer iterations than Jacobi-PCG and than the
    same flexible CG with the network zeroed (Jacobi), on every one of them."""
    fam = jfem.workloads.learned_family(32, seed_item=40)
    ev = jfem.workloads.learned_family(3, seed_item=40 + 100000)
    with jfem.Context(0) as ctx:
        _setup(ctx, fam[0])
        ctx.set_coarse_space(0)
        ctx.mpnn_init(3)
        for w in fam:
            _setup(ctx, w, mesh=False)
            n = ctx.mpnn_collect(8, 1e-10)
        assert n == 8 * len(fam)
        l1 = ctx.mpnn_train(30, 32, 3e-3, seed=1)
        l2 = ctx.mpnn_train(30, 32, 1e-3, seed=2)
        assert l2[-1] < l1[0] < 1.0
        trained = ctx.mpnn_get_weights()
        zero = np.zeros_like(trained)
        gains, gains0 = [], []
        for w in ev:
            _setup(ctx, w, mesh=False)
            uj, sj, rcj = ctx.solve(method=jfem._abi.PCG_JACOBI, precision=1, tol=1e-8, max_iter=100000)
            ctx.mpnn_set_weights(zero)
            _, s0, rc0 = ctx.solve(method=jfem._abi.FCG_LEARNED, precision=1, tol=1e-8, max_iter=100000)
            ctx.mpnn_set_weights(trained)
            ul, sl, rcl = ctx.solve(method=jfem._abi.FCG_LEARNED, precision=1, tol=1e-8, max_iter=100000)
            assert rcj == 0 and rc0 == 0 and rcl == 0 and sl.residual <= 1e-8 and sl.fallbacks == 0
            assert rel_err(ul, uj) <= 1e-6
            gains.append(sj.cg_iterations / sl.cg_iterations)
            gains0.append(s0.cg_iterations / sl.cg_iterations)
        assert min(gains) > 1.05 and min(gains0) > 1.05, (gains, gains0)


def test_fcg_falls_back_to_jacobi_when_the_network_fails(jfem):
    """A network that produces NaN: the FP64 true residual judges the iterate
    non-finite, the solve continues with Jacobi from the best iterate and still
    converges (status JFEM_STALL, one fallback)."""
    w = jfem.workloads.learned_family(1, seed_item=902)[0]
    with jfem.Context(0) as ctx:
        _setup(ctx, w)
        ctx.mpnn_set_weights(np.full(jfem._abi.MPNN_PARAMS, np.nan, np.float32))
        u, st, rc = ctx.solve(method=jfem._abi.FCG_LEARNED, precision=1, tol=1e-8, max_iter=100000)
        uj, sj, _ = ctx.solve(method=jfem._abi.PCG_JACOBI, precision=1, tol=1e-8, max_iter=100000)
    assert rc == jfem._abi.STALL and st.fallbacks == 1 and st.residual <= 1e-8
    assert rel_err(u, uj) <= 1e-6


def test_weights_survive_a_new_mesh(jfem):
    w1 = _small(jfem)
    w2 = jfem.workloads.learned_family(1, seed_item=903, nx=8, ny=2, nz=2, L=4.0)[0]
    with jfem.Context(0) as ctx:
        _setup(ctx, w1)
        ctx.mpnn_init(5)
        p1 = ctx.mpnn_get_weights()
        _setup(ctx, w2)
        assert np.array_equal(ctx.mpnn_get_weights(), p1)
        with pytest.raises(jfem.JFEMError):
            ctx.mpnn_train(1, 8, 1e-3)          # pairs belong to the previous mesh


def test_two_level_learned_network_gain(jfem):
    """Two-level (coarse space on, the default): the network trained on pairs
    carrying the coarse term learns the fine-level correction the coarse space
    leaves.  On 3 unseen systems of the family, learned two-level FCG reaches
    1e-8 in fewer iterations in total than the same solver with the network
    zeroed (two-level Jacobi), and both need several times fewer than
    Jacobi-PCG; every solve matches Jacobi-PCG's displacement."""
    fam = jfem.workloads.learned_family(32, seed_item=40)
    ev = jfem.workloads.learned_family(3, seed_item=40 + 100000)
    abi = jfem._abi
    with jfem.Context(0) as ctx:
        _setup(ctx, fam[0])
        ctx.mpnn_init(3)
        for w in fam:
            _setup(ctx, w, mesh=False)
            ctx.mpnn_collect(8, 1e-10)
        l1 = ctx.mpnn_train(30, 32, 3e-3, seed=1)
        l2 = ctx.mpnn_train(30, 32, 1e-3, seed=2)
        assert l2[-1] < l1[0] < 1.0
        trained = ctx.mpnn_get_weights()
        its_j, its_0, its_l = [], [], []
        for w in ev:
            _setup(ctx, w, mesh=False)
            uj, sj, rcj = ctx.solve(method=abi.PCG_JACOBI, precision=1, tol=1e-8, max_iter=100000)
            u0, s0, rc0 = ctx.solve(method=abi.FCG_TWO_LEVEL, precision=1, tol=1e-8, max_iter=100000)
            ctx.mpnn_set_weights(np.zeros_like(trained))
            uz, sz, rcz = ctx.solve(method=abi.FCG_LEARNED, precision=1, tol=1e-8, max_iter=100000)
            ctx.mpnn_set_weights(trained)
            ul, sl, rcl = ctx.solve(method=abi.FCG_LEARNED, precision=1, tol=1e-8, max_iter=100000)
            assert rcj == rc0 == rcz == rcl == 0 and sl.fallbacks == 0 and sl.residual <= 1e-8
            # zeroed network = two-level Jacobi up to rounding (z = √d(√d r) instead of d r in FP32)
            assert abs(sz.cg_iterations - s0.cg_iterations) <= max(2, 0.05 * s0.cg_iterations)
            for u in (u0, uz, ul):
                assert rel_err(u, uj) <= 1e-6
            its_j.append(sj.cg_iterations)
            its_0.append(s0.cg_iterations)
            its_l.append(sl.cg_iterations)
    assert sum(its_l) < sum(its_0) and 4 * sum(its_0) <= sum(its_j), (its_j, its_0, its_l)
