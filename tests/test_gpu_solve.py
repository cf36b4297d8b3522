"""GPU solves through the C ABI and the reference-shaped host API."""
import numpy as np
import pytest

from conftest import GOLDEN, rel_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [0, 1])
def test_pcg_tet4_cantilever(jfem, gpu_ctx_factory, precision):
    w = jfem.workloads.cfg_tet4_cantilever()
    d = np.load(GOLDEN / "tet4_cantilever.npz")
    with gpu_ctx_factory(w) as ctx:
        u, st, rc = ctx.solve(method=0, precision=precision, tol=1e-10, max_iter=100000)
    assert rc == 0 and st.residual <= 1e-10
    assert rel_err(u, d["u"]) <= 1e-8
    assert np.all(u[w.fixed_dofs] == 0.0)


def test_pcg_tet10_small_cantilever_mixed(jfem, gpu_ctx_factory):
    w = jfem.workloads.cantilever(10, 40, 4, 4, 4.0, 0.4, 0.4)
    d = np.load(GOLDEN / "tet10_cantilever_small.npz")
    with gpu_ctx_factory(w) as ctx:
        u, st, rc = ctx.solve(method=0, precision=1, tol=1e-10, max_iter=200000)
        u2, st2, _ = ctx.solve(method=0, precision=1, tol=1e-10, max_iter=200000)
    assert rc == 0 and rel_err(u, d["u"]) <= 1e-8
    assert st.refinements >= 1
    assert np.array_equal(u, u2) and st.cg_iterations == st2.cg_iterations    # bit-reproducible


def test_patch_test_reference_fixture_gpu(jfem, gpu_ctx_factory):
    d = np.load(GOLDEN / "cube_tet4.npz")
    with gpu_ctx_factory() as ctx:
        ctx.set_mesh(4, d["X"], d["conn"])
        ctx.set_material(float(d["E"]), float(d["nu"]))
        ctx.set_dirichlet(d["dofs"], d["vals"])
        ctx.set_surface_load(3, d["faces"], p=d["p"])
        u, st, rc = ctx.solve(method=0, precision=0, tol=1e-12, max_iter=1000)
    assert np.abs(u - d["u_exact"]).max() <= 1e-10 * np.abs(d["u_exact"]).max()


def test_prescribed_nonzero_displacement(jfem, orc, gpu_ctx_factory):
    w = jfem.workloads.cantilever(4, 8, 2, 2, 4.0, 1.0, 1.0, traction=(0, 0, 0))
    m = w.mesh
    tip = m.nodes_where(0, 4.0)
    dofs = np.concatenate([w.fixed_dofs, 3 * tip + 2])
    vals = np.concatenate([np.zeros(w.fixed_dofs.size), np.full(tip.size, -0.01)])
    cp, rv, nz, _ = orc.assemble_coo(4, m.X, m.conn, 210e3, 0.3)
    fixed = np.zeros(m.n_dofs, bool)
    fixed[dofs] = True
    g = np.zeros(m.n_dofs)
    g[dofs] = vals
    uo = orc.direct_solve(cp, rv, nz, np.zeros(m.n_dofs), fixed, g=g)
    with gpu_ctx_factory() as ctx:
        ctx.set_mesh(4, m.X, m.conn)
        ctx.set_material(210e3, 0.3)
        ctx.set_dirichlet(dofs, vals)
        u, st, rc = ctx.solve(method=0, precision=1, tol=1e-10, max_iter=100000)
    assert rc == 0 and rel_err(u, uo) <= 1e-8


def test_newton_neo_hookean_cube(jfem, gpu_ctx_factory):
    w = jfem.workloads.cube_compression(n=4, steps=5, top_uz=-0.1)
    d = np.load(GOLDEN / "hex8_neohookean_small.npz")
    for precision in (0, 1):
        with gpu_ctx_factory(w) as ctx:
            u, st, rc = ctx.solve(method=2, precision=precision, tol=1e-10, newton_tol=1e-11, max_newton=30,
                                  max_cg_per_newton=2000, n_load_steps=5)
        assert rc == 0, st.status
        assert rel_err(u, d["u"]) <= 1e-8
        assert st.history_len == st.newton_iterations > 0


def test_newton_tangent_cache_follows_the_state(jfem, gpu_ctx_factory):
    """The mixed Newton solve reads a per-step cache of the Neo-Hookean point
    state; after the solve (u moved on) and after set_state, the FP32 tiled
    tangent apply at the current state must agree with the FP64 apply, so a
    stale cache cannot be used."""
    w = jfem.workloads.cube_compression(n=6, steps=3, top_uz=-0.1)
    v = np.random.default_rng(5).standard_normal(w.mesh.n_dofs)
    with gpu_ctx_factory(w) as ctx:
        u, st, rc = ctx.solve(method=2, precision=1, tol=1e-10, newton_tol=1e-10, max_newton=30,
                              max_cg_per_newton=2000, n_load_steps=3)
        assert rc == 0 and st.newton_iterations > 0
        ctx.set_state(u)
        y32, y64 = ctx.apply(v, fp32=True, masked=True), ctx.apply(v, fp32=False, masked=True)
        assert rel_err(y32, y64) <= 1e-5
        ctx.set_state(0.5 * u)
        z32, z64 = ctx.apply(v, fp32=True, masked=True), ctx.apply(v, fp32=False, masked=True)
        assert rel_err(z32, z64) <= 1e-5 and rel_err(z64, y64) > 1e-3
        u2, st2, rc2 = ctx.solve(method=2, precision=1, tol=1e-10, newton_tol=1e-10, max_newton=30,
                                 max_cg_per_newton=2000, n_load_steps=3)
    assert rc2 == 0 and rel_err(u2, u) <= 1e-7


def test_solve_api_physics(jfem):
    w = jfem.workloads.cfg_tet4_cantilever()
    d = np.load(GOLDEN / "tet4_cantilever.npz")
    ph = jfem.Physics(jfem.Tet4, w.mesh.X, w.mesh.conn, E=210e3, nu=0.3)
    jfem.add_dirichlet_(ph, w.mesh.nodes_where(0, 0.0))
    jfem.add_neumann_(ph, jfem.Tri3, w.faces, (0.0, 0.0, -1.0))
    sol = jfem.solve_(ph, backend=jfem.GPU(), tol=1e-10, max_iter=100000)
    assert isinstance(sol, jfem.ElasticitySolution)
    assert sol.newton_iterations == 1 and sol.cg_iterations > 0 and sol.residual <= 1e-10
    assert rel_err(sol.u, d["u"]) <= 1e-8


def test_legacy_problem_assemble_and_run(jfem, orc):
    d = np.load(GOLDEN / "cube_tet4.npz")
    X, conn, ids = d["X"], d["conn"], d["node_ids"]
    geom = {int(ids[i]): X[i] for i in range(len(ids))}
    body = jfem.Problem(jfem.Elasticity, "body", 3)
    els = [jfem.Element(jfem.Tet4, [int(ids[n]) for n in c]) for c in conn]
    jfem.update_(els, "geometry", geom)
    jfem.update_(els, "youngs modulus", float(d["E"]))
    jfem.update_(els, "poissons ratio", float(d["nu"]))
    surf = [jfem.Element(jfem.Tri3, [int(ids[n]) for n in f]) for f in d["faces"]]
    jfem.update_(surf, "geometry", geom)
    jfem.update_(surf, "surface pressure", 1.0)
    jfem.add_elements_(body, els + surf)
    asm = jfem.assemble_(body, 0.0)
    cp, rv, nz, _ = orc.assemble_coo(4, X, conn, float(d["E"]), float(d["nu"]))
    assert np.array_equal(asm.K.indptr, cp) and rel_err(asm.K.data, nz) <= 1e-12
    assert abs(asm.f.reshape(-1, 3)[:, 2].sum() + 100.0) < 1e-10           # 1.0 × area 100
    # Dirichlet problems: symmetry planes from the fixture's boundary DOFs
    bc = jfem.Problem(jfem.Dirichlet, "symmetry", 3, "displacement")
    for dof in d["dofs"]:
        el = jfem.Element(jfem.Tet4, [int(ids[dof // 3])] * 4)
        jfem.update_(el, f"displacement {dof % 3 + 1}", 0.0)
        bc.elements.append(el)
    an = jfem.Analysis(jfem.Linear)
    jfem.add_problems_(an, [body, bc])
    an.properties["tol"] = 1e-12
    u = jfem.run_(an)
    uu = np.concatenate([u[int(n)] for n in ids])
    assert np.abs(uu - d["u_exact"]).max() <= 1e-10 * np.abs(d["u_exact"]).max()


@pytest.mark.parametrize("method", [0, 1])
def test_time_budget_returns_best_iterate(jfem, gpu_ctx_factory, method):
    """A solve whose time budget (1 µs) runs out after its first chunk of CG
    iterations returns JFEM_ERR_TIMEOUT (a host-side check between graph
    launches; no kernel waits on anything), hands back the better of the
    current and the best FP64 iterate — finite, prescribed DOFs kept, its true
    relative residual in the stats — and the iteration count reached, and the
    context stays usable: the next solve converges."""
    import ctypes as C
    w = jfem.workloads.cantilever(10, 20, 2, 2, 10.0, 1.0, 1.0)
    abi = jfem._abi
    with gpu_ctx_factory(w) as ctx:
        if method == 1:
            ctx.mpnn_init(3)
        o = jfem.default_opts(method=abi.FCG_LEARNED if method else abi.PCG_JACOBI, precision=abi.MIXED,
                              tol=1e-10, max_iter=100000)
        o.time_budget_s = 1e-6
        u = np.full(w.mesh.n_dofs, np.nan)
        st = abi.Stats()
        rc = ctx._lib.jfem_solve(ctx._h, C.byref(o), u.ctypes.data_as(C.POINTER(C.c_double)), C.byref(st))
        assert rc == abi.ERR_TIMEOUT and st.status == abi.ERR_TIMEOUT
        assert "time budget" in ctx._lib.jfem_last_error(ctx._h).decode()
        assert np.all(np.isfinite(u)) and np.all(u[w.fixed_dofs] == 0.0)
        assert 0 < st.cg_iterations < 1000 and 0.0 < st.residual <= 1.0 + 1e-12   # never worse than x0
        o.time_budget_s = 0.0
        u2, st2, rc2 = ctx.solve(o)
        assert rc2 in (0, abi.STALL) and st2.residual <= 1e-10


def test_absolute_tolerance_mode(jfem, gpu_ctx_factory):
    """tol_absolute = 1 stops CG on ‖f − K u‖ ≤ tol, the reference's absolute
    test (src/backend/cpu.jl:230,244): with tol = 1e-9·‖f‖ it converges to the
    same relative level as the default mode with tol = 1e-9, and a tighter
    absolute tol reaches a smaller relative residual."""
    w = jfem.workloads.cantilever(4, 20, 4, 4, 10.0, 1.0, 1.0)
    abi = jfem._abi
    with gpu_ctx_factory(w) as ctx:
        _, _, _, f = ctx.assemble_csc(0)
        fn = float(np.linalg.norm(f[~w.fixed_mask().astype(bool)]))
        _, st_rel, rc1 = ctx.solve(method=abi.PCG_JACOBI, precision=abi.MIXED, tol=1e-9, max_iter=100000)
        _, st_abs, rc2 = ctx.solve(method=abi.PCG_JACOBI, precision=abi.MIXED, tol=1e-9 * fn, max_iter=100000,
                                   tol_absolute=1)
        _, st_abs2, rc3 = ctx.solve(method=abi.PCG_JACOBI, precision=abi.MIXED, tol=1e-10 * fn,
                                    max_iter=100000, tol_absolute=1)
    assert rc1 == rc2 == rc3 == 0
    assert st_rel.residual <= 1e-9 and st_abs.residual * fn <= 1e-9 * fn
    assert st_abs2.residual <= 1e-10 and st_abs2.cg_iterations >= st_abs.cg_iterations


def test_newton_neo_hookean_cube_16_against_oracle(jfem, orc, gpu_ctx_factory):
    """The Newton–Krylov configuration at a representative size: Hex8
    Neo-Hookean unit cube of 16³ cells (14,739 DOFs), per-element lognormal E
    (σ_log 0.2, seeded), ν = 0.3, bottom clamped, top u_z ramped to −0.1 over
    10 load steps.  The GPU's mixed-precision Newton–Krylov (FP32 tangent
    apply, FP64 residuals) against the oracle's FP64 Newton with consistent
    tangents and direct solves (src/solvers.jl:575-620), stored in
    tests/golden/hex8_neohookean_16.npz by tests/golden/make_golden.py:
    u within 1e-8."""
    w = jfem.workloads.cube_compression(n=16, steps=10, top_uz=-0.1)
    d = np.load(GOLDEN / "hex8_neohookean_16.npz")
    # the fixture's E (np.exp may differ in the last bit between host architectures)
    assert np.abs(d["E"] - w.E).max() <= 1e-14 * np.abs(w.E).max()
    w.E = d["E"]
    with gpu_ctx_factory(w) as ctx:
        u, st, rc = ctx.solve(method=2, precision=1, tol=1e-10, newton_tol=1e-10, max_newton=30,
                              max_cg_per_newton=20000, n_load_steps=10, max_iter=200000)
    assert rc == 0 and st.newton_iterations >= 10
    assert rel_err(u, d["u"]) <= 1e-8
