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
