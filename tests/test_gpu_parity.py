"""GPU parity through the C ABI: assembly, apply, internal force against the oracle."""
import hashlib

import numpy as np
import pytest

from conftest import GOLDEN, rel_err

pytestmark = pytest.mark.gpu


def _hash(cp, rv):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(cp, dtype=np.int64).tobytes())
    h.update(np.ascontiguousarray(rv, dtype=np.int64).tobytes())
    return h.hexdigest()


def test_csc_tet4_cantilever_matches_oracle_and_golden(jfem, orc, gpu_ctx_factory):
    w = jfem.workloads.cfg_tet4_cantilever()
    m = w.mesh
    with gpu_ctx_factory(w) as ctx:
        cp, rv, nz, f = ctx.assemble_csc(0)
    ocp, orv, onz, _ = orc.assemble_coo(4, m.X, m.conn, w.E, w.nu)
    assert np.array_equal(cp, ocp) and np.array_equal(rv, orv)          # pattern bit-exact
    assert rel_err(nz, onz) <= 1e-12                                      # K entries
    fo = orc.traction(w.face_type, w.faces, m.X, w.traction)
    assert rel_err(f, fo) <= 1e-12                                        # f = f_ext − f_int(0)
    d = np.load(GOLDEN / "tet4_cantilever.npz")
    assert _hash(cp, rv) == str(d["pattern_sha256"])
    assert rel_err(nz[d["sample_idx"]], d["sample_val"]) <= 1e-12


@pytest.mark.parametrize("et,dims", [(10, (4, 2, 3)), (8, (3, 4, 2)), (4, (5, 3, 2))])
def test_csc_small_meshes_per_element_material(jfem, orc, gpu_ctx_factory, et, dims):
    m = jfem.mesh.box_mesh(et, *dims, 2.0, 1.3, 0.9)
    g = np.random.default_rng(et)
    # mildly distorted nodes: non-affine Hex8/Tet10 exercise the per-point geometry path
    X = m.X + 0.02 * g.standard_normal(m.X.shape)
    E = g.uniform(50e3, 300e3, m.n_elem)
    nu = g.uniform(0.2, 0.45, m.n_elem)
    with gpu_ctx_factory() as ctx:
        ctx.set_mesh(et, X, m.conn + 1, index_base=1)
        ctx.set_material(E, nu)
        cp, rv, nz, f = ctx.assemble_csc(1)
    ocp, orv, onz, _ = orc.assemble_coo(et, X, m.conn, E, nu)
    assert np.array_equal(cp - 1, ocp) and np.array_equal(rv - 1, orv)
    assert rel_err(nz, onz) <= 1e-12


@pytest.mark.parametrize("model", [0, 1])
@pytest.mark.parametrize("et", [8, 10, 4])
def test_csc_finite_strain_tangent(jfem, orc, gpu_ctx_factory, et, model):
    m = jfem.mesh.box_mesh(et, 3, 2, 2, 1.0, 0.8, 0.6)
    g = np.random.default_rng(11)
    u = 0.01 * g.standard_normal(m.n_dofs)
    with gpu_ctx_factory() as ctx:
        ctx.set_mesh(et, m.X, m.conn)
        ctx.set_material(200e3, 0.3, model)
        ctx.set_formulation(True, True)
        ctx.set_state(u)
        cp, rv, nz, f = ctx.assemble_csc(0)
        fi = ctx.internal_force()
    ocp, orv, onz, ofi = orc.assemble_coo(et, m.X, m.conn, 200e3, 0.3, u=u, model=model, finite=True, geom=True)
    assert np.array_equal(cp, ocp) and np.array_equal(rv, orv)
    assert rel_err(nz, onz) <= 1e-12
    assert rel_err(-f, ofi) <= 1e-12            # f = f_ext − f_int with no surface load
    assert rel_err(fi, ofi) <= 1e-12            # matrix-free FP64 internal force


def test_assembly_is_deterministic(jfem, gpu_ctx_factory):
    w = jfem.workloads.cantilever(10, 6, 3, 3, 3.0, 1.0, 1.0)
    with gpu_ctx_factory(w) as ctx:
        a = ctx.assemble_csc(0)
        b = ctx.assemble_csc(0)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_assembly_timing_hook_runs_the_same_assembly(jfem, gpu_ctx_factory):
    """jfem_time_assembly times the two assembly launches into scratch and
    leaves the assembled K unchanged; its entry count is K's."""
    w = jfem.workloads.cantilever(10, 6, 3, 3, 3.0, 1.0, 1.0)
    with gpu_ctx_factory(w) as ctx:
        a = ctx.assemble_csc(0)
        ms_q, ms_s, nnz = ctx.time_assembly(reps=2)
        b = ctx.assemble_csc(0)
        with pytest.raises(jfem.JFEMError):
            ctx.time_assembly(reps=0)
    assert ms_q > 0.0 and ms_s > 0.0 and nnz == a[2].size
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("et", [4, 10, 8])
def test_apply_fp64_and_fp32(jfem, orc, gpu_ctx_factory, et):
    m = jfem.mesh.box_mesh(et, 5, 3, 3, 5.0, 1.0, 1.0)
    g = np.random.default_rng(3)
    v = g.standard_normal(m.n_dofs)
    E = g.uniform(100e3, 300e3, m.n_elem)
    with gpu_ctx_factory() as ctx:
        ctx.set_mesh(et, m.X, m.conn)
        ctx.set_material(E, 0.3)
        y64 = ctx.apply(v)
        y32 = ctx.apply(v, fp32=True)
        y64b = ctx.apply(v)
    yo = orc.apply(et, m.X, m.conn, E, 0.3, v)
    assert rel_err(y64, yo) <= 1e-12
    assert rel_err(y32, yo) <= 2e-5          # FP32 element arithmetic
    assert np.array_equal(y64, y64b)        # deterministic gather


@pytest.mark.parametrize("et,dims", [(10, (8, 4, 4)), (8, (8, 6, 6)), (4, (10, 5, 5))])
def test_apply_fp32_distorted_multi_tile(jfem, orc, gpu_ctx_factory, et, dims):
    """Tiled FP32 apply on distorted (non-affine for Tet10/Hex8) meshes of
    several tiles: per-point geometry records read from HBM, tile-shared nodes
    through the boundary pass; small strain and the Neo-Hookean tangent."""
    m = jfem.mesh.box_mesh(et, *dims, 2.0, 1.0, 1.0)
    g = np.random.default_rng(20 + et)
    X = m.X + 0.01 * g.standard_normal(m.X.shape)
    E = g.uniform(100e3, 300e3, m.n_elem)
    v = g.standard_normal(m.n_dofs)
    u = 0.01 * g.standard_normal(m.n_dofs)
    with gpu_ctx_factory() as ctx:
        ctx.set_mesh(et, X, m.conn)
        ctx.set_material(E, 0.3)
        y32 = ctx.apply(v, fp32=True)
        ctx.set_material(E, 0.3, 1)
        ctx.set_formulation(True, True)
        ctx.set_state(u)
        t32 = ctx.apply(v, fp32=True)
    assert m.n_elem > 256                     # several tiles, so shared nodes exist
    assert rel_err(y32, orc.apply(et, X, m.conn, E, 0.3, v)) <= 2e-5
    to = orc.apply(et, X, m.conn, E, 0.3, v, u=u, model=1, finite=True, geom=True)
    assert rel_err(t32, to) <= 1e-4


def test_apply_masked(jfem, gpu_ctx_factory, orc):
    w = jfem.workloads.cantilever(4, 6, 2, 2, 3.0, 1.0, 1.0)
    m = w.mesh
    v = np.random.default_rng(5).standard_normal(m.n_dofs)
    with gpu_ctx_factory(w) as ctx:
        y = ctx.apply(v, masked=True)
    vm = v.copy()
    vm[w.fixed_dofs] = 0
    yo = orc.apply(4, m.X, m.conn, w.E, w.nu, vm)
    yo[w.fixed_dofs] = 0
    assert rel_err(y, yo) <= 1e-12


@pytest.mark.parametrize("model", [0, 1])
def test_tangent_apply_matches_assembled_tangent(jfem, orc, gpu_ctx_factory, model):
    m = jfem.mesh.box_mesh(8, 4, 3, 3, 1.0, 0.7, 0.7)
    g = np.random.default_rng(8)
    u = 0.02 * g.standard_normal(m.n_dofs)
    v = g.standard_normal(m.n_dofs)
    with gpu_ctx_factory() as ctx:
        ctx.set_mesh(8, m.X, m.conn)
        ctx.set_material(210e3, 0.3, model)
        ctx.set_formulation(True, True)
        ctx.set_state(u)
        y64 = ctx.apply(v)
        y32 = ctx.apply(v, fp32=True)
    yo = orc.apply(8, m.X, m.conn, 210e3, 0.3, v, u=u, model=model, finite=True, geom=True)
    assert rel_err(y64, yo) <= 1e-12
    assert rel_err(y32, yo) <= 1e-4


def test_error_paths(jfem, gpu_ctx_factory):
    m = jfem.mesh.box_mesh(4, 2, 1, 1)
    with gpu_ctx_factory() as ctx:
        ctx.set_mesh(4, m.X, m.conn)
        with pytest.raises(jfem.JFEMError) as e:
            ctx.set_mesh(4, m.X, m.conn + 100)
        assert e.value.code == jfem._abi.ERR_INVALID
        with pytest.raises(jfem.JFEMError) as e:           # the failed call left no (partial) mesh
            ctx.set_material(210e3, 0.3)
        assert e.value.code == jfem._abi.ERR_INVALID and "set_mesh" in str(e.value)
        ctx.set_mesh(4, m.X, m.conn)
        ctx.set_material(210e3, 0.3)
        ft, fc = m.face(0, 1)
        ctx.set_traction(ft, fc, np.ones((fc.shape[0], 3)))
        with pytest.raises(jfem.JFEMError) as e:           # a face node outside the mesh
            ctx.set_traction(ft, fc + m.n_nodes, np.ones((fc.shape[0], 3)))
        assert e.value.code == jfem._abi.ERR_INVALID
        _, _, _, f = ctx.assemble_csc(0)                   # ...left no surface load: f = −f_int(0) = 0
        assert not np.any(f)
        ctx.set_mesh(4, m.X, m.conn)
        with pytest.raises(jfem.JFEMError):
            ctx.apply(np.zeros(m.n_dofs))                  # material not set
        with pytest.raises(jfem.JFEMError):
            ctx.set_material(210e3, 0.5)                   # incompressible ν rejected
        bad = m.conn.copy()
        bad[0, [1, 2]] = bad[0, [2, 1]]                    # inverted element
        ctx.set_mesh(4, m.X, bad)
        ctx.set_material(210e3, 0.3)
        with pytest.raises(jfem.JFEMError) as e:
            ctx.assemble_csc(0)
        assert e.value.code == jfem._abi.ERR_NEG_JACOBIAN
        with pytest.raises(jfem.JFEMError) as e:
            ctx.apply(np.zeros(m.n_dofs))
        assert e.value.code == jfem._abi.ERR_NEG_JACOBIAN


@pytest.mark.parametrize("et", [4, 10, 8])
@pytest.mark.parametrize("kind", ["traction", "pressure", "both"])
def test_surface_loads_match_oracle(jfem, orc, gpu_ctx_factory, et, kind):
    """k_face_load against the oracle's consistent integration
    (problems_elasticity.jl:454-502): per-face traction and pressure on all six
    faces of a distorted box — Tri3 (Tet4), curved Tri6 (Tet10), warped Quad4
    (Hex8) — read back as f = f_ext − f_int(0) from jfem_assemble_csc; ≤ 1e-12."""
    m = jfem.mesh.box_mesh(et, 3, 2, 2, 1.4, 1.0, 0.8)
    X = m.X + 0.03 * np.random.default_rng(et).standard_normal(m.X.shape)
    faces = []
    for axis in range(3):
        for side in range(2):
            ft, fc = m.face(axis, side)
            faces.append(fc)
    faces = np.concatenate(faces)
    g = np.random.default_rng(20 + et)
    t = g.standard_normal((faces.shape[0], 3)) if kind != "pressure" else None
    p = g.uniform(0.5, 2.0, faces.shape[0]) if kind != "traction" else None
    with gpu_ctx_factory() as ctx:
        ctx.set_mesh(et, X, m.conn)
        ctx.set_material(210e3, 0.3)
        ctx.set_surface_load(ft, faces, t=t, p=p)
        _, _, _, f = ctx.assemble_csc(0)
    fo = np.zeros(m.n_dofs)
    if t is not None:
        fo += orc.traction(ft, faces, X, t)
    if p is not None:
        fo += orc.pressure(ft, faces, X, p)
    assert rel_err(f, fo) <= 1e-12
