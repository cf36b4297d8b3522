"""Checkpoint files with the GPU: a network written to a weight file and read
into a fresh context preconditions bit-identically, and a load-stepped Newton
solve stopped after two of four steps and resumed from its load-step file in a
fresh context ends where one jfem_solve call over the four steps ends."""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def test_network_file_preconditions_identically(jfem, tmp_path):
    w = jfem.workloads.learned_family(1, seed_item=900, nx=6, ny=2, nz=2, L=3.0)[0]
    m = w.mesh
    weights = np.random.default_rng(8).standard_normal(jfem._abi.MPNN_PARAMS).astype(np.float32) * 0.05
    r = np.random.default_rng(9).standard_normal(m.n_dofs)
    path = tmp_path / "net.jfemnet"

    def setup(ctx):
        ctx.set_mesh(m.elem_type, m.X, m.conn)
        ctx.set_material(w.E, w.nu)
        ctx.set_dirichlet(w.fixed_dofs, w.fixed_values)
        ctx.set_traction(w.face_type, w.faces, w.traction)

    with jfem.Context(0) as ctx:
        setup(ctx)
        ctx.mpnn_set_weights(weights)                 # rounded to BF16 on the way in
        z1 = ctx.mpnn_precondition(r)
        jfem.checkpoint.save_network(path, ctx, meta={"note": "test"})
        w1 = ctx.mpnn_get_weights()
    with jfem.Context(0) as ctx:
        setup(ctx)
        wl, header = jfem.checkpoint.load_network(path, ctx)
        z2 = ctx.mpnn_precondition(r)
        w2 = ctx.mpnn_get_weights()
    assert header["meta"] == {"note": "test"}
    assert np.array_equal(w2, w1) and np.array_equal(wl, w1)
    assert np.array_equal(z2, z1)


def test_newton_resumed_from_load_step_file_matches_one_call(jfem, gpu_ctx_factory, tmp_path):
    w = jfem.workloads.cube_compression(n=4, steps=4, top_uz=-0.1)
    kw = dict(precision=0, tol=1e-10, newton_tol=1e-11, max_newton=30, max_cg_per_newton=2000)
    with gpu_ctx_factory(w) as ctx:
        u_ref, st, rc = ctx.solve(method=2, n_load_steps=4, **kw)
    assert rc == 0
    ck = tmp_path / "steps.bin"
    with gpu_ctx_factory(w) as ctx:                   # stopped after two of the four steps
        u2, info2 = jfem.checkpoint.newton_load_steps(ctx, 4, w.fixed_dofs, w.fixed_values, checkpoint=ck,
                                                      stop_after=2, **kw)
    u_file, step, steps = jfem.checkpoint.load_load_step(ck)
    assert (step, steps) == (2, 4) and info2["steps_done"] == 2 and np.array_equal(u_file, u2)
    with gpu_ctx_factory(w) as ctx:                   # a fresh context resumes from the file
        u4, info4 = jfem.checkpoint.newton_load_steps(ctx, 4, w.fixed_dofs, w.fixed_values, checkpoint=ck,
                                                      resume=True, **kw)
    assert info4["status"] == 0 and info4["steps_done"] == 4
    assert jfem.checkpoint.load_load_step(ck)[1] == 4
    assert all(k >= 1 for k, _, _ in info2["per_step"] + info4["per_step"])
    assert rel_err(u4, u_ref) <= 1e-7
