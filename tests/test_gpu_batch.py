"""Batched persistent solves (jfem_batch_*) against the oracle's direct solves."""
import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


def _oracle_u(orc, w):
    m = w.mesh
    cp, rv, nz, _ = orc.assemble_coo(4, m.X, m.conn, w.E, w.nu)
    f = orc.traction(w.face_type, w.faces, m.X, w.traction)
    return orc.direct_solve(cp, rv, nz, f, w.fixed_mask().astype(bool))


def test_batch_matches_oracle_and_is_deterministic(jfem, orc):
    """Uneven Tet4 cantilevers (8..14 cubes along x, random E, ν, end traction)
    solved together to 1e-10: each displacement within 1e-8 of the oracle's
    direct solve; a second launch gives identical bits."""
    ws = jfem.workloads.batch_instances(count=12, nmin=8, nmax=14, seed_item=77)
    with jfem.Batch(0) as b:
        for k, w in enumerate(ws):
            assert b.add_workload(w) == k
        us, it, st, res, lat, t = b.solve(tol=1e-10, max_iter=50000, block_size=256)
        us2, it2, *_ = b.solve(tol=1e-10, max_iter=50000, block_size=256)
    assert np.all(st == 0) and np.all(res <= 1e-10) and np.all(it > 0)
    assert np.all(lat > 0) and t > 0 and lat.max() <= t * 1.01
    for w, u in zip(ws, us):
        assert rel_err(u, _oracle_u(orc, w)) <= 1e-8
        assert np.all(u[w.fixed_dofs] == 0.0)
    assert all(np.array_equal(a, c) for a, c in zip(us, us2)) and np.array_equal(it, it2)


def test_batch_autotune_and_block_sizes_agree(jfem):
    ws = jfem.workloads.batch_instances(count=6, nmin=8, nmax=10, seed_item=78)
    with jfem.Batch(0) as b:
        for w in ws:
            b.add_workload(w)
        ref, *_ = b.solve(tol=1e-9, block_size=128)
        for bs in (512, 1024):
            us, _, st, *_ = b.solve(tol=1e-9, block_size=bs)
            assert np.all(st == 0)
            for a, c in zip(us, ref):
                assert rel_err(a, c) <= 1e-7
        us, _, st, *_ = b.solve(tol=1e-9, block_size=0)
        bs, grid = b.config()
        assert bs in (128, 256, 512, 1024) and 1 <= grid <= len(ws)
        assert np.all(st == 0)


@pytest.mark.parametrize("cluster,block", [(2, 512), (4, 256), (8, 256)])
def test_cluster_teams_match_single_cta_teams(jfem, cluster, block):
    """The largest half of the instances solved by thread-block clusters (one
    instance per cluster, cluster-barrier synchronised, sums exchanged through
    distributed shared memory in rank order) gives the single-CTA solutions to
    the solver tolerance, every instance converged, and repeats bit for bit."""
    ws = jfem.workloads.batch_instances(count=10, nmin=8, nmax=16, seed_item=80)
    with jfem.Batch(0) as b:
        for w in ws:
            b.add_workload(w)
        b.set_config(256)
        ref, it0, st0, *_ = b.solve(tol=1e-9, max_iter=50000)
        assert b.cluster_config() == (1, 0, 0)
        b.set_config(256, cluster, 5, block)
        us, it, st, res, lat, t = b.solve(tol=1e-9, max_iter=50000)
        us2, it2, *_ = b.solve(tol=1e-9, max_iter=50000)
        assert b.cluster_config() == (cluster, 5, block)
        with pytest.raises(jfem.JFEMError):
            b.set_config(256, 3, 5, block)
    assert np.all(st0 == 0) and np.all(st == 0) and np.all(res <= 1e-9) and np.all(lat > 0)
    for a, c in zip(us, ref):
        assert rel_err(a, c) <= 1e-6
    assert all(np.array_equal(a, c) for a, c in zip(us, us2)) and np.array_equal(it, it2)


def test_batch_rejects_invalid_instances(jfem):
    w = jfem.workloads.batch_instances(count=1, nmin=8, nmax=8, seed_item=79)[0]
    m = w.mesh
    with jfem.Batch(0) as b:
        bad = m.conn.copy()
        bad[0, 0] = m.n_nodes + 5
        with pytest.raises(jfem.JFEMError):
            b.add(m.X, bad, w.E, w.nu, w.fixed_dofs, w.faces, w.traction)
        flipped = m.conn.copy()
        flipped[:, [1, 2]] = flipped[:, [2, 1]]
        with pytest.raises(jfem.JFEMError):
            b.add(m.X, flipped, w.E, w.nu, w.fixed_dofs, w.faces, w.traction)
        with pytest.raises(jfem.JFEMError):
            b.add(m.X, m.conn, -1.0, w.nu, w.fixed_dofs, w.faces, w.traction)
        with pytest.raises(jfem.JFEMError):
            b.solve()                    # nothing added


def test_cluster_teams_large_instances_against_oracle(jfem, orc):
    """The largest instances of the batched configuration (28..32 cubes along
    x, up to 8,019 DOFs), the half that the autotuner puts on thread-block
    clusters, solved on 4-CTA clusters to 1e-10: every displacement within 1e-8
    of the oracle's direct solve (not only of the single-CTA teams)."""
    ws = jfem.workloads.batch_instances(count=6, nmin=28, nmax=32, seed_item=81)
    with jfem.Batch(0) as b:
        for w in ws:
            b.add_workload(w)
        b.set_config(256, 4, 3, 256)
        us, it, st, res, lat, t = b.solve(tol=1e-10, max_iter=100000)
        assert b.cluster_config() == (4, 3, 256)
    assert np.all(st == 0) and np.all(res <= 1e-10)
    for w, u in zip(ws, us):
        assert rel_err(u, _oracle_u(orc, w)) <= 1e-8


def test_autotuner_cache_reused_by_a_new_batch(jfem, tmp_path, monkeypatch):
    """The autotuned configuration is cached by (GPU, element type, batch
    shape): a second batch object of the same shape takes it without timing
    candidates (tune source 2, same configuration, same bits), and the cache
    file named by JFEM_AUTOTUNE_CACHE holds the entry as JSON."""
    import json
    cache = tmp_path / "autotune.json"
    monkeypatch.setenv("JFEM_AUTOTUNE_CACHE", str(cache))
    ws = jfem.workloads.batch_instances(count=9, nmin=8, nmax=11, seed_item=82)
    runs = []
    for _ in range(2):
        with jfem.Batch(0) as b:
            for w in ws:
                b.add_workload(w)
            us, it, st, *_ = b.solve(tol=1e-9, max_iter=50000, block_size=0)
            runs.append((b.tune_source, b.config(), b.cluster_config(), us, it))
    assert runs[0][0] in (1, 2) and runs[1][0] == 2
    assert runs[0][1:3] == runs[1][1:3]
    assert all(np.array_equal(a, c) for a, c in zip(runs[0][3], runs[1][3]))
    if runs[0][0] == 1:
        entries = json.loads(cache.read_text())
        assert len(entries) >= 1 and all("bs" in e and "ms" in e for e in entries.values())
