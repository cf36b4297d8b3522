"""Checkpoint files on the CPU: BF16 rounding (against torch's bfloat16 and the
oracle's), the network weight file and the Newton load-step file round trips
and their rejections, and the per-step Newton driver's bookkeeping (staged
run, resume) against a stand-in context.  The GPU side (a loaded network
preconditions bit-identically; a resumed Newton run equals one call) is in
tests/test_zzz_checkpoint_gpu.py."""
import struct
from types import SimpleNamespace

import numpy as np
import pytest

import mpnn_oracle as mo


@pytest.fixture(scope="module")
def ck(jfem):
    return jfem.checkpoint


def _edge_floats():
    bits = np.array([0x00000000, 0x80000000, 0x3F800000, 0x3F808000, 0x3F818000, 0x3F807FFF, 0x3F808001,
                     0x7F7FFFFF, 0xFF7FFFFF, 0x7F800000, 0xFF800000, 0x00000001, 0x807FFFFF, 0x00400000,
                     0x7F7F8000, 0x7F7F7FFF], dtype=np.uint32)
    return bits.view(np.float32)


def test_bf16_rounding_is_nearest_even(ck):
    torch = pytest.importorskip("torch")
    g = np.random.default_rng(3)
    w = np.concatenate([g.standard_normal(20000).astype(np.float32) * np.float32(10.0) ** g.integers(-30, 30, 20000),
                        _edge_floats()]).astype(np.float32)
    want = torch.from_numpy(w).to(torch.bfloat16).view(torch.int16).numpy().view(np.uint16)
    got = ck.to_bf16(w)
    assert np.array_equal(got, want)
    assert np.array_equal(ck.from_bf16(got), mo.bf16_round(w))
    nan = ck.to_bf16(np.array([np.nan], np.float32))
    assert np.isnan(ck.from_bf16(nan)[0])


def test_network_file_round_trip(ck, tmp_path, jfem):
    w = np.random.default_rng(1).standard_normal(jfem._abi.MPNN_PARAMS).astype(np.float32) * 0.1
    p = tmp_path / "net.jfemnet"
    ck.save_network(p, w, meta={"train_systems": 512, "loss_last": 0.87})
    data = p.read_bytes()
    assert data[:8] == b"JFEMNET\x01"
    (hl,) = struct.unpack_from("<I", data, 8)
    assert len(data) == 12 + hl + 2 * jfem._abi.MPNN_PARAMS
    w2, header = ck.load_network(p)
    assert w2.dtype == np.float32 and np.array_equal(w2, mo.bf16_round(w))
    assert header["meta"] == {"train_systems": 512, "loss_last": 0.87}
    assert header["params"] == jfem._abi.MPNN_PARAMS and header["dtype"] == "bfloat16"
    assert [s["name"] for s in header["segments"]] == ["Ws1", "Wn1", "Ws2", "Wn2", "Ws3", "Wn3", "Wo"]
    # saving what was loaded changes nothing (BF16 values are fixed points)
    ck.save_network(tmp_path / "again", w2, meta=header["meta"])
    assert (tmp_path / "again").read_bytes() == data


def test_network_file_rejects(ck, tmp_path, jfem):
    with pytest.raises(ValueError):
        ck.save_network(tmp_path / "short", np.zeros(10, np.float32))
    p = tmp_path / "net"
    ck.save_network(p, np.zeros(jfem._abi.MPNN_PARAMS, np.float32))
    data = p.read_bytes()
    for bad in (b"XXXXXXXX" + data[8:], data[:-2], data[:20]):
        q = tmp_path / "bad"
        q.write_bytes(bad)
        with pytest.raises(ValueError):
            ck.load_network(q)


def test_load_step_file_round_trip(ck, tmp_path):
    u = np.random.default_rng(2).standard_normal(3 * 125)
    p = tmp_path / "steps.bin"
    ck.save_load_step(p, u, 3, 10)
    u2, s, n = ck.load_load_step(p)
    assert (s, n) == (3, 10) and np.array_equal(u2, u)
    data = p.read_bytes()
    for bad in (data[:-8], b"JFEMSTEQ" + data[8:], data[:8] + struct.pack("<I", 2) + data[12:]):
        (tmp_path / "bad").write_bytes(bad)
        with pytest.raises(ValueError):
            ck.load_load_step(tmp_path / "bad")
    with pytest.raises(ValueError):
        ck.save_load_step(p, u, 11, 10)


class _FakeContext:
    """Stands in for jfem.Context: records the Dirichlet values and states the
    driver sets, and 'solves' a step by moving every DOF to the step's
    fraction (so the state after step s is s/S everywhere)."""

    def __init__(self, n_nodes):
        self.n_nodes = n_nodes
        self.calls = []
        self.state = None
        self.vals = None

    def set_dirichlet(self, dofs, values):
        self.vals = np.array(values)
        self.calls.append(("dirichlet", float(values[0])))

    def set_surface_load(self, ft, faces, t=None, p=None):
        self.calls.append(("surface", float(np.asarray(t).ravel()[0])))

    def set_state(self, u):
        self.state = np.array(u)
        self.calls.append(("state", float(u[0])))

    def solve(self, **kw):
        assert kw["method"] == 2 and kw["n_load_steps"] == 1 and kw["precision"] == 0
        frac = float(self.vals[0])
        self.state = np.full(3 * self.n_nodes, frac)
        self.calls.append(("solve", frac))
        return self.state.copy(), SimpleNamespace(newton_iterations=3, cg_iterations=10, residual=1e-12), 0


def test_newton_driver_stages_and_resumes(ck, tmp_path):
    p = tmp_path / "steps.bin"
    ctx = _FakeContext(5)
    surf = (3, np.zeros((1, 3), np.int64), np.ones((1, 3)), None)
    u, info = ck.newton_load_steps(ctx, 4, [0, 1], [1.0, 1.0], surface=surf, checkpoint=p, stop_after=2,
                                   precision=0)
    assert info["steps_done"] == 2 and info["newton_iterations"] == 6 and np.allclose(u, 0.5)
    assert [c for c in ctx.calls if c[0] == "solve"] == [("solve", 0.25), ("solve", 0.5)]
    assert ("surface", 0.25) in ctx.calls and ("surface", 0.5) in ctx.calls
    us, s, n = ck.load_load_step(p)
    assert (s, n) == (2, 4) and np.allclose(us, 0.5)
    fresh = _FakeContext(5)
    u4, info4 = ck.newton_load_steps(fresh, 4, [0, 1], [1.0, 1.0], surface=surf, checkpoint=p, resume=True,
                                     precision=0)
    assert fresh.calls[0] == ("state", 0.5)             # the resumed run starts from the file's state
    assert [c for c in fresh.calls if c[0] == "solve"] == [("solve", 0.75), ("solve", 1.0)]
    assert info4["steps_done"] == 4 and np.allclose(u4, 1.0) and ck.load_load_step(p)[1] == 4
    done = _FakeContext(5)                               # nothing left: the file's last state comes back
    u5, info5 = ck.newton_load_steps(done, 4, [0, 1], [1.0, 1.0], checkpoint=p, resume=True, precision=0)
    assert info5["steps_done"] == 4 and np.allclose(u5, 1.0)
    assert not [c for c in done.calls if c[0] == "solve"]
    new = _FakeContext(5)                                # resume without a file yet: from step 1
    u6, info6 = ck.newton_load_steps(new, 2, [0], [1.0], checkpoint=tmp_path / "none.bin", resume=True,
                                     precision=0)
    assert [c for c in new.calls if c[0] == "solve"] == [("solve", 0.5), ("solve", 1.0)]
    assert not [c for c in new.calls if c[0] == "state"] and ck.load_load_step(tmp_path / "none.bin")[1] == 2
    with pytest.raises(ValueError):
        ck.newton_load_steps(_FakeContext(5), 5, [0], [1.0], checkpoint=p, resume=True, precision=0)
    with pytest.raises(ValueError):
        ck.newton_load_steps(_FakeContext(5), 4, [0], [1.0], resume=True, precision=0)
    with pytest.raises(ValueError):
        ck.newton_load_steps(_FakeContext(6), 4, [0], [1.0], checkpoint=p, resume=True, precision=0)
