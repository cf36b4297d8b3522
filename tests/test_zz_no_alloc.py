"""jfem_apply_noalloc: the matrix-free apply for callers that cannot allocate.

Some callers of this library may not call cudaMalloc: a host application that
owns all device memory through its own arena or pool (an embedding simulation,
a Julia CUDA memory pool), or a latency-critical loop in which an allocation
could stall the device.  jfem_apply_noalloc takes their device buffers for the
mesh, material, v and y and does its work in one fixed device array.  These
tests call it through the C ABI and compare it with the context-based FP64
apply (jfem_apply_device) and with the oracle's FP64 element-by-element apply
on two calls in a row, at the tolerance of the other FP64 apply tests (1e-12
relative); they check that a mesh too large for the fixed array is refused, and
that a node number one past the end or an inadmissible material is reported as
JFEM_ERR_INVALID (the element kernel range-checks every node before it reads
X or v, so such input never reads outside the caller's buffers).  The file is
named to be collected last.
"""
import ctypes

import numpy as np
import pytest

from conftest import rel_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("et,dims", [(10, (6, 3, 3)), (4, (8, 3, 2)), (8, (5, 4, 3))])
def test_noalloc_apply_matches_context_apply(jfem, orc, et, dims):
    import torch
    dev = torch.device("cuda", 0)
    m = jfem.mesh.box_mesh(et, *dims, 3.0, 1.0, 0.8)
    g = np.random.default_rng(et)
    E = g.uniform(50e3, 300e3, m.n_elem)
    nu = g.uniform(0.2, 0.45, m.n_elem)
    X_d = torch.tensor(m.X, dtype=torch.float64, device=dev)
    conn_d = torch.tensor(m.conn + 1, dtype=torch.int64, device=dev)      # 1-based, like Julia
    E_d = torch.tensor(E, dtype=torch.float64, device=dev)
    nu_d = torch.tensor(nu, dtype=torch.float64, device=dev)
    lib = jfem.load()
    stream = torch.cuda.current_stream(dev).cuda_stream
    with jfem.Context(0) as ctx:
        ctx.set_mesh(et, m.X, m.conn)
        ctx.set_material(E, nu)
        for call in range(2):
            v_d = torch.tensor(g.standard_normal(m.n_dofs), dtype=torch.float64, device=dev)
            y_ref = torch.empty_like(v_d)
            ctx.apply_device(v_d.data_ptr(), y_ref.data_ptr(), fp32=False, masked=False)
            y_d = torch.full_like(v_d, float("nan"))
            torch.cuda.synchronize()
            rc = lib.jfem_apply_noalloc(et, m.n_nodes, X_d.data_ptr(), m.n_elem, conn_d.data_ptr(), 1,
                                        E_d.data_ptr(), nu_d.data_ptr(), v_d.data_ptr(), y_d.data_ptr(),
                                        ctypes.c_void_p(stream))
            assert rc == 0, f"call {call}: status {rc}"
            y = y_d.cpu().numpy()
            assert rel_err(y, y_ref.cpu().numpy()) <= 1e-12, f"call {call}"
            y_orc = orc.apply(et, m.X, m.conn, E, nu, v_d.cpu().numpy())
            assert rel_err(y, y_orc) <= 1e-12, f"call {call} against the oracle"


def test_noalloc_refuses_oversize_mesh(jfem):
    import torch
    dev = torch.device("cuda", 0)
    dummy = torch.zeros(4, dtype=torch.float64, device=dev)
    lib = jfem.load()
    # 240,000 Tet10 elements need more than the 64 MiB working array
    N, E = 201 * 41 * 41, 240000
    p = dummy.data_ptr()
    rc = lib.jfem_apply_noalloc(10, N, p, E, p, 0, p, p, p, p, None)
    assert rc == jfem._abi.ERR_TOO_LARGE


@pytest.mark.parametrize("bad", ["node_past_end", "node_negative", "nu_half", "E_zero"])
def test_noalloc_rejects_bad_input(jfem, bad):
    """A tiny Tet4 mesh with one node number one past the end (or below the
    base), or one element with ν = 1/2 or E = 0: status JFEM_ERR_INVALID; a
    good call on the same buffers afterwards still succeeds."""
    import torch
    dev = torch.device("cuda", 0)
    m = jfem.mesh.box_mesh(4, 2, 1, 1, 1.0, 1.0, 1.0)
    conn = m.conn.copy()
    E = np.full(m.n_elem, 210e3)
    nu = np.full(m.n_elem, 0.3)
    if bad == "node_past_end":
        conn[3, 2] = m.n_nodes          # 0-based: one past the last node
    elif bad == "node_negative":
        conn[1, 0] = -1
    elif bad == "nu_half":
        nu[2] = 0.5
    else:
        E[4] = 0.0
    lib = jfem.load()
    X_d = torch.tensor(m.X, dtype=torch.float64, device=dev)
    good_d = torch.tensor(m.conn, dtype=torch.int64, device=dev)
    conn_d = torch.tensor(conn, dtype=torch.int64, device=dev)
    E_d = torch.tensor(E, dtype=torch.float64, device=dev)
    nu_d = torch.tensor(nu, dtype=torch.float64, device=dev)
    E_ok = torch.full_like(E_d, 210e3)
    nu_ok = torch.full_like(nu_d, 0.3)
    v_d = torch.ones(m.n_dofs, dtype=torch.float64, device=dev)
    y_d = torch.zeros_like(v_d)
    torch.cuda.synchronize()
    rc = lib.jfem_apply_noalloc(4, m.n_nodes, X_d.data_ptr(), m.n_elem, conn_d.data_ptr(), 0, E_d.data_ptr(),
                                nu_d.data_ptr(), v_d.data_ptr(), y_d.data_ptr(), None)
    assert rc == jfem._abi.ERR_INVALID
    rc = lib.jfem_apply_noalloc(4, m.n_nodes, X_d.data_ptr(), m.n_elem, good_d.data_ptr(), 0, E_ok.data_ptr(),
                                nu_ok.data_ptr(), v_d.data_ptr(), y_d.data_ptr(), None)
    assert rc == 0
    assert np.abs(y_d.cpu().numpy()).max() <= 1e-6 * 210e3      # v = constant translation: K v = 0
