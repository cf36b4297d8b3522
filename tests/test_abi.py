"""The C-ABI library builds, loads and exports every symbol include/jfem.h declares."""
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    text = (ROOT / "include" / "jfem.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(jfem_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_boundary():
    syms = declared_symbols()
    for s in ["jfem_create", "jfem_destroy", "jfem_last_error", "jfem_set_mesh", "jfem_set_material",
              "jfem_set_dirichlet", "jfem_set_traction", "jfem_assemble_csc", "jfem_apply", "jfem_solve"]:
        assert s in syms


def test_library_exports_every_declared_symbol(jfem):
    lib = jfem.load()
    for s in declared_symbols():
        assert hasattr(lib, s), f"{s} missing from libjfem_cuda.so"
    assert set(declared_symbols()) <= set(jfem._abi.SIGNATURES)
    assert lib.jfem_version().startswith(b"jfem-gb300")


def test_library_targets_sm103a():
    import subprocess
    so = ROOT / "juliafem.jl_gb300" / "libjfem_cuda.so"
    out = subprocess.run(["cuobjdump", "--list-elf", str(so)], capture_output=True, text=True)
    if out.returncode != 0:
        import pytest
        pytest.skip("cuobjdump unavailable")
    assert "sm_103a" in out.stdout


def test_default_opts_match_reference_defaults(jfem):
    o = jfem.default_opts()
    assert (o.tol, o.max_iter, o.newton_tol, o.max_newton, o.max_cg_per_newton) == (1e-6, 1000, 1e-6, 20, 50)
    assert (o.forcing_power, o.forcing_max) == (0.5, 0.9)


def test_no_device_fails_loudly(jfem):
    import torch
    if torch.cuda.is_available():
        import pytest
        pytest.skip("a GPU is present")
    import pytest
    with pytest.raises(jfem.JFEMError):
        jfem.Context(0)


def test_host_exception_does_not_cross_the_abi(jfem):
    """A host allocation failure inside the library comes back as
    JFEM_ERR_OOM, not as a C++ exception through the C interface (which would
    end this process).  jfem_rcm runs on the host only: a node count of 10^15
    makes its first per-node array (tens of PB) fail to allocate before
    anything is written to perm."""
    import ctypes as C
    import numpy as np
    conn = np.array([[0, 1, 2, 3]], np.int64)
    perm = np.zeros(4, np.int64)
    b0, b1 = C.c_int64(0), C.c_int64(0)
    lib = jfem.load()
    rc = lib.jfem_rcm(10 ** 15, 1, 4, conn.ctypes.data_as(C.POINTER(C.c_int64)), 0, 0,
                      perm.ctypes.data_as(C.POINTER(C.c_int64)), C.byref(b0), C.byref(b1))
    assert rc == jfem._abi.ERR_OOM
    assert not perm.any()
    # the library still works afterwards
    p, _, _ = jfem._abi.rcm(conn, 4, start=0)
    assert sorted(p.tolist()) == [0, 1, 2, 3]
