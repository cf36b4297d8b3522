"""Shared test set-up: marker registration, package / oracle loading, builders.

The oracle (oracle/) is test infrastructure: it is the checker the GPU results
are compared with, never the thing under test.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

import jfem_loader  # noqa: E402

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libjfem_cuda.so")


@pytest.fixture(scope="session")
def jfem():
    pkg = jfem_loader.load_package()
    from jfem_gb300 import build as _build
    _build.build()          # incremental: recompiles only stale translation units
    return pkg


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def npo():
    import np_oracle
    return np_oracle


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.abs(b).max()
    return float(np.abs(a - b).max() / (den if den > 0 else 1.0))


@pytest.fixture(scope="session")
def gpu_ctx_factory(jfem):
    """Context factory for GPU tests; fails (does not skip) when the library or
    the device is unusable, so a silent fallback cannot pass."""
    def make(w=None):
        ctx = jfem.Context(0)
        if w is not None:
            ctx.set_mesh(w.mesh.elem_type, w.mesh.X, w.mesh.conn)
            ctx.set_material(w.E, w.nu, w.model)
            ctx.set_formulation(w.finite, w.finite)
            ctx.set_dirichlet(w.fixed_dofs, w.fixed_values)
            if w.faces is not None:
                ctx.set_traction(w.face_type, w.faces, w.traction)
        return ctx
    return make
