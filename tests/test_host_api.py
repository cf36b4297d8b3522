"""Host-side logic of the reference-shaped API (no GPU needed)."""
import numpy as np
import pytest


def test_cpu_backend_request_raises(jfem):
    with pytest.raises(RuntimeError, match="CPU backend"):
        jfem.select_backend(jfem.CPU(4))


def test_element_validation(jfem):
    with pytest.raises(ValueError):
        jfem.Element(jfem.Tet10, [1, 2, 3, 4])
    el = jfem.Element(jfem.Tet4, [1, 2, 3, 4])
    jfem.update_(el, "youngs modulus", 210e3)
    assert el.haskey("youngs modulus") and el("youngs modulus") == 210e3


def test_get_gdofs_interleaved(jfem):
    assert list(jfem.get_gdofs([1, 3])) == [0, 1, 2, 6, 7, 8]


def test_overconstrained_dirichlet_raises(jfem):
    from jfem_gb300.problem import _dirichlet_arrays
    ph = jfem.Physics(jfem.Tet4, np.zeros((4, 3)), np.array([[0, 1, 2, 3]]))
    jfem.add_dirichlet_(ph, [0, 1], (1, 2))
    jfem.add_dirichlet_(ph, [1], (2,))
    with pytest.raises(RuntimeError, match="overconstrained"):
        _dirichlet_arrays(ph)


def test_unsupported_element_in_problem(jfem):
    from jfem_gb300.problem import _pack_volume
    p = jfem.Problem(jfem.Elasticity, "body", 3)
    el = jfem.Element(jfem.Tet4, [1, 2, 3, 4])
    el.etype = "Seg3"
    jfem.add_elements_(p, [el])
    with pytest.raises(RuntimeError, match="unsupported elements"):
        _pack_volume(p)


def test_batch_instances_are_seeded(jfem):
    a = jfem.workloads.batch_instances(count=5)
    b = jfem.workloads.batch_instances(count=5)
    for x, y in zip(a, b):
        assert x.mesh.n_elem == y.mesh.n_elem and x.E == y.E and np.array_equal(x.traction, y.traction)
    sizes = [w.mesh.shape[0] for w in jfem.workloads.batch_instances(count=64)]
    assert min(sizes) >= 8 and max(sizes) <= 32
