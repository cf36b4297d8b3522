"""The Neo-Hookean tangent action the cached-state GPU apply evaluates
(flux_tangent_cached in csrc/jfem_apply_kernels.cuh), restated in numpy and
checked against central finite differences of the first Piola stress
P(F) = F S(FᵀF), S = μ(I − C⁻¹) + λ ln J C⁻¹ (the closed form of
src/materials/neo_hookean.jl:129-143).  The cache holds F, C⁻¹ and
cc = μ − λ ln J per point; then S = μ I − cc C⁻¹ and
δS = λ (C⁻¹:δE) C⁻¹ + 2 cc C⁻¹ δE C⁻¹, δP = F δS + ∇v S."""
import numpy as np


def _pk1(F, lam, mu):
    C = F.T @ F
    Ci = np.linalg.inv(C)
    lnJ = 0.5 * np.log(np.linalg.det(C))
    S = mu * (np.eye(3) - Ci) + lam * lnJ * Ci
    return F @ S


def _cached_state(F, lam, mu):
    C = F.T @ F
    Ci = np.linalg.inv(C)
    cc = mu - lam * 0.5 * np.log(np.linalg.det(C))
    return Ci, cc


def _tangent_action(F, Ci, cc, lam, mu, gv):
    FtG = F.T @ gv
    dE = 0.5 * (FtG + FtG.T)
    CidE = Ci @ dE
    tr = np.trace(CidE)
    S = mu * np.eye(3) - cc * Ci
    dS = lam * tr * Ci + 2.0 * cc * (CidE @ Ci)
    return F @ dS + gv @ S


def test_cached_tangent_matches_finite_differences_of_pk1():
    g = np.random.default_rng(11)
    lam, mu = 121153.8, 80769.2          # E = 210e3, ν = 0.3
    for _ in range(20):
        F = np.eye(3) + 0.15 * g.standard_normal((3, 3))
        if np.linalg.det(F) <= 0.2:
            continue
        gv = g.standard_normal((3, 3))
        Ci, cc = _cached_state(F, lam, mu)
        dP = _tangent_action(F, Ci, cc, lam, mu, gv)
        h = 1e-6
        fd = (_pk1(F + h * gv, lam, mu) - _pk1(F - h * gv, lam, mu)) / (2 * h)
        assert np.abs(dP - fd).max() <= 1e-6 * np.abs(fd).max()


def test_cached_stress_equals_closed_form():
    g = np.random.default_rng(12)
    lam, mu = 5.0, 2.0
    F = np.eye(3) + 0.1 * g.standard_normal((3, 3))
    Ci, cc = _cached_state(F, lam, mu)
    C = F.T @ F
    S_closed = mu * (np.eye(3) - np.linalg.inv(C)) + lam * 0.5 * np.log(np.linalg.det(C)) * np.linalg.inv(C)
    assert np.allclose(mu * np.eye(3) - cc * Ci, S_closed, rtol=1e-13, atol=1e-13)
