"""Independent numpy/scipy restatement of the elasticity hot path (FP64).

TEST INFRASTRUCTURE ONLY (a second oracle used to cross-check the C++ one).

It is written in the reference's *tensor* form rather than the B-matrix form of
oracle/jfem_oracle.cpp, so the two share no arithmetic:

* shape functions from barycentric coordinates (Tet4 N = L, Tet10 N = L(2L−1)
  and 4LᵢLⱼ, Hex8 trilinear) — same functions as
  src/basis/lagrange_generated.jl:229-311, different expressions;
* small strain: Kᵃᵇᵢⱼ = Σ_q w (λ ∂ᵢNₐ ∂ⱼN_b + μ ∂ⱼNₐ ∂ᵢN_b + μ δᵢⱼ ∇Nₐ·∇N_b)
  (src/physics/assembly_helpers.jl:201-226 contraction ∇Nᵢ·𝔻·∇Nⱼ);
* finite strain (total Lagrangian): P = F S, 𝔸ᵢⱼₖₗ = Fᵢₘ 𝔻ₘⱼₙₗ Fₖₙ + δᵢₖ Sⱼₗ,
  Kᵃᵇᵢₖ = Σ_q w ∂ⱼNₐ 𝔸ᵢⱼₖₗ ∂ₗN_b, fᵃᵢ = Σ_q w Pᵢⱼ ∂ⱼNₐ — algebraically the
  BL(F)ᵀ𝔻BL(F) + BNLᵀŜBNL of src/problems_elasticity.jl:269-404;
* Neo-Hookean S, 𝔻 from ψ (src/materials/neo_hookean.jl:129-143,205-231);
* global assembly through scipy COO→CSC (sums duplicates, keeps explicit zeros),
  the same semantics as SparseArrays.sparse used at src/sparse/sparse.jl:53.
"""
from __future__ import annotations

import numpy as np

_SQ3 = 1.0 / np.sqrt(3.0)


def rule(et):
    if et == 4:
        return np.array([[0.25, 0.25, 0.25]]), np.array([1.0 / 6.0])
    if et == 10:
        a = (5.0 + 3.0 * np.sqrt(5.0)) / 20.0
        b = (5.0 - np.sqrt(5.0)) / 20.0
        return np.array([[a, b, b], [b, a, b], [b, b, a], [b, b, b]]), np.full(4, 1.0 / 24.0)
    if et == 8:
        p = np.array([-_SQ3, _SQ3])
        pts = np.array([[p[i], p[j], p[k]] for k in range(2) for j in range(2) for i in range(2)])
        return pts, np.ones(8)
    raise ValueError(et)


def basis(et, xi):
    """(N[n_en], dN[n_en, 3]) at one reference point."""
    xi = np.asarray(xi, dtype=np.float64)
    if et in (4, 10):
        L = np.array([1.0 - xi.sum(), xi[0], xi[1], xi[2]])
        dL = np.array([[-1.0, -1.0, -1.0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=np.float64)
        if et == 4:
            return L.copy(), dL.copy()
        N = np.empty(10)
        dN = np.empty((10, 3))
        for i in range(4):
            N[i] = L[i] * (2 * L[i] - 1)
            dN[i] = (4 * L[i] - 1) * dL[i]
        for m, (i, j) in enumerate(((0, 1), (1, 2), (2, 0), (0, 3), (1, 3), (2, 3))):
            N[4 + m] = 4 * L[i] * L[j]
            dN[4 + m] = 4 * (dL[i] * L[j] + L[i] * dL[j])
        return N, dN
    if et == 8:
        s = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                      [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], dtype=np.float64)
        f = 1 + s * xi  # (8,3)
        N = 0.125 * f.prod(axis=1)
        dN = np.empty((8, 3))
        dN[:, 0] = 0.125 * s[:, 0] * f[:, 1] * f[:, 2]
        dN[:, 1] = 0.125 * f[:, 0] * s[:, 1] * f[:, 2]
        dN[:, 2] = 0.125 * f[:, 0] * f[:, 1] * s[:, 2]
        return N, dN
    raise ValueError(et)


def lame(E, nu):
    E = np.asarray(E, dtype=np.float64)
    nu = np.asarray(nu, dtype=np.float64)
    return E * nu / ((1 + nu) * (1 - 2 * nu)), E / (2 * (1 + nu))


def element_arrays(et, X, conn, E, nu, u=None, model=0, finite=False):
    """Ke (n_elem, 3n, 3n) with DOF order 3a+i, fe (n_elem, 3n)."""
    X = np.asarray(X, dtype=np.float64)
    conn = np.asarray(conn, dtype=np.int64)
    ne, nn = conn.shape
    la, mu = lame(np.broadcast_to(E, (ne,)), np.broadcast_to(nu, (ne,)))
    Xe = X[conn]                                           # (ne, nn, 3)
    ue = np.zeros_like(Xe) if u is None else np.asarray(u).reshape(-1, 3)[conn]
    pts, wts = rule(et)
    K = np.zeros((ne, nn, 3, nn, 3))
    f = np.zeros((ne, nn, 3))
    I3 = np.eye(3)
    for xi, wq in zip(pts, wts):
        _, dN = basis(et, xi)
        J = np.einsum("ak,eab->ekb", dN, Xe)              # J[k,b] = Σ_a dN_a[k] X_a[b]
        detJ = np.linalg.det(J)
        if np.any(detJ <= 0):
            raise ValueError("non-positive Jacobian")
        g = np.einsum("ekl,al->eak", np.linalg.inv(J), dN)  # ∇N_a = J⁻¹ dN_a
        w = wq * detJ
        if not finite:
            Kq = (la[:, None, None, None, None] * np.einsum("eai,ebj->eaibj", g, g)
                  + mu[:, None, None, None, None] * np.einsum("eaj,ebi->eaibj", g, g)
                  + mu[:, None, None, None, None] * np.einsum("eak,ebk,ij->eaibj", g, g, I3))
            gu = np.einsum("eai,eaj->eij", ue, g)
            eps = 0.5 * (gu + gu.transpose(0, 2, 1))
            sig = (la * np.trace(eps, axis1=1, axis2=2))[:, None, None] * I3 + 2 * mu[:, None, None] * eps
            fq = np.einsum("eij,eaj->eai", sig, g)
        else:
            gu = np.einsum("eai,eaj->eij", ue, g)
            F = I3 + gu
            Cm = np.einsum("eki,ekj->eij", F, F)
            if model == 1:
                Ci = np.linalg.inv(Cm)
                lnJ = 0.5 * np.log(np.linalg.det(Cm))
                S = mu[:, None, None] * (I3 - Ci) + (la * lnJ)[:, None, None] * Ci
                c = mu - la * lnJ
                D = (la[:, None, None, None, None] * np.einsum("eij,ekl->eijkl", Ci, Ci)
                     + c[:, None, None, None, None] * (np.einsum("eik,ejl->eijkl", Ci, Ci)
                                                       + np.einsum("eil,ejk->eijkl", Ci, Ci)))
            else:
                Egl = 0.5 * (Cm - I3)
                S = (la * np.trace(Egl, axis1=1, axis2=2))[:, None, None] * I3 + 2 * mu[:, None, None] * Egl
                D = (la[:, None, None, None, None] * np.einsum("ij,kl->ijkl", I3, I3)[None]
                     + mu[:, None, None, None, None] * (np.einsum("ik,jl->ijkl", I3, I3)
                                                        + np.einsum("il,jk->ijkl", I3, I3))[None])
            A = np.einsum("eim,emjnl,ekn->eijkl", F, D, F) + np.einsum("ik,ejl->eijkl", I3, S)
            Kq = np.einsum("eaj,eijkl,ebl->eaibk", g, A, g)
            P = np.einsum("eik,ekj->eij", F, S)
            fq = np.einsum("eij,eaj->eai", P, g)
        K += w[:, None, None, None, None] * Kq
        f += w[:, None, None] * fq
    return K.reshape(ne, 3 * nn, 3 * nn), f.reshape(ne, 3 * nn)


def assemble(et, X, conn, E, nu, u=None, model=0, finite=False):
    """scipy CSC K (sorted indices, duplicates summed, zeros kept) and f_int."""
    import scipy.sparse as sp
    X = np.asarray(X, dtype=np.float64)
    conn = np.asarray(conn, dtype=np.int64)
    Ke, fe = element_arrays(et, X, conn, E, nu, u=u, model=model, finite=finite)
    ne, nn = conn.shape
    gd = (3 * conn[:, :, None] + np.arange(3)[None, None, :]).reshape(ne, 3 * nn)
    rows = np.repeat(gd[:, :, None], 3 * nn, axis=2).ravel()
    cols = np.repeat(gd[:, None, :], 3 * nn, axis=1).ravel()
    n = 3 * X.shape[0]
    K = sp.coo_matrix((Ke.ravel(), (rows, cols)), shape=(n, n)).tocsc()
    K.sum_duplicates()
    K.sort_indices()
    fint = np.zeros(n)
    np.add.at(fint, gd.ravel(), fe.ravel())
    return K, fint


def traction(ft, fconn, X, t, p=None):
    """Consistent surface load: Σ w‖∂X/∂ξ₁×∂X/∂ξ₂‖ t Nᵢ, plus, when the
    per-face pressure p is given, Σ w (∂X/∂ξ₁×∂X/∂ξ₂)(−p) Nᵢ (the normal
    times the area element; problems_elasticity.jl:486-493)."""
    X = np.asarray(X, dtype=np.float64)
    fconn = np.asarray(fconn, dtype=np.int64)
    nf = fconn.shape[0]
    t = np.broadcast_to(np.asarray(t, dtype=np.float64), (nf, 3))
    pf = None if p is None else np.broadcast_to(np.asarray(p, dtype=np.float64), (nf,))
    if ft == 3:
        pts, wts = np.array([[1 / 3, 1 / 3]]), np.array([0.5])
    elif ft == 6:
        pts = np.array([[2 / 3, 1 / 6], [1 / 6, 2 / 3], [1 / 6, 1 / 6]])
        wts = np.full(3, 1 / 6)
    elif ft == 4:
        p = np.array([-_SQ3, _SQ3])
        pts = np.array([[p[i], p[j]] for j in range(2) for i in range(2)])
        wts = np.ones(4)
    else:
        raise ValueError(ft)
    f = np.zeros(3 * X.shape[0])
    for xi, wq in zip(pts, wts):
        u, v = xi
        if ft == 3:
            N = np.array([1 - u - v, u, v])
            dN = np.array([[-1, -1], [1, 0], [0, 1]], dtype=float)
        elif ft == 6:
            L = np.array([1 - u - v, u, v])
            dL = np.array([[-1, -1], [1, 0], [0, 1]], dtype=float)
            N = np.empty(6)
            dN = np.empty((6, 2))
            for i in range(3):
                N[i] = L[i] * (2 * L[i] - 1)
                dN[i] = (4 * L[i] - 1) * dL[i]
            for m, (i, j) in enumerate(((0, 1), (1, 2), (2, 0))):
                N[3 + m] = 4 * L[i] * L[j]
                dN[3 + m] = 4 * (dL[i] * L[j] + L[i] * dL[j])
        else:
            s = np.array([[-1, -1], [1, -1], [1, 1], [-1, 1]], dtype=float)
            N = 0.25 * (1 + s[:, 0] * u) * (1 + s[:, 1] * v)
            dN = np.stack([0.25 * s[:, 0] * (1 + s[:, 1] * v), 0.25 * (1 + s[:, 0] * u) * s[:, 1]], 1)
        Xf = X[fconn]                                    # (nf, nfn, 3)
        T = np.einsum("ak,fab->fkb", dN, Xf)             # (nf, 2, 3)
        area = np.linalg.norm(np.cross(T[:, 0], T[:, 1]), axis=1)
        load = t if pf is None else t - pf[:, None] * np.cross(T[:, 0], T[:, 1]) / area[:, None]
        contrib = (wq * area)[:, None, None] * load[:, None, :] * N[None, :, None]
        np.add.at(f, (3 * fconn[:, :, None] + np.arange(3)).ravel(), contrib.ravel())
    return f


def mass_rule(et):
    """Rules exact for N·Nᵀ: GLTET4 (Tet4), GLTET15 (Tet10, the points and
    weights of src/quadrature/gltet.jl:46-63), GLHEX8 (Hex8)."""
    if et == 4:
        return rule(10)
    if et == 8:
        return rule(8)
    s15 = np.sqrt(15.0)
    a = 0.25
    b1, b2 = (7 + s15) / 34, (7 - s15) / 34
    c1, c2 = (13 - 3 * s15) / 34, (13 + 3 * s15) / 34
    d, f = (5 - s15) / 20, (5 + s15) / 20
    w1, w2, w3, w4 = 8 / 405, (2665 - 14 * s15) / 226800, (2665 + 14 * s15) / 226800, 5 / 567
    pts = [(a, a, a), (b1, b1, b1), (b1, b1, c1), (b1, c1, b1), (c1, b1, b1), (b2, b2, b2), (b2, b2, c2),
           (b2, c2, b2), (c2, b2, b2), (d, d, f), (d, f, d), (f, d, d), (d, f, f), (f, d, f), (f, f, d)]
    return np.array(pts), np.array([w1] + [w2] * 4 + [w3] * 4 + [w4] * 6)


def lsq_fit(et, X, conn, E, nu, u, field):
    """Least-squares nodal fit of the small-strain strain (field 0) or stress
    (field 1) vector (order 11, 22, 33, 12, 23, 13, tensor shear components) as
    lsq_fit + get_strain_vector / get_stress_vector of
    src/problems_elasticity.jl:521-583: A = Σ w N Nᵀ, b = Σ w N f, A x = b on
    the nodes the elements touch (scipy's spsolve standing in for ldlt).  The
    integration uses mass_rule(et): the elements' own rules (GLTET1 / GLTET4)
    make A singular on simplices, a defect not replicated."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    X = np.asarray(X, dtype=np.float64)
    conn = np.asarray(conn, dtype=np.int64)
    ne, nn = conn.shape
    nnode = X.shape[0]
    la, mu = lame(np.broadcast_to(E, (ne,)), np.broadcast_to(nu, (ne,)))
    Xe = X[conn]
    ue = np.asarray(u, dtype=np.float64).reshape(-1, 3)[conn]
    pts, wts = mass_rule(et)
    rows, cols, vals = [], [], []
    b = np.zeros((nnode, 6))
    I3 = np.eye(3)
    for xi, wq in zip(pts, wts):
        N, dN = basis(et, xi)
        J = np.einsum("ak,eab->ekb", dN, Xe)
        detJ = np.linalg.det(J)
        g = np.einsum("ekl,al->eak", np.linalg.inv(J), dN)
        gu = np.einsum("eai,eaj->eij", ue, g)
        eps = 0.5 * (gu + gu.transpose(0, 2, 1))
        if field == 0:
            t = eps
        else:
            t = (la * np.trace(eps, axis1=1, axis2=2))[:, None, None] * I3 + 2 * mu[:, None, None] * eps
        f = np.stack([t[:, 0, 0], t[:, 1, 1], t[:, 2, 2], t[:, 0, 1], t[:, 1, 2], t[:, 0, 2]], axis=1)
        w = wq * detJ
        for a in range(nn):
            np.add.at(b, conn[:, a], (w * N[a])[:, None] * f)
            for c in range(nn):
                rows.append(conn[:, a])
                cols.append(conn[:, c])
                vals.append(w * N[a] * N[c])
    A = sp.csc_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(nnode, nnode))
    A = 0.5 * (A + A.T)
    nz = np.unique(conn)
    x = np.zeros((nnode, 6))
    x[nz] = spla.spsolve(A[nz][:, nz].tocsc(), b[nz])
    return x
