"""numpy/scipy restatement of the two-level preconditioner's coarse level.

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker of the CUDA coarse
space (juliafem.jl_gb300/csrc/jfem_coarse.cu); the product never imports it.

The reference has no coarse space (its CG is unpreconditioned,
src/backend/cpu.jl:221-254, ext/JuliaFEMCUDAExt.jl:531-577); its GPU solver
design note recommends a multigrid-type coarse correction
(docs/src/book/design/gpu_solver_strategy_expert_validated.md:114-156).  The
semantics restated here are the library's own:

* aggregation — nodes binned into nb[d] = max(1, round(ext_d / H)) equal boxes
  per axis over the bounding box, H = (ext_x·ext_y·ext_z / (target/6))^(1/3),
  ext_d = max(hi_d − lo_d, 1e-9·max_d ext), box index
  min(nb_d − 1, floor((X_d − lo_d)/ext_d·nb_d)); occupied boxes numbered in
  ascending (x fastest) box order;
* P — for aggregate a and node i in it, d_i = X_i − c_a (c_a the mean of the
  aggregate's node coordinates): columns 6a..6a+2 the unit translations,
  6a+3..6a+5 the rotations e_k × d_i; rows of prescribed DOFs zero;
* A_c = Pᵀ K P with K the oracle's FP64 assembled stiffness;
* M r = D⁻¹ r + P A_c⁻¹ Pᵀ r on the free DOFs (zero on prescribed ones).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp


def auto_coarse_dofs(n_dofs: int) -> int:
    return int(min(2304, max(192, n_dofs // 1000)))


def aggregates(X, target_nc: int):
    """(aggregate of each node, number of aggregates, bins per axis)."""
    X = np.asarray(X, dtype=np.float64).reshape(-1, 3)
    lo, hi = X.min(0), X.max(0)
    emax = float((hi - lo).max())
    ext = np.maximum(hi - lo, 1e-9 * emax)
    n_target = max(1, target_nc // 6)
    H = np.cbrt(ext[0] * ext[1] * ext[2] / n_target)
    nb = np.maximum(1, np.floor(ext / H + 0.5)).astype(np.int64)
    b = np.minimum(nb - 1, np.floor((X - lo) / ext * nb).astype(np.int64))
    b = np.maximum(b, 0)
    cell = b[:, 0] + nb[0] * (b[:, 1] + nb[1] * b[:, 2])
    occupied, agg = np.unique(cell, return_inverse=True)
    return agg.astype(np.int64), occupied.size, tuple(int(v) for v in nb)


def prolongation(X, agg, n_agg, fixed_mask):
    """P (3N × 6·n_agg, CSC) of the rigid-body modes of each aggregate."""
    X = np.asarray(X, dtype=np.float64).reshape(-1, 3)
    n = X.shape[0]
    cen = np.zeros((n_agg, 3))
    np.add.at(cen, agg, X)
    cen /= np.bincount(agg, minlength=n_agg)[:, None]
    d = X - cen[agg]
    nodes = np.arange(n)
    rows, cols, vals = [], [], []
    for c in range(3):                                   # translations
        rows.append(3 * nodes + c)
        cols.append(6 * agg + c)
        vals.append(np.ones(n))
    rot = [((1, -d[:, 2]), (2, d[:, 1])),                # e_x × d
           ((0, d[:, 2]), (2, -d[:, 0])),                # e_y × d
           ((0, -d[:, 1]), (1, d[:, 0]))]                # e_z × d
    for k, comps in enumerate(rot):
        for c, v in comps:
            rows.append(3 * nodes + c)
            cols.append(6 * agg + 3 + k)
            vals.append(v)
    P = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                      shape=(3 * n, 6 * n_agg))
    free = (np.asarray(fixed_mask).reshape(-1) == 0).astype(np.float64)
    return (sp.diags(free) @ P).tocsc()


def coarse_matrix(K, P):
    """A_c = Pᵀ K P (dense)."""
    return np.asarray((P.T @ (K @ P)).todense())


def two_level(K, P, fixed_mask):
    """The preconditioner r ↦ D⁻¹ r + P A_c⁻¹ Pᵀ r (free DOFs) as a function."""
    free = np.asarray(fixed_mask).reshape(-1) == 0
    dinv = np.where(free, 1.0 / K.diagonal(), 0.0)
    Ac = coarse_matrix(K, P)
    return lambda r: dinv * r + np.where(free, P @ np.linalg.solve(Ac, P.T @ r), 0.0)


def pcg(K, b, fixed_mask, M, tol=1e-8, maxit=20000):
    """PCG on the free DOFs, stopping on the recursive residual ‖r‖ ≤ tol‖b_free‖;
    returns (x, iterations)."""
    fr = (np.asarray(fixed_mask).reshape(-1) == 0).astype(np.float64)
    x = np.zeros_like(b)
    r = b * fr
    z = M(r)
    p = z.copy()
    rz = r @ z
    bb = np.sqrt(r @ r)
    for it in range(1, maxit + 1):
        q = (K @ (p * fr)) * fr
        a = rz / (p @ q)
        x += a * p
        r -= a * q
        if np.sqrt(r @ r) <= tol * bb:
            return x, it
        z = M(r)
        rzn = r @ z
        p = z + (rzn / rz) * p
        rz = rzn
    return x, maxit
