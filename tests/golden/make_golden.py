"""Mint the golden fixtures of the elasticity hot path.

Run from the repository root:  python tests/golden/make_golden.py

* cube_tet4.npz — the reference's own fixture test/testdata/cube_tet4.inp
  (10 nodes, 17 C3D4, symmetry planes, unit pressure on the top face) parsed by
  the package's Abaqus reader, plus its analytic solution: a linear field
  u = (νx/E, νy/E, −z/E) that Tet4 must reproduce exactly (patch test).
  Needs a JuliaFEM.jl source tree named by the environment variable
  JFEM_REFERENCE_ROOT; skipped when it is unset or the file is absent.
* tet4_cantilever.npz — oracle outputs for the Tet4 40×4×4 cantilever: a
  SHA-256 of the CSC pattern, nnz, seeded samples of K, K·w for a seeded w,
  f, and u from the elimination + sparse direct solve (the oracle's stand-in
  for CHOLMOD ldlt, src/solvers.jl:192-216).
* tet10_cantilever_small.npz — the same for the Tet10 40×4×4 cantilever on
  [0,4]×[0,0.4]² (19,683 DOFs).
* hex8_neohookean_small.npz — load-stepped Newton (oracle, FP64, direct
  solves) on a 4×4×4 Hex8 Neo-Hookean cube, top u_z = −0.1 over 5 steps.
* hex8_neohookean_16.npz — the Newton–Krylov configuration at a
  representative size: 16³ Hex8 Neo-Hookean cube, per-element lognormal E
  (σ_log 0.2), top u_z = −0.1 over 10 load steps, oracle Newton to 1e-11
  (about a minute of direct solves, hence a fixture rather than a test-time
  oracle run).

`python tests/golden/make_golden.py hex8_16` writes only the last one.

The oracle is the restatement in oracle/jfem_oracle.cpp, cross-checked against
oracle/np_oracle.py before anything is written.
"""
from __future__ import annotations

import hashlib
import os
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))
import jfem_loader  # noqa: E402
import np_oracle  # noqa: E402
import oracle  # noqa: E402

OUT = Path(__file__).resolve().parent
REF_INP = Path(os.environ.get("JFEM_REFERENCE_ROOT", "")) / "test" / "testdata" / "cube_tet4.inp" \
    if os.environ.get("JFEM_REFERENCE_ROOT") else None


def pattern_hash(colptr, rowval) -> str:
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(colptr, dtype=np.int64).tobytes())
    h.update(np.ascontiguousarray(rowval, dtype=np.int64).tobytes())
    return h.hexdigest()


def linear_case(w, samples=4096):
    m = w.mesh
    cp, rv, nz, _ = oracle.assemble_coo(m.elem_type, m.X, m.conn, w.E, w.nu)
    K2, _ = np_oracle.assemble(m.elem_type, m.X, m.conn, w.E, w.nu)
    assert np.array_equal(K2.indptr, cp) and np.array_equal(K2.indices, rv)
    assert np.abs(K2.data - nz).max() <= 1e-13 * np.abs(nz).max()
    f = oracle.traction(w.face_type, w.faces, m.X, w.traction)
    f2 = np_oracle.traction(w.face_type, w.faces, m.X, w.traction)
    assert np.abs(f - f2).max() <= 1e-14
    g = np.random.Generator(np.random.Philox(key=7))
    idx = np.sort(g.choice(nz.size, size=min(samples, nz.size), replace=False))
    wv = g.standard_normal(m.n_dofs)
    Kw = oracle.spmv(cp, rv, nz, wv)
    u = oracle.direct_solve(cp, rv, nz, f, w.fixed_mask().astype(bool))
    up, it, rr, st = oracle.pcg(cp, rv, nz, f, w.fixed_mask(), tol=1e-12, maxit=200000)
    assert np.abs(up - u).max() <= 1e-8 * np.abs(u).max()
    return dict(pattern_sha256=pattern_hash(cp, rv), nnz=nz.size, n=m.n_dofs, sample_idx=idx,
                sample_val=nz[idx], K_fro=np.sqrt((nz ** 2).sum()), w=wv, Kw=Kw, f=f, u=u,
                pcg_iters_1e12=it)


def newton_16(jfem):
    w = jfem.workloads.cube_compression(n=16, steps=10, top_uz=-0.1)
    m = w.mesh
    u, its = oracle.newton(m.elem_type, m.X, m.conn, w.E, w.nu, w.fixed_mask().astype(bool), w.prescribed(),
                           n_steps=10, tol=1e-11, max_newton=25, model=1)
    np.savez_compressed(OUT / "hex8_neohookean_16.npz", u=u, newton_its=np.array(its), E=w.E)


def main():
    jfem = jfem_loader.load_package()
    wl = jfem.workloads
    oracle.build()
    if sys.argv[1:] == ["hex8_16"]:
        newton_16(jfem)
        print("golden fixture written to", OUT)
        return
    newton_16(jfem)
    # Tet4 cantilever
    w1 = wl.cfg_tet4_cantilever()
    np.savez_compressed(OUT / "tet4_cantilever.npz", **linear_case(w1))
    # Tet10 small cantilever
    w2 = wl.cantilever(10, 40, 4, 4, 4.0, 0.4, 0.4, name="tet10_small")
    np.savez_compressed(OUT / "tet10_cantilever_small.npz", **linear_case(w2, samples=8192))
    # Hex8 Neo-Hookean Newton
    w3 = wl.cube_compression(n=4, steps=5, top_uz=-0.1)
    m = w3.mesh
    u, its = oracle.newton(m.elem_type, m.X, m.conn, w3.E, w3.nu, w3.fixed_mask().astype(bool),
                           w3.prescribed(), n_steps=w3.n_load_steps, tol=1e-10, max_newton=25, model=1)
    np.savez_compressed(OUT / "hex8_neohookean_small.npz", u=u, newton_its=np.array(its), E=w3.E)
    # reference fixture (patch test)
    if REF_INP is not None and REF_INP.exists():
        ab = jfem.abaqus.read(str(REF_INP))
        et, X, conn, index, eids = ab.to_arrays()
        dofs, vals = jfem.abaqus.boundary_dofs(ab, index)
        faces = []
        p = []
        for sname, kind, val in ab.dsload:
            assert kind == "P"
            for ft, nodes in ab.surface_elements(sname):
                faces.append([index[n] for n in nodes])
                p.append(val)
        E, nu = ab.elastic
        P = p[0]
        # uniaxial compression σ_zz = −P with symmetry planes x=0, y=0, z=0
        u_exact = np.stack([nu * P * X[:, 0] / E, nu * P * X[:, 1] / E, -P * X[:, 2] / E], 1).ravel()
        np.savez_compressed(OUT / "cube_tet4.npz", X=X, conn=conn, dofs=dofs, vals=vals,
                            faces=np.array(faces, dtype=np.int64), p=np.array(p), E=E, nu=nu,
                            u_exact=u_exact, node_ids=np.array(sorted(index)), elem_ids=np.array(eids))
    print("golden fixtures written to", OUT)


if __name__ == "__main__":
    main()
