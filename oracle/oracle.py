"""ctypes front end of the C++ FP64 oracle (oracle/jfem_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline legs as the checker.  The product never imports it.

Parity status: "parity unpinned" by the reference (no executable reference, no
golden vectors for this path in its tests); pinned by the reference fixture
test/testdata/cube_tet4.inp as a patch test, by closed forms, and by the
independent numpy restatement in oracle/np_oracle.py.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "jfem_oracle.cpp"
LIB = HERE / "_build" / "libjfem_oracle.so"

_i64p = C.POINTER(C.c_int64)
_f64p = C.POINTER(C.c_double)
_u8p = C.POINTER(C.c_uint8)

NEN = {4: 4, 10: 10, 8: 8}
NFN = {3: 3, 6: 6, 4: 4}


def build(force: bool = False) -> Path:
    """Compile the oracle shared library (g++, OpenMP, no -march flags)."""
    LIB.parent.mkdir(parents=True, exist_ok=True)
    if force or not LIB.exists() or LIB.stat().st_mtime < SRC.stat().st_mtime:
        cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-shared", "-fPIC",
               str(SRC), "-o", str(LIB)]
        subprocess.run(cmd, check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        L.orc_element.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _f64p, _f64p,
                                  C.c_double, C.c_double, _f64p, _f64p]
        L.orc_assemble_coo.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int64, _f64p,
                                       C.c_int64, _i64p, _f64p, _f64p, C.c_int, _f64p,
                                       _i64p, _i64p, _i64p, _f64p, _f64p]
        L.orc_pattern.argtypes = [C.c_int, C.c_int64, C.c_int64, _i64p, _i64p, _i64p, _i64p]
        L.orc_assemble_pattern.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int64, _f64p,
                                           C.c_int64, _i64p, _f64p, _f64p, C.c_int, _f64p,
                                           _i64p, _i64p, _f64p, _f64p]
        L.orc_traction.argtypes = [C.c_int, C.c_int64, _i64p, _f64p, _f64p, _f64p]
        L.orc_pressure.argtypes = [C.c_int, C.c_int64, _i64p, _f64p, _f64p, _f64p]
        L.orc_csc_spmv.argtypes = [C.c_int64, _i64p, _i64p, _f64p, _f64p, _f64p]
        L.orc_csc_spmv.restype = None
        L.orc_pcg.argtypes = [C.c_int64, _i64p, _i64p, _f64p, _f64p, _u8p, C.c_double, C.c_int,
                              _f64p, C.POINTER(C.c_int), _f64p]
        L.orc_apply.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int64, _f64p, C.c_int64,
                                _i64p, _f64p, _f64p, C.c_int, _f64p, _f64p, _f64p]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_set_threads.restype = None
        L.orc_get_threads.restype = C.c_int
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t) if a is not None else None


def _f(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def _mat(E, nu, n_elem):
    E = np.atleast_1d(np.asarray(E, dtype=np.float64))
    nu = np.atleast_1d(np.asarray(nu, dtype=np.float64))
    per = int(E.size > 1 or nu.size > 1)
    if per:
        E = np.broadcast_to(E, (n_elem,)).copy()
        nu = np.broadcast_to(nu, (n_elem,)).copy()
    return E, nu, per


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def get_threads() -> int:
    return int(lib().orc_get_threads())


def element(et, Xe, E, nu, ue=None, model=0, finite=False, geom=False):
    """Element stiffness (column-major (3n)²) and internal force (3n)."""
    nn = NEN[et]
    Xe = np.ascontiguousarray(Xe, dtype=np.float64).reshape(nn, 3)
    ue = None if ue is None else np.ascontiguousarray(ue, dtype=np.float64).reshape(nn, 3)
    Ke = np.zeros((3 * nn) * (3 * nn))
    fe = np.zeros(3 * nn)
    rc = lib().orc_element(et, model, int(finite), int(geom), _p(Xe, _f64p), _p(ue, _f64p),
                           float(E), float(nu), _p(Ke, _f64p), _p(fe, _f64p))
    if rc != 0:
        raise RuntimeError(f"orc_element failed with status {rc}")
    return Ke.reshape(3 * nn, 3 * nn, order="F"), fe


def assemble_coo(et, X, conn, E, nu, u=None, model=0, finite=False, geom=False):
    """Global (colptr, rowval, nzval, fint) by COO push + sparse() semantics."""
    X = _f(X)
    conn = np.ascontiguousarray(conn, dtype=np.int64)
    E, nu, per = _mat(E, nu, conn.shape[0])
    u = _f(u)
    L = lib()
    n = 3 * X.shape[0]
    nnz = C.c_int64(0)
    args = (et, model, int(finite), int(geom), X.shape[0], _p(X, _f64p), conn.shape[0],
            _p(conn, _i64p), _p(E, _f64p), _p(nu, _f64p), per, _p(u, _f64p))
    rc = L.orc_assemble_coo(*args, C.byref(nnz), None, None, None, None)
    if rc != 0:
        raise RuntimeError(f"orc_assemble_coo failed with status {rc}")
    colptr = np.zeros(n + 1, np.int64)
    rowval = np.zeros(nnz.value, np.int64)
    nzval = np.zeros(nnz.value)
    fint = np.zeros(n)
    rc = L.orc_assemble_coo(*args, C.byref(nnz), _p(colptr, _i64p), _p(rowval, _i64p),
                            _p(nzval, _f64p), _p(fint, _f64p))
    if rc != 0:
        raise RuntimeError(f"orc_assemble_coo failed with status {rc}")
    return colptr, rowval, nzval, fint


def pattern(et, n_nodes, conn):
    conn = np.ascontiguousarray(conn, dtype=np.int64)
    L = lib()
    nnz = C.c_int64(0)
    rc = L.orc_pattern(et, n_nodes, conn.shape[0], _p(conn, _i64p), C.byref(nnz), None, None)
    if rc != 0:
        raise RuntimeError("orc_pattern failed")
    colptr = np.zeros(3 * n_nodes + 1, np.int64)
    rowval = np.zeros(nnz.value, np.int64)
    rc = L.orc_pattern(et, n_nodes, conn.shape[0], _p(conn, _i64p), C.byref(nnz),
                       _p(colptr, _i64p), _p(rowval, _i64p))
    if rc != 0:
        raise RuntimeError("orc_pattern failed")
    return colptr, rowval


def assemble_pattern(et, X, conn, E, nu, colptr, rowval, u=None, model=0, finite=False,
                     geom=False):
    """In-place add into a fixed CSC pattern (sparsematrixcsc.jl:69-98 semantics)."""
    X = _f(X)
    conn = np.ascontiguousarray(conn, dtype=np.int64)
    E, nu, per = _mat(E, nu, conn.shape[0])
    u = _f(u)
    nzval = np.zeros(rowval.size)
    fint = np.zeros(3 * X.shape[0])
    rc = lib().orc_assemble_pattern(et, model, int(finite), int(geom), X.shape[0],
                                    _p(X, _f64p), conn.shape[0], _p(conn, _i64p),
                                    _p(E, _f64p), _p(nu, _f64p), per, _p(u, _f64p),
                                    _p(colptr, _i64p), _p(rowval, _i64p), _p(nzval, _f64p),
                                    _p(fint, _f64p))
    if rc != 0:
        raise RuntimeError(f"orc_assemble_pattern failed with status {rc}")
    return nzval, fint


def traction(ft, fconn, X, t, n_nodes=None):
    """Consistent surface load vector; t is (3,) or (n_faces, 3)."""
    X = _f(X)
    fconn = np.ascontiguousarray(fconn, dtype=np.int64)
    nf = fconn.shape[0]
    t = np.ascontiguousarray(np.broadcast_to(np.asarray(t, dtype=np.float64), (nf, 3)))
    f = np.zeros(3 * (X.shape[0] if n_nodes is None else n_nodes))
    rc = lib().orc_traction(ft, nf, _p(fconn, _i64p), _p(X, _f64p), _p(t, _f64p), _p(f, _f64p))
    if rc != 0:
        raise RuntimeError("orc_traction failed")
    return f


def pressure(ft, fconn, X, p, n_nodes=None):
    """Consistent surface-pressure load (problems_elasticity.jl:486-493); p is a
    scalar or one value per face, positive towards the surface."""
    X = _f(X)
    fconn = np.ascontiguousarray(fconn, dtype=np.int64)
    nf = fconn.shape[0]
    p = np.ascontiguousarray(np.broadcast_to(np.asarray(p, dtype=np.float64), (nf,)))
    f = np.zeros(3 * (X.shape[0] if n_nodes is None else n_nodes))
    rc = lib().orc_pressure(ft, nf, _p(fconn, _i64p), _p(X, _f64p), _p(p, _f64p), _p(f, _f64p))
    if rc != 0:
        raise RuntimeError("orc_pressure failed")
    return f


def spmv(colptr, rowval, nzval, x):
    x = _f(x)
    y = np.zeros(colptr.size - 1)
    lib().orc_csc_spmv(colptr.size - 1, _p(colptr, _i64p), _p(rowval, _i64p),
                       _p(nzval, _f64p), _p(x, _f64p), _p(y, _f64p))
    return y


def pcg(colptr, rowval, nzval, b, fixed, tol=1e-10, maxit=100000, x0=None):
    """Jacobi-PCG with prescribed DOFs eliminated; returns (x, iters, relres, status)."""
    n = colptr.size - 1
    b = _f(b)
    fx = np.ascontiguousarray(fixed, dtype=np.uint8)
    x = np.zeros(n) if x0 is None else _f(x0).copy()
    it = C.c_int(0)
    rr = C.c_double(0)
    rc = lib().orc_pcg(n, _p(colptr, _i64p), _p(rowval, _i64p), _p(nzval, _f64p), _p(b, _f64p),
                       _p(fx, _u8p), float(tol), int(maxit), _p(x, _f64p), C.byref(it),
                       C.byref(rr))
    return x, it.value, rr.value, rc


def apply(et, X, conn, E, nu, v, u=None, model=0, finite=False, geom=False):
    """Matrix-free y = K(u)·v in FP64, element by element."""
    X = _f(X)
    conn = np.ascontiguousarray(conn, dtype=np.int64)
    E, nu, per = _mat(E, nu, conn.shape[0])
    v = _f(v)
    u = _f(u)
    y = np.zeros(3 * X.shape[0])
    rc = lib().orc_apply(et, model, int(finite), int(geom), X.shape[0], _p(X, _f64p),
                         conn.shape[0], _p(conn, _i64p), _p(E, _f64p), _p(nu, _f64p), per,
                         _p(u, _f64p), _p(v, _f64p), _p(y, _f64p))
    if rc != 0:
        raise RuntimeError(f"orc_apply failed with status {rc}")
    return y


def to_scipy(colptr, rowval, nzval, n=None):
    import scipy.sparse as sp
    n = colptr.size - 1 if n is None else n
    return sp.csc_matrix((nzval, rowval, colptr), shape=(n, n))


def direct_solve(colptr, rowval, nzval, b, fixed, g=None):
    """Elimination + sparse direct solve (solvers.jl:192-216 with scipy for CHOLMOD).

    K = ½(K + Kᵀ) first (solvers.jl:289-292).
    """
    import scipy.sparse.linalg as spl
    K = to_scipy(colptr, rowval, nzval)
    K = (0.5 * (K + K.T)).tocsc()
    n = K.shape[0]
    fixed = np.asarray(fixed, dtype=bool)
    u = np.zeros(n)
    if g is not None:
        u[fixed] = np.asarray(g)[fixed]
    Ifree = np.nonzero(~fixed)[0]
    B = np.nonzero(fixed)[0]
    rhs = np.asarray(b)[Ifree] - K[Ifree][:, B] @ u[B]
    u[Ifree] = spl.spsolve(K[Ifree][:, Ifree].tocsc(), rhs)
    return u


def newton(et, X, conn, E, nu, fixed, g_final, f_ext=None, n_steps=10, tol=1e-8, max_newton=20,
           model=1):
    """Load-stepped Newton with the consistent tangent (Km + Kg) and a direct solve.

    Legacy nonlinear loop of src/solvers.jl:575-620 (re-assemble, solve, u += Δu).
    The prescribed values enter incrementally as in src/problems_dirichlet.jl:60-89
    (g = u_prescribed − u_prev): the first iteration of a step carries the whole
    increment of the prescribed DOFs, later iterations keep them fixed.  A step has
    converged when ‖R_free‖ ≤ tol·‖f_int‖ (FP64; f_int includes the reactions).
    g_final holds the prescribed values at the last step; step s prescribes
    s/n_steps of them.  Returns (u, newton_iterations_per_step).
    """
    n = 3 * X.shape[0]
    fixed = np.asarray(fixed, dtype=bool)
    u = np.zeros(n)
    f_ext = np.zeros(n) if f_ext is None else np.asarray(f_ext, dtype=np.float64)
    colptr, rowval = pattern(et, X.shape[0], conn)
    its = []
    for s in range(1, n_steps + 1):
        frac = s / n_steps
        target = frac * np.asarray(g_final, dtype=np.float64)
        k = 0
        for k in range(1, max_newton + 1):
            nz, fint = assemble_pattern(et, X, conn, E, nu, colptr, rowval, u=u, model=model,
                                        finite=True, geom=True)
            R = frac * f_ext - fint
            R[fixed] = 0.0
            rn = np.linalg.norm(R)
            if k > 1 and rn <= tol * max(np.linalg.norm(fint), 1e-300):
                break
            g = np.zeros(n)
            g[fixed] = target[fixed] - u[fixed]
            du = direct_solve(colptr, rowval, nz, R, fixed, g=g)
            u += du
        its.append(k)
    return u, its


def rcm(conn, n_nodes, start=0):
    """Reverse Cuthill–McKee as symrcm of src/graph/graph_ordering.jl:21-98
    (breadth-first from `start`, neighbours by increasing degree with a stable
    sort, reversed), on the node graph with ascending adjacency lists; nodes
    unreachable from `start` continue from the lowest unvisited node.
    Pure Python: small graphs only."""
    conn = np.asarray(conn, dtype=np.int64)
    nb = [set() for _ in range(n_nodes)]
    for el in conn:
        for a in el:
            nb[a].update(int(b) for b in el if b != a)
    adj = [sorted(s) for s in nb]
    deg = [len(a) for a in adj]
    visited = [False] * n_nodes
    order = []
    s = start
    while len(order) < n_nodes:
        visited[s] = True
        head = len(order)
        order.append(s)
        while head < len(order):
            v = order[head]
            head += 1
            for w in sorted(adj[v], key=lambda j: deg[j]):      # stable: ties keep ascending order
                if not visited[w]:
                    visited[w] = True
                    order.append(w)
        rest = [k for k in range(n_nodes) if not visited[k]]
        if rest:
            s = rest[0]
    perm = np.array(order[::-1], dtype=np.int64)
    newpos = np.empty(n_nodes, np.int64)
    newpos[perm] = np.arange(n_nodes)
    bw = lambda pos: 2 * max(abs(int(pos[v]) - int(pos[w])) for v in range(n_nodes) for w in adj[v]) + 1
    return perm, bw(np.arange(n_nodes)), bw(newpos)
