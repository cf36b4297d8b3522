"""ctypes binding of libjfem_cuda.so (include/jfem.h).

The library is the product: there is no CPU fallback.  Loading fails loudly
when the shared object has not been built (``build()`` in __graft_entry__ or
``python juliafem.jl_gb300/build.py``).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libjfem_cuda.so"

OK, NOT_CONVERGED, STALL = 0, 1, 2
ERR_INVALID, ERR_CUDA, ERR_OOM, ERR_NEG_JACOBIAN, ERR_NAN, ERR_TIMEOUT, ERR_TOO_LARGE = -1, -2, -3, -4, -5, -6, -7
NOALLOC_SCRATCH_BYTES = 64 << 20
TET4, TET10, HEX8 = 4, 10, 8
TRI3, TRI6, QUAD4 = 3, 6, 4
LINEAR_ELASTIC, NEO_HOOKEAN = 0, 1
PCG_JACOBI, FCG_LEARNED, NEWTON, FCG_TWO_LEVEL = 0, 1, 2, 3
FP64, MIXED = 0, 1
APPLY_FP32, APPLY_MASKED = 1, 2
HISTORY_MAX = 256
MPNN_WIDTH, MPNN_PARAMS = 32, 4384

NEN = {TET4: 4, TET10: 10, HEX8: 8}
NFN = {TRI3: 3, TRI6: 6, QUAD4: 4}

_ERRNAMES = {ERR_INVALID: "invalid argument", ERR_CUDA: "CUDA error", ERR_OOM: "out of memory",
             ERR_NEG_JACOBIAN: "non-positive Jacobian", ERR_NAN: "NaN / invalid material state",
             ERR_TIMEOUT: "time budget exceeded", ERR_TOO_LARGE: "mesh too large for the fixed scratch"}


class JFEMError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{_ERRNAMES.get(code, 'error')} ({code}): {msg}")
        self.code = code


class SolveOpts(C.Structure):
    _fields_ = [("method", C.c_int), ("precision", C.c_int), ("tol", C.c_double), ("max_iter", C.c_int),
                ("newton_tol", C.c_double), ("max_newton", C.c_int), ("max_cg_per_newton", C.c_int),
                ("n_load_steps", C.c_int), ("forcing_power", C.c_double), ("forcing_max", C.c_double),
                ("time_budget_s", C.c_double), ("refine_drop", C.c_double), ("tol_absolute", C.c_int)]


class Stats(C.Structure):
    _fields_ = [("status", C.c_int), ("newton_iterations", C.c_int), ("cg_iterations", C.c_int),
                ("refinements", C.c_int), ("fallbacks", C.c_int), ("residual", C.c_double),
                ("solve_time_s", C.c_double), ("history_len", C.c_int),
                ("history", C.c_double * (3 * HISTORY_MAX))]

    def history_list(self):
        return [(int(self.history[3 * i]), float(self.history[3 * i + 1]), float(self.history[3 * i + 2]))
                for i in range(self.history_len)]


# Every symbol include/jfem.h declares, with its ctypes signature.
_P = C.c_void_p
_i64 = C.c_int64
_i64p = C.POINTER(C.c_int64)
_f64p = C.POINTER(C.c_double)
_f32p = C.POINTER(C.c_float)
SIGNATURES = {
    "jfem_version": (C.c_char_p, []),
    "jfem_default_opts": (None, [C.POINTER(SolveOpts)]),
    "jfem_create": (C.c_int, [C.POINTER(_P), C.c_int]),
    "jfem_destroy": (C.c_int, [_P]),
    "jfem_last_error": (C.c_char_p, [_P]),
    "jfem_set_mesh": (C.c_int, [_P, C.c_int, _i64, _f64p, _i64, _i64p, C.c_int]),
    "jfem_set_material": (C.c_int, [_P, C.c_int, _f64p, _f64p, C.c_int]),
    "jfem_set_formulation": (C.c_int, [_P, C.c_int, C.c_int]),
    "jfem_set_dirichlet": (C.c_int, [_P, _i64, _i64p, _f64p, C.c_int]),
    "jfem_set_traction": (C.c_int, [_P, C.c_int, _i64, _i64p, _f64p, C.c_int]),
    "jfem_set_surface_load": (C.c_int, [_P, C.c_int, _i64, _i64p, _f64p, _f64p, C.c_int]),
    "jfem_set_state": (C.c_int, [_P, _f64p]),
    "jfem_assemble_csc": (C.c_int, [_P, C.c_int, _i64p, _i64p, _i64p, _f64p, _f64p]),
    "jfem_apply": (C.c_int, [_P, _f64p, _f64p, C.c_int]),
    "jfem_apply_device": (C.c_int, [_P, _P, _P, C.c_int]),
    "jfem_internal_force": (C.c_int, [_P, _f64p]),
    "jfem_solve": (C.c_int, [_P, C.POINTER(SolveOpts), _f64p, C.POINTER(Stats)]),
    "jfem_solve_device": (C.c_int, [_P, C.POINTER(SolveOpts), _P, C.POINTER(Stats)]),
    "jfem_kernel_launches": (_i64, [_P]),
    "jfem_last_apply_ms": (C.c_double, [_P]),
    "jfem_stream": (C.c_void_p, [_P]),
    "jfem_time_apply": (C.c_int, [_P, C.c_int, C.c_int, _f64p, _f64p]),
    "jfem_time_assembly": (C.c_int, [_P, C.c_int, _f64p, _f64p, _i64p]),
    "jfem_apply_noalloc": (C.c_int, [C.c_int, _i64, _P, _i64, _P, C.c_int, _P, _P, _P, _P, _P]),
    "jfem_mpnn_init": (C.c_int, [_P, C.c_uint64]),
    "jfem_mpnn_set_weights": (C.c_int, [_P, _f32p]),
    "jfem_mpnn_get_weights": (C.c_int, [_P, _f32p]),
    "jfem_mpnn_collect": (C.c_int, [_P, C.c_int, C.c_double]),
    "jfem_mpnn_clear": (C.c_int, [_P]),
    "jfem_mpnn_train": (C.c_int, [_P, C.c_int, C.c_int, C.c_double, C.c_uint64, _f64p]),
    "jfem_mpnn_loss_grad": (C.c_int, [_P, _f64p, _f64p, _f64p, _f32p]),
    "jfem_mpnn_precondition": (C.c_int, [_P, _f64p, _f64p]),
    "jfem_set_coarse_space": (C.c_int, [_P, C.c_int]),
    "jfem_coarse_info": (C.c_int, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int64),
                                   C.POINTER(C.c_double)]),
    "jfem_coarse_matrix": (C.c_int, [_P, _f64p, C.POINTER(C.c_int)]),
    "jfem_coarse_precondition": (C.c_int, [_P, _f64p, _f64p]),
    "jfem_batch_create": (C.c_int, [C.POINTER(_P), C.c_int]),
    "jfem_batch_destroy": (C.c_int, [_P]),
    "jfem_batch_last_error": (C.c_char_p, [_P]),
    "jfem_batch_add": (C.c_int, [_P, _i64, _f64p, _i64, _i64p, C.c_int, C.c_double, C.c_double, _i64, _i64p,
                                 _i64, _i64p, _f64p]),
    "jfem_batch_solve": (C.c_int, [_P, C.c_double, C.c_int, C.c_int, _f64p, C.POINTER(C.c_int),
                                   C.POINTER(C.c_int), _f64p, _f64p, _f64p]),
    "jfem_batch_config": (C.c_int, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "jfem_batch_tune_source": (C.c_int, [_P]),
    "jfem_batch_cluster_config": (C.c_int, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "jfem_batch_set_config": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, C.c_int]),
    "jfem_rcm": (C.c_int, [_i64, _i64, C.c_int, _i64p, C.c_int, _i64, _i64p, _i64p, _i64p]),
    "jfem_recover_field": (C.c_int, [_P, _f64p, C.c_int, C.c_double, C.c_int, _f64p, C.POINTER(C.c_int)]),
}

_lib = None


def load(path: Path | str | None = None):
    """Load the shared library (raises if it is missing — there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p.name} is not built; run __graft_entry__.build() "
                           "(the CUDA library is required, there is no CPU path)")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _ptr(a, t):
    return None if a is None else a.ctypes.data_as(t)


def default_opts(**kw) -> SolveOpts:
    o = SolveOpts()
    load().jfem_default_opts(C.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise TypeError(f"unknown solve option {k}")
        setattr(o, k, v)
    return o


class Context:
    """One device context (one mesh on one GPU) behind the C ABI."""

    def __init__(self, device: int = 0):
        self._lib = load()
        h = C.c_void_p()
        rc = self._lib.jfem_create(C.byref(h), int(device))
        if rc != 0:
            raise JFEMError(rc, "jfem_create failed (no usable CUDA device?)")
        self._h = h
        self.n_nodes = 0
        self.n_elem = 0
        self.elem_type = 0

    def close(self):
        if getattr(self, "_h", None):
            self._lib.jfem_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc: int) -> int:
        if rc < 0:
            raise JFEMError(rc, self._lib.jfem_last_error(self._h).decode())
        return rc

    # -- model -----------------------------------------------------------------
    def set_mesh(self, elem_type: int, X, conn, index_base: int = 0):
        X = np.ascontiguousarray(X, dtype=np.float64).reshape(-1, 3)
        conn = np.ascontiguousarray(conn, dtype=np.int64).reshape(-1, NEN[elem_type])
        self._check(self._lib.jfem_set_mesh(self._h, elem_type, X.shape[0], _ptr(X, _f64p), conn.shape[0],
                                            _ptr(conn, _i64p), index_base))
        self.n_nodes, self.n_elem, self.elem_type = X.shape[0], conn.shape[0], elem_type

    def set_material(self, E, nu, model: int = LINEAR_ELASTIC):
        E = np.atleast_1d(np.asarray(E, dtype=np.float64))
        nu = np.atleast_1d(np.asarray(nu, dtype=np.float64))
        per = int(E.size > 1 or nu.size > 1)
        if per:
            E = np.ascontiguousarray(np.broadcast_to(E, (self.n_elem,)))
            nu = np.ascontiguousarray(np.broadcast_to(nu, (self.n_elem,)))
        self._check(self._lib.jfem_set_material(self._h, model, _ptr(E, _f64p), _ptr(nu, _f64p), per))

    def set_formulation(self, finite_strain: bool, geometric_stiffness: bool):
        self._check(self._lib.jfem_set_formulation(self._h, int(finite_strain), int(geometric_stiffness)))

    def set_dirichlet(self, dofs, values=None, index_base: int = 0):
        dofs = np.ascontiguousarray(dofs, dtype=np.int64)
        vals = None if values is None else np.ascontiguousarray(np.broadcast_to(values, dofs.shape),
                                                                 dtype=np.float64)
        self._check(self._lib.jfem_set_dirichlet(self._h, dofs.size, _ptr(dofs, _i64p), _ptr(vals, _f64p),
                                                 index_base))

    def set_traction(self, face_type: int, face_conn, t, index_base: int = 0):
        fc = np.ascontiguousarray(face_conn, dtype=np.int64).reshape(-1, NFN[face_type])
        t = np.ascontiguousarray(np.broadcast_to(np.asarray(t, dtype=np.float64), (fc.shape[0], 3)))
        self._check(self._lib.jfem_set_traction(self._h, face_type, fc.shape[0], _ptr(fc, _i64p),
                                                _ptr(t, _f64p), index_base))

    def set_surface_load(self, face_type: int, face_conn, t=None, p=None, index_base: int = 0):
        fc = np.ascontiguousarray(face_conn, dtype=np.int64).reshape(-1, NFN[face_type])
        nf = fc.shape[0]
        t = None if t is None else np.ascontiguousarray(np.broadcast_to(np.asarray(t, dtype=np.float64), (nf, 3)))
        p = None if p is None else np.ascontiguousarray(np.broadcast_to(np.asarray(p, dtype=np.float64), (nf,)))
        self._check(self._lib.jfem_set_surface_load(self._h, face_type, nf, _ptr(fc, _i64p), _ptr(t, _f64p),
                                                    _ptr(p, _f64p), index_base))

    def set_state(self, u=None):
        u = None if u is None else np.ascontiguousarray(u, dtype=np.float64)
        self._check(self._lib.jfem_set_state(self._h, _ptr(u, _f64p)))

    # -- operators -------------------------------------------------------------
    def assemble_csc(self, index_base: int = 0, want_f: bool = True):
        nnz = C.c_int64(0)
        self._check(self._lib.jfem_assemble_csc(self._h, index_base, C.byref(nnz), None, None, None, None))
        n = 3 * self.n_nodes
        colptr = np.empty(n + 1, np.int64)
        rowval = np.empty(nnz.value, np.int64)
        nzval = np.empty(nnz.value, np.float64)
        f = np.empty(n, np.float64) if want_f else None
        self._check(self._lib.jfem_assemble_csc(self._h, index_base, C.byref(nnz), _ptr(colptr, _i64p),
                                                _ptr(rowval, _i64p), _ptr(nzval, _f64p), _ptr(f, _f64p)))
        return colptr, rowval, nzval, f

    def apply(self, v, fp32: bool = False, masked: bool = False):
        v = np.ascontiguousarray(v, dtype=np.float64)
        y = np.empty_like(v)
        flags = (APPLY_FP32 if fp32 else 0) | (APPLY_MASKED if masked else 0)
        self._check(self._lib.jfem_apply(self._h, _ptr(v, _f64p), _ptr(y, _f64p), flags))
        return y

    def apply_device(self, v_ptr: int, y_ptr: int, fp32: bool = True, masked: bool = False):
        flags = (APPLY_FP32 if fp32 else 0) | (APPLY_MASKED if masked else 0)
        self._check(self._lib.jfem_apply_device(self._h, C.c_void_p(v_ptr), C.c_void_p(y_ptr), flags))

    def internal_force(self):
        f = np.empty(3 * self.n_nodes)
        self._check(self._lib.jfem_internal_force(self._h, _ptr(f, _f64p)))
        return f

    def solve(self, opts: SolveOpts | None = None, **kw):
        o = opts if opts is not None else default_opts(**kw)
        u = np.empty(3 * self.n_nodes)
        st = Stats()
        rc = self._check(self._lib.jfem_solve(self._h, C.byref(o), _ptr(u, _f64p), C.byref(st)))
        return u, st, rc

    def solve_device(self, u_ptr: int, opts: SolveOpts | None = None, **kw):
        o = opts if opts is not None else default_opts(**kw)
        st = Stats()
        rc = self._check(self._lib.jfem_solve_device(self._h, C.byref(o), C.c_void_p(u_ptr), C.byref(st)))
        return st, rc

    @property
    def kernel_launches(self) -> int:
        return int(self._lib.jfem_kernel_launches(self._h))

    @property
    def last_apply_ms(self) -> float:
        return float(self._lib.jfem_last_apply_ms(self._h))

    @property
    def stream(self) -> int:
        return int(self._lib.jfem_stream(self._h) or 0)

    def recover_field(self, u, field: int = 1, tol: float = 1e-12, max_iter: int = 10000):
        """Nodal strain (field 0) or stress (field 1) by the least-squares fit:
        array [n_nodes, 6] (11, 22, 33, 12, 23, 13)."""
        u = np.ascontiguousarray(u, dtype=np.float64)
        out = np.empty((self.n_nodes, 6))
        it = C.c_int(0)
        self._check(self._lib.jfem_recover_field(self._h, _ptr(u, _f64p), int(field), float(tol), int(max_iter),
                                                 _ptr(out, _f64p), C.byref(it)))
        return out

    # -- learned preconditioner ---------------------------------------------------
    def mpnn_init(self, seed: int = 0):
        self._check(self._lib.jfem_mpnn_init(self._h, int(seed)))

    def mpnn_set_weights(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        if w.size != MPNN_PARAMS:
            raise ValueError(f"expected {MPNN_PARAMS} weights, got {w.size}")
        self._check(self._lib.jfem_mpnn_set_weights(self._h, _ptr(w, _f32p)))

    def mpnn_get_weights(self):
        w = np.empty(MPNN_PARAMS, np.float32)
        self._check(self._lib.jfem_mpnn_get_weights(self._h, _ptr(w, _f32p)))
        return w

    def mpnn_collect(self, max_pairs: int = 6, tol: float = 1e-10) -> int:
        """Solve the current system and keep (residual, error) pairs from its iterates."""
        return self._check(self._lib.jfem_mpnn_collect(self._h, int(max_pairs), float(tol)))

    def mpnn_clear(self):
        self._check(self._lib.jfem_mpnn_clear(self._h))

    def mpnn_train(self, epochs: int, batch: int = 32, lr: float = 1e-3, seed: int = 0):
        losses = np.zeros(epochs)
        self._check(self._lib.jfem_mpnn_train(self._h, int(epochs), int(batch), float(lr), int(seed),
                                              _ptr(losses, _f64p)))
        return losses

    def mpnn_loss_grad(self, r, e):
        r = np.ascontiguousarray(r, dtype=np.float64)
        e = np.ascontiguousarray(e, dtype=np.float64)
        L = C.c_double(0)
        g = np.empty(MPNN_PARAMS, np.float32)
        self._check(self._lib.jfem_mpnn_loss_grad(self._h, _ptr(r, _f64p), _ptr(e, _f64p), C.byref(L),
                                                  _ptr(g, _f32p)))
        return L.value, g

    def mpnn_precondition(self, r):
        r = np.ascontiguousarray(r, dtype=np.float64)
        z = np.empty_like(r)
        self._check(self._lib.jfem_mpnn_precondition(self._h, _ptr(r, _f64p), _ptr(z, _f64p)))
        return z

    # -- two-level preconditioner ------------------------------------------------
    def set_coarse_space(self, coarse_dofs: int = -1):
        """0: no coarse space; < 0: automatic size; > 0: about that many coarse DOFs."""
        self._check(self._lib.jfem_set_coarse_space(self._h, int(coarse_dofs)))

    def coarse_info(self):
        """(aggregates, coarse DOFs, elements evaluated for A_c, set-up ms)."""
        a, n, ms = C.c_int(0), C.c_int(0), C.c_double(0)
        e = C.c_int64(0)
        self._check(self._lib.jfem_coarse_info(self._h, C.byref(a), C.byref(n), C.byref(e), C.byref(ms)))
        return a.value, n.value, e.value, ms.value

    def coarse_matrix(self):
        """(A_c [nc, nc], aggregate of each node)."""
        _, nc, _, _ = self.coarse_info()
        Ac = np.empty((nc, nc))
        agg = np.empty(self.n_nodes, dtype=np.int32)
        self._check(self._lib.jfem_coarse_matrix(self._h, _ptr(Ac, _f64p), agg.ctypes.data_as(C.POINTER(C.c_int))))
        return Ac, agg

    def coarse_precondition(self, r):
        r = np.ascontiguousarray(r, dtype=np.float64)
        z = np.empty_like(r)
        self._check(self._lib.jfem_coarse_precondition(self._h, _ptr(r, _f64p), _ptr(z, _f64p)))
        return z

    def time_apply(self, reps: int = 20, fp32: bool = True, masked: bool = True):
        """Mean CUDA-event ms of (element kernel, gather kernel) of one apply."""
        a, b = C.c_double(0), C.c_double(0)
        flags = (APPLY_FP32 if fp32 else 0) | (APPLY_MASKED if masked else 0)
        self._check(self._lib.jfem_time_apply(self._h, flags, int(reps), C.byref(a), C.byref(b)))
        return a.value, b.value

    def time_assembly(self, reps: int = 3):
        """Mean CUDA-event ms of (integration-point kernel, CSC scatter kernel) of
        the FP64 assembly of K's values and f_int, and K's stored entry count."""
        a, b, n = C.c_double(0), C.c_double(0), C.c_int64(0)
        self._check(self._lib.jfem_time_assembly(self._h, int(reps), C.byref(a), C.byref(b), C.byref(n)))
        return a.value, b.value, n.value


class Batch:
    """Many small independent Tet4 solves in one persistent launch (jfem_batch_*)."""

    def __init__(self, device: int = 0):
        self._lib = load()
        h = C.c_void_p()
        rc = self._lib.jfem_batch_create(C.byref(h), int(device))
        if rc != 0:
            raise JFEMError(rc, "jfem_batch_create failed (no usable CUDA device?)")
        self._h = h
        self.node_counts = []

    def close(self):
        if getattr(self, "_h", None):
            self._lib.jfem_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc: int) -> int:
        if rc < 0:
            raise JFEMError(rc, self._lib.jfem_batch_last_error(self._h).decode())
        return rc

    def add(self, X, conn, E: float, nu: float, fixed_dofs, face_conn, t, index_base: int = 0) -> int:
        X = np.ascontiguousarray(X, dtype=np.float64).reshape(-1, 3)
        conn = np.ascontiguousarray(conn, dtype=np.int64).reshape(-1, 4)
        fd = np.ascontiguousarray(fixed_dofs, dtype=np.int64)
        fc = np.ascontiguousarray(face_conn, dtype=np.int64).reshape(-1, 3)
        t = np.ascontiguousarray(np.broadcast_to(np.asarray(t, dtype=np.float64), (fc.shape[0], 3)))
        k = self._check(self._lib.jfem_batch_add(self._h, X.shape[0], _ptr(X, _f64p), conn.shape[0], _ptr(conn, _i64p),
                                                 index_base, float(E), float(nu), fd.size, _ptr(fd, _i64p),
                                                 fc.shape[0], _ptr(fc, _i64p), _ptr(t, _f64p)))
        self.node_counts.append(X.shape[0])
        return k

    def add_workload(self, w) -> int:
        return self.add(w.mesh.X, w.mesh.conn, w.E, w.nu, w.fixed_dofs, w.faces, w.traction)

    def solve(self, tol: float = 1e-8, max_iter: int = 100000, block_size: int = 0):
        """Returns (list of u per instance, iterations, status, residual, latency_s, solve_s)."""
        n = len(self.node_counts)
        tot = 3 * sum(self.node_counts)
        u = np.empty(tot)
        it = np.empty(n, np.int32)
        stv = np.empty(n, np.int32)
        res = np.empty(n)
        lat = np.empty(n)
        t = C.c_double(0)
        self._check(self._lib.jfem_batch_solve(self._h, float(tol), int(max_iter), int(block_size), _ptr(u, _f64p),
                                               it.ctypes.data_as(C.POINTER(C.c_int)),
                                               stv.ctypes.data_as(C.POINTER(C.c_int)), _ptr(res, _f64p),
                                               _ptr(lat, _f64p), C.byref(t)))
        offs = np.concatenate([[0], np.cumsum(3 * np.asarray(self.node_counts))])
        us = [u[offs[k]:offs[k + 1]] for k in range(n)]
        return us, it, stv, res, lat, t.value

    @property
    def tune_source(self) -> int:
        """0 none yet, 1 autotuned by this object, 2 taken from the autotuner cache."""
        return int(self._lib.jfem_batch_tune_source(self._h))

    def config(self):
        bs, g = C.c_int(0), C.c_int(0)
        self._check(self._lib.jfem_batch_config(self._h, C.byref(bs), C.byref(g)))
        return bs.value, g.value

    def set_config(self, block_size: int, cluster_size: int = 1, n_clustered: int = 0, cluster_block: int = 0):
        """Fix the launch configuration used by solve(block_size=0); block_size 0
        returns to the autotuner."""
        self._check(self._lib.jfem_batch_set_config(self._h, int(block_size), int(cluster_size), int(n_clustered),
                                                     int(cluster_block)))

    def cluster_config(self):
        """(cluster size, number of instances solved on clusters, their block size)."""
        cs, nl, bc = C.c_int(0), C.c_int(0), C.c_int(0)
        self._check(self._lib.jfem_batch_cluster_config(self._h, C.byref(cs), C.byref(nl), C.byref(bc)))
        return cs.value, nl.value, bc.value


def rcm(conn, n_nodes: int, start: int = 0, index_base: int = 0):
    """Reverse Cuthill–McKee order of the node graph (jfem_rcm): returns
    (perm, bandwidth_before, bandwidth_after); perm[k] = old node at position k."""
    conn = np.ascontiguousarray(conn, dtype=np.int64)
    nen = conn.shape[1] if conn.ndim == 2 else 1
    perm = np.empty(n_nodes, np.int64)
    b0, b1 = C.c_int64(0), C.c_int64(0)
    rc = load().jfem_rcm(int(n_nodes), conn.shape[0], nen, _ptr(conn, _i64p), index_base, int(start),
                         _ptr(perm, _i64p), C.byref(b0), C.byref(b1))
    if rc != 0:
        raise JFEMError(rc, "jfem_rcm")
    return perm, b0.value, b1.value
