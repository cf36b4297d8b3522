"""Checkpoint and resume: learned-preconditioner weights and Newton load steps.

The reference writes results only (XDMF/HDF5, src/io.jl) and has neither; the
two files here are what a long training run or a load-stepped Newton solve
needs to stop and carry on.

Network weights (``save_network`` / ``load_network``): the JFEM_MPNN_PARAMS
values in the layout of include/jfem.h (Ws1 32×3, Wn1 32×3, Ws2, Wn2, Ws3, Wn3
32×32, Wo 3×32, row-major [out][in]) as BF16 — the precision the inference and
training kernels read — behind a JSON header::

    8 bytes   magic  b"JFEMNET\\x01"
    4 bytes   header length H, uint32 little-endian
    H bytes   header, UTF-8 JSON: format, version, dtype "bfloat16",
              byte_order "little", params, width, layers, segments
              [{name, shape}], meta (caller's dict, e.g. the training record)
    2·P bytes the weights, BF16 little-endian

Rounding to BF16 is to nearest, ties to even (the kernels' __float2bfloat16_rn),
so a loaded network gives bit-identical preconditioner output.

Newton load-step state (``save_load_step`` / ``load_load_step``): the
displacement after a completed load step, raw FP64::

    8 bytes   magic  b"JFEMSTEP"
    4 × uint32 version 1, step s (completed), steps S, reserved 0
    uint64    n (DOFs)
    8·n bytes u, float64 little-endian

``newton_load_steps`` runs the load steps of the library's Newton–Krylov
solve one call per step — step s of S applies s/S of the prescribed values and
surface loads, as jfem_solve does inside one call (src/solvers.jl:575-620) — and
writes the state after each step, so a solve that stops (time budget, process
end) resumes in a fresh context from the last completed step.
"""
from __future__ import annotations

import json
import os
import struct
from pathlib import Path

import numpy as np

from . import _abi

NET_MAGIC = b"JFEMNET\x01"
STEP_MAGIC = b"JFEMSTEP"
NET_FORMAT = "jfem-mpnn-weights"
NET_VERSION = 1
STEP_VERSION = 1
NET_SEGMENTS = [("Ws1", (32, 3)), ("Wn1", (32, 3)), ("Ws2", (32, 32)), ("Wn2", (32, 32)),
                ("Ws3", (32, 32)), ("Wn3", (32, 32)), ("Wo", (3, 32))]
assert sum(a * b for _, (a, b) in NET_SEGMENTS) == _abi.MPNN_PARAMS


# ---------------------------------------------------------------------------
# BF16
# ---------------------------------------------------------------------------
def to_bf16(w) -> np.ndarray:
    """float32 → BF16 bit patterns (uint16), round to nearest, ties to even;
    NaN stays a (quiet) NaN, ±inf stays ±inf."""
    bits = np.ascontiguousarray(w, dtype=np.float32).view(np.uint32).astype(np.uint64)
    rounded = ((bits + 0x7FFF + ((bits >> 16) & 1)) >> 16).astype(np.uint16)
    nan = np.isnan(np.ascontiguousarray(w, dtype=np.float32))
    return np.where(nan, ((bits >> 16).astype(np.uint16) | np.uint16(0x0040)), rounded).astype(np.uint16)


def from_bf16(b) -> np.ndarray:
    """BF16 bit patterns → float32 (exact)."""
    return (np.ascontiguousarray(b, dtype=np.uint16).astype(np.uint32) << 16).view(np.float32)


# ---------------------------------------------------------------------------
# network weights
# ---------------------------------------------------------------------------
def _atomic_write(path: Path, data: bytes) -> None:
    tmp = path.with_name(path.name + ".tmp")
    with open(tmp, "wb") as f:
        f.write(data)
        f.flush()
        os.fsync(f.fileno())
    os.replace(tmp, path)


def save_network(path, weights, meta: dict | None = None) -> None:
    """Write the network (JFEM_MPNN_PARAMS float values, or a Context whose
    weights are read with jfem_mpnn_get_weights) as a BF16 weight file."""
    if isinstance(weights, _abi.Context):
        weights = weights.mpnn_get_weights()
    w = np.ascontiguousarray(weights, dtype=np.float32).reshape(-1)
    if w.size != _abi.MPNN_PARAMS:
        raise ValueError(f"expected {_abi.MPNN_PARAMS} weights, got {w.size}")
    header = {"format": NET_FORMAT, "version": NET_VERSION, "dtype": "bfloat16", "byte_order": "little",
              "params": int(w.size), "width": _abi.MPNN_WIDTH, "layers": 3,
              "segments": [{"name": n, "shape": list(s)} for n, s in NET_SEGMENTS], "meta": meta or {}}
    hb = json.dumps(header, sort_keys=True).encode("utf-8")
    blob = to_bf16(w).astype("<u2").tobytes()
    _atomic_write(Path(path), NET_MAGIC + struct.pack("<I", len(hb)) + hb + blob)


def load_network(path, ctx: _abi.Context | None = None):
    """Read a weight file: (float32 weights, header).  With ctx the weights are
    also set in that context (jfem_mpnn_set_weights)."""
    data = Path(path).read_bytes()
    if len(data) < 12 or data[:8] != NET_MAGIC:
        raise ValueError(f"{path}: not a network weight file")
    (hl,) = struct.unpack_from("<I", data, 8)
    if 12 + hl > len(data):
        raise ValueError(f"{path}: truncated header")
    header = json.loads(data[12:12 + hl].decode("utf-8"))
    if header.get("format") != NET_FORMAT or header.get("version") != NET_VERSION:
        raise ValueError(f"{path}: unsupported format {header.get('format')!r} version {header.get('version')!r}")
    if header.get("dtype") != "bfloat16" or header.get("byte_order") != "little":
        raise ValueError(f"{path}: unsupported dtype or byte order")
    p = int(header.get("params", -1))
    shapes = [(s["name"], tuple(s["shape"])) for s in header.get("segments", [])]
    if p != _abi.MPNN_PARAMS or shapes != NET_SEGMENTS:
        raise ValueError(f"{path}: network of {p} parameters in another layout")
    blob = data[12 + hl:]
    if len(blob) != 2 * p:
        raise ValueError(f"{path}: {len(blob)} weight bytes, expected {2 * p}")
    w = from_bf16(np.frombuffer(blob, dtype="<u2"))
    if ctx is not None:
        ctx.mpnn_set_weights(w)
    return w, header


# ---------------------------------------------------------------------------
# Newton load steps
# ---------------------------------------------------------------------------
def save_load_step(path, u, step: int, steps: int) -> None:
    """Write the displacement after completed load step `step` of `steps`."""
    u = np.ascontiguousarray(u, dtype="<f8").reshape(-1)
    if not (0 <= step <= steps) or steps < 1:
        raise ValueError(f"load step {step} of {steps}")
    head = STEP_MAGIC + struct.pack("<4IQ", STEP_VERSION, int(step), int(steps), 0, u.size)
    _atomic_write(Path(path), head + u.tobytes())


def load_load_step(path):
    """Read a load-step file: (u, completed step, steps)."""
    data = Path(path).read_bytes()
    hs = 8 + struct.calcsize("<4IQ")
    if len(data) < hs or data[:8] != STEP_MAGIC:
        raise ValueError(f"{path}: not a load-step file")
    ver, step, steps, _, n = struct.unpack_from("<4IQ", data, 8)
    if ver != STEP_VERSION:
        raise ValueError(f"{path}: unsupported version {ver}")
    if len(data) != hs + 8 * n:
        raise ValueError(f"{path}: {len(data) - hs} state bytes, expected {8 * n}")
    if not (0 <= step <= steps) or steps < 1:
        raise ValueError(f"{path}: load step {step} of {steps}")
    return np.frombuffer(data, dtype="<f8", offset=hs).astype(np.float64), int(step), int(steps)


def newton_load_steps(ctx: _abi.Context, steps: int, fixed_dofs, fixed_values, surface=None, checkpoint=None,
                      resume: bool = False, stop_after: int | None = None, **solve_kw):
    """Newton–Krylov over `steps` load steps, one jfem_solve call per step.

    Step s sets the prescribed values to s/steps · fixed_values and, with
    ``surface = (face_type, faces, t, p)`` (t, p may be None), the surface
    loads to s/steps of t and p, then runs JFEM_NEWTON with one load step from
    the context's current state — the same iteration jfem_solve runs for step
    s inside one call.  With ``checkpoint`` the state is written after every
    step; ``resume=True`` starts from the state in that file when it exists (a
    fresh context gets it through jfem_set_state) and from step 1 when it does
    not, so a job script can always pass it.  ``stop_after`` ends the run after that
    step (for a staged run).  Other keywords are jfem_solve_opts fields
    (precision, tol, newton_tol, max_newton, max_cg_per_newton, …).

    Returns (u, info) with info: status (worst of the steps: 0 converged, 1 a
    step did not converge), steps_done, newton_iterations, cg_iterations,
    residual (last step's), per_step [(newton_iterations, cg_iterations,
    residual)]."""
    if steps < 1:
        raise ValueError("steps must be >= 1")
    dofs = np.ascontiguousarray(fixed_dofs, dtype=np.int64)
    vals = np.ascontiguousarray(np.broadcast_to(np.asarray(fixed_values, dtype=np.float64), dofs.shape))
    first = 1
    if resume and checkpoint is None:
        raise ValueError("resume needs a checkpoint file")
    if resume and Path(checkpoint).exists():
        u0, done, n_file = load_load_step(checkpoint)
        if n_file != steps:
            raise ValueError(f"checkpoint holds a run of {n_file} load steps, not {steps}")
        if u0.size != 3 * ctx.n_nodes:
            raise ValueError("checkpoint state does not match the mesh")
        ctx.set_state(u0)
        first = done + 1
    kw = dict(solve_kw)
    kw.update(method=_abi.NEWTON, n_load_steps=1)
    info = {"status": 0, "steps_done": first - 1, "newton_iterations": 0, "cg_iterations": 0, "residual": 0.0,
            "per_step": []}
    u = None
    last = steps if stop_after is None else min(steps, int(stop_after))
    for s in range(first, last + 1):
        frac = s / steps
        ctx.set_dirichlet(dofs, vals * frac)
        if surface is not None:
            ft, faces, t, p = surface
            ctx.set_surface_load(ft, faces, t=None if t is None else np.asarray(t, dtype=np.float64) * frac,
                                 p=None if p is None else np.asarray(p, dtype=np.float64) * frac)
        u, st, rc = ctx.solve(**kw)
        info["status"] = max(info["status"], int(rc))
        info["steps_done"] = s
        info["newton_iterations"] += st.newton_iterations
        info["cg_iterations"] += st.cg_iterations
        info["residual"] = st.residual
        info["per_step"].append((st.newton_iterations, st.cg_iterations, st.residual))
        if checkpoint is not None:
            save_load_step(checkpoint, u, s, steps)
    if u is None:   # nothing left to run: the checkpoint already holds the last step
        u = load_load_step(checkpoint)[0] if checkpoint is not None else np.zeros(3 * ctx.n_nodes)
    return u, info
