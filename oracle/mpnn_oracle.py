"""numpy restatement of the learned preconditioner (FP64).

TEST INFRASTRUCTURE ONLY: the checker for the GPU forward, adjoint and
gradient kernels of juliafem.jl_gb300/csrc/jfem_mpnn.cu.  The reference has no
learned preconditioner (it is new in this build), so this file defines the
semantics the CUDA kernels must reproduce; it is pinned by finite differences
and by symmetry checks (tests/test_mpnn_oracle.py), not by reference golden
vectors.

Network N (node graph of the mesh: i ~ j when nodes i ≠ j share an element),
linear message passing, 3 layers of width 32, no biases:

    agg(h)_i = (1/deg_i) Σ_{j ~ i} h_j
    h1 = y  W1sᵀ + agg(y)  W1nᵀ              y: [N, 3] → h1: [N, 32]
    h2 = h1 W2sᵀ + agg(h1) W2nᵀ
    h3 = h2 W3sᵀ + agg(h2) W3nᵀ
    N(y) = mask ⊙ (h3 Woᵀ)                   → [N, 3]

Weights are BF16 values (the flat layout of PARAM_SHAPES, row-major [out][in]).
Nᵀ is the adjoint of N (its backward-data pass).

Preconditioner (symmetric positive definite for any weights):

    y = mask ⊙ D^{-1/2} r,   z = D^{-1/2} (y + Nᵀ N y)

Jacobi plus a learned positive semi-definite correction, so flexible CG keeps
the convergence of PCG.  Training pairs (r, e) with r = K e, scaled by s (RMS
of D^{-1/2} r over the free DOFs): y = mask ⊙ D^{-1/2} r / s, t = mask ⊙ e / s,
r̃ = r / s = D^{1/2} y.  Loss per pair:

    ℓ = 1 − (zᵀ r̃)² / ((zᵀ K z)(tᵀ r̃)) = 1 − cos²_K(z, t),

the fraction of the energy norm of the error left after one optimally scaled
step along z.
"""
from __future__ import annotations

import numpy as np

WIDTH = 32
PARAM_SHAPES = [("W1s", (WIDTH, 3)), ("W1n", (WIDTH, 3)),
                ("W2s", (WIDTH, WIDTH)), ("W2n", (WIDTH, WIDTH)),
                ("W3s", (WIDTH, WIDTH)), ("W3n", (WIDTH, WIDTH)),
                ("Wo", (3, WIDTH))]
N_PARAMS = sum(a * b for _, (a, b) in PARAM_SHAPES)


def bf16_round(w: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    a = np.ascontiguousarray(w, dtype=np.float32).view(np.uint32).astype(np.uint64)
    lsb = (a >> 16) & 1
    a = (a + 0x7FFF + lsb) & 0xFFFF0000
    return a.astype(np.uint32).view(np.float32)


def unpack(flat: np.ndarray) -> dict:
    out, k = {}, 0
    for name, (a, b) in PARAM_SHAPES:
        out[name] = np.asarray(flat[k:k + a * b], dtype=np.float64).reshape(a, b)
        k += a * b
    return out


def pack(d: dict) -> np.ndarray:
    return np.concatenate([d[name].reshape(-1) for name, _ in PARAM_SHAPES])


def node_graph(nb_ptr: np.ndarray, nbr: np.ndarray):
    """Neighbour lists without the node itself: (ptr, neighbour, row) arrays."""
    n = nb_ptr.size - 1
    rows = np.repeat(np.arange(n), np.diff(nb_ptr))
    keep = nbr != rows
    ptr = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(np.bincount(rows[keep], minlength=n), out=ptr[1:])
    return ptr, nbr[keep].astype(np.int64), rows[keep]


def _inv_deg(ptr):
    deg = np.diff(ptr).astype(np.float64)
    return np.where(deg > 0, 1.0 / np.maximum(deg, 1.0), 0.0)


def _agg(h, graph):
    ptr, idx, rows = graph
    s = np.zeros_like(h)
    np.add.at(s, rows, h[idx])
    return s * _inv_deg(ptr)[:, None]


def _agg_t(g, graph):
    """Transpose of _agg: (aggᵀ g)_j = Σ_{i ~ j} g_i / deg_i."""
    ptr, idx, rows = graph
    gi = g * _inv_deg(ptr)[:, None]
    s = np.zeros_like(g)
    np.add.at(s, idx, gi[rows])
    return s


def forward(params, y, graph, mask3):
    """N(y) and the per-layer (input, aggregate) pairs."""
    W = unpack(params)
    cache = []
    h = y
    for l in (1, 2, 3):
        a = _agg(h, graph)
        cache.append((h, a))
        h = h @ W[f"W{l}s"].T + a @ W[f"W{l}n"].T
    cache.append((h, None))
    return (h @ W["Wo"].T) * mask3, cache


def adjoint(params, u, graph, mask3):
    """Nᵀ u."""
    W = unpack(params)
    g = (u * mask3) @ W["Wo"]
    for l in (3, 2, 1):
        g = g @ W[f"W{l}s"] + _agg_t(g @ W[f"W{l}n"], graph)
    return g


def weight_grad(params, cache, dout, graph, mask3):
    """∂⟨dout, N(y)⟩/∂W for the activations of one forward pass."""
    W = unpack(params)
    g = {}
    dout = dout * mask3
    g["Wo"] = dout.T @ cache[3][0]
    dh = dout @ W["Wo"]
    for l in (3, 2, 1):
        h, a = cache[l - 1]
        g[f"W{l}s"] = dh.T @ h
        g[f"W{l}n"] = dh.T @ a
        if l > 1:
            dh = dh @ W[f"W{l}s"] + _agg_t(dh @ W[f"W{l}n"], graph)
    return g


def apply_scaled(params, y, sq, graph, mask3):
    """z = (y + NᵀN y) / sq (scaled units; sq = D^{1/2})."""
    u, _ = forward(params, y, graph, mask3)
    v = adjoint(params, u, graph, mask3)
    return (y + v) * mask3 / np.where(sq > 0, sq, 1.0)


def loss(params, y, t, sq, graph, mask3, kmul, c=None):
    """kmul(v [N,3]) → K v with prescribed rows and columns removed.  c (same
    shape as y, may be None): a term added to z that does not depend on the
    weights — the coarse correction P A_c⁻¹ Pᵀ r̃ of the two-level
    preconditioner, in the same scaled units."""
    z = apply_scaled(params, y, sq, graph, mask3)
    if c is not None:
        z = z + c * mask3
    rt = sq * y
    a = float(np.sum(z * rt))
    q = float(np.sum(z * kmul(z)))
    return 1.0 - a * a / (q * float(np.sum(t * rt)))


def loss_and_grad(params, y, t, sq, graph, mask3, kmul, c=None):
    """Loss and its gradient with respect to the (BF16-valued) parameters; c as
    in loss() (it shifts z, so ∂ℓ/∂z changes through a, q and Kz, while
    ∂z/∂(NᵀN y) = D^{-1/2} stays as without it)."""
    u, cache_y = forward(params, y, graph, mask3)
    v = adjoint(params, u, graph, mask3)
    isq = np.where(sq > 0, 1.0 / np.where(sq > 0, sq, 1.0), 0.0)
    z = (y + v) * mask3 * isq
    if c is not None:
        z = z + c * mask3
    rt = sq * y
    kz = kmul(z)
    a = float(np.sum(z * rt))
    q = float(np.sum(z * kz))
    den = float(np.sum(t * rt))
    L = 1.0 - a * a / (q * den)
    gz = (-2.0 * a / (q * den) * rt + 2.0 * a * a / (q * q * den) * kz) * mask3
    gh = gz * isq                                   # ∂ℓ/∂(NᵀN y) = D^{-1/2} ∂ℓ/∂z
    w, cache_g = forward(params, gh, graph, mask3)  # N ĝ
    g1 = weight_grad(params, cache_y, w, graph, mask3)   # ⟨N ĝ, dN y⟩
    g2 = weight_grad(params, cache_g, u, graph, mask3)   # ⟨dN ĝ, N y⟩
    return L, pack({k: g1[k] + g2[k] for k in g1})


def init_params(seed: int) -> np.ndarray:
    """Glorot-uniform weights scaled by 0.5 (the untrained correction is small
    beside Jacobi); BF16-rounded."""
    g = np.random.Generator(np.random.Philox(key=int(seed)))
    parts = []
    for name, (a, b) in PARAM_SHAPES:
        lim = 0.5 * np.sqrt(6.0 / (a + b))
        parts.append(g.uniform(-lim, lim, size=a * b))
    return bf16_round(np.concatenate(parts).astype(np.float32)).astype(np.float64)


def precondition(params, r, dinv, graph, mask3):
    """z = D^{-1/2}(y + NᵀN y), y = mask ⊙ D^{-1/2} r (flat in, flat out)."""
    r = np.asarray(r, dtype=np.float64).reshape(-1, 3)
    isq = np.sqrt(np.asarray(dinv, dtype=np.float64).reshape(-1, 3)) * mask3
    y = isq * r
    u, _ = forward(params, y, graph, mask3)
    v = adjoint(params, u, graph, mask3)
    return (isq * (y + v)).reshape(-1)
