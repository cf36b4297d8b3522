"""Structured box meshes for the elasticity hot path (host-side input generation).

The reference exports a structured mesh generator whose source file is missing
from its tree (src/JuliaFEM.jl:432-434 includes mesh/structured.jl, absent), so
the split is defined here:

* vertex lattice index ``i + (nx+1)*(j + (ny+1)*k)`` (0-based);
* every cube is split into 6 tetrahedra along its (0,0,0)→(1,1,1) diagonal
  (Kuhn/Freudenthal split, one tet per axis permutation, conforming across
  cubes); odd permutations swap their 2nd and 3rd vertex so that every element
  has a positive Jacobian;
* Tet10 uses the doubled lattice (2nx+1)(2ny+1)(2nz+1) (every doubled-lattice
  point is an edge, face-diagonal or body-diagonal midpoint of the split) with
  mid-edge order 5:(1-2) 6:(2-3) 7:(3-1) 8:(1-4) 9:(2-4) 10:(3-4)
  (src/topology/tetrahedra.jl:213-235, src/basis/lagrange_generated.jl:257-283);
* Hex8 node order follows src/basis/lagrange_generated.jl:285-311
  ((-1,-1,-1),(1,-1,-1),(1,1,-1),(-1,1,-1), then the same at ξ₃ = +1).

Connectivity is returned element-major ``conn[e, a]`` (0-based int64), node
coordinates as ``X[n, 3]`` float64.
"""
from __future__ import annotations

import itertools
from dataclasses import dataclass, field

import numpy as np

TET4, TET10, HEX8 = 4, 10, 8
TRI3, TRI6, QUAD4 = 3, 6, 4

_PERMS = list(itertools.permutations((0, 1, 2)))


@dataclass
class BoxMesh:
    elem_type: int
    X: np.ndarray            # (N, 3) float64
    conn: np.ndarray         # (E, n_en) int64, 0-based
    shape: tuple             # (nx, ny, nz) cubes
    size: tuple              # (Lx, Ly, Lz)
    lattice: tuple           # node lattice dims (mx, my, mz)
    faces: dict = field(default_factory=dict)

    @property
    def n_nodes(self) -> int:
        return int(self.X.shape[0])

    @property
    def n_elem(self) -> int:
        return int(self.conn.shape[0])

    @property
    def n_dofs(self) -> int:
        return 3 * self.n_nodes

    def nodes_where(self, axis: int, value: float, tol: float = 1e-9) -> np.ndarray:
        return np.nonzero(np.abs(self.X[:, axis] - value) <= tol)[0].astype(np.int64)

    def face(self, axis: int, side: int):
        """Surface elements on the box face ``axis = 0 (side 0) or L (side 1)``.

        Returns ``(face_type, face_conn[n_faces, n_fn])``.
        """
        return _box_face(self, axis, side)


def _lattice_index(mx, my):
    def idx(i, j, k):
        return i + mx * (j + my * k)
    return idx


def _cube_corners(nx, ny, nz, step, mx, my):
    """Lattice index of corner (a,b,c) of every cube, shape (ncubes, 2, 2, 2)."""
    i = np.arange(nx)
    j = np.arange(ny)
    k = np.arange(nz)
    K, J, I = np.meshgrid(k, j, i, indexing="ij")   # cube index = i + nx*(j + ny*k)
    I = I.ravel() * step
    J = J.ravel() * step
    K = K.ravel() * step
    out = np.empty((I.size, 2, 2, 2), dtype=np.int64)
    for a in (0, 1):
        for b in (0, 1):
            for c in (0, 1):
                out[:, a, b, c] = (I + a * step) + mx * ((J + b * step) + my * (K + c * step))
    return out


def _kuhn_vertices():
    """Per permutation: the 4 corner offsets (a,b,c) of the tet, orientation-fixed."""
    tets = []
    for p in _PERMS:
        v0 = [0, 0, 0]
        v1 = list(v0); v1[p[0]] = 1
        v2 = list(v1); v2[p[1]] = 1
        v3 = [1, 1, 1]
        parity = np.linalg.det(np.array([v1, v2, v3], dtype=float))
        if parity < 0:
            v1, v2 = v2, v1
        tets.append((tuple(v0), tuple(v1), tuple(v2), tuple(v3)))
    return tets


_TET10_EDGES = ((0, 1), (1, 2), (2, 0), (0, 3), (1, 3), (2, 3))


def box_mesh(elem_type: int, nx: int, ny: int, nz: int,
             Lx: float = 1.0, Ly: float = 1.0, Lz: float = 1.0) -> BoxMesh:
    """Structured [0,Lx]×[0,Ly]×[0,Lz] mesh of nx×ny×nz cubes."""
    if elem_type not in (TET4, TET10, HEX8):
        raise ValueError(f"unsupported element type {elem_type}")
    step = 2 if elem_type == TET10 else 1
    mx, my, mz = step * nx + 1, step * ny + 1, step * nz + 1
    kk, jj, ii = np.meshgrid(np.arange(mz), np.arange(my), np.arange(mx), indexing="ij")
    X = np.stack([ii.ravel() * (Lx / (step * nx)),
                  jj.ravel() * (Ly / (step * ny)),
                  kk.ravel() * (Lz / (step * nz))], axis=1).astype(np.float64)
    corners = _cube_corners(nx, ny, nz, step, mx, my)
    nc = corners.shape[0]
    if elem_type == HEX8:
        order = ((0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0),
                 (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1))
        conn = np.stack([corners[:, a, b, c] for (a, b, c) in order], axis=1)
    else:
        tets = _kuhn_vertices()
        conn4 = np.empty((nc, 6, 4), dtype=np.int64)
        for t, verts in enumerate(tets):
            for a, (p, q, r) in enumerate(verts):
                conn4[:, t, a] = corners[:, p, q, r]
        conn4 = conn4.reshape(nc * 6, 4)
        if elem_type == TET4:
            conn = conn4
        else:
            # midpoint of two doubled-lattice nodes is again a lattice node
            def coords(n):
                return n % mx, (n // mx) % my, n // (mx * my)
            mids = []
            for (p, q) in _TET10_EDGES:
                ip, jp, kp = coords(conn4[:, p])
                iq, jq, kq = coords(conn4[:, q])
                mids.append(((ip + iq) // 2) + mx * (((jp + jq) // 2) + my * ((kp + kq) // 2)))
            conn = np.concatenate([conn4, np.stack(mids, axis=1)], axis=1)
    return BoxMesh(elem_type, X, np.ascontiguousarray(conn, dtype=np.int64),
                   (nx, ny, nz), (Lx, Ly, Lz), (mx, my, mz))


def _box_face(mesh: BoxMesh, axis: int, side: int):
    """Boundary faces on a box side, consistent with the volume split."""
    nx, ny, nz = mesh.shape
    mx, my, _ = mesh.lattice
    step = 2 if mesh.elem_type == TET10 else 1
    n = (nx, ny, nz)
    # the two in-plane axes, in increasing order
    u_ax, v_ax = [d for d in range(3) if d != axis]
    iu, iv = np.meshgrid(np.arange(n[u_ax]), np.arange(n[v_ax]), indexing="ij")
    iu = iu.ravel()
    iv = iv.ravel()
    fixed = side * n[axis]

    def node(du, dv):
        # lattice coordinates in doubled units where needed
        c = [None, None, None]
        c[axis] = np.full(iu.shape, fixed * step)
        c[u_ax] = iu * step + du
        c[v_ax] = iv * step + dv
        return c[0] + mx * (c[1] + my * c[2])

    if mesh.elem_type == HEX8:
        quads = np.stack([node(0, 0), node(1, 0), node(1, 1), node(0, 1)], axis=1)
        return QUAD4, quads.astype(np.int64)
    s = step
    # Kuhn face diagonal runs from the (u,v) = (0,0) to (1,1) corner of each square
    # (both corners lie on the cube's main diagonal projection).
    t1 = [(0, 0), (s, 0), (s, s)]
    t2 = [(0, 0), (s, s), (0, s)]
    tris = []
    for t in (t1, t2):
        verts = [node(du, dv) for (du, dv) in t]
        if mesh.elem_type == TET4:
            tris.append(np.stack(verts, axis=1))
        else:
            mids = []
            for (p, q) in ((0, 1), (1, 2), (2, 0)):
                du = (t[p][0] + t[q][0]) // 2
                dv = (t[p][1] + t[q][1]) // 2
                mids.append(node(du, dv))
            tris.append(np.stack(verts + mids, axis=1))
    faces = np.concatenate(tris, axis=0).astype(np.int64)
    return (TRI3 if mesh.elem_type == TET4 else TRI6), faces


def clamp_dofs(nodes: np.ndarray, comps=(0, 1, 2)) -> np.ndarray:
    """Interleaved global DOFs 3*node + comp (src/assembly/problems.jl:466-478)."""
    nodes = np.asarray(nodes, dtype=np.int64)
    return np.sort(np.concatenate([3 * nodes + c for c in comps])).astype(np.int64)
