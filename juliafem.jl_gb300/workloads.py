"""Synthetic workloads of the elasticity hot path (seeded, reproducible).

* ``cantilever`` — box [0,L]×[0,W]×[0,H], x = 0 face clamped, uniform traction
  on the x = L face (the linear-elastic cantilever configurations: Tet4
  40×4×4 cubes on [0,10]×[0,1]², Tet10 200×20×20 on [0,20]×[0,2]²);
* ``cube_compression`` — Hex8 Neo-Hookean unit cube, bottom clamped, top face
  z-displacement prescribed, per-element lognormal E (seeded);
* ``batch_instances`` — many uneven Tet4 cantilevers with random E, ν and end
  tractions.

Random numbers come from numpy's Philox bit generator with a global seed and a
per-item offset, so inputs are identical on every machine.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import mesh as _mesh

SEED = 20261203


def rng(item: int = 0) -> np.random.Generator:
    return np.random.Generator(np.random.Philox(key=SEED + int(item)))


@dataclass
class Workload:
    name: str
    mesh: _mesh.BoxMesh
    E: np.ndarray | float
    nu: np.ndarray | float
    fixed_dofs: np.ndarray
    fixed_values: np.ndarray
    face_type: int = 0
    faces: np.ndarray | None = None
    traction: np.ndarray | None = None
    model: int = 0                    # 0 linear elastic, 1 Neo-Hookean
    finite: bool = False
    n_load_steps: int = 1
    extra: dict = field(default_factory=dict)

    @property
    def n_dofs(self) -> int:
        return self.mesh.n_dofs

    def fixed_mask(self) -> np.ndarray:
        m = np.zeros(self.n_dofs, dtype=np.uint8)
        m[self.fixed_dofs] = 1
        return m

    def prescribed(self) -> np.ndarray:
        g = np.zeros(self.n_dofs)
        g[self.fixed_dofs] = self.fixed_values
        return g


def cantilever(elem_type: int, nx: int, ny: int, nz: int, L: float, W: float, H: float,
               E=210e3, nu=0.3, traction=(0.0, 0.0, -1.0), name: str = "cantilever") -> Workload:
    m = _mesh.box_mesh(elem_type, nx, ny, nz, L, W, H)
    clamp = m.nodes_where(0, 0.0)
    dofs = _mesh.clamp_dofs(clamp)
    ft, faces = m.face(0, 1)
    t = np.broadcast_to(np.asarray(traction, dtype=np.float64), (faces.shape[0], 3)).copy()
    return Workload(name, m, E, nu, dofs, np.zeros(dofs.size), ft, faces, t)


def cfg_tet4_cantilever() -> Workload:
    """Tet4 40×4×4 cubes on [0,10]×[0,1]²: 3,840 elements, 1,025 nodes, 3,075 DOFs."""
    return cantilever(_mesh.TET4, 40, 4, 4, 10.0, 1.0, 1.0, name="tet4_cantilever_40x4x4")


def cfg_tet10_cantilever(nx: int = 200, ny: int = 20, nz: int = 20) -> Workload:
    """Tet10 cantilever on [0,20]×[0,2]² (200×20×20 cubes: 480,000 elements,
    674,081 nodes, 2,022,243 DOFs); smaller nx,ny,nz keep the aspect."""
    return cantilever(_mesh.TET10, nx, ny, nz, 20.0 * nx / 200, 2.0 * ny / 20, 2.0 * nz / 20,
                      name=f"tet10_cantilever_{nx}x{ny}x{nz}")


def cube_compression(n: int = 128, steps: int = 10, top_uz: float = -0.1, sigma_log: float = 0.2,
                     nu: float = 0.3, E_median: float = 210e3) -> Workload:
    """Hex8 Neo-Hookean unit cube: bottom clamped, top u_z ramped to top_uz."""
    m = _mesh.box_mesh(_mesh.HEX8, n, n, n, 1.0, 1.0, 1.0)
    z = rng(3).standard_normal(m.n_elem)
    E = E_median * np.exp(sigma_log * z)
    bottom = m.nodes_where(2, 0.0)
    top = m.nodes_where(2, 1.0)
    d_b = _mesh.clamp_dofs(bottom)
    d_t = 3 * top + 2
    dofs = np.concatenate([d_b, d_t])
    vals = np.concatenate([np.zeros(d_b.size), np.full(d_t.size, top_uz)])
    order = np.argsort(dofs)
    return Workload(f"hex8_neohookean_{n}^3", m, E, nu, dofs[order], vals[order], model=1, finite=True,
                    n_load_steps=steps)


def batch_instances(count: int = 256, nmin: int = 8, nmax: int = 32, seed_item: int = 5):
    """Uneven Tet4 cantilevers: n ~ U{nmin..nmax} cubes along x (length 4), n/4
    (rounded, ≥ 2) across; E ~ U[50e3, 300e3], ν ~ U[0.2, 0.45]; random end traction."""
    g = rng(seed_item)
    out = []
    for i in range(count):
        n = int(g.integers(nmin, nmax + 1))
        k = max(2, int(round(n / 4)))
        E = float(g.uniform(50e3, 300e3))
        nu = float(g.uniform(0.2, 0.45))
        t = g.standard_normal(3)
        w = cantilever(_mesh.TET4, n, k, k, 4.0, 1.0, 1.0, E=E, nu=nu, traction=t, name=f"batch_{i}")
        out.append(w)
    return out


def learned_family(count: int, seed_item: int = 40, nx: int = 40, ny: int = 4, nz: int = 4,
                   L: float = 10.0, W: float = 1.0, H: float = 1.0, sigma_log: float = 0.5,
                   patches: int = 2, elem_type: int = _mesh.TET10):
    """Training / evaluation systems of the learned preconditioner: the Tet10
    cantilever on [0,10]×[0,1]² (40×4×4 cubes, the geometry of the Tet4
    parity case) with per-element E = 210e3·exp(σ z), z ~ N(0,1) (σ = 0.5),
    ν = 0.3, x = 0 clamped, and `patches` tractions with components N(0,1) on
    random rectangular patches of the five unclamped faces.  Item k of a family
    draws from the generator of seed_item + k, so a family of unseen systems is
    a disjoint seed range."""
    m = _mesh.box_mesh(elem_type, nx, ny, nz, L, W, H)
    clamp = m.nodes_where(0, 0.0)
    dofs = _mesh.clamp_dofs(clamp)
    sides = [(0, 1), (1, 0), (1, 1), (2, 0), (2, 1)]
    face_sets = []
    for axis, side in sides:
        ft, faces = m.face(axis, side)
        face_sets.append((axis, ft, faces, m.X[faces].mean(axis=1)))
    out = []
    for k in range(count):
        g = rng(seed_item + k)
        E = 210e3 * np.exp(sigma_log * g.standard_normal(m.n_elem))
        sel_faces, sel_t = [], []
        for _ in range(patches):
            axis, ft, faces, cen = face_sets[int(g.integers(len(face_sets)))]
            u_ax, v_ax = [d for d in range(3) if d != axis]
            lu, lv = m.size[u_ax], m.size[v_ax]
            u = np.sort(g.uniform(0.0, lu, 2))
            v = np.sort(g.uniform(0.0, lv, 2))
            inside = ((cen[:, u_ax] >= u[0]) & (cen[:, u_ax] <= u[1]) &
                      (cen[:, v_ax] >= v[0]) & (cen[:, v_ax] <= v[1]))
            if not inside.any():   # at least the face nearest the patch centre
                c = np.array([0.0, 0.0, 0.0])
                c[u_ax], c[v_ax] = u.mean(), v.mean()
                inside[np.argmin(np.sum((cen[:, [u_ax, v_ax]] - c[[u_ax, v_ax]]) ** 2, axis=1))] = True
            t = g.standard_normal(3)
            sel_faces.append(faces[inside])
            sel_t.append(np.broadcast_to(t, (int(inside.sum()), 3)))
        faces = np.concatenate(sel_faces)
        trac = np.ascontiguousarray(np.concatenate(sel_t))
        out.append(Workload(f"learned_{seed_item + k}", m, E, 0.3, dofs, np.zeros(dofs.size),
                            face_sets[0][1], faces, trac))
    return out
