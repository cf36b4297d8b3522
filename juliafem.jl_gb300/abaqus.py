"""Abaqus ``.inp`` mesh reader (volume meshes, node/element sets, element surfaces).

Behaviour of the reference reader src/readers/parse_mesh.jl (keywords *NODE,
*ELEMENT TYPE=…, *NSET / *ELSET with optional GENERATE, *SURFACE TYPE=ELEMENT)
and the side tables of src/readers/create_surface_elements.jl:10-27 (sides
ordered so that ∂X/∂ξ₁ × ∂X/∂ξ₂ points out of the element).  Also reads the
*ELASTIC constants, *BOUNDARY (set, first[, last[, value]]) and *DSLOAD
(surface, P, value) records of a single static step.

Node and element ids stay the file's 1-based ids; ``to_arrays`` renumbers them
densely (0-based) for the C ABI.
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field

import numpy as np

ELEMENT_TYPES = {   # parse_mesh.jl:8-35
    "C3D4": "Tet4", "C3D4H": "Tet4", "C3D10": "Tet10", "C3D10H": "Tet10",
    "C3D8": "Hex8", "C3D8R": "Hex8",
}
NODES_PER = {"Tet4": 4, "Tet10": 10, "Hex8": 8}

# element side → (surface element, local node list, 1-based)
SIDES = {
    "Tet4": {"S1": ("Tri3", [1, 3, 2]), "S2": ("Tri3", [1, 2, 4]), "S3": ("Tri3", [2, 3, 4]),
             "S4": ("Tri3", [1, 4, 3])},
    "Tet10": {"S1": ("Tri6", [1, 3, 2, 7, 6, 5]), "S2": ("Tri6", [1, 2, 4, 5, 9, 8]),
              "S3": ("Tri6", [2, 3, 4, 6, 10, 9]), "S4": ("Tri6", [1, 4, 3, 8, 10, 7])},
    "Hex8": {"S1": ("Quad4", [1, 2, 3, 4]), "S2": ("Quad4", [5, 8, 7, 6]), "S3": ("Quad4", [1, 5, 6, 2]),
             "S4": ("Quad4", [2, 6, 7, 3]), "S5": ("Quad4", [3, 7, 8, 4]), "S6": ("Quad4", [4, 8, 5, 1])},
}


@dataclass
class AbaqusMesh:
    nodes: dict = field(default_factory=dict)            # id → (x, y, z)
    elements: dict = field(default_factory=dict)         # id → (type, [node ids])
    node_sets: dict = field(default_factory=dict)        # name → [ids]
    element_sets: dict = field(default_factory=dict)     # name → [ids]
    surface_sets: dict = field(default_factory=dict)     # name → [(elem id, side)]
    elastic: tuple | None = None                          # (E, nu)
    boundary: list = field(default_factory=list)         # (set or node, first, last, value)
    dsload: list = field(default_factory=list)           # (surface, 'P', value)

    def surface_elements(self, name: str):
        """[(face type, [node ids])] of a surface (create_surface_elements.jl)."""
        out = []
        for eid, side in self.surface_sets[name]:
            et, conn = self.elements[eid]
            ft, loc = SIDES[et][side]
            out.append((ft, [conn[i - 1] for i in loc]))
        return out

    def to_arrays(self):
        """(element type, X (N,3), conn (E, n_en) 0-based, node ids, element ids)."""
        ids = sorted(self.nodes)
        index = {n: i for i, n in enumerate(ids)}
        X = np.array([self.nodes[n] for n in ids], dtype=np.float64)
        eids = sorted(self.elements)
        types = {self.elements[e][0] for e in eids}
        if len(types) != 1:
            raise ValueError(f"one volume element type expected, found {sorted(types)}")
        conn = np.array([[index[n] for n in self.elements[e][1]] for e in eids], dtype=np.int64)
        return types.pop(), X, conn, index, eids


def _opts(line: str) -> dict:
    parts = [p.strip() for p in line.split(",")]
    out = {"_kw": parts[0].upper()}
    for p in parts[1:]:
        if "=" in p:
            k, v = p.split("=", 1)
            out[k.strip().upper()] = v.strip()
        elif p:
            out[p.upper()] = True
    return out


def _nums(line: str):
    return [t for t in (s.strip() for s in line.split(",")) if t]


def read(path_or_text: str) -> AbaqusMesh:
    text = path_or_text
    if "\n" not in path_or_text and not path_or_text.lstrip().startswith("*"):
        with open(path_or_text) as fh:
            text = fh.read()
    m = AbaqusMesh()
    kw = None
    opts: dict = {}
    pending_elem: list = []
    for raw in text.splitlines():
        line = raw.strip()
        if not line or line.startswith("**"):
            continue
        if line.startswith("*"):
            opts = _opts(line)
            kw = opts["_kw"]
            pending_elem = []
            if kw == "*ELEMENT":
                etype = opts.get("TYPE", "").upper()
                if etype not in ELEMENT_TYPES:
                    raise ValueError(f"unsupported element type {etype}")
            continue
        vals = _nums(line)
        if kw == "*NODE":
            nid = int(vals[0])
            m.nodes[nid] = tuple(float(v) for v in vals[1:4])
            if "NSET" in opts:
                m.node_sets.setdefault(opts["NSET"], []).append(nid)
        elif kw == "*ELEMENT":
            et = ELEMENT_TYPES[opts["TYPE"].upper()]
            pending_elem.extend(int(v) for v in vals)
            need = NODES_PER[et] + 1
            if len(pending_elem) >= need:
                eid = pending_elem[0]
                m.elements[eid] = (et, pending_elem[1:need])
                if "ELSET" in opts:
                    m.element_sets.setdefault(opts["ELSET"], []).append(eid)
                pending_elem = []
        elif kw in ("*NSET", "*ELSET"):
            target = m.node_sets if kw == "*NSET" else m.element_sets
            name = opts.get("NSET" if kw == "*NSET" else "ELSET")
            ids = target.setdefault(name, [])
            if opts.get("GENERATE"):
                a, b = int(vals[0]), int(vals[1])
                step = int(vals[2]) if len(vals) > 2 else 1
                ids.extend(range(a, b + 1, step))
            else:
                for v in vals:
                    if re.fullmatch(r"-?\d+", v):
                        ids.append(int(v))
                    else:
                        ids.extend(target.get(v, []))
        elif kw == "*SURFACE":
            name = opts.get("NAME")
            lst = m.surface_sets.setdefault(name, [])
            ref, side = vals[0], vals[1].upper()
            if re.fullmatch(r"\d+", ref):
                lst.append((int(ref), side))
            else:
                lst.extend((e, side) for e in m.element_sets.get(ref, []))
        elif kw == "*ELASTIC":
            m.elastic = (float(vals[0]), float(vals[1]))
        elif kw == "*BOUNDARY":
            first = int(vals[1])
            last = int(vals[2]) if len(vals) > 2 and vals[2] else first
            value = float(vals[3]) if len(vals) > 3 else 0.0
            m.boundary.append((vals[0], first, last, value))
        elif kw == "*DSLOAD":
            m.dsload.append((vals[0], vals[1].upper(), float(vals[2])))
    return m


def boundary_dofs(mesh: AbaqusMesh, index: dict):
    """0-based interleaved DOFs and values of the *BOUNDARY records."""
    dofs, vals = {}, {}
    for target, first, last, value in mesh.boundary:
        nodes = mesh.node_sets.get(target)
        if nodes is None:
            nodes = [int(target)]
        for n in nodes:
            for comp in range(first, last + 1):
                d = 3 * index[n] + comp - 1
                dofs[d] = True
                vals[d] = value
    d = np.array(sorted(dofs), dtype=np.int64)
    return d, np.array([vals[k] for k in d], dtype=np.float64)
