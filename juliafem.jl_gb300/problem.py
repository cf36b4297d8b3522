"""Host-side mirror of JuliaFEM's elasticity API over the C ABI.

Julia is not available on this machine, so the reference-facing layer is
written in Python with the reference's names (``!`` becomes a trailing ``_``),
argument meaning and error behaviour.  Every numeric step runs in
libjfem_cuda.so; this module only packs element data into flat arrays (the
host packing of ext/JuliaFEMCUDAExt.jl:86-217) and unpacks results.

Two entry styles, as in the reference:

* legacy — ``Problem(Elasticity, name, 3)``, ``Element(Tet10, conn)``,
  ``update_(elements, "youngs modulus", E)``, ``add_elements_``,
  ``assemble_(problem, time)`` filling ``problem.assembly.K / .f``
  (src/problems_elasticity.jl:65-81, src/assembly/problems.jl:14-40) and
  ``Analysis(Linear)`` + ``run_`` (src/solvers.jl:641-657);
* backend plugin — ``solve_(physics; backend=GPU(), tol, max_iter, newton_tol,
  max_newton, max_cg_per_newton)`` returning ``ElasticitySolution``
  (src/backend/abstract.jl:138-217) through ``initialize_backend`` and
  ``solve_backend_`` (ext/JuliaFEMCUDAExt.jl:867-916).
"""
from __future__ import annotations

import time as _time
import warnings
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from ._abi import Context, JFEMError

# element / face types (names of the reference's Element{Tet10} etc.)
Tet4, Tet10, Hex8 = "Tet4", "Tet10", "Hex8"
Tri3, Tri6, Quad4 = "Tri3", "Tri6", "Quad4"
_VOLUME = {Tet4: _abi.TET4, Tet10: _abi.TET10, Hex8: _abi.HEX8}
_SURFACE = {Tri3: _abi.TRI3, Tri6: _abi.TRI6, Quad4: _abi.QUAD4}
_NNODES = {Tet4: 4, Tet10: 10, Hex8: 8, Tri3: 3, Tri6: 6, Quad4: 4}


# ---------------------------------------------------------------------------
# problems and elements (legacy API)
# ---------------------------------------------------------------------------
@dataclass
class Elasticity:
    """Problem properties (src/problems_elasticity.jl:36-50)."""
    formulation: str = "continuum"
    finite_strain: bool = False
    geometric_stiffness: bool = False
    store_fields: list = field(default_factory=list)
    material_model: str = "linear_elastic"   # or "neo_hookean" (src/materials/neo_hookean.jl)


@dataclass
class Dirichlet:
    """Nodal-collocation Dirichlet problem (src/problems_dirichlet.jl:37-95)."""
    formulation: str = "incremental"
    variational: bool = False


class Element:
    """Element{T}(connectivity) with named fields (src/elements/elements.jl)."""

    def __init__(self, etype: str, connectivity):
        if etype not in _NNODES:
            raise ValueError(f"unsupported element type {etype}")
        conn = tuple(int(c) for c in connectivity)
        if len(conn) != _NNODES[etype]:
            raise ValueError(f"{etype} needs {_NNODES[etype]} nodes, got {len(conn)}")
        self.etype = etype
        self.connectivity = conn
        self.fields: dict = {}

    def __len__(self):
        return len(self.connectivity)

    def haskey(self, name: str) -> bool:
        return name in self.fields

    def __call__(self, name: str):
        return self.fields[name]


def update_(elements, name: str, value):
    """update!(elements, field, value): a constant, a dict node→value (geometry),
    or a callable of the element."""
    if isinstance(elements, Element):
        elements = [elements]
    for el in elements:
        el.fields[name] = value(el) if callable(value) else value


class Assembly:
    """Global arrays of a problem after assemble_ (src/assembly/problems.jl:14-40)."""

    def __init__(self):
        self.K = None          # scipy.sparse.csc_matrix
        self.f = None          # numpy (3N,)
        self.colptr = self.rowval = self.nzval = None

    def isempty(self) -> bool:
        return self.K is None

    def empty_(self):
        self.__init__()


class Problem:
    """Problem{P}(name, dim[, parent_field]) (src/assembly/problems.jl:95-141)."""

    def __init__(self, kind, name: str, dim: int = 3, parent_field: str | None = None):
        self.properties = kind() if isinstance(kind, type) else kind
        self.name = name
        self.dim = dim
        self.parent_field_name = parent_field
        self.elements: list[Element] = []
        self.assembly = Assembly()
        self._ctx: Context | None = None
        self._node_map = None

    def get_unknown_field_name(self) -> str:
        return "displacement"


def add_elements_(problem: Problem, elements):
    problem.elements.extend(elements)


def get_gdofs(node_ids, dim: int = 3):
    """Interleaved global DOFs 3(n−1)+j for 1-based node ids (problems.jl:466-478), 0-based."""
    node_ids = np.asarray(node_ids, dtype=np.int64)
    return (dim * (node_ids[:, None] - 1) + np.arange(dim)[None, :]).ravel()


def _node_table(elements):
    """Renumber 1-based node ids to a dense 0-based range (ext/JuliaFEMCUDAExt.jl:100-108)."""
    ids = sorted({n for el in elements for n in el.connectivity})
    return {n: i for i, n in enumerate(ids)}, ids


def _pack_volume(problem: Problem):
    vols = [el for el in problem.elements if el.etype in _VOLUME]
    surfs = [el for el in problem.elements if el.etype in _SURFACE]
    others = [el for el in problem.elements if el.etype not in _VOLUME and el.etype not in _SURFACE]
    if others:
        raise RuntimeError(f"Tried to assemble unsupported elements of type {others[0].etype} "
                           "to 3d continuum problem.")     # problems_elasticity.jl:510-518
    types = {el.etype for el in vols}
    if len(types) != 1:
        raise RuntimeError("one volume element type per problem is supported "
                           f"(found {sorted(types) or 'none'})")
    etype = types.pop()
    node_map, ids = _node_table(problem.elements)
    N = len(ids)
    X = np.zeros((N, 3))
    seen = np.zeros(N, bool)
    for el in vols + surfs:
        geo = el.fields.get("geometry")
        if geo is None:
            continue
        for n in el.connectivity:
            X[node_map[n]] = geo[n]
            seen[node_map[n]] = True
    if not seen.all():
        raise RuntimeError("field 'geometry' missing for some nodes")
    conn = np.array([[node_map[n] for n in el.connectivity] for el in vols], dtype=np.int64)
    E = np.array([float(el.fields["youngs modulus"]) for el in vols])
    nu = np.array([float(el.fields["poissons ratio"]) for el in vols])
    faces = []
    for el in surfs:
        t = np.zeros(3)
        pr = 0.0
        has = False
        if "displacement traction force" in el.fields:
            t += np.asarray(el.fields["displacement traction force"], dtype=float)
            has = True
        for i in range(3):
            key = f"displacement traction force {i + 1}"
            if key in el.fields:
                t[i] += float(el.fields[key])
                has = True
        if "surface pressure" in el.fields:
            pr = float(el.fields["surface pressure"])
            has = True
        if has:
            faces.append((el.etype, [node_map[n] for n in el.connectivity], t, pr))
    return _VOLUME[etype], X, conn, E, nu, faces, node_map, ids


def _context_for(problem: Problem) -> Context:
    ftype, X, conn, E, nu, faces, node_map, ids = _pack_volume(problem)
    ctx = Context(0)
    ctx.set_mesh(ftype, X, conn)
    props = problem.properties
    model = _abi.NEO_HOOKEAN if getattr(props, "material_model", "") == "neo_hookean" else _abi.LINEAR_ELASTIC
    ctx.set_material(E, nu, model)
    ctx.set_formulation(bool(props.finite_strain), bool(props.geometric_stiffness))
    if faces:
        kinds = {f[0] for f in faces}
        if len(kinds) != 1:
            raise RuntimeError("one surface element type per problem is supported")
        k = kinds.pop()
        ctx.set_surface_load(_SURFACE[k], np.array([f[1] for f in faces], dtype=np.int64),
                             np.array([f[2] for f in faces]), np.array([f[3] for f in faces]))
    problem._ctx = ctx
    problem._node_map = (node_map, ids)
    return ctx


def assemble_(problem: Problem, time: float = 0.0):
    """assemble!(problem, time): global K (CSC) and f = f_ext − f_int on the GPU.

    Fills ``problem.assembly.K`` (scipy CSC in the problem's dense node order,
    interleaved DOFs) and ``problem.assembly.f``.
    """
    import scipy.sparse as sp
    if not isinstance(problem.properties, Elasticity):
        raise TypeError("assemble_ on the GPU path supports Problem{Elasticity}")
    if not problem.assembly.isempty():
        warnings.warn(f"Assemble problem {problem.name}: problem.assembly is not empty")
    ctx = _context_for(problem)
    u = problem.__dict__.get("_u_state")
    if u is not None:
        ctx.set_state(u)
    colptr, rowval, nzval, f = ctx.assemble_csc(0)
    n = colptr.size - 1
    problem.assembly.colptr, problem.assembly.rowval, problem.assembly.nzval = colptr, rowval, nzval
    problem.assembly.K = sp.csc_matrix((nzval, rowval, colptr), shape=(n, n))
    problem.assembly.f = f
    return problem.assembly


# ---------------------------------------------------------------------------
# backends and the new solve! API
# ---------------------------------------------------------------------------
class AbstractBackend:
    pass


class Auto(AbstractBackend):
    pass


class GPU(AbstractBackend):
    pass


class CPU(AbstractBackend):
    def __init__(self, nthreads: int = 1):
        self.nthreads = nthreads


def select_backend(backend: AbstractBackend) -> AbstractBackend:
    """select_backend (src/backend/abstract.jl:72-112).  This package only
    provides the GPU backend; CPU requests raise instead of silently running
    elsewhere."""
    if isinstance(backend, CPU):
        raise RuntimeError("CPU backend is not provided by the GB300 package")
    _abi.load()
    return GPU()


@dataclass
class ElasticitySolution:
    """src/backend/abstract.jl:138-151."""
    u: np.ndarray
    newton_iterations: int
    cg_iterations: int
    residual: float
    solve_time: float
    history: list


@dataclass
class DirichletBC:
    """Prescribed displacement components on nodes (0-based node indices)."""
    nodes: np.ndarray
    components: tuple = (1, 2, 3)     # 1-based like "displacement 1..3"
    value: float | np.ndarray = 0.0


@dataclass
class NeumannBC:
    """Surface traction on faces (0-based node indices)."""
    face_type: str
    faces: np.ndarray
    traction: np.ndarray


@dataclass
class Physics:
    """Physics{Elasticity}: mesh arrays, material, BCs (src/physics.jl:42-64)."""
    element_type: str
    X: np.ndarray
    conn: np.ndarray
    E: float | np.ndarray = 210e3
    nu: float | np.ndarray = 0.3
    material_model: str = "linear_elastic"
    finite_strain: bool = False
    geometric_stiffness: bool = False
    dirichlet: list = field(default_factory=list)
    neumann: list = field(default_factory=list)
    n_load_steps: int = 1
    precision: str = "mixed"      # "mixed" (FP32 apply + FP64 refinement) or "fp64"


def add_dirichlet_(physics: Physics, nodes, components=(1, 2, 3), value=0.0):
    physics.dirichlet.append(DirichletBC(np.asarray(nodes, dtype=np.int64), tuple(components), value))


def add_neumann_(physics: Physics, face_type: str, faces, traction):
    physics.neumann.append(NeumannBC(face_type, np.asarray(faces, dtype=np.int64),
                                     np.asarray(traction, dtype=np.float64)))


def _dirichlet_arrays(physics: Physics):
    dofs, vals = [], []
    for bc in physics.dirichlet:
        v = np.broadcast_to(np.asarray(bc.value, dtype=np.float64), (len(bc.nodes),))
        for c in bc.components:
            dofs.append(3 * bc.nodes + (c - 1))
            vals.append(v)
    if not dofs:
        return np.zeros(0, np.int64), np.zeros(0)
    d = np.concatenate(dofs)
    v = np.concatenate(vals)
    if np.unique(d).size != d.size:
        raise RuntimeError("problem is overconstrained, not continuing to solution.")   # solvers.jl:96-130
    return d, v


def initialize_backend(backend: AbstractBackend, physics: Physics, time: float = 0.0) -> Context:
    """Upload mesh, material, Dirichlet masks and traction table; build adjacency
    and sparsity pattern on the device (ext/JuliaFEMCUDAExt.jl:86-217)."""
    ctx = Context(0)
    et = _VOLUME[physics.element_type]
    ctx.set_mesh(et, physics.X, physics.conn)
    model = _abi.NEO_HOOKEAN if physics.material_model == "neo_hookean" else _abi.LINEAR_ELASTIC
    ctx.set_material(physics.E, physics.nu, model)
    ctx.set_formulation(physics.finite_strain, physics.geometric_stiffness)
    d, v = _dirichlet_arrays(physics)
    ctx.set_dirichlet(d, v)
    if physics.neumann:
        kinds = {bc.face_type for bc in physics.neumann}
        if len(kinds) != 1:
            raise RuntimeError("one surface element type per problem is supported")
        faces = np.concatenate([bc.faces for bc in physics.neumann])
        trac = np.concatenate([np.broadcast_to(bc.traction, (len(bc.faces), 3)) for bc in physics.neumann])
        ctx.set_traction(_SURFACE[kinds.pop()], faces, trac)
    return ctx


def solve_backend_(data: Context, physics: Physics, tol=1e-6, max_iter=1000, newton_tol=1e-6, max_newton=20,
                   max_cg_per_newton=50, method: str | None = None):
    """solve_backend!: returns (u, newton_iters, cg_iters, residual, history)."""
    nonlinear = physics.finite_strain
    m = {"pcg": _abi.PCG_JACOBI, "newton": _abi.NEWTON, "fcg": _abi.FCG_LEARNED}
    meth = m[method] if method else (_abi.NEWTON if nonlinear else _abi.PCG_JACOBI)
    opts = _abi.default_opts(method=meth, precision=_abi.MIXED if physics.precision == "mixed" else _abi.FP64,
                             tol=tol, max_iter=max_iter, newton_tol=newton_tol, max_newton=max_newton,
                             max_cg_per_newton=max_cg_per_newton, n_load_steps=physics.n_load_steps)
    u, st, rc = data.solve(opts)
    if rc == _abi.NOT_CONVERGED:
        warnings.warn(f"CG did not converge in {max_iter} iterations")   # ext/JuliaFEMCUDAExt.jl:630
    return u, st.newton_iterations, st.cg_iterations, st.residual, st.history_list()


def solve_(physics: Physics, backend: AbstractBackend | None = None, time: float = 0.0, tol: float = 1e-6,
           max_iter: int = 1000, newton_tol: float = 1e-6, max_newton: int = 20, max_cg_per_newton: int = 50,
           method: str | None = None) -> ElasticitySolution:
    """solve!(physics; backend, time, tol, max_iter, newton_tol, max_newton,
    max_cg_per_newton) (src/backend/abstract.jl:181-217)."""
    select_backend(backend or Auto())
    t0 = _time.perf_counter_ns()
    data = initialize_backend(GPU(), physics, time)
    try:
        u, ni, ci, res, hist = solve_backend_(data, physics, tol=tol, max_iter=max_iter, newton_tol=newton_tol,
                                              max_newton=max_newton, max_cg_per_newton=max_cg_per_newton,
                                              method=method)
    finally:
        data.close()
    t1 = _time.perf_counter_ns()
    return ElasticitySolution(np.asarray(u), ni, ci, res, (t1 - t0) / 1e9, hist)


# ---------------------------------------------------------------------------
# legacy Analysis{Linear} driver
# ---------------------------------------------------------------------------
class Linear:
    pass


class Analysis:
    def __init__(self, kind=Linear, name: str = "analysis"):
        self.kind = kind
        self.name = name
        self.problems: list[Problem] = []
        self.u = None
        self.properties = {"tol": 1e-10, "max_iter": 100000}


def add_problems_(analysis: Analysis, problems):
    analysis.problems.extend(problems)


def run_(analysis: Analysis, time: float = 0.0):
    """run!(Analysis{Linear}) (src/solvers.jl:641-657): field problem + nodal
    Dirichlet problems, solved on the GPU (elimination of prescribed DOFs)."""
    fields = [p for p in analysis.problems if isinstance(p.properties, Elasticity)]
    bcs = [p for p in analysis.problems if isinstance(p.properties, Dirichlet)]
    if len(fields) != 1:
        raise RuntimeError("exactly one Elasticity problem is supported")
    prob = fields[0]
    ctx = _context_for(prob)
    node_map, ids = prob._node_map
    dofs, vals = {}, {}
    for bc in bcs:
        # within one Dirichlet problem later values overwrite earlier ones
        # (field_vals dict of src/problems_dirichlet.jl:60-89); a DOF constrained by
        # two problems is an error (check_for_overconstrained_dofs, src/solvers.jl:96-130)
        mine = {}
        for el in bc.elements:
            for i in range(3):
                key = f"{bc.parent_field_name or 'displacement'} {i + 1}"
                if key not in el.fields:
                    continue
                for n in el.connectivity:
                    mine[3 * node_map[n] + i] = float(el.fields[key])
        if set(mine) & set(dofs):
            raise RuntimeError("problem is overconstrained, not continuing to solution.")
        dofs.update({d: True for d in mine})
        vals.update(mine)
    d = np.array(sorted(dofs), dtype=np.int64)
    ctx.set_dirichlet(d, np.array([vals[k] for k in d]) if d.size else None)
    u, st, rc = ctx.solve(method=_abi.PCG_JACOBI, precision=_abi.FP64, tol=analysis.properties["tol"],
                          max_iter=analysis.properties["max_iter"])
    if rc == _abi.NOT_CONVERGED:
        warnings.warn("linear solve did not converge")
    analysis.u = {nid: u[3 * i:3 * i + 3] for i, nid in enumerate(ids)}
    analysis.stats = st
    ctx.close()
    prob._ctx = None
    return analysis.u
