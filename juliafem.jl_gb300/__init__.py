"""juliafem.jl_gb300 — GB300-native (sm_103a) JuliaFEM elasticity hot path.

The compute lives in libjfem_cuda.so (C ABI, include/jfem.h); this package is
its Python binding (``_abi``), the reference-shaped host API (``problem``), the
structured box mesher (``mesh``), the Abaqus input reader (``abaqus``) and the
weight and load-step checkpoint files (``checkpoint``).

The directory name contains a dot, so it is loaded by path; ``load_package()``
in __graft_entry__.py (and tests/conftest.py) registers it as ``jfem_gb300``.
"""
from . import _abi, abaqus, checkpoint, mesh, workloads
from ._abi import Batch, Context, JFEMError, SolveOpts, Stats, default_opts, load
from .problem import (CPU, GPU, Analysis, Auto, Dirichlet, DirichletBC, Elasticity, ElasticitySolution,
                      Element, Hex8, Linear, NeumannBC, Physics, Problem, Quad4, Tet4, Tet10, Tri3, Tri6,
                      add_dirichlet_, add_elements_, add_neumann_, add_problems_, assemble_, get_gdofs,
                      initialize_backend, run_, select_backend, solve_, solve_backend_, update_)

__all__ = [n for n in dir() if not n.startswith("__")]
