"""GB300-native global step of warp-mfem's mixed variational FEM solver.

``MixedFEMSolver`` (alias ``RefinementSolver``) keeps the reference solver's
constructor and ``step(state_in, state_out, control, contacts, dt)``; all
compute runs in libmfem_gb300.so (hand-written sm_103a CUDA, C ABI in
include/mfem_gb300.h).
"""
from . import beams
from .model import Model, State

__all__ = ["beams", "Model", "State", "MixedFEMSolver", "RefinementSolver"]


def __getattr__(name):
    # the solver loads the CUDA library; import it lazily so mesh generation
    # and the build work on machines without a GPU
    if name in ("MixedFEMSolver", "RefinementSolver"):
        from . import solver
        return getattr(solver, name)
    raise AttributeError(name)
