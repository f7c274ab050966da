"""GB300-native ODIL engine.

Host API mirroring the reference (odil22/odil util_op.py / util.py /
optimizer.py / linsolver.py) over hand-written sm_103a CUDA kernels in
libodil_gb300.so (C ABI, include/odil_gb300.h).  There is no CPU fallback:
without the built library every compute call raises.
"""
from .domain import Domain, State
from .problem import Context, Problem
from .wave import WaveOperator, WaveKernels, extrap_quadh
from ._capi import OdilError
# The names of the reference's facade module (odil.py): the solver modules,
# History and MultigridDecomp.
from . import history, linsolver, optimizer, util
from .history import History
from .multigrid import MultigridDecomp

util_history = history

__all__ = [
    "Domain", "State", "Context", "Problem", "WaveOperator", "WaveKernels",
    "extrap_quadh", "OdilError", "History", "MultigridDecomp", "util",
    "linsolver", "optimizer", "history", "util_history"
]
