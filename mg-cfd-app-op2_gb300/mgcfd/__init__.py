"""Python binding of mgcfd_gb300, the GB300-native MG-CFD multigrid Euler hot path.

The compute path is libmgcfd_gb300.so (hand-written sm_103a CUDA behind the C
ABI of include/mgcfd_gb300.h); this package only binds it with ctypes.
"""
from . import _build, _lib  # noqa: F401
from .mesh import HostMesh, Level, freestream, h5_read, level_views_from_arrays, renumber_nodes  # noqa: F401
from .solver import Batch, Solver, options, solve  # noqa: F401
from .solver import Q_FLUXES, Q_OLD_VARIABLES, Q_RESIDUALS, Q_STEP_FACTORS, Q_VARIABLES, Q_VOLUMES  # noqa: F401
from .server import Server  # noqa: F401
from .op2_vcycle import LoopSolver  # noqa: F401
