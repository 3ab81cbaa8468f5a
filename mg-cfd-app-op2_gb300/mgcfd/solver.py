"""Device-resident multigrid solver (mgcfd_solver_* in include/mgcfd_gb300.h)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .mesh import HostMesh, level_views_from_arrays

PRECISION = {"fp64": 0, "mixed": 1, "dw": 2}
INCREMENT = {"auto": 0, "atomic": 1, "gather": 2, "fused": 3, "coloured": 4}
RENUMBER = {"none": 0, "spatial": 1, "rcm": 2}
ACCUMULATION = {"fp64": 0, "pair32": 1}
Q_VARIABLES, Q_FLUXES, Q_STEP_FACTORS, Q_VOLUMES, Q_RESIDUALS, Q_OLD_VARIABLES = range(6)


def options(precision="fp64", increment="auto", renumber="spatial", use_graph=True, measure_mem_bound=False,
            block_size=0, time_kernels=False, host_setup=False, accumulation="fp64",
            stage_neighbour_ids=False, edge_parallel_stage=False) -> _lib.SolverOptions:
    o = _lib.SolverOptions()
    _lib.load().mgcfd_solver_default_options(C.byref(o))
    o.precision = PRECISION[precision]
    o.increment = INCREMENT[increment]
    o.renumber = RENUMBER[renumber]
    o.use_graph = int(use_graph)
    o.measure_mem_bound = int(measure_mem_bound)
    o.block_size = int(block_size)
    o.time_kernels = int(time_kernels)
    o.host_setup = int(host_setup)
    o.accumulation = ACCUMULATION[accumulation]
    o.stage_neighbour_ids = int(stage_neighbour_ids)
    o.edge_parallel_stage = int(edge_parallel_stage)
    return o


class Solver:
    """Owns a mesh on the GPU and runs V-cycles (euler3d.cpp:452-641)."""

    def __init__(self, mesh, mach: float, aoa_deg: float, stream: int | None = None, **opts):
        self._lib = _lib.load()
        if isinstance(mesh, HostMesh):
            views = mesh.level_views()
            self._nn = [mesh.level_view(l).nnodes for l in range(mesh.num_levels)]
        else:  # list of mgcfd.mesh.Level
            self._keep = mesh
            views = level_views_from_arrays(mesh)
            self._nn = [L.nnodes for L in mesh]
        self.options = options(**opts)
        h = C.c_void_p()
        _lib.check(self._lib.mgcfd_solver_create(len(views), views, mach, aoa_deg, C.byref(self.options),
                                                 C.c_void_p(stream) if stream else None, C.byref(h)))
        self._h = h

    @property
    def num_levels(self) -> int:
        return len(self._nn)

    def run(self, ncycles: int) -> None:
        _lib.check(self._lib.mgcfd_solver_run(self._h, ncycles))

    def step(self):
        """One smoothing step plus its transfer; returns (level smoothed, cycles done)."""
        lvl, cyc = C.c_int32(), C.c_int64()
        _lib.check(self._lib.mgcfd_solver_step(self._h, C.byref(lvl), C.byref(cyc)))
        return lvl.value, cyc.value

    def synchronize(self) -> int:
        """Waits; returns the status code (0 = ok) without raising."""
        return self._lib.mgcfd_solver_synchronize(self._h)

    def reset(self) -> None:
        _lib.check(self._lib.mgcfd_solver_reset(self._h))

    def fetch(self, level: int, quantity: int = Q_VARIABLES) -> np.ndarray:
        n = self._nn[level]
        width = 1 if quantity in (Q_STEP_FACTORS, Q_VOLUMES) else 5
        out = np.empty((n, width) if width > 1 else (n,), dtype=np.float64)
        _lib.check(self._lib.mgcfd_solver_fetch(self._h, level, quantity, out.ctypes.data_as(_lib.c_double_p)))
        return out

    def norms(self):
        """(status, rms_l0, density_rms_l0) after synchronising: the level-0
        residual norms of the last level-0 smoothing step (euler3d.cpp:533-537)."""
        rms, rho = C.c_double(), C.c_double()
        st = self._lib.mgcfd_solver_mesh_status(self._h, 0, C.byref(rms), C.byref(rho))
        return st, rms.value, rho.value

    def stats(self) -> _lib.SolverStats:
        s = _lib.SolverStats()
        _lib.check(self._lib.mgcfd_solver_get_stats(self._h, C.byref(s)))
        return s

    def close(self):
        if getattr(self, "_h", None):
            self._lib.mgcfd_solver_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def solve(levels, mach, aoa_deg, ncycles, **opts):
    """One full solve through host buffers (mgcfd_solve); returns per-level variables."""
    lib = _lib.load()
    views = level_views_from_arrays(levels)
    outs = [np.empty((L.nnodes, 5), dtype=np.float64) for L in levels]
    ptrs = (_lib.c_double_p * len(levels))(*[o.ctypes.data_as(_lib.c_double_p) for o in outs])
    o = options(**opts)
    _lib.check(lib.mgcfd_solve(len(levels), views, mach, aoa_deg, ncycles, C.byref(o), ptrs))
    return outs


class Batch(Solver):
    """Many independent meshes solved together, one launch per V-cycle stage
    (mgcfd_batch_create).  Each mesh has its own Mach number, angle of attack,
    min_dt and outcome."""

    def __init__(self, meshes, machs, aoas, stream: int | None = None, **opts):
        self._lib = _lib.load()
        level_lists = [m.levels() if isinstance(m, HostMesh) else m for m in meshes]
        nl = len(level_lists[0])
        if any(len(L) != nl for L in level_lists):
            raise ValueError("all meshes of a batch need the same number of levels")
        self._keep = (meshes, level_lists)
        self._views = [level_views_from_arrays(L) for L in level_lists]
        ptrs = (C.POINTER(_lib.LevelView) * len(meshes))(*[C.cast(v, C.POINTER(_lib.LevelView)) for v in self._views])
        self._mesh_nn = [[L.nnodes for L in levels] for levels in level_lists]
        self._nn = [sum(nn[l] for nn in self._mesh_nn) for l in range(nl)]
        mach = (C.c_double * len(meshes))(*machs)
        aoa = (C.c_double * len(meshes))(*aoas)
        self.options = options(**opts)
        h = C.c_void_p()
        _lib.check(self._lib.mgcfd_batch_create(len(meshes), nl, ptrs, mach, aoa, C.byref(self.options),
                                                C.c_void_p(stream) if stream else None, C.byref(h)))
        self._h = h

    @property
    def num_meshes(self) -> int:
        return len(self._mesh_nn)

    def fetch_mesh(self, mesh: int, level: int, quantity: int = Q_VARIABLES) -> np.ndarray:
        n = self._mesh_nn[mesh][level]
        width = 1 if quantity in (Q_STEP_FACTORS, Q_VOLUMES) else 5
        out = np.empty((n, width) if width > 1 else (n,), dtype=np.float64)
        _lib.check(self._lib.mgcfd_solver_fetch_mesh(self._h, mesh, level, quantity,
                                                     out.ctypes.data_as(_lib.c_double_p)))
        return out

    def fetch_meshes(self, level: int, quantity: int = Q_VARIABLES):
        """Every mesh's rows of one level with a single device-to-host copy:
        a list of arrays (views into one buffer), in mesh order."""
        whole = self.fetch(level, quantity)
        bounds = np.cumsum([0] + [nn[level] for nn in self._mesh_nn])
        return [whole[bounds[m]:bounds[m + 1]] for m in range(len(self._mesh_nn))]

    def mesh_status(self, mesh: int):
        """(status, rms_l0, density_rms_l0) of one mesh after synchronising."""
        rms, rho = C.c_double(), C.c_double()
        st = self._lib.mgcfd_solver_mesh_status(self._h, mesh, C.byref(rms), C.byref(rho))
        return st, rms.value, rho.value
