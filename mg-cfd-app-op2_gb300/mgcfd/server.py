"""Serving loop binding (mgcfd_server_* in include/mgcfd_gb300.h)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .mesh import HostMesh, level_views_from_arrays
from .solver import ACCUMULATION, INCREMENT, PRECISION


def estimate_bytes(mesh, precision: str = "fp64", increment: str = "auto") -> int:
    """Device bytes the server charges against its budget for a request on this
    mesh (mgcfd_request_estimate_bytes)."""
    levels = mesh.levels() if isinstance(mesh, HostMesh) else mesh
    views = level_views_from_arrays(levels)
    b = C.c_int64()
    _lib.check(_lib.load().mgcfd_request_estimate_bytes(len(levels), views, PRECISION[precision],
                                                        INCREMENT[increment], C.byref(b)))
    return b.value


class Server:
    """Continuous-batching solve server on one GPU.  batch_max_meshes > 1
    admits small requests (at most batch_max_nodes level-0 nodes) that wait
    next to each other as cohorts solved in shared launches."""

    def __init__(self, hbm_budget_gb: float = 150.0, max_active: int = 16, precision: str = "fp64",
                 increment: str = "auto", max_cycles: int = 50, residual_drop: float = 1e-6,
                 accumulation: str = "fp64", batch_max_meshes: int = 0, batch_max_nodes: int = 0):
        self._lib = _lib.load()
        o = _lib.ServerOptions()
        self._lib.mgcfd_server_default_options(C.byref(o))
        o.hbm_budget_bytes = int(hbm_budget_gb * (1 << 30))
        o.max_active = max_active
        o.precision = PRECISION[precision]
        o.increment = INCREMENT[increment]
        o.max_cycles = max_cycles
        o.residual_drop = residual_drop
        o.accumulation = ACCUMULATION[accumulation]
        o.batch_max_meshes = batch_max_meshes
        o.batch_max_nodes = batch_max_nodes
        h = C.c_void_p()
        _lib.check(self._lib.mgcfd_server_create(C.byref(o), C.byref(h)))
        self._h = h
        self._keep = {}  # request id -> (levels, views, output) kept alive until completion

    def submit(self, mesh, mach: float, aoa_deg: float, want_result: bool = False, mesh_key: int | None = None,
               resident: bool = True) -> int:
        """Queue a solve.  A HostMesh is kept resident on the device between
        requests (keyed by the HostMesh object) unless resident=False; a list
        of Level arrays is resident only under an explicit mesh_key."""
        levels = mesh.levels() if isinstance(mesh, HostMesh) else mesh
        if mesh_key is None:
            mesh_key = mesh.serial if (resident and isinstance(mesh, HostMesh)) else 0
        views = level_views_from_arrays(levels)
        out = np.empty((levels[0].nnodes, 5)) if want_result else None
        rid = C.c_int64()
        _lib.check(self._lib.mgcfd_server_submit(self._h, len(levels), views, mach, aoa_deg, int(mesh_key),
                                                 out.ctypes.data_as(_lib.c_double_p) if out is not None else None,
                                                 C.byref(rid)))
        self._keep[rid.value] = (mesh, levels, views, out)
        return rid.value

    def poll(self):
        """Completed requests since the last poll: list of (result dict, final level-0 variables or None)."""
        buf = (_lib.RequestResult * 256)()
        n = C.c_int32()
        done = []
        while True:
            _lib.check(self._lib.mgcfd_server_poll(self._h, buf, 256, C.byref(n)))
            for i in range(n.value):
                r = buf[i]
                keep = self._keep.pop(r.id, None)
                done.append(({"id": r.id, "status": r.status, "cycles": r.cycles, "submit_s": r.submit_s,
                              "admit_s": r.admit_s, "finish_s": r.finish_s, "rho_rms_first": r.rho_rms_first,
                              "rho_rms_last": r.rho_rms_last, "device_begin_s": r.device_begin_s,
                              "device_end_s": r.device_end_s}, keep[3] if keep else None))
            if n.value < 256:
                return done

    def drain(self, timeout_s: float = 600.0) -> None:
        _lib.check(self._lib.mgcfd_server_drain(self._h, timeout_s))

    def stats(self) -> dict:
        s = _lib.ServerStats()
        _lib.check(self._lib.mgcfd_server_get_stats(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in s._fields_ if k != "reserved"}

    def close(self):
        if getattr(self, "_h", None):
            self._lib.mgcfd_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
