"""ORACLE TEST INFRASTRUCTURE -- not part of the product.

ctypes wrapper of oracle/_build/liboracle.so (the C restatement of the
reference path, mgcfd_oracle.c) and a runner for the reference binary
oracle/_ref/euler3d_ref.  Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg use this module, and only as the checker.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
sys.path.insert(0, str(HERE))
import recipe as _recipe  # noqa: E402  (oracle/recipe.py)

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class Freestream(C.Structure):
    _fields_ = [("smoothing_coefficient", C.c_double), ("ff_variable", C.c_double * 5),
                ("ff_flux_contribution_momentum_x", C.c_double * 3),
                ("ff_flux_contribution_momentum_y", C.c_double * 3),
                ("ff_flux_contribution_momentum_z", C.c_double * 3),
                ("ff_flux_contribution_density_energy", C.c_double * 3)]


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        _recipe.build_oracle()
        L = C.CDLL(str(_recipe.ORACLE_LIB))
        L.orc_freestream_init.argtypes = [C.c_double, C.c_double, C.POINTER(Freestream)]
        L.orc_mesh_create.restype = C.c_void_p
        L.orc_mesh_create.argtypes = [C.c_int]
        L.orc_mesh_set_level.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, _dp, _ip, _ip, _ip,
                                         _dp, _dp, _ip]
        L.orc_run.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_int, C.c_int, C.c_int, _dp]
        L.orc_get.argtypes = [C.c_void_p, C.c_int, C.c_int, _dp]
        L.orc_smoothing_steps.restype = C.c_long
        L.orc_smoothing_steps.argtypes = [C.c_void_p]
        L.orc_mesh_destroy.argtypes = [C.c_void_p]
        L.orc_mesh_set_volumes.argtypes = [C.c_void_p, C.c_int, _dp]
        L.orc_loop_get_min_dt.restype = C.c_double
        L.orc_loop_calc_rms.restype = C.c_double
        _LIB = L
    return _LIB


def dptr(a):
    return a.ctypes.data_as(_dp) if a is not None else None


def iptr(a):
    return a.ctypes.data_as(_ip) if a is not None else None


def freestream(mach, aoa):
    ff = Freestream()
    lib().orc_freestream_init(mach, aoa, C.byref(ff))
    return ff


Q_VARIABLES, Q_FLUXES, Q_STEP_FACTORS, Q_VOLUMES, Q_RESIDUALS, Q_EWT, Q_BWT, Q_OLD = range(8)


class OracleRun:
    """Whole-run oracle over a list of mgcfd.mesh.Level objects."""

    def __init__(self, levels):
        L = lib()
        self._h = L.orc_mesh_create(len(levels))
        self.levels = levels
        for i, lv in enumerate(levels):
            arrs = [np.ascontiguousarray(a) for a in (lv.coords, lv.edge_to_nodes, lv.bnd_to_node, lv.bnd_group,
                                                       lv.edge_weights, lv.bnd_weights)]
            n2mg = np.ascontiguousarray(lv.node_to_mg) if lv.node_to_mg is not None else None
            rc = L.orc_mesh_set_level(self._h, i, lv.nnodes, lv.nedges, lv.nbnd, dptr(arrs[0]), iptr(arrs[1]),
                                      iptr(arrs[2]), iptr(arrs[3]), dptr(arrs[4]), dptr(arrs[5]), iptr(n2mg))
            assert rc == 0
            if getattr(lv, "volumes", None) is not None:
                self._vols = getattr(self, "_vols", []) + [np.ascontiguousarray(lv.volumes)]
                assert L.orc_mesh_set_volumes(self._h, i, dptr(self._vols[-1])) == 0

    def run(self, mach, aoa, ncycles, nthreads=1, measure_mem_bound=False):
        t = C.c_double()
        st = lib().orc_run(self._h, mach, aoa, ncycles, nthreads, int(measure_mem_bound), C.byref(t))
        return st, t.value

    def get(self, level, what):
        lv = self.levels[level]
        shape = {Q_VARIABLES: (lv.nnodes, 5), Q_FLUXES: (lv.nnodes, 5), Q_STEP_FACTORS: (lv.nnodes,),
                 Q_VOLUMES: (lv.nnodes,), Q_RESIDUALS: (lv.nnodes, 5), Q_EWT: (lv.nedges, 3),
                 Q_BWT: (lv.nbnd, 3), Q_OLD: (lv.nnodes, 5)}[what]
        out = np.empty(shape, dtype=np.float64)
        assert lib().orc_get(self._h, level, what, dptr(out)) == 0
        return out

    @property
    def smoothing_steps(self):
        return lib().orc_smoothing_steps(self._h)

    def close(self):
        if self._h:
            lib().orc_mesh_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_reference_binary(workdir, ncycles, mach, aoa, extra_args=(), prefix="solution."):
    """Run oracle/_ref/euler3d_ref on workdir/input.dat; returns CompletedProcess."""
    exe = _recipe.build_reference()
    if exe is None:
        raise FileNotFoundError("reference sources are not available on this host")
    env = dict(os.environ, MGCFD_MACH=repr(float(mach)), MGCFD_AOA_DEG=repr(float(aoa)))
    cmd = [str(exe), "-i", "input.dat", "-g", str(ncycles), "--output-variables", "--output-step-factors",
           "-o", prefix, *extra_args]
    return subprocess.run(cmd, cwd=workdir, env=env, capture_output=True, text=True)
