"""ctypes binding of libmgcfd_gb300.so (declarations in include/mgcfd_gb300.h).

The library is the product; there is no Python or CPU fallback.  Loading
fails with an ImportError naming the missing file when it has not been built.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from . import _build

c_double_p = C.POINTER(C.c_double)
c_int32_p = C.POINTER(C.c_int32)


class Freestream(C.Structure):
    _fields_ = [("smoothing_coefficient", C.c_double),
                ("ff_variable", C.c_double * 5),
                ("ff_flux_contribution_momentum_x", C.c_double * 3),
                ("ff_flux_contribution_momentum_y", C.c_double * 3),
                ("ff_flux_contribution_momentum_z", C.c_double * 3),
                ("ff_flux_contribution_density_energy", C.c_double * 3)]


class LevelView(C.Structure):
    _fields_ = [("nnodes", C.c_int32), ("nedges", C.c_int32), ("nbnd", C.c_int32), ("n_axis", C.c_int32),
                ("coords", c_double_p), ("edge_to_nodes", c_int32_p), ("bnd_to_node", c_int32_p),
                ("bnd_group", c_int32_p), ("edge_weights", c_double_p), ("bnd_weights", c_double_p),
                ("node_to_mg", c_int32_p), ("volumes", c_double_p)]


class SolverOptions(C.Structure):
    _fields_ = [("precision", C.c_int32), ("increment", C.c_int32), ("renumber", C.c_int32),
                ("use_graph", C.c_int32), ("measure_mem_bound", C.c_int32), ("block_size", C.c_int32),
                ("time_kernels", C.c_int32), ("host_setup", C.c_int32), ("accumulation", C.c_int32),
                ("stage_neighbour_ids", C.c_int32), ("edge_parallel_stage", C.c_int32),
                ("reserved", C.c_int32 * 5)]


class SolverStats(C.Structure):
    _fields_ = [("cycles", C.c_int64), ("smoothing_steps", C.c_int64), ("flux_sweeps_l0", C.c_int64),
                ("flux_ms_l0", C.c_double), ("kernel_launches", C.c_int64), ("device_bytes", C.c_int64),
                ("rms_l0", C.c_double), ("status", C.c_int32), ("ncolors_reserved", C.c_int32)]


class ServerOptions(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_int64), ("max_active", C.c_int32), ("precision", C.c_int32),
                ("increment", C.c_int32), ("max_cycles", C.c_int32), ("residual_drop", C.c_double),
                ("accumulation", C.c_int32), ("batch_max_meshes", C.c_int32), ("batch_max_nodes", C.c_int32),
                ("reserved", C.c_int32 * 5)]


class RequestResult(C.Structure):
    _fields_ = [("id", C.c_int64), ("status", C.c_int32), ("cycles", C.c_int32), ("submit_s", C.c_double),
                ("admit_s", C.c_double), ("finish_s", C.c_double), ("rho_rms_first", C.c_double),
                ("rho_rms_last", C.c_double), ("device_begin_s", C.c_double), ("device_end_s", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("failed", C.c_int64), ("active", C.c_int64),
                ("pending", C.c_int64), ("used_bytes", C.c_int64), ("peak_bytes", C.c_int64),
                ("peak_active", C.c_int64), ("cache_hits", C.c_int64), ("cached_solvers", C.c_int64),
                ("cohorts", C.c_int64), ("cohort_requests", C.c_int64)]


OK = 0
ERR_INVALID, ERR_CUDA, ERR_NOMEM, ERR_IO, ERR_NEGATIVE_DT, ERR_BAD_VALUES, ERR_TIMEOUT, ERR_BUDGET = range(1, 9)

_vp = C.c_void_p
_i32 = C.c_int32
_pp = C.POINTER

# name -> (restype, argtypes); every symbol declared in include/mgcfd_gb300.h.
SIGNATURES = {
    "mgcfd_abi_version": (C.c_int, []),
    "mgcfd_status_string": (C.c_char_p, [C.c_int]),
    "mgcfd_last_error": (C.c_char_p, []),
    "mgcfd_freestream_init": (C.c_int, [C.c_double, C.c_double, _pp(Freestream)]),
    "mgcfd_host_mesh_generate": (C.c_int, [C.c_int, C.c_int, C.c_uint64, _pp(_vp)]),
    "mgcfd_host_mesh_load": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int, _pp(_vp)]),
    "mgcfd_host_mesh_write": (C.c_int, [_vp, C.c_char_p, C.c_char_p, _i32]),
    "mgcfd_host_mesh_num_levels": (C.c_int, [_vp]),
    "mgcfd_host_mesh_level": (C.c_int, [_vp, C.c_int, _pp(LevelView)]),
    "mgcfd_host_mesh_destroy": (None, [_vp]),
    "mgcfd_host_mesh_from_views": (C.c_int, [_i32, _pp(LevelView), _pp(_vp)]),
    "mgcfd_renumber_nodes": (C.c_int, [C.c_int, _i32, c_double_p, _i32, c_int32_p, c_int32_p]),
    "mgcfd_host_mesh_renumber": (C.c_int, [_vp, C.c_int, C.POINTER(_vp)]),
    "mgcfd_h5_dataset_shape": (C.c_int, [C.c_char_p, C.c_char_p, _pp(C.c_int64), _pp(C.c_int)]),
    "mgcfd_h5_read_f64": (C.c_int, [C.c_char_p, C.c_char_p, c_double_p, C.c_int64]),
    "mgcfd_h5_read_i32": (C.c_int, [C.c_char_p, C.c_char_p, c_int32_p, C.c_int64]),
    "mgcfd_h5_write_f64": (C.c_int, [C.c_char_p, C.c_char_p, c_double_p, C.c_int64, C.c_int64]),
    "mgcfd_op_initialize_variables": (C.c_int, [_i32, _pp(Freestream), _vp, _vp]),
    "mgcfd_op_zero": (C.c_int, [_i32, _i32, _vp, _vp]),
    "mgcfd_op_calculate_cell_volumes": (C.c_int, [_i32, _i32, _vp, _vp, _vp, _vp, _vp]),
    "mgcfd_op_dampen_ewt": (C.c_int, [_i32, _vp, _vp]),
    "mgcfd_op_copy_double": (C.c_int, [_i32, _vp, _vp, _vp]),
    "mgcfd_op_calculate_dt": (C.c_int, [_i32, _vp, _vp, _vp, _vp]),
    "mgcfd_op_get_min_dt": (C.c_int, [_i32, _vp, _vp, _vp]),
    "mgcfd_op_compute_step_factor": (C.c_int, [_i32, _vp, _vp, _vp, _vp, _vp]),
    "mgcfd_op_compute_flux_edge": (C.c_int, [_i32, _i32, _vp, _vp, _vp, C.c_double, _vp, _vp]),
    "mgcfd_op_compute_bnd_node_flux": (C.c_int, [_i32, _i32, _vp, _vp, _vp, _vp, _pp(Freestream), _vp, _vp]),
    "mgcfd_op_time_step": (C.c_int, [_i32, _i32, _vp, _vp, _vp, _vp, _vp]),
    "mgcfd_op_unstructured_stream": (C.c_int, [_i32, _i32, _vp, _vp, _vp, _vp, _vp]),
    "mgcfd_op_residual": (C.c_int, [_i32, _vp, _vp, _vp, _vp]),
    "mgcfd_op_calc_rms": (C.c_int, [_i32, _vp, _vp, _vp]),
    "mgcfd_op_count_bad_vals": (C.c_int, [_i32, _vp, _vp, _vp]),
    "mgcfd_op_up_pre": (C.c_int, [_i32, _i32, _vp, _vp, _vp, _vp]),
    "mgcfd_op_up": (C.c_int, [_i32, _i32, _vp, _vp, _vp, _vp, _vp]),
    "mgcfd_op_up_post": (C.c_int, [_i32, _vp, _vp, _vp]),
    "mgcfd_op_down": (C.c_int, [_i32, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "mgcfd_op_plans_mode": (C.c_int, [_i32]),
    "mgcfd_op_flux_precision": (C.c_int, [_i32]),
    "mgcfd_op_plan_release": (C.c_int, [_vp]),
    "mgcfd_op_plans_release": (C.c_int, []),
    "mgcfd_op_plans_info": (C.c_int, [_pp(C.c_int64), _pp(C.c_int64), _pp(C.c_int64), _pp(C.c_int64)]),
    "mgcfd_op_map_errors": (C.c_int, [_pp(C.c_int64), _i32]),
    "mgcfd_op_restrict_noalloc": (C.c_int, [_i32, _i32, _vp, _vp, _vp, _vp]),
    "mgcfd_op_count_differences": (C.c_int, [_i32, _vp, _vp, _vp, _vp]),
    "mgcfd_solver_default_options": (None, [_pp(SolverOptions)]),
    "mgcfd_solver_create": (C.c_int, [_i32, _pp(LevelView), C.c_double, C.c_double, _pp(SolverOptions), _vp,
                                      _pp(_vp)]),
    "mgcfd_solver_reset": (C.c_int, [_vp]),
    "mgcfd_solver_run": (C.c_int, [_vp, _i32]),
    "mgcfd_solver_synchronize": (C.c_int, [_vp]),
    "mgcfd_solver_step": (C.c_int, [_vp, _pp(_i32), _pp(C.c_int64)]),
    "mgcfd_solver_fetch": (C.c_int, [_vp, _i32, _i32, c_double_p]),
    "mgcfd_solver_get_stats": (C.c_int, [_vp, _pp(SolverStats)]),
    "mgcfd_solver_destroy": (None, [_vp]),
    "mgcfd_solver_table": (C.c_int, [_vp, _i32, _i32, _vp, C.c_int64, _pp(C.c_int64)]),
    "mgcfd_batch_create": (C.c_int, [_i32, _i32, _pp(_pp(LevelView)), _pp(C.c_double), _pp(C.c_double),
                                     _pp(SolverOptions), _vp, _pp(_vp)]),
    "mgcfd_solver_num_meshes": (C.c_int, [_vp]),
    "mgcfd_solver_fetch_mesh": (C.c_int, [_vp, _i32, _i32, _i32, c_double_p]),
    "mgcfd_solver_mesh_status": (C.c_int, [_vp, _i32, _pp(C.c_double), _pp(C.c_double)]),
    "mgcfd_server_default_options": (None, [_pp(ServerOptions)]),
    "mgcfd_server_create": (C.c_int, [_pp(ServerOptions), _pp(_vp)]),
    "mgcfd_server_submit": (C.c_int, [_vp, _i32, _pp(LevelView), C.c_double, C.c_double, C.c_int64,
                                      c_double_p, _pp(C.c_int64)]),
    "mgcfd_server_poll": (C.c_int, [_vp, _pp(RequestResult), _i32, _pp(_i32)]),
    "mgcfd_server_drain": (C.c_int, [_vp, C.c_double]),
    "mgcfd_server_get_stats": (C.c_int, [_vp, _pp(ServerStats)]),
    "mgcfd_server_destroy": (None, [_vp]),
    "mgcfd_request_estimate_bytes": (C.c_int, [_i32, _pp(LevelView), _i32, _i32, _pp(C.c_int64)]),
    "mgcfd_solve": (C.c_int, [_i32, _pp(LevelView), C.c_double, C.c_double, _i32, _pp(SolverOptions),
                              _pp(c_double_p)]),
}

_LIB = None


class MgcfdError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"mgcfd status {status}: {message}")
        self.status = status


def lib_path() -> Path:
    return _build.LIB


def load(build_if_missing: bool = False):
    """Load libmgcfd_gb300.so (building it first if asked and missing)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    p = lib_path()
    if not p.exists():
        if build_if_missing:
            _build.build_library()
        else:
            raise ImportError(f"{p} is not built; run __graft_entry__.build() (the CUDA library is required)")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def check(status: int) -> None:
    if status != OK:
        lib = load()
        msg = lib.mgcfd_last_error().decode(errors="replace") or lib.mgcfd_status_string(status).decode()
        raise MgcfdError(status, msg)
