"""Per-loop drop-in entry points (mgcfd_op_* in include/mgcfd_gb300.h).

Each function takes device pointers (ints, e.g. torch.Tensor.data_ptr()) to
arrays in OP2's dat layout and enqueues one op_par_loop's worth of work on
`stream` (an int cudaStream_t handle, 0 = default stream).
"""
from __future__ import annotations

import ctypes as C

from . import _lib


def _call(name, *args):
    _lib.check(getattr(_lib.load(), name)(*args))


def _p(x):
    return C.c_void_p(int(x)) if x else None


def initialize_variables(n, ff, variables, stream=0):
    _call("mgcfd_op_initialize_variables", n, C.byref(ff), _p(variables), _p(stream))


def zero(n, dim, array, stream=0):
    _call("mgcfd_op_zero", n, dim, _p(array), _p(stream))


def calculate_cell_volumes(nedges, nnodes, edge_to_nodes, coords, edge_weights, volumes, stream=0):
    _call("mgcfd_op_calculate_cell_volumes", nedges, nnodes, _p(edge_to_nodes), _p(coords), _p(edge_weights), _p(volumes),
          _p(stream))


def dampen_ewt(n, weights, stream=0):
    _call("mgcfd_op_dampen_ewt", n, _p(weights), _p(stream))


def copy_double(n, variables, old_variables, stream=0):
    _call("mgcfd_op_copy_double", n, _p(variables), _p(old_variables), _p(stream))


def calculate_dt(n, variables, volumes, dt, stream=0):
    _call("mgcfd_op_calculate_dt", n, _p(variables), _p(volumes), _p(dt), _p(stream))


def get_min_dt(n, dt, min_dt, stream=0):
    _call("mgcfd_op_get_min_dt", n, _p(dt), _p(min_dt), _p(stream))


def compute_step_factor(n, variables, volumes, min_dt, step_factors, stream=0):
    _call("mgcfd_op_compute_step_factor", n, _p(variables), _p(volumes), _p(min_dt), _p(step_factors), _p(stream))


def compute_flux_edge(nedges, nnodes, edge_to_nodes, variables, edge_weights, smoothing_coefficient, fluxes,
                      stream=0):
    _call("mgcfd_op_compute_flux_edge", nedges, nnodes, _p(edge_to_nodes), _p(variables), _p(edge_weights),
          C.c_double(smoothing_coefficient), _p(fluxes), _p(stream))


def compute_bnd_node_flux(nbnd, nnodes, bnd_to_node, bnd_group, bnd_weights, variables, ff, fluxes, stream=0):
    _call("mgcfd_op_compute_bnd_node_flux", nbnd, nnodes, _p(bnd_to_node), _p(bnd_group), _p(bnd_weights), _p(variables),
          C.byref(ff), _p(fluxes), _p(stream))


def time_step(n, rk, step_factors, fluxes, old_variables, variables, stream=0):
    _call("mgcfd_op_time_step", n, rk, _p(step_factors), _p(fluxes), _p(old_variables), _p(variables), _p(stream))


def unstructured_stream(nedges, nnodes, edge_to_nodes, variables, edge_weights, fluxes, stream=0):
    _call("mgcfd_op_unstructured_stream", nedges, nnodes, _p(edge_to_nodes), _p(variables), _p(edge_weights), _p(fluxes),
          _p(stream))


def residual(n, old_variables, variables, residuals, stream=0):
    _call("mgcfd_op_residual", n, _p(old_variables), _p(variables), _p(residuals), _p(stream))


def calc_rms(n, residuals, rms, stream=0):
    _call("mgcfd_op_calc_rms", n, _p(residuals), _p(rms), _p(stream))


def count_bad_vals(n, variables, count, stream=0):
    _call("mgcfd_op_count_bad_vals", n, _p(variables), _p(count), _p(stream))


def count_differences(n, test, master, count, stream=0):
    _call("mgcfd_op_count_differences", n, _p(test), _p(master), _p(count), _p(stream))


def up_pre(nfine, ncoarse, node_to_mg, coarse_variables, up_scratch, stream=0):
    _call("mgcfd_op_up_pre", nfine, ncoarse, _p(node_to_mg), _p(coarse_variables), _p(up_scratch), _p(stream))


def up(nfine, ncoarse, node_to_mg, fine_variables, coarse_variables, up_scratch, stream=0):
    _call("mgcfd_op_up", nfine, ncoarse, _p(node_to_mg), _p(fine_variables), _p(coarse_variables), _p(up_scratch),
          _p(stream))


def up_post(ncoarse, coarse_variables, up_scratch, stream=0):
    _call("mgcfd_op_up_post", ncoarse, _p(coarse_variables), _p(up_scratch), _p(stream))


def down(nfine, ncoarse, node_to_mg, fine_variables, fine_residuals, fine_coords, coarse_residuals, coarse_coords,
         stream=0):
    _call("mgcfd_op_down", nfine, ncoarse, _p(node_to_mg), _p(fine_variables), _p(fine_residuals), _p(fine_coords),
          _p(coarse_residuals), _p(coarse_coords), _p(stream))


def map_errors(reset=False) -> int:
    """Elements skipped because a map entry was out of range (device counter)."""
    v = C.c_int64()
    _call("mgcfd_op_map_errors", C.byref(v), int(reset))
    return v.value


PLANS = {"off": 0, "auto": 1, "reorder": 2, "caller_order": 3}


def plans_mode(mode="auto"):
    """How plans built from now on order the nodes ("auto", "reorder",
    "caller_order"), or "off" for the plan-free kernels."""
    _call("mgcfd_op_plans_mode", PLANS[mode])


def flux_precision(precision="fp64"):
    """Arithmetic of compute_flux_edge calls through plans: "fp64" (default)
    or "dw" (double-word primitives and fluxes, no atomics; the FP64 bar)."""
    _call("mgcfd_op_flux_precision", {"fp64": 0, "dw": 2}[precision])


def plan_release(map_ptr):
    """Free the plans built from the map at this device address (before the
    map's memory is freed or reused; synchronises the device)."""
    _call("mgcfd_op_plan_release", _p(map_ptr))


def plans_release():
    """Free every cached plan (synchronises the device)."""
    _call("mgcfd_op_plans_release")


def plans_info():
    """{edge_plans, child_plans, reordered, device_bytes} of the plans held."""
    v = [C.c_int64() for _ in range(4)]
    _call("mgcfd_op_plans_info", *[C.byref(x) for x in v])
    return dict(zip(("edge_plans", "child_plans", "reordered", "device_bytes"), (x.value for x in v)))
