"""Parity metrics shared by the tests.

The bar for the FP64 path is relative 1e-10 against the oracle:
    err_state = max over nodes of |x - r| / max(|r|, column scale)
where the column scale is the largest |r| of that variable on the level (so a
variable that is near zero everywhere, like w-momentum at zero sideslip, is
judged against its own magnitude rather than against 0).  Because the damped
edge weights keep the state near freestream, the change from the initial
state is also compared:
    err_delta = max |(x - x0) - (r - x0)| / max |r - x0|
"""
import numpy as np

STATE_TOL = 1e-10     # FP64 drop-in bar
DELTA_TOL = 1e-7      # FP64: rounding noise relative to the change the solver made
MIXED_TOL = 1e-6      # mixed precision bar on the final state


def state_error(x, r):
    x = np.asarray(x, dtype=np.float64).reshape(r.shape)
    r = np.asarray(r, dtype=np.float64)
    if r.ndim == 1:
        r = r[:, None]
        x = x[:, None]
    scale = np.maximum(np.abs(r), np.abs(r).max(axis=0, keepdims=True) * 1e-3)
    scale = np.where(scale == 0, 1.0, scale)
    return float(np.max(np.abs(x - r) / scale))


def delta_error(x, r, x0):
    x = np.asarray(x, dtype=np.float64).reshape(r.shape)
    d_ref = r - x0
    denom = np.abs(d_ref).max(axis=0)
    denom = np.where(denom == 0, 1.0, denom)
    return float(np.max(np.abs((x - x0) - d_ref).max(axis=0) / denom))


def per_variable_errors(x, r):
    """Max and L2 relative error per variable (density, 3 momenta, energy)."""
    x = np.asarray(x).reshape(r.shape)
    mx = np.abs(x - r).max(axis=0) / np.maximum(np.abs(r).max(axis=0), 1e-300)
    l2 = np.sqrt(((x - r) ** 2).sum(axis=0)) / np.maximum(np.sqrt((r ** 2).sum(axis=0)), 1e-300)
    return mx, l2
