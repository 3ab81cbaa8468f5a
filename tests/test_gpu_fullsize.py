"""Parity at the benchmark's full size: the 200^3 lattice (8,000,000 nodes,
23,880,000 edges, 4 levels) at Mach 0.8 and 3 degrees.

The oracle's OpenMP form (coloured edges on every host core) runs this mesh
at about half a V-cycle per second on 16 cores, so the FP64 path and the
double-word form are checked against it directly over the 25 V-cycles the
workload names (about a minute); the other checks are size-independent properties: the fused
mixed-precision stage equals the gather stage bit for bit, mixed precision
stays within 1e-6 of FP64 after 25 V-cycles (the mixed-precision workload),
and renumbering the nodes only relabels the solution."""
import os

import numpy as np
import pytest

import mgcfd
import oracle as O
from parity import DELTA_TOL, MIXED_TOL, STATE_TOL, delta_error, per_variable_errors, state_error

pytestmark = pytest.mark.gpu

N, LEVELS, SEED, MACH, AOA = 200, 4, 20240501, 0.8, 3.0


@pytest.fixture(scope="module")
def mesh():
    return mgcfd.HostMesh.generate(N, LEVELS, SEED)


def _solve(mesh, cycles, **opts):
    s = mgcfd.Solver(mesh, MACH, AOA, **opts)
    s.run(cycles)
    assert s.synchronize() == 0
    out = [s.fetch(l) for l in range(LEVELS)]
    s.close()
    return out


@pytest.fixture(scope="module")
def oracle25(mesh):
    ref = O.OracleRun(mesh.levels())
    assert ref.run(MACH, AOA, 25, nthreads=os.cpu_count() or 1)[0] == 0
    out = [ref.get(l, O.Q_VARIABLES) for l in range(LEVELS)]
    ref.close()
    return out


@pytest.mark.parametrize("opts", [dict(), dict(precision="dw", increment="fused")], ids=["fp64", "dw_fused"])
def test_matches_oracle_at_8m_nodes(mesh, oracle25, opts):
    """FP64, and the double-word form at the same bar, over the workload's 25 V-cycles."""
    got = _solve(mesh, 25, **opts)
    x0 = np.asarray(list(mgcfd.freestream(MACH, AOA).ff_variable))
    for l in range(LEVELS):
        assert state_error(got[l], oracle25[l]) <= STATE_TOL, (l, state_error(got[l], oracle25[l]))
        assert delta_error(got[l], oracle25[l], x0) <= DELTA_TOL


def test_fused_equals_gather_at_8m_nodes(mesh):
    a = _solve(mesh, 2, precision="mixed", increment="gather")
    b = _solve(mesh, 2, precision="mixed", increment="fused")
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


def test_mixed_precision_error_after_25_cycles(mesh):
    ref = _solve(mesh, 25)
    got = _solve(mesh, 25, precision="mixed")
    for l in range(LEVELS):
        mx, l2 = per_variable_errors(got[l], ref[l])
        assert mx.max() <= MIXED_TOL and l2.max() <= MIXED_TOL, (l, mx, l2)


def test_renumbering_only_relabels(mesh):
    a = _solve(mesh, 2, renumber="none")
    b = _solve(mesh, 2, renumber="spatial")
    for l in range(LEVELS):
        assert state_error(b[l], a[l]) <= STATE_TOL
