"""The device solver on irregular meshes against the oracle (GPU)."""
import numpy as np
import pytest

import mgcfd
import oracle as O
from irregular import irregular_levels
from parity import DELTA_TOL, MIXED_TOL, STATE_TOL, delta_error, per_variable_errors, state_error

pytestmark = pytest.mark.gpu

MACH, AOA, CYCLES = 0.6, 2.0, 3


@pytest.fixture(scope="module")
def case():
    levels = irregular_levels(3000, 3, seed=11)
    ref = O.OracleRun(levels)
    assert ref.run(MACH, AOA, CYCLES)[0] == 0
    return levels, [ref.get(l, O.Q_VARIABLES) for l in range(3)]


@pytest.mark.parametrize("opts", [dict(increment="atomic"), dict(increment="gather"),
                                  dict(increment="atomic", host_setup=True), dict(increment="gather", renumber="rcm"),
                                  dict(increment="atomic", renumber="none")])
def test_fp64_matches_oracle(case, opts):
    levels, ref = case
    s = mgcfd.Solver(levels, MACH, AOA, **opts)
    s.run(CYCLES)
    assert s.synchronize() == 0
    x0 = np.array(O.freestream(MACH, AOA).ff_variable[:])
    for l in range(3):
        got = s.fetch(l)
        assert state_error(got, ref[l]) <= STATE_TOL
        assert delta_error(got, ref[l], x0) <= DELTA_TOL
    s.close()


@pytest.mark.parametrize("accumulation", ["fp64", "pair32"])
def test_mixed_matches_oracle(case, accumulation):
    levels, ref = case
    out = {}
    for inc in ("gather", "fused"):
        s = mgcfd.Solver(levels, MACH, AOA, precision="mixed", increment=inc, accumulation=accumulation)
        s.run(CYCLES)
        assert s.synchronize() == 0
        out[inc] = [s.fetch(l) for l in range(3)]
        s.close()
    for l in range(3):
        np.testing.assert_array_equal(out["fused"][l], out["gather"][l])
        mx, l2 = per_variable_errors(out["fused"][l], ref[l])
        assert mx.max() <= MIXED_TOL and l2.max() <= MIXED_TOL
