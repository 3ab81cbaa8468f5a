"""The device solver against the golden fixtures written by the reference
binary (tests/golden/make_golden.py), at the FP64 parity bar (GPU)."""
import json
from pathlib import Path

import numpy as np
import pytest

import mgcfd
from parity import DELTA_TOL, STATE_TOL, delta_error, state_error

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = sorted(p.stem for p in GOLDEN.glob("*.npz"))


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("increment", ["atomic", "gather"])
def test_solver_matches_reference_fixture(name, increment):
    z = np.load(GOLDEN / f"{name}.npz")
    meta = json.loads(str(z["meta"]))
    mesh = mgcfd.HostMesh.generate(meta["n"], meta["levels"], meta["seed"])
    s = mgcfd.Solver(mesh, meta["mach"], meta["aoa"], increment=increment)
    s.run(meta["cycles"])
    assert s.synchronize() == 0
    x0 = np.array(mgcfd.freestream(meta["mach"], meta["aoa"]).ff_variable[:])
    for l in range(meta["levels"]):
        var = s.fetch(l)
        sf = s.fetch(l, mgcfd.Q_STEP_FACTORS)
        if meta["full"]:
            ref, ref_sf = z[f"variables_L{l}"], z[f"step_factors_L{l}"]
        else:
            idx = z[f"rows_L{l}"]
            var, sf = var[idx], sf[idx]
            ref, ref_sf = z[f"variables_rows_L{l}"], z[f"step_factors_rows_L{l}"]
        assert state_error(var, ref) <= STATE_TOL, (l, state_error(var, ref))
        assert delta_error(var, ref, x0) <= DELTA_TOL, (l, delta_error(var, ref, x0))
        np.testing.assert_allclose(sf, ref_sf, rtol=1e-12)
