"""The oracle against the golden fixtures written by the reference binary
(tests/golden/make_golden.py), and the mesh generator against the fixtures'
array digests.  CPU only."""
import hashlib
import json
import platform
from pathlib import Path

import numpy as np
import pytest

import mgcfd
import oracle as O
from parity import STATE_TOL, state_error

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = sorted(p.stem for p in GOLDEN.glob("*.npz"))
EXACT = platform.machine() in ("x86_64", "AMD64")  # fixtures were written on x86_64


def load(name):
    z = np.load(GOLDEN / f"{name}.npz")
    return json.loads(str(z["meta"])), z


def same(a, b):
    if EXACT:
        np.testing.assert_array_equal(a, b)
    else:
        np.testing.assert_allclose(a, b, rtol=1e-12, atol=0)


@pytest.mark.parametrize("name", CASES)
def test_generator_reproduces_fixture_mesh(name):
    meta, _ = load(name)
    mesh = mgcfd.HostMesh.generate(meta["n"], meta["levels"], meta["seed"])
    for l, L in enumerate(mesh.levels()):
        for key, digest in meta["mesh_sha256"].items():
            lev, arr = key.split(".")
            if lev != f"L{l}":
                continue
            got = hashlib.sha256(np.ascontiguousarray(getattr(L, arr)).tobytes()).hexdigest()
            assert got == digest, key


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_fixture(name):
    meta, z = load(name)
    mesh = mgcfd.HostMesh.generate(meta["n"], meta["levels"], meta["seed"])
    run = O.OracleRun(mesh.levels())
    st, _ = run.run(meta["mach"], meta["aoa"], meta["cycles"])
    assert st == 0
    for l in range(meta["levels"]):
        var = run.get(l, O.Q_VARIABLES)
        sf = run.get(l, O.Q_STEP_FACTORS)
        if meta["full"]:
            same(var, z[f"variables_L{l}"])
            same(sf, z[f"step_factors_L{l}"])
        else:
            idx = z[f"rows_L{l}"]
            same(var[idx], z[f"variables_rows_L{l}"])
            same(sf[idx], z[f"step_factors_rows_L{l}"])
            stats = np.stack([var.sum(axis=0), (var * var).sum(axis=0), var.min(axis=0), var.max(axis=0)])
            np.testing.assert_allclose(stats, z[f"stats_L{l}"], rtol=1e-15 if EXACT else 1e-12)


def test_openmp_oracle_close_to_sequential():
    mesh = mgcfd.HostMesh.generate(16, 3, 8)
    levels = mesh.levels()
    a, b = O.OracleRun(levels), O.OracleRun(levels)
    assert a.run(0.5, 3.0, 3)[0] == 0
    assert b.run(0.5, 3.0, 3, nthreads=4)[0] == 0
    for l in range(3):
        assert state_error(b.get(l, O.Q_VARIABLES), a.get(l, O.Q_VARIABLES)) <= STATE_TOL
