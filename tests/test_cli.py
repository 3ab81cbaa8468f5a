"""euler3d_gb300, the euler3d-compatible driver (config.h, euler3d.cpp:69-826)."""
import json
import subprocess
from pathlib import Path

import numpy as np
import pytest

import mgcfd
from mgcfd import _build
from parity import STATE_TOL, state_error

GOLDEN = Path(__file__).resolve().parent / "golden"


def cli(*args, cwd=None):
    return subprocess.run([str(_build.CLI), *map(str, args)], cwd=cwd, capture_output=True, text=True, timeout=600)


def test_help_and_missing_input():
    r = cli("-h")
    assert r.returncode == 1 and "Usage" in r.stderr
    r = cli()
    assert r.returncode == 1 and "input_file not set" in r.stdout


def test_bad_deck_is_reported(tmp_path):
    (tmp_path / "input.dat").write_text("size=1\nnum_levels=1\nmesh_name=nope\n[levels]\n0=a.h5\n")
    r = cli("-i", "input.dat", "-d", tmp_path)
    assert r.returncode == 1 and "Unknown mesh_name" in r.stderr


def test_config_file_keys(tmp_path):
    (tmp_path / "run.conf").write_text("# comment\ninput_file=missing.dat\ncycles=3\nbogus=1\n")
    r = cli("-c", tmp_path / "run.conf")
    assert "Unknown key 'bogus'" in r.stdout
    assert r.returncode == 1 and "Could not open input file" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [[], ["--precision", "dw"]], ids=["fp64", "dw"])
def test_run_output_and_validate_against_reference_fixture(tmp_path, precision):
    """The driver's --output-variables files match the reference's solution
    (golden fixture), and -v accepts them as the reference's -v would; the
    double-word form (--precision dw) at the same bar."""
    z = np.load(GOLDEN / "lattice9_l3_c3.npz")
    meta = json.loads(str(z["meta"]))
    mesh = mgcfd.HostMesh.generate(meta["n"], meta["levels"], meta["seed"])
    mesh.write(str(tmp_path), "m_")
    args = ["-i", "input.dat", "-d", tmp_path, "-g", meta["cycles"], *precision, "--mach", meta["mach"],
            "--aoa", meta["aoa"]]
    r = cli(*args, "--output-variables", "--output-step-factors", "-o", f"{tmp_path}/solution.")
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count("Performing MG cycle") == meta["cycles"] and "Max total runtime" in r.stdout
    for l in range(meta["levels"]):
        got = mgcfd.h5_read(tmp_path / f"solution.variables.L{l}.cycles={meta['cycles']}.h5",
                            f"p_variables_result_L{l}")
        assert state_error(got, z[f"variables_L{l}"]) <= STATE_TOL
        sf = mgcfd.h5_read(tmp_path / f"solution.step_factors.L{l}.cycles={meta['cycles']}.h5",
                           f"p_step_factors_result_L{l}")
        np.testing.assert_allclose(sf.reshape(-1), z[f"step_factors_L{l}"], rtol=1e-12)
    r = cli(*args, "-v")
    assert r.returncode == 0 and "Validation passed" in r.stdout, r.stdout
    r = cli(*args[:-4], "-v", "--mach", 0.3, "--aoa", 0.0)  # different flow: must fail validation
    assert "Validation failed" in r.stdout


@pytest.mark.gpu
def test_flow_interval_snapshots(tmp_path):
    mesh = mgcfd.HostMesh.generate(8, 2, 4)
    mesh.write(str(tmp_path), "m_")
    r = cli("-i", "input.dat", "-d", tmp_path, "-g", 4, "-I", 2, "-o", f"{tmp_path}/snap.", "--mach", 0.5)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count("Performing MG cycle") == 4
    a = mgcfd.h5_read(tmp_path / "snap.variables.L0.cycle=2.h5", "p_variables")
    b = mgcfd.h5_read(tmp_path / "snap.variables.L0.cycle=4.h5", "p_variables")
    assert a.shape == (512, 5) and not np.array_equal(a, b)
    assert not (tmp_path / "snap.variables.L0.cycle=1.h5").exists()


@pytest.mark.gpu
def test_legacy_mode_and_mem_bound_flag(tmp_path):
    mesh = mgcfd.HostMesh.generate(8, 2, 21)
    mesh.write(str(tmp_path), "m_", legacy_datasets=True)
    outs = []
    for extra in ([], ["-l"], ["-b"], ["-n"]):
        pre = f"{tmp_path}/o{len(outs)}."
        r = cli("-i", "input.dat", "-d", tmp_path, "-g", 2, "--mach", 0.5, "--aoa", 3.0, "--output-variables",
                "-o", pre, *extra)
        assert r.returncode == 0, r.stdout + r.stderr
        outs.append(mgcfd.h5_read(f"{pre}variables.L0.cycles=2.h5", "p_variables_result_L0"))
    for o in outs[1:]:
        assert state_error(o, outs[0]) <= STATE_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("extra", [["--precision", "mixed"], ["--precision", "mixed", "--accumulation", "pair32"],
                                   ["--precision", "mixed", "--increment", "gather"]])
def test_mixed_precision_flags(tmp_path, extra):
    """--precision mixed (with the increment and accumulation choices) stays
    within the mixed-precision bar of the FP64 run's solution files."""
    from parity import MIXED_TOL, per_variable_errors
    mesh = mgcfd.HostMesh.generate(10, 2, 33)
    mesh.write(str(tmp_path), "m_")
    base = ["-i", "input.dat", "-d", tmp_path, "-g", 3, "--mach", 0.6, "--aoa", 2.0, "--output-variables"]
    assert cli(*base, "-o", f"{tmp_path}/f.").returncode == 0
    r = cli(*base, "-o", f"{tmp_path}/m.", *extra)
    assert r.returncode == 0, r.stdout + r.stderr
    for l in range(2):
        a = mgcfd.h5_read(tmp_path / f"f.variables.L{l}.cycles=3.h5", f"p_variables_result_L{l}")
        b = mgcfd.h5_read(tmp_path / f"m.variables.L{l}.cycles=3.h5", f"p_variables_result_L{l}")
        mx, l2 = per_variable_errors(b, a)
        assert mx.max() <= MIXED_TOL and l2.max() <= MIXED_TOL
        assert not np.array_equal(a, b)  # the flag took effect


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [[], ["--precision", "dw"]], ids=["fp64", "dw"])
def test_per_loop_run_matches_reference_fixture(tmp_path, precision):
    """--per-loop runs the reference's loop sequence through the mgcfd_op_*
    entry points on OP2-layout dats: its solution files match the reference's
    (golden fixture) and -v accepts them; with --precision dw the flux calls
    run in the DW form, at the same bar."""
    z = np.load(GOLDEN / "lattice9_l3_c3.npz")
    meta = json.loads(str(z["meta"]))
    mesh = mgcfd.HostMesh.generate(meta["n"], meta["levels"], meta["seed"])
    mesh.write(str(tmp_path), "m_")
    args = ["-i", "input.dat", "-d", tmp_path, "-g", meta["cycles"], "--mach", meta["mach"], "--aoa", meta["aoa"],
            "--per-loop", *precision]
    r = cli(*args, "--output-variables", "--output-step-factors", "--output-fluxes", "-o", f"{tmp_path}/solution.")
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count("Performing MG cycle") == meta["cycles"] and "Max total runtime" in r.stdout
    for l in range(meta["levels"]):
        got = mgcfd.h5_read(tmp_path / f"solution.variables.L{l}.cycles={meta['cycles']}.h5",
                            f"p_variables_result_L{l}")
        assert state_error(got, z[f"variables_L{l}"]) <= STATE_TOL
        sf = mgcfd.h5_read(tmp_path / f"solution.step_factors.L{l}.cycles={meta['cycles']}.h5",
                           f"p_step_factors_result_L{l}")
        np.testing.assert_allclose(sf.reshape(-1), z[f"step_factors_L{l}"], rtol=1e-12)
        fx = mgcfd.h5_read(tmp_path / f"solution.fluxes.L{l}.cycles={meta['cycles']}.h5", f"p_fluxes_result_L{l}")
        assert not fx.any()  # time_step_kernel leaves the fluxes at zero (time_stepping_kernels.h:84)
    r = cli(*args, "-v")
    assert r.returncode == 0 and "Validation passed" in r.stdout, r.stdout


@pytest.mark.gpu
def test_per_loop_flags_match_the_solver(tmp_path):
    """-l (legacy datasets), -b (unstructured_stream each stage) and -I
    (level-0 snapshots) through the per-loop entry points give the device
    solver's results; --precision mixed is refused with --per-loop."""
    mesh = mgcfd.HostMesh.generate(8, 2, 21)
    mesh.write(str(tmp_path), "m_", legacy_datasets=True)
    base = ["-i", "input.dat", "-d", tmp_path, "-g", 4, "--mach", 0.5, "--aoa", 3.0, "--output-variables"]
    for extra in ([], ["-l"], ["-b"], ["-I", 2]):
        outs = []
        for mode in ([], ["--per-loop"]):
            pre = f"{tmp_path}/{'p' if mode else 's'}{len(extra)}{''.join(map(str, extra))}."
            r = cli(*base, "-o", pre, *extra, *mode)
            assert r.returncode == 0, r.stdout + r.stderr
            outs.append([mgcfd.h5_read(f"{pre}variables.L{l}.cycles=4.h5", f"p_variables_result_L{l}")
                         for l in range(2)])
            if extra == ["-I", 2]:
                snap = mgcfd.h5_read(f"{pre}variables.L0.cycle=2.h5", "p_variables")
                outs[-1].append(snap)
        for a, b in zip(outs[0], outs[1]):
            assert state_error(b, a) <= STATE_TOL, extra
    r = cli(*base, "-o", f"{tmp_path}/x.", "--per-loop", "--precision", "mixed")
    assert r.returncode == 1 and "--per-loop" in r.stdout
