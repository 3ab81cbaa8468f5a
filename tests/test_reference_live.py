"""Live comparison against the reference binary (the unmodified reference
euler3d.cpp built against the sequential OP2 stand-in).  Runs only where the
reference sources are present; elsewhere the committed golden fixtures carry
the same evidence (test_golden_oracle.py)."""
import numpy as np
import pytest

import mgcfd
import oracle as O

pytestmark = pytest.mark.reference


@pytest.fixture(autouse=True)
def _need_reference(reference_available):
    if not reference_available:
        pytest.skip("reference sources not present on this host")


@pytest.mark.parametrize("n,nl,seed,mach,aoa,cycles", [(7, 2, 3, 0.7, 1.0, 3), (10, 3, 11, 0.4, 5.0, 2),
                                                       (5, 2, 1, 1.2, 0.0, 6)])
def test_oracle_bitwise_equal_to_reference(tmp_path, n, nl, seed, mach, aoa, cycles):
    mesh = mgcfd.HostMesh.generate(n, nl, seed)
    mesh.write(str(tmp_path), "m_")
    r = O.run_reference_binary(tmp_path, cycles, mach, aoa)
    assert r.returncode == 0, r.stderr
    assert "Max total runtime" in r.stdout
    run = O.OracleRun(mesh.levels())
    assert run.run(mach, aoa, cycles)[0] == 0
    for l in range(nl):
        ref = mgcfd.h5_read(tmp_path / f"solution.variables.L{l}.cycles={cycles}.h5", f"p_variables_result_L{l}")
        np.testing.assert_array_equal(run.get(l, O.Q_VARIABLES), ref)


def test_reference_validation_flow_accepts_its_own_solution(tmp_path):
    """euler3d.cpp:658-718: -v compares against solution.variables.L*.cycles=N.h5."""
    mesh = mgcfd.HostMesh.generate(9, 2, 4)
    mesh.write(str(tmp_path), "m_")
    assert O.run_reference_binary(tmp_path, 3, 0.5, 3.0).returncode == 0
    r = O.run_reference_binary(tmp_path, 3, 0.5, 3.0, extra_args=["-v"], prefix="again.")
    assert r.returncode == 0
    assert "Validation passed" in r.stdout


def test_measure_mem_bound_flag_leaves_solution_unchanged(tmp_path):
    mesh = mgcfd.HostMesh.generate(8, 2, 6)
    mesh.write(str(tmp_path), "m_")
    assert O.run_reference_binary(tmp_path, 2, 0.5, 3.0, prefix="a.").returncode == 0
    assert O.run_reference_binary(tmp_path, 2, 0.5, 3.0, extra_args=["-b"], prefix="b.").returncode == 0
    for l in range(2):
        a = mgcfd.h5_read(tmp_path / f"a.variables.L{l}.cycles=2.h5", f"p_variables_result_L{l}")
        b = mgcfd.h5_read(tmp_path / f"b.variables.L{l}.cycles=2.h5", f"p_variables_result_L{l}")
        np.testing.assert_array_equal(a, b)


def test_legacy_mode_files(tmp_path):
    """-l reads "areas" and "edge_weights.recalculated" (euler3d.cpp:247-309);
    with those written as misc.h:40-76 computes them, legacy and non-legacy
    runs agree bit for bit, and so does the oracle fed the legacy arrays."""
    mesh = mgcfd.HostMesh.generate(8, 2, 21)
    mesh.write(str(tmp_path), "m_", legacy_datasets=True)
    assert O.run_reference_binary(tmp_path, 2, 0.5, 3.0, prefix="a.").returncode == 0
    r = O.run_reference_binary(tmp_path, 2, 0.5, 3.0, extra_args=["-l"], prefix="b.")
    assert r.returncode == 0, r.stdout + r.stderr
    legacy = mgcfd.HostMesh.load("input.dat", str(tmp_path), legacy=True)
    run = O.OracleRun(legacy.levels())
    assert run.run(0.5, 3.0, 2)[0] == 0
    for l in range(2):
        a = mgcfd.h5_read(tmp_path / f"a.variables.L{l}.cycles=2.h5", f"p_variables_result_L{l}")
        b = mgcfd.h5_read(tmp_path / f"b.variables.L{l}.cycles=2.h5", f"p_variables_result_L{l}")
        np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(run.get(l, O.Q_VARIABLES), b)


def test_reference_solution_unchanged_by_flipped_edges(tmp_path):
    """The reference itself, on a mesh whose edges are partly stored end for
    end: calculate_cell_volumes (misc.h:40-76) uses each input weight's
    magnitude only and re-derives its direction from b - a, and flux.h:41-208
    mirrors end a's expressions for end b, so the solution is the same bit
    for bit.  This is the identity behind the device tables' a < b
    orientation and the node-centric stages (each edge evaluated from either
    end)."""
    mesh = mgcfd.HostMesh.generate(9, 2, 8)
    levels = mesh.levels()
    rng = np.random.default_rng(2)
    flipped = []
    for L in levels:
        flip = rng.random(L.nedges) < 0.5
        e2n = np.array(L.edge_to_nodes, dtype=np.int32, copy=True)
        e2n[flip] = e2n[flip][:, ::-1]
        w = np.array(L.edge_weights, copy=True)
        w[flip] = -w[flip]  # any sign: only |w| is read
        flipped.append(mgcfd.Level(coords=np.array(L.coords), edge_to_nodes=np.ascontiguousarray(e2n),
                                   bnd_to_node=np.array(L.bnd_to_node), bnd_group=np.array(L.bnd_group),
                                   edge_weights=np.ascontiguousarray(w), bnd_weights=np.array(L.bnd_weights),
                                   node_to_mg=None if L.node_to_mg is None else np.array(L.node_to_mg),
                                   n_axis=L.n_axis))
    (tmp_path / "a").mkdir()
    (tmp_path / "b").mkdir()
    mesh.write(str(tmp_path / "a"), "m_")
    mgcfd.HostMesh.from_levels(flipped).write(str(tmp_path / "b"), "m_")
    for d in ("a", "b"):
        r = O.run_reference_binary(tmp_path / d, 3, 0.7, 2.0)
        assert r.returncode == 0, r.stderr
    for l in range(len(levels)):
        a = mgcfd.h5_read(tmp_path / "a" / f"solution.variables.L{l}.cycles=3.h5", f"p_variables_result_L{l}")
        b = mgcfd.h5_read(tmp_path / "b" / f"solution.variables.L{l}.cycles=3.h5", f"p_variables_result_L{l}")
        np.testing.assert_array_equal(a, b)
