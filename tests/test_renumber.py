"""Mesh renumbering as a standalone step (mgcfd_renumber_nodes,
mgcfd_host_mesh_renumber, the mgcfd_renumber tool): bit-exact integer work
against the oracle's restatement of the orders, and the reference's contract
that a relabelled mesh gives the same solution, permuted (euler3d.cpp:377)."""
import subprocess

import numpy as np
import pytest

import mgcfd
import oracle as O
import renumber_orders as R
from mgcfd import _build
from parity import STATE_TOL, state_error

FIELDS = ("coords", "edge_to_nodes", "edge_weights", "bnd_to_node", "bnd_group", "bnd_weights", "node_to_mg")


def as_dict(L):
    return {k: getattr(L, k) for k in FIELDS}


@pytest.mark.parametrize("n,seed", [(6, 1), (11, 7), (17, 3)])
def test_morton_order_bitwise(n, seed):
    mesh = mgcfd.HostMesh.generate(n, 1, seed)
    L = mesh.level(0)
    np.testing.assert_array_equal(mgcfd.renumber_nodes("spatial", L.coords), R.morton_order(L.coords))


@pytest.mark.parametrize("n,seed", [(5, 2), (9, 4)])
def test_rcm_order_bitwise(n, seed):
    mesh = mgcfd.HostMesh.generate(n, 1, seed)
    L = mesh.level(0)
    got = mgcfd.renumber_nodes("rcm", L.coords, L.edge_to_nodes)
    np.testing.assert_array_equal(got, R.rcm_order(L.nnodes, L.edge_to_nodes))


def test_rcm_disconnected_components_and_isolated_nodes():
    # two triangles and two isolated nodes
    e2n = np.array([[0, 1], [1, 2], [2, 0], [5, 6], [6, 7], [7, 5]], dtype=np.int32)
    coords = np.zeros((8, 3))
    got = mgcfd.renumber_nodes("rcm", coords, e2n)
    np.testing.assert_array_equal(got, R.rcm_order(8, e2n))
    assert sorted(got.tolist()) == list(range(8))


def test_morton_ties_and_degenerate_boxes():
    coords = np.zeros((7, 3))  # every node at one point: identity (stable)
    np.testing.assert_array_equal(mgcfd.renumber_nodes("spatial", coords), np.arange(7))
    line = np.zeros((9, 3))
    line[:, 1] = np.array([4, 1, 1, 0, 3, 2, 2, 5, 0], dtype=float)  # flat in x and z, ties
    np.testing.assert_array_equal(mgcfd.renumber_nodes("spatial", line), R.morton_order(line))


def test_bad_arguments_are_rejected():
    with pytest.raises(mgcfd._lib.MgcfdError):
        mgcfd.renumber_nodes("rcm", np.zeros((3, 3)), np.array([[0, 3]], dtype=np.int32))
    with pytest.raises(KeyError):
        mgcfd.renumber_nodes("scotch", np.zeros((3, 3)))


@pytest.mark.parametrize("method", ["spatial", "rcm"])
def test_mesh_relabelling_matches_oracle(method):
    mesh = mgcfd.HostMesh.generate(9, 3, 12)
    out = mesh.renumber(method)
    levels = mesh.levels()
    perms = [mgcfd.renumber_nodes(method, L.coords, L.edge_to_nodes) for L in levels]
    for l, L in enumerate(levels):
        want = R.relabel(as_dict(L), perms[l], perms[l + 1] if l + 1 < len(levels) else None)
        got = out.level(l)
        for k, v in want.items():
            np.testing.assert_array_equal(getattr(got, k), v, err_msg=f"level {l} {k}")
        if l + 1 == len(levels):
            assert got.node_to_mg is None


def test_renumbering_is_idempotent_for_spatial_order():
    once = mgcfd.HostMesh.generate(10, 2, 5).renumber("spatial")
    twice = once.renumber("spatial")
    for l in range(2):
        for k in FIELDS:
            a, b = getattr(once.level(l), k), getattr(twice.level(l), k)
            if a is None:
                assert b is None
            else:
                np.testing.assert_array_equal(a, b)


def test_solution_is_invariant_under_relabelling():
    """Oracle solves on the original and the renumbered mesh agree after
    undoing the permutation (only the edge order's rounding differs)."""
    mesh = mgcfd.HostMesh.generate(8, 3, 9)
    out = mesh.renumber("spatial")
    a = O.OracleRun(mesh.levels())
    b = O.OracleRun(out.levels())
    assert a.run(0.6, 2.0, 3)[0] == 0 and b.run(0.6, 2.0, 3)[0] == 0
    for l in range(3):
        perm = mgcfd.renumber_nodes("spatial", mesh.level(l).coords)
        ref = a.get(l, O.Q_VARIABLES)[perm]
        assert state_error(b.get(l, O.Q_VARIABLES), ref) <= STATE_TOL


def test_tool_writes_a_mesh_the_loader_reads_back(tmp_path):
    mesh = mgcfd.HostMesh.generate(7, 2, 31)
    (tmp_path / "in").mkdir()
    (tmp_path / "out").mkdir()
    mesh.write(str(tmp_path / "in"), "m_")
    r = subprocess.run([str(_build.RENUMBER_CLI), "-i", "input.dat", "-d", str(tmp_path / "in"), "-o",
                        str(tmp_path / "out"), "-m", "rcm"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    back = mgcfd.HostMesh.load("input.dat", str(tmp_path / "out"))
    want = mesh.renumber("rcm")
    for l in range(2):
        for k in FIELDS:
            a, b = getattr(back.level(l), k), getattr(want.level(l), k)
            if a is None:
                assert b is None
            else:
                np.testing.assert_array_equal(a, b)
    r = subprocess.run([str(_build.RENUMBER_CLI), "-i", "input.dat", "-d", str(tmp_path / "in")],
                       capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "Usage" in r.stderr


@pytest.mark.reference
@pytest.mark.parametrize("legacy", [False, True])
def test_reference_solution_is_invariant_under_the_tool(tmp_path, reference_available, legacy):
    """The reference binary run on the tool's output (standard or legacy
    ".renumbered" datasets) gives its own solution on the input, permuted."""
    if not reference_available:
        pytest.skip("reference sources not present on this host")
    mesh = mgcfd.HostMesh.generate(8, 2, 17)
    src, dst = tmp_path / "in", tmp_path / "out"
    src.mkdir()
    dst.mkdir()
    mesh.write(str(src), "m_")
    args = [str(_build.RENUMBER_CLI), "-i", "input.dat", "-d", str(src), "-o", str(dst)]
    if legacy:
        args.append("--legacy-datasets")
    assert subprocess.run(args, capture_output=True, timeout=120).returncode == 0
    extra = ["-l"] if legacy else []
    assert O.run_reference_binary(src, 3, 0.7, 4.0).returncode == 0
    assert O.run_reference_binary(dst, 3, 0.7, 4.0, extra_args=extra).returncode == 0
    for l in range(2):
        perm = mgcfd.renumber_nodes("spatial", mesh.level(l).coords)
        a = mgcfd.h5_read(src / f"solution.variables.L{l}.cycles=3.h5", f"p_variables_result_L{l}")
        b = mgcfd.h5_read(dst / f"solution.variables.L{l}.cycles=3.h5", f"p_variables_result_L{l}")
        assert state_error(b, a[perm]) <= STATE_TOL
