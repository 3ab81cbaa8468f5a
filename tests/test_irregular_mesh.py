"""Irregular meshes (random nodes, parallel and reversed edges, several
boundary entries per node, ignored boundary groups, coarse nodes without
children): the oracle against the reference binary, and the C ABI's host
mesh built from arbitrary arrays."""
import numpy as np
import pytest

import mgcfd
import oracle as O
from irregular import irregular_levels


def test_host_mesh_from_arrays_round_trips_through_files(tmp_path):
    levels = irregular_levels(400, 2, seed=5)
    mesh = mgcfd.HostMesh.from_levels(levels)
    mesh.write(str(tmp_path), "irr_")
    back = mgcfd.HostMesh.load("input.dat", str(tmp_path))
    for l, L in enumerate(levels):
        got = back.level(l)
        for k in ("coords", "edge_to_nodes", "bnd_to_node", "bnd_group", "edge_weights", "bnd_weights"):
            np.testing.assert_array_equal(getattr(got, k), getattr(L, k))
        if L.node_to_mg is not None:
            np.testing.assert_array_equal(got.node_to_mg, L.node_to_mg)


def test_incomplete_levels_are_rejected():
    levels = irregular_levels(100, 2, seed=1)
    levels[0].node_to_mg = None
    with pytest.raises(mgcfd._lib.MgcfdError):
        mgcfd.HostMesh.from_levels(levels)


@pytest.mark.reference
@pytest.mark.parametrize("seed,nl,cycles", [(3, 3, 3), (8, 2, 4)])
def test_oracle_bitwise_equal_to_reference_on_irregular_mesh(tmp_path, reference_available, seed, nl, cycles):
    if not reference_available:
        pytest.skip("reference sources not present on this host")
    levels = irregular_levels(900, nl, seed=seed)
    mgcfd.HostMesh.from_levels(levels).write(str(tmp_path), "irr_")
    r = O.run_reference_binary(tmp_path, cycles, 0.6, 2.0)
    assert r.returncode == 0, r.stderr
    run = O.OracleRun(levels)
    assert run.run(0.6, 2.0, cycles)[0] == 0
    for l in range(nl):
        ref = mgcfd.h5_read(tmp_path / f"solution.variables.L{l}.cycles={cycles}.h5", f"p_variables_result_L{l}")
        np.testing.assert_array_equal(run.get(l, O.Q_VARIABLES), ref)
