"""Batched solves: many meshes concatenated into one launch per stage (GPU)."""
import numpy as np
import pytest

import mgcfd
import oracle as O
from parity import MIXED_TOL, STATE_TOL, per_variable_errors, state_error

pytestmark = pytest.mark.gpu

SIZES = [(9, 11), (16, 3), (12, 7), (20, 5), (7, 13), (10, 2)]
MACH = [0.3, 0.5, 0.8, 0.6, 0.45, 0.7]
AOA = [0.0, 3.0, 6.0, 1.5, 4.5, 2.0]


@pytest.fixture(scope="module")
def meshes():
    return [mgcfd.HostMesh.generate(n, 3, seed) for n, seed in SIZES]


@pytest.mark.parametrize("increment", ["atomic", "gather"])
def test_batch_equals_individual_solves(meshes, increment):
    cycles = 3
    b = mgcfd.Batch(meshes, MACH, AOA, increment=increment)
    b.run(cycles)
    assert b.synchronize() == 0
    for m, mesh in enumerate(meshes):
        s = mgcfd.Solver(mesh, MACH[m], AOA[m], increment=increment)
        s.run(cycles)
        assert s.synchronize() == 0
        ref = O.OracleRun(mesh.levels())
        assert ref.run(MACH[m], AOA[m], cycles)[0] == 0
        assert b.mesh_status(m)[0] == 0
        for l in range(3):
            got, alone = b.fetch_mesh(m, l), s.fetch(l)
            if increment == "gather":  # deterministic: the batch does exactly the same arithmetic
                np.testing.assert_array_equal(got, alone)
            assert state_error(got, alone) <= STATE_TOL
            assert state_error(got, ref.get(l, O.Q_VARIABLES)) <= STATE_TOL
            np.testing.assert_allclose(b.fetch_mesh(m, l, mgcfd.Q_STEP_FACTORS), s.fetch(l, mgcfd.Q_STEP_FACTORS),
                                       rtol=1e-13)
    # the concatenated fetch is the meshes' rows in order
    whole = b.fetch(0)
    np.testing.assert_array_equal(whole[: meshes[0].level(0).nnodes], b.fetch_mesh(0, 0))
    for m, rows in enumerate(b.fetch_meshes(1)):
        np.testing.assert_array_equal(rows, b.fetch_mesh(m, 1))


def test_failing_mesh_is_isolated(meshes):
    levels = [m.levels() for m in meshes[:3]]
    poisoned = [mgcfd.Level(**{k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in L.__dict__.items()
                               if k != "owner"}) for L in levels[1]]
    poisoned[0].edge_weights[0, :] = np.nan
    b = mgcfd.Batch([levels[0], poisoned, levels[2]], MACH[:3], AOA[:3])
    b.run(2)
    assert b.synchronize() == 0
    assert b.mesh_status(1)[0] == mgcfd._lib.ERR_BAD_VALUES
    for m in (0, 2):
        assert b.mesh_status(m)[0] == 0
        ref = O.OracleRun(levels[m])
        assert ref.run(MACH[m], AOA[m], 2)[0] == 0
        assert state_error(b.fetch_mesh(m, 0), ref.get(0, O.Q_VARIABLES)) <= STATE_TOL


@pytest.mark.parametrize("increment,accumulation", [("gather", "fp64"), ("fused", "fp64"), ("fused", "pair32")])
def test_mixed_precision_batch(meshes, increment, accumulation):
    b = mgcfd.Batch(meshes, MACH, AOA, precision="mixed", increment=increment, accumulation=accumulation)
    b.run(3)
    assert b.synchronize() == 0
    for m, mesh in enumerate(meshes):
        ref = O.OracleRun(mesh.levels())
        assert ref.run(MACH[m], AOA[m], 3)[0] == 0
        mx, l2 = per_variable_errors(b.fetch_mesh(m, 0), ref.get(0, O.Q_VARIABLES))
        assert mx.max() <= MIXED_TOL and l2.max() <= MIXED_TOL
        if increment == "fused":  # deterministic: equal to the mesh solved alone
            s = mgcfd.Solver(mesh, MACH[m], AOA[m], precision="mixed", increment="fused", accumulation=accumulation)
            s.run(3)
            assert s.synchronize() == 0
            np.testing.assert_array_equal(b.fetch_mesh(m, 0), s.fetch(0))
            s.close()


@pytest.mark.parametrize("increment", ["atomic", "gather"])
def test_residual_norms_match_oracle(meshes, increment):
    """Each mesh's level-0 residual norm (calc_rms_kernel, validation.h:37-44,
    summed over the mesh and taken as sqrt(rms / N) at euler3d.cpp:533-537)
    against the oracle's own calc_rms on its residual after the same cycles:
    the last level-0 smoothing step is the first step of the last cycle in
    both.  Summation order moves the residuals by ~1e-22 against residuals of
    ~1e-6, so the FP64 bar holds for the norms."""
    cycles = 2
    b = mgcfd.Batch(meshes[:4], MACH[:4], AOA[:4], increment=increment)
    b.run(cycles)
    assert b.synchronize() == 0
    for m in range(4):
        st, rms, rho = b.mesh_status(m)
        run = O.OracleRun(meshes[m].levels())
        assert run.run(MACH[m], AOA[m], cycles)[0] == 0
        res = run.get(0, O.Q_RESIDUALS)
        n0 = res.shape[0]
        rms_ref = np.sqrt(O.lib().orc_loop_calc_rms(n0, O.dptr(np.ascontiguousarray(res))) / n0)
        rho_ref = np.sqrt(O.lib().orc_loop_calc_rms(n0, O.dptr(np.ascontiguousarray(
            np.column_stack([res[:, 0], np.zeros((n0, 4))])))) / n0)
        assert st == 0
        assert rms == pytest.approx(rms_ref, rel=STATE_TOL, abs=0.0), (m, rms, rms_ref)
        assert rho == pytest.approx(rho_ref, rel=STATE_TOL, abs=0.0), (m, rho, rho_ref)
        run.close()
