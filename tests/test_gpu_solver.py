"""Full V-cycle parity of the device solver against the oracle (GPU)."""
import numpy as np
import pytest

import mgcfd
import oracle as O
from parity import DELTA_TOL, MIXED_TOL, STATE_TOL, delta_error, per_variable_errors, state_error

pytestmark = pytest.mark.gpu


def _oracle(levels, mach, aoa, cycles):
    run = O.OracleRun(levels)
    st, _ = run.run(mach, aoa, cycles)
    assert st == 0
    return run


def _ff(mach, aoa):
    return np.array(O.freestream(mach, aoa).ff_variable[:])


@pytest.mark.parametrize("n,nl,cycles", [(6, 1, 3), (8, 2, 3), (9, 3, 2), (16, 3, 4), (20, 4, 2)])
@pytest.mark.parametrize("increment", ["atomic", "gather"])
def test_small_meshes_fp64(n, nl, cycles, increment):
    mesh = mgcfd.HostMesh.generate(n, nl, 1000 + n)
    levels = mesh.levels()
    mach, aoa = 0.5, 3.0
    ref = _oracle(levels, mach, aoa, cycles)
    s = mgcfd.Solver(mesh, mach, aoa, increment=increment)
    s.run(cycles)
    assert s.synchronize() == 0
    x0 = _ff(mach, aoa)
    for l in range(nl):
        r = ref.get(l, O.Q_VARIABLES)
        x = s.fetch(l)
        assert state_error(x, r) <= STATE_TOL, (l, state_error(x, r))
        assert delta_error(x, r, x0) <= DELTA_TOL, (l, delta_error(x, r, x0))
        np.testing.assert_allclose(s.fetch(l, mgcfd.Q_VOLUMES), ref.get(l, O.Q_VOLUMES), rtol=1e-14)
        np.testing.assert_allclose(s.fetch(l, mgcfd.Q_STEP_FACTORS), ref.get(l, O.Q_STEP_FACTORS), rtol=1e-12)
        np.testing.assert_allclose(s.fetch(l, mgcfd.Q_RESIDUALS), ref.get(l, O.Q_RESIDUALS),
                                   rtol=0, atol=1e-9 * np.abs(ref.get(l, O.Q_RESIDUALS)).max() + 1e-300)


@pytest.mark.parametrize("renumber", ["none", "spatial", "rcm"])
@pytest.mark.parametrize("use_graph", [True, False])
def test_config0_mesh_fp64(renumber, use_graph):
    """48^3, 3 levels, 10 V-cycles, Mach 0.5, 3 degrees: the reference's CPU case."""
    mesh = mgcfd.HostMesh.generate(48, 3, 1234)
    levels = mesh.levels()
    mach, aoa, cycles = 0.5, 3.0, 10
    ref = _oracle(levels, mach, aoa, cycles)
    s = mgcfd.Solver(mesh, mach, aoa, renumber=renumber, use_graph=use_graph)
    s.run(cycles)
    assert s.synchronize() == 0
    st = s.stats()
    assert st.cycles == cycles and st.smoothing_steps == ref.smoothing_steps
    x0 = _ff(mach, aoa)
    for l in range(3):
        r = ref.get(l, O.Q_VARIABLES)
        x = s.fetch(l)
        assert state_error(x, r) <= STATE_TOL
        assert delta_error(x, r, x0) <= DELTA_TOL


def test_mixed_precision_error_bound():
    mesh = mgcfd.HostMesh.generate(32, 3, 77)
    levels = mesh.levels()
    mach, aoa, cycles = 0.8, 3.0, 5
    ref = _oracle(levels, mach, aoa, cycles)
    s = mgcfd.Solver(mesh, mach, aoa, precision="mixed")
    s.run(cycles)
    assert s.synchronize() == 0
    x0 = _ff(mach, aoa)
    for l in range(3):
        r = ref.get(l, O.Q_VARIABLES)
        x = s.fetch(l)
        mx, l2 = per_variable_errors(x, r)  # relative to each variable's magnitude
        assert mx.max() <= MIXED_TOL and l2.max() <= MIXED_TOL, (mx, l2)
        assert delta_error(x, r, x0) <= 1e-4   # FP32 flux: the change itself is right to ~1e-6


def test_mixed_precision_pair_accumulation():
    """MGCFD_ACCUM_PAIR32: node sums in compensated FP32 pairs; same bar
    against the oracle, and within 1e-8 of the FP64-accumulated mixed run."""
    mesh = mgcfd.HostMesh.generate(24, 3, 78)
    levels = mesh.levels()
    mach, aoa, cycles = 0.7, 2.0, 4
    ref = _oracle(levels, mach, aoa, cycles)
    runs = {}
    for acc in ("fp64", "pair32"):
        s = mgcfd.Solver(mesh, mach, aoa, precision="mixed", increment="gather", accumulation=acc)
        s.run(cycles)
        assert s.synchronize() == 0
        runs[acc] = [s.fetch(l) for l in range(3)]
        s.close()
    for l in range(3):
        mx, l2 = per_variable_errors(runs["pair32"][l], ref.get(l, O.Q_VARIABLES))
        assert mx.max() <= MIXED_TOL and l2.max() <= MIXED_TOL, (mx, l2)
        mx, _ = per_variable_errors(runs["pair32"][l], runs["fp64"][l])
        assert mx.max() <= 1e-8, mx


@pytest.mark.parametrize("accumulation", ["fp64", "pair32"])
@pytest.mark.parametrize("n,nl,cycles,host_setup", [(12, 3, 3, False), (17, 2, 2, True), (48, 3, 2, False)])
def test_fused_stage_equals_gather_bitwise(n, nl, cycles, host_setup, accumulation):
    """The fused node-centric stage computes each edge's FP32 flux at both
    ends from the same inputs and sums in the gather order: the gather
    strategy's results bit for bit, on every level."""
    mesh = mgcfd.HostMesh.generate(n, nl, 100 + n)
    out = {}
    for inc in ("gather", "fused"):
        s = mgcfd.Solver(mesh, 0.75, 2.5, precision="mixed", increment=inc, accumulation=accumulation,
                         host_setup=host_setup)
        s.run(cycles)
        assert s.synchronize() == 0
        out[inc] = [s.fetch(l) for l in range(nl)] + [s.fetch(0, mgcfd.Q_RESIDUALS)]
        s.close()
    for a, b in zip(out["gather"], out["fused"]):
        np.testing.assert_array_equal(a, b)


def _dense_levels(n=3000, per_node=20, seed=6):
    """One level of random nodes with `per_node` random edges each: about ten
    edges per node on each side, so a block of 128 nodes holds more a-side
    and b-side edges than the staged id capacity (1,024) and the edge loop
    falls back to global loads past it."""
    rng = np.random.default_rng(seed)
    coords = rng.random((n, 3))
    a = np.repeat(np.arange(n), per_node)
    b = (a + rng.integers(1, n, len(a))) % n
    e = np.stack([a, b], 1)[rng.permutation(len(a))].astype(np.int32)
    d = coords[e[:, 1]] - coords[e[:, 0]]
    w = 1e-3 * d / np.linalg.norm(d, axis=1, keepdims=True)
    bn = rng.choice(n, n // 10, replace=False).astype(np.int32)
    return [mgcfd.Level(coords=coords, edge_to_nodes=np.ascontiguousarray(e), bnd_to_node=bn,
                        bnd_group=rng.integers(0, 8, len(bn)).astype(np.int32),
                        edge_weights=np.ascontiguousarray(w), bnd_weights=rng.normal(size=(len(bn), 3)) * 1e-3,
                        node_to_mg=None)]


@pytest.mark.parametrize("variant", ["stage_neighbour_ids", "edge_parallel_stage"])
@pytest.mark.parametrize("accumulation", ["fp64", "pair32"])
@pytest.mark.parametrize("mesh_kind", ["lattice", "dense"])
def test_fused_stage_variants_give_the_same_bits(mesh_kind, accumulation, variant):
    """The fused stage's variants change only where values travel: neighbour
    ids from shared memory filled by cp.async (global memory past the staged
    capacity), or every edge end of a block computed at once into shared
    memory and summed per node afterwards (in several chunks on the dense
    mesh).  The results are the per-node loop's bits, alone and batched."""
    levels = mgcfd.HostMesh.generate(20, 3, 8).levels() if mesh_kind == "lattice" else _dense_levels()
    out = {}
    for on in (False, True):
        s = mgcfd.Solver(levels, 0.6, 1.5, precision="mixed", increment="fused", accumulation=accumulation,
                         **{variant: on})
        s.run(3)
        assert s.synchronize() == 0
        out[on] = [s.fetch(l) for l in range(len(levels))] + [s.fetch(0, mgcfd.Q_RESIDUALS)]
        s.close()
    for a, b in zip(out[False], out[True]):
        np.testing.assert_array_equal(a, b)
    if mesh_kind == "lattice":
        other = mgcfd.HostMesh.generate(9, 3, 4).levels()
        b = mgcfd.Batch([levels, other], [0.6, 0.4], [1.5, 0.0], precision="mixed", increment="fused",
                        accumulation=accumulation, **{variant: True})
        b.run(3)
        assert b.synchronize() == 0
        for l in range(len(levels)):
            np.testing.assert_array_equal(b.fetch_mesh(0, l), out[False][l])
        b.close()


@pytest.mark.parametrize("host_setup", [False, True])
@pytest.mark.parametrize("kind", ["lattice", "irregular", "dense"])
def test_coloured_increment_matches_oracle_and_repeats_bitwise(kind, host_setup):
    """The coloured FP64 increment (one launch per colour class, plain
    increments): within the FP64 bar of the oracle on every level, and the
    same bits on a second run (no atomics, a fixed order per node)."""
    from irregular import irregular_levels
    levels = {"lattice": lambda: mgcfd.HostMesh.generate(14, 3, 61).levels(),
              "irregular": lambda: irregular_levels(1500, 3, 9),
              "dense": lambda: _dense_levels(per_node=8)}[kind]()
    mach, aoa, cycles = 0.7, 2.0, 3
    runs = []
    for _ in range(2):
        s = mgcfd.Solver(levels, mach, aoa, increment="coloured", host_setup=host_setup)
        s.run(cycles)
        assert s.synchronize() == 0
        runs.append([s.fetch(l) for l in range(len(levels))])
        s.close()
    ref = _oracle(levels, mach, aoa, cycles)
    x0 = _ff(mach, aoa)
    for l in range(len(levels)):
        np.testing.assert_array_equal(runs[0][l], runs[1][l])
        r = ref.get(l, O.Q_VARIABLES)
        assert state_error(runs[0][l], r) <= STATE_TOL, (l, state_error(runs[0][l], r))
        assert delta_error(runs[0][l], r, x0) <= DELTA_TOL


def test_coloured_increment_is_fp64_and_single_mesh():
    mesh = mgcfd.HostMesh.generate(6, 2, 1)
    with pytest.raises(mgcfd._lib.MgcfdError):
        mgcfd.Solver(mesh, 0.5, 0.0, precision="mixed", increment="coloured")
    with pytest.raises(mgcfd._lib.MgcfdError):
        mgcfd.Batch([mesh, mesh], [0.5, 0.6], [0.0, 1.0], increment="coloured")
    # A node with 70 edges needs more colour classes than the 64 the set-up keeps.
    star = _dense_levels(n=200, per_node=1)[0]
    e = np.concatenate([star.edge_to_nodes, np.stack([np.zeros(70), np.arange(1, 71)], 1).astype(np.int32)])
    star.edge_to_nodes = np.ascontiguousarray(e.astype(np.int32))
    d = star.coords[e[:, 1]] - star.coords[e[:, 0]]
    star.edge_weights = np.ascontiguousarray(1e-3 * d / np.linalg.norm(d, axis=1, keepdims=True))
    with pytest.raises(mgcfd._lib.MgcfdError, match="64"):
        mgcfd.Solver([star], 0.5, 0.0, increment="coloured")
    s = mgcfd.Solver([star], 0.5, 0.0, increment="atomic")  # the same mesh is fine otherwise
    s.close()


def test_fused_needs_mixed_precision():
    mesh = mgcfd.HostMesh.generate(6, 1, 1)
    with pytest.raises(mgcfd._lib.MgcfdError):
        mgcfd.Solver(mesh, 0.5, 0.0, precision="fp64", increment="fused")


def test_run_in_pieces_equals_one_run():
    mesh = mgcfd.HostMesh.generate(12, 3, 5)
    a = mgcfd.Solver(mesh, 0.5, 3.0, increment="gather")
    a.run(4)
    assert a.synchronize() == 0
    b = mgcfd.Solver(mesh, 0.5, 3.0, increment="gather")
    b.run(1)
    b.run(3)
    assert b.synchronize() == 0
    for l in range(3):
        np.testing.assert_array_equal(a.fetch(l), b.fetch(l))  # gather strategy is deterministic
    b.reset()
    b.run(4)
    assert b.synchronize() == 0
    np.testing.assert_array_equal(a.fetch(0), b.fetch(0))


def test_negative_volume_reports_negative_dt():
    """Legacy-mode volumes (the "areas" dataset) with a negative entry give
    min_dt < 0; the device detects it (euler3d.cpp:480-484) and the host gets a
    status, the same outcome as the oracle's abort."""
    mesh = mgcfd.HostMesh.generate(8, 2, 3)
    levels = mesh.levels()
    ref = O.OracleRun(levels)
    assert ref.run(0.5, 3.0, 1)[0] == 0
    legacy = []
    for l, L in enumerate(levels):
        vols = ref.get(l, O.Q_VOLUMES).copy()
        if l == 1:
            vols[3] = -vols[3]
        legacy.append(mgcfd.Level(coords=L.coords, edge_to_nodes=L.edge_to_nodes, bnd_to_node=L.bnd_to_node,
                                  bnd_group=L.bnd_group, edge_weights=ref.get(l, O.Q_EWT) / 1e-7,
                                  bnd_weights=L.bnd_weights, node_to_mg=L.node_to_mg, volumes=vols))
    assert O.OracleRun(legacy).run(0.5, 3.0, 2)[0] == 1
    s = mgcfd.Solver(legacy, 0.5, 3.0)
    s.run(2)
    assert s.synchronize() == mgcfd._lib.ERR_NEGATIVE_DT
    assert "min_dt" in mgcfd._lib.load().mgcfd_last_error().decode()


def test_legacy_volumes_match_oracle():
    mesh = mgcfd.HostMesh.generate(10, 2, 11)
    levels = mesh.levels()
    ref = O.OracleRun(levels)
    assert ref.run(0.5, 3.0, 0)[0] == 0
    legacy = [mgcfd.Level(coords=L.coords, edge_to_nodes=L.edge_to_nodes, bnd_to_node=L.bnd_to_node,
                          bnd_group=L.bnd_group, edge_weights=ref.get(l, O.Q_EWT) / 1e-7 * 1.0,
                          bnd_weights=L.bnd_weights, node_to_mg=L.node_to_mg,
                          volumes=ref.get(l, O.Q_VOLUMES) * 1.5)
              for l, L in enumerate(levels)]
    ref2 = _oracle(legacy, 0.5, 3.0, 3)
    s = mgcfd.Solver(legacy, 0.5, 3.0)
    s.run(3)
    assert s.synchronize() == 0
    for l in range(2):
        assert state_error(s.fetch(l), ref2.get(l, O.Q_VARIABLES)) <= STATE_TOL


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nan_state_reports_bad_values(precision):
    # mixed precision uses the fused stage, whose level-0 NaN count is taken
    # in the restriction that follows the step; FP64 counts in the last stage
    mesh = mgcfd.HostMesh.generate(8, 2, 3)
    levels = mesh.levels()
    bad = [mgcfd.Level(**{k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in L.__dict__.items()
                          if k != "owner"}) for L in levels]
    bad[0].edge_weights[0, :] = np.nan  # poisons the flux of two nodes at level 0
    s = mgcfd.Solver(bad, 0.5, 3.0, precision=precision)
    s.run(2)
    assert s.synchronize() == mgcfd._lib.ERR_BAD_VALUES
    assert "Bad variable values" in mgcfd._lib.load().mgcfd_last_error().decode()
    with pytest.raises(mgcfd._lib.MgcfdError):
        s.run(1)


def test_solve_entry_point_matches_solver():
    mesh = mgcfd.HostMesh.generate(10, 2, 9)
    levels = mesh.levels()
    outs = mgcfd.solve(levels, 0.6, 2.0, 3, increment="gather")
    s = mgcfd.Solver(levels, 0.6, 2.0, increment="gather")
    s.run(3)
    assert s.synchronize() == 0
    for l in range(2):
        np.testing.assert_array_equal(outs[l], s.fetch(l))


def _norms(mesh, cycles, **opts):
    s = mgcfd.Solver(mesh, 0.7, 2.0, **opts)
    s.run(cycles)
    st, rms, rho = s.norms()
    assert st == 0
    res = s.fetch(0, mgcfd.Q_RESIDUALS)
    s.close()
    return rms, rho, res


@pytest.mark.parametrize("nl", [1, 3])
def test_level0_norms_match_residuals_and_oracle(nl):
    """rms of the last level-0 step (euler3d.cpp:533-537), taken in the last RK
    stage (FP64, gather) or in the restriction after it (fused stage): both
    equal sqrt(sum res^2 / N) of the residual the solver returns, and the
    FP64 value matches the oracle's residual."""
    mesh = mgcfd.HostMesh.generate(12, nl, 77)
    n0 = mesh.level(0).nnodes
    cycles = 3
    ref = _oracle(mesh.levels(), 0.7, 2.0, cycles)
    r_ref = ref.get(0, O.Q_RESIDUALS)
    rms_ref = np.sqrt(np.sum(r_ref ** 2) / n0)
    rms64, rho64, res64 = _norms(mesh, cycles)
    assert rms64 == pytest.approx(np.sqrt(np.sum(res64 ** 2) / n0), rel=1e-12)
    assert rho64 == pytest.approx(np.sqrt(np.sum(res64[:, 0] ** 2) / n0), rel=1e-12)
    # The residual is the last step's change (~1e-6 against a state of ~1);
    # summation order moves it by ~1e-22, so the FP64 bar applies to its norm.
    assert rms64 == pytest.approx(rms_ref, rel=STATE_TOL, abs=0.0)
    rms_f, rho_f, res_f = _norms(mesh, cycles, precision="mixed", increment="fused")
    rms_g, rho_g, res_g = _norms(mesh, cycles, precision="mixed", increment="gather")
    np.testing.assert_array_equal(res_f, res_g)  # same residuals, norms from different kernels
    assert rms_f == pytest.approx(rms_g, rel=1e-12) and rho_f == pytest.approx(rho_g, rel=1e-12)
    assert rms_f == pytest.approx(np.sqrt(np.sum(res_f ** 2) / n0), rel=1e-12)
