"""Serving loop: continuous admission under an HBM budget, overlapping
requests, and identical results alone and in the mix (GPU)."""
import time

import numpy as np
import pytest

import mgcfd
from mgcfd import server
import oracle as O
from parity import MIXED_TOL, STATE_TOL, per_variable_errors, state_error

pytestmark = pytest.mark.gpu

CASES = [(14, 3, 1, 0.4, 1.0), (9, 2, 2, 0.8, 5.0), (18, 3, 3, 0.6, 3.0), (11, 3, 4, 0.3, 0.0), (20, 4, 5, 0.7, 2.0)]


@pytest.fixture(scope="module")
def meshes():
    return [mgcfd.HostMesh.generate(n, nl, seed) for n, nl, seed, _, _ in CASES]


def run_requests(srv, meshes, idx):
    ids = {srv.submit(meshes[i], CASES[i][3], CASES[i][4], want_result=True): i for i in idx}
    srv.drain(300)
    out = {}
    for res, var in srv.poll():
        out[ids[res["id"]]] = (res, var)
    return out


def test_alone_equals_mix_bitwise_with_gather(meshes):
    alone = {}
    for i in range(len(CASES)):
        srv = mgcfd.Server(max_active=1, increment="gather", max_cycles=4)
        alone.update(run_requests(srv, meshes, [i]))
        srv.close()
    srv = mgcfd.Server(max_active=4, increment="gather", max_cycles=4)
    mix = run_requests(srv, meshes, range(len(CASES)))
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(CASES) and st["failed"] == 0 and st["peak_active"] >= 2
    for i in range(len(CASES)):
        ra, va = alone[i]
        rm, vm = mix[i]
        assert ra["status"] == rm["status"] == 0 and ra["cycles"] == rm["cycles"] == 4
        np.testing.assert_array_equal(va, vm)
        ref = O.OracleRun(meshes[i].levels())
        assert ref.run(CASES[i][3], CASES[i][4], 4)[0] == 0
        assert state_error(vm, ref.get(0, O.Q_VARIABLES)) <= STATE_TOL


@pytest.mark.parametrize("accumulation", ["fp64", "pair32"])
def test_served_mixed_alone_equals_mix_bitwise(meshes, accumulation):
    """The served mixed-precision form (fused node-centric stage, FP64 or
    compensated FP32-pair node sums): every request gives the same bits alone
    and in a mix of overlapping requests, and stays within the mixed bar of
    the FP64 oracle."""
    cycles = 4
    alone = {}
    for i in range(len(CASES)):
        srv = mgcfd.Server(max_active=1, precision="mixed", increment="fused", accumulation=accumulation,
                           max_cycles=cycles)
        alone.update(run_requests(srv, meshes, [i]))
        srv.close()
    srv = mgcfd.Server(max_active=4, precision="mixed", increment="fused", accumulation=accumulation,
                       max_cycles=cycles)
    mix = run_requests(srv, meshes, range(len(CASES)))
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(CASES) and st["failed"] == 0 and st["peak_active"] >= 2
    for i in range(len(CASES)):
        ra, va = alone[i]
        rm, vm = mix[i]
        assert ra["status"] == rm["status"] == 0 and ra["cycles"] == rm["cycles"] == cycles
        np.testing.assert_array_equal(va, vm)
        ref = O.OracleRun(meshes[i].levels())
        assert ref.run(CASES[i][3], CASES[i][4], cycles)[0] == 0
        mx, l2 = per_variable_errors(vm, ref.get(0, O.Q_VARIABLES))
        assert mx.max() <= MIXED_TOL and l2.max() <= MIXED_TOL, (i, mx, l2)


def test_served_dw_alone_equals_mix_bitwise(meshes):
    """The served double-word form (fused node-centric stage): the same bits
    alone and in a mix of overlapping requests, at the FP64 bar of the oracle."""
    cycles = 4
    alone = {}
    for i in range(len(CASES)):
        srv = mgcfd.Server(max_active=1, precision="dw", max_cycles=cycles)
        alone.update(run_requests(srv, meshes, [i]))
        srv.close()
    srv = mgcfd.Server(max_active=4, precision="dw", max_cycles=cycles)
    mix = run_requests(srv, meshes, range(len(CASES)))
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(CASES) and st["failed"] == 0 and st["peak_active"] >= 2
    for i in range(len(CASES)):
        ra, va = alone[i]
        rm, vm = mix[i]
        assert ra["status"] == rm["status"] == 0 and ra["cycles"] == rm["cycles"] == cycles
        np.testing.assert_array_equal(va, vm)
        ref = O.OracleRun(meshes[i].levels())
        assert ref.run(CASES[i][3], CASES[i][4], cycles)[0] == 0
        assert state_error(vm, ref.get(0, O.Q_VARIABLES)) <= STATE_TOL


def test_alone_equals_mix_within_tolerance_with_atomics(meshes):
    srv = mgcfd.Server(max_active=1, increment="atomic", max_cycles=3)
    alone = run_requests(srv, meshes, range(3))
    srv.close()
    srv = mgcfd.Server(max_active=3, increment="atomic", max_cycles=3)
    mix = run_requests(srv, meshes, range(3))
    srv.close()
    for i in range(3):
        assert state_error(mix[i][1], alone[i][1]) <= STATE_TOL


def test_budget_admits_one_at_a_time_and_rejects_oversized(meshes):
    small = mgcfd.HostMesh.generate(10, 2, 8)
    one = server.estimate_bytes(small)
    assert server.estimate_bytes(meshes[4]) > 1.5 * one
    srv = mgcfd.Server(hbm_budget_gb=1.5 * one / 2 ** 30, max_active=8, max_cycles=2)  # room for one small request
    ids = [srv.submit(small, 0.5, 1.0) for _ in range(4)]
    big = srv.submit(meshes[4], 0.5, 1.0)
    srv.drain(300)
    results = {r["id"]: r for r, _ in srv.poll()}
    st = srv.stats()
    srv.close()
    assert st["peak_active"] == 1
    assert all(results[i]["status"] == 0 for i in ids)
    assert results[big]["status"] == mgcfd._lib.ERR_BUDGET
    # admitted strictly one after another
    spans = sorted((results[i]["admit_s"], results[i]["finish_s"]) for i in ids)
    assert all(spans[k + 1][0] >= spans[k][1] - 1e-6 for k in range(len(spans) - 1))


def test_later_arrival_overlaps_running_request(meshes):
    big = mgcfd.HostMesh.generate(48, 3, 2)
    srv = mgcfd.Server(max_active=4, max_cycles=400, residual_drop=0.0)
    first = srv.submit(big, 0.5, 1.0)
    t0 = time.perf_counter()
    while srv.stats()["active"] == 0 and time.perf_counter() - t0 < 60:
        time.sleep(0.001)
    second = srv.submit(meshes[0], 0.6, 2.0)
    srv.drain(300)
    res = {r["id"]: r for r, _ in srv.poll()}
    srv.close()
    assert res[first]["status"] == res[second]["status"] == 0
    assert res[second]["admit_s"] < res[first]["finish_s"]  # joined while the first was running
    # and its V-cycles ran on the GPU while the first one's did (CUDA-event
    # timestamps of both requests' first chunk start and last chunk end)
    b1, e1 = res[first]["device_begin_s"], res[first]["device_end_s"]
    b2, e2 = res[second]["device_begin_s"], res[second]["device_end_s"]
    assert 0 <= b1 < e1 and 0 <= b2 < e2
    assert b2 < e1 and b1 < e2


def test_failing_request_does_not_disturb_others(meshes):
    levels = meshes[1].levels()
    bad = [mgcfd.Level(**{k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in L.__dict__.items()
                          if k != "owner"}) for L in levels]
    bad[0].edge_weights[3, :] = np.nan
    srv = mgcfd.Server(max_active=4, increment="gather", max_cycles=3)
    good = srv.submit(meshes[0], CASES[0][3], CASES[0][4], want_result=True)
    broken = srv.submit(bad, 0.5, 1.0)
    srv.drain(300)
    res = {r["id"]: (r, v) for r, v in srv.poll()}
    srv.close()
    assert res[broken][0]["status"] == mgcfd._lib.ERR_BAD_VALUES
    assert res[good][0]["status"] == 0
    ref = O.OracleRun(meshes[0].levels())
    assert ref.run(CASES[0][3], CASES[0][4], 3)[0] == 0
    assert state_error(res[good][1], ref.get(0, O.Q_VARIABLES)) <= STATE_TOL


def test_device_stop_rule_ends_the_solve_at_the_right_cycle(meshes):
    """residual_drop = 10 is met as soon as it is tested (second cycle): the
    server stops there although it has enqueued more cycles, and the result
    is that of a plain 2-cycle solve, bit for bit (gather increment)."""
    srv = mgcfd.Server(max_active=2, increment="gather", max_cycles=50, residual_drop=10.0)
    out = run_requests(srv, meshes, [2])
    srv.close()
    res, var = out[2]
    assert res["status"] == 0 and res["cycles"] == 2
    assert res["rho_rms_first"] > 0 and res["rho_rms_last"] > 0
    s = mgcfd.Solver(meshes[2], CASES[2][3], CASES[2][4], increment="gather")
    s.run(2)
    assert s.synchronize() == 0
    np.testing.assert_array_equal(var, s.fetch(0))
    s.close()


def test_resident_mesh_reused_across_freestreams(meshes):
    """Requests on the same HostMesh reuse its device tables (cache hits),
    and each result equals a fresh solver's for that request's freestream."""
    flows = [(0.5, 1.0), (0.8, 4.0), (0.35, 0.0)]
    srv = mgcfd.Server(max_active=1, increment="gather", max_cycles=3)
    got = {}
    for mach, aoa in flows:
        rid = srv.submit(meshes[1], mach, aoa, want_result=True)
        srv.drain(300)
        for res, var in srv.poll():
            assert res["id"] == rid and res["status"] == 0
            got[(mach, aoa)] = var
    st = srv.stats()
    srv.close()
    assert st["cache_hits"] == 2 and st["cached_solvers"] == 1
    for mach, aoa in flows:
        s = mgcfd.Solver(meshes[1], mach, aoa, increment="gather")
        s.run(3)
        assert s.synchronize() == 0
        np.testing.assert_array_equal(got[(mach, aoa)], s.fetch(0))
        s.close()


def test_idle_meshes_are_evicted_for_new_ones(meshes):
    a, b = meshes[0], meshes[2]
    budget = max(server.estimate_bytes(a), server.estimate_bytes(b)) * 1.5  # one resident mesh at a time
    srv = mgcfd.Server(hbm_budget_gb=budget / 2 ** 30, max_active=2, max_cycles=2)
    for mesh in (a, b, a):
        srv.submit(mesh, 0.5, 1.0)
        srv.drain(300)
    res = [r for r, _ in srv.poll()]
    st = srv.stats()
    srv.close()
    assert [r["status"] for r in res] == [0, 0, 0]
    assert st["cache_hits"] == 0 and st["cached_solvers"] == 1 and st["used_bytes"] <= budget


# Cohorts: small requests that wait together are solved as one batched solver.
COHORT = [(30, 3, 21, 0.5, 2.0), (12, 3, 22, 0.7, 1.0), (9, 3, 23, 0.35, 4.0), (16, 3, 24, 0.8, 0.5),
          (11, 3, 25, 0.6, 3.0), (14, 3, 26, 0.45, 6.0)]


@pytest.fixture(scope="module")
def cohort_meshes():
    return [mgcfd.HostMesh.generate(n, nl, seed) for n, nl, seed, _, _ in COHORT]


def run_cohort_stream(meshes, cases, **opts):
    """One slot, every request queued at once: the first is admitted alone
    and the rest wait behind it, so they are admitted as a cohort."""
    srv = mgcfd.Server(max_active=1, batch_max_meshes=16, batch_max_nodes=10 ** 7, **opts)
    ids = {srv.submit(m, c[3], c[4], want_result=True): i for i, (m, c) in enumerate(zip(meshes, cases))}
    srv.drain(300)
    out = {ids[r["id"]]: (r, v) for r, v in srv.poll()}
    st = srv.stats()
    srv.close()
    return out, st


@pytest.mark.parametrize("opts", [dict(precision="mixed", increment="fused", accumulation="fp64"),
                                  dict(precision="mixed", increment="fused", accumulation="pair32"),
                                  dict(precision="fp64", increment="gather"), dict(precision="dw")])
def test_cohort_results_equal_requests_alone_bitwise(cohort_meshes, opts):
    cycles = 4
    mix, st = run_cohort_stream(cohort_meshes, COHORT, max_cycles=cycles, **opts)
    assert st["cohorts"] >= 1 and st["cohort_requests"] >= 2 and st["failed"] == 0
    for i, (m, c) in enumerate(zip(cohort_meshes, COHORT)):
        srv = mgcfd.Server(max_active=1, max_cycles=cycles, **opts)
        rid = srv.submit(m, c[3], c[4], want_result=True)
        srv.drain(300)
        (ra, va), = [(r, v) for r, v in srv.poll() if r["id"] == rid]
        srv.close()
        rm, vm = mix[i]
        assert ra["status"] == rm["status"] == 0 and ra["cycles"] == rm["cycles"] == cycles
        # The norms are sums over blocks with FP64 atomics (order not fixed,
        # alone or batched); the states are compared bit for bit.
        assert ra["rho_rms_first"] == pytest.approx(rm["rho_rms_first"], rel=1e-12)
        assert ra["rho_rms_last"] == pytest.approx(rm["rho_rms_last"], rel=1e-12)
        np.testing.assert_array_equal(va, vm)
        if opts["precision"] == "mixed":
            ref = O.OracleRun(m.levels())
            assert ref.run(c[3], c[4], cycles)[0] == 0
            mx, l2 = per_variable_errors(vm, ref.get(0, O.Q_VARIABLES))
            assert mx.max() <= MIXED_TOL and l2.max() <= MIXED_TOL
        elif opts["precision"] == "dw":
            ref = O.OracleRun(m.levels())
            assert ref.run(c[3], c[4], cycles)[0] == 0
            assert state_error(vm, ref.get(0, O.Q_VARIABLES)) <= STATE_TOL


def test_cohort_stop_rule_is_per_request(cohort_meshes):
    """residual_drop = 10 is met at every request's second cycle: each stops
    there although the cohort has more cycles enqueued, and its result is a
    plain 2-cycle solve's, bit for bit."""
    mix, st = run_cohort_stream(cohort_meshes, COHORT, increment="gather", max_cycles=50, residual_drop=10.0)
    assert st["cohort_requests"] >= 2
    for i, (m, c) in enumerate(zip(cohort_meshes, COHORT)):
        r, v = mix[i]
        assert r["status"] == 0 and r["cycles"] == 2 and r["rho_rms_first"] > 0
        s = mgcfd.Solver(m, c[3], c[4], increment="gather")
        s.run(2)
        assert s.synchronize() == 0
        np.testing.assert_array_equal(v, s.fetch(0))
        s.close()


def test_failing_request_in_a_cohort_stops_alone(cohort_meshes):
    levels = cohort_meshes[2].levels()
    bad = [mgcfd.Level(**{k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in L.__dict__.items()
                          if k != "owner"}) for L in levels]
    bad[0].edge_weights[5, :] = np.nan
    meshes = list(cohort_meshes)
    meshes[2] = bad
    mix, st = run_cohort_stream(meshes, COHORT, precision="mixed", increment="fused", max_cycles=3)
    assert st["cohort_requests"] >= 2 and st["failed"] == 1
    assert mix[2][0]["status"] == mgcfd._lib.ERR_BAD_VALUES
    for i in (1, 3, 4, 5):
        r, v = mix[i]
        assert r["status"] == 0 and r["cycles"] == 3
        s = mgcfd.Solver(cohort_meshes[i], COHORT[i][3], COHORT[i][4], precision="mixed", increment="fused")
        s.run(3)
        assert s.synchronize() == 0
        np.testing.assert_array_equal(v, s.fetch(0))
        s.close()
