"""Per-loop parity: each mgcfd_op_* entry point (one op_par_loop of
euler3d.cpp) against the oracle's sequential loop, on device buffers in OP2's
dat layout (GPU)."""
import ctypes as C

import numpy as np
import pytest

import mgcfd
from mgcfd import ops
import oracle as O
from parity import STATE_TOL, state_error

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


_KEEP = []  # device buffers live until the module ends, so a data_ptr() never dangles


def dev(a):
    t = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    _KEEP.append(t)
    return t


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


@pytest.fixture(scope="module")
def case():
    mesh = mgcfd.HostMesh.generate(14, 2, 42)
    levels = mesh.levels()
    rng = np.random.default_rng(7)
    ff = O.freestream(0.7, 2.0)
    fv = np.array(ff.ff_variable[:])
    var = np.tile(fv, (levels[0].nnodes, 1)) * (1.0 + 0.01 * rng.standard_normal((levels[0].nnodes, 5)))
    ref = O.OracleRun(levels)
    assert ref.run(0.7, 2.0, 0)[0] == 0  # init only: volumes and damped weights
    return dict(mesh=mesh, levels=levels, var=var, ff=ff, ref=ref, rng=rng)


def test_initialize_zero_dampen_copy(case):
    L0 = case["levels"][0]
    n = L0.nnodes
    v = torch.empty((n, 5), dtype=torch.float64, device="cuda")
    ops.initialize_variables(n, mgcfd.freestream(0.7, 2.0), v.data_ptr())
    exp = np.empty((n, 5))
    O.lib().orc_loop_initialize_variables(n, C.byref(case["ff"]), dp(exp))
    np.testing.assert_array_equal(host(v), exp)
    ops.zero(n, 5, v.data_ptr())
    assert not host(v).any()
    w = dev(L0.edge_weights)
    ops.dampen_ewt(L0.nedges, w.data_ptr())
    exp = L0.edge_weights.copy()
    O.lib().orc_loop_dampen_ewt(L0.nedges, dp(exp))
    np.testing.assert_array_equal(host(w), exp)
    src = dev(case["var"])
    dst = torch.zeros_like(src)
    ops.copy_double(n, src.data_ptr(), dst.data_ptr())
    np.testing.assert_array_equal(host(dst), case["var"])


def test_calculate_cell_volumes(case):
    L0 = case["levels"][0]
    e2n, xyz, w = dev(L0.edge_to_nodes), dev(L0.coords), dev(L0.edge_weights)
    vol = torch.zeros(L0.nnodes, dtype=torch.float64, device="cuda")
    ops.calculate_cell_volumes(L0.nedges, L0.nnodes, e2n.data_ptr(), xyz.data_ptr(), w.data_ptr(), vol.data_ptr())
    ev, ew = np.zeros(L0.nnodes), L0.edge_weights.copy()
    O.lib().orc_loop_calculate_cell_volumes(L0.nedges, ip(L0.edge_to_nodes), dp(L0.coords), dp(ew), dp(ev))
    np.testing.assert_allclose(host(vol), ev, rtol=1e-14)
    np.testing.assert_allclose(host(w), ew, rtol=1e-14, atol=1e-30)


def test_dt_min_step_factor(case):
    L0, ref = case["levels"][0], case["ref"]
    n = L0.nnodes
    vol = ref.get(0, O.Q_VOLUMES)
    v, vd = dev(case["var"]), dev(vol)
    dt = torch.empty(n, dtype=torch.float64, device="cuda")
    ops.calculate_dt(n, v.data_ptr(), vd.data_ptr(), dt.data_ptr())
    edt = np.empty(n)
    O.lib().orc_loop_calculate_dt(n, dp(case["var"]), dp(vol), dp(edt))
    np.testing.assert_allclose(host(dt), edt, rtol=1e-14)
    md = torch.empty(1, dtype=torch.float64, device="cuda")
    ops.get_min_dt(n, dt.data_ptr(), md.data_ptr())
    assert host(md)[0] == host(dt).min()
    np.testing.assert_allclose(host(md)[0], O.lib().orc_loop_get_min_dt(n, dp(edt)), rtol=1e-14)
    sf = torch.empty(n, dtype=torch.float64, device="cuda")
    ops.compute_step_factor(n, v.data_ptr(), vd.data_ptr(), md.data_ptr(), sf.data_ptr())
    np.testing.assert_array_equal(host(sf), host(md)[0] / vol)
    # NaN entries never win the minimum; an empty set gives DBL_MAX.
    dt_nan = dt.clone()
    dt_nan[::7] = float("nan")
    ops.get_min_dt(n, dt_nan.data_ptr(), md.data_ptr())
    assert host(md)[0] == np.nanmin(host(dt_nan))
    ops.get_min_dt(0, dt.data_ptr(), md.data_ptr())
    assert host(md)[0] == np.finfo(np.float64).max


def test_calculate_dt_volume_plan(case):
    """calculate_dt through its volume plan (cube roots cached per vol dat,
    checked against the volumes' bits) gives the plan-free kernel's bits on
    the first call, on a repeat, and after volumes change in place."""
    L0, ref = case["levels"][0], case["ref"]
    n = L0.nnodes
    vol = ref.get(0, O.Q_VOLUMES).copy()
    v, vd = dev(case["var"]), dev(vol)

    def run(mode):
        ops.plans_mode(mode)
        try:
            dt = torch.empty(n, dtype=torch.float64, device="cuda")
            ops.calculate_dt(n, v.data_ptr(), vd.data_ptr(), dt.data_ptr())
            return host(dt)
        finally:
            ops.plans_mode("auto")

    ops.plans_release()
    free = run("off")
    assert ops.plans_info()["device_bytes"] == 0
    np.testing.assert_array_equal(run("auto"), free)
    assert ops.plans_info()["device_bytes"] >= 16 * n
    np.testing.assert_array_equal(run("auto"), free)
    vd[::5] *= 1.5  # in place: the plan must notice the new bits
    vd[3] = float("nan")
    free2 = run("off")
    got = run("auto")
    np.testing.assert_array_equal(got, free2)
    edt = np.empty(n)
    O.lib().orc_loop_calculate_dt(n, dp(case["var"]), dp(host(vd)), dp(edt))
    np.testing.assert_allclose(got, edt, rtol=1e-14)
    assert not np.array_equal(got, free)
    ops.plan_release(vd.data_ptr())
    assert ops.plans_info()["device_bytes"] == 0


@pytest.mark.parametrize("level", [0, 1])
def test_flux_edge_and_boundary(case, level):
    L, ref, ff = case["levels"][level], case["ref"], case["ff"]
    n = L.nnodes
    var = case["var"][:n] if level == 0 else np.tile(np.array(ff.ff_variable[:]), (n, 1)) * 1.002
    ewt, bwt = ref.get(level, O.Q_EWT), ref.get(level, O.Q_BWT)
    flux = torch.zeros((n, 5), dtype=torch.float64, device="cuda")
    ops.compute_flux_edge(L.nedges, n, dev(L.edge_to_nodes).data_ptr(), dev(var).data_ptr(), dev(ewt).data_ptr(),
                          ff.smoothing_coefficient, flux.data_ptr())
    exp = np.zeros((n, 5))
    O.lib().orc_loop_compute_flux_edge(L.nedges, ip(L.edge_to_nodes), dp(var), dp(ewt), C.c_double(ff.smoothing_coefficient),
                                       dp(exp))
    got = host(flux)
    assert state_error(got, exp) <= STATE_TOL, state_error(got, exp)
    ops.compute_bnd_node_flux(L.nbnd, n, dev(L.bnd_to_node).data_ptr(), dev(L.bnd_group).data_ptr(),
                              dev(bwt).data_ptr(), dev(var).data_ptr(), mgcfd.freestream(0.7, 2.0), flux.data_ptr())
    O.lib().orc_loop_compute_bnd_node_flux(L.nbnd, ip(L.bnd_to_node), ip(L.bnd_group), dp(bwt), dp(var),
                                           C.byref(ff), dp(exp))
    got = host(flux)
    assert state_error(got, exp) <= STATE_TOL, state_error(got, exp)


def test_time_step_residual_rms_bad(case):
    L0 = case["levels"][0]
    n = L0.nnodes
    rng = case["rng"]
    old = case["var"]
    flux = rng.standard_normal((n, 5)) * 1e-3
    sf = rng.random(n) + 0.5
    for rk in range(3):
        v = torch.zeros((n, 5), dtype=torch.float64, device="cuda")
        f = dev(flux)
        ops.time_step(n, rk, dev(sf).data_ptr(), f.data_ptr(), dev(old).data_ptr(), v.data_ptr())
        ev, ef = np.zeros((n, 5)), flux.copy()
        O.lib().orc_loop_time_step(n, rk, dp(sf), dp(ef), dp(old), dp(ev))
        np.testing.assert_allclose(host(v), ev, rtol=1e-15)
        assert not host(f).any()
    new = old + flux
    res = torch.empty((n, 5), dtype=torch.float64, device="cuda")
    ops.residual(n, dev(old).data_ptr(), dev(new).data_ptr(), res.data_ptr())
    er = np.empty((n, 5))
    O.lib().orc_loop_residual(n, dp(old), dp(new), dp(er))
    np.testing.assert_array_equal(host(res), er)
    rms = torch.zeros(1, dtype=torch.float64, device="cuda")
    ops.calc_rms(n, res.data_ptr(), rms.data_ptr())
    np.testing.assert_allclose(host(rms)[0], O.lib().orc_loop_calc_rms(n, dp(er)), rtol=1e-12)
    bad = new.copy()
    bad[5, 2] = np.nan
    bad[9, 0] = np.inf
    bad[9, 4] = -np.inf
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    ops.count_bad_vals(n, dev(bad).data_ptr(), cnt.data_ptr())
    assert host(cnt)[0] == O.lib().orc_loop_count_bad_vals(n, dp(bad)) == 3
    test = new.copy()
    test[3, 1] *= 1 + 1e-6
    test[4, 4] *= 1 + 1e-9   # inside the reference tolerance
    cnt.zero_()
    ops.count_differences(n, dev(test).data_ptr(), dev(new).data_ptr(), cnt.data_ptr())
    diff = np.empty((n, 5))
    O.lib().orc_loop_identify_differences(n, dp(test), dp(new), dp(diff))
    assert host(cnt)[0] == O.lib().orc_loop_count_non_zeros(n, dp(diff)) == 1


def test_restrict_prolong(case):
    lv = case["levels"]
    F, Cl = lv[0], lv[1]
    rng = case["rng"]
    fv = case["var"]
    cv0 = np.tile(np.array(case["ff"].ff_variable[:]), (Cl.nnodes, 1))
    cv = dev(cv0)
    scratch = torch.zeros(Cl.nnodes, dtype=torch.int32, device="cuda")
    m = dev(F.node_to_mg)
    ops.up_pre(F.nnodes, Cl.nnodes, m.data_ptr(), cv.data_ptr(), scratch.data_ptr())
    ops.up(F.nnodes, Cl.nnodes, m.data_ptr(), dev(fv).data_ptr(), cv.data_ptr(), scratch.data_ptr())
    ops.up_post(Cl.nnodes, cv.data_ptr(), scratch.data_ptr())
    ecv, esc = cv0.copy(), np.zeros(Cl.nnodes, dtype=np.int32)
    O.lib().orc_loop_up_pre(F.nnodes, ip(F.node_to_mg), dp(ecv), ip(esc))
    O.lib().orc_loop_up(F.nnodes, ip(F.node_to_mg), dp(fv), dp(ecv), ip(esc))
    O.lib().orc_loop_up_post(Cl.nnodes, dp(ecv), ip(esc))
    np.testing.assert_allclose(host(cv), ecv, rtol=1e-14)
    np.testing.assert_array_equal(host(scratch), esc)
    fres = rng.standard_normal((F.nnodes, 5)) * 1e-4
    cres = rng.standard_normal((Cl.nnodes, 5)) * 1e-4
    out = dev(fv)
    ops.down(F.nnodes, Cl.nnodes, m.data_ptr(), out.data_ptr(), dev(fres).data_ptr(), dev(F.coords).data_ptr(),
             dev(cres).data_ptr(), dev(Cl.coords).data_ptr())
    efv = fv.copy()
    O.lib().orc_loop_down(F.nnodes, ip(F.node_to_mg), dp(efv), dp(fres), dp(F.coords), dp(cres), dp(Cl.coords))
    np.testing.assert_allclose(host(out), efv, rtol=1e-14)


def test_unstructured_stream(case):
    L0 = case["levels"][0]
    n = L0.nnodes
    var = case["var"]
    ewt = case["ref"].get(0, O.Q_EWT)
    out = torch.zeros((n, 5), dtype=torch.float64, device="cuda")
    ops.unstructured_stream(L0.nedges, n, dev(L0.edge_to_nodes).data_ptr(), dev(var).data_ptr(), dev(ewt).data_ptr(),
                            out.data_ptr())
    exp = np.zeros((n, 5))
    O.lib().orc_loop_unstructured_stream(L0.nedges, ip(L0.edge_to_nodes), dp(var), dp(ewt), dp(exp))
    np.testing.assert_allclose(host(out), exp, rtol=1e-14)


def test_invalid_arguments_are_rejected(case):
    with pytest.raises(mgcfd._lib.MgcfdError):
        ops.time_step(10, 3, 1, 1, 1, 1)        # rk_cycle out of range
    with pytest.raises(mgcfd._lib.MgcfdError):
        ops.compute_flux_edge(10, 10, 0, 0, 0, 0.1, 0)  # null pointers
    ops.compute_flux_edge(0, 0, 0, 0, 0, 0.1, 0)       # empty set: nothing to do


def test_out_of_range_map_entries_are_skipped(case):
    """A map entry outside [0, nnodes) is range-checked in the kernel: the
    element is skipped and counted, the rest of the loop runs normally."""
    L0, ref, ff = case["levels"][0], case["ref"], case["ff"]
    n = L0.nnodes
    var = case["var"]
    ewt = ref.get(0, O.Q_EWT)
    e2n = L0.edge_to_nodes.copy()
    e2n[3, 0] = n          # one past the end
    e2n[7, 1] = -5         # negative
    ops.map_errors(reset=True)
    flux = torch.zeros((n, 5), dtype=torch.float64, device="cuda")
    ops.compute_flux_edge(L0.nedges, n, dev(e2n).data_ptr(), dev(var).data_ptr(), dev(ewt).data_ptr(),
                          ff.smoothing_coefficient, flux.data_ptr())
    torch.cuda.synchronize()
    assert ops.map_errors(reset=True) == 2
    keep = np.ones(L0.nedges, dtype=bool)
    keep[[3, 7]] = False
    e_ok = np.ascontiguousarray(L0.edge_to_nodes[keep])
    w_ok = np.ascontiguousarray(ewt[keep])
    exp = np.zeros((n, 5))
    O.lib().orc_loop_compute_flux_edge(int(keep.sum()), ip(e_ok), dp(var), dp(w_ok),
                                       C.c_double(ff.smoothing_coefficient), dp(exp))
    assert state_error(host(flux), exp) <= STATE_TOL
