"""The reference's V-cycle driven loop by loop through the per-loop entry
points -- mgcfd.LoopSolver runs euler3d.cpp:413-641 as mgcfd_op_* calls on
device dats in OP2 layout -- and the execution plans behind the edge flux and
the restriction (plans.cu), against the oracle (GPU)."""
import ctypes as C

import numpy as np
import pytest

import mgcfd
from mgcfd import ops
import oracle as O
from irregular import irregular_levels
from parity import DELTA_TOL, STATE_TOL, delta_error, state_error

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

MACH, AOA = 0.7, 2.0


def _levels(kind):
    if kind == "lattice":  # node and edge ids randomly permuted, as the generator writes them
        return mgcfd.HostMesh.generate(14, 3, 42).levels()
    if kind == "renumbered":  # Morton order, as after the renumbering tool
        return mgcfd.HostMesh.generate(14, 3, 42).renumber("spatial").levels()
    return irregular_levels(1500, 3, 5)


def _run_loops(levels, cycles, mode, precision="fp64"):
    ops.plans_mode(mode)
    ops.flux_precision(precision)
    s = mgcfd.LoopSolver(levels, MACH, AOA)
    s.run(cycles)
    st, rms = s.synchronize()
    out = [s.fetch(l) for l in range(len(levels))]
    res0 = s.fetch(0, "res")
    info = ops.plans_info()
    s.close()
    assert ops.plans_info()["device_bytes"] == 0  # close() releases every plan it built
    ops.plans_mode("auto")
    ops.flux_precision("fp64")
    return st, rms, out, res0, info


@pytest.mark.parametrize("kind", ["lattice", "renumbered", "irregular"])
@pytest.mark.parametrize("mode,precision", [("reorder", "fp64"), ("caller_order", "fp64"), ("off", "fp64"),
                                            ("reorder", "dw"), ("caller_order", "dw")])
def test_vcycle_through_loops_matches_oracle(kind, mode, precision):
    """Also with the flux calls in the DW form (double-word primitives and
    fluxes through the plans, node-centric, no atomics), at the same bar."""
    levels = _levels(kind)
    cycles = 3
    st, rms, got, res0, info = _run_loops(levels, cycles, mode, precision)
    assert st == 0
    ref = O.OracleRun(levels)
    assert ref.run(MACH, AOA, cycles)[0] == 0
    x0 = np.asarray(list(mgcfd.freestream(MACH, AOA).ff_variable))
    for l in range(len(levels)):
        r = ref.get(l, O.Q_VARIABLES)
        assert state_error(got[l], r) <= STATE_TOL, (l, state_error(got[l], r))
        assert delta_error(got[l], r, x0) <= DELTA_TOL
    r0 = ref.get(0, O.Q_RESIDUALS)
    n0 = r0.shape[0]
    assert rms == pytest.approx(np.sqrt(O.lib().orc_loop_calc_rms(n0, O.dptr(np.ascontiguousarray(r0))) / n0),
                                rel=STATE_TOL, abs=0.0)
    if mode == "off":
        assert info["edge_plans"] == 0 and info["child_plans"] == 0
    else:
        assert info["edge_plans"] == len(levels) and info["child_plans"] == len(levels) - 1
        assert info["reordered"] == (len(levels) if mode == "reorder" else 0)


def test_auto_mode_reorders_only_scattered_numberings():
    """At 100^3 nodes the generator's permuted ids join far-apart nodes and
    the plan reorders; the Morton-renumbered mesh keeps the caller's order."""
    for kind, reordered in (("permuted", 1), ("spatial", 0)):
        mesh = mgcfd.HostMesh.generate(100, 1, 7)
        if kind == "spatial":
            mesh = mesh.renumber("spatial")
        L = mesh.level(0)
        e2n = torch.from_numpy(np.ascontiguousarray(L.edge_to_nodes)).cuda()
        var = torch.from_numpy(np.tile(np.array(mgcfd.freestream(MACH, AOA).ff_variable[:]), (L.nnodes, 1))).cuda()
        w = torch.from_numpy(np.ascontiguousarray(L.edge_weights)).cuda()
        flux = torch.zeros_like(var)
        ops.compute_flux_edge(L.nedges, L.nnodes, e2n.data_ptr(), var.data_ptr(), w.data_ptr(), 0.2, flux.data_ptr())
        torch.cuda.synchronize()
        info = ops.plans_info()
        assert info["edge_plans"] == 1 and info["reordered"] == reordered, (kind, info)
        ops.plan_release(e2n.data_ptr())


def _flux_case(rng, nn, e2n, sc=0.2):
    fv = np.array(mgcfd.freestream(MACH, AOA).ff_variable[:])
    var = np.tile(fv, (nn, 1)) * (1.0 + 0.01 * rng.standard_normal((nn, 5)))
    w = rng.standard_normal((len(e2n), 3)) * 1e-3
    return var, w


def _oracle_flux(e2n, var, w, sc, nn):
    keep = np.all((e2n >= 0) & (e2n < nn), axis=1)
    e_ok, w_ok = np.ascontiguousarray(e2n[keep]), np.ascontiguousarray(w[keep])
    exp = np.zeros((nn, 5))
    O.lib().orc_loop_compute_flux_edge(int(keep.sum()), e_ok.ctypes.data_as(C.POINTER(C.c_int)), O.dptr(var),
                                       O.dptr(w_ok), C.c_double(sc), O.dptr(exp))
    return exp, int((~keep).sum())


@pytest.mark.parametrize("mode", ["reorder", "caller_order"])
@pytest.mark.parametrize("precision", ["fp64", "dw"])
def test_plan_on_disconnected_graph_with_isolated_nodes_and_bad_entries(mode, precision):
    """Two separate lattices, isolated nodes (no edges), parallel and reversed
    edges and out-of-range map entries, all under a random relabelling: the
    Cuthill-McKee search covers every component and leaves isolated nodes at
    the end; skipped edges are counted on every call."""
    rng = np.random.default_rng(11)
    a, b = mgcfd.HostMesh.generate(9, 1, 1).level(0), mgcfd.HostMesh.generate(7, 1, 2).level(0)
    n_iso = 17
    nn = a.nnodes + b.nnodes + n_iso
    e = np.concatenate([a.edge_to_nodes, b.edge_to_nodes + a.nnodes])
    e = np.concatenate([e, e[:40], e[40:60, ::-1]])
    relabel = rng.permutation(nn).astype(np.int32)
    e = relabel[e]
    e[[5, 77]] = [nn, 3]
    e[123, 1] = -2
    e = np.ascontiguousarray(e[rng.permutation(len(e))].astype(np.int32))
    var, w = _flux_case(rng, nn, e)
    exp, nbad = _oracle_flux(e, var, w, 0.2, nn)
    assert nbad == 3
    ops.plans_mode(mode)
    ops.flux_precision(precision)
    ops.map_errors(reset=True)
    d_e, d_v, d_w = (torch.from_numpy(x).cuda() for x in (e, var, w))
    for call in range(2):  # the second call reuses the plan and the weight memo
        flux = torch.zeros((nn, 5), dtype=torch.float64, device="cuda")
        ops.compute_flux_edge(len(e), nn, d_e.data_ptr(), d_v.data_ptr(), d_w.data_ptr(), 0.2, flux.data_ptr())
        torch.cuda.synchronize()
        assert state_error(flux.cpu().numpy(), exp) <= STATE_TOL, call
    assert ops.map_errors(reset=True) == 2 * nbad
    info = ops.plans_info()
    assert info["edge_plans"] == 1 and info["reordered"] == (1 if mode == "reorder" else 0)
    ops.plan_release(d_e.data_ptr())


@pytest.mark.parametrize("precision", ["fp64", "dw"])
def test_weight_memo_follows_changed_weights_and_smoothing(precision):
    """The plan keeps each edge's |w| term for the weight bits it last saw:
    new weights and a new smoothing coefficient give the oracle's fluxes for
    the new inputs, including weights whose halves are not normal numbers."""
    rng = np.random.default_rng(4)
    L = mgcfd.HostMesh.generate(12, 1, 9).level(0)
    e = np.ascontiguousarray(L.edge_to_nodes)
    nn = L.nnodes
    var, w = _flux_case(rng, nn, e)
    d_e, d_v = torch.from_numpy(e).cuda(), torch.from_numpy(var).cuda()
    ops.plans_mode("reorder")
    ops.flux_precision(precision)
    w2 = w * 1.5
    w2[3] = [0.0, 1e-3, -1e-3]          # a zero component
    w2[8] = [5e-324, 1e-3, 2e-308]      # subnormal / smallest normal components
    for weights, sc in ((w, 0.2), (w, 0.2), (w2, 0.2), (w2, 0.35), (w, 0.35)):
        d_w = torch.from_numpy(np.ascontiguousarray(weights)).cuda()
        flux = torch.zeros((nn, 5), dtype=torch.float64, device="cuda")
        ops.compute_flux_edge(len(e), nn, d_e.data_ptr(), d_v.data_ptr(), d_w.data_ptr(), sc, flux.data_ptr())
        exp, _ = _oracle_flux(e, var, weights, sc, nn)
        torch.cuda.synchronize()
        assert state_error(flux.cpu().numpy(), exp) <= STATE_TOL
    ops.plan_release(d_e.data_ptr())


def test_dw_and_fp64_flux_calls_share_a_plan():
    """FP64 and DW calls alternate on one plan while the weights change: each
    keeps its own memo, both stay within the FP64 bar of the oracle, and the
    DW form gives the same bits on every call (no atomics)."""
    rng = np.random.default_rng(17)
    L = mgcfd.HostMesh.generate(11, 1, 3).level(0)
    e = np.ascontiguousarray(L.edge_to_nodes)
    nn = L.nnodes
    var, w = _flux_case(rng, nn, e)
    d_e, d_v = torch.from_numpy(e).cuda(), torch.from_numpy(var).cuda()
    ops.plans_mode("reorder")
    dw_bits = {}
    for k, (weights, prec) in enumerate(((w, "fp64"), (w, "dw"), (w * 2, "fp64"), (w * 2, "dw"), (w, "dw"),
                                         (w, "fp64"), (w * 2, "dw"))):
        ops.flux_precision(prec)
        d_w = torch.from_numpy(np.ascontiguousarray(weights)).cuda()
        flux = torch.zeros((nn, 5), dtype=torch.float64, device="cuda")
        ops.compute_flux_edge(len(e), nn, d_e.data_ptr(), d_v.data_ptr(), d_w.data_ptr(), 0.2, flux.data_ptr())
        got = flux.cpu().numpy()
        exp, _ = _oracle_flux(e, var, weights, 0.2, nn)
        assert state_error(got, exp) <= STATE_TOL, (k, prec)
        if prec == "dw":
            key = float(weights[0, 0])
            if key in dw_bits:
                np.testing.assert_array_equal(got, dw_bits[key])
            dw_bits[key] = got
    assert ops.plans_info()["edge_plans"] == 1
    ops.flux_precision("fp64")
    ops.plan_release(d_e.data_ptr())


def test_restriction_plan_is_a_deterministic_gather():
    """up_pre/up/up_post through the children plan: the oracle's sums bit for
    bit (children added in fine-node order), counts equal, and coarse nodes
    without children keep their state (mg.h:58)."""
    levels = irregular_levels(1200, 2, 3)
    F, Cl = levels[0], levels[1]
    rng = np.random.default_rng(2)
    fv = rng.standard_normal((F.nnodes, 5))
    cv0 = rng.standard_normal((Cl.nnodes, 5))
    m = torch.from_numpy(np.ascontiguousarray(F.node_to_mg)).cuda()
    d_fv = torch.from_numpy(fv).cuda()
    for call in range(2):
        cv = torch.from_numpy(cv0.copy()).cuda()
        scratch = torch.full((Cl.nnodes,), 7, dtype=torch.int32, device="cuda")
        ops.up_pre(F.nnodes, Cl.nnodes, m.data_ptr(), cv.data_ptr(), scratch.data_ptr())
        ops.up(F.nnodes, Cl.nnodes, m.data_ptr(), d_fv.data_ptr(), cv.data_ptr(), scratch.data_ptr())
        ops.up_post(Cl.nnodes, cv.data_ptr(), scratch.data_ptr())
        ecv, esc = cv0.copy(), np.full(Cl.nnodes, 7, dtype=np.int32)
        ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))  # noqa: E731
        O.lib().orc_loop_up_pre(F.nnodes, ip(F.node_to_mg), O.dptr(ecv), ip(esc))
        O.lib().orc_loop_up(F.nnodes, ip(F.node_to_mg), O.dptr(fv), O.dptr(ecv), ip(esc))
        O.lib().orc_loop_up_post(Cl.nnodes, O.dptr(ecv), ip(esc))
        torch.cuda.synchronize()
        np.testing.assert_array_equal(cv.cpu().numpy(), ecv)
        np.testing.assert_array_equal(scratch.cpu().numpy(), esc)
    assert ops.plans_info()["child_plans"] == 1
    ops.plan_release(m.data_ptr())
    assert ops.plans_info()["child_plans"] == 0


def test_plan_on_a_chain_longer_than_the_search_cap():
    """A chain of 20,000 nodes has as many breadth-first levels; the search
    stops at its cap (16,384 levels) and the rest follows in id order, with
    the same fluxes."""
    rng = np.random.default_rng(21)
    nn = 20000
    relabel = rng.permutation(nn).astype(np.int32)
    e = np.ascontiguousarray(relabel[np.stack([np.arange(nn - 1), np.arange(1, nn)], 1)].astype(np.int32))
    var, w = _flux_case(rng, nn, e)
    exp, _ = _oracle_flux(e, var, w, 0.2, nn)
    ops.plans_mode("reorder")
    d_e, d_v, d_w = (torch.from_numpy(x).cuda() for x in (e, var, w))
    flux = torch.zeros((nn, 5), dtype=torch.float64, device="cuda")
    ops.compute_flux_edge(len(e), nn, d_e.data_ptr(), d_v.data_ptr(), d_w.data_ptr(), 0.2, flux.data_ptr())
    torch.cuda.synchronize()
    assert state_error(flux.cpu().numpy(), exp) <= STATE_TOL
    assert ops.plans_info()["reordered"] == 1
    ops.plan_release(d_e.data_ptr())
