"""Size-independent properties of the oracle's per-loop restatement
(oracle/mgcfd_oracle.c, which follows flux.h, mg.h and time_stepping_kernels.h
term for term), checked on the CPU.  They are the identities the device
kernels are built on:

* an edge flipped end for end with its weight negated gives the same node
  increments, bit for bit (flux.h:41-208 computes end b's increment with
  end a's expressions mirrored), which is what lets the edge tables orient
  every edge a < b and the node-centric stages evaluate an edge from either
  end;
* the increments of one edge cancel between its ends up to rounding, so the
  sum of all node increments is zero to rounding (OP_INC of +f and -f);
* restriction of a constant field is that constant (mg.h:29-64), and the
  time step is old + sf/(RK+1-rk) * flux with the flux zeroed
  (time_stepping_kernels.h:66-86)."""
import ctypes as C

import numpy as np
import pytest

import mgcfd
import oracle as O


def dp(a):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_double))


def ip(a):
    assert a.dtype == np.int32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_int))


@pytest.fixture(scope="module")
def case():
    mesh = mgcfd.HostMesh.generate(12, 2, 11)
    levels = mesh.levels()
    rng = np.random.default_rng(5)
    ff = O.freestream(0.8, 3.0)
    fv = np.array(ff.ff_variable[:])
    var = np.ascontiguousarray(np.tile(fv, (levels[0].nnodes, 1))
                               * (1.0 + 0.05 * rng.standard_normal((levels[0].nnodes, 5))))
    return dict(levels=levels, var=var, ff=ff, rng=rng)


def edge_flux(nn, e2n, var, ewt, sc):
    out = np.zeros((nn, 5))
    O.lib().orc_loop_compute_flux_edge(len(e2n), ip(e2n), dp(var), dp(ewt), C.c_double(sc), dp(out))
    return out


def test_flipped_edges_with_negated_weights_give_the_same_bits(case):
    L, var, ff = case["levels"][0], case["var"], case["ff"]
    e2n = np.ascontiguousarray(L.edge_to_nodes, dtype=np.int32)
    ewt = np.ascontiguousarray(L.edge_weights, dtype=np.float64)
    want = edge_flux(L.nnodes, e2n, var, ewt, ff.smoothing_coefficient)
    flip = case["rng"].random(len(e2n)) < 0.5
    e2 = e2n.copy()
    e2[flip] = e2[flip][:, ::-1]
    w2 = ewt.copy()
    w2[flip] = -w2[flip]
    got = edge_flux(L.nnodes, np.ascontiguousarray(e2), var, np.ascontiguousarray(w2), ff.smoothing_coefficient)
    assert flip.sum() > len(e2n) // 3
    np.testing.assert_array_equal(got, want)


def test_edge_increments_cancel_over_the_mesh(case):
    L, var, ff = case["levels"][0], case["var"], case["ff"]
    e2n = np.ascontiguousarray(L.edge_to_nodes, dtype=np.int32)
    ewt = np.ascontiguousarray(L.edge_weights, dtype=np.float64)
    f = edge_flux(L.nnodes, e2n, var, ewt, ff.smoothing_coefficient)
    scale = np.abs(f).sum(axis=0)
    assert (scale > 0).all()
    assert (np.abs(f.sum(axis=0)) <= 1e-13 * scale).all(), f.sum(axis=0) / scale
    # One edge alone: its two ends' increments are negatives of each other to rounding.
    one = edge_flux(L.nnodes, e2n[:1].copy(), var, ewt[:1].copy(), ff.smoothing_coefficient)
    a, b = e2n[0]
    np.testing.assert_allclose(one[a], -one[b], rtol=4e-16, atol=0)


def test_restriction_of_a_constant_field_is_the_constant(case):
    F, Cl = case["levels"][0], case["levels"][1]
    fv = np.ascontiguousarray(np.tile(np.array(case["ff"].ff_variable[:]), (F.nnodes, 1)))
    cv = np.full((Cl.nnodes, 5), np.nan)
    scratch = np.zeros(Cl.nnodes, dtype=np.int32)
    n2mg = np.ascontiguousarray(F.node_to_mg, dtype=np.int32)
    O.lib().orc_loop_up_pre(F.nnodes, ip(n2mg), dp(cv), ip(scratch))
    O.lib().orc_loop_up(F.nnodes, ip(n2mg), dp(fv), dp(cv), ip(scratch))
    O.lib().orc_loop_up_post(Cl.nnodes, dp(cv), ip(scratch))
    assert (scratch >= 1).all() and scratch.sum() == F.nnodes  # every coarse node has a child
    np.testing.assert_allclose(cv, fv[: Cl.nnodes], rtol=4.5e-16, atol=0)


@pytest.mark.parametrize("rk", [0, 1, 2])
def test_time_step_is_the_rk_update_and_zeroes_the_flux(case, rk):
    n = 257
    rng = np.random.default_rng(rk)
    sf, old = rng.random(n) + 0.5, rng.standard_normal((n, 5))
    flux = rng.standard_normal((n, 5))
    want = old + (sf / (3 + 1 - rk))[:, None] * flux
    v = np.empty((n, 5))
    O.lib().orc_loop_time_step(n, rk, dp(sf), dp(flux), dp(old), dp(v))
    np.testing.assert_array_equal(v, want)
    assert not flux.any()
