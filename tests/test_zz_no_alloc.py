"""mgcfd_op_restrict_noalloc: the restriction entry point that allocates
nothing, for callers that cannot call cudaMalloc (a host framework that owns
all device memory, or code that must not allocate between time steps).

It keeps the per-coarse-node child counts in a fixed array inside the library
instead of a caller buffer, so it is checked against the existing entry
points mgcfd_op_up_pre/up/up_post (which take the counts from the caller) on
two calls in a row: the second call must not see the first call's counts.
This file is collected last so that a failure here leaves every other test
already run."""
import ctypes as C

import numpy as np
import pytest

import mgcfd
from mgcfd import _lib, ops

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _restrict_with_caller_scratch(nfine, ncoarse, node_to_mg, fine, coarse0):
    cv = torch.from_numpy(coarse0.copy()).cuda()
    fv = torch.from_numpy(np.ascontiguousarray(fine)).cuda()
    m = torch.from_numpy(np.ascontiguousarray(node_to_mg)).cuda()
    scratch = torch.zeros(ncoarse, dtype=torch.int32, device="cuda")
    ops.up_pre(nfine, ncoarse, m.data_ptr(), cv.data_ptr(), scratch.data_ptr())
    ops.up(nfine, ncoarse, m.data_ptr(), fv.data_ptr(), cv.data_ptr(), scratch.data_ptr())
    ops.up_post(ncoarse, cv.data_ptr(), scratch.data_ptr())
    torch.cuda.synchronize()
    ops.plan_release(m.data_ptr())  # the map's memory is freed on return
    return cv.cpu().numpy()


def _restrict_noalloc(nfine, ncoarse, node_to_mg, fine, coarse0):
    cv = torch.from_numpy(coarse0.copy()).cuda()
    fv = torch.from_numpy(np.ascontiguousarray(fine)).cuda()
    m = torch.from_numpy(np.ascontiguousarray(node_to_mg)).cuda()
    lib = _lib.load()
    _lib.check(lib.mgcfd_op_restrict_noalloc(nfine, ncoarse, C.c_void_p(m.data_ptr()),
                                             C.c_void_p(fv.data_ptr()), C.c_void_p(cv.data_ptr()), None))
    torch.cuda.synchronize()
    return cv.cpu().numpy()


def _states(rng, ff, n):
    return np.tile(ff, (n, 1)) * (1.0 + 0.01 * rng.standard_normal((n, 5)))


def test_restrict_noalloc_matches_caller_scratch_twice():
    mesh = mgcfd.HostMesh.generate(22, 2, 99)
    F, Cl = mesh.level(0), mesh.level(1)
    rng = np.random.default_rng(3)
    ff = np.array(mgcfd.freestream(0.6, 4.0).ff_variable[:])
    for call in range(2):  # the second call must start from cleared counts
        fine, coarse0 = _states(rng, ff, F.nnodes), _states(rng, ff, Cl.nnodes)
        expect = _restrict_with_caller_scratch(F.nnodes, Cl.nnodes, F.node_to_mg, fine, coarse0)
        got = _restrict_noalloc(F.nnodes, Cl.nnodes, F.node_to_mg, fine, coarse0)
        np.testing.assert_allclose(got, expect, rtol=1e-14, err_msg=f"call {call}")


def test_restrict_noalloc_larger_then_smaller_level():
    """A call on a larger coarse level leaves higher counts in the shared
    array; the next, smaller call must neither see nor use them."""
    mesh = mgcfd.HostMesh.generate(26, 3, 17)
    rng = np.random.default_rng(5)
    ff = np.array(mgcfd.freestream(0.7, 2.0).ff_variable[:])
    for lf in (0, 1):  # level 0 -> 1 (larger coarse level), then level 1 -> 2
        F, Cl = mesh.level(lf), mesh.level(lf + 1)
        fine, coarse0 = _states(rng, ff, F.nnodes), _states(rng, ff, Cl.nnodes)
        expect = _restrict_with_caller_scratch(F.nnodes, Cl.nnodes, F.node_to_mg, fine, coarse0)
        got = _restrict_noalloc(F.nnodes, Cl.nnodes, F.node_to_mg, fine, coarse0)
        np.testing.assert_allclose(got, expect, rtol=1e-14, err_msg=f"fine level {lf}")


def test_restrict_noalloc_skips_and_counts_out_of_range_entries():
    mesh = mgcfd.HostMesh.generate(12, 2, 23)
    F, Cl = mesh.level(0), mesh.level(1)
    rng = np.random.default_rng(9)
    ff = np.array(mgcfd.freestream(0.5, 1.0).ff_variable[:])
    node_to_mg = F.node_to_mg.copy()
    bad = rng.choice(F.nnodes, 5, replace=False)
    node_to_mg[bad[:3]] = Cl.nnodes  # one past the end
    node_to_mg[bad[3:]] = -1
    fine, coarse0 = _states(rng, ff, F.nnodes), _states(rng, ff, Cl.nnodes)
    ops.map_errors(reset=True)
    expect = _restrict_with_caller_scratch(F.nnodes, Cl.nnodes, node_to_mg, fine, coarse0)
    assert ops.map_errors(reset=True) == 2 * len(bad)  # up_pre and up each skip and count them
    got = _restrict_noalloc(F.nnodes, Cl.nnodes, node_to_mg, fine, coarse0)
    assert ops.map_errors(reset=True) == len(bad)
    np.testing.assert_allclose(got, expect, rtol=1e-14)


def test_restrict_noalloc_rejects_oversized_level():
    lib = _lib.load()
    st = lib.mgcfd_op_restrict_noalloc(10, (1 << 20) + 1, None, None, None, None)
    assert st == _lib.ERR_INVALID
    assert "capacity" in lib.mgcfd_last_error().decode()
