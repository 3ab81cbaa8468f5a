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


def _restrict_with_caller_scratch(F, Cl, fine, coarse0):
    cv = torch.from_numpy(coarse0.copy()).cuda()
    fv = torch.from_numpy(np.ascontiguousarray(fine)).cuda()
    m = torch.from_numpy(np.ascontiguousarray(F.node_to_mg)).cuda()
    scratch = torch.zeros(Cl.nnodes, dtype=torch.int32, device="cuda")
    ops.up_pre(F.nnodes, Cl.nnodes, m.data_ptr(), cv.data_ptr(), scratch.data_ptr())
    ops.up(F.nnodes, Cl.nnodes, m.data_ptr(), fv.data_ptr(), cv.data_ptr(), scratch.data_ptr())
    ops.up_post(Cl.nnodes, cv.data_ptr(), scratch.data_ptr())
    torch.cuda.synchronize()
    return cv.cpu().numpy()


def _restrict_noalloc(F, Cl, fine, coarse0):
    cv = torch.from_numpy(coarse0.copy()).cuda()
    fv = torch.from_numpy(np.ascontiguousarray(fine)).cuda()
    m = torch.from_numpy(np.ascontiguousarray(F.node_to_mg)).cuda()
    lib = _lib.load()
    _lib.check(lib.mgcfd_op_restrict_noalloc(F.nnodes, Cl.nnodes, C.c_void_p(m.data_ptr()),
                                             C.c_void_p(fv.data_ptr()), C.c_void_p(cv.data_ptr()), None))
    torch.cuda.synchronize()
    return cv.cpu().numpy()


def test_restrict_noalloc_matches_caller_scratch_twice():
    mesh = mgcfd.HostMesh.generate(22, 2, 99)
    F, Cl = mesh.level(0), mesh.level(1)
    rng = np.random.default_rng(3)
    ff = np.array(mgcfd.freestream(0.6, 4.0).ff_variable[:])
    for call in range(2):  # the second call must start from cleared counts
        fine = np.tile(ff, (F.nnodes, 1)) * (1.0 + 0.01 * rng.standard_normal((F.nnodes, 5)))
        coarse0 = np.tile(ff, (Cl.nnodes, 1)) * (1.0 + 0.01 * rng.standard_normal((Cl.nnodes, 5)))
        expect = _restrict_with_caller_scratch(F, Cl, fine, coarse0)
        got = _restrict_noalloc(F, Cl, fine, coarse0)
        np.testing.assert_allclose(got, expect, rtol=1e-14, err_msg=f"call {call}")


def test_restrict_noalloc_rejects_oversized_level():
    lib = _lib.load()
    st = lib.mgcfd_op_restrict_noalloc(10, (1 << 20) + 1, None, None, None, None)
    assert st == _lib.ERR_INVALID
    assert "capacity" in lib.mgcfd_last_error().decode()
