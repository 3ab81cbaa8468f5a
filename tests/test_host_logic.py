"""Host-side logic that needs no GPU: the autotuner's choice and cache (driven
by stand-in solvers with set timings), and the server's HBM admission
estimate (a host function of the C ABI)."""
import ctypes as C
import time

import pytest

import mgcfd
from mgcfd import _lib, autotune, server


class FakeRun:
    """Stands in for a Solver or Batch: run() sleeps for the candidate's set
    time per cycle; synchronize() returns the candidate's status."""

    made = []

    def __init__(self, ms_per_cycle, status=0, **opts):
        self.ms, self.status, self.opts = ms_per_cycle, status, opts
        self.closed = False
        FakeRun.made.append(self)

    def run(self, cycles):
        time.sleep(self.ms * 1e-3 * cycles)

    def synchronize(self):
        return self.status

    def close(self):
        self.closed = True


def maker(table, status=None):
    status = status or {}

    def make(increment, block_size, precision):
        key = (increment, block_size)
        return FakeRun(table[key], status.get(key, 0), increment=increment, block_size=block_size,
                       precision=precision)
    return make


@pytest.fixture(autouse=True)
def clean_cache():
    autotune._CACHE.clear()
    FakeRun.made.clear()
    yield
    autotune._CACHE.clear()


def test_autotune_picks_the_fastest_candidate_and_closes_every_run():
    table = {("atomic", 128): 30, ("atomic", 256): 25, ("gather", 128): 8, ("gather", 256): 20, ("fused", 0): 1}
    best, timings = autotune.tune(maker(table), 1000, "fp64", cycles=1)
    assert best == {"increment": "gather", "block_size": 128, "precision": "fp64"}
    # The fused stage exists for mixed precision only: never tried in FP64.
    assert ("fused", 0) not in timings and len(timings) == 4
    assert all(r.closed for r in FakeRun.made)
    best, _ = autotune.tune(maker(table), 1000, "mixed", cycles=1)
    assert best["increment"] == "fused"
    # ... and for the double-word form.
    best, timings = autotune.tune(maker(table), 1000, "dw", cycles=1)
    assert best == {"increment": "fused", "block_size": 0, "precision": "dw"} and len(timings) == 5


def test_autotune_skips_failed_candidates():
    table = {("atomic", 128): 1, ("atomic", 256): 25, ("gather", 128): 5, ("gather", 256): 25, ("fused", 0): 1}
    best, timings = autotune.tune(maker(table, status={("atomic", 128): _lib.ERR_NEGATIVE_DT}), 1000, "fp64",
                                  cycles=1)
    assert ("atomic", 128) not in timings
    assert (best["increment"], best["block_size"]) == ("gather", 128)


def test_autotune_caches_by_size_class_and_precision():
    table = {("atomic", 128): 1, ("atomic", 256): 2, ("gather", 128): 2, ("gather", 256): 2, ("fused", 0): 2}
    first = autotune.tune(maker(table), 1000, "fp64", cycles=1)
    made = len(FakeRun.made)
    # Same power-of-two size class (512..1023 nodes), same precision: cached, nothing rebuilt.
    assert autotune.tune(maker(table), 600, "fp64", cycles=1) is first
    assert len(FakeRun.made) == made
    # Another size class or precision is tuned afresh.
    autotune.tune(maker(table), 5000, "fp64", cycles=1)
    autotune.tune(maker(table), 1000, "mixed", cycles=1)
    assert len(FakeRun.made) == made + 4 + 5


def test_server_estimate_grows_with_mesh_and_strategy():
    small, big = mgcfd.HostMesh.generate(8, 2, 1), mgcfd.HostMesh.generate(16, 3, 1)
    atomic = server.estimate_bytes(small, "fp64", "atomic")
    assert atomic > 1 << 20
    assert server.estimate_bytes(big, "fp64", "atomic") > 4 * (atomic - (1 << 20))
    # Per-edge fluxes (gather) and the FP32 copies (mixed) cost memory.
    assert server.estimate_bytes(small, "fp64", "gather") > atomic
    assert server.estimate_bytes(small, "mixed", "atomic") > atomic
    # auto means atomics in FP64 and the fused stage in mixed precision.
    assert server.estimate_bytes(small, "fp64", "auto") == atomic
    assert server.estimate_bytes(small, "mixed", "auto") == server.estimate_bytes(small, "mixed", "fused")
    # DW: the pair-word primitives and weights on top of FP64's arrays; auto is the fused stage.
    assert server.estimate_bytes(small, "dw", "atomic") > atomic
    assert server.estimate_bytes(small, "dw", "auto") == server.estimate_bytes(small, "dw", "fused")
    assert server.estimate_bytes(small, "dw", "fused") > server.estimate_bytes(small, "dw", "atomic")


def test_server_estimate_rejects_bad_arguments():
    lib = _lib.load()
    out = C.c_int64()
    assert lib.mgcfd_request_estimate_bytes(0, None, 0, 0, C.byref(out)) == _lib.ERR_INVALID
    views = mgcfd.level_views_from_arrays(mgcfd.HostMesh.generate(8, 2, 1).levels())
    assert lib.mgcfd_request_estimate_bytes(2, views, 0, 0, None) == _lib.ERR_INVALID
    with pytest.raises(_lib.MgcfdError):
        _lib.check(lib.mgcfd_request_estimate_bytes(0, None, 0, 0, C.byref(out)))
