"""Autotuner: picks the edge-kernel block size and the increment strategy
(FP64 atomics or the deterministic edge-flux gather) for a mesh or a batch by
timing V-cycles of each candidate on the device, and caches the choice by
problem size and precision."""
from __future__ import annotations

import time

from .solver import Batch, Solver

_CACHE: dict = {}
CANDIDATES = [("atomic", 128), ("atomic", 256), ("gather", 128), ("gather", 256), ("fused", 0)]


def _key(total_nodes: int, precision: str):
    # size class: powers of two of the level-0 node count
    return (max(total_nodes, 1).bit_length(), precision)


def tune(make, total_nodes: int, precision: str = "fp64", cycles: int = 2, candidates=CANDIDATES):
    """make(increment=..., block_size=..., precision=...) -> Solver or Batch.

    Returns (best options dict, {candidate: ms per cycle}).  Results are cached
    per size class and precision."""
    key = _key(total_nodes, precision)
    if key in _CACHE:
        return _CACHE[key]
    timings = {}
    for inc, bs in candidates:
        if inc == "fused" and precision not in ("mixed", "dw"):
            continue  # the fused node-centric stage exists for mixed precision and DW
        s = make(increment=inc, block_size=bs, precision=precision)
        s.run(1)  # warm-up, graph capture
        if s.synchronize() != 0:
            s.close()
            continue
        t0 = time.perf_counter()
        s.run(cycles)
        s.synchronize()
        timings[(inc, bs)] = 1e3 * (time.perf_counter() - t0) / cycles
        s.close()
    best = min(timings, key=timings.get)
    result = ({"increment": best[0], "block_size": best[1], "precision": precision}, timings)
    _CACHE[key] = result
    return result


def tune_solver(mesh, mach, aoa, precision="fp64", **kw):
    n = mesh.level(0).nnodes if hasattr(mesh, "level") else mesh[0].nnodes
    return tune(lambda **o: Solver(mesh, mach, aoa, **o), n, precision, **kw)


def tune_batch(meshes, machs, aoas, precision="fp64", **kw):
    n = sum(m.level(0).nnodes if hasattr(m, "level") else m[0].nnodes for m in meshes)
    return tune(lambda **o: Batch(meshes, machs, aoas, **o), n, precision, **kw)
