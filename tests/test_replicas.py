"""Replica aggregation across ranks (gloo, world size 2, CPU): a barrier and
the job throughput = all ranks' units / the slowest rank's time."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    from mgcfd import replicas
    dist = replicas.init("gloo")
    replicas.barrier(dist)
    thr, tmax = replicas.job_throughput(10.0 * (rank + 1), [1.5, 2.5][rank], dist)
    out.put((rank, thr, tmax))
    dist.destroy_process_group()


def test_two_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, thr, tmax in res:
        assert tmax == 2.5
        assert thr == pytest.approx(30.0 / 2.5)


def test_single_process_needs_no_group(monkeypatch):
    from mgcfd import replicas
    monkeypatch.delenv("WORLD_SIZE", raising=False)
    assert replicas.init() is None
    assert replicas.job_throughput(8.0, 2.0, None) == (4.0, 2.0)
