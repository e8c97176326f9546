"""Replica timing across ranks on the CPU (gloo, world size 2): the bench's
rank setup, barrier and max-over-ranks reduction that turn N independent
replicas of the suffix-sort step into one whole-job number.  No data moves
between ranks; only the step times are reduced."""
import multiprocessing as mp
import os
import socket

import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out):
    os.environ.update({"WORLD_SIZE": str(world), "RANK": str(rank), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    import bench
    w, r, local, dist = bench.dist_setup()
    try:
        bench.barrier(dist)
        step_s = 0.010 * (r + 1)                 # rank 1 is the slower replica
        slowest = bench.reduce_max(dist, step_s)
        n = 1 << 20
        value = w * n / 1e6 / slowest            # whole-job MB/s, as bench.py reports it
        out.put((r, w, local, slowest, value))
    finally:
        dist.destroy_process_group()


def test_two_replicas_reduce_to_the_slowest():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r for r, *_ in res] == [0, 1]
    for r, w, local, slowest, value in res:
        assert w == 2 and local == r
        assert slowest == pytest.approx(0.020)
        assert value == pytest.approx(2 * (1 << 20) / 1e6 / 0.020)


def test_single_process_has_no_group(monkeypatch):
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    import bench
    w, r, local, dist = bench.dist_setup()
    assert (w, r, local, dist) == (1, 0, 0, None)
    assert bench.reduce_max(dist, 1.25) == 1.25
