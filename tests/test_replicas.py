"""The multi-rank path of bench.py on CPU: world_size 2 over gloo.  Each
rank runs an independent scan (replicas, no data exchange); the job's time
is the slowest rank's and its rate counts every rank's units."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r "took" 10 (r + 1) ms over 5 scans of 1e6 units
        slow_ms = bench.max_over_ranks(10.0 * (rank + 1), dist, "cpu")
        dist.barrier()
        q.put((rank, slow_ms, bench.whole_job_rate(1e6, 5, world, slow_ms * 1e-3)))
    finally:
        dist.destroy_process_group()


def test_replicas_time_the_slowest_rank():
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r for r, _, _ in got] == [0, 1]
    for _, slow_ms, rate in got:
        assert slow_ms == 20.0
        assert rate == pytest.approx(1e6 * 5 * 2 / 0.020)


def test_single_rank_needs_no_group():
    import bench

    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.whole_job_rate(10.0, 2, 1, 4.0) == 5.0
