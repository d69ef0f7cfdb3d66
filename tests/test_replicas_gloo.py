"""The multi-GPU form of the bench is independent replicas (the iteration has no
exchange step on one GPU per rank): these world_size-2 runs on CPU (gloo) check
the aggregation over ranks and that the reference arm works on rank 0 only."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
mp = pytest.importorskip("torch.multiprocessing")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        # rank r timed (r + 1) * 10 ms for 5 steps of 1000 events
        max_ms, value = bench.replica_value(10.0 * (rank + 1), 1000, 5, world)
        # the reference arm runs on rank 0 only: other ranks return at once
        from jpet_strip.workloads import WORKLOADS

        out = None
        if rank != 0:
            out = bench.reference_arm(None, WORKLOADS["plain-5mm-1M"], world, rank)
        dist.barrier()
        q.put((rank, max_ms, value, out))
    finally:
        dist.destroy_process_group()


def test_replica_aggregation_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, max_ms, value, out in res:
        assert max_ms == pytest.approx(20.0)
        # both ranks' events over the slowest rank's time
        assert value == pytest.approx(2 * 1000 * 5 / 0.020)
        assert out is None


def test_single_rank_value():
    sys.path.insert(0, ROOT)
    import bench

    max_ms, value = bench.replica_value(25.0, 2000, 4, 1)
    assert max_ms == 25.0 and value == pytest.approx(2000 * 4 / 0.025)
