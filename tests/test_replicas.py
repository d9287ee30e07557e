"""The multi-GPU path is replicas only (the step does not shard): bench.py
runs one independent solver per rank and aggregates throughput over the
slowest rank. This checks that aggregation with two gloo ranks on CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys

    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench

    w, r, _ = bench.dist_setup()
    assert (w, r) == (world, rank)
    bench.barrier(w)
    # rank 1 is the slow one: 40 ms vs 10 ms for the same work
    value, ms = bench.replica_throughput(10.0 if rank == 0 else 40.0, w, cells=1000, steps=4)
    out.put((rank, value, ms))
    dist.destroy_process_group()


def test_two_replicas_aggregate_over_the_slowest_rank():
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
    for rank, value, ms in res:
        assert ms == pytest.approx(40.0)
        assert value == pytest.approx(2 * 1000 * 4 / 0.040 / 1e9)
