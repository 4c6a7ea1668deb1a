"""Multi-process path of the bench on CPU (gloo, world size 2).

The solve does not shard: under torchrun every rank solves its own replica
and the job's rate is the ranks' total work over the slowest rank's time.
These tests run that aggregation across two real processes: the timing
that reaches rank 0 is the maximum over the ranks, the rate counts every
rank's work, and the reference arm's other ranks leave without work.
"""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")

WS = 2


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as sk:
        sk.bind(("127.0.0.1", 0))
        return sk.getsockname()[1]


def _worker(rank, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(WS),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=WS)
    try:
        import bench
        # per-rank step times 1.5 s and 2.5 s: every rank sees the slowest
        t = bench.max_over_ranks(1.5 + rank, WS, "cpu")
        rate = bench.replica_throughput(960000 * 5, WS, t)
        ws, r, local = bench.dist_env()
        # the reference arm: ranks other than 0 return at once
        ref_left = None
        if rank != 0:
            sys.argv = ["bench.py", "--impl", "reference"]
            ref_left = bench.run_reference(bench.parse()) is None
        dist.barrier()
        q.put((rank, t, rate, ws, r, ref_left))
    finally:
        dist.destroy_process_group()


def test_replica_timing_is_the_max_over_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, port, q)) for r in range(WS)]
    for p in procs:
        p.start()
    try:
        res = sorted(q.get(timeout=180) for _ in range(WS))
    finally:
        for p in procs:
            p.join(timeout=60)
    assert [p.exitcode for p in procs] == [0] * WS
    for rank, t, rate, ws, r, ref_left in res:
        assert t == 2.5
        assert rate == pytest.approx(WS * 960000 * 5 / 2.5)
        assert ws == WS and r == rank
        assert ref_left is (None if rank == 0 else True)


def test_single_rank_aggregation_is_identity():
    import bench
    assert bench.max_over_ranks(0.25, 1) == 0.25
    assert bench.replica_throughput(10.0, 1, 2.0) == 5.0
