"""The multi-GPU layout is replicas: each rank evaluates its own parameter
vectors and the slowest rank's time counts.  This checks bench.py's
cross-rank reduction with two gloo ranks on the CPU."""
import os

import pytest
import torch.multiprocessing as mp


def _worker(rank, world, port, q):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    dev_ms, wall, span = bench.reduce_over_ranks([10.0 + rank, 1.0 + 2 * rank, 5.0 - rank], dist, device="cpu")
    evals = bench.whole_job_evals(batch=4, steps=3, world=world)
    q.put((rank, dev_ms, wall, span, evals))
    dist.destroy_process_group()


def test_two_rank_reduction():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29517
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, dev_ms, wall, span, evals in out:
        assert dev_ms == 11.0 and wall == 3.0 and span == 5.0
        assert evals == 24
