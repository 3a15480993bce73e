"""The N > 1 benchmark path: replicas, max-over-ranks timing (gloo, 2 ranks on CPU)."""
import os
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    vals = bench.aggregate_over_ranks([10.0 + rank, 5.0 - rank])
    dist.barrier()
    out.put((rank, vals))
    dist.destroy_process_group()


def test_aggregate_over_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 1000)
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert res[0] == res[1] == [11.0, 5.0]


def test_aggregate_single_process():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.aggregate_over_ranks([1.0, 2.0]) == [1.0, 2.0]
