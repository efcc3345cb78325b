"""The multi-GPU form is replicas only: each rank evaluates its own slice of
the parameter vectors, and the only exchange is bench.py's timing barrier
and max over ranks.  Exercised here with world size 2 over gloo on CPU."""
import os

import numpy as np
import pytest
import torch.multiprocessing as mp


def _rank(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port), XPSI_BENCH_BACKEND="gloo")
    import bench
    import torch.distributed as dist
    r, w = bench.dist_init()
    assert (r, w) == (rank, world)
    bench.barrier(w)
    # each rank reports a different step time; every rank sees the maximum
    t = bench.max_over_ranks(0.25 + rank, w)
    shard = bench.shard_vectors(4, r, w)
    out.put((rank, t, shard))
    dist.destroy_process_group()


def test_replicas_shard_and_time_over_gloo():
    world, port = 2, 29517 + os.getpid() % 1000
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = {}
    for _ in range(world):
        rank, t, shard = q.get(timeout=120)
        res[rank] = (t, shard)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert all(t == pytest.approx(1.25) for t, _ in res.values())
    from xpsi_gb300 import synthetic as SY
    full = SY.config3_vectors(8, seed=3)
    np.testing.assert_array_equal(np.concatenate([res[0][1], res[1][1]]), full)
