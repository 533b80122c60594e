"""Host-side logic of the multi-rank bench (replicas: one independent job per
GPU, no data-path collective) on two CPU ranks over gloo: barrier, the
max-over-ranks time and the whole-job aggregate."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist

    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    ws, r, local = bench.dist_env()
    d = bench.init_dist(ws, "gloo")
    bench.barrier(d)
    ms = 100.0 + 50.0 * rank          # rank 1 is the slow one
    worst = bench.max_over_ranks(d, ms)
    total = bench.sum_over_ranks(d, 7.0)
    V, steps = 1000, 4
    value = ws * V * steps / (worst / 1e3)
    q.put((rank, ws, worst, total, value))
    bench.barrier(d)
    dist.destroy_process_group()


def test_two_rank_replica_aggregation():
    import torch.multiprocessing as mp
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
    for rank, ws, worst, total, value in res:
        assert ws == 2 and worst == 150.0 and total == 14.0
        assert value == pytest.approx(2 * 1000 * 4 / 0.150)
