"""Multi-GPU is replicas only: every rank runs its own allocator and nothing on
the data path is exchanged.  What bench.py does across ranks — a barrier
around the timed region, the slowest rank's time, the sum of all ranks' ops —
is host logic; it runs here with world_size 2 on the gloo backend (CPU)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.barrier(world)
        secs = bench.max_over_ranks(1.0 + rank, world)     # rank 1 is the slow one
        ops = bench.sum_over_ranks(100.0 * (rank + 1), world)
        q.put((rank, secs, ops, ops / secs))
    finally:
        dist.destroy_process_group()


def test_replica_reductions_world2():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, secs, ops, value in got:
        assert secs == 2.0 and ops == 300.0 and value == 150.0


def test_single_rank_passthrough():
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.sum_over_ranks(7.0, 1) == 7.0
