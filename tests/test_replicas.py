"""The N>1 path of bench.py runs independent replicas (the time-stepping
path does not shard): ranks meet only at a barrier and a max-over-ranks
reduction of their timings.  World size 2 on gloo, CPU only."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench.barrier(dist)
    t = bench.max_over_ranks(dist, 1.0 + rank * 0.5)
    out.put((rank, t))
    dist.destroy_process_group()


def test_max_over_ranks_world2():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == {0: 1.5, 1: 1.5}


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.dist_init(1)[:2] == (0, 1)
    assert bench.max_over_ranks(None, 2.5) == 2.5
