"""Multi-rank path of bench.py on CPU: world_size 2 over gloo.

Each rank integrates its own network instance (distinct seed); the whole-job
units are the sum over ranks and the time the max over ranks.
"""
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


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    seed = bench.instance_seed(rank)
    units, ms = bench.combine_ranks(1000 * (rank + 1), 10.0 + rank, "cpu")
    q.put((rank, seed, units, ms))
    dist.destroy_process_group()


def test_two_rank_combination():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    seeds = [o[1] for o in out]
    assert len(set(seeds)) == 2
    for _, _, units, ms in out:
        assert units == 3000 and ms == 11.0


def test_single_process_combination_is_identity():
    import bench
    assert bench.combine_ranks(123, 4.5, "cpu") == (123.0, 4.5)
