"""bench.py's replica timing on several ranks: every rank gets the largest time of any rank
(gloo process group on the CPU, world size 2)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        assert bench.dist_env()[:2] == (rank, world)
        out[rank] = bench.max_over_ranks(1.5 + rank, world)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_on_two_gloo_ranks():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=120)
        assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
        assert dict(out) == {0: 2.5, 1: 2.5}


def test_one_rank_keeps_its_time():
    import bench
    assert bench.max_over_ranks(3.25, 1) == 3.25
