"""Multi-rank bench logic on CPU: world_size-2 gloo processes emulate the
replicas-only multi-GPU run (barrier, max over ranks, whole-job value)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, times, out):
    import torch
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    dist.barrier()
    t = torch.tensor([times[rank]], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    import bench

    value, tmax = bench.aggregate([float(t.item())] * world, cells_per_rank=1000, steps=10)
    out[rank] = (value, tmax)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_max_over_ranks():
    world = 2
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()  # no fork of a process that may hold OpenMP threads
    out = mgr.dict()
    times = [0.5, 0.8]
    mp.spawn(_worker, args=(world, port, times, out), nprocs=world, join=True)
    for r in range(world):
        value, tmax = out[r]
        assert tmax == pytest.approx(0.8)
        assert value == pytest.approx(world * 1000 * 10 / 0.8)


def test_aggregate_uses_slowest_rank():
    import bench

    v, t = bench.aggregate([1.0, 2.0, 4.0], cells_per_rank=10, steps=2)
    assert t == 4.0 and v == pytest.approx(3 * 10 * 2 / 4.0)
