"""The replica aggregation of bench.py under torch.distributed: two gloo
ranks on CPU, each with its own timed region and unit count; rank 0 must
see the slowest rank's time and the sum of the units."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms, units = bench.reduce_over_ranks(10.0 + rank, 100 * (rank + 1))
    out[rank] = (ms, units)
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_take_max_time_and_sum_units():
    world = 2
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        mp.start_processes(_rank, args=(world, _free_port(), out), nprocs=world,
                           start_method="spawn", join=True)
        res = dict(out)
    for r in range(world):
        assert res[r] == (11.0, 300.0)
