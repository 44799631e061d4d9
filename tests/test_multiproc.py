"""World-size-2 checks of the multi-process bench path on CPU (gloo).

The path shards by replica: every rank advances its own copy of the box and
the only cross-rank operations are a barrier and the max of the timed
region."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as tmp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms_local = 100.0 * (rank + 1)
    value, t_max = bench.aggregate(world, 1000, 5, ms_local)
    dist.barrier()
    out[rank] = (value, t_max)
    dist.destroy_process_group()


def test_aggregate_two_ranks_gloo():
    world = 2
    port = _free_port()
    mgr = tmp.get_context("spawn").Manager()
    out = mgr.dict()
    tmp.start_processes(_worker, args=(world, port, out), nprocs=world,
                        start_method="spawn")
    for r in range(world):
        value, t_max = out[r]
        assert t_max == 200.0
        assert value == pytest.approx(world * 1000 * 5 / 0.2)


def test_aggregate_single_rank():
    import bench
    v, t = bench.aggregate(1, 1000, 4, 50.0)
    assert t == 50.0 and v == pytest.approx(1000 * 4 / 0.05)
