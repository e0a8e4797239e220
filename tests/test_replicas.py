"""The replica path of bench.py (N GPUs = N independent replicas): the job-wide value
uses the slowest rank's time and the edges of all ranks. Two gloo ranks on the CPU."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms, edges = bench.reduce_over_ranks(10.0 + 5.0 * rank, 1000.0 * (rank + 1), torch.device("cpu"), world)
    out[rank] = (ms, edges)
    dist.destroy_process_group()


def test_reduce_over_ranks_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world, port = 2, _free_port()
    with mp.Manager() as mgr:
        out = mgr.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        assert res[r] == (15.0, 3000.0)


def test_reduce_over_ranks_single():
    import bench
    assert bench.reduce_over_ranks(7.0, 42, None, 1) == (7.0, 42.0)
