"""Multi-rank host logic (replicas only: no data-path collective) on CPU with
the gloo backend, world size 2."""
import os

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from pyticles_gb300 import replicas


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms, work = replicas.combine(10.0 + rank, 100.0 * (rank + 1), dist, device="cpu")
    out[rank] = (ms, work, replicas.shard(list(range(7)), rank, world))
    dist.destroy_process_group()


def test_combine_takes_max_time_and_sums_work():
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    port = 29500 + os.getpid() % 1000
    mp.start_processes(_worker, args=(2, port, out), nprocs=2, join=True,
                       start_method="spawn")
    assert out[0][:2] == (11.0, 300.0) and out[1][:2] == (11.0, 300.0)
    assert out[0][2] == [0, 2, 4, 6] and out[1][2] == [1, 3, 5]


def test_combine_without_process_group_is_identity():
    assert replicas.combine(3.5, 42, None) == (3.5, 42.0)
