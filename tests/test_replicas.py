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


def _served_worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    jobs = replicas.shard(list(range(11)), rank, world)
    recs = [{"job": k, "error": None, "visible": 0.1 * k, "admitted": 0.1 * k + 0.05,
             "finished": 0.1 * k + 1.0 + k, "latency": 1.0 + k, "queue": 0.05}
            for k in jobs]
    rep = {"jobs": len(jobs), "completed": len(jobs), "failed": 0, "rejected": 0,
           "unfinished_running": 0, "unfinished_waiting": 0,
           "work_pair_interactions": 100.0 * len(jobs), "peak_hbm_bytes": 10,
           "offered_pair_interactions": 1000.0 * len(jobs), "makespan_s": 5.0 + rank,
           "arrival_window_s": 1.0, "job_records": recs}
    merged = replicas.merge_served(replicas.gather(rep, dist))
    out[rank] = (jobs, merged)
    dist.destroy_process_group()


def test_served_shares_cover_every_job_once_and_merge():
    """Under torchrun each rank serves a round-robin share of one arrival
    stream; the shares cover every job exactly once and the merged report
    adds the work up over the slowest rank and takes the latency
    percentiles over all ranks' jobs."""
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    port = 30500 + os.getpid() % 1000
    mp.start_processes(_served_worker, args=(2, port, out), nprocs=2, join=True,
                       start_method="spawn")
    shares = [out[0][0], out[1][0]]
    assert sorted(shares[0] + shares[1]) == list(range(11))
    assert not set(shares[0]) & set(shares[1])
    for rank in (0, 1):
        m = out[rank][1]
        assert m["jobs"] == m["completed"] == 11 and m["ranks"] == 2
        assert m["makespan_s"] == 6.0
        assert m["achieved_pair_interactions_per_s"] == 1100.0 / 6.0
        assert m["latency_s"]["n"] == 11 and m["latency_s"]["p50"] == 6.0
        assert sorted(r["job"] for r in m["job_records"]) == list(range(11))


def test_batched_shares_are_disjoint_and_complete():
    sims = list(range(512))
    for world in (1, 2, 4, 8):
        parts = [replicas.shard(sims, r, world) for r in range(world)]
        assert sorted(x for p in parts for x in p) == sims
        assert max(len(p) for p in parts) - min(len(p) for p in parts) <= 1
