"""Replica bookkeeping for multi-GPU runs.

Simulations do not exchange data, so N GPUs run N independent replicas (or
disjoint sets of simulations): no collective sits on the data path.  Only the
measurement is combined: the job time is the slowest rank's time and the work
is the sum over ranks.
"""


def combine(ms, work, dist=None, device=None):
    """Returns (max ms over ranks, summed work) -- identity without a
    process group."""
    if dist is None or not dist.is_available() or not dist.is_initialized():
        return float(ms), float(work)
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    w = torch.tensor([float(work)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(w, op=dist.ReduceOp.SUM)
    return float(t.item()), float(w.item())


def shard(items, rank, world):
    """Round-robin share of independent simulations for this rank."""
    return [x for k, x in enumerate(items) if k % world == rank]
