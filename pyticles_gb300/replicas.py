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
    """Round-robin share of independent simulations (or jobs) for this rank."""
    return [x for k, x in enumerate(items) if k % world == rank]


def gather(obj, dist=None):
    """Every rank's obj, in rank order, on every rank ([obj] without a
    process group).  Host objects only (job records, reports): the
    measurement, never the data path."""
    if dist is None or not dist.is_available() or not dist.is_initialized():
        return [obj]
    out = [None] * dist.get_world_size()
    dist.all_gather_object(out, obj)
    return out


def merge_served(reports):
    """One served-window report from the ranks' reports over disjoint job
    shares: job counts and work add up, the makespan is the slowest rank's,
    and latency, queueing and service percentiles are taken over the job
    records of all ranks."""
    import numpy as np
    if len(reports) == 1:
        return reports[0]
    recs = [r for rep in reports for r in rep["job_records"]]

    def pct(x):
        x = np.asarray(x, dtype=np.float64)
        if len(x) == 0:
            return {"p50": None, "p99": None, "n": 0}
        return {"p50": float(np.percentile(x, 50)), "p99": float(np.percentile(x, 99)),
                "n": int(len(x))}

    done = [r for r in recs if r.get("error") is None and r.get("finished") is not None]
    out = dict(reports[0])
    for k in ("jobs", "completed", "failed", "rejected", "unfinished_running",
              "unfinished_waiting", "work_pair_interactions", "peak_hbm_bytes",
              "offered_pair_interactions"):
        if k in reports[0]:
            out[k] = sum(rep[k] for rep in reports)
    out["makespan_s"] = max(rep["makespan_s"] for rep in reports)
    out["arrival_window_s"] = max(rep["arrival_window_s"] for rep in reports)
    out["latency_s"] = pct([r["latency"] for r in done])
    out["queue_s"] = pct([r["queue"] for r in recs if r.get("queue") is not None])
    out["service_s"] = pct([r["finished"] - r["admitted"] for r in done])
    out["latency_p50_s"], out["latency_p99_s"] = out["latency_s"]["p50"], out["latency_s"]["p99"]
    out["queue_p50_s"], out["service_p50_s"] = out["queue_s"]["p50"], out["service_s"]["p50"]
    out["achieved_pair_interactions_per_s"] = (out["work_pair_interactions"] / out["makespan_s"]
                                               if out["makespan_s"] > 0 else 0.0)
    if "offered_pair_interactions" in out:
        out["offered_pair_interactions_per_s"] = (out["offered_pair_interactions"]
                                                  / max(out["arrival_window_s"], 1e-9))
    out["job_records"] = recs
    out["ranks"] = len(reports)
    return out
