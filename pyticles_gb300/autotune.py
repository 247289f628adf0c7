"""Autotuner for the engine's launch and grid knobs.

Knobs (struct sph_tuning): threads per block of the pair passes, the
cell-edge / cutoff ratio (1 -> cells of the cutoff and a 3^d window, 1/2 ->
5^d, 1/3 -> 7^d, cells beyond the cutoff culled per particle), for batches
in mixed precision the launch form of the cell-window passes (one thread
per particle, or persistent grids that walk the flattened table) and the
pair scheme in mixed precision: cell windows, per-particle pair lists or
cluster pairs (3D; the cluster scheme has its own fixed launch shape).  A candidate is
timed with CUDA events over a few graph-captured steps on a clone of the
simulations (same parameters, same current states), so tuning neither
advances the live simulations nor shifts their thermostat schedules.  Results
are cached per workload signature for the life of the process.
"""
import math

import numpy as np

from .engine import Engine

BLOCKS = (64, 128, 256)
RATIOS = (1.0, 0.5, 1.0 / 3.0)

_cache = {}


def signature(group, precision, counts):
    """Workload key: group flags, precision and the particle-count profile."""
    total = int(sum(counts))
    return (group.dim, group.kernel, group.viscosity, group.heat_flux, group.integrator,
            precision, int(round(math.log2(max(total, 1)))), len(counts) > 1)


def cluster_candidate(group, precision, sims):
    """Whether the cluster-pair scheme can apply: 3D simulations in mixed
    precision without collisions (the engine itself checks the boxes)."""
    return group.dim == 3 and precision == "mixed" and group.collision == 0


def list_candidate(group, precision, sims):
    """Whether per-particle pair lists can apply: mixed precision without
    collisions (the engine itself checks the grids and the slot count)."""
    return precision == "mixed" and group.collision == 0


def time_candidate(group, precision, sims, block, ratio, steps, warmup, stream, scheme=0,
                   persistent=0):
    import torch
    total = sum(len(s[1]) for s in sims)
    with Engine(group, precision, max_particles=total, max_sims=len(sims),
                stream=stream.cuda_stream) as e:
        for prm, r, v, m, u in sims:
            e.add(prm, r, v, m, u)
        e.set_tuning(block_size=block, cell_ratio=ratio, steps_per_graph=steps, use_graph=1,
                     pair_scheme=scheme, persistent=persistent)
        e.advance(warmup)
        e.prepare()
        e.sync()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        e.advance(steps)
        t1.record(stream)
        t1.synchronize()
        e.sync()
        return t0.elapsed_time(t1) / steps


def tune(group, precision, sims, steps=4, warmup=2, blocks=BLOCKS, ratios=RATIOS,
         use_cache=True):
    """Times every (block, ratio) candidate of the cell scheme, and the
    cluster scheme where it can apply, on the given simulations
    [(params, r, v, m, u), ...]; returns (best_knobs, table)."""
    import torch
    key = signature(group, precision, [len(s[1]) for s in sims])
    if use_cache and key in _cache:
        return _cache[key]
    stream = torch.cuda.Stream()
    table = []
    for ratio in ratios:
        for block in blocks:
            ms = time_candidate(group, precision, sims, block, ratio, steps, warmup, stream)
            table.append({"block_size": block, "cell_ratio": ratio, "pair_scheme": 0,
                          "persistent": 0, "ms_per_step": ms})
    if precision == "mixed" and len(sims) > 1:
        # the persistent launch form, at the best cell-window shape
        cell = min(table, key=lambda row: row["ms_per_step"])
        ms = time_candidate(group, precision, sims, cell["block_size"], cell["cell_ratio"], steps,
                            warmup, stream, persistent=1)
        table.append(dict(cell, persistent=1, ms_per_step=ms))
    if list_candidate(group, precision, sims):
        for block in (128, 256):
            ms = time_candidate(group, precision, sims, block, 0.5, steps, warmup, stream,
                                scheme=2)
            table.append({"block_size": block, "cell_ratio": 0.5, "pair_scheme": 2,
                          "persistent": 0, "ms_per_step": ms})
    if cluster_candidate(group, precision, sims):
        ms = time_candidate(group, precision, sims, 128, 0.5, steps, warmup, stream, scheme=1)
        table.append({"block_size": 128, "cell_ratio": 0.5, "pair_scheme": 1, "persistent": 0,
                      "ms_per_step": ms})
    best = min(table, key=lambda row: row["ms_per_step"])
    knobs = {"block_size": best["block_size"], "cell_ratio": best["cell_ratio"],
             "pair_scheme": best["pair_scheme"], "persistent": best["persistent"]}
    _cache[key] = (knobs, table)
    return knobs, table


def tune_engine(engine, sims, precision, **kw):
    """Tunes on a clone of `sims` and applies the best knobs to `engine`."""
    knobs, table = tune(engine.group, precision, sims, **kw)
    engine.set_tuning(**knobs)
    return knobs, table


def sample_sims(sims, max_particles):
    """A subset of the simulations (every k-th) holding about max_particles,
    for tuning large batches quickly."""
    total = sum(len(s[1]) for s in sims)
    if total <= max_particles:
        return list(sims)
    stride = int(np.ceil(total / max_particles))
    return list(sims[::stride])
