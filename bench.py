"""Benchmark of the SPH step on GB300: pair-interactions/s.

Workload (one "step" = one improved-Euler step = 2 derivative evaluations):
2D van der Waals fluid, N = 1,048,576 (1024^2 lattice, spacing 1, jitter
+-0.1, T = 0.6, Lucy kernel, h_s = 3, h_l = 6, a = 2, b = 0.5, artificial
viscosity, dt = 1e-3), periodic box, mixed precision, every step captured in
one CUDA graph.  Synthetic seeded inputs (no dataset exists for this path).

metric value = (unordered pairs with r < h_l by the FP64 minimum-image
test) x 2 evaluations x K steps / device time of the K steps.

    python bench.py [--steps K] [--warmup W] [--side 1024] [--impl ours|reference]

Under torchrun (N > 1) each rank runs an independent replica (the
simulations do not exchange data); value sums the ranks' work over the
slowest rank's time.
"""
import argparse
import json
import math
import os
import re
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "pair-interactions/s & p50/p99 job latency, mixed vs plain FP64, 1 GB300"
UNIT = "pair-interactions/s"
L2_BYTES = 129e6
WORKLOAD_2D = ("2D van der Waals fluid, {side}^2 lattice, Lucy h_s=3 h_l=6, viscosity, "
               "improved Euler dt=1e-3, periodic")


def rank_info():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.lines = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.device)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        time.sleep(0.25)
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for name, val in zip(names, parts[4:8]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)),
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured", float(d.get("sm_max_mhz", 2070.0))
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback", 2070.0


def committed_figure(name, key):
    """A per-particle figure (`key: X` line) of one launch from a committed ncu
    summary under profiles/, or None."""
    path = os.path.join(ROOT, "profiles", name)
    try:
        txt = open(path).read()
    except OSError:
        return None
    m = re.search(key + r":\s*([0-9.eE+-]+)", txt)
    return float(m.group(1)) if m else None


def committed_traffic(name):
    """DRAM bytes per particle of one force launch from the committed ncu
    summary (`dram_bytes_per_particle: X` line), or None."""
    return committed_figure(name, "dram_bytes_per_particle")


def initial_state(side, seed):
    from pyticles_gb300 import workloads
    prm, r, v, m, T0 = workloads.config_2d(side, seed, viscosity=True)
    return prm, r, v, m, T0


def gpu_initial_energy(prm, r, v, m, T0, stream):
    """u0 = k_B T0 - a rho0 with rho0 from one GPU density evaluation."""
    from pyticles_gb300 import Engine
    with Engine(prm, "fp64", max_particles=len(r), stream=stream) as e:
        s = e.add(prm, r, v, m, np.zeros(len(r)))
        rho = e.derivatives(s)["rho"]
    return T0 * prm.kbdash - prm.adash * rho


def run_timed(prm, r, v, m, u, precision, steps, warmup, torch, stream, profile=True,
              knobs=None, sims=None):
    """Device time of `steps` graph-captured steps (one graph; with cluster
    pairs, graphs of 20 steps each captured on fresh event slots), with
    per-pass CUDA events recorded inside the graphs.  `sims` [(params, r, v, m, u)]
    replaces the single simulation for batched runs."""
    from pyticles_gb300 import Engine
    sims = sims or [(prm, r, v, m, u)]
    total = sum(len(x[1]) for x in sims)
    e = Engine(sims[0][0], precision, max_particles=total, max_sims=len(sims),
               stream=stream.cuda_stream)
    for sm in sims:
        e.add(*sm)
    if knobs:
        e.set_tuning(**knobs)
    e.set_tuning(steps_per_graph=max(1, steps), use_graph=1)
    e.advance(max(1, warmup))
    e.sync()
    if profile:
        e.profile(True)
    e.prepare()
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    e.advance(steps)
    t1.record(stream)
    t1.synchronize()
    ms = t0.elapsed_time(t1)
    e.sync()
    passes = e.profile_read() if profile else None
    pairs = e.last_pair_total()
    kps = e.kernels_per_step()
    e.profile(False)
    e.close()
    return ms, pairs, passes, kps


def batched_workload(nsims, ramp_steps=500):
    """512 independent 2D simulations: N log-uniform in [256, 65536], T in
    [0.2, 1.2], areal density in [0.4, 0.9], thermostat quench T -> T/2 over
    500 steps; u0 = k_B T0 - a n (n the number density)."""
    from pyticles_gb300 import workloads
    sims = []
    for prm, r, v, m, T0 in workloads.batched_2d(nsims, seed_base=4000,
                                                  ramp_steps=ramp_steps):
        dens = 1.0 / (prm.box[0] / math.sqrt(len(r))) ** 2
        u = workloads.vdw_energy(np.full(len(r), dens), T0)
        sims.append((prm, r, v, m, u))
    return sims


def batched_arm(sims, steps, torch, stream, dist=None):
    """The batched workload after autotuning the knobs on a sample.  The cell
    windows are timed with one thread per particle ("grid") and as
    persistent launches (tuning.persistent) over the flattened table, and
    the pair lists ("lists", which launch one thread per particle) when the
    tuner chose them; the fastest is the arm's value.  Under torchrun each
    rank runs its round-robin share of the simulations (replicas.shard); the
    work adds up over the slowest rank's time."""
    from pyticles_gb300 import replicas
    from pyticles_gb300 import autotune
    knobs, _ = autotune.tune(sims[0][0], "mixed", autotune.sample_sims(sims, 1 << 20), steps=3,
                             warmup=2)
    forms = {"grid": dict(knobs, rebin=0, persistent=0, pair_scheme=0),
             "persistent": dict(knobs, rebin=0, persistent=1, pair_scheme=0)}
    if knobs.get("pair_scheme") == 2:
        forms["lists"] = dict(knobs, rebin=0, persistent=0)
    variants, used = {}, {}
    for name, k in forms.items():
        ms, pairs, passes, kps = run_timed(None, None, None, None, None, "mixed", steps, 3,
                                           torch, stream, knobs=k, sims=sims)
        ms, pairs = replicas.combine(ms, pairs, dist, device="cuda")
        variants[name] = {
            "ms_per_step": ms / steps, "value": pairs * 2 * steps / (ms * 1e-3),
            "pass_ms_per_step": {kk: p["ms"] / steps for kk, p in passes.items()},
            "pairs_per_eval": pairs}
        used[name] = {kk: k[kk] for kk in ("block_size", "cell_ratio", "pair_scheme",
                                            "persistent") if kk in k}
    best = min(variants, key=lambda name: variants[name]["ms_per_step"])
    b = variants[best]
    nall = replicas.combine(0.0, sum(len(x[1]) for x in sims), dist, device="cuda")[1]
    sall = replicas.combine(0.0, len(sims), dist, device="cuda")[1]
    return {"sims": int(sall), "n": int(nall), "steps": steps,
            "ms_per_step": b["ms_per_step"], "pairs_per_eval": b["pairs_per_eval"],
            "value": b["value"], "unit": UNIT, "tuning": used[best],
            "launch": best, "variants": variants,
            "pass_ms_per_step": b["pass_ms_per_step"]}


def batched_accuracy(sims, steps, stream, knobs):
    """Mixed precision against the FP64 oracle for the smallest, median and
    largest simulation of the batch, each advanced `steps` steps from the
    same initial state (the quench included): relative L2 of r, v, u after
    the steps, and of rho, vdot, udot of one evaluation at the GPU's final
    state.  The three run in an engine of their own (on cell windows a
    simulation gives the same bits there as in the full batch; on pair
    lists the same to rounding)."""
    from oracle import oracle
    from pyticles_gb300 import Engine
    order = sorted(range(len(sims)), key=lambda k: len(sims[k][1]))
    picks = {"smallest": order[0], "median": order[len(order) // 2], "largest": order[-1]}
    group = [sims[k] for k in picks.values()]
    total = sum(len(x[1]) for x in group)
    out = {}
    with Engine(group[0][0], "mixed", max_particles=total, max_sims=len(group),
                stream=stream.cuda_stream) as e:
        ids = [e.add(*st) for st in group]
        e.set_tuning(**dict(knobs, rebin=0, steps_per_graph=min(steps, 100)))
        e.advance(steps)
        e.sync()
        states = [e.get_state(i) for i in ids]
        evals = [e.derivatives(i) for i in ids]
        e.sync()
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    for (name, k), (prm, r, v, m, u), (rr, vv, uu), g in zip(picks.items(), group, states, evals):
        t0 = time.perf_counter()
        r1, v1, u1, _ = oracle.advance(prm, r, v, m, u, steps)
        ref = oracle.derivatives(prm, rr, vv, m, uu)
        out[name] = {"sim": k, "n": len(r), "oracle_s": time.perf_counter() - t0,
                     "r": rel(rr, r1), "v": rel(vv, v1), "u": rel(uu, u1),
                     "rho": rel(g["rho"], ref["rho"]), "vdot": rel(g["vdot"], ref["vdot"]),
                     "udot": rel(g["udot"], ref["udot"])}
    return out


def fluid3d_workload(side):
    """3D fluid at number density 0.7 (side^3 particles), cubic spline with
    support radii 2.735 / 5.148 (about 60 / 400 neighbours), viscosity, heat
    flux."""
    from pyticles_gb300 import workloads
    prm, r, v, m, T0 = workloads.config_3d(side, 3000)
    u = workloads.vdw_energy(np.full(len(r), 0.7), T0)
    return [(prm, r, v, m, u)]


def timed_workload(sims, steps, warmup, torch, stream, tune=True, rebin=0):
    """Autotunes on a sample, then times `steps` graph-captured steps."""
    knobs = None
    if tune:
        from pyticles_gb300 import autotune
        knobs, _ = autotune.tune(sims[0][0], "mixed",
                                 autotune.sample_sims(sims, 1 << 20), steps=3, warmup=2)
    knobs = dict(knobs or {}, rebin=rebin)
    ms, pairs, passes, kps = run_timed(None, None, None, None, None, "mixed", steps, warmup,
                                       torch, stream, knobs=knobs, sims=sims)
    n = sum(len(x[1]) for x in sims)
    return {"sims": len(sims), "n": n, "steps": steps, "ms_per_step": ms / steps,
            "pairs_per_eval": pairs, "value": pairs * 2 * steps / (ms * 1e-3),
            "unit": UNIT, "tuning": knobs,
            "pass_ms_per_step": {k: p["ms"] / steps for k, p in passes.items()}}


def serve_window(njobs, time_limit, budget_gb, seed=5000, dist=None, schemes=(0, 1)):
    """A fixed Poisson arrival window of the served workload (20 jobs/s, 70%
    2D, N log-uniform in [1e3, 1e6], steps uniform in [100, 5000]), served in
    real time within an HBM budget small enough that admission queues.  The
    offered load (about 1.5e12 pair-interactions/s) exceeds one GPU, so the
    run stops at the time limit: jobs still running or still waiting then
    are reported as unfinished, and the work they did counts toward the
    achieved load.  Offered load counts each job's pairs from the fluid's
    density (56.5 unordered pairs per particle in 2D, about 200 in 3D) x 2
    evaluations x its steps, over the arrival window.  schemes: the 2D and
    3D groups' pair schemes."""
    from pyticles_gb300 import replicas, serve
    jobs = serve.poisson_jobs(njobs, seed=seed)
    if dist is not None and dist.is_initialized():
        # each rank serves its round-robin share of the one arrival stream
        jobs = replicas.shard(jobs, dist.get_rank(), dist.get_world_size())
    offered = sum(j.n * (56.5 if j.dim == 2 else 200.0) * 2 * j.steps for j in jobs)
    srv = serve.Server(budget_gb * 1e9, chunk=25, max_sims=256, pair_scheme_2d=schemes[0],
                       pair_scheme_3d=schemes[1])
    rep = srv.run(jobs, realtime=True, time_limit=time_limit)
    rep["pair_schemes"] = {"2d": schemes[0], "3d": schemes[1]}
    rep["job_records"] = srv.job_records(jobs)
    srv.close()
    rep["offered_pair_interactions_per_s"] = offered / max(rep["arrival_window_s"], 1e-9)
    rep["offered_pair_interactions"] = offered
    rep["time_limit_s"] = time_limit
    return replicas.merge_served(replicas.gather(rep, dist))


def run_e2e(prm, r, v, m, u, steps, torch, stream, knobs=None):
    """Through the C ABI with host (pinned) buffers: every step copies the
    state in, advances one step and reads the state back (the timed arm's
    knobs; a state set from the host is binned, and with pair lists listed,
    before its step)."""
    from pyticles_gb300 import Engine
    n, d = r.shape
    pin = lambda shape: torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
    hr, hv, hm, hu = pin((n, d)), pin((n, d)), pin((n,)), pin((n,))
    hr[:], hv[:], hm[:], hu[:] = r, v, m, u
    e = Engine(prm, "mixed", max_particles=n, stream=stream.cuda_stream)
    s = e.add(prm, hr, hv, hm, hu)
    if knobs:
        e.set_tuning(**knobs)
    e.set_tuning(steps_per_graph=1, use_graph=1)
    for _ in range(3):
        e.set_state(s, hr, hv, hm, hu)
        e.advance(1)
        e.get_state(s, hr, hv, hu)
    e.sync()
    t = time.perf_counter()
    for _ in range(steps):
        e.set_state(s, hr, hv, hm, hu)
        e.advance(1)
        e.get_state(s, hr, hv, hu)
    e.sync()
    wall = time.perf_counter() - t
    pairs = e.last_pair_total()
    e.close()
    return wall, pairs, n * (2 * d + 2) * 8, n * (2 * d + 1) * 8


def accuracy_track(prm, r, v, m, u, steps, every, stream, knobs=None):
    """Mixed-precision accuracy along the benchmarked trajectory: every
    `every` steps the GPU evaluates f(x) at its current state and the FP64
    oracle re-evaluates it at the same state; relative L2 of rho, vdot and
    udot."""
    from oracle import oracle
    from pyticles_gb300 import Engine
    out = []
    with Engine(prm, "mixed", max_particles=len(r), stream=stream.cuda_stream) as e:
        s = e.add(prm, r, v, m, u)
        e.set_tuning(**dict(knobs or {}, rebin=1, steps_per_graph=every))
        done = 0
        while done < steps:
            e.advance(every)
            done += every
            rs, vs, us = e.get_state(s)
            g = e.derivatives(s)
            e.sync()
            t0 = time.perf_counter()
            ref = oracle.derivatives(prm, rs, vs, m, us)
            t_ref = time.perf_counter() - t0
            row = {"step": done,
                   # the same evaluation on the host cores: the CPU baseline
                   # of this workload (one evaluation = its pair count)
                   "oracle_eval": {"value": ref["nip"] / t_ref, "unit": UNIT,
                                   "seconds": t_ref, "cores": oracle.threads(),
                                   "cpu": cpu_model(), "kind": "port"}}
            for k in ("rho", "vdot", "udot"):
                row[k] = float(np.linalg.norm(g[k] - ref[k]) / np.linalg.norm(ref[k]))
            out.append(row)
    return out


def cpu_model():
    """The host CPU as /proc/cpuinfo names it (model name, else the Arm
    implementer/part codes), else the machine type."""
    import platform
    try:
        info = open("/proc/cpuinfo").read().splitlines()
    except OSError:
        info = []
    fields = {}
    for line in info:
        if ":" in line:
            k, _, val = line.partition(":")
            fields.setdefault(k.strip(), val.strip())
    if fields.get("model name"):
        return fields["model name"]
    if fields.get("CPU part"):
        return (f"{platform.machine()} (CPU implementer {fields.get('CPU implementer', '?')}, "
                f"part {fields['CPU part']})")
    return platform.processor() or platform.machine()


def oracle_rate(side, seed, budget_s, max_steps):
    """FP64 C oracle (OpenMP, all host threads) on a bounded sample."""
    from oracle import oracle
    prm, r, v, m, T0 = initial_state(side, seed)
    u = oracle.initial_energy(prm, r, v, m, T0)
    nip = oracle.derivatives(prm, r, v, m, u)["nip"]
    steps, t = 0, 0.0
    while steps < max_steps and (steps == 0 or t < budget_s):
        t0 = time.perf_counter()
        r, v, u, _ = oracle.advance(prm, r, v, m, u, 1)
        t += time.perf_counter() - t0
        steps += 1
    return nip * 2 * steps / t, steps, t, oracle.threads(), len(r)


def reference_arm(args):
    """The reference path's CPU implementation: the FP64 oracle port (the
    reference is Python and its compiled parts do not build), all host
    threads, one improved-Euler step of a 512^2 sample of the workload per
    bench step."""
    rank, world, _ = rank_info()
    if rank != 0:
        return 0
    # a bounded sample of the workload: 512^2 (256^2 for long runs, so that
    # the whole run stays within a few minutes on the host cores)
    side = min(args.side, 512 if args.steps <= 300 else 256)
    from oracle import oracle
    prm, r, v, m, T0 = initial_state(side, 1000)
    u = oracle.initial_energy(prm, r, v, m, T0)
    nip = oracle.derivatives(prm, r, v, m, u)["nip"]
    r, v, u, _ = oracle.advance(prm, r, v, m, u, max(0, min(args.warmup, 2)))
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r, v, u, _ = oracle.advance(prm, r, v, m, u, 1)
    wall = time.perf_counter() - t0
    value = nip * 2 * args.steps / wall
    sample = (f"2D van der Waals fluid N={len(r)} ({side}^2 lattice, same density, kernels, "
              f"viscosity and dt as the GPU workload), {args.steps} improved-Euler steps")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": WORKLOAD_2D.format(side=args.side), "n": args.side ** 2,
                       "evals_per_step": 2, "precision": "fp64 (the reference's arithmetic)",
                       "sample": {"n": len(r), "pairs_per_eval": nip}},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": oracle.threads(),
                             "cpu": cpu_model(), "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def profile_case(args):
    """A few eager (non-graph) steps of one workload for profilers: each step
    launches the binning kernels, then per integrator stage k_density,
    [k_heat,] k_force; with --steps 2 the second step's launches are the ones
    to capture.  2D: the fluid of the bench line at --side^2; 3D: the fluid at
    density 0.7 at --side^3 (cubic spline, viscosity, heat flux)."""
    from pyticles_gb300 import Engine, build, workloads
    build.build()
    if args.profile_case == "2d":
        prm, r, v, m, T0 = workloads.config_2d(args.side, 1000, viscosity=True)
        u = workloads.vdw_energy(np.ones(len(r)), T0)
    else:
        prm, r, v, m, T0 = workloads.config_3d(args.side, 3000)
        u = workloads.vdw_energy(np.full(len(r), 0.7), T0)
    with Engine(prm, args.precision, max_particles=len(r)) as e:
        e.add(prm, r, v, m, u)
        e.set_tuning(use_graph=0, pair_scheme=args.pair_scheme or 0)
        e.advance(args.steps)
        e.sync()
        print(f"{args.profile_case} n={len(r)} steps={args.steps} "
              f"pairs/eval={e.last_pair_total()} tuning={e.tuning}")
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--side", type=int, default=1024)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--fp64-steps", type=int, default=10)
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-tune", action="store_true",
                    help="use the engine's default knobs (stable launch counts for profilers)")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the batched, 3D and served sub-workloads")
    ap.add_argument("--batched-sims", type=int, default=512)
    ap.add_argument("--batched-steps", type=int, default=500,
                    help="steps of the batched workload (its quench ramps over 500)")
    ap.add_argument("--side3d", type=int, default=128)
    ap.add_argument("--steps3d", type=int, default=200)
    ap.add_argument("--serve-jobs", type=int, default=200)
    ap.add_argument("--serve-budget-gb", type=float, default=3.0,
                    help="HBM budget of the served workload's engines")
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    ap.add_argument("--accuracy-steps", type=int, default=1000,
                    help="trajectory length of the mixed-vs-FP64 accuracy report (0: skip)")
    ap.add_argument("--rebin", type=int, default=1, choices=[0, 1],
                    help="single-simulation workloads: 1 bins into cells on demand "
                         "(tuning.rebin), 0 every step")
    ap.add_argument("--profile-case", choices=["2d", "3d"], default=None,
                    help="profiling driver: --steps eager steps of one workload "
                         "(--side, --precision, --pair-scheme), no timing")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--pair-scheme", type=int, default=None, choices=[0, 1, 2],
                    help="force the pair scheme (profiling case: default 0; the timed "
                         "2D workload: the tuner's choice)")
    args = ap.parse_args()
    if args.profile_case:
        return profile_case(args)
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return reference_arm(args)

    import torch
    from pyticles_gb300 import build
    build.build()
    rank, world, local = rank_info()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    stream = torch.cuda.Stream()
    prm, r, v, m, T0 = initial_state(args.side, 1000 + rank)
    u = gpu_initial_energy(prm, r, v, m, T0, stream.cuda_stream)
    n = len(r)
    hbm_peak, peak_kind, sm_max = measured_peaks()

    from pyticles_gb300 import autotune
    knobs = None
    if not args.no_tune:
        knobs, _ = autotune.tune(prm, "mixed", [(prm, r, v, m, u)], steps=3, warmup=2)
    knobs = dict(knobs or {}, rebin=args.rebin)
    if args.pair_scheme is not None:
        knobs["pair_scheme"] = args.pair_scheme
    if dist:
        dist.barrier()
    with ClockSampler(local) as clocks:
        ms, pairs, passes, kps = run_timed(prm, r, v, m, u, "mixed", args.steps, args.warmup,
                                           torch, stream, knobs=knobs)
    from pyticles_gb300 import replicas
    ms, pairs_all = replicas.combine(ms, pairs, dist, device="cuda")
    value = pairs_all * 2 * args.steps / (ms * 1e-3)

    # plain FP64 GPU step on the same workload
    ms64, pairs64, _, _ = run_timed(prm, r, v, m, u, "fp64", args.fp64_steps, 3, torch, stream,
                                    profile=False, knobs=knobs)
    fp64_value = pairs64 * 2 * args.fp64_steps / (ms64 * 1e-3)

    # end to end through the C ABI with pinned host buffers
    wall, pairs_e, h2d, d2h = run_e2e(prm, r, v, m, u, args.e2e_steps, torch, stream,
                                      knobs=knobs)
    e2e_value = pairs_e * 2 * args.e2e_steps / wall

    # roofline of the dominant pass (force + integrator epilogue): the pair
    # lists' k_force_vl when the tuner chose them, else the cell windows'
    # k_force; pair lists bin on demand whatever `rebin` says
    lists = knobs.get("pair_scheme") == 2
    fprof = "k_force_vl_2d_mixed.md" if lists else "k_force_2d_mixed.md"
    f = passes["force"]
    nlaunch = max(1, f["launches"])
    avg_ms = f["ms"] / nlaunch
    from pyticles_gb300 import opcount
    bpp = opcount.force_bytes_per_step_average(2, 4, reuse=bool(args.rebin) or lists)
    achieved = bpp * n / (avg_ms * 1e-3) / 1e9
    trafpp = committed_traffic(fprof)
    # the binding limit, instruction issue: from one ncu launch, its warp
    # instructions over its own duration and clock against SMs x 4 issue
    # slots per cycle (both from the same launch); the live figure scales
    # that launch's instruction count to the bench's in-graph launch time
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    winst_pp = committed_figure(fprof, "warp_instructions_per_particle")
    ncu_ms = committed_figure(fprof, "launch_ms")
    ncu_mhz = committed_figure(fprof, "sm_mhz")
    ncu_issue = None
    if winst_pp is not None and ncu_ms and ncu_mhz:
        ncu_issue = winst_pp * n / (sms * 4 * ncu_mhz * 1e6 * ncu_ms * 1e-3)
    flops = opcount.FLOPS_FORCE[2] * pairs / (avg_ms * 1e-3) / 1e12
    fp32_peak = sms * 128 * 2 * sm_max * 1e6 / 1e12
    total_pass_ms = sum(p["ms"] for p in passes.values())

    extras = {}
    if not args.no_extras:
        # every rank: the batched and served arms split their simulations and
        # jobs over the ranks; the 3D fluid runs as a replica per rank
        bsims = batched_workload(args.batched_sims)
        extras["batched"] = batched_arm(replicas.shard(bsims, rank, world), args.batched_steps,
                                        torch, stream, dist)
        if rank == 0 and not args.no_cpu:
            extras["batched"]["accuracy"] = batched_accuracy(
                bsims, args.batched_steps, stream, extras["batched"]["tuning"])
        w3 = fluid3d_workload(args.side3d)
        extras["fluid3d"] = timed_workload(w3, args.steps3d, 3, torch, stream,
                                           rebin=args.rebin)
        f3 = extras["fluid3d"]
        ms3, work3 = replicas.combine(f3["ms_per_step"] * f3["steps"],
                                      f3["pairs_per_eval"] * 2 * f3["steps"], dist, device="cuda")
        f3["value"] = work3 / (ms3 * 1e-3)
        f3["replicas"] = world
        if rank == 0 and not args.no_cpu:
            acc3 = accuracy_track(*w3[0], args.steps3d, args.steps3d, stream,
                                  knobs=extras["fluid3d"]["tuning"])
            extras["fluid3d"]["cpu_baseline"] = dict(
                acc3[-1].pop("oracle_eval"),
                sample="one FP64 oracle evaluation (pair search, density, heat flux, force) "
                       "of the 128^3 state after the timed steps")
            extras["fluid3d"]["accuracy"] = {
                "what": "relative L2 of the mixed-precision evaluation against the FP64 "
                        "oracle at the GPU state after the timed steps",
                **acc3[-1]}
        extras["serve"] = serve_window(args.serve_jobs, args.serve_seconds, args.serve_budget_gb,
                                       dist=dist)

    accuracy = None
    if rank == 0 and not args.no_cpu and args.accuracy_steps > 0:
        accuracy = accuracy_track(prm, r, v, m, u, args.accuracy_steps,
                                  max(1, min(100, args.accuracy_steps)), stream, knobs=knobs)
        for row in accuracy:
            row.pop("oracle_eval")

    cpu = None
    if rank == 0 and not args.no_cpu:
        rate, csteps, ct, cores, cn = oracle_rate(min(args.side, 512), 1000, args.cpu_seconds,
                                                  50)
        cpu = {"value": rate, "unit": UNIT, "cores": cores, "cpu": cpu_model(), "kind": "port",
               "sample": f"FP64 C oracle, 2D vdW fluid N={cn}, {csteps} improved-Euler steps, "
                         f"{ct:.1f} s"}
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0
    working_set = n * (2 * 56 + 2 * 16 + 16 + 16 + 40 + 48)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded lattice + jitter, Maxwell velocities)",
        "config": {
            "workload": WORKLOAD_2D.format(side=args.side),
            "n": n, "pairs_per_eval": pairs, "evals_per_step": 2,
            "precision": "mixed: f32 pair arithmetic + compensated sums, f64 pair test, "
                         "integrator and reductions",
            "graph": f"{args.steps} steps in one CUDA graph",
            "l2": f"working set ~{working_set / 1e6:.0f} MB per step > 129 MB L2 (no flush)",
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
            "fp64_value": fp64_value, "mixed_over_fp64": value / fp64_value,
            "tuning": knobs,
            "pass_ms_per_step": {k: p["ms"] / args.steps for k, p in passes.items()},
        },
        "roofline": {
            # the HBM roofline of the dominant pass, as the metric asks; the
            # pass is bound by instruction issue (FP32 pair arithmetic), whose
            # fraction is `binding`
            "bound": "issue",
            "kernel": ("k_force_vl<lucy> (pair lists; force + energy rate + integrator)"
                       if lists else
                       "k_force<float,2,lucy> (force + energy rate + integrator)"),
            "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
            "frac": achieved / hbm_peak, "peak_kind": peak_kind,
            "bytes_per_particle": bpp,
            "traffic": None if trafpp is None else trafpp * n,
            "traffic_note": ("DRAM bytes of one ncu launch (" + fprof + "); with pair lists "
                             "they include the list entries streamed per pass (4 B each), "
                             "which the algorithmic bytes do not count"),
            "binding": None if winst_pp is None else {
                "limit": "instruction issue (FP32 pair arithmetic)",
                "frac": ncu_issue,
                "frac_live": winst_pp * n / (avg_ms * 1e-3) / (sms * 4 * sm_max * 1e6),
                "warp_instructions_per_particle": winst_pp,
                "sms": sms,
                "note": "frac: warp instructions of one ncu launch over that launch's own "
                        "duration x SMs x 4 issue slots x its SM clock; frac_live: the same "
                        "instruction count over the live in-graph launch time at the maximum "
                        "clock"},
            "fp32_pipe": {"achieved_tflops": flops, "peak_tflops": fp32_peak,
                          "frac": flops / fp32_peak,
                          "note": "algorithmic flops of the force pass over SMs x 128 FP32 "
                                  "lanes x 2 x max SM clock (SM count from the device)"},
            "force_share_of_step": f["ms"] / total_pass_ms if total_pass_ms > 0 else None,
        },
        "cpu_baseline": cpu,
        "accuracy": None if accuracy is None else {
            "what": "relative L2 of the mixed-precision evaluation against the FP64 oracle "
                    "at the GPU state, every 100 steps of the benchmarked trajectory",
            "max": {k: max(row[k] for row in accuracy) for k in ("rho", "vdot", "udot")},
            "track": accuracy},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "steps": args.e2e_steps},
        "gpu_launches": kps * args.steps,
        "clocks": clocks.summary(),
    }
    if extras:
        sv = extras.get("serve", {})
        line["latency"] = {"p50_s": sv.get("latency_p50_s"), "p99_s": sv.get("latency_p99_s"),
                           "workload": "served Poisson window (see workloads.serve)"}
        line["workloads"] = extras
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
