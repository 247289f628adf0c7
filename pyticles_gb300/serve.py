"""Continuous-batching SPH job server.

Jobs -- independent 2D or 3D simulations with their own size, parameters and
step count -- arrive over time.  Each dimension group (2D: Lucy kernel,
viscosity; 3D: cubic spline, viscosity, heat flux) owns one engine on its own
CUDA stream, whose particle capacity is its share of an HBM budget.  A job is
admitted into its group's engine as soon as a simulation slot and enough
particle capacity are free (first fit over the waiting queue), joins the
engine's next chunk of steps, and leaves -- state copied back, capacity
released -- when its steps are done.  The 2D and 3D engines run their chunks
concurrently.  Per job: queueing delay (admission - arrival), service time
(completion - admission) and latency (completion - arrival).

Failure handling: a malformed job (array shapes that disagree with its
dimension or size, no steps) or one larger than its group's whole capacity is
rejected at admission; a job the engine refuses to add (an allocation or
parameter error) fails with that status; a job whose state turns non-finite
(or whose particles outrun the cell slack) is retired with that error after
the chunk in which it happened.  The other jobs continue unaffected (their
particles never interact).  The report carries the HBM budget, each group's
particle capacity and its peak use.
"""
import collections
import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from .engine import Engine
from .workloads import lattice_system, rng_for, vdw_energy

# Bytes of engine state per particle (mirrors alloc_particles in
# csrc/sph_engine.cu): FP64 state A/B, evaluation positions/velocities, cell
# origins (3 axes x 8 arrays x 8 B), rates and factors in the pass precision,
# ids and sort scratch, seven packed vectors (positions and velocities of two
# stages, force factors, heat factors, the force pass's neighbour record),
# staging.
def bytes_per_particle(precision="mixed", integrator="ieuler", cluster=False, lists=0):
    """HBM an engine holds per particle of capacity.  lists = the dimension
    of a group on per-particle pair lists (0: none)."""
    rs = 4 if precision == "mixed" else 8
    v4 = 4 * rs
    b = 3 * 8 * 8 + 9 * rs + 5 * 8 + 9 * 4 + 7 * v4 + 10 * rs + 8 * 8
    if integrator == "rk4":
        b += 7 * 8
    if cluster and precision == "mixed":
        # cluster pairs (csrc/sph_cluster.cu): slot records (72 B a slot),
        # sort scratch (16 B), cluster boxes and references (16 B), and the
        # lists: 1.4 times the longest, about 415 entries of 8 B per cluster
        # of 8 in a fluid at n = 0.7 (denser fluids need proportionally more)
        b += 72 + 16 + 16 + 440
    if lists and precision == "mixed":
        # pair lists (csrc/sph_vlist.cu): rows of 1.25 times the longest
        # list of 4-byte entries -- about 180 in the served 2D fluid (spacing
        # 1, cutoff 6) and 600 in the 3D one (n = 0.7, cutoff 5.148) -- the
        # counts and the build positions
        b += 4 * (180 if lists == 2 else 600) + 4 + 16
    return b


@dataclass
class Job:
    job_id: int
    arrival: float            # seconds after the server starts
    dim: int
    steps: int
    params: object            # SphParams
    r: np.ndarray
    v: np.ndarray
    m: np.ndarray
    u: np.ndarray
    visible: float = None     # server time at which the job was seen
    admitted: float = None
    finished: float = None
    result: tuple = None
    error: str = None
    sim: int = None
    remaining: int = 0
    work: float = 0.0         # pair-interactions done

    @property
    def n(self):
        return len(self.r)


def make_job(job_id, arrival, dim, n, steps, seed, precision_kw=None):
    """A job of the served workload: 2D van der Waals fluid (spacing 1, Lucy
    h = 3, 6, viscosity) or 3D fluid at density 0.7 (cubic spline, support
    2.735 / 5.148, viscosity, heat flux), about n particles, T ~ U[0.4, 0.8]."""
    rng = rng_for(seed)
    temp = rng.uniform(0.4, 0.8)
    if dim == 2:
        side = max(16, int(round(math.sqrt(n))))
        prm, r, v, m, T0 = lattice_system(side, 2, spacing=1.0, jitter=0.1, temperature=temp,
                                          seed=seed, kernel="lucy", h_short=3.0, h_long=6.0,
                                          viscosity=True, dt=1e-3)
        rho0 = 1.0
    else:
        dens = 0.7
        side = max(10, int(round(n ** (1.0 / 3.0))))
        prm, r, v, m, T0 = lattice_system(side, 3, spacing=dens ** (-1.0 / 3.0), jitter=0.1,
                                          temperature=temp, seed=seed, kernel="cubic",
                                          h_short=2.735 / 2, h_long=5.148 / 2, viscosity=True,
                                          heat_flux=True, dt=1e-3)
        rho0 = dens
    u = vdw_energy(np.full(len(r), rho0), T0)
    return Job(job_id, arrival, dim, steps, prm, r, v, m, u)


def poisson_jobs(njobs, rate=20.0, frac2d=0.7, n_lo=1e3, n_hi=1e6, steps_lo=100,
                 steps_hi=5000, seed=5000):
    """The served workload: Poisson arrivals at `rate` jobs/s, 2D with
    probability frac2d, N log-uniform in [n_lo, n_hi], steps uniform in
    [steps_lo, steps_hi]; seeded."""
    rng = rng_for(seed)
    t = 0.0
    jobs = []
    for k in range(njobs):
        t += rng.exponential(1.0 / rate)
        dim = 2 if rng.uniform() < frac2d else 3
        n = int(math.exp(rng.uniform(math.log(n_lo), math.log(n_hi))))
        steps = int(rng.integers(steps_lo, steps_hi + 1))
        jobs.append(make_job(k, t, dim, n, steps, seed + 1 + k))
    return jobs


class Group:
    """One engine (one dimension group) and its jobs."""

    def __init__(self, dim, params, capacity, max_sims, precision, chunk, engine_factory,
                 stream, pair_scheme=0):
        self.dim = dim
        self.capacity = int(capacity)
        self.max_sims = max_sims
        self.chunk = chunk
        self.engine = engine_factory(params, precision, self.capacity, max_sims, stream)
        self.engine.set_tuning(steps_per_graph=chunk, use_graph=1, pair_scheme=pair_scheme)
        self.active = {}          # sim id -> job
        self.live = 0
        self.peak = 0

    def fits(self, job):
        return len(self.active) < self.max_sims and self.live + job.n <= self.capacity

    def admit(self, job, now):
        job.sim = self.engine.add(job.params, job.r, job.v, job.m, job.u)
        job.admitted = now
        job.remaining = job.steps
        self.active[job.sim] = job
        self.live += job.n
        self.peak = max(self.peak, self.live)

    def launch(self):
        """Enqueues one chunk (asynchronous); returns its step count."""
        if not self.active:
            return 0
        steps = min(self.chunk, min(j.remaining for j in self.active.values()))
        self.engine.advance(steps)
        return steps

    def finish(self, steps, now):
        """Waits for the chunk, accounts work and retires finished or failed
        jobs.  Returns the retired jobs."""
        if steps == 0:
            return []
        failed = set()
        try:
            self.engine.sync()
        except _abi.SphError:
            for sim, job in self.active.items():
                code = self.engine.status(sim)
                if code:
                    job.error = _abi.STATUS_NAMES.get(code, str(code))
                    failed.add(sim)
        # each job's own pair set (of the chunk's last step) x 2 evaluations
        # per step x the chunk's steps
        counts = self.engine.last_pair_counts(max(self.active) + 1)
        done = []
        for sim, job in list(self.active.items()):
            job.remaining -= steps
            job.work += 2.0 * steps * float(counts[sim])
            if sim in failed or job.remaining <= 0:
                if sim not in failed:
                    job.result = self.engine.get_state(sim)
                job.finished = now()
                self.engine.remove(sim)
                del self.active[sim]
                self.live -= job.n
                done.append(job)
        return done

    def close(self):
        self.engine.close()


def malformed(job):
    """Why a job cannot be served as given, or None."""
    if job.dim not in (2, 3):
        return "dimension must be 2 or 3"
    n = len(job.r)
    if n == 0:
        return "no particles"
    for name, a, shape in (("r", job.r, (n, job.dim)), ("v", job.v, (n, job.dim)),
                           ("m", job.m, (n,)), ("u", job.u, (n,))):
        if np.shape(a) != shape:
            return f"{name} has shape {np.shape(a)}, expected {shape}"
    if job.steps <= 0:
        return "no steps"
    if job.params is not None and getattr(job.params, "dim", job.dim) != job.dim:
        return "parameters of another dimension"
    return None


def default_engine_factory(params, precision, capacity, max_sims, stream):
    return Engine(params, precision, max_particles=capacity, max_sims=max_sims, stream=stream)


class Server:
    """Continuous batching over a 2D and a 3D engine within an HBM budget."""

    def __init__(self, hbm_budget_bytes, precision="mixed", chunk=25, max_sims=256,
                 share_2d=0.6, engine_factory=default_engine_factory, clock=time.perf_counter,
                 streams=None, group_params=None, pair_scheme_3d=1, pair_scheme_2d=0):
        """pair_scheme_2d / _3d: each group's pair scheme.  The defaults (cell
        windows; cluster pairs, whose tables and lists count against the
        group's share of the budget) give every job the bits it would have
        alone; pair lists (2) are faster, and a job's results then follow
        the engine's list builds (equal to the job alone to rounding)."""
        self.precision = precision
        self.chunk = chunk
        self.clock = clock
        self.hbm_budget = float(hbm_budget_bytes)
        self.bpp = {2: bytes_per_particle(precision, lists=2 if pair_scheme_2d == 2 else 0),
                    3: bytes_per_particle(precision, cluster=pair_scheme_3d == 1,
                                          lists=3 if pair_scheme_3d == 2 else 0)}
        caps = {2: hbm_budget_bytes * share_2d / self.bpp[2],
                3: hbm_budget_bytes * (1 - share_2d) / self.bpp[3]}
        if group_params is None:
            group_params = {2: make_job(0, 0.0, 2, 256, 1, 1).params,
                            3: make_job(0, 0.0, 3, 1000, 1, 2).params}
        streams = streams or {2: None, 3: None}
        schemes = {2: pair_scheme_2d, 3: pair_scheme_3d}
        self.groups = {d: Group(d, group_params[d], caps[d], max_sims, precision, chunk,
                                engine_factory, streams[d], schemes[d]) for d in (2, 3)}
        self.rejected = []

    def run(self, jobs, realtime=True, time_limit=None, concurrent=True):
        """Serves `jobs`.  With realtime, a job becomes visible at its arrival
        time on the server clock; otherwise all jobs are visible at once.
        Latency and queueing delay are measured from when a job is visible.

        concurrent: each dimension group runs its own loop on its own host
        thread (admission, chunk, retirement), so a group starts its next
        chunk as soon as its last one finished instead of waiting for the
        other group's chunk; the engines' calls release the interpreter
        lock while they wait on their streams.  Otherwise one loop launches
        both groups' chunks and waits for both before the next."""
        if concurrent:
            return self._run_concurrent(jobs, realtime, time_limit)
        jobs = sorted(jobs, key=lambda j: j.arrival)
        pending = collections.deque(jobs)
        waiting = []
        completed = []
        t0 = self.clock()
        now = lambda: self.clock() - t0
        while pending or waiting or any(g.active for g in self.groups.values()):
            t = now()
            if time_limit is not None and t > time_limit:
                break
            while pending and (not realtime or pending[0].arrival <= t):
                job = pending.popleft()
                job.visible = t
                waiting.append(job)
            # admission: first fit in arrival order
            still = []
            for job in waiting:
                why = malformed(job)
                if why is not None:
                    job.error = "rejected: " + why
                    job.finished = t
                    self.rejected.append(job)
                    continue
                g = self.groups[job.dim]
                if job.n > g.capacity:
                    job.error = "rejected: larger than the group's HBM budget"
                    job.finished = t
                    self.rejected.append(job)
                elif g.fits(job):
                    try:
                        g.admit(job, t)
                    except _abi.SphError as exc:
                        job.error = _abi.STATUS_NAMES.get(exc.status, str(exc.status))
                        job.finished = t
                        completed.append(job)
                else:
                    still.append(job)
            waiting = still
            if not any(g.active for g in self.groups.values()):
                if pending:
                    wait = pending[0].arrival - now()
                    if realtime and wait > 0:
                        time.sleep(min(wait, 0.05))
                continue
            launched = {d: g.launch() for d, g in self.groups.items()}
            for d, g in self.groups.items():
                completed.extend(g.finish(launched[d], now))
        makespan = now()
        return self.report(completed, makespan, jobs)

    def _admit(self, g, waiting, t, completed):
        """First-fit admission of the visible jobs into group g; returns the
        jobs still waiting.  Malformed and oversized jobs are rejected."""
        still = []
        for job in waiting:
            why = malformed(job)
            if why is not None:
                job.error = "rejected: " + why
                job.finished = t
                self.rejected.append(job)
                continue
            if job.n > g.capacity:
                job.error = "rejected: larger than the group's HBM budget"
                job.finished = t
                self.rejected.append(job)
            elif g.fits(job):
                try:
                    g.admit(job, t)
                except _abi.SphError as exc:
                    job.error = _abi.STATUS_NAMES.get(exc.status, str(exc.status))
                    job.finished = t
                    completed.append(job)
            else:
                still.append(job)
        return still

    def _run_concurrent(self, jobs, realtime, time_limit):
        import threading
        jobs = sorted(jobs, key=lambda j: j.arrival)
        queues = {d: collections.deque() for d in self.groups}
        for job in jobs:
            # a job of no served dimension goes to the 2D loop, which rejects it
            queues[job.dim if job.dim in self.groups else 2].append(job)
        completed = []
        lock = threading.Lock()
        errors = []
        t0 = self.clock()
        now = lambda: self.clock() - t0

        def serve_group(d):
            g = self.groups[d]
            pending, waiting = queues[d], []
            try:
                while pending or waiting or g.active:
                    t = now()
                    if time_limit is not None and t > time_limit:
                        break
                    while pending and (not realtime or pending[0].arrival <= t):
                        job = pending.popleft()
                        job.visible = t
                        waiting.append(job)
                    done = []
                    with lock:
                        waiting = self._admit(g, waiting, t, done)
                        completed.extend(done)
                    if not g.active:
                        if pending and realtime:
                            wait = pending[0].arrival - now()
                            if wait > 0:
                                time.sleep(min(wait, 0.05))
                        continue
                    steps = g.launch()
                    retired = g.finish(steps, now)
                    with lock:
                        completed.extend(retired)
            except Exception as exc:   # re-raised in the calling thread
                errors.append(exc)

        threads = [threading.Thread(target=serve_group, args=(d,)) for d in self.groups]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        if errors:
            raise errors[0]
        makespan = now()
        return self.report(completed, makespan, jobs)

    def report(self, completed, makespan, jobs):
        """Latency (completion - visible), queueing delay (admission -
        visible) and service time (completion - admission) at p50 / p99 over
        the jobs that completed; jobs still running or still waiting when a
        time limit stopped the run are counted as such, and the work they
        did counts toward the achieved load."""
        ok = [j for j in completed if j.error is None]

        def pct(x):
            x = np.asarray(x, dtype=np.float64)
            if len(x) == 0:
                return {"p50": None, "p99": None, "n": 0}
            return {"p50": float(np.percentile(x, 50)), "p99": float(np.percentile(x, 99)),
                    "n": int(len(x))}

        lat = pct([j.finished - j.visible for j in ok])
        admitted = [j for j in jobs if j.admitted is not None and j.visible is not None]
        queue = pct([j.admitted - j.visible for j in admitted])
        service = pct([j.finished - j.admitted for j in ok])
        work = sum(j.work for j in jobs)
        window = max(j.arrival for j in jobs) if jobs else 0.0
        running = [j for j in jobs if j.admitted is not None and j.finished is None]
        waiting = [j for j in jobs if j.admitted is None and j.finished is None]
        return {
            "hbm_budget_bytes": self.hbm_budget,
            "capacity_particles": {d: g.capacity for d, g in self.groups.items()},
            "peak_particles": {d: g.peak for d, g in self.groups.items()},
            "peak_hbm_bytes": sum(g.peak * self.bpp[d] for d, g in self.groups.items()),
            "jobs": len(jobs), "completed": len(ok),
            "failed": len([j for j in completed if j.error]), "rejected": len(self.rejected),
            "unfinished_running": len(running), "unfinished_waiting": len(waiting),
            "latency_s": lat, "queue_s": queue, "service_s": service,
            "latency_p50_s": lat["p50"], "latency_p99_s": lat["p99"],
            "queue_p50_s": queue["p50"], "service_p50_s": service["p50"],
            "makespan_s": makespan, "arrival_window_s": window,
            "work_pair_interactions": work,
            "achieved_pair_interactions_per_s": work / makespan if makespan > 0 else 0.0,
        }

    @staticmethod
    def job_records(jobs):
        """One structured record per job (JSON-ready): size, timing in server
        seconds, latency split, pair-interactions done and the error if any."""
        out = []
        for j in jobs:
            rec = {"job": j.job_id, "dim": j.dim, "n": j.n, "steps": j.steps,
                   "arrival": j.arrival, "visible": j.visible, "admitted": j.admitted,
                   "finished": j.finished, "pair_interactions": j.work, "error": j.error}
            if j.finished is not None and j.visible is not None:
                rec["latency"] = j.finished - j.visible
            if j.admitted is not None and j.visible is not None:
                rec["queue"] = j.admitted - j.visible
            out.append(rec)
        return out

    def close(self):
        for g in self.groups.values():
            g.close()
