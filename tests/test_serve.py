"""Continuous-batching server: admission, retirement, failure isolation and
latency accounting on CPU with a fake engine; a real 2D + 3D run on the GPU
where each job's result equals the same job run alone."""
import numpy as np
import pytest

from pyticles_gb300 import _abi, serve
from pyticles_gb300.serve import Job, Server, make_job


class FakeEngine:
    """Records calls; a simulation's 'state' is the number of steps it ran."""

    def __init__(self, params, precision, capacity, max_sims, stream):
        self.capacity = capacity
        self.sims = {}
        self.next_id = 0
        self.fail = set()
        self.err = False
        self.log = []

    def set_tuning(self, **kw):
        pass

    def add(self, prm, r, v, m, u):
        if len(r) == 77:          # an allocation the device refuses
            raise _abi.SphError(_abi.SPH_ENOMEM, "sph_sim_add")
        sid = self.next_id
        self.next_id += 1
        self.sims[sid] = {"n": len(r), "steps": 0, "nan": bool(np.isnan(u).any())}
        self.log.append(("add", sid))
        return sid

    def remove(self, sid):
        self.log.append(("remove", sid))
        del self.sims[sid]

    def advance(self, k):
        self.log.append(("advance", k, tuple(sorted(self.sims))))
        for s in self.sims.values():
            s["steps"] += k
            if s["nan"]:
                self.err = True

    def sync(self):
        if self.err:
            self.err = False
            raise _abi.SphError(_abi.SPH_ENAN, "device")

    def status(self, sid):
        return _abi.SPH_ENAN if self.sims[sid]["nan"] else 0

    def get_state(self, sid):
        return (self.sims[sid]["steps"],)

    def last_pair_total(self):
        return sum(s["n"] for s in self.sims.values()) * 10

    def last_pair_counts(self, nslots):
        out = np.zeros(nslots, dtype=np.int64)
        for sid, s in self.sims.items():
            if sid < nslots:
                out[sid] = s["n"] * 10
        return out

    def close(self):
        pass


def fake_job(k, arrival, dim, n, steps, nan=False):
    u = np.zeros(n)
    if nan:
        u[0] = np.nan
    return Job(k, arrival, dim, steps, None, np.zeros((n, dim)), np.zeros((n, dim)),
               np.ones(n), u)


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        self.t += 0.001
        return self.t


def fake_server(budget_particles, chunk=10, max_sims=4):
    bpp = serve.bytes_per_particle("mixed")
    return Server(budget_particles * bpp / 0.5, chunk=chunk, max_sims=max_sims, share_2d=0.5,
                  engine_factory=FakeEngine, clock=FakeClock(), group_params={2: None, 3: None})


@pytest.mark.parametrize("concurrent", [True, False])
def test_jobs_run_exactly_their_steps_and_leave(concurrent):
    """Both loops: one host thread per dimension group (the default) and the
    single loop that waits for both groups' chunks."""
    srv = fake_server(1000)
    jobs = [fake_job(0, 0.0, 2, 100, 25), fake_job(1, 0.0, 2, 200, 40),
            fake_job(2, 0.0, 3, 50, 7)]
    rep = srv.run(jobs, realtime=False, concurrent=concurrent)
    assert rep["completed"] == 3 and rep["failed"] == 0
    assert [j.result[0] for j in jobs] == [25, 40, 7]
    assert not srv.groups[2].active and srv.groups[2].live == 0


@pytest.mark.parametrize("concurrent", [True, False])
def test_each_job_is_credited_its_own_pairs(concurrent):
    """A job's work is its own pair count x 2 evaluations x its steps, not a
    share of the chunk's total (the fake engine's pair set is 10 n)."""
    srv = fake_server(1000)
    jobs = [fake_job(0, 0.0, 2, 100, 25), fake_job(1, 0.0, 2, 200, 40),
            fake_job(2, 0.0, 3, 50, 7)]
    srv.run(jobs, realtime=False, concurrent=concurrent)
    for j in jobs:
        assert j.work == 2.0 * j.steps * 10 * j.n


def test_time_limit_reports_unfinished_jobs():
    """A run stopped by its time limit reports the jobs still running and
    still waiting, counts their partial work, and splits latency, queueing
    and service time at p50 / p99 over the jobs that finished."""
    srv = fake_server(300, chunk=5, max_sims=2)
    jobs = [fake_job(0, 0.0, 2, 100, 5), fake_job(1, 0.0, 2, 200, 10000),
            fake_job(2, 0.0, 2, 250, 10), fake_job(3, 0.0, 2, 50, 10)]
    rep = srv.run(jobs, realtime=False, time_limit=0.5)
    assert rep["completed"] >= 1
    assert rep["unfinished_running"] >= 1 and rep["unfinished_waiting"] >= 1
    assert rep["completed"] + rep["unfinished_running"] + rep["unfinished_waiting"] == 4
    assert rep["work_pair_interactions"] > sum(j.work for j in jobs if j.finished is not None)
    for k in ("latency_s", "queue_s", "service_s"):
        assert rep[k]["n"] >= 1 and rep[k]["p99"] >= rep[k]["p50"] >= 0


def test_admission_waits_for_capacity_and_slots():
    srv = fake_server(300, chunk=5, max_sims=2)
    jobs = [fake_job(0, 0.0, 2, 200, 10), fake_job(1, 0.0, 2, 200, 10),
            fake_job(2, 0.0, 2, 50, 10), fake_job(3, 0.0, 2, 50, 10)]
    srv.run(jobs, realtime=False)
    adv = [e for e in srv.groups[2].engine.log if e[0] == "advance"]
    # capacity 300: job 1 (200) cannot join job 0 (200); first fit lets job 2 in
    assert all(len(e[2]) <= 2 for e in adv)
    assert jobs[1].admitted > jobs[2].admitted
    assert all(j.result[0] == 10 for j in jobs)


def test_oversized_job_is_rejected_not_run():
    srv = fake_server(100)
    jobs = [fake_job(0, 0.0, 2, 500, 10), fake_job(1, 0.0, 2, 20, 10)]
    rep = srv.run(jobs, realtime=False)
    assert rep["rejected"] == 1 and jobs[0].error.startswith("rejected")
    assert jobs[1].result == (10,)


def test_failed_job_is_retired_and_others_continue():
    srv = fake_server(1000, chunk=5)
    jobs = [fake_job(0, 0.0, 2, 100, 20), fake_job(1, 0.0, 2, 100, 20, nan=True),
            fake_job(2, 0.0, 2, 100, 20)]
    rep = srv.run(jobs, realtime=False)
    assert jobs[1].error == "SPH_ENAN" and jobs[1].result is None
    assert jobs[0].result == (20,) and jobs[2].result == (20,)
    assert rep["failed"] == 1 and rep["completed"] == 2


def test_malformed_and_refused_jobs_fail_alone():
    """Host-side injected failures: a malformed request and an allocation
    the engine refuses; the other jobs complete with their full steps."""
    srv = fake_server(1000, chunk=5)
    bad = fake_job(1, 0.0, 2, 50, 10)
    bad.r = np.zeros((50, 3))                     # 3 columns in the 2D group
    nomem = fake_job(2, 0.0, 2, 77, 10)
    nosteps = fake_job(3, 0.0, 3, 20, 0)
    good = [fake_job(0, 0.0, 2, 100, 20), fake_job(4, 0.0, 3, 60, 15)]
    rep = srv.run(good + [bad, nomem, nosteps], realtime=False)
    assert bad.error.startswith("rejected: r has shape")
    assert nosteps.error == "rejected: no steps"
    assert nomem.error == "SPH_ENOMEM" and nomem.result is None
    assert [j.result[0] for j in good] == [20, 15]
    assert rep["completed"] == 2 and rep["rejected"] == 2 and rep["failed"] == 1
    assert rep["peak_particles"][2] == 100 and rep["peak_particles"][3] == 60
    # the 3D group on cluster pairs counts their tables and lists too
    assert rep["peak_hbm_bytes"] == (100 * serve.bytes_per_particle("mixed")
                                     + 60 * serve.bytes_per_particle("mixed", cluster=True))


def test_latency_accounting_uses_arrival_times():
    srv = fake_server(1000, chunk=10)
    jobs = [fake_job(0, 0.0, 2, 10, 10), fake_job(1, 0.5, 2, 10, 10)]
    rep = srv.run(jobs, realtime=False)
    for j in jobs:
        assert j.finished >= j.admitted >= j.visible
    assert rep["arrival_window_s"] == 0.5
    assert rep["latency_p99_s"] >= rep["latency_p50_s"] > 0


def test_job_records_are_json_lines():
    import json
    srv = fake_server(1000, chunk=10)
    jobs = [fake_job(0, 0.0, 2, 10, 10), fake_job(1, 0.5, 3, 10, 20)]
    srv.run(jobs, realtime=False)
    recs = [json.loads(json.dumps(r)) for r in srv.job_records(jobs)]
    assert [r["job"] for r in recs] == [0, 1]
    assert all(r["latency"] >= r["queue"] >= 0 and r["error"] is None for r in recs)
    assert all(r["pair_interactions"] > 0 for r in recs)


def test_poisson_workload_shape():
    jobs = serve.poisson_jobs(60, n_lo=1e3, n_hi=2e3, steps_lo=100, steps_hi=200, seed=9)
    arr = np.array([j.arrival for j in jobs])
    assert np.all(np.diff(arr) > 0)
    assert 1.0 < arr[-1] < 6.0                      # ~3 s at 20 jobs/s
    frac2d = np.mean([j.dim == 2 for j in jobs])
    assert 0.5 < frac2d < 0.9
    assert all(100 <= j.steps <= 200 for j in jobs)
    assert all(j.params.dim == j.dim for j in jobs)


# ---- on the GPU ----

def small_jobs(seed=77):
    # the 3D jobs: one too small for columns (cell windows), two on cluster
    # pairs, sharing the 3D engine
    specs = [(2, 900, 30), (3, 1000, 20), (2, 1600, 45), (2, 400, 15), (3, 8000, 25),
             (2, 2500, 35), (3, 10648, 12)]
    return [make_job(k, 0.01 * k, d, n, s, seed + k) for k, (d, n, s) in enumerate(specs)]


def run_alone(job, precision="mixed"):
    """The job in an engine of its own, on the pair scheme of its server
    group (cluster pairs for 3D)."""
    from pyticles_gb300 import Engine
    with Engine(job.params, precision, max_particles=job.n) as e:
        s = e.add(job.params, job.r, job.v, job.m, job.u)
        e.set_tuning(pair_scheme=1 if job.dim == 3 else 0)
        e.advance(job.steps)
        e.sync()
        return e.get_state(s)


@pytest.mark.gpu
def test_served_results_equal_alone():
    jobs = small_jobs()
    srv = Server(2e9, chunk=10, max_sims=8)
    rep = srv.run(jobs, realtime=False)
    srv.close()
    assert rep["completed"] == len(jobs) and rep["failed"] == 0
    assert rep["latency_p99_s"] >= rep["latency_p50_s"] > 0
    for job in jobs:
        alone = run_alone(job)
        for a, b in zip(alone, job.result):
            assert np.array_equal(a, b), job.job_id


@pytest.mark.gpu
def test_nan_job_does_not_disturb_the_mix():
    jobs = small_jobs(seed=91)
    bad = make_job(99, 0.0, 2, 900, 30, 1234)
    bad.u[5] = np.nan
    srv = Server(2e9, chunk=10, max_sims=8)
    srv.run(jobs + [bad], realtime=False)
    srv.close()
    assert bad.error == "SPH_ENAN"
    for job in jobs:
        assert job.error is None
        alone = run_alone(job)
        for a, b in zip(alone, job.result):
            assert np.array_equal(a, b), job.job_id


@pytest.mark.gpu
def test_served_on_pair_lists_match_alone_to_rounding():
    """Both groups on pair lists: every job completes, and its state equals
    the same job run alone on lists to rounding (the list builds follow the
    engine, not the job)."""
    from pyticles_gb300 import Engine
    jobs = small_jobs(seed=83)
    srv = Server(2e9, chunk=10, max_sims=8, pair_scheme_2d=2, pair_scheme_3d=2)
    rep = srv.run(jobs, realtime=False)
    srv.close()
    assert rep["completed"] == len(jobs) and rep["failed"] == 0
    for job in jobs:
        with Engine(job.params, "mixed", max_particles=job.n) as e:
            s = e.add(job.params, job.r, job.v, job.m, job.u)
            e.set_tuning(pair_scheme=2)
            e.advance(job.steps)
            e.sync()
            alone = e.get_state(s)
        for a, b in zip(alone, job.result):
            assert np.linalg.norm(a - b) <= 1e-6 * np.linalg.norm(a), job.job_id


def test_budget_counts_the_pair_lists():
    """A group on pair lists counts their rows against the HBM budget: the
    2D fluid's lists (about 180 entries of 4 bytes) and the 3D fluid's
    (about 600), plus counts and build positions; FP64 engines have none."""
    base = serve.bytes_per_particle("mixed")
    assert serve.bytes_per_particle("mixed", lists=2) == base + 4 * 180 + 20
    assert serve.bytes_per_particle("mixed", lists=3) == base + 4 * 600 + 20
    assert serve.bytes_per_particle("fp64", lists=2) == serve.bytes_per_particle("fp64")
    srv = Server(1e9, share_2d=0.5, engine_factory=FakeEngine, clock=FakeClock(),
                 group_params={2: None, 3: None}, pair_scheme_2d=2, pair_scheme_3d=2)
    assert srv.groups[2].capacity == int(0.5e9 / (base + 740))
    assert srv.groups[3].capacity == int(0.5e9 / (base + 2420))
