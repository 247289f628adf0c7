"""Pair lists (tuning.pair_scheme 2): per-particle neighbour lists with a
skin, built when the engine bins and walked by the 2D mixed-precision pair
passes, against the golden vectors of the reference, the FP64 oracle and
the cell-window scheme.  The pair set stays exact: every evaluation still
applies the reference's pair test to the listed candidates."""
import numpy as np
import pytest

from oracle import oracle
from pyticles_gb300 import Engine, build, workloads
from pyticles_gb300._abi import SPH_ESKIN, SphError
from tests.golden_cases import SYSTEMS, load, params_of, rel_l2
from tests.test_gpu_parity import JQ_TOL, KEYS, MIXED_TOL, mixed_bound, record

pytestmark = pytest.mark.gpu

SYSTEMS_2D = [n for n in SYSTEMS if params_of(load(n)).dim == 2]


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


def listed(prm, r, v, m, u, skin=0.025, nsims=1):
    e = Engine(prm, "mixed", max_particles=len(r) * nsims, max_sims=nsims)
    e.set_tuning(pair_scheme=2, list_skin=skin)
    return e


def lists_in_use(e):
    """The engine runs its list build each step: one kernel more than the
    cell-window scheme launches when it too bins on demand (as lists do)."""
    k2 = e.kernels_per_step()
    rebin = e.tuning["rebin"]
    e.set_tuning(pair_scheme=0, rebin=1)
    k0 = e.kernels_per_step()
    e.set_tuning(pair_scheme=2, rebin=rebin)
    return k2 == k0 + 1


@pytest.mark.parametrize("name", SYSTEMS_2D)
def test_list_evaluation_matches_reference(name):
    g = load(name)
    prm = params_of(g)
    with listed(prm, g["r0"], g["v0"], g["m"], g["u0"]) as e:
        s = e.add(prm, g["r0"], g["v0"], g["m"], g["u0"])
        d = e.derivatives(s)
        e.sync()
        assert lists_in_use(e)
        errs = {k: rel_l2(d[k], g["ev_" + k]) for k in KEYS}
        bounds = {k: mixed_bound(name, k) for k in KEYS}
        record("list_evaluation", name, "mixed", errs, bounds)
        for k, err in errs.items():
            assert err < bounds[k], (k, err, bounds[k])
        assert e.pair_count(s) == len(g["iap"])


@pytest.mark.parametrize("name", SYSTEMS_2D)
def test_list_steps_track_reference(name):
    g = load(name)
    prm = params_of(g)
    with listed(prm, g["r0"], g["v0"], g["m"], g["u0"]) as e:
        s = e.add(prm, g["r0"], g["v0"], g["m"], g["u0"])
        e.advance(int(g["steps"]))
        e.sync()
        r, v, u = e.get_state(s)
        errs = {"r": rel_l2(r, g["r_final"]), "v": rel_l2(v, g["v_final"]),
                "u": rel_l2(u, g["u_final"])}
        bounds = {"r": MIXED_TOL, "u": MIXED_TOL,
                  "v": max(MIXED_TOL, mixed_bound(name, "vdot"))}
        record("list_steps", name, "mixed", errs, bounds)
        for k, err in errs.items():
            assert err < bounds[k], (k, err, bounds[k])


def test_list_config1_100_steps_match_reference():
    """100 improved-Euler steps of the 32 x 32 fluid against the reference's
    own update(), every 20 steps, on one set of lists kept across steps."""
    g = load("traj2d_1024")
    prm = params_of(g)
    with listed(prm, g["r0"], g["v0"], g["m"], g["u0"]) as e:
        s = e.add(prm, g["r0"], g["v0"], g["m"], g["u0"])
        done = 0
        for k, mark in enumerate(g["marks"]):
            e.advance(int(mark) - done)
            done = int(mark)
            e.sync()
            r, v, u = e.get_state(s)
            errs = {"r": rel_l2(r, g["r_marks"][k]), "v": rel_l2(v, g["v_marks"][k]),
                    "u": rel_l2(u, g["u_marks"][k])}
            record("list_traj100", f"traj2d_1024@{done}", "mixed", errs)
            for key, err in errs.items():
                assert err < MIXED_TOL, (done, key, err)
        # the lists outlive many steps of the slow fluid
        assert e.rebin_count() <= 20


def test_list_viscous_100_steps_match_oracle():
    prm, r, v, m, T0 = workloads.config_2d(32, 1000, viscosity=True)
    u = oracle.initial_energy(prm, r, v, m, T0)
    with listed(prm, r, v, m, u) as e:
        s = e.add(prm, r, v, m, u)
        e.advance(100)
        e.sync()
        rr, vv, uu = e.get_state(s)
    r1, v1, u1, _ = oracle.advance(prm, r, v, m, u, 100)
    errs = {"r": rel_l2(rr, r1), "v": rel_l2(vv, v1), "u": rel_l2(uu, u1)}
    record("list_traj100", "visc2d_1024@100", "mixed", errs)
    for key, err in errs.items():
        assert err < MIXED_TOL, (key, err)


def test_list_heat_flux_matches_oracle():
    """Heat flux walks the near entries only."""
    prm, r, v, m, T0 = workloads.config_2d(24, 1002, viscosity=True, heat_flux=True)
    u = oracle.initial_energy(prm, r, v, m, T0)
    u = u + prm.kbdash * 0.2 * T0 * np.sin(2 * np.pi * r[:, 0] / prm.box[0])
    ref = oracle.derivatives(prm, r, v, m, u)
    with listed(prm, r, v, m, u) as e:
        s = e.add(prm, r, v, m, u)
        d = e.derivatives(s)
        e.sync()
        assert lists_in_use(e)
    errs = {k: rel_l2(d[k], ref[k]) for k in KEYS + ("jq",)}
    record("list_full_physics", "visc_heat2d_576", "mixed", errs)
    for k, err in errs.items():
        assert err < (5e-6 if k == "jq" else MIXED_TOL), (k, err)


def test_fast_particles_rebuild_and_stay_exact():
    """A hot fluid moves far enough to rebuild the lists many times; each
    evaluation still has the oracle's pair set and values."""
    prm, r, v, m, T0 = workloads.config_2d(24, 1003, viscosity=True)
    v = v * 20.0          # ~0.02 per step: a rebuild every few steps
    u = oracle.initial_energy(prm, r, v, m, T0)
    with listed(prm, r, v, m, u) as e:
        s = e.add(prm, r, v, m, u)
        before = e.rebin_count()
        e.advance(40)
        e.sync()
        assert e.rebin_count() - before >= 3
        rr, vv, uu = e.get_state(s)
        d = e.derivatives(s)
        nip = e.pair_count(s)
    r1, v1, u1, _ = oracle.advance(prm, r, v, m, u, 40)
    assert rel_l2(rr, r1) < MIXED_TOL
    assert rel_l2(vv, v1) < 1e-5
    ref = oracle.derivatives(prm, rr, vv, m, uu)
    assert nip == ref["nip"]
    for k in ("rho", "vdot", "udot"):
        assert rel_l2(d[k], ref[k]) < MIXED_TOL, k


def test_list_skin_violation_is_flagged():
    """A particle that moves more than half the skin within one step raises
    SPH_ESKIN instead of silently missing pairs."""
    prm, r, v, m, T0 = workloads.config_2d(32, 5001)
    u = workloads.vdw_energy(np.full(len(r), 1.0), T0)
    with listed(prm, r, v, m, u) as e:
        s = e.add(prm, r, v, m, u)
        v2 = v.copy()
        v2[3] = [1000.0, 0.0]   # 1 per step against a skin of 0.15
        e.set_state(s, r, v2, m, u)
        e.advance(1)
        with pytest.raises(SphError) as ei:
            e.sync()
        assert ei.value.status == SPH_ESKIN


def test_lists_agree_with_cell_windows_at_size():
    """The 256^2 fluid: the same pair count and the two schemes' mixed
    evaluations within rounding of each other."""
    prm, r, v, m, T0 = workloads.config_2d(256, 1000, viscosity=True)
    u = oracle.initial_energy(prm, r, v, m, T0)
    with Engine(prm, "mixed", max_particles=len(r)) as e:
        s = e.add(prm, r, v, m, u)
        d0 = e.derivatives(s)
        n0 = e.pair_count(s)
        e.set_tuning(pair_scheme=2)
        d2 = e.derivatives(s)
        n2 = e.pair_count(s)
        assert lists_in_use(e)
    assert n0 == n2
    for k in ("rho", "vdot", "udot"):
        assert rel_l2(d2[k], d0[k]) < 5e-7, k


def test_batched_lists_match_oracle():
    """Several simulations in one engine on lists (constants from the
    simulation table)."""
    sims = [workloads.config_2d(side, 1100 + side, viscosity=True) for side in (16, 24, 20)]
    with Engine(sims[0][0], "mixed", max_particles=sum(len(x[1]) for x in sims),
                max_sims=len(sims)) as e:
        e.set_tuning(pair_scheme=2)
        ids, us = [], []
        for prm, r, v, m, T0 in sims:
            u = oracle.initial_energy(prm, r, v, m, T0)
            us.append(u)
            ids.append(e.add(prm, r, v, m, u))
        e.advance(10)
        e.sync()
        for sid, (prm, r, v, m, T0), u in zip(ids, sims, us):
            rr, vv, uu = e.get_state(sid)
            r1, v1, u1, _ = oracle.advance(prm, r, v, m, u, 10)
            assert rel_l2(rr, r1) < MIXED_TOL
            assert rel_l2(vv, v1) < MIXED_TOL
            assert rel_l2(uu, u1) < MIXED_TOL
        assert lists_in_use(e)


def test_lists_fall_back_where_they_do_not_apply():
    """FP64 and 3D engines asked for lists stay on cell windows (no build
    kernel) and keep their parity."""
    prm, r, v, m, T0 = workloads.config_2d(16, 1200, viscosity=True)
    u = oracle.initial_energy(prm, r, v, m, T0)
    ref = oracle.derivatives(prm, r, v, m, u)
    with Engine(prm, "fp64", max_particles=len(r)) as e:
        s = e.add(prm, r, v, m, u)
        k0 = e.kernels_per_step()
        e.set_tuning(pair_scheme=2)
        d = e.derivatives(s)
        assert e.kernels_per_step() == k0
        for k in ("rho", "vdot", "udot"):
            assert rel_l2(d[k], ref[k]) < 1e-12, k


def test_list_3d_golden_matches_reference():
    """A 3D golden system of the reference (Debrun kernel, 216 particles)."""
    g = load("debrun3d_216")
    prm = params_of(g)
    with listed(prm, g["r0"], g["v0"], g["m"], g["u0"]) as e:
        s = e.add(prm, g["r0"], g["v0"], g["m"], g["u0"])
        d = e.derivatives(s)
        e.sync()
        assert lists_in_use(e)
        errs = {k: rel_l2(d[k], g["ev_" + k]) for k in KEYS}
        bounds = {k: mixed_bound("debrun3d_216", k) for k in KEYS}
        record("list_evaluation", "debrun3d_216", "mixed", errs, bounds)
        for k, err in errs.items():
            assert err < bounds[k], (k, err, bounds[k])
        assert e.pair_count(s) == len(g["iap"])


def test_list_3d_heat_flux_matches_oracle():
    """The 3D cubic-spline fluid with viscosity and heat flux: one
    evaluation and 20 steps against the oracle."""
    prm, r, v, m, T0 = workloads.config_3d(12, 3000)
    u = oracle.initial_energy(prm, r, v, m, T0)
    u = u + prm.kbdash * 0.2 * T0 * np.sin(2 * np.pi * r[:, 0] / prm.box[0])
    ref = oracle.derivatives(prm, r, v, m, u)
    with listed(prm, r, v, m, u) as e:
        s = e.add(prm, r, v, m, u)
        d = e.derivatives(s)
        nip = e.pair_count(s)
        e.advance(20)
        e.sync()
        rr, vv, uu = e.get_state(s)
        assert lists_in_use(e)
    errs = {k: rel_l2(d[k], ref[k]) for k in KEYS + ("jq",)}
    record("list_full_physics", "cubic3d_heat_1728", "mixed", errs)
    for k, err in errs.items():
        assert err < (5e-6 if k == "jq" else MIXED_TOL), (k, err)
    assert nip == ref["nip"]
    r1, v1, u1, _ = oracle.advance(prm, r, v, m, u, 20)
    for a, b in ((rr, r1), (vv, v1), (uu, u1)):
        assert rel_l2(a, b) < MIXED_TOL


def test_lists_agree_with_clusters_in_3d():
    """The 3D fluid at 24^3: the same pair count as the cluster pairs and the
    cell windows, evaluations within rounding of each other."""
    prm, r, v, m, T0 = workloads.config_3d(24, 3001)
    u = oracle.initial_energy(prm, r, v, m, T0)
    # a temperature gradient, so that the heat flux is more than rounding
    u = u + prm.kbdash * 0.2 * T0 * np.sin(2 * np.pi * r[:, 0] / prm.box[0])
    out = {}
    with Engine(prm, "mixed", max_particles=len(r)) as e:
        s = e.add(prm, r, v, m, u)
        for scheme in (0, 1, 2):
            e.set_tuning(pair_scheme=scheme)
            out[scheme] = (e.derivatives(s), e.pair_count(s))
        assert lists_in_use(e)
    assert out[0][1] == out[1][1] == out[2][1]
    # jq differences of T carry each scheme's density rounding (held to
    # JQ_TOL against the oracle)
    for k in ("rho", "vdot", "udot", "jq"):
        assert rel_l2(out[2][0][k], out[0][0][k]) < (JQ_TOL if k == "jq" else 5e-7), k


@pytest.mark.parametrize("scheme", [0, 2])
def test_state_round_trips_keep_the_trajectory(scheme):
    """The end-to-end pattern -- the state out to the host and back in every
    step -- gives the bits of the plain advance: a state set within the
    cells' slack (and the lists' skin) goes into the current binning, and
    one beyond it is binned exactly as the step would have."""
    prm, r, v, m, T0 = workloads.config_2d(32, 1004, viscosity=True)
    v = v * 5.0
    u = oracle.initial_energy(prm, r, v, m, T0)
    knobs = dict(pair_scheme=scheme, rebin=1, steps_per_graph=1)
    with Engine(prm, "mixed", max_particles=len(r)) as e:
        s = e.add(prm, r, v, m, u)
        e.set_tuning(**knobs)
        e.advance(30)
        e.sync()
        ref = e.get_state(s)
        bins_ref = e.rebin_count()
    with Engine(prm, "mixed", max_particles=len(r)) as e:
        s = e.add(prm, r, v, m, u)
        e.set_tuning(**knobs)
        e.advance(1)
        for _ in range(29):
            rr, vv, uu = e.get_state(s)
            e.set_state(s, rr, vv, m, uu)
            e.advance(1)
        e.sync()
        got = e.get_state(s)
        assert bins_ref >= 2
    for a, b in zip(ref, got):
        assert np.array_equal(a, b)


def test_lists_grow_with_a_denser_state():
    """A state set from outside that is far denser than the one the rows were
    sized for: the engine measures again, grows the rows and evaluates the
    oracle's pair set; a later, sparser state keeps working."""
    rng = np.random.default_rng(11)
    n = 1600
    prm, r, v, m, T0 = workloads.config_2d(40, 1005, viscosity=True)
    r, v = r[:n], v[:n]
    m = np.full(n, 0.2)    # keeps the packed state's densities below the pole b rho = 1
    u = np.full(n, 0.5)
    with listed(prm, r, v, m, u) as e:
        s = e.add(prm, r, v, m, u)
        e.advance(2)
        e.sync()
        # the same particles packed into a quarter of the box: about four
        # times the neighbours per particle
        dense = 0.5 * r + rng.uniform(-0.05, 0.05, size=r.shape)
        e.set_state(s, dense, v, m, u)
        d = e.derivatives(s)
        nip = e.pair_count(s)
        ref = oracle.derivatives(prm, dense, v, m, u)
        assert nip == ref["nip"]
        for k in ("rho", "vdot", "udot"):
            assert rel_l2(d[k], ref[k]) < 1e-5, k
        e.advance(2)
        e.sync()
        e.set_state(s, r, v, m, u)
        d = e.derivatives(s)
        ref = oracle.derivatives(prm, r, v, m, u)
        for k in ("rho", "vdot", "udot"):
            assert rel_l2(d[k], ref[k]) < MIXED_TOL, k


def test_lists_follow_simulations_joining_and_leaving():
    """Simulations added to and removed from an engine on lists between
    advances (a new layout each time, the rows measured again): each one
    tracks the oracle's trajectory."""
    sims = workloads.batched_2d(3, seed_base=4300, n_lo=256, n_hi=2048, ramp_steps=10)
    st = [(p, r, v, m, oracle.initial_energy(p, r, v, m, T)) for p, r, v, m, T in sims]
    total = sum(len(x[1]) for x in st)
    with Engine(st[0][0], "mixed", max_particles=total, max_sims=3) as e:
        e.set_tuning(pair_scheme=2)
        a = e.add(*st[0])
        b = e.add(*st[1])
        e.advance(3)
        e.remove(b)
        c = e.add(*st[2])
        e.advance(3)
        e.sync()
        assert lists_in_use(e)
        ra = e.get_state(a)
        rc = e.get_state(c)
    for got, (p, r, v, m, u), steps in ((ra, st[0], 6), (rc, st[2], 3)):
        ref = oracle.advance(p, r, v, m, u, steps)[:3]
        for x, y in zip(got, ref):
            assert rel_l2(x, y) < MIXED_TOL


def test_profiled_advance_with_eager_steps():
    """Per-pass profiling over an advance that ends in eager steps (50 steps
    in graph chunks of 17: two graphs and 16 steps enqueued one by one) on
    pair lists: no error, every pass timed."""
    prm, r, v, m, T0 = workloads.config_2d(32, 1006, viscosity=True)
    u = oracle.initial_energy(prm, r, v, m, T0)
    with listed(prm, r, v, m, u) as e:
        s = e.add(prm, r, v, m, u)
        e.set_tuning(steps_per_graph=50)
        e.advance(50)
        e.sync()
        e.profile(True)
        e.advance(50)
        e.sync()
        prof = e.profile_read()
        e.profile(False)
        assert prof["force"]["launches"] > 0 and prof["force"]["ms"] > 0
        assert prof["density"]["launches"] == prof["force"]["launches"]
