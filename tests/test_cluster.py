"""The cluster-pair scheme (tuning pair_scheme = 1): 3D simulations in
mixed precision, their pairs evaluated as 8 x 4 blocks of compact particle
clusters from box-culled lists of each simulation.  The pair set is the reference's exact set
(neighbour_list.py:168-178), the results meet the mixed-precision bounds
against the FP64 oracle like the cell-window scheme, runs are deterministic,
and the cell scheme runs wherever the cluster scheme does not apply."""
import numpy as np
import pytest

from oracle import oracle
from pyticles_gb300 import Engine, SphError, build, make_params, workloads
from pyticles_gb300._abi import SPH_ESKIN
from tests.golden_cases import position_floor, rel_l2

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-6
JQ_TOL = 5e-6          # jq sums T_j - T_i: the pressure-only bound of the cell scheme's tests
# Debrun's gradient factor (h - r)^2 / r weighs the closest pairs most: on the
# Debrun system below the cell scheme shows 1.3e-6 (vdot, udot), this one 1.0e-6
DEBRUN_TOL = 2e-6
KEYS = ("rho", "rho_lr", "t", "p", "vdot", "udot")


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


def with_gradient(prm, r, v, m, T0):
    """Initial u with T = T0 (1 + 0.2 sin(2 pi x / L)) so the heat flux is real."""
    u = oracle.initial_energy(prm, r, v, m, T0)
    return u + prm.kbdash * 0.2 * T0 * np.sin(2 * np.pi * r[:, 0] / prm.box[0])


def case(name):
    if name == "cubic_heat_8000":
        prm, r, v, m, T0 = workloads.config_3d(20, 3100)
    elif name == "lucy_heat_4096":
        prm, r, v, m, T0 = workloads.config_3d(16, 3101, kernel="lucy", h_short=1.4, h_long=2.5)
    elif name == "gauss_4096":
        prm, r, v, m, T0 = workloads.config_3d(16, 3102, kernel="gaussian", h_short=0.9,
                                               h_long=1.4, cutoff=3.0, heat_flux=False)
    elif name == "debrun_rk4_4096":
        prm, r, v, m, T0 = workloads.config_3d(16, 3103, kernel="debrun", h_short=1.4,
                                               h_long=2.5, integrator="rk4")
    else:
        raise KeyError(name)
    return prm, r, v, m, with_gradient(prm, r, v, m, T0)


def engine(prm, r, v, m, u, scheme, precision="mixed", cap=1, **tune):
    e = Engine(prm, precision, max_particles=cap * len(r), max_sims=2)
    s = e.add(prm, r, v, m, u)
    e.set_tuning(pair_scheme=scheme, **tune)
    return e, s


CASES = ["cubic_heat_8000", "lucy_heat_4096", "gauss_4096", "debrun_rk4_4096"]


@pytest.mark.parametrize("name", CASES)
def test_cluster_scheme_matches_oracle(name):
    prm, r, v, m, u = case(name)
    ref = oracle.derivatives(prm, r, v, m, u)
    e, s = engine(prm, r, v, m, u, 1)
    with e:
        d = e.derivatives(s)
        e.sync()
        keys = KEYS + (("jq",) if prm.heat_flux else ())
        errs = {k: rel_l2(d[k], ref[k]) for k in keys}
        print(name, errs)
        tol = DEBRUN_TOL if name.startswith("debrun") else MIXED_TOL
        for k, err in errs.items():
            assert err < (JQ_TOL if k == "jq" else tol), (k, err)
        assert e.last_pair_total() == ref["nip"]
        e.advance(5)
        e.sync()
        rr, vv, uu = e.get_state(s)
    r5, v5, u5, _ = oracle.advance(prm, r, v, m, u, 5)
    assert rel_l2(rr, r5) < tol
    assert rel_l2(vv, v5) < tol
    assert rel_l2(uu, u5) < tol


@pytest.mark.parametrize("integ", ["euler", "ieuler", "rk4"])
def test_cluster_scheme_agrees_with_cell_scheme(integ):
    """Same pair set (pair counts equal) and trajectories equal to rounding
    over 12 steps, in graphs of 4."""
    prm, r, v, m, T0 = workloads.config_3d(20, 3110, integrator=integ)
    u = workloads.vdw_energy(np.full(len(r), 0.7), T0)
    out = {}
    for scheme in (0, 1):
        e, s = engine(prm, r, v, m, u, scheme, steps_per_graph=4)
        with e:
            d = e.derivatives(s)
            e.sync()
            pairs = e.last_pair_total()
            ks = e.kernels_per_step()
            e.advance(12)
            e.sync()
            out[scheme] = (d, pairs, ks, e.get_state(s))
    (d0, p0, k0, st0), (d1, p1, k1, st1) = out[0], out[1]
    assert p0 == p1
    assert k1 != k0                   # the cluster passes ran
    for k in ("rho", "vdot", "udot", "jq"):
        assert rel_l2(d1[k], d0[k]) < (JQ_TOL if k == "jq" else MIXED_TOL), k
    for a, b in zip(st1, st0):
        assert rel_l2(a, b) < MIXED_TOL


def test_cluster_scheme_is_deterministic():
    """Lists and sums follow the state only: eager steps, graphs of 5 and a
    second engine give the same bits."""
    prm, r, v, m, u = case("cubic_heat_8000")
    states = []
    for per, graph in ((5, 1), (1, 0), (5, 1)):
        e, s = engine(prm, r, v, m, u, 1, steps_per_graph=per, use_graph=graph)
        with e:
            e.advance(10)
            e.sync()
            states.append(e.get_state(s))
    for st in states[1:]:
        for a, b in zip(st, states[0]):
            assert np.array_equal(a, b)


def test_pass_profile_counts_every_chunk_of_an_advance():
    """With cluster pairs an advance replays its graph chunk by chunk; the
    pass profile times every launch, so 60 steps count three times the
    passes of 20 (graphs of 200 steps requested, chunks of 20 run)."""
    prm, r, v, m, u = case("cubic_heat_8000")
    launches = {}
    for steps in (20, 60):
        e, s = engine(prm, r, v, m, u, 1, steps_per_graph=200)
        with e:
            e.advance(2)
            e.sync()
            e.profile(True)
            e.prepare()
            e.advance(steps)
            e.sync()
            passes = e.profile_read()
            launches[steps] = {k: p["launches"] for k, p in passes.items()}
            assert all(p["ms"] >= 0.0 for p in passes.values())
    assert launches[20]["force"] > 0
    for k, n in launches[20].items():
        assert launches[60][k] == 3 * n, k


def test_cluster_scheme_with_binning_on_demand_and_thermostat():
    prm, r, v, m, T0 = workloads.config_3d(20, 3120, integrator="rk4", dt=2e-3)
    prm.thermostat = 1
    prm.thermostat_temp = 0.6
    prm.thermostat_temp_end = 0.3
    prm.thermostat_ramp_steps = 10
    u = workloads.vdw_energy(np.full(len(r), 0.7), T0)
    e, s = engine(prm, r, v, m, u, 1, rebin=1, steps_per_graph=4)
    with e:
        e.advance(12)
        e.sync()
        rr, vv, uu = e.get_state(s)
    ro, vo, uo, _ = oracle.advance(prm, r, v, m, u, 12)
    assert rel_l2(rr, ro) < MIXED_TOL
    assert rel_l2(vv, vo) < MIXED_TOL
    assert rel_l2(uu, uo) < MIXED_TOL


@pytest.mark.parametrize("what", ["2d", "fp64", "small_box"])
def test_cell_scheme_runs_where_clusters_do_not_apply(what):
    """pair_scheme = 1 leaves a 2D engine, an FP64 engine and a simulation
    whose box is narrower than five columns on the cell scheme: the same
    launches and the same bits as pair_scheme = 0."""
    precision = "mixed"
    if what == "2d":
        prm, r, v, m, T0 = workloads.config_2d(48, 3130)
    elif what == "small_box":
        prm, r, v, m, T0 = workloads.config_3d(12, 3131)
    else:
        prm, r, v, m, T0 = workloads.config_3d(20, 3132)
        precision = "fp64"
    u = workloads.vdw_energy(np.full(len(r), 0.7), T0)
    res = []
    for scheme in (0, 1):
        e, s = engine(prm, r, v, m, u, scheme, precision=precision, cap=2)
        with e:
            e.advance(3)
            e.sync()
            res.append((e.kernels_per_step(), e.get_state(s)))
    assert res[0][0] == res[1][0]
    for a, b in zip(res[0][1], res[1][1]):
        assert np.array_equal(a, b)


def test_cluster_scheme_flags_a_skin_violation():
    """A particle that outruns the allowed drift within a step raises
    SPH_ESKIN: the lists were culled with that drift as margin."""
    prm, r, v, m, u = case("cubic_heat_8000")
    e, s = engine(prm, r, v, m, u, 1)
    with e:
        v2 = v.copy()
        v2[7] = [5000.0, 0.0, 0.0]
        e.set_state(s, r, v2, m, u)
        e.advance(1)
        with pytest.raises(SphError) as ei:
            e.sync()
        assert ei.value.status == SPH_ESKIN


def test_cluster_scheme_full_size_invariants():
    """N = 110,592 (48^3): the pair count equals the oracle's, forces cancel
    pairwise and momentum is conserved over 5 steps."""
    prm, r, v, m, T0 = workloads.config_3d(48, 3140)
    u = workloads.vdw_energy(np.full(len(r), 0.7), T0)
    n_ref = len(oracle.pairs(prm, r)[0])
    e, s = engine(prm, r, v, m, u, 1)
    with e:
        d = e.derivatives(s)
        assert e.last_pair_total() == n_ref
        net = np.abs(d["vdot"].sum(axis=0)) / np.abs(d["vdot"]).sum(axis=0)
        assert np.all(net < 1e-6), net
        p0 = np.array(e.diagnostics(s)["momentum"])
        e.advance(5)
        e.sync()
        p1 = np.array(e.diagnostics(s)["momentum"])
    assert np.all(np.abs(p1 - p0) / np.abs(v).sum() < 1e-7), (p0, p1)


def test_autotuner_times_the_cluster_scheme_for_one_3d_simulation():
    """Cell windows, the pair lists (two block sizes) and the cluster pairs."""
    from pyticles_gb300 import autotune
    prm, r, v, m, T0 = workloads.config_3d(20, 3150)
    u = workloads.vdw_energy(np.full(len(r), 0.7), T0)
    knobs, table = autotune.tune(prm, "mixed", [(prm, r, v, m, u)], steps=2, warmup=1,
                                 blocks=(128,), ratios=(0.5,), use_cache=False)
    assert [row["pair_scheme"] for row in table] == [0, 2, 2, 1]
    assert knobs["pair_scheme"] in (0, 1, 2)
    _, table2 = autotune.tune(prm, "fp64", [(prm, r, v, m, u)], steps=2, warmup=1,
                              blocks=(128,), ratios=(0.5,), use_cache=False)
    assert [row["pair_scheme"] for row in table2] == [0]


def test_autotuner_times_the_persistent_launch_for_batches():
    """A mixed-precision batch: the cell-window candidates, then the
    persistent launch form at the best of them, then the 2D pair lists; a
    single simulation and an FP64 batch get no persistent candidate, and
    FP64 no lists."""
    from pyticles_gb300 import autotune
    sims = [(p, r, v, m, oracle.initial_energy(p, r, v, m, T))
            for p, r, v, m, T in workloads.batched_2d(3, seed_base=4600, n_lo=256, n_hi=1024,
                                                      ramp_steps=10)]
    knobs, table = autotune.tune(sims[0][0], "mixed", sims, steps=2, warmup=1,
                                 blocks=(64, 128), ratios=(0.5,), use_cache=False)
    cells = [row for row in table if row["pair_scheme"] == 0]
    assert [row["persistent"] for row in cells] == [0, 0, 1]
    best_cell = min(cells[:2], key=lambda row: row["ms_per_step"])
    assert cells[2]["block_size"] == best_cell["block_size"]
    assert [row["pair_scheme"] for row in table] == [0, 0, 0, 2, 2]
    assert knobs["persistent"] in (0, 1)
    _, one = autotune.tune(sims[0][0], "mixed", sims[:1], steps=2, warmup=1, blocks=(128,),
                           ratios=(0.5,), use_cache=False)
    _, fp64 = autotune.tune(sims[0][0], "fp64", sims, steps=2, warmup=1, blocks=(128,),
                            ratios=(0.5,), use_cache=False)
    assert [(row["pair_scheme"], row["persistent"]) for row in one] == [(0, 0), (2, 0), (2, 0)]
    assert [(row["pair_scheme"], row["persistent"]) for row in fp64] == [(0, 0)]


def droplet(seed=3160, gas=False):
    """8000 particles at density 1.4 in a cube of side 17.9 inside a periodic
    box of side 40 (mean density 0.125), or with gas=True the same particles
    spread uniformly over the box.  Columns follow the mean density; the
    lists of the dense region are about four times longer than a uniform
    fluid's at that mean."""
    rng = np.random.Generator(np.random.PCG64(seed))
    side, dens, L = 20, 1.4, 40.0
    if gas:
        r = rng.uniform(0.0, L, size=(side ** 3, 3))
    else:
        s = dens ** (-1.0 / 3.0)
        g = (np.arange(side) + 0.5) * s
        r = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
        r = r + rng.uniform(-0.1, 0.1, r.shape) * s + 4.0
    prm = make_params(dim=3, kernel="cubic", box=[L] * 3, h_short=2.735 / 2, h_long=5.148 / 2,
                      viscosity=True, heat_flux=True, dt=1e-3)
    v = rng.normal(0.0, np.sqrt(0.6), size=r.shape)
    v -= v.mean(axis=0)
    m = np.ones(len(r))
    return prm, r, v, m, oracle.initial_energy(prm, r, v, m, 0.6)


def test_cluster_lists_are_sized_by_measurement_for_a_dense_droplet():
    prm, r, v, m, u = droplet()
    ref = oracle.derivatives(prm, r, v, m, u)
    kps = {}
    for scheme in (0, 1):
        e, s = engine(prm, r, v, m, u, scheme)
        with e:
            d = e.derivatives(s)
            e.sync()
            kps[scheme] = e.kernels_per_step()
            if scheme == 1:
                for k in ("rho", "vdot", "udot"):
                    assert rel_l2(d[k], ref[k]) < MIXED_TOL, k
                assert e.last_pair_total() == ref["nip"]
                e.advance(4)
                e.sync()                     # no SPH_ECAPACITY
    assert kps[1] != kps[0]


def test_cluster_lists_follow_a_state_that_condenses():
    """A gas whose state is replaced by the droplet (set_state): the engine
    measures the lists again before the next step."""
    prm, r, v, m, u = droplet(gas=True)
    _, rd, vd, md, ud = droplet()
    e, s = engine(prm, r, v, m, u, 1, steps_per_graph=2)
    with e:
        e.advance(4)
        e.sync()
        e.set_state(s, rd, vd, md, ud)
        e.advance(4)
        e.sync()                             # no SPH_ECAPACITY
        rr, vv, uu = e.get_state(s)
    ro, vo, uo, _ = oracle.advance(prm, rd, vd, md, ud, 4)
    assert rel_l2(rr, ro) < MIXED_TOL and rel_l2(uu, uo) < MIXED_TOL


def test_cluster_lists_grow_within_one_advance():
    """A gas imploding towards the box centre (v = -(r - c)): over 200 steps
    in one call the densest lists grow by more than the 1.4 times headroom of
    a measurement, so the call must re-measure between its chunks of steps.
    It runs without SPH_ECAPACITY, gives the bits of the same steps taken in
    calls of 10, and its final state has the oracle's pair set."""
    spatial = pytest.importorskip("scipy.spatial")
    prm, r, v, m, u = droplet(gas=True)
    L = prm.box[0]
    v = v - (r - 0.5 * L)
    rc = prm.cutoff
    counts0 = spatial.cKDTree(r, boxsize=L).query_ball_point(r, rc, return_length=True)
    out = []
    for calls in ((200,), (10,) * 20):
        e, s = engine(prm, r, v, m, u, 1, steps_per_graph=200)
        with e:
            for n in calls:
                e.advance(n)
            e.sync()                         # no SPH_ECAPACITY
            out.append(e.get_state(s) + (e.pair_count(s),))
    for a, b in zip(out[0][:3], out[1][:3]):
        assert np.array_equal(a, b)
    rr, vv, uu, npairs = out[0]
    counts1 = spatial.cKDTree(np.mod(rr, L), boxsize=L).query_ball_point(
        np.mod(rr, L), rc, return_length=True)
    assert counts1.max() > 1.5 * counts0.max()
    assert npairs == oracle.derivatives(prm, rr, vv, m, uu)["nip"]


def test_particle_system_with_cluster_pairs():
    """SmoothParticleSystem(d=3, precision='mixed', pair_scheme=1).run: the
    Python API path on cluster pairs, against the FP64 oracle."""
    from pyticles_gb300 import PeriodicBox, SmoothParticleSystem, SpamComplete, VerletList
    prm, r, v, m, u = case("cubic_heat_8000")
    n = len(r)
    L = prm.box[0]
    p = SmoothParticleSystem(n, d=3, maxn=n, hshort=prm.h_short, hlong=prm.h_long,
                             simbox=PeriodicBox(xmax=L, ymax=L, zmax=L), precision="mixed",
                             pair_scheme=1)
    p.r[:] = r
    p.v[:] = v
    p.m[:] = m
    p.u[:] = u
    nl = VerletList(p, cutoff=prm.cutoff, tolerance=0.0)
    p.nlists.append(nl)
    p.nl_default = nl
    p.forces.append(SpamComplete(p, nl, eta=prm.visc_alpha, zeta=prm.visc_beta,
                                 cutoff=prm.cutoff, kernel="cubic", heat_flux=True))
    p.run(prm.dt, 6)
    assert p._engine.tuning["pair_scheme"] == 1
    ro, vo, uo, _ = oracle.advance(prm, r, v, m, u, 6)
    assert rel_l2(p.r[:n], ro) < MIXED_TOL and rel_l2(p.v[:n], vo) < MIXED_TOL
    assert rel_l2(p.u[:n], uo) < MIXED_TOL
    p.close()


def test_cluster_scheme_in_a_rectangular_box():
    """Different extents per axis (different column counts and slab
    heights): pair count and derivatives against the oracle, 3 RK4 steps."""
    rng = np.random.Generator(np.random.PCG64(3170))
    s = 0.7 ** (-1.0 / 3.0)
    nx, ny, nz = 26, 19, 15
    g = [(np.arange(k) + 0.5) * s for k in (nx, ny, nz)]
    r = np.stack(np.meshgrid(*g, indexing="ij"), -1).reshape(-1, 3)
    r = r + rng.uniform(-0.1, 0.1, r.shape) * s
    box = [nx * s, ny * s, nz * s]
    prm = make_params(dim=3, kernel="cubic", box=box, h_short=2.735 / 2, h_long=5.148 / 2,
                      viscosity=True, heat_flux=True, dt=1e-3, integrator="rk4")
    v = rng.normal(0.0, np.sqrt(0.6), size=r.shape)
    v -= v.mean(axis=0)
    m = np.ones(len(r))
    u = with_gradient(prm, r, v, m, 0.6)
    ref = oracle.derivatives(prm, r, v, m, u)
    kps = []
    for scheme in (0, 1):
        e, s_ = engine(prm, r, v, m, u, scheme)
        with e:
            kps.append(e.kernels_per_step())
            if scheme == 0:
                continue
            d = e.derivatives(s_)
            e.sync()
            for k in ("rho", "vdot", "udot"):
                assert rel_l2(d[k], ref[k]) < MIXED_TOL, k
            assert e.last_pair_total() == ref["nip"]
            e.advance(3)
            e.sync()
            rr, vv, uu = e.get_state(s_)
    assert kps[1] != kps[0]
    ro, vo, uo, _ = oracle.advance(prm, r, v, m, u, 3)
    assert rel_l2(rr, ro) < MIXED_TOL and rel_l2(uu, uo) < MIXED_TOL


def batch_of_3d():
    """Three 3D fluids of different size, density and temperature (the same
    kernel and flags: one engine group)."""
    sims = []
    for side, dens, T, seed in ((20, 0.7, 0.6, 3180), (24, 0.55, 0.9, 3181), (18, 0.8, 0.5, 3182)):
        prm, r, v, m, T0 = workloads.config_3d(side, seed, density=dens, integrator="rk4")
        sims.append((prm, r, v, m, with_gradient(prm, r, v, m, T)))
    return sims


def test_cluster_scheme_batched_equals_alone():
    """Each simulation's columns, clusters and lists are its own, and its
    sums follow them alone: a simulation gives the same bits in a batch of
    three as alone."""
    sims = batch_of_3d()
    total = sum(len(x[1]) for x in sims)
    with Engine(sims[0][0], "mixed", max_particles=total, max_sims=3) as e:
        ids = [e.add(*x) for x in sims]
        e.set_tuning(pair_scheme=1, steps_per_graph=4)
        ks = e.kernels_per_step()
        e.advance(8)
        e.sync()
        batched = [e.get_state(i) for i in ids]
    with Engine(sims[0][0], "mixed", max_particles=total, max_sims=3) as e0:
        for x in sims:
            e0.add(*x)
        assert e0.kernels_per_step() != ks           # the cluster passes ran
    for x, got in zip(sims, batched):
        e, s = engine(*x, 1, steps_per_graph=4)
        with e:
            e.advance(8)
            e.sync()
            alone = e.get_state(s)
        for a, b in zip(got, alone):
            assert np.array_equal(a, b)


def test_cluster_scheme_batch_matches_oracle():
    sims = batch_of_3d()
    total = sum(len(x[1]) for x in sims)
    with Engine(sims[0][0], "mixed", max_particles=total, max_sims=3) as e:
        ids = [e.add(*x) for x in sims]
        e.set_tuning(pair_scheme=1)
        derivs = [e.derivatives(i) for i in ids]
        e.sync()
        assert e.last_pair_total() == sum(oracle.derivatives(*x)["nip"] for x in sims)
    for x, d in zip(sims, derivs):
        ref = oracle.derivatives(*x)
        for k in ("rho", "vdot", "udot"):
            assert rel_l2(d[k], ref[k]) < MIXED_TOL, k


def test_schemes_side_by_side_keep_each_simulation_alone():
    """A simulation whose box admits columns runs on cluster pairs, one whose
    box does not on cell windows, in the same engine and the same steps; each
    gives the bits it gives alone (where its scheme is the same choice)."""
    big = workloads.config_3d(20, 3190, integrator="rk4")
    small = workloads.config_3d(12, 3191, integrator="rk4")
    sims = []
    for prm, r, v, m, T0 in (big, small):
        sims.append((prm, r, v, m, with_gradient(prm, r, v, m, T0)))
    total = sum(len(x[1]) for x in sims)
    with Engine(sims[0][0], "mixed", max_particles=total, max_sims=2) as e:
        ids = [e.add(*x) for x in sims]
        e.set_tuning(pair_scheme=1, steps_per_graph=3)
        ks = e.kernels_per_step()
        d = [e.derivatives(i) for i in ids]
        e.sync()
        assert e.last_pair_total() == sum(oracle.derivatives(*x)["nip"] for x in sims)
        for x, di in zip(sims, d):
            ref = oracle.derivatives(*x)
            for k in ("rho", "vdot", "udot"):
                assert rel_l2(di[k], ref[k]) < MIXED_TOL, k
        e.advance(6)
        e.sync()
        mixed = [e.get_state(i) for i in ids]
    with Engine(sims[0][0], "mixed", max_particles=total, max_sims=2) as e0:
        for x in sims:
            e0.add(*x)
        assert e0.kernels_per_step() < ks        # both schemes' passes ran
    for x, got in zip(sims, mixed):
        e, s = engine(*x, 1, steps_per_graph=3)
        with e:
            e.advance(6)
            e.sync()
            alone = e.get_state(s)
        for a, b in zip(got, alone):
            assert np.array_equal(a, b)


def random_system(seed):
    """A 3D system with random kernel, smoothing lengths, box shape and
    density, placement (uniform, clumped, or with an empty slab), flags and
    integrator."""
    rng = np.random.Generator(np.random.PCG64(seed))
    kernel = ["cubic", "lucy", "gaussian", "debrun"][seed % 4]
    h_s = rng.uniform(0.8, 1.4)
    h_l = h_s * rng.uniform(1.3, 2.0)
    cutoff = (2.0 if kernel == "cubic" else 1.0) * h_l
    if kernel == "gaussian":
        cutoff = 2.0 * h_l
    dens = rng.uniform(0.3, 1.0)
    box = rng.uniform(4.5, 6.5, size=3) * cutoff
    n = int(dens * box.prod())
    kind = seed % 3
    if kind == 0:
        r = rng.uniform(0.0, 1.0, size=(n, 3)) * box
    elif kind == 1:                 # clumps
        centres = rng.uniform(0.0, 1.0, size=(6, 3)) * box
        r = (centres[rng.integers(0, 6, n)] + rng.normal(0.0, 1.2 * h_s, size=(n, 3))) % box
    else:                           # an empty slab across z
        r = rng.uniform(0.0, 1.0, size=(n, 3)) * box * np.array([1.0, 1.0, 0.6])
    prm = make_params(dim=3, kernel=kernel, box=list(box), h_short=h_s, h_long=h_l,
                      cutoff=cutoff, viscosity=bool(seed % 2), heat_flux=bool((seed // 2) % 2),
                      dt=5e-4, integrator=["euler", "ieuler", "rk4"][seed % 3])
    v = rng.normal(0.0, 0.6, size=r.shape)
    v -= v.mean(axis=0)
    m = rng.uniform(0.8, 1.2, size=n)
    u = oracle.initial_energy(prm, r, v, m, 0.6)
    return prm, r, v, m, u


@pytest.mark.parametrize("seed", range(12))
def test_random_3d_systems_match_oracle(seed):
    """Random systems (sparse and dense columns, clusters spread over many
    slabs, z windows wrapping the box, some boxes too small for columns):
    pair counts exact, and the mixed-precision errors against the oracle no
    larger than the cell scheme's on the same system.  Uniformly random
    placements put particles nearly on top of each other and push local
    densities past the van der Waals pole (b rho = 1), so on some systems
    FP32 rounding of the positions alone moves the FP64 forces by 1e-5 to
    3e-4 (the position floor): there both schemes' errors are that floor
    times a random factor, and the bound is a small multiple of it."""
    prm, r, v, m, u = random_system(4000 + seed)
    floor = position_floor(prm, r, v, m, u)
    ref = oracle.derivatives(prm, r, v, m, u)
    ro, vo, uo, _ = oracle.advance(prm, r, v, m, u, 3)
    errs = {}
    for scheme in (0, 1):
        e, s = engine(prm, r, v, m, u, scheme)
        with e:
            d = e.derivatives(s)
            e.sync()
            assert e.last_pair_total() == ref["nip"], scheme
            e.advance(3)
            e.sync()
            rr, vv, uu = e.get_state(s)
        errs[scheme] = {k: rel_l2(d[k], ref[k]) for k in ("rho", "vdot", "udot")}
        errs[scheme].update(r3=rel_l2(rr, ro), u3=rel_l2(uu, uo))
    print(seed, errs, {k: floor[k] for k in ("rho", "vdot", "udot")})
    for k, err in errs[1].items():
        assert err < 2 * max(errs[0][k], 3 * floor.get(k, 0.0), MIXED_TOL), (k, errs, floor)
