"""The reference-facing API (pyticles_gb300 mirrors of particles.py,
neighbour_list.py, forces.py, spam_complete_force.py, box.py), with the
reference's own unit tests re-expressed (test/neighbour_list_test.py,
test/force_test.py) and a run script in the shape of run_scripts/bspana_profile.py.
Host-side logic runs on CPU; anything that evaluates runs on the GPU."""
import numpy as np
import pytest

from oracle import oracle
from pyticles_gb300 import (CohesiveSpamForce, CohesiveSpamForce2d, MirrorBox, NeighbourList,
                            ParticleSystem, PeriodicBox, SmoothParticleSystem, SortedVerletList,
                            SpamComplete, SpamForce, SpamForce2d, VerletList, integrator,
                            workloads)
from pyticles_gb300.box import wrap_teleport
from tests.golden_cases import load, params_of, rel_l2, sort_pairs


# ---- host logic (CPU) ----

def test_minimum_image_matches_reference_rule():
    dr = np.array([3.0, -3.0, 0.4])
    NeighbourList.minimum_image(dr, 5.0, 5.0, 1.0)
    assert np.allclose(dr, [-2.0, 2.0, 0.4])
    dr = np.array([2.5, -2.5, 0.5])   # exactly L/2: strict comparisons keep it
    NeighbourList.minimum_image(dr, 5.0, 5.0, 1.0)
    assert np.allclose(dr, [2.5, -2.5, 0.5])


def test_ponder_rebuild_host_logic():
    """test/neighbour_list_test.py:48-53: False after build, True once a
    particle moved further than the tolerance."""
    p = ParticleSystem(3, d=3, maxn=3)
    nl = VerletList(p, cutoff=10, tolerance=2)
    nl.r_old[:, :] = p.r[:, :]
    nl.ponder_rebuild()
    assert nl.rebuild_list is False
    p.r[0, :] = (100.0, 100.0, 100.0)
    nl.ponder_rebuild()
    assert nl.rebuild_list is True


def _filled_system(d, n=5, maxn=7, seed=11):
    rng = np.random.Generator(np.random.PCG64(seed))
    p = SmoothParticleSystem(n, d=d, maxn=maxn)
    for a in (p.r, p.v, p.m, p.rho, p.p, p.pco, p.u, p.vdot, p.udot, p.rhodot):
        a[...] = rng.uniform(0.5, 2.0, a.shape)
    p.rdot = p.v
    return p


@pytest.mark.parametrize("d", [2, 3])
def test_state_vector_rows_follow_the_reference(d):
    """gather_state / gather_derivatives fill the reference's 11 rows
    (particles.py:496-511, 528-542): m, x, y, z, vx, vy, vz, rho, p, pco, u
    and mdot, rdot, vdot, rhodot, 0, 0, udot; a 2D system leaves the z rows
    at zero."""
    p = _filled_system(d)
    n = p.n
    x = p.gather_state()
    assert x.shape == (11, p.maxn)
    assert np.array_equal(x[0, :n], p.m[:n])
    for a in range(3):
        want_r = p.r[:n, a] if a < d else np.zeros(n)
        want_v = p.v[:n, a] if a < d else np.zeros(n)
        assert np.array_equal(x[1 + a, :n], want_r)
        assert np.array_equal(x[4 + a, :n], want_v)
    for row, arr in zip(range(7, 11), (p.rho, p.p, p.pco, p.u)):
        assert np.array_equal(x[row, :n], arr[:n])
    assert not x[:, n:].any()                  # rows beyond n stay untouched
    xd = p.gather_derivatives()
    assert np.array_equal(xd[0, :n], p.mdot[:n])
    for a in range(d):
        assert np.array_equal(xd[1 + a, :n], p.v[:n, a])
        assert np.array_equal(xd[4 + a, :n], p.vdot[:n, a])
    assert np.array_equal(xd[7, :n], p.rhodot[:n])
    assert not xd[8:10].any()
    assert np.array_equal(xd[10, :n], p.udot[:n])


@pytest.mark.parametrize("d", [2, 3])
def test_scatter_state_inverts_gather_state(d):
    p = _filled_system(d)
    x = p.gather_state().copy()
    x[:, :p.n] *= 3.0
    q = _filled_system(d, seed=12)
    q.scatter_state(x)
    assert np.array_equal(q.gather_state(), x)
    assert np.array_equal(q.r[:q.n], 3.0 * p.r[:p.n])
    assert np.array_equal(q.u[:q.n], 3.0 * p.u[:p.n])


def test_create_particle_appends_with_the_last_mass():
    """particles.py:171-178: the new particle takes index n and the mass of
    particle n - 1; the system refuses more than maxn particles."""
    p = _filled_system(3, n=5, maxn=6)
    p.create_particle((1.0, 2.0, 3.0))
    assert p.n == 6
    assert np.array_equal(p.r[5], [1.0, 2.0, 3.0])
    assert p.m[5] == p.m[4]
    assert not p.v[5].any()
    with pytest.raises(ValueError):
        p.create_particle((0.0, 0.0, 0.0))


def test_property_formulas(capsys):
    """properties.py:24-60: the equations of state and the Hamiltonian
    (kinetic energy plus the unweighted sum of u), printed and returned."""
    from pyticles_gb300 import properties
    rho, t = np.array([0.5, 1.5]), np.array([0.6, 1.2])
    assert np.array_equal(properties.ideal_isothermal(rho, t), rho)
    assert np.array_equal(properties.art_water(rho, t), rho - 1.0)
    assert np.allclose(properties.vdw_temp(rho, properties.vdw_energy(rho, t)), t)
    p = _filled_system(3)
    want = sum(0.5 * p.m[i] * (p.v[i] @ p.v[i]) + p.u[i] for i in range(p.n))
    assert properties.hamiltonian(p) == pytest.approx(want, rel=1e-14)
    assert float(capsys.readouterr().out) == pytest.approx(want, rel=1e-14)


def test_periodic_box_teleports():
    r = np.array([[5.5, -0.1], [0.0, 5.0], [-2.0, 7.0]])
    wrap_teleport(r, (5.0, 5.0))
    assert np.array_equal(r, [[0.0, 5.0], [0.0, 5.0], [5.0, 0.0]])


def test_mirror_box_is_refused_by_the_engine():
    p = SmoothParticleSystem(4, d=2, maxn=4)
    nl = VerletList(p, cutoff=1.0, tolerance=0.0)
    p.nlists.append(nl)
    p.forces.append(SpamComplete(p, nl))
    assert isinstance(p.box, MirrorBox)
    with pytest.raises(NotImplementedError):
        p.engine_params(1e-3)


def test_engine_params_from_reference_objects():
    box = PeriodicBox(xmax=20, ymax=20, zmax=1)
    p = SmoothParticleSystem(400, d=2, maxn=400, hshort=3.0, hlong=6.0, simbox=box,
                             integrator="ieuler", thermostat=True, thermostat_temp=0.4)
    nl = VerletList(p, cutoff=6.0, tolerance=0.5)
    p.nlists.append(nl)
    p.nl_default = nl
    p.forces.append(SpamComplete(p, nl, eta=0.8, zeta=0.2))
    prm = p.engine_params(2e-3)
    assert (prm.dim, prm.kernel, prm.viscosity, prm.thermostat) == (2, 2, 1, 1)
    assert (prm.visc_alpha, prm.visc_beta, prm.cutoff, prm.tolerance) == (0.8, 0.2, 6.0, 0.5)
    assert (prm.h_short, prm.h_long, prm.dt, prm.thermostat_temp) == (3.0, 6.0, 2e-3, 0.4)
    p.forces = [SpamForce(p, nl), CohesiveSpamForce(p, nl)]
    assert p.engine_params(1e-3).viscosity == 0
    # the 2D classes (forces.py:246-318) configure the same evaluation
    p.forces = [SpamForce2d(p, nl), CohesiveSpamForce2d(p, nl)]
    prm2 = p.engine_params(1e-3)
    assert (prm2.kernel, prm2.viscosity, prm2.heat_flux) == (2, 0, 0)
    assert p.engine_params(1e-3, thermostat=False).thermostat == 0


def test_integrator_runs_any_callbacks_like_the_reference():
    """integrator.euler/imp_euler/rk4 run the engine step for the system
    whose gather_state, derivatives, gather_derivatives and scatter_state
    they get; any other callables get the reference's generic scheme
    (integrator.py:14-103): here a harmonic oscillator x' = v, v' = -x, one
    step of each against the scheme written out."""
    p = SmoothParticleSystem(4, d=2, maxn=4)
    q = SmoothParticleSystem(4, d=2, maxn=4)
    own = (p.gather_state, p.derivatives, p.gather_derivatives, p.scatter_state)
    assert integrator._system(*own) is p
    mixed = (p.gather_state, q.derivatives, p.gather_derivatives, p.scatter_state)
    assert integrator._system(*mixed) is None

    class Osc:
        def __init__(self):
            self.x = np.array([1.0, 0.5])
            self.calls = 0

        def get_state(self):
            return self.x.copy()

        def calc(self):
            self.calls += 1
            self.rate = np.array([self.x[1], -self.x[0]])

        def get_derivs(self):
            return self.rate

        def set_state(self, x):
            self.x = np.asarray(x, dtype=float)

    f = lambda x: np.array([x[1], -x[0]])
    dt = 0.1
    x0 = np.array([1.0, 0.5])
    c1 = f(x0) * dt
    want = {"euler": x0 + c1,
            "imp_euler": x0 + (c1 + f(x0 + c1) * dt) / 2}
    k2 = f(x0 + c1 / 2) * dt
    k3 = f(x0 + k2 / 2) * dt
    k4 = f(x0 + k3) * dt
    want["rk4"] = x0 + (1.0 / 6.0) * (c1 + 2. * k2 + 2. * k3 + k4)
    for name, evals in (("euler", 1), ("imp_euler", 2), ("rk4", 4)):
        o = Osc()
        getattr(integrator, name)(o.get_state, o.calc, o.get_derivs, o.set_state, dt)
        assert np.array_equal(o.x, want[name]), name
        assert o.calls == evals
    # a system the engine refuses (no periodic box) keeps its own integrator
    nl = VerletList(p, cutoff=1.0, tolerance=0.0)
    p.nlists.append(nl)
    p.forces.append(SpamComplete(p, nl))
    for step in (integrator.euler, integrator.rk4):
        with pytest.raises(NotImplementedError):
            step(*own, 1e-3)
        assert p.integrator == "ieuler"


def test_spam_complete_reports_the_terms_it_does_not_compute():
    """sigma / rcoef (repulsive core) raise; cgrad (density-gradient term,
    reference default 1.0) warns once and is not computed; cgrad = 0, as the
    reference's drivers pass it, is silent."""
    import warnings

    from pyticles_gb300 import forces
    p = SmoothParticleSystem(4, d=2, maxn=4)
    nl = VerletList(p, cutoff=1.0, tolerance=0.0)
    with pytest.raises(NotImplementedError):
        SpamComplete(p, nl, sigma=1.0, cgrad=0.0)
    with pytest.raises(NotImplementedError):
        SpamComplete(p, nl, rcoef=1.0, cgrad=0.0)
    forces._cgrad_warned = False
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        SpamComplete(p, nl, cgrad=0.0)
        assert not w
        SpamComplete(p, nl)                 # the reference default cgrad = 1.0
        SpamComplete(p, nl, cgrad=0.5)
    assert len(w) == 1 and issubclass(w[0].category, RuntimeWarning)
    assert "cgrad" in str(w[0].message)


# ---- evaluation (GPU) ----

@pytest.mark.gpu
def test_reference_nlist_tests():
    """test/neighbour_list_test.py:8-53 through the GPU pair export."""
    p = ParticleSystem(3, d=3, maxn=3)
    p.r[0, :] = (0.0, 0.0, 0.0)
    p.r[1, :] = (1.0, 0.0, 0.0)
    p.r[2, :] = (0.0, 0.0, 1.0)
    nl = NeighbourList(p)
    nl.build()
    nl.separations()
    k = nl.find_pair(0, 1)
    assert nl.rij[k] == 1.0
    nl2 = VerletList(p, cutoff=10, tolerance=2)
    nl2.build()
    nl2.compress()
    nl2.separations()
    assert nl2.rij[0] == 1.0
    nl2.ponder_rebuild()
    assert nl2.rebuild_list is False
    p.r[0, :] = (100.0, 100.0, 100.0)
    nl2.ponder_rebuild()
    assert nl2.rebuild_list is True
    nl.close()
    nl2.close()


@pytest.mark.gpu
def test_sorted_verlet_list_matches_reference_pairs():
    g = load("lucy2d_400")
    box = PeriodicBox(xmax=20, ymax=20, zmax=1)
    p = SmoothParticleSystem(400, d=2, maxn=400, simbox=box)
    p.r[:] = g["r0"]
    p.v[:] = g["v0"]
    nl = SortedVerletList(p, cutoff=6.0, tolerance=0.0)
    nl.build()
    got, _ = sort_pairs(nl.iap)
    ref, _ = sort_pairs(g["iap"])
    assert np.array_equal(got, ref)
    assert np.all(np.diff(nl.rsq) <= 0)   # descending separation
    nl.close()


def bspana_like(g, precision, steps):
    """run_scripts/bspana_profile.py:39-61 with the periodic box."""
    box = PeriodicBox(xmax=float(g["box"][0]), ymax=float(g["box"][1]), zmax=1)
    n = len(g["r0"])
    p = SmoothParticleSystem(n, d=2, maxn=n, hshort=float(g["h_short"]),
                             hlong=float(g["h_long"]), simbox=box, integrator="ieuler",
                             precision=precision)
    p.r[:] = g["r0"]
    p.v[:] = g["v0"]
    p.m[:] = g["m"]
    p.u[:] = g["u0"]
    nl = VerletList(p, cutoff=float(g["cutoff"]), tolerance=0.0)
    p.nlists.append(nl)
    p.nl_default = nl
    p.forces.append(SpamComplete(p, nl, eta=0.0, zeta=0.0))
    for _ in range(steps):
        p.update(float(g["dt"]))
    return p


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 5e-6)])
def test_update_matches_reference_trajectory(precision, tol):
    g = load("lucy2d_400")
    p = bspana_like(g, precision, int(g["steps"]))
    assert rel_l2(p.r, g["r_final"]) < tol
    assert rel_l2(p.v, g["v_final"]) < tol
    assert rel_l2(p.u, g["u_final"]) < tol
    for k in ("rho", "rho_lr", "t", "p", "pco", "vdot", "udot"):
        assert rel_l2(getattr(p, k), g["after_" + k]) < tol, k
    assert p.steps == int(g["steps"])
    p.close()


@pytest.mark.gpu
def test_force_apply_writes_reference_arrays():
    """SpamComplete.apply / p.derivatives() fill rho, p, pco, t, vdot, udot
    (spam_complete_force.py:171-183) with one evaluation."""
    g = load("lucy2d_1024")
    p = bspana_like(g, "fp64", 0)
    p.forces[0].apply()
    for k in ("rho", "rho_lr", "t", "p", "pco", "vdot", "udot"):
        assert rel_l2(getattr(p, k), g["ev_" + k]) < 1e-12, k
    p.close()


@pytest.mark.gpu
def test_run_many_steps_equals_update_loop():
    prm, r, v, m, T0 = workloads.config_2d(24, 77, viscosity=True)
    u = oracle.initial_energy(prm, r, v, m, T0)
    out = []
    for mode in ("update", "run"):
        box = PeriodicBox(xmax=24, ymax=24, zmax=1)
        p = SmoothParticleSystem(len(r), d=2, maxn=len(r), hshort=3.0, hlong=6.0, simbox=box,
                                 precision="mixed")
        p.r[:], p.v[:], p.m[:], p.u[:] = r, v, m, u
        nl = VerletList(p, cutoff=6.0, tolerance=0.0)
        p.nlists.append(nl)
        p.forces.append(SpamComplete(p, nl))
        if mode == "update":
            for _ in range(4):
                p.update(1e-3)
        else:
            p.run(1e-3, 4)
        out.append((p.r.copy(), p.v.copy(), p.u.copy()))
        p.close()
    for a, b in zip(*out):
        assert np.array_equal(a, b)


@pytest.mark.gpu
def test_spam_properties_matches_reference():
    """properties.spam_properties(p, nl) on the GPU against the reference's
    own output (tests/golden/spam_props.npz)."""
    from pyticles_gb300 import properties
    g = load("spam_props")
    n = len(g["r"])
    box = PeriodicBox(xmax=3.3, ymax=3.3, zmax=3.3)
    p = SmoothParticleSystem(n, d=3, maxn=n, hshort=float(g["h"]), hlong=float(g["hlr"]),
                             simbox=box)
    p.r[:] = g["r"]
    p.v[:] = g["v"]
    p.m[:] = g["m"]
    p.t[:] = float(g["T0"])
    nl = VerletList(p, cutoff=float(g["cutoff"]), tolerance=0.0)
    properties.spam_properties(p, nl)
    for k in ("rho", "p", "pco", "u", "t"):
        a, b = getattr(p, k)[:n], g[k]
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < 1e-12, k
    # spam_properties_ls: the same, plus rho_lr at the long length (the
    # oracle's long density of the same state)
    q = SmoothParticleSystem(n, d=3, maxn=n, hshort=float(g["h"]), hlong=float(g["hlr"]),
                             simbox=box)
    q.r[:] = g["r"]
    q.v[:] = g["v"]
    q.m[:] = g["m"]
    q.t[:] = float(g["T0"])
    properties.spam_properties_ls(q, nl)
    for k in ("rho", "p", "pco", "u", "t"):
        assert np.array_equal(getattr(q, k)[:n], getattr(p, k)[:n]), k
    prm = params_of({"dim": 3, "kernel": "lucy", "box": [3.3] * 3, "h_short": float(g["h"]),
                     "h_long": float(g["hlr"]), "cutoff": float(g["cutoff"]), "tolerance": 0.0,
                     "dt": 1.0, "integrator": "ieuler", "thermostat": 0, "thermostat_temp": 1.0})
    ref = oracle.derivatives(prm, q.r[:n], q.v[:n], q.m[:n], np.zeros(n))["rho_lr"]
    assert np.linalg.norm(q.rho_lr[:n] - ref) / np.linalg.norm(ref) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("name,fn", [("ieuler", integrator.imp_euler), ("rk4", integrator.rk4),
                                     ("euler", integrator.euler)])
def test_integrator_functions_run_the_engine_step(name, fn):
    """integrator.<fn>(p.gather_state, p.derivatives, p.gather_derivatives,
    p.scatter_state, dt) followed by the box wrap gives the bits of update(dt)
    on a twin system set to that integrator (particles.py:485-488)."""
    g = load("lucy2d_400")
    twins = []
    for integ in ("ieuler", name):
        box = PeriodicBox(xmax=float(g["box"][0]), ymax=float(g["box"][1]), zmax=1)
        n = len(g["r0"])
        p = SmoothParticleSystem(n, d=2, maxn=n, hshort=float(g["h_short"]),
                                 hlong=float(g["h_long"]), simbox=box, integrator=integ,
                                 precision="fp64")
        p.r[:] = g["r0"]
        p.v[:] = g["v0"]
        p.m[:] = g["m"]
        p.u[:] = g["u0"]
        nl = VerletList(p, cutoff=float(g["cutoff"]), tolerance=0.0)
        p.nlists.append(nl)
        p.nl_default = nl
        p.forces.append(SpamComplete(p, nl, eta=0.0, zeta=0.0))
        twins.append(p)
    a, b = twins
    dt = float(g["dt"])
    for _ in range(3):
        fn(a.gather_state, a.derivatives, a.gather_derivatives, a.scatter_state, dt)
        a.box.apply(a)
        b.update(dt)
    assert a.integrator == "ieuler"          # the call leaves the system's own choice
    for k in ("r", "v", "u", "rho", "vdot", "udot"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    a.close()
    b.close()



@pytest.mark.gpu
@pytest.mark.parametrize("name,fn", [("ieuler", integrator.imp_euler), ("rk4", integrator.rk4),
                                     ("euler", integrator.euler)])
def test_generic_integrator_over_gpu_derivatives(name, fn):
    """The generic scheme (callables that are not one system's own bound
    methods, here wrappers of them) with the GPU evaluation as calc_derivs,
    followed by the box wrap, agrees with update(dt) of a twin system to the
    FP64 step tolerance over three steps."""
    g = load("lucy2d_400")
    twins = []
    for integ in ("ieuler", name):
        box = PeriodicBox(xmax=float(g["box"][0]), ymax=float(g["box"][1]), zmax=1)
        n = len(g["r0"])
        p = SmoothParticleSystem(n, d=2, maxn=n, hshort=float(g["h_short"]),
                                 hlong=float(g["h_long"]), simbox=box, integrator=integ,
                                 precision="fp64")
        p.r[:] = g["r0"]
        p.v[:] = g["v0"]
        p.m[:] = g["m"]
        p.u[:] = g["u0"]
        nl = VerletList(p, cutoff=float(g["cutoff"]), tolerance=0.0)
        p.nlists.append(nl)
        p.nl_default = nl
        p.forces.append(SpamComplete(p, nl, eta=0.0, zeta=0.0, cgrad=0.0))
        twins.append(p)
    a, b = twins
    dt = float(g["dt"])
    fns = (lambda: a.gather_state(), lambda: a.derivatives(), lambda: a.gather_derivatives(),
           lambda x: a.scatter_state(x))
    assert integrator._system(*fns) is None
    for _ in range(3):
        fn(*fns, dt)
        a.box.apply(a)
        b.update(dt)
    n = len(g["r0"])
    for x, y in ((a.r[:n], b.r[:n]), (a.v[:n], b.v[:n]), (a.u[:n], b.u[:n])):
        assert np.linalg.norm(x - y) / np.linalg.norm(y) < 1e-10
