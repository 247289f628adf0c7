"""Binning on demand (tuning.rebin = 1): the cells of the last binning are
kept until a particle has used half of its cell slack -- the skin reuse of
VerletList.compress / ponder_rebuild (neighbour_list.py:191-234).  The pair
set stays exact at every evaluation, so trajectories track the FP64 oracle
as closely as binning every step does; only the summation order (rounding)
differs."""
import numpy as np
import pytest

from oracle import oracle
from pyticles_gb300 import Engine, build, workloads
from tests.golden_cases import rel_l2

pytestmark = pytest.mark.gpu

STEP_TOL = 1e-10


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


def hot_fluid(integ, side=24, temperature=4.0, dt=4e-3, seed=71):
    """A hot 2D fluid whose particles cross cell boundaries within a few
    steps (so bins are both reused and renewed)."""
    prm, r, v, m, T0 = workloads.lattice_system(side, 2, spacing=1.0, jitter=0.1,
                                                temperature=temperature, seed=seed,
                                                kernel="lucy", h_short=2.0, h_long=3.0,
                                                viscosity=True, dt=dt, integrator=integ)
    u = oracle.initial_energy(prm, r, v, m, T0)
    return prm, r, v, m, u


def run(prm, r, v, m, u, precision, steps, rebin, per_graph=1):
    with Engine(prm, precision, max_particles=len(r)) as e:
        s = e.add(prm, r, v, m, u)
        e.set_tuning(rebin=rebin, steps_per_graph=per_graph)
        e.advance(steps)
        e.sync()
        return e.get_state(s), e.rebin_count()


@pytest.mark.parametrize("integ", ["ieuler", "rk4"])
def test_rebin_on_demand_tracks_oracle(integ):
    prm, r, v, m, u = hot_fluid(integ)
    steps = 40
    (rg, vg, ug), bins = run(prm, r, v, m, u, "fp64", steps, rebin=1, per_graph=8)
    ro, vo, uo, _ = oracle.advance(prm, r, v, m, u, steps)
    errs = (rel_l2(rg, ro), rel_l2(vg, vo), rel_l2(ug, uo))
    print(integ, "bins", bins, "of", steps, errs)
    assert max(errs) < STEP_TOL
    assert 2 <= bins < steps          # reused, and renewed after drift


def test_rebin_on_demand_matches_every_step_binning():
    prm, r, v, m, u = hot_fluid("ieuler", side=32)
    (r1, v1, u1), b1 = run(prm, r, v, m, u, "mixed", 60, rebin=0, per_graph=10)
    (r2, v2, u2), b2 = run(prm, r, v, m, u, "mixed", 60, rebin=1, per_graph=10)
    assert b1 == 60 and b2 < 60
    assert rel_l2(r2, r1) < 1e-6 and rel_l2(v2, v1) < 1e-6 and rel_l2(u2, u1) < 1e-6


def test_rebin_steps_are_independent_of_call_boundaries():
    """The gate lives on the device: 30 steps in one call, in graphs of 5,
    and one by one give the same bits."""
    prm, r, v, m, u = hot_fluid("ieuler", side=20)
    out = []
    for chunks in ([30], [5] * 6, [1] * 30):
        with Engine(prm, "mixed", max_particles=len(r)) as e:
            s = e.add(prm, r, v, m, u)
            e.set_tuning(rebin=1, steps_per_graph=5)
            for c in chunks:
                e.advance(c)
            e.sync()
            out.append((e.get_state(s), e.rebin_count()))
    for (state, bins) in out[1:]:
        assert bins == out[0][1]
        for a, b in zip(state, out[0][0]):
            assert np.array_equal(a, b)


def test_euler_bins_every_step():
    prm, r, v, m, u = hot_fluid("euler", side=16)
    _, bins = run(prm, r, v, m, u, "mixed", 12, rebin=1)
    assert bins == 12


def test_state_upload_forces_a_binning():
    prm, r, v, m, u = hot_fluid("ieuler", side=16)
    with Engine(prm, "mixed", max_particles=len(r)) as e:
        s = e.add(prm, r, v, m, u)
        e.set_tuning(rebin=1)
        e.advance(3)
        e.sync()
        b0 = e.rebin_count()
        rr, vv, uu = e.get_state(s)
        e.set_state(s, rr[::-1].copy(), vv[::-1].copy(), m, uu[::-1].copy())
        e.advance(1)
        e.sync()
        assert e.rebin_count() == b0 + 1


def test_rebin_with_collisions_and_thermostat_tracks_oracle():
    """Binning on demand combined with hard collisions (extra collision and
    integrator passes) and the thermostat ramp, RK4."""
    from pyticles_gb300 import _abi
    prm, r, v, m, u = hot_fluid("rk4", side=20, temperature=2.0, dt=2e-3, seed=72)
    prm.collision = _abi.SPH_COLLIDE_EXCHANGE
    prm.collision_cutoff = 0.9
    prm.thermostat = 1
    prm.thermostat_temp = 2.0
    prm.thermostat_temp_end = 1.0
    prm.thermostat_ramp_steps = 20
    steps = 24
    (rg, vg, ug), bins = run(prm, r, v, m, u, "fp64", steps, rebin=1, per_graph=6)
    ro, vo, uo, _ = oracle.advance(prm, r, v, m, u, steps)
    errs = (rel_l2(rg, ro), rel_l2(vg, vo), rel_l2(ug, uo))
    print("bins", bins, errs)
    assert max(errs) < STEP_TOL
    assert bins < steps


def test_particle_system_run_with_rebin():
    """SmoothParticleSystem(rebin=True).run: the Python API path."""
    from pyticles_gb300 import PeriodicBox, SmoothParticleSystem, SpamComplete, VerletList
    prm, r, v, m, u = hot_fluid("ieuler", side=20)
    n = len(r)
    box = PeriodicBox(xmax=20.0, ymax=20.0, zmax=1)
    p = SmoothParticleSystem(n, d=2, maxn=n, hshort=2.0, hlong=3.0, simbox=box,
                             precision="fp64", rebin=True)
    p.r[:] = r
    p.v[:] = v
    p.m[:] = m
    p.u[:] = u
    nl = VerletList(p, cutoff=3.0, tolerance=0.0)
    p.nlists.append(nl)
    p.nl_default = nl
    p.forces.append(SpamComplete(p, nl, eta=prm.visc_alpha, zeta=prm.visc_beta))
    p.run(prm.dt, 30)
    assert p._engine.rebin_count() < 30
    ro, vo, uo, _ = oracle.advance(prm, r, v, m, u, 30)
    assert rel_l2(p.r[:n], ro) < STEP_TOL and rel_l2(p.v[:n], vo) < STEP_TOL
    p.close()
