"""Hard collisions (forces.py:87-243, 454-474) on the GPU.

* sph_collide_pairs -- Force.apply over a reference pair list -- equals the
  oracle's sequential loop bit for bit (same FP64 operations in the same
  per-particle order; the dependency levels only reorder independent
  pairs) and the reference's own output to a few ulp (it squares with pow).
* The engine step with a CollisionForce after the SPH forces reproduces the
  reference's SmoothParticleSystem.update (golden collide2d_144) and the
  oracle; batched simulations with collisions equal the same simulations
  run alone.
CPU-only tests at the end cover the Python wiring.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle
from pyticles_gb300 import (CohesiveSpamForce, CollisionForce, CollisionForce3d, Engine,
                            FortranCollisionForce, PeriodicBox, SmoothParticleSystem,
                            SpamForce, VerletList, _abi, build, workloads)
from tests.golden_cases import collide_params, load, rel_l2

STEP_TOL = 1e-10
MIXED_TOL = 1e-6


@pytest.fixture(scope="module")
def built():
    build.build()


def collide_host(tag, mode, g, iap=None):
    r, v = g["r_" + tag].copy(), g["v_" + tag].copy()
    m = g["m_" + tag].copy()
    iap = np.ascontiguousarray(g["iap_" + tag] if iap is None else iap, dtype=np.int64)
    drij, rij = g["drij_" + tag].copy(), g["rij_" + tag].copy()
    n, d = v.shape
    st = _abi.lib().sph_collide_pairs(d, mode, n, r.ctypes.data, v.ctypes.data, m.ctypes.data,
                                      len(iap), iap.ctypes.data, drij.ctypes.data,
                                      rij.ctypes.data, float(g["cutoff_" + tag]), _abi.SPH_HOST,
                                      None)
    return st, r, v, drij, rij


@pytest.mark.gpu
@pytest.mark.parametrize("tag, mode", [("2d", 1), ("3d", 2), ("3d", 1)])
def test_collide_pairs_equals_sequential_oracle(built, tag, mode):
    g = load("collide_lists")
    st, r, v, drij, rij = collide_host(tag, mode, g)
    assert st == 0
    ro, vo, drijo, rijo = oracle.collide_pairs(mode, g["r_" + tag], g["v_" + tag],
                                               g["m_" + tag], g["iap_" + tag],
                                               g["drij_" + tag], g["rij_" + tag],
                                               float(g["cutoff_" + tag]))
    assert np.array_equal(v, vo)
    assert np.array_equal(r, ro)
    assert np.array_equal(drij, drijo)
    assert np.array_equal(rij, rijo)
    if mode == 2:
        assert np.abs(r - g["r_" + tag]).max() > 0.01          # pushback happened
        np.testing.assert_allclose(v, g["v_after_" + tag], rtol=0, atol=1e-13)


@pytest.mark.gpu
def test_collide_pairs_device_memory(built):
    import torch
    g = load("collide_lists")
    tag = "2d"
    dev = torch.device("cuda:0")
    t = {k: torch.tensor(g[k + "_" + tag], device=dev)
         for k in ("r", "v", "m", "iap", "drij", "rij")}
    n, d = t["v"].shape
    st = _abi.lib().sph_collide_pairs(d, 1, n, t["r"].data_ptr(), t["v"].data_ptr(),
                                      t["m"].data_ptr(), t["iap"].shape[0],
                                      t["iap"].data_ptr(), t["drij"].data_ptr(),
                                      t["rij"].data_ptr(), float(g["cutoff_" + tag]),
                                      _abi.SPH_DEVICE, None)
    assert st == 0
    _, vo, _, _ = oracle.collide_pairs(1, g["r_2d"], g["v_2d"], g["m_2d"], g["iap_2d"],
                                       g["drij_2d"], g["rij_2d"], float(g["cutoff_2d"]))
    assert np.array_equal(t["v"].cpu().numpy(), vo)


@pytest.mark.gpu
def test_collide_pairs_rejects_bad_indices(built):
    g = load("collide_lists")
    iap = g["iap_2d"].copy()
    iap[3, 1] = len(g["v_2d"])            # out of range
    st, _, v, _, _ = collide_host("2d", 1, g, iap=iap)
    assert st == _abi.SPH_EINVAL
    assert np.array_equal(v, g["v_2d"])   # nothing applied


def run_engine(prm, g, precision, steps):
    with Engine(prm, precision, max_particles=len(g["r0"])) as e:
        s = e.add(prm, g["r0"], g["v0"], g["m"], g["u0"])
        out = []
        for _ in range(steps):
            e.advance(1)
            e.sync()
            out.append(e.get_state(s))
        return out


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_engine_collision_steps_match_reference(built, precision):
    g = load("collide2d_144")
    prm = collide_params(g)
    states = run_engine(prm, g, precision, int(g["steps"]))
    tol = STEP_TOL if precision == "fp64" else MIXED_TOL
    for k, (r, v, u) in enumerate(states, start=1):
        errs = (rel_l2(r, g[f"r_step{k}"]), rel_l2(v, g[f"v_step{k}"]),
                rel_l2(u, g[f"u_step{k}"]))
        print(precision, k, errs)
        assert max(errs) < tol, (k, errs)


@pytest.mark.gpu
@pytest.mark.parametrize("integ", ["euler", "ieuler", "rk4"])
def test_engine_collisions_3d_match_oracle(built, integ):
    """3D fluid with viscosity and heat flux, FortranCollisionForce's
    exchange after every evaluation, each integrator."""
    prm, r, v, m, T0 = workloads.lattice_system(6, 3, spacing=1.0, jitter=0.12,
                                                temperature=0.8, seed=31, kernel="lucy",
                                                h_short=1.3, h_long=1.9, viscosity=True,
                                                heat_flux=True, dt=2e-3, integrator=integ)
    prm.collision = _abi.SPH_COLLIDE_EXCHANGE
    prm.collision_cutoff = 0.9
    u = oracle.initial_energy(prm, r, v, m, T0)
    ro, vo, uo, _ = oracle.advance(prm, r, v, m, u, 4)
    with Engine(prm, "fp64", max_particles=len(r)) as e:
        s = e.add(prm, r, v, m, u)
        e.advance(4)
        e.sync()
        rg, vg, ug = e.get_state(s)
    assert rel_l2(rg, ro) < STEP_TOL and rel_l2(vg, vo) < STEP_TOL and rel_l2(ug, uo) < STEP_TOL
    free = oracle.advance(collide_params_off(prm), r, v, m, u, 4)[1]
    assert rel_l2(free, vo) > 1e-3       # collisions happened


def collide_params_off(prm):
    p = _abi.params_from_dict(_abi.params_dict(prm))
    p.collision = 0
    p.collision_cutoff = 0.0
    return p


@pytest.mark.gpu
def test_collision_batched_equals_alone(built):
    g = load("collide2d_144")
    sims = []
    for k, coll in enumerate((0.95, 0.9, 0.8)):
        prm, r, v, m, T0 = workloads.lattice_system(12 + k, 2, spacing=1.0, jitter=0.1,
                                                    temperature=0.6, seed=60 + k,
                                                    kernel="lucy", h_short=2.0, h_long=3.0,
                                                    dt=1e-3)
        prm.collision = _abi.SPH_COLLIDE_EXCHANGE
        prm.collision_cutoff = coll
        u = oracle.initial_energy(prm, r, v, m, T0)
        sims.append((prm, r, v, m, u))
    alone = []
    for prm, r, v, m, u in sims:
        with Engine(prm, "mixed", max_particles=len(r)) as e:
            s = e.add(prm, r, v, m, u)
            e.advance(5)
            e.sync()
            alone.append(e.get_state(s))
    with Engine(sims[0][0], "mixed", max_particles=sum(len(x[1]) for x in sims),
                max_sims=4) as e:
        ids = [e.add(*x) for x in sims]
        e.advance(5)
        e.sync()
        for sid, ref in zip(ids, alone):
            for a, b in zip(e.get_state(sid), ref):
                assert np.array_equal(a, b)
    assert g is not None


def api_system(g, coll_force):
    n = len(g["r0"])
    L = [float(x) for x in g["box"][:2]]
    box = PeriodicBox(xmax=L[0], ymax=L[1], zmax=1)
    p = SmoothParticleSystem(n, d=2, maxn=n, hshort=float(g["h_short"]),
                             hlong=float(g["h_long"]), simbox=box)
    p.r[:, :] = g["r0"]
    p.v[:, :] = g["v0"]
    p.m[:] = g["m"]
    p.u[:] = g["u0"]
    nl = VerletList(p, cutoff=float(g["cutoff"]), tolerance=0.0)
    p.nlists.append(nl)
    p.nl_default = nl
    p.forces.append(SpamForce(p, nl))
    p.forces.append(CohesiveSpamForce(p, nl))
    if coll_force is not None:
        p.forces.append(coll_force(p, nl, cutoff=float(g["collision_cutoff"])))
    return p


@pytest.mark.gpu
@pytest.mark.parametrize("force", [CollisionForce, FortranCollisionForce])
def test_api_update_with_collision_force(built, force):
    g = load("collide2d_144")
    p = api_system(g, force)
    n = p.n
    for k in range(1, int(g["steps"]) + 1):
        p.update(float(g["dt"]))
        assert rel_l2(p.r[:n], g[f"r_step{k}"]) < STEP_TOL
        assert rel_l2(p.v[:n], g[f"v_step{k}"]) < STEP_TOL
    p.close()


# ---- CPU: wiring ----

def test_engine_params_take_the_collision_force():
    g = load("collide2d_144")
    p = api_system(g, CollisionForce)
    prm = p.engine_params(1e-3)
    assert prm.collision == _abi.SPH_COLLIDE_EXCHANGE
    assert prm.collision_cutoff == float(g["collision_cutoff"])
    q = api_system(g, None)
    assert q.engine_params(1e-3).collision == 0


def test_pushback_and_misordered_collisions_are_refused_in_the_step():
    g = load("collide2d_144")
    p = api_system(g, CollisionForce3d)
    with pytest.raises(NotImplementedError):
        p.engine_params(1e-3)
    q = api_system(g, None)
    q.forces.insert(0, CollisionForce(q, q.nl_default, cutoff=0.9))
    with pytest.raises(NotImplementedError):
        q.engine_params(1e-3)


def test_collision_params_survive_the_dict_roundtrip():
    prm = _abi.make_params(collision_cutoff=0.5)
    back = _abi.params_from_dict(_abi.params_dict(prm))
    assert back.collision == 1 and back.collision_cutoff == 0.5
    assert ctypes.sizeof(back) == ctypes.sizeof(_abi.SphParams)


@pytest.mark.gpu
def test_collision_capacity_overflow_is_reported(built):
    """More colliding pairs than particles in one evaluation: the engine
    reports SPH_ECAPACITY and applies none of them."""
    prm, r, v, m, T0 = workloads.lattice_system(12, 2, spacing=1.0, jitter=0.1,
                                                temperature=0.6, seed=81, kernel="lucy",
                                                h_short=2.0, h_long=3.0, dt=1e-3)
    prm.collision = _abi.SPH_COLLIDE_EXCHANGE
    prm.collision_cutoff = 2.9       # ~25 partners per particle
    u = oracle.initial_energy(prm, r, v, m, T0)
    with Engine(prm, "mixed", max_particles=len(r)) as e:
        s = e.add(prm, r, v, m, u)
        e.advance(1)
        with pytest.raises(_abi.SphError) as ei:
            e.sync()
        assert ei.value.status == _abi.SPH_ECAPACITY
        assert e.status(s) == _abi.SPH_ECAPACITY


def test_collision_over_sorted_list_is_refused_in_the_step():
    from pyticles_gb300 import SortedVerletList
    g = load("collide2d_144")
    p = api_system(g, None)
    snl = SortedVerletList(p, cutoff=float(g["cutoff"]), tolerance=0.0)
    p.forces.append(CollisionForce(p, snl, cutoff=0.9))
    with pytest.raises(NotImplementedError):
        p.engine_params(1e-3)
