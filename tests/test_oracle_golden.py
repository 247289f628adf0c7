"""Pins the FP64 oracle (oracle/sph_oracle.c) to golden vectors produced by
the reference's own Python (tests/golden/make_golden.py).  CPU only."""
import numpy as np
import pytest

from oracle import oracle
from tests.golden_cases import SYSTEMS, load, params_of, rel_l2, sort_pairs

# FP64 with different summation order: one evaluation agrees to 1e-12
# relative L2; a few integrator steps to 1e-10.  Squared distances: the
# reference squares with `dx**2`, which numpy evaluates through pow() and
# which on this platform is occasionally 1 ulp away from the correctly
# rounded dx*dx that the oracle and the kernels use; rsq is compared to
# 2 ulp while the pair SET must be identical.
EVAL_TOL = 1e-12


def assert_rsq_close(a, b):
    assert np.all(np.abs(a - b) <= 2 * np.spacing(np.abs(b)))
STEP_TOL = 1e-10


def test_kernel_table():
    """spkernel.lucy_kernel / gauss_kernel / debrun_kernel at 1, 2, 3 D."""
    tab = load("kernels")["table"]
    for kid, dim, r, h, w_ref, g_ref in tab:
        w, g = oracle.kernel(int(kid), int(dim), r, h)
        if int(kid) == 1:
            g_ref = -g_ref  # spkernel.py:51 gradient sign; Lucy's convention here
        assert w == pytest.approx(w_ref, rel=1e-13, abs=1e-300), (kid, dim, r, h)
        if r > 0:  # at r == 0 dwdx = g * 0 = 0 whatever g is
            assert g == pytest.approx(g_ref, rel=1e-12, abs=1e-14), (kid, dim, r, h)


def test_known_answers():
    """test/neighbour_list_test.py and test/kernel_test.py."""
    k = load("kat")
    assert float(k["brute_rij"]) == 1.0
    assert float(k["verlet_rij0"]) == 1.0
    assert not bool(k["rebuild_before"]) and bool(k["rebuild_after"])
    w, _ = oracle.kernel(2, 3, 0.0, 2.0)
    assert w == float(k["lucy_w0_h2_3d"]) == pytest.approx(105.0 / (128.0 * np.pi))
    prm = params_of({"dim": 3, "kernel": "lucy", "box": k["mirror_box"], "h_short": 1.0,
                     "h_long": 1.0, "cutoff": 10.0, "tolerance": 2.0, "dt": 1e-3,
                     "integrator": "ieuler", "thermostat": 0, "thermostat_temp": 1.0})
    iap, rsq = oracle.pairs(prm, k["positions"], brute=True)
    assert [tuple(x) for x in iap] == [(0, 1), (0, 2), (1, 2)]
    assert np.sqrt(rsq[0]) == 1.0


@pytest.mark.parametrize("case", ["exact_cut", "tol3d", "faces2d"])
def test_pair_edge_cases(case):
    """Bit-exact pair sets: distances exactly at the cutoff, faces and
    corners, positions outside the box, a quadrature skin."""
    g = load("pairs_edge")
    r = g[case + "_r"]
    prm = params_of({"dim": int(g[case + "_dim"]), "kernel": "lucy", "box": g[case + "_box"],
                     "h_short": 1.0, "h_long": 1.0, "cutoff": float(g[case + "_cutoff"]),
                     "tolerance": float(g[case + "_tol"]), "dt": 1e-3,
                     "integrator": "ieuler", "thermostat": 0, "thermostat_temp": 1.0})
    ref, idx = sort_pairs(g[case + "_iap"])
    ref_rsq = g[case + "_rsq"][idx]
    for brute in (True, False):
        iap, rsq = oracle.pairs(prm, r, brute=brute)
        assert np.array_equal(iap, ref)
        assert_rsq_close(rsq, ref_rsq)


@pytest.mark.parametrize("name", SYSTEMS)
def test_pair_set_matches_reference(name):
    g = load(name)
    prm = params_of(g)
    ref, idx = sort_pairs(g["iap"])
    iap, rsq = oracle.pairs(prm, g["r0"])
    assert np.array_equal(iap, ref)
    assert_rsq_close(rsq, g["rsq"][idx])


@pytest.mark.parametrize("name", SYSTEMS)
def test_evaluation_matches_reference(name):
    g = load(name)
    prm = params_of(g)
    d = oracle.derivatives(prm, g["r0"], g["v0"], g["m"], g["u0"])
    assert d["nip"] == len(g["iap"])
    for k in ("rho", "rho_lr", "t", "p", "pco", "vdot", "udot"):
        err = rel_l2(d[k], g["ev_" + k])
        assert err < EVAL_TOL, (k, err)


@pytest.mark.parametrize("name", SYSTEMS)
def test_steps_match_reference(name):
    g = load(name)
    prm = params_of(g)
    steps = int(g["steps"])
    r, v, u, props = oracle.advance(prm, g["r0"], g["v0"], g["m"], g["u0"], steps)
    assert rel_l2(r, g["r_final"]) < STEP_TOL
    assert rel_l2(v, g["v_final"]) < STEP_TOL
    assert rel_l2(u, g["u_final"]) < STEP_TOL
    for k in ("rho", "rho_lr", "t", "p", "pco", "vdot", "udot"):
        err = rel_l2(props[k], g["after_" + k])
        assert err < STEP_TOL, (k, err)


# Collisions: the reference squares with pow() (`dr[0]**2`), 1 ulp away from
# dr*dr for ~0.3% of inputs, and rij after a pushback is np.linalg.norm; both
# leave last-bit differences in chained updates.
COLLIDE_ULP = 8


def assert_ulp_close(a, b, ulp=COLLIDE_ULP):
    a, b = np.asarray(a), np.asarray(b)
    assert np.all(np.abs(a - b) <= ulp * np.spacing(np.maximum(np.abs(a), np.abs(b))))


@pytest.mark.parametrize("tag, mode", [("2d", 1), ("3d", 2)])
def test_collision_lists_match_reference(tag, mode):
    """CollisionForce (2D) and CollisionForce3d (pushback) Force.apply on a
    reference VerletList (forces.py:38-42, 87-243)."""
    g = load("collide_lists")
    r, v, drij, rij = oracle.collide_pairs(mode, g["r_" + tag], g["v_" + tag], g["m_" + tag],
                                           g["iap_" + tag], g["drij_" + tag],
                                           g["rij_" + tag], float(g["cutoff_" + tag]))
    c = float(g["cutoff_" + tag])
    assert np.count_nonzero(g["rij_" + tag] ** 2 <= c * c) > 100   # long chains of pairs
    assert_ulp_close(v, g["v_after_" + tag])
    assert_ulp_close(r, g["r_after_" + tag])
    assert_ulp_close(drij, g["drij_after_" + tag])
    assert_ulp_close(rij, g["rij_after_" + tag])


def test_collision_steps_match_reference():
    """SmoothParticleSystem.update with SpamForce + CohesiveSpamForce and a
    CollisionForce after them: the extra first evaluation's collisions and
    each stage's collided velocities (particles.py:459-494, integrator.py)."""
    from tests.golden_cases import collide_params
    g = load("collide2d_144")
    prm = collide_params(g)
    r, v, u = g["r0"], g["v0"], g["u0"]
    for k in range(1, int(g["steps"]) + 1):
        r, v, u, _ = oracle.advance(prm, r, v, g["m"], u, 1, step0=k - 1)
        assert rel_l2(r, g[f"r_step{k}"]) < 1e-15
        assert rel_l2(v, g[f"v_step{k}"]) < 1e-15
        assert rel_l2(u, g[f"u_step{k}"]) < 1e-15
    # the collisions matter: without them the velocities differ at O(1)
    _, v_free, _, _ = oracle.advance(collide_params(g, collision_cutoff=0.0), g["r0"], g["v0"],
                                     g["m"], g["u0"], int(g["steps"]))
    assert rel_l2(v_free, g["v_step3"]) > 0.1


def test_spam_properties_formulas_match_reference():
    """properties.spam_properties: the EOS steps applied to the reference's
    own densities reproduce its pressures, energies and temperatures bit for
    bit; the oracle's density matches the reference's."""
    from pyticles_gb300 import properties
    g = load("spam_props")
    rho = g["rho"]
    p, pco = properties.vdw(rho, np.full(len(rho), float(g["T0"])))
    assert np.array_equal(p, g["p"]) and np.array_equal(pco, g["pco"])
    u = properties.vdw_energy(rho, float(g["T0"]))
    assert np.array_equal(u, g["u"])
    assert np.array_equal(properties.vdw_temp(rho, u), g["t"])
    prm = params_of({"dim": 3, "kernel": "lucy", "box": g["box"], "h_short": float(g["h"]),
                     "h_long": float(g["hlr"]), "cutoff": float(g["cutoff"]), "tolerance": 0.0,
                     "dt": 1e-3, "integrator": "ieuler", "thermostat": 0,
                     "thermostat_temp": 1.0})
    d = oracle.derivatives(prm, g["r"], g["v"], g["m"], np.zeros(len(rho)))
    assert rel_l2(d["rho"], rho) < EVAL_TOL


def test_floors_fixture_is_what_the_oracle_computes():
    """tests/golden/floors.json (make_floors.py) holds the conditioning floors
    the mixed-precision parity bounds are built on; recomputing them from the
    oracle gives the committed numbers."""
    from tests.golden.make_floors import floors
    from tests.golden_cases import load_floors
    committed = load_floors()
    fresh = floors()
    assert sorted(committed) == sorted(fresh) == sorted(SYSTEMS)
    for name in SYSTEMS:
        for kind in ("position", "geometry"):
            for k, x in fresh[name][kind].items():
                assert committed[name][kind][k] == pytest.approx(x, rel=1e-9), (name, kind, k)


def test_geometry_floor_only_rounds_the_pair_geometry():
    """The FP32-geometry mode keeps the pair set and moves the evaluation by
    FP32-sized amounts, not more."""
    g = load("lucy2d_400")
    prm = params_of(g)
    a = oracle.derivatives(prm, g["r0"], g["v0"], g["m"], g["u0"])
    b = oracle.derivatives(prm, g["r0"], g["v0"], g["m"], g["u0"], geometry32=True)
    c = oracle.derivatives(prm, g["r0"], g["v0"], g["m"], g["u0"])
    assert a["nip"] == b["nip"] == len(g["iap"])
    assert 0 < rel_l2(b["rho"], a["rho"]) < 1e-7
    assert 0 < rel_l2(b["vdot"], a["vdot"]) < 1e-5
    for k in ("rho", "vdot", "udot"):       # the mode is off again afterwards
        assert np.array_equal(a[k], c[k])


def test_oracle_follows_the_reference_for_100_steps():
    """The plain small configuration at its own length: 100 improved-Euler
    steps of the 32 x 32 fluid (SmoothParticleSystem.update, particles.py:
    459-494), compared every 20 steps and in the properties after the last."""
    g = load("traj2d_1024")
    prm = params_of(g)
    r, v, u = g["r0"], g["v0"], g["u0"]
    done = 0
    for k, mark in enumerate(g["marks"]):
        r, v, u, props = oracle.advance(prm, r, v, g["m"], u, int(mark) - done, step0=done)
        done = int(mark)
        for got, key in ((r, "r_marks"), (v, "v_marks"), (u, "u_marks")):
            assert rel_l2(got, g[key][k]) < STEP_TOL, (mark, key)
    assert done == int(g["steps"]) == 100
    for key in ("rho", "rho_lr", "t", "p", "pco", "vdot", "udot"):
        assert rel_l2(props[key], g["after_" + key]) < STEP_TOL, key
