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
