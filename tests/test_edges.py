"""Edge cases through the C ABI: tiny and isolated systems, empty engines,
single-cell boxes, capacity limits and argument errors (the reference's
own tests use 2- and 3-particle systems, test/neighbour_list_test.py and
test/force_test.py)."""
import numpy as np
import pytest

from oracle import oracle
from pyticles_gb300 import Engine, SphError, _abi, build, make_params
from tests.golden_cases import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


def small(dim, n, L, seed, **kw):
    rng = np.random.Generator(np.random.PCG64(seed))
    r = rng.uniform(0.0, L, size=(n, dim))
    v = rng.normal(0.0, 0.5, size=(n, dim))
    m = np.ones(n)
    prm = make_params(dim=dim, box=[L] * dim, h_short=1.0, h_long=2.0, viscosity=True, **kw)
    u = oracle.initial_energy(prm, r, v, m, 0.6)
    return prm, r, v, m, u


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("dim, n", [(2, 1), (2, 2), (3, 1), (3, 3)])
def test_tiny_systems_match_oracle(dim, n, precision):
    """One to three particles: self terms only, or a single pair."""
    prm, r, v, m, u = small(dim, n, 3.0, 10 + n)
    r[:] = np.linspace(0.5, 1.5, n)[:, None] * np.ones(dim)
    u = oracle.initial_energy(prm, r, v, m, 0.6)
    ref = oracle.derivatives(prm, r, v, m, u)
    ro, vo, uo, _ = oracle.advance(prm, r, v, m, u, 3)
    with Engine(prm, precision, max_particles=n) as e:
        s = e.add(prm, r, v, m, u)
        d = e.derivatives(s)
        e.advance(3)
        e.sync()
        rg, vg, ug = e.get_state(s)
        assert e.pair_count(s) == ref["nip"]
    tol = 1e-12 if precision == "fp64" else 1e-6
    assert rel_l2(d["rho"], ref["rho"]) < tol
    assert np.allclose(d["vdot"], ref["vdot"], rtol=tol * 10, atol=1e-12)
    assert rel_l2(rg, ro) < max(tol, 1e-10) and rel_l2(ug, uo) < max(tol, 1e-10)


def test_isolated_particles_have_no_pairs():
    """Particles further apart than the cutoff: no pairs, only self density."""
    prm = make_params(dim=2, box=[40.0, 40.0], h_short=1.0, h_long=2.0)
    r = np.array([[5.0, 5.0], [15.0, 5.0], [5.0, 15.0], [25.0, 25.0]])
    v, m = np.zeros((4, 2)), np.ones(4)
    u = np.full(4, 0.5)
    with Engine(prm, "mixed", max_particles=4) as e:
        s = e.add(prm, r, v, m, u)
        d = e.derivatives(s)
        e.sync()
        assert e.pair_count(s) == 0
        assert e.pairs(s)["iap"].shape == (0, 2)
        assert np.all(d["vdot"] == 0) and np.all(d["udot"] == 0)
        assert np.allclose(d["rho"], d["rho"][0])


@pytest.mark.parametrize("dim", [2, 3])
def test_single_cell_box_uses_minimum_image(dim):
    """A box smaller than three cells per axis collapses to one cell per axis;
    the pair pass then applies the minimum image itself."""
    prm, r, v, m, u = small(dim, 40 if dim == 2 else 60, 4.0, 33)
    ref = oracle.derivatives(prm, r, v, m, u)
    with Engine(prm, "fp64", max_particles=len(r)) as e:
        s = e.add(prm, r, v, m, u)
        d = e.derivatives(s)
        e.sync()
        assert e.pair_count(s) == ref["nip"]
    for k in ("rho", "vdot", "udot"):
        assert rel_l2(d[k], ref[k]) < 1e-12


def test_empty_engine_and_removed_simulations():
    prm, r, v, m, u = small(2, 64, 8.0, 5)
    with Engine(prm, "mixed", max_particles=64, max_sims=2) as e:
        e.advance(5)                    # nothing to do
        e.sync()
        s = e.add(prm, r, v, m, u)
        e.advance(2)
        e.remove(s)
        e.advance(3)                    # empty again
        e.sync()
        out = np.empty((64, 2))
        st = _abi.lib().sph_sim_get_state(e._h, s, out.ctypes.data, None, None, _abi.SPH_HOST)
        assert st == _abi.SPH_ENOTFOUND


def test_argument_errors_are_reported():
    prm, r, v, m, u = small(2, 16, 8.0, 6)
    with Engine(prm, "mixed", max_particles=16, max_sims=1) as e:
        with pytest.raises(SphError) as ei:
            e.add(prm, r[:0], v[:0], m[:0], u[:0])          # empty simulation
        assert ei.value.status == _abi.SPH_EINVAL
        bad = make_params(dim=2, box=[8.0, 8.0], h_short=1.0, h_long=2.0, kernel="cubic")
        with pytest.raises(SphError) as ei:
            e.add(bad, r, v, m, u)                          # other kernel than the group
        assert ei.value.status == _abi.SPH_EINVAL
        s = e.add(prm, r, v, m, u)
        with pytest.raises(SphError) as ei:
            e.add(prm, r, v, m, u)                          # no simulation slot left
        assert ei.value.status == _abi.SPH_ECAPACITY
        # output pointers that are NULL are refused, not written through
        lib, h = _abi.lib(), e._h
        assert lib.sph_sim_count(h, s, None) == _abi.SPH_EINVAL
        assert lib.sph_sim_pair_count(h, s, None) == _abi.SPH_EINVAL
        assert lib.sph_sim_diagnostics(h, s, None) == _abi.SPH_EINVAL
        # a partial state update is refused before anything is written
        before = e.get_state(s)
        r2 = np.ascontiguousarray(r + 0.5)
        assert lib.sph_sim_set_state(h, s, r2.ctypes.data, None, None, None,
                                     _abi.SPH_HOST) == _abi.SPH_EINVAL
        for a, b in zip(e.get_state(s), before):
            assert np.array_equal(a, b)


@pytest.mark.parametrize("dim", [2, 3])
def test_sparse_system_in_a_huge_box(dim):
    """A few hundred particles in a box millions of cutoffs wide: the cell
    table is coarsened to a multiple of the particle count and the pair set
    and forces stay exact."""
    L = 2.0e5 if dim == 2 else 4.0e3
    rng = np.random.Generator(np.random.PCG64(90 + dim))
    n = 300
    centres = rng.uniform(0.0, L, size=(30, dim))
    r = (centres[:, None, :] + rng.uniform(-1.5, 1.5, size=(30, 10, dim))).reshape(n, dim) % L
    v = rng.normal(0.0, 0.5, size=(n, dim))
    m = np.ones(n)
    prm = make_params(dim=dim, box=[L] * dim, h_short=1.0, h_long=2.0, viscosity=True)
    u = oracle.initial_energy(prm, r, v, m, 0.6)
    ref = oracle.derivatives(prm, r, v, m, u)
    with Engine(prm, "fp64", max_particles=n) as e:
        s = e.add(prm, r, v, m, u)
        d = e.derivatives(s)
        e.sync()
        assert e.pair_count(s) == ref["nip"] > 0
    for k in ("rho", "vdot", "udot"):
        assert rel_l2(d[k], ref[k]) < 1e-12
