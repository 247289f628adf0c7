"""The smoothing kernels of the pair passes through sph_kernel_eval and the
spkernel mirror, against the reference's kernel table (spkernel.py:39-153,
tests/golden/kernels.npz), its known answer (test/kernel_test.py:12: Lucy
W(0, h = 2) = 105 / (128 pi) in 3D) and, for the M4 cubic spline that the
reference lacks, the oracle."""

import numpy as np
import pytest

from oracle import oracle
from pyticles_gb300 import _abi, spkernel
from tests.golden_cases import load

# FP64: the device evaluates the reference's formulas in another order (q
# from a hi/lo reciprocal of h instead of r / h), relative to each value and
# to the kernel's scale: near the support's edge (1 - q)^3 turns one ulp of q
# into 1e-13 relative (the table holds q = 0.999)
W_TOL64, G_TOL64 = 1e-13, 1e-12
# mixed: FP32 arithmetic on FP32-rounded r, relative to the kernel's scale
# (W(0) for W, the largest |g| of the table's radii for g)
TOL32 = 4e-6


def _eval(kid, dim, h, r, precision=_abi.SPH_FP64, n=None, mem=_abi.SPH_HOST):
    r = np.ascontiguousarray(r, dtype=np.float64)
    w, g = np.zeros_like(r), np.zeros_like(r)
    st = _abi.lib().sph_kernel_eval(kid, dim, h, precision, r.size if n is None else n,
                                    r.ctypes.data, w.ctypes.data, g.ctypes.data, mem, None)
    return st, w, g


def _table():
    """Rows (kid, dim, h, r, W, g) at 2 and 3 D, g = (dW/dr)/r in Lucy's sign."""
    rows = []
    for kid, dim, r, h, w_ref, g_ref in load("kernels")["table"]:
        if int(dim) in (2, 3):
            rows.append((int(kid), int(dim), float(h), float(r), float(w_ref),
                         -float(g_ref) if int(kid) == 1 else float(g_ref)))
    return rows


# ---- host checks (CPU): arguments are refused before any device work ----

@pytest.mark.parametrize("args", [
    dict(kid=0), dict(kid=5), dict(dim=1), dict(dim=4), dict(h=0.0), dict(h=-1.0),
    dict(h=float("inf")), dict(h=float("nan")), dict(precision=2), dict(n=-1), dict(mem=7)])
def test_kernel_eval_refuses_bad_arguments(args):
    a = dict(kid=2, dim=3, h=1.0, precision=_abi.SPH_FP64, n=None, mem=_abi.SPH_HOST)
    a.update(args)
    st, _, _ = _eval(a["kid"], a["dim"], a["h"], np.zeros(4), a["precision"], a["n"], a["mem"])
    assert st == _abi.SPH_EINVAL


def test_kernel_eval_of_nothing_is_ok():
    st = _abi.lib().sph_kernel_eval(2, 3, 1.0, _abi.SPH_FP64, 0, None, None, None,
                                    _abi.SPH_HOST, None)
    assert st == _abi.SPH_OK


def test_spkernel_refuses_one_dimension():
    with pytest.raises(NotImplementedError):
        spkernel.lucy_kernel(0.5, [0.5], 1.0)


# ---- device evaluation (GPU) ----

@pytest.mark.gpu
def test_known_answer_lucy_3d():
    """test/kernel_test.py:12: W(0, h = 2) = 105 / (128 pi), in both precisions."""
    for prec in (_abi.SPH_FP64, _abi.SPH_MIXED):
        st, w, _ = _eval(2, 3, 2.0, np.zeros(1), prec)
        assert st == _abi.SPH_OK
        assert w[0] == float(load("kat")["lucy_w0_h2_3d"]) == pytest.approx(105 / (128 * np.pi))


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_kernel_table(precision):
    """Gaussian, Lucy and Debrun at 2 and 3 D against the reference's values."""
    rows = _table()
    groups = {}
    for row in rows:
        groups.setdefault(row[:3], []).append(row)
    for (kid, dim, h), rs in groups.items():
        r = np.array([x[3] for x in rs])
        w_ref = np.array([x[4] for x in rs])
        g_ref = np.array([x[5] for x in rs])
        prec = _abi.SPH_MIXED if precision == "mixed" else _abi.SPH_FP64
        st, w, g = _eval(kid, dim, h, r, prec)
        assert st == _abi.SPH_OK
        live = r > 0          # at r = 0 dwdx = g * 0 whatever g is
        w0 = oracle.kernel(kid, dim, 0.0, h)[0]
        gs = np.max(np.abs(g_ref[live]))
        if precision == "fp64":
            assert np.allclose(w, w_ref, rtol=W_TOL64, atol=W_TOL64 * w0), (kid, dim, h)
            assert np.allclose(g[live], g_ref[live], rtol=G_TOL64, atol=G_TOL64 * gs), \
                (kid, dim, h)
        else:
            assert np.all(np.abs(w - w_ref) <= TOL32 * w0), (kid, dim, h)
            assert np.all(np.abs(g[live] - g_ref[live]) <= TOL32 * gs), (kid, dim, h)


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [2, 3])
def test_cubic_spline_against_the_oracle(dim):
    rng = np.random.Generator(np.random.PCG64(7100 + dim))
    h = 1.3
    r = np.concatenate([[0.0, h, 2 * h, 2.5 * h], rng.uniform(0.0, 2.2 * h, 200)])
    st, w, g = _eval(4, dim, h, r)
    assert st == _abi.SPH_OK
    ref = np.array([oracle.kernel(4, dim, x, h) for x in r])
    assert np.allclose(w, ref[:, 0], rtol=W_TOL64, atol=W_TOL64 * ref[0, 0])
    live = r > 0
    gs = np.max(np.abs(ref[live, 1]))
    assert np.allclose(g[live], ref[live, 1], rtol=G_TOL64, atol=G_TOL64 * gs)


@pytest.mark.gpu
def test_spkernel_mirror_conventions():
    """Return conventions of spkernel.py: one pair gives (float W, dwdx of
    dx's length); 0 gradient at r = 0; the Gaussian's +2 W dx / h^2
    (spkernel.py:51); lucy_w / lucy_w3d; arrays of pairs at once."""
    h = 2.0
    dx = np.array([0.3, -0.4, 1.2])
    r = float(np.linalg.norm(dx))
    w, dwdx = spkernel.lucy_kernel(r, dx, h)
    wk, gk = oracle.kernel(2, 3, r, h)
    assert isinstance(w, float) and dwdx.shape == (3,)
    assert w == pytest.approx(wk, rel=1e-13) and np.allclose(dwdx, gk * dx, rtol=1e-12)
    w0, d0 = spkernel.lucy_kernel(0.0, np.zeros(2), h)
    assert w0 == pytest.approx(5 / (np.pi * h * h), rel=1e-14) and not d0.any()
    wg, dg = spkernel.gauss_kernel(r, dx, h)
    assert np.allclose(dg, 2.0 * wg * dx / (h * h), rtol=1e-12)
    assert spkernel.kernel(r, dx, h, "debrun")[0] == pytest.approx(oracle.kernel(3, 3, r, h)[0],
                                                                    rel=1e-13)
    assert spkernel.lucy_w(0.5, h) == pytest.approx(oracle.kernel(2, 2, 0.5, h)[0], rel=1e-13)
    w3 = spkernel.lucy_w3d(0.5, h)
    assert w3.shape == (1,) and w3[0] == pytest.approx(oracle.kernel(2, 3, 0.5, h)[0], rel=1e-13)
    rs = np.array([0.1, 0.9, 1.7, 2.5])
    dxs = np.stack([rs, np.zeros(4)], axis=1)
    ws, ds = spkernel.lucy_kernel(rs, dxs, h, precision="mixed")
    assert ws.shape == (4,) and ds.shape == (4, 2) and ws[-1] == 0.0 and not ds[-1].any()
    ref = np.array([oracle.kernel(2, 2, x, h)[0] for x in rs])
    assert np.all(np.abs(ws - ref) <= TOL32 * ref[0])
