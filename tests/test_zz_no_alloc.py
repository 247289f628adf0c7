"""The allocation-free entry point sph_derivatives_noalloc, called through
the C ABI with caller-owned device buffers, against the engine's own
evaluation (sph_sim_derivatives) on the same inputs, twice in a row (the
second call runs on the scratch the first one left behind).

It serves callers that cannot let a library allocate device memory (a host
framework that owns the device's memory pool, a loop that may not block in
the allocator); it must give the engine's results.  This file is collected
last on purpose: a failure here leaves every other test already run.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle
from pyticles_gb300 import Engine, build, workloads
from pyticles_gb300._abi import (NOALLOC_MAX_PARTICLES, SPH_ECAPACITY, SPH_EINVAL, SPH_FP64,
                                 SPH_MIXED, lib, make_params)

pytestmark = pytest.mark.gpu

TOL = 1e-12  # the FP64 evaluation tolerance of the parity tests
KEYS = ("rho", "rho_lr", "t", "p", "pco", "vdot", "udot", "jq")


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


def noalloc(prm, precision, r, v, m, u):
    import torch
    dev = torch.device("cuda:0")
    n, d = r.shape
    t_in = [torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device=dev)
            for a in (r, v, m, u)]
    out = {k: torch.zeros(n, dtype=torch.float64, device=dev)
           for k in ("rho", "rho_lr", "t", "p", "pco", "udot")}
    out["vdot"] = torch.zeros((n, d), dtype=torch.float64, device=dev)
    out["jq"] = torch.zeros((n, d), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    prec = SPH_MIXED if precision == "mixed" else SPH_FP64
    st = lib().sph_derivatives_noalloc(
        ctypes.byref(prm), prec, n, *[x.data_ptr() for x in t_in],
        *[out[k].data_ptr() for k in ("rho", "rho_lr", "t", "p", "pco", "vdot", "udot", "jq")],
        ctypes.c_void_p(stream))
    assert st == 0, st
    return {k: val.cpu().numpy() for k, val in out.items()}


def cases():
    p2, r2, v2, m2, T2 = workloads.config_2d(32, 1000, viscosity=True)
    p3, r3, v3, m3, T3 = workloads.config_3d(12, 3000)
    return {"visc2d_1024": (p2, r2, v2, m2, T2), "cubic3d_heat_1728": (p3, r3, v3, m3, T3)}


def rel(a, b):
    den = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (den if den > 0 else 1.0)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("case", ["visc2d_1024", "cubic3d_heat_1728"])
def test_noalloc_matches_engine_twice(case, precision):
    prm, r, v, m, T0 = cases()[case]
    u = oracle.initial_energy(prm, r, v, m, T0)
    u = u + 0.1 * T0 * np.sin(2 * np.pi * r[:, 0] / prm.box[0])
    with Engine(prm, precision, max_particles=len(r)) as e:
        s = e.add(prm, r, v, m, u)
        ref = e.derivatives(s)
        e.sync()
    for _ in range(2):
        out = noalloc(prm, precision, r, v, m, u)
        for k in KEYS:
            assert rel(out[k], ref[k]) <= TOL, (k, rel(out[k], ref[k]))


def test_noalloc_coarser_cells_in_a_sparse_box():
    """A sparse 2D box that needs more cells than the scratch holds at half
    the cutoff: the call falls back to coarser cells (up to four times the
    cutoff) and still gives the oracle's FP64 evaluation; a box too large
    even for those is refused with SPH_ECAPACITY, twice in a row."""
    rng = np.random.default_rng(7)
    n = 3000
    prm = make_params(dim=2, box=(400.0, 400.0), kernel="lucy", h_short=1.5, h_long=2.0,
                      cutoff=2.0, viscosity=True)
    r = rng.uniform(0.0, 400.0, size=(n, 2))
    # clumps, so that pairs exist at this density
    r[: n // 2] = (r[: n // 2] % 40.0) + 100.0
    v = rng.normal(0.0, 0.5, size=(n, 2))
    m = np.full(n, 0.3)      # keeps every density well below the pole b rho = 1
    u = np.full(n, 0.4)
    ref = oracle.derivatives(prm, r, v, m, u)
    assert ref["nip"] > 1000
    for _ in range(2):
        out = noalloc(prm, "fp64", r, v, m, u)
        for k in KEYS:
            assert rel(out[k], ref[k]) <= TOL, (k, rel(out[k], ref[k]))
    big = make_params(dim=2, box=(5000.0, 5000.0), kernel="lucy", h_short=1.5, h_long=2.0,
                      cutoff=2.0)
    rb = rng.uniform(0.0, 5000.0, size=(200, 2))
    import torch
    bufs = [torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda:0")
            for a in (rb, np.zeros((200, 2)), np.ones(200), np.zeros(200))]
    outb = torch.zeros(200, dtype=torch.float64, device="cuda:0")
    for _ in range(2):
        st = lib().sph_derivatives_noalloc(ctypes.byref(big), SPH_FP64, 200,
                                           *[b.data_ptr() for b in bufs], outb.data_ptr(),
                                           *([None] * 7), None)
        assert st == SPH_ECAPACITY


def test_noalloc_rejects_sizes_beyond_its_limit():
    n = NOALLOC_MAX_PARTICLES + 1
    prm = make_params(dim=2, box=(400.0, 400.0))
    r = np.random.default_rng(0).uniform(0, 400, size=(n, 2))
    import torch
    buf = torch.zeros(n * 2, dtype=torch.float64, device="cuda:0")
    st = lib().sph_derivatives_noalloc(ctypes.byref(prm), SPH_MIXED, n, buf.data_ptr(),
                                       buf.data_ptr(), buf.data_ptr(), buf.data_ptr(),
                                       *([None] * 8), None)
    assert st == SPH_EINVAL
    del r
