"""Headless splash rendering against the reference's own
interpolate.splash_map_2d / splash_map_3d (golden images from
tests/golden/make_golden.py)."""
import numpy as np
import pytest

from tests.golden_cases import load, rel_l2

pytestmark = pytest.mark.gpu


def test_splash_map_2d_matches_reference():
    from pyticles_gb300 import interpolate
    g = load("splat")
    Z = interpolate.splash_map_2d(g["x"], g["y"], g["r"], g["m"], g["rho"], g["a"], g["h"],
                                  (0.0, 20.0, 0.0, 20.0), 5.0)
    assert Z.shape == g["Z2"].shape
    assert rel_l2(Z, g["Z2"]) < 1e-12


def test_splash_map_3d_matches_reference():
    from pyticles_gb300 import interpolate
    g = load("splat")
    Z = interpolate.splash_map_3d(g["x3"], g["y3"], 3.0, g["r3"], g["m3"], g["rho3"], g["rho3"],
                                  g["h3"], (0.0, 6.0, 0.0, 6.0), 1.5)
    assert rel_l2(Z, g["Z3"]) < 1e-12


def test_splash_map_device_buffers():
    import ctypes
    import torch
    from pyticles_gb300 import _abi
    g = load("splat")
    dev = "cuda:0"
    t = {k: torch.as_tensor(g[k], dtype=torch.float64, device=dev)
         for k in ("r", "m", "rho", "a", "h", "x", "y")}
    Z = torch.zeros((40, 40), dtype=torch.float64, device=dev)
    b = (ctypes.c_double * 4)(0.0, 20.0, 0.0, 20.0)
    torch.cuda.synchronize()
    st = _abi.lib().sph_splash_map(2, 400, t["r"].data_ptr(), 2, t["m"].data_ptr(),
                                   t["rho"].data_ptr(), t["a"].data_ptr(), t["h"].data_ptr(),
                                   40, 40, t["x"].data_ptr(), t["y"].data_ptr(), 0.0, b, 5.0,
                                   Z.data_ptr(), _abi.SPH_DEVICE, None)
    assert st == 0
    assert rel_l2(Z.cpu().numpy(), g["Z2"]) < 1e-12
