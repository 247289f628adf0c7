"""Headless SPH splash rendering, mirroring pyticles' interpolate.py.

splash_map_2d / splash_map_3d keep the reference signatures
(interpolate.py:39-149) and return the pixel grid Z[nx, ny] computed on the
GPU by libsph's sph_splash_map (a device buffer in place of the GL blit of
SmoothParticleView.render_density, pview.py:483-519).
"""
import ctypes

import numpy as np

from . import _abi


def _splash(mode, x, y, z, r, m, rho, a, h, bounds, cutoff):
    r = np.ascontiguousarray(r, dtype=np.float64)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    arrs = [np.ascontiguousarray(q, dtype=np.float64) for q in (m, rho, a, h)]
    b = (ctypes.c_double * 4)(*[float(v) for v in bounds])
    Z = np.zeros((x.size, y.size))
    _abi.check(_abi.lib().sph_splash_map(
        mode, r.shape[0], r.ctypes.data, r.shape[1], *[q.ctypes.data for q in arrs],
        x.size, y.size, x.ctypes.data, y.ctypes.data, float(z), b, float(cutoff),
        Z.ctypes.data, _abi.SPH_HOST, None), "sph_splash_map")
    return Z


def splash_map_2d(x, y, r, m, rho, a, h, bounds, cutoff):
    """Particles of a 2D system onto the (x, y) pixel grid (interpolate.py:39-88)."""
    return _splash(2, x, y, 0.0, r, m, rho, a, h, bounds, cutoff)


def splash_map_3d(x, y, z, r, m, rho, a, h, bounds, cutoff):
    """Particles of a 3D system onto the plane at height z (interpolate.py:90-149)."""
    return _splash(3, x, y, z, r, m, rho, a, h, bounds, cutoff)
