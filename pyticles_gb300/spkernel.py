"""Smoothing kernels, mirroring pyticles' spkernel.py.

The functions keep the reference signatures and return conventions
(spkernel.py:22-153) and evaluate the kernels of the pair passes on the GPU
(libsph's sph_kernel_eval), for one pair or for arrays of pairs at once:
r has shape (n,) or is a scalar, dx the matching (n, dim) or (dim,).

  lucy_kernel, debrun_kernel -> w, dwdx = (dW/dr) dx / r (0 at r = 0)
  cubic_kernel               -> the same for the M4 spline
  gauss_kernel               -> w, dwdx = -(dW/dr) dx / r, the reference's
                                sign (spkernel.py:51)
  kernel(r, dx, h, type)     -> by name ('gaussian', 'lucy', 'debrun', and
                                'cubic', the M4 spline the engine adds)
  lucy_w, lucy_w3d           -> W only, 2D and 3D

Dimensions 2 and 3 (those the engine runs); dx decides the dimension as in
the reference.  precision='mixed' evaluates as the mixed-precision passes do.
"""
import numpy as np

from . import _abi
from .engine import PRECISIONS

ktable = {1: "gaussian", 2: "lucy", 3: "debrun", 4: "cubic"}
_IDS = {name: k for k, name in ktable.items()}


def evaluate(r, h, kernel="lucy", dim=3, precision="fp64"):
    """W(r, h) and g = (dW/dr)/r at the distances r (arrays of r's shape)."""
    r = np.asarray(r, dtype=np.float64)
    flat = np.ascontiguousarray(np.abs(r).ravel())
    w = np.empty_like(flat)
    g = np.empty_like(flat)
    kid = kernel if isinstance(kernel, (int, np.integer)) else _IDS[kernel]
    _abi.check(_abi.lib().sph_kernel_eval(
        int(kid), int(dim), float(h), PRECISIONS[precision], flat.size, flat.ctypes.data,
        w.ctypes.data, g.ctypes.data, _abi.SPH_HOST, None), "sph_kernel_eval")
    return w.reshape(r.shape), g.reshape(r.shape)


def _with_gradient(kid, r, dx, h, sign, precision):
    dx = np.atleast_1d(np.asarray(dx, dtype=np.float64))
    dim = dx.shape[-1]
    if dim not in (2, 3):
        raise NotImplementedError("the engine's kernels are 2D and 3D")
    w, g = evaluate(r, h, kid, dim, precision)
    # dwdx = g dx; at r = 0 Lucy and Debrun return 0 (spkernel.py:108-109,
    # 143-144), the Gaussian its finite g dx
    gg = sign * g
    if kid in (2, 3):
        gg = np.where(np.asarray(r) == 0.0, 0.0, gg)
    dwdx = np.asarray(gg)[..., None] * dx
    if np.ndim(r) == 0:
        return float(w), dwdx.reshape(dim)
    return w, dwdx


def gauss_kernel(r, dx, h, precision="fp64"):
    """Gaussian W and the reference's gradient +2 W dx / h^2 (spkernel.py:39-52)."""
    return _with_gradient(1, r, dx, h, -1.0, precision)


def lucy_kernel(r, dx, h, precision="fp64"):
    """Lucy W and dwdx (spkernel.py:86-118)."""
    return _with_gradient(2, r, dx, h, 1.0, precision)


def debrun_kernel(r, dx, h, precision="fp64"):
    """Debrun's spiky W and dwdx (spkernel.py:120-153)."""
    return _with_gradient(3, r, dx, h, 1.0, precision)


def cubic_kernel(r, dx, h, precision="fp64"):
    """M4 cubic spline (Monaghan & Lattanzio 1985, support 2h) W and dwdx."""
    return _with_gradient(4, r, dx, h, 1.0, precision)


def kernel(r, dx, h, type, precision="fp64"):
    """W and dwdx of the kernel named `type` (spkernel.py:22-37)."""
    fn = {"gaussian": gauss_kernel, "lucy": lucy_kernel, "debrun": debrun_kernel,
          "cubic": cubic_kernel}[type]
    return fn(r, dx, h, precision)


def lucy_w(r, h):
    """2D Lucy W (spkernel.py:54-63)."""
    w, _ = evaluate(r, h, 2, 2)
    return float(w) if np.ndim(r) == 0 else w


def lucy_w3d(r, h):
    """3D Lucy W as a one-element array (spkernel.py:65-84)."""
    w, _ = evaluate(r, h, 2, 3)
    return np.atleast_1d(w)
