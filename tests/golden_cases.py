"""Loads the golden fixtures of tests/golden/ (made by make_golden.py from
the reference's own Python) into oracle / engine inputs."""
import os

import numpy as np

from pyticles_gb300._abi import make_params

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

SYSTEMS = ["lucy3d_27", "lucy2d_400", "lucy2d_1024", "gauss2d_256", "debrun3d_216",
           "thermo2d_400", "euler2d_144", "rk4_2d_144"]


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False))


def params_of(g, **over):
    kw = dict(dim=int(g["dim"]), kernel=str(g["kernel"]), box=[float(x) for x in g["box"]],
              h_short=float(g["h_short"]), h_long=float(g["h_long"]),
              cutoff=float(g["cutoff"]), tolerance=float(g["tolerance"]), dt=float(g["dt"]),
              integrator=str(g["integrator"]), thermostat=bool(int(g["thermostat"])),
              thermostat_temp=float(g["thermostat_temp"]), viscosity=False, heat_flux=False)
    kw.update(over)
    return make_params(**kw)


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (den if den > 0 else 1.0))


def sort_pairs(iap):
    iap = np.asarray(iap, dtype=np.int64)
    lo = np.minimum(iap[:, 0], iap[:, 1])
    hi = np.maximum(iap[:, 0], iap[:, 1])
    idx = np.lexsort((hi, lo))
    return np.stack([lo[idx], hi[idx]], axis=1), idx


def collide_params(g, **over):
    """Engine parameters of a collision fixture (collision_case in make_golden.py)."""
    kw = dict(dim=int(g["dim"]), kernel=str(g["kernel"]), box=[float(x) for x in g["box"]],
              h_short=float(g["h_short"]), h_long=float(g["h_long"]),
              cutoff=float(g["cutoff"]), tolerance=0.0, dt=float(g["dt"]),
              integrator=str(g["integrator"]), viscosity=False, heat_flux=False,
              collision_cutoff=float(g["collision_cutoff"]))
    kw.update(over)
    return make_params(**kw)
