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


# ---- conditioning floors of the mixed-precision evaluation ----------------
# Both use the FP64 oracle only (test infrastructure).

FLOOR_KEYS = ("rho", "rho_lr", "t", "p", "pco", "vdot", "udot")


def position_floor(prm, r, v, m, u, shifts=4, seed=0):
    """Floor A: the largest relative L2 change of the FP64 evaluation when the
    positions are rounded to FP32 in cell-local frames (cells of half the
    cutoff, as the passes store them), over a few random frame offsets.
    No evaluation that starts from FP32 cell-local positions can be more
    accurate than this on the given system."""
    from oracle import oracle
    r = np.asarray(r, dtype=np.float64)
    ref = oracle.derivatives(prm, r, v, m, u)
    edge = 0.5 * float(prm.cutoff)
    rng = np.random.Generator(np.random.PCG64(seed))
    worst = {k: 0.0 for k in FLOOR_KEYS}
    for _ in range(shifts):
        shift = rng.uniform(-0.5, 0.5, size=r.shape[1]) * edge
        cen = (np.floor((r - shift) / edge) + 0.5) * edge + shift
        rp = cen + (r - cen).astype(np.float32).astype(np.float64)
        d = oracle.derivatives(prm, rp, v, m, u)
        for k in FLOOR_KEYS:
            worst[k] = max(worst[k], rel_l2(d[k], ref[k]))
    return worst


def geometry_floor(prm, r, v, m, u):
    """Floor B: the relative L2 change of the FP64 evaluation when every
    pair's separation vector and distance are the nearest FP32 numbers
    (oracle.derivatives(geometry32=True)) and all other arithmetic is FP64:
    the floor of any evaluation that carries pair geometry in FP32."""
    from oracle import oracle
    ref = oracle.derivatives(prm, r, v, m, u)
    d = oracle.derivatives(prm, r, v, m, u, geometry32=True)
    return {k: rel_l2(d[k], ref[k]) for k in FLOOR_KEYS}


def load_floors():
    import json
    with open(os.path.join(GOLDEN, "floors.json")) as f:
        return json.load(f)
