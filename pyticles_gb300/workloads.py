"""Seeded synthetic initial states for the SPH workloads.

Positions: a square (cubic) lattice of spacing s with uniform jitter
U(-j s, +j s), particle k at ((i + 1/2) s + jitter); velocities Gaussian with
variance k_B T / m per component, mean momentum removed; m = 1.  Seeds use
numpy.random.Generator(PCG64(seed)) with seed = workload index * 1000 + sim
index.  The internal energy starts at the van der Waals value
u = k_B T - a rho (properties.py:44-46) and is set by the caller once the
initial density is known.
"""
import math

import numpy as np

from ._abi import make_params


def rng_for(seed):
    return np.random.Generator(np.random.PCG64(seed))


def lattice(side, dim, spacing, jitter, rng):
    """side**dim lattice points with cell-centred offsets and jitter."""
    axes = [(np.arange(side) + 0.5) * spacing] * dim
    grid = np.meshgrid(*axes, indexing="ij")
    r = np.stack([g.reshape(-1) for g in grid], axis=1).astype(np.float64)
    if jitter > 0:
        r += rng.uniform(-jitter * spacing, jitter * spacing, size=r.shape)
    return r


def maxwell(n, dim, temperature, mass, rng, kbdash=1.0):
    v = rng.normal(0.0, math.sqrt(kbdash * temperature / mass), size=(n, dim))
    v -= v.mean(axis=0, keepdims=True)
    return v


def lattice_system(side, dim, spacing=1.0, jitter=0.1, temperature=0.6, seed=1000,
                   mass=1.0, **param_kw):
    """Returns (params, r, v, m, T0) for a periodic lattice system whose box
    is side * spacing per axis."""
    rng = rng_for(seed)
    r = lattice(side, dim, spacing, jitter, rng)
    n = r.shape[0]
    v = maxwell(n, dim, temperature, mass, rng, param_kw.get("kbdash", 1.0))
    m = np.full(n, mass, dtype=np.float64)
    L = side * spacing
    box = [L] * dim + [1.0] * (3 - dim)
    params = make_params(dim=dim, box=box, **param_kw)
    return params, r, v, m, temperature


def config_2d(side, seed, viscosity=True, **kw):
    """The 2D van der Waals fluid: spacing 1, jitter 0.1, T=0.6, Lucy,
    h_s = 3, h_l = 6 spacings, a=2, b=0.5, dt=1e-3, improved Euler."""
    kw.setdefault("kernel", "lucy")
    kw.setdefault("h_short", 3.0)
    kw.setdefault("h_long", 6.0)
    kw.setdefault("dt", 1e-3)
    return lattice_system(side, 2, spacing=1.0, jitter=0.1, temperature=0.6, seed=seed,
                          viscosity=viscosity, **kw)


def config_3d(side, seed, density=0.7, **kw):
    """3D periodic cube at number density 0.7 with the cubic spline: support
    radii 2.735 (short, about 60 neighbours) and 5.148 (long, about 400),
    heat flux on."""
    spacing = density ** (-1.0 / 3.0)
    kw.setdefault("kernel", "cubic")
    kw.setdefault("h_short", 2.735 / 2.0)
    kw.setdefault("h_long", 5.148 / 2.0)
    kw.setdefault("dt", 1e-3)
    kw.setdefault("viscosity", True)
    kw.setdefault("heat_flux", True)
    return lattice_system(side, 3, spacing=spacing, jitter=0.1, temperature=0.6, seed=seed,
                          **kw)


def batched_2d(nsims, seed_base=4000, n_lo=256, n_hi=65536, t_lo=0.2, t_hi=1.2,
               dens_lo=0.4, dens_hi=0.9, ramp_steps=500, **kw):
    """512-simulation batched workload: N log-uniform in [n_lo, n_hi]
    (rounded to a square lattice), T ~ U[t_lo, t_hi], areal density ~
    U[dens_lo, dens_hi] (spacing n^-1/2, h in spacings as in the 2D fluid),
    thermostat quench T -> T/2 over ramp_steps steps."""
    meta = rng_for(seed_base)
    sims = []
    for s in range(nsims):
        n_target = math.exp(meta.uniform(math.log(n_lo), math.log(n_hi)))
        side = max(8, int(round(math.sqrt(n_target))))
        temp = meta.uniform(t_lo, t_hi)
        dens = meta.uniform(dens_lo, dens_hi)
        spacing = dens ** -0.5
        kw2 = dict(kw)
        kw2.setdefault("kernel", "lucy")
        kw2.setdefault("dt", 1e-3)
        kw2.setdefault("viscosity", True)
        kw2["h_short"] = 3.0 * spacing
        kw2["h_long"] = 6.0 * spacing
        kw2["thermostat"] = True
        kw2["thermostat_temp"] = temp
        kw2["thermostat_temp_end"] = 0.5 * temp
        kw2["thermostat_ramp_steps"] = ramp_steps
        sims.append(lattice_system(side, 2, spacing=spacing, jitter=0.1, temperature=temp,
                                   seed=seed_base + s, **kw2))
    return sims


def vdw_energy(rho, temperature, adash=2.0, kbdash=1.0):
    """u = k_B T - a rho (properties.py:44-46)."""
    return temperature * kbdash - adash * rho
