"""Smooth-particle properties, mirroring pyticles' properties.py.

spam_properties(p, nl) -- the summation density of every particle (Lucy
kernel at the short smoothing length, self term W(0, h) without m_i), then
the van der Waals pressures from the current temperatures and the energies
those temperatures imply (properties.py:63-120).  The density comes from
libsph's density pass at the current positions (the pair set of a freshly
built list); the velocity gradient tensor p.gradv, which no force uses, is
not computed.  pyticles' run scripts call it once to initialise u from T.

vdw, vdw_energy, vdw_temp -- the equation-of-state formulas of
properties.py:38-49 on host arrays, for setting up states; ideal_isothermal
and art_water, the reference's other equations of state (properties.py:
24-36), likewise (the engine's step uses van der Waals).

spam_properties_ls(p, nl) -- the same with rho_lr at the long length.

hamiltonian(p) -- the total energy sum(m v^2 / 2) + sum(u) of the host
arrays, printed and returned (properties.py:55-60).
"""
import numpy as np

from . import _abi
from .engine import Engine

# properties.py:18-21
ADASH = 2.0
BDASH = 0.5
KBDASH = 1.0
RHONAUGHT = 1.0


def ideal_isothermal(rho, t):
    """Isothermal kinetic pressure rho k_B (properties.py:24-29)."""
    return rho * KBDASH


def art_water(rho, t):
    """Compressible liquid about the reference density (properties.py:32-36)."""
    return (rho - RHONAUGHT) * KBDASH


def vdw(rho, t):
    """Repulsive and cohesive van der Waals pressure (properties.py:38-41)."""
    return (rho * KBDASH * t) / (1 - rho * BDASH), -ADASH * rho * rho


def vdw_energy(rho, t):
    """u = k_B T - a rho (properties.py:44-46)."""
    return t * KBDASH - ADASH * rho


def vdw_temp(rho, u):
    """T = (u + a rho) / k_B (properties.py:48-49)."""
    return (u + ADASH * rho) / KBDASH


calc_pressure = vdw


def hamiltonian(p):
    """Kinetic plus internal energy of the first p.n particles, the internal
    energy summed without a mass factor as in properties.py:55-60."""
    n = p.n
    v = np.asarray(p.v[:n], dtype=np.float64)
    h = float(np.sum(0.5 * p.m[:n] * np.sum(v * v, axis=1)) + np.sum(p.u[:n]))
    print(h)
    return h


def summation_density(p, nl, precision=None):
    """rho at the short smoothing length p.h[0] on the GPU (Lucy kernel)."""
    return _densities(p, nl, precision)[0]


def _densities(p, nl, precision=None):
    """rho and rho_lr at p.h[0] and p.hlr[0] on the GPU (Lucy kernel)."""
    n = p.n
    cutoff, tol = nl._cutoff_tol()
    prm = _abi.make_params(dim=p.dim, kernel="lucy", box=p.box.extents,
                           h_short=float(p.h[0]), h_long=float(p.hlr[0]), cutoff=cutoff,
                           tolerance=tol, adash=ADASH, bdash=BDASH, kbdash=KBDASH, dt=1.0)
    precision = precision or getattr(p, "precision", "fp64")
    with Engine(prm, precision, max_particles=max(n, 1)) as e:
        s = e.add(prm, p.r[:n], p.v[:n], p.m[:n], np.zeros(n))
        out = e.derivatives(s)
        e.sync()
    return out["rho"], out["rho_lr"]


def spam_properties(p, nl):
    """properties.spam_properties: density, pressures from the current
    temperatures, u = vdw_energy(rho, T), T = vdw_temp(rho, u)."""
    n = p.n
    rho = summation_density(p, nl)
    p.rho[:n] = rho
    p.p[:n], p.pco[:n] = calc_pressure(p.rho[:n], p.t[:n])
    p.u[:n] = vdw_energy(p.rho[:n], p.t[:n])
    p.t[:n] = vdw_temp(p.rho[:n], p.u[:n])


def spam_properties_ls(p, nl):
    """properties.spam_properties_ls (properties.py:123-188): spam_properties
    with the density at the long smoothing length, p.rho_lr, as well (the
    reference's body names the long length h_lr, which it never defines; it
    is p.hlr).  Pressures and energies follow the short density, as there."""
    n = p.n
    rho, rho_lr = _densities(p, nl)
    p.rho[:n] = rho
    p.rho_lr[:n] = rho_lr
    p.p[:n], p.pco[:n] = calc_pressure(p.rho[:n], p.t[:n])
    p.u[:n] = vdw_energy(p.rho[:n], p.t[:n])
    p.t[:n] = vdw_temp(p.rho[:n], p.u[:n])
