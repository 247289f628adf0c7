"""Pair forces, mirroring pyticles' forces.py and spam_complete_force.py.

The force objects describe which terms the GPU derivative evaluation
computes; the arithmetic runs in libsph's force pass:

* SpamForce + CohesiveSpamForce (forces.py:321-405), and their 2D forms
  SpamForce2d + CohesiveSpamForce2d (:246-318): van der Waals repulsive
  pressure on the short smoothing length and cohesive pressure on the long
  one, energy rate du = a.dv/2 per pair.
* SpamComplete (spam_complete_force.py:19-183): the same plus artificial
  viscosity (eta, zeta) and optionally the heat flux, in one call.
* SpamConduction (c_forces.pyx:185-239): adds the heat-flux energy term.

Force.apply() runs one evaluation of the whole derivative for the
particle system it belongs to and writes p.rho, p.rho_lr, p.t, p.p, p.pco,
p.vdot, p.udot and p.jq, as SpamComplete.apply does (:171-183).

Hard collisions (forces.py:87-243, 454-474) mutate p.v (and, for
CollisionForce3d, p.r) over the neighbour list's pairs on the device
(sph_collide_pairs); inside SmoothParticleSystem.update the engine applies
CollisionForce / FortranCollisionForce after every evaluation itself.
"""
import warnings

import numpy as np

from . import _abi


class Force:
    """A generic pairwise force (forces.py:22-42)."""

    def __init__(self, particles, nl, cutoff=100.0):
        self.p = particles
        self.nl = nl
        self.cutoff = cutoff
        self.cutoffsq = cutoff * cutoff

    def apply(self):
        self.p.derivatives()


class SpamForce(Force):
    """Repulsive van der Waals pressure force (forces.py:321-368)."""

    def __init__(self, particles, neighbour_list, cutoff=5.0):
        Force.__init__(self, particles, neighbour_list, cutoff=cutoff)


class CohesiveSpamForce(Force):
    """Cohesive pressure force on the long smoothing length (forces.py:371-405)."""

    def __init__(self, particles, neighbour_list, cutoff=10.0):
        Force.__init__(self, particles, neighbour_list, cutoff=cutoff)


class SpamForce2d(SpamForce):
    """The 2D form of SpamForce (forces.py:246-274): the same terms, which
    the engine evaluates in the system's dimension."""


class CohesiveSpamForce2d(CohesiveSpamForce):
    """The 2D cohesive force (forces.py:277-318).  The reference's active body
    repeats the repulsive pressure term (p / rho^2, :300-318) and keeps the
    cohesive one (pco / rho^2) commented out (:286-298); the engine computes
    the cohesive term, as CohesiveSpamForce does in 3D."""


class SpamConduction(Force):
    """Heat conduction energy rate with the full heat-flux vector
    (c_forces.pyx:185-239)."""

    def __init__(self, particles, nl):
        Force.__init__(self, particles, nl)


_cgrad_warned = False


def _warn_cgrad():
    global _cgrad_warned
    if not _cgrad_warned:
        _cgrad_warned = True
        warnings.warn("SpamComplete: the density-gradient term (cgrad) of the reference's "
                      "absent Fortran force is not computed; the evaluation runs without it "
                      "(pass cgrad=0.0 to silence this warning)", RuntimeWarning, stacklevel=3)


class SpamComplete(Force):
    """All smooth-particle properties and forces in one evaluation
    (spam_complete_force.py:19-60).

    adash, bdash, kbdash -- van der Waals a, b, k_B
    sigma, rcoef         -- the repulsive core (spam_complete_force.py:40-41,
                            55-56) lives in the absent Fortran: non-zero
                            values raise NotImplementedError
    cgrad                -- the density-gradient term (spam_complete_force.py:
                            42, 57) lives in the absent Fortran too and is NOT
                            computed at any value, its reference default 1.0
                            included: a non-zero cgrad warns once
                            (RuntimeWarning) and the evaluation runs without
                            the term, as the reference's own drivers
                            configure it (nanobox_quench.py:93 passes
                            cgrad=0.0)
    eta, zeta            -- artificial viscosity: Monaghan alpha = eta,
                            beta = zeta, sound speed 1 (the reference passes
                            c = 1, :142)
    kernel_type          -- ignored, as in the reference (:60 forces Lucy)
    kernel               -- extension: 'lucy', 'gaussian', 'debrun', 'cubic'
    heat_flux            -- extension: Fourier heat flux + conduction rate
    """

    def __init__(self, particles, neighbour_list, adash=2.0, bdash=0.5, kbdash=1.0,
                 sigma=0.0, rcoef=0.0, cgrad=1.0, eta=1.0, zeta=0.1, kernel_type=2,
                 cutoff=5.0, kernel="lucy", heat_flux=False, thermalk=1.0, visc_eps=0.01,
                 sound_speed=1.0):
        Force.__init__(self, particles, neighbour_list, cutoff=cutoff)
        if sigma != 0.0 or rcoef != 0.0:
            raise NotImplementedError("the repulsive core (sigma, rcoef) has no source in "
                                      "pyticles and is not implemented")
        if cgrad != 0.0:
            _warn_cgrad()
        self.adash, self.bdash, self.kbdash = adash, bdash, kbdash
        self.sigma, self.rcoef, self.cgrad = sigma, rcoef, cgrad
        self.eta, self.zeta = eta, zeta
        self.kernel_type = 2
        self.kernel = kernel
        self.heat_flux = heat_flux
        self.thermalk = thermalk
        self.visc_eps = visc_eps
        self.sound_speed = sound_speed


def collide(p, nl, cutoff, mode, dims=None):
    """Force.apply of a collision force (forces.py:38-42): pairs of nl with
    rij^2 <= cutoff^2, in list order, on the GPU.  dims: the velocity
    components the force acts on (CollisionForce: x and y)."""
    n, ni = p.n, nl.nip
    if ni == 0 or n == 0:
        return
    dim = p.dim if dims is None else dims
    v = np.ascontiguousarray(p.v[:n, :dim], dtype=np.float64)
    r = np.ascontiguousarray(p.r[:n, :dim], dtype=np.float64)
    m = np.ascontiguousarray(p.m[:n], dtype=np.float64)
    iap = np.ascontiguousarray(nl.iap[:ni], dtype=np.int64)
    drij = np.ascontiguousarray(nl.drij[:ni, :dim], dtype=np.float64)
    rij = np.ascontiguousarray(nl.rij[:ni], dtype=np.float64)
    _abi.check(_abi.lib().sph_collide_pairs(dim, mode, n, r.ctypes.data, v.ctypes.data,
                                            m.ctypes.data, ni, iap.ctypes.data,
                                            drij.ctypes.data, rij.ctypes.data, float(cutoff),
                                            _abi.SPH_HOST, None), "sph_collide_pairs")
    p.v[:n, :dim] = v
    if mode == _abi.SPH_COLLIDE_PUSHBACK:
        p.r[:n, :dim] = r
        nl.drij[:ni, :dim] = drij
        nl.rij[:ni] = rij


class CollisionForce(Force):
    """Hard 2D collisions (forces.py:87-156): a pair that is not separating
    trades the x/y velocity components along its separation, scaled by the
    mass ratio."""

    mode = _abi.SPH_COLLIDE_EXCHANGE
    dims = 2

    def __init__(self, particles, neighbour_list, cutoff=5.0):
        Force.__init__(self, particles, neighbour_list, cutoff=cutoff)

    def apply(self):
        collide(self.p, self.nl, self.cutoff, self.mode, min(self.dims, self.p.dim))


class CollisionForce3d(CollisionForce):
    """Hard 3D collisions with the pushback that separates the pair to
    cutoff + 0.01 (forces.py:158-243)."""

    mode = _abi.SPH_COLLIDE_PUSHBACK
    dims = 3


class FortranCollisionForce(CollisionForce):
    """forces.py:454-474.  Its collide3d (Fortran) is absent from pyticles;
    it is restated as CollisionForce3d's velocity exchange, without the
    pushback (collide3d receives no positions)."""

    dims = 3

    def __init__(self, particles, neighbour_list, cutoff=1.0):
        CollisionForce.__init__(self, particles, neighbour_list, cutoff=cutoff)
