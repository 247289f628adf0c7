"""Pair forces, mirroring pyticles' forces.py and spam_complete_force.py.

The force objects describe which terms the GPU derivative evaluation
computes; the arithmetic runs in libsph's force pass:

* SpamForce + CohesiveSpamForce (forces.py:321-405): van der Waals
  repulsive pressure on the short smoothing length and cohesive pressure on
  the long one, energy rate du = a.dv/2 per pair.
* SpamComplete (spam_complete_force.py:19-183): the same plus artificial
  viscosity (eta, zeta) and optionally the heat flux, in one call.
* SpamConduction (c_forces.pyx:185-239): adds the heat-flux energy term.

Force.apply() runs one evaluation of the whole derivative for the
particle system it belongs to and writes p.rho, p.rho_lr, p.t, p.p, p.pco,
p.vdot, p.udot and p.jq, as SpamComplete.apply does (:171-183).
"""


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


class SpamConduction(Force):
    """Heat conduction energy rate with the full heat-flux vector
    (c_forces.pyx:185-239)."""

    def __init__(self, particles, nl):
        Force.__init__(self, particles, nl)


class SpamComplete(Force):
    """All smooth-particle properties and forces in one evaluation
    (spam_complete_force.py:19-60).

    adash, bdash, kbdash -- van der Waals a, b, k_B
    sigma, rcoef, cgrad  -- accepted for compatibility; the repulsive core and
                            density-gradient terms live in the absent Fortran
                            and are not computed (sigma = rcoef = 0 defaults)
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
        self.adash, self.bdash, self.kbdash = adash, bdash, kbdash
        self.sigma, self.rcoef, self.cgrad = sigma, rcoef, cgrad
        self.eta, self.zeta = eta, zeta
        self.kernel_type = 2
        self.kernel = kernel
        self.heat_flux = heat_flux
        self.thermalk = thermalk
        self.visc_eps = visc_eps
        self.sound_speed = sound_speed
