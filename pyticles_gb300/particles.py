"""Particle systems, mirroring pyticles' particles.py.

SmoothParticleSystem keeps the reference's constructor, state arrays
(r, v, m, rho, rho_lr, t, u, p, pco, vdot, udot, jq, h, hlr ...), its
nlists / forces / nl_default wiring and update(dt).  update() uploads the
host state to libsph, runs one integrator step on the GPU (density ->
EOS -> forces/rates -> integrator -> periodic wrap -> thermostat) and copies
the state and properties back, with the reference's post-update semantics
(particles.py:459-494, 496-542).  run(dt, nsteps) advances several steps
with a single upload and download.  gather_state / scatter_state /
gather_derivatives and create_particle keep the reference's state-vector
interface for callers that drive their own integrator or add particles.

The engine configuration is derived from the attached objects:
  box      PeriodicBox (box.py:28-47) -> periodic extents
  nlist    VerletList(cutoff, tolerance) -> pair set; NeighbourList -> all pairs
  forces   SpamComplete -> Lucy (or its `kernel`), viscosity eta/zeta,
           optional heat flux; SpamForce + CohesiveSpamForce -> no viscosity;
           SpamConduction -> heat flux
  h, hlr   uniform short / long smoothing lengths
"""
import time

import numpy as np

from . import _abi
from .box import MirrorBox, PeriodicBox
from .neighbour_list import SortedVerletList
from .engine import Engine
from .forces import (CohesiveSpamForce, CollisionForce, CollisionForce3d, SpamComplete,
                     SpamConduction, SpamForce)

XMAX = 5
YMAX = 5
ZMAX = 1
VMAX = 0.1
VSPLIT = 10.0
RAMAL = 0.5

# properties.py:18-20
ADASH = 2.0
BDASH = 0.5
KBDASH = 1.0


class ParticleSystem:
    """Particles with basic mechanical properties (particles.py:69-195)."""

    # Rows of the state vector x: m, r (3 rows), v (3 rows); the reference
    # lays them out for 3D (particles.py:198-233), and a 2D system leaves the
    # z rows at zero so that every row keeps its number.
    N_VARIABLES = 7

    def __init__(self, n, d=3, maxn=125, controllers=(), xmax=XMAX, ymax=YMAX, zmax=ZMAX,
                 vmax=VMAX, simbox=None, mass=1.0, rinit=None, source=None, side=(5, 5, 5),
                 integrator="rk4", spacing=0.1):
        if d not in (2, 3):
            raise ValueError("the GB300 engine runs 2D and 3D systems")
        self.n = n
        self.dim = d
        self.maxn = maxn
        self.dt = 0.0
        self.steps = 0
        self.box = simbox if simbox else MirrorBox(p=self, xmax=xmax, ymax=ymax, zmax=zmax)
        if integrator not in _abi.INTEGRATORS:
            raise KeyError(integrator)
        self.integrator = integrator
        self.r = self.box.xmax * np.random.random([self.maxn, self.dim])
        self.m = np.zeros(self.maxn, dtype=float)
        self.v = vmax * (np.random.random([self.maxn, self.dim]) - 0.5)
        self.rdot = np.zeros(self.r.shape)
        self.vdot = np.zeros(self.v.shape)
        self.mdot = np.zeros(self.m.shape)
        if rinit in ("grid", "fcc", "load"):
            raise NotImplementedError(f"rinit={rinit!r} needs pyticles' absent configuration / "
                                      "netCDF modules; set p.r directly")
        self.m[:] = mass
        self.colour = 1.0, 0.0, 0.0
        # state vectors of the integrators (particles.py:151-154)
        self.x = np.zeros([self.N_VARIABLES, self.maxn])
        self.xdot = np.zeros([self.N_VARIABLES, self.maxn])
        self.nlists = []
        self.forces = []
        self.controllers = list(controllers)
        self.timing = {"force time": -1, "deriv time": -1, "pairsep time": -1,
                       "update time": -1, "integrate time": -1}

    def rebuild_lists(self):
        for nl in self.nlists:
            if nl.rebuild_list:
                nl.build()

    def create_particle(self, r, v=None):
        """Appends a particle at index n with the mass of particle n - 1
        (particles.py:171-178); v defaults to rest."""
        if self.n >= self.maxn:
            raise ValueError(f"the system holds maxn = {self.maxn} particles already")
        self.r[self.n] = r
        self.m[self.n] = self.m[self.n - 1]
        self.v[self.n] = 0.0 if v is None else v
        self.n += 1
        self.rebuild_lists()

    def gather_state(self):
        """The state vector x of the first n particles (particles.py:200-210)."""
        n, d = self.n, self.dim
        self.x[0, :n] = self.m[:n]
        self.x[1:1 + d, :n] = self.r[:n].T
        self.x[4:4 + d, :n] = self.v[:n].T
        return self.x

    def scatter_state(self, x):
        """Particle arrays from the state vector x (particles.py:212-221)."""
        n, d = self.n, self.dim
        self.m[:n] = x[0, :n]
        self.r[:n] = x[1:1 + d, :n].T
        self.v[:n] = x[4:4 + d, :n].T

    def gather_derivatives(self):
        """The rates xdot of the state vector (particles.py:223-233)."""
        n, d = self.n, self.dim
        self.xdot[0, :n] = self.mdot[:n]
        self.xdot[1:1 + d, :n] = self.rdot[:n].T
        self.xdot[4:4 + d, :n] = self.vdot[:n].T
        return self.xdot


class SmoothParticleSystem(ParticleSystem):
    """Long/short smoothing-length SPH system (particles.py:256-571).

    precision -- 'fp64' (default: the reference's arithmetic) or 'mixed'
                 (FP32 pair arithmetic, FP64 pair test and integrator)
    rebin     -- keep the cell list of the last binning across steps of run()
                 until a particle has used half of its cell slack (the skin
                 reuse of VerletList.compress/ponder_rebuild); the pair set
                 stays exact, the summation order follows the binning times
    pair_scheme -- 0: cell-window pair passes; 1: cluster pairs (a 3D system
                 in mixed precision, 1.5x faster; elsewhere the cell scheme
                 runs); 2: per-particle pair lists with a skin, rebuilt when
                 a particle has moved a quarter of it (mixed precision, 2D
                 or 3D; 1.5x the cell scheme in 2D, 1.7x the cluster pairs
                 in 3D); same pair set, rounding differs
    """

    N_VARIABLES = 11   # + rho, p, pco, u (particles.py:355-358)

    def __init__(self, n, d=3, maxn=100, controllers=(), xmax=XMAX, ymax=YMAX, zmax=ZMAX,
                 vmax=VMAX, rinit=None, side=None, mass=1.0, spacing=None, temperature=1.0,
                 thermostat_temp=1.0, thermostat=False, hshort=1.0, hlong=3.0, source=None,
                 integrator="ieuler", simbox=None, precision="fp64", rebin=False,
                 pair_scheme=0):
        ParticleSystem.__init__(self, n=n, d=d, xmax=xmax, ymax=ymax, zmax=zmax, rinit=rinit,
                                side=side, mass=mass, source=source, spacing=spacing,
                                integrator=integrator, vmax=vmax, maxn=maxn, simbox=simbox,
                                controllers=controllers)
        self.V_split = VSPLIT
        self.r_amalg = RAMAL
        self.rho = np.zeros(self.maxn)
        self.rho_lr = np.zeros(self.maxn)
        self.rhodot = np.zeros(self.rho.shape)
        self.gradv = np.zeros([self.maxn, self.dim, self.dim])
        self.jq = np.zeros([self.maxn, self.dim])
        self.t = np.ones(self.maxn)
        self.t[:] = temperature
        self.thermostat = thermostat
        self.u = np.ones(self.maxn, dtype=float)
        self.udot = np.zeros(self.maxn, dtype=float)
        self.h = np.zeros(self.maxn)
        self.hlr = np.zeros(self.maxn)
        self.h[:] = hshort
        self.hlr[:] = hlong
        self.p = np.zeros([self.maxn])
        self.pco = np.zeros([self.maxn])
        self.P = np.zeros([self.maxn, self.dim, self.dim])
        self.thermostat_temp = thermostat_temp
        self.precision = precision
        self.rebin = bool(rebin)
        self.pair_scheme = int(pair_scheme)
        self.timing["SPAM time"] = -1
        self.timing["nlist rebuild time"] = -1
        self._engine = None
        self._engine_key = None
        self._sim = None

    # -- engine configuration ------------------------------------------------
    def _nlist(self):
        nl = getattr(self, "nl_default", None)
        if nl is None and self.nlists:
            nl = self.nlists[0]
        if nl is None:
            raise RuntimeError("attach a neighbour list (p.nlists / p.nl_default)")
        return nl

    def engine_params(self, dt, thermostat=None):
        """sph_params for the attached box, neighbour list and forces
        (thermostat overrides the system's own switch)."""
        if not isinstance(self.box, PeriodicBox):
            raise NotImplementedError("the GB300 engine needs a PeriodicBox "
                                      f"(got {type(self.box).__name__})")
        n = self.n
        hs, hl = self.h[:n], self.hlr[:n]
        if n and (np.any(hs != hs[0]) or np.any(hl != hl[0])):
            raise NotImplementedError("per-particle smoothing lengths are not supported")
        nl = self._nlist()
        cutoff, tol = nl._cutoff_tol()
        kw = dict(dim=self.dim, box=self.box.extents, h_short=float(hs[0]),
                  h_long=float(hl[0]), cutoff=cutoff, tolerance=tol, dt=float(dt),
                  integrator=self.integrator,
                  thermostat=bool(self.thermostat if thermostat is None else thermostat),
                  thermostat_temp=float(self.thermostat_temp), adash=ADASH, bdash=BDASH,
                  kbdash=KBDASH)
        comp = [f for f in self.forces if isinstance(f, SpamComplete)]

        def has(cls):
            return any(isinstance(f, cls) for f in self.forces)

        if comp:
            f = comp[0]
            kw.update(kernel=f.kernel, adash=f.adash, bdash=f.bdash, kbdash=f.kbdash,
                      viscosity=(f.eta != 0.0 or f.zeta != 0.0), visc_alpha=f.eta,
                      visc_beta=f.zeta, visc_eps=f.visc_eps, sound_speed=f.sound_speed,
                      heat_flux=bool(f.heat_flux), thermalk=f.thermalk)
        elif has(SpamForce) and has(CohesiveSpamForce):
            kw.update(kernel="lucy", viscosity=False)
        else:
            raise NotImplementedError("the GB300 engine evaluates SpamComplete or the "
                                      "SpamForce + CohesiveSpamForce pair")
        if has(SpamConduction):
            kw["heat_flux"] = True
        kw["collision_cutoff"] = self._collision_cutoff(cutoff, tol)
        return _abi.make_params(**kw)

    def _collision_forces(self):
        return [f for f in self.forces if isinstance(f, CollisionForce)]

    def _collision_cutoff(self, cutoff, tol):
        """The engine's collision range: CollisionForce / FortranCollisionForce
        placed after the SPH forces (bspana.py:45-46, fspana.py:117-119)."""
        coll = self._collision_forces()
        if not coll:
            return 0.0
        f = coll[0]
        if len(coll) > 1 or isinstance(f, CollisionForce3d):
            raise NotImplementedError(
                "the engine step runs one CollisionForce or FortranCollisionForce; "
                "CollisionForce3d's pushback moves particles inside the step -- apply() it "
                "between steps instead")
        if self.forces.index(f) != len(self.forces) - 1:
            raise NotImplementedError("a collision force must come after the SPH forces")
        if self.dim == 3 and f.dims == 2:
            raise NotImplementedError("CollisionForce (x/y only) in a 3D engine step")
        if isinstance(f.nl, SortedVerletList):
            # the engine applies collisions in VerletList's (i, j) order; the
            # reference's sort_by_r permutes rij twice (neighbour_list.py:276-278),
            # so its sorted-list collision order has no consistent meaning
            raise NotImplementedError("collision forces over a SortedVerletList in the engine "
                                      "step; apply() them over the list instead")
        fc, ft = f.nl._cutoff_tol()
        if f.cutoff ** 2 > min(cutoff * cutoff + tol * tol, fc * fc + ft * ft):
            raise NotImplementedError("collision range beyond the neighbour list's pairs")
        return float(f.cutoff)

    def _ensure_engine(self, dt, thermostat=None):
        prm = self.engine_params(dt, thermostat)
        key = (repr(sorted(_abi.params_dict(prm).items())), self.n, self.precision)
        n = self.n
        if self._engine is None or self._engine_key != key:
            if self._engine is not None:
                self._engine.close()
            self._engine = Engine(prm, precision=self.precision, max_particles=max(n, 1),
                                  max_sims=1)
            self._engine.set_tuning(rebin=int(self.rebin), pair_scheme=self.pair_scheme)
            self._sim = self._engine.add(prm, self.r[:n], self.v[:n], self.m[:n], self.u[:n])
            self._engine_key = key
        else:
            self._engine.set_state(self._sim, self.r[:n], self.v[:n], self.m[:n], self.u[:n])
        return self._engine

    def _download(self, props_fn):
        n = self.n
        e = self._engine
        r, v, u = e.get_state(self._sim)
        self.r[:n] = r
        self.v[:n] = v
        self.u[:n] = u
        out = props_fn(self._sim)
        self.rho[:n] = out["rho"]
        self.rho_lr[:n] = out["rho_lr"]
        self.t[:n] = out["t"]
        self.p[:n] = out["p"]
        self.pco[:n] = out["pco"]
        self.vdot[:n] = out["vdot"]
        self.udot[:n] = out["udot"]
        self.jq[:n] = out["jq"]
        self.rdot = self.v

    # -- the reference's step API ---------------------------------------------
    def derivatives(self):
        """One evaluation of the rates at the current state on the GPU
        (particles.py:544-567 with SpamComplete.apply)."""
        t = time.time()
        e = self._ensure_engine(self.dt if self.dt > 0 else 1.0)
        out = e.derivatives(self._sim)
        e.sync()
        n = self.n
        self.rho[:n] = out["rho"]
        self.rho_lr[:n] = out["rho_lr"]
        self.t[:n] = out["t"]
        self.p[:n] = out["p"]
        self.pco[:n] = out["pco"]
        self.vdot[:n] = out["vdot"]
        self.udot[:n] = out["udot"]
        self.jq[:n] = out["jq"]
        # collision forces mutate v after the rates (particles.py:562-564)
        for f in self._collision_forces():
            f.nl.separations()
            f.apply()
        self.rdot = self.v
        self.timing["force time"] = time.time() - t

    def update(self, dt):
        """One integrator step (particles.py:459-494)."""
        self.run(dt, 1)

    def run(self, dt, nsteps):
        """nsteps integrator steps with one upload and one download."""
        t1 = time.time()
        t = time.time()
        self.rebuild_lists()
        self.timing["nlist rebuild time"] = time.time() - t
        self._advance(dt, nsteps)
        self.steps += nsteps
        self.timing["update time"] = time.time() - t1

    def _advance(self, dt, nsteps, thermostat=None):
        """nsteps engine steps from the host arrays back into them."""
        self.dt = dt
        e = self._ensure_engine(dt, thermostat)
        t = time.time()
        e.advance(nsteps)
        e.sync()
        self.timing["integrate time"] = time.time() - t
        self._download(e.properties)

    def gather_state(self):
        """x with the smooth particle rows rho, p, pco, u (particles.py:496-511)."""
        n = self.n
        ParticleSystem.gather_state(self)
        for row, a in zip(range(7, 11), (self.rho, self.p, self.pco, self.u)):
            self.x[row, :n] = a[:n]
        return self.x

    def scatter_state(self, x):
        """The inverse of gather_state (particles.py:513-526)."""
        n = self.n
        ParticleSystem.scatter_state(self, x)
        for row, a in zip(range(7, 11), (self.rho, self.p, self.pco, self.u)):
            a[:n] = x[row, :n]

    def gather_derivatives(self):
        """xdot with rhodot, zero rates for p and pco, and udot
        (particles.py:528-542)."""
        n = self.n
        ParticleSystem.gather_derivatives(self)
        self.xdot[7, :n] = self.rhodot[:n]
        self.xdot[8:10, :n] = 0.0
        self.xdot[10, :n] = self.udot[:n]
        return self.xdot

    def apply_thermostat(self, target_temp):
        """Scaling thermostat on the host arrays (particles.py:450-457); the
        GPU step applies it itself when `thermostat` is set."""
        tav = self.t.mean()
        self.t = self.t * (target_temp / tav)
        self.u = self.t * KBDASH - ADASH * self.rho

    def close(self):
        if self._engine is not None:
            self._engine.close()
            self._engine = None
