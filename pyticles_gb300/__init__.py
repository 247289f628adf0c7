"""pyticles_gb300 -- pyticles' SPH step (cell-list neighbour search,
summation density, van der Waals pressure forces with viscosity and heat
flux, improved-Euler integrator, periodic box) on GB300 (sm_103a) CUDA
kernels behind a C ABI (include/sph.h, libsph.so).

Reference-facing API (same names as andrewcharles/pyticles):
    SmoothParticleSystem, ParticleSystem      particles.py
    NeighbourList, VerletList, SortedVerletList neighbour_list.py
    Force, SpamForce, CohesiveSpamForce, SpamForce2d, CohesiveSpamForce2d,
    SpamConduction, SpamComplete
    CollisionForce, CollisionForce3d, FortranCollisionForce
    PeriodicBox
    properties.spam_properties, vdw, vdw_energy, vdw_temp
    integrator.euler, imp_euler, rk4         (the engine step of a system)
    spkernel.kernel, lucy_kernel, gauss_kernel, debrun_kernel, lucy_w, lucy_w3d
Engine-level API: Engine (many simulations per engine), workloads, serve.
"""
from ._abi import KERNELS, SphError, SphParams, make_params  # noqa: F401
from .box import Box, MirrorBox, PeriodicBox  # noqa: F401
from .engine import Engine  # noqa: F401
from .forces import (CohesiveSpamForce, CohesiveSpamForce2d, CollisionForce,  # noqa: F401
                     CollisionForce3d, Force, FortranCollisionForce, SpamComplete,
                     SpamConduction, SpamForce, SpamForce2d)
from .neighbour_list import NeighbourList, SortedVerletList, VerletList  # noqa: F401
from .particles import ParticleSystem, SmoothParticleSystem  # noqa: F401
from . import integrator, properties, spkernel  # noqa: F401

__version__ = "0.1.0"
