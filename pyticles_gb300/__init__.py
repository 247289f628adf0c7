"""pyticles_gb300 -- pyticles' SPH step (cell-list neighbour search,
summation density, van der Waals pressure forces with viscosity and heat
flux, improved-Euler integrator, periodic box) on GB300 (sm_103a) CUDA
kernels behind a C ABI (include/sph.h, libsph.so).

Reference-facing API (same names as andrewcharles/pyticles):
    SmoothParticleSystem, ParticleSystem      particles.py
    NeighbourList, VerletList, SortedVerletList neighbour_list.py
    Force, SpamForce, CohesiveSpamForce, SpamConduction, SpamComplete
    CollisionForce, CollisionForce3d, FortranCollisionForce
    PeriodicBox
    properties.spam_properties, vdw, vdw_energy, vdw_temp
Engine-level API: Engine (many simulations per engine), workloads, serve.
"""
from ._abi import KERNELS, SphError, SphParams, make_params  # noqa: F401
from .box import Box, MirrorBox, PeriodicBox  # noqa: F401
from .engine import Engine  # noqa: F401
from .forces import (CohesiveSpamForce, CollisionForce, CollisionForce3d,  # noqa: F401
                     Force, FortranCollisionForce, SpamComplete, SpamConduction, SpamForce)
from .neighbour_list import NeighbourList, SortedVerletList, VerletList  # noqa: F401
from .particles import ParticleSystem, SmoothParticleSystem  # noqa: F401
from . import properties  # noqa: F401

__version__ = "0.1.0"
