"""Simulation boxes, mirroring pyticles' box.py.

PeriodicBox is the box of the GPU step: its teleport wrap (r > L -> 0,
r < 0 -> L per axis, box.py:33-47) runs inside the engine's final force
pass.  PeriodicBox.apply(p) is kept for callers that wrap positions
themselves.  MirrorBox is not supported by the engine.
"""
import numpy as np


class Box:
    def __init__(self, p="none", xmax=64, ymax=48, zmax=100):
        self.p = p
        self.xmax = xmax
        self.ymax = ymax
        self.zmax = zmax

    @property
    def extents(self):
        return (float(self.xmax), float(self.ymax), float(self.zmax))

    def apply(self, p):
        return


class PeriodicBox(Box):
    """Periodic box with the reference's teleport wrap."""

    def apply(self, p):
        n = p.n
        for a, L in enumerate(self.extents[:p.dim]):
            x = p.r[:n, a]
            x[x > L] = 0
            x[x < 0] = L


class MirrorBox(Box):
    """Reflecting walls (box.py:49-73).  The GPU step has no reflecting
    boundary; systems using it cannot run on the engine."""

    def apply(self, p):
        raise NotImplementedError("MirrorBox is not supported by the GB300 engine; "
                                  "use PeriodicBox")


def wrap_teleport(r, extents):
    """Vectorised PeriodicBox wrap of an (n, d) array, in place."""
    for a in range(r.shape[1]):
        x = r[:, a]
        x[x > extents[a]] = 0
        x[x < 0] = extents[a]
    return r


__all__ = ["Box", "PeriodicBox", "MirrorBox", "wrap_teleport", "np"]
