"""Neighbour lists, mirroring pyticles' neighbour_list.py.

The pair set is produced on the GPU by libsph's cell list with the
reference's FP64 test (i<j, dr = r_j - r_i, one minimum-image shift per axis,
rsq < cutoff^2 + tolerance^2; neighbour_list.py:105-123, 160-189), bit-exact
as a set.  build(), compress() and separations() export it with the
NeighbourList attributes nip, iap, rsq, rij, drij, dv; the step itself does
not need the exported list (it bins particles every step).
"""
import numpy as np

from . import _abi
from .engine import Engine


class NeighbourList:
    """All pairs (neighbour_list.py:16-124): the cutoff covers the box."""

    def __init__(self, particle):
        self.nip = 0
        self.particle = particle
        self.iap = np.zeros((0, 2), dtype=np.int64)
        self.rij = np.zeros(0)
        self.rsq = np.zeros(0)
        self.drij = np.zeros((0, particle.dim))
        self.dv = np.zeros((0, particle.dim))
        self.wij = np.zeros(0)
        self.wij_lr = np.zeros(0)
        self.dwij = np.zeros((0, particle.dim))
        self.dwij_lr = np.zeros((0, particle.dim))
        self.rebuild_list = False
        self.nforce = 0
        self.forces = []
        self._engine = None
        self._key = None

    # the pair-set cutoff of a brute-force list: every pair of the box
    def _cutoff_tol(self):
        ext = self.particle.box.extents[:self.particle.dim]
        return float(np.sqrt(sum(L * L for L in ext))) * 2.0 + 1.0, 0.0

    def _export(self):
        p = self.particle
        n = p.n
        cutoff, tol = self._cutoff_tol()
        prm = _abi.make_params(dim=p.dim, kernel="lucy", box=p.box.extents, h_short=1.0,
                               h_long=1.0, cutoff=cutoff, tolerance=tol, dt=1.0)
        key = (n, p.dim, cutoff, tol, p.box.extents)
        if self._engine is None or self._key != key:
            if self._engine is not None:
                self._engine.close()
            self._engine = Engine(prm, precision="fp64", max_particles=max(n, 1), max_sims=1)
            self._sim = self._engine.add(prm, p.r[:n], p.v[:n], p.m[:n], np.zeros(n))
            self._key = key
        else:
            self._engine.set_state(self._sim, p.r[:n], p.v[:n], p.m[:n], np.zeros(n))
        out = self._engine.pairs(self._sim)
        self.iap = out["iap"]
        self.rsq = out["rsq"]
        self.drij = out["drij"]
        self.dv = out["dv"]
        self.rij = np.sqrt(self.rsq)
        self.nip = len(self.iap)
        self.wij = np.zeros(self.nip)
        self.wij_lr = np.zeros(self.nip)
        self.dwij = np.zeros((self.nip, p.dim))
        self.dwij_lr = np.zeros((self.nip, p.dim))

    def build(self):
        self.rebuild_list = False
        self._export()

    def compress(self):
        print("Cannot compress a brute list")

    def separations(self):
        """drij (minimum image), rij, rsq and dv of the pairs at the current
        positions (neighbour_list.py:63-83)."""
        self._export()

    def find_pair(self, i, j):
        hit = np.nonzero((self.iap[:self.nip, 0] == i) & (self.iap[:self.nip, 1] == j))[0]
        return int(hit[0]) if len(hit) else -1

    def apply_minimum_image(self):
        ext = self.particle.box.extents
        for k in range(self.nip):
            self.minimum_image(self.drij[k, :], *ext)

    @staticmethod
    def minimum_image(dr, xmax, ymax, zmax):
        """One shift per axis with strict comparisons (neighbour_list.py:105-123)."""
        for a, L in enumerate((xmax, ymax, zmax)[:len(dr)]):
            if dr[a] > L / 2.:
                dr[a] = dr[a] - L
            if dr[a] < -L / 2.:
                dr[a] = dr[a] + L

    def close(self):
        if self._engine is not None:
            self._engine.close()
            self._engine = None


class VerletList(NeighbourList):
    """Pairs within cutoff plus a tolerance added in quadrature
    (neighbour_list.py:127-252)."""

    def __init__(self, particle, cutoff=2.0, tolerance=1.0):
        NeighbourList.__init__(self, particle)
        self.cutoff_radius = cutoff
        self.cutoff_radius_sq = cutoff ** 2
        self.tolerance = tolerance
        self.tolerance_sq = tolerance * tolerance
        self.r_old = np.zeros(particle.r.shape)

    def _cutoff_tol(self):
        return float(self.cutoff_radius), float(self.tolerance)

    def build(self):
        self.rebuild_list = False
        self.r_old[:, :] = self.particle.r[:, :]
        self._export()

    def compress(self):
        """Drops pairs outside cutoff + tolerance at the current positions and
        ponders a rebuild (neighbour_list.py:191-223)."""
        self._export()
        self.ponder_rebuild()

    def ponder_rebuild(self):
        """rebuild_list = True once any particle moved further than the
        tolerance since build (neighbour_list.py:225-234)."""
        dr = self.r_old - self.particle.r
        dsq = np.max(np.sum(dr * dr, axis=1))
        if dsq > self.tolerance_sq:
            self.rebuild_list = True

    def separations(self):
        self._export()


class SortedVerletList(VerletList):
    """A Verlet list sorted by descending separation (neighbour_list.py:262-301)."""

    def separations(self):
        VerletList.separations(self)
        self.sort_by_r()

    def sort_by_r(self):
        idx = np.argsort(self.rsq[:self.nip])[::-1]
        for name in ("iap", "rij", "rsq", "dv", "drij", "wij", "dwij", "wij_lr", "dwij_lr"):
            setattr(self, name, getattr(self, name)[idx])

    def build(self):
        VerletList.build(self)
        self.sort_by_r()

    def compress(self):
        VerletList.compress(self)
        self.sort_by_r()
