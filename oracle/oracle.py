"""TEST INFRASTRUCTURE ONLY: ctypes wrapper of the FP64 CPU oracle
(oracle/sph_oracle.c).  Imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference legs only, to compare results against.

build() compiles oracle/sph_oracle.c with gcc (-O2 -fopenmp
-ffp-contract=off) into oracle/_build/liboracle.so.
"""
import ctypes
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SRC = os.path.join(HERE, "sph_oracle.c")

sys.path.insert(0, ROOT)
from pyticles_gb300._abi import SphParams  # noqa: E402  (struct layout only)


def build(force=False):
    os.makedirs(BUILD, exist_ok=True)
    hdr = os.path.join(ROOT, "include", "sph.h")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) > max(os.path.getmtime(SRC), os.path.getmtime(hdr))):
        return LIB
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-fast-math", SRC, "-o", LIB + ".tmp", "-lm"]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        P = ctypes.POINTER
        vp, i64 = ctypes.c_void_p, ctypes.c_int64
        L.orc_pairs.argtypes = [P(SphParams), i64, vp, i64, vp, vp, P(i64)]
        L.orc_pairs_brute.argtypes = [P(SphParams), i64, vp, i64, vp, vp, P(i64)]
        L.orc_derivatives.argtypes = [P(SphParams), i64, vp, vp, vp, vp] + [vp] * 8 + [P(i64)]
        L.orc_advance.argtypes = ([P(SphParams), i64, vp, vp, vp, vp, ctypes.c_int32, i64]
                                  + [vp] * 8)
        L.orc_kernel.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                 P(ctypes.c_double), P(ctypes.c_double)]
        L.orc_kernel.restype = None
        L.orc_collide_pairs.argtypes = [ctypes.c_int32, ctypes.c_int32, i64, vp, vp, vp, i64,
                                        vp, vp, vp, ctypes.c_double]
        L.orc_collide_pairs.restype = ctypes.c_int
        L.orc_set_geometry32.argtypes = [ctypes.c_int]
        L.orc_set_geometry32.restype = None
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_set_threads.restype = None
        L.orc_get_threads.restype = ctypes.c_int
        for f in ("orc_pairs", "orc_pairs_brute", "orc_derivatives", "orc_advance"):
            getattr(L, f).restype = ctypes.c_int
        _lib = L
    return _lib


def _c(a, dtype=np.float64):
    return np.ascontiguousarray(a, dtype=dtype)


def set_threads(n):
    lib().orc_set_threads(int(n))


def threads():
    return lib().orc_get_threads()


def kernel(ktype, dim, r, h):
    w, g = ctypes.c_double(), ctypes.c_double()
    lib().orc_kernel(int(ktype), int(dim), float(r), float(h), ctypes.byref(w), ctypes.byref(g))
    return w.value, g.value


def pairs(params, r, brute=False):
    """Pair set (i<j) sorted by (i, j); returns (iap[nip,2], rsq[nip])."""
    r = _c(r)
    n = r.shape[0]
    fn = lib().orc_pairs_brute if brute else lib().orc_pairs
    nip = ctypes.c_int64()
    st = fn(ctypes.byref(params), n, r.ctypes.data, 0, None, None, ctypes.byref(nip))
    cap = nip.value
    iap = np.zeros((max(cap, 1), 2), dtype=np.int64)
    rsq = np.zeros(max(cap, 1))
    st = fn(ctypes.byref(params), n, r.ctypes.data, cap, iap.ctypes.data, rsq.ctypes.data,
            ctypes.byref(nip))
    assert st == 0, st
    return iap[:cap], rsq[:cap]


def derivatives(params, r, v, m, u, geometry32=False):
    """One evaluation f(x).  Returns a dict of rho, rho_lr, t, p, pco, vdot,
    udot, jq and nip.  geometry32: each pair's separation and distance
    rounded to the nearest FP32 numbers (the FP32-geometry error floor;
    the pair set is unchanged)."""
    r, v, m, u = _c(r), _c(v), _c(m), _c(u)
    n, d = r.shape
    out = {k: np.zeros(n) for k in ("rho", "rho_lr", "t", "p", "pco", "udot")}
    out["vdot"] = np.zeros((n, d))
    out["jq"] = np.zeros((n, d))
    nip = ctypes.c_int64()
    lib().orc_set_geometry32(1 if geometry32 else 0)
    try:
        st = lib().orc_derivatives(ctypes.byref(params), n, r.ctypes.data, v.ctypes.data,
                                   m.ctypes.data, u.ctypes.data, out["rho"].ctypes.data,
                                   out["rho_lr"].ctypes.data, out["t"].ctypes.data,
                                   out["p"].ctypes.data, out["pco"].ctypes.data,
                                   out["vdot"].ctypes.data, out["udot"].ctypes.data,
                                   out["jq"].ctypes.data, ctypes.byref(nip))
    finally:
        lib().orc_set_geometry32(0)
    assert st == 0, st
    out["nip"] = nip.value
    return out


def advance(params, r, v, m, u, nsteps, step0=0):
    """nsteps integrator steps; returns (r, v, u, props) with the reference's
    post-update property semantics."""
    r, v, m, u = _c(r).copy(), _c(v).copy(), _c(m), _c(u).copy()
    n, d = r.shape
    props = {k: np.zeros(n) for k in ("rho", "rho_lr", "t", "p", "pco", "udot")}
    props["vdot"] = np.zeros((n, d))
    props["jq"] = np.zeros((n, d))
    st = lib().orc_advance(ctypes.byref(params), n, r.ctypes.data, v.ctypes.data,
                           m.ctypes.data, u.ctypes.data, int(nsteps), int(step0),
                           props["rho"].ctypes.data, props["rho_lr"].ctypes.data,
                           props["t"].ctypes.data, props["p"].ctypes.data,
                           props["pco"].ctypes.data, props["vdot"].ctypes.data,
                           props["udot"].ctypes.data, props["jq"].ctypes.data)
    assert st == 0, st
    return r, v, u, props


def initial_energy(params, r, v, m, temperature):
    """u = k_B T - a rho with rho the initial short-range density
    (properties.py:44-46, 116-119)."""
    d = derivatives(params, r, v, m, np.zeros(r.shape[0]))
    return temperature * params.kbdash - params.adash * d["rho"]


def collide_pairs(mode, r, v, m, iap, drij, rij, cutoff):
    """Force.apply of a collision force over a pair list, sequentially
    (forces.py:38-42, 87-243).  Returns updated copies (r, v, drij, rij)."""
    r, v, m = _c(r).copy(), _c(v).copy(), _c(m)
    iap = _c(iap, np.int64)
    drij, rij = _c(drij).copy(), _c(rij).copy()
    n, d = v.shape
    st = lib().orc_collide_pairs(d, int(mode), n, r.ctypes.data, v.ctypes.data,
                                 m.ctypes.data, len(iap), iap.ctypes.data, drij.ctypes.data,
                                 rij.ctypes.data, float(cutoff))
    assert st == 0, st
    return r, v, drij, rij
