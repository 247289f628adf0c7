"""Python handle on libsph's engine (include/sph.h).

Arrays may be numpy (host memory, copied by the library on its stream) or
CUDA torch tensors (device memory, used in place).  Torch tensors produced
on torch's stream must be complete before the call (the methods call
torch.cuda.current_stream().synchronize() for device inputs).  Every error
status raises SphError; there is no CPU path.
"""
import ctypes

import numpy as np

from . import _abi
from ._abi import SPH_DEVICE, SPH_HOST, SphParams, SphTuning, check, lib, ptr

PRECISIONS = {"fp64": _abi.SPH_FP64, "mixed": _abi.SPH_MIXED}


def _is_torch(a):
    return a is not None and not isinstance(a, np.ndarray) and hasattr(a, "data_ptr")


def _mem(*arrays):
    dev = [_is_torch(a) and a.is_cuda for a in arrays if a is not None]
    if dev and all(dev):
        import torch
        torch.cuda.current_stream().synchronize()
        return SPH_DEVICE
    if any(dev):
        raise ValueError("mixing host and device arrays in one call")
    return SPH_HOST


def _host(a, shape=None):
    if a is None:
        return None
    if _is_torch(a):
        if a.dtype != __import__("torch").float64 or not a.is_contiguous():
            raise ValueError("device arrays must be contiguous float64")
        return a
    out = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None:
        out = out.reshape(shape)
    return out


class Engine:
    """Many simulations of one dim / kernel / flags group in one engine."""

    def __init__(self, group, precision="mixed", max_particles=1 << 20, max_sims=1,
                 stream=None):
        self._lib = lib()
        self.group = group
        self.dim = group.dim
        self.precision = PRECISIONS[precision] if isinstance(precision, str) else int(precision)
        h = ctypes.c_void_p()
        st = ctypes.c_void_p(stream) if stream else None
        check(self._lib.sph_engine_create(ctypes.byref(h), ctypes.byref(group), self.precision,
                                          int(max_particles), int(max_sims), st),
              "sph_engine_create")
        self._h = h
        self.counts = {}
        self.sim_params = {}

    # -- lifetime --
    def close(self):
        if getattr(self, "_h", None):
            self._lib.sph_engine_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- simulations --
    def add(self, params, r, v, m, u):
        n = int(r.shape[0])
        r, v, m, u = _host(r), _host(v), _host(m), _host(u)
        mem = _mem(r, v, m, u)
        sid = ctypes.c_int32()
        check(self._lib.sph_sim_add(self._h, ctypes.byref(params), n, ptr(r), ptr(v), ptr(m),
                                    ptr(u), mem, ctypes.byref(sid)), "sph_sim_add")
        self.counts[sid.value] = n
        self.sim_params[sid.value] = params
        return sid.value

    def remove(self, sim):
        check(self._lib.sph_sim_remove(self._h, int(sim)), "sph_sim_remove")
        self.counts.pop(sim, None)
        self.sim_params.pop(sim, None)

    def set_state(self, sim, r, v, m, u):
        r, v, m, u = _host(r), _host(v), _host(m), _host(u)
        mem = _mem(r, v, m, u)
        check(self._lib.sph_sim_set_state(self._h, int(sim), ptr(r), ptr(v), ptr(m), ptr(u),
                                          mem), "sph_sim_set_state")

    def get_state(self, sim, r=None, v=None, u=None):
        """Fills the given buffers (numpy or CUDA tensors); allocates numpy
        arrays when none are given.  Returns (r, v, u)."""
        n, d = self.counts[sim], self.dim
        if r is None and v is None and u is None:
            r, v, u = np.empty((n, d)), np.empty((n, d)), np.empty(n)
        mem = _mem(r, v, u)
        check(self._lib.sph_sim_get_state(self._h, int(sim), ptr(r), ptr(v), ptr(u), mem),
              "sph_sim_get_state")
        return r, v, u

    def _props(self, fn, sim, out):
        n, d = self.counts[sim], self.dim
        if out is None:
            out = {k: np.empty(n) for k in ("rho", "rho_lr", "t", "p", "pco", "udot")}
            out["vdot"] = np.empty((n, d))
            out["jq"] = np.empty((n, d))
        keys = ("rho", "rho_lr", "t", "p", "pco", "vdot", "udot", "jq")
        mem = _mem(*[out.get(k) for k in keys])
        check(fn(self._h, int(sim), *[ptr(out.get(k)) for k in keys], mem), fn.__name__)
        return out

    def derivatives(self, sim, out=None):
        """One evaluation f(x) at the current state (no state change)."""
        return self._props(self._lib.sph_sim_derivatives, sim, out)

    def properties(self, sim, out=None):
        """Per-particle properties left by the last step (reference semantics)."""
        return self._props(self._lib.sph_sim_get_properties, sim, out)

    def steps(self, sim):
        n = ctypes.c_int64()
        check(self._lib.sph_sim_steps(self._h, int(sim), ctypes.byref(n)), "sph_sim_steps")
        return n.value

    def set_steps(self, sim, steps):
        check(self._lib.sph_sim_set_steps(self._h, int(sim), int(steps)), "sph_sim_set_steps")

    def advance(self, nsteps=1):
        check(self._lib.sph_advance(self._h, int(nsteps)), "sph_advance")

    def sync(self):
        """Waits for the device; raises on a device-side error flag."""
        check(self._lib.sph_sync(self._h), "device")

    def status(self, sim):
        s = ctypes.c_int32()
        check(self._lib.sph_sim_status(self._h, int(sim), ctypes.byref(s)), "sph_sim_status")
        return s.value

    def pair_count(self, sim):
        n = ctypes.c_int64()
        check(self._lib.sph_sim_pair_count(self._h, int(sim), ctypes.byref(n)),
              "sph_sim_pair_count")
        return n.value

    def pairs(self, sim, with_geometry=True):
        """Pair set (i<j, original indices) ordered by (i, j) plus drij, rsq, dv."""
        nip = ctypes.c_int64()
        # capacity query
        st = self._lib.sph_sim_export_pairs(self._h, int(sim), 0, None, None, None, None,
                                            ctypes.byref(nip), SPH_HOST)
        if st not in (_abi.SPH_OK, _abi.SPH_ECAPACITY):
            check(st, "sph_sim_export_pairs")
        cap = nip.value
        d = self.dim
        iap = np.zeros((max(cap, 1), 2), dtype=np.int64)
        rsq = np.zeros(max(cap, 1)) if with_geometry else None
        drij = np.zeros((max(cap, 1), d)) if with_geometry else None
        dv = np.zeros((max(cap, 1), d)) if with_geometry else None
        check(self._lib.sph_sim_export_pairs(self._h, int(sim), cap, ptr(iap), ptr(drij),
                                             ptr(rsq), ptr(dv), ctypes.byref(nip), SPH_HOST),
              "sph_sim_export_pairs")
        k = nip.value
        out = {"iap": iap[:k]}
        if with_geometry:
            out.update(rsq=rsq[:k], drij=drij[:k], dv=dv[:k])
        return out

    def last_pair_total(self):
        """Unordered pairs of one evaluation (all simulations): the first
        evaluation of the last step or derivative call."""
        n = ctypes.c_int64()
        check(self._lib.sph_last_pair_total(self._h, ctypes.byref(n)), "sph_last_pair_total")
        return n.value

    def last_pair_counts(self, nslots):
        """The same per simulation slot: an int64 array of length nslots."""
        out = np.zeros(int(nslots), dtype=np.int64)
        check(self._lib.sph_last_pair_counts(self._h, out.ctypes.data_as(
            ctypes.POINTER(ctypes.c_int64)), int(nslots)), "sph_last_pair_counts")
        return out

    def diagnostics(self, sim):
        out = (ctypes.c_double * 6)()
        check(self._lib.sph_sim_diagnostics(self._h, int(sim), out), "sph_sim_diagnostics")
        return {"kinetic": out[0], "internal": out[1], "momentum": list(out[2:5]),
                "mean_t": out[5]}

    @property
    def tuning(self):
        t = SphTuning()
        check(self._lib.sph_get_tuning(self._h, ctypes.byref(t)), "sph_get_tuning")
        return {"block_size": t.block_size, "use_graph": t.use_graph,
                "steps_per_graph": t.steps_per_graph, "rebin": t.rebin,
                "cell_ratio": t.cell_ratio, "pair_scheme": t.pair_scheme,
                "persistent": t.persistent, "list_skin": t.list_skin}

    def set_tuning(self, **kw):
        """block_size, use_graph, steps_per_graph, cell_ratio, rebin (1: bin
        into cells only when a particle has used half of the cell slack,
        VerletList.ponder_rebuild's skin reuse; 0: every step),
        pair_scheme (0: cell windows; 1: cluster pairs, for 3D simulations
        in mixed precision without collisions; 2: per-particle pair lists
        with a skin, for 2D simulations in mixed precision without
        collisions), list_skin (the lists' skin as a fraction of the
        cutoff) and persistent (1: the cell-window passes as persistent
        grid-stride launches)."""
        cur = self.tuning
        cur.update(kw)
        t = SphTuning(block_size=int(cur["block_size"]), use_graph=int(cur["use_graph"]),
                      steps_per_graph=int(cur["steps_per_graph"]), rebin=int(cur["rebin"]),
                      cell_ratio=float(cur["cell_ratio"]),
                      pair_scheme=int(cur["pair_scheme"]),
                      persistent=int(cur["persistent"]),
                      list_skin=float(cur["list_skin"]))
        check(self._lib.sph_set_tuning(self._h, ctypes.byref(t)), "sph_set_tuning")

    def rebin_count(self):
        """Binnings (cell-list builds) performed so far."""
        n = ctypes.c_int64()
        check(self._lib.sph_rebin_count(self._h, ctypes.byref(n)), "sph_rebin_count")
        return n.value

    # -- launch-ready graphs and per-pass timing --
    def prepare(self):
        check(self._lib.sph_prepare(self._h), "sph_prepare")

    def profile(self, enable=True):
        check(self._lib.sph_profile(self._h, 1 if enable else 0), "sph_profile")

    def profile_read(self):
        ms = (ctypes.c_double * 5)()
        n = (ctypes.c_int64 * 5)()
        check(self._lib.sph_profile_read(self._h, ms, n), "sph_profile_read")
        return {name: {"ms": ms[k], "launches": n[k]} for k, name in enumerate(_abi.PASSES)}

    def kernels_per_step(self):
        n = ctypes.c_int64()
        check(self._lib.sph_kernels_per_step(self._h, ctypes.byref(n)), "sph_kernels_per_step")
        return n.value

