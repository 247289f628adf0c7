"""ctypes mirror of include/sph.h and the loader of libsph.so.

The library is built in-tree by pyticles_gb300/build.py.  Loading fails
loudly: there is no CPU fallback for any entry point.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# PYTICLES_CHECKS=1 selects the checking build (device-side index checks that
# report SPH_EBOUNDS instead of accessing out of range), made by
# build.build(checks=True)
CHECKS = os.environ.get("PYTICLES_CHECKS", "0") == "1"
LIB_PATH = os.path.join(HERE, "_build", "libsph_checks.so" if CHECKS else "libsph.so")

# status codes (enum sph_status)
SPH_OK = 0
SPH_EINVAL = 1
SPH_ENOMEM = 2
SPH_ECELL_OVERFLOW = 3
SPH_ETIMEOUT = 4
SPH_ENAN = 5
SPH_ECUDA = 6
SPH_ESKIN = 7
SPH_ECAPACITY = 8
SPH_ENOTFOUND = 9
SPH_EBOUNDS = 10
PASSES = ("sort", "density", "heat", "tsum", "force")
NOALLOC_MAX_PARTICLES = 16384

STATUS_NAMES = {
    0: "SPH_OK", 1: "SPH_EINVAL", 2: "SPH_ENOMEM", 3: "SPH_ECELL_OVERFLOW",
    4: "SPH_ETIMEOUT", 5: "SPH_ENAN", 6: "SPH_ECUDA", 7: "SPH_ESKIN",
    8: "SPH_ECAPACITY", 9: "SPH_ENOTFOUND", 10: "SPH_EBOUNDS",
}

# kernel ids follow spkernel.ktable (spkernel.py:20) plus the cubic spline
KERNELS = {"gaussian": 1, "lucy": 2, "debrun": 3, "cubic": 4}
SPH_FP64 = 0
SPH_MIXED = 1
INTEGRATORS = {"euler": 0, "ieuler": 1, "rk4": 2}
SPH_DEVICE = 0
SPH_HOST = 1
# enum sph_collision
SPH_COLLIDE_OFF = 0
SPH_COLLIDE_EXCHANGE = 1
SPH_COLLIDE_PUSHBACK = 2


class SphParams(ctypes.Structure):
    """struct sph_params (include/sph.h)."""
    _fields_ = [
        ("dim", ctypes.c_int32),
        ("kernel", ctypes.c_int32),
        ("viscosity", ctypes.c_int32),
        ("heat_flux", ctypes.c_int32),
        ("thermostat", ctypes.c_int32),
        ("integrator", ctypes.c_int32),
        ("collision", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("box", ctypes.c_double * 3),
        ("h_short", ctypes.c_double),
        ("h_long", ctypes.c_double),
        ("cutoff", ctypes.c_double),
        ("tolerance", ctypes.c_double),
        ("adash", ctypes.c_double),
        ("bdash", ctypes.c_double),
        ("kbdash", ctypes.c_double),
        ("visc_alpha", ctypes.c_double),
        ("visc_beta", ctypes.c_double),
        ("visc_eps", ctypes.c_double),
        ("sound_speed", ctypes.c_double),
        ("thermalk", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("thermostat_temp", ctypes.c_double),
        ("thermostat_temp_end", ctypes.c_double),
        ("thermostat_ramp_steps", ctypes.c_int64),
        ("collision_cutoff", ctypes.c_double),
    ]


class SphTuning(ctypes.Structure):
    """struct sph_tuning (include/sph.h)."""
    _fields_ = [
        ("block_size", ctypes.c_int32),
        ("use_graph", ctypes.c_int32),
        ("steps_per_graph", ctypes.c_int32),
        ("rebin", ctypes.c_int32),
        ("cell_ratio", ctypes.c_double),
        ("pair_scheme", ctypes.c_int32),
        ("persistent", ctypes.c_int32),
        ("list_skin", ctypes.c_double),
    ]


def make_params(dim=2, kernel="lucy", box=(32.0, 32.0, 1.0), h_short=3.0, h_long=6.0,
                cutoff=None, tolerance=0.0, adash=2.0, bdash=0.5, kbdash=1.0,
                viscosity=False, visc_alpha=1.0, visc_beta=0.1, visc_eps=0.01,
                sound_speed=1.0, heat_flux=False, thermalk=1.0, dt=1e-3,
                integrator="ieuler", thermostat=False, thermostat_temp=1.0,
                thermostat_temp_end=None, thermostat_ramp_steps=0, collision_cutoff=0.0):
    """Builds an SphParams.  Defaults follow the reference: a=2, b=0.5,
    k_B=1 (properties.py:18-20), eta=1, zeta=0.1, c=1
    (spam_complete_force.py:36-46,142), thermalk=1 (f_properties.py:14).
    collision_cutoff > 0 turns on hard collisions (the velocity exchange of
    CollisionForce / FortranCollisionForce) after every evaluation."""
    p = SphParams()
    p.dim = int(dim)
    p.kernel = KERNELS[kernel] if isinstance(kernel, str) else int(kernel)
    p.viscosity = int(bool(viscosity))
    p.heat_flux = int(bool(heat_flux))
    p.thermostat = int(bool(thermostat))
    p.integrator = INTEGRATORS[integrator] if isinstance(integrator, str) else int(integrator)
    b = list(box) + [1.0] * (3 - len(box))
    for a in range(3):
        p.box[a] = float(b[a])
    p.h_short = float(h_short)
    p.h_long = float(h_long)
    if cutoff is None:
        support = 2.0 if p.kernel == KERNELS["cubic"] else 1.0
        cutoff = support * max(h_short, h_long)
    p.cutoff = float(cutoff)
    p.tolerance = float(tolerance)
    p.adash, p.bdash, p.kbdash = float(adash), float(bdash), float(kbdash)
    p.visc_alpha, p.visc_beta, p.visc_eps = float(visc_alpha), float(visc_beta), float(visc_eps)
    p.sound_speed = float(sound_speed)
    p.thermalk = float(thermalk)
    p.dt = float(dt)
    p.thermostat_temp = float(thermostat_temp)
    p.thermostat_temp_end = float(thermostat_temp if thermostat_temp_end is None
                                  else thermostat_temp_end)
    p.thermostat_ramp_steps = int(thermostat_ramp_steps)
    p.collision = SPH_COLLIDE_EXCHANGE if collision_cutoff > 0 else SPH_COLLIDE_OFF
    p.reserved = 0
    p.collision_cutoff = float(collision_cutoff)
    return p


def params_dict(p):
    """SphParams -> plain dict (for logs and fixtures)."""
    out = {}
    for name, _ in SphParams._fields_:
        val = getattr(p, name)
        out[name] = list(val) if name == "box" else val
    return out


def params_from_dict(d):
    p = SphParams()
    for name, _ in SphParams._fields_:
        if name == "box":
            for a in range(3):
                p.box[a] = float(d["box"][a])
        elif name in d:
            setattr(p, name, d[name])
    return p


class SphError(RuntimeError):
    def __init__(self, status, where=""):
        self.status = status
        super().__init__(f"{where}: {STATUS_NAMES.get(status, status)}")


_lib = None


def _declare(lib):
    c_i32, c_i64, vp = ctypes.c_int32, ctypes.c_int64, ctypes.c_void_p
    P = ctypes.POINTER
    sig = {
        "sph_engine_create": [P(vp), P(SphParams), c_i32, c_i64, c_i32, vp],
        "sph_engine_destroy": [vp],
        "sph_sim_add": [vp, P(SphParams), c_i64, vp, vp, vp, vp, c_i32, P(c_i32)],
        "sph_sim_remove": [vp, c_i32],
        "sph_sim_set_state": [vp, c_i32, vp, vp, vp, vp, c_i32],
        "sph_sim_get_state": [vp, c_i32, vp, vp, vp, c_i32],
        "sph_sim_get_properties": [vp, c_i32, vp, vp, vp, vp, vp, vp, vp, vp, c_i32],
        "sph_sim_count": [vp, c_i32, P(c_i64)],
        "sph_sim_steps": [vp, c_i32, P(c_i64)],
        "sph_sim_set_steps": [vp, c_i32, c_i64],
        "sph_advance": [vp, c_i32],
        "sph_sim_derivatives": [vp, c_i32, vp, vp, vp, vp, vp, vp, vp, vp, c_i32],
        "sph_sim_pair_count": [vp, c_i32, P(c_i64)],
        "sph_sim_export_pairs": [vp, c_i32, c_i64, vp, vp, vp, vp, P(c_i64), c_i32],
        "sph_last_pair_total": [vp, P(c_i64)],
        "sph_last_pair_counts": [vp, P(c_i64), c_i32],
        "sph_sim_diagnostics": [vp, c_i32, P(ctypes.c_double)],
        "sph_get_tuning": [vp, P(SphTuning)],
        "sph_set_tuning": [vp, P(SphTuning)],
        "sph_prepare": [vp],
        "sph_rebin_count": [vp, P(c_i64)],
        "sph_profile": [vp, c_i32],
        "sph_profile_read": [vp, P(ctypes.c_double), P(c_i64)],
        "sph_kernels_per_step": [vp, P(c_i64)],
        "sph_sync": [vp],
        "sph_sim_status": [vp, c_i32, P(c_i32)],
        "sph_derivatives_noalloc": [P(SphParams), c_i32, c_i64] + [vp] * 13,
        "sph_splash_map": [c_i32, c_i64, vp, c_i32, vp, vp, vp, vp, c_i32, c_i32, vp, vp,
                           ctypes.c_double, vp, ctypes.c_double, vp, c_i32, vp],
        "sph_kernel_eval": [c_i32, c_i32, ctypes.c_double, c_i32, c_i64, vp, vp, vp, c_i32, vp],
        "sph_collide_pairs": [c_i32, c_i32, c_i64, vp, vp, vp, c_i64, vp, vp, vp,
                              ctypes.c_double, c_i32, vp],
        "sph_status_string": [ctypes.c_int],
        "sph_version": [],
    }
    for name, args in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    lib.sph_status_string.restype = ctypes.c_char_p
    return lib


def exported_symbols():
    """Names of every entry point declared in include/sph.h."""
    return ["sph_engine_create", "sph_engine_destroy", "sph_sim_add", "sph_sim_remove",
            "sph_sim_set_state", "sph_sim_get_state", "sph_sim_get_properties",
            "sph_sim_count", "sph_sim_steps", "sph_sim_set_steps", "sph_advance", "sph_sim_derivatives", "sph_sim_pair_count",
            "sph_sim_export_pairs", "sph_last_pair_total", "sph_last_pair_counts",
            "sph_sim_diagnostics",
            "sph_get_tuning", "sph_set_tuning", "sph_rebin_count", "sph_prepare", "sph_profile",
            "sph_profile_read", "sph_kernels_per_step", "sph_sync", "sph_sim_status",
            "sph_splash_map", "sph_kernel_eval", "sph_collide_pairs", "sph_derivatives_noalloc",
            "sph_status_string", "sph_version"]


def lib():
    """Loads libsph.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"libsph.so not built at {LIB_PATH}; run pyticles_gb300.build.build() "
                "(the CUDA engine has no CPU fallback)")
        _lib = _declare(ctypes.CDLL(LIB_PATH))
    return _lib


def check(status, where=""):
    if status != SPH_OK:
        raise SphError(status, where)


def ptr(a):
    """Address of a numpy array / torch tensor (or None -> NULL)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()
