"""The integrator interface of pyticles (integrator.py:14-103) over the GPU
step.

euler, imp_euler and rk4 take (get_state, calc_derivs, get_derivs,
set_state, dt) as in pyticles.  Given the bound gather_state, derivatives,
gather_derivatives and scatter_state of one SmoothParticleSystem -- the
call SmoothParticleSystem.update makes (particles.py:485-486) -- each runs
its integrator's step for that system in the engine, from the host arrays
back into them.  The engine's step ends with the periodic teleport wrap,
which the reference applies after the call (particles.py:488): a second
wrap leaves wrapped positions unchanged.  The thermostat is not applied:
as in the reference, the caller does that after the call (:490-491).

Any other callables are refused: the library has no host integrator.
"""
from .particles import SmoothParticleSystem

_METHODS = ("gather_state", "derivatives", "gather_derivatives", "scatter_state")


def _system(get_state, calc_derivs, get_derivs, set_state):
    """The SmoothParticleSystem whose own methods the four callables are."""
    p = getattr(get_state, "__self__", None)
    if isinstance(p, SmoothParticleSystem):
        for name, f in zip(_METHODS, (get_state, calc_derivs, get_derivs, set_state)):
            if getattr(f, "__self__", None) is not p or \
                    getattr(f, "__func__", None) is not getattr(type(p), name):
                break
        else:
            return p
    raise NotImplementedError(
        "the GB300 engine integrates a SmoothParticleSystem: pass its gather_state, "
        "derivatives, gather_derivatives and scatter_state")


def _step(integrator, dt, fns):
    p = _system(*fns)
    saved = p.integrator
    p.integrator = integrator
    try:
        p._advance(dt, 1, thermostat=False)
    finally:
        p.integrator = saved


def euler(get_state, calc_derivs, get_derivs, set_state, dt):
    """x <- x + dt f(x) (integrator.py:14-41)."""
    _step("euler", dt, (get_state, calc_derivs, get_derivs, set_state))


def imp_euler(get_state, calc_derivs, get_derivs, set_state, dt):
    """Predictor-corrector: x <- x + dt (f(x) + f(x + dt f(x))) / 2
    (integrator.py:44-59)."""
    _step("ieuler", dt, (get_state, calc_derivs, get_derivs, set_state))


def rk4(get_state, calc_derivs, get_derivs, set_state, dt):
    """Classical fourth-order Runge-Kutta (integrator.py:62-103)."""
    _step("rk4", dt, (get_state, calc_derivs, get_derivs, set_state))
