"""The integrator interface of pyticles (integrator.py:14-103).

euler, imp_euler and rk4 take (get_state, calc_derivs, get_derivs,
set_state, dt) as in pyticles.

Given the bound gather_state, derivatives, gather_derivatives and
scatter_state of one SmoothParticleSystem -- the call
SmoothParticleSystem.update makes (particles.py:485-486) -- each runs its
integrator's step for that system in the GPU engine, from the host arrays
back into them.  The engine's step ends with the periodic teleport wrap,
which the reference applies after the call (particles.py:488): a second
wrap leaves wrapped positions unchanged.  The thermostat is not applied: as
in the reference, the caller does that after the call (:490-491).

Any other callables get the reference's generic scheme: the state vector
from get_state, rates from calc_derivs then get_derivs, the stage states
given back through set_state, with the stage arithmetic of integrator.py
(c = xdot dt; x = x0 + c; x0 + (c1 + c2)/2; x0 + (c1 + 2 c2 + 2 c3 + c4)/6).
That arithmetic runs on the host on the state vectors the callables
exchange; the rates are whatever calc_derivs computes (a system's
derivatives() evaluates them on the GPU).
"""
import numpy as np

from .particles import SmoothParticleSystem

_METHODS = ("gather_state", "derivatives", "gather_derivatives", "scatter_state")


def _system(get_state, calc_derivs, get_derivs, set_state):
    """The SmoothParticleSystem whose own methods the four callables are, or
    None."""
    p = getattr(get_state, "__self__", None)
    if isinstance(p, SmoothParticleSystem):
        for name, f in zip(_METHODS, (get_state, calc_derivs, get_derivs, set_state)):
            if getattr(f, "__self__", None) is not p or \
                    getattr(f, "__func__", None) is not getattr(type(p), name):
                return None
        return p
    return None


def _step(integrator, dt, fns):
    p = _system(*fns)
    if p is None:
        return False
    saved = p.integrator
    p.integrator = integrator
    try:
        p._advance(dt, 1, thermostat=False)
    finally:
        p.integrator = saved
    return True


def _rates(calc_derivs, get_derivs, dt):
    calc_derivs()
    return np.asarray(get_derivs()) * dt


def euler(get_state, calc_derivs, get_derivs, set_state, dt):
    """x <- x + dt f(x) (integrator.py:14-41)."""
    if _step("euler", dt, (get_state, calc_derivs, get_derivs, set_state)):
        return
    c = _rates(calc_derivs, get_derivs, dt)
    set_state(np.asarray(get_state()) + c)


def imp_euler(get_state, calc_derivs, get_derivs, set_state, dt):
    """Predictor-corrector: x <- x + dt (f(x) + f(x + dt f(x))) / 2
    (integrator.py:44-59)."""
    if _step("ieuler", dt, (get_state, calc_derivs, get_derivs, set_state)):
        return
    c1 = _rates(calc_derivs, get_derivs, dt)
    x0 = np.array(get_state(), copy=True)
    set_state(x0 + c1)
    c2 = _rates(calc_derivs, get_derivs, dt)
    set_state(x0 + (c1 + c2) / 2)


def rk4(get_state, calc_derivs, get_derivs, set_state, dt):
    """Classical fourth-order Runge-Kutta (integrator.py:62-103)."""
    if _step("rk4", dt, (get_state, calc_derivs, get_derivs, set_state)):
        return
    c1 = _rates(calc_derivs, get_derivs, dt)
    x0 = np.array(get_state(), copy=True)
    set_state(x0 + c1 / 2.0)
    c2 = _rates(calc_derivs, get_derivs, dt)
    set_state(x0 + c2 / 2.0)
    c3 = _rates(calc_derivs, get_derivs, dt)
    set_state(x0 + c3)
    c4 = _rates(calc_derivs, get_derivs, dt)
    set_state(x0 + (1.0 / 6.0) * (c1 + 2. * c2 + 2. * c3 + c4))
