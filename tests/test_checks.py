"""The checking build (libsph_checks.so, -DSPH_DEBUG_CHECKS): the binning,
pair and collision kernels test every cell and particle index they derive
and report SPH_EBOUNDS instead of accessing out of range.  Ordinary
workloads -- batched, 2D and 3D, binning on demand, collisions, small
single-cell boxes, cluster pairs beside cell windows, pair lists in 2D
batches and in 3D -- run clean under it and give the release build's bits.
The library is loaded in a child process (PYTICLES_CHECKS=1)."""
import os
import subprocess
import sys

import pytest

from pyticles_gb300 import build

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import sys, numpy as np
sys.path.insert(0, ROOT)
from pyticles_gb300 import Engine, _abi, workloads
assert _abi.LIB_PATH.endswith(LIBNAME), _abi.LIB_PATH
out = []
prm, r, v, m, T0 = workloads.config_2d(48, 7001, viscosity=True)
u = workloads.vdw_energy(np.ones(len(r)), T0)
sims = [(prm, r, v, m, u)]
for k, side in enumerate((12, 20, 7)):
    p2, r2, v2, m2, T2 = workloads.lattice_system(side, 2, spacing=1.0, jitter=0.1,
        temperature=0.8, seed=7100 + k, kernel="lucy", h_short=2.0, h_long=3.0,
        viscosity=True, dt=2e-3)
    p2.collision = _abi.SPH_COLLIDE_EXCHANGE if k == 0 else 0
    p2.collision_cutoff = 0.9 if k == 0 else 0.0
    sims.append((p2, r2, v2, m2, workloads.vdw_energy(np.ones(len(r2)), T2)))
for group in ([sims[0]], sims[1:2], sims[2:]):
    with Engine(group[0][0], "mixed", max_particles=sum(len(x[1]) for x in group),
                max_sims=len(group)) as e:
        ids = [e.add(*x) for x in group if x[0].collision == group[0][0].collision]
        e.set_tuning(rebin=1, steps_per_graph=4)
        e.advance(12)
        e.sync()
        for s in ids:
            e.derivatives(s)
            e.pairs(s)
            out.append(e.get_state(s)[0].sum())
        e.sync()
p3, r3, v3, m3, T3 = workloads.config_3d(16, 7002)
with Engine(p3, "mixed", max_particles=len(r3)) as e:
    s = e.add(p3, r3, v3, m3, workloads.vdw_energy(np.full(len(r3), 0.7), T3))
    e.advance(6)
    e.sync()
    out.append(e.get_state(s)[0].sum())
# cluster pairs beside cell windows: a box too small for columns, a larger one
p5, r5, v5, m5, T5 = workloads.config_3d(12, 7004, integrator="rk4")
p4, r4, v4, m4, T4 = workloads.config_3d(20, 7003, integrator="rk4")
with Engine(p4, "mixed", max_particles=len(r5) + len(r4), max_sims=2) as e:
    ids = [e.add(p5, r5, v5, m5, workloads.vdw_energy(np.full(len(r5), 0.7), T5)),
           e.add(p4, r4, v4, m4, workloads.vdw_energy(np.full(len(r4), 0.7), T4))]
    e.set_tuning(pair_scheme=1, steps_per_graph=3)
    e.advance(6)
    e.sync()
    for s in ids:
        e.derivatives(s)
        out.append(e.get_state(s)[0].sum())
    e.sync()
# pair lists: a batch of two 2D simulations, and the 3D fluid
with Engine(sims[0][0], "mixed", max_particles=len(sims[0][1]) + len(sims[2][1]),
            max_sims=2) as e:
    ids = [e.add(*sims[0]), e.add(*sims[2])]
    e.set_tuning(pair_scheme=2, steps_per_graph=4)
    e.advance(12)
    e.sync()
    for s in ids:
        e.derivatives(s)
        out.append(e.get_state(s)[0].sum())
    e.sync()
with Engine(p3, "mixed", max_particles=len(r3)) as e:
    s = e.add(p3, r3, v3, m3, workloads.vdw_energy(np.full(len(r3), 0.7), T3))
    e.set_tuning(pair_scheme=2, steps_per_graph=3)
    e.advance(6)
    e.sync()
    out.append(e.get_state(s)[0].sum())
print(repr([float(x) for x in out]))
"""


def run_child(checks):
    env = dict(os.environ, PYTICLES_CHECKS="1" if checks else "0")
    code = CHILD.replace("ROOT", repr(ROOT)).replace(
        "LIBNAME", repr("libsph_checks.so" if checks else "libsph.so"))
    res = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True,
                         text=True, timeout=600)
    assert res.returncode == 0, res.stderr[-3000:]
    return res.stdout.strip().splitlines()[-1]


def test_checking_build_runs_clean_and_matches_release():
    build.build()
    build.build(checks=True)
    assert run_child(True) == run_child(False)
