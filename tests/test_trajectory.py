"""Trajectory files in the schema of spam_nc.py, and checkpoint / resume."""
import numpy as np
import pytest
from scipy.io import netcdf_file

from pyticles_gb300 import trajectory


class P:
    def __init__(self, n, dim, seed):
        rng = np.random.default_rng(seed)
        self.n = n
        self.r = rng.uniform(0, 5, (n, dim))
        self.v = rng.normal(size=(n, dim))
        self.u = rng.normal(size=n)
        self.m = np.ones(n)


def test_schema_and_round_trip(tmp_path):
    fn = str(tmp_path / "traj.nc")
    trajectory.create_sph_ncfile(fn, {"system": "vdw2d"}, 50, 2)
    steps = [P(50, 2, k) for k in range(3)]
    for p in steps:
        trajectory.write_step(fn, p)
    f = netcdf_file(fn, "r", mmap=False)
    assert f.dimensions["particle"] == 50 and f.dimensions["spatial"] == 2
    assert f.dimensions["timestep"] is None
    assert f.variables["position"].shape == (3, 50, 2)
    assert f.variables["internal_energy"].shape == (3, 50)
    assert list(f.variables["timestep"][:]) == [1.0, 2.0, 3.0]
    assert f.system == b"vdw2d" and f.Creator == b"ac"
    f.close()
    r, v, u, m = trajectory.read_arrays(fn, step=1)
    assert np.array_equal(r, steps[1].r) and np.array_equal(u, steps[1].u)
    q = P(50, 2, 99)
    trajectory.read_step(fn, q)
    assert np.array_equal(q.r, steps[2].r) and np.array_equal(q.v, steps[2].v)


@pytest.mark.gpu
def test_checkpoint_resume_is_bit_identical(tmp_path):
    from oracle import oracle
    from pyticles_gb300 import Engine, workloads
    prm, r, v, m, T0 = workloads.lattice_system(24, 2, spacing=1.0, jitter=0.1,
                                                temperature=0.8, seed=31, viscosity=True,
                                                thermostat=True, thermostat_temp=0.8,
                                                thermostat_temp_end=0.4, thermostat_ramp_steps=20)
    u = oracle.initial_energy(prm, r, v, m, T0)
    with Engine(prm, "mixed", max_particles=len(r)) as e:
        s = e.add(prm, r, v, m, u)
        e.advance(12)
        e.sync()
        full = e.get_state(s)
    with Engine(prm, "mixed", max_particles=len(r)) as e:
        s = e.add(prm, r, v, m, u)
        e.advance(5)
        trajectory.save_checkpoint(str(tmp_path / "ck.npz"), e, [s], [m])
    entries = trajectory.load_checkpoint(str(tmp_path / "ck.npz"))
    assert entries[0][5] == 5
    with Engine(prm, "mixed", max_particles=len(r)) as e:
        (s,) = trajectory.restore(e, entries)
        e.advance(7)
        e.sync()
        resumed = e.get_state(s)
        assert e.steps(s) == 12
    for a, b in zip(full, resumed):
        assert np.array_equal(a, b)


@pytest.mark.gpu
def test_async_writer_records_engine_steps(tmp_path):
    from pyticles_gb300 import Engine, workloads
    prm, r, v, m, T0 = workloads.config_2d(20, 41)
    u = workloads.vdw_energy(np.ones(len(r)), T0)
    fn = str(tmp_path / "run.nc")
    with Engine(prm, "mixed", max_particles=len(r)) as e:
        s = e.add(prm, r, v, m, u)
        w = trajectory.AsyncTrajectoryWriter(fn, e, s, m, {"workload": "config1"})
        states = []
        for _ in range(3):
            e.advance(2)
            w.snapshot()
            states.append(e.get_state(s))
        w.close()
    for k, (rr, vv, uu) in enumerate(states):
        got = trajectory.read_arrays(fn, k)
        assert np.array_equal(got[0], rr) and np.array_equal(got[2], uu)
