"""Trajectories and checkpoints.

Trajectory files keep the schema of pyticles' spam_nc.py (spam_nc.py:28-170):
netCDF classic, dimensions `timestep` (unlimited), `particle`, `spatial`;
coordinate variables `timestep`, `particle`, `spatial`; per step `position`
and `velocity` (timestep, particle, spatial), `internal_energy` and `mass`
(timestep, particle); global attributes `Date`, `Creator` and the caller's.
netCDF4 is not available here, so files are written in the classic format
through scipy.io.netcdf_file, which any netCDF reader opens.

`AsyncTrajectoryWriter` copies the state out of the engine (device -> host)
and hands the file write to a background thread, so the GPU keeps stepping.

Checkpoints (`save_checkpoint` / `load_checkpoint`) hold, per simulation,
r, v, u, m, the parameters and the step count; a restored run reproduces the
uninterrupted trajectory bit for bit (every step is a function of the state
alone, and the step count fixes the thermostat schedule).
"""
import json
import queue
import threading

import numpy as np
from scipy.io import netcdf_file

from . import _abi


def create_sph_ncfile(filename, attribs, n, dim):
    """Creates an empty trajectory file (spam_nc.py:28-119)."""
    f = netcdf_file(filename, "w", version=1)
    f.Date = 1
    f.Creator = "ac"
    for name, val in attribs.items():
        setattr(f, name, val)
    f.createDimension("timestep", None)
    f.createDimension("particle", n)
    f.createDimension("spatial", dim)
    f.createVariable("timestep", "d", ("timestep",))
    part = f.createVariable("particle", "i", ("particle",))
    space = f.createVariable("spatial", "i", ("spatial",))
    part[:] = np.arange(n, dtype=np.int32)
    space[:] = np.arange(dim, dtype=np.int32)
    f.createVariable("position", "d", ("timestep", "particle", "spatial"))
    f.createVariable("velocity", "d", ("timestep", "particle", "spatial"))
    f.createVariable("internal_energy", "d", ("timestep", "particle"))
    f.createVariable("mass", "d", ("timestep", "particle"))
    f.flush()
    f.close()


def write_arrays(filename, r, v, u, m):
    """Appends one step (spam_nc.py:121-145)."""
    f = netcdf_file(filename, "a")
    i = f.variables["timestep"].shape[0]
    f.variables["timestep"][i] = i + 1
    n = r.shape[0]
    f.variables["position"][i, :n, :] = r
    f.variables["velocity"][i, :n, :] = v
    f.variables["internal_energy"][i, :n] = u
    f.variables["mass"][i, :n] = m
    f.flush()
    f.close()


def write_step(filename, p):
    """spam_nc.write_step for a particle system p (p.r, p.v, p.u, p.m, p.n)."""
    n = p.n
    write_arrays(filename, p.r[:n], p.v[:n], p.u[:n], p.m[:n])


def read_arrays(filename, step="last"):
    """(r, v, u, m) of one step (spam_nc.py:148-170 reads r, v and m)."""
    f = netcdf_file(filename, "r", mmap=False)
    nsteps = f.variables["timestep"].shape[0]
    i = nsteps - 1 if step == "last" else int(step)
    out = tuple(np.array(f.variables[k][i]) for k in
                ("position", "velocity", "internal_energy", "mass"))
    f.close()
    return out


def read_step(filename, p, step="last"):
    """spam_nc.read_step: makes step i the state of particle system p."""
    r, v, u, m = read_arrays(filename, step)
    n = p.n
    p.r[:n] = r[:n]
    p.v[:n] = v[:n]
    p.m[:n] = m[:n]


class AsyncTrajectoryWriter:
    """Writes an engine simulation's steps without stalling the GPU: the
    state is read back on the caller's thread (a device -> host copy) and
    the file write runs on a background thread."""

    def __init__(self, filename, engine, sim, mass, attribs=None):
        n = engine.counts[sim]
        create_sph_ncfile(filename, attribs or {}, n, engine.dim)
        self.filename = filename
        self.engine = engine
        self.sim = sim
        self.mass = np.asarray(mass, dtype=np.float64)
        self.q = queue.Queue(maxsize=8)
        self.err = None
        self.thread = threading.Thread(target=self._run, daemon=True)
        self.thread.start()

    def _run(self):
        while True:
            item = self.q.get()
            if item is None:
                return
            try:
                write_arrays(self.filename, *item)
            except Exception as exc:  # surfaced by close()
                self.err = exc

    def snapshot(self):
        r, v, u = self.engine.get_state(self.sim)
        self.q.put((r, v, u, self.mass))

    def close(self):
        self.q.put(None)
        self.thread.join()
        if self.err:
            raise self.err


def save_checkpoint(path, engine, sims, masses):
    """Writes every listed simulation's state, parameters and step count."""
    data = {"nsims": len(sims)}
    for k, (sim, m) in enumerate(zip(sims, masses)):
        r, v, u = engine.get_state(sim)
        prm = _abi.params_dict(engine_params(engine, sim))
        data[f"s{k}_r"], data[f"s{k}_v"], data[f"s{k}_u"] = r, v, u
        data[f"s{k}_m"] = np.asarray(m, dtype=np.float64)
        data[f"s{k}_steps"] = engine.steps(sim)
        data[f"s{k}_params"] = np.array(json.dumps(prm))
    np.savez(path, **data)


def engine_params(engine, sim):
    return engine.sim_params[sim]


def load_checkpoint(path):
    """[(params, r, v, m, u, steps), ...] from save_checkpoint."""
    d = np.load(path, allow_pickle=False)
    out = []
    for k in range(int(d["nsims"])):
        prm = json.loads(str(d[f"s{k}_params"]))
        out.append((_abi.params_from_dict(prm), d[f"s{k}_r"], d[f"s{k}_v"], d[f"s{k}_m"],
                    d[f"s{k}_u"], int(d[f"s{k}_steps"])))
    return out


def restore(engine, entries):
    """Adds checkpointed simulations to an engine; returns their ids."""
    ids = []
    for prm, r, v, m, u, steps in entries:
        sim = engine.add(prm, r, v, m, u)
        engine.set_steps(sim, steps)
        ids.append(sim)
    return ids
