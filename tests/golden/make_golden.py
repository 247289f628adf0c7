"""Generates the golden vectors in tests/golden/ by running the reference's
own pure-Python SPH code (andrewcharles/pyticles, Python 2 sources).

Usage (in a container that has the reference sources):

    python tests/golden/make_golden.py /root/reference

The reference cannot be imported as shipped (Python 2 print statements,
missing Fortran/Cython modules).  This script copies the pure-Python modules
it needs into a temporary directory and applies only mechanical edits:

  * `print x` statements become `print(x)`;
  * neighbour_list.py:32 `/ 2` becomes `// 2` (an int array size in Py3);
  * spkernel.lucy_w3d returns `w[0]` instead of the 1-element array `w`
    (NumPy 2 no longer assigns it into a scalar slot, interpolate.py:147);
  * stub modules replace the absent compiled ones: pairsep (Cython),
    fkernel, collision (Fortran), configuration, spam_nc (netCDF),
    neighbours (vasp) and f_properties (re-exports properties);
    eos.get_vdw_u is restated as the reference's own properties.vdw_energy
    (properties.py:44-46), fkernel's 3D Lucy kernel as spkernel.lucy_kernel's
    3D branch, neighbours.minimum_image as neighbour_list.py:105-123 on two
    axes.

The derivative evaluation composes reference functions in the order of
SpamComplete.apply (spam_complete_force.py:63-183), whose Fortran is absent:
VerletList.build (neighbour_list.py:160-189) -> NeighbourList.separations
(:63-83, minimum image) -> spkernel.lucy_kernel / gauss_kernel /
debrun_kernel per pair at h and h_lr -> spdensity.sum_density for Lucy (the
same loop for the other kernels) -> properties.vdw_temp, T clamped at 0,
properties.vdw (p from rho, pco from rho_lr) -> forces.SpamForce.apply and
forces.CohesiveSpamForce.apply.  Steps run SmoothParticleSystem.update
(particles.py:459-494) with integrator.imp_euler/euler/rk4 and
box.PeriodicBox.  2D systems run the reference's 3-column arrays with z = 0
and pass the 2-component displacement to the kernel (spkernel.py:97-98), so
the 2D normalisation applies.  Gaussian gradients are stored in the
reference's own sign (spkernel.py:51); the test flips it.
"""
import os
import re
import shutil
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from pyticles_gb300 import workloads  # noqa: E402  (seeded initial states only)

MODULES = ["spkernel.py", "spdensity.py", "properties.py", "forces.py", "neighbour_list.py",
           "integrator.py", "box.py", "controller.py", "particles.py", "interpolate.py"]

STUBS = {
    "pairsep.py": "def pairsep(nl):\n    pass\n",
    # lucy_w3d's Fortran kernel, restated as the 3D Lucy kernel (spkernel.py:86-118)
    "fkernel.py": ("import math\n"
                   "class _Kernel:\n"
                   "    @staticmethod\n"
                   "    def lucy_kernel(r, dr, h, w, dwdx):\n"
                   "        q = 105. / (math.pi * 16. * (h ** 3))\n"
                   "        w[0] = q * (1 + 3. * r / h) * ((1. - r / h)) ** 3 if r < h else 0.0\n"
                   "kernel = _Kernel()\n"),
    # the vasp `neighbours` module is absent: its minimum_image restated with
    # the rule of neighbour_list.py:105-123 on the first two axes
    "neighbours.py": ("def minimum_image(dr, xmax, ymax):\n"
                      "    if dr[0] > xmax / 2.:\n        dr[0] = dr[0] - xmax\n"
                      "    if dr[1] > ymax / 2.:\n        dr[1] = dr[1] - ymax\n"
                      "    if dr[0] < -xmax / 2.:\n        dr[0] = dr[0] + xmax\n"
                      "    if dr[1] < -ymax / 2.:\n        dr[1] = dr[1] + ymax\n"),
    "collision.py": "collision = None\n",
    "configuration.py": "",
    "spam_nc.py": "def read_step(*a, **k):\n    raise RuntimeError('netCDF4 absent')\n",
    "f_properties.py": "from properties import *\n",
    "eos.py": ("import properties\n"
               "def get_vdw_u(t, rho):\n"
               "    return properties.vdw_energy(rho, t)\n"),
}

PRINT_RE = re.compile(r"^(\s*)print(\s+(.*))?\s*$")
INLINE_PRINT_RE = re.compile(r"^(\s*if .*:\s*)print\s+(.*?)\s*$")


def py3(src):
    out = []
    for line in src.splitlines():
        mi = INLINE_PRINT_RE.match(line)
        if mi:
            out.append(f"{mi.group(1)}print({mi.group(2)})")
            continue
        m = PRINT_RE.match(line)
        if m and not line.strip().startswith("print("):
            body = m.group(3) or ""
            out.append(f"{m.group(1)}print({body})")
        else:
            out.append(line)
    return "\n".join(out) + "\n"


def shim(refdir):
    tmp = tempfile.mkdtemp(prefix="pyticles_shim_")
    for name in MODULES:
        src = open(os.path.join(refdir, name)).read()
        src = py3(src)
        if name == "spkernel.py":
            # NumPy 2 no longer assigns a 1-element array to a scalar slot
            # (interpolate.py:147 adds lucy_w3d's result into Z[x, y])
            src = src.replace("    kfc(r,dr,h,w,dwdx)\n    return w\n",
                              "    kfc(r,dr,h,w,dwdx)\n    return w[0]\n")
        if name == "neighbour_list.py":
            src = src.replace("(particle.maxn * particle.maxn) / 2 - 1",
                              "(particle.maxn * particle.maxn) // 2 - 1")
        open(os.path.join(tmp, name), "w").write(src)
    for name, body in STUBS.items():
        open(os.path.join(tmp, name), "w").write(body)
    sys.path.insert(0, tmp)
    return tmp


def load_reference(refdir):
    tmp = shim(refdir)
    import box
    import forces
    import interpolate
    import integrator
    import neighbour_list
    import particles
    import properties
    import spdensity
    import spkernel
    return tmp, dict(box=box, forces=forces, integrator=integrator, interpolate=interpolate,
                     neighbour_list=neighbour_list, particles=particles,
                     properties=properties, spdensity=spdensity, spkernel=spkernel)


KNAMES = {1: "gaussian", 2: "lucy", 3: "debrun"}


def make_complete_force(R, dim, kname):
    """SpamComplete.apply's sequence built from the reference's Python."""
    forces, nlm, spk = R["forces"], R["neighbour_list"], R["spkernel"]
    spd, props = R["spdensity"], R["properties"]
    kfun = {"lucy": spk.lucy_kernel, "gaussian": spk.gauss_kernel,
            "debrun": spk.debrun_kernel}[kname]

    def kernel_rows(nl, h, w_out, dw_out):
        for k in range(nl.nip):
            i = nl.iap[k, 0]
            w, dw = kfun(nl.rij[k], nl.drij[k, :dim], h[i])
            w_out[k] = w
            dw_out[k, :] = 0.0
            dw_out[k, :dim] = dw

    def density(p, nl, h, w):
        n, ni = p.n, nl.nip
        if kname == "lucy":
            return spd.sum_density(p.m[0:n], h[0:n], nl.iap[0:ni, :], nl.rij[0:ni],
                                   nl.drij[0:ni, :dim])
        # spdensity.sum_density's loop (spdensity.py:40-56) with this kernel
        rho = np.zeros(n)
        rho[:] = kfun(0.0, np.zeros(dim), h[0])[0]
        for k in range(ni):
            i, j = nl.iap[k]
            rho[i] += w[k] * p.m[j]
            rho[j] += w[k] * p.m[i]
        return rho

    class RefComplete(forces.Force):
        def __init__(self, p, nl):
            forces.Force.__init__(self, p, nl, cutoff=1e30)
            self.last_nip = 0

        def apply(self):
            p, nl = self.p, self.nl
            n = p.n
            nl.build()
            nlm.NeighbourList.separations(nl)
            ni = nl.nip
            self.last_nip = ni
            kernel_rows(nl, p.h, nl.wij, nl.dwij)
            kernel_rows(nl, p.hlr, nl.wij_lr, nl.dwij_lr)
            p.rho[0:n] = density(p, nl, p.h, nl.wij)
            p.rho_lr[0:n] = density(p, nl, p.hlr, nl.wij_lr)
            T = props.vdw_temp(p.rho[0:n], p.u[0:n])
            T[T < 0.0] = 0.0
            p.t[0:n] = T
            p.p[0:n] = props.vdw(p.rho[0:n], T)[0]
            p.pco[0:n] = props.vdw(p.rho_lr[0:n], T)[1]
            if kname == "gaussian":
                # gauss_kernel's gradient has the opposite sign to Lucy's
                # (spkernel.py:51 vs :112-113); forces need Lucy's convention.
                nl.dwij[0:ni] *= -1.0
                nl.dwij_lr[0:ni] *= -1.0
            forces.SpamForce(p, nl, cutoff=1e30).apply()
            forces.CohesiveSpamForce(p, nl, cutoff=1e30).apply()
            if kname == "gaussian":
                nl.dwij[0:ni] *= -1.0
                nl.dwij_lr[0:ni] *= -1.0

    return RefComplete


def build_system(R, r, v, m, u, box_len, dim, hs, hl, cutoff, tol, kname, integ="ieuler",
                 thermostat=False, t_target=1.0):
    particles, nlm, boxm = R["particles"], R["neighbour_list"], R["box"]
    n = r.shape[0]
    L = list(box_len) + [1.0] * (3 - len(box_len))
    zmax = L[2] if dim == 3 else 1.0
    sbox = boxm.PeriodicBox(xmax=L[0], ymax=L[1], zmax=zmax)
    p = particles.SmoothParticleSystem(n, d=3, maxn=n, xmax=L[0], ymax=L[1], zmax=zmax,
                                       hshort=hs, hlong=hl, integrator=integ, simbox=sbox,
                                       thermostat=thermostat, thermostat_temp=t_target)
    sbox.p = p
    p.r[:, :] = 0.0
    p.v[:, :] = 0.0
    p.r[:, :dim] = r
    p.v[:, :dim] = v
    p.m[:] = m
    p.u[:] = u
    nl = nlm.VerletList(p, cutoff=cutoff, tolerance=tol)
    p.nlists.append(nl)
    p.nl_default = nl
    force = make_complete_force(R, dim, kname)(p, nl)
    p.forces.append(force)
    return p, nl, force


def ref_initial_energy(R, r, v, m, box_len, dim, hs, hl, cutoff, tol, kname, T0):
    """u0 = vdw_energy(rho0, T0) after one density evaluation
    (properties.py:116-119, the run scripts' spam_properties call)."""
    p, nl, force = build_system(R, r, v, m, np.zeros(len(r)), box_len, dim, hs, hl, cutoff,
                                tol, kname)
    force.apply()
    return R["properties"].vdw_energy(p.rho[:len(r)].copy(), T0)


def snapshot(p, dim, n):
    return dict(rho=p.rho[:n].copy(), rho_lr=p.rho_lr[:n].copy(), t=p.t[:n].copy(),
                p=p.p[:n].copy(), pco=p.pco[:n].copy(), vdot=p.vdot[:n, :dim].copy(),
                udot=p.udot[:n].copy())


def run_case(R, name, r, v, m, box_len, dim, hs, hl, cutoff, tol, kname, T0, steps,
             integ="ieuler", dt=1e-3, thermostat=False, t_target=1.0, u=None):
    t0 = time.time()
    n = r.shape[0]
    if u is None:
        u = ref_initial_energy(R, r, v, m, box_len, dim, hs, hl, cutoff, tol, kname, T0)
    p, nl, force = build_system(R, r, v, m, u, box_len, dim, hs, hl, cutoff, tol, kname,
                                integ, thermostat, t_target)
    # one derivative evaluation at the initial state
    p.derivatives()
    ev = snapshot(p, dim, n)
    ni = nl.nip
    iap = nl.iap[:ni].copy()
    rsq = nl.rsq[:ni].copy()
    drij = nl.drij[:ni, :dim].copy()
    dv = nl.dv[:ni, :dim].copy()
    wij, dwij = nl.wij[:ni].copy(), nl.dwij[:ni, :dim].copy()
    wij_lr, dwij_lr = nl.wij_lr[:ni].copy(), nl.dwij_lr[:ni, :dim].copy()
    traj = []
    for s in range(steps):
        p.update(dt)
        traj.append((p.r[:n, :dim].copy(), p.v[:n, :dim].copy(), p.u[:n].copy()))
    after = snapshot(p, dim, n)
    out = dict(
        name=name, dim=dim, kernel=kname, box=np.array(list(box_len) + [1.0] * (3 - dim)),
        h_short=hs, h_long=hl, cutoff=cutoff, tolerance=tol, dt=dt, integrator=integ,
        thermostat=int(thermostat), thermostat_temp=t_target, T0=T0, steps=steps,
        r0=r, v0=v, m=m, u0=u, iap=iap.astype(np.int32), rsq=rsq,
        r_final=traj[-1][0] if traj else r, v_final=traj[-1][1] if traj else v,
        u_final=traj[-1][2] if traj else u,
    )
    if ni <= 10000:
        # per-pair NeighbourList attributes for the smaller systems only
        out.update(drij=drij, dv=dv, wij=wij, dwij=dwij, wij_lr=wij_lr, dwij_lr=dwij_lr)
    for k, val in ev.items():
        out["ev_" + k] = val
    for k, val in after.items():
        out["after_" + k] = val
    if traj:
        out["r_step1"], out["v_step1"], out["u_step1"] = traj[0]
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    print(f"{name}: n={n} nip={ni} steps={steps} {time.time() - t0:.1f}s -> {path}")


def trajectory_case(R, name, r, v, m, box_len, dim, hs, hl, cutoff, kname, T0, steps, every,
                    dt=1e-3, integ="ieuler"):
    """A long trajectory of SmoothParticleSystem.update (particles.py:459-494):
    the state every `every` steps and the properties after the last step."""
    t0 = time.time()
    n = r.shape[0]
    u = ref_initial_energy(R, r, v, m, box_len, dim, hs, hl, cutoff, 0.0, kname, T0)
    p, nl, force = build_system(R, r, v, m, u, box_len, dim, hs, hl, cutoff, 0.0, kname, integ)
    marks, rs, vs, us = [], [], [], []
    for s in range(1, steps + 1):
        p.update(dt)
        if s % every == 0:
            marks.append(s)
            rs.append(p.r[:n, :dim].copy())
            vs.append(p.v[:n, :dim].copy())
            us.append(p.u[:n].copy())
    after = snapshot(p, dim, n)
    out = dict(name=name, dim=dim, kernel=kname,
               box=np.array(list(box_len) + [1.0] * (3 - dim)), h_short=hs, h_long=hl,
               cutoff=cutoff, tolerance=0.0, dt=dt, integrator=integ, thermostat=0,
               thermostat_temp=1.0, T0=T0, steps=steps, r0=r, v0=v, m=m, u0=u,
               marks=np.array(marks), r_marks=np.array(rs), v_marks=np.array(vs),
               u_marks=np.array(us))
    for k, val in after.items():
        out["after_" + k] = val
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    print(f"{name}: n={n} steps={steps} {time.time() - t0:.1f}s -> {path}")


def collision_case(R, name, r, v, m, box_len, dim, hs, hl, cutoff, kname, T0, steps, coll,
                   dt=1e-3, integ="ieuler"):
    """SmoothParticleSystem.update with p.forces = [SpamComplete's sequence,
    forces.CollisionForce(p, nl, cutoff=coll)] -- the order of the run scripts
    (bspana.py:45-46, fspana.py:117-119)."""
    t0 = time.time()
    n = r.shape[0]
    u = ref_initial_energy(R, r, v, m, box_len, dim, hs, hl, cutoff, 0.0, kname, T0)
    p, nl, force = build_system(R, r, v, m, u, box_len, dim, hs, hl, cutoff, 0.0, kname, integ)
    p.forces.append(R["forces"].CollisionForce(p, nl, cutoff=coll))
    traj = []
    for s in range(steps):
        p.update(dt)
        traj.append((p.r[:n, :dim].copy(), p.v[:n, :dim].copy(), p.u[:n].copy()))
    out = dict(name=name, dim=dim, kernel=kname, box=np.array(list(box_len) + [1.0] * (3 - dim)),
               h_short=hs, h_long=hl, cutoff=cutoff, collision_cutoff=coll, dt=dt,
               integrator=integ, steps=steps, r0=r, v0=v, m=m, u0=u)
    for k, (rr, vv, uu) in enumerate(traj):
        out[f"r_step{k + 1}"], out[f"v_step{k + 1}"], out[f"u_step{k + 1}"] = rr, vv, uu
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(f"{name}: n={n} steps={steps} {time.time() - t0:.1f}s")


def collision_lists(R):
    """Force.apply of CollisionForce (2D) and CollisionForce3d (pushback) on
    a VerletList built by the reference (neighbour_list.py:160-189)."""
    particles, nlm, forces = R["particles"], R["neighbour_list"], R["forces"]
    rng = np.random.Generator(np.random.PCG64(4242))
    out = {}
    for dim, n, L, cut, coll in ((2, 150, 10.0, 1.5, 0.9), (3, 200, 5.0, 1.2, 0.75)):
        p = particles.SmoothParticleSystem(n, d=3, maxn=n, xmax=L, ymax=L, zmax=L)
        p.r[:, :] = 0.0
        p.v[:, :] = 0.0
        p.r[:, :dim] = rng.uniform(0.0, L, size=(n, dim))
        p.v[:, :dim] = rng.normal(0.0, 1.0, size=(n, dim))
        p.m[:] = rng.uniform(0.5, 2.0, size=n)
        nl = nlm.VerletList(p, cutoff=cut, tolerance=0.0)
        nl.build()
        # NeighbourList.separations (neighbour_list.py:63-83): VerletList's
        # own leaves rij to the absent Cython pairsep
        nlm.NeighbourList.separations(nl)
        ni = nl.nip
        tag = f"{dim}d"
        out[f"r_{tag}"] = p.r[:n, :dim].copy()
        out[f"v_{tag}"] = p.v[:n, :dim].copy()
        out[f"m_{tag}"] = p.m[:n].copy()
        out[f"iap_{tag}"] = nl.iap[:ni].astype(np.int64)
        out[f"drij_{tag}"] = nl.drij[:ni, :dim].copy()
        out[f"rij_{tag}"] = nl.rij[:ni].copy()
        out[f"cutoff_{tag}"] = coll
        f = (forces.CollisionForce if dim == 2 else forces.CollisionForce3d)(p, nl, cutoff=coll)
        f.apply()
        out[f"v_after_{tag}"] = p.v[:n, :dim].copy()
        out[f"r_after_{tag}"] = p.r[:n, :dim].copy()
        out[f"drij_after_{tag}"] = nl.drij[:ni, :dim].copy()
        out[f"rij_after_{tag}"] = nl.rij[:ni].copy()
    np.savez_compressed(os.path.join(HERE, "collide_lists.npz"), **out)
    print("collide_lists:", {k: v.shape for k, v in out.items() if k.startswith("iap")})


def spam_properties_case(R):
    """properties.spam_properties (properties.py:63-120) on the 3D lattice of
    lucy3d_27 with T = T0: densities, pressures, u from T."""
    particles, nlm, boxm, props = R["particles"], R["neighbour_list"], R["box"], R["properties"]
    prm, r, v, m, T0 = workloads.lattice_system(3, 3, spacing=1.1, jitter=0.1,
                                                temperature=0.6, seed=11)
    n = len(r)
    sbox = boxm.PeriodicBox(xmax=3.3, ymax=3.3, zmax=3.3)
    p = particles.SmoothParticleSystem(n, d=3, maxn=n, xmax=3.3, ymax=3.3, zmax=3.3,
                                       hshort=1.2, hlong=1.6, simbox=sbox)
    sbox.p = p
    p.r[:, :] = r
    p.v[:, :] = v
    p.m[:] = m
    p.t[:] = T0
    nl = nlm.VerletList(p, cutoff=1.6, tolerance=0.0)
    nl.build()
    nlm.NeighbourList.separations(nl)
    props.spam_properties(p, nl)
    np.savez_compressed(os.path.join(HERE, "spam_props.npz"), r=r, v=v, m=m, T0=T0,
                        box=np.array([3.3, 3.3, 3.3]), h=1.2, hlr=1.6, cutoff=1.6,
                        rho=p.rho[:n].copy(), p=p.p[:n].copy(), pco=p.pco[:n].copy(),
                        u=p.u[:n].copy(), t=p.t[:n].copy())
    print("spam_props:", n, float(p.rho[:n].mean()))


def kernel_table(R):
    spk = R["spkernel"]
    rows = []
    for kname, fn in (("lucy", spk.lucy_kernel), ("gaussian", spk.gauss_kernel),
                      ("debrun", spk.debrun_kernel)):
        kid = {"gaussian": 1, "lucy": 2, "debrun": 3}[kname]
        for dim in (1, 2, 3):
            for h in (0.7, 2.0, 3.0):
                for frac in (0.0, 0.1, 0.37, 0.5, 0.8, 0.999, 1.0, 1.3):
                    r = frac * h
                    dx = np.zeros(dim)
                    dx[0] = r
                    w, dw = fn(r, dx if dim > 1 else r, h)
                    dw = np.atleast_1d(np.asarray(dw, dtype=float))
                    g = 0.0 if (r == 0.0 or dw.size == 0) else float(dw[0]) / r
                    rows.append((kid, dim, r, h, float(w), g))
    arr = np.array(rows)
    np.savez_compressed(os.path.join(HERE, "kernels.npz"), table=arr)
    print(f"kernels: {len(rows)} rows")


def kat_nlist(R):
    """The reference's own known-answer tests (test/neighbour_list_test.py)."""
    particles, nlm = R["particles"], R["neighbour_list"]
    p = particles.ParticleSystem(3, d=3, maxn=5)
    p.r[0, :] = (0.0, 0.0, 0.0)
    p.r[1, :] = (1.0, 0.0, 0.0)
    p.r[2, :] = (0.0, 0.0, 1.0)
    nl = nlm.NeighbourList(p)
    nl.build()
    nl.separations()
    k = nl.find_pair(0, 1)
    brute_rij = float(nl.rij[k])
    nl2 = nlm.VerletList(p, cutoff=10, tolerance=2)
    nl2.build()
    nl2.compress()
    nlm.NeighbourList.separations(nl2)
    verlet_rij0 = float(nl2.rij[0])
    nl2.ponder_rebuild()
    before = bool(nl2.rebuild_list)
    p.r[0, :] = (100.0, 100.0, 100.0)
    nl2.ponder_rebuild()
    after = bool(nl2.rebuild_list)
    w0 = R["spkernel"].lucy_kernel(0.0, [0.0, 0.0, 0.0], 2.0)[0]
    box = np.array([p.box.xmax, p.box.ymax, p.box.zmax], dtype=float)
    np.savez_compressed(os.path.join(HERE, "kat.npz"), brute_rij=brute_rij,
                        verlet_rij0=verlet_rij0, rebuild_before=before,
                        rebuild_after=after, lucy_w0_h2_3d=w0, mirror_box=box,
                        positions=np.array([[0.0, 0, 0], [1.0, 0, 0], [0.0, 0, 1]]))
    print(f"kat: rij={brute_rij} verlet={verlet_rij0} rebuild {before}->{after} w0={w0}")


def pair_edge_cases(R):
    """Pair sets from VerletList.build on adversarial inputs: distances exactly
    at the cutoff, positions on 0 and L, outside the box (predictor states),
    and a skin tolerance."""
    particles, nlm = R["particles"], R["neighbour_list"]
    rng = np.random.Generator(np.random.PCG64(99))
    cases = {}
    # (a) lattice at spacing exactly cutoff/2: many pairs at rsq == cutoff^2
    side, s, L = 8, 1.5, 12.0
    g = (np.arange(side) * s)
    r = np.stack(np.meshgrid(g, g, indexing="ij"), -1).reshape(-1, 2)
    cases["exact_cut"] = (r, (L, L, 1.0), 2, 3.0, 0.0)
    # (b) random 3D with tolerance and positions slightly outside [0, L]
    r = rng.uniform(-0.05, 10.05, size=(300, 3))
    cases["tol3d"] = (r, (10.0, 10.0, 10.0), 3, 2.5, 1.0)
    # (c) particles on the box faces and corners
    r = rng.uniform(0, 9.0, size=(200, 2))
    r[:20, 0] = 0.0
    r[20:40, 0] = 9.0
    r[40:60, 1] = 9.0
    cases["faces2d"] = (r, (9.0, 9.0, 1.0), 2, 2.9, 0.0)
    out = {}
    for name, (r, L, dim, cut, tol) in cases.items():
        n = r.shape[0]
        p = particles.ParticleSystem(n, d=3, maxn=n, xmax=L[0], ymax=L[1], zmax=L[2])
        p.r[:, :] = 0.0
        p.r[:, :dim] = r
        nl = nlm.VerletList(p, cutoff=cut, tolerance=tol)
        nl.build()
        out[name + "_r"] = r
        out[name + "_box"] = np.array(L, dtype=float)
        out[name + "_dim"] = dim
        out[name + "_cutoff"] = cut
        out[name + "_tol"] = tol
        out[name + "_iap"] = nl.iap[:nl.nip].copy()
        out[name + "_rsq"] = nl.rsq[:nl.nip].copy()
        print(f"pairs {name}: n={n} nip={nl.nip}")
    np.savez_compressed(os.path.join(HERE, "pairs_edge.npz"), **out)


def splat_maps(R):
    """interpolate.splash_map_2d / splash_map_3d on golden systems."""
    ip = R["interpolate"]
    g = dict(np.load(os.path.join(HERE, "lucy2d_400.npz")))
    r, m, rho = g["r0"], g["m"], g["ev_rho"]
    a = rho.copy()
    h = np.full(len(r), 3.0)
    x = np.arange(40) * 0.5
    y = np.arange(40) * 0.5
    Z2 = ip.splash_map_2d(x, y, r, m, rho, a, h, (0.0, 20.0, 0.0, 20.0), 5.0)
    g3 = dict(np.load(os.path.join(HERE, "debrun3d_216.npz")))
    r3, m3, rho3 = g3["r0"], g3["m"], g3["ev_rho"]
    h3 = np.full(len(r3), 1.3)
    x3 = np.arange(24) * 0.25
    y3 = np.arange(24) * 0.25
    Z3 = ip.splash_map_3d(x3, y3, 3.0, r3, m3, rho3, rho3.copy(), h3, (0.0, 6.0, 0.0, 6.0), 1.5)
    np.savez_compressed(os.path.join(HERE, "splat.npz"), x=x, y=y, r=r, m=m, rho=rho, a=a, h=h,
                        Z2=Z2, x3=x3, y3=y3, r3=r3, m3=m3, rho3=rho3, h3=h3, Z3=Z3)
    print(f"splat: 2d {Z2.shape} sum={Z2.sum():.6f}  3d {Z3.shape} sum={Z3.sum():.6f}")


def main():
    if len(sys.argv) < 2:
        sys.exit("usage: make_golden.py REFERENCE_DIR [case ...]")
    refdir = sys.argv[1]
    which = set(sys.argv[2:])
    tmp, R = load_reference(refdir)
    try:
        def want(name):
            return not which or name in which

        if want("kernels"):
            kernel_table(R)
        if want("kat"):
            kat_nlist(R)
        if want("pairs"):
            pair_edge_cases(R)
        if want("splat"):
            splat_maps(R)
        if want("spam_props"):
            spam_properties_case(R)
        if want("collide_lists"):
            collision_lists(R)
        if want("collide2d_144"):
            prm, r, v, m, T0 = workloads.lattice_system(12, 2, spacing=1.0, jitter=0.1,
                                                        temperature=0.6, seed=18)
            collision_case(R, "collide2d_144", r, v, m, (12.0, 12.0), 2, 2.0, 3.0, 3.0, "lucy",
                           T0, steps=3, coll=0.95)
        if want("lucy3d_27"):
            prm, r, v, m, T0 = workloads.lattice_system(3, 3, spacing=1.1, jitter=0.1,
                                                        temperature=0.6, seed=11)
            run_case(R, "lucy3d_27", r, v, m, (3.3, 3.3, 3.3), 3, 1.2, 1.6, 1.6, 0.0, "lucy",
                     T0, steps=3)
        if want("lucy2d_400"):
            prm, r, v, m, T0 = workloads.config_2d(20, 12)
            run_case(R, "lucy2d_400", r, v, m, (20.0, 20.0), 2, 3.0, 6.0, 6.0, 0.0, "lucy",
                     T0, steps=5)
        if want("lucy2d_1024"):
            prm, r, v, m, T0 = workloads.config_2d(32, 1000)
            run_case(R, "lucy2d_1024", r, v, m, (32.0, 32.0), 2, 3.0, 6.0, 6.0, 0.0, "lucy",
                     T0, steps=2)
        if "traj2d_1024" in which:
            # the plain small configuration at its own length: the 32^2 fluid
            # of lucy2d_1024, 100 improved-Euler steps at dt = 1e-3 (no
            # viscosity: the reference has none); slow, so only on request
            prm, r, v, m, T0 = workloads.config_2d(32, 1000)
            trajectory_case(R, "traj2d_1024", r, v, m, (32.0, 32.0), 2, 3.0, 6.0, 6.0, "lucy",
                            T0, steps=100, every=20)
        if want("gauss2d_256"):
            prm, r, v, m, T0 = workloads.lattice_system(16, 2, spacing=1.0, jitter=0.1,
                                                        temperature=0.6, seed=13)
            run_case(R, "gauss2d_256", r, v, m, (16.0, 16.0), 2, 1.0, 1.5, 4.0, 0.0,
                     "gaussian", T0, steps=2)
        if want("debrun3d_216"):
            prm, r, v, m, T0 = workloads.lattice_system(6, 3, spacing=1.0, jitter=0.1,
                                                        temperature=0.6, seed=14)
            run_case(R, "debrun3d_216", r, v, m, (6.0, 6.0, 6.0), 3, 1.3, 1.9, 1.9, 0.0,
                     "debrun", T0, steps=2)
        if want("thermo2d_400"):
            prm, r, v, m, T0 = workloads.config_2d(20, 15)
            run_case(R, "thermo2d_400", r, v, m, (20.0, 20.0), 2, 3.0, 6.0, 6.0, 0.0, "lucy",
                     T0, steps=3, thermostat=True, t_target=0.4)
        if want("euler2d_144"):
            prm, r, v, m, T0 = workloads.lattice_system(12, 2, spacing=1.0, jitter=0.1,
                                                        temperature=0.6, seed=16)
            run_case(R, "euler2d_144", r, v, m, (12.0, 12.0), 2, 2.0, 3.0, 3.0, 0.0, "lucy",
                     T0, steps=3, integ="euler")
        if want("rk4_2d_144"):
            prm, r, v, m, T0 = workloads.lattice_system(12, 2, spacing=1.0, jitter=0.1,
                                                        temperature=0.6, seed=17)
            run_case(R, "rk4_2d_144", r, v, m, (12.0, 12.0), 2, 2.0, 3.0, 3.0, 0.0, "lucy",
                     T0, steps=3, integ="rk4")
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


if __name__ == "__main__":
    main()
