"""Times the reference's own pure-Python SPH step (andrewcharles/pyticles,
through the same mechanical Python-3 shim as make_golden.py) on the 2D
configuration it can run: a 32 x 32 lattice (N = 1024), Lucy h = 3 / 6,
improved Euler.  Prints pair-interactions/s with the metric's counting (the
unordered pairs of one evaluation x 2 evaluations per step), single-threaded
on this host, as the measured speed of the reference path.

Usage (in a container that has the reference sources):

    python tests/golden/time_reference.py /root/reference [steps]
"""
import os
import platform
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import make_golden  # noqa: E402
from pyticles_gb300 import workloads  # noqa: E402


def main():
    if len(sys.argv) < 2:
        sys.exit("usage: time_reference.py REFERENCE_DIR [steps]")
    refdir = sys.argv[1]
    steps = int(sys.argv[2]) if len(sys.argv) > 2 else 1
    tmp, R = make_golden.load_reference(refdir)
    prm, r, v, m, T0 = workloads.config_2d(32, 1000)
    u = make_golden.ref_initial_energy(R, r, v, m, (32.0, 32.0), 2, 3.0, 6.0, 6.0, 0.0, "lucy",
                                       T0)
    p, nl, force = make_golden.build_system(R, r, v, m, u, (32.0, 32.0), 2, 3.0, 6.0, 6.0, 0.0,
                                            "lucy")
    t0 = time.perf_counter()
    for _ in range(steps):
        p.update(1e-3)
    dt = time.perf_counter() - t0
    pairs = force.last_nip
    rate = pairs * 2 * steps / dt
    print(f"reference Python step, N=1024 (2D), {steps} step(s): {dt:.1f} s, "
          f"{pairs} pairs per evaluation, {rate:.3e} pair-interactions/s "
          f"({platform.processor() or platform.machine()}, 1 thread)")


if __name__ == "__main__":
    main()
