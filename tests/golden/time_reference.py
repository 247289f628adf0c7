"""Times the reference's own pure-Python SPH step (andrewcharles/pyticles,
through the same mechanical Python-3 shim as make_golden.py) on the 2D
configuration it can run: a side x side lattice (32: N = 1024, the plain
small configuration; 64: N = 4096), Lucy h = 3 / 6, improved Euler.  Prints
pair-interactions/s with the metric's counting (the unordered pairs of one
evaluation x 2 evaluations per step), single-threaded on this host, as the
measured speed of the reference path.  Its pair build is O(N^2) Python, so
larger lattices are out of reach.

Usage (in a container that has the reference sources):

    python tests/golden/time_reference.py REFERENCE_DIR [steps] [side]
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
        sys.exit("usage: time_reference.py REFERENCE_DIR [steps] [side]")
    refdir = sys.argv[1]
    steps = int(sys.argv[2]) if len(sys.argv) > 2 else 1
    side = int(sys.argv[3]) if len(sys.argv) > 3 else 32
    tmp, R = make_golden.load_reference(refdir)
    prm, r, v, m, T0 = workloads.config_2d(side, 1000)
    box = (float(side), float(side))
    u = make_golden.ref_initial_energy(R, r, v, m, box, 2, 3.0, 6.0, 6.0, 0.0, "lucy", T0)
    p, nl, force = make_golden.build_system(R, r, v, m, u, box, 2, 3.0, 6.0, 6.0, 0.0, "lucy")
    t0 = time.perf_counter()
    for _ in range(steps):
        p.update(1e-3)
    dt = time.perf_counter() - t0
    pairs = force.last_nip
    rate = pairs * 2 * steps / dt
    print(f"reference Python step, N={side * side} (2D), {steps} step(s): {dt:.1f} s, "
          f"{pairs} pairs per evaluation, {rate:.3e} pair-interactions/s "
          f"({platform.processor() or platform.machine()}, 1 thread)")


if __name__ == "__main__":
    main()
