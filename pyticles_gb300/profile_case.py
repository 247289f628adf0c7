"""Runs a few eager (non-graph) steps of a named workload, for profilers.

    python -m pyticles_gb300.profile_case --case 2d --side 1024 --steps 2
    python -m pyticles_gb300.profile_case --case 3d --side 64 --steps 2
    python -m pyticles_gb300.profile_case --case 3d --side 64 --steps 2 --pair-scheme 1

Each step launches the sort kernels, then per integrator stage k_density,
[k_heat,] k_force; with --steps 2 and one warm-up step the second step's
launches are the ones to capture (skip the first step's)."""
import argparse

import numpy as np

from . import build, workloads
from .engine import Engine


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", choices=["2d", "3d"], default="2d")
    ap.add_argument("--side", type=int, default=1024)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--precision", default="mixed")
    ap.add_argument("--pair-scheme", type=int, default=0, choices=[0, 1])
    args = ap.parse_args()
    build.build()
    if args.case == "2d":
        prm, r, v, m, T0 = workloads.config_2d(args.side, 1000, viscosity=True)
        u = workloads.vdw_energy(np.ones(len(r)), T0)
    else:
        prm, r, v, m, T0 = workloads.config_3d(args.side, 3000)
        u = workloads.vdw_energy(np.full(len(r), 0.7), T0)
    with Engine(prm, args.precision, max_particles=len(r)) as e:
        e.add(prm, r, v, m, u)
        e.set_tuning(use_graph=0, pair_scheme=args.pair_scheme)
        e.advance(args.steps)
        e.sync()
        print(f"{args.case} n={len(r)} steps={args.steps} pairs/eval={e.last_pair_total()} "
              f"tuning={e.tuning}")


if __name__ == "__main__":
    main()
