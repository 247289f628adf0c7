"""Writes tests/golden/floors.json: the conditioning floors of the
mixed-precision evaluation on every golden system, from the FP64 oracle
(test infrastructure) alone.

    python tests/golden/make_floors.py

Per system and quantity (rho, rho_lr, t, p, pco, vdot, udot):

  position  floor A: relative L2 change of the FP64 evaluation when the
            positions are rounded to FP32 in cell-local frames (largest over
            four random frame offsets);
  geometry  floor B: relative L2 change of the FP64 evaluation when each
            pair's separation vector and distance are the nearest FP32
            numbers, all else FP64 -- the floor of any evaluation with FP32
            pair geometry.

tests/test_gpu_parity.py holds the mixed-precision force of each system to
a fixed multiple of its floor B; tests/test_oracle_golden.py checks that
this file is what the oracle computes.
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from tests.golden_cases import (SYSTEMS, geometry_floor, load, params_of,  # noqa: E402
                                position_floor)


def floors():
    out = {}
    for name in SYSTEMS:
        g = load(name)
        prm = params_of(g)
        args = (prm, g["r0"], g["v0"], g["m"], g["u0"])
        out[name] = {"position": position_floor(*args), "geometry": geometry_floor(*args)}
    return out


def main():
    path = os.path.join(HERE, "floors.json")
    with open(path, "w") as f:
        json.dump(floors(), f, indent=1, sort_keys=True)
        f.write("\n")
    print("wrote", path)


if __name__ == "__main__":
    main()
