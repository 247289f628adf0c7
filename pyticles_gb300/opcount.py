"""Algorithmic work units of the SPH step, the numerators of the rooflines.

Flops per unordered pair per derivative evaluation (add/mul/div/sqrt = 1,
fma = 2; compares and the minimum image count 0), from the formulas the
passes evaluate: density 3d + 24 (two kernels and two weighted sums), force
10d + 42 (two gradients, pressure and cohesive terms, viscosity, energy
rate); the heat flux adds 7d + 12 for q and 3d + 4 for its energy term.

Bytes per particle per force launch: every array the launch must touch, read
or written once (the HBM minimum of an unfused design); the measured DRAM
traffic of a launch (ncu) is compared against it.
"""

FLOPS_DENSITY = {2: 3 * 2 + 24, 3: 3 * 3 + 24}
FLOPS_FORCE = {2: 10 * 2 + 42, 3: 10 * 3 + 42}
FLOPS_HEAT = {2: (7 * 2 + 12) + (3 * 2 + 4), 3: (7 * 3 + 12) + (3 * 3 + 4)}


def flops_per_pair(dim, heat=False):
    """Flops of one unordered pair in one evaluation (all passes)."""
    f = FLOPS_DENSITY[dim] + FLOPS_FORCE[dim]
    return f + (FLOPS_HEAT[dim] if heat else 0)


def force_bytes_per_particle(dim, rsize, stage_final, heat=False, reuse=False):
    """Unique bytes one force launch moves per particle.

    Reads: the packed position and neighbour record (and rho in 3D, the heat
    factors with heat flux), cell and simulation ids, FP64 x0, v0, the
    evaluation velocity, u0 and m, the cell origin (next-stage packing),
    the stage-0 rates on the last stage.  Writes: the rates, then either the
    next evaluation's state (FP64 x, v, u, stage-0 rates, packed copies) or
    the final state (FP64 x, v, u, m, ids); with binning on demand (reuse) the
    last stage also writes the next step's B state and packed copies.
    """
    v4 = 4 * rsize
    reads = 2 * v4 + (rsize if dim == 3 else 0) + (v4 if heat else 0)
    reads += 8 + 3 * 8 * dim + 16
    writes = (dim + 1) * rsize                      # vdot, udot
    if stage_final:
        reads += (dim + 1) * rsize                  # stage-0 rates
        writes += 8 * (2 * dim + 2) + 8             # final x, v, u, m, ids
        if reuse:
            reads += 8 * dim                        # cell origin
            writes += 8 * (2 * dim + 1) + 2 * v4    # next B state + packed
    else:
        reads += 8 * dim                            # cell origin
        writes += (dim + 1) * rsize + 8 * (2 * dim + 1) + 2 * v4
    return reads + writes


def force_bytes_per_step_average(dim, rsize, heat=False, reuse=False, nstage=2):
    """Average over one step's force launches (the roofline numerator)."""
    first = force_bytes_per_particle(dim, rsize, False, heat)
    last = force_bytes_per_particle(dim, rsize, True, heat, reuse)
    return (first * (nstage - 1) + last) / nstage
