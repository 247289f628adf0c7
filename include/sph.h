/*
 * sph.h -- C ABI of libsph, the sm_103a (GB300) engine for pyticles' SPH step:
 * cell-list neighbour search -> summation density (short and long smoothing
 * lengths) -> van der Waals pressure forces, artificial viscosity, heat flux
 * and energy rates -> improved-Euler (or Euler / RK4) update -> periodic box.
 *
 * Plain C types only: no torch, no CUDA types in the signatures.  Pointers
 * tagged `mem` are device pointers when mem == SPH_DEVICE (e.g. from
 * torch.Tensor.data_ptr()) and host pointers when mem == SPH_HOST; the
 * library copies host data on its own stream.  Every call returns an
 * int status (SPH_OK == 0).  The library never keeps a pointer the caller
 * passed in: state is copied into engine-owned, cell-sorted device arrays.
 *
 * Reference interfaces replaced (andrewcharles/pyticles, file:line):
 *   sph_engine_create / sph_sim_add     SmoothParticleSystem.__init__   particles.py:271-359
 *                                       SpamComplete.__init__            spam_complete_force.py:36-60
 *   sph_advance                         SmoothParticleSystem.update      particles.py:459-494
 *                                       integrator.imp_euler/euler/rk4   integrator.py:14-103
 *                                       PeriodicBox.apply                box.py:33-47
 *                                       apply_thermostat                 particles.py:450-457
 *   sph_sim_derivatives                 SpamComplete.apply               spam_complete_force.py:63-183
 *                                       (calc_sphforce3d call            spam_complete_force.py:158-165)
 *                                       properties.spam_properties       properties.py:63-120
 *                                       forces.SpamForce/CohesiveSpamForce forces.py:321-405
 *   sph_sim_pair_count / export_pairs   VerletList.build + separations   neighbour_list.py:160-189, 63-83
 *   sph_tuning.rebin, sph_rebin_count   VerletList.compress/ponder_rebuild neighbour_list.py:191-234
 *   sph_kernel_eval                     spkernel.kernel / lucy_kernel ... spkernel.py:22-153
 *   sph_collide_pairs                   CollisionForce / CollisionForce3d forces.py:87-243
 *                                       FortranCollisionForce            forces.py:454-474
 *                                       Force.apply (cutoff test)        forces.py:38-42
 */
#ifndef PYTICLES_GB300_SPH_H
#define PYTICLES_GB300_SPH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
enum sph_status {
    SPH_OK = 0,
    SPH_EINVAL = 1,          /* bad argument (size, dim, kernel, box ...)       */
    SPH_ENOMEM = 2,          /* device allocation failed or HBM budget exceeded */
    SPH_ECELL_OVERFLOW = 3,  /* a cell holds more particles than a kernel can stage */
    SPH_ETIMEOUT = 4,        /* a bounded device wait gave up                    */
    SPH_ENAN = 5,            /* a non-finite density, pressure or rate appeared  */
    SPH_ECUDA = 6,           /* a CUDA runtime call failed                       */
    SPH_ESKIN = 7,           /* a particle moved further within one step than the
                                cell slack allows (cell list would miss pairs),
                                or with pair lists further from its position
                                at the lists' build than half the skin       */
    SPH_ECAPACITY = 8,       /* engine particle / simulation capacity exceeded,
                                or a cluster or particle pair list outgrew its
                                region                                          */
    SPH_ENOTFOUND = 9,       /* unknown simulation id                           */
    SPH_EBOUNDS = 10         /* an index check failed and the access was
                                skipped: the checking build's checks, and in
                                every build the cluster pair lists' agreement
                                between counting and writing                 */
};

/* Kernel ids follow spkernel.ktable (spkernel.py:20): 1 gaussian, 2 lucy,
 * 3 debrun; 4 is the M4 cubic spline (support 2h), which pyticles lacks. */
enum sph_kernel {
    SPH_KERNEL_GAUSSIAN = 1,
    SPH_KERNEL_LUCY = 2,
    SPH_KERNEL_DEBRUN = 3,
    SPH_KERNEL_CUBIC = 4
};

/* Arithmetic of the pair passes.  SPH_FP64: everything in FP64.
 * SPH_MIXED: FP32 pair arithmetic on cell-local coordinates with
 * compensated FP32 per-particle sums; FP64 pair-set test (exact fallback
 * for borderline pairs), FP64 integrator and FP64 global reductions. */
enum sph_precision { SPH_FP64 = 0, SPH_MIXED = 1 };

/* integrator names follow particles.py:119-121 */
enum sph_integrator { SPH_EULER = 0, SPH_IEULER = 1, SPH_RK4 = 2 };

enum sph_memory { SPH_DEVICE = 0, SPH_HOST = 1 };

/* Per-simulation parameters (POD).  dim, kernel, viscosity, heat_flux and
 * integrator must agree across all simulations of one engine; the rest may
 * differ per simulation. */
typedef struct sph_params {
    int32_t dim;            /* 2 or 3                                                */
    int32_t kernel;         /* enum sph_kernel                                       */
    int32_t viscosity;      /* 1: Monaghan (1992) artificial viscosity, short h     */
    int32_t heat_flux;      /* 1: Fourier heat flux q and conduction energy rate    */
    int32_t thermostat;     /* 1: scaling thermostat after every step               */
    int32_t integrator;     /* enum sph_integrator                                   */
    int32_t collision;      /* enum sph_collision: hard-sphere velocity exchange on
                               pairs within collision_cutoff after every evaluation */
    int32_t reserved;       /* 0                                                     */
    double box[3];          /* periodic extents xmax, ymax, zmax (box.py:18-22)     */
    double h_short;         /* repulsive smoothing length  (particles.py:286, p.h)  */
    double h_long;          /* cohesive smoothing length   (particles.py:287, p.hlr)*/
    double cutoff;          /* pair set: rsq < cutoff^2 + tolerance^2               */
    double tolerance;       /*   (neighbour_list.py:153-157, 178)                   */
    double adash, bdash, kbdash;   /* van der Waals a, b, k_B (properties.py:18-20) */
    double visc_alpha;      /* Monaghan alpha (SpamComplete eta)                    */
    double visc_beta;       /* Monaghan beta  (SpamComplete zeta)                   */
    double visc_eps;        /* epsilon in mu = h v.r / (r^2 + eps h^2)              */
    double sound_speed;     /* c in the viscosity (spam_complete_force.py:142: 1)   */
    double thermalk;        /* conductivity kappa (f_properties.py:14)              */
    double dt;              /* time step                                             */
    double thermostat_temp;      /* target temperature at step 0                    */
    double thermostat_temp_end;  /* target after thermostat_ramp_steps (linear)     */
    int64_t thermostat_ramp_steps;
    double collision_cutoff;     /* pairs with rij^2 <= cutoff^2 collide (forces.py:38-42) */
} sph_params;

/* Hard collisions (forces.py:87-243, 454-474): after each derivative
 * evaluation every pair (i<j in list order) with rij^2 <= collision_cutoff^2
 * that is not separating exchanges the components of its velocities along
 * the pair axis, scaled by the mass ratio, in the pair list's order.
 * SPH_COLLIDE_EXCHANGE is CollisionForce (2D) / FortranCollisionForce
 * (collide3d restated); SPH_COLLIDE_PUSHBACK adds CollisionForce3d's
 * separation of the pair to cutoff + 0.01 (sph_collide_pairs only). */
enum sph_collision { SPH_COLLIDE_OFF = 0, SPH_COLLIDE_EXCHANGE = 1, SPH_COLLIDE_PUSHBACK = 2 };

typedef struct sph_engine sph_engine;

/* Creates an engine for up to max_particles particles in up to max_sims
 * simulations of the same dim/kernel/flags as `group`.  stream is a
 * cudaStream_t (NULL: the engine creates its own non-blocking stream).
 * Device scratch is allocated here and grown by sph_sim_add if needed. */
int sph_engine_create(sph_engine **out, const sph_params *group, int32_t precision,
                      int64_t max_particles, int32_t max_sims, void *stream);
int sph_engine_destroy(sph_engine *e);

/* Adds a simulation of n particles.  r and v are n x dim row-major
 * (the layout of ParticleSystem.r / .v), m and u have length n.
 * Positions must lie within [-box/4, 5 box/4] per axis (the teleport wrap
 * keeps them in [0, box] once stepping).  Writes its id to *sim_id. */
int sph_sim_add(sph_engine *e, const sph_params *p, int64_t n, const double *r,
                const double *v, const double *m, const double *u, int32_t mem,
                int32_t *sim_id);
int sph_sim_remove(sph_engine *e, int32_t sim_id);
/* Replaces the state of an existing simulation (same n): r, v, m and u
 * together (all NULL changes nothing; some NULL is SPH_EINVAL, and then
 * nothing is written). */
int sph_sim_set_state(sph_engine *e, int32_t sim_id, const double *r, const double *v,
                      const double *m, const double *u, int32_t mem);
/* Reads the state back in the caller's original particle order.
 * Any pointer may be NULL to skip it. */
int sph_sim_get_state(sph_engine *e, int32_t sim_id, double *r, double *v, double *u,
                      int32_t mem);
/* Reads the per-particle properties left by the last step, with the
 * reference's semantics: rho, p, pco of the step's first evaluation
 * (scatter_state restores them, particles.py:513-526) and t, rho_lr,
 * vdot, udot, jq of the last evaluation.  Any pointer may be NULL. */
int sph_sim_get_properties(sph_engine *e, int32_t sim_id, double *rho, double *rho_lr,
                           double *t, double *p, double *pco, double *vdot, double *udot,
                           double *jq, int32_t mem);
int sph_sim_count(sph_engine *e, int32_t sim_id, int64_t *n);
/* Steps a simulation has taken (the thermostat ramp position); set it when
 * resuming from a checkpoint (particles.py:110 `steps`). */
int sph_sim_steps(sph_engine *e, int32_t sim_id, int64_t *steps);
int sph_sim_set_steps(sph_engine *e, int32_t sim_id, int64_t steps);

/* Advances every simulation by nsteps steps of its integrator, applying
 * the periodic box after each step and the thermostat when enabled.
 * Asynchronous except with cluster pairs or pair lists on
 * (sph_tuning.pair_scheme 1 or 2), where
 * steps run in graph chunks of steps_per_graph steps (at most 32; a longer
 * setting is split into even chunks of about 20) and the call returns once
 * all but its last chunk finished: each chunk's longest pair list is
 * checked before the chunk after next is queued, and the lists are
 * re-measured in between when one filled its region past 80%. */
int sph_advance(sph_engine *e, int32_t nsteps);

/* One derivative evaluation f(x) of every simulation at its current state
 * (no state change), then copies simulation sim_id's results out in the
 * caller's order.  vdot and jq are n x dim.  Any pointer may be NULL. */
int sph_sim_derivatives(sph_engine *e, int32_t sim_id, double *rho, double *rho_lr,
                        double *t, double *p, double *pco, double *vdot, double *udot,
                        double *jq, int32_t mem);

/* Number of unordered pairs (i<j) in the pair set at the current state. */
int sph_sim_pair_count(sph_engine *e, int32_t sim_id, int64_t *nip);
/* Exports the pair set with NeighbourList attributes: iap (nip x 2, int64,
 * i<j, original indices), drij (nip x dim, r_j - r_i minimum-imaged), rsq
 * (nip), dv (nip x dim, v_j - v_i).  Pairs are ordered by (i, j).  cap is
 * the capacity in pairs; *nip receives the count (SPH_ECAPACITY if larger
 * than cap).  Any array pointer may be NULL. */
int sph_sim_export_pairs(sph_engine *e, int32_t sim_id, int64_t cap, int64_t *iap,
                         double *drij, double *rsq, double *dv, int64_t *nip, int32_t mem);

/* Sum over all simulations of the pair-set size (unordered pairs) of one
 * evaluation: the first evaluation of the last step, or of the last
 * derivative call (the metric's unit of work per evaluation). */
int sph_last_pair_total(sph_engine *e, int64_t *pairs);

/* The same per simulation: counts[sim_id] for sim_id < cap (0 for empty
 * slots).  No counterpart in the reference; the job server attributes
 * each job's work from it. */
int sph_last_pair_counts(sph_engine *e, int64_t *counts, int32_t cap);

/* Per-simulation diagnostics of the current state, FP64 reductions:
 * out[0] kinetic energy, out[1] internal energy, out[2..4] momentum,
 * out[5] mean temperature of the last evaluation. */
int sph_sim_diagnostics(sph_engine *e, int32_t sim_id, double out[6]);

/* Tuning knobs (chosen by the autotuner, pyticles_gb300/autotune.py). */
typedef struct sph_tuning {
    int32_t block_size;       /* threads per block of the pair passes          */
    int32_t use_graph;        /* capture each advance chunk as a CUDA graph     */
    int32_t steps_per_graph;  /* steps unrolled into one graph                  */
    int32_t rebin;            /* 0: bin the particles into cells every step.
                                 1: keep the cells of the last binning until a
                                 particle has used half of the cell slack --
                                 VerletList.compress / ponder_rebuild's skin
                                 reuse (neighbour_list.py:191-234); the pair
                                 set stays exact at every evaluation.  Improved
                                 Euler and RK4 (Euler bins every step).  The
                                 summation order then depends on when the
                                 engine last binned, so a simulation equals
                                 itself alone only to rounding             */
    double cell_ratio;        /* cell edge / (cutoff + skin): 1 -> cells of the
                                 cutoff and a 3^d window, 1/2 -> half-size cells
                                 and a 5^d window, 1/3 -> 7^d (down to 1/5);
                                 cells beyond the cutoff from a particle are
                                 skipped                                       */
    int32_t pair_scheme;      /* 0: cell windows, a particle per lane.
                                 1: cluster pairs -- clusters of 8 compact
                                 particles against listed clusters of 4, 8 x 4
                                 pairs per warp step, for each simulation of
                                 a 3D mixed-precision engine without
                                 collisions whose box spans at least five
                                 columns of about 8 particles per axis; the
                                 other simulations stay on cell windows in
                                 the same steps.  The choice and the lists
                                 (built every step) are per simulation, so a
                                 simulation gives the same bits alone or in a
                                 batch; same pair set, rounding differs from
                                 scheme 0.
                                 2: pair lists -- per particle the neighbours
                                 within the cutoff plus list_skin, built when
                                 the engine bins and kept while every particle
                                 stays within a quarter of the skin of where
                                 it was at the build (VerletList.build with
                                 its skin and ponder_rebuild,
                                 neighbour_list.py:160-234); the passes walk
                                 the lists and still apply the exact pair test
                                 at every evaluation.  Mixed-precision
                                 engines (up to 67 M particles in 2D, 8.4 M
                                 in 3D) without collisions whose boxes span at least
                                 2W+1 cells per axis (W <= 3); otherwise cell
                                 windows.  Bins on demand like rebin = 1 for
                                 improved Euler and RK4, so the summation
                                 order depends on when the engine last built;
                                 same pair set, rounding differs from
                                 scheme 0                                     */
    int32_t persistent;       /* 0: the cell-window density, heat-flux and
                                 force passes launch one thread per particle.
                                 1: each launches only the blocks the device
                                 holds at once (SMs x resident blocks), which
                                 walk the flattened particle table grid-
                                 stride: one persistent launch per pass over
                                 all simulations.  Each particle's sums are
                                 the same either way (same bits)           */
    double list_skin;         /* pair_scheme 2: the lists' skin as a fraction of
                                 the cutoff (0.01 .. 0.5; default 0.025); at
                                 least 32 dt vmax is used                     */
} sph_tuning;
int sph_get_tuning(sph_engine *e, sph_tuning *t);
int sph_set_tuning(sph_engine *e, const sph_tuning *t);

/* Binnings (counting sorts into cells) performed since the engine was
 * created: one per step with tuning.rebin == 0. */
int sph_rebin_count(sph_engine *e, int64_t *n);

/* Instantiates (and caches) the CUDA graph of tuning.steps_per_graph steps
 * for the current layout without running it, so a later sph_advance starts
 * without host-side graph construction. */
int sph_prepare(sph_engine *e);

/* Per-pass device timing with CUDA events recorded on the engine's stream,
 * also inside captured graphs (the graph is rebuilt when this toggles).
 * sph_profile(e, 1) clears the records and starts recording; after the
 * work, sph_profile_read sums the elapsed time and the launch count per
 * pass; sph_profile(e, 0) stops.  When a graph is replayed several times
 * the events hold its last replay. */
enum sph_pass {
    SPH_PASS_SORT = 0,      /* binning, scan, scatter, in-cell order, permute */
    SPH_PASS_DENSITY = 1,
    SPH_PASS_HEAT = 2,
    SPH_PASS_TSUM = 3,      /* thermostat reductions */
    SPH_PASS_FORCE = 4,     /* force + energy rate + integrator stage */
    SPH_NPASS = 5
};
int sph_profile(sph_engine *e, int32_t enable);
int sph_profile_read(sph_engine *e, double ms[5], int64_t launches[5]);
/* CUDA kernels one step launches (for launch accounting). */
int sph_kernels_per_step(sph_engine *e, int64_t *n);

/* Waits for the engine's stream; returns the first device-side error
 * (SPH_ENAN, SPH_ESKIN, ...) raised since the last call, then clears it. */
int sph_sync(sph_engine *e);
/* Per-simulation device error word (0 = ok). */
int sph_sim_status(sph_engine *e, int32_t sim_id, int32_t *status);

/* Headless splash rendering (interpolate.splash_map_2d / splash_map_3d,
 * interpolate.py:39-149; replaces the GL path of
 * SmoothParticleView.render_density, pview.py:483-519).  mode 2: particles
 * of a 2D system onto the (x, y) grid; mode 3: particles of a 3D system onto
 * the plane at height z.  r is n x r_cols row-major; m, rho, a, h have
 * length n (a may be NULL: a = rho); x (nx) and y (ny) are the regular pixel
 * coordinates; bounds = {xmin, xmax, ymin, ymax} is host memory in both
 * modes; Z receives nx x ny values, Z[ix * ny + iy].  Each particle adds
 * a m / rho W_lucy(s, h) to the pixels of its box whose minimum-imaged
 * distance s is below the cutoff.  mem tags all other pointers. */
int sph_splash_map(int32_t mode, int64_t n, const double *r, int32_t r_cols, const double *m,
                   const double *rho, const double *a, const double *h, int32_t nx, int32_t ny,
                   const double *x, const double *y, double z, const double *bounds,
                   double cutoff, double *Z, int32_t mem, void *stream);

/* The smoothing kernel of the pair passes at n distances r (spkernel.kernel,
 * gauss_kernel, lucy_kernel, debrun_kernel, lucy_w, lucy_w3d,
 * spkernel.py:22-153): w[k] = W(r[k], h) and g[k] = (dW/dr)/r, so that
 * dwdx = g (r_j - r_i) in Lucy's sign convention for every kernel (the
 * reference's Gaussian returns -g dx, spkernel.py:51).  kernel: enum
 * sph_kernel; dim 2 or 3; precision: the arithmetic of the pair passes
 * (SPH_MIXED evaluates in FP32 on FP32-rounded r).  mem tags r, w and g.
 * Runs on `stream` (NULL: the default stream) and returns once w and g are
 * written. */
int sph_kernel_eval(int32_t kernel, int32_t dim, double h, int32_t precision, int64_t n,
                    const double *r, double *w, double *g, int32_t mem, void *stream);

/* Hard collisions over a given pair list: Force.apply of CollisionForce
 * (mode SPH_COLLIDE_EXCHANGE, dim 2), FortranCollisionForce (EXCHANGE, the
 * absent collide3d restated) and CollisionForce3d (SPH_COLLIDE_PUSHBACK).
 * Pairs k = 0 .. nip-1 with rij[k]^2 <= cutoff^2 are applied in list order,
 * as the reference's sequential loop does; pairs that share no particle run
 * concurrently (dependency levels), with results identical to the
 * sequential order.  r and v (n x dim) are updated in place; with PUSHBACK
 * so are r, drij[k] (r_j - r_i, not minimum-imaged) and rij[k] of the pairs
 * that were pushed apart.  iap is nip x 2 (int64, 0-based), drij nip x dim.
 * mem tags every array pointer; returns after the work has finished. */
int sph_collide_pairs(int32_t dim, int32_t mode, int64_t n, double *r, double *v,
                      const double *m, int64_t nip, const int64_t *iap, double *drij,
                      double *rij, double cutoff, int32_t mem, void *stream);

/* ---- allocation-free evaluation (no counterpart in the reference) ------
 * One derivative evaluation of one simulation -- the passes of
 * sph_sim_derivatives -- for callers that cannot let a library allocate
 * device memory: a host application or framework that budgets the whole
 * device up front and hands out memory only from its own pool, or a
 * latency-critical loop that may not block in the allocator.  All pointers
 * are device pointers owned by the caller: r, v (n x dim), m, u (n) in;
 * rho, rho_lr, t, p, pco, udot (n) and vdot, jq (n x dim) out, in the
 * caller's particle order (any output may be NULL).  stream is a
 * cudaStream_t (NULL: the legacy default stream); the call returns after the
 * work has finished, with the device error word (SPH_ENAN) as its status.
 * It calls no cudaMalloc / cudaFree: all intermediate arrays live in one
 * file-scope static device array of SPH_NOALLOC_SCRATCH_BYTES, which every
 * GPU that loads the library holds until the process exits.  Limits:
 * n <= SPH_NOALLOC_MAX_PARTICLES (SPH_EINVAL beyond), at most
 * SPH_NOALLOC_MAX_CELLS cells (coarser cells are chosen when the box needs
 * more; SPH_ECAPACITY if even those exceed it).  The first call on a device
 * looks up the array's device address; make that first call before any
 * stream capture.  All calls share the array: calls whose work overlaps on
 * the GPU (two threads, or unordered streams) race on it. */
#define SPH_NOALLOC_MAX_PARTICLES 16384
#define SPH_NOALLOC_MAX_CELLS 16384
#define SPH_NOALLOC_SCRATCH_BYTES (16384u * 512u + 16384u * 32u + (256u << 10))
int sph_derivatives_noalloc(const sph_params *p, int32_t precision, int64_t n, const double *r,
                            const double *v, const double *m, const double *u, double *rho,
                            double *rho_lr, double *t, double *pres, double *pco, double *vdot,
                            double *udot, double *jq, void *stream);

const char *sph_status_string(int status);
int sph_version(void);

#ifdef __cplusplus
}
#endif

#endif /* PYTICLES_GB300_SPH_H */
