// sph_internal.h -- device data layout shared by the engine and its kernels.
//
// HBM layout (all arrays flattened over the engine's simulations):
//  * state A  (canonical, cell-sorted as of the last step):  pos[3][P], vel[3][P],
//    u[P], m[P] in FP64 SoA, plus id[P] (original index within its simulation)
//    and sim[P].  New simulations are appended unsorted at the tail.
//  * state B  (this step's start state x0 after the counting sort): same fields.
//  * evaluation arrays (B order): packed cell-local positions / velocities
//    (float4 in mixed mode, double4 in FP64 mode), FP64 raw evaluation
//    positions xe (exact pair test), ue, ve; densities, EOS outputs, packed
//    force factors, heat flux, rates and integrator accumulators.
//  * cell table: per simulation a Morton-ordered cell range; cell_start[C+1],
//    the packed integer coordinates of every cell and, per simulation, the
//    linear-cell -> Morton-rank map used to find neighbour cells.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/sph.h"

namespace sph {

// Pair-pass constants of one simulation in the arithmetic type of the
// passes, precomputed on the host so that no thread spends FP64 work (or a
// division) deriving them.  Index 0 = short smoothing length, 1 = long.
template <typename R> struct SimConst {
    R thr_lo, thr_hi;            // fast-test band around cutoff^2 + tolerance^2
    R thr_s;                     // short kernel's support^2 (grown by a margin, at
                                 // most thr_hi): beyond it W_s = grad W_s = 0
    R edge[3], L[3], hL[3];
    R edge_lo[3];                // edge - (R)edge: cell offsets as a hi/lo pair
    R ext[3];                    // half cell extent + allowed drift (culling)
    R h[2], h_lo[2], inv_h[2], inv_h_lo[2], sig[2], g0[2], g0_h2[2];
    R inv_h2[2], inv_h2_lo[2];
    R g0_pl, g0_h2_pl;           // the long kernel's g0 and g0/h^2 times the cohesive
                                 // factor pco_i/rho_l,i^2 + pco_j/rho_l,j^2 = -2a
    R hs, eps_h2, alpha_c, beta, kappa;
    // pair lists (tuning.pair_scheme 2): the build takes pairs with FP32
    // rsq <= vl_thr ((cutoff + skin)^2 grown by a margin) and files those
    // with rsq < vl_near ((short support + skin)^2, grown) as near
    R vl_thr, vl_near;
};

// Normalisation sigma of a smoothing kernel (W = sigma w(q)) in dim 2 or 3:
// Lucy and Debrun as spkernel.py:86-153, the Gaussian's 1/(h^d pi^(d/2))
// (spkernel.py:39-52), the M4 cubic spline's 10/(7 pi h^2) and 1/(pi h^3).
double kernel_sigma(int kernel, int dim, double h);

// Device constants of one smoothing length: h and 1/h as hi/lo pairs, sigma
// and the gradient factor g0 (Lucy -12 sigma/h^2, Gaussian -2/h^2 with sigma
// applied in the kernel, cubic sigma/h^2, Debrun -3 sigma).  The pair passes'
// tables and sph_kernel_eval take them from here alike.
// Gradient factor g0 of a kernel at smoothing length h (sigma applied where
// the kernel's gradient carries it): Lucy -12 sigma/h^2, Gaussian -2/h^2
// (sigma applied in the kernel), cubic sigma/h^2, Debrun -3 sigma.
inline double kernel_g0(int kernel, double h, double sig) {
    switch (kernel) {
        case SPH_KERNEL_LUCY: return -12.0 * sig / (h * h);
        case SPH_KERNEL_GAUSSIAN: return -2.0 / (h * h);
        case SPH_KERNEL_CUBIC: return sig / (h * h);
        default: return -3.0 * sig;
    }
}

template <typename R>
inline void kernel_consts(int kernel, double h, double sig, R &h_r, R &h_lo, R &inv_h,
                          R &inv_h_lo, R &sig_r, R &g0, R &g0_h2, R &inv_h2,
                          R &inv_h2_lo) {
    h_r = (R)h;
    h_lo = (R)(h - (double)h_r);
    inv_h = (R)(1.0 / h);
    inv_h_lo = (R)(1.0 / h - (double)inv_h);
    sig_r = (R)sig;
    g0 = (R)kernel_g0(kernel, h, sig);
    g0_h2 = (R)((double)g0 / (h * h));
    inv_h2 = (R)(1.0 / (h * h));
    inv_h2_lo = (R)(1.0 / (h * h) - (double)inv_h2);
}

// Per-simulation constants on the device.
struct SimDev {
    double L[3], half_L[3], inv_L[3];
    double edge[3], inv_edge[3];
    double slack_half[3];   // max displacement per axis between binning and an evaluation
    double box_half[3];     // 0.5 edge + slack_half: a particle must stay this close
                            // to its cell centre (SPH_ESKIN beyond)
    double rebin_half[3];   // 0.5 edge + slack_half / 2: past it, bin again (rebin mode)
    double vl_gate2;        // pair lists: squared displacement from the build position
                            // past which the engine builds again (skin/4)^2
    double vl_eskin2;       // ... and past which the lists may miss pairs (skin/2)^2
    int nc[3];
    int win[3];             // neighbour window: +-win cells per axis (0 on single-cell axes)
    int small_mask;         // bit a set: axis a has one cell (minimum image in the pair pass)
    int active;
    int cell_off, ncells;
    int part_off, n;        // range in B (sorted) order
    int chunk_first, nchunk;  // this simulation's reduction chunks
    int thermostat;
    double thr;             // cutoff^2 + tolerance^2 (FP64, the reference's value)
    double hs, hl;          // smoothing lengths
    double sig_s, sig_l;    // kernel normalisations
    double ws0, wl0;        // self terms W(0, h)
    double a, b, kb;        // van der Waals
    double alpha, beta, eps, c;   // Monaghan viscosity
    double kappa;           // conductivity
    double dt, hdt;         // time step and dt/2
    double inv_kb;
    double T0, T1;          // thermostat ramp ends
    long long ramp;
    int coll_on;            // hard collisions after each evaluation
    int cl_on;              // the pair passes run on cluster pairs (sph_cluster.cu);
                            // the cell-window passes skip this simulation
    int coll_win[3];        // +-cells searched for collision partners
    double coll_c2;         // collision_cutoff^2 (Force.cutoffsq, forces.py:33)
    SimConst<float> cf;
    SimConst<double> cd;
};

// Pointers of the engine buffers (device addresses), passed by value.
struct View {
    int np;                 // particles in B (sorted, active)
    int dim;
    SimDev *sims;
    // state A
    double *a_pos[3], *a_vel[3], *a_u, *a_m;
    int *a_id, *a_sim;
    // state B
    double *b_pos[3], *b_vel[3], *b_u, *b_m;
    int *b_id, *b_sim;
    // sort scratch
    int *cell_of;           // A order: global cell, -1 dropped
    int *rank;              // A order: arrival rank within cell
    int *order_tmp, *order; // B slot -> A index
    int *cell_count, *cell_start, *cell_b;  // cell_b: B order cell id
    int *morton;            // per simulation: linear cell -> Morton rank
    int *cell_xyz;          // global cell -> packed cell coordinates (11/11/10 bits)
    double *org[3];         // B order: FP64 origin of the particle's cell-local frame
    // evaluation (stage s reads *_in, its force pass writes stage s+1's *_out)
    void *pk_pos_in, *pk_vel_in;     // float4 / double4: {xl, yl, zl, m}, {vx, vy, vz, 0}
    void *pk_pos_out, *pk_vel_out;
    void *pk_f, *pk_q;               // {p/rho^2, rho, T_hi, T_lo}, {q/rho^2, rho}
    void *pk_fv;                     // force-pass view of j: 2D {vx, vy, p/rho^2, rho},
                                     // 3D {vx, vy, vz, p/rho^2} (rho from `rho`)
    double *xe_in[3], *xe_out[3];    // FP64 raw evaluation positions (exact pair test)
    double *ve_in[3], *ve_out[3];    // FP64 evaluation velocities (rdot)
    double *ue_in, *ue_out;          // FP64 evaluation internal energy
    void *rho, *rho_l, *temp, *pres, *pco;  // R arrays of the current evaluation
    void *rho0, *pres0, *pco0;              // first evaluation of the step
    void *q[3];                             // heat flux vector (jq)
    void *vdot[3], *udot;                   // rates of the current evaluation
    void *f0v[3], *f0u;                     // stage-0 rates (improved Euler)
    double *acc_r[3], *acc_v[3], *acc_u;    // RK4 accumulators
    // reductions
    double *tsum_part;      // per chunk
    int *chunk_sim, *chunk_start, *chunk_len;
    int nchunks;
    double *t_scale;        // per sim thermostat factor
    long long *steps;       // per sim steps done
    unsigned long long *pair_count;  // per sim (pairs x2 counted by gather)
    int *err;               // per sim error word
    int *err_any;
    // binning on demand (tuning.rebin): the binning kernels run only while
    // *rebin_gate != 0; with reuse set the last stage also writes B and the
    // stage-0 packed arrays for the next step and raises *rebin_gate once a
    // particle has used half of its cell slack
    int *rebin_gate;
    int reuse;
    unsigned long long *bin_count;
    // one_sim: every particle belongs to simulation `one` (a copy of
    // sims[that id]); the pair kernels then read its constants from the
    // kernel parameters instead of holding them in registers
    int one_sim;
    // persist: the pair passes launch pass_grid()'s resident blocks, which
    // walk the particles grid-stride (tuning.persistent)
    int persist;
    // pair lists (tuning.pair_scheme 2, VList): entries four to a group,
    // group row g of particle i at int4 slot g * vl_stride + i; near
    // entries from row 0 up, far ones from row vl_cap/4 - 1 down (see
    // VList); vl_cnt[i] = near | far << 16; vl_x0[i] the particle's
    // cell-local position at the build
    int vl_on;
    int vl_cap;
    long long vl_stride;
    const int *vl_ent;
    const unsigned *vl_cnt;
    float4 *vl_x0;
    SimDev one;
};

// Strided view of an n x 3 (SoA, stride 1) or n x dim (row-major, stride
// dim) FP64 array: element (slot, axis a) is p[a][slot * stride].
struct Vec3Ref {
    double *p[3];
    int stride;
};

// Colliding pairs of one evaluation in the order the reference applies
// them, and the dependency levels that let pairs without a shared particle
// run concurrently (sph_collide.cu).
struct CollideSet {
    int cap;                        // candidate capacity
    int np;                         // particle slots
    int *row_count, *row_start;     // [np + 1] per row (sequence order)
    int *scan_tmp;                  // scan blocks
    int *ci, *cj;                   // [cap] particle slots of i (first) and j
    double *dr[3];                  // [cap] r_j - r_i, minimum-imaged
    double *rij;                    // [cap] |dr| as listed
    int *src;                       // [cap] index in the caller's pair list
    int *touch_count, *touch_start, *touch_fill;  // [np + 1]
    int *touch;                     // [2 cap] candidates of each particle
    int *pred;                      // [2 cap] previous candidate on side i / j
    int *level;                     // [cap]
    int *info;                      // [4]: count, overflow, max level, solver status
};

// Cluster-pair scheme (tuning.pair_scheme = 1, sph_cluster.cu): each 3D
// simulation's particles are binned into columns (x, y) of about eight
// particles' width and thin z slabs, ordered by slab within a column and cut
// into clusters of 8 consecutive particles (padded slots at a column's end).
// Each cluster keeps its positions relative to a lattice point of its own
// (column centre, slab floor), so a cluster pair's shift is an integer
// lattice offset.  A list per i-cluster (8 particles) names the j-clusters
// (halves of 4) of the same simulation whose bounding boxes lie within the
// cutoff plus the allowed drift; a warp evaluates 8 i x 4 j pairs per list
// entry.  Lists live in fixed regions of lstride entries, built in one pass.
// Per simulation: its lattice and its ranges in the flattened column and
// fine-cell tables.
struct ClGeom {
    int ncx, ncy, nslab;          // columns per axis, slabs per column
    int rx, ry;                   // +-columns searched per axis
    int col_off, fine_off;        // first column / fine cell of the simulation
    float wx, wy, gz;             // lattice steps
    double wxd, wyd, gzd;
    float drift2[3];              // twice the allowed drift per axis (list margin)
};

struct ClusterSet {
    int on;                       // the scheme runs for this layout
    int ncol, nfine;              // columns / fine cells of all simulations
    int ncl_max, slots_max;
    int nall;                     // particle slots of the per-particle arrays
    int lstride;                  // list entries reserved per i-cluster
    const ClGeom *geom;           // [simulation slots]
    ClGeom g1;                    // an engine with one simulation: its lattice,
    int sim1;                     // and its slot, as kernel parameters
    int *colsim;                  // [ncol] simulation of each column
    int *csim;                    // [ncl_max] simulation of each cluster
    int *fcount, *fstart, *fkey, *frank, *ford, *scan_tmp;
    int *colcnt, *colcl;          // [ncol + 1]: clusters per column, prefix
    int *slot_idx, *slot_of;      // slot -> sorted index (-1 padding), inverse
    int4 *cref;                   // per cluster {kx, ky, kz, global column}
    float4 *ibox, *jbox;          // bounding boxes (lo, hi) of clusters / halves
    int *lnear, *lfar;            // [ncl_max] entries within / beyond the short
                                  // support: the near ones from the front of the
                                  // i-cluster's lstride slots, the far ones from
                                  // the back
    int2 *ent;                    // {j half | near << 31, lattice offset dx|dy<<8|dz<<16}
    int *maxfill;                 // longest list since the host last read it
    float4 *cpos, *cfv, *cf, *cq; // per slot: {x, y, z, m} local, {v, p/rho^2},
                                  // {p/rho^2, 1/rho, T_hi, T_lo}, {q/rho^2, 0}
    float *crho;
};

// ---- launch wrappers (sph_cluster.cu) ----
// Cluster build of the step (stage-0 positions) and its pair lists; with
// store false the lists are only measured (c.maxfill), not written.
void launch_cluster_build(const View &v, const ClusterSet &c, cudaStream_t s, bool store = true);
// Cluster-local packed positions of evaluation `stage` (stage > 0 also
// checks each particle's drift since the build).
void launch_cluster_pack(const View &v, const ClusterSet &c, int stage, cudaStream_t s);
void launch_cluster_density(const View &v, const ClusterSet &c, int kernel, int stage,
                            cudaStream_t s);
void launch_cluster_heat(const View &v, const ClusterSet &c, int kernel, cudaStream_t s);
void launch_cluster_force(const View &v, const ClusterSet &c, int kernel, int viscosity, int heat,
                          cudaStream_t s);
int cluster_build_kernels();

// Pair lists of the mixed-precision cell-window engine (tuning.pair_scheme
// 2, sph_vlist.cu).  An entry packs the neighbour's B-order index (the low
// vl_index_bits(D) bits: 26 in 2D, 23 in 3D) and its cell's window offset
// from the particle's cell, o + 3 in three bits per axis above it (x, y[, z]
// upward, z in the top bits).
struct VList {
    int on;
    int cap;                      // entries reserved per particle (a multiple of 4)
    long long stride;             // particle slots per group row
    int *ent;                     // [cap/4][stride][4]: four entries of one particle
                                  // per 16-byte group; near entry k at group row k/4,
                                  // slot k%4; far entry k at group row cap/4 - 1 - k/4,
                                  // slot 3 - k%4
    unsigned *cnt;                // [stride] near | far << 16
    float4 *x0;                   // [stride] cell-local position at the build
    int *maxfill;                 // longest list since the host last read it
};
__host__ __device__ constexpr int vl_index_bits(int dim) { return 32 - 3 * dim; }
__host__ __device__ constexpr int vl_index_mask(int dim) { return (1 << vl_index_bits(dim)) - 1; }
constexpr int kVlMaxWindow = 3;   // window offsets -3 .. 3

// Builds every particle's list from the binned stage-0 state (gated like
// the binning) and records the longest (maxfill, in entries of whole groups:
// the near and the far run each fill whole groups).  kVlCount only counts;
// kVlStore stores and reports a list that outgrew its rows (SPH_ECAPACITY,
// its first entries kept); kVlStoreQuiet stores without reporting (the
// engine's measuring build, which resizes the rows instead).
enum { kVlCount = 0, kVlStore = 1, kVlStoreQuiet = 2 };
void launch_vlist_build(const View &v, const VList &l, const int *gate, int mode,
                        cudaStream_t s);

// ---- launch wrappers (sph_collide.cu) ----
// Engine path: candidates of every simulation with collisions on, found
// with the cell list at the evaluation positions v.xe_in.
void launch_collide_find(const View &v, const CollideSet &c, cudaStream_t s);
// Touch lists, predecessors and dependency levels of the current set.
void launch_collide_levels(const CollideSet &c, cudaStream_t s);
// Applies the set level by level to velocities vel (and positions pos with
// push_cut > 0: CollisionForce3d's pushback).  m is indexed by slot.  With
// pk_vel non-null the packed evaluation velocities are refreshed too.
// err/err_any (may be null) receive SPH_ECAPACITY for nsims simulations on
// overflow.
void launch_collide_apply(const CollideSet &c, int dim, Vec3Ref vel, Vec3Ref pos,
                          const double *m, double push_cut, void *pk_vel, int precision,
                          int *err, int *err_any, int nsims, cudaStream_t s);
// Engine path: the integrator stage from the stored rates (collisions on;
// with cl_only, the simulations on cluster pairs alone).
void launch_integrate(const View &v, int precision, int integrator, int stage, cudaStream_t s,
                      int cl_only = 0);

// ---- launch wrappers (sph_sort.cu) ----
void launch_bin(const View &v, int np_a, cudaStream_t s);
void launch_scan(int *count, int *start, int n, int *block_tmp, cudaStream_t s,
                 const int *gate = nullptr);
void launch_scatter(const View &v, int np_a, cudaStream_t s);
void launch_cellsort(const View &v, int ncells, cudaStream_t s);
void launch_permute(const View &v, int precision, cudaStream_t s);
// A simulation's state just set in A (identity order from a_off) into its B
// slots [b0, b0 + n) of the current binning; raises *far if it needs a new
// binning (sph_sort.cu).
void launch_restage(const View &v, int precision, int a_off, int b0, int n, int *far,
                    cudaStream_t s);
void launch_load_aos(double *dst[3], const double *src, int n, int dim, cudaStream_t s);
void launch_store_aos(double *dst, double *const src[3], const int *id, int off, int n, int dim,
                      cudaStream_t s);
void launch_store_scalar(double *dst, const double *src, const int *id, int off, int n,
                         cudaStream_t s);
void launch_store_R(double *dst, const void *src, int precision, const int *id, int off, int n,
                    cudaStream_t s);
void launch_fill_int(int *dst, int val, int n, cudaStream_t s, const int *gate = nullptr);
// After a gated binning: clears the gate and counts the binning.
void launch_rebin_close(int *gate, unsigned long long *bin_count, cudaStream_t s);
void launch_iota_sim(int *id, int *sim, int sim_id, int n, cudaStream_t s);

// ---- launch wrappers (sph_pairs.cu) ----
// stage: evaluation index within the step; nstage: evaluations per step;
// mode: 0 derivative only, 1 advance.
void launch_density(const View &v, int precision, int kernel, int stage, int block,
                    cudaStream_t s);
void launch_heat(const View &v, int precision, int kernel, int block, cudaStream_t s);
void launch_force(const View &v, int precision, int kernel, int viscosity, int heat,
                  int integrator, int stage, int mode, int block, cudaStream_t s);
void launch_tsum(const View &v, int precision, int nsims, cudaStream_t s);
void launch_pair_rows(const View &v, int precision, int sim_off, int n, long long *row_count,
                      cudaStream_t s);
void launch_pair_write(const View &v, int precision, int sim_off, int n,
                       const long long *row_start, long long *iap, double *drij, double *rsq,
                       double *dv, cudaStream_t s);
void launch_scan64(long long *data, int n, cudaStream_t s);

}  // namespace sph
