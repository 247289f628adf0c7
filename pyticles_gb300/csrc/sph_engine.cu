// sph_engine.cu -- host side of libsph: the engine object behind the C ABI
// declared in include/sph.h.
//
// One engine holds many simulations of the same dim / kernel / flags in
// flattened device arrays.  A step is: counting-sort binning of every
// simulation's particles into its own Morton-ordered cell range (one global
// cell table), then per integrator stage a density pass, an optional heat
// pass and a force pass whose epilogue writes the next stage's state (or the
// final state with the periodic wrap and thermostat).  The step is captured
// once as a CUDA graph and replayed; the graph is rebuilt when simulations
// join or leave.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "sph_internal.h"

using namespace sph;

namespace {

#define CK(call)                                                   \
    do {                                                           \
        cudaError_t _e = (call);                                   \
        if (_e != cudaSuccess) {                                   \
            fprintf(stderr, "libsph: %s failed: %s (%s:%d)\n", #call, \
                    cudaGetErrorString(_e), __FILE__, __LINE__);   \
            return SPH_ECUDA;                                      \
        }                                                          \
    } while (0)

#define TRY(call)                 \
    do {                          \
        int _st = (call);         \
        if (_st != SPH_OK) return _st; \
    } while (0)

struct Sim {
    sph_params prm;
    int64_t n = 0;
    bool active = false;
    int nc[3] = {1, 1, 1};
    int win[3] = {0, 0, 0};
    double edge[3] = {1, 1, 1};
    int ncells = 0;
    std::vector<int> morton;   // linear cell -> Morton rank
    std::vector<int> rank_lin; // Morton rank -> linear cell
    int cell_off = 0;
    int part_off = 0;          // B layout
    int a_off = 0;             // contiguous range in A
    int chunk_first = 0, nchunk = 0;
    int64_t steps = 0;
    double vmax = 0.0;
    double vl_skin = 0.0;      // pair lists: skin (absolute) the grid leaves room for
};

template <typename T>
int dalloc(T **p, size_t n) {
    *p = nullptr;
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void **)p, n * sizeof(T));
    if (e != cudaSuccess) {
        cudaGetLastError();
        return SPH_ENOMEM;
    }
    return SPH_OK;
}

}  // namespace

struct sph_engine {
    sph_params group;
    int precision = SPH_MIXED;
    int dim = 2, nstage = 2;
    size_t rsize = 4, v4size = 16;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int64_t cap_p = 0;
    int cap_s = 0;
    int64_t cap_c = 0;
    int64_t cap_chunks = 0;
    sph_tuning tune;

    std::vector<Sim> sims;        // indexed by id (device slot)
    bool layout_dirty = true;
    int np_b = 0;                 // particles in the current B layout
    int a_extent = 0;             // used extent of A
    int ncells_total = 0;
    int nchunks = 0;
    bool any_thermostat = false;

    // device buffers
    double *a_pos[3] = {}, *a_vel[3] = {}, *a_u = nullptr, *a_m = nullptr;
    int *a_id = nullptr, *a_sim = nullptr;
    double *b_pos[3] = {}, *b_vel[3] = {}, *b_u = nullptr, *b_m = nullptr;
    int *b_id = nullptr, *b_sim = nullptr;
    int *cell_of = nullptr, *rank = nullptr, *order_tmp = nullptr, *order = nullptr;
    int *cell_b = nullptr;
    int *cell_count = nullptr, *cell_start = nullptr, *morton = nullptr;
    int *cell_xyz = nullptr;
    double *org[3] = {};
    int *scan_tmp = nullptr;
    void *pk_pos[2] = {}, *pk_vel[2] = {}, *pk_f = nullptr, *pk_q = nullptr, *pk_fv = nullptr;
    double *xe[2][3] = {}, *ve[3] = {}, *ue = nullptr;
    void *rho = nullptr, *rho_l = nullptr, *temp = nullptr, *pres = nullptr, *pco = nullptr;
    void *rho0 = nullptr, *pres0 = nullptr, *pco0 = nullptr;
    void *q[3] = {}, *vdot[3] = {}, *udot = nullptr, *f0v[3] = {}, *f0u = nullptr;
    double *acc_r[3] = {}, *acc_v[3] = {}, *acc_u = nullptr;
    double *stage_buf = nullptr;  // host transfers: two AoS regions (3 cap_p each), two
                                  // components (cap_p each), so that one call's
                                  // copies need no wait between them
    SimDev *sims_d = nullptr;
    double *t_scale = nullptr, *tsum_part = nullptr;
    long long *steps_d = nullptr;
    unsigned long long *pair_count = nullptr;
    int *err = nullptr, *err_any = nullptr;
    int *chunk_sim = nullptr, *chunk_start = nullptr, *chunk_len = nullptr;
    CollideSet coll = {};          // hard-collision candidates (group.collision)
    int *rebin_gate = nullptr;     // tuning.rebin: bin before the next step
    int *restage_far = nullptr;    // set_state kept the binning unless raised
    unsigned long long *bin_count = nullptr;
    bool bins_valid = false;       // B, its packed copies and the cells match A
    bool one_sim = false;          // exactly one live simulation (one_dev)
    int n_cell_sims = 0;           // live simulations on the cell-window passes
    bool cl_disabled = false;      // cluster lists did not fit: cell passes only
    SimDev one_dev;
    ClusterSet cl = {};            // tuning.pair_scheme = 1 (sph_cluster.cu)
    ClGeom *cl_geom_d = nullptr;   // per simulation slot
    int cl_geom_cap = 0;
    int64_t cl_np = 0, cl_fine = 0, cl_col = 0, cl_ncl = 0;  // allocated sizes
    long long cl_ent = 0;
    int cl_need = 0;               // list entries per i-cluster last measured (x margin)
    bool cl_stale = true;          // the state changed since the lists were measured
    int *cl_fill_host = nullptr;   // pinned: longest list of the last advance
    cudaEvent_t cl_fill_ev = nullptr;
    bool cl_fill_pending = false;
    VList vl = {};                 // tuning.pair_scheme = 2 (sph_vlist.cu)
    bool vl_disabled = false;      // the pair lists did not fit: cell windows
    long long vl_alloc = 0;        // entries allocated in vl.ent

    // profiling: event pairs recorded around each pass
    bool prof_on = false;
    std::vector<cudaEvent_t> prof_pool;
    size_t prof_used = 0;
    struct ProfRec { int kind; cudaEvent_t a, b; };
    std::vector<ProfRec> prof_recs;

    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    int graph_steps = 0;
    bool graph_launched = false;   // its event slots hold a launch's profile
    bool props_valid = false;
};

namespace {

int nstage_of(int integ) { return integ == SPH_EULER ? 1 : (integ == SPH_RK4 ? 4 : 2); }

double kernel_w0(int kernel, int dim, double h) {
    double sig = kernel_sigma(kernel, dim, h);
    switch (kernel) {
        case SPH_KERNEL_DEBRUN: return sig * h * h * h;
        default: return sig;  // Lucy, Gaussian, cubic spline: W(0) = sigma
    }
}

uint64_t part1by1(uint64_t x) {
    x &= 0xffffffffull;
    x = (x | (x << 16)) & 0x0000ffff0000ffffull;
    x = (x | (x << 8)) & 0x00ff00ff00ff00ffull;
    x = (x | (x << 4)) & 0x0f0f0f0f0f0f0f0full;
    x = (x | (x << 2)) & 0x3333333333333333ull;
    x = (x | (x << 1)) & 0x5555555555555555ull;
    return x;
}

uint64_t part1by2(uint64_t x) {
    x &= 0x1fffffull;
    x = (x | (x << 32)) & 0x1f00000000ffffull;
    x = (x | (x << 16)) & 0x1f0000ff0000ffull;
    x = (x | (x << 8)) & 0x100f00f00f00f00full;
    x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

int validate_params(const sph_engine *e, const sph_params *p) {
    if (p->dim != e->dim || p->kernel != e->group.kernel || p->viscosity != e->group.viscosity ||
        p->heat_flux != e->group.heat_flux || p->integrator != e->group.integrator ||
        p->collision != e->group.collision)
        return SPH_EINVAL;
    if (p->collision != SPH_COLLIDE_OFF) {
        // the engine runs the velocity exchange; a collision range beyond the
        // pair set would need pairs the cell list does not visit
        if (p->collision != SPH_COLLIDE_EXCHANGE || !(p->collision_cutoff > 0) ||
            p->collision_cutoff * p->collision_cutoff >
                p->cutoff * p->cutoff + p->tolerance * p->tolerance)
            return SPH_EINVAL;
    }
    for (int a = 0; a < p->dim; ++a)
        if (!(p->box[a] > 0.0) || !std::isfinite(p->box[a])) return SPH_EINVAL;
    if (!(p->h_short > 0) || !(p->h_long > 0) || !(p->cutoff > 0) || p->tolerance < 0)
        return SPH_EINVAL;
    if (!(p->kbdash > 0) || !(p->dt > 0)) return SPH_EINVAL;
    return SPH_OK;
}

// Cell grid of one simulation.  reach = cutoff + 8 dt vmax: the cutoff plus
// room for the largest displacement between binning and an evaluation of
// the step (checked on the device, SPH_ESKIN); with pair lists (list_skin =
// the tuning's skin as a fraction of the cutoff, 0 otherwise) cutoff + skin,
// the skin at least 32 dt vmax.  Cells are r * reach wide
// (r = tuning.cell_ratio) and the pair passes scan +-W cells per axis with
// W = ceil(1/r) for r < 1 (1 otherwise), culling cells beyond the cutoff.
// An axis with fewer than 2W+1 cells becomes a single cell (the passes then
// apply the minimum image on it).
void make_grid(Sim &S, int dim, double ratio, double list_skin = 0.0) {
    double rc = std::sqrt(S.prm.cutoff * S.prm.cutoff + S.prm.tolerance * S.prm.tolerance);
    S.vl_skin = list_skin > 0.0 ? std::max(list_skin * rc, 32.0 * S.prm.dt * S.vmax) : 0.0;
    double reach = rc + std::max(8.0 * S.prm.dt * S.vmax, S.vl_skin);
    // cells of ratio x reach; the window spans the W = ceil(1/ratio) cells
    // per side that cover the reach (1/2 -> 2, 1/3 -> 3, 0.6 -> 2 with room
    // to spare)
    int W = ratio < 1.0 ? std::max(1, (int)std::ceil(1.0 / ratio - 1e-9)) : 1;
    double need = reach * ratio * (1.0 + 1e-9);
    S.ncells = 1;
    for (int a = 0; a < 3; ++a) {
        S.win[a] = 0;
        if (a >= dim) {
            S.nc[a] = 1;
            S.edge[a] = 1.0;
            continue;
        }
        int nc = (int)std::floor(S.prm.box[a] / need);
        if (nc < 2 * W + 1) {
            nc = 1;
        } else {
            if (nc > (a < 2 ? 2047 : 1023)) nc = (a < 2 ? 2047 : 1023);  // packed coordinates
            S.win[a] = W;
        }
        S.nc[a] = nc;
    }
    // A sparse simulation in a large box gets coarser cells: at most 8 cells
    // per particle (at least 2^16, at most 2^24 cells), so the cell table
    // stays proportional to the particles.  Larger cells keep the +-W window
    // covering the reach.
    const int64_t limit =
        std::min<int64_t>(int64_t(1) << 24, std::max<int64_t>(int64_t(1) << 16, 8 * S.n));
    for (;;) {
        int64_t total = int64_t(S.nc[0]) * S.nc[1] * S.nc[2];
        if (total <= limit) break;
        int a = 0;
        for (int b = 1; b < dim; ++b)
            if (S.nc[b] > S.nc[a]) a = b;
        int nc = std::max(1, (int)(S.nc[a] * 0.9));
        if (nc < 2 * W + 1) {
            nc = 1;
            S.win[a] = 0;
        }
        S.nc[a] = nc;
    }
    for (int a = 0; a < 3; ++a) {
        S.edge[a] = a < dim ? S.prm.box[a] / S.nc[a] : 1.0;
        S.ncells *= S.nc[a];
    }
    // Morton order of the grid cells
    std::vector<std::pair<uint64_t, int>> codes(S.ncells);
    for (int c = 0; c < S.ncells; ++c) {
        int cx = c % S.nc[0], cy = (c / S.nc[0]) % S.nc[1], cz = c / (S.nc[0] * S.nc[1]);
        uint64_t code = dim == 2 ? (part1by1(cx) | (part1by1(cy) << 1))
                                 : (part1by2(cx) | (part1by2(cy) << 1) | (part1by2(cz) << 2));
        codes[c] = {code, c};
    }
    std::sort(codes.begin(), codes.end());
    S.morton.assign(S.ncells, 0);
    S.rank_lin.assign(S.ncells, 0);
    for (int r = 0; r < S.ncells; ++r) {
        S.morton[codes[r].second] = r;
        S.rank_lin[r] = codes[r].second;
    }
}

template <typename R>
void fill_const(SimConst<R> &c, const sph_engine *e, const Sim &S, const SimDev &d,
                double margin) {
    const sph_params &p = S.prm;
    c.thr_lo = (R)(d.thr * (1.0 - margin));
    c.thr_hi = (R)(d.thr * (1.0 + margin));
    // compact short kernels vanish beyond h (Lucy, Debrun) or 2h (cubic); the
    // margin keeps every pair the FP32 kernel could still see as q < 1
    double supp = p.kernel == SPH_KERNEL_CUBIC ? 2.0 * p.h_short : p.h_short;
    c.thr_s = c.thr_hi;
    if (p.kernel != SPH_KERNEL_GAUSSIAN && supp * supp * (1.0 + 1.0 / 1024.0) < d.thr)
        c.thr_s = (R)(supp * supp * (1.0 + 1.0 / 1024.0));
    for (int a = 0; a < 3; ++a) {
        c.edge[a] = (R)S.edge[a];
        c.edge_lo[a] = (R)(S.edge[a] - (double)c.edge[a]);
        c.L[a] = (R)p.box[a];
        c.hL[a] = (R)d.half_L[a];
        // rounded up so no reachable cell is culled; single-cell axes never are
        c.ext[a] = (a < e->dim && S.win[a] > 0) ? (R)((0.5 * S.edge[a] + d.slack_half[a]) * 1.0001)
                                               : (R)1e30;
    }
    if (S.vl_skin > 0.0) {
        // pair lists: the build's FP32 squared distances carry ~1e-6; the
        // 2^-10 margin files every pair that can enter the cutoff (or the
        // short support) while the lists hold
        const double rc = std::sqrt(d.thr), sk = S.vl_skin;
        c.vl_thr = (R)((rc + sk) * (rc + sk) * (1.0 + 1.0 / 1024.0));
        double near = (rc + sk) * (rc + sk);
        if (p.kernel != SPH_KERNEL_GAUSSIAN && supp * supp * (1.0 + 1.0 / 1024.0) < d.thr) {
            const double sq = supp * std::sqrt(1.0 + 1.0 / 1024.0);
            near = std::min(near, (sq + sk) * (sq + sk));
        }
        c.vl_near = (R)(near * (1.0 + 1.0 / 1024.0));
    } else {
        c.vl_thr = c.vl_near = (R)0;
    }
    const double hh[2] = {p.h_short, p.h_long}, sg[2] = {d.sig_s, d.sig_l};
    for (int k = 0; k < 2; ++k)
        kernel_consts<R>(p.kernel, hh[k], sg[k], c.h[k], c.h_lo[k], c.inv_h[k], c.inv_h_lo[k],
                         c.sig[k], c.g0[k], c.g0_h2[k], c.inv_h2[k], c.inv_h2_lo[k]);
    c.hs = (R)p.h_short;
    c.eps_h2 = (R)(p.visc_eps * p.h_short * p.h_short);
    c.alpha_c = (R)(p.visc_alpha * p.sound_speed);
    c.beta = (R)p.visc_beta;
    // the cohesive factor -2a folded into the long kernel's gradient
    // constants: the force passes take -2a grad W_l as one kernel evaluation
    const double g0l = kernel_g0(p.kernel, p.h_long, d.sig_l);
    c.g0_pl = (R)(g0l * (-2.0 * p.adash));
    c.g0_h2_pl = (R)(g0l / (p.h_long * p.h_long) * (-2.0 * p.adash));
    c.kappa = (R)p.thermalk;
}

SimDev make_simdev(const sph_engine *e, const Sim &S) {
    SimDev d;
    memset(&d, 0, sizeof(d));
    const sph_params &p = S.prm;
    double rc = std::sqrt(p.cutoff * p.cutoff + p.tolerance * p.tolerance);
    for (int a = 0; a < 3; ++a) {
        d.L[a] = p.box[a];
        d.half_L[a] = p.box[a] / 2.;
        d.inv_L[a] = 1.0 / p.box[a];
        d.edge[a] = S.edge[a];
        d.inv_edge[a] = 1.0 / S.edge[a];
        d.nc[a] = S.nc[a];
        d.win[a] = S.win[a];
        d.slack_half[a] = (a < e->dim && S.win[a] > 0) ? 0.5 * (S.win[a] * S.edge[a] - rc) : 1e300;
        d.box_half[a] = (a < e->dim && S.win[a] > 0) ? 0.5 * S.edge[a] + d.slack_half[a] : 1e300;
        d.rebin_half[a] =
            (a < e->dim && S.win[a] > 0) ? 0.5 * S.edge[a] + 0.5 * d.slack_half[a] : 1e300;
        if (a < e->dim && S.nc[a] == 1) d.small_mask |= (1 << a);
    }
    d.vl_gate2 = S.vl_skin > 0.0 ? 0.0625 * S.vl_skin * S.vl_skin : 1e300;
    d.vl_eskin2 = S.vl_skin > 0.0 ? 0.25 * S.vl_skin * S.vl_skin : 1e300;
    d.active = S.active ? 1 : 0;
    d.cell_off = S.cell_off;
    d.ncells = S.ncells;
    d.part_off = S.part_off;
    d.n = (int)S.n;
    d.chunk_first = S.chunk_first;
    d.nchunk = S.nchunk;
    d.thermostat = p.thermostat;
    d.thr = p.cutoff * p.cutoff + p.tolerance * p.tolerance;
    d.hs = p.h_short;
    d.hl = p.h_long;
    d.sig_s = kernel_sigma(p.kernel, e->dim, p.h_short);
    d.sig_l = kernel_sigma(p.kernel, e->dim, p.h_long);
    d.ws0 = kernel_w0(p.kernel, e->dim, p.h_short);
    d.wl0 = kernel_w0(p.kernel, e->dim, p.h_long);
    d.a = p.adash;
    d.b = p.bdash;
    d.kb = p.kbdash;
    d.alpha = p.visc_alpha;
    d.beta = p.visc_beta;
    d.eps = p.visc_eps;
    d.c = p.sound_speed;
    d.kappa = p.thermalk;
    d.dt = p.dt;
    d.hdt = 0.5 * p.dt;
    d.inv_kb = 1.0 / p.kbdash;
    d.T0 = p.thermostat_temp;
    d.T1 = p.thermostat_temp_end;
    d.ramp = p.thermostat_ramp_steps;
    d.coll_on = p.collision == SPH_COLLIDE_EXCHANGE ? 1 : 0;
    d.coll_c2 = p.collision_cutoff * p.collision_cutoff;
    for (int a = 0; a < 3; ++a) {
        // two particles within the collision range sit at most this many
        // cells apart (each may have drifted by slack_half since binning)
        int w = 0;
        if (d.coll_on && a < e->dim && S.nc[a] > 1)
            w = std::min(S.win[a], (int)std::ceil((p.collision_cutoff + 2.0 * d.slack_half[a]) /
                                                  S.edge[a]));
        d.coll_win[a] = w;
    }
    // fast-test guard band: 2^-12 relative in FP32 (cell-local coordinates
    // keep the FP32 squared distance within 5e-6 of the FP64 one), 1e-9 in FP64
    fill_const<float>(d.cf, e, S, d, 1.0 / 4096.0);
    fill_const<double>(d.cd, e, S, d, 1e-9);
    return d;
}

void free_graph(sph_engine *e) {
    if (e->graph_exec) cudaGraphExecDestroy(e->graph_exec);
    if (e->graph) cudaGraphDestroy(e->graph);
    e->graph_exec = nullptr;
    e->graph = nullptr;
    e->graph_steps = 0;
    e->graph_launched = false;
}

void cluster_free(sph_engine *e) {
    ClusterSet &c = e->cl;
    void *ptrs[] = {c.fcount, c.fstart,  c.fkey,    c.frank, c.ford, c.scan_tmp, c.colcnt,
                    c.colcl,  c.slot_idx, c.slot_of, c.cref,  c.ibox, c.jbox,     c.lnear,
                    c.lfar,   c.ent,     c.cpos,    c.cfv,   c.cf,   c.cq,       c.crho,
                    c.maxfill, c.colsim, c.csim};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    c = ClusterSet{};
    e->cl_np = e->cl_fine = e->cl_col = e->cl_ncl = 0;
    e->cl_ent = 0;
}

// Cluster geometry of the live 3D simulations (tuning.pair_scheme = 1):
// columns about 8 particles wide (the cube root of the volume of 8 at the
// simulation's mean density), slabs a quarter of that, the column reach of
// the cutoff plus twice the allowed drift, each simulation's range in the
// flattened column and fine-cell tables, and the buffers.  A simulation whose
// box is too narrow for the columns stays on the cell-window passes (the
// choice depends on the simulation alone); sd[s].cl_on marks the others.
// c.on = 0 if none runs on cluster pairs.
int cluster_setup(sph_engine *e, std::vector<SimDev> &sd) {
    ClusterSet &c = e->cl;
    c.on = 0;
    for (auto &d : sd) d.cl_on = 0;
    if (e->tune.pair_scheme != 1 || e->cl_disabled || e->dim != 3 || e->precision != SPH_MIXED ||
        e->group.collision != SPH_COLLIDE_OFF || e->np_b < 8)
        return SPH_OK;
    std::vector<ClGeom> geom(e->cap_s);
    std::vector<int> colsim;
    int64_t ncol = 0, nfine = 0, ncl_max = 0, np = 0;
    double per_est = 64.0;
    for (int sid = 0; sid < (int)e->sims.size(); ++sid) {
        const Sim &S = e->sims[sid];
        memset(&geom[sid], 0, sizeof(ClGeom));
        if (!S.active || S.n < 8) continue;
        const SimDev &d = sd[sid];
        const double *L = S.prm.box;
        const double vol = L[0] * L[1] * L[2];
        const double wt = std::cbrt(8.0 * vol / (double)S.n);
        const int ncx = std::max(1, (int)std::floor(L[0] / wt));
        const int ncy = std::max(1, (int)std::floor(L[1] / wt));
        const int nslab = std::max(1, (int)std::floor(L[2] / (0.25 * wt)));
        const double wx = L[0] / ncx, wy = L[1] / ncy, gz = L[2] / nslab;
        const double rc = std::sqrt(d.thr);
        double drift[3];
        bool fits = true;
        for (int a = 0; a < 3; ++a) {
            drift[a] = 2.0 * d.slack_half[a];
            fits &= drift[a] < 0.25 * L[a];   // not a single-cell axis, slack room
        }
        if (!fits) continue;
        // a column dx over lies at least (|dx| - 1) widths away
        const int rx = (int)std::ceil((rc + drift[0] + 1e-3) / wx);
        const int ry = (int)std::ceil((rc + drift[1] + 1e-3) / wy);
        // every column and every z image within reach must be distinct
        if (2 * rx + 1 > ncx || 2 * ry + 1 > ncy || rx > 100 || ry > 100) continue;
        if (L[2] < 2.0 * (rc + drift[2]) + 4.0 * gz || nslab > 30000) continue;
        const int64_t sfine = (int64_t)ncx * ncy * nslab;
        if (sfine > std::max<int64_t>(int64_t(1) << 16, 16 * S.n)) continue;
        sd[sid].cl_on = 1;
        ClGeom &g = geom[sid];
        g.ncx = ncx;
        g.ncy = ncy;
        g.nslab = nslab;
        g.rx = rx;
        g.ry = ry;
        g.col_off = (int)ncol;
        g.fine_off = (int)nfine;
        g.wxd = wx;
        g.wyd = wy;
        g.gzd = gz;
        g.wx = (float)wx;
        g.wy = (float)wy;
        g.gz = (float)gz;
        for (int a = 0; a < 3; ++a) g.drift2[a] = (float)drift[a];
        for (int k = 0; k < ncx * ncy; ++k) colsim.push_back(sid);
        ncol += (int64_t)ncx * ncy;
        nfine += sfine;
        ncl_max += S.n / 8 + (int64_t)ncx * ncy + 1;
        np += S.n;
        // list length before any measurement: 2.6 times the mean of a uniform
        // fluid (the j-halves in the box of an i-cluster grown by the reach)
        const double rho_n = (double)S.n / vol;
        const double R = rc + std::max(drift[0], std::max(drift[1], drift[2]));
        const double hz = 8.0 / (rho_n * wx * wy) + gz;
        const double box = (2 * wx + 2 * R) * (2 * wy + 2 * R) * (2 * hz + 2 * R);
        per_est = std::max(per_est, std::ceil(rho_n * box / 4.0));
    }
    if (ncol == 0 || nfine > (int64_t(1) << 30) || 8 * ncl_max > (int64_t(1) << 30)) {
        for (auto &d : sd) d.cl_on = 0;
        return SPH_OK;
    }
    // afterwards what the longest list measured needs (cluster_measure)
    const int per = e->cl_need > 0 ? e->cl_need : (int)std::min(65536.0, per_est);
    const long long cap = (long long)per * ncl_max;
    // fkey, frank and slot_of are indexed by the particle's place in the
    // engine's sorted order, so they hold every live particle, not only the
    // simulations on cluster pairs
    const int64_t nall = std::max<int64_t>(e->np_b, np);
    if (nall > e->cl_np || nfine > e->cl_fine || ncol > e->cl_col || ncl_max > e->cl_ncl ||
        cap > e->cl_ent) {
        cluster_free(e);
        const int64_t scan = std::max(nfine, ncol) / 4096 + 2;
        TRY(dalloc(&c.fcount, nfine));
        TRY(dalloc(&c.fstart, nfine + 1));
        TRY(dalloc(&c.fkey, nall));
        TRY(dalloc(&c.frank, nall));
        TRY(dalloc(&c.ford, nall));
        TRY(dalloc(&c.scan_tmp, scan));
        TRY(dalloc(&c.colcnt, ncol));
        TRY(dalloc(&c.colcl, ncol + 1));
        TRY(dalloc(&c.colsim, ncol));
        TRY(dalloc(&c.csim, ncl_max));
        TRY(dalloc(&c.slot_idx, 8 * ncl_max));
        TRY(dalloc(&c.slot_of, nall));
        TRY(dalloc(&c.cref, ncl_max));
        TRY(dalloc(&c.ibox, 2 * ncl_max));
        TRY(dalloc(&c.jbox, 4 * ncl_max));
        TRY(dalloc(&c.lnear, ncl_max));
        TRY(dalloc(&c.lfar, ncl_max));
        TRY(dalloc(&c.ent, cap));
        TRY(dalloc(&c.cpos, 8 * ncl_max));
        TRY(dalloc(&c.cfv, 8 * ncl_max));
        TRY(dalloc(&c.cf, 8 * ncl_max));
        TRY(dalloc(&c.cq, 8 * ncl_max));
        TRY(dalloc(&c.crho, 8 * ncl_max));
        TRY(dalloc(&c.maxfill, 1));
        CK(cudaMemset(c.maxfill, 0, sizeof(int)));
        e->cl_np = nall;
        e->cl_fine = nfine;
        e->cl_col = ncol;
        e->cl_ncl = ncl_max;
        e->cl_ent = cap;
    }
    if (!e->cl_geom_d || e->cl_geom_cap < e->cap_s) {
        cudaFree(e->cl_geom_d);
        e->cl_geom_d = nullptr;
        TRY(dalloc(&e->cl_geom_d, e->cap_s));
        e->cl_geom_cap = e->cap_s;
    }
    CK(cudaMemcpy(e->cl_geom_d, geom.data(), sizeof(ClGeom) * e->cap_s, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c.colsim, colsim.data(), sizeof(int) * ncol, cudaMemcpyHostToDevice));
    c.geom = e->cl_geom_d;
    c.sim1 = -1;
    memset(&c.g1, 0, sizeof(ClGeom));
    if (e->one_sim)
        for (int sid = 0; sid < (int)e->sims.size(); ++sid)
            if (e->sims[sid].active) {
                c.sim1 = sid;
                c.g1 = geom[sid];
            }
    c.ncol = (int)ncol;
    c.nfine = (int)nfine;
    c.ncl_max = (int)ncl_max;
    c.slots_max = (int)(8 * ncl_max);
    c.nall = (int)e->cl_np;
    c.lstride = per;
    c.on = 1;
    e->cl_stale = true;
    return SPH_OK;
}

int alloc_cells(sph_engine *e, int64_t cells) {
    if (cells <= e->cap_c) return SPH_OK;
    int64_t c = std::max<int64_t>(cells, e->cap_c * 2);
    cudaFree(e->cell_count);
    cudaFree(e->cell_start);
    cudaFree(e->morton);
    cudaFree(e->scan_tmp);
    e->cap_c = 0;
    TRY(dalloc(&e->cell_count, c));
    TRY(dalloc(&e->cell_start, c + 1));
    TRY(dalloc(&e->morton, c));
    cudaFree(e->cell_xyz);
    TRY(dalloc(&e->cell_xyz, c));
    TRY(dalloc(&e->scan_tmp, c / 4096 + 2));
    e->cap_c = c;
    free_graph(e);
    return SPH_OK;
}

View make_view(const sph_engine *e) {
    View v;
    memset(&v, 0, sizeof(v));
    v.np = e->np_b;
    v.persist = e->tune.persistent;
    v.dim = e->dim;
    v.sims = e->sims_d;
    for (int a = 0; a < 3; ++a) {
        v.a_pos[a] = e->a_pos[a];
        v.a_vel[a] = e->a_vel[a];
        v.b_pos[a] = e->b_pos[a];
        v.b_vel[a] = e->b_vel[a];
        v.q[a] = e->q[a];
        v.vdot[a] = e->vdot[a];
        v.f0v[a] = e->f0v[a];
        v.acc_r[a] = e->acc_r[a];
        v.acc_v[a] = e->acc_v[a];
    }
    v.a_u = e->a_u;
    v.a_m = e->a_m;
    v.a_id = e->a_id;
    v.a_sim = e->a_sim;
    v.b_u = e->b_u;
    v.b_m = e->b_m;
    v.b_id = e->b_id;
    v.b_sim = e->b_sim;
    v.cell_of = e->cell_of;
    v.rank = e->rank;
    v.order_tmp = e->order_tmp;
    v.order = e->order;
    v.cell_count = e->cell_count;
    v.cell_start = e->cell_start;
    v.cell_b = e->cell_b;
    v.morton = e->morton;
    v.cell_xyz = e->cell_xyz;
    for (int a = 0; a < 3; ++a) v.org[a] = e->org[a];
    v.pk_f = e->pk_f;
    v.pk_q = e->pk_q;
    v.pk_fv = e->pk_fv;
    v.rho = e->rho;
    v.rho_l = e->rho_l;
    v.temp = e->temp;
    v.pres = e->pres;
    v.pco = e->pco;
    v.rho0 = e->rho0;
    v.pres0 = e->pres0;
    v.pco0 = e->pco0;
    v.udot = e->udot;
    v.f0u = e->f0u;
    v.acc_u = e->acc_u;
    v.tsum_part = e->tsum_part;
    v.chunk_sim = e->chunk_sim;
    v.chunk_start = e->chunk_start;
    v.chunk_len = e->chunk_len;
    v.nchunks = e->nchunks;
    v.t_scale = e->t_scale;
    v.steps = e->steps_d;
    v.pair_count = e->pair_count;
    v.err = e->err;
    v.err_any = e->err_any;
    v.bin_count = e->bin_count;
    v.one_sim = e->one_sim ? 1 : 0;
    if (e->one_sim) v.one = e->one_dev;
    // pair lists once their rows exist (measured)
    if (e->vl.on && e->vl.ent && e->vl.cap > 0) {
        v.vl_on = 1;
        v.vl_cap = e->vl.cap;
        v.vl_stride = e->vl.stride;
        v.vl_ent = e->vl.ent;
        v.vl_cnt = e->vl.cnt;
        v.vl_x0 = e->vl.x0;
    }
    return v;
}

// Binning on demand applies to multi-stage integrators: their last stage
// writes packed buffer 0, which no evaluation of that stage reads.  Pair
// lists always bin (and build) on demand.
bool rebin_on_demand(const sph_engine *e) {
    return (e->tune.rebin != 0 || e->vl.on) && e->nstage > 1;
}

// The pair lists' skin as a fraction of the cutoff, 0 without them.
double list_skin_of(const sph_engine *e) {
    return e->tune.pair_scheme == 2 ? e->tune.list_skin : 0.0;
}

// Pair lists (cluster or particle) whose fill the host tracks.
bool lists_on(const sph_engine *e) { return e->cl.on || e->vl.on; }
int *list_maxfill(const sph_engine *e) { return e->cl.on ? e->cl.maxfill : e->vl.maxfill; }
int list_room(const sph_engine *e) { return e->cl.on ? e->cl.lstride : e->vl.cap; }

// Pair lists of a mixed-precision engine (tuning.pair_scheme = 2): on when
// every live simulation's grid has a window of 1 to 3 cells per axis and
// room for it, without collisions, and the slots fit the entries' index
// field.  The rows are sized by vl_measure before the next use.
int vl_setup(sph_engine *e) {
    VList &l = e->vl;
    l.on = 0;
    if (e->tune.pair_scheme != 2 || e->vl_disabled || e->precision != SPH_MIXED ||
        e->group.collision != SPH_COLLIDE_OFF || e->np_b <= 0 ||
        e->np_b > vl_index_mask(e->dim))
        return SPH_OK;
    for (const auto &S : e->sims) {
        if (!S.active) continue;
        if (!(S.vl_skin > 0.0)) return SPH_OK;
        for (int a = 0; a < e->dim; ++a)
            if (S.win[a] < 1 || S.win[a] > kVlMaxWindow || S.nc[a] < 2 * S.win[a] + 1)
                return SPH_OK;
    }
    if (!l.cnt) {
        TRY(dalloc(&l.cnt, e->cap_p));
        TRY(dalloc(&l.x0, e->cap_p));
        TRY(dalloc(&l.maxfill, 1));
        CK(cudaMemset(l.maxfill, 0, sizeof(int)));
    }
    const long long stride = ((long long)e->np_b + 31) & ~31LL;
    if (stride != l.stride) {
        // rows of the old layout: measured again before the next use
        cudaFree(l.ent);
        l.ent = nullptr;
        l.cap = 0;
        e->vl_alloc = 0;
        l.stride = stride;
    }
    l.on = 1;
    e->cl_stale = true;
    return SPH_OK;
}

// Evaluation buffers of stage s: stage 0 reads the permuted x0 (B) and
// packed buffer 0; stage s >= 1 reads what stage s-1's force pass wrote.
void stage_view(const sph_engine *e, View &v, int s) {
    int pin = s & 1, pout = (s + 1) & 1;
    v.pk_pos_in = e->pk_pos[pin];
    v.pk_vel_in = e->pk_vel[pin];
    v.pk_pos_out = e->pk_pos[pout];
    v.pk_vel_out = e->pk_vel[pout];
    for (int a = 0; a < 3; ++a) {
        v.xe_in[a] = s == 0 ? e->b_pos[a] : e->xe[(s - 1) & 1][a];
        v.xe_out[a] = e->xe[s & 1][a];
        v.ve_in[a] = s == 0 ? e->b_vel[a] : e->ve[a];
        v.ve_out[a] = e->ve[a];
    }
    v.ue_in = s == 0 ? e->b_u : e->ue;
    v.ue_out = e->ue;
}

// Rebuilds the host-side layout: cell offsets, concatenated Morton and
// neighbour tables, particle offsets and reduction chunks; uploads them.
int relayout(sph_engine *e) {
    e->bins_valid = false;
    int cell_off = 0, part_off = 0;
    e->any_thermostat = false;
    for (auto &S : e->sims) {
        if (!S.active) continue;
        S.cell_off = cell_off;
        S.part_off = part_off;
        cell_off += S.ncells;
        part_off += (int)S.n;
        if (S.prm.thermostat) e->any_thermostat = true;
    }
    TRY(alloc_cells(e, std::max(cell_off, 1)));
    e->ncells_total = cell_off;
    e->np_b = part_off;
    std::vector<int> mort(std::max(cell_off, 1));
    std::vector<int> cxyz(std::max(cell_off, 1), 0);
    std::vector<int> csim, cstart, clen;
    for (auto &S : e->sims) {
        if (!S.active) continue;
        for (int lin = 0; lin < S.ncells; ++lin) mort[S.cell_off + lin] = S.morton[lin];
        for (int r = 0; r < S.ncells; ++r) {
            int lin = S.rank_lin[r];
            int c[3] = {lin % S.nc[0], (lin / S.nc[0]) % S.nc[1], lin / (S.nc[0] * S.nc[1])};
            cxyz[S.cell_off + r] = c[0] | (c[1] << 11) | (c[2] << 22);
        }
        S.chunk_first = (int)csim.size();
        S.nchunk = (int)((S.n + 1023) / 1024);
        for (int64_t b = 0; b < S.n; b += 1024) {
            csim.push_back((int)(&S - &e->sims[0]));
            cstart.push_back(S.part_off + (int)b);
            clen.push_back((int)std::min<int64_t>(1024, S.n - b));
        }
    }
    e->nchunks = (int)csim.size();
    if (e->nchunks > e->cap_chunks) {
        cudaFree(e->chunk_sim);
        cudaFree(e->chunk_start);
        cudaFree(e->chunk_len);
        cudaFree(e->tsum_part);
        int64_t c = std::max<int64_t>(e->nchunks, 2 * e->cap_chunks);
        TRY(dalloc(&e->chunk_sim, c));
        TRY(dalloc(&e->chunk_start, c));
        TRY(dalloc(&e->chunk_len, c));
        TRY(dalloc(&e->tsum_part, c));
        e->cap_chunks = c;
    }
    cudaStream_t st = e->stream;
    if (cell_off > 0) {
        CK(cudaMemcpyAsync(e->morton, mort.data(), sizeof(int) * cell_off, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(e->cell_xyz, cxyz.data(), sizeof(int) * cell_off,
                           cudaMemcpyHostToDevice, st));
    }
    if (e->nchunks > 0) {
        CK(cudaMemcpyAsync(e->chunk_sim, csim.data(), sizeof(int) * e->nchunks, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(e->chunk_start, cstart.data(), sizeof(int) * e->nchunks, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(e->chunk_len, clen.data(), sizeof(int) * e->nchunks, cudaMemcpyHostToDevice, st));
    }
    std::vector<SimDev> sd(e->cap_s);
    for (int s = 0; s < e->cap_s; ++s) {
        if (s < (int)e->sims.size()) sd[s] = make_simdev(e, e->sims[s]);
        else memset(&sd[s], 0, sizeof(SimDev));
    }
    // a single live simulation: its constants travel as kernel parameters
    int live = 0, last = -1;
    for (int s = 0; s < (int)e->sims.size(); ++s)
        if (e->sims[s].active) ++live, last = s;
    e->one_sim = live == 1;
    // marks the simulations that run on cluster pairs (SimDev.cl_on)
    TRY(cluster_setup(e, sd));
    TRY(vl_setup(e));
    e->n_cell_sims = 0;
    for (int s = 0; s < (int)e->sims.size(); ++s)
        if (e->sims[s].active && !sd[s].cl_on) ++e->n_cell_sims;
    if (e->one_sim) e->one_dev = sd[last];
    CK(cudaMemcpyAsync(e->sims_d, sd.data(), sizeof(SimDev) * e->cap_s, cudaMemcpyHostToDevice, st));
    CK(cudaStreamSynchronize(st));
    free_graph(e);
    e->layout_dirty = false;
    return SPH_OK;
}

// Event pair around one pass when profiling is on (pool grows outside capture).
struct ProfScope {
    sph_engine *e;
    cudaStream_t st;
    int kind;
    cudaEvent_t b = nullptr;
    unsigned flags = cudaEventRecordDefault;
    ProfScope(sph_engine *e_, int kind_, cudaStream_t st_) : e(e_), st(st_), kind(kind_) {
        if (!e->prof_on || e->prof_used + 2 > e->prof_pool.size()) return;
        cudaEvent_t a = e->prof_pool[e->prof_used++];
        b = e->prof_pool[e->prof_used++];
        // external record nodes when captured, so the events are timeable;
        // plain records for the eager steps of an advance (the external
        // flag is refused outside a capture)
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        cudaStreamIsCapturing(st, &cs);
        if (cs == cudaStreamCaptureStatusActive) flags = cudaEventRecordExternal;
        cudaEventRecordWithFlags(a, st, flags);
        e->prof_recs.push_back({kind, a, b});
    }
    ~ProfScope() {
        if (b) cudaEventRecordWithFlags(b, st, flags);
    }
};

constexpr int kSortKernels = 7;  // bin, 3 scan, scatter, in-cell order, permute

// Counting sort of A into B plus the packed first-evaluation copies.  Gated:
// the kernels run only if the device gate is raised (binning on demand); the
// close kernel then lowers it and counts the binning.
void enqueue_prepare(sph_engine *e, cudaStream_t st, bool gated = false, bool lists = true) {
    ProfScope ps(e, SPH_PASS_SORT, st);
    View v = make_view(e);
    stage_view(e, v, 0);
    v.pk_pos_out = e->pk_pos[0];
    v.pk_vel_out = e->pk_vel[0];
    const int *gate = gated ? e->rebin_gate : nullptr;
    v.rebin_gate = gated ? e->rebin_gate : nullptr;
    if (gated)
        launch_fill_int(e->cell_count, 0, std::max(e->ncells_total, 1), st, gate);
    else
        cudaMemsetAsync(e->cell_count, 0, sizeof(int) * std::max(e->ncells_total, 1), st);
    cudaMemsetAsync(e->pair_count, 0, sizeof(unsigned long long) * e->cap_s, st);
    launch_bin(v, e->a_extent, st);
    launch_scan(e->cell_count, e->cell_start, e->ncells_total, e->scan_tmp, st, gate);
    launch_scatter(v, e->a_extent, st);
    launch_cellsort(v, e->ncells_total, st);
    launch_permute(v, e->precision, st);
    // a binning renumbers the slots: the pair lists are built again
    if (lists && e->vl.on && e->vl.ent && e->vl.cap > 0)
        launch_vlist_build(v, e->vl, gate, kVlStore, st);
    if (gated) launch_rebin_close(e->rebin_gate, e->bin_count, st);
}

// Collision candidates at the evaluation positions of v and their levels.
void enqueue_collide_find(sph_engine *e, const View &v, cudaStream_t st) {
    CollideSet c = e->coll;
    c.np = e->np_b;
    cudaMemsetAsync(c.info, 0, sizeof(int) * 4, st);
    launch_collide_find(v, c, st);
    launch_collide_levels(c, st);
}

// Collisions on the velocities of evaluation s (stage 0: the start state).
void enqueue_collide_apply(sph_engine *e, int s, bool packed, cudaStream_t st) {
    CollideSet c = e->coll;
    c.np = e->np_b;
    double *const *vel = s == 0 ? e->b_vel : e->ve;
    Vec3Ref vr{{vel[0], vel[1], vel[2]}, 1};
    launch_collide_apply(c, e->dim, vr, vr, e->b_m, 0.0, packed ? e->pk_vel[0] : nullptr,
                         e->precision, e->err, e->err_any, (int)e->sims.size(), st);
}

// One evaluation of the step.  With hard collisions the reference's
// derivatives() mutates the velocities after the rates are computed
// (forces after SpamComplete in p.forces), before the integrator reads
// them as rdot and, on the first evaluation, as x_start; the step's extra
// first evaluation (particles.py:480) leaves its collisions behind too.  The
// force pass then stops at the rates and a separate pass integrates.
void enqueue_stage(sph_engine *e, int s, int mode, cudaStream_t st) {
    View v = make_view(e);
    stage_view(e, v, s);
    if (mode == 1 && s == e->nstage - 1 && rebin_on_demand(e)) {
        v.reuse = 1;
        v.rebin_gate = e->rebin_gate;
    }
    const bool cells = e->n_cell_sims > 0;
    if (e->cl.on) {
        // the simulations on cluster pairs: build at the step's first
        // evaluation, repack at the later ones; their rates pass leaves the
        // stage update to k_integrate.  The cell-window passes below skip
        // them (SimDev.cl_on) and run only if some simulation remains.
        const ClusterSet &c = e->cl;
        const int kern = e->group.kernel;
        if (s == 0) {
            ProfScope ps(e, SPH_PASS_SORT, st);
            launch_cluster_build(v, c, st);
        }
        {
            ProfScope ps(e, SPH_PASS_DENSITY, st);
            if (s > 0) launch_cluster_pack(v, c, s, st);
            launch_cluster_density(v, c, kern, s, st);
            if (cells) launch_density(v, e->precision, kern, s, e->tune.block_size, st);
        }
        if (e->group.heat_flux) {
            ProfScope ps(e, SPH_PASS_HEAT, st);
            launch_cluster_heat(v, c, kern, st);
            if (cells) launch_heat(v, e->precision, kern, e->tune.block_size, st);
        }
        if (mode == 1 && s == e->nstage - 1 && e->any_thermostat) {
            ProfScope ps(e, SPH_PASS_TSUM, st);
            launch_tsum(v, e->precision, (int)e->sims.size(), st);
        }
        {
            ProfScope ps(e, SPH_PASS_FORCE, st);
            launch_cluster_force(v, c, kern, e->group.viscosity, e->group.heat_flux, st);
            if (mode == 1) launch_integrate(v, e->precision, e->group.integrator, s, st, 1);
            if (cells)
                launch_force(v, e->precision, kern, e->group.viscosity, e->group.heat_flux,
                             e->group.integrator, s, mode, e->tune.block_size, st);
        }
        return;
    }
    int blk = e->tune.block_size;
    const bool coll = mode == 1 && e->group.collision != SPH_COLLIDE_OFF;
    if (coll && s == 0) {
        ProfScope ps(e, SPH_PASS_FORCE, st);
        enqueue_collide_find(e, v, st);
        enqueue_collide_apply(e, 0, true, st);
    }
    {
        ProfScope ps(e, SPH_PASS_DENSITY, st);
        launch_density(v, e->precision, e->group.kernel, s, blk, st);
    }
    if (e->group.heat_flux) {
        ProfScope ps(e, SPH_PASS_HEAT, st);
        launch_heat(v, e->precision, e->group.kernel, blk, st);
    }
    if (mode == 1 && s == e->nstage - 1 && e->any_thermostat) {
        ProfScope ps(e, SPH_PASS_TSUM, st);
        launch_tsum(v, e->precision, (int)e->sims.size(), st);
    }
    {
        ProfScope ps(e, SPH_PASS_FORCE, st);
        launch_force(v, e->precision, e->group.kernel, e->group.viscosity, e->group.heat_flux,
                     e->group.integrator, s, coll ? 0 : mode, blk, st);
        if (coll) {
            if (s > 0) enqueue_collide_find(e, v, st);
            enqueue_collide_apply(e, s, false, st);
            launch_integrate(v, e->precision, e->group.integrator, s, st);
        }
    }
}

void enqueue_step(sph_engine *e, cudaStream_t st) {
    enqueue_prepare(e, st, rebin_on_demand(e));
    for (int s = 0; s < e->nstage; ++s) enqueue_stage(e, s, 1, st);
}

// Measures the longest pair list of the current state (a binning and a
// list build that only counts) and sizes the list regions to 1.4 times it,
// growing or shrinking the entry buffer.  Runs before an advance or an
// evaluation whenever the state was set from outside or the layout changed,
// and within an advance once a chunk of steps filled a region past 80% (a
// fluid condensing into denser regions): the chunk already queued then has
// 25% of headroom left, and an overflow is still reported (SPH_ECAPACITY).  Lists that
// do not fit in device memory leave the layout on the cell scheme.
int cluster_measure(sph_engine *e) {
    ClusterSet &c = e->cl;
    if (!c.on) return SPH_OK;
    cudaStream_t st = e->stream;
    const bool prof = e->prof_on;
    e->prof_on = false;
    CK(cudaMemsetAsync(c.maxfill, 0, sizeof(int), st));
    enqueue_prepare(e, st);
    View v = make_view(e);
    stage_view(e, v, 0);
    launch_cluster_build(v, c, st, false);
    e->prof_on = prof;
    int fill = 0;
    CK(cudaMemcpyAsync(&fill, c.maxfill, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaMemsetAsync(c.maxfill, 0, sizeof(int), st));
    CK(cudaStreamSynchronize(st));
    e->cl_stale = false;
    e->cl_fill_pending = false;   // read of the old regions: superseded
    const int need = std::max(64, (int)std::ceil(1.4 * fill) + 8);
    if (need == c.lstride) return SPH_OK;
    free_graph(e);
    // regions are addressed with 64-bit offsets: the buffer may exceed 2^31
    // entries (a simulation of tens of millions of particles)
    cudaFree(c.ent);
    c.ent = nullptr;
    const int st_alloc = dalloc(&c.ent, (int64_t)need * c.ncl_max);
    if (st_alloc != SPH_OK) {
        // no room for the lists: the layout is rebuilt on the cell scheme
        c.on = 0;
        e->cl_ent = 0;
        e->cl_disabled = true;
        e->layout_dirty = true;
        return SPH_OK;
    }
    c.lstride = need;
    e->cl_need = need;
    e->cl_ent = (long long)need * c.ncl_max;
    return SPH_OK;
}

// Bins the current state and builds the pair lists into the existing rows
// (only counts without rows), reading back the longest list: the lists are
// kept if it left a fifth of the rows free, otherwise the rows are resized
// to 1.25 times it (+8, at least 40, whole groups of four; the near and far
// runs each fill whole groups) and the lists built again.
// Either way the cells and lists then match the state, so the next step
// need not bin.  Lists longer than the count field or rows that do not fit
// in device memory leave the layout on cell windows.
int vl_measure(sph_engine *e) {
    VList &l = e->vl;
    if (!l.on) return SPH_OK;
    cudaStream_t st = e->stream;
    const bool prof = e->prof_on;
    e->prof_on = false;
    CK(cudaMemsetAsync(l.maxfill, 0, sizeof(int), st));
    enqueue_prepare(e, st, false, false);
    const bool have = l.ent && l.cap > 0;
    {
        View v = make_view(e);
        stage_view(e, v, 0);
        VList m = l;
        if (!have) m.cap = 0;
        launch_vlist_build(v, m, nullptr, have ? kVlStoreQuiet : kVlCount, st);
    }
    int fill = 0;
    CK(cudaMemcpyAsync(&fill, l.maxfill, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaMemsetAsync(l.maxfill, 0, sizeof(int), st));
    CK(cudaStreamSynchronize(st));
    e->prof_on = prof;
    e->cl_stale = false;
    e->cl_fill_pending = false;
    if (have && fill <= 0.8 * l.cap) {
        e->bins_valid = true;
        return SPH_OK;
    }
    const int need = (std::max(40, (int)std::ceil(1.25 * fill) + 8) + 3) & ~3;
    if (need != l.cap || !l.ent) {
        free_graph(e);
        cudaFree(l.ent);
        l.ent = nullptr;
        l.cap = 0;
        e->vl_alloc = 0;
        if (need > 0xffff || dalloc(&l.ent, (size_t)need * (size_t)l.stride) != SPH_OK) {
            l.on = 0;
            e->vl_disabled = true;
            e->layout_dirty = true;
            e->bins_valid = false;
            return SPH_OK;
        }
        l.cap = need;
        e->vl_alloc = (long long)need * l.stride;
    }
    View v = make_view(e);
    stage_view(e, v, 0);
    launch_vlist_build(v, l, nullptr, kVlStoreQuiet, st);
    e->bins_valid = true;
    return SPH_OK;
}

// Before an advance or an evaluation with cluster pairs or pair lists:
// re-measure if the state changed or the last advance filled a list past
// 80% of its room.
int cluster_check(sph_engine *e) {
    if (!lists_on(e)) return SPH_OK;
    if (e->cl_fill_pending && cudaEventQuery(e->cl_fill_ev) == cudaSuccess) {
        e->cl_fill_pending = false;
        if (*e->cl_fill_host > 0.8 * list_room(e)) e->cl_stale = true;
    }
    if (e->cl_stale) TRY(e->cl.on ? cluster_measure(e) : vl_measure(e));
    if (e->layout_dirty) TRY(relayout(e));   // the lists did not fit
    if (e->vl.on && e->cl_stale) TRY(vl_measure(e));   // set up again by the relayout
    return SPH_OK;
}

// After an advance: the longest list of its steps, read back without a
// wait (checked by the next cluster_check).
int cluster_note_fill(sph_engine *e) {
    if (!lists_on(e)) return SPH_OK;
    if (!e->cl_fill_host) {
        CK(cudaMallocHost((void **)&e->cl_fill_host, sizeof(int)));
        CK(cudaEventCreateWithFlags(&e->cl_fill_ev, cudaEventDisableTiming));
    }
    if (e->cl_fill_pending) return SPH_OK;   // the previous read is still in flight
    int *fill = list_maxfill(e);
    CK(cudaMemcpyAsync(e->cl_fill_host, fill, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
    CK(cudaMemsetAsync(fill, 0, sizeof(int), e->stream));
    CK(cudaEventRecord(e->cl_fill_ev, e->stream));
    e->cl_fill_pending = true;
    return SPH_OK;
}

int64_t kernels_per_step(const sph_engine *e) {
    if (e->cl.on) {
        // cluster build; per evaluation density, [heat,] force and the stage
        // update; the later evaluations' repacking; the cell-window passes of
        // the other simulations
        int64_t k = kSortKernels + cluster_build_kernels();
        k += (int64_t)e->nstage * (3 + (e->group.heat_flux ? 1 : 0)) + (e->nstage - 1);
        if (e->n_cell_sims > 0) k += (int64_t)e->nstage * (2 + (e->group.heat_flux ? 1 : 0));
        if (e->any_thermostat) k += 2;
        if (rebin_on_demand(e)) k += 2;
        return k;
    }
    int64_t k = kSortKernels + (e->vl.on ? 1 : 0);   // + the pair lists' build
    k += (int64_t)e->nstage * (2 + (e->group.heat_flux ? 1 : 0));
    if (e->any_thermostat) k += 2;
    // collisions: per find 5 kernels + 7 for the levels, one apply per
    // evaluation plus the extra first one, one integrator pass per stage
    if (e->group.collision != SPH_COLLIDE_OFF) k += (int64_t)e->nstage * 14 + 1;
    if (rebin_on_demand(e)) k += 2;   // gated cell-count fill and close
    return k;
}

int ensure_prof_pool(sph_engine *e, size_t need) {
    while (e->prof_pool.size() < need) {
        cudaEvent_t ev;
        CK(cudaEventCreate(&ev));
        e->prof_pool.push_back(ev);
    }
    return SPH_OK;
}

// Captures `per` steps as the engine's graph, unless that graph exists.
// With profiling on, a graph already launched is captured again on fresh
// event slots, so every launch's passes are timed (not only the last one).
int build_graph(sph_engine *e, int per) {
    if (e->graph_exec && e->graph_steps == per && !(e->prof_on && e->graph_launched))
        return SPH_OK;
    free_graph(e);
    if (e->prof_on) {
        TRY(ensure_prof_pool(e, e->prof_used + (size_t)per * 2 * (1 + 4 * e->nstage) + 8));
    }
    cudaStream_t st = e->stream;
    CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < per; ++k) enqueue_step(e, st);
    CK(cudaStreamEndCapture(st, &e->graph));
    CK(cudaGraphInstantiate(&e->graph_exec, e->graph, 0));
    e->graph_steps = per;
    return SPH_OK;
}


void after_advance(sph_engine *e, int steps) {
    e->a_extent = e->np_b;
    for (auto &S : e->sims)
        if (S.active) {
            S.a_off = S.part_off;
            S.steps += steps;
        }
    e->props_valid = true;
}

int ensure_layout(sph_engine *e) {
    if (e->layout_dirty) TRY(relayout(e));
    return SPH_OK;
}

int check_sim(sph_engine *e, int32_t id) {
    if (!e || id < 0 || id >= (int)e->sims.size() || !e->sims[id].active) return SPH_ENOTFOUND;
    return SPH_OK;
}

// Staging regions (offsets in cap_p units): positions, velocities, a scalar.
constexpr int kStageR = 0, kStageV = 3, kStageU = 6;

// Copies n*k doubles from caller memory into staging region `region`.
int stage_in(sph_engine *e, const double *src, size_t count, int mem, int region, double **out) {
    if (mem == SPH_DEVICE) {
        *out = const_cast<double *>(src);
        return SPH_OK;
    }
    double *dst = e->stage_buf + (size_t)region * e->cap_p;
    CK(cudaMemcpyAsync(dst, src, sizeof(double) * count, cudaMemcpyHostToDevice, e->stream));
    *out = dst;
    return SPH_OK;
}

int write_state_range(sph_engine *e, int off, int64_t n, const double *r, const double *v,
                      const double *m, const double *u, int mem) {
    cudaStream_t st = e->stream;
    double *pos[3] = {e->a_pos[0] + off, e->a_pos[1] + off, e->a_pos[2] + off};
    double *vel[3] = {e->a_vel[0] + off, e->a_vel[1] + off, e->a_vel[2] + off};
    double *src;
    if (r) {
        TRY(stage_in(e, r, (size_t)n * e->dim, mem, kStageR, &src));
        launch_load_aos(pos, src, (int)n, e->dim, st);
    }
    if (v) {
        TRY(stage_in(e, v, (size_t)n * e->dim, mem, kStageV, &src));
        launch_load_aos(vel, src, (int)n, e->dim, st);
    }
    cudaMemcpyKind k = mem == SPH_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (m) CK(cudaMemcpyAsync(e->a_m + off, m, sizeof(double) * n, k, st));
    if (u) CK(cudaMemcpyAsync(e->a_u + off, u, sizeof(double) * n, k, st));
    if (mem == SPH_HOST) CK(cudaStreamSynchronize(st));
    return SPH_OK;
}

int copy_out(sph_engine *e, double *dst, size_t count, int mem, double *dev_src) {
    if (mem == SPH_DEVICE) return SPH_OK;  // written in place
    CK(cudaMemcpyAsync(dst, dev_src, sizeof(double) * count, cudaMemcpyDeviceToHost, e->stream));
    return SPH_OK;
}

// Gathers an R array (B order) of simulation s into caller order.
int gather_R(sph_engine *e, const Sim &S, void *src, double *dst, int mem) {
    if (!dst) return SPH_OK;
    double *d = mem == SPH_DEVICE ? dst : e->stage_buf;
    launch_store_R(d, src, e->precision, e->b_id, S.part_off, (int)S.n, e->stream);
    TRY(copy_out(e, dst, (size_t)S.n, mem, d));
    if (mem == SPH_HOST) CK(cudaStreamSynchronize(e->stream));
    return SPH_OK;
}

int gather_R_vec(sph_engine *e, const Sim &S, void *const src[3], double *dst, int mem) {
    if (!dst) return SPH_OK;
    double *d = mem == SPH_DEVICE ? dst : e->stage_buf;
    // component-wise into AoS: store each component with stride dim via temp
    for (int a = 0; a < e->dim; ++a) {
        double *tmp = e->stage_buf + (size_t)e->cap_p * 3;  // past the 3 cap_p AoS region
        launch_store_R(tmp, src[a], e->precision, e->b_id, S.part_off, (int)S.n, e->stream);
        CK(cudaMemcpy2DAsync(d + a, sizeof(double) * e->dim, tmp, sizeof(double), sizeof(double),
                             (size_t)S.n, cudaMemcpyDeviceToDevice, e->stream));
    }
    TRY(copy_out(e, dst, (size_t)S.n * e->dim, mem, d));
    if (mem == SPH_HOST) CK(cudaStreamSynchronize(e->stream));
    return SPH_OK;
}

int alloc_particles(sph_engine *e) {
    int64_t P = e->cap_p;
    for (int a = 0; a < 3; ++a) {
        TRY(dalloc(&e->a_pos[a], P));
        TRY(dalloc(&e->a_vel[a], P));
        TRY(dalloc(&e->b_pos[a], P));
        TRY(dalloc(&e->b_vel[a], P));
        TRY(dalloc(&e->xe[0][a], P));
        TRY(dalloc(&e->xe[1][a], P));
        TRY(dalloc(&e->ve[a], P));
        TRY(dalloc(&e->org[a], P));
        TRY(dalloc((char **)&e->q[a], P * e->rsize));
        TRY(dalloc((char **)&e->vdot[a], P * e->rsize));
        TRY(dalloc((char **)&e->f0v[a], P * e->rsize));
        if (e->group.integrator == SPH_RK4) {
            TRY(dalloc(&e->acc_r[a], P));
            TRY(dalloc(&e->acc_v[a], P));
        }
    }
    TRY(dalloc(&e->a_u, P));
    TRY(dalloc(&e->a_m, P));
    TRY(dalloc(&e->a_id, P));
    TRY(dalloc(&e->a_sim, P));
    TRY(dalloc(&e->b_u, P));
    TRY(dalloc(&e->b_m, P));
    TRY(dalloc(&e->b_id, P));
    TRY(dalloc(&e->b_sim, P));
    TRY(dalloc(&e->cell_of, P));
    TRY(dalloc(&e->rank, P));
    TRY(dalloc(&e->order_tmp, P));
    TRY(dalloc(&e->order, P));
    TRY(dalloc(&e->cell_b, P));
    TRY(dalloc(&e->ue, P));
    for (int b = 0; b < 2; ++b) {
        TRY(dalloc((char **)&e->pk_pos[b], P * e->v4size));
        TRY(dalloc((char **)&e->pk_vel[b], P * e->v4size));
    }
    TRY(dalloc((char **)&e->pk_f, P * e->v4size));
    TRY(dalloc((char **)&e->pk_q, P * e->v4size));
    TRY(dalloc((char **)&e->pk_fv, P * e->v4size));
    void **rs[] = {&e->rho, &e->rho_l, &e->temp, &e->pres, &e->pco, &e->rho0, &e->pres0,
                   &e->pco0, &e->udot, &e->f0u};
    for (void **p : rs) TRY(dalloc((char **)p, P * e->rsize));
    if (e->group.integrator == SPH_RK4) TRY(dalloc(&e->acc_u, P));
    TRY(dalloc(&e->stage_buf, P * 8));
    if (e->group.collision != SPH_COLLIDE_OFF) {
        // up to one colliding pair per particle per evaluation (SPH_ECAPACITY beyond)
        CollideSet &c = e->coll;
        c.cap = (int)P;
        TRY(dalloc(&c.row_count, P + 1));
        TRY(dalloc(&c.row_start, P + 1));
        TRY(dalloc(&c.scan_tmp, P / 4096 + 2));
        TRY(dalloc(&c.ci, P));
        TRY(dalloc(&c.cj, P));
        for (int a = 0; a < 3; ++a) TRY(dalloc(&c.dr[a], P));
        TRY(dalloc(&c.rij, P));
        TRY(dalloc(&c.src, P));
        TRY(dalloc(&c.touch_count, P + 1));
        TRY(dalloc(&c.touch_start, P + 1));
        TRY(dalloc(&c.touch_fill, P + 1));
        TRY(dalloc(&c.touch, 2 * P));
        TRY(dalloc(&c.pred, 2 * P));
        TRY(dalloc(&c.level, P));
        TRY(dalloc(&c.info, 4));
    }
    // pk_q must read as zero when heat flux is off
    CK(cudaMemset(e->pk_q, 0, P * e->v4size));
    CK(cudaMemset(e->a_sim, 0xff, P * sizeof(int)));
    return SPH_OK;
}

int alloc_sims(sph_engine *e) {
    int S = e->cap_s;
    TRY(dalloc(&e->sims_d, S));
    TRY(dalloc(&e->t_scale, S));
    TRY(dalloc(&e->steps_d, S));
    TRY(dalloc(&e->pair_count, S));
    TRY(dalloc(&e->err, S));
    TRY(dalloc(&e->err_any, 1));
    TRY(dalloc(&e->rebin_gate, 1));
    TRY(dalloc(&e->restage_far, 1));
    TRY(dalloc(&e->bin_count, 1));
    CK(cudaMemset(e->rebin_gate, 0, sizeof(int)));
    CK(cudaMemset(e->bin_count, 0, sizeof(unsigned long long)));
    CK(cudaMemset(e->err, 0, sizeof(int) * S));
    CK(cudaMemset(e->err_any, 0, sizeof(int)));
    CK(cudaMemset(e->steps_d, 0, sizeof(long long) * S));
    CK(cudaMemset(e->pair_count, 0, sizeof(unsigned long long) * S));
    std::vector<double> one(S, 1.0);
    CK(cudaMemcpy(e->t_scale, one.data(), sizeof(double) * S, cudaMemcpyHostToDevice));
    return SPH_OK;
}

void free_all(sph_engine *e) {
    free_graph(e);
    void *ptrs[] = {e->a_u, e->a_m, e->a_id, e->a_sim, e->b_u, e->b_m, e->b_id, e->b_sim,
                    e->cell_of, e->rank, e->order_tmp, e->order, e->cell_b, e->cell_count,
                    e->cell_start, e->morton, e->scan_tmp, e->pk_pos[0], e->pk_pos[1],
                    e->pk_vel[0], e->pk_vel[1], e->pk_f, e->pk_q, e->pk_fv, e->ue, e->rho, e->rho_l,
                    e->temp, e->pres, e->pco, e->rho0, e->pres0, e->pco0, e->udot, e->f0u,
                    e->acc_u, e->stage_buf, e->sims_d, e->t_scale, e->tsum_part, e->steps_d,
                    e->pair_count, e->err, e->err_any, e->rebin_gate, e->restage_far,
                    e->bin_count,
                    e->chunk_sim, e->chunk_start,
                    e->chunk_len, e->cell_xyz};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    const CollideSet &c = e->coll;
    void *cp[] = {c.row_count, c.row_start, c.scan_tmp, c.ci,   c.cj,    c.dr[0],
                  c.dr[1],     c.dr[2],     c.rij,      c.src,  c.touch_count,
                  c.touch_start, c.touch_fill, c.touch, c.pred, c.level, c.info};
    for (void *p : cp)
        if (p) cudaFree(p);
    cluster_free(e);
    void *vp[] = {e->vl.ent, e->vl.cnt, e->vl.x0, e->vl.maxfill};
    for (void *p : vp)
        if (p) cudaFree(p);
    e->vl = VList{};
    e->vl_alloc = 0;
    if (e->cl_geom_d) cudaFree(e->cl_geom_d);
    e->cl_geom_d = nullptr;
    if (e->cl_fill_host) cudaFreeHost(e->cl_fill_host);
    if (e->cl_fill_ev) cudaEventDestroy(e->cl_fill_ev);
    e->cl_fill_host = nullptr;
    e->cl_fill_ev = nullptr;
    for (int a = 0; a < 3; ++a) {
        void *pa[] = {e->org[a], e->a_pos[a], e->a_vel[a], e->b_pos[a], e->b_vel[a], e->xe[0][a],
                      e->xe[1][a], e->ve[a], e->q[a], e->vdot[a], e->f0v[a], e->acc_r[a],
                      e->acc_v[a]};
        for (void *p : pa)
            if (p) cudaFree(p);
    }
}

// Moves every live particle to the front of A in the current sorted layout.
int compact(sph_engine *e) {
    TRY(ensure_layout(e));
    cudaStream_t st = e->stream;
    enqueue_prepare(e, st);
    size_t n = (size_t)e->np_b;
    for (int a = 0; a < e->dim; ++a) {
        CK(cudaMemcpyAsync(e->a_pos[a], e->b_pos[a], n * 8, cudaMemcpyDeviceToDevice, st));
        CK(cudaMemcpyAsync(e->a_vel[a], e->b_vel[a], n * 8, cudaMemcpyDeviceToDevice, st));
    }
    CK(cudaMemcpyAsync(e->a_u, e->b_u, n * 8, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(e->a_m, e->b_m, n * 8, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(e->a_id, e->b_id, n * 4, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(e->a_sim, e->b_sim, n * 4, cudaMemcpyDeviceToDevice, st));
    if ((int64_t)n < e->cap_p)
        CK(cudaMemsetAsync(e->a_sim + n, 0xff, (e->cap_p - n) * sizeof(int), st));
    CK(cudaStreamSynchronize(st));
    e->a_extent = (int)n;
    for (auto &S : e->sims)
        if (S.active) S.a_off = S.part_off;
    return SPH_OK;
}

}  // namespace

extern "C" {

const char *sph_status_string(int status) {
    switch (status) {
        case SPH_OK: return "SPH_OK";
        case SPH_EINVAL: return "SPH_EINVAL: invalid argument";
        case SPH_ENOMEM: return "SPH_ENOMEM: device allocation failed";
        case SPH_ECELL_OVERFLOW: return "SPH_ECELL_OVERFLOW: cell occupancy too large";
        case SPH_ETIMEOUT: return "SPH_ETIMEOUT: bounded device wait gave up";
        case SPH_ENAN: return "SPH_ENAN: non-finite density, pressure or rate";
        case SPH_ECUDA: return "SPH_ECUDA: CUDA runtime error";
        case SPH_ESKIN: return "SPH_ESKIN: displacement within a step exceeded the cell slack";
        case SPH_ECAPACITY: return "SPH_ECAPACITY: engine capacity exceeded";
        case SPH_ENOTFOUND: return "SPH_ENOTFOUND: unknown simulation id";
        case SPH_EBOUNDS: return "SPH_EBOUNDS: an index check failed";
        default: return "unknown status";
    }
}

int sph_version(void) { return 10000; }

int sph_engine_create(sph_engine **out, const sph_params *group, int32_t precision,
                      int64_t max_particles, int32_t max_sims, void *stream) {
    if (!out || !group) return SPH_EINVAL;
    *out = nullptr;
    if (group->dim != 2 && group->dim != 3) return SPH_EINVAL;
    if (group->kernel < 1 || group->kernel > 4) return SPH_EINVAL;
    if (group->integrator < 0 || group->integrator > 2) return SPH_EINVAL;
    if (group->collision != SPH_COLLIDE_OFF && group->collision != SPH_COLLIDE_EXCHANGE)
        return SPH_EINVAL;
    if (precision != SPH_FP64 && precision != SPH_MIXED) return SPH_EINVAL;
    if (max_particles <= 0 || max_particles > (int64_t)0x7fffffff / 2 || max_sims <= 0)
        return SPH_EINVAL;
    sph_engine *e = new sph_engine();
    e->group = *group;
    e->precision = precision;
    e->dim = group->dim;
    e->nstage = nstage_of(group->integrator);
    e->rsize = precision == SPH_MIXED ? 4 : 8;
    e->v4size = precision == SPH_MIXED ? 16 : 32;
    e->cap_p = max_particles;
    e->cap_s = max_sims;
    e->tune.block_size = 128;
    e->tune.rebin = 0;
    // measured on GB300: half-cutoff cells in 2D and 3D (autotune.py re-tunes)
    e->tune.cell_ratio = 0.5;
    e->tune.use_graph = 1;
    e->tune.steps_per_graph = 1;
    e->tune.pair_scheme = 0;
    e->tune.persistent = 0;
    // measured on GB300 (2D 1M fluid): 0.02-0.03 of the cutoff balance the
    // lists' length against how often they are built
    e->tune.list_skin = 0.025;
    if (stream) {
        e->stream = (cudaStream_t)stream;
    } else {
        if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess) {
            delete e;
            return SPH_ECUDA;
        }
        e->own_stream = true;
    }
    int st = alloc_particles(e);
    if (st == SPH_OK) st = alloc_sims(e);
    if (st == SPH_OK) st = alloc_cells(e, 1024);
    if (st != SPH_OK) {
        free_all(e);
        if (e->own_stream) cudaStreamDestroy(e->stream);
        delete e;
        return st;
    }
    *out = e;
    return SPH_OK;
}

int sph_engine_destroy(sph_engine *e) {
    if (!e) return SPH_EINVAL;
    cudaStreamSynchronize(e->stream);
    free_all(e);
    for (cudaEvent_t ev : e->prof_pool) cudaEventDestroy(ev);
    if (e->own_stream) cudaStreamDestroy(e->stream);
    delete e;
    return SPH_OK;
}

int sph_sim_add(sph_engine *e, const sph_params *p, int64_t n, const double *r, const double *v,
                const double *m, const double *u, int32_t mem, int32_t *sim_id) {
    if (!e || !p || !r || !v || !m || !u || !sim_id || n <= 0) return SPH_EINVAL;
    TRY(validate_params(e, p));
    // simulation slot
    int id = -1;
    for (int s = 0; s < (int)e->sims.size(); ++s)
        if (!e->sims[s].active) {
            id = s;
            break;
        }
    if (id < 0) {
        if ((int)e->sims.size() >= e->cap_s) return SPH_ECAPACITY;
        id = (int)e->sims.size();
        e->sims.emplace_back();
    }
    int64_t live = 0;
    for (auto &S : e->sims)
        if (S.active) live += S.n;
    if (live + n > e->cap_p) return SPH_ECAPACITY;
    if (e->a_extent + n > e->cap_p) TRY(compact(e));
    // velocity bound for the cell slack and a host-side position check
    std::vector<double> hv((size_t)n * p->dim), hr((size_t)n * p->dim);
    cudaMemcpyKind k = mem == SPH_DEVICE ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost;
    CK(cudaMemcpy(hv.data(), v, sizeof(double) * hv.size(), k));
    CK(cudaMemcpy(hr.data(), r, sizeof(double) * hr.size(), k));
    double vmax = 0.0;
    for (double x : hv) vmax = std::max(vmax, std::fabs(x));
    for (int64_t i = 0; i < n; ++i)
        for (int a = 0; a < p->dim; ++a) {
            double x = hr[(size_t)i * p->dim + a];
            // within a quarter box of [0, L]: the reference's single minimum-image
            // shift then equals the true minimum image for every pair
            if (!(x >= -0.25 * p->box[a] && x <= 1.25 * p->box[a])) return SPH_EINVAL;
        }
    Sim &S = e->sims[id];
    S = Sim();
    S.prm = *p;
    S.n = n;
    S.vmax = vmax;
    make_grid(S, e->dim, e->tune.cell_ratio, list_skin_of(e));
    int off = e->a_extent;
    TRY(write_state_range(e, off, n, r, v, m, u, mem));
    launch_iota_sim(e->a_id + off, e->a_sim + off, id, (int)n, e->stream);
    CK(cudaMemsetAsync(e->err + id, 0, sizeof(int), e->stream));
    CK(cudaMemsetAsync(e->steps_d + id, 0, sizeof(long long), e->stream));
    CK(cudaStreamSynchronize(e->stream));
    S.active = true;
    S.a_off = off;
    e->a_extent += (int)n;
    e->layout_dirty = true;
    e->props_valid = false;
    e->bins_valid = false;
    *sim_id = id;
    return SPH_OK;
}

int sph_sim_remove(sph_engine *e, int32_t id) {
    TRY(check_sim(e, id));
    Sim &S = e->sims[id];
    launch_fill_int(e->a_sim + S.a_off, -1, (int)S.n, e->stream);
    CK(cudaStreamSynchronize(e->stream));
    S.active = false;
    e->layout_dirty = true;
    e->props_valid = false;
    e->bins_valid = false;
    return SPH_OK;
}

int sph_sim_set_state(sph_engine *e, int32_t id, const double *r, const double *v,
                      const double *m, const double *u, int32_t mem) {
    TRY(check_sim(e, id));
    const bool all = r && v && m && u;
    // the state is given in original order, which holds for a full update
    // only (checked before anything is written)
    if (!all && (r || v || m || u)) return SPH_EINVAL;
    Sim &S = e->sims[id];
    // A holds the simulation in slot order a_off + k with id[k]; the caller
    // gives original order, so reset ids to identity for the range.
    TRY(write_state_range(e, S.a_off, S.n, r, v, m, u, mem));
    if (all) launch_iota_sim(e->a_id + S.a_off, e->a_sim + S.a_off, id, (int)S.n, e->stream);
    // With binning on demand the current cells (and pair lists) are kept
    // when the new state lies within their slack: it goes straight into the
    // simulation's B slots in the current order.  Otherwise the next step
    // bins (and measures the lists) again.
    bool kept = false;
    if (all && rebin_on_demand(e) && e->bins_valid && !e->layout_dirty && !e->cl.on &&
        (!e->vl.on || (e->vl.ent && !e->cl_stale))) {
        cudaStream_t st = e->stream;
        int far = 1;
        CK(cudaMemsetAsync(e->restage_far, 0, sizeof(int), st));
        View vw = make_view(e);
        stage_view(e, vw, 0);
        launch_restage(vw, e->precision, S.a_off, S.part_off, (int)S.n, e->restage_far, st);
        CK(cudaMemcpyAsync(&far, e->restage_far, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        kept = far == 0;
    } else {
        CK(cudaStreamSynchronize(e->stream));
    }
    e->props_valid = false;
    if (!kept) {
        e->bins_valid = false;
        e->cl_stale = true;
    }
    return SPH_OK;
}

int sph_sim_get_state(sph_engine *e, int32_t id, double *r, double *v, double *u, int32_t mem) {
    TRY(check_sim(e, id));
    Sim &S = e->sims[id];
    cudaStream_t st = e->stream;
    int n = (int)S.n;
    // each component in its own staging region: the copies follow their
    // gathers back to back, and one wait at the end covers them all
    const size_t P = (size_t)e->cap_p;
    if (r) {
        double *d = mem == SPH_DEVICE ? r : e->stage_buf + kStageR * P;
        launch_store_aos(d, e->a_pos, e->a_id, S.a_off, n, e->dim, st);
        TRY(copy_out(e, r, (size_t)n * e->dim, mem, d));
    }
    if (v) {
        double *d = mem == SPH_DEVICE ? v : e->stage_buf + kStageV * P;
        launch_store_aos(d, e->a_vel, e->a_id, S.a_off, n, e->dim, st);
        TRY(copy_out(e, v, (size_t)n * e->dim, mem, d));
    }
    if (u) {
        double *d = mem == SPH_DEVICE ? u : e->stage_buf + kStageU * P;
        launch_store_scalar(d, e->a_u, e->a_id, S.a_off, n, st);
        TRY(copy_out(e, u, (size_t)n, mem, d));
    }
    if (mem == SPH_HOST) CK(cudaStreamSynchronize(st));
    CK(cudaGetLastError());
    return SPH_OK;
}

int sph_sim_count(sph_engine *e, int32_t id, int64_t *n) {
    TRY(check_sim(e, id));
    if (!n) return SPH_EINVAL;
    *n = e->sims[id].n;
    return SPH_OK;
}

int sph_sim_steps(sph_engine *e, int32_t id, int64_t *steps) {
    TRY(check_sim(e, id));
    if (!steps) return SPH_EINVAL;
    *steps = e->sims[id].steps;
    return SPH_OK;
}

int sph_sim_set_steps(sph_engine *e, int32_t id, int64_t steps) {
    TRY(check_sim(e, id));
    if (steps < 0) return SPH_EINVAL;
    long long s = (long long)steps;
    CK(cudaMemcpyAsync(e->steps_d + id, &s, sizeof(s), cudaMemcpyHostToDevice, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    e->sims[id].steps = steps;
    return SPH_OK;
}

// Steps per graph launch with cluster pairs: a long advance runs in chunks
// of at most kClMaxChunk steps (a longer graph is split into even chunks of
// about kClChunk), and the longest list of each chunk is checked while the
// next one runs.
constexpr int kClChunk = 20, kClMaxChunk = 32;

// Between two chunks of an advance with cluster pairs: waits for the longest
// list of the chunk before the one just queued (finished by now; the queued
// chunk keeps the device busy), queues the read of the one just queued, and
// reports whether a region was filled past 80% (re-measure before more steps).
int cluster_between(sph_engine *e, bool *over) {
    if (e->cl_fill_pending) {
        CK(cudaEventSynchronize(e->cl_fill_ev));
        e->cl_fill_pending = false;
        if (*e->cl_fill_host > 0.8 * list_room(e)) e->cl_stale = true;
    }
    TRY(cluster_note_fill(e));
    *over = e->cl_stale;
    return SPH_OK;
}

// Steps per graph launch of an advance.
int graph_chunk(const sph_engine *e) {
    const int per = std::max(1, e->tune.steps_per_graph);
    if (!lists_on(e) || per <= kClMaxChunk) return per;
    const int n = (per + kClChunk - 1) / kClChunk;
    return (per + n - 1) / n;
}

// Queues up to n steps in the current layout; stops early (*ran < n) when a
// cluster list region needs re-measuring before further steps.
int advance_span(sph_engine *e, int n, int *ran) {
    cudaStream_t st = e->stream;
    const bool cl = lists_on(e);
    const int per = graph_chunk(e);
    int done = 0;
    *ran = 0;
    if (e->prof_on) TRY(ensure_prof_pool(e, e->prof_used + (size_t)n * 2 * (1 + 4 * e->nstage) + 8));
    if (rebin_on_demand(e) && !e->bins_valid) {
        // the state or the layout changed since the last step: bin first
        launch_fill_int(e->rebin_gate, 1, 1, st);
        e->bins_valid = true;
    }
    // The binning pass covers A's used extent.  After simulations joined or
    // left, A holds dropped or unsorted particles beyond the live count;
    // that first step runs eagerly, after which A is compact (extent == live).
    if (e->a_extent != e->np_b) {
        enqueue_step(e, st);
        after_advance(e, 1);
        ++done;
    }
    while (done < n) {
        int k;
        if (e->tune.use_graph && n - done >= per) {
            TRY(build_graph(e, per));
            CK(cudaGraphLaunch(e->graph_exec, st));
            e->graph_launched = true;
            k = per;
        } else {
            k = cl ? std::min(n - done, per) : n - done;
            for (int i = 0; i < k; ++i) enqueue_step(e, st);
        }
        after_advance(e, k);
        done += k;
        if (cl) {
            bool over = false;
            TRY(cluster_between(e, &over));
            if (over) break;
        }
    }
    *ran = done;
    return SPH_OK;
}

int sph_advance(sph_engine *e, int32_t nsteps) {
    if (!e || nsteps < 0) return SPH_EINVAL;
    int done = 0;
    while (done < nsteps) {
        TRY(ensure_layout(e));
        if (e->np_b == 0) return SPH_OK;
        TRY(cluster_check(e));
        int ran = 0;
        TRY(advance_span(e, nsteps - done, &ran));
        done += ran;
    }
    CK(cudaGetLastError());
    return SPH_OK;
}

int sph_sim_derivatives(sph_engine *e, int32_t id, double *rho, double *rho_lr, double *t,
                        double *p, double *pco, double *vdot, double *udot, double *jq,
                        int32_t mem) {
    TRY(check_sim(e, id));
    TRY(ensure_layout(e));
    TRY(cluster_check(e));
    cudaStream_t st = e->stream;
    enqueue_prepare(e, st);
    enqueue_stage(e, 0, 0, st);
    CK(cudaGetLastError());
    e->props_valid = true;
    const Sim &S = e->sims[id];
    TRY(gather_R(e, S, e->rho, rho, mem));
    TRY(gather_R(e, S, e->rho_l, rho_lr, mem));
    TRY(gather_R(e, S, e->temp, t, mem));
    TRY(gather_R(e, S, e->pres, p, mem));
    TRY(gather_R(e, S, e->pco, pco, mem));
    TRY(gather_R(e, S, e->udot, udot, mem));
    TRY(gather_R_vec(e, S, e->vdot, vdot, mem));
    if (jq) {
        if (e->group.heat_flux) TRY(gather_R_vec(e, S, e->q, jq, mem));
        else if (mem == SPH_DEVICE) CK(cudaMemsetAsync(jq, 0, sizeof(double) * S.n * e->dim, st));
        else memset(jq, 0, sizeof(double) * S.n * e->dim);
    }
    CK(cudaStreamSynchronize(st));
    return SPH_OK;
}

int sph_sim_get_properties(sph_engine *e, int32_t id, double *rho, double *rho_lr, double *t,
                           double *p, double *pco, double *vdot, double *udot, double *jq,
                           int32_t mem) {
    TRY(check_sim(e, id));
    if (!e->props_valid || e->layout_dirty) return sph_sim_derivatives(e, id, rho, rho_lr, t, p, pco, vdot, udot, jq, mem);
    const Sim &S = e->sims[id];
    TRY(gather_R(e, S, e->rho0, rho, mem));
    TRY(gather_R(e, S, e->rho_l, rho_lr, mem));
    TRY(gather_R(e, S, e->temp, t, mem));
    TRY(gather_R(e, S, e->pres0, p, mem));
    TRY(gather_R(e, S, e->pco0, pco, mem));
    TRY(gather_R(e, S, e->udot, udot, mem));
    TRY(gather_R_vec(e, S, e->vdot, vdot, mem));
    if (jq) {
        if (e->group.heat_flux) TRY(gather_R_vec(e, S, e->q, jq, mem));
        else if (mem == SPH_DEVICE) CK(cudaMemsetAsync(jq, 0, sizeof(double) * S.n * e->dim, e->stream));
        else memset(jq, 0, sizeof(double) * S.n * e->dim);
    }
    CK(cudaStreamSynchronize(e->stream));
    return SPH_OK;
}

int sph_sim_pair_count(sph_engine *e, int32_t id, int64_t *nip) {
    TRY(check_sim(e, id));
    if (!nip) return SPH_EINVAL;
    TRY(ensure_layout(e));
    TRY(cluster_check(e));
    cudaStream_t st = e->stream;
    if (e->cl.on) {
        // simulations on cluster pairs count in the cluster density pass
        enqueue_prepare(e, st);
        enqueue_stage(e, 0, 0, st);
    } else {
        enqueue_prepare(e, st);
        View v = make_view(e);
        stage_view(e, v, 0);
        launch_density(v, e->precision, e->group.kernel, 0, e->tune.block_size, st);
    }
    unsigned long long c = 0;
    CK(cudaMemcpyAsync(&c, e->pair_count + id, sizeof(c), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    *nip = (int64_t)(c / 2);
    return SPH_OK;
}

int sph_sim_export_pairs(sph_engine *e, int32_t id, int64_t cap, int64_t *iap, double *drij,
                         double *rsq, double *dv, int64_t *nip, int32_t mem) {
    TRY(check_sim(e, id));
    if (!nip) return SPH_EINVAL;
    TRY(ensure_layout(e));
    cudaStream_t st = e->stream;
    enqueue_prepare(e, st);
    const Sim &S = e->sims[id];
    View v = make_view(e);
    stage_view(e, v, 0);
    long long *rows = nullptr;
    TRY(dalloc(&rows, (size_t)S.n + 1));
    CK(cudaMemsetAsync(rows, 0, sizeof(long long) * (S.n + 1), st));
    launch_pair_rows(v, e->precision, S.part_off, (int)S.n, rows, st);
    launch_scan64(rows, (int)S.n, st);
    long long total = 0;
    CK(cudaMemcpyAsync(&total, rows + S.n, sizeof(total), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    *nip = total;
    if (total > cap) {
        cudaFree(rows);
        return SPH_ECAPACITY;
    }
    if (total > 0 && (iap || drij || rsq || dv)) {
        long long *d_iap = nullptr;
        double *d_drij = nullptr, *d_rsq = nullptr, *d_dv = nullptr;
        bool host = mem == SPH_HOST;
        int st1 = SPH_OK;
        if (host || !iap) st1 = dalloc(&d_iap, (size_t)total * 2);
        else d_iap = (long long *)iap;
        if (st1 == SPH_OK && drij) {
            if (host) st1 = dalloc(&d_drij, (size_t)total * e->dim);
            else d_drij = drij;
        }
        if (st1 == SPH_OK && rsq) {
            if (host) st1 = dalloc(&d_rsq, (size_t)total);
            else d_rsq = rsq;
        }
        if (st1 == SPH_OK && dv) {
            if (host) st1 = dalloc(&d_dv, (size_t)total * e->dim);
            else d_dv = dv;
        }
        if (st1 == SPH_OK) {
            launch_pair_write(v, e->precision, S.part_off, (int)S.n, rows, d_iap, d_drij, d_rsq,
                              d_dv, st);
            if (host) {
                if (iap) cudaMemcpyAsync(iap, d_iap, sizeof(long long) * total * 2, cudaMemcpyDeviceToHost, st);
                if (drij) cudaMemcpyAsync(drij, d_drij, sizeof(double) * total * e->dim, cudaMemcpyDeviceToHost, st);
                if (rsq) cudaMemcpyAsync(rsq, d_rsq, sizeof(double) * total, cudaMemcpyDeviceToHost, st);
                if (dv) cudaMemcpyAsync(dv, d_dv, sizeof(double) * total * e->dim, cudaMemcpyDeviceToHost, st);
            }
            cudaStreamSynchronize(st);
        }
        if (host || !iap) cudaFree(d_iap);
        if (host) {
            cudaFree(d_drij);
            cudaFree(d_rsq);
            cudaFree(d_dv);
        }
        if (st1 != SPH_OK) {
            cudaFree(rows);
            return st1;
        }
    }
    cudaFree(rows);
    CK(cudaGetLastError());
    return SPH_OK;
}

int sph_last_pair_total(sph_engine *e, int64_t *pairs) {
    if (!e || !pairs) return SPH_EINVAL;
    std::vector<unsigned long long> c(e->cap_s);
    CK(cudaMemcpyAsync(c.data(), e->pair_count, sizeof(unsigned long long) * e->cap_s,
                       cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    unsigned long long t = 0;
    for (int s = 0; s < (int)e->sims.size(); ++s)
        if (e->sims[s].active) t += c[s];
    *pairs = (int64_t)(t / 2);
    return SPH_OK;
}

int sph_last_pair_counts(sph_engine *e, int64_t *counts, int32_t cap) {
    if (!e || !counts || cap < 0) return SPH_EINVAL;
    std::vector<unsigned long long> c(e->cap_s);
    CK(cudaMemcpyAsync(c.data(), e->pair_count, sizeof(unsigned long long) * e->cap_s,
                       cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    for (int s = 0; s < cap; ++s) {
        const bool live = s < (int)e->sims.size() && e->sims[s].active;
        counts[s] = live ? (int64_t)(c[s] / 2) : 0;
    }
    return SPH_OK;
}

int sph_sim_diagnostics(sph_engine *e, int32_t id, double out[6]) {
    TRY(check_sim(e, id));
    if (!out) return SPH_EINVAL;
    const Sim &S = e->sims[id];
    size_t n = (size_t)S.n, d = (size_t)e->dim;
    std::vector<double> v(n * d), u(n), m(n), t(n, 0.0);
    TRY(sph_sim_get_state(e, id, nullptr, v.data(), u.data(), SPH_HOST));
    CK(cudaMemcpy(m.data(), e->a_m + S.a_off, sizeof(double) * n, cudaMemcpyDeviceToHost));
    double ke = 0, ue = 0, mom[3] = {0, 0, 0}, tav = 0;
    for (size_t i = 0; i < n; ++i) {
        double v2 = 0;
        for (size_t a = 0; a < d; ++a) {
            v2 += v[i * d + a] * v[i * d + a];
            mom[a] += m[i] * v[i * d + a];
        }
        ke += 0.5 * m[i] * v2;
        ue += u[i];
    }
    if (e->props_valid && !e->layout_dirty) {
        TRY(gather_R(e, S, e->temp, t.data(), SPH_HOST));
        for (double x : t) tav += x;
        tav /= (double)n;
    }
    out[0] = ke;
    out[1] = ue;
    out[2] = mom[0];
    out[3] = mom[1];
    out[4] = mom[2];
    out[5] = tav;
    return SPH_OK;
}

int sph_get_tuning(sph_engine *e, sph_tuning *t) {
    if (!e || !t) return SPH_EINVAL;
    *t = e->tune;
    return SPH_OK;
}

int sph_set_tuning(sph_engine *e, const sph_tuning *t) {
    if (!e || !t) return SPH_EINVAL;
    if (t->block_size < 32 || t->block_size > 256 || (t->block_size & 31) ||
        !(t->cell_ratio >= 0.2 && t->cell_ratio <= 4.0) || (t->rebin != 0 && t->rebin != 1) ||
        t->steps_per_graph < 1 || t->pair_scheme < 0 || t->pair_scheme > 2 ||
        (t->persistent != 0 && t->persistent != 1) ||
        !(t->list_skin >= 0.01 && t->list_skin <= 0.5))
        return SPH_EINVAL;
    // the grid's reach holds the pair lists' skin
    const double skin_old = list_skin_of(e);
    bool regrid = t->cell_ratio != e->tune.cell_ratio;
    if (t->pair_scheme != e->tune.pair_scheme) {
        e->layout_dirty = true;
        e->cl_disabled = false;
        e->vl_disabled = false;
    }
    e->tune = *t;
    regrid |= list_skin_of(e) != skin_old;
    free_graph(e);
    if (regrid) {
        for (auto &S : e->sims)
            if (S.active) make_grid(S, e->dim, e->tune.cell_ratio, list_skin_of(e));
        e->layout_dirty = true;
        e->props_valid = false;
    }
    e->bins_valid = false;
    return SPH_OK;
}

int sph_rebin_count(sph_engine *e, int64_t *n) {
    if (!e || !n) return SPH_EINVAL;
    unsigned long long c = 0;
    CK(cudaMemcpyAsync(&c, e->bin_count, sizeof(c), cudaMemcpyDeviceToHost, e->stream));
    CK(cudaStreamSynchronize(e->stream));
    *n = (int64_t)c;
    return SPH_OK;
}

int sph_prepare(sph_engine *e) {
    if (!e) return SPH_EINVAL;
    TRY(ensure_layout(e));
    if (e->np_b == 0 || !e->tune.use_graph) return SPH_OK;
    TRY(cluster_check(e));
    if (e->a_extent != e->np_b) return SPH_OK;  // first step after a change runs eagerly
    return build_graph(e, graph_chunk(e));
}

int sph_profile(sph_engine *e, int32_t enable) {
    if (!e) return SPH_EINVAL;
    CK(cudaStreamSynchronize(e->stream));
    bool on = enable != 0;
    if (on != e->prof_on) free_graph(e);
    e->prof_on = on;
    e->prof_recs.clear();
    e->prof_used = 0;
    if (on) TRY(ensure_prof_pool(e, 64));
    return SPH_OK;
}

int sph_profile_read(sph_engine *e, double ms[5], int64_t launches[5]) {
    if (!e || !ms || !launches) return SPH_EINVAL;
    CK(cudaStreamSynchronize(e->stream));
    for (int k = 0; k < SPH_NPASS; ++k) {
        ms[k] = 0.0;
        launches[k] = 0;
    }
    for (auto &r : e->prof_recs) {
        float t = 0.0f;
        if (cudaEventElapsedTime(&t, r.a, r.b) != cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        ms[r.kind] += t;
        launches[r.kind] += r.kind == SPH_PASS_SORT ? kSortKernels : (r.kind == SPH_PASS_TSUM ? 2 : 1);
    }
    return SPH_OK;
}

int sph_kernels_per_step(sph_engine *e, int64_t *n) {
    if (!e || !n) return SPH_EINVAL;
    TRY(ensure_layout(e));
    *n = kernels_per_step(e);
    return SPH_OK;
}

int sph_sync(sph_engine *e) {
    if (!e) return SPH_EINVAL;
    CK(cudaStreamSynchronize(e->stream));
    CK(cudaGetLastError());
    int code = 0;
    CK(cudaMemcpy(&code, e->err_any, sizeof(int), cudaMemcpyDeviceToHost));
    if (code) CK(cudaMemset(e->err_any, 0, sizeof(int)));
    return code;
}

int sph_sim_status(sph_engine *e, int32_t id, int32_t *status) {
    TRY(check_sim(e, id));
    if (!status) return SPH_EINVAL;
    CK(cudaStreamSynchronize(e->stream));
    CK(cudaMemcpy(status, e->err + id, sizeof(int), cudaMemcpyDeviceToHost));
    return SPH_OK;
}

}  // extern "C"

namespace sph {

double kernel_sigma(int kernel, int dim, double h) {
    const double pi = 3.14159265358979323846;
    switch (kernel) {
        case SPH_KERNEL_LUCY:
            return dim == 2 ? 5.0 / (pi * h * h) : 105.0 / (pi * 16.0 * (h * h * h));
        case SPH_KERNEL_GAUSSIAN:
            return 1.0 / (std::pow(h, dim) * std::pow(pi, dim / 2.0));
        case SPH_KERNEL_DEBRUN: {
            double h2 = h * h, h6 = h2 * h2 * h2;
            return dim == 2 ? 10.0 / (pi * h6) : 15.0 / (pi * h6);
        }
        default:
            return dim == 2 ? 10.0 / (7.0 * pi * h * h) : 1.0 / (pi * h * h * h);
    }
}

// Host-side tables of one simulation laid out on its own (cell offset 0,
// particle offset 0): device constants, linear-cell -> Morton map and packed
// cell coordinates, for callers that provide all device memory themselves.
// cell_ratio as in sph_tuning; vmax bounds |v| for the cell slack.
int single_sim_tables(const sph_params *p, int64_t n, double cell_ratio, double vmax,
                      SimDev *dev, std::vector<int> *morton, std::vector<int> *cell_xyz) {
    if (!p || !dev || !morton || !cell_xyz || n <= 0) return SPH_EINVAL;
    sph_engine cfg;
    cfg.group = *p;
    cfg.dim = p->dim;
    int st = validate_params(&cfg, p);
    if (st != SPH_OK) return st;
    Sim S;
    S.prm = *p;
    S.n = n;
    S.vmax = vmax;
    S.active = true;
    make_grid(S, p->dim, cell_ratio);
    S.cell_off = 0;
    S.part_off = 0;
    *dev = make_simdev(&cfg, S);
    *morton = S.morton;
    cell_xyz->assign(S.ncells, 0);
    for (int r = 0; r < S.ncells; ++r) {
        int lin = S.rank_lin[r];
        int c0 = lin % S.nc[0], c1 = (lin / S.nc[0]) % S.nc[1], c2 = lin / (S.nc[0] * S.nc[1]);
        (*cell_xyz)[r] = c0 | (c1 << 11) | (c2 << 22);
    }
    return SPH_OK;
}

}  // namespace sph
