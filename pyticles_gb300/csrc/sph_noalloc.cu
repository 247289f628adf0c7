// sph_noalloc.cu -- one derivative evaluation of one simulation with no
// device allocation at all.
//
// The engine (sph_engine.cu) owns its working memory and grows it with
// cudaMalloc.  Some callers cannot let a library allocate: a host application
// or framework that budgets the whole device up front and hands out memory
// only from its own pool, or a latency-critical loop that may not block in
// the allocator.  For them, sph_derivatives_noalloc runs the same sort,
// density, heat and force passes on caller-owned inputs and outputs, with
// every intermediate array carved out of one statically sized device array
// (g_noalloc_scratch below, SPH_NOALLOC_SCRATCH_BYTES bytes, held by every
// GPU that loads the library until the process exits).
//
// The array is shared by all calls and keeps the last call's contents: each
// call rewrites everything it reads and clears what must start at zero (cell
// counts, pair counts, error words).  Calls whose work overlaps on the GPU --
// from two threads, or on two streams without ordering -- race on it.
#include <mutex>
#include <vector>

#include "sph_internal.h"

namespace sph {
int single_sim_tables(const sph_params *p, int64_t n, double cell_ratio, double vmax,
                      SimDev *dev, std::vector<int> *morton, std::vector<int> *cell_xyz);
}

using namespace sph;

namespace {

constexpr size_t kAlign = 256;
// Per particle, in FP64 (the larger case), what sph_derivatives_noalloc
// carves below: positions and velocities of states A and B and the cell
// origins (5 x 3 x 8), the heat-flux and vdot components (2 x 3 x 8), u and m
// of A and B (4 x 8), ids, simulations and sort scratch (9 x 4), five packed
// vectors -- position, velocity, force factors, heat factors, neighbour
// record -- (5 x 32), nine scalar outputs (9 x 8) and one output staging
// column (8): 476 B, within the 512 B budgeted.  Per cell: count, start,
// Morton rank, coordinates.  The per-array alignment padding is covered by
// the 256 KiB added to the total.
constexpr size_t kBytesUsedPerParticle =
    5 * 3 * 8 + 2 * 3 * 8 + 4 * 8 + 9 * 4 + 5 * 32 + 9 * 8 + 8;
constexpr size_t kBytesPerParticle = 512;
static_assert(kBytesUsedPerParticle <= kBytesPerParticle,
              "the per-particle carving outgrew the scratch budget");
constexpr size_t kBytesPerCell = 32;
constexpr size_t kScratchBytes = (size_t)SPH_NOALLOC_MAX_PARTICLES * kBytesPerParticle +
                                 (size_t)SPH_NOALLOC_MAX_CELLS * kBytesPerCell + (256u << 10);
static_assert(kScratchBytes == SPH_NOALLOC_SCRATCH_BYTES, "header and scratch size disagree");

// The scratch itself.  In host code this name is only a stand-in for the
// device symbol: its address must come from cudaGetSymbolAddress on the
// current device before a kernel may use it.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mu;
constexpr int kMaxDevices = 256;
void *g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch on the current device, looked up once per
// device (the first call on a device performs this set-up).
int scratch_address(void **out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return SPH_ECUDA;
    }
    if (dev < 0 || dev >= kMaxDevices) return SPH_EINVAL;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return SPH_ECUDA;
        }
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return SPH_OK;
}

struct Carver {
    char *base;
    size_t off, cap;
    bool ok = true;
    template <typename T>
    T *take(size_t count) {
        size_t o = (off + kAlign - 1) / kAlign * kAlign;
        size_t bytes = count * sizeof(T);
        if (o + bytes > cap) {
            ok = false;
            return nullptr;
        }
        off = o + bytes;
        return (T *)(base + o);
    }
};

#define NA_CK(call)                            \
    do {                                       \
        if ((call) != cudaSuccess) {           \
            cudaGetLastError();                \
            return SPH_ECUDA;                  \
        }                                      \
    } while (0)

}  // namespace

extern "C" int sph_derivatives_noalloc(const sph_params *p, int32_t precision, int64_t n,
                                       const double *r, const double *v, const double *m,
                                       const double *u, double *rho, double *rho_lr,
                                       double *t, double *pres, double *pco, double *vdot,
                                       double *udot, double *jq, void *stream) {
    if (!p || !r || !v || !m || !u) return SPH_EINVAL;
    if (precision != SPH_FP64 && precision != SPH_MIXED) return SPH_EINVAL;
    if (p->dim != 2 && p->dim != 3) return SPH_EINVAL;
    if (p->kernel < 1 || p->kernel > 4) return SPH_EINVAL;
    if (n <= 0 || n > SPH_NOALLOC_MAX_PARTICLES) return SPH_EINVAL;  // size limit
    const int dim = p->dim;
    cudaStream_t st = (cudaStream_t)stream;

    // host-side layout (the engine's default cells of half the cutoff, so the
    // summation order is the engine's); coarser cells if the box needs more
    // than the cell limit
    SimDev sd;
    std::vector<int> morton, cxyz;
    const double ratios[] = {0.5, 1.0, 2.0, 4.0};
    int status = SPH_ECAPACITY;
    for (double ratio : ratios) {
        status = single_sim_tables(p, n, ratio, 0.0, &sd, &morton, &cxyz);
        if (status != SPH_OK) return status;
        if ((int64_t)morton.size() <= SPH_NOALLOC_MAX_CELLS) break;
        status = SPH_ECAPACITY;
    }
    if ((int64_t)morton.size() > SPH_NOALLOC_MAX_CELLS) return SPH_ECAPACITY;
    const int ncells = (int)morton.size();
    sd.n = (int)n;

    void *base = nullptr;
    int s0 = scratch_address(&base);
    if (s0 != SPH_OK) return s0;

    // carve the scratch
    const size_t rs = precision == SPH_MIXED ? 4 : 8, v4 = 4 * rs;
    Carver c{(char *)base, 0, kScratchBytes};
    const size_t N = (size_t)n;
    View w;
    memset(&w, 0, sizeof(w));
    w.np = (int)n;
    w.dim = dim;
    w.sims = c.take<SimDev>(1);
    for (int a = 0; a < 3; ++a) {
        w.a_pos[a] = c.take<double>(N);
        w.a_vel[a] = c.take<double>(N);
        w.b_pos[a] = c.take<double>(N);
        w.b_vel[a] = c.take<double>(N);
        w.org[a] = c.take<double>(N);
        w.q[a] = c.take<char>(N * rs);
        w.vdot[a] = c.take<char>(N * rs);
    }
    w.a_u = c.take<double>(N);
    w.a_m = c.take<double>(N);
    w.a_id = c.take<int>(N);
    w.a_sim = c.take<int>(N);
    w.b_u = c.take<double>(N);
    w.b_m = c.take<double>(N);
    w.b_id = c.take<int>(N);
    w.b_sim = c.take<int>(N);
    w.cell_of = c.take<int>(N);
    w.rank = c.take<int>(N);
    w.order_tmp = c.take<int>(N);
    w.order = c.take<int>(N);
    w.cell_b = c.take<int>(N);
    w.cell_count = c.take<int>((size_t)ncells);
    w.cell_start = c.take<int>((size_t)ncells + 1);
    w.morton = c.take<int>((size_t)ncells);
    w.cell_xyz = c.take<int>((size_t)ncells);
    int *scan_tmp = c.take<int>((size_t)ncells / 4096 + 2);
    w.pk_pos_in = w.pk_pos_out = c.take<char>(N * v4);
    w.pk_vel_in = w.pk_vel_out = c.take<char>(N * v4);
    w.pk_f = c.take<char>(N * v4);
    w.pk_q = c.take<char>(N * v4);
    w.pk_fv = c.take<char>(N * v4);
    void **scalars[] = {&w.rho, &w.rho_l, &w.temp, &w.pres, &w.pco, &w.rho0, &w.pres0, &w.pco0,
                        &w.udot};
    for (void **sp : scalars) *sp = c.take<char>(N * rs);
    double *column = c.take<double>(N);
    w.pair_count = c.take<unsigned long long>(1);
    w.err = c.take<int>(1);
    w.err_any = c.take<int>(1);
    w.t_scale = c.take<double>(1);
    w.steps = c.take<long long>(1);
    if (!c.ok) return SPH_ECAPACITY;
    // the first evaluation reads the sorted state itself
    for (int a = 0; a < 3; ++a) {
        w.xe_in[a] = w.b_pos[a];
        w.ve_in[a] = w.b_vel[a];
    }
    w.ue_in = w.b_u;

    // inputs and tables; what must start at zero is cleared here
    NA_CK(cudaMemcpyAsync(w.sims, &sd, sizeof(SimDev), cudaMemcpyHostToDevice, st));
    w.one_sim = 1;
    w.one = sd;
    NA_CK(cudaMemcpyAsync(w.morton, morton.data(), sizeof(int) * ncells, cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemcpyAsync(w.cell_xyz, cxyz.data(), sizeof(int) * ncells, cudaMemcpyHostToDevice, st));
    NA_CK(cudaMemsetAsync(w.err, 0, sizeof(int), st));
    NA_CK(cudaMemsetAsync(w.err_any, 0, sizeof(int), st));
    NA_CK(cudaMemsetAsync(w.pair_count, 0, sizeof(unsigned long long), st));
    NA_CK(cudaMemsetAsync(w.cell_count, 0, sizeof(int) * ncells, st));
    NA_CK(cudaMemsetAsync(w.pk_q, 0, N * v4, st));
    launch_load_aos(w.a_pos, r, (int)n, dim, st);
    launch_load_aos(w.a_vel, v, (int)n, dim, st);
    NA_CK(cudaMemcpyAsync(w.a_m, m, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
    NA_CK(cudaMemcpyAsync(w.a_u, u, sizeof(double) * N, cudaMemcpyDeviceToDevice, st));
    launch_iota_sim(w.a_id, w.a_sim, 0, (int)n, st);

    // the engine's passes: counting sort, density, heat, force (no state update)
    launch_bin(w, (int)n, st);
    launch_scan(w.cell_count, w.cell_start, ncells, scan_tmp, st);
    launch_scatter(w, (int)n, st);
    launch_cellsort(w, ncells, st);
    launch_permute(w, precision, st);
    launch_density(w, precision, p->kernel, 0, 128, st);
    if (p->heat_flux) launch_heat(w, precision, p->kernel, 128, st);
    launch_force(w, precision, p->kernel, p->viscosity, p->heat_flux, p->integrator, 0, 0, 128,
                 st);

    // outputs in the caller's particle order
    void *const *srcs[] = {&w.rho, &w.rho_l, &w.temp, &w.pres, &w.pco, &w.udot};
    double *dsts[] = {rho, rho_lr, t, pres, pco, udot};
    for (int k = 0; k < 6; ++k)
        if (dsts[k]) launch_store_R(dsts[k], *srcs[k], precision, w.b_id, 0, (int)n, st);
    double *vecs[] = {vdot, jq};
    void *const *vsrc[] = {w.vdot, w.q};
    for (int k = 0; k < 2; ++k) {
        if (!vecs[k]) continue;
        if (k == 1 && !p->heat_flux) {
            NA_CK(cudaMemsetAsync(jq, 0, sizeof(double) * N * dim, st));
            continue;
        }
        for (int a = 0; a < dim; ++a) {
            launch_store_R(column, vsrc[k][a], precision, w.b_id, 0, (int)n, st);
            NA_CK(cudaMemcpy2DAsync(vecs[k] + a, sizeof(double) * dim, column, sizeof(double),
                                    sizeof(double), N, cudaMemcpyDeviceToDevice, st));
        }
    }
    NA_CK(cudaGetLastError());
    int code = 0;
    NA_CK(cudaMemcpyAsync(&code, w.err_any, sizeof(int), cudaMemcpyDeviceToHost, st));
    NA_CK(cudaStreamSynchronize(st));
    return code;
}
