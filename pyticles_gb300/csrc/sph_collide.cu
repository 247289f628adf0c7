// sph_collide.cu -- hard collisions: CollisionForce (forces.py:87-156),
// CollisionForce3d (forces.py:158-243) and FortranCollisionForce
// (forces.py:454-474, whose collide3d is restated as CollisionForce3d's
// velocity exchange), applied through Force.apply's cutoff test
// rij^2 <= cutoff^2 (forces.py:38-42).
//
// The reference walks its pair list once and mutates the velocities of each
// colliding pair in place, so a pair sees the velocities left by every
// earlier pair that shares a particle with it.  Here each candidate pair k
// records its predecessor on either particle (the previous candidate in list
// order touching that particle); its dependency level is one more than the
// larger level of the two predecessors.  Pairs of one level share no
// particle, so a level is applied concurrently and the levels in order:
// every particle sees exactly the sequence of updates of the sequential
// loop, with the same FP64 operations (no contraction), so results equal
// the reference's bit for bit.
//
// Candidate sources:
//  * engine: at each evaluation the cell list yields, per particle i, the
//    partners j with a larger original index whose minimum-imaged FP64
//    distance passes both the pair-set test (rsq < cutoff^2 + tol^2) and the
//    collision test; rows are laid out in (i, j) order -- VerletList.build's
//    order (neighbour_list.py:160-189);
//  * sph_collide_pairs: the caller's pair list, filtered in list order.
#include <algorithm>
#include <cstring>
#include <vector>

#include "sph_device.cuh"

namespace sph {
namespace {

__device__ __forceinline__ double m_(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double a_(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double s_(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double q_(double a, double b) { return __ddiv_rn(a, b); }

__device__ __forceinline__ double &at(const Vec3Ref &r, int slot, int a) {
    return r.p[a][(size_t)slot * r.stride];
}

__device__ __forceinline__ int wrap_cell(int c, int n) {
    c += c < 0 ? n : 0;
    c -= c >= n ? n : 0;
    return c;
}

// Partners j of particle slot i with a larger original index that collide
// with it at the evaluation positions: f(j, idj, dr, rij).
template <int D, typename F>
__device__ void for_partners(const View &v, const SimDev &S, int i, F f) {
    const int cp = v.cell_xyz[v.cell_b[i]];
    const int c0 = cp & 2047, c1 = (cp >> 11) & 2047, c2 = (cp >> 22) & 1023;
    const int *mort = v.morton + S.cell_off;
    const int idi = v.b_id[i];
    double xi[3] = {0, 0, 0};
    for (int a = 0; a < D; ++a) xi[a] = v.xe_in[a][i];
    const int w0 = S.coll_win[0], w1 = S.coll_win[1], w2 = D == 3 ? S.coll_win[2] : 0;
    for (int oz = -w2; oz <= w2; ++oz) {
        const int z = D == 3 ? wrap_cell(c2 + oz, S.nc[2]) : 0;
        for (int oy = -w1; oy <= w1; ++oy) {
            const int y = wrap_cell(c1 + oy, S.nc[1]);
            for (int ox = -w0; ox <= w0; ++ox) {
                const int x = wrap_cell(c0 + ox, S.nc[0]);
                const int lin = (z * S.nc[1] + y) * S.nc[0] + x;
                if (!SPH_IN_BOUNDS(lin >= 0 && lin < S.ncells, v.err_any)) continue;
                const int gc = S.cell_off + mort[lin];
                const int jb = v.cell_start[gc], je = v.cell_start[gc + 1];
                if (!SPH_IN_BOUNDS(jb >= 0 && jb <= je && je <= v.np, v.err_any)) continue;
                for (int j = jb; j < je; ++j) {
                    const int idj = v.b_id[j];
                    if (idj <= idi) continue;
                    double dr[3] = {0, 0, 0}, rsq = 0.0;
                    for (int a = 0; a < D; ++a) {
                        double d = s_(v.xe_in[a][j], xi[a]);
                        if (d > S.half_L[a]) d = s_(d, S.L[a]);
                        if (d < -S.half_L[a]) d = a_(d, S.L[a]);
                        dr[a] = d;
                        rsq = a == 0 ? m_(d, d) : a_(rsq, m_(d, d));
                    }
                    if (!(rsq < S.thr)) continue;             // in the pair list
                    const double rij = __dsqrt_rn(rsq);
                    if (!(m_(rij, rij) <= S.coll_c2)) continue;  // Force.apply
                    f(j, idj, dr, rij);
                }
            }
        }
    }
}

template <int D>
__global__ void k_coll_rows(View v, CollideSet c) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.np) return;
    const SimDev &S = v.sims[v.b_sim[i]];
    int cnt = 0;
    if (S.coll_on) for_partners<D>(v, S, i, [&](int, int, const double *, double) { ++cnt; });
    c.row_count[S.part_off + v.b_id[i]] = cnt;
}

template <int D>
__global__ void k_coll_write(View v, CollideSet c) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.np) return;
    const SimDev &S = v.sims[v.b_sim[i]];
    if (!S.coll_on) return;
    const int row = S.part_off + v.b_id[i];
    const int base = c.row_start[row];
    if (c.row_start[row + 1] > c.cap) return;  // overflow: reported, nothing applied
    int m = 0;
    for_partners<D>(v, S, i, [&](int j, int idj, const double *dr, double rij) {
        // insertion into the row, ordered by j's original index
        int p = base + m;
        while (p > base && v.b_id[c.cj[p - 1]] > idj) {
            c.ci[p] = c.ci[p - 1];
            c.cj[p] = c.cj[p - 1];
            for (int a = 0; a < 3; ++a) c.dr[a][p] = c.dr[a][p - 1];
            c.rij[p] = c.rij[p - 1];
            --p;
        }
        c.ci[p] = i;
        c.cj[p] = j;
        for (int a = 0; a < 3; ++a) c.dr[a][p] = a < D ? dr[a] : 0.0;
        c.rij[p] = rij;
        ++m;
    });
}

// info[0] = candidates, info[1] = overflow; touch counts per particle
__global__ void k_coll_touch_count(CollideSet c, const int *total) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = *total;
    if (k == 0) {
        c.info[0] = n;
        c.info[1] = n > c.cap ? 1 : 0;
    }
    if (n > c.cap || k >= n) return;
    if (c.ci[k] < 0) return;
    atomicAdd(&c.touch_count[c.ci[k]], 1);
    atomicAdd(&c.touch_count[c.cj[k]], 1);
}

__global__ void k_coll_touch_fill(CollideSet c) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = c.info[0];
    if (n > c.cap || k >= n || c.ci[k] < 0) return;
    const int a = c.ci[k], b = c.cj[k];
    c.touch[c.touch_start[a] + atomicAdd(&c.touch_fill[a], 1)] = k;
    c.touch[c.touch_start[b] + atomicAdd(&c.touch_fill[b], 1)] = k;
}

// Per particle: its candidates in list order; each one's predecessor on
// this particle's side is the previous entry.
__global__ void k_coll_pred(CollideSet c) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= c.np || c.info[1]) return;
    const int b = c.touch_start[a], e = c.touch_start[a + 1];
    for (int q = b + 1; q < e; ++q) {
        const int x = c.touch[q];
        int p = q;
        while (p > b && c.touch[p - 1] > x) {
            c.touch[p] = c.touch[p - 1];
            --p;
        }
        c.touch[p] = x;
    }
    for (int q = b; q < e; ++q) {
        const int k = c.touch[q];
        const int side = c.ci[k] == a ? 0 : 1;
        c.pred[2 * k + side] = q > b ? c.touch[q - 1] : -1;
    }
}

constexpr int kSolveThreads = 1024;

// Dependency levels by monotone relaxation in one block: a level only ever
// grows towards its fixed point, so a sweep without a change ends it.  The
// longest chain bounds the sweeps; the loop stops after n + 1 regardless.
__global__ void __launch_bounds__(kSolveThreads) k_coll_levels(CollideSet c) {
    __shared__ int changed, maxl;
    const int n = c.info[0];
    if (n > c.cap) return;
    for (int k = threadIdx.x; k < n; k += blockDim.x) c.level[k] = 0;
    if (threadIdx.x == 0) maxl = 0;
    __syncthreads();
    int sweeps = 0;
    for (;;) {
        if (threadIdx.x == 0) changed = 0;
        __syncthreads();
        for (int k = threadIdx.x; k < n; k += blockDim.x) {
            if (c.ci[k] < 0) continue;
            const int pa = c.pred[2 * k], pb = c.pred[2 * k + 1];
            int l = 0;
            if (pa >= 0) l = max(l, c.level[pa] + 1);
            if (pb >= 0) l = max(l, c.level[pb] + 1);
            if (l != c.level[k]) {
                c.level[k] = l;
                changed = 1;
            }
        }
        __syncthreads();
        const int more = changed;
        __syncthreads();
        if (!more) break;
        if (++sweeps > n + 1) {
            if (threadIdx.x == 0) c.info[3] = 1;
            break;
        }
    }
    for (int k = threadIdx.x; k < n; k += blockDim.x)
        if (c.ci[k] >= 0) atomicMax(&maxl, c.level[k]);
    __syncthreads();
    if (threadIdx.x == 0) c.info[2] = maxl;
}

template <typename R, int D>
__device__ void collide_one(const CollideSet &c, int k, Vec3Ref vel, Vec3Ref pos,
                            const double *m, double push_cut, void *pk_vel, double *list_drij,
                            double *list_rij) {
    const int i = c.ci[k], j = c.cj[k];
    double dr[3], vi[3], vj[3];
    for (int a = 0; a < D; ++a) {
        dr[a] = c.dr[a][k];
        vi[a] = at(vel, i, a);
        vj[a] = at(vel, j, a);
    }
    double drsq = m_(dr[0], dr[0]);
    double vidotr = m_(vi[0], dr[0]), vjdotr = m_(vj[0], dr[0]);
    for (int a = 1; a < D; ++a) {
        drsq = a_(drsq, m_(dr[a], dr[a]));
        vidotr = a_(vidotr, m_(vi[a], dr[a]));
        vjdotr = a_(vjdotr, m_(vj[a], dr[a]));
    }
    // moving away from each other: nothing to do
    if (vidotr < 0 && vjdotr > 0) return;
    const double fi = q_(vidotr, drsq), fj = q_(vjdotr, drsq);
    const double mji = q_(m[j], m[i]), mij = q_(m[i], m[j]);
    for (int a = 0; a < D; ++a) {
        const double vti = m_(fi, dr[a]), vtj = m_(fj, dr[a]);
        const double vni = s_(vi[a], vti), vnj = s_(vj[a], vtj);
        // the components along the pair axis trade places, scaled by mass
        vi[a] = a_(m_(vtj, mji), vni);
        vj[a] = a_(m_(vti, mij), vnj);
        at(vel, i, a) = vi[a];
        at(vel, j, a) = vj[a];
    }
    if (pk_vel) {
        using T4 = typename V4<R>::T;
        T4 *P = (T4 *)pk_vel;
        P[i] = make_v4<R>((R)vi[0], (R)vi[1], D == 3 ? (R)vi[2] : (R)0, (R)0);
        P[j] = make_v4<R>((R)vj[0], (R)vj[1], D == 3 ? (R)vj[2] : (R)0, (R)0);
    }
    if (push_cut > 0 && drsq < m_(push_cut, push_cut)) {
        // CollisionForce3d: move both particles apart to cutoff + 0.01
        const double rij = c.rij[k];
        const double ro = q_(s_(a_(push_cut, 0.01), rij), 2.0);
        double d[3] = {0, 0, 0}, nsq = 0.0;
        for (int a = 0; a < D; ++a) {
            const double dro = m_(q_(dr[a], rij), ro);
            at(pos, i, a) = s_(at(pos, i, a), dro);
            at(pos, j, a) = a_(at(pos, j, a), dro);
            d[a] = s_(at(pos, j, a), at(pos, i, a));
            nsq = a == 0 ? m_(d[a], d[a]) : a_(nsq, m_(d[a], d[a]));
        }
        if (list_drij) {
            const int s = c.src[k];
            for (int a = 0; a < D; ++a) list_drij[(size_t)s * D + a] = d[a];
            list_rij[s] = __dsqrt_rn(nsq);
        }
    }
}

template <typename R, int D>
__global__ void __launch_bounds__(kSolveThreads)
    k_coll_apply(CollideSet c, Vec3Ref vel, Vec3Ref pos, const double *m, double push_cut,
                 void *pk_vel, int *err, int *err_any, int nsims, double *list_drij,
                 double *list_rij) {
    const int n = c.info[0];
    if (n > c.cap || c.info[3]) {
        if (err)
            for (int s = threadIdx.x; s < nsims; s += blockDim.x)
                set_err(err, err_any, s, c.info[3] ? SPH_ETIMEOUT : SPH_ECAPACITY);
        return;
    }
    const int top = c.info[2];
    for (int l = 0; l <= top; ++l) {
        for (int k = threadIdx.x; k < n; k += blockDim.x)
            if (c.ci[k] >= 0 && c.level[k] == l)
                collide_one<R, D>(c, k, vel, pos, m, push_cut, pk_vel, list_drij, list_rij);
        __syncthreads();
    }
}

// ---- pair-list source ----
// Candidate flags; a pair with an index outside [0, n) (or i == j) anywhere
// in the list makes the whole call an error and nothing is applied.
__global__ void k_list_flag(int64_t nip, const int64_t *iap, int64_t n, const double *rij,
                            double c2, int *flag, int *info) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nip) return;
    const int64_t i = iap[2 * k], j = iap[2 * k + 1];
    if (i < 0 || j < 0 || i >= n || j >= n || i == j) {
        atomicExch(&info[3], 2);
        flag[k] = 0;
        return;
    }
    flag[k] = m_(rij[k], rij[k]) <= c2 ? 1 : 0;
}

__global__ void k_list_compact(int64_t nip, const int64_t *iap, const double *drij,
                               const double *rij, int dim, int64_t n, const int *flag,
                               const int *start, CollideSet c) {
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nip || !flag[k]) return;
    const int p = start[k];
    const int64_t i = iap[2 * k], j = iap[2 * k + 1];
    if (i < 0 || j < 0 || i >= n || j >= n || i == j) {
        c.ci[p] = -1;
        c.cj[p] = -1;
        atomicExch(&c.info[3], 2);
        return;
    }
    c.ci[p] = (int)i;
    c.cj[p] = (int)j;
    for (int a = 0; a < 3; ++a) c.dr[a][p] = a < dim ? drij[k * dim + a] : 0.0;
    c.rij[p] = rij[k];
    c.src[p] = (int)k;
}

int blocks_for(int64_t n, int t) { return (int)((n + t - 1) / t); }

}  // namespace

void launch_collide_find(const View &v, const CollideSet &c, cudaStream_t s) {
    if (v.np <= 0) return;
    const int nb = blocks_for(v.np, 128);
    if (v.dim == 2) k_coll_rows<2><<<nb, 128, 0, s>>>(v, c);
    else k_coll_rows<3><<<nb, 128, 0, s>>>(v, c);
    launch_scan(c.row_count, c.row_start, v.np, c.scan_tmp, s);
    if (v.dim == 2) k_coll_write<2><<<nb, 128, 0, s>>>(v, c);
    else k_coll_write<3><<<nb, 128, 0, s>>>(v, c);
}

static void collide_levels(const CollideSet &c, const int *total, cudaStream_t s) {
    cudaMemsetAsync(c.touch_count, 0, sizeof(int) * (c.np + 1), s);
    cudaMemsetAsync(c.touch_fill, 0, sizeof(int) * (c.np + 1), s);
    const int nk = blocks_for(c.cap > 0 ? c.cap : 1, 256);
    k_coll_touch_count<<<nk, 256, 0, s>>>(c, total);
    launch_scan(c.touch_count, c.touch_start, c.np, c.scan_tmp, s);
    k_coll_touch_fill<<<nk, 256, 0, s>>>(c);
    k_coll_pred<<<blocks_for(c.np > 0 ? c.np : 1, 256), 256, 0, s>>>(c);
    k_coll_levels<<<1, kSolveThreads, 0, s>>>(c);
}

void launch_collide_levels(const CollideSet &c, cudaStream_t s) {
    collide_levels(c, c.row_start + c.np, s);
}

void launch_collide_apply(const CollideSet &c, int dim, Vec3Ref vel, Vec3Ref pos,
                          const double *m, double push_cut, void *pk_vel, int precision,
                          int *err, int *err_any, int nsims, cudaStream_t s) {
#define SPH_CA(R_, D_)                                                                     \
    k_coll_apply<R_, D_><<<1, kSolveThreads, 0, s>>>(c, vel, pos, m, push_cut, pk_vel, err, \
                                                     err_any, nsims, nullptr, nullptr)
    if (precision == SPH_MIXED) {
        if (dim == 2) SPH_CA(float, 2);
        else SPH_CA(float, 3);
    } else {
        if (dim == 2) SPH_CA(double, 2);
        else SPH_CA(double, 3);
    }
#undef SPH_CA
}

}  // namespace sph

using namespace sph;

namespace {

template <typename T>
int tmp_alloc(T **p, size_t n, std::vector<void *> &owned) {
    if (cudaMalloc((void **)p, sizeof(T) * (n ? n : 1)) != cudaSuccess) {
        cudaGetLastError();
        return SPH_ENOMEM;
    }
    owned.push_back(*p);
    return SPH_OK;
}

}  // namespace

extern "C" int sph_collide_pairs(int32_t dim, int32_t mode, int64_t n, double *r, double *v,
                                 const double *m, int64_t nip, const int64_t *iap,
                                 double *drij, double *rij, double cutoff, int32_t mem,
                                 void *stream) {
    if ((dim != 2 && dim != 3) || (mode != SPH_COLLIDE_EXCHANGE && mode != SPH_COLLIDE_PUSHBACK))
        return SPH_EINVAL;
    if (n < 0 || nip < 0 || n > (1 << 30) || nip > (1 << 30) || !(cutoff >= 0)) return SPH_EINVAL;
    if (nip > 0 && (!v || !m || !iap || !drij || !rij)) return SPH_EINVAL;
    if (mode == SPH_COLLIDE_PUSHBACK && nip > 0 && !r) return SPH_EINVAL;
    if (mem != SPH_DEVICE && mem != SPH_HOST) return SPH_EINVAL;
    if (nip == 0 || n == 0) return SPH_OK;
    cudaStream_t st = (cudaStream_t)stream;
    std::vector<void *> owned;
    int status = SPH_OK;
    auto run = [&]() -> int {
        const size_t nd = (size_t)n * dim, pd = (size_t)nip * dim;
        double *dr_ = r, *dv = v, *dm = (double *)m, *ddrij = drij, *drij_ = rij;
        const int64_t *diap = iap;
        if (mem == SPH_HOST) {
            if (tmp_alloc(&dv, nd, owned) || tmp_alloc(&dm, (size_t)n, owned) ||
                tmp_alloc(&ddrij, pd, owned) || tmp_alloc(&drij_, (size_t)nip, owned) ||
                tmp_alloc((int64_t **)&diap, 2 * (size_t)nip, owned))
                return SPH_ENOMEM;
            if (r && tmp_alloc(&dr_, nd, owned)) return SPH_ENOMEM;
            cudaMemcpyAsync(dv, v, sizeof(double) * nd, cudaMemcpyHostToDevice, st);
            cudaMemcpyAsync(dm, m, sizeof(double) * n, cudaMemcpyHostToDevice, st);
            cudaMemcpyAsync(ddrij, drij, sizeof(double) * pd, cudaMemcpyHostToDevice, st);
            cudaMemcpyAsync(drij_, rij, sizeof(double) * nip, cudaMemcpyHostToDevice, st);
            cudaMemcpyAsync((void *)diap, iap, sizeof(int64_t) * 2 * nip, cudaMemcpyHostToDevice,
                            st);
            if (r) cudaMemcpyAsync(dr_, r, sizeof(double) * nd, cudaMemcpyHostToDevice, st);
        }
        CollideSet c;
        memset(&c, 0, sizeof(c));
        c.cap = (int)nip;
        c.np = (int)n;
        int *flag = nullptr, *fstart = nullptr;
        int tmp_n = (int)std::max<int64_t>(nip, n) / 4096 + 2;
        if (tmp_alloc(&flag, (size_t)nip + 1, owned) || tmp_alloc(&fstart, (size_t)nip + 1, owned) ||
            tmp_alloc(&c.scan_tmp, (size_t)tmp_n, owned) || tmp_alloc(&c.ci, (size_t)nip, owned) ||
            tmp_alloc(&c.cj, (size_t)nip, owned) || tmp_alloc(&c.dr[0], (size_t)nip, owned) ||
            tmp_alloc(&c.dr[1], (size_t)nip, owned) || tmp_alloc(&c.dr[2], (size_t)nip, owned) ||
            tmp_alloc(&c.rij, (size_t)nip, owned) || tmp_alloc(&c.src, (size_t)nip, owned) ||
            tmp_alloc(&c.touch_count, (size_t)n + 1, owned) ||
            tmp_alloc(&c.touch_start, (size_t)n + 1, owned) ||
            tmp_alloc(&c.touch_fill, (size_t)n + 1, owned) ||
            tmp_alloc(&c.touch, 2 * (size_t)nip, owned) ||
            tmp_alloc(&c.pred, 2 * (size_t)nip, owned) || tmp_alloc(&c.level, (size_t)nip, owned) ||
            tmp_alloc(&c.info, 4, owned))
            return SPH_ENOMEM;
        cudaMemsetAsync(c.info, 0, sizeof(int) * 4, st);
        const int nb = blocks_for(nip, 256);
        k_list_flag<<<nb, 256, 0, st>>>(nip, diap, n, drij_, cutoff * cutoff, flag, c.info);
        launch_scan(flag, fstart, (int)nip, c.scan_tmp, st);
        k_list_compact<<<nb, 256, 0, st>>>(nip, diap, ddrij, drij_, dim, n, flag, fstart, c);
        collide_levels(c, fstart + nip, st);
        Vec3Ref vel{{dv, dv + 1, dv + (dim == 3 ? 2 : 1)}, dim};
        Vec3Ref pos{{dr_, dr_ ? dr_ + 1 : nullptr, dr_ ? dr_ + (dim == 3 ? 2 : 1) : nullptr}, dim};
        const double push = mode == SPH_COLLIDE_PUSHBACK ? cutoff : 0.0;
#define SPH_CL(D_)                                                                         \
    k_coll_apply<double, D_><<<1, kSolveThreads, 0, st>>>(c, vel, pos, dm, push, nullptr,  \
                                                          nullptr, nullptr, 0, ddrij, drij_)
        if (dim == 2) SPH_CL(2);
        else SPH_CL(3);
#undef SPH_CL
        int info[4] = {0, 0, 0, 0};
        cudaMemcpyAsync(info, c.info, sizeof(info), cudaMemcpyDeviceToHost, st);
        if (mem == SPH_HOST) {
            cudaMemcpyAsync(v, dv, sizeof(double) * nd, cudaMemcpyDeviceToHost, st);
            if (mode == SPH_COLLIDE_PUSHBACK) {
                cudaMemcpyAsync(r, dr_, sizeof(double) * nd, cudaMemcpyDeviceToHost, st);
                cudaMemcpyAsync(drij, ddrij, sizeof(double) * pd, cudaMemcpyDeviceToHost, st);
                cudaMemcpyAsync(rij, drij_, sizeof(double) * nip, cudaMemcpyDeviceToHost, st);
            }
        }
        if (cudaStreamSynchronize(st) != cudaSuccess || cudaGetLastError() != cudaSuccess)
            return SPH_ECUDA;
        if (info[3] == 2) return SPH_EINVAL;
        if (info[3] == 1) return SPH_ETIMEOUT;
        return SPH_OK;
    };
    status = run();
    if (status != SPH_OK) cudaStreamSynchronize(st);
    for (void *p : owned) cudaFree(p);
    return status;
}
