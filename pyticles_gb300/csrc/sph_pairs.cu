// sph_pairs.cu -- density and heat-flux passes of one derivative evaluation,
// the thermostat reductions and the pair-set export.
//
//   k_density : rho_s, rho_l summation (self term W(0,h), no m_i:
//               properties.py:77-91), fused EOS epilogue (T from u, clamp,
//               p, pco: properties.py:38-49, spam_complete_force.py:134-152)
//   k_heat    : Fourier heat flux q_i (f_properties.py:129-130 restated)
#include <map>
#include <mutex>
#include <utility>

#include "sph_pairs.cuh"

namespace sph {

// At most 64 registers (4 blocks of 256 per SM): the two loop bodies of
// for_pairs would otherwise take 80 and cost 5-20% in occupancy.  A single
// simulation (its constants are kernel parameters): 2D mixed precision at
// 32 registers (7 blocks, 60 B spilled), measured 6.3% faster than 48 and 2%
// faster than 40; 3D and FP64 at 51.
// LIST: the pair lists (tuning.pair_scheme 2) instead of the cell windows.
template <typename R, int D, int K, bool ONE, bool LIST = false>
__device__ __forceinline__ void density_one(const View &v, int stage, int i) {
    const bool active = i < v.np;
    const int ii = active ? i : v.np - 1;
    using T4 = typename V4<R>::T;
    const T4 *__restrict__ P = (const T4 *)v.pk_pos_in;
    const int s = v.b_sim[ii];
    const SimDev &S = ONE ? v.one : v.sims[s];
    if (S.cl_on) return;   // evaluated by the cluster passes
    KConst<R> ks = make_kconst<R>(S, 0);
    KConst<R> kl = make_kconst<R>(S, 1);
    BAcc<R> rs, rl;
    rs.init((R)0);
    rl.init((R)0);
    unsigned cnt = 0;
    auto body = [&](int j, const T4 &pj, const R *d, R rsq, auto near) {
        const Dist<R> dd = plain_dist<R>(rsq);
        R w, g;
        if constexpr (decltype(near)::value) {
            kernel_wg<K, R>(ks, dd, &w, &g);
            rs.add(pj.w * w);
        }
        kernel_wg<K, R>(kl, dd, &w, &g);
        rl.add(pj.w * w);
        ++cnt;
    };
    auto cell_done = [&]() {
        rs.flush();
        rl.flush();
    };
    if (!active) return;
    {
        PairFrame<R, D> fr;
        fr.init(S);
        if constexpr (LIST) for_list<R, D, true>(v, S, fr, P, i, P[i], body, cell_done);
        else for_pairs<R, D>(v, S, fr, P, i, P[i], body, cell_done);
    }
    // EOS in FP64 from the compensated sums plus the FP64 self term
    // (properties.py:77-78): the temperature T = (u + a rho)/k_B cancels
    // strongly, so rho enters it with the bits the FP32 sum carried in its
    // compensation.  p/rho^2 = k_B T / (rho (1 - b rho)); the cohesive factor
    // pco/rho_l^2 is exactly -a and needs no storage.
    double rho = S.ws0 + S.sig_s * rs.get64();
    double rhol = S.wl0 + S.sig_l * rl.get64();
    double T = (v.ue_in[i] + S.a * rho) * S.inv_kb;
    if (T < 0.0) T = 0.0;
    double den = rho * (1.0 - S.b * rho);
    double fs = S.kb * T * recip64<R>(den);
    double p = fs * rho * rho;
    double pco = -S.a * rhol * rhol;
    R Th = (R)T;
    ((R *)v.rho)[i] = (R)rho;
    ((R *)v.rho_l)[i] = (R)rhol;
    ((R *)v.temp)[i] = Th;
    ((R *)v.pres)[i] = (R)p;
    ((R *)v.pco)[i] = (R)pco;
    if (stage == 0) {
        ((R *)v.rho0)[i] = (R)rho;
        ((R *)v.pres0)[i] = (R)p;
        ((R *)v.pco0)[i] = (R)pco;
    }
    // {p/rho^2, rho, T_hi, T_lo}: T as a hi/lo pair so that T_j - T_i in the
    // heat pass does not lose the low bits
    ((T4 *)v.pk_f)[i] = make_v4<R>((R)fs, (R)rho, Th, (R)(T - (double)Th));
    // what the force pass reads of a neighbour, in one 16-byte load in 2D
    const T4 vi = ((const T4 *)v.pk_vel_in)[i];
    ((T4 *)v.pk_fv)[i] = D == 2 ? make_v4<R>(vi.x, vi.y, (R)fs, (R)rho)
                                : make_v4<R>(vi.x, vi.y, vi.z, (R)fs);
    if (!isfinite((R)p) || !isfinite((R)rho) || !isfinite((R)rhol))
        set_err(v.err, v.err_any, s, SPH_ENAN);
    // the pair set of one evaluation: counted at the step's first one only
    // (the counters are cleared once per step)
    if (stage == 0) add_pair_count(v.pair_count, s, cnt);
}

// One thread per particle; PERSIST: the resident blocks of pass_grid walk
// the particles grid-stride (the same per-particle work, the same bits).
template <typename R, int D, int K, bool ONE, bool PERSIST>
__global__ void __launch_bounds__(256, ONE ? ((D == 2 && sizeof(R) == 4) ? 7 : 5) : 4) k_density(const __grid_constant__ View v, int stage) {
    if constexpr (PERSIST) {
        for (int base = blockIdx.x * blockDim.x; base < v.np; base += gridDim.x * blockDim.x)
            density_one<R, D, K, ONE>(v, stage, base + threadIdx.x);
    } else {
        density_one<R, D, K, ONE>(v, stage, blockIdx.x * blockDim.x + threadIdx.x);
    }
}

// The density pass over the pair lists (mixed precision); a single
// simulation at SPH_VL_DENSITY_BLOCKS (2D) / SPH_VL_DENSITY3_BLOCKS (3D)
// resident blocks of 256 per SM, several at SPH_VL_DENSITY_MULTI_BLOCKS
// (5: 6.5% faster than 4 for 512 batched 2D simulations).
#ifndef SPH_VL_DENSITY_BLOCKS
#define SPH_VL_DENSITY_BLOCKS 7
#endif
#ifndef SPH_VL_DENSITY3_BLOCKS
#define SPH_VL_DENSITY3_BLOCKS 6
#endif
#ifndef SPH_VL_DENSITY_MULTI_BLOCKS
#define SPH_VL_DENSITY_MULTI_BLOCKS 5
#endif
template <int D, int K, bool ONE>
__global__ void __launch_bounds__(256, ONE ? (D == 2 ? SPH_VL_DENSITY_BLOCKS : SPH_VL_DENSITY3_BLOCKS) : SPH_VL_DENSITY_MULTI_BLOCKS)
    k_density_vl(const __grid_constant__ View v, int stage) {
    density_one<float, D, K, ONE, true>(v, stage, blockIdx.x * blockDim.x + threadIdx.x);
}

// At most 64 registers (4 blocks of 256 per SM): 8% faster in 3D than 80.
template <typename R, int D, int K, bool ONE, bool LIST = false>
__device__ __forceinline__ void heat_one(const View &v, int i) {
    const bool active = i < v.np;
    const int ii = active ? i : v.np - 1;
    using T4 = typename V4<R>::T;
    const T4 *__restrict__ P = (const T4 *)v.pk_pos_in;
    const T4 *__restrict__ F = (const T4 *)v.pk_f;
    const int s = v.b_sim[ii];
    const SimDev &S = ONE ? v.one : v.sims[s];
    if (S.cl_on) return;   // evaluated by the cluster passes
    KConst<R> ks = make_kconst<R>(S, 0);
    const T4 fi = F[ii];
    BAcc<R> q[3];
    q[0].init(0);
    q[1].init(0);
    q[2].init(0);
    auto body = [&](int j, const T4 &pj, const R *d, R rsq, auto) {
        R g = kernel_g<K, R, true>(ks, make_dist<R>(rsq));
        T4 fj = F[j];
        R dT = (fj.z - fi.z) + (fj.w - fi.w);
        R f = pj.w * rrcp<R>(fj.y) * dT * g;
        q[0].add(f * d[0]);
        q[1].add(f * d[1]);
        if (D == 3) q[2].add(f * d[2]);
    };
    auto cell_done = [&]() {
        q[0].flush();
        q[1].flush();
        if (D == 3) q[2].flush();
    };
    if (!active) return;
    {
        PairFrame<R, D> fr;
        fr.init(S);
        // only the short kernel enters q: cells and pairs beyond its support
        // contribute exactly zero and are not visited
        fr.thr_hi = fr.thr_s;
        if constexpr (LIST) for_list<R, D, false>(v, S, fr, P, i, P[i], body, cell_done);
        else for_pairs<R, D, D == 3, false>(v, S, fr, P, i, P[i], body, cell_done);
    }
    R kap = sconst<R>(S).kappa;
    R qq[3] = {kap * q[0].get(), kap * q[1].get(), kap * q[2].get()};
    R ir2 = (R)1 / (fi.y * fi.y);
    for (int a = 0; a < D; ++a) ((R *)v.q[a])[i] = qq[a];
    // {q/rho^2, rho}: the force pass's heat record, which in 3D also gives
    // it the neighbour's density
    ((T4 *)v.pk_q)[i] = make_v4<R>(qq[0] * ir2, qq[1] * ir2, qq[2] * ir2, fi.y);
}

template <typename R, int D, int K, bool ONE, bool PERSIST>
__global__ void __launch_bounds__(256, 4) k_heat(const __grid_constant__ View v) {
    if constexpr (PERSIST) {
        for (int base = blockIdx.x * blockDim.x; base < v.np; base += gridDim.x * blockDim.x)
            heat_one<R, D, K, ONE>(v, base + threadIdx.x);
    } else {
        heat_one<R, D, K, ONE>(v, blockIdx.x * blockDim.x + threadIdx.x);
    }
}

template <int D, int K, bool ONE>
__global__ void __launch_bounds__(256, 4) k_heat_vl(const __grid_constant__ View v) {
    heat_one<float, D, K, ONE, true>(v, blockIdx.x * blockDim.x + threadIdx.x);
}

// The persistent form is instantiated for the mixed-precision passes only;
// FP64 engines launch one thread per particle whatever tuning.persistent says.
// Pair lists (v.vl_on) exist for mixed-precision engines only.
template <typename R, int D, int K, bool ONE>
void density_launch(const View &v, int stage, int block, cudaStream_t s) {
    if constexpr (std::is_same<R, float>::value) {
        if (v.vl_on) {
            k_density_vl<D, K, ONE><<<(v.np + block - 1) / block, block, 0, s>>>(v, stage);
            return;
        }
    }
    if (std::is_same<R, float>::value && v.persist) {
        auto *fn = k_density<R, D, K, ONE, std::is_same<R, float>::value>;
        fn<<<pass_grid(v, fn, block), block, 0, s>>>(v, stage);
    } else {
        k_density<R, D, K, ONE, false><<<(v.np + block - 1) / block, block, 0, s>>>(v, stage);
    }
}

template <typename R, int D, int K, bool ONE>
void heat_launch(const View &v, int block, cudaStream_t s) {
    if constexpr (std::is_same<R, float>::value) {
        if (v.vl_on) {
            k_heat_vl<D, K, ONE><<<(v.np + block - 1) / block, block, 0, s>>>(v);
            return;
        }
    }
    if (std::is_same<R, float>::value && v.persist) {
        auto *fn = k_heat<R, D, K, ONE, std::is_same<R, float>::value>;
        fn<<<pass_grid(v, fn, block), block, 0, s>>>(v);
    } else {
        k_heat<R, D, K, ONE, false><<<(v.np + block - 1) / block, block, 0, s>>>(v);
    }
}

void launch_density(const View &v, int precision, int kernel, int stage, int block,
                    cudaStream_t s) {
    if (v.np <= 0) return;
    if (v.one_sim)
        SPH_DISPATCH(precision, v.dim, kernel, (density_launch<R, D, K, true>(v, stage, block, s)));
    else
        SPH_DISPATCH(precision, v.dim, kernel, (density_launch<R, D, K, false>(v, stage, block, s)));
}

void launch_heat(const View &v, int precision, int kernel, int block, cudaStream_t s) {
    if (v.np <= 0) return;
    if (v.one_sim)
        SPH_DISPATCH(precision, v.dim, kernel, (heat_launch<R, D, K, true>(v, block, s)));
    else
        SPH_DISPATCH(precision, v.dim, kernel, (heat_launch<R, D, K, false>(v, block, s)));
}

int resident_blocks(const void *kernel, int block) {
    static std::mutex mu;
    static std::map<std::pair<const void *, int>, int> cache;
    std::lock_guard<std::mutex> lock(mu);
    int dev = 0;
    cudaGetDevice(&dev);
    const auto key = std::make_pair(kernel, block * 64 + dev);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    int sms = 0, per = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, block, 0);
    const int cap = (sms > 0 ? sms : 1) * (per > 0 ? per : 1);
    cache[key] = cap;
    return cap;
}

// ---- thermostat: per-chunk FP64 partial sums of T, then one thread per
// simulation sums its chunks in order (deterministic) ----
template <typename R>
__global__ void k_tsum_chunks(View v) {
    int c = blockIdx.x;
    int b = v.chunk_start[c], n = v.chunk_len[c];
    double x = 0.0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) x += (double)((const R *)v.temp)[b + k];
    __shared__ double sh[256];
    sh[threadIdx.x] = x;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) v.tsum_part[c] = sh[0];
}

__global__ void k_tsum_sims(View v, int nsims) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsims) return;
    SimDev &S = v.sims[s];
    if (!S.active) return;
    long long done = v.steps[s] + 1;
    v.steps[s] = done;
    if (!S.thermostat) return;
    double sum = 0.0;
    for (int c = S.chunk_first; c < S.chunk_first + S.nchunk; ++c) sum += v.tsum_part[c];
    double tav = sum / (double)S.n;
    double target = S.T0;
    if (S.ramp > 0) {
        double f = (double)done / (double)S.ramp;
        if (f > 1.0) f = 1.0;
        target = S.T0 + (S.T1 - S.T0) * f;
    }
    v.t_scale[s] = target / tav;
}

void launch_tsum(const View &v, int precision, int nsims, cudaStream_t s) {
    if (v.nchunks > 0) {
        if (precision == SPH_MIXED) k_tsum_chunks<float><<<v.nchunks, 256, 0, s>>>(v);
        else k_tsum_chunks<double><<<v.nchunks, 256, 0, s>>>(v);
    }
    k_tsum_sims<<<(nsims + 127) / 128, 128, 0, s>>>(v, nsims);
}

// ---- pair-set export (VerletList.build + NeighbourList.separations
// attributes): the same pair iteration, rows keyed by original index ----
template <typename R, int D>
__global__ void k_pair_rows(View v, int off, int n, long long *row_count) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int i = off + k;
    const SimDev &S = v.sims[v.b_sim[i]];
    using T4 = typename V4<R>::T;
    const T4 *__restrict__ P = (const T4 *)v.pk_pos_in;
    PairFrame<R, D> fr;
    fr.init(S);
    const int idi = v.b_id[i];
    long long c = 0;
    for_pairs<R, D>(
        v, S, fr, P, i, P[i], [&](int j, const T4 &, const R *, R, auto) {
            if (v.b_id[j] > idi) ++c;
        },
        [] {});
    row_count[idi] = c;
}

template <typename R, int D>
__global__ void k_pair_write(View v, int off, int n, const long long *row_start, long long *iap,
                             double *drij, double *rsq, double *dv) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int i = off + k;
    const SimDev &S = v.sims[v.b_sim[i]];
    using T4 = typename V4<R>::T;
    const T4 *__restrict__ P = (const T4 *)v.pk_pos_in;
    PairFrame<R, D> fr;
    fr.init(S);
    const int idi = v.b_id[i];
    const long long base = row_start[idi];
    long long m = 0;
    for_pairs<R, D>(v, S, fr, P, i, P[i], [&](int j, const T4 &, const R *, R, auto) {
        const int idj = v.b_id[j];
        if (idj < idi) return;
        // insertion into the row, ordered by j's original index
        long long p = base + m;
        while (p > base && iap[2 * (p - 1) + 1] > idj) {
            iap[2 * p] = iap[2 * (p - 1)];
            iap[2 * p + 1] = iap[2 * (p - 1) + 1];
            if (rsq) rsq[p] = rsq[p - 1];
            if (drij)
                for (int a = 0; a < D; ++a) drij[p * D + a] = drij[(p - 1) * D + a];
            if (dv)
                for (int a = 0; a < D; ++a) dv[p * D + a] = dv[(p - 1) * D + a];
            --p;
        }
        iap[2 * p] = idi;
        iap[2 * p + 1] = idj;
        double r2 = 0.0;
        for (int a = 0; a < D; ++a) {
            double d = __dsub_rn(v.xe_in[a][j], v.xe_in[a][i]);
            if (d > S.half_L[a]) d = __dsub_rn(d, S.L[a]);
            if (d < -S.half_L[a]) d = __dadd_rn(d, S.L[a]);
            r2 = (a == 0) ? __dmul_rn(d, d) : __dadd_rn(r2, __dmul_rn(d, d));
            if (drij) drij[p * D + a] = d;
            if (dv) dv[p * D + a] = __dsub_rn(v.ve_in[a][j], v.ve_in[a][i]);
        }
        if (rsq) rsq[p] = r2;
        ++m;
    }, [] {});
}

void launch_pair_rows(const View &v, int precision, int sim_off, int n, long long *row_count,
                      cudaStream_t s) {
    if (n <= 0) return;
    int nb = (n + 127) / 128;
    if (precision == SPH_MIXED) {
        if (v.dim == 2) k_pair_rows<float, 2><<<nb, 128, 0, s>>>(v, sim_off, n, row_count);
        else k_pair_rows<float, 3><<<nb, 128, 0, s>>>(v, sim_off, n, row_count);
    } else {
        if (v.dim == 2) k_pair_rows<double, 2><<<nb, 128, 0, s>>>(v, sim_off, n, row_count);
        else k_pair_rows<double, 3><<<nb, 128, 0, s>>>(v, sim_off, n, row_count);
    }
}

void launch_pair_write(const View &v, int precision, int sim_off, int n,
                       const long long *row_start, long long *iap, double *drij, double *rsq,
                       double *dv, cudaStream_t s) {
    if (n <= 0) return;
    int nb = (n + 127) / 128;
#define SPH_PW(R_, D_) \
    k_pair_write<R_, D_><<<nb, 128, 0, s>>>(v, sim_off, n, row_start, iap, drij, rsq, dv)
    if (precision == SPH_MIXED) {
        if (v.dim == 2) SPH_PW(float, 2);
        else SPH_PW(float, 3);
    } else {
        if (v.dim == 2) SPH_PW(double, 2);
        else SPH_PW(double, 3);
    }
#undef SPH_PW
}

// exclusive scan of n+1 int64 entries in place (export path only)
__global__ void k_scan64(long long *data, int n) {
    __shared__ long long sh[1024];
    __shared__ long long carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base <= n; base += 1024) {
        int i = base + threadIdx.x;
        long long x = (i <= n) ? data[i] : 0;
        sh[threadIdx.x] = x;
        __syncthreads();
        for (int o = 1; o < 1024; o <<= 1) {
            long long y = threadIdx.x >= (unsigned)o ? sh[threadIdx.x - o] : 0;
            __syncthreads();
            sh[threadIdx.x] += y;
            __syncthreads();
        }
        if (i <= n) data[i] = sh[threadIdx.x] - x + carry;
        __syncthreads();
        if (threadIdx.x == 1023) carry += sh[1023];
        __syncthreads();
    }
}

void launch_scan64(long long *data, int n, cudaStream_t s) {
    k_scan64<<<1, 1024, 0, s>>>(data, n);
}

}  // namespace sph
