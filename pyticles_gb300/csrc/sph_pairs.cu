// sph_pairs.cu -- the pair passes of one derivative evaluation and the
// fused integrator epilogue.
//
//   k_density : rho_s, rho_l summation (self term W(0,h), no m_i:
//               properties.py:77-91), fused EOS epilogue (T from u, clamp,
//               p, pco: properties.py:38-49, spam_complete_force.py:134-152)
//   k_heat    : Fourier heat flux q_i (f_properties.py:129-130 restated)
//   k_force   : pressure + cohesive accelerations, Monaghan viscosity, energy
//               rate incl. conduction (forces.py:338-405, c_forces.pyx:96-111,
//               163-178, 224-237) fused with the integrator stage update
//               (integrator.py:14-103), periodic teleport (box.py:33-47) and the
//               thermostat (particles.py:450-457).
//
// Every pass is a gather: thread i sums over all neighbours j in the 3^dim
// cells around its own cell, so each unordered pair is evaluated from both
// sides and no atomics touch particle data.  Positions are cell-local
// (relative to the particle's cell centre), which keeps FP32 differences
// accurate; the pair-set test runs on those FP32 distances with a 2^-12
// guard band and falls back to the reference's FP64 test for pairs inside
// the band, so the pair set is bit-exact.
#include <type_traits>

#include "sph_device.cuh"

namespace sph {

__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }

// 1/x for the EOS: FP64 division in FP64 mode; in mixed mode an FP32
// reciprocal refined by one FP64 Newton step (relative error ~1e-14), which
// spares the narrow FP64 pipe a full division per particle.
template <typename R> __device__ __forceinline__ double recip64(double x);
template <> __device__ __forceinline__ double recip64<double>(double x) { return 1.0 / x; }
template <> __device__ __forceinline__ double recip64<float>(double x) {
    double r = (double)__frcp_rn((float)x);
    return r * fma(-x, r, 2.0);
}
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }

template <typename R, int D>
struct PairFrame {
    R thr_lo, thr_hi, thr_s;
    R edge[3], L[3], hL[3];
    R ext[3];       // half extent of a cell including the allowed drift
    int small_mask;
    __device__ __forceinline__ void init(const SimDev &S) {
        const SimConst<R> &c = sconst<R>(S);
        thr_lo = c.thr_lo;
        thr_hi = c.thr_hi;
        thr_s = c.thr_s;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            edge[a] = c.edge[a];
            L[a] = c.L[a];
            hL[a] = c.hL[a];
            ext[a] = c.ext[a];
        }
        small_mask = S.small_mask;
    }
    __device__ __forceinline__ void min_image(R *d) const {
        if (small_mask) {
#pragma unroll
            for (int a = 0; a < D; ++a)
                if (small_mask & (1 << a)) {
                    if (d[a] > hL[a]) d[a] -= L[a];
                    if (d[a] < -hL[a]) d[a] += L[a];
                }
        }
    }
};

template <int D> struct NbrCount { static constexpr int value = D == 2 ? 9 : 27; };

// max(|c| - ext, 0): distance along one axis from particle i to a cell whose
// centre sits at c relative to i
template <typename R> __device__ __forceinline__ R fmaxf_(R c, R ext) {
    R a = (c < (R)0 ? -c : c) - ext;
    return a > (R)0 ? a : (R)0;
}

// Iterates the pair set of particle i.  body(j, pj, d[3], rsq, near) is called
// for every j != i that passes the exact pair test, in a fixed order: neighbour
// cells in raster order (z, y, x) of their offset from i's cell, particles in
// cell order.  The order depends only on i's cell, never on which particles
// share a warp or a launch, so every particle sums its pairs identically
// whether its simulation runs alone or in a batch.
//
// Cells are (cutoff + skin)/W wide and the window spans +-W cells per axis;
// a cell whose box (grown by the allowed drift) lies beyond the cutoff from
// particle i is skipped before any of its particles is loaded.
//
// near is std::true_type unless the cell lies beyond the short kernel's
// support from every lane of the warp that visits it (a warp-uniform choice,
// so the two loop bodies never diverge); with std::false_type the body may
// drop every short-kernel term, which is exactly zero there.
//
// PF: load the next candidate's position before testing the current one
// (measured: 4-7% faster for the 3D heat and force passes, slower for the
// 2D passes and for density, where more warps already hide the latency).
template <typename R, int D, bool PF = false, typename T4, typename F, typename G>
__device__ __forceinline__ void for_pairs(const View &v, const SimDev &S,
                                          const PairFrame<R, D> &fr, const T4 *__restrict__ P,
                                          int i, const T4 &pi, F body, G cell_done) {
    const int cp = v.cell_xyz[v.cell_b[i]];
    const int c0 = cp & 2047, c1 = (cp >> 11) & 2047, c2 = (cp >> 22) & 1023;
    const int w0 = S.win[0], w1 = S.win[1], w2 = D == 3 ? S.win[2] : 0;
    const int n0 = S.nc[0], n1 = S.nc[1], n2 = S.nc[2];
    const int *mort = v.morton + S.cell_off;
    for (int oz = -w2; oz <= w2; ++oz) {
        R dz = (R)0;
        int z = 0;
        if (D == 3) {
            dz = fmaxf_((R)oz * fr.edge[2] - pi.z, fr.ext[2]);
            z = c2 + oz;
            z += (z < 0) ? n2 : 0;
            z -= (z >= n2) ? n2 : 0;
        }
        for (int oy = -w1; oy <= w1; ++oy) {
            R dy = fmaxf_((R)oy * fr.edge[1] - pi.y, fr.ext[1]);
            R dyz = dy * dy + dz * dz;
            if (dyz > fr.thr_hi) continue;
            int y = c1 + oy;
            y += (y < 0) ? n1 : 0;
            y -= (y >= n1) ? n1 : 0;
            const int row = (z * n1 + y) * n0;
            for (int ox = -w0; ox <= w0; ++ox) {
                R dx = fmaxf_((R)ox * fr.edge[0] - pi.x, fr.ext[0]);
                if (dx * dx + dyz > fr.thr_hi) continue;
                int x = c0 + ox;
                x += (x < 0) ? n0 : 0;
                x -= (x >= n0) ? n0 : 0;
                const int gc = S.cell_off + mort[row + x];
                const R ox_ = (R)ox * fr.edge[0] - pi.x;
                const R oy_ = (R)oy * fr.edge[1] - pi.y;
                const R oz_ = (D == 3) ? (R)oz * fr.edge[2] - pi.z : (R)0;
                const int jb = v.cell_start[gc], je = v.cell_start[gc + 1];
                auto scan = [&](auto near) {
                    T4 pn;
                    if (PF) pn = P[jb < je ? jb : i];
                    for (int j = jb; j < je; ++j) {
                        T4 pj;
                        if (PF) {
                            pj = pn;
                            if (j + 1 < je) pn = P[j + 1];
                        }
                        if (j == i) continue;
                        if (!PF) pj = P[j];
                        R d[3];
                        d[0] = pj.x + ox_;
                        d[1] = pj.y + oy_;
                        d[2] = (D == 3) ? pj.z + oz_ : (R)0;
                        fr.min_image(d);
                        R rsq = d[0] * d[0] + d[1] * d[1];
                        if (D == 3) rsq += d[2] * d[2];
                        if (rsq > fr.thr_hi) continue;
                        if (rsq >= fr.thr_lo && !exact_in_set<D>(v.xe_in, &S, i, j)) continue;
                        body(j, pj, d, rsq, near);
                    }
                };
                if (__any_sync(__activemask(), dx * dx + dyz < fr.thr_s))
                    scan(std::true_type{});
                else
                    scan(std::false_type{});
                cell_done();
            }
        }
    }
}

// Warp-aggregated per-simulation counter update.
__device__ __forceinline__ void add_pair_count(unsigned long long *cnt, int s, unsigned c) {
    unsigned act = __activemask();
    unsigned grp = __match_any_sync(act, s);
    unsigned long long tot = 0;
    // sum over the group (lanes with the same simulation)
    for (int l = 0; l < 32; ++l) {
        if (!(act & (1u << l))) continue;
        unsigned x = __shfl_sync(act, c, l);
        if (grp & (1u << l)) tot += x;
    }
    int leader = __ffs(grp) - 1;
    if ((threadIdx.x & 31) == leader) atomicAdd(&cnt[s], tot);
}

// At most 64 registers (4 blocks of 256 per SM): the two loop bodies of
// for_pairs would otherwise take 80 and cost 5-20% in occupancy.
template <typename R, int D, int K>
__global__ void __launch_bounds__(256, 4) k_density(View v, int stage) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = i < v.np;
    const int ii = active ? i : v.np - 1;
    using T4 = typename V4<R>::T;
    const T4 *__restrict__ P = (const T4 *)v.pk_pos_in;
    const int s = v.b_sim[ii];
    const SimDev &S = v.sims[s];
    KConst<R> ks = make_kconst<R>(S, 0);
    KConst<R> kl = make_kconst<R>(S, 1);
    BAcc<R> rs, rl;
    rs.init((R)0);
    rl.init((R)0);
    unsigned cnt = 0;
    auto body = [&](int j, const T4 &pj, const R *d, R rsq, auto near) {
        R r = rsqrt_<R>(rsq);
        R w, g;
        if constexpr (decltype(near)::value) {
            kernel_wg<K, R>(ks, r, &w, &g);
            rs.add(pj.w * w);
        }
        kernel_wg<K, R>(kl, r, &w, &g);
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
        for_pairs<R, D>(v, S, fr, P, i, P[i], body, cell_done);
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
    add_pair_count(v.pair_count, s, cnt);
}

// At most 64 registers (4 blocks of 256 per SM): 8% faster in 3D than 80.
template <typename R, int D, int K>
__global__ void __launch_bounds__(256, 4) k_heat(View v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = i < v.np;
    const int ii = active ? i : v.np - 1;
    using T4 = typename V4<R>::T;
    const T4 *__restrict__ P = (const T4 *)v.pk_pos_in;
    const T4 *__restrict__ F = (const T4 *)v.pk_f;
    const int s = v.b_sim[ii];
    const SimDev &S = v.sims[s];
    KConst<R> ks = make_kconst<R>(S, 0);
    const T4 fi = F[ii];
    BAcc<R> q[3];
    q[0].init(0);
    q[1].init(0);
    q[2].init(0);
    auto body = [&](int j, const T4 &pj, const R *d, R rsq, auto) {
        R r = fsqrt<R>(rsq);
        R g = kernel_g<K, R>(ks, r);
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
        for_pairs<R, D, D == 3>(v, S, fr, P, i, P[i], body, cell_done);
    }
    R kap = sconst<R>(S).kappa;
    R qq[3] = {kap * q[0].get(), kap * q[1].get(), kap * q[2].get()};
    R ir2 = (R)1 / (fi.y * fi.y);
    for (int a = 0; a < D; ++a) ((R *)v.q[a])[i] = qq[a];
    ((T4 *)v.pk_q)[i] = make_v4<R>(qq[0] * ir2, qq[1] * ir2, qq[2] * ir2, (R)0);
}

// Next evaluation state: positions/velocities/energy in FP64 plus packed
// cell-local copies relative to the particle's cell (binned at x0).
template <typename R, int D>
__device__ __forceinline__ void write_eval_state(const View &v, const SimDev &S, int i,
                                                 const double *x, const double *vel, double u,
                                                 double m) {
    using T4 = typename V4<R>::T;
    R xl[3] = {0, 0, 0}, vv[3] = {0, 0, 0};
    bool skin = false;
#pragma unroll
    for (int a = 0; a < D; ++a) {
        // relative to the cell the particle was binned in; with binning on
        // demand the step may have started from a wrapped position
        double d = x[a] - v.org[a][i];
        if (d > S.half_L[a]) d -= S.L[a];
        if (d < -S.half_L[a]) d += S.L[a];
        xl[a] = (R)d;
        vv[a] = (R)vel[a];
        v.xe_out[a][i] = x[a];
        v.ve_out[a][i] = vel[a];
        // the cell list finds every pair while each particle stays within its
        // cell grown by the slack
        skin |= fabs(d) > S.box_half[a];
    }
    if (skin) set_err(v.err, v.err_any, v.b_sim[i], SPH_ESKIN);
    v.ue_out[i] = u;
    ((T4 *)v.pk_pos_out)[i] = make_v4<R>(xl[0], xl[1], xl[2], (R)m);
    ((T4 *)v.pk_vel_out)[i] = make_v4<R>(vv[0], vv[1], vv[2], (R)0);
}

// Final state of the step into A (same slot as B), with the teleport wrap.
// In rebin mode it is also the next step's start state in B and its packed
// stage-0 copies, relative to the unchanged cells (the final stage writes
// pk_*_out == buffer 0 for improved Euler and RK4); a particle past half of
// its cell slack asks for a binning before the next step.
template <typename R, int D>
__device__ __forceinline__ void write_final_state(const View &v, const SimDev &S, int i,
                                                  double *x, const double *vel, double u) {
    using T4 = typename V4<R>::T;
    R xl[3] = {0, 0, 0}, vv[3] = {0, 0, 0};
    bool far = false;
#pragma unroll
    for (int a = 0; a < D; ++a) {
        double L = S.L[a];
        if (x[a] > L) x[a] = 0;
        if (x[a] < 0) x[a] = L;
        v.a_pos[a][i] = x[a];
        v.a_vel[a][i] = vel[a];
        if (v.reuse) {
            double d = x[a] - v.org[a][i];
            if (d > S.half_L[a]) d -= L;   // the wrap moved it across the box
            if (d < -S.half_L[a]) d += L;
            far |= fabs(d) > S.rebin_half[a];
            xl[a] = (R)d;
            vv[a] = (R)vel[a];
            v.b_pos[a][i] = x[a];
            v.b_vel[a][i] = vel[a];
        }
    }
    v.a_u[i] = u;
    v.a_m[i] = v.b_m[i];
    v.a_id[i] = v.b_id[i];
    v.a_sim[i] = v.b_sim[i];
    if (v.reuse) {
        v.b_u[i] = u;
        ((T4 *)v.pk_pos_out)[i] = make_v4<R>(xl[0], xl[1], xl[2], (R)v.b_m[i]);
        ((T4 *)v.pk_vel_out)[i] = make_v4<R>(vv[0], vv[1], vv[2], (R)0);
        if (far) *v.rebin_gate = 1;
    }
}

// Integrator stage of particle i (c = xdot dt as in integrator.py:14-103)
// from its rates vdr, udr, followed on the last stage by the teleport wrap
// and the thermostat.
template <typename R, int D>
__device__ __forceinline__ void integrate_stage(const View &v, const SimDev &S, int i, int s,
                                                int stage, int integ, const R *vdr, R udr) {
    const double dt = S.dt;
    double x0[3] = {0, 0, 0}, v0[3] = {0, 0, 0}, rd[3] = {0, 0, 0}, vd[3] = {0, 0, 0};
#pragma unroll
    for (int a = 0; a < D; ++a) {
        x0[a] = v.b_pos[a][i];
        v0[a] = v.b_vel[a][i];
        rd[a] = v.ve_in[a][i];
        vd[a] = (double)vdr[a];
    }
    double u0 = v.b_u[i], udd = (double)udr, m = v.b_m[i];
    double x[3] = {0, 0, 0}, vel[3] = {0, 0, 0}, u;
    bool final_stage = false;
    // Euler and improved Euler in FMA form: x0 + dt f and x0 + dt/2 (f0 + f1)
    // (integrator.py:14-59 round c = f dt and (c1 + c2)/2 separately; the
    // difference is one rounding per step, far below the FP64 tolerance)
    if (integ == SPH_EULER) {
        for (int a = 0; a < D; ++a) {
            x[a] = fma(dt, rd[a], x0[a]);
            vel[a] = fma(dt, vd[a], v0[a]);
        }
        u = fma(dt, udd, u0);
        final_stage = true;
    } else if (integ == SPH_IEULER) {
        if (stage == 0) {
            for (int a = 0; a < D; ++a) {
                ((R *)v.f0v[a])[i] = vdr[a];
                x[a] = fma(dt, rd[a], x0[a]);
                vel[a] = fma(dt, vd[a], v0[a]);
            }
            ((R *)v.f0u)[i] = udr;
            u = fma(dt, udd, u0);
            write_eval_state<R, D>(v, S, i, x, vel, u, m);
        } else {
            const double hdt = S.hdt;
            for (int a = 0; a < D; ++a) {
                x[a] = fma(hdt, v0[a] + rd[a], x0[a]);
                vel[a] = fma(hdt, (double)((const R *)v.f0v[a])[i] + vd[a], v0[a]);
            }
            u = fma(hdt, (double)((const R *)v.f0u)[i] + udd, u0);
            final_stage = true;
        }
    } else {  // RK4
        double cr[3], cv[3], cu = dmul(udd, dt);
        for (int a = 0; a < D; ++a) {
            cr[a] = dmul(rd[a], dt);
            cv[a] = dmul(vd[a], dt);
        }
        if (stage == 0) {
            for (int a = 0; a < D; ++a) {
                v.acc_r[a][i] = cr[a];
                v.acc_v[a][i] = cv[a];
                x[a] = dadd(x0[a], cr[a] / 2.0);
                vel[a] = dadd(v0[a], cv[a] / 2.0);
            }
            v.acc_u[i] = cu;
            u = dadd(u0, cu / 2.0);
            write_eval_state<R, D>(v, S, i, x, vel, u, m);
        } else if (stage < 3) {
            for (int a = 0; a < D; ++a) {
                v.acc_r[a][i] = dadd(v.acc_r[a][i], dmul(2.0, cr[a]));
                v.acc_v[a][i] = dadd(v.acc_v[a][i], dmul(2.0, cv[a]));
                x[a] = stage == 1 ? dadd(x0[a], cr[a] / 2.0) : dadd(x0[a], cr[a]);
                vel[a] = stage == 1 ? dadd(v0[a], cv[a] / 2.0) : dadd(v0[a], cv[a]);
            }
            v.acc_u[i] = dadd(v.acc_u[i], dmul(2.0, cu));
            u = stage == 1 ? dadd(u0, cu / 2.0) : dadd(u0, cu);
            write_eval_state<R, D>(v, S, i, x, vel, u, m);
        } else {
            for (int a = 0; a < D; ++a) {
                x[a] = dadd(x0[a], dmul(1.0 / 6.0, dadd(v.acc_r[a][i], cr[a])));
                vel[a] = dadd(v0[a], dmul(1.0 / 6.0, dadd(v.acc_v[a][i], cv[a])));
            }
            u = dadd(u0, dmul(1.0 / 6.0, dadd(v.acc_u[i], cu)));
            final_stage = true;
        }
    }
    if (final_stage) {
        if (S.thermostat) {
            // particles.py:450-457: T <- T * target / mean(T); u <- k_B T - a rho
            R *tp = (R *)v.temp;
            double T = (double)tp[i] * v.t_scale[s];
            u = dadd(dmul(T, S.kb), -dmul(S.a, (double)((const R *)v.rho0)[i]));
            tp[i] = (R)T;
        }
        write_final_state<R, D>(v, S, i, x, vel, u);
    }
}

// VH: bit 0 viscosity, bit 1 heat flux (compile-time, so a workload without
// them carries neither their registers nor their branches)
// At most 64 registers (4 blocks of 256 per SM): measured 17% faster than the
// unconstrained 80-104 despite a few spilled words outside the pair loop.
template <typename R, int D, int K, int VH>
__global__ void __launch_bounds__(256, 4) k_force(View v, int stage, int mode, int integ) {
    constexpr bool visc = (VH & 1) != 0;
    constexpr bool heat = (VH & 2) != 0;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = i < v.np;
    const int ii = active ? i : v.np - 1;
    using T4 = typename V4<R>::T;
    const T4 *__restrict__ P = (const T4 *)v.pk_pos_in;
    const T4 *__restrict__ FV = (const T4 *)v.pk_fv;
    const R *__restrict__ RHO = (const R *)v.rho;
    const T4 *__restrict__ Q = (const T4 *)v.pk_q;
    const int s = v.b_sim[ii];
    const SimDev &S = v.sims[s];
    KConst<R> ks = make_kconst<R>(S, 0);
    KConst<R> kl = make_kconst<R>(S, 1);
    const SimConst<R> &sc = sconst<R>(S);
    const R hs = sc.hs, eps_h2 = sc.eps_h2;
    const R alpha_c = sc.alpha_c, beta = sc.beta;
    const R pl2 = sc.pl2;  // pco_i/rho_l,i^2 + pco_j/rho_l,j^2 = -2a
    // own velocity, p/rho^2 and rho
    const T4 fvi = FV[ii];
    const R vix = fvi.x, viy = fvi.y, viz = D == 3 ? fvi.z : (R)0;
    const R fsi = D == 2 ? fvi.z : fvi.w;
    const R rhoi = D == 2 ? fvi.w : RHO[ii];
    const T4 qi = heat ? Q[ii] : make_v4<R>(0, 0, 0, 0);
    BAcc<R> ax[3], ud;
    ax[0].init(0);
    ax[1].init(0);
    ax[2].init(0);
    ud.init(0);
    auto body = [&](int j, const T4 &pj, const R *d, R rsq, auto near) {
        constexpr bool NEAR = decltype(near)::value;
        R r = fsqrt<R>(rsq);
        R gl = kernel_g<K, R>(kl, r);
        const T4 fvj = FV[j];
        R dvdx = (fvj.x - vix) * d[0] + (fvj.y - viy) * d[1];
        if (D == 3) dvdx += (fvj.z - viz) * d[2];
        // beyond the short support gs = 0: the pressure and viscosity terms
        // vanish and gsum = pl2 gl bit for bit
        R gsum = pl2 * gl, gs = (R)0;
        if constexpr (NEAR) {
            gs = kernel_g<K, R>(ks, r);
            R ps = fsi + (D == 2 ? fvj.z : fvj.w);
            if (visc && dvdx < (R)0) {
                // Monaghan viscosity on approaching pairs
                const R rhoj = D == 2 ? fvj.w : RHO[j];
                R mu = fdiv<R>(hs * dvdx, rsq + eps_h2);
                ps += fdiv<R>((R)2 * (-alpha_c * mu + beta * mu * mu), rhoi + rhoj);
            }
            gsum = ps * gs + pl2 * gl;
        }
        ax[0].add(gsum * d[0]);
        ax[1].add(gsum * d[1]);
        if (D == 3) ax[2].add(gsum * d[2]);
        R du = (R)0.5 * gsum * dvdx * pj.w;
        if (heat && NEAR) {
            T4 qj = Q[j];
            R dq = (qi.x + qj.x) * d[0] + (qi.y + qj.y) * d[1];
            if (D == 3) dq += (qi.z + qj.z) * d[2];
            du -= dq * gs * pj.w;
        }
        ud.add(du);
    };
    auto cell_done = [&]() {
        ax[0].flush();
        ax[1].flush();
        if (D == 3) ax[2].flush();
        ud.flush();
    };
    if (!active) return;
    {
        PairFrame<R, D> fr;
        fr.init(S);
        for_pairs<R, D, D == 3>(v, S, fr, P, i, P[i], body, cell_done);
    }
    R vdr[3] = {ax[0].get(), ax[1].get(), ax[2].get()};
    R udr = ud.get();
    for (int a = 0; a < D; ++a) ((R *)v.vdot[a])[i] = vdr[a];
    ((R *)v.udot)[i] = udr;
    if (!isfinite(vdr[0]) || !isfinite(udr)) set_err(v.err, v.err_any, s, SPH_ENAN);
    if (mode == 0) return;

    integrate_stage<R, D>(v, S, i, s, stage, integ, vdr, udr);
}

// Integrator stage from the stored rates: the epilogue of k_force as a pass
// of its own, for steps whose velocities change between the force pass and
// the update (hard collisions).
template <typename R, int D>
__global__ void __launch_bounds__(256) k_integrate(View v, int stage, int integ) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.np) return;
    const int s = v.b_sim[i];
    const SimDev &S = v.sims[s];
    if (!S.active) return;
    R vdr[3] = {0, 0, 0};
    for (int a = 0; a < D; ++a) vdr[a] = ((const R *)v.vdot[a])[i];
    integrate_stage<R, D>(v, S, i, s, stage, integ, vdr, ((const R *)v.udot)[i]);
}

// ---- dispatch ----
#define SPH_DISPATCH(PREC, DIM, KERN, CALL)                                       \
    do {                                                                          \
        if (PREC == SPH_MIXED) {                                                  \
            using R = float;                                                      \
            if (DIM == 2) { constexpr int D = 2; SPH_DISPATCH_K(KERN, CALL); }    \
            else { constexpr int D = 3; SPH_DISPATCH_K(KERN, CALL); }             \
        } else {                                                                  \
            using R = double;                                                     \
            if (DIM == 2) { constexpr int D = 2; SPH_DISPATCH_K(KERN, CALL); }    \
            else { constexpr int D = 3; SPH_DISPATCH_K(KERN, CALL); }             \
        }                                                                         \
    } while (0)
#define SPH_DISPATCH_K(KERN, CALL)                                                \
    switch (KERN) {                                                               \
        case SPH_KERNEL_GAUSSIAN: { constexpr int K = SPH_KERNEL_GAUSSIAN; CALL; break; } \
        case SPH_KERNEL_LUCY: { constexpr int K = SPH_KERNEL_LUCY; CALL; break; }         \
        case SPH_KERNEL_DEBRUN: { constexpr int K = SPH_KERNEL_DEBRUN; CALL; break; }     \
        default: { constexpr int K = SPH_KERNEL_CUBIC; CALL; break; }                     \
    }

void launch_density(const View &v, int precision, int kernel, int stage, int block,
                    cudaStream_t s) {
    if (v.np <= 0) return;
    int nb = (v.np + block - 1) / block;
    SPH_DISPATCH(precision, v.dim, kernel, (k_density<R, D, K><<<nb, block, 0, s>>>(v, stage)));
}

void launch_heat(const View &v, int precision, int kernel, int block, cudaStream_t s) {
    if (v.np <= 0) return;
    int nb = (v.np + block - 1) / block;
    SPH_DISPATCH(precision, v.dim, kernel, (k_heat<R, D, K><<<nb, block, 0, s>>>(v)));
}

void launch_force(const View &v, int precision, int kernel, int viscosity, int heat,
                  int integrator, int stage, int mode, int block, cudaStream_t s) {
    if (v.np <= 0) return;
    int nb = (v.np + block - 1) / block;
    const int vh = (viscosity ? 1 : 0) | (heat ? 2 : 0);
#define SPH_FORCE(VH_) k_force<R, D, K, VH_><<<nb, block, 0, s>>>(v, stage, mode, integrator)
    SPH_DISPATCH(precision, v.dim, kernel, ({
                     switch (vh) {
                         case 0: SPH_FORCE(0); break;
                         case 1: SPH_FORCE(1); break;
                         case 2: SPH_FORCE(2); break;
                         default: SPH_FORCE(3); break;
                     }
                 }));
#undef SPH_FORCE
}

void launch_integrate(const View &v, int precision, int integrator, int stage, cudaStream_t s) {
    if (v.np <= 0) return;
    int nb = (v.np + 255) / 256;
    if (precision == SPH_MIXED) {
        if (v.dim == 2) k_integrate<float, 2><<<nb, 256, 0, s>>>(v, stage, integrator);
        else k_integrate<float, 3><<<nb, 256, 0, s>>>(v, stage, integrator);
    } else {
        if (v.dim == 2) k_integrate<double, 2><<<nb, 256, 0, s>>>(v, stage, integrator);
        else k_integrate<double, 3><<<nb, 256, 0, s>>>(v, stage, integrator);
    }
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
