// sph_force.cuh -- the force pass and the integrator stage:
//
//   k_force   : pressure + cohesive accelerations, Monaghan viscosity, energy
//               rate incl. conduction (forces.py:338-405, c_forces.pyx:96-111,
//               163-178, 224-237) fused with the integrator stage update
//               (integrator.py:14-103), periodic teleport (box.py:33-47) and the
//               thermostat (particles.py:450-457).
//
// Instantiated per precision in sph_force_f32.cu / sph_force_f64.cu.
#pragma once

#include "sph_pairs.cuh"

namespace sph {

// Next evaluation state: positions/velocities/energy in FP64 plus packed
// cell-local copies relative to the particle's cell (binned at x0).
template <typename R, int D>
__device__ __forceinline__ void write_eval_state(const View &v, const SimDev &S, int i,
                                                 const double *x, const double *vel, double u,
                                                 double m) {
    using T4 = typename V4<R>::T;
    R xl[3] = {0, 0, 0}, vv[3] = {0, 0, 0};
    bool skin = false;
    double moved = 0.0;   // squared displacement from the pair lists' build
#pragma unroll
    for (int a = 0; a < D; ++a) {
        // relative to the cell the particle was binned in; with binning on
        // demand the step may have started from a wrapped position
        double d = x[a] - v.org[a][i];
        if (d > S.half_L[a]) d -= S.L[a];
        if (d < -S.half_L[a]) d += S.L[a];
        if (v.vl_on) {
            const float4 x0 = v.vl_x0[i];
            const double m = d - (double)(a == 0 ? x0.x : (a == 1 ? x0.y : x0.z));
            moved += m * m;
        }
        xl[a] = (R)d;
        vv[a] = (R)vel[a];
        v.xe_out[a][i] = x[a];
        v.ve_out[a][i] = vel[a];
        // the cell list finds every pair while each particle stays within its
        // cell grown by the slack
        skin |= fabs(d) > S.box_half[a];
    }
    // with pair lists: a pair can be missing from them once a particle has
    // moved half the skin
    skin |= moved > S.vl_eskin2;
    if (skin) set_err(v.err, v.err_any, v.b_sim[i], SPH_ESKIN);
    v.ue_out[i] = u;
    ((T4 *)v.pk_pos_out)[i] = make_v4<R>(xl[0], xl[1], xl[2], (R)m);
    ((T4 *)v.pk_vel_out)[i] = make_v4<R>(vv[0], vv[1], vv[2], (R)0);
}

// Final state of the step into A (same slot as B), with the teleport wrap.
// In rebin mode it is also the next step's start state in B and its packed
// stage-0 copies, relative to the unchanged cells (the final stage writes
// pk_*_out == buffer 0 for improved Euler and RK4); a particle past half of
// its cell slack -- with pair lists, one that has moved a quarter of the
// skin since their build -- asks for a binning before the next step.
template <typename R, int D>
__device__ __forceinline__ void write_final_state(const View &v, const SimDev &S, int i,
                                                  double *x, const double *vel, double u) {
    using T4 = typename V4<R>::T;
    R xl[3] = {0, 0, 0}, vv[3] = {0, 0, 0};
    bool far = false;
    double moved = 0.0;
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
            if (v.vl_on) {
                const float4 x0 = v.vl_x0[i];
                const double m = d - (double)(a == 0 ? x0.x : (a == 1 ? x0.y : x0.z));
                moved += m * m;
            } else {
                far |= fabs(d) > S.rebin_half[a];
            }
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
        far |= moved > S.vl_gate2;
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
// them carries neither their registers nor their branches).  ONE: a single
// simulation, whose constants come from the kernel parameters.
// Register caps: 64 (4 blocks of 256 per SM) measured 17% faster than the
// unconstrained 80-104 despite a few spilled words outside the pair loop; a
// single 2D simulation, with its constants out of registers, runs best at 51
// (5 blocks), 3D at 64.
// LIST: the pair lists (tuning.pair_scheme 2) instead of the cell windows.
template <typename R, int D, int K, int VH, bool ONE, bool LIST = false>
__device__ __forceinline__ void force_one(const View &v, int stage, int mode, int integ, int i) {
    constexpr bool visc = (VH & 1) != 0;
    constexpr bool heat = (VH & 2) != 0;
    const bool active = i < v.np;
    const int ii = active ? i : v.np - 1;
    using T4 = typename V4<R>::T;
    const T4 *__restrict__ P = (const T4 *)v.pk_pos_in;
    const T4 *__restrict__ FV = (const T4 *)v.pk_fv;
    const R *__restrict__ RHO = (const R *)v.rho;
    const T4 *__restrict__ Q = (const T4 *)v.pk_q;
    const int s = v.b_sim[ii];
    const SimDev &S = ONE ? v.one : v.sims[s];
    if (S.cl_on) return;   // evaluated (and integrated) by the cluster passes
    KConst<R> ks = make_kconst<R>(S, 0);
    // the long kernel with pco_i/rho_l,i^2 + pco_j/rho_l,j^2 = -2a folded in
    KConst<R> kl = make_kconst_cohesive<R>(S);
    const SimConst<R> &sc = sconst<R>(S);
    const R hs = sc.hs, eps_h2 = sc.eps_h2;
    const R alpha_c = sc.alpha_c, beta = sc.beta;
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
        const Dist<R> dd = make_dist<R>(rsq);
        const R gl = kernel_g<K, R, true>(kl, dd);   // -2a grad W_l / r
        const T4 fvj = FV[j];
        R dvdx = (fvj.x - vix) * d[0] + (fvj.y - viy) * d[1];
        if (D == 3) dvdx += (fvj.z - viz) * d[2];
        // beyond the short support gs = 0: the pressure and viscosity terms
        // vanish and gsum = gl bit for bit
        R gsum = gl, gs = (R)0;
        // the heat record {q/rho^2, rho}: with heat flux in 3D it also
        // carries the density the viscosity needs
        T4 qj = make_v4<R>(0, 0, 0, 0);
        if constexpr (NEAR) {
            if (heat) qj = Q[j];
            gs = kernel_g<K, R, true>(ks, dd);
            R ps = fsi + (D == 2 ? fvj.z : fvj.w);
            // Monaghan viscosity on approaching pairs within the short
            // support (beyond it gs = 0, so ps no longer enters gsum and the
            // warp skips the block when none of its pairs needs it)
            if (visc && dvdx < (R)0 && gs != (R)0) {
                const R rhoj = D == 2 ? fvj.w : (heat ? qj.w : RHO[j]);
                R mu = fdiv<R>(hs * dvdx, rsq + eps_h2);
                ps += fdiv<R>((R)2 * (-alpha_c * mu + beta * mu * mu), rhoi + rhoj);
            }
            gsum = ps * gs + gl;
        }
        ax[0].add(gsum * d[0]);
        ax[1].add(gsum * d[1]);
        if (D == 3) ax[2].add(gsum * d[2]);
        // twice the energy-rate term; the sum is halved once at the end
        // (scaling by 2 is exact, so the bits are those of the halved terms)
        R du = gsum * dvdx * pj.w;
        if (heat && NEAR) {
            R dq = (qi.x + qj.x) * d[0] + (qi.y + qj.y) * d[1];
            if (D == 3) dq += (qi.z + qj.z) * d[2];
            du -= (R)2 * dq * gs * pj.w;
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
        if constexpr (LIST) for_list<R, D, true>(v, S, fr, P, i, P[i], body, cell_done);
        else for_pairs<R, D, D == 3, false>(v, S, fr, P, i, P[i], body, cell_done);
    }
    R vdr[3] = {ax[0].get(), ax[1].get(), ax[2].get()};
    R udr = (R)0.5 * ud.get();
    for (int a = 0; a < D; ++a) ((R *)v.vdot[a])[i] = vdr[a];
    ((R *)v.udot)[i] = udr;
    if (!isfinite(vdr[0]) || !isfinite(udr)) set_err(v.err, v.err_any, s, SPH_ENAN);
    if (mode == 0) return;

    integrate_stage<R, D>(v, S, i, s, stage, integ, vdr, udr);
}

// One thread per particle; PERSIST: the resident blocks of pass_grid walk
// the particles grid-stride (the same per-particle work, the same bits).
template <typename R, int D, int K, int VH, bool ONE, bool PERSIST>
__global__ void __launch_bounds__(256, (ONE && D == 2) ? 5 : 4) k_force(const __grid_constant__ View v, int stage,
                                                  int mode, int integ) {
    if constexpr (PERSIST) {
        for (int base = blockIdx.x * blockDim.x; base < v.np; base += gridDim.x * blockDim.x)
            force_one<R, D, K, VH, ONE>(v, stage, mode, integ, base + threadIdx.x);
    } else {
        force_one<R, D, K, VH, ONE>(v, stage, mode, integ, blockIdx.x * blockDim.x + threadIdx.x);
    }
}

// The force pass over the pair lists (mixed precision); a single
// simulation at SPH_VL_FORCE_BLOCKS (2D) / SPH_VL_FORCE3_BLOCKS (3D)
// resident blocks of 256 per SM.
#ifndef SPH_VL_FORCE_BLOCKS
#define SPH_VL_FORCE_BLOCKS 5
#endif
#ifndef SPH_VL_FORCE3_BLOCKS
#define SPH_VL_FORCE3_BLOCKS 4
#endif
#ifndef SPH_VL_FORCE_MULTI_BLOCKS
#define SPH_VL_FORCE_MULTI_BLOCKS 4
#endif
template <int D, int K, int VH, bool ONE>
__global__ void __launch_bounds__(256, ONE ? (D == 2 ? SPH_VL_FORCE_BLOCKS : SPH_VL_FORCE3_BLOCKS) : SPH_VL_FORCE_MULTI_BLOCKS)
    k_force_vl(const __grid_constant__ View v, int stage, int mode, int integ) {
    force_one<float, D, K, VH, ONE, true>(v, stage, mode, integ,
                                          blockIdx.x * blockDim.x + threadIdx.x);
}

// Integrator stage from the stored rates: the epilogue of k_force as a pass
// of its own, for steps whose velocities change between the force pass and
// the update (hard collisions).
template <typename R, int D>
__global__ void __launch_bounds__(256) k_integrate(View v, int stage, int integ, int cl_only) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.np) return;
    const int s = v.b_sim[i];
    const SimDev &S = v.sims[s];
    if (!S.active || (cl_only && !S.cl_on)) return;
    R vdr[3] = {0, 0, 0};
    for (int a = 0; a < D; ++a) vdr[a] = ((const R *)v.vdot[a])[i];
    integrate_stage<R, D>(v, S, i, s, stage, integ, vdr, ((const R *)v.udot)[i]);
}

// the persistent form for the mixed-precision pass only (see density_launch)
template <typename R, int D, int K, int VH, bool ONE>
void force_launch(const View &v, int stage, int mode, int integ, int block, cudaStream_t s) {
    if constexpr (std::is_same<R, float>::value) {
        if (v.vl_on) {
            k_force_vl<D, K, VH, ONE>
                <<<(v.np + block - 1) / block, block, 0, s>>>(v, stage, mode, integ);
            return;
        }
    }
    if (std::is_same<R, float>::value && v.persist) {
        auto *fn = k_force<R, D, K, VH, ONE, std::is_same<R, float>::value>;
        fn<<<pass_grid(v, fn, block), block, 0, s>>>(v, stage, mode, integ);
    } else {
        k_force<R, D, K, VH, ONE, false>
            <<<(v.np + block - 1) / block, block, 0, s>>>(v, stage, mode, integ);
    }
}

template <typename R>
void launch_force_t(const View &v, int kernel, int viscosity, int heat, int integrator, int stage,
                    int mode, int block, cudaStream_t s) {
    if (v.np <= 0) return;
    const int vh = (viscosity ? 1 : 0) | (heat ? 2 : 0);
#define SPH_FORCE(VH_)                                                                   \
    (v.one_sim ? force_launch<R, D, K, VH_, true>(v, stage, mode, integrator, block, s)  \
               : force_launch<R, D, K, VH_, false>(v, stage, mode, integrator, block, s))
#define SPH_FORCE_VH                                                                     \
    switch (vh) {                                                                        \
        case 0: SPH_FORCE(0); break;                                                     \
        case 1: SPH_FORCE(1); break;                                                     \
        case 2: SPH_FORCE(2); break;                                                     \
        default: SPH_FORCE(3); break;                                                    \
    }
    if (v.dim == 2) {
        constexpr int D = 2;
        SPH_DISPATCH_K(kernel, SPH_FORCE_VH);
    } else {
        constexpr int D = 3;
        SPH_DISPATCH_K(kernel, SPH_FORCE_VH);
    }
#undef SPH_FORCE_VH
#undef SPH_FORCE
}

template <typename R>
void launch_integrate_t(const View &v, int integrator, int stage, cudaStream_t s, int cl_only) {
    if (v.np <= 0) return;
    int nb = (v.np + 255) / 256;
    if (v.dim == 2) k_integrate<R, 2><<<nb, 256, 0, s>>>(v, stage, integrator, cl_only);
    else k_integrate<R, 3><<<nb, 256, 0, s>>>(v, stage, integrator, cl_only);
}

}  // namespace sph
