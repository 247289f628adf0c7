// sph_device.cuh -- device helpers shared by the binning and pair kernels.
#pragma once

#include <cuda_runtime.h>

#include <type_traits>

#include "sph_internal.h"

namespace sph {

template <typename R> struct V4;
template <> struct V4<float> { using T = float4; };
template <> struct V4<double> { using T = double4_32a; };

template <typename R>
__device__ __forceinline__ typename V4<R>::T make_v4(R x, R y, R z, R w) {
    typename V4<R>::T o;
    o.x = x; o.y = y; o.z = z; o.w = w;
    return o;
}

// Cell coordinate of position x on axis a: the position is first wrapped
// into [0, L) (shift = L floor(x/L)), then binned with the cell edge.  The
// binning kernel and every pass that needs a particle's cell centre call
// this same function so the results agree bit for bit.
__device__ __forceinline__ int cell_coord(double x, const SimDev &S, int a, double *shift) {
    double k = floor(x * S.inv_L[a]);
    double sh = k * S.L[a];
    double xw = x - sh;
    int ci = (int)(xw * S.inv_edge[a]);
    if (ci < 0) ci = 0;
    if (ci >= S.nc[a]) ci = S.nc[a] - 1;
    *shift = sh;
    return ci;
}

__device__ __forceinline__ double cell_centre(int ci, const SimDev &S, int a) {
    return ((double)ci + 0.5) * S.edge[a];
}

// The reference's FP64 pair test (neighbour_list.py:168-178): dr = r_j - r_i,
// one minimum-image shift per axis with strict comparisons against L/2,
// rsq = dx*dx + dy*dy (+ dz*dz) summed left to right, no FMA contraction.
template <int D>
__device__ __forceinline__ double exact_rsq(double *const xe[3], const SimDev &S, int i, int j) {
    double rsq = 0.0;
#pragma unroll
    for (int a = 0; a < D; ++a) {
        double d = __dsub_rn(xe[a][j], xe[a][i]);
        if (d > S.half_L[a]) d = __dsub_rn(d, S.L[a]);
        if (d < -S.half_L[a]) d = __dadd_rn(d, S.L[a]);
        double sq = __dmul_rn(d, d);
        rsq = (a == 0) ? sq : __dadd_rn(rsq, sq);
    }
    return rsq;
}

// The exact test behind the rare guard-band branch.  Kept out of line: when
// inlined, the compiler predicates it and every candidate then pays its
// FP64 instructions, which on GB300's narrow FP64 pipe dominate the pass.
template <int D>
__device__ __noinline__ bool exact_in_set(double *const *xe, const SimDev *S, int i, int j) {
    double rsq = 0.0;
#pragma unroll
    for (int a = 0; a < D; ++a) {
        double d = __dsub_rn(xe[a][j], xe[a][i]);
        if (d > S->half_L[a]) d = __dsub_rn(d, S->L[a]);
        if (d < -S->half_L[a]) d = __dadd_rn(d, S->L[a]);
        double sq = __dmul_rn(d, d);
        rsq = (a == 0) ? sq : __dadd_rn(rsq, sq);
    }
    return rsq < S->thr;
}

// Compensated (Kahan) accumulation for FP32 sums; FP64 sums are plain.
template <typename R> struct Acc;
template <> struct Acc<float> {
    float s, c;
    __device__ __forceinline__ void init(float x) { s = x; c = 0.0f; }
    __device__ __forceinline__ void add(float x) {
        float y = __fsub_rn(x, c);
        float t = __fadd_rn(s, y);
        c = __fsub_rn(__fsub_rn(t, s), y);
        s = t;
    }
    __device__ __forceinline__ float get() const { return s; }
    // the compensated value in FP64: s - c carries the bits s lost
    __device__ __forceinline__ double get64() const { return (double)s - (double)c; }
};
template <> struct Acc<double> {
    double s;
    __device__ __forceinline__ void init(double x) { s = x; }
    __device__ __forceinline__ void add(double x) { s += x; }
    __device__ __forceinline__ double get() const { return s; }
    __device__ __forceinline__ double get64() const { return s; }
};

// Blocked compensated sum: the terms of one neighbour cell (a handful) are
// added plainly into `part`, which is folded into the compensated total once
// per cell.  The per-cell partials carry a few ulp; the compensation keeps
// the sum over cells from growing further.
template <typename R> struct BAcc {
    Acc<R> total;
    R part;
    __device__ __forceinline__ void init(R x) { total.init(x); part = (R)0; }
    __device__ __forceinline__ void add(R x) { part += x; }
    __device__ __forceinline__ void flush() { total.add(part); part = (R)0; }
    __device__ __forceinline__ R get() { flush(); return total.get(); }
    __device__ __forceinline__ double get64() { flush(); return total.get64(); }
};

// Approximate single-precision division for terms that do not enter a
// cancelling sum (viscosity): MUFU reciprocal, about 2 ulp; exact in FP64.
template <typename R> __device__ __forceinline__ R fdiv(R a, R b);
template <> __device__ __forceinline__ float fdiv<float>(float a, float b) {
    return __fdividef(a, b);
}
template <> __device__ __forceinline__ double fdiv<double>(double a, double b) { return a / b; }


// ---- smoothing kernels: W(r) and g = (dW/dr)/r, so dwdx = g (r_j - r_i) ----
// Lucy (spkernel.py:86-118), Gaussian (spkernel.py:39-52, Lucy's gradient
// sign), Debrun (spkernel.py:120-153), M4 cubic spline (support 2h).
template <typename R> struct KConst {
    R h, h_lo, inv_h, inv_h_lo, sig, g0;  // g0: Lucy -12 sig/h^2, Gaussian -2/h^2, cubic sig/h^2
    R g0_h2;                              // g0 / h^2 (the refined Lucy gradient)
    R inv_h2, inv_h2_lo;                  // 1/h^2 as a hi/lo pair (the refined Gaussian)
};

template <typename R> __device__ __forceinline__ const SimConst<R> &sconst(const SimDev &S);
template <> __device__ __forceinline__ const SimConst<float> &sconst<float>(const SimDev &S) {
    return S.cf;
}
template <> __device__ __forceinline__ const SimConst<double> &sconst<double>(const SimDev &S) {
    return S.cd;
}

// Kernel constants of smoothing length `which` (0 short, 1 long).  h and 1/h
// are hi/lo pairs: q = fma(r, hi, r*lo) is unbiased to ~0.5 ulp instead of
// carrying the rounding of 1/h into every term alike, and h - r keeps the
// part of h that (float)h misses, which near the support edge would shift
// every term's vanishing factor alike.
template <typename R>
__device__ __forceinline__ KConst<R> make_kconst(const SimDev &S, int which) {
    const SimConst<R> &c = sconst<R>(S);
    KConst<R> k;
    k.h = c.h[which];
    k.h_lo = c.h_lo[which];
    k.inv_h = c.inv_h[which];
    k.inv_h_lo = c.inv_h_lo[which];
    k.sig = c.sig[which];
    k.g0 = c.g0[which];
    k.g0_h2 = c.g0_h2[which];
    k.inv_h2 = c.inv_h2[which];
    k.inv_h2_lo = c.inv_h2_lo[which];
    return k;
}

// The long kernel's constants with the cohesive factor -2a folded into its
// gradient (the force passes need only -2a grad W_l).
template <typename R>
__device__ __forceinline__ KConst<R> make_kconst_cohesive(const SimDev &S) {
    KConst<R> k = make_kconst<R>(S, 1);
    const SimConst<R> &c = sconst<R>(S);
    k.g0 = c.g0_pl;
    k.g0_h2 = c.g0_h2_pl;
    return k;
}

template <typename R> __device__ __forceinline__ R rexp(R x);
template <> __device__ __forceinline__ float rexp<float>(float x) { return expf(x); }
template <> __device__ __forceinline__ double rexp<double>(double x) { return exp(x); }
// correctly rounded reciprocal (cheaper than a division)
template <typename R> __device__ __forceinline__ R rrcp(R x);
template <> __device__ __forceinline__ float rrcp<float>(float x) { return __frcp_rn(x); }
template <> __device__ __forceinline__ double rrcp<double>(double x) { return 1.0 / x; }

// 1/sqrt(x) by the MUFU approximation, 0 at x = 0
__device__ __forceinline__ float rsqrt0(float x) { return x > 0.0f ? rsqrtf(x) : 0.0f; }

// The distance of a pair, in one of two forms.
//
// Refined (make_dist; the force and heat-flux passes, whose pair gradients
// enter sums that cancel): in FP32, r = rsq * ir with ir the MUFU reciprocal
// square root (about 2 ulp) and e = (rsq - r^2) / r, so that r + e/2 is
// sqrt(rsq) to O(eps^2).  The compact kernels then form their vanishing
// factor h - r as ((h_hi - r) + h_lo) - e/2: h_hi - r is exact for r in
// [h/2, 2h] (Sterbenz), so the factor keeps its relative accuracy up to the
// support edge instead of inheriting the roundings of sqrt and r/h.  On the
// pressure-only golden systems, whose near-lattice pair forces cancel to
// well below their terms, this removes about a fifth of the net force's
// error for two operations per pair.  The cubic spline keeps its direct
// form (its passes are the 3D workload's, which meets 1e-6 without).
//
// Plain (plain_dist; the density passes and the kernel-table call):
// r = sqrt(rsq) correctly rounded, e = 0, and the kernels in their direct
// forms of q = r/h.
//
// FP64 passes use the direct forms with r = sqrt(rsq) either way.
template <typename R> struct Dist {
    R rsq, r, e, ir;   // ir = 1/r where a kernel needs it (0 at r = 0)
};
template <typename R> __device__ __forceinline__ Dist<R> make_dist(R rsq);
template <> __device__ __forceinline__ Dist<float> make_dist<float>(float rsq) {
    Dist<float> d;
    d.rsq = rsq;
    d.ir = rsqrt0(rsq);
    d.r = rsq * d.ir;
    d.e = __fmaf_rn(-d.r, d.r, rsq) * d.ir;
    return d;
}
template <> __device__ __forceinline__ Dist<double> make_dist<double>(double rsq) {
    Dist<double> d;
    d.rsq = rsq;
    d.r = sqrt(rsq);
    d.e = 0.0;
    d.ir = d.r > 0.0 ? 1.0 / d.r : 0.0;
    return d;
}
template <typename R> __device__ __forceinline__ Dist<R> dist_of(R r) {
    Dist<R> d;
    d.rsq = r * r;
    d.r = r;
    d.e = (R)0;
    d.ir = r > (R)0 ? rrcp<R>(r) : (R)0;
    return d;
}
template <typename R> __device__ __forceinline__ Dist<R> plain_dist(R rsq) {
    return dist_of<R>(sqrt(rsq));
}

// REF: the refined FP32 forms (see Dist); they apply to FP32 only
template <typename R, bool REF>
constexpr bool refined_v = REF && std::is_same<R, float>::value;

// q = r/h with 1/h as a hi/lo pair (refined: with the correction e/2)
template <typename R, bool REF>
__device__ __forceinline__ R qof(const KConst<R> &k, const Dist<R> &d) {
    if constexpr (std::is_same<R, double>::value) {
        return d.r * k.inv_h;
    } else if constexpr (REF) {
        return __fmaf_rn(d.r, k.inv_h, __fmaf_rn(d.e, 0.5f * k.inv_h, d.r * k.inv_h_lo));
    } else {
        return __fmaf_rn(d.r, k.inv_h, d.r * k.inv_h_lo);
    }
}
// h - r in FP32, refined: ((h_hi - r) + h_lo) - e/2
__device__ __forceinline__ float h_minus_r(const KConst<float> &k, const Dist<float> &d) {
    return __fmaf_rn(-0.5f, d.e, (k.h - d.r) + k.h_lo);
}

// *w receives W/sigma (the normalisation is applied once per particle in
// FP64, which keeps its rounding out of every term); *g the full (dW/dr)/r.
template <int K, typename R, bool REF = false>
__device__ __forceinline__ void kernel_wg(const KConst<R> &k, const Dist<R> &d, R *w, R *g) {
    constexpr bool refined = refined_v<R, REF>;
    if (K == SPH_KERNEL_LUCY) {
        if constexpr (refined) {
            // t = h - r = h (1 - q): W/sigma = (1 + 3q)(1 - q)^3 and
            // g = g0 (1 - q)^2 = (g0 / h^2) t^2 (g0_h2 rounded once: a scale
            // common to every term of the sum)
            const float t = h_minus_r(k, d);
            if (t > 0.0f) {
                const float s = t * k.inv_h;
                *w = (4.0f - 3.0f * s) * (s * s * s);
                *g = k.g0_h2 * (t * t);
            } else {
                *w = 0.0f;
                *g = 0.0f;
            }
        } else {
            const R q = qof<R, REF>(k, d);
            if (q < (R)1) {
                const R s = (R)1 - q;
                const R s2 = s * s;
                *w = ((R)1 + (R)3 * q) * (s2 * s);
                *g = k.g0 * s2;
            } else {
                *w = (R)0;
                *g = (R)0;
            }
        }
    } else if (K == SPH_KERNEL_GAUSSIAN) {
        R q2;
        if constexpr (refined) {
            // q^2 = rsq / h^2 in one rounding (1/h^2 as a hi/lo pair)
            q2 = __fmaf_rn(d.rsq, k.inv_h2, d.rsq * k.inv_h2_lo);
        } else {
            const R q = qof<R, REF>(k, d);
            q2 = q * q;
        }
        const R e = rexp<R>(-q2);
        *w = e;
        *g = k.g0 * k.sig * e;
    } else if (K == SPH_KERNEL_DEBRUN) {
        R s;
        if constexpr (refined) s = h_minus_r(k, d);
        else s = k.h - d.r;
        if (s > (R)0) {
            *w = s * s * s;
            *g = k.g0 * s * s * d.ir;
        } else {
            *w = (R)0;
            *g = (R)0;
        }
    } else {  // cubic spline, direct form, evaluated without branches (selects)
        const R q = qof<R, false>(k, d);
        R s = (R)2 - q;
        s = s > (R)0 ? s : (R)0;
        const R w_in = (R)1 - (R)1.5 * q * q + (R)0.75 * q * q * q;
        const R g_in = k.g0 * ((R)-3 + (R)2.25 * q);
        const R w_out = (R)0.25 * s * s * s;
        // -0.75 sig s^2 / (h r) = g0 * (-0.75 s^2 h / r) with g0 = sig/h^2
        const R g_out = k.g0 * ((R)-0.75 * s * s * k.h) * d.ir;
        const bool inner = q < (R)1;
        *w = inner ? w_in : w_out;
        *g = inner ? g_in : g_out;
    }
}

template <int K, typename R, bool REF = false>
__device__ __forceinline__ R kernel_g(const KConst<R> &k, const Dist<R> &d) {
    R w, g;
    kernel_wg<K, R, REF>(k, d, &w, &g);
    return g;
}

__device__ __forceinline__ void set_err(int *err, int *err_any, int s, int code) {
    atomicCAS(&err[s], 0, code);
    atomicCAS(err_any, 0, code);
}

// Index checks of the checking build (-DSPH_DEBUG_CHECKS): a failed check
// records SPH_EBOUNDS and the caller skips the access; the release build
// compiles them away.
#ifdef SPH_DEBUG_CHECKS
__device__ __forceinline__ bool sph_in_bounds(bool ok, int *err_any) {
    if (!ok && err_any) atomicCAS(err_any, 0, SPH_EBOUNDS);
    return ok;
}
#define SPH_IN_BOUNDS(cond, err_any) sph_in_bounds((cond), (err_any))
#else
#define SPH_IN_BOUNDS(cond, err_any) true
#endif

}  // namespace sph
