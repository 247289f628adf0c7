// sph_device.cuh -- device helpers shared by the binning and pair kernels.
#pragma once

#include <cuda_runtime.h>

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

// Approximate single-precision helpers for terms that do not enter a
// cancelling sum (viscosity, force-pass distances): MUFU reciprocal and
// reciprocal square root, about 2 ulp; exact operations in FP64 mode.
template <typename R> __device__ __forceinline__ R fdiv(R a, R b);
template <> __device__ __forceinline__ float fdiv<float>(float a, float b) {
    return __fdividef(a, b);
}
template <> __device__ __forceinline__ double fdiv<double>(double a, double b) { return a / b; }
template <typename R> __device__ __forceinline__ R fsqrt(R x);
template <> __device__ __forceinline__ float fsqrt<float>(float x) {
    return x > 0.0f ? x * rsqrtf(x) : 0.0f;
}
template <> __device__ __forceinline__ double fsqrt<double>(double x) { return sqrt(x); }


// ---- smoothing kernels: W(r) and g = (dW/dr)/r, so dwdx = g (r_j - r_i) ----
// Lucy (spkernel.py:86-118), Gaussian (spkernel.py:39-52, Lucy's gradient
// sign), Debrun (spkernel.py:120-153), M4 cubic spline (support 2h).
template <typename R> struct KConst {
    R h, inv_h, inv_h_lo, sig, g0;  // g0: Lucy -12 sig/h^2, Gaussian -2/h^2, cubic sig/h^2
};

template <typename R> __device__ __forceinline__ const SimConst<R> &sconst(const SimDev &S);
template <> __device__ __forceinline__ const SimConst<float> &sconst<float>(const SimDev &S) {
    return S.cf;
}
template <> __device__ __forceinline__ const SimConst<double> &sconst<double>(const SimDev &S) {
    return S.cd;
}

// Kernel constants of smoothing length `which` (0 short, 1 long).  1/h is a
// hi/lo pair: q = fma(r, hi, r*lo) is unbiased to ~0.5 ulp instead of
// carrying the rounding of 1/h into every term alike.
template <typename R>
__device__ __forceinline__ KConst<R> make_kconst(const SimDev &S, int which) {
    const SimConst<R> &c = sconst<R>(S);
    KConst<R> k;
    k.h = c.h[which];
    k.inv_h = c.inv_h[which];
    k.inv_h_lo = c.inv_h_lo[which];
    k.sig = c.sig[which];
    k.g0 = c.g0[which];
    return k;
}

template <typename R> __device__ __forceinline__ R rexp(R x);
template <> __device__ __forceinline__ float rexp<float>(float x) { return expf(x); }
template <> __device__ __forceinline__ double rexp<double>(double x) { return exp(x); }
template <typename R> __device__ __forceinline__ R rsqrt_(R x);
template <> __device__ __forceinline__ float rsqrt_<float>(float x) { return sqrtf(x); }
template <> __device__ __forceinline__ double rsqrt_<double>(double x) { return sqrt(x); }

template <typename R> __device__ __forceinline__ R qof(const KConst<R> &k, R r);
template <> __device__ __forceinline__ float qof<float>(const KConst<float> &k, float r) {
    return __fmaf_rn(r, k.inv_h, r * k.inv_h_lo);
}
template <> __device__ __forceinline__ double qof<double>(const KConst<double> &k, double r) {
    return r * k.inv_h;
}

// *w receives W/sigma (the normalisation is applied once per particle in
// FP64, which keeps its rounding out of every term); *g the full (dW/dr)/r.
// correctly rounded reciprocal (cheaper than a division)
template <typename R> __device__ __forceinline__ R rrcp(R x);
template <> __device__ __forceinline__ float rrcp<float>(float x) { return __frcp_rn(x); }
template <> __device__ __forceinline__ double rrcp<double>(double x) { return 1.0 / x; }

template <int K, typename R>
__device__ __forceinline__ void kernel_wg(const KConst<R> &k, R r, R *w, R *g) {
    if (K == SPH_KERNEL_LUCY) {
        R q = qof<R>(k, r);
        if (q < (R)1) {
            R s = (R)1 - q;
            R s2 = s * s;
            *w = ((R)1 + (R)3 * q) * (s2 * s);
            *g = k.g0 * s2;
        } else {
            *w = (R)0;
            *g = (R)0;
        }
    } else if (K == SPH_KERNEL_GAUSSIAN) {
        R q = qof<R>(k, r);
        R e = rexp<R>(-q * q);
        *w = e;
        *g = k.g0 * k.sig * e;
    } else if (K == SPH_KERNEL_DEBRUN) {
        if (r < k.h) {
            R s = k.h - r;
            *w = s * s * s;
            *g = (r > (R)0) ? k.g0 * s * s * rrcp<R>(r) : (R)0;
        } else {
            *w = (R)0;
            *g = (R)0;
        }
    } else {  // cubic spline, evaluated without branches (selects)
        R q = qof<R>(k, r);
        R s = (R)2 - q;
        s = s > (R)0 ? s : (R)0;
        R w_in = (R)1 - (R)1.5 * q * q + (R)0.75 * q * q * q;
        R g_in = k.g0 * ((R)-3 + (R)2.25 * q);
        R w_out = (R)0.25 * s * s * s;
        // -0.75 sig s^2 / (h r) = g0 * (-0.75 s^2 h / r) with g0 = sig/h^2
        R g_out = k.g0 * ((R)-0.75 * s * s * k.h) * rrcp<R>(r);
        bool inner = q < (R)1;
        *w = inner ? w_in : w_out;
        *g = inner ? g_in : g_out;
    }
}

template <int K, typename R>
__device__ __forceinline__ R kernel_g(const KConst<R> &k, R r) {
    R w, g;
    kernel_wg<K, R>(k, r, &w, &g);
    return g;
}

// (dW/dr)/r given r and ir = 1/r (0 at r = 0) in FP32: the cubic spline's
// outer branch and Debrun take ir instead of a correctly rounded reciprocal
// of r; the other kernels are kernel_g.
template <int K>
__device__ __forceinline__ float kernel_g_ir(const KConst<float> &k, float r, float ir) {
    if (K == SPH_KERNEL_CUBIC) {
        const float q = qof<float>(k, r);
        float s = 2.0f - q;
        s = s > 0.0f ? s : 0.0f;
        const float g_in = k.g0 * (-3.0f + 2.25f * q);
        const float g_out = k.g0 * (-0.75f * s * s * k.h) * ir;
        return q < 1.0f ? g_in : g_out;
    } else if (K == SPH_KERNEL_DEBRUN) {
        if (r < k.h) {
            const float s = k.h - r;
            return k.g0 * s * s * ir;
        }
        return 0.0f;
    } else {
        return kernel_g<K, float>(k, r);
    }
}

// 1/sqrt(x) by the MUFU approximation, 0 at x = 0 (r = x * ir is then the
// same as fsqrt's x * rsqrt(x))
__device__ __forceinline__ float rsqrt0(float x) { return x > 0.0f ? rsqrtf(x) : 0.0f; }

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
