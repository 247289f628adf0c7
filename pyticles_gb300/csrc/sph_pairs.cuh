// sph_pairs.cuh -- shared pieces of the pair passes: the pair iteration
// (cell windows, culling, FP32 fast test with exact FP64 fallback), the
// accumulation helpers and the precision/dimension/kernel dispatch.
//
// Every pass is a gather: thread i sums over all neighbours j in the 3^dim
// cells around its own cell, so each unordered pair is evaluated from both
// sides and no atomics touch particle data.  Positions are cell-local
// (relative to the particle's cell centre), which keeps FP32 differences
// accurate; the pair-set test runs on those FP32 distances with a 2^-12
// guard band and falls back to the reference's FP64 test for pairs inside
// the band, so the pair set is bit-exact.
#pragma once

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
    R edge_lo[3];   // FP32: the part of the cell edge that (float)edge misses
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
            edge_lo[a] = c.edge_lo[a];
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
//
// SELF: skip j == i, which only the home cell (offset 0) can hold, so only its
// loop tests for it.  A pass whose pair terms all carry the separation d
// (force, heat flux) may leave the test out: for j == i, d = 0 exactly and
// every kernel's gradient factor is finite at r = 0, so the terms add +0 and
// the sums keep their bits.
template <typename R, int D, bool PF = false, bool SELF = true, typename T4, typename F,
          typename G>
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
                if (!SPH_IN_BOUNDS(row + x >= 0 && row + x < S.ncells, v.err_any)) continue;
                const int gc = S.cell_off + mort[row + x];
                if (!SPH_IN_BOUNDS(gc >= S.cell_off && gc < S.cell_off + S.ncells, v.err_any))
                    continue;
                // offset of the window cell's frame from particle i; in FP32
                // the cell edge is a hi/lo pair, so that the offset carries one
                // rounding instead of the edge's rounding times the cell count
                R ox_ = (R)ox * fr.edge[0] - pi.x;
                R oy_ = (R)oy * fr.edge[1] - pi.y;
                R oz_ = (D == 3) ? (R)oz * fr.edge[2] - pi.z : (R)0;
                if constexpr (std::is_same<R, float>::value) {
                    ox_ = __fmaf_rn((R)ox, fr.edge_lo[0], ox_);
                    oy_ = __fmaf_rn((R)oy, fr.edge_lo[1], oy_);
                    if (D == 3) oz_ = __fmaf_rn((R)oz, fr.edge_lo[2], oz_);
                }
                const int jb = v.cell_start[gc], je = v.cell_start[gc + 1];
                if (!SPH_IN_BOUNDS(jb >= 0 && jb <= je && je <= v.np, v.err_any)) continue;
                auto scan = [&](auto near, auto self, auto mi) {
                    T4 pn;
                    if (PF) pn = P[jb < je ? jb : i];
                    for (int j = jb; j < je; ++j) {
                        T4 pj;
                        if (PF) {
                            pj = pn;
                            if (j + 1 < je) pn = P[j + 1];
                        }
                        if (decltype(self)::value && j == i) continue;
                        if (!PF) pj = P[j];
                        R d[3];
                        d[0] = pj.x + ox_;
                        d[1] = pj.y + oy_;
                        d[2] = (D == 3) ? pj.z + oz_ : (R)0;
                        if constexpr (decltype(mi)::value) fr.min_image(d);
                        R rsq = d[0] * d[0] + d[1] * d[1];
                        if (D == 3) rsq += d[2] * d[2];
                        if (rsq > fr.thr_hi) continue;
                        if (rsq >= fr.thr_lo && !exact_in_set<D>(v.xe_in, &S, i, j)) continue;
                        body(j, pj, d, rsq, near);
                    }
                };
                // the minimum image applies only on single-cell axes: the scan
                // is compiled with and without it (4.7% of the 2D density
                // pass, which otherwise tested small_mask per candidate)
                if (fr.small_mask) {
                    if (SELF && ox == 0 && oy == 0 && oz == 0)
                        scan(std::true_type{}, std::true_type{}, std::true_type{});
                    else if (__any_sync(__activemask(), dx * dx + dyz < fr.thr_s))
                        scan(std::true_type{}, std::false_type{}, std::true_type{});
                    else
                        scan(std::false_type{}, std::false_type{}, std::true_type{});
                } else {
                    if (SELF && ox == 0 && oy == 0 && oz == 0)
                        scan(std::true_type{}, std::true_type{}, std::false_type{});
                    else if (__any_sync(__activemask(), dx * dx + dyz < fr.thr_s))
                        scan(std::true_type{}, std::false_type{}, std::false_type{});
                    else
                        scan(std::false_type{}, std::false_type{}, std::false_type{});
                }
                cell_done();
            }
        }
    }
}

// Window offset k - 3 of a list entry's 3-bit field k, as an exact float:
// 2^23 + k built from its bits, minus 2^23 + 3.
__device__ __forceinline__ float vl_offset(unsigned k) {
    return __fsub_rn(__int_as_float(0x4B000000 | k), 8388611.0f);
}

// Iterates the pair set of particle i from its pair list (tuning.pair_scheme
// 2; FP32): the near entries, then with FAR the far ones, each in the
// order of the build (window cells in raster order, particles in cell
// order), with the same fast test and exact FP64 fallback as for_pairs.
// body(j, pj, d, rsq, near) as in for_pairs; cell_done() folds the blocked
// sums every 16 entries.  A far entry lay beyond the short support plus the
// skin at the build, so while the lists hold it stays beyond the support:
// the far bodies drop the short-kernel terms, which are exactly zero.
//
// Entries come four to a 16-byte group (near groups from row 0 up, far
// groups from row cap/4 - 1 down, a far group's entries from its last slot
// back); the next group is loaded before the current one is evaluated, so
// that the stream of entries from HBM overlaps the arithmetic.
//
// The separation is rebuilt from the entry's window offset: d = (p_j - p_i)
// + o e + o e_lo with the cell edge as a hi/lo pair, every rounding at the
// magnitude of d.
template <typename R, int D, bool FAR, typename T4, typename F, typename G>
__device__ __forceinline__ void for_list(const View &v, const SimDev &S,
                                         const PairFrame<R, D> &fr, const T4 *__restrict__ P,
                                         int i, const T4 &pi, F body, G cell_done) {
    static_assert(std::is_same<R, float>::value, "pair lists: mixed precision");
    constexpr int kBits = vl_index_bits(D);
    const unsigned cnt = v.vl_cnt[i];
    const int nn = (int)(cnt & 0xffffu), nf = (int)(cnt >> 16);
    const long long st = v.vl_stride;
    auto one = [&](int code, auto near) {
        const int j = code & vl_index_mask(D);
        if (!SPH_IN_BOUNDS(j >= 0 && j < v.np, v.err_any)) return;
        const unsigned t = (unsigned)code >> kBits;
        const float fx = vl_offset(t & 7u);
        const float fy = vl_offset(D == 3 ? (t >> 3) & 7u : t >> 3);
        const T4 pj = P[j];
        R d[3];
        d[0] = __fmaf_rn(fx, fr.edge_lo[0], __fmaf_rn(fx, fr.edge[0], __fsub_rn(pj.x, pi.x)));
        d[1] = __fmaf_rn(fy, fr.edge_lo[1], __fmaf_rn(fy, fr.edge[1], __fsub_rn(pj.y, pi.y)));
        d[2] = (R)0;
        R rsq = d[0] * d[0] + d[1] * d[1];
        if (D == 3) {
            const float fz = vl_offset(t >> 6);
            d[2] = __fmaf_rn(fz, fr.edge_lo[2], __fmaf_rn(fz, fr.edge[2], __fsub_rn(pj.z, pi.z)));
            rsq += d[2] * d[2];
        }
        if (rsq > fr.thr_hi) return;
        if (rsq >= fr.thr_lo && !exact_in_set<D>(v.xe_in, &S, i, j)) return;
        body(j, pj, d, rsq, near);
    };
    // n entries from group pointer g, stepping `dir` rows per group; slots
    // in order 0..3 (near) or 3..0 (far).  Measured on the 2D fluid: a
    // lookahead of one group is enough (two, or the group's four records
    // loaded ahead of their tests, were 3-6% slower: more registers)
    auto walk = [&](const int4 *g, long long dir, int n, auto near, auto rev) {
        const int ng = (n + 3) >> 2;
        int4 cur = ng > 0 ? *g : make_int4(0, 0, 0, 0);
        for (int k = 0; k < ng; ++k) {
            const int4 nxt = k + 1 < ng ? g[(k + 1) * dir] : cur;
            const int left = n - 4 * k;
            if constexpr (decltype(rev)::value) {
                one(cur.w, near);
                if (left > 1) one(cur.z, near);
                if (left > 2) one(cur.y, near);
                if (left > 3) one(cur.x, near);
            } else {
                one(cur.x, near);
                if (left > 1) one(cur.y, near);
                if (left > 2) one(cur.z, near);
                if (left > 3) one(cur.w, near);
            }
            if ((k & 3) == 3) cell_done();
            cur = nxt;
        }
        cell_done();
    };
    const int4 *E = (const int4 *)v.vl_ent + i;
    walk(E, st, nn, std::true_type{}, std::false_type{});
    if constexpr (FAR)
        walk(E + (long long)((v.vl_cap >> 2) - 1) * st, -st, nf, std::false_type{},
             std::true_type{});
}

// Blocks of a pair-pass launch: one thread per particle, or with v.persist
// only the blocks the device holds at once (SMs x resident blocks of this
// kernel at this block size, cached per kernel), which then walk the
// particles grid-stride.
int resident_blocks(const void *kernel, int block);
template <typename F> inline int pass_grid(const View &v, F *kernel, int block) {
    const int nb = (v.np + block - 1) / block;
    if (!v.persist) return nb;
    const int cap = resident_blocks((const void *)kernel, block);
    return nb < cap ? nb : cap;
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

}  // namespace sph
