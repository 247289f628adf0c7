// sph_cluster.cu -- the cluster-pair scheme of the pair passes (tuning
// pair_scheme = 1): 3D simulations in mixed precision, each with its own
// columns, clusters and lists in flattened tables.
//
// The cell-window passes (sph_pairs.cu, sph_force.cuh) give every lane its own
// particle and its own neighbour cells; in 3D the lanes of a warp then sit in
// two or three home cells, cull different window cells and run different trip
// counts, and 62% of the candidates they test lie beyond the cutoff.  Here a
// warp takes a cluster of 8 spatially compact particles and walks a list of
// 4-particle j-clusters whose bounding boxes come within the cutoff: every
// list entry is 8 x 4 pair tests on all 32 lanes, with the j positions read
// as four 16-byte records, and the j-clusters are culled box to box once per
// step instead of cell by cell in every pass.
//
// Build (each step, at the stage-0 positions):
//   k_cl_key/scatter/fsort : counting sort of the particles into fine cells
//                            (columns of about 8 particles' width in x and y,
//                            slabs of a quarter of that in z), ordered by slab
//                            within a column, by sorted index within a slab
//   k_cl_cols/slots        : clusters of 8 consecutive particles per column
//                            (the last one padded), slot <-> particle maps and
//                            each cluster's lattice reference point
//   k_cl_pack              : cluster-local FP32 positions (every evaluation)
//   k_cl_bbox, k_cl_list   : boxes of the clusters and of their halves; per
//                            i-cluster the j-halves of the same simulation
//                            within the cutoff plus twice the allowed drift,
//                            with the shift between the two lattice points,
//                            the entries within the short kernel's support in
//                            front, into a region of lstride entries (sized
//                            by the engine from a measured build)
// Passes: k_cl_density (+ EOS), k_cl_heat, k_cl_force (rates; the integrator
// stage runs as k_integrate).  Simulations whose boxes are too narrow for
// the columns stay on the cell-window passes in the same steps.
//
// Each particle sums its pairs in list order (j-clusters in a fixed order
// derived from its simulation's state), each lane over its quarter of every
// j-cluster, and the four quarters are added in a fixed tree, so the results
// are deterministic and the same alone or in a batch; they differ from the
// cell scheme's in rounding only.
#include <type_traits>

#include "sph_pairs.cuh"

namespace sph {
namespace {

constexpr int kBlock = 256;
constexpr float kFar = 1.0e18f;    // padding slots: beyond any cutoff and lattice shift
constexpr float kEmpty = 1.0e30f;  // box of an empty half: lo > hi

int nblocks(long long n, int block) { return (int)std::max<long long>(1, (n + block - 1) / block); }

__global__ void k_cl_key(const __grid_constant__ View v, const __grid_constant__ ClusterSet c) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.np) return;
    if (!SPH_IN_BOUNDS(i < c.nall, v.err_any)) return;
    const int sim = v.b_sim[i];
    const SimDev &S = v.sims[sim];
    if (!S.cl_on) {   // on the cell-window passes
        c.fkey[i] = -1;
        return;
    }
    const ClGeom &g = c.geom[sim];
    const double step[3] = {g.wxd, g.wyd, g.gzd};
    const int nk[3] = {g.ncx, g.ncy, g.nslab};
    int k[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double x = v.xe_in[a][i];
        const double xw = x - S.L[a] * floor(x * S.inv_L[a]);
        int q = (int)(xw / step[a]);
        q = q < 0 ? 0 : (q >= nk[a] ? nk[a] - 1 : q);
        k[a] = q;
    }
    const int key = g.fine_off + (k[1] * g.ncx + k[0]) * g.nslab + k[2];
    if (!SPH_IN_BOUNDS(key >= 0 && key < c.nfine, v.err_any)) return;
    c.fkey[i] = key;
    c.frank[i] = atomicAdd(&c.fcount[key], 1);
}

__global__ void k_cl_scatter(const __grid_constant__ View v, const __grid_constant__ ClusterSet c) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.np) return;
    if (!SPH_IN_BOUNDS(i < c.nall, v.err_any)) return;
    const int key = c.fkey[i];
    if (key < 0) return;
    const int dst = c.fstart[key] + c.frank[i];
    if (SPH_IN_BOUNDS(dst >= 0 && dst < v.np, v.err_any)) c.ford[dst] = i;
}

// Members of a fine cell in ascending sorted index: the atomic ranks of the
// scatter depend on timing, this order does not.
__global__ void k_cl_fsort(const __grid_constant__ ClusterSet c) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= c.nfine) return;
    const int b = c.fstart[f], e = c.fstart[f + 1];
    for (int p = b + 1; p < e; ++p) {
        const int x = c.ford[p];
        int q = p - 1;
        while (q >= b && c.ford[q] > x) {
            c.ford[q + 1] = c.ford[q];
            --q;
        }
        c.ford[q + 1] = x;
    }
}

// First fine cell of global column col.
__device__ __forceinline__ int col_fine(const ClGeom &g, int col) {
    return g.fine_off + (col - g.col_off) * g.nslab;
}

__global__ void k_cl_cols(const __grid_constant__ ClusterSet c) {
    const int col = blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= c.ncol) return;
    const ClGeom &g = c.geom[c.colsim[col]];
    const int f0 = col_fine(g, col);
    const int cnt = c.fstart[f0 + g.nslab] - c.fstart[f0];
    c.colcnt[col] = (cnt + 7) >> 3;
}

__global__ void k_cl_slots(const __grid_constant__ View v, const __grid_constant__ ClusterSet c) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= c.fstart[c.nfine]) return;   // the particles on cluster pairs
    if (!SPH_IN_BOUNDS(p < c.nall, v.err_any)) return;
    const int i = c.ford[p];
    if (!SPH_IN_BOUNDS(i >= 0 && i < v.np && i < c.nall, v.err_any)) return;
    const int sim = v.b_sim[i];
    const ClGeom &g = c.geom[sim];
    const int local = c.fkey[i] - g.fine_off;
    const int lcol = local / g.nslab;
    const int col = g.col_off + lcol;
    const int q = p - c.fstart[g.fine_off + lcol * g.nslab];
    if (!SPH_IN_BOUNDS(col >= 0 && col < c.ncol, v.err_any)) return;
    const int cl = c.colcl[col] + (q >> 3);
    const int slot = cl * 8 + (q & 7);
    if (!SPH_IN_BOUNDS(cl >= 0 && cl < c.ncl_max, v.err_any)) return;
    c.slot_idx[slot] = i;
    c.slot_of[i] = slot;
    // the first particle of a cluster lies in its lowest slab
    if ((q & 7) == 0) {
        c.cref[cl] = make_int4(lcol % g.ncx, lcol / g.ncx, local % g.nslab, col);
        c.csim[cl] = sim;
    }
}

// Positions relative to the cluster's lattice point (column centre in x and
// y, slab floor in z), with one periodic correction; evaluations after the
// first also check the drift since the build against the allowed slack.
__global__ void k_cl_pack(const __grid_constant__ View v, const __grid_constant__ ClusterSet c,
                          int stage) {
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= c.slots_max || slot >= 8 * c.colcl[c.ncol]) return;
    const int i = c.slot_idx[slot];
    if (i < 0) {
        c.cpos[slot] = make_float4(kFar, kFar, kFar, 0.0f);
        return;
    }
    const int sim = c.csim[slot >> 3];
    const SimDev &S = v.sims[sim];
    const ClGeom &g = c.geom[sim];
    const int4 r = c.cref[slot >> 3];
    const double ref[3] = {(r.x + 0.5) * g.wxd, (r.y + 0.5) * g.wyd, r.z * g.gzd};
    float l[3];
    bool skin = false;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const double x = v.xe_in[a][i];
        double d = x - ref[a];
        if (d > S.half_L[a]) d -= S.L[a];
        if (d < -S.half_L[a]) d += S.L[a];
        l[a] = (float)d;
        if (stage > 0) {
            double m = x - v.b_pos[a][i];
            if (m > S.half_L[a]) m -= S.L[a];
            if (m < -S.half_L[a]) m += S.L[a];
            skin |= fabs(m) > S.slack_half[a];
        }
    }
    if (skin) set_err(v.err, v.err_any, sim, SPH_ESKIN);
    c.cpos[slot] = make_float4(l[0], l[1], l[2], (float)v.b_m[i]);
}

__global__ void k_cl_bbox(const __grid_constant__ ClusterSet c) {
    const int cl = blockIdx.x * blockDim.x + threadIdx.x;
    if (cl >= c.ncl_max || cl >= c.colcl[c.ncol]) return;
    float lo[2][3], hi[2][3];
    for (int h = 0; h < 2; ++h)
        for (int a = 0; a < 3; ++a) {
            lo[h][a] = kEmpty;
            hi[h][a] = -kEmpty;
        }
    for (int k = 0; k < 8; ++k) {
        const int slot = cl * 8 + k;
        if (c.slot_idx[slot] < 0) continue;
        const float4 p = c.cpos[slot];
        const float x[3] = {p.x, p.y, p.z};
        const int h = k >> 2;
        for (int a = 0; a < 3; ++a) {
            lo[h][a] = fminf(lo[h][a], x[a]);
            hi[h][a] = fmaxf(hi[h][a], x[a]);
        }
    }
    for (int h = 0; h < 2; ++h) {
        c.jbox[2 * (2 * cl + h)] = make_float4(lo[h][0], lo[h][1], lo[h][2], 0.0f);
        c.jbox[2 * (2 * cl + h) + 1] = make_float4(hi[h][0], hi[h][1], hi[h][2], 0.0f);
    }
    c.ibox[2 * cl] = make_float4(fminf(lo[0][0], lo[1][0]), fminf(lo[0][1], lo[1][1]),
                                 fminf(lo[0][2], lo[1][2]), 0.0f);
    c.ibox[2 * cl + 1] = make_float4(fmaxf(hi[0][0], hi[1][0]), fmaxf(hi[0][1], hi[1][1]),
                                     fmaxf(hi[0][2], hi[1][2]), 0.0f);
}

// The list build's arithmetic is written in explicitly rounded operations,
// so that no compiler contraction makes its box tests differ from the
// bounds they are derived for (a counting and a writing pass once
// disagreed on entries at the cutoff that way).
// Gap between the intervals [alo, ahi] and [blo, bhi], less the margin m.
__device__ __forceinline__ float gap_less(float alo, float ahi, float blo, float bhi, float m) {
    const float g = fmaxf(0.0f, fmaxf(__fsub_rn(blo, ahi), __fsub_rn(alo, bhi)));
    return fmaxf(0.0f, __fsub_rn(g, m));
}
__device__ __forceinline__ float sq_add(float acc, float g) { return __fadd_rn(acc, __fmul_rn(g, g)); }

// Per-i-cluster constants of the list build (with its simulation's lattice).
struct ListFrame {
    ClGeom g;
    float4 ilo, ihi;
    int4 ri;
    float thr, thr_s, m0, m1, m2;
    int slo, shi;   // slab window (absolute, may leave [0, nslab))
};

// The j-halves of one column (dy, dx) within reach of the i box: the
// clusters holding a particle in the slab window, each tested as a whole and
// then by halves, every z image whose gap is in reach.  Writes the entries in
// enumeration order (clusters in index order, images in ascending offset,
// halves): the k-th within the short support at at_near + k, the k-th beyond
// it at at_far - k, only inside [lo_end, hi_end); nn and nf count them.
template <bool STORE>
__device__ void cl_column(const ClusterSet &c, const ListFrame &f, int dy, int dx,
                          long long at_near, long long at_far, long long lo_end,
                          long long hi_end, int &nn, int &nf) {
    nn = 0;
    nf = 0;
    const ClGeom &g = f.g;
    const float sy = __fmul_rn((float)dy, g.wy), sx = __fmul_rn((float)dx, g.wx);
    const float hwy = __fmul_rn(0.5f, g.wy), hwx = __fmul_rn(0.5f, g.wx);
    const float gy = gap_less(f.ilo.y, f.ihi.y, __fsub_rn(sy, hwy), __fadd_rn(sy, hwy), f.m1);
    const float gx = gap_less(f.ilo.x, f.ihi.x, __fsub_rn(sx, hwx), __fadd_rn(sx, hwx), f.m0);
    if (sq_add(__fmul_rn(gx, gx), gy) >= f.thr) return;
    int ky = (f.ri.y + dy) % g.ncy;
    ky += ky < 0 ? g.ncy : 0;
    int kx = (f.ri.x + dx) % g.ncx;
    kx += kx < 0 ? g.ncx : 0;
    const int lcol = ky * g.ncx + kx;
    const int col = g.col_off + lcol;
    const int cb = c.colcl[col], ce = c.colcl[col + 1];
    if (cb == ce) return;
    const int f0 = g.fine_off + lcol * g.nslab;
    const int pstart = c.fstart[f0];
    // first cluster holding a particle of slab >= s (0 <= s <= nslab);
    // one past the last holding a particle of slab <= s (-1 <= s < nslab)
    auto first_cl = [&](int s) { return cb + ((c.fstart[f0 + s] - pstart) >> 3); };
    auto end_cl = [&](int s) { return cb + ((c.fstart[f0 + s + 1] - pstart + 7) >> 3); };
    int b0 = cb, b1 = cb, a0, a1;
    if (f.shi - f.slo + 1 >= g.nslab) {
        a0 = cb;
        a1 = ce;
    } else if (f.slo < 0) {
        b1 = end_cl(f.shi);
        a0 = max(first_cl(f.slo + g.nslab), b1);
        a1 = ce;
    } else if (f.shi >= g.nslab) {
        a0 = first_cl(f.slo);
        a1 = ce;
        b1 = min(end_cl(f.shi - g.nslab), a0);
    } else {
        a0 = first_cl(f.slo);
        a1 = end_cl(f.shi);
    }
    for (int part = 0; part < 2; ++part) {
        const int r0 = part == 0 ? b0 : a0, r1 = part == 0 ? b1 : a1;
        for (int cj = r0; cj < r1; ++cj) {
            const float4 clo = c.ibox[2 * cj], chi = c.ibox[2 * cj + 1];
            const float cx = gap_less(f.ilo.x, f.ihi.x, __fadd_rn(clo.x, sx), __fadd_rn(chi.x, sx), f.m0);
            const float cy = gap_less(f.ilo.y, f.ihi.y, __fadd_rn(clo.y, sy), __fadd_rn(chi.y, sy), f.m1);
            const float cxy = sq_add(__fmul_rn(cx, cx), cy);
            if (cxy >= f.thr) continue;
            const int dz0 = c.cref[cj].z - f.ri.z;
            for (int img = -1; img <= 1; ++img) {
                const int dz = dz0 + img * g.nslab;
                const float sz = __fmul_rn((float)dz, g.gz);
                const float cz = gap_less(f.ilo.z, f.ihi.z, __fadd_rn(clo.z, sz), __fadd_rn(chi.z, sz), f.m2);
                if (sq_add(cxy, cz) >= f.thr) continue;
                for (int h = 0; h < 2; ++h) {
                    const float4 lo = c.jbox[2 * (2 * cj + h)], hi = c.jbox[2 * (2 * cj + h) + 1];
                    if (lo.x > hi.x) continue;
                    const float hx = gap_less(f.ilo.x, f.ihi.x, __fadd_rn(lo.x, sx), __fadd_rn(hi.x, sx), f.m0);
                    const float hy = gap_less(f.ilo.y, f.ihi.y, __fadd_rn(lo.y, sy), __fadd_rn(hi.y, sy), f.m1);
                    const float hz = gap_less(f.ilo.z, f.ihi.z, __fadd_rn(lo.z, sz), __fadd_rn(hi.z, sz), f.m2);
                    const float g2 = sq_add(sq_add(__fmul_rn(hx, hx), hy), hz);
                    if (g2 >= f.thr) continue;
                    const bool near = g2 < f.thr_s;
                    // near entries from the front, far ones from the back
                    const long long at = near ? at_near + nn : at_far - nf;
                    if (STORE && at >= lo_end && at < hi_end)
                        c.ent[at] = make_int2(
                            (int)((unsigned)(2 * cj + h) | (near ? 0x80000000u : 0u)),
                            (dx & 0xff) | ((dy & 0xff) << 8) | (dz << 16));
                    nn += near ? 1 : 0;
                    nf += near ? 0 : 1;
                }
            }
        }
    }
}

// The list of i-cluster cl (a thread per i-cluster) in one pass, into its
// region of lstride entries: the columns of the (2 ry + 1) x (2 rx + 1)
// window in (dy, dx) raster order, the entries within the short support from
// the front, the others from the back, each in enumeration order (columns in
// raster order, then each column's own order).  A list longer than the
// region raises SPH_ECAPACITY and keeps only what fits.  (A warp per
// i-cluster with a lane per column measured 3x slower: the lanes' columns
// differ widely in work.)  Every thread also records its list length into
// c.maxfill; with STORE false nothing else is written (the engine sizes the
// regions from that measurement).
template <bool STORE>
__device__ int cl_list_one(const View &v, const ClusterSet &c, int cl) {
    const long long base = (long long)cl * c.lstride, top = base + c.lstride;
    const int sim = c.csim[cl];
    ListFrame f;
    f.g = c.geom[sim];
    const SimConst<float> &k = v.sims[sim].cf;
    f.thr = k.thr_hi;
    f.thr_s = k.thr_s;
    const float eps = 1.0e-3f;  // rounding of boxes and shifts, far above it
    f.m0 = f.g.drift2[0] + eps;
    f.m1 = f.g.drift2[1] + eps;
    f.m2 = f.g.drift2[2] + eps;
    f.ilo = c.ibox[2 * cl];
    f.ihi = c.ibox[2 * cl + 1];
    f.ri = c.cref[cl];
    const float reach_z = __fadd_rn(__fsqrt_rn(f.thr), f.m2);
    const float zref = __fmul_rn((float)f.ri.z, f.g.gz);
    const float zlo = __fsub_rn(__fadd_rn(zref, f.ilo.z), reach_z);
    const float zhi = __fadd_rn(__fadd_rn(zref, f.ihi.z), reach_z);
    f.slo = (int)floorf(__fdiv_rn(zlo, f.g.gz)) - 1;
    f.shi = (int)floorf(__fdiv_rn(zhi, f.g.gz)) + 1;
    int tot_near = 0, tot_far = 0;
    for (int dy = -f.g.ry; dy <= f.g.ry; ++dy)
        for (int dx = -f.g.rx; dx <= f.g.rx; ++dx) {
            int nn, nf;
            // the regions stay apart: near entries below top - tot_far, far above
            cl_column<STORE>(c, f, dy, dx, base + tot_near, top - 1 - tot_far, base + tot_near,
                             top - tot_far, nn, nf);
            tot_near += nn;
            tot_far += nf;
        }
    const int total = tot_near + tot_far;
    if (!STORE) return total;
    if (total > c.lstride) {
        set_err(v.err, v.err_any, sim, SPH_ECAPACITY);
        tot_far = 0;
        tot_near = min(tot_near, c.lstride);
    }
    c.lnear[cl] = tot_near;
    c.lfar[cl] = tot_far;
    return total;
}

// A thread per i-cluster; the warp's longest list goes to c.maxfill.
template <bool STORE>
__global__ void __launch_bounds__(128) k_cl_list(const __grid_constant__ View v,
                                                 const __grid_constant__ ClusterSet c) {
    const int cl = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = cl < c.ncl_max && cl < c.colcl[c.ncol];
    int total = 0;
    if (live) total = cl_list_one<STORE>(v, c, cl);
    const int wmax = __reduce_max_sync(0xffffffffu, total);
    if ((threadIdx.x & 31) == 0 && wmax > 0) atomicMax(c.maxfill, wmax);
}

// Prefetching the next entry and its j record, per pass: measured faster
// for the force pass only (3D, N = 2,097,152: force 15.26 -> 14.65 ms per
// step; density 8.29 -> 8.98 and heat 2.47 -> 2.63 with it).
constexpr bool kPfDensity = false, kPfHeat = false, kPfForce = true;

// Pairs of one lane over n entries from p (step +1 or -1): i = slot si (lane
// & 7 of the warp's cluster; gi its particle, -1 for a padding slot, which
// takes no pairs: two padding slots lie at the same far point), j = the
// lane's quarter (lane >> 3) of each listed j-cluster.  body(sj, pj, d, rsq,
// near) for every pair of the exact set (FP32 test, FP64 in the guard band);
// near is NEAR, the segment's kind (the front of a list holds its entries
// within the short support, the back the others); flush() after every 16th
// entry of the list (blocked compensated sums).

// The lattice steps of the warp's simulation and its constants.
struct PairCtx {
    const SimDev *S;
    float wx, wy, gz;
    float thr_lo, thr_hi;
};

template <bool PF, bool NEAR, typename F, typename G>
__device__ __forceinline__ void cl_segment(const View &v, const ClusterSet &c, const PairCtx &x,
                                           int si, int gi, const float4 &pi, const int2 *p, int n,
                                           int step, int &flushes, F body, G flush) {
    const int jj = (threadIdx.x & 31) >> 3;
    int2 en_n = make_int2(0, 0);
    float4 pj_n = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (PF && n > 0) {
        en_n = *p;
        pj_n = c.cpos[(en_n.x & 0x7fffffff) * 4 + jj];
    }
    for (int e = 0; e < n; ++e, p += step) {
        int2 en;
        float4 pj;
        if (PF) {
            en = en_n;
            pj = pj_n;
            if (e + 1 < n) {
                en_n = p[step];
                pj_n = c.cpos[(en_n.x & 0x7fffffff) * 4 + jj];
            }
        } else {
            en = *p;
            pj = c.cpos[(en.x & 0x7fffffff) * 4 + jj];
        }
        const int sj = (en.x & 0x7fffffff) * 4 + jj;
        if (!SPH_IN_BOUNDS(sj < c.slots_max, v.err_any)) continue;
        const float sx = (float)(signed char)(en.y & 0xff) * x.wx;
        const float sy = (float)(signed char)((en.y >> 8) & 0xff) * x.wy;
        const float sz = (float)(en.y >> 16) * x.gz;
        float d[3];
        d[0] = (pj.x + sx) - pi.x;
        d[1] = (pj.y + sy) - pi.y;
        d[2] = (pj.z + sz) - pi.z;
        const float rsq = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        if (gi >= 0 && rsq <= x.thr_hi && sj != si &&
            (rsq < x.thr_lo || exact_in_set<3>(v.xe_in, x.S, gi, c.slot_idx[sj]))) {
            body(sj, pj, d, rsq, std::integral_constant<bool, NEAR>{});
        }
        if ((++flushes & 15) == 0) flush();
    }
}

// The near entries from the front of the i-cluster's region, then (unless
// NEAR_ONLY) the far ones from its back, in list order.
template <bool NEAR_ONLY, bool PF, typename F, typename G>
__device__ __forceinline__ void cl_for_pairs(const View &v, const ClusterSet &c, const PairCtx &x,
                                             int wid, int si, int gi, const float4 &pi, F body,
                                             G flush) {
    const int2 *region = c.ent + (long long)wid * c.lstride;
    int flushes = 0;
    // a list's front holds exactly its entries within the short support
    cl_segment<PF, true>(v, c, x, si, gi, pi, region, c.lnear[wid], 1, flushes, body, flush);
    if (!NEAR_ONLY)
        cl_segment<PF, false>(v, c, x, si, gi, pi, region + c.lstride - 1, c.lfar[wid], -1,
                              flushes, body, flush);
}

// The warp's simulation: kernel parameters for a single simulation (ONE),
// else its table entries.
template <bool ONE>
__device__ __forceinline__ const SimDev &cl_sim(const View &v, int sim) {
    if constexpr (ONE) return v.one;
    else return v.sims[sim];
}
template <bool ONE>
__device__ __forceinline__ const ClGeom &cl_geom(const ClusterSet &c, int sim) {
    if constexpr (ONE) return c.g1;
    else return c.geom[sim];
}
template <bool ONE>
__device__ __forceinline__ int cl_simid(const ClusterSet &c, int wid) {
    if constexpr (ONE) return c.sim1;
    else return c.csim[wid];
}

__device__ __forceinline__ PairCtx pair_ctx(const SimDev &S, const ClGeom &g, float thr_hi) {
    PairCtx x;
    x.S = &S;
    x.wx = g.wx;
    x.wy = g.wy;
    x.gz = g.gz;
    x.thr_lo = S.cf.thr_lo;
    x.thr_hi = thr_hi;
    return x;
}

// Sum over the four lanes that share i (lanes ii, ii + 8, ii + 16, ii + 24),
// in a fixed order; the result is valid on lanes 0..7.
__device__ __forceinline__ double quad_sum(double x) {
    x += __shfl_down_sync(0xffffffffu, x, 16);
    x += __shfl_down_sync(0xffffffffu, x, 8);
    return x;
}

// Whether warp wid has a cluster to work on (uniform per warp).
__device__ __forceinline__ bool cl_live(const ClusterSet &c, int wid) {
    return wid < c.ncl_max && wid < c.colcl[c.ncol];
}

// Density and heat passes at 40 registers (6 blocks of 256 per SM, a few
// words spilled): measured on the 3D 128^3 fluid 6% (density) and 9% (heat)
// faster than the 48 the compiler takes unconstrained.

template <int K, bool ONE>
__global__ void __launch_bounds__(kBlock, 6) k_cl_density(const __grid_constant__ View v,
                                                       const __grid_constant__ ClusterSet c,
                                                       int stage) {
    const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (!cl_live(c, wid)) return;
    const int lane = threadIdx.x & 31, ii = lane & 7, jj = lane >> 3;
    const int si = wid * 8 + ii;
    const float4 pi = c.cpos[si];
    const int gi = c.slot_idx[si];
    const int sim = cl_simid<ONE>(c, wid);
    const SimDev &S = cl_sim<ONE>(v, sim);
    const PairCtx x = pair_ctx(S, cl_geom<ONE>(c, sim), S.cf.thr_hi);
    const KConst<float> ks = make_kconst<float>(S, 0), kl = make_kconst<float>(S, 1);
    BAcc<float> rs, rl;
    rs.init(0.0f);
    rl.init(0.0f);
    unsigned cnt = 0;
    cl_for_pairs<false, kPfDensity>(
        v, c, x, wid, si, gi, pi,
        [&](int, const float4 &pj, const float *, float rsq, auto near) {
            const Dist<float> dd = plain_dist<float>(rsq);
            float w, g;
            if constexpr (decltype(near)::value) {
                kernel_wg<K, float>(ks, dd, &w, &g);
                rs.add(pj.w * w);
            }
            kernel_wg<K, float>(kl, dd, &w, &g);
            rl.add(pj.w * w);
            ++cnt;
        },
        [&]() {
            rs.flush();
            rl.flush();
        });
    const double sum_s = quad_sum(rs.get64()), sum_l = quad_sum(rl.get64());
    // the pair set of one evaluation: counted at the step's first one only
    if (stage == 0) {
        for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
        if (lane == 0) atomicAdd(&v.pair_count[sim], (unsigned long long)cnt);
    }
    if (jj != 0 || gi < 0) return;
    // EOS in FP64, as in the cell-window density pass (k_density)
    const double rho = S.ws0 + S.sig_s * sum_s;
    const double rhol = S.wl0 + S.sig_l * sum_l;
    double T = (v.ue_in[gi] + S.a * rho) * S.inv_kb;
    if (T < 0.0) T = 0.0;
    const double den = rho * (1.0 - S.b * rho);
    const double fs = S.kb * T * recip64<float>(den);
    const double p = fs * rho * rho;
    const double pco = -S.a * rhol * rhol;
    const float Th = (float)T;
    ((float *)v.rho)[gi] = (float)rho;
    ((float *)v.rho_l)[gi] = (float)rhol;
    ((float *)v.temp)[gi] = Th;
    ((float *)v.pres)[gi] = (float)p;
    ((float *)v.pco)[gi] = (float)pco;
    if (stage == 0) {
        ((float *)v.rho0)[gi] = (float)rho;
        ((float *)v.pres0)[gi] = (float)p;
        ((float *)v.pco0)[gi] = (float)pco;
    }
    // the heat pass reads 1/rho (rounded once from FP64, no reciprocal per pair)
    c.cf[si] = make_float4((float)fs, (float)recip64<float>(rho), Th, (float)(T - (double)Th));
    c.crho[si] = (float)rho;
    const float4 vi = ((const float4 *)v.pk_vel_in)[gi];
    c.cfv[si] = make_float4(vi.x, vi.y, vi.z, (float)fs);
    if (!isfinite((float)p) || !isfinite((float)rho) || !isfinite((float)rhol))
        set_err(v.err, v.err_any, sim, SPH_ENAN);
}

template <int K, bool ONE>
__global__ void __launch_bounds__(kBlock, 6) k_cl_heat(const __grid_constant__ View v,
                                                    const __grid_constant__ ClusterSet c) {
    const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (!cl_live(c, wid)) return;
    const int lane = threadIdx.x & 31, ii = lane & 7, jj = lane >> 3;
    const int si = wid * 8 + ii;
    const float4 pi = c.cpos[si];
    const int gi = c.slot_idx[si];
    const int sim = cl_simid<ONE>(c, wid);
    const SimDev &S = cl_sim<ONE>(v, sim);
    const SimConst<float> &k = S.cf;
    // only the short kernel enters q: the pair test stops at its support
    const PairCtx x = pair_ctx(S, cl_geom<ONE>(c, sim), k.thr_s);
    const KConst<float> ks = make_kconst<float>(S, 0);
    const float4 fi = c.cf[si];
    BAcc<float> q[3];
    q[0].init(0.0f);
    q[1].init(0.0f);
    q[2].init(0.0f);
    // only the short kernel enters q: entries beyond its support are skipped
    cl_for_pairs<true, kPfHeat>(
        v, c, x, wid, si, gi, pi,
        [&](int sj, const float4 &pj, const float *d, float rsq, auto) {
            const float g = kernel_g<K, float, true>(ks, make_dist<float>(rsq));
            const float4 fj = c.cf[sj];   // {p/rho^2, 1/rho, T_hi, T_lo}
            const float dT = (fj.z - fi.z) + (fj.w - fi.w);
            const float f = pj.w * fj.y * dT * g;
            q[0].add(f * d[0]);
            q[1].add(f * d[1]);
            q[2].add(f * d[2]);
        },
        [&]() {
            q[0].flush();
            q[1].flush();
            q[2].flush();
        });
    double s[3];
    for (int a = 0; a < 3; ++a) s[a] = quad_sum(q[a].get64());
    if (jj != 0 || gi < 0) return;
    const float ir2 = fi.y * fi.y;   // 1/rho^2
    float qq[3];
    for (int a = 0; a < 3; ++a) {
        qq[a] = k.kappa * (float)s[a];
        ((float *)v.q[a])[gi] = qq[a];
    }
    c.cq[si] = make_float4(qq[0] * ir2, qq[1] * ir2, qq[2] * ir2, 0.0f);
}

// Register caps: 64 for a single simulation (constants in the kernel
// parameters); 85 for several, whose constants come from the table (64
// spilled 168 bytes).
template <int K, int VH, bool ONE>
__global__ void __launch_bounds__(kBlock, ONE ? 4 : 3) k_cl_force(const __grid_constant__ View v,
                                                     const __grid_constant__ ClusterSet c) {
    constexpr bool visc = (VH & 1) != 0;
    constexpr bool heat = (VH & 2) != 0;
    const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (!cl_live(c, wid)) return;
    const int lane = threadIdx.x & 31, ii = lane & 7, jj = lane >> 3;
    const int si = wid * 8 + ii;
    const float4 pi = c.cpos[si];
    const int gi = c.slot_idx[si];
    const int sim = cl_simid<ONE>(c, wid);
    const SimDev &S = cl_sim<ONE>(v, sim);
    const SimConst<float> &sc = S.cf;
    const PairCtx x = pair_ctx(S, cl_geom<ONE>(c, sim), sc.thr_hi);
    // the long kernel with the cohesive factor -2a folded in (see k_force)
    const KConst<float> ks = make_kconst<float>(S, 0), kl = make_kconst_cohesive<float>(S);
    const float hs = sc.hs, eps_h2 = sc.eps_h2, alpha_c = sc.alpha_c, beta = sc.beta;
    const float4 fvi = c.cfv[si];
    const float rhoi = c.crho[si];
    const float4 qi = heat ? c.cq[si] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    BAcc<float> ax[3], ud;
    ax[0].init(0.0f);
    ax[1].init(0.0f);
    ax[2].init(0.0f);
    ud.init(0.0f);
    // the pair terms of k_force (forces.py:338-405, c_forces.pyx:96-111, 163-178, 224-237)
    cl_for_pairs<false, kPfForce>(
        v, c, x, wid, si, gi, pi,
        [&](int sj, const float4 &pj, const float *d, float rsq, auto near) {
            constexpr bool NEAR = decltype(near)::value;
            const Dist<float> dd = make_dist<float>(rsq);
            const float gl = kernel_g<K, float, true>(kl, dd);
            const float4 fvj = c.cfv[sj];
            const float dvdx = (fvj.x - fvi.x) * d[0] + (fvj.y - fvi.y) * d[1] + (fvj.z - fvi.z) * d[2];
            float gsum = gl, gs = 0.0f;
            if constexpr (NEAR) {
                gs = kernel_g<K, float, true>(ks, dd);
                float ps = fvi.w + fvj.w;
                if (visc && dvdx < 0.0f && gs != 0.0f) {   // gs = 0: ps does not enter
                    const float rhoj = c.crho[sj];
                    const float mu = fdiv<float>(hs * dvdx, rsq + eps_h2);
                    ps += fdiv<float>(2.0f * (-alpha_c * mu + beta * mu * mu), rhoi + rhoj);
                }
                gsum = ps * gs + gl;
            }
            ax[0].add(gsum * d[0]);
            ax[1].add(gsum * d[1]);
            ax[2].add(gsum * d[2]);
            float du = gsum * dvdx * pj.w;   // twice the term, halved at the end
            if (heat && NEAR) {
                const float4 qj = c.cq[sj];
                const float dq = (qi.x + qj.x) * d[0] + (qi.y + qj.y) * d[1] + (qi.z + qj.z) * d[2];
                du -= 2.0f * dq * gs * pj.w;
            }
            ud.add(du);
        },
        [&]() {
            ax[0].flush();
            ax[1].flush();
            ax[2].flush();
            ud.flush();
        });
    float vd[3];
    for (int a = 0; a < 3; ++a) vd[a] = (float)quad_sum(ax[a].get64());
    const float u = (float)(0.5 * quad_sum(ud.get64()));
    if (jj != 0 || gi < 0) return;
    for (int a = 0; a < 3; ++a) ((float *)v.vdot[a])[gi] = vd[a];
    ((float *)v.udot)[gi] = u;
    if (!isfinite(vd[0]) || !isfinite(u)) set_err(v.err, v.err_any, sim, SPH_ENAN);
}

int warp_blocks(const ClusterSet &c) { return nblocks((long long)c.ncl_max * 32, kBlock); }

}  // namespace

int cluster_build_kernels() { return 15; }

void launch_cluster_build(const View &v, const ClusterSet &c, cudaStream_t s, bool store) {
    if (v.np <= 0) return;
    cudaMemsetAsync(c.fcount, 0, sizeof(int) * c.nfine, s);
    k_cl_key<<<nblocks(v.np, kBlock), kBlock, 0, s>>>(v, c);
    launch_scan(c.fcount, c.fstart, c.nfine, c.scan_tmp, s);
    k_cl_scatter<<<nblocks(v.np, kBlock), kBlock, 0, s>>>(v, c);
    k_cl_fsort<<<nblocks(c.nfine, kBlock), kBlock, 0, s>>>(c);
    k_cl_cols<<<nblocks(c.ncol, kBlock), kBlock, 0, s>>>(c);
    launch_scan(c.colcnt, c.colcl, c.ncol, c.scan_tmp, s);
    launch_fill_int(c.slot_idx, -1, c.slots_max, s);
    k_cl_slots<<<nblocks(v.np, kBlock), kBlock, 0, s>>>(v, c);
    k_cl_pack<<<nblocks(c.slots_max, kBlock), kBlock, 0, s>>>(v, c, 0);
    k_cl_bbox<<<nblocks(c.ncl_max, kBlock), kBlock, 0, s>>>(c);
    if (store) k_cl_list<true><<<nblocks(c.ncl_max, 128), 128, 0, s>>>(v, c);
    else k_cl_list<false><<<nblocks(c.ncl_max, 128), 128, 0, s>>>(v, c);
}

void launch_cluster_pack(const View &v, const ClusterSet &c, int stage, cudaStream_t s) {
    k_cl_pack<<<nblocks(c.slots_max, kBlock), kBlock, 0, s>>>(v, c, stage);
}

#define SPH_CL_KERNELS(...)                                                                  \
    switch (kernel) {                                                                        \
        case SPH_KERNEL_GAUSSIAN: { constexpr int K = SPH_KERNEL_GAUSSIAN; __VA_ARGS__; break; } \
        case SPH_KERNEL_LUCY: { constexpr int K = SPH_KERNEL_LUCY; __VA_ARGS__; break; }         \
        case SPH_KERNEL_DEBRUN: { constexpr int K = SPH_KERNEL_DEBRUN; __VA_ARGS__; break; }     \
        default: { constexpr int K = SPH_KERNEL_CUBIC; __VA_ARGS__; break; }                     \
    }

void launch_cluster_density(const View &v, const ClusterSet &c, int kernel, int stage,
                            cudaStream_t s) {
    if (v.one_sim) {
        SPH_CL_KERNELS(k_cl_density<K, true><<<warp_blocks(c), kBlock, 0, s>>>(v, c, stage));
    } else {
        SPH_CL_KERNELS(k_cl_density<K, false><<<warp_blocks(c), kBlock, 0, s>>>(v, c, stage));
    }
}

void launch_cluster_heat(const View &v, const ClusterSet &c, int kernel, cudaStream_t s) {
    if (v.one_sim) {
        SPH_CL_KERNELS(k_cl_heat<K, true><<<warp_blocks(c), kBlock, 0, s>>>(v, c));
    } else {
        SPH_CL_KERNELS(k_cl_heat<K, false><<<warp_blocks(c), kBlock, 0, s>>>(v, c));
    }
}

void launch_cluster_force(const View &v, const ClusterSet &c, int kernel, int viscosity, int heat,
                          cudaStream_t s) {
    const int vh = (viscosity ? 1 : 0) | (heat ? 2 : 0);
#define SPH_CL_FORCE(VH_)                                                                \
    do {                                                                                 \
        if (v.one_sim) {                                                                 \
            SPH_CL_KERNELS(k_cl_force<K, VH_, true><<<warp_blocks(c), kBlock, 0, s>>>(v, c));  \
        } else {                                                                         \
            SPH_CL_KERNELS(k_cl_force<K, VH_, false><<<warp_blocks(c), kBlock, 0, s>>>(v, c)); \
        }                                                                                \
    } while (0)
    switch (vh) {
        case 0: SPH_CL_FORCE(0); break;
        case 1: SPH_CL_FORCE(1); break;
        case 2: SPH_CL_FORCE(2); break;
        default: SPH_CL_FORCE(3); break;
    }
#undef SPH_CL_FORCE
}

#undef SPH_CL_KERNELS

}  // namespace sph
