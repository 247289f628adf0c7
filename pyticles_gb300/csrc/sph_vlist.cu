// sph_vlist.cu -- per-particle pair lists of the mixed-precision engine
// (tuning.pair_scheme 2): VerletList.build with a skin (neighbour_list.py:
// 160-189), kept across steps until a particle has moved a quarter of the
// skin from where it was at the build (VerletList.ponder_rebuild,
// neighbour_list.py:191-234, with the displacement bound a skin list needs).
//
// The build runs right after a binning, on the binned stage-0 state: each
// particle scans its cell window once and files every neighbour within the
// cutoff plus the skin, near ones (within the short support plus the skin)
// from the front of its column of the ELL table, far ones from the back.
// Lists name neighbours by their B-order slot, so they are rebuilt whenever
// the engine bins.  The pair passes then walk the lists (for_list) and apply
// the exact pair test at every evaluation: the pair set stays the
// reference's while every particle remains within half the skin of its
// build position (checked in the force pass, SPH_ESKIN beyond).
#include "sph_pairs.cuh"

namespace sph {

// One thread per particle, FP32 cell-local positions (pk_pos_in holds the
// stage-0 packed state); mode as launch_vlist_build.
template <int D>
__global__ void __launch_bounds__(256) k_vlist_build(const __grid_constant__ View v, VList l,
                                                     const int *gate, int mode) {
    if (gate && *gate == 0) return;
    const bool store = mode != kVlCount;
    constexpr int kBits = vl_index_bits(D);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = i < v.np;
    const int ii = active ? i : v.np - 1;
    const int s = v.b_sim[ii];
    const SimDev &S = v.one_sim ? v.one : v.sims[s];
    const SimConst<float> &c = S.cf;
    const float4 *__restrict__ P = (const float4 *)v.pk_pos_in;
    const float4 pi = P[ii];
    int nn = 0, nf = 0;   // entries found
    int wn = 0, wf = 0;   // entries within the rows
    if (active) {
        if (store) l.x0[i] = pi;
        const int cp = v.cell_xyz[v.cell_b[i]];
        const int c0 = cp & 2047, c1 = (cp >> 11) & 2047, c2 = (cp >> 22) & 1023;
        const int w0 = S.win[0], w1 = S.win[1], w2 = D == 3 ? S.win[2] : 0;
        const int n0 = S.nc[0], n1 = S.nc[1], n2 = S.nc[2];
        const int *mort = v.morton + S.cell_off;
        const float thr = c.vl_thr, thr_n = c.vl_near;
        // entry k of the near run sits in group row k/4, slot k%4; far
        // entry k in group row cap/4 - 1 - k/4, slot 3 - k%4.  Each run
        // collects a group in registers and stores it whole (16 bytes).
        int4 *rows = (int4 *)l.ent + i;
        const long long far0 = (long long)((l.cap >> 2) - 1) * l.stride;
        int4 gn = make_int4(0, 0, 0, 0), gf = make_int4(0, 0, 0, 0);
        for (int oz = -w2; oz <= w2; ++oz) {
            float dz = 0.f, oz_ = 0.f;
            int z = 0;
            if (D == 3) {
                dz = fmaxf_((float)oz * c.edge[2] - pi.z, c.ext[2]);
                if (dz * dz > thr) continue;
                z = c2 + oz;
                z += (z < 0) ? n2 : 0;
                z -= (z >= n2) ? n2 : 0;
                oz_ = __fmaf_rn((float)oz, c.edge_lo[2], (float)oz * c.edge[2] - pi.z);
            }
            for (int oy = -w1; oy <= w1; ++oy) {
                const float dy = fmaxf_((float)oy * c.edge[1] - pi.y, c.ext[1]);
                const float dyz = dy * dy + dz * dz;
                if (dyz > thr) continue;
                int y = c1 + oy;
                y += (y < 0) ? n1 : 0;
                y -= (y >= n1) ? n1 : 0;
                const int row = (z * n1 + y) * n0;
                const float oy_ =
                    __fmaf_rn((float)oy, c.edge_lo[1], (float)oy * c.edge[1] - pi.y);
                for (int ox = -w0; ox <= w0; ++ox) {
                    const float dx = fmaxf_((float)ox * c.edge[0] - pi.x, c.ext[0]);
                    if (dx * dx + dyz > thr) continue;
                    int x = c0 + ox;
                    x += (x < 0) ? n0 : 0;
                    x -= (x >= n0) ? n0 : 0;
                    if (!SPH_IN_BOUNDS(row + x >= 0 && row + x < S.ncells, v.err_any)) continue;
                    const int gc = S.cell_off + mort[row + x];
                    const float ox_ =
                        __fmaf_rn((float)ox, c.edge_lo[0], (float)ox * c.edge[0] - pi.x);
                    const int jb = v.cell_start[gc], je = v.cell_start[gc + 1];
                    if (!SPH_IN_BOUNDS(jb >= 0 && jb <= je && je <= v.np, v.err_any)) continue;
                    unsigned t = (unsigned)(ox + 3) | ((unsigned)(oy + 3) << 3);
                    if (D == 3) t |= (unsigned)(oz + 3) << 6;
                    const int tag = (int)(t << kBits);
                    for (int j = jb; j < je; ++j) {
                        if (j == i) continue;
                        const float4 pj = P[j];
                        const float ddx = pj.x + ox_, ddy = pj.y + oy_;
                        float rsq = ddx * ddx + ddy * ddy;
                        if (D == 3) {
                            const float ddz = pj.z + oz_;
                            rsq += ddz * ddz;
                        }
                        if (rsq > thr) continue;
                        const bool near = rsq < thr_n;
                        nn += near ? 1 : 0;
                        nf += near ? 0 : 1;
                        if (!store) continue;
                        // groups fill as shift registers: near entries enter
                        // at w (the oldest ends in x), far ones at x (the
                        // oldest ends in w); whole groups only, so the near
                        // and far runs never share one
                        const int code = j | tag;
                        const int rows_cap = l.cap >> 2;
                        if (near) {
                            if (((wn + 4) >> 2) + ((wf + 3) >> 2) <= rows_cap) {
                                gn = make_int4(gn.y, gn.z, gn.w, code);
                                if ((++wn & 3) == 0)
                                    rows[(long long)((wn >> 2) - 1) * l.stride] = gn;
                            }
                        } else {
                            if (((wn + 3) >> 2) + ((wf + 4) >> 2) <= rows_cap) {
                                gf = make_int4(code, gf.x, gf.y, gf.z);
                                if ((++wf & 3) == 0)
                                    rows[far0 - (long long)((wf >> 2) - 1) * l.stride] = gf;
                            }
                        }
                    }
                }
            }
        }
        if (store) {
            // the partial last groups, shifted into place (their unused
            // slots are never read)
            if (wn & 3) {
                for (int t = wn & 3; t < 4; ++t) gn = make_int4(gn.y, gn.z, gn.w, 0);
                rows[(long long)(wn >> 2) * l.stride] = gn;
            }
            if (wf & 3) {
                for (int t = wf & 3; t < 4; ++t) gf = make_int4(0, gf.x, gf.y, gf.z);
                rows[far0 - (long long)(wf >> 2) * l.stride] = gf;
            }
            // an overflowing list keeps the entries that fit (the first cap
            // of the scan) and its simulation reports the overflow
            if (mode == kVlStore && (wn < nn || wf < nf))
                set_err(v.err, v.err_any, s, SPH_ECAPACITY);
            l.cnt[i] = (unsigned)wn | ((unsigned)wf << 16);
        }
    }
    // the longest list of the warp in whole groups, one atomic per warp
    const int need = 4 * (((nn + 3) >> 2) + ((nf + 3) >> 2));
    const int tot = __reduce_max_sync(0xffffffffu, active ? need : 0);
    if ((threadIdx.x & 31) == 0 && tot > 0) atomicMax(l.maxfill, tot);
}

void launch_vlist_build(const View &v, const VList &l, const int *gate, int mode,
                        cudaStream_t s) {
    if (v.np <= 0 || !l.on) return;
    if (v.dim == 2)
        k_vlist_build<2><<<(v.np + 255) / 256, 256, 0, s>>>(v, l, gate, mode);
    else
        k_vlist_build<3><<<(v.np + 255) / 256, 256, 0, s>>>(v, l, gate, mode);
}

}  // namespace sph
