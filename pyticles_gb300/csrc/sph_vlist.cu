// sph_vlist.cu -- per-particle pair lists of the 2D mixed-precision engine
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

// One thread per particle, 2D, FP32 cell-local positions (pk_pos_in holds the
// stage-0 packed state); mode as launch_vlist_build.
__global__ void __launch_bounds__(256) k_vlist_build(const __grid_constant__ View v, VList l,
                                                     const int *gate, int mode) {
    const bool store = mode != kVlCount;
    if (gate && *gate == 0) return;
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
        if (store) l.x0[i] = make_float2(pi.x, pi.y);
        const int cp = v.cell_xyz[v.cell_b[i]];
        const int c0 = cp & 2047, c1 = (cp >> 11) & 2047;
        const int w0 = S.win[0], w1 = S.win[1];
        const int n0 = S.nc[0], n1 = S.nc[1];
        const int *mort = v.morton + S.cell_off;
        const float thr = c.vl_thr, thr_n = c.vl_near;
        // entry k of the near run sits in group row k/4, slot k%4; far
        // entry k in group row cap/4 - 1 - k/4, slot 3 - k%4
        int *near_row = l.ent + 4 * (long long)i;
        int *far_row = l.ent + 4 * ((long long)((l.cap >> 2) - 1) * l.stride + i) + 3;
        for (int oy = -w1; oy <= w1; ++oy) {
            const float dy = fmaxf_((float)oy * c.edge[1] - pi.y, c.ext[1]);
            if (dy * dy > thr) continue;
            int y = c1 + oy;
            y += (y < 0) ? n1 : 0;
            y -= (y >= n1) ? n1 : 0;
            const int row = y * n0;
            const float oy_ = __fmaf_rn((float)oy, c.edge_lo[1], (float)oy * c.edge[1] - pi.y);
            for (int ox = -w0; ox <= w0; ++ox) {
                const float dx = fmaxf_((float)ox * c.edge[0] - pi.x, c.ext[0]);
                if (dx * dx + dy * dy > thr) continue;
                int x = c0 + ox;
                x += (x < 0) ? n0 : 0;
                x -= (x >= n0) ? n0 : 0;
                if (!SPH_IN_BOUNDS(row + x >= 0 && row + x < S.ncells, v.err_any)) continue;
                const int gc = S.cell_off + mort[row + x];
                const float ox_ =
                    __fmaf_rn((float)ox, c.edge_lo[0], (float)ox * c.edge[0] - pi.x);
                const int jb = v.cell_start[gc], je = v.cell_start[gc + 1];
                if (!SPH_IN_BOUNDS(jb >= 0 && jb <= je && je <= v.np, v.err_any)) continue;
                const int tag = ((ox + 3) << 26) | (int)((unsigned)(oy + 3) << 29);
                for (int j = jb; j < je; ++j) {
                    if (j == i) continue;
                    const float4 pj = P[j];
                    const float ddx = pj.x + ox_, ddy = pj.y + oy_;
                    const float rsq = ddx * ddx + ddy * ddy;
                    if (rsq > thr) continue;
                    const bool room = wn + wf < l.cap;
                    if (rsq < thr_n) {
                        if (room) {
                            if (store) near_row[4 * (long long)(wn >> 2) * l.stride + (wn & 3)] = j | tag;
                            ++wn;
                        }
                        ++nn;
                    } else {
                        if (room) {
                            if (store) far_row[-4 * (long long)(wf >> 2) * l.stride - (wf & 3)] = j | tag;
                            ++wf;
                        }
                        ++nf;
                    }
                }
            }
        }
        if (store) {
            // an overflowing list keeps the entries that fit (the first cap
            // of the scan) and its simulation reports the overflow
            if (mode == kVlStore && nn + nf > l.cap) set_err(v.err, v.err_any, s, SPH_ECAPACITY);
            l.cnt[i] = (unsigned)wn | ((unsigned)wf << 16);
        }
    }
    // the longest list of the warp, one atomic per warp
    const int tot = __reduce_max_sync(0xffffffffu, active ? nn + nf : 0);
    if ((threadIdx.x & 31) == 0 && tot > 0) atomicMax(l.maxfill, tot);
}

void launch_vlist_build(const View &v, const VList &l, const int *gate, int mode,
                        cudaStream_t s) {
    if (v.np <= 0 || !l.on) return;
    k_vlist_build<<<(v.np + 255) / 256, 256, 0, s>>>(v, l, gate, mode);
}

}  // namespace sph
