// sph_sort.cu -- counting-sort cell binning into Morton-ordered cells, the
// permutation of the state into cell order, and host<->engine layout copies.
//
// Per step: k_bin (cell id + arrival rank, one atomic per particle) ->
// exclusive scan of the cell counts -> k_scatter -> k_cellsort (within each
// cell, order members by original particle index, which makes the layout and
// every sum order a function of the state alone) -> k_permute (gather the FP64 state into
// B and write the packed cell-local FP32/FP64 copies of the first evaluation).
#include "sph_device.cuh"

namespace sph {

// Grids of the binning kernels are capped (grid-stride loops), so that the
// gated launches of a step that keeps its cells cost little.
constexpr int kSortMaxBlocks = 152 * 16;

inline int sort_blocks(long long work, int per_block) {
    long long nb = (work + per_block - 1) / per_block;
    return (int)(nb < 1 ? 1 : (nb > kSortMaxBlocks ? kSortMaxBlocks : nb));
}

__device__ __forceinline__ void bin_one(const View &v, int k) {
    int s = v.a_sim[k];
    int c = -1, rk = 0;
    if (s >= 0) {
        const SimDev &S = v.sims[s];
        if (S.active) {
            int lin = 0, mul = 1;
            for (int a = 0; a < v.dim; ++a) {
                double sh;
                int ci = cell_coord(v.a_pos[a][k], S, a, &sh);
                lin += ci * mul;
                mul *= S.nc[a];
            }
            if (SPH_IN_BOUNDS(lin >= 0 && lin < S.ncells, v.err_any)) {
                c = S.cell_off + v.morton[S.cell_off + lin];
                if (SPH_IN_BOUNDS(c >= S.cell_off && c < S.cell_off + S.ncells, v.err_any))
                    rk = atomicAdd(&v.cell_count[c], 1);
                else
                    c = -1;
            }
        }
    }
    v.cell_of[k] = c;
    v.rank[k] = rk;
}


__global__ void k_bin(View v, int np_a) {
    if (v.rebin_gate && *v.rebin_gate == 0) return;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < np_a; k += gridDim.x * blockDim.x)
        bin_one(v, k);
}

void launch_bin(const View &v, int np_a, cudaStream_t s) {
    if (np_a <= 0) return;
    k_bin<<<sort_blocks(np_a, 256), 256, 0, s>>>(v, np_a);
}

// ---- exclusive scan of int counts: start[i] = sum count[<i], start[n] = total ----
constexpr int kScanBlock = 1024;
constexpr int kScanPer = 4;
constexpr int kScanTile = kScanBlock * kScanPer;

__device__ __forceinline__ int block_excl_scan(int x, int *total) {
    __shared__ int warp_sums[33];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warp_sums[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        int nw = blockDim.x >> 5;
        int ws = lane < nw ? warp_sums[lane] : 0;
        int wi = ws;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += y;
        }
        if (lane < nw) warp_sums[lane] = wi - ws;
        if (lane == nw - 1) warp_sums[32] = wi;
    }
    __syncthreads();
    int res = incl - x + warp_sums[wid];
    *total = warp_sums[32];
    __syncthreads();
    return res;
}

__global__ void k_scan_reduce(const int *count, int n, int *block_tmp, const int *gate) {
    if (gate && *gate == 0) return;
    int base = blockIdx.x * kScanTile;
    int sum = 0;
    for (int t = 0; t < kScanPer; ++t) {
        int i = base + t * kScanBlock + threadIdx.x;
        if (i < n) sum += count[i];
    }
    int total;
    block_excl_scan(sum, &total);
    if (threadIdx.x == 0) block_tmp[blockIdx.x] = total;
}

__global__ void k_scan_top(int *block_tmp, int nb, const int *gate) {
    if (gate && *gate == 0) return;
    // single block, sequential chunks of 1024
    int carry = 0;
    for (int base = 0; base < nb; base += kScanBlock) {
        int i = base + threadIdx.x;
        int x = i < nb ? block_tmp[i] : 0;
        int total;
        int e = block_excl_scan(x, &total);
        if (i < nb) block_tmp[i] = e + carry;
        carry += total;
    }
    if (threadIdx.x == 0) block_tmp[nb] = carry;
}

__global__ void k_scan_apply(const int *count, int *start, int n, const int *block_tmp, int nb,
                             const int *gate) {
    if (gate && *gate == 0) return;
    int base = blockIdx.x * kScanTile;
    // each thread owns kScanPer consecutive elements
    int i0 = base + threadIdx.x * kScanPer;
    int loc[kScanPer];
    int sum = 0;
#pragma unroll
    for (int t = 0; t < kScanPer; ++t) {
        loc[t] = (i0 + t < n) ? count[i0 + t] : 0;
        sum += loc[t];
    }
    int total;
    int e = block_excl_scan(sum, &total) + block_tmp[blockIdx.x];
#pragma unroll
    for (int t = 0; t < kScanPer; ++t) {
        if (i0 + t < n) start[i0 + t] = e;
        e += loc[t];
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) start[n] = block_tmp[nb];
}

void launch_scan(int *count, int *start, int n, int *block_tmp, cudaStream_t s,
                 const int *gate) {
    int nb = (n + kScanTile - 1) / kScanTile;
    if (nb < 1) nb = 1;
    k_scan_reduce<<<nb, kScanBlock, 0, s>>>(count, n, block_tmp, gate);
    k_scan_top<<<1, kScanBlock, 0, s>>>(block_tmp, nb, gate);
    k_scan_apply<<<nb, kScanBlock, 0, s>>>(count, start, n, block_tmp, nb, gate);
}

__global__ void k_scatter(View v, int np_a) {
    if (v.rebin_gate && *v.rebin_gate == 0) return;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < np_a; k += gridDim.x * blockDim.x) {
        int c = v.cell_of[k];
        if (c >= 0) {
            const int dst = v.cell_start[c] + v.rank[k];
            if (SPH_IN_BOUNDS(dst >= 0 && dst < v.np, v.err_any)) v.order_tmp[dst] = k;
        }
    }
}

void launch_scatter(const View &v, int np_a, cudaStream_t s) {
    if (np_a <= 0) return;
    k_scatter<<<sort_blocks(np_a, 256), 256, 0, s>>>(v, np_a);
}

// One warp per cell: the rank of each member is the number of members with a
// smaller original particle index (unique within a cell: a cell belongs to
// one simulation).  The order inside a cell is therefore canonical -- it
// depends neither on the order in which the atomics of k_bin arrived nor on
// the layout the state had before -- so every pass sums its pairs in an order
// that is a function of the positions alone.
__global__ void k_cellsort(View v, int ncells) {
    if (v.rebin_gate && *v.rebin_gate == 0) return;
    const int lane = threadIdx.x & 31;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int cell = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; cell < ncells;
         cell += nwarps) {
        int b = v.cell_start[cell], e = v.cell_start[cell + 1];
        int m = e - b;
        for (int x = lane; x < m; x += 32) {
            int val = v.order_tmp[b + x];
            int key = v.a_id[val];
            int r = 0;
            for (int t = 0; t < m; ++t) r += (v.a_id[v.order_tmp[b + t]] < key) ? 1 : 0;
            v.order[b + r] = val;
            v.cell_b[b + r] = cell;
        }
    }
}

void launch_cellsort(const View &v, int ncells, cudaStream_t s) {
    if (ncells <= 0) return;
    k_cellsort<<<sort_blocks((long long)ncells * 32, 256), 256, 0, s>>>(v, ncells);
}

// Gather the state into B (cell order) and pack the first evaluation's
// cell-local coordinates: xl = wrap(x) - centre of the particle's cell.
template <typename R>
__device__ __forceinline__ void permute_one(const View &v, int j) {
    int k = v.order[j];
    int s = v.a_sim[k];
    const SimDev &S = v.sims[s];
    R xl[3] = {0, 0, 0}, vv[3] = {0, 0, 0};
    for (int a = 0; a < v.dim; ++a) {
        double x = v.a_pos[a][k];
        double vel = v.a_vel[a][k];
        v.b_pos[a][j] = x;
        v.b_vel[a][j] = vel;
        double sh;
        int ci = cell_coord(x, S, a, &sh);
        double org = sh + cell_centre(ci, S, a);
        v.org[a][j] = org;
        xl[a] = (R)(x - org);
        vv[a] = (R)vel;
    }
    double m = v.a_m[k];
    v.b_u[j] = v.a_u[k];
    v.b_m[j] = m;
    v.b_id[j] = v.a_id[k];
    v.b_sim[j] = s;
    using T4 = typename V4<R>::T;
    ((T4 *)v.pk_pos_out)[j] = make_v4<R>(xl[0], xl[1], xl[2], (R)m);
    ((T4 *)v.pk_vel_out)[j] = make_v4<R>(vv[0], vv[1], vv[2], (R)0);
}

template <typename R>
__global__ void k_permute(View v) {
    if (v.rebin_gate && *v.rebin_gate == 0) return;
    const int first = blockIdx.x * blockDim.x + threadIdx.x;
    if (first == 0 && !v.rebin_gate && v.bin_count) ++*v.bin_count;
    for (int j = first; j < v.np; j += gridDim.x * blockDim.x) permute_one<R>(v, j);
}

// A state set from the host (A in identity order from a_off) into the B
// slots [b0, b0 + n) of the current binning, keeping the cells, the order
// and the pair lists: B and the stage-0 packed copies relative to the cells'
// frames.  *far is raised if some particle lies past half of its cell slack
// or, with pair lists, a quarter of the skin from its position at their
// build -- the caller then bins again.  The check is write_final_state's.
template <typename R>
__global__ void k_restage(View v, int a_off, int b0, int n, int *far) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int j = b0 + k;
    const int a = a_off + v.b_id[j];
    const SimDev &S = v.one_sim ? v.one : v.sims[v.b_sim[j]];
    R xl[3] = {0, 0, 0}, vv[3] = {0, 0, 0};
    bool out = false;
    double moved = 0.0;
    for (int d = 0; d < v.dim; ++d) {
        const double x = v.a_pos[d][a], vel = v.a_vel[d][a];
        v.b_pos[d][j] = x;
        v.b_vel[d][j] = vel;
        double r = x - v.org[d][j];
        if (r > S.half_L[d]) r -= S.L[d];
        if (r < -S.half_L[d]) r += S.L[d];
        if (v.vl_on) {
            const float4 x0 = v.vl_x0[j];
            const double m = r - (double)(d == 0 ? x0.x : (d == 1 ? x0.y : x0.z));
            moved += m * m;
        } else {
            out |= fabs(r) > S.rebin_half[d];
        }
        xl[d] = (R)r;
        vv[d] = (R)vel;
    }
    out |= moved > S.vl_gate2;
    const double m = v.a_m[a];
    v.b_u[j] = v.a_u[a];
    v.b_m[j] = m;
    using T4 = typename V4<R>::T;
    ((T4 *)v.pk_pos_out)[j] = make_v4<R>(xl[0], xl[1], xl[2], (R)m);
    ((T4 *)v.pk_vel_out)[j] = make_v4<R>(vv[0], vv[1], vv[2], (R)0);
    if (out) *far = 1;
}

void launch_restage(const View &v, int precision, int a_off, int b0, int n, int *far,
                    cudaStream_t s) {
    if (n <= 0) return;
    if (precision == SPH_MIXED)
        k_restage<float><<<(n + 255) / 256, 256, 0, s>>>(v, a_off, b0, n, far);
    else
        k_restage<double><<<(n + 255) / 256, 256, 0, s>>>(v, a_off, b0, n, far);
}

void launch_permute(const View &v, int precision, cudaStream_t s) {
    if (v.np <= 0) return;
    int nb = sort_blocks(v.np, 256);
    if (precision == SPH_MIXED) k_permute<float><<<nb, 256, 0, s>>>(v);
    else k_permute<double><<<nb, 256, 0, s>>>(v);
}

// ---- layout copies ----
__global__ void k_load_aos(double *d0, double *d1, double *d2, const double *src, int n, int dim) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    d0[i] = src[(size_t)i * dim + 0];
    d1[i] = src[(size_t)i * dim + 1];
    if (dim == 3) d2[i] = src[(size_t)i * dim + 2];
}

void launch_load_aos(double *dst[3], const double *src, int n, int dim, cudaStream_t s) {
    if (n <= 0) return;
    k_load_aos<<<(n + 255) / 256, 256, 0, s>>>(dst[0], dst[1], dst[2], src, n, dim);
}

__global__ void k_store_aos(double *dst, const double *s0, const double *s1, const double *s2,
                            const int *id, int off, int n, int dim) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int i = id[off + k];
    dst[(size_t)i * dim + 0] = s0[off + k];
    dst[(size_t)i * dim + 1] = s1[off + k];
    if (dim == 3) dst[(size_t)i * dim + 2] = s2[off + k];
}

void launch_store_aos(double *dst, double *const src[3], const int *id, int off, int n, int dim,
                      cudaStream_t s) {
    if (n <= 0) return;
    k_store_aos<<<(n + 255) / 256, 256, 0, s>>>(dst, src[0], src[1], src[2], id, off, n, dim);
}

__global__ void k_store_scalar(double *dst, const double *src, const int *id, int off, int n) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    dst[id[off + k]] = src[off + k];
}

void launch_store_scalar(double *dst, const double *src, const int *id, int off, int n,
                         cudaStream_t s) {
    if (n <= 0) return;
    k_store_scalar<<<(n + 255) / 256, 256, 0, s>>>(dst, src, id, off, n);
}

template <typename R>
__global__ void k_store_R(double *dst, const R *src, const int *id, int off, int n) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    dst[id[off + k]] = (double)src[off + k];
}

void launch_store_R(double *dst, const void *src, int precision, const int *id, int off, int n,
                    cudaStream_t s) {
    if (n <= 0) return;
    int nb = (n + 255) / 256;
    if (precision == SPH_MIXED) k_store_R<float><<<nb, 256, 0, s>>>(dst, (const float *)src, id, off, n);
    else k_store_R<double><<<nb, 256, 0, s>>>(dst, (const double *)src, id, off, n);
}

__global__ void k_fill_int(int *dst, int val, int n, const int *gate) {
    if (gate && *gate == 0) return;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
        dst[k] = val;
}

void launch_fill_int(int *dst, int val, int n, cudaStream_t s, const int *gate) {
    if (n <= 0) return;
    k_fill_int<<<sort_blocks(n, 256), 256, 0, s>>>(dst, val, n, gate);
}

__global__ void k_rebin_close(int *gate, unsigned long long *bin_count) {
    if (*gate) {
        *gate = 0;
        ++*bin_count;
    }
}

void launch_rebin_close(int *gate, unsigned long long *bin_count, cudaStream_t s) {
    k_rebin_close<<<1, 1, 0, s>>>(gate, bin_count);
}

__global__ void k_iota_sim(int *id, int *sim, int sim_id, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        id[i] = i;
        sim[i] = sim_id;
    }
}

void launch_iota_sim(int *id, int *sim, int sim_id, int n, cudaStream_t s) {
    if (n <= 0) return;
    k_iota_sim<<<(n + 255) / 256, 256, 0, s>>>(id, sim, sim_id, n);
}

}  // namespace sph
