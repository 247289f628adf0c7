// sph_kfunc.cu -- the smoothing kernels of the pair passes as a callable
// function (sph_kernel_eval): W(r) and g = (dW/dr)/r at given distances, in
// the device arithmetic of the cell-window passes (kernel_wg with the
// constants of kernel_consts), for pyticles' spkernel interface
// (spkernel.py:22-153).  W is the kernel's w(q) times sigma, applied in FP64
// as the density pass applies it to its sums; g carries sigma already.
#include <cmath>

#include "sph_device.cuh"

namespace sph {
namespace {

template <int K, typename R>
__global__ void k_kernel_eval(int64_t n, const double *r, double *w, double *g, KConst<R> k,
                              double sig) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    R wv, gv;
    kernel_wg<K, R>(k, dist_of<R>((R)r[i]), &wv, &gv);
    w[i] = sig * (double)wv;
    g[i] = (double)gv;
}

template <typename R>
void launch_kernel_eval(int kernel, int dim, double h, int64_t n, const double *r, double *w,
                        double *g, cudaStream_t st) {
    const double sig = kernel_sigma(kernel, dim, h);
    KConst<R> k;
    kernel_consts<R>(kernel, h, sig, k.h, k.h_lo, k.inv_h, k.inv_h_lo, k.sig, k.g0,
                     k.g0_h2, k.inv_h2, k.inv_h2_lo);
    const int block = 256;
    const unsigned grid = (unsigned)((n + block - 1) / block);
    switch (kernel) {
        case SPH_KERNEL_GAUSSIAN:
            k_kernel_eval<SPH_KERNEL_GAUSSIAN, R><<<grid, block, 0, st>>>(n, r, w, g, k, sig);
            break;
        case SPH_KERNEL_LUCY:
            k_kernel_eval<SPH_KERNEL_LUCY, R><<<grid, block, 0, st>>>(n, r, w, g, k, sig);
            break;
        case SPH_KERNEL_DEBRUN:
            k_kernel_eval<SPH_KERNEL_DEBRUN, R><<<grid, block, 0, st>>>(n, r, w, g, k, sig);
            break;
        default:
            k_kernel_eval<SPH_KERNEL_CUBIC, R><<<grid, block, 0, st>>>(n, r, w, g, k, sig);
            break;
    }
}

}  // namespace
}  // namespace sph

extern "C" int sph_kernel_eval(int32_t kernel, int32_t dim, double h, int32_t precision,
                               int64_t n, const double *r, double *w, double *g, int32_t mem,
                               void *stream) {
    if (kernel < SPH_KERNEL_GAUSSIAN || kernel > SPH_KERNEL_CUBIC) return SPH_EINVAL;
    if ((dim != 2 && dim != 3) || !(h > 0.0) || !std::isfinite(h)) return SPH_EINVAL;
    if ((precision != SPH_FP64 && precision != SPH_MIXED) || n < 0) return SPH_EINVAL;
    if (mem != SPH_HOST && mem != SPH_DEVICE) return SPH_EINVAL;
    if (n == 0) return SPH_OK;
    if (!r || !w || !g) return SPH_EINVAL;
    if (n > (int64_t)INT32_MAX * 256) return SPH_EINVAL;   // one launch's grid
    cudaStream_t st = (cudaStream_t)stream;
    const double *dr = r;
    double *dw = w, *dg = g, *buf = nullptr;
    if (mem == SPH_HOST) {
        if (cudaMalloc(&buf, sizeof(double) * 3 * (size_t)n) != cudaSuccess) {
            cudaGetLastError();
            return SPH_ENOMEM;
        }
        dw = buf;
        dg = buf + n;
        double *rin = buf + 2 * n;
        if (cudaMemcpyAsync(rin, r, sizeof(double) * n, cudaMemcpyHostToDevice, st) !=
            cudaSuccess) {
            cudaFree(buf);
            return SPH_ECUDA;
        }
        dr = rin;
    }
    if (precision == SPH_MIXED)
        sph::launch_kernel_eval<float>(kernel, dim, h, n, dr, dw, dg, st);
    else
        sph::launch_kernel_eval<double>(kernel, dim, h, n, dr, dw, dg, st);
    int status = cudaGetLastError() == cudaSuccess ? SPH_OK : SPH_ECUDA;
    if (status == SPH_OK && mem == SPH_HOST) {
        if (cudaMemcpyAsync(w, dw, sizeof(double) * n, cudaMemcpyDeviceToHost, st) !=
                cudaSuccess ||
            cudaMemcpyAsync(g, dg, sizeof(double) * n, cudaMemcpyDeviceToHost, st) != cudaSuccess)
            status = SPH_ECUDA;
    }
    if (cudaStreamSynchronize(st) != cudaSuccess) status = SPH_ECUDA;
    if (buf) cudaFree(buf);
    return status;
}
