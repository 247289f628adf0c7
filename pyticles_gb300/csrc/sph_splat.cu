// sph_splat.cu -- headless SPH splash rendering of particles onto a pixel
// grid (interpolate.splash_map_2d / splash_map_3d, interpolate.py:39-149),
// replacing the GL path of SmoothParticleView.render_density
// (pview.py:483-519) with a device buffer.
//
// Each particle adds a_i m_i / rho_i W(|r_i - g|, h_i) to every pixel g of
// its pixel box [floor((r - cutoff - min)/res), floor((r + cutoff - min)/res))
// -- upper end excluded, as range() does in the reference -- whose
// minimum-imaged distance is below the cutoff.  Pixel indices wrap
// periodically; the minimum image acts on x and y with the box maxima
// (neighbours.minimum_image(dr, xmax, ymax)).  W is the 2D Lucy kernel
// (spkernel.lucy_w, spkernel.py:54-63) or, for the 3D map of particles onto
// the plane z, the 3D Lucy kernel.  FP64 throughout; contributions are added
// with atomics, so the last bits of a pixel may depend on arrival order.
#include <cmath>

#include "sph_internal.h"

namespace {

__device__ __forceinline__ double lucy_w(double s, double h, int dim3) {
    const double pi = 3.14159265358979323846;
    double q = dim3 ? 105.0 / (pi * 16.0 * (h * h * h)) : 5.0 / (pi * h * h);
    if (s < 0) s = -s;
    if (s < h) {
        double t = 1.0 - s / h;
        return q * (1.0 + 3.0 * s / h) * (t * t * t);
    }
    return 0.0;
}

__device__ __forceinline__ double min_image(double d, double L) {
    if (d > L / 2.) d = d - L;
    if (d < -L / 2.) d = d + L;
    return d;
}

// one thread per particle; r is n x cols row-major
__global__ void k_splat(int n, const double *r, int cols, const double *m, const double *rho,
                        const double *a, const double *h, int nx, int ny, const double *x,
                        const double *y, double z, double xmin, double xmax, double ymin,
                        double ymax, double cutoff, int dim3, double *Z) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double rx = r[(size_t)i * cols], ry = r[(size_t)i * cols + 1];
    const double rz = dim3 ? r[(size_t)i * cols + 2] : 0.0;
    if (dim3 && (rz - z) > cutoff) return;
    const double res = x[1] - x[0];
    const int xa = (int)floor((rx - cutoff - xmin) / res);
    const int ya = (int)floor((ry - cutoff - ymin) / res);
    const int xb = (int)floor((rx + cutoff - xmin) / res);
    const int yb = (int)floor((ry + cutoff - ymin) / res);
    const double wgt = a[i] * m[i] / rho[i];
    const double hi = h[i], c2 = cutoff * cutoff;
    for (int ypx = ya; ypx < yb; ++ypx) {
        int yy = ypx;
        if (yy >= ny) yy -= ny;
        if (yy < 0) yy += ny;
        if (yy < 0 || yy >= ny) continue;  // boxes wider than the grid
        for (int xpx = xa; xpx < xb; ++xpx) {
            int xx = xpx;
            if (xx >= nx) xx -= nx;
            if (xx < 0) xx += nx;
            if (xx < 0 || xx >= nx) continue;
            double dx, dy, dz = 0.0;
            if (dim3) {
                dx = rx - x[xx];
                dy = ry - y[yy];
                dz = rz - z;
            } else {
                dx = rx - x[xx];
                dy = y[yy] - ry;
            }
            dx = min_image(dx, xmax);
            dy = min_image(dy, ymax);
            double rsq = dx * dx + dy * dy + dz * dz;
            if (rsq < c2) atomicAdd(&Z[(size_t)xx * ny + yy], wgt * lucy_w(sqrt(rsq), hi, dim3));
        }
    }
}

}  // namespace

extern "C" int sph_splash_map(int32_t mode, int64_t n, const double *r, int32_t r_cols,
                              const double *m, const double *rho, const double *a,
                              const double *h, int32_t nx, int32_t ny, const double *x,
                              const double *y, double z, const double *bounds, double cutoff,
                              double *Z, int32_t mem, void *stream) {
    if ((mode != 2 && mode != 3) || n < 0 || nx < 2 || ny < 1 || !bounds || !Z || !x || !y)
        return SPH_EINVAL;
    if (r_cols < (mode == 3 ? 3 : 2)) return SPH_EINVAL;
    if (!(cutoff > 0)) return SPH_EINVAL;
    cudaStream_t st = (cudaStream_t)stream;
    size_t npix = (size_t)nx * ny;
    // device copies of host inputs (this entry point is not on the step path)
    const double *dr = r, *dm = m, *drho = rho, *da = a, *dh = h, *dx = x, *dy = y;
    double *dZ = Z;
    double *buf = nullptr;
    if (mem == SPH_HOST) {
        size_t need = (size_t)n * (r_cols + 4) + nx + ny + npix;
        if (cudaMalloc(&buf, sizeof(double) * (need ? need : 1)) != cudaSuccess) {
            cudaGetLastError();
            return SPH_ENOMEM;
        }
        double *p = buf;
        auto up = [&](const double *src, size_t cnt) {
            cudaMemcpyAsync(p, src, sizeof(double) * cnt, cudaMemcpyHostToDevice, st);
            double *q = p;
            p += cnt;
            return (const double *)q;
        };
        dr = up(r, (size_t)n * r_cols);
        dm = up(m, n);
        drho = up(rho, n);
        da = up(a ? a : rho, n);
        dh = up(h, n);
        dx = up(x, nx);
        dy = up(y, ny);
        dZ = p;
    } else if (!a) {
        da = rho;
    }
    cudaMemsetAsync(dZ, 0, sizeof(double) * npix, st);
    if (n > 0)
        k_splat<<<(int)((n + 127) / 128), 128, 0, st>>>(
            (int)n, dr, r_cols, dm, drho, da, dh, nx, ny, dx, dy, z, bounds[0], bounds[1],
            bounds[2], bounds[3], cutoff, mode == 3 ? 1 : 0, dZ);
    int status = SPH_OK;
    if (mem == SPH_HOST) {
        if (cudaMemcpyAsync(Z, dZ, sizeof(double) * npix, cudaMemcpyDeviceToHost, st) !=
            cudaSuccess)
            status = SPH_ECUDA;
    }
    if (cudaStreamSynchronize(st) != cudaSuccess || cudaGetLastError() != cudaSuccess)
        status = SPH_ECUDA;
    if (buf) cudaFree(buf);
    return status;
}
