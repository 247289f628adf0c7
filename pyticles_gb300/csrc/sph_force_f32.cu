// sph_force_f32.cu -- the mixed-precision (FP32 pair arithmetic) force pass and
// integrator stage, and the precision dispatch of both.
#include "sph_force.cuh"

namespace sph {

extern template void launch_force_t<double>(const View &, int, int, int, int, int, int, int,
                                            cudaStream_t);
extern template void launch_integrate_t<double>(const View &, int, int, cudaStream_t, int);
template void launch_force_t<float>(const View &, int, int, int, int, int, int, int,
                                    cudaStream_t);
template void launch_integrate_t<float>(const View &, int, int, cudaStream_t, int);

void launch_force(const View &v, int precision, int kernel, int viscosity, int heat,
                  int integrator, int stage, int mode, int block, cudaStream_t s) {
    if (precision == SPH_MIXED)
        launch_force_t<float>(v, kernel, viscosity, heat, integrator, stage, mode, block, s);
    else
        launch_force_t<double>(v, kernel, viscosity, heat, integrator, stage, mode, block, s);
}

void launch_integrate(const View &v, int precision, int integrator, int stage, cudaStream_t s,
                      int cl_only) {
    if (precision == SPH_MIXED) launch_integrate_t<float>(v, integrator, stage, s, cl_only);
    else launch_integrate_t<double>(v, integrator, stage, s, cl_only);
}

}  // namespace sph
