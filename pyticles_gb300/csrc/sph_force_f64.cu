// sph_force_f64.cu -- the FP64 force pass and integrator stage.
#include "sph_force.cuh"

namespace sph {

template void launch_force_t<double>(const View &, int, int, int, int, int, int, int,
                                     cudaStream_t);
template void launch_integrate_t<double>(const View &, int, int, cudaStream_t, int);

}  // namespace sph
