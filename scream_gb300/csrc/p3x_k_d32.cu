/* Column kernel instantiation: rate type double, 32 lanes per column. */
#include "p3x_kernels_impl.cuh"

namespace p3x {
template cudaError_t launch_p3_part<double, 32>(const dev::Inst&, const dev::KParams<double>&,
                                                 const LaunchSpec&, int, int, cudaStream_t);
}  // namespace p3x
