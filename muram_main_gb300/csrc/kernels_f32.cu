// FP32 kernels: state storage and stencil arithmetic in single precision.
#define GPUMHD_LAUNCH_IMPL
#include "gpumhd_launch.cuh"

namespace gpumhd {
template struct Launch<float>;
}  // namespace gpumhd
