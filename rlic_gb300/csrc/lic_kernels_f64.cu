// float64 instantiation of the convolution kernels (see lic_kernels.cuh).
#include "lic_kernels.cuh"

namespace rlic {
RLIC_DEFINE_LAUNCHERS(double)
}  // namespace rlic
