// float64 instantiation of the convolution kernels (see lic_kernels.cuh).
#include "lic_kernels.cuh"

namespace rlic {
RLIC_DEFINE_LAUNCHERS(double)

// Self-check of the screened float64 division of the streamline step
// (quotient_screened): q[i] = its |a[i] / b[i]|, certified[i] = whether it
// certified the result.
__global__ void quotient_check_kernel(const double* __restrict__ a, const double* __restrict__ b,
                                      int64_t n, double* __restrict__ q,
                                      int32_t* __restrict__ certified) {
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n; k += stride) {
        double r;
        certified[k] = quotient_screened(a[k], b[k], r) ? 1 : 0;
        q[k] = r;
    }
}

cudaError_t launch_quotient_check(const double* a, const double* b, int64_t n, double* q,
                                  int32_t* certified, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    quotient_check_kernel<<<stream_blocks(n), 256, 0, stream>>>(a, b, n, q, certified);
    count_launch();
    return cudaGetLastError();
}
}  // namespace rlic
