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

// Self-check of the integer numerator of the float64 step
// (numerator_two_int): g[i] = its fma(2, 0.5 - f[i], f[i]) and in_range[i]
// = whether f[i] lay in its range [0, 1] (g[i] is then 0 otherwise).
__global__ void numerator_check_kernel(const double* __restrict__ f, int64_t n,
                                       double* __restrict__ g, int32_t* __restrict__ in_range) {
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n; k += stride) {
        double r = 0.0;
        const bool ok = numerator_two_int(f[k], r);
        in_range[k] = ok ? 1 : 0;
        g[k] = ok ? r : 0.0;
    }
}

cudaError_t launch_numerator_check(const double* f, int64_t n, double* g, int32_t* in_range,
                                   cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    numerator_check_kernel<<<stream_blocks(n), 256, 0, stream>>>(f, n, g, in_range);
    count_launch();
    return cudaGetLastError();
}
}  // namespace rlic
