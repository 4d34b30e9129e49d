// float32 instantiation of the convolution kernels (see lic_kernels.cuh).
#include "lic_kernels.cuh"

#include <mutex>

namespace rlic {
RLIC_DEFINE_LAUNCHERS(float)

// A device word that stays zero: the "no NaN sample" flag of fields the
// caller vouches for (RLIC_FLAG_FIELD_NAN_FREE).  It lives in this
// translation unit, whose kernels every call loads anyway, so that looking
// its address up never loads the module of the C ABI's unit (which holds the
// no-allocation entry point's static scratch).
__device__ unsigned g_zero_flag = 0u;

const unsigned* zero_flag(cudaError_t* err) {
    static std::mutex mu;
    static const unsigned* addr[64] = {};
    int dev = 0;
    *err = cudaGetDevice(&dev);
    if (*err != cudaSuccess) return nullptr;
    if (dev < 0 || dev >= 64) {
        *err = cudaErrorInvalidDevice;
        return nullptr;
    }
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void* p = nullptr;
        *err = cudaGetSymbolAddress(&p, g_zero_flag);
        if (*err != cudaSuccess) return nullptr;
        addr[dev] = static_cast<const unsigned*>(p);
    }
    return addr[dev];
}
}  // namespace rlic
