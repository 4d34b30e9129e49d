// lic_lowp.cuh -- device helpers of the reduced-precision replay (FP16 or
// BF16 storage, FP32 compensated accumulation), shared by lic_lowp.cu and
// the TMA-staged replay (lic_stage.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "lic_device.cuh"

namespace rlic {

template <typename S> struct StorageTraits;
template <> struct StorageTraits<__half> {
    __device__ static float load(const __half* p) { return __half2float(__ldg(p)); }
    __device__ static __half from_float(float x) { return __float2half_rn(x); }
};
template <> struct StorageTraits<__nv_bfloat16> {
    __device__ static float load(const __nv_bfloat16* p) { return __bfloat162float(__ldg(p)); }
    __device__ static __nv_bfloat16 from_float(float x) { return __float2bfloat16_rn(x); }
};

// Compensated accumulation of w * x (Kahan): `sum` carries the total, `comp`
// the low-order part lost by the previous addition.
__device__ __forceinline__ void kahan_add(float& sum, float& comp, float w, float x) {
    const float y = __fmaf_rn(w, x, -comp);
    const float t = __fadd_rn(sum, y);
    comp = __fsub_rn(__fsub_rn(t, sum), y);
    sum = t;
}

template <typename S, typename I>
__device__ __forceinline__ void gather8_lowp(I& cell, uint32_t wd, const I* table,
                                             const S* __restrict__ tex, float x[8]) {
#pragma unroll
    for (int b = 0; b < 8; ++b) {
        cell += table[(wd >> (4 * b)) & 15u];
        x[b] = StorageTraits<S>::load(tex + cell);
    }
}

// The steps of one half, in the order of the traced pass.  Full words
// without a stop code are gathered one word ahead, as in replay_half: the 8
// loads of word q+1 are in flight while word q's compensated sums run.
template <typename S, typename I>
__device__ __forceinline__ void replay_half_lowp(float& sum, float& comp, I p,
                                                 const uint32_t* __restrict__ words, int64_t npix,
                                                 int count, const float* w, const I* table,
                                                 const S* __restrict__ tex) {
    I cell = p;
    const int full = count >> 3;
    int q = 0;
    if (full > 0) {
        uint32_t wd = __ldg(words);
        if (!word_has_stop(wd)) {
            float x[8];
            gather8_lowp<S, I>(cell, wd, table, tex, x);
            for (q = 1; q < full; ++q) {
                wd = __ldg(words + size_t(q) * size_t(npix));
                if (word_has_stop(wd)) break;
                float y[8];
                gather8_lowp<S, I>(cell, wd, table, tex, y);
                const float* wq = w + 8 * (q - 1);
#pragma unroll
                for (int b = 0; b < 8; ++b) kahan_add(sum, comp, wq[b], x[b]);
#pragma unroll
                for (int b = 0; b < 8; ++b) x[b] = y[b];
            }
            const float* wq = w + 8 * (q - 1);
#pragma unroll
            for (int b = 0; b < 8; ++b) kahan_add(sum, comp, wq[b], x[b]);
        }
    }
    // remaining steps one by one: a word with a stop code, or the last partial word
    for (; q <= full; ++q) {
        const int n = (q < full) ? 8 : (count & 7);
        if (n == 0) break;
        const uint32_t wd = __ldg(words + size_t(q) * size_t(npix));
        const float* wq = w + 8 * q;
        for (int b = 0; b < n; ++b) {
            const uint32_t code = (wd >> (4 * b)) & 15u;
            if (code == kStop) return;
            cell += table[code];
            kahan_add(sum, comp, wq[b], StorageTraits<S>::load(tex + cell));
        }
    }
}

}  // namespace rlic
