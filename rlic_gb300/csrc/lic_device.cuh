// lic_device.cuh -- device-side streamline arithmetic of rLIC, for sm_103a.
//
// Every function here reproduces one function of the reference's native core
// (neutrinoceros/rlic, src/lib.rs) operation for operation, in the input
// dtype, so that streamline cell paths match the reference index for index:
//
//   * products and sums that Rust rounds separately use the __*_rn
//     intrinsics, which the compiler never contracts into an FMA;
//   * Rust's `mul_add` is fma()/fmaf() (one rounding);
//   * divisions are __fdiv_rn / __ddiv_rn (IEEE round-to-nearest), never an
//     approximate reciprocal;
//   * the library is also built with -fmad=false -prec-div=true -ftz=false as
//     a second guard.
//
// Coordinates are signed here; a step left from 0 gives -1, which plays the
// role of the reference's usize::wrapping_sub result usize::MAX
// (src/lib.rs:221, 84).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace rlic {

template <typename T> struct Vec2;
template <> struct Vec2<float> { using type = float2; };
template <> struct Vec2<double> { using type = double2; };

__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float abs_(float a) { return fabsf(a); }
__device__ __forceinline__ double abs_(double a) { return fabs(a); }

// num-traits Signed::signum for floats (std f32/f64::signum): -1 when the sign
// bit is set (including -0.0 and -inf), +1 otherwise, NaN for NaN.
template <typename T>
__device__ __forceinline__ T signum(T x) {
    return isnan(x) ? x : (signbit(x) ? T(-1) : T(1));
}

// time_to_next_pixel, src/lib.rs:157-180.
//   branchless + fma (default build):  |fma(1 + signum(v), 0.5 - f, f) / v|
//   branchless, no fma:                |((1 + signum(v)) * (0.5 - f) + f) / v|
//   branchy:  v > 0: (1 - f) / v;  v < 0: -(f / v);  else +inf
template <typename T, bool FMA, bool BRANCHLESS>
__device__ __forceinline__ T time_to_next_pixel(T vel, T frac) {
    if constexpr (BRANCHLESS) {
        const T s = add_rn(T(1), signum(vel));
        const T d = sub_rn(T(0.5), frac);
        T rem;
        if constexpr (FMA) {
            rem = fma_rn(s, d, frac);
        } else {
            rem = add_rn(mul_rn(s, d), frac);
        }
        return abs_(div_rn(rem, vel));
    } else {
        if (vel > T(0)) return div_rn(sub_rn(T(1), frac), vel);
        if (vel < T(0)) return -div_rn(frac, vel);
        return T(INFINITY);
    }
}

// One image axis with its two boundary rules (BoundaryPair, src/lib.rs:70-96),
// pre-resolved: a coordinate that stepped to -1 becomes `lo_to`, one that
// stepped to `size` becomes `hi_to` (closed: clamp; periodic: wrap).
template <typename I>
struct Axis {
    I size;
    I lo_to;
    I hi_to;
};

template <typename I>
__host__ __device__ inline Axis<I> make_axis(I size, int left, int right) {
    // 0 = closed, 1 = periodic  (src/lib.rs:84-95)
    Axis<I> a;
    a.size = size;
    a.lo_to = (left == 0) ? I(0) : size - 1;
    a.hi_to = (right == 0) ? size - 1 : I(0);
    return a;
}

template <typename I>
__device__ __forceinline__ I apply_axis(I c, const Axis<I>& a) {
    c = (c == I(-1)) ? a.lo_to : c;
    c = (c == a.size) ? a.hi_to : c;
    return c;
}

// advance, src/lib.rs:236-273, with update_state (src/lib.rs:209-233) inlined.
// (u, v) is the already sign-adjusted local velocity.  Ties and NaN times
// take the y branch (`tx < ty` is false).  Both axes get the boundary rule
// after every step (src/lib.rs:270-272); only the moved axis can be out of
// range, and applying the rule to an in-range coordinate is the identity.
template <typename T, bool FMA, bool BRANCHLESS, typename I>
__device__ __forceinline__ void advance(T u, T v, I& i, I& j, T& fx, T& fy,
                                        const Axis<I>& ax, const Axis<I>& ay) {
    if (u == T(0) && v == T(0)) return;
    const T tx = time_to_next_pixel<T, FMA, BRANCHLESS>(u, fx);
    const T ty = time_to_next_pixel<T, FMA, BRANCHLESS>(v, fy);
    const bool xstep = tx < ty;
    const T vpar = xstep ? u : v;
    const T vorth = xstep ? v : u;
    const T t = xstep ? tx : ty;
    T forth = xstep ? fy : fx;
    if constexpr (FMA) {
        forth = fma_rn(t, vorth, forth);
    } else {
        forth = add_rn(forth, mul_rn(t, vorth));
    }
    const bool up = vpar >= T(0);  // -0.0 counts as >= 0 (src/lib.rs:217)
    const T fpar = up ? T(0) : T(1);
    const I d = up ? I(1) : I(-1);
    if (xstep) {
        j = apply_axis(j + d, ax);
        fx = fpar;
        fy = forth;
    } else {
        i = apply_axis(i + d, ay);
        fy = fpar;
        fx = forth;
    }
}

// Read-only cached loads.
template <typename V>
__device__ __forceinline__ V ldg(const V* p) { return __ldg(p); }

// One half of convole_single_pixel (src/lib.rs:305-362): the forward trace
// (taps kmid+1 .. klen-1, ascending) or the backward trace (taps kmid-1 .. 0,
// descending), accumulating kernel[k] * input[cell] into `acc` after each
// step.  The reference reads u and v at the current cell, stops on NaN,
// flips the sample against the previous one in polarization mode (the dot
// product is two separately rounded products and a rounded sum,
// src/lib.rs:341), negates it for the backward trace, advances, then samples
// the texture at the new cell.
//
// `Rec` receives (step, linear cell) after each step when RECORD is true.
template <typename T, bool FMA, bool BRANCHLESS, bool POL, bool BACKWARD, bool RECORD,
          typename I, typename Rec>
__device__ __forceinline__ void trace_half(T& acc, I i, I j, I nx,
                                           const typename Vec2<T>::type* __restrict__ uv,
                                           const T* __restrict__ tex,
                                           const T* __restrict__ weights, int k0, int count,
                                           const Axis<I>& ax, const Axis<I>& ay, Rec rec) {
    T fx = T(0.5), fy = T(0.5);
    T lu = T(0), lv = T(0);
    for (int s = 0; s < count; ++s) {
        const int k = BACKWARD ? k0 - s : k0 + s;
        const auto p = ldg(uv + (i * nx + j));
        T pu = p.x, pv = p.y;
        if (isnan(pu) || isnan(pv)) break;
        if constexpr (POL) {
            const T dot = add_rn(mul_rn(pu, lu), mul_rn(pv, lv));
            if (dot < T(0)) {
                pu = -pu;
                pv = -pv;
            }
            lu = pu;
            lv = pv;
        }
        if constexpr (BACKWARD) {
            pu = -pu;
            pv = -pv;
        }
        advance<T, FMA, BRANCHLESS>(pu, pv, i, j, fx, fy, ax, ay);
        const I cell = i * nx + j;
        if constexpr (RECORD) {
            rec(s, cell);
        } else {
            const T x = ldg(tex + cell);
            const T w = weights[k];
            if constexpr (FMA) {
                acc = fma_rn(w, x, acc);
            } else {
                acc = add_rn(acc, mul_rn(w, x));
            }
        }
    }
}

struct NoRecord {
    template <typename I>
    __device__ __forceinline__ void operator()(int, I) const {}
};

}  // namespace rlic
