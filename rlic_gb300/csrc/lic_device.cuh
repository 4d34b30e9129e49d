// lic_device.cuh -- device-side streamline arithmetic of rLIC, for sm_103a.
//
// Every function here reproduces one function of the reference's native core
// (neutrinoceros/rlic, src/lib.rs) operation for operation, in the input
// dtype, so that streamline cell paths match the reference index for index:
//
//   * products and sums that Rust rounds separately use the __*_rn
//     intrinsics, which the compiler never contracts into an FMA;
//   * Rust's `mul_add` is __fmaf_rn / __fma_rn (one rounding);
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
// Bit patterns of float64 values moved through an opaque register move.  A
// plain bit cast would let the compiler turn integer tests and sign-bit
// edits back into FP64 compares, abs and negations, and GB300 runs FP64
// instructions at a small fraction of its FP32 rate (see the predicates
// below).
__device__ __forceinline__ uint64_t bits_of(double x) {
    uint64_t r;
    asm("mov.b64 %0, %1;" : "=l"(r) : "d"(x));
    return r;
}
__device__ __forceinline__ double from_bits(uint64_t b) {
    double r;
    asm("mov.b64 %0, %1;" : "=d"(r) : "l"(b));
    return r;
}

__device__ __forceinline__ float abs_(float a) { return fabsf(a); }
// float64 |a| and -a clear or flip the sign bit with an integer instruction
// (the same results as fabs and negation) and keep them off the FP64 pipe
__device__ __forceinline__ double abs_(double a) {
    return from_bits(bits_of(a) & 0x7FFFFFFFFFFFFFFFull);
}
__device__ __forceinline__ float neg_(float a) { return -a; }
__device__ __forceinline__ double neg_(double a) { return from_bits(bits_of(a) ^ (1ull << 63)); }
// signbit for the numerator's 1 + signum(v) (exactly 0 or 2)
__device__ __forceinline__ bool sign_set(float x) { return signbit(x); }
__device__ __forceinline__ bool sign_set(double x) { return (bits_of(x) >> 63) != 0; }

// Packed pairs of float32 operations (sm_100-family f32x2 instructions): each
// lane is rounded exactly as the scalar __fmaf_rn / __fsub_rn / __fmul_rn.
// The x and y halves of a streamline step are independent, so they share one
// instruction.
__device__ __forceinline__ float2 fma2_rn(float2 a, float2 b, float2 c) {
    float2 r;
    asm("{.reg .b64 pa, pb, pc, pd;\n\t"
        "mov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\tmov.b64 pc, {%6, %7};\n\t"
        "fma.rn.f32x2 pd, pa, pb, pc;\n\tmov.b64 {%0, %1}, pd;}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
    return r;
}
__device__ __forceinline__ float2 sub2_rn(float2 a, float2 b) {
    float2 r;
    asm("{.reg .b64 pa, pb, pd;\n\t"
        "mov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "sub.rn.f32x2 pd, pa, pb;\n\tmov.b64 {%0, %1}, pd;}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}
__device__ __forceinline__ float2 mul2_rn(float2 a, float2 b) {
    float2 r;
    asm("{.reg .b64 pa, pb, pd;\n\t"
        "mov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
        "mul.rn.f32x2 pd, pa, pb;\n\tmov.b64 {%0, %1}, pd;}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}

// Predicates of the streamline step.  GB300 executes FP64 instructions,
// comparisons included, at a small fraction of its FP32 rate, and the
// float64 trace is bound by that pipe; for float64 these predicates read the
// IEEE-754 bit patterns with integer instructions instead, with the same
// results as the comparisons they replace.  float32 keeps plain comparisons.
constexpr uint64_t kMagMask64 = 0x7FFFFFFFFFFFFFFFull;
constexpr uint64_t kInfBits64 = 0x7FF0000000000000ull;

// x == 0 (either sign)
__device__ __forceinline__ bool is_zero(float x) { return x == 0.f; }
__device__ __forceinline__ bool is_zero(double x) { return (bits_of(x) & kMagMask64) == 0; }
// isnan(x)
__device__ __forceinline__ bool is_nan(float x) { return isnan(x); }
__device__ __forceinline__ bool is_nan(double x) { return (bits_of(x) & kMagMask64) > kInfBits64; }
// x >= 0 for x not NaN (true for -0.0)
__device__ __forceinline__ bool nonneg(float x) { return x >= 0.f; }
__device__ __forceinline__ bool nonneg(double x) {
    const uint64_t b = bits_of(x);
    return (b >> 63) == 0 || (b & kMagMask64) == 0;
}
// a < b for a, b with the sign bit clear (|.| results: magnitudes, +inf, NaN).
// Such bit patterns order as unsigned integers the way the values do, NaN
// above +inf; a NaN on either side gives false, as the comparison.
__device__ __forceinline__ bool less_mag(float a, float b) { return a < b; }
__device__ __forceinline__ bool less_mag(double a, double b) {
    return bits_of(a) < bits_of(b) && bits_of(b) <= kInfBits64;
}
// add_rn(p, q) < 0.  The rounded sum has the sign of the exact sum: a nonzero
// sum of two floating-point numbers never rounds to zero (a sum that
// underflows is exact), an exact zero rounds to +0 (-0 only from -0 + -0,
// which is not below 0), and overflow keeps the sign.  So the sum is
// negative when both operands are negative and not both zero, or when the
// negative operand has the larger magnitude; NaN operands and inf + -inf
// (NaN) give false.
__device__ __forceinline__ bool sum_negative(float p, float q) { return add_rn(p, q) < 0.f; }
__device__ __forceinline__ bool sum_negative(double p, double q) {
    const uint64_t bp = bits_of(p), bq = bits_of(q);
    const uint64_t mp = bp & kMagMask64, mq = bq & kMagMask64;
    const bool np = (bp >> 63) != 0, nq = (bq >> 63) != 0;
    const bool neg = np ? (nq ? ((mp | mq) != 0) : (mp > mq)) : (nq && mq > mp);
    return neg && mp <= kInfBits64 && mq <= kInfBits64;
}

// Accumulation of one kernel-weighted sample: `mul_add` in the default build
// (src/lib.rs:357-360, 380-383), a rounded product then a rounded sum without
// the `fma` feature (src/lib.rs:353-356, 376-379).
template <typename T, bool FMA>
__device__ __forceinline__ T accumulate(T w, T x, T acc) {
    if constexpr (FMA) {
        return fma_rn(w, x, acc);
    } else {
        return add_rn(acc, mul_rn(w, x));
    }
}

// float32 steps: 1 = a lane whose velocity is zero (its state stays as it
// is) leaves the step by a branch, which spares the other lanes the selects
// that would keep its state (the float32 traced pass is bound by the ALU
// pipe those selects use); 0 = it runs the step with stand-in velocities
// and selects keep its state.  float64 steps always take the selects,
// which measured faster there.
#ifndef RLIC_STILL_BRANCH_F32
#define RLIC_STILL_BRANCH_F32 1
#endif


// Which operands of the time divisions are routed around the division
// sequence (see abs_quotient): 0 none; 1 zero numerators, with selects of
// the fixed results; 2 zero numerators and zero denominators; 3 zero
// numerators, with the result from a multiply by zero.  3 is the fastest on
// the at-scale workload (8192^2 float32; 1.6% ahead of 1 on the traced pass,
// whose ALU pipe the selects load): zero numerators are frequent
// (reversals), zero components rare, and the full guard's extra selects
// cost more than the slow paths it saves.
#ifndef RLIC_QUOTIENT_GUARD
#define RLIC_QUOTIENT_GUARD 3
#endif

// |a / b| rounded to nearest, for b not NaN.  A zero numerator or a zero
// denominator sends the division sequence to its slow path, and a warp whose
// lanes take it runs it for all of them.  Such operands are common here: a
// streamline that reverses direction meets a zero numerator every other
// step, and axis-aligned flows have a zero velocity component at every step.
// Their IEEE results are fixed, so they are produced by selects and the
// division only sees fast-path operands:
//   b == +-0:  a == +-0 or NaN -> NaN, otherwise inf
//   a == +-0:  0 (b is not NaN)
template <typename T>
__device__ __forceinline__ T abs_quotient(T a, T b) {
#if RLIC_QUOTIENT_GUARD == 0
    return abs_(div_rn(a, b));
#elif RLIC_QUOTIENT_GUARD == 1
    const bool a0 = is_zero(a);
    const T q = abs_(div_rn(a0 ? T(1) : a, b));
    return a0 ? (is_zero(b) ? T(NAN) : T(0)) : q;
#elif RLIC_QUOTIENT_GUARD == 3
    // a zero numerator divides a small power of two instead (2^-24 for
    // float32, 2^-53 for float64: the quotient stays finite for every
    // nonzero b, subnormals included) and keeps q * 0: 0 for b nonzero,
    // NaN for b zero (q = inf), as |0 / b|
    const bool a0 = is_zero(a);
    const T tiny = sizeof(T) == 4 ? T(0x1p-24) : T(0x1p-53);
    const T q = abs_(div_rn(a0 ? tiny : a, b));
    return a0 ? mul_rn(q, T(0)) : q;
#else
    const bool a0 = is_zero(a);
    const bool a0n = a0 || is_nan(a);
    const bool b0 = is_zero(b);
    const T q = abs_(div_rn((a0 | b0) ? T(1) : a, b0 ? T(1) : b));
    return b0 ? (a0n ? T(NAN) : T(INFINITY)) : (a0 ? T(0) : q);
#endif
}

// Signed quotient a / b, for the branchy variant (b nonzero and not NaN).
template <typename T>
__device__ __forceinline__ T signed_quotient(T a, T b) {
    const bool a0 = is_zero(a);
    const T q = div_rn(a0 ? T(1) : a, b);
    return a0 ? ((signbit(a) != signbit(b)) ? T(-0.0) : T(0.0)) : q;
}

// time_to_next_pixel, src/lib.rs:157-180.
//   branchless + fma (default build):  |fma(1 + signum(v), 0.5 - f, f) / v|
//   branchless, no fma:                |((1 + signum(v)) * (0.5 - f) + f) / v|
//   branchy:  v > 0: (1 - f) / v;  v < 0: -(f / v);  else +inf
// On the branchless path v is never NaN here (a NaN sample stops the trace
// before any advance, src/lib.rs:336-338), so 1 + signum(v) is exactly 2 when
// the sign bit of v is clear and exactly 0 when it is set (num-traits
// signum: -0.0 -> -1).
template <typename T, bool FMA, bool BRANCHLESS>
__device__ __forceinline__ T time_to_next_pixel(T vel, T frac) {
    if constexpr (BRANCHLESS) {
        const T s = sign_set(vel) ? T(0) : T(2);
        const T d = sub_rn(T(0.5), frac);
        T rem;
        if constexpr (FMA) {
            rem = fma_rn(s, d, frac);
        } else {
            rem = add_rn(mul_rn(s, d), frac);
        }
        return abs_quotient(rem, vel);
    } else {
        if (vel > T(0)) return signed_quotient(sub_rn(T(1), frac), vel);
        if (vel < T(0)) return -signed_quotient(frac, vel);
        return T(INFINITY);
    }
}

// Both times of one step, tx for (u, fx) and ty for (v, fy).  The default
// float32 build computes the x and y halves of the branchless formula as
// packed pairs; every other case is time_to_next_pixel twice.
template <typename T, bool FMA, bool BRANCHLESS>
__device__ __forceinline__ void times_to_next_pixel(T u, T v, T fx, T fy, T& tx, T& ty) {
    if constexpr (BRANCHLESS && FMA && sizeof(T) == 4) {
        const float2 s = make_float2(signbit(u) ? 0.f : 2.f, signbit(v) ? 0.f : 2.f);
        const float2 f = make_float2(fx, fy);
        const float2 rem = fma2_rn(s, sub2_rn(make_float2(0.5f, 0.5f), f), f);
        tx = abs_quotient(rem.x, float(u));
        ty = abs_quotient(rem.y, float(v));
    } else {
        tx = time_to_next_pixel<T, FMA, BRANCHLESS>(u, fx);
        ty = time_to_next_pixel<T, FMA, BRANCHLESS>(v, fy);
    }
}

// The branchless numerator fma(1 + signum(v), 0.5 - f, f) of
// time_to_next_pixel (src/lib.rs:168-179), before its division.
template <typename T, bool FMA>
__device__ __forceinline__ T time_numerator(T vel, T frac) {
    const T s = sign_set(vel) ? T(0) : T(2);
    const T d = sub_rn(T(0.5), frac);
    return FMA ? fma_rn(s, d, frac) : add_rn(mul_rn(s, d), frac);
}

// Axis of a trace's last move: before the first move both fractions are
// 0.5; after a move along an axis, that axis's fraction is exactly 0 or 1
// (update_state, src/lib.rs:217-223).
constexpr int kLastNone = 0, kLastX = 1, kLastY = 2;

// The numerator fma(1 + signum(v), 0.5 - f, f) for f exactly 0, 0.5 or 1,
// without FP64 instructions: 0.5 for f = 0.5; for f in {0, 1} with
// s = 1 + signum(v) in {0, 2}, s = 2 gives 1 - f and s = 0 gives f, all
// exact (2 * 0.5 + 0 = 1, 2 * -0.5 + 1 = +0, 0 * x + f = f).  The product
// and sum of the branchless build without `fma` give the same values.
__device__ __forceinline__ double known_numerator(double vel, double frac, bool centre) {
    const bool s2 = !sign_set(vel);
    const bool one = (bits_of(frac) >> 52) == 0x3FFull;  // frac == 1.0 (else +0)
    return centre ? 0.5 : ((s2 != one) ? 1.0 : 0.0);
}

// The numerator fma(2, 0.5 - f, f) (1 + signum(v) = 2: the sign bit of v
// clear) rounded to nearest, for 0 <= f <= 1, with integer instructions
// only.  The FP64 pipe bounds the float64 step, and this replaces its
// subtraction and its FMA.  Returns false, leaving g unset, for f outside
// [0, 1] (the sign bit set, -0 included), where the caller uses FP64.
//
// With f = m 2^(E - 1075) (E its biased exponent, m its 53-bit
// significand), d = RN(0.5 - f) and g = RN(2 d + f):
//   * f = 1: 2 (0.5 - 1) + 1 = +0;
//   * f in [0.5, 1): d = 0.5 - f exactly (Sterbenz), so g = 1 - f exactly,
//     r 2^-53 with r = 2^53 - m, normalised by its leading zeros;
//   * f in [2^-55, 0.5): d lies in [0.25, 0.5], a multiple of 2^-54.  With
//     s1 = 1021 - E, f = (K + lo1 / 2^s1) 2^-54 for K = m >> s1, and
//     d = (2^53 - K - c1) 2^-54, c1 rounding the remainder lo1 against
//     half a unit h1 = 2^(s1-1) (ties to the even D; s1 = 0, f in
//     [0.25, 0.5), is exact).  In units of 2^-53, 2 d + f = 2^53 - K - c1 +
//     K / 2 exactly plus the remainder (K odd: half a unit and lo1), so
//     g = (2^53 - ceil(K / 2) - c1 + c2) 2^-53, c2 rounding that remainder
//     (ties to even); a result of 2^53 units is 1.0;
//   * f < 2^-55 (subnormals and zero included): d = 0.5 and g = RN(1 + f)
//     = 1.
// Checked against the FP64 sequence on random and constructed operands,
// rounding ties included (rlic_check_numerators_f64).
constexpr uint64_t kMant52 = (uint64_t(1) << 52) - 1;
constexpr uint64_t kOneBits64 = 0x3FF0000000000000ull;

__device__ __forceinline__ bool numerator_two_int(double f, double& g) {
    const uint64_t b = bits_of(f);
    const uint32_t E = uint32_t(b >> 52);  // the sign bit included: f < 0 gives E >= 2048
    const uint64_t m = (b & kMant52) | (uint64_t(1) << 52);
    // f in [0.5, 1)
    const uint64_t r1 = (uint64_t(1) << 53) - m;
    const int lz = __clzll(r1 | 1u);
    const uint64_t g_half = (uint64_t(uint32_t(1033 - lz) & 0x7FFu) << 52) |
                            ((r1 << (lz > 11 ? lz - 11 : 0)) & kMant52);
    // f in [2^-55, 0.5)
    int s1 = 1021 - int(E);
    s1 = s1 < 0 ? 0 : (s1 > 53 ? 53 : s1);
    const uint64_t K = m >> s1;
    const uint64_t lo1 = m & ((uint64_t(1) << s1) - 1);
    const uint64_t h1 = (uint64_t(1) << s1) >> 1;
    const uint64_t c1 = (s1 > 0 && (lo1 > h1 || (lo1 == h1 && (K & 1)))) ? 1u : 0u;
    const uint64_t G0 = (uint64_t(1) << 53) - ((K + 1) >> 1) - c1;
    const uint64_t c2 = ((K & 1) && (lo1 != 0 || (G0 & 1))) ? 1u : 0u;
    const uint64_t G = G0 + c2;
    const uint64_t g_low =
        G >= (uint64_t(1) << 53) ? kOneBits64 : ((uint64_t(1022) << 52) | (G & kMant52));
    uint64_t r = E < 968u ? kOneBits64 : (E <= 1021u ? g_low : g_half);
    r = b == kOneBits64 ? 0u : r;
    g = from_bits(r);
    return E < 1023u || b == kOneBits64;
}

// Both numerators of a float64 step, computing only the one of the axis
// whose fraction is not known exactly (the axis not moved last; x before
// the first move, when both are 0.5): f when the velocity's sign bit is set
// (1 + signum(v) = 0: 0 (0.5 - f) + f = f), otherwise by integer
// instructions (numerator_two_int), and with FP64 instructions only for a
// fraction outside [0, 1].  The branchless build without `fma` rounds
// 2 (0.5 - f) exactly and then the sum, the same value.
// INT_NUM = false computes it with FP64 instructions instead (the paired
// pass on small images, which waits on latency more than on the FP64 pipe:
// the integer sequence lengthens each step's chain there).
template <bool FMA, bool INT_NUM = true>
__device__ __forceinline__ void time_numerators(double u, double v, double fx, double fy,
                                                int last, double& ax, double& ay) {
    const bool gen_y = (last == kLastX);
    const double vel = gen_y ? v : u;
    const double frac = gen_y ? fy : fx;
    double g;
    if constexpr (INT_NUM) {
        g = frac;
        if (!sign_set(vel)) {
            if (!numerator_two_int(frac, g)) g = time_numerator<double, FMA>(vel, frac);
        }
    } else {
        g = time_numerator<double, FMA>(vel, frac);
    }
    const double k = known_numerator(gen_y ? u : v, gen_y ? fx : fy, last == kLastNone);
    ax = gen_y ? k : g;
    ay = gen_y ? g : k;
}

// float64 step choice with one division where two are not needed.
//
// A step compares tx = |ax / u| with ty = |ay / v| (both rounded), then uses
// only the chosen one.  The float64 division is the bulk of the FP64 work
// of a step, so the comparison is settled first, when it provably can be,
// from the cross products |ax|*|v| and |ay|*|u| (tx < ty exactly when the
// first is the smaller, up to the rounding of the quotients):
//
//   * every operand is truncated to float32 from its bit pattern (integer
//     instructions): x' <= |x| < x' (1 + 2^-23);
//   * the float32 products p1 = x'y' carry a further 2^-24 rounding, so
//     p1 < p2 (1 - 2^-16) implies |ax||v| < |ay||u| (1 - 2^-17): the exact
//     quotients differ by far more than one unit in the last place, hence
//     so do the rounded ones, and tx < ty; symmetrically p1 > p2 (1 + 2^-16)
//     implies tx > ty;
//   * the screen runs only when u, v and the nonzero numerators are normal
//     with binary exponents in [-60, 60], so that x', the products and the
//     quotients stay normal and finite;
//   * a zero numerator needs no division: |0 / u| = 0 for u nonzero, so
//     tx < ty exactly when ax is zero and ay is not, and the time is 0.
//
// Returns false when the screen cannot decide (operands out of range, or
// products within 2^-16 of each other); the caller then divides both.
__device__ __forceinline__ bool screen_in_range(uint32_t hi) {
    const uint32_t e = (hi >> 20) & 0x7FFu;  // biased exponent
    return e - (1023u - 60u) <= 120u;
}
__device__ __forceinline__ float truncate_to_f32(double x) {
    // |x| with 23 mantissa bits kept, for exponents in [-60, 60]
    const uint64_t b = bits_of(x);
    const uint32_t hi = uint32_t(b >> 32), lo = uint32_t(b);
    const uint32_t e = ((hi >> 20) & 0x7FFu) - (1023u - 127u);
    return __uint_as_float((e << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29));
}
// |a| / |b| rounded to nearest for nonzero a and b whose binary exponents
// lie in [-60, 60] (the screened range), with 4 FP64 instructions instead of
// a general division; returns false when it cannot certify the result (the
// caller then divides with __ddiv_rn).  Methods: Newton-Raphson refinement
// of a reciprocal from a float32 seed (Markstein, "Computation of elementary
// functions on the IBM RISC System/6000 processor", IBM J. Res. Dev. 1990),
// and the exact FMA remainder r = a - b q of a quotient within one ulp
// (Boldo and Daumas, "Representable correcting terms for possibly
// underflowing floating point operations", ARITH 2003), used here only as a
// certificate:
//
//   y0 = rcp.approx(float32(|b|))          relative error < 2^-21
//   y1 = y0 + y0 (1 - |b| y0)               relative error ~2^-42 (FP32
//                                           pipe, reciprocal_seed)
//   q0 = |a| y1;  q1 = q0 + y1 (|a| - |b| q0)
//   r  = fma(-|b|, q1, |a|)
//
// q1 is the rounded quotient exactly when |a/b - q1| < ulp(q1)/2, i.e.
// R = |r| / (|b| ulp(q1)) < 1/2 (q1 not a power of two, whose lower
// neighbour is only half an ulp away: those are refused).  R is bounded
// from r's and b's exponents and 23-bit mantissas with a 2^-16 margin; a
// refused R (near a rounding tie, or q1 off by an ulp) falls back.  An
// inexact r (q1 off by more than an ulp) has R near or above 1 and is
// refused as well.  Every intermediate stays normal: |b| and |a| in
// [2^-60, 2^61), quotients in (2^-121, 2^121), and a nonzero r is a
// multiple of 2^-285.

// 1: the reciprocal seed's Newton step runs on the FP32 pipe
// (reciprocal_seed); 0: it runs as two FP64 FMAs.
#ifndef RLIC_F64_SEED_FP32
#define RLIC_F64_SEED_FP32 1
#endif

__device__ __forceinline__ double f32_to_f64_bits(float x) {
    // exact widening of a normal positive float32 with integer instructions
    const uint32_t b = __float_as_uint(x);
    const uint64_t e = uint64_t(((b >> 23) & 0xFFu) + (1023u - 127u));
    return from_bits((e << 52) | (uint64_t(b & 0x7FFFFFu) << 29));
}
__device__ __forceinline__ float mantissa_f32(double x) {
    // the 23 leading fraction bits of x as a float32 in [1, 2)
    const uint64_t b = bits_of(x);
    return __uint_as_float((127u << 23) | uint32_t((b >> 29) & 0x7FFFFFu));
}
// The Newton step y1 = y0 + y0 (1 - B y0) on the FP32 pipe: B is split into
// its leading 24 bits bh and the next 24 bits bm, the product bh y0 is
// taken exactly (its rounding error by an FMA), and the correction
// y0 (1 - (bh + bm) y0), about 2^-21 y0, is accurate to about 2^-45 y0.  y1
// is assembled as a float64 from y0 and the correction with 64-bit integer
// arithmetic (truncated to 53 bits).  Its accuracy, about 2^-42, only
// affects how often the certificate of quotient_screened accepts, never
// the correctness of an accepted quotient.
__device__ __forceinline__ double reciprocal_seed(double B) {
    const uint64_t bb = bits_of(B);
    const uint32_t eb = uint32_t(bb >> 52) & 0x7FFu;  // biased exponent of B
    const float bh = truncate_to_f32(B);
    // bits 28..0 of the significand, value lo29 * 2^(eb - 1075), as a float
    const uint32_t lo29 = uint32_t(bb) & 0x1FFFFFFFu;
    const float lo_f = __uint2float_rz(lo29);  // exact leading 24 bits
    const float bm = lo29 ? __uint_as_float(__float_as_uint(lo_f) - ((1075u - eb) << 23)) : 0.f;
    float r0;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r0) : "f"(bh));
    const float hi = __fmul_rn(bh, r0);
    const float lo = __fmaf_rn(bh, r0, -hi);  // exact: bh r0 = hi + lo
    const float e = __fmaf_rn(-bm, r0, __fsub_rn(__fsub_rn(1.f, hi), lo));
    const float c = __fmul_rn(r0, e);
    // y1 = r0 + c: significands as 64-bit fixed point, r0's leading bit at 61
    const uint32_t rb = __float_as_uint(r0), cb = __float_as_uint(c);
    const int kr = int((rb >> 23) & 0xFFu), kc = int((cb >> 23) & 0xFFu);
    int64_t y = int64_t((rb & 0x7FFFFFu) | 0x800000u) << 38;
    const int d = kr - kc;
    if ((cb & 0x7FFFFFFFu) != 0u && d >= 0 && d <= 61) {
        const int64_t cs = (int64_t((cb & 0x7FFFFFu) | 0x800000u) << 38) >> d;
        y = (cb >> 31) ? y - cs : y + cs;
    }
    const int msb = 63 - __clzll(y);  // 60, 61 or 62
    const uint64_t mant = (uint64_t(y) >> (msb - 52)) & 0xFFFFFFFFFFFFFull;
    return from_bits((uint64_t(msb + kr + 835) << 52) | mant);
}

__device__ __forceinline__ bool quotient_screened(double a, double b, double& q) {
    const double A = abs_(a), B = abs_(b);
#if RLIC_F64_SEED_FP32
    const double y1 = reciprocal_seed(B);
#else
    float r0;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r0) : "f"(truncate_to_f32(B)));
    const double y0 = f32_to_f64_bits(r0);
    const double y1 = fma_rn(y0, fma_rn(-B, y0, 1.0), y0);
#endif
    const double q0 = mul_rn(A, y1);
    const double q1 = fma_rn(fma_rn(-B, q0, A), y1, q0);
    const double r = fma_rn(-B, q1, A);
    q = q1;
    const uint64_t bq = bits_of(q1), br = bits_of(r) & kMagMask64;
    if ((bq & 0xFFFFFFFFFFFFFull) == 0) return false;  // power of two
    if (br == 0) return true;                            // exact quotient
    const int k = int(br >> 52) - int(bits_of(B) >> 52) - int(bq >> 52) + (1023 + 52);
    if (k <= -3) return true;   // R < 2 * 2^-3
    if (k >= 0) return false;   // R > 1/2
    const float lhs = __fmul_rn(mantissa_f32(r), k == -1 ? 0.5f : 0.25f);
    return lhs < __fmul_rn(mantissa_f32(B), 0.5f - 0x1p-17f);
}

__device__ __forceinline__ bool screen_step(double ax, double ay, double u, double v,
                                            bool& xstep) {
    const bool ax0 = is_zero(ax), ay0 = is_zero(ay);
    const bool in_range = screen_in_range(uint32_t(bits_of(u) >> 32)) &&
                          screen_in_range(uint32_t(bits_of(v) >> 32)) &&
                          (ax0 || screen_in_range(uint32_t(bits_of(ax) >> 32))) &&
                          (ay0 || screen_in_range(uint32_t(bits_of(ay) >> 32)));
    const float p1 = __fmul_rn(truncate_to_f32(ax), truncate_to_f32(v));
    const float p2 = __fmul_rn(truncate_to_f32(ay), truncate_to_f32(u));
    const bool lt = p1 < __fmul_rn(p2, 1.0f - 0x1p-16f);
    const bool gt = p1 > __fmul_rn(p2, 1.0f + 0x1p-16f);
    const bool any0 = ax0 || ay0;
    xstep = any0 ? (ax0 && !ay0) : lt;
    return in_range && (any0 || lt || gt);
}

// One image axis with its two boundary rules (BoundaryPair, src/lib.rs:70-96),
// pre-resolved: a coordinate that stepped to -1 becomes `lo_to`, one that
// stepped to `size` becomes `hi_to` (closed: clamp; periodic: wrap).  The
// fraction is left alone, as in the reference.
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

// Image geometry of one launch.
template <typename I>
struct Geometry {
    I ny, nx;
    Axis<I> ax, ay;
};

// Step codes of the path cache: 4 bits per streamline step, two 2-bit
// fields: bits 0-1 the column move dx, bits 2-3 the row move dy, each 00 = 0,
// 01 = +1, 11 = -1 (two's complement), 10 = a wrap across a periodic edge.
//   0x0    no move (zero velocity, or a move cancelled by a closed boundary)
//   0x1, 0x3   +1 / -1 column         0x4, 0xC   +1 / -1 row
//   0x2, 0x6   wrap right -> left (-(nx-1)) / left -> right (+(nx-1))
//   0x8, 0x9   wrap bottom -> top (-(ny-1) rows) / top -> bottom (+(ny-1) rows)
//   0xF    the trace stopped on a NaN sample (a step never moves both axes)
// The table below maps every code to its linear-index delta.  Replaying the
// deltas from the start pixel visits exactly the cells the trace visited.
constexpr uint32_t kStop = 15u;

// True when one of the 8 codes of a word is the stop code (all four bits set).
__device__ __forceinline__ bool word_has_stop(uint32_t wd) {
    return (wd & (wd >> 1) & (wd >> 2) & (wd >> 3) & 0x11111111u) != 0u;
}

template <typename I>
__device__ __forceinline__ void fill_delta_table(I* table, I nx, I ny) {
    // called by one thread
    for (int c = 0; c < 16; ++c) table[c] = 0;
    table[0x1] = 1;
    table[0x3] = -1;
    table[0x4] = nx;
    table[0xC] = -nx;
    table[0x2] = -(nx - 1);
    table[0x6] = nx - 1;
    table[0x8] = -(ny - 1) * nx;
    table[0x9] = (ny - 1) * nx;
}

// advance, src/lib.rs:236-273, with update_state (src/lib.rs:209-233) folded
// in, on one pixel state.  (u, v) is the sign-adjusted local velocity.
//
// Ties and NaN times take the y branch (`tx < ty` is false); -0.0 counts as
// >= 0 (src/lib.rs:217).  A zero velocity leaves everything unchanged
// (src/lib.rs:242-244); this is applied with selects rather than a branch so
// that a warp whose lanes sit on zero cells stays converged.
//
// EDGE = false is the interior fast path: the caller guarantees no step can
// reach the image border, so the boundary rule (src/lib.rs:270-272) is the
// identity and only the linear index is tracked.  EDGE = true tracks the row
// and column and applies the rule to the moved axis (the other axis is in
// range already, and the rule is the identity on in-range coordinates).
//
// Returns the step code (see above).
template <typename T, bool FMA, bool BRANCHLESS, bool EDGE, typename I, bool INT_NUM = true>
__device__ __forceinline__ uint32_t advance(T u, T v, T& fx, T& fy, I& cell, I& i, I& j,
                                            int& last, const Geometry<I>& g) {
    const bool still = is_zero(u) & is_zero(v);
    if constexpr (sizeof(T) == 4 && RLIC_STILL_BRANCH_F32) {
        if (still) return 0u;  // the state stays as it is (src/lib.rs:242-244)
    }
    // A still lane keeps its state whatever the times are; giving it unit
    // velocities keeps its divisions on the fast path (a division by zero
    // takes the slow one) and its lane in step with the warp.
    const T su = still ? T(1) : u;
    const T sv = still ? T(1) : v;
    bool xstep;
    T t;
    if constexpr (BRANCHLESS && sizeof(T) == 8) {
        // one division when the screen settles the comparison, else both;
        // one numerator computed in FP64 (see known_numerator)
        T ax, ay;
        time_numerators<FMA, INT_NUM>(su, sv, fx, fy, last, ax, ay);
        const bool settled = screen_step(ax, ay, su, sv, xstep);
        const bool first_x = !settled || xstep;
        const T num = first_x ? ax : ay;
        const T den = first_x ? su : sv;
        // settled lanes: the screened division (a zero numerator gives 0)
        const bool num0 = is_zero(num);
        T q;
        const bool certified = quotient_screened(num0 ? T(1) : num, den, q);
        t = num0 ? T(0) : q;
        if (!(settled && certified)) {  // rare: general divisions
            const T q1 = abs_quotient(num, den);
            t = q1;
            if (!settled) {
                const T ty = abs_quotient(ay, sv);
                xstep = less_mag(q1, ty);
                t = xstep ? q1 : ty;
            }
        }
    } else {
        T tx, ty;
        times_to_next_pixel<T, FMA, BRANCHLESS>(su, sv, fx, fy, tx, ty);
        // the branchless times are magnitudes (|.|, +inf or NaN): less_mag applies
        xstep = BRANCHLESS ? less_mag(tx, ty) : (tx < ty);
        t = xstep ? tx : ty;
    }
    // the orthogonal update of either branch (update_state, src/lib.rs:225-232):
    // an x step moves fy by t * v, a y step moves fx by t * u.  float32
    // computes both in one packed instruction and keeps one; float64 computes
    // only the one kept.
    T cx, cy;
    if constexpr (FMA && sizeof(T) == 4) {
        const float2 c = fma2_rn(make_float2(t, t), make_float2(su, sv), make_float2(fx, fy));
        cx = c.x;
        cy = c.y;
    } else {
        const T vo = xstep ? sv : su;
        const T fo = xstep ? fy : fx;
        const T o = FMA ? fma_rn(t, vo, fo) : add_rn(fo, mul_rn(t, vo));
        cx = o;
        cy = o;
    }
    const T vpar = xstep ? su : sv;
    const bool up = nonneg(vpar);
    const T fpar = up ? T(0) : T(1);
    const T nfx = xstep ? fpar : cx;
    const T nfy = xstep ? cy : fpar;
    fx = still ? fx : nfx;
    fy = still ? fy : nfy;
    last = still ? last : (xstep ? kLastX : kLastY);
    if constexpr (!EDGE) {
        const I step = xstep ? I(1) : g.nx;
        cell += still ? I(0) : (up ? step : -step);
        const uint32_t code = xstep ? (up ? 0x1u : 0x3u) : (up ? 0x4u : 0xCu);
        return still ? 0u : code;
    } else {
        const I c_old = xstep ? j : i;
        const I size = xstep ? g.ax.size : g.ay.size;
        const I lo_to = xstep ? g.ax.lo_to : g.ay.lo_to;
        const I hi_to = xstep ? g.ax.hi_to : g.ay.hi_to;
        I c = c_old + (up ? I(1) : I(-1));
        c = (c == I(-1)) ? lo_to : c;
        c = (c == size) ? hi_to : c;
        c = still ? c_old : c;
        const I dd = c - c_old;
        if (xstep) {
            j = c;
        } else {
            i = c;
        }
        cell += xstep ? dd : dd * g.nx;
        uint32_t code;
        if (dd == I(0)) {
            code = 0u;
        } else if (dd == I(1)) {
            code = xstep ? 0x1u : 0x4u;
        } else if (dd == I(-1)) {
            code = xstep ? 0x3u : 0xCu;
        } else if (dd < I(0)) {
            code = xstep ? 0x2u : 0x8u;
        } else {
            code = xstep ? 0x6u : 0x9u;
        }
        return code;
    }
}

// A load of kernel input: through the read-only data cache (NC, the
// default: the data does not change while the kernel runs), or a plain
// coherent load, for data that other CTAs of the same launch wrote before
// an acquire (the persistent batched kernel).
template <bool NC, typename V>
__device__ __forceinline__ V ld_in(const V* p) {
    if constexpr (NC) {
        return __ldg(p);
    } else {
        return *p;
    }
}

// 8 consecutive values from 16-byte aligned (shared) memory, with vector loads.
__device__ __forceinline__ void load8_aligned(const float* w, float out[8]) {
    const float4 a = reinterpret_cast<const float4*>(w)[0];
    const float4 b = reinterpret_cast<const float4*>(w)[1];
    out[0] = a.x; out[1] = a.y; out[2] = a.z; out[3] = a.w;
    out[4] = b.x; out[5] = b.y; out[6] = b.z; out[7] = b.w;
}
__device__ __forceinline__ void load8_aligned(const double* w, double out[8]) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const double2 a = reinterpret_cast<const double2*>(w)[k];
        out[2 * k] = a.x;
        out[2 * k + 1] = a.y;
    }
}

// Per-trace state of convole_single_pixel (src/lib.rs:314-323).
template <typename T, typename I>
struct TraceState {
    T fx, fy;  // position inside the cell, starting at the centre (0.5, 0.5)
    T lu, lv;  // previous sample in polarization mode, starting at (0, 0)
    int last;  // axis of the last move (kLastNone before the first)
    I cell, i, j;
    bool back;  // direction chosen at run time (kDirRuntime): backward
};

// Direction of a half-trace: forward, backward, or chosen per thread at run
// time (TraceState::back), for kernels whose lanes trace both halves.
constexpr int kDirForward = 0, kDirBackward = 1, kDirRuntime = 2;

// -x when n is set, x otherwise: a sign-bit edit (integer instruction).
__device__ __forceinline__ float neg_if(float x, bool n) {
    return __uint_as_float(__float_as_uint(x) ^ (n ? 0x80000000u : 0u));
}
__device__ __forceinline__ double neg_if(double x, bool n) {
    return from_bits(bits_of(x) ^ (uint64_t(n) << 63));
}

// One step of convole_single_pixel (src/lib.rs:331-361): read u and v at the
// current cell, stop on NaN (returns false), flip the sample against the
// previous one in polarization mode (the dot product is two separately
// rounded products and a rounded sum, src/lib.rs:341), negate it for the
// backward trace, advance, then accumulate weight * texture at the new cell.
// `code` receives the step code; `x_out`, when given, the texture sample.
// INT_NUM: see time_numerators (float64 only).
template <typename T, bool FMA, bool BRANCHLESS, bool POL, int DIR, bool EDGE,
          bool SAMPLE, typename I, bool NAN_CHECK = true, bool NC = true, bool INT_NUM = true>
__device__ __forceinline__ bool trace_step(TraceState<T, I>& st, T& acc, T w,
                                           const Geometry<I>& g,
                                           const typename Vec2<T>::type* __restrict__ uv,
                                           const T* __restrict__ tex, uint32_t& code,
                                           T* x_out = nullptr) {
    const auto p = ld_in<NC>(uv + st.cell);
    T pu = p.x, pv = p.y;
    // (NAN_CHECK false: the caller knows the field holds no NaN sample)
    if (NAN_CHECK && (is_nan(pu) || is_nan(pv))) return false;
    if constexpr (POL) {
        bool flip;
        if constexpr (sizeof(T) == 4) {
            const float2 pr = mul2_rn(make_float2(pu, pv), make_float2(st.lu, st.lv));
            flip = sum_negative(pr.x, pr.y);
        } else {
            flip = sum_negative(mul_rn(pu, st.lu), mul_rn(pv, st.lv));
        }
        if (flip) {
            pu = neg_(pu);
            pv = neg_(pv);
        }
        st.lu = pu;
        st.lv = pv;
    }
    if constexpr (DIR == kDirBackward) {
        pu = neg_(pu);
        pv = neg_(pv);
    } else if constexpr (DIR == kDirRuntime) {
        pu = neg_if(pu, st.back);
        pv = neg_if(pv, st.back);
    }
    code = advance<T, FMA, BRANCHLESS, EDGE, I, INT_NUM>(pu, pv, st.fx, st.fy, st.cell, st.i,
                                                         st.j, st.last, g);
    if constexpr (SAMPLE) {
        const T x = ld_in<NC>(tex + st.cell);
        acc = accumulate<T, FMA>(w, x, acc);
        if (x_out) *x_out = x;
    }
    return true;
}

// Steps of a code word unrolled in trace_half, per element type.  The
// float64 step is long, and 8 unrolled steps overflow the instruction cache
// (ncu: warps waiting on instruction fetch): 2 measured 10-12% faster than 8
// (4096^2, 129 taps, one pass: 30.4 against 33.9 ms; 2048^2, 65 taps: 3.92
// against 4.42 ms), 4 in between.  The float32 step keeps the whole word.
#ifndef RLIC_TRACE_UNROLL_F64
#define RLIC_TRACE_UNROLL_F64 2
#endif
#ifndef RLIC_TRACE_UNROLL_F32
#define RLIC_TRACE_UNROLL_F32 8
#endif
template <typename T> struct TraceUnroll { static constexpr int value = RLIC_TRACE_UNROLL_F32; };
template <> struct TraceUnroll<double> { static constexpr int value = RLIC_TRACE_UNROLL_F64; };

// One half of convole_single_pixel (src/lib.rs:305-362): the forward trace
// (taps kmid+1 .. klen-1, ascending) or the backward trace (taps kmid-1 .. 0,
// descending), accumulating kernel[k] * input[cell] into `acc` after each
// step.  `w` holds this half's weights in step order (w[s] is the tap of
// step s), 8-entry aligned.  When SAMPLE is false the texture is not read.
//
// Steps run in groups of 8, one 32-bit word of step codes per group; with
// RECORD the word is stored at words[group * stride].  A trace that stops on
// NaN stores the stop code in place of its step and nothing after it.
template <typename T, bool FMA, bool BRANCHLESS, bool POL, int DIR, bool EDGE,
          bool SAMPLE, bool RECORD, typename I, bool NAN_CHECK = true, bool NC = true>
__device__ __forceinline__ void trace_half(T& acc, I i, I j, const Geometry<I>& g,
                                           const typename Vec2<T>::type* __restrict__ uv,
                                           const T* __restrict__ tex, const T* w, int count,
                                           uint32_t* __restrict__ words, size_t stride) {
    TraceState<T, I> st;
    st.last = kLastNone;
    st.fx = T(0.5);
    st.fy = T(0.5);
    st.lu = T(0);
    st.lv = T(0);
    st.cell = i * g.nx + j;
    st.i = i;
    st.j = j;
    st.back = DIR == kDirBackward;
    const int full = count >> 3;
    for (int q = 0; q < full; ++q) {
        const T* wq = w + 8 * q;
        uint32_t word = 0;
#pragma unroll(TraceUnroll<T>::value)
        for (int b = 0; b < 8; ++b) {
            uint32_t code = 0;
            if (!trace_step<T, FMA, BRANCHLESS, POL, DIR, EDGE, SAMPLE, I, NAN_CHECK, NC>(
                    st, acc, SAMPLE ? wq[b] : T(0), g, uv, tex, code)) {
                if constexpr (RECORD) words[size_t(q) * stride] = word | (kStop << (4 * b));
                return;
            }
            word |= code << (4 * b);
        }
        if constexpr (RECORD) words[size_t(q) * stride] = word;
    }
    const int rest = count & 7;
    if (rest) {
        uint32_t word = 0;
        for (int b = 0; b < rest; ++b) {
            uint32_t code = 0;
            if (!trace_step<T, FMA, BRANCHLESS, POL, DIR, EDGE, SAMPLE, I, NAN_CHECK, NC>(
                    st, acc, SAMPLE ? w[8 * full + b] : T(0), g, uv, tex, code)) {
                if constexpr (RECORD) words[size_t(full) * stride] = word | (kStop << (4 * b));
                return;
            }
            word |= code << (4 * b);
        }
        if constexpr (RECORD) words[size_t(full) * stride] = word;
    }
}

// The same walk for path parity checks: reports the cell reached by every
// step to `rec(s, cell)`.
template <typename T, bool FMA, bool BRANCHLESS, bool POL, int DIR, typename I, typename Rec>
__device__ __forceinline__ void walk_half(I i, I j, const Geometry<I>& g,
                                          const typename Vec2<T>::type* __restrict__ uv,
                                          int count, Rec rec) {
    TraceState<T, I> st;
    st.last = kLastNone;
    st.fx = T(0.5);
    st.fy = T(0.5);
    st.lu = T(0);
    st.lv = T(0);
    st.cell = i * g.nx + j;
    st.i = i;
    st.j = j;
    st.back = DIR == kDirBackward;
    T acc = T(0);
    for (int s = 0; s < count; ++s) {
        uint32_t code = 0;
        if (!trace_step<T, FMA, BRANCHLESS, POL, DIR, true, false>(
                st, acc, T(0), g, uv, static_cast<const T*>(nullptr), code))
            return;
        rec(s, st.cell);
    }
}

}  // namespace rlic
