// lic_kernels.cuh -- CUDA kernels of the convolution core and their launchers.
//
// Included by exactly one translation unit per element type
// (lic_kernels_f32.cu, lic_kernels_f64.cu), which instantiate the launchers
// declared in lic_launch.h.
//
// Kernels
//   pack_uv_kernel     u, v -> interleaved (u, v) pairs (one load per step)
//   lic_pass_kernel    one convolution pass (src/lib.rs:364-406): one thread
//                      per pixel, centre tap, forward trace, backward trace;
//                      optionally records every step's code (path cache)
//   lic_gather_kernel  one convolution pass replayed from recorded step codes:
//                      the same cells, weights and accumulation order as the
//                      traced pass, without re-running the streamline
//                      arithmetic (the path of a pixel does not depend on the
//                      texture, src/lib.rs:433-440 reuses u, v every pass)
//   trace_cells_kernel streamline cells of selected pixels (parity checks)
//
// Work distribution: CTAs of block_x x block_y threads own pixel tiles of the
// same shape, numbered row-major.  The traced pass launches one CTA per tile
// (tiles cost unevenly, and the hardware scheduler balances them); the
// replay, whose tiles all cost the same, sizes its grid to the CTAs that fit
// on the device at once and strides over tiles, so its shared-memory set-up
// (weights, delta table) happens once per CTA.  A tile whose streamlines
// cannot reach the border (every pixel farther than klen/2 cells from it)
// takes the interior path without boundary logic.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "lic_device.cuh"
#include "lic_launch.h"

// Minimum resident CTAs per SM requested from the register allocator for the
// traced passes (256-thread CTAs; 8 = full occupancy at 32 registers per
// thread).  1 leaves the allocation to the compiler: the float32 pass is
// bound by instruction issue and gains nothing from more warps.  The float64
// pass waits on FP64 results: 3 CTAs (85 registers, no spills) measured 9%
// faster than the 2 that its 86 unconstrained registers allow.
#ifndef RLIC_PASS_MIN_BLOCKS_F64
#define RLIC_PASS_MIN_BLOCKS_F64 3
#endif
#ifndef RLIC_PASS_MIN_BLOCKS_F32
#define RLIC_PASS_MIN_BLOCKS_F32 1
#endif

namespace rlic {

// Minimum resident CTAs per SM for the float32 / 32-bit-index replay
// kernel's register allocation (8: 32 registers, full occupancy; measured
// fastest at 8192^2: 2.10 ms per replay against 2.11 for 7 and 2.25 for 6).
// Wider types need more registers and keep fewer CTAs.
#ifndef RLIC_GATHER_MIN_BLOCKS
#define RLIC_GATHER_MIN_BLOCKS 8
#endif

template <typename T, typename I> struct PassMinBlocks { static constexpr int value = 1; };

// The paired pass (two threads per pixel, CTAs of at most kPairedMaxThreads
// threads): the float64 form waits on FP64 results and wants every pixel of
// a small image resident at once; 7 CTAs of 128 threads per SM (72
// registers) hold a 256^2 image's 131072 threads in one wave.
constexpr int kPairedMaxThreads = 128;
#ifndef RLIC_PAIRED_MIN_BLOCKS_F64
#define RLIC_PAIRED_MIN_BLOCKS_F64 7
#endif
template <typename T> struct PairedMinBlocks { static constexpr int value = 1; };
template <> struct PairedMinBlocks<double> {
    static constexpr int value = RLIC_PAIRED_MIN_BLOCKS_F64;
};

template <typename T, typename I> struct GatherMinBlocks { static constexpr int value = 4; };
template <> struct GatherMinBlocks<float, int32_t> {
    static constexpr int value = RLIC_GATHER_MIN_BLOCKS;
};
template <> struct GatherMinBlocks<float, int64_t> { static constexpr int value = 6; };
template <typename I> struct PassMinBlocks<float, I> {
    static constexpr int value = RLIC_PASS_MIN_BLOCKS_F32;
};
// (64-bit indices, images beyond 2^31 pixels, need more registers: 1)
template <> struct PassMinBlocks<double, int32_t> {
    static constexpr int value = RLIC_PASS_MIN_BLOCKS_F64;
};

template <typename T>
__global__ void pack_uv_kernel(const T* __restrict__ u, const T* __restrict__ v,
                               typename Vec2<T>::type* __restrict__ uv, int64_t n,
                               unsigned* __restrict__ nan_flag) {
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    bool nan = false;
    for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n; k += stride) {
        typename Vec2<T>::type p;
        p.x = u[k];
        p.y = v[k];
        nan |= isnan(p.x) || isnan(p.y);
        uv[k] = p;
    }
    if (nan && nan_flag) atomicOr(nan_flag, 1u);
}

// Tile bookkeeping shared by the pass and gather kernels.
template <typename I>
struct TileGrid {
    I tiles_x, ntiles;
    int bx, by;
    int radius;  // max cells a streamline can move away from its pixel
    I tile_base; // first tile of this launch (traced passes)
};

template <typename I>
__device__ __forceinline__ bool tile_is_interior(I ti, I tj, const TileGrid<I>& tg,
                                                 const Geometry<I>& g) {
    const I r0 = ti * tg.by, c0 = tj * tg.bx;
    const I r = tg.radius;
    return r0 - r >= 0 && r0 + tg.by - 1 + r <= g.ny - 1 && c0 - r >= 0 &&
           c0 + tg.bx - 1 + r <= g.nx - 1;
}

// Shared-memory layout: forward weights in step order (wf[s] = kernel[kmid+1+s]),
// then backward weights in step order (wb[s] = kernel[kmid-1-s]), each padded
// to a multiple of 8 entries; then (gather only) the 16-entry delta table.
template <typename T>
__device__ __forceinline__ void load_step_weights(T* smem, const T* __restrict__ kernel, int klen,
                                                  int nf_pad) {
    const int kmid = klen / 2;
    const int nf = klen - kmid - 1;
    const int nthreads = blockDim.x * blockDim.y;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    for (int s = tid; s < nf; s += nthreads) smem[s] = kernel[kmid + 1 + s];
    for (int s = tid; s < kmid; s += nthreads) smem[nf_pad + s] = kernel[kmid - 1 - s];
}

// Path-cache word addressing: codes[word * npix + pixel], 8 steps per word,
// forward words first, then backward words (word-major so that a warp's
// 32 consecutive pixels read or write 128 contiguous bytes).
struct CodeLayout {
    int64_t npix;
    int words_f;  // ceil(nf / 8)
};

// What a traced pass does with each step: sample the texture (kSample),
// sample and record the step codes (kSampleRecord), or only record them
// (kRecordOnly, no texture read and no output).
enum PassMode : int { kSample = 0, kSampleRecord = 1, kRecordOnly = 2 };

template <typename T, bool FMA, bool BRANCHLESS, bool POL, bool EDGE, int MODE, typename I,
          bool NAN_CHECK = true, bool NC = true>
__device__ __forceinline__ T convolve_pixel(I i, I j, const Geometry<I>& g,
                                            const typename Vec2<T>::type* __restrict__ uv,
                                            const T* __restrict__ tex, const T* wf, const T* wb,
                                            T wmid, int nf, int kmid, uint32_t* __restrict__ codes,
                                            const CodeLayout& cl) {
    constexpr bool SAMPLE = MODE != kRecordOnly;
    constexpr bool RECORD = MODE != kSample;
    const I p = i * g.nx + j;
    T acc = T(0);
    if constexpr (SAMPLE) acc = accumulate<T, FMA>(wmid, ld_in<NC>(tex + p), T(0));
    uint32_t* words_f = RECORD ? codes + p : nullptr;
    uint32_t* words_b = RECORD ? codes + size_t(cl.words_f) * size_t(cl.npix) + p : nullptr;
    trace_half<T, FMA, BRANCHLESS, POL, kDirForward, EDGE, SAMPLE, RECORD, I, NAN_CHECK, NC>(
        acc, i, j, g, uv, tex, wf, nf, words_f, cl.npix);
    trace_half<T, FMA, BRANCHLESS, POL, kDirBackward, EDGE, SAMPLE, RECORD, I, NAN_CHECK, NC>(
        acc, i, j, g, uv, tex, wb, kmid, words_b, cl.npix);
    return acc;
}

// One convolution pass, one pixel tile per CTA (the hardware balances CTAs of
// uneven cost, e.g. streamlines that stop early).
template <typename T, bool FMA, bool BRANCHLESS, bool POL, int MODE, typename I>
__global__ void __launch_bounds__(256, (PassMinBlocks<T, I>::value))
lic_pass_kernel(const T* __restrict__ tex_in, const typename Vec2<T>::type* __restrict__ uv,
                const T* __restrict__ kernel, int klen, Geometry<I> g, TileGrid<I> tg,
                T* __restrict__ tex_out, uint32_t* __restrict__ codes, CodeLayout cl,
                const unsigned* __restrict__ field_nan) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* wsm = reinterpret_cast<T*>(smem_raw);
    const int kmid = klen / 2;
    const int nf = klen - kmid - 1;
    const int nf_pad = (nf + 7) & ~7;
    if constexpr (MODE != kRecordOnly) {
        load_step_weights(wsm, kernel, klen, nf_pad);
        __syncthreads();
    }
    const T wmid = (MODE != kRecordOnly) ? __ldg(kernel + kmid) : T(0);
    const I tile = tg.tile_base + I(blockIdx.x);
    const I ti = tile / tg.tiles_x;
    const I tj = tile - ti * tg.tiles_x;
    const I i = ti * tg.by + I(threadIdx.y);
    const I j = tj * tg.bx + I(threadIdx.x);
    T acc;
    // a field known to hold no NaN sample spares interior tiles the per-step
    // NaN test (and the stop-code exits of the recording loop)
    const bool nan_free = field_nan != nullptr && __ldg(field_nan) == 0u;
    if (tile_is_interior(ti, tj, tg, g)) {
        if (nan_free) {
            acc = convolve_pixel<T, FMA, BRANCHLESS, POL, false, MODE, I, false>(
                i, j, g, uv, tex_in, wsm, wsm + nf_pad, wmid, nf, kmid, codes, cl);
        } else {
            acc = convolve_pixel<T, FMA, BRANCHLESS, POL, false, MODE, I, true>(
                i, j, g, uv, tex_in, wsm, wsm + nf_pad, wmid, nf, kmid, codes, cl);
        }
    } else if (i < g.ny && j < g.nx) {
        acc = convolve_pixel<T, FMA, BRANCHLESS, POL, true, MODE>(
            i, j, g, uv, tex_in, wsm, wsm + nf_pad, wmid, nf, kmid, codes, cl);
    } else {
        return;
    }
    if constexpr (MODE != kRecordOnly) tex_out[i * g.nx + j] = acc;
}

// Steps of a code word unrolled in the paired pass's loop (8: the whole
// word).  The float64 pass's unrolled steps overflow the instruction cache
// (ncu: warps waiting on instruction fetch); 4 measured 7% faster than 8 on
// a 256^2 image (0.0955 against 0.1031 ms per call), 2 and 1 within 1% of 4.
#ifndef RLIC_PAIRED_UNROLL_F64
#define RLIC_PAIRED_UNROLL_F64 4
#endif
#ifndef RLIC_PAIRED_UNROLL_F32
#define RLIC_PAIRED_UNROLL_F32 8
#endif
template <typename T> struct PairedUnroll { static constexpr int value = RLIC_PAIRED_UNROLL_F32; };
template <> struct PairedUnroll<double> { static constexpr int value = RLIC_PAIRED_UNROLL_F64; };

// One half of a pixel's streamline for the paired pass below: the direction
// is the thread's (st.back); every step's texture sample is accumulated into
// `acc` with this half's weights `w` and, on backward threads, also stored
// at sink[s * sink_stride] for step s.  Records step codes like trace_half.
// Returns the number of steps sampled (count, or the step that met a NaN
// sample and stopped the trace).
template <typename T, bool FMA, bool BRANCHLESS, bool POL, bool EDGE, bool RECORD, typename I,
          bool NAN_CHECK>
__device__ __forceinline__ int trace_paired_half(T& acc, I i, I j, bool back,
                                                 const Geometry<I>& g,
                                                 const typename Vec2<T>::type* __restrict__ uv,
                                                 const T* __restrict__ tex, const T* w,
                                                 int count, uint32_t* __restrict__ words,
                                                 size_t stride, T* sink, int sink_stride) {
    TraceState<T, I> st;
    st.last = kLastNone;
    st.fx = T(0.5);
    st.fy = T(0.5);
    st.lu = T(0);
    st.lv = T(0);
    st.cell = i * g.nx + j;
    st.i = i;
    st.j = j;
    st.back = back;
    for (int q = 0; 8 * q < count; ++q) {
        const int n = count - 8 * q < 8 ? count - 8 * q : 8;
        const T* wq = w + 8 * q;
        uint32_t word = 0;
#pragma unroll(PairedUnroll<T>::value)
        for (int b = 0; b < 8; ++b) {
            if (b < n) {
                uint32_t code = 0;
                T x;
                if (!trace_step<T, FMA, BRANCHLESS, POL, kDirRuntime, EDGE, true, I, NAN_CHECK,
                                true, false>(
                        st, acc, wq[b], g, uv, tex, code, &x)) {
                    if constexpr (RECORD) words[size_t(q) * stride] = word | (kStop << (4 * b));
                    return 8 * q + b;
                }
                if (back) sink[(8 * q + b) * sink_stride] = x;
                word |= code << (4 * b);
            }
        }
        if constexpr (RECORD) words[size_t(q) * stride] = word;
    }
    return count;
}

// One convolution pass with each pixel's two half-streamlines traced by two
// threads of one warp: lanes 0-15 trace the forward halves of 16 pixels,
// lanes 16-31 the backward halves of the same pixels.  On images whose
// tiles cannot fill the GPU this doubles the threads that run the serial
// streamline arithmetic (each thread's chain of steps is half as long).  The
// output keeps the reference's accumulation order (centre tap, forward taps
// ascending, backward taps descending, src/lib.rs:376-403): the forward
// thread accumulates the centre and its own samples as it steps, while the
// backward thread stores its samples in shared memory; the forward thread
// then adds them in step order.  A CTA of 2 * bx * by threads owns a tile of
// bx x by pixels (bx * by a multiple of 16, at most 64); pixel slot
// 16 * warp + (lane & 15) is tile row slot / bx, column slot % bx.
template <typename T, bool FMA, bool BRANCHLESS, bool POL, int MODE, typename I>
__global__ void __launch_bounds__(kPairedMaxThreads, (PairedMinBlocks<T>::value))
lic_pass_paired_kernel(const T* __restrict__ tex_in, const typename Vec2<T>::type* __restrict__ uv,
                       const T* __restrict__ kernel, int klen, Geometry<I> g, TileGrid<I> tg,
                       T* __restrict__ tex_out, uint32_t* __restrict__ codes, CodeLayout cl,
                       const unsigned* __restrict__ field_nan) {
    static_assert(MODE != kRecordOnly, "the paired pass samples the texture");
    constexpr bool RECORD = MODE == kSampleRecord;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* wsm = reinterpret_cast<T*>(smem_raw);
    const int kmid = klen / 2;
    const int nf = klen - kmid - 1;
    const int nf_pad = (nf + 7) & ~7;
    const int nb_pad = (kmid + 7) & ~7;
    const int npx = tg.bx * tg.by;
    T* samples = wsm + nf_pad + nb_pad;  // [kmid][npx]: backward samples by step
    load_step_weights(wsm, kernel, klen, nf_pad);
    __syncthreads();
    const T wmid = __ldg(kernel + kmid);
    const I tile = tg.tile_base + I(blockIdx.x);
    const I ti = tile / tg.tiles_x;
    const I tj = tile - ti * tg.tiles_x;
    const int lane = int(threadIdx.x) & 31;
    const bool back = lane >= 16;
    const int slot = (int(threadIdx.x) >> 5) * 16 + (lane & 15);
    const int r = slot / tg.bx;
    const I i = ti * tg.by + I(r);
    const I j = tj * tg.bx + I(slot - r * tg.bx);
    const bool interior = tile_is_interior(ti, tj, tg, g);
    const bool valid = interior || (i < g.ny && j < g.nx);
    const bool nan_free = field_nan != nullptr && __ldg(field_nan) == 0u;
    const I p = valid ? i * g.nx + j : I(0);
    T acc = T(0);
    int sampled = 0;
    if (valid) {
        acc = accumulate<T, FMA>(wmid, __ldg(tex_in + p), T(0));
        uint32_t* words =
            RECORD ? codes + (back ? size_t(cl.words_f) * size_t(cl.npix) : size_t(0)) + p
                   : nullptr;
        const T* w = back ? wsm + nf_pad : wsm;
        const int count = back ? kmid : nf;
        T* sink = samples + slot;
#define RLIC_PAIRED(EDGE, CHECK)                                                          \
    trace_paired_half<T, FMA, BRANCHLESS, POL, EDGE, RECORD, I, CHECK>(                   \
        acc, i, j, back, g, uv, tex_in, w, count, words, size_t(cl.npix), sink, npx)
        if (interior && nan_free) sampled = RLIC_PAIRED(false, false);
        else if (interior) sampled = RLIC_PAIRED(false, true);
        else sampled = RLIC_PAIRED(true, true);
#undef RLIC_PAIRED
    }
    __syncwarp();
    // the backward partner's sample count (every lane takes part in the shuffle)
    const int nback = __shfl_sync(0xffffffffu, sampled, (lane & 15) + 16);
    if (!valid || back) return;
    const T* wb = wsm + nf_pad;
    for (int s = 0; s < nback; ++s) acc = accumulate<T, FMA>(wb[s], samples[s * npx + slot], acc);
    tex_out[p] = acc;
}

// Replays `count` recorded steps of one half from pixel p.  A word holds 8
// steps.  Words without a stop code (all of them unless the field holds
// NaNs) are gathered branch-free, and one word ahead: the 8 texture loads of
// word q+1 are in flight while the 8 ordered FMAs of word q run, so the
// accumulation order (that of the traced pass) is kept while the load
// latency is hidden.
template <typename T, typename I, bool NC = true>
__device__ __forceinline__ void gather8(I& cell, uint32_t wd, const I* table,
                                        const T* __restrict__ tex, T x[8]) {
#pragma unroll
    for (int b = 0; b < 8; ++b) {
        cell += table[(wd >> (4 * b)) & 15u];
        x[b] = ld_in<NC>(tex + cell);
    }
}

template <typename T, bool FMA, typename I, bool NC = true>
__device__ __forceinline__ void replay_half(T& acc, I p, const uint32_t* __restrict__ words,
                                            int64_t npix, int count, const T* w, const I* table,
                                            const T* __restrict__ tex) {
    I cell = p;
    const int full = count >> 3;
    int q = 0;
    // pipelined run of full words without stop codes
    if (full > 0) {
        uint32_t wd = ld_in<NC>(words);
        if (!word_has_stop(wd)) {
            T x[8];
            gather8<T, I, NC>(cell, wd, table, tex, x);
            for (q = 1; q < full; ++q) {
                wd = ld_in<NC>(words + size_t(q) * size_t(npix));
                if (word_has_stop(wd)) break;
                T y[8];
                gather8<T, I, NC>(cell, wd, table, tex, y);
                const T* wq = w + 8 * (q - 1);
#pragma unroll
                for (int b = 0; b < 8; ++b) acc = accumulate<T, FMA>(wq[b], x[b], acc);
#pragma unroll
                for (int b = 0; b < 8; ++b) x[b] = y[b];
            }
            const T* wq = w + 8 * (q - 1);
#pragma unroll
            for (int b = 0; b < 8; ++b) acc = accumulate<T, FMA>(wq[b], x[b], acc);
        }
    }
    // remaining steps one by one: a word with a stop code, or the last partial word
    for (; q <= full; ++q) {
        const int n = (q < full) ? 8 : (count & 7);
        if (n == 0) break;
        const uint32_t wd = ld_in<NC>(words + size_t(q) * size_t(npix));
        const T* wq = w + 8 * q;
        for (int b = 0; b < n; ++b) {
            const uint32_t code = (wd >> (4 * b)) & 15u;
            if (code == kStop) return;
            cell += table[code];
            acc = accumulate<T, FMA>(wq[b], ld_in<NC>(tex + cell), acc);
        }
    }
}

template <typename T, bool FMA, typename I>
__global__ void __launch_bounds__(256, (GatherMinBlocks<T, I>::value))
lic_gather_kernel(const T* __restrict__ tex_in, const uint32_t* __restrict__ codes,
                  const T* __restrict__ kernel, int klen, Geometry<I> g, TileGrid<I> tg,
                  T* __restrict__ tex_out, CodeLayout cl) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* wsm = reinterpret_cast<T*>(smem_raw);
    const int kmid = klen / 2;
    const int nf = klen - kmid - 1;
    const int nf_pad = (nf + 7) & ~7;
    const int nb_pad = (kmid + 7) & ~7;
    I* table = reinterpret_cast<I*>(smem_raw + sizeof(T) * size_t(nf_pad + nb_pad));
    load_step_weights(wsm, kernel, klen, nf_pad);
    if (threadIdx.x == 0 && threadIdx.y == 0) fill_delta_table(table, g.nx, g.ny);
    __syncthreads();
    const T wmid = __ldg(kernel + kmid);
    const uint32_t* codes_b = codes + size_t(cl.words_f) * size_t(cl.npix);
    for (I tile = blockIdx.x; tile < tg.ntiles; tile += gridDim.x) {
        const I ti = tile / tg.tiles_x;
        const I tj = tile - ti * tg.tiles_x;
        const I i = ti * tg.by + I(threadIdx.y);
        const I j = tj * tg.bx + I(threadIdx.x);
        if (i >= g.ny || j >= g.nx) continue;
        const I p = i * g.nx + j;
        T acc = accumulate<T, FMA>(wmid, __ldg(tex_in + p), T(0));
        replay_half<T, FMA, I>(acc, p, codes + p, cl.npix, nf, wsm, table, tex_in);
        replay_half<T, FMA, I>(acc, p, codes_b + p, cl.npix, kmid, wsm + nf_pad, table, tex_in);
        tex_out[p] = acc;
    }
}

// Cells visited by the streamlines of selected pixels (path parity checks).
template <typename T, bool FMA, bool BRANCHLESS, bool POL>
__global__ void trace_cells_kernel(const typename Vec2<T>::type* __restrict__ uv,
                                   Geometry<int64_t> g, int klen, int64_t npix,
                                   const int64_t* __restrict__ pix, int64_t* __restrict__ cells) {
    const int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    const int steps = klen - 1;
    const int kmid = klen / 2;
    const int nf = klen - kmid - 1;
    int64_t* dst = cells + p * steps;
    for (int s = 0; s < steps; ++s) dst[s] = -1;
    const int64_t lin = pix[p];
    if (lin < 0 || lin >= g.ny * g.nx) return;  // invalid pixel: row stays -1
    const int64_t i = lin / g.nx;
    const int64_t j = lin - i * g.nx;
    walk_half<T, FMA, BRANCHLESS, POL, kDirForward>(i, j, g, uv, nf,
                                              [dst](int s, int64_t c) { dst[s] = c; });
    walk_half<T, FMA, BRANCHLESS, POL, kDirBackward>(i, j, g, uv, kmid,
                                             [dst, nf](int s, int64_t c) { dst[nf + s] = c; });
}

// ------------------------------------------------------------ adjoint pass --
//
// One pass of the convolution is linear in the texture: out = A x with
// A[p, c_k(p)] += kernel[k], c_k(p) the cell that pixel p's streamline samples
// with tap k (c_kmid(p) = p).  Its transpose scatters: y[c_k(p)] += kernel[k]
// * g[p].  Both kernels below walk the recorded step codes from every pixel,
// so they see exactly the cells of the traced pass.

// Calls f(k, cell) for every tap of pixel p, centre first, then the forward
// taps ascending, then the backward taps descending.
template <typename I, typename F>
__device__ __forceinline__ void for_each_tap(I p, const uint32_t* __restrict__ codes,
                                             const CodeLayout& cl, int klen, const I* table,
                                             F f) {
    const int kmid = klen / 2;
    const int nf = klen - kmid - 1;
    f(kmid, p);
    for (int half = 0; half < 2; ++half) {
        const uint32_t* words =
            codes + (half ? size_t(cl.words_f) * size_t(cl.npix) : size_t(0)) + p;
        const int count = half ? kmid : nf;
        I cell = p;
        for (int s = 0; s < count; ++s) {
            const uint32_t wd = __ldg(words + size_t(s >> 3) * size_t(cl.npix));
            const uint32_t code = (wd >> (4 * (s & 7))) & 15u;
            if (code == kStop) break;
            cell += table[code];
            f(half ? kmid - 1 - s : kmid + 1 + s, cell);
        }
    }
}

// y = A^T g (y zeroed by the caller).  One thread per pixel, grid-stride.
template <typename T, typename I>
__global__ void __launch_bounds__(256)
lic_scatter_kernel(const T* __restrict__ g, const uint32_t* __restrict__ codes,
                   const T* __restrict__ kernel, int klen, Geometry<I> geo, CodeLayout cl,
                   T* __restrict__ y) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* w = reinterpret_cast<T*>(smem_raw);
    I* table = reinterpret_cast<I*>(smem_raw + sizeof(T) * size_t((klen + 1) & ~1));
    for (int k = threadIdx.x; k < klen; k += blockDim.x) w[k] = kernel[k];
    if (threadIdx.x == 0) fill_delta_table(table, geo.nx, geo.ny);
    __syncthreads();
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; q < cl.npix; q += stride) {
        const I p = I(q);
        const T gp = g[p];
        for_each_tap(p, codes, cl, klen, table,
                     [&](int k, I cell) { atomicAdd(y + cell, mul_rn(w[k], gp)); });
    }
}

// Sum of v over the warp, added by lane 0 to *addr (shared memory).  Every
// lane of the warp must call it.
template <typename T>
__device__ __forceinline__ void warp_add_to(T* addr, T v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(addr, v);
}

// dw[k] += sum_p g[p] * x[c_k(p)]: the gradient of <g, A x> with respect to
// kernel[k].  The lanes of a warp walk their pixels' taps in step, so every
// tap's 32 products are summed across the warp with shuffles and added to
// the CTA's shared partial sum by one lane (32 lanes adding to one shared
// address would serialise); one global (float64) atomic per tap per CTA.
// A lane past the image or past a stop code contributes zero.
template <typename T, typename I>
__global__ void __launch_bounds__(256)
lic_kernel_grad_kernel(const T* __restrict__ g, const T* __restrict__ x,
                       const uint32_t* __restrict__ codes, int klen, Geometry<I> geo,
                       CodeLayout cl, double* __restrict__ dw) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* acc = reinterpret_cast<T*>(smem_raw);
    I* table = reinterpret_cast<I*>(smem_raw + sizeof(T) * size_t((klen + 1) & ~1));
    for (int k = threadIdx.x; k < klen; k += blockDim.x) acc[k] = T(0);
    if (threadIdx.x == 0) fill_delta_table(table, geo.nx, geo.ny);
    __syncthreads();
    const int kmid = klen / 2;
    const int nf = klen - kmid - 1;
    const int lane = threadIdx.x & 31;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    // the loop bound is the warp's first pixel, so the whole warp iterates
    for (int64_t q0 = int64_t(blockIdx.x) * blockDim.x + (threadIdx.x & ~31); q0 < cl.npix;
         q0 += stride) {
        const int64_t q = q0 + lane;
        const bool active = q < cl.npix;
        const I p = active ? I(q) : I(0);
        const T gp = active ? g[p] : T(0);
        warp_add_to(acc + kmid, active ? mul_rn(gp, __ldg(x + p)) : T(0));
        for (int half = 0; half < 2; ++half) {
            const uint32_t* words =
                codes + (half ? size_t(cl.words_f) * size_t(cl.npix) : size_t(0)) + p;
            const int count = half ? kmid : nf;
            I cell = p;
            bool stopped = !active;
            for (int s = 0; s < count; ++s) {
                const uint32_t wd = __ldg(words + size_t(s >> 3) * size_t(cl.npix));
                const uint32_t code = (wd >> (4 * (s & 7))) & 15u;
                stopped = stopped || code == kStop;
                if (!stopped) cell += table[code];
                const T v = stopped ? T(0) : mul_rn(gp, __ldg(x + cell));
                warp_add_to(acc + (half ? kmid - 1 - s : kmid + 1 + s), v);
            }
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < klen; k += blockDim.x) atomicAdd(dw + k, double(acc[k]));
}

// ------------------------------------------------------- strided inputs --
//
// Inputs given as strided views (element strides, possibly zero or
// negative: numpy broadcasts, transposes, reversed or sliced arrays) are read
// in place, from device memory or, on devices with pageable-memory access,
// from the caller's host memory.  A zero stride re-reads the same elements,
// which then come from cache.

// ------------------------------------------------ host-memory uploads --
//
// Kernels that read the caller's host arrays in place (pageable-memory
// access over NVLink-C2C).  Those reads are latency-bound: a small grid with
// several independent loads per thread in flight reaches the link's
// bandwidth, and leaves the other SMs to the traced pass that runs on the
// rows already uploaded.  RLIC_UPLOAD_CTAS bounds the grid; every thread
// keeps kUploadUnroll loads in flight.

#ifndef RLIC_UPLOAD_CTAS
#define RLIC_UPLOAD_CTAS 32
#endif
constexpr int kUploadUnroll = 8;

// dst[i * nx + j] = src[i * s0 + j * s1]; with neg_flag, also sets *neg_flag
// when an element is below zero (NaN and -0.0 are not: the test of numpy's
// `np.any(texture < 0)`, src/rlic/_lib.py:174), so the texture's check needs
// no pass of its own.
template <typename T>
__global__ void gather_strided_kernel(const T* __restrict__ src, int64_t s0, int64_t s1,
                                      T* __restrict__ dst, int64_t ny, int64_t nx,
                                      unsigned* __restrict__ neg_flag) {
    const int64_t span = int64_t(blockDim.x) * kUploadUnroll;
    bool neg = false;
    for (int64_t i = blockIdx.y; i < ny; i += gridDim.y) {
        for (int64_t j0 = int64_t(blockIdx.x) * span + threadIdx.x; j0 < nx;
             j0 += int64_t(gridDim.x) * span) {
            T r[kUploadUnroll];
#pragma unroll
            for (int k = 0; k < kUploadUnroll; ++k) {
                const int64_t j = j0 + int64_t(k) * blockDim.x;
                if (j < nx) r[k] = src[i * s0 + j * s1];
            }
#pragma unroll
            for (int k = 0; k < kUploadUnroll; ++k) {
                const int64_t j = j0 + int64_t(k) * blockDim.x;
                if (j < nx) {
                    neg |= r[k] < T(0);
                    dst[i * nx + j] = r[k];
                }
            }
        }
    }
    if (neg && neg_flag) atomicOr(neg_flag, 1u);
}

// uv[i * nx + j] = (u[i * su0 + j * su1], v[i * sv0 + j * sv1])
template <typename T>
__global__ void pack_uv_strided_kernel(const T* __restrict__ u, int64_t su0, int64_t su1,
                                       const T* __restrict__ v, int64_t sv0, int64_t sv1,
                                       typename Vec2<T>::type* __restrict__ uv, int64_t ny,
                                       int64_t nx, unsigned* __restrict__ nan_flag) {
    constexpr int U = kUploadUnroll / 2;  // two loads per element
    const int64_t span = int64_t(blockDim.x) * U;
    bool nan = false;
    for (int64_t i = blockIdx.y; i < ny; i += gridDim.y) {
        for (int64_t j0 = int64_t(blockIdx.x) * span + threadIdx.x; j0 < nx;
             j0 += int64_t(gridDim.x) * span) {
            typename Vec2<T>::type r[U];
#pragma unroll
            for (int k = 0; k < U; ++k) {
                const int64_t j = j0 + int64_t(k) * blockDim.x;
                if (j < nx) {
                    r[k].x = u[i * su0 + j * su1];
                    r[k].y = v[i * sv0 + j * sv1];
                }
            }
#pragma unroll
            for (int k = 0; k < U; ++k) {
                const int64_t j = j0 + int64_t(k) * blockDim.x;
                if (j < nx) {
                    nan |= isnan(r[k].x) || isnan(r[k].y);
                    uv[i * nx + j] = r[k];
                }
            }
        }
    }
    if (nan && nan_flag) atomicOr(nan_flag, 1u);
}

// Whether an element of a 16-byte vector of T is below zero (NaN and -0.0
// are not).
template <typename T>
__device__ __forceinline__ bool negative_in(uint4 w) {
    if constexpr (sizeof(T) == 4) {
        return (__uint_as_float(w.x) < 0.f) | (__uint_as_float(w.y) < 0.f) |
               (__uint_as_float(w.z) < 0.f) | (__uint_as_float(w.w) < 0.f);
    } else {
        const double a = __longlong_as_double(static_cast<long long>(uint64_t(w.y) << 32 | w.x));
        const double b = __longlong_as_double(static_cast<long long>(uint64_t(w.w) << 32 | w.z));
        return (a < 0.0) | (b < 0.0);
    }
}

// Contiguous rows with 16-byte aligned starts: plain 16-byte vector copies of
// elements of type T; with neg_flag, as gather_strided_kernel.
template <typename T>
__global__ void copy_vec16_kernel(const uint4* __restrict__ src, uint4* __restrict__ dst,
                                  int64_t nvec, unsigned* __restrict__ neg_flag) {
    const int64_t span = int64_t(blockDim.x) * kUploadUnroll;
    bool neg = false;
    for (int64_t b = int64_t(blockIdx.x) * span + threadIdx.x; b < nvec;
         b += int64_t(gridDim.x) * span) {
        uint4 r[kUploadUnroll];
#pragma unroll
        for (int k = 0; k < kUploadUnroll; ++k) {
            const int64_t q = b + int64_t(k) * blockDim.x;
            if (q < nvec) r[k] = src[q];
        }
#pragma unroll
        for (int k = 0; k < kUploadUnroll; ++k) {
            const int64_t q = b + int64_t(k) * blockDim.x;
            if (q < nvec) {
                neg |= negative_in<T>(r[k]);
                dst[q] = r[k];
            }
        }
    }
    if (neg && neg_flag) atomicOr(neg_flag, 1u);
}

// Contiguous u, v with 16-byte aligned rows: 16-byte vectors of u and of v
// interleaved into two 16-byte vectors of (u, v) pairs.  ELEM_WORDS is the
// element size in 32-bit words (1: float, 2: double).
// A NaN has all exponent bits set and a nonzero fraction.
__device__ __forceinline__ bool nan_in(uint4 w, int elem_words) {
    if (elem_words == 1) {
        return ((w.x & 0x7FFFFFFFu) > 0x7F800000u) || ((w.y & 0x7FFFFFFFu) > 0x7F800000u) ||
               ((w.z & 0x7FFFFFFFu) > 0x7F800000u) || ((w.w & 0x7FFFFFFFu) > 0x7F800000u);
    }
    const uint64_t a = (uint64_t(w.y) << 32 | w.x) & 0x7FFFFFFFFFFFFFFFull;
    const uint64_t b = (uint64_t(w.w) << 32 | w.z) & 0x7FFFFFFFFFFFFFFFull;
    return a > 0x7FF0000000000000ull || b > 0x7FF0000000000000ull;
}

template <int ELEM_WORDS>
__global__ void pack_vec16_kernel(const uint4* __restrict__ u, const uint4* __restrict__ v,
                                  uint4* __restrict__ uv, int64_t nvec,
                                  unsigned* __restrict__ nan_flag) {
    constexpr int U = kUploadUnroll / 2;
    const int64_t span = int64_t(blockDim.x) * U;
    bool nan = false;
    for (int64_t b = int64_t(blockIdx.x) * span + threadIdx.x; b < nvec;
         b += int64_t(gridDim.x) * span) {
        uint4 a[U], c[U];
#pragma unroll
        for (int k = 0; k < U; ++k) {
            const int64_t q = b + int64_t(k) * blockDim.x;
            if (q < nvec) {
                a[k] = u[q];
                c[k] = v[q];
            }
        }
#pragma unroll
        for (int k = 0; k < U; ++k) {
            const int64_t q = b + int64_t(k) * blockDim.x;
            if (q < nvec) {
                nan |= nan_in(a[k], ELEM_WORDS) || nan_in(c[k], ELEM_WORDS);
                if constexpr (ELEM_WORDS == 1) {
                    uv[2 * q] = make_uint4(a[k].x, c[k].x, a[k].y, c[k].y);
                    uv[2 * q + 1] = make_uint4(a[k].z, c[k].z, a[k].w, c[k].w);
                } else {
                    uv[2 * q] = make_uint4(a[k].x, a[k].y, c[k].x, c[k].y);
                    uv[2 * q + 1] = make_uint4(a[k].z, a[k].w, c[k].z, c[k].w);
                }
            }
        }
    }
    if (nan && nan_flag) atomicOr(nan_flag, 1u);
}

// Grid of an upload over ny rows of nx elements, `per_thread` elements per
// thread per round, at most RLIC_UPLOAD_CTAS CTAs of 256 threads.
inline dim3 upload_grid(int64_t ny, int64_t nx, int per_thread) {
    const int64_t span = 256 * int64_t(per_thread);
    int64_t gx = (nx + span - 1) / span;
    gx = gx < 1 ? 1 : (gx > RLIC_UPLOAD_CTAS ? RLIC_UPLOAD_CTAS : gx);
    int64_t gy = RLIC_UPLOAD_CTAS / gx;
    gy = gy < 1 ? 1 : (gy > ny ? ny : gy);
    return dim3(unsigned(gx), unsigned(gy < 1 ? 1 : gy));
}

inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// --------------------------------------------------------- input checks --

// Sets *flag when some element of x is below zero (NaN is not: the same test
// as numpy's `np.any(texture < 0)`, src/rlic/_lib.py:174).
template <typename T>
__global__ void check_negative_kernel(const T* __restrict__ x, int64_t n,
                                      unsigned* __restrict__ flag) {
    bool neg = false;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n; k += stride)
        neg |= x[k] < T(0);
    if (__any_sync(0xffffffffu, neg) && (threadIdx.x & 31) == 0) atomicOr(flag, 1u);
}

// ------------------------------------------------ reduced-precision helpers --

// Float copy of the kernel, 1/sum(|kernel|) as used by the reduced-precision
// replays, and the factor that undoes `iterations` of those normalisations
// (computed from the float factor actually applied).  One CTA of 256 threads.
template <typename T>
__global__ void lowp_prepare_kernel(const T* __restrict__ kernel, int klen, int64_t iterations,
                                    float* __restrict__ w32, float* __restrict__ inv_scale,
                                    double* __restrict__ undo) {
    __shared__ double part[256];
    double s = 0.0;
    for (int k = threadIdx.x; k < klen; k += blockDim.x) {
        w32[k] = float(kernel[k]);
        s += fabs(double(kernel[k]));
    }
    part[threadIdx.x] = s;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if (int(threadIdx.x) < h) part[threadIdx.x] += part[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double total = part[0];
        if (!(total > 0.0) || !isfinite(total)) total = 1.0;
        const float inv = float(1.0 / total);
        inv_scale[0] = inv;
        undo[0] = pow(1.0 / double(inv), double(iterations));
    }
}

__device__ __forceinline__ __half to_half(float x) { return __float2half_rn(x); }
__device__ __forceinline__ __half to_half(double x) { return __double2half(x); }
__device__ __forceinline__ __nv_bfloat16 to_bf16(float x) { return __float2bfloat16_rn(x); }
__device__ __forceinline__ __nv_bfloat16 to_bf16(double x) { return __double2bfloat16(x); }

template <typename T>
__global__ void to_storage_kernel(const T* __restrict__ src, void* __restrict__ dst, int storage,
                                  int64_t n) {
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n; k += stride) {
        if (storage == kStorageFP16)
            static_cast<__half*>(dst)[k] = to_half(src[k]);
        else
            static_cast<__nv_bfloat16*>(dst)[k] = to_bf16(src[k]);
    }
}

template <typename T>
__global__ void from_storage_kernel(const void* __restrict__ src, int storage,
                                    const double* __restrict__ undo, T* __restrict__ dst,
                                    int64_t n) {
    const double f = *undo;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n; k += stride) {
        const float x = (storage == kStorageFP16)
                            ? __half2float(static_cast<const __half*>(src)[k])
                            : __bfloat162float(static_cast<const __nv_bfloat16*>(src)[k]);
        dst[k] = T(double(x) * f);
    }
}

// ---------------------------------------------------------------- launchers --

inline int64_t tiles_of(int64_t n, int b) { return (n + b - 1) / b; }

template <typename I>
Geometry<I> make_geometry(const Shape& sh) {
    Geometry<I> g;
    g.ny = I(sh.ny);
    g.nx = I(sh.nx);
    g.ax = make_axis<I>(I(sh.nx), sh.bnd[0], sh.bnd[1]);
    g.ay = make_axis<I>(I(sh.ny), sh.bnd[2], sh.bnd[3]);
    return g;
}

template <typename I>
TileGrid<I> make_tiles(const Shape& sh, const LaunchConfig& lc, int klen) {
    TileGrid<I> tg;
    tg.bx = lc.block_x;
    tg.by = lc.block_y;
    tg.tiles_x = I(tiles_of(sh.nx, lc.block_x));
    tg.ntiles = tg.tiles_x * I(tiles_of(sh.ny, lc.block_y));
    tg.radius = klen / 2;
    tg.tile_base = I(lc.tile_begin);
    return tg;
}

inline CodeLayout make_code_layout(const Shape& sh, int klen) {
    CodeLayout cl;
    cl.npix = sh.ny * sh.nx;
    const int nf = klen - klen / 2 - 1;
    cl.words_f = (nf + 7) / 8;
    return cl;
}

inline size_t weights_smem_bytes(int klen, size_t elem) {
    const int kmid = klen / 2;
    const int nf = klen - kmid - 1;
    return elem * size_t(((nf + 7) & ~7) + ((kmid + 7) & ~7));
}

// Grid size for a persistent-stride kernel: CTAs resident at once, capped by
// the number of tiles.
template <typename K>
cudaError_t persistent_grid(K kernel, int threads, size_t smem, int64_t ntiles,
                            unsigned* grid) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    if (smem > 48 * 1024) {
        e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e != cudaSuccess) return e;
    }
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    int64_t g = int64_t(sms) * per_sm;
    if (g > ntiles) g = ntiles;
    if (g < 1) g = 1;
    *grid = unsigned(g);
    return cudaSuccess;
}

template <typename T>
cudaError_t launch_pack_t(const T* u, const T* v, void* uv, int64_t n, cudaStream_t stream,
                          unsigned* nan_flag) {
    int64_t blocks = (n + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (blocks < 1) blocks = 1;
    pack_uv_kernel<T><<<unsigned(blocks), 256, 0, stream>>>(
        u, v, static_cast<typename Vec2<T>::type*>(uv), n, nan_flag);
    count_launch();
    return cudaGetLastError();
}

// The paired pass's shared memory holds the step weights, then kmid
// backward samples of each of the tile's pixels (paired_smem_bytes in
// lic_launch.h); paired_launch_fits says when a launch takes that form.
static_assert(kPairedMaxThreads == kPairedMaxThreadsHost, "paired CTA limit");

inline bool paired_fits(const Shape& sh, const LaunchConfig& lc, int klen, size_t elem) {
    return paired_launch_fits(sh.ny * sh.nx, lc.block_x, lc.block_y, klen, elem);
}

template <typename T, bool FMA, bool BRANCHLESS, bool POL, int MODE>
cudaError_t launch_paired_t(const T* tex_in, const void* uv, const T* kernel, int klen,
                            const Shape& sh, const LaunchConfig& lc, T* tex_out, uint32_t* codes,
                            cudaStream_t stream) {
    const auto g = make_geometry<int32_t>(sh);
    const auto tg = make_tiles<int32_t>(sh, lc, klen);
    const auto cl = make_code_layout(sh, klen);
    const int npx = lc.block_x * lc.block_y;
    const size_t smem = paired_smem_bytes(klen, npx, sizeof(T));
    auto kfn = lic_pass_paired_kernel<T, FMA, BRANCHLESS, POL, MODE, int32_t>;
    if (smem > 48 * 1024) {
        cudaError_t e =
            cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e != cudaSuccess) return e;
    }
    const int64_t count = lc.tile_count ? lc.tile_count : int64_t(tg.ntiles) - lc.tile_begin;
    if (count <= 0) return cudaSuccess;
    kfn<<<unsigned(count), unsigned(2 * npx), smem, stream>>>(
        tex_in, static_cast<const typename Vec2<T>::type*>(uv), kernel, klen, g, tg, tex_out,
        codes, cl, lc.field_nan);
    count_launch();
    return cudaGetLastError();
}

template <typename T, int MODE>
cudaError_t launch_paired_m(const Variant& var, const T* tex_in, const void* uv, const T* kernel,
                            int klen, const Shape& sh, const LaunchConfig& lc, T* tex_out,
                            uint32_t* codes, cudaStream_t stream) {
    const int code = (var.fma ? 4 : 0) | (var.branchless ? 2 : 0) | (var.pol ? 1 : 0);
#define RLIC_PAIRED_CASE(C, F, B, P)                                                        \
    case C:                                                                                 \
        return launch_paired_t<T, F, B, P, MODE>(tex_in, uv, kernel, klen, sh, lc, tex_out, \
                                                 codes, stream);
    switch (code) {
        RLIC_PAIRED_CASE(0, false, false, false)
        RLIC_PAIRED_CASE(1, false, false, true)
        RLIC_PAIRED_CASE(2, false, true, false)
        RLIC_PAIRED_CASE(3, false, true, true)
        RLIC_PAIRED_CASE(4, true, false, false)
        RLIC_PAIRED_CASE(5, true, false, true)
        RLIC_PAIRED_CASE(6, true, true, false)
        RLIC_PAIRED_CASE(7, true, true, true)
    }
#undef RLIC_PAIRED_CASE
    return cudaErrorInvalidValue;
}

template <typename T, bool FMA, bool BRANCHLESS, bool POL, int MODE, typename I>
cudaError_t launch_pass_t(const T* tex_in, const void* uv, const T* kernel, int klen,
                          const Shape& sh, const LaunchConfig& lc, T* tex_out, uint32_t* codes,
                          cudaStream_t stream) {
    const auto g = make_geometry<I>(sh);
    const auto tg = make_tiles<I>(sh, lc, klen);
    const auto cl = make_code_layout(sh, klen);
    const size_t smem = (MODE == kRecordOnly) ? 0 : weights_smem_bytes(klen, sizeof(T));
    if (int64_t(tg.ntiles) > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
    auto kfn = lic_pass_kernel<T, FMA, BRANCHLESS, POL, MODE, I>;
    if (smem > 48 * 1024) {
        cudaError_t e =
            cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e != cudaSuccess) return e;
    }
    const int64_t count = lc.tile_count ? lc.tile_count : int64_t(tg.ntiles) - lc.tile_begin;
    if (count <= 0) return cudaSuccess;
    kfn<<<unsigned(count), dim3(lc.block_x, lc.block_y), smem, stream>>>(
        tex_in, static_cast<const typename Vec2<T>::type*>(uv), kernel, klen, g, tg, tex_out,
        codes, cl, lc.field_nan);
    count_launch();
    return cudaGetLastError();
}

template <typename T, int MODE, typename I>
cudaError_t launch_pass_m(const Variant& var, const T* tex_in, const void* uv, const T* kernel,
                          int klen, const Shape& sh, const LaunchConfig& lc, T* tex_out,
                          uint32_t* codes, cudaStream_t stream) {
    const int code = (var.fma ? 4 : 0) | (var.branchless ? 2 : 0) | (var.pol ? 1 : 0);
#define RLIC_PASS_CASE(C, F, B, P)                                                          \
    case C:                                                                                 \
        return launch_pass_t<T, F, B, P, MODE, I>(tex_in, uv, kernel, klen, sh, lc, tex_out, \
                                                  codes, stream);
    switch (code) {
        RLIC_PASS_CASE(0, false, false, false)
        RLIC_PASS_CASE(1, false, false, true)
        RLIC_PASS_CASE(2, false, true, false)
        RLIC_PASS_CASE(3, false, true, true)
        RLIC_PASS_CASE(4, true, false, false)
        RLIC_PASS_CASE(5, true, false, true)
        RLIC_PASS_CASE(6, true, true, false)
        RLIC_PASS_CASE(7, true, true, true)
    }
#undef RLIC_PASS_CASE
    return cudaErrorInvalidValue;
}

template <typename T, typename I>
cudaError_t launch_pass_i(const Variant& var, int mode, const T* tex_in, const void* uv,
                          const T* kernel, int klen, const Shape& sh, const LaunchConfig& lc,
                          T* tex_out, uint32_t* codes, cudaStream_t stream) {
    if (lc.paired && mode != kRecordOnly && paired_fits(sh, lc, klen, sizeof(T))) {
        return mode == kSample
                   ? launch_paired_m<T, kSample>(var, tex_in, uv, kernel, klen, sh, lc, tex_out,
                                                 codes, stream)
                   : launch_paired_m<T, kSampleRecord>(var, tex_in, uv, kernel, klen, sh, lc,
                                                       tex_out, codes, stream);
    }
    switch (mode) {
        case kSample:
            return launch_pass_m<T, kSample, I>(var, tex_in, uv, kernel, klen, sh, lc, tex_out,
                                                codes, stream);
        case kSampleRecord:
            return launch_pass_m<T, kSampleRecord, I>(var, tex_in, uv, kernel, klen, sh, lc,
                                                      tex_out, codes, stream);
        case kRecordOnly:
            return launch_pass_m<T, kRecordOnly, I>(var, tex_in, uv, kernel, klen, sh, lc,
                                                    tex_out, codes, stream);
    }
    return cudaErrorInvalidValue;
}

template <typename T, bool FMA, typename I>
cudaError_t launch_gather_t(const T* tex_in, const uint32_t* codes, const T* kernel, int klen,
                            const Shape& sh, const LaunchConfig& lc, T* tex_out,
                            cudaStream_t stream) {
    const auto g = make_geometry<I>(sh);
    const auto cl = make_code_layout(sh, klen);
    const auto tg = make_tiles<I>(sh, lc, klen);
    const size_t smem = weights_smem_bytes(klen, sizeof(T)) + 16 * sizeof(I);
    auto kfn = lic_gather_kernel<T, FMA, I>;
    unsigned grid = 0;
    cudaError_t e = persistent_grid(kfn, lc.block_x * lc.block_y, smem, int64_t(tg.ntiles), &grid);
    if (e != cudaSuccess) return e;
    kfn<<<grid, dim3(lc.block_x, lc.block_y), smem, stream>>>(tex_in, codes, kernel, klen, g, tg,
                                                              tex_out, cl);
    count_launch();
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_trace_cells_t(const Variant& var, const void* uv, const Shape& sh, int klen,
                                 int64_t npix, const int64_t* pix, int64_t* cells,
                                 cudaStream_t stream) {
    const auto g = make_geometry<int64_t>(sh);
    const auto* p = static_cast<const typename Vec2<T>::type*>(uv);
    const unsigned blocks = unsigned((npix + 127) / 128);
    const int code = (var.fma ? 4 : 0) | (var.branchless ? 2 : 0) | (var.pol ? 1 : 0);
#define RLIC_TRACE_CASE(C, F, B, P)                                                       \
    case C:                                                                               \
        trace_cells_kernel<T, F, B, P><<<blocks, 128, 0, stream>>>(p, g, klen, npix, pix, \
                                                                   cells);                \
        break;
    switch (code) {
        RLIC_TRACE_CASE(0, false, false, false)
        RLIC_TRACE_CASE(1, false, false, true)
        RLIC_TRACE_CASE(2, false, true, false)
        RLIC_TRACE_CASE(3, false, true, true)
        RLIC_TRACE_CASE(4, true, false, false)
        RLIC_TRACE_CASE(5, true, false, true)
        RLIC_TRACE_CASE(6, true, true, false)
        RLIC_TRACE_CASE(7, true, true, true)
    }
#undef RLIC_TRACE_CASE
    count_launch();
    return cudaGetLastError();
}

inline unsigned stream_blocks(int64_t n) {
    int64_t blocks = (n + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    return unsigned(blocks < 1 ? 1 : blocks);
}

// Rows [0, ny) of strided u, v into the packed field.  Contiguous rows with
// 16-byte aligned starts take the vector kernel.
template <typename T>
cudaError_t launch_pack_strided_t(const T* u, int64_t su0, int64_t su1, const T* v, int64_t sv0,
                                  int64_t sv1, void* uv, int64_t ny, int64_t nx,
                                  cudaStream_t stream, unsigned* nan_flag) {
    const int64_t per_vec = 16 / int64_t(sizeof(T));
    if (su1 == 1 && sv1 == 1 && su0 == nx && sv0 == nx && nx % per_vec == 0 && aligned16(u) &&
        aligned16(v) && aligned16(uv)) {
        const int64_t nvec = ny * nx / per_vec;
        const dim3 grid = upload_grid(1, nvec, kUploadUnroll / 2);
        pack_vec16_kernel<int(sizeof(T) / 4)><<<grid.x, 256, 0, stream>>>(
            reinterpret_cast<const uint4*>(u), reinterpret_cast<const uint4*>(v),
            static_cast<uint4*>(uv), nvec, nan_flag);
    } else {
        pack_uv_strided_kernel<T><<<upload_grid(ny, nx, kUploadUnroll / 2), 256, 0, stream>>>(
            u, su0, su1, v, sv0, sv1, static_cast<typename Vec2<T>::type*>(uv), ny, nx, nan_flag);
    }
    count_launch();
    return cudaGetLastError();
}

// Rows [0, ny) of a strided array into a contiguous one.
template <typename T>
cudaError_t launch_gather_strided_t(const T* src, int64_t s0, int64_t s1, T* dst, int64_t ny,
                                    int64_t nx, cudaStream_t stream, unsigned* neg_flag) {
    const int64_t per_vec = 16 / int64_t(sizeof(T));
    if (s1 == 1 && s0 == nx && nx % per_vec == 0 && aligned16(src) && aligned16(dst)) {
        const int64_t nvec = ny * nx / per_vec;
        const dim3 grid = upload_grid(1, nvec, kUploadUnroll);
        copy_vec16_kernel<T><<<grid.x, 256, 0, stream>>>(
            reinterpret_cast<const uint4*>(src), reinterpret_cast<uint4*>(dst), nvec, neg_flag);
    } else {
        gather_strided_kernel<T><<<upload_grid(ny, nx, kUploadUnroll), 256, 0, stream>>>(
            src, s0, s1, dst, ny, nx, neg_flag);
    }
    count_launch();
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_check_negative_t(const T* x, int64_t n, unsigned* flag, cudaStream_t stream) {
    // whole warps only: every lane of a launched warp reaches the vote
    check_negative_kernel<T><<<stream_blocks(n), 256, 0, stream>>>(x, n, flag);
    count_launch();
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_lowp_prepare_t(const T* kernel, int klen, int64_t iterations, float* w32,
                                  float* inv_scale, double* undo, cudaStream_t stream) {
    lowp_prepare_kernel<T><<<1, 256, 0, stream>>>(kernel, klen, iterations, w32, inv_scale, undo);
    count_launch();
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_to_storage_t(const T* src, void* dst, int storage, int64_t n,
                                cudaStream_t stream) {
    to_storage_kernel<T><<<stream_blocks(n), 256, 0, stream>>>(src, dst, storage, n);
    count_launch();
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_from_storage_t(const void* src, int storage, const double* undo, T* dst,
                                  int64_t n, cudaStream_t stream) {
    from_storage_kernel<T><<<stream_blocks(n), 256, 0, stream>>>(src, storage, undo, dst, n);
    count_launch();
    return cudaGetLastError();
}

inline unsigned pixel_blocks(int64_t npix) {
    int64_t blocks = (npix + 255) / 256;
    if (blocks > 152 * 8) blocks = 152 * 8;
    return unsigned(blocks < 1 ? 1 : blocks);
}

template <typename T, typename I>
cudaError_t launch_scatter_t(const T* g, const uint32_t* codes, const T* kernel, int klen,
                             const Shape& sh, T* y, cudaStream_t stream) {
    const auto geo = make_geometry<I>(sh);
    const auto cl = make_code_layout(sh, klen);
    const size_t smem = sizeof(T) * size_t((klen + 1) & ~1) + 16 * sizeof(I);
    auto kfn = lic_scatter_kernel<T, I>;
    if (smem > 48 * 1024) {
        cudaError_t e =
            cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e != cudaSuccess) return e;
    }
    cudaError_t e = cudaMemsetAsync(y, 0, size_t(cl.npix) * sizeof(T), stream);
    if (e != cudaSuccess) return e;
    kfn<<<pixel_blocks(cl.npix), 256, smem, stream>>>(g, codes, kernel, klen, geo, cl, y);
    count_launch();
    return cudaGetLastError();
}

template <typename T, typename I>
cudaError_t launch_kernel_grad_t(const T* g, const T* x, const uint32_t* codes, int klen,
                                 const Shape& sh, double* dw, cudaStream_t stream) {
    const auto geo = make_geometry<I>(sh);
    const auto cl = make_code_layout(sh, klen);
    const size_t smem = sizeof(T) * size_t((klen + 1) & ~1) + 16 * sizeof(I);
    auto kfn = lic_kernel_grad_kernel<T, I>;
    if (smem > 48 * 1024) {
        cudaError_t e =
            cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
        if (e != cudaSuccess) return e;
    }
    kfn<<<pixel_blocks(cl.npix), 256, smem, stream>>>(g, x, codes, klen, geo, cl, dw);
    count_launch();
    return cudaGetLastError();
}

// Definitions of the per-type overloads declared in lic_launch.h.
#define RLIC_DEFINE_LAUNCHERS(T)                                                             \
    cudaError_t launch_pack(const T* u, const T* v, void* uv, int64_t n, cudaStream_t stream, \
                            unsigned* nan_flag) {                                            \
        return launch_pack_t<T>(u, v, uv, n, stream, nan_flag);                              \
    }                                                                                        \
    cudaError_t launch_pass(const Variant& var, int mode, const T* tex_in, const void* uv,    \
                            const T* kernel, int klen, const Shape& sh,                      \
                            const LaunchConfig& lc, T* tex_out, uint32_t* codes,             \
                            cudaStream_t stream) {                                           \
        if (sh.small_index())                                                                \
            return launch_pass_i<T, int32_t>(var, mode, tex_in, uv, kernel, klen, sh, lc,    \
                                             tex_out, codes, stream);                        \
        return launch_pass_i<T, int64_t>(var, mode, tex_in, uv, kernel, klen, sh, lc,        \
                                         tex_out, codes, stream);                            \
    }                                                                                        \
    cudaError_t launch_gather(bool fma, const T* tex_in, const uint32_t* codes,              \
                              const T* kernel, int klen, const Shape& sh,                    \
                              const LaunchConfig& lc, T* tex_out, cudaStream_t stream) {     \
        if (sh.small_index())                                                                \
            return fma ? launch_gather_t<T, true, int32_t>(tex_in, codes, kernel, klen, sh,  \
                                                           lc, tex_out, stream)              \
                       : launch_gather_t<T, false, int32_t>(tex_in, codes, kernel, klen, sh, \
                                                            lc, tex_out, stream);            \
        return fma ? launch_gather_t<T, true, int64_t>(tex_in, codes, kernel, klen, sh, lc,  \
                                                       tex_out, stream)                      \
                   : launch_gather_t<T, false, int64_t>(tex_in, codes, kernel, klen, sh, lc, \
                                                        tex_out, stream);                    \
    }                                                                                        \
    cudaError_t launch_trace_cells(const Variant& var, const T* /*type tag*/, const void* uv, \
                                   const Shape& sh, int klen, int64_t npix,                  \
                                   const int64_t* pix, int64_t* cells, cudaStream_t stream) { \
        return launch_trace_cells_t<T>(var, uv, sh, klen, npix, pix, cells, stream);         \
    }                                                                                        \
    cudaError_t launch_lowp_prepare(const T* kernel, int klen, int64_t iterations,           \
                                    float* w32, float* inv_scale, double* undo,              \
                                    cudaStream_t stream) {                                   \
        return launch_lowp_prepare_t<T>(kernel, klen, iterations, w32, inv_scale, undo,      \
                                        stream);                                             \
    }                                                                                        \
    cudaError_t launch_to_storage(const T* src, void* dst, int storage, int64_t n,           \
                                  cudaStream_t stream) {                                     \
        return launch_to_storage_t<T>(src, dst, storage, n, stream);                         \
    }                                                                                        \
    cudaError_t launch_from_storage(const void* src, int storage, const double* undo, T* dst, \
                                    int64_t n, cudaStream_t stream) {                        \
        return launch_from_storage_t<T>(src, storage, undo, dst, n, stream);                 \
    }                                                                                        \
    cudaError_t launch_check_negative(const T* x, int64_t n, unsigned* flag,                 \
                                      cudaStream_t stream) {                                 \
        return launch_check_negative_t<T>(x, n, flag, stream);                               \
    }                                                                                        \
    cudaError_t launch_pack_strided(const T* u, int64_t su0, int64_t su1, const T* v,        \
                                    int64_t sv0, int64_t sv1, void* uv, int64_t ny,          \
                                    int64_t nx, cudaStream_t stream, unsigned* nan_flag) {   \
        return launch_pack_strided_t<T>(u, su0, su1, v, sv0, sv1, uv, ny, nx, stream,        \
                                        nan_flag);                                           \
    }                                                                                        \
    cudaError_t launch_gather_strided(const T* src, int64_t s0, int64_t s1, T* dst,          \
                                      int64_t ny, int64_t nx, cudaStream_t stream,           \
                                      unsigned* neg_flag) {                                  \
        return launch_gather_strided_t<T>(src, s0, s1, dst, ny, nx, stream, neg_flag);       \
    }                                                                                        \
    cudaError_t launch_scatter(const T* g, const uint32_t* codes, const T* kernel, int klen, \
                               const Shape& sh, T* y, cudaStream_t stream) {                 \
        return sh.small_index()                                                              \
                   ? launch_scatter_t<T, int32_t>(g, codes, kernel, klen, sh, y, stream)     \
                   : launch_scatter_t<T, int64_t>(g, codes, kernel, klen, sh, y, stream);    \
    }                                                                                        \
    cudaError_t launch_kernel_grad(const T* g, const T* x, const uint32_t* codes, int klen,  \
                                   const Shape& sh, double* dw, cudaStream_t stream) {       \
        return sh.small_index()                                                              \
                   ? launch_kernel_grad_t<T, int32_t>(g, x, codes, klen, sh, dw, stream)     \
                   : launch_kernel_grad_t<T, int64_t>(g, x, codes, klen, sh, dw, stream);    \
    }

}  // namespace rlic
