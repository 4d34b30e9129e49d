// lic_stage.cu -- the replayed pass with its texture staged in shared memory
// by the Tensor Memory Accelerator (TMA).
//
// A replayed pass (lic_gather_kernel) gathers K texture cells per pixel along
// the recorded streamline.  Every cell a pixel samples lies within
// kmid = klen / 2 cells of it along each axis (one cell per step,
// src/lib.rs:325-329), so a super-tile of SX x SY pixels samples only a box of
// (SX + 2 HX) x (SY + 2 HY) cells around it, HX >= kmid and HY = kmid.  This
// kernel is persistent: each CTA loops over super-tiles; for each one a
// single thread issues one `cp.async.bulk.tensor.2d` copy of the box from HBM
// (through L2) into shared memory, and one `cp.async.bulk.tensor.3d` copy of
// the super-tile's code words (all words of its pixels), both completing on
// one mbarrier, and the CTA then replays its pixels from shared memory.  The
// copy engine fills the box and the codes, so the fill costs the load/store
// pipe nothing; the gathers, which bound the L1-cached replay, become
// shared-memory loads, and no step waits on a code word from HBM.
//
// Super-tiles whose box would cross a periodic image edge (their streamlines
// may wrap to the far side) replay through L1/L2 as lic_gather_kernel does.
// Boxes that cross a closed edge are staged: the copy fills cells outside the
// image with zeros, and no streamline reaches them (a closed edge clamps).
// Accumulation order and weights are those of the traced pass, so the results
// are bit-identical to lic_gather_kernel's.
//
// Every wait on the mbarrier is bounded: after kStageWaitLimit polls the CTA
// sets the library's stage-timeout word and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdlib>
#include <mutex>
#include <type_traits>

#include "lic_kernels.cuh"
#include "lic_lowp.cuh"

namespace rlic {

namespace {

constexpr int kStageThreadsX = 64;  // CTA: 64 x 4 threads, one column per thread
constexpr int kStageThreadsY = 4;
constexpr int kStageBoxOffset = 128;  // box start in shared memory (after the mbarrier)
constexpr uint32_t kStageWaitLimit = 1u << 22;
// The staged form needs at least two resident CTAs per SM to hide a copy
// behind the other CTA's work: a box larger than this (129 float64 taps)
// replays through L1 instead, which measured faster than one CTA per SM
// (the 8192^2 float64, 129-tap path cache: 270 against 301 ms).
constexpr size_t kStageMaxSmem = 113 * 1024;

__device__ unsigned g_stage_timeout = 0u;

struct StageGrid {
    int sx, sy;       // super-tile, pixels
    int hx, hy;       // halo, cells
    int bw, bh;       // staged box, cells (bw is the shared-memory row pitch)
    int tiles_x, ntiles;
    bool wrap_x, wrap_y;  // an axis with a periodic side
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// Polls the barrier's phase `parity` at most kStageWaitLimit times.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
    for (uint32_t k = 0; k < kStageWaitLimit; ++k)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// One 2-D tiled copy of the box at (x, y) (elements; x aligned to 16 bytes,
// negative or out-of-range coordinates read zeros) into shared memory.
__device__ __forceinline__ void tma_load_box(void* dst, const CUtensorMap* map, int x, int y,
                                             uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3}], [%4];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
        : "memory");
}

// The cell offset of step b of a code word inside a staged box of row pitch
// `pitch`: the column move (bits 4b..4b+1) and the row move (bits
// 4b+2..4b+3) as signed 2-bit fields.  A staged box never meets the wrap
// codes, and stop codes are handled before a word gets here, so only
// 0 / +1 / -1 occur; decoding by arithmetic keeps the gathers the only
// shared-memory loads of a step.
__device__ __forceinline__ int box_delta(uint32_t wd, int b, int pitch) {
    const int dx = int(wd << (30 - 4 * b)) >> 30;
    const int dy = int(wd << (28 - 4 * b)) >> 30;
    return dy * pitch + dx;
}

// Word q of one half's codes (0 past the last word of the half).
__device__ __forceinline__ uint32_t code_word(const uint32_t* __restrict__ words, int64_t npix,
                                              int q, int nwords) {
    return q < nwords ? __ldg(words + size_t(q) * size_t(npix)) : 0u;
}

// Where a half's code words come from: global memory (word q of the pixel
// at words[q * npix]) or a shared-memory copy of the super-tile's codes
// (word q at words[q * stride]).
struct GlobalWords {
    const uint32_t* __restrict__ words;
    int64_t npix;
    __device__ __forceinline__ uint32_t operator()(int q, int nwords) const {
        return code_word(words, npix, q, nwords);
    }
};
struct SharedWords {
    const uint32_t* words;
    int stride;
    __device__ __forceinline__ uint32_t operator()(int q, int nwords) const {
        return q < nwords ? words[q * stride] : 0u;
    }
};

// The 8 cells of one code word, gathered from the box into x.
template <typename T>
__device__ __forceinline__ void gather_word(int& cell, uint32_t wd, int pitch, const T* box,
                                            T x[8]) {
#pragma unroll
    for (int b = 0; b < 8; ++b) {
        cell += box_delta(wd, b, pitch);
        x[b] = box[cell];
    }
}

// The 8 ordered kernel-weighted samples of one code word.
template <typename T, bool FMA>
__device__ __forceinline__ void accumulate_word(T& acc, const T x[8], const T* w) {
    T wq[8];
    load8_aligned(w, wq);
#pragma unroll
    for (int b = 0; b < 8; ++b) acc = accumulate<T, FMA>(wq[b], x[b], acc);
}

// replay_half (lic_kernels.cuh) on the staged box: the same walk in the
// traced pass's accumulation order, with shared-memory gathers and
// arithmetic decoding.  The 8 gathers of word q + 1 are in flight while
// word q accumulates; the two word buffers alternate, two words per loop
// turn, so that no register copies are needed.  Code words are loaded two
// ahead: the caller passes the half's first two words (w0, w1), loaded
// when the pixel starts, and word q + 2 is requested while word q's
// gathers are issued.  (Requesting four words ahead measured slower: the
// extra registers cost a resident CTA.)  STOPS = false: the field holds no
// NaN sample, so no word holds a stop code and none is tested.
template <typename T, bool FMA, bool STOPS, typename WS>
__device__ __forceinline__ void replay_half_staged(T& acc, int cell, WS words, int count,
                                                   uint32_t w0, uint32_t w1, const T* w,
                                                   int pitch, const T* box) {
    const int full = count >> 3;
    const int nwords = (count + 7) >> 3;
    int q = 0;
    if (full > 0 && !(STOPS && word_has_stop(w0))) {
        T x[8], y[8];
        gather_word(cell, w0, pitch, box, x);
        uint32_t wn = w1;
        bool in_x = true;  // which buffer holds word q - 1, gathered, not yet accumulated
        for (q = 1; q < full;) {
            uint32_t wd = wn;
            wn = words(q + 1, nwords);
            if (STOPS && word_has_stop(wd)) break;
            gather_word(cell, wd, pitch, box, y);
            accumulate_word<T, FMA>(acc, x, w + 8 * (q - 1));
            in_x = false;
            if (++q >= full) break;
            wd = wn;
            wn = words(q + 1, nwords);
            if (STOPS && word_has_stop(wd)) break;
            gather_word(cell, wd, pitch, box, x);
            accumulate_word<T, FMA>(acc, y, w + 8 * (q - 1));
            in_x = true;
            ++q;
        }
        if (in_x) {
            accumulate_word<T, FMA>(acc, x, w + 8 * (q - 1));
        } else {
            accumulate_word<T, FMA>(acc, y, w + 8 * (q - 1));
        }
    }
    // a word with a stop code, or the last partial word, step by step
    for (; q < nwords; ++q) {
        const int n = (q < full) ? 8 : (count & 7);
        const uint32_t wd = q == 0 ? w0 : (q == 1 ? w1 : words(q, nwords));
        const T* wq = w + 8 * q;
        for (int b = 0; b < n; ++b) {
            if (STOPS && ((wd >> (4 * b)) & 15u) == kStop) return;
            cell += box_delta(wd, b, pitch);
            acc = accumulate<T, FMA>(wq[b], box[cell], acc);
        }
    }
}

// One staged pixel: the centre tap, then both halves, from word sources
// `fw` (forward) and `bw` (backward).
template <typename T, bool FMA, typename WS>
__device__ __forceinline__ T staged_pixel(int cell, WS fw, WS bw, int nf, int kmid, T wmid,
                                          const T* wsm, int nf_pad, int pitch, const T* box,
                                          bool nan_free) {
    const int nwf = (nf + 7) >> 3, nwb = (kmid + 7) >> 3;
    // both halves' first two code words, four loads in flight
    const uint32_t f0 = fw(0, nwf), f1 = fw(1, nwf);
    const uint32_t b0 = bw(0, nwb), b1 = bw(1, nwb);
    T acc = accumulate<T, FMA>(wmid, box[cell], T(0));
    if (nan_free) {
        replay_half_staged<T, FMA, false>(acc, cell, fw, nf, f0, f1, wsm, pitch, box);
        replay_half_staged<T, FMA, false>(acc, cell, bw, kmid, b0, b1, wsm + nf_pad, pitch, box);
    } else {
        replay_half_staged<T, FMA, true>(acc, cell, fw, nf, f0, f1, wsm, pitch, box);
        replay_half_staged<T, FMA, true>(acc, cell, bw, kmid, b0, b1, wsm + nf_pad, pitch, box);
    }
    return acc;
}

// A 3-D tiled copy of the super-tile's code words, box (64, sy, words) at
// (x, y, 0), into shared memory.
__device__ __forceinline__ void tma_load_codes(void* dst, const CUtensorMap* map, int x, int y,
                                               uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(0), "r"(smem_addr(bar))
        : "memory");
}

// CODES: the super-tile's code words come into shared memory by a second
// copy on the same mbarrier (a 3-D box over the word-major code array), so
// no step waits on a code word from HBM.
template <typename T, bool FMA, bool CODES>
__global__ void __launch_bounds__(kStageThreadsX * kStageThreadsY)
lic_gather_staged_kernel(const __grid_constant__ CUtensorMap map,
                         const __grid_constant__ CUtensorMap code_map,
                         const T* __restrict__ tex_in, const uint32_t* __restrict__ codes,
                         const T* __restrict__ kernel, int klen, Geometry<int32_t> g,
                         StageGrid sg, T* __restrict__ tex_out, CodeLayout cl,
                         const unsigned* __restrict__ field_nan) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
    T* box = reinterpret_cast<T*>(smem_raw + kStageBoxOffset);
    const int kmid = klen / 2;
    const int nf = klen - kmid - 1;
    const int nf_pad = (nf + 7) & ~7;
    const int nb_pad = (kmid + 7) & ~7;
    const int nwf = (nf + 7) >> 3, nwb = (kmid + 7) >> 3;
    const size_t box_bytes_al = (size_t(sg.bw) * size_t(sg.bh) * sizeof(T) + 127) & ~size_t(127);
    uint32_t* scodes = reinterpret_cast<uint32_t*>(smem_raw + kStageBoxOffset + box_bytes_al);
    const uint32_t code_bytes = CODES ? uint32_t(kStageThreadsX * sg.sy * (nwf + nwb) * 4) : 0u;
    T* wsm = reinterpret_cast<T*>(smem_raw + kStageBoxOffset + box_bytes_al + code_bytes);
    int* gtab = reinterpret_cast<int*>(wsm + nf_pad + nb_pad);  // image deltas
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    load_step_weights(wsm, kernel, klen, nf_pad);
    if (tid == 0) {
        fill_delta_table(gtab, g.nx, g.ny);
        mbar_init(bar);
    }
    __syncthreads();
    const T wmid = __ldg(kernel + kmid);
    // codes of a field known to hold no NaN sample have no stop code
    const bool nan_free = field_nan != nullptr && __ldg(field_nan) == 0u;
    const uint32_t* codes_b = codes + size_t(cl.words_f) * size_t(cl.npix);
    const uint32_t box_bytes = uint32_t(sg.bw) * uint32_t(sg.bh) * uint32_t(sizeof(T));
    const int word_stride = kStageThreadsX * sg.sy;  // between a pixel's words in scodes
    uint32_t parity = 0;
    for (int tile = blockIdx.x; tile < sg.ntiles; tile += gridDim.x) {
        const int ti = tile / sg.tiles_x;
        const int tj = tile - ti * sg.tiles_x;
        const int x0 = tj * sg.sx, y0 = ti * sg.sy;
        const int bx0 = x0 - sg.hx, by0 = y0 - sg.hy;
        const bool staged = !(sg.wrap_x && (bx0 < 0 || bx0 + sg.bw > g.nx)) &&
                            !(sg.wrap_y && (by0 < 0 || by0 + sg.bh > g.ny));
        if (staged) {
            if (tid == 0) {
                // order this CTA's earlier shared-memory reads before the copy
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                mbar_expect_tx(bar, box_bytes + code_bytes);
                tma_load_box(box, &map, bx0, by0, bar);
                if constexpr (CODES) tma_load_codes(scodes, &code_map, x0, y0, bar);
            }
            const bool arrived = mbar_wait_bounded(bar, parity);
            // the whole CTA leaves together if any thread gave up waiting
            if (__syncthreads_or(!arrived)) {
                if (tid == 0) atomicExch(&g_stage_timeout, 1u);
                if (!arrived) mbar_wait_bounded(bar, parity);  // the copy in flight, once more
                return;
            }
            parity ^= 1u;
        }
        for (int r = threadIdx.y; r < sg.sy; r += kStageThreadsY) {
            const int c = threadIdx.x;
            const int i = y0 + r, j = x0 + c;
            if (i >= g.ny || j >= g.nx) continue;
            const int p = i * g.nx + j;
            T acc;
            if (staged) {
                const int cell = (r + sg.hy) * sg.bw + (c + sg.hx);
                if constexpr (CODES) {
                    const uint32_t* mine = scodes + r * kStageThreadsX + c;
                    acc = staged_pixel<T, FMA>(cell, SharedWords{mine, word_stride},
                                               SharedWords{mine + nwf * word_stride, word_stride},
                                               nf, kmid, wmid, wsm, nf_pad, sg.bw, box, nan_free);
                } else {
                    acc = staged_pixel<T, FMA>(cell, GlobalWords{codes + p, cl.npix},
                                               GlobalWords{codes_b + p, cl.npix}, nf, kmid, wmid,
                                               wsm, nf_pad, sg.bw, box, nan_free);
                }
            } else {
                acc = accumulate<T, FMA>(wmid, __ldg(tex_in + p), T(0));
                replay_half<T, FMA, int32_t>(acc, p, codes + p, cl.npix, nf, wsm, gtab, tex_in);
                replay_half<T, FMA, int32_t>(acc, p, codes_b + p, cl.npix, kmid, wsm + nf_pad,
                                             gtab, tex_in);
            }
            tex_out[p] = acc;
        }
        __syncthreads();  // every read of the box precedes the next copy into it
    }
}

// ----------------------------------- reduced-precision staged replay --
//
// The same staging for the FP16 / BF16 storage form (lic_lowp.cu): the box
// holds 2-byte cells, each converted to FP32 when gathered, and the samples
// accumulate by compensated (Kahan) summation in the order of the traced
// pass, exactly as lic_gather_lowp_kernel does, so the results are the same
// bits.

__device__ __forceinline__ float stored_to_f32(__half h) { return __half2float(h); }
__device__ __forceinline__ float stored_to_f32(__nv_bfloat16 h) { return __bfloat162float(h); }

template <typename S>
__device__ __forceinline__ void gather_word_lowp(int& cell, uint32_t wd, int pitch, const S* box,
                                                 float x[8]) {
#pragma unroll
    for (int b = 0; b < 8; ++b) {
        cell += box_delta(wd, b, pitch);
        x[b] = stored_to_f32(box[cell]);
    }
}

__device__ __forceinline__ void kahan_word(float& sum, float& comp, const float x[8],
                                           const float* w) {
    float wq[8];
    load8_aligned(w, wq);
#pragma unroll
    for (int b = 0; b < 8; ++b) kahan_add(sum, comp, wq[b], x[b]);
}

// replay_half_staged with FP16/BF16 cells and compensated FP32 sums.
template <typename S, bool STOPS>
__device__ __forceinline__ void replay_half_staged_lowp(float& sum, float& comp, int cell,
                                                        const uint32_t* __restrict__ words,
                                                        int64_t npix, int count, uint32_t w0,
                                                        uint32_t w1, const float* w, int pitch,
                                                        const S* box) {
    const int full = count >> 3;
    const int nwords = (count + 7) >> 3;
    int q = 0;
    if (full > 0 && !(STOPS && word_has_stop(w0))) {
        float x[8], y[8];
        gather_word_lowp(cell, w0, pitch, box, x);
        uint32_t wn = w1;
        bool in_x = true;
        for (q = 1; q < full;) {
            uint32_t wd = wn;
            wn = code_word(words, npix, q + 1, nwords);
            if (STOPS && word_has_stop(wd)) break;
            gather_word_lowp(cell, wd, pitch, box, y);
            kahan_word(sum, comp, x, w + 8 * (q - 1));
            in_x = false;
            if (++q >= full) break;
            wd = wn;
            wn = code_word(words, npix, q + 1, nwords);
            if (STOPS && word_has_stop(wd)) break;
            gather_word_lowp(cell, wd, pitch, box, x);
            kahan_word(sum, comp, y, w + 8 * (q - 1));
            in_x = true;
            ++q;
        }
        if (in_x) {
            kahan_word(sum, comp, x, w + 8 * (q - 1));
        } else {
            kahan_word(sum, comp, y, w + 8 * (q - 1));
        }
    }
    for (; q < nwords; ++q) {
        const int n = (q < full) ? 8 : (count & 7);
        const uint32_t wd = q == 0 ? w0 : (q == 1 ? w1 : code_word(words, npix, q, nwords));
        const float* wq = w + 8 * q;
        for (int b = 0; b < n; ++b) {
            if (STOPS && ((wd >> (4 * b)) & 15u) == kStop) return;
            cell += box_delta(wd, b, pitch);
            kahan_add(sum, comp, wq[b], stored_to_f32(box[cell]));
        }
    }
}

template <typename S>
__global__ void __launch_bounds__(kStageThreadsX * kStageThreadsY)
lic_gather_staged_lowp_kernel(const __grid_constant__ CUtensorMap map,
                              const S* __restrict__ tex_in, const uint32_t* __restrict__ codes,
                              const float* __restrict__ w32, int klen,
                              const float* __restrict__ inv_scale, Geometry<int32_t> g,
                              StageGrid sg, S* __restrict__ tex_out, CodeLayout cl,
                              const unsigned* __restrict__ field_nan) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
    S* box = reinterpret_cast<S*>(smem_raw + kStageBoxOffset);
    const int kmid = klen / 2;
    const int nf = klen - kmid - 1;
    const int nf_pad = (nf + 7) & ~7;
    const int nb_pad = (kmid + 7) & ~7;
    // weights after the box, 16-byte aligned
    const size_t box_bytes_al = (size_t(sg.bw) * size_t(sg.bh) * sizeof(S) + 15) & ~size_t(15);
    float* wsm = reinterpret_cast<float*>(smem_raw + kStageBoxOffset + box_bytes_al);
    int* gtab = reinterpret_cast<int*>(wsm + nf_pad + nb_pad);
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    load_step_weights(wsm, w32, klen, nf_pad);
    if (tid == 0) {
        fill_delta_table(gtab, g.nx, g.ny);
        mbar_init(bar);
    }
    __syncthreads();
    const float wmid = __ldg(w32 + kmid);
    const float scale = __ldg(inv_scale);
    const bool nan_free = field_nan != nullptr && __ldg(field_nan) == 0u;
    const uint32_t* codes_b = codes + size_t(cl.words_f) * size_t(cl.npix);
    const uint32_t box_bytes = uint32_t(sg.bw) * uint32_t(sg.bh) * uint32_t(sizeof(S));
    const int nwf = (nf + 7) >> 3, nwb = (kmid + 7) >> 3;
    uint32_t parity = 0;
    for (int tile = blockIdx.x; tile < sg.ntiles; tile += gridDim.x) {
        const int ti = tile / sg.tiles_x;
        const int tj = tile - ti * sg.tiles_x;
        const int x0 = tj * sg.sx, y0 = ti * sg.sy;
        const int bx0 = x0 - sg.hx, by0 = y0 - sg.hy;
        const bool staged = !(sg.wrap_x && (bx0 < 0 || bx0 + sg.bw > g.nx)) &&
                            !(sg.wrap_y && (by0 < 0 || by0 + sg.bh > g.ny));
        if (staged) {
            if (tid == 0) {
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                mbar_expect_tx(bar, box_bytes);
                tma_load_box(box, &map, bx0, by0, bar);
            }
            const bool arrived = mbar_wait_bounded(bar, parity);
            if (__syncthreads_or(!arrived)) {
                if (tid == 0) atomicExch(&g_stage_timeout, 1u);
                if (!arrived) mbar_wait_bounded(bar, parity);
                return;
            }
            parity ^= 1u;
        }
        for (int r = threadIdx.y; r < sg.sy; r += kStageThreadsY) {
            const int c = threadIdx.x;
            const int i = y0 + r, j = x0 + c;
            if (i >= g.ny || j >= g.nx) continue;
            const int p = i * g.nx + j;
            float sum = 0.f, comp = 0.f;
            if (staged) {
                const uint32_t f0 = code_word(codes + p, cl.npix, 0, nwf);
                const uint32_t f1 = code_word(codes + p, cl.npix, 1, nwf);
                const uint32_t b0 = code_word(codes_b + p, cl.npix, 0, nwb);
                const uint32_t b1 = code_word(codes_b + p, cl.npix, 1, nwb);
                const int cell = (r + sg.hy) * sg.bw + (c + sg.hx);
                kahan_add(sum, comp, wmid, stored_to_f32(box[cell]));
                if (nan_free) {
                    replay_half_staged_lowp<S, false>(sum, comp, cell, codes + p, cl.npix, nf, f0,
                                                      f1, wsm, sg.bw, box);
                    replay_half_staged_lowp<S, false>(sum, comp, cell, codes_b + p, cl.npix, kmid,
                                                      b0, b1, wsm + nf_pad, sg.bw, box);
                } else {
                    replay_half_staged_lowp<S, true>(sum, comp, cell, codes + p, cl.npix, nf, f0,
                                                     f1, wsm, sg.bw, box);
                    replay_half_staged_lowp<S, true>(sum, comp, cell, codes_b + p, cl.npix, kmid,
                                                     b0, b1, wsm + nf_pad, sg.bw, box);
                }
            } else {
                kahan_add(sum, comp, wmid, StorageTraits<S>::load(tex_in + p));
                replay_half_lowp<S, int32_t>(sum, comp, p, codes + p, cl.npix, nf, wsm, gtab,
                                             tex_in);
                replay_half_lowp<S, int32_t>(sum, comp, p, codes_b + p, cl.npix, kmid,
                                             wsm + nf_pad, gtab, tex_in);
            }
            tex_out[p] = StorageTraits<S>::from_float(__fmul_rn(sum, scale));
        }
        __syncthreads();
    }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn(cudaError_t* err) {
    static std::mutex mu;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::lock_guard<std::mutex> lock(mu);
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        *err = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                                cudaEnableDefault, &q);
        if (*err != cudaSuccess) return nullptr;
        if (q != cudaDriverEntryPointSuccess || !p) {
            *err = cudaErrorNotSupported;
            return nullptr;
        }
        fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    *err = cudaSuccess;
    return fn;
}

int g_stage_rows = 16;  // super-tile height in pixels (a multiple of 4)

// Extra cells per box row (a multiple of 4): a wider box changes the row
// pitch, and with it which gathers of a warp share a shared-memory bank.
// RLIC_STAGE_PAD in the environment sets it (tuning only).
int stage_pad() {
    static const int pad = [] {
        const char* e = std::getenv("RLIC_STAGE_PAD");
        const int v = e ? std::atoi(e) : 0;
        return (v >= 0 && v <= 64 && v % 4 == 0) ? v : 0;
    }();
    return pad;
}

// Super-tile, halo and box of a staged replay of `elem`-byte cells, and the
// tensor map over the texture; cudaErrorNotSupported when the image or the
// kernel does not fit the form.
cudaError_t plan_stage(const void* tex_in, size_t elem, CUtensorMapDataType dtype, int klen,
                       const Shape& sh, size_t weights_bytes, StageGrid* sg, size_t* smem,
                       CUtensorMap* map) {
    const int kmid = klen / 2;
    const int align = int(16 / elem);  // x of a copy: 16-byte aligned
    if (!sh.small_index() || klen < 2 || (sh.nx * int64_t(elem)) % 16 != 0 ||
        (reinterpret_cast<uintptr_t>(tex_in) & 15u) != 0)
        return cudaErrorNotSupported;
    sg->sx = kStageThreadsX;
    sg->sy = g_stage_rows;
    sg->hx = (kmid + align - 1) / align * align;
    sg->hy = kmid;
    sg->bw = sg->sx + 2 * sg->hx + (stage_pad() + align - 1) / align * align;
    sg->bh = sg->sy + 2 * sg->hy;
    if (sg->bw > 256 || sg->bh > 256) return cudaErrorNotSupported;  // box limit of a copy
    sg->tiles_x = int(tiles_of(sh.nx, sg->sx));
    const int64_t ntiles = int64_t(sg->tiles_x) * tiles_of(sh.ny, sg->sy);
    if (ntiles > 0x7fffffffLL) return cudaErrorNotSupported;
    sg->ntiles = int(ntiles);
    sg->wrap_x = sh.bnd[0] == 1 || sh.bnd[1] == 1;
    sg->wrap_y = sh.bnd[2] == 1 || sh.bnd[3] == 1;
    const size_t box = (elem * size_t(sg->bw) * size_t(sg->bh) + 15) & ~size_t(15);
    *smem = kStageBoxOffset + box + weights_bytes + 16 * sizeof(int);
    if (*smem > kStageMaxSmem) return cudaErrorNotSupported;
    cudaError_t e = cudaSuccess;
    auto encode = encode_fn(&e);
    if (!encode) return e;
    const cuuint64_t dims[2] = {cuuint64_t(sh.nx), cuuint64_t(sh.ny)};
    const cuuint64_t strides[1] = {cuuint64_t(sh.nx) * elem};
    const cuuint32_t boxdim[2] = {cuuint32_t(sg->bw), cuuint32_t(sg->bh)};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult cr = encode(map, dtype, 2, const_cast<void*>(tex_in), dims, strides, boxdim,
                               estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                               CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return cr == CUDA_SUCCESS ? cudaSuccess : cudaErrorNotSupported;
}

template <typename S>
cudaError_t launch_gather_staged_lowp_t(const void* tex_in, const uint32_t* codes,
                                        const float* w32, int klen, const float* inv_scale,
                                        const Shape& sh, const unsigned* field_nan,
                                        void* tex_out, cudaStream_t stream) {
    const int kmid = klen / 2;
    const int nf = klen - kmid - 1;
    StageGrid sg;
    size_t smem = 0;
    CUtensorMap map;
    const CUtensorMapDataType dt = sizeof(S) == 2 && std::is_same<S, __half>::value
                                       ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16
                                       : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
    cudaError_t e = plan_stage(tex_in, sizeof(S), dt, klen, sh,
                               sizeof(float) * size_t(((nf + 7) & ~7) + ((kmid + 7) & ~7)), &sg,
                               &smem, &map);
    if (e != cudaSuccess) return e;
    auto kfn = lic_gather_staged_lowp_kernel<S>;
    unsigned grid = 0;
    e = persistent_grid(kfn, kStageThreadsX * kStageThreadsY, smem, sg.ntiles, &grid);
    if (e != cudaSuccess) return e;
    const auto g = make_geometry<int32_t>(sh);
    const auto cl = make_code_layout(sh, klen);
    kfn<<<grid, dim3(kStageThreadsX, kStageThreadsY), smem, stream>>>(
        map, static_cast<const S*>(tex_in), codes, w32, klen, inv_scale, g, sg,
        static_cast<S*>(tex_out), cl, field_nan);
    count_launch();
    return cudaGetLastError();
}

// Whether staged replays also copy their super-tile's code words into
// shared memory (the default: 1.63 against 1.73 ms per replay at 8192^2,
// with 16-row super-tiles; RLIC_STAGE_CODES=0 in the environment turns it
// off, for tuning).
bool stage_codes() {
    static const bool on = [] {
        const char* e = std::getenv("RLIC_STAGE_CODES");
        return !(e != nullptr && e[0] == '0');
    }();
    return on;
}

template <typename T, bool FMA>
cudaError_t launch_gather_staged_t(const T* tex_in, const uint32_t* codes, const T* kernel,
                                   int klen, const Shape& sh, const unsigned* field_nan,
                                   T* tex_out, cudaStream_t stream) {
    const int kmid = klen / 2;
    const int nf = klen - kmid - 1;
    const size_t wbytes = sizeof(T) * size_t(((nf + 7) & ~7) + ((kmid + 7) & ~7));
    StageGrid sg;
    size_t smem = 0;
    CUtensorMap map, code_map;
    cudaError_t e = plan_stage(
        tex_in, sizeof(T),
        sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, klen,
        sh, wbytes, &sg, &smem, &map);
    if (e != cudaSuccess) return e;
    const int words = int((nf + 7) / 8 + (kmid + 7) / 8);
    bool with_codes = stage_codes() && sh.nx % 4 == 0 &&
                      (reinterpret_cast<uintptr_t>(codes) & 15u) == 0 && words <= 256;
    if (with_codes) {
        const size_t box_al = (sizeof(T) * size_t(sg.bw) * size_t(sg.bh) + 127) & ~size_t(127);
        const size_t smem_c = kStageBoxOffset + box_al +
                              size_t(kStageThreadsX) * sg.sy * words * 4 + wbytes +
                              16 * sizeof(int);
        cudaError_t ce = cudaSuccess;
        auto encode = encode_fn(&ce);
        const cuuint64_t dims[3] = {cuuint64_t(sh.nx), cuuint64_t(sh.ny), cuuint64_t(words)};
        const cuuint64_t strides[2] = {cuuint64_t(sh.nx) * 4,
                                       cuuint64_t(sh.nx) * cuuint64_t(sh.ny) * 4};
        const cuuint32_t boxdim[3] = {cuuint32_t(kStageThreadsX), cuuint32_t(sg.sy),
                                      cuuint32_t(words)};
        const cuuint32_t estr[3] = {1, 1, 1};
        with_codes = smem_c <= kStageMaxSmem && encode != nullptr &&
                     encode(&code_map, CU_TENSOR_MAP_DATA_TYPE_UINT32, 3,
                            const_cast<uint32_t*>(codes), dims, strides, boxdim, estr,
                            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
        if (with_codes) smem = smem_c;
    }
    if (!with_codes) code_map = map;  // unused
    auto kfn = with_codes ? lic_gather_staged_kernel<T, FMA, true>
                          : lic_gather_staged_kernel<T, FMA, false>;
    if (!with_codes) {
        // the layout without codes: the box rounded to 128 bytes, then weights
        const size_t box_al = (sizeof(T) * size_t(sg.bw) * size_t(sg.bh) + 127) & ~size_t(127);
        smem = kStageBoxOffset + box_al + wbytes + 16 * sizeof(int);
        if (smem > kStageMaxSmem) return cudaErrorNotSupported;
    }
    unsigned grid = 0;
    e = persistent_grid(kfn, kStageThreadsX * kStageThreadsY, smem, sg.ntiles, &grid);
    if (e != cudaSuccess) return e;
    const auto g = make_geometry<int32_t>(sh);
    const auto cl = make_code_layout(sh, klen);
    kfn<<<grid, dim3(kStageThreadsX, kStageThreadsY), smem, stream>>>(
        map, code_map, tex_in, codes, kernel, klen, g, sg, tex_out, cl, field_nan);
    count_launch();
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_gather_staged(bool fma, const float* tex_in, const uint32_t* codes,
                                 const float* kernel, int klen, const Shape& sh,
                                 const unsigned* field_nan, float* tex_out,
                                 cudaStream_t stream) {
    return fma ? launch_gather_staged_t<float, true>(tex_in, codes, kernel, klen, sh, field_nan,
                                                     tex_out, stream)
               : launch_gather_staged_t<float, false>(tex_in, codes, kernel, klen, sh, field_nan,
                                                      tex_out, stream);
}

cudaError_t launch_gather_staged(bool fma, const double* tex_in, const uint32_t* codes,
                                 const double* kernel, int klen, const Shape& sh,
                                 const unsigned* field_nan, double* tex_out,
                                 cudaStream_t stream) {
    return fma ? launch_gather_staged_t<double, true>(tex_in, codes, kernel, klen, sh, field_nan,
                                                      tex_out, stream)
               : launch_gather_staged_t<double, false>(tex_in, codes, kernel, klen, sh,
                                                       field_nan, tex_out, stream);
}

cudaError_t launch_gather_staged_lowp(int storage, const void* tex_in, const uint32_t* codes,
                                      const float* w32, int klen, const float* inv_scale,
                                      const Shape& sh, const unsigned* field_nan,
                                      void* tex_out, cudaStream_t stream) {
    if (storage == kStorageFP16)
        return launch_gather_staged_lowp_t<__half>(tex_in, codes, w32, klen, inv_scale, sh,
                                                   field_nan, tex_out, stream);
    if (storage == kStorageBF16)
        return launch_gather_staged_lowp_t<__nv_bfloat16>(tex_in, codes, w32, klen, inv_scale,
                                                          sh, field_nan, tex_out, stream);
    return cudaErrorInvalidValue;
}

void set_stage_rows(int rows) { g_stage_rows = rows; }

cudaError_t stage_timeout_seen(bool* seen) {
    unsigned v = 0;
    cudaError_t e = cudaMemcpyFromSymbol(&v, g_stage_timeout, sizeof(v));
    *seen = v != 0;
    return e;
}

}  // namespace rlic
