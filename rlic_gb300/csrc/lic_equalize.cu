// lic_equalize.cu -- histogram equalization of an image on the GPU.
//
// The reference declares equalize_histogram{,_sliding_tile,
// _tile_interpolation}_{f32,f64} in its native-module stubs
// (src/rlic/_core.pyi:30-57) without implementing them (README.md:19-23
// points to the separate `ahe` package), so the definitions here are this
// library's own; oracle/histogram.py states them in numpy and the GPU
// results match it bit for bit.  Every step rounds once in the image's
// dtype, in the order of that definition.
//
// Work, for an ny x nx image:
//   1. finite min / max / count: one pass, block reductions, one atomic per
//      block on order-preserving integer encodings;
//   2. bin of every pixel (int32, -1 for non-finite);
//   3a. global: shared-memory histograms per block, merged with atomics,
//       one-block inclusive scan, then out = cdf[bin] / count;
//   3b. tile interpolation: one CTA per tile builds its histogram in shared
//       memory, scans it and writes the tile's mapping; each pixel then
//       blends the mappings of its four nearest tile centres;
//   3c. sliding tile: each thread slides one column's window down a run of
//       rows, keeping the window's histogram in shared memory (2 tw cell
//       updates per pixel); windows beyond 65535 cells or more than 256
//       bins count every window cell per pixel instead.
#include "../../include/rlic_gb300.h"
#include "lic_equalize.h"
#include "lic_launch.h"

#include <cstdint>
#include <cuda_runtime.h>

namespace rlic {
namespace {

// Order-preserving unsigned encodings of finite floats (for atomic min/max).
__device__ __forceinline__ uint32_t order_key(float x) {
    const uint32_t b = __float_as_uint(x);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ unsigned long long order_key(double x) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x));
    return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ float from_key(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}
__device__ __forceinline__ double from_key(unsigned long long k) {
    return __longlong_as_double(static_cast<long long>(
        (k & 0x8000000000000000ull) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k));
}

template <typename T> struct KeyOf;
template <> struct KeyOf<float> { using type = uint32_t; };
template <> struct KeyOf<double> { using type = unsigned long long; };

template <typename T>
struct Stats {
    typename KeyOf<T>::type lo_key, hi_key;
    unsigned long long count;
};

template <typename T> __device__ __forceinline__ T div_rn_(T a, T b);
template <> __device__ __forceinline__ float div_rn_(float a, float b) { return __fdiv_rn(a, b); }
template <> __device__ __forceinline__ double div_rn_(double a, double b) { return __ddiv_rn(a, b); }
template <typename T> __device__ __forceinline__ T sub_rn_(T a, T b);
template <> __device__ __forceinline__ float sub_rn_(float a, float b) { return __fsub_rn(a, b); }
template <> __device__ __forceinline__ double sub_rn_(double a, double b) { return __dsub_rn(a, b); }
template <typename T> __device__ __forceinline__ T mul_rn_(T a, T b);
template <> __device__ __forceinline__ float mul_rn_(float a, float b) { return __fmul_rn(a, b); }
template <> __device__ __forceinline__ double mul_rn_(double a, double b) { return __dmul_rn(a, b); }
template <typename T> __device__ __forceinline__ T add_rn_(T a, T b);
template <> __device__ __forceinline__ float add_rn_(float a, float b) { return __fadd_rn(a, b); }
template <> __device__ __forceinline__ double add_rn_(double a, double b) { return __dadd_rn(a, b); }
// integer count -> T, rounded to nearest (as numpy's int64 -> float cast)
template <typename T> __device__ __forceinline__ T from_count(unsigned long long c);
template <> __device__ __forceinline__ float from_count(unsigned long long c) {
    return __ull2float_rn(c);
}
template <> __device__ __forceinline__ double from_count(unsigned long long c) {
    return __ull2double_rn(c);
}

template <typename T>
__global__ void stats_init_kernel(Stats<T>* st) {
    st->lo_key = ~typename KeyOf<T>::type(0);
    st->hi_key = 0;
    st->count = 0;
}

template <typename T>
__global__ void minmax_kernel(const T* __restrict__ x, int64_t n, Stats<T>* st) {
    using K = typename KeyOf<T>::type;
    K lo = ~K(0), hi = K(0);
    unsigned long long cnt = 0;
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n; k += stride) {
        const T v = x[k];
        if (isfinite(v)) {
            const K key = order_key(v);
            lo = key < lo ? key : lo;
            hi = key > hi ? key : hi;
            ++cnt;
        }
    }
    __shared__ K s_lo[32], s_hi[32];
    __shared__ unsigned long long s_cnt[32];
    for (int off = 16; off > 0; off >>= 1) {
        const K olo = __shfl_down_sync(0xffffffffu, lo, off);
        const K ohi = __shfl_down_sync(0xffffffffu, hi, off);
        cnt += __shfl_down_sync(0xffffffffu, cnt, off);
        lo = olo < lo ? olo : lo;
        hi = ohi > hi ? ohi : hi;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        s_lo[warp] = lo;
        s_hi[warp] = hi;
        s_cnt[warp] = cnt;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < int(blockDim.x >> 5); ++w) {
            lo = s_lo[w] < lo ? s_lo[w] : lo;
            hi = s_hi[w] > hi ? s_hi[w] : hi;
            cnt += s_cnt[w];
        }
        if (cnt) {
            atomicMin(&st->lo_key, lo);
            atomicMax(&st->hi_key, hi);
            atomicAdd(&st->count, cnt);
        }
    }
}

// bin(p) as defined in oracle/histogram.py; -1 for non-finite pixels.
template <typename T>
__global__ void bins_kernel(const T* __restrict__ x, int64_t n, const Stats<T>* st, int nbins,
                            int32_t* __restrict__ bins) {
    const T lo = from_key(st->lo_key), hi = from_key(st->hi_key);
    const T span = sub_rn_(hi, lo);
    const bool spread = st->count > 0 && hi > lo && isfinite(span);
    const T scale = spread ? div_rn_(T(nbins), span) : T(0);
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n; k += stride) {
        const T v = x[k];
        int32_t b = -1;
        if (isfinite(v)) {
            b = 0;
            if (spread) {
                const T s = floor(mul_rn_(sub_rn_(v, lo), scale));
                b = s >= T(nbins - 1) ? nbins - 1 : int32_t(s);
            }
        }
        bins[k] = b;
    }
}

// Global histogram: shared-memory counts per block when they fit.
__global__ void hist_kernel(const int32_t* __restrict__ bins, int64_t n, int nbins,
                            unsigned long long* __restrict__ hist, bool shared) {
    extern __shared__ uint32_t s_hist[];
    if (shared) {
        for (int k = threadIdx.x; k < nbins; k += blockDim.x) s_hist[k] = 0u;
        __syncthreads();
    }
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n; k += stride) {
        const int32_t b = bins[k];
        if (b >= 0) {
            if (shared) {
                atomicAdd(&s_hist[b], 1u);
            } else {
                atomicAdd(&hist[b], 1ull);
            }
        }
    }
    if (shared) {
        __syncthreads();
        for (int k = threadIdx.x; k < nbins; k += blockDim.x)
            if (s_hist[k]) atomicAdd(&hist[k], (unsigned long long)s_hist[k]);
    }
}

// Inclusive scan of v[0..n) by one block of 1024 threads, in chunks.
template <typename V>
__device__ void block_inclusive_scan(V* v, int64_t n) {
    __shared__ V s_part[1024];
    __shared__ V s_carry;
    if (threadIdx.x == 0) s_carry = V(0);
    __syncthreads();
    for (int64_t base = 0; base < n; base += blockDim.x) {
        const int64_t k = base + threadIdx.x;
        s_part[threadIdx.x] = k < n ? v[k] : V(0);
        __syncthreads();
        for (int off = 1; off < int(blockDim.x); off <<= 1) {
            const V add = threadIdx.x >= unsigned(off) ? s_part[threadIdx.x - off] : V(0);
            __syncthreads();
            s_part[threadIdx.x] += add;
            __syncthreads();
        }
        if (k < n) v[k] = s_part[threadIdx.x] + s_carry;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) s_carry += s_part[threadIdx.x];
        __syncthreads();
    }
}

__global__ void scan_kernel(unsigned long long* hist, int nbins) {
    block_inclusive_scan(hist, nbins);
}

template <typename T>
__global__ void map_global_kernel(const T* __restrict__ x, const int32_t* __restrict__ bins,
                                  int64_t n, const unsigned long long* __restrict__ cdf,
                                  const Stats<T>* st, T* __restrict__ out) {
    const T count = from_count<T>(st->count);
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n; k += stride) {
        const int32_t b = bins[k];
        out[k] = b >= 0 ? div_rn_(from_count<T>(cdf[b]), count) : x[k];
    }
}

// One CTA per tile: histogram in shared memory, scan, mapping m_t(k).
template <typename T>
__global__ void tile_maps_kernel(const int32_t* __restrict__ bins, int64_t ny, int64_t nx,
                                 int64_t th, int64_t tw, int64_t ntx, int nbins,
                                 T* __restrict__ maps) {
    extern __shared__ uint32_t s_cdf[];
    __shared__ uint32_t s_n;
    const int64_t t = blockIdx.x;
    const int64_t a = t / ntx, c = t - a * ntx;
    const int64_t r0 = a * th, r1 = (r0 + th < ny) ? r0 + th : ny;
    const int64_t c0 = c * tw, c1 = (c0 + tw < nx) ? c0 + tw : nx;
    for (int k = threadIdx.x; k < nbins; k += blockDim.x) s_cdf[k] = 0u;
    if (threadIdx.x == 0) s_n = 0u;
    __syncthreads();
    const int64_t w = c1 - c0, cells = (r1 - r0) * w;
    uint32_t mine = 0;
    for (int64_t q = threadIdx.x; q < cells; q += blockDim.x) {
        const int64_t i = r0 + q / w, j = c0 + q % w;
        const int32_t b = bins[i * nx + j];
        if (b >= 0) {
            atomicAdd(&s_cdf[b], 1u);
            ++mine;
        }
    }
    if (mine) atomicAdd(&s_n, mine);
    __syncthreads();
    block_inclusive_scan(s_cdf, nbins);
    __syncthreads();
    const uint32_t nt = s_n;
    T* m = maps + t * nbins;
    const T tn = from_count<T>(nt);
    for (int k = threadIdx.x; k < nbins; k += blockDim.x)
        m[k] = nt ? div_rn_(from_count<T>(s_cdf[k]), tn) : T(0);
}

// Tile centre (r0 + r1 - 1) / 2 of tile a along an axis of n cells in tiles of t.
template <typename T>
__device__ __forceinline__ T tile_centre(int64_t a, int64_t t, int64_t n) {
    const int64_t r0 = a * t, r1 = (r0 + t < n) ? r0 + t : n;
    return mul_rn_(T(r0 + r1 - 1), T(0.5));  // exact: the halving of an integer
}

// (a0, a1, f) of position i against the tile centres of one axis.
template <typename T>
__device__ __forceinline__ void interp_axis(int64_t i, int64_t t, int64_t n, int64_t nt,
                                            int64_t& a0, int64_t& a1, T& f) {
    const T pos = T(i);
    const T first = tile_centre<T>(0, t, n), last = tile_centre<T>(nt - 1, t, n);
    f = T(0);
    if (!(pos > first)) {
        a0 = a1 = 0;
        return;
    }
    if (!(pos < last)) {
        a0 = a1 = nt - 1;
        return;
    }
    // the last centre <= i: centres of full tiles are a t + (t - 1) / 2
    int64_t a = (2 * i - (t - 1)) / (2 * t);
    if (a < 0) a = 0;
    if (a > nt - 1) a = nt - 1;
    while (a + 1 < nt && !(tile_centre<T>(a + 1, t, n) > pos)) ++a;
    while (a > 0 && tile_centre<T>(a, t, n) > pos) --a;
    a0 = a;
    a1 = a + 1;
    const T c0 = tile_centre<T>(a0, t, n), c1 = tile_centre<T>(a1, t, n);
    f = div_rn_(sub_rn_(pos, c0), sub_rn_(c1, c0));
}

template <typename T>
__device__ __forceinline__ T lerp_rn(T u, T w, T f) {
    return add_rn_(u, mul_rn_(f, sub_rn_(w, u)));
}

// (a0, a1, f) of every row (blockIdx.y == 0) or column (== 1) of the image.
template <typename T>
__global__ void axis_tables_kernel(int64_t ny, int64_t nx, int64_t th, int64_t tw, int64_t nty,
                                   int64_t ntx, int32_t* __restrict__ a0, int32_t* __restrict__ a1,
                                   T* __restrict__ f) {
    const bool cols = blockIdx.y == 1;
    const int64_t n = cols ? nx : ny, t = cols ? tw : th, nt = cols ? ntx : nty;
    const int64_t base = cols ? ny : 0;
    for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += int64_t(gridDim.x) * blockDim.x) {
        int64_t lo, hi;
        T w;
        interp_axis<T>(i, t, n, nt, lo, hi, w);
        a0[base + i] = int32_t(lo);
        a1[base + i] = int32_t(hi);
        f[base + i] = w;
    }
}

template <typename T>
__global__ void map_tiles_kernel(const T* __restrict__ x, const int32_t* __restrict__ bins,
                                 int64_t ny, int64_t nx, int64_t ntx, int nbins,
                                 const int32_t* __restrict__ a0, const int32_t* __restrict__ a1,
                                 const T* __restrict__ f, const T* __restrict__ maps,
                                 T* __restrict__ out) {
    const int64_t j = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= nx) return;
    const int64_t ca0 = a0[ny + j], ca1 = a1[ny + j];
    const T fx = f[ny + j];
    for (int64_t i = blockIdx.y; i < ny; i += gridDim.y) {
        const int64_t k = i * nx + j;
        const int32_t b = bins[k];
        if (b < 0) {
            out[k] = x[k];
            continue;
        }
        const int64_t ra0 = a0[i], ra1 = a1[i];
        const T fy = f[i];
        const T m00 = maps[(ra0 * ntx + ca0) * nbins + b];
        const T m01 = maps[(ra0 * ntx + ca1) * nbins + b];
        const T m10 = maps[(ra1 * ntx + ca0) * nbins + b];
        const T m11 = maps[(ra1 * ntx + ca1) * nbins + b];
        out[k] = lerp_rn(lerp_rn(m00, m01, fx), lerp_rn(m10, m11, fx), fy);
    }
}

template <typename T>
__device__ __forceinline__ void sliding_pixel(const T* __restrict__ x,
                                              const int32_t* __restrict__ bins, int64_t ny,
                                              int64_t nx, int64_t th, int64_t tw, bool all_finite,
                                              int64_t i, int64_t j, T* __restrict__ out);

// Sliding tile: rank of the pixel's bin within its window.
template <typename T>
__global__ void sliding_kernel(const T* __restrict__ x, const int32_t* __restrict__ bins,
                               int64_t ny, int64_t nx, int64_t th, int64_t tw,
                               const Stats<T>* st, T* __restrict__ out) {
    const int64_t j = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= nx) return;
    const bool all_finite = st->count == (unsigned long long)(ny * nx);
    for (int64_t i = int64_t(blockIdx.y) * blockDim.y + threadIdx.y; i < ny;
         i += int64_t(gridDim.y) * blockDim.y) {
        sliding_pixel(x, bins, ny, nx, th, tw, all_finite, i, j, out);
    }
}

template <typename T>
__device__ __forceinline__ void sliding_pixel(const T* __restrict__ x,
                                              const int32_t* __restrict__ bins, int64_t ny,
                                              int64_t nx, int64_t th, int64_t tw, bool all_finite,
                                              int64_t i, int64_t j, T* __restrict__ out) {
    const int64_t k = i * nx + j;
    const int32_t b = bins[k];
    if (b < 0) {
        out[k] = x[k];
        return;
    }
    const int64_t r0 = i - th / 2 < 0 ? 0 : i - th / 2;
    const int64_t r1 = i - th / 2 + th > ny ? ny : i - th / 2 + th;
    const int64_t c0 = j - tw / 2 < 0 ? 0 : j - tw / 2;
    const int64_t c1 = j - tw / 2 + tw > nx ? nx : j - tw / 2 + tw;
    // a non-finite cell holds -1, which as an unsigned value is above every
    // bin: one unsigned compare counts the finite cells whose bin is <= b
    const uint32_t ub = uint32_t(b);
    const int w = int(c1 - c0);
    uint32_t below = 0, invalid = 0;
    for (int64_t r = r0; r < r1; ++r) {
        const int32_t* row = bins + r * nx + c0;
        for (int c = 0; c < w; ++c) below += uint32_t(__ldg(row + c)) <= ub;
        if (!all_finite)
            for (int c = 0; c < w; ++c) invalid += __ldg(row + c) < 0;
    }
    const uint32_t valid = uint32_t((r1 - r0) * w) - invalid;
    out[k] = div_rn_(from_count<T>(below), from_count<T>(valid));
}

// Sliding tile with the bins of a CTA's 32 x 8 pixels and their windows
// staged in shared memory (cells outside the image hold -1, which no count
// includes).  Used when that region fits; the counts are the same as
// sliding_pixel's.
constexpr int kSlideBx = 32, kSlideBy = 8;

template <typename T>
__global__ void __launch_bounds__(kSlideBx * kSlideBy)
sliding_smem_kernel(const T* __restrict__ x, const int32_t* __restrict__ bins, int64_t ny,
                    int64_t nx, int th, int tw, const Stats<T>* st, T* __restrict__ out) {
    extern __shared__ int32_t s_bins[];
    const int rw = kSlideBx + tw - 1, rh = kSlideBy + th - 1;  // region
    const int64_t j0 = int64_t(blockIdx.x) * kSlideBx, i0 = int64_t(blockIdx.y) * kSlideBy;
    const int64_t ri0 = i0 - th / 2, rj0 = j0 - tw / 2;
    const int tid = threadIdx.y * kSlideBx + threadIdx.x;
    for (int q = tid; q < rw * rh; q += kSlideBx * kSlideBy) {
        const int qr = q / rw, qc = q - qr * rw;
        const int64_t gi = ri0 + qr, gj = rj0 + qc;
        s_bins[q] = (gi >= 0 && gi < ny && gj >= 0 && gj < nx) ? __ldg(bins + gi * nx + gj) : -1;
    }
    __syncthreads();
    const int64_t i = i0 + threadIdx.y, j = j0 + threadIdx.x;
    if (i >= ny || j >= nx) return;
    const int64_t k = i * nx + j;
    const int32_t b = s_bins[(threadIdx.y + th / 2) * rw + threadIdx.x + tw / 2];
    if (b < 0) {
        out[k] = x[k];
        return;
    }
    const bool all_finite = st->count == (unsigned long long)(ny * nx);
    const uint32_t ub = uint32_t(b);
    uint32_t below = 0, valid = 0;
    for (int r = 0; r < th; ++r) {
        const int32_t* row = s_bins + (threadIdx.y + r) * rw + threadIdx.x;
        for (int c = 0; c < tw; ++c) below += uint32_t(row[c]) <= ub;
        if (!all_finite)
            for (int c = 0; c < tw; ++c) valid += row[c] >= 0;
    }
    if (all_finite) {  // the window clipped to the image
        const int64_t r0 = i - th / 2 < 0 ? 0 : i - th / 2;
        const int64_t r1 = i - th / 2 + th > ny ? ny : i - th / 2 + th;
        const int64_t c0 = j - tw / 2 < 0 ? 0 : j - tw / 2;
        const int64_t c1 = j - tw / 2 + tw > nx ? nx : j - tw / 2 + tw;
        valid = uint32_t((r1 - r0) * (c1 - c0));
    }
    out[k] = div_rn_(from_count<T>(below), from_count<T>(valid));
}

// The same counts with each thread ranking kSlideRows vertically adjacent
// pixels: their windows share all but kSlideRows - 1 rows, so every bin
// loaded from shared memory is compared with up to kSlideRows pixel bins
// (one load serves several compares, where sliding_smem_kernel loads each
// bin once per pixel).  A CTA covers 32 x (8 * kSlideRows) pixels.
constexpr int kSlideRows = 4;

template <typename T>
__global__ void __launch_bounds__(kSlideBx * kSlideBy)
sliding_smem_rows_kernel(const T* __restrict__ x, const int32_t* __restrict__ bins, int64_t ny,
                         int64_t nx, int th, int tw, const Stats<T>* st, T* __restrict__ out) {
    extern __shared__ int32_t s_bins[];
    constexpr int kTileY = kSlideBy * kSlideRows;
    const int rw = kSlideBx + tw - 1, rh = kTileY + th - 1;  // region
    const int64_t j0 = int64_t(blockIdx.x) * kSlideBx, i0 = int64_t(blockIdx.y) * kTileY;
    const int64_t ri0 = i0 - th / 2, rj0 = j0 - tw / 2;
    const int tid = threadIdx.y * kSlideBx + threadIdx.x;
    for (int q = tid; q < rw * rh; q += kSlideBx * kSlideBy) {
        const int qr = q / rw, qc = q - qr * rw;
        const int64_t gi = ri0 + qr, gj = rj0 + qc;
        s_bins[q] = (gi >= 0 && gi < ny && gj >= 0 && gj < nx) ? __ldg(bins + gi * nx + gj) : -1;
    }
    __syncthreads();
    const int64_t j = j0 + threadIdx.x;
    if (j >= nx) return;
    // this thread's pixels: rows ty0 .. ty0 + kSlideRows - 1 of the tile
    const int ty0 = threadIdx.y * kSlideRows;
    uint32_t ub[kSlideRows], below[kSlideRows];
#pragma unroll
    for (int k = 0; k < kSlideRows; ++k) {
        // -1 (a non-finite pixel, or a row below the image) ranks nothing
        // useful; its count is discarded below
        ub[k] = uint32_t(s_bins[(ty0 + k + th / 2) * rw + threadIdx.x + tw / 2]);
        below[k] = 0;
    }
    const bool all_finite = st->count == (unsigned long long)(ny * nx);
    // region row ty0 + r lies in the window of pixel k when k <= r < k + th
    uint32_t valid_acc[kSlideRows];
#pragma unroll
    for (int k = 0; k < kSlideRows; ++k) valid_acc[k] = 0;
    for (int r = 0; r < th + kSlideRows - 1; ++r) {
        const int32_t* row = s_bins + (ty0 + r) * rw + threadIdx.x;
        uint32_t cnt[kSlideRows];
#pragma unroll
        for (int k = 0; k < kSlideRows; ++k) cnt[k] = 0;
        uint32_t nvalid = 0;
        for (int c = 0; c < tw; ++c) {
            const uint32_t v = uint32_t(row[c]);
#pragma unroll
            for (int k = 0; k < kSlideRows; ++k) cnt[k] += v <= ub[k];
            if (!all_finite) nvalid += int32_t(v) >= 0;
        }
#pragma unroll
        for (int k = 0; k < kSlideRows; ++k) {
            const bool in = r >= k && r < k + th;
            below[k] += in ? cnt[k] : 0u;
            valid_acc[k] += in ? nvalid : 0u;
        }
    }
#pragma unroll
    for (int k = 0; k < kSlideRows; ++k) {
        const int64_t i = i0 + ty0 + k;
        if (i >= ny) break;
        const int64_t idx = i * nx + j;
        if (int32_t(ub[k]) < 0) {
            out[idx] = x[idx];
            continue;
        }
        uint32_t valid = valid_acc[k];
        if (all_finite) {  // the window clipped to the image
            const int64_t r0 = i - th / 2 < 0 ? 0 : i - th / 2;
            const int64_t r1 = i - th / 2 + th > ny ? ny : i - th / 2 + th;
            const int64_t c0 = j - tw / 2 < 0 ? 0 : j - tw / 2;
            const int64_t c1 = j - tw / 2 + tw > nx ? nx : j - tw / 2 + tw;
            valid = uint32_t((r1 - r0) * (c1 - c0));
        }
        out[idx] = div_rn_(from_count<T>(below[k]), from_count<T>(valid));
    }
}

// Sliding windows kept as running histograms.  Each thread owns one output
// column j and a run of `rows` consecutive output rows, and keeps the
// histogram of its current window in shared memory: the counts of bins 2m
// and 2m + 1 packed in word m (16 bits each, so a window holds at most
// 65535 cells), word m of thread t at s_hist[m * kHistThreads + t] (every
// lane of a warp in its own bank).  Moving down one row subtracts the
// window's top row and adds the row below it: 2 tw cells per pixel instead
// of the th tw cells that a full count reads.  The rank of the pixel's bin
// is the sum of the words below it (the packed halves add without carry,
// each half's total being at most the window's cell count) plus the pixel's
// own word.  Shared-memory atomics do the updates: their results are never
// read back, so they issue without waiting on one another.  ALL_FINITE:
// the image has no non-finite pixel, so every cell inside the image counts
// and the clipped window's area is the valid count.
constexpr int kHistThreads = 128;

template <typename T, bool ALL_FINITE>
__device__ __forceinline__ void sliding_hist_run(const T* __restrict__ x,
                                                 const int32_t* __restrict__ bins, int64_t ny,
                                                 int64_t nx, int th, int tw, int nbins, int rows,
                                                 T* __restrict__ out, uint32_t* s_hist) {
    const int words = (nbins + 1) / 2;
    const int t = threadIdx.x;
    uint32_t* hist = s_hist + t;
    for (int m = 0; m < words; ++m) hist[m * kHistThreads] = 0u;
    const int64_t j = int64_t(blockIdx.x) * kHistThreads + t;
    if (j >= nx) return;  // (each thread works on its own words only)
    const int64_t i0 = int64_t(blockIdx.y) * rows;
    const int64_t i1 = i0 + rows < ny ? i0 + rows : ny;
    // window columns [cl, cr) as 32-bit offsets (a row has fewer than 2^31)
    const int cl = int(j - tw / 2 < 0 ? 0 : j - tw / 2);
    const int cr = int(j - tw / 2 + tw > nx ? nx : j - tw / 2 + tw);
    int32_t nvalid = 0;
    // adds (SIGN 1) or removes (SIGN -1) one cell of bin b: word b / 2, half
    // b % 2.  A non-finite cell (b = -1, only when !ALL_FINITE) adds 0 to
    // word 0.  No branch: the atomics issue back to back.
    auto apply = [&](int32_t b, int sign) {
        uint32_t ub = uint32_t(b), inc;
        if (ALL_FINITE) {
            inc = (ub & 1u) * 0xFFFFu + 1u;
        } else {
            const bool ok = b >= 0;
            ub = ok ? ub : 0u;
            inc = ok ? (ub & 1u) * 0xFFFFu + 1u : 0u;
            nvalid += ok ? sign : 0;
        }
        uint32_t* w = hist + (ub >> 1) * kHistThreads;
        if (sign > 0) {
            atomicAdd(w, inc);
        } else {
            atomicSub(w, inc);
        }
    };
    // the window's cells of image row r (inside the image) enter it (sign 1)
    // or leave it (sign -1); the bins are loaded 8 columns at a time before
    // any is applied, so that 8 loads are in flight
    auto row_update = [&](int64_t r, int sign) {
        const int32_t* p = bins + r * nx;
        int c = cl;
        for (; c + 8 <= cr; c += 8) {
            int32_t b[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) b[k] = __ldg(p + c + k);
#pragma unroll
            for (int k = 0; k < 8; ++k) apply(b[k], sign);
        }
        for (; c < cr; ++c) apply(__ldg(p + c), sign);
    };
    // the first window: rows [i0 - th/2, i0 - th/2 + th) inside the image
    {
        const int64_t r0 = i0 - th / 2 < 0 ? 0 : i0 - th / 2;
        const int64_t r1 = i0 - th / 2 + th > ny ? ny : i0 - th / 2 + th;
        for (int64_t r = r0; r < r1; ++r) row_update(r, 1);
    }
    const int64_t c_span = int64_t(cr - cl);
    for (int64_t i = i0; i < i1; ++i) {
        if (i > i0) {
            const int64_t r_out = i - 1 - th / 2, r_in = i - th / 2 + th - 1;
            if (r_out >= 0) row_update(r_out, -1);
            if (r_in < ny) row_update(r_in, 1);
        }
        const int64_t k = i * nx + j;
        const int32_t b = __ldg(bins + k);
        if (!ALL_FINITE && b < 0) {
            out[k] = x[k];
            continue;
        }
        const uint32_t hb = uint32_t(b) >> 1;
        uint32_t a0 = 0, a1 = 0, a2 = 0, a3 = 0;
        uint32_t m = 0;
        for (; m + 4 <= hb; m += 4) {
            a0 += hist[m * kHistThreads];
            a1 += hist[(m + 1) * kHistThreads];
            a2 += hist[(m + 2) * kHistThreads];
            a3 += hist[(m + 3) * kHistThreads];
        }
        for (; m < hb; ++m) a0 += hist[m * kHistThreads];
        const uint32_t acc = a0 + a1 + a2 + a3;
        const uint32_t own = hist[hb * kHistThreads];
        const uint32_t below = (acc & 0xFFFFu) + (acc >> 16) + (own & 0xFFFFu) +
                               ((uint32_t(b) & 1u) ? (own >> 16) : 0u);
        uint32_t valid = uint32_t(nvalid);
        if (ALL_FINITE) {  // the window clipped to the image
            const int64_t r0 = i - th / 2 < 0 ? 0 : i - th / 2;
            const int64_t r1 = i - th / 2 + th > ny ? ny : i - th / 2 + th;
            valid = uint32_t((r1 - r0) * c_span);
        }
        out[k] = div_rn_(from_count<T>(below), from_count<T>(valid));
    }
}

template <typename T>
__global__ void __launch_bounds__(kHistThreads)
sliding_hist_kernel(const T* __restrict__ x, const int32_t* __restrict__ bins, int64_t ny,
                    int64_t nx, int th, int tw, int nbins, int rows, const Stats<T>* st,
                    T* __restrict__ out) {
    extern __shared__ uint32_t s_hist[];
    if (st->count == (unsigned long long)(ny * nx)) {
        sliding_hist_run<T, true>(x, bins, ny, nx, th, tw, nbins, rows, out, s_hist);
    } else {
        sliding_hist_run<T, false>(x, bins, ny, nx, th, tw, nbins, rows, out, s_hist);
    }
}

unsigned grid_for(int64_t n) {
    int64_t blocks = (n + 255) / 256;
    if (blocks > 152 * 8) blocks = 152 * 8;
    return unsigned(blocks < 1 ? 1 : blocks);
}

}  // namespace

size_t equalize_scratch_bytes(int64_t ny, int64_t nx, int64_t nbins, int strategy,
                              int64_t th, int64_t tw, size_t elem) {
    const int64_t n = ny * nx;
    auto up = [](size_t b) { return (b + 255) & ~size_t(255); };
    size_t total = up(sizeof(Stats<double>)) + up(size_t(n) * sizeof(int32_t));
    if (strategy == RLIC_EQUALIZE_GLOBAL) total += up(size_t(nbins) * 8);
    if (strategy == RLIC_EQUALIZE_TILE_INTERPOLATION) {
        const int64_t ntiles = ((ny + th - 1) / th) * ((nx + tw - 1) / tw);
        total += up(size_t(ntiles) * size_t(nbins) * elem);
        total += 2 * up(size_t(ny + nx) * sizeof(int32_t)) + up(size_t(ny + nx) * elem);
    }
    return total;
}

template <typename T>
cudaError_t launch_equalize_t(const T* x, int64_t ny, int64_t nx, int nbins, int strategy,
                              int64_t th, int64_t tw, T* out, void* scratch,
                              cudaStream_t stream) {
    const int64_t n = ny * nx;
    auto up = [](size_t b) { return (b + 255) & ~size_t(255); };
    unsigned char* base = static_cast<unsigned char*>(scratch);
    Stats<T>* st = reinterpret_cast<Stats<T>*>(base);
    int32_t* bins = reinterpret_cast<int32_t*>(base + up(sizeof(Stats<double>)));
    unsigned char* rest = base + up(sizeof(Stats<double>)) + up(size_t(n) * sizeof(int32_t));
    cudaError_t e = cudaSuccess;
    stats_init_kernel<T><<<1, 1, 0, stream>>>(st);
    count_launch();
    minmax_kernel<T><<<grid_for(n), 256, 0, stream>>>(x, n, st);
    count_launch();
    bins_kernel<T><<<grid_for(n), 256, 0, stream>>>(x, n, st, nbins, bins);
    count_launch();
    if (strategy == RLIC_EQUALIZE_GLOBAL) {
        unsigned long long* hist = reinterpret_cast<unsigned long long*>(rest);
        e = cudaMemsetAsync(hist, 0, size_t(nbins) * 8, stream);
        if (e != cudaSuccess) return e;
        const bool shared = nbins <= 12288;
        hist_kernel<<<grid_for(n), 256, shared ? size_t(nbins) * 4 : 0, stream>>>(
            bins, n, nbins, hist, shared);
        count_launch();
        scan_kernel<<<1, 1024, 0, stream>>>(hist, nbins);
        count_launch();
        map_global_kernel<T><<<grid_for(n), 256, 0, stream>>>(x, bins, n, hist, st, out);
        count_launch();
    } else if (strategy == RLIC_EQUALIZE_TILE_INTERPOLATION) {
        const int64_t nty = (ny + th - 1) / th, ntx = (nx + tw - 1) / tw;
        T* maps = reinterpret_cast<T*>(rest);
        const size_t smem = size_t(nbins) * 4;
        auto kfn = tile_maps_kernel<T>;
        if (smem > 48 * 1024) {
            e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
            if (e != cudaSuccess) return e;
        }
        kfn<<<unsigned(nty * ntx), 1024, smem, stream>>>(bins, ny, nx, th, tw, ntx, nbins, maps);
        count_launch();
        unsigned char* tab = rest + up(size_t(nty * ntx) * size_t(nbins) * sizeof(T));
        int32_t* a0 = reinterpret_cast<int32_t*>(tab);
        int32_t* a1 = reinterpret_cast<int32_t*>(tab + up(size_t(ny + nx) * sizeof(int32_t)));
        T* f = reinterpret_cast<T*>(tab + 2 * up(size_t(ny + nx) * sizeof(int32_t)));
        const int64_t longest = ny > nx ? ny : nx;
        axis_tables_kernel<T><<<dim3(unsigned((longest + 255) / 256), 2), 256, 0, stream>>>(
            ny, nx, th, tw, nty, ntx, a0, a1, f);
        count_launch();
        const int64_t gy = ny < 1024 ? ny : 1024;
        map_tiles_kernel<T><<<dim3(unsigned((nx + 255) / 256), unsigned(gy)), 256, 0, stream>>>(
            x, bins, ny, nx, ntx, nbins, a0, a1, f, maps, out);
        count_launch();
    } else if (nbins <= 256 && th * tw <= 65535 && nx < (int64_t(1) << 30)) {
        // running window histograms: one wave of CTAs, each sliding its
        // 128 columns down one run of rows (the first window of a run costs
        // th * tw cells, every later one 2 tw), runs of at least 32 rows
        const size_t smem = size_t((nbins + 1) / 2) * kHistThreads * 4;
        auto kfn = sliding_hist_kernel<T>;
        if (smem > 48 * 1024) {
            e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
            if (e != cudaSuccess) return e;
        }
        int dev = 0, sms = 0, per_sm = 0;
        e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, kHistThreads, smem);
        if (e != cudaSuccess) return e;
        const int64_t gx = (nx + kHistThreads - 1) / kHistThreads;
        int64_t gy = int64_t(sms) * (per_sm < 1 ? 1 : per_sm) / gx;
        const int64_t most = (ny + 31) / 32;
        gy = gy < 1 ? 1 : (gy > most ? most : gy);
        const int64_t rows = (ny + gy - 1) / gy;
        gy = (ny + rows - 1) / rows;
        kfn<<<dim3(unsigned(gx), unsigned(gy)), kHistThreads, smem, stream>>>(
            x, bins, ny, nx, int(th), int(tw), nbins, int(rows), st, out);
        count_launch();
    } else {
        const int64_t gy = (ny + 7) / 8;
        const int64_t gy_rows = (ny + kSlideBy * kSlideRows - 1) / (kSlideBy * kSlideRows);
        const size_t smem = size_t(kSlideBx + tw - 1) * size_t(kSlideBy + th - 1) * 4;
        const size_t smem_rows =
            size_t(kSlideBx + tw - 1) * size_t(kSlideBy * kSlideRows + th - 1) * 4;
        if (smem_rows <= 200 * 1024 && gy_rows <= 65535) {
            auto kfn = sliding_smem_rows_kernel<T>;
            if (smem_rows > 48 * 1024) {
                e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         int(smem_rows));
                if (e != cudaSuccess) return e;
            }
            kfn<<<dim3(unsigned((nx + kSlideBx - 1) / kSlideBx), unsigned(gy_rows)),
                  dim3(kSlideBx, kSlideBy), smem_rows, stream>>>(x, bins, ny, nx, int(th),
                                                                 int(tw), st, out);
        } else if (smem <= 200 * 1024 && gy <= 65535) {
            auto kfn = sliding_smem_kernel<T>;
            if (smem > 48 * 1024) {
                e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         int(smem));
                if (e != cudaSuccess) return e;
            }
            kfn<<<dim3(unsigned((nx + kSlideBx - 1) / kSlideBx), unsigned(gy)),
                  dim3(kSlideBx, kSlideBy), smem, stream>>>(x, bins, ny, nx, int(th), int(tw),
                                                            st, out);
        } else {
            const dim3 block(32, 8);
            const dim3 grid(unsigned((nx + 31) / 32), unsigned(gy < 65535 ? gy : 65535));
            sliding_kernel<T><<<grid, block, 0, stream>>>(x, bins, ny, nx, th, tw, st, out);
        }
        count_launch();
    }
    return cudaGetLastError();
}

cudaError_t launch_equalize(const float* x, int64_t ny, int64_t nx, int nbins, int strategy,
                            int64_t th, int64_t tw, float* out, void* scratch,
                            cudaStream_t stream) {
    return launch_equalize_t<float>(x, ny, nx, nbins, strategy, th, tw, out, scratch, stream);
}
cudaError_t launch_equalize(const double* x, int64_t ny, int64_t nx, int nbins, int strategy,
                            int64_t th, int64_t tw, double* out, void* scratch,
                            cudaStream_t stream) {
    return launch_equalize_t<double>(x, ny, nx, nbins, strategy, th, tw, out, scratch, stream);
}

}  // namespace rlic
