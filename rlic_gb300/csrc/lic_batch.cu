// lic_batch.cu -- the batched form: many independent float32 convolutions,
// of uneven sizes, kernel lengths, boundaries, uv modes and iteration counts,
// run together, one kernel launch per pass level over all of them.
//
// Level 1 is the traced pass of every instance (recording its path cache when
// it has two or more iterations); level L >= 2 replays instances that have at
// least L iterations.  Each level's launch covers the tiles of all its
// instances in one 1-D grid: a CTA finds its instance by binary search over
// the level's tile prefix sums (kept in shared memory), then loads that
// instance's weights and delta table.  Tile shapes (tile_x x tile_y = 256
// pixels) may differ per instance.  The arithmetic is the default build's
// (features `fma` + `branchless`), bit-identical to rlic_convolve_f32.
#include "lic_batch.h"
#include "lic_kernels.cuh"

namespace rlic {

namespace {

constexpr int kMaxBatchInSmem = 1024;  // instances per level resolved in shared memory

// Instance of the level's CTA: binary search of `tile` in starts[0..m).
__device__ __forceinline__ int find_instance(const int64_t* starts, int m, int64_t tile) {
    int lo = 0, hi = m - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (starts[mid] <= tile) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ float* level_dst(const BatchInstance& b, int level) {
    return ((b.iterations - level) % 2 == 0) ? b.out : b.tmp;
}

__device__ __forceinline__ const float* level_src(const BatchInstance& b, int level) {
    return level == 1 ? b.texture : level_dst(b, level - 1);
}

// Stages the level's (instance, first tile) table into shared memory.
__device__ __forceinline__ int load_level(const BatchLevel& lv, int64_t* starts, int* index) {
    const int m = lv.count;
    for (int k = threadIdx.x; k < m; k += blockDim.x) {
        starts[k] = lv.tile_start[k];
        index[k] = lv.instance[k];
    }
    __syncthreads();
    return m;
}

__global__ void __launch_bounds__(256)
batch_pass_kernel(const BatchInstance* __restrict__ insts, BatchLevel lv) {
    __shared__ int64_t starts[kMaxBatchInSmem];
    __shared__ int index[kMaxBatchInSmem];
    __shared__ __align__(16) float wsm[2 * kBatchMaxHalf];
    const int m = load_level(lv, starts, index);
    const int64_t tile = blockIdx.x;
    const int slot = find_instance(starts, m, tile);
    const BatchInstance& b = insts[index[slot]];
    const int64_t local = tile - starts[slot];
    const int klen = b.klen;
    const int kmid = klen / 2;
    const int nf = klen - kmid - 1;
    const int nf_pad = (nf + 7) & ~7;
    load_step_weights(wsm, b.kernel, klen, nf_pad);
    __syncthreads();
    Geometry<int32_t> g;
    g.ny = b.ny;
    g.nx = b.nx;
    g.ax = make_axis<int32_t>(b.nx, b.bnd[0], b.bnd[1]);
    g.ay = make_axis<int32_t>(b.ny, b.bnd[2], b.bnd[3]);
    TileGrid<int32_t> tg;
    tg.bx = b.tile_x;
    tg.by = b.tile_y;
    tg.tiles_x = b.tiles_x;
    tg.ntiles = b.ntiles;
    tg.radius = kmid;
    CodeLayout cl;
    cl.npix = int64_t(b.ny) * b.nx;
    cl.words_f = (nf + 7) / 8;
    const int ti = int(local / b.tiles_x);
    const int tj = int(local - int64_t(ti) * b.tiles_x);
    const int tid = threadIdx.x;
    const int i = ti * b.tile_y + tid / b.tile_x;
    const int j = tj * b.tile_x + tid % b.tile_x;
    const float wmid = __ldg(b.kernel + kmid);
    const float* src = level_src(b, 1);
    const auto* uv = reinterpret_cast<const float2*>(b.uv);
    const bool record = b.iterations >= 2;
    const bool interior = tile_is_interior(ti, tj, tg, g);
    if (!interior && (i >= b.ny || j >= b.nx)) return;
    // interior tiles of a field without NaN samples skip the per-step NaN test
    const bool fast = interior && __ldg(b.nan_flag) == 0u;
    float acc;
#define RLIC_BATCH_PIXEL(POL, EDGE, MODE, CHECK)                                           \
    acc = convolve_pixel<float, true, true, POL, EDGE, MODE, int32_t, CHECK>(               \
        i, j, g, uv, src, wsm, wsm + nf_pad, wmid, nf, kmid, b.codes, cl)
    if (b.pol) {
        if (record) {
            if (fast) RLIC_BATCH_PIXEL(true, false, kSampleRecord, false);
            else if (interior) RLIC_BATCH_PIXEL(true, false, kSampleRecord, true);
            else RLIC_BATCH_PIXEL(true, true, kSampleRecord, true);
        } else {
            if (fast) RLIC_BATCH_PIXEL(true, false, kSample, false);
            else if (interior) RLIC_BATCH_PIXEL(true, false, kSample, true);
            else RLIC_BATCH_PIXEL(true, true, kSample, true);
        }
    } else {
        if (record) {
            if (fast) RLIC_BATCH_PIXEL(false, false, kSampleRecord, false);
            else if (interior) RLIC_BATCH_PIXEL(false, false, kSampleRecord, true);
            else RLIC_BATCH_PIXEL(false, true, kSampleRecord, true);
        } else {
            if (fast) RLIC_BATCH_PIXEL(false, false, kSample, false);
            else if (interior) RLIC_BATCH_PIXEL(false, false, kSample, true);
            else RLIC_BATCH_PIXEL(false, true, kSample, true);
        }
    }
#undef RLIC_BATCH_PIXEL
    level_dst(b, 1)[int64_t(i) * b.nx + j] = acc;
}

__global__ void __launch_bounds__(256)
batch_gather_kernel(const BatchInstance* __restrict__ insts, BatchLevel lv, int level) {
    __shared__ int64_t starts[kMaxBatchInSmem];
    __shared__ int index[kMaxBatchInSmem];
    __shared__ __align__(16) float wsm[2 * kBatchMaxHalf];
    __shared__ int32_t table[16];
    const int m = load_level(lv, starts, index);
    const int64_t tile = blockIdx.x;
    const int slot = find_instance(starts, m, tile);
    const BatchInstance& b = insts[index[slot]];
    const int64_t local = tile - starts[slot];
    const int klen = b.klen;
    const int kmid = klen / 2;
    const int nf = klen - kmid - 1;
    const int nf_pad = (nf + 7) & ~7;
    load_step_weights(wsm, b.kernel, klen, nf_pad);
    if (threadIdx.x == 0) fill_delta_table(table, int32_t(b.nx), int32_t(b.ny));
    __syncthreads();
    const int ti = int(local / b.tiles_x);
    const int tj = int(local - int64_t(ti) * b.tiles_x);
    const int tid = threadIdx.x;
    const int i = ti * b.tile_y + tid / b.tile_x;
    const int j = tj * b.tile_x + tid % b.tile_x;
    if (i >= b.ny || j >= b.nx) return;
    const int64_t npix = int64_t(b.ny) * b.nx;
    const int p = i * b.nx + j;
    const float* src = level_src(b, level);
    float acc = accumulate<float, true>(__ldg(b.kernel + kmid), __ldg(src + p), 0.f);
    replay_half<float, true, int32_t>(acc, p, b.codes + p, npix, nf, wsm, table, src);
    replay_half<float, true, int32_t>(acc, p, b.codes + size_t((nf + 7) / 8) * npix + p, npix,
                                      kmid, wsm + nf_pad, table, src);
    level_dst(b, level)[p] = acc;
}

// Packs (u, v) of every instance: blockIdx.y selects the instance.
__global__ void batch_pack_kernel(const BatchInstance* __restrict__ insts) {
    const BatchInstance& b = insts[blockIdx.y];
    const int64_t n = int64_t(b.ny) * b.nx;
    float2* uv = static_cast<float2*>(b.uv);
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    bool nan = false;
    for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n; k += stride) {
        const float2 p = make_float2(b.u[k], b.v[k]);
        nan |= isnan(p.x) || isnan(p.y);
        uv[k] = p;
    }
    if (nan) atomicOr(b.nan_flag, 1u);
}

}  // namespace

cudaError_t launch_batch_pack(const BatchInstance* dev, int count, int64_t max_pixels,
                              cudaStream_t stream) {
    if (count <= 0) return cudaSuccess;
    if (count > 65535) return cudaErrorInvalidConfiguration;
    int64_t bx = (max_pixels + 255) / 256;
    if (bx > 512) bx = 512;
    if (bx < 1) bx = 1;
    batch_pack_kernel<<<dim3(unsigned(bx), unsigned(count)), 256, 0, stream>>>(dev);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_batch_level(const BatchInstance* dev, const BatchLevel& lv, int level,
                               cudaStream_t stream) {
    if (lv.count <= 0 || lv.total_tiles <= 0) return cudaSuccess;
    if (lv.count > kMaxBatchInSmem || lv.total_tiles > 0x7fffffffLL)
        return cudaErrorInvalidConfiguration;
    if (level == 1)
        batch_pass_kernel<<<unsigned(lv.total_tiles), 256, 0, stream>>>(dev, lv);
    else
        batch_gather_kernel<<<unsigned(lv.total_tiles), 256, 0, stream>>>(dev, lv, level);
    count_launch();
    return cudaGetLastError();
}

}  // namespace rlic
