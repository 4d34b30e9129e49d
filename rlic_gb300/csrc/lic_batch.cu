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

// Tile `local` of instance b's traced pass (level 1), by the CTA's 256
// threads; `wsm` receives the weights (the caller synchronises after).
// NC: read the field and texture through the read-only cache (they do not
// change during the launch); false in the persistent kernel, where the pack
// of the same launch wrote the field.
template <bool NC>
__device__ __forceinline__ void trace_tile(const BatchInstance& b, int64_t local, float* wsm) {
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
    const bool fast = interior && *reinterpret_cast<const volatile unsigned*>(b.nan_flag) == 0u;
    float acc;
#define RLIC_BATCH_PIXEL(POL, EDGE, MODE, CHECK)                                           \
    acc = convolve_pixel<float, true, true, POL, EDGE, MODE, int32_t, CHECK, NC>(           \
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

// Loads instance b's step weights and delta table into shared memory (the
// caller synchronises after).
__device__ __forceinline__ void replay_setup(const BatchInstance& b, float* wsm, int32_t* table) {
    const int kmid = b.klen / 2;
    const int nf = b.klen - kmid - 1;
    load_step_weights(wsm, b.kernel, b.klen, (nf + 7) & ~7);
    if (threadIdx.x == 0) fill_delta_table(table, int32_t(b.nx), int32_t(b.ny));
}

// Tile `local` of instance b's replayed pass at `level` (weights and delta
// table already in shared memory).
template <bool NC>
__device__ __forceinline__ void replay_tile(const BatchInstance& b, int64_t local, int level,
                                            const float* wsm, const int32_t* table) {
    const int klen = b.klen;
    const int kmid = klen / 2;
    const int nf = klen - kmid - 1;
    const int nf_pad = (nf + 7) & ~7;
    const int ti = int(local / b.tiles_x);
    const int tj = int(local - int64_t(ti) * b.tiles_x);
    const int tid = threadIdx.x;
    const int i = ti * b.tile_y + tid / b.tile_x;
    const int j = tj * b.tile_x + tid % b.tile_x;
    if (i >= b.ny || j >= b.nx) return;
    const int64_t npix = int64_t(b.ny) * b.nx;
    const int p = i * b.nx + j;
    const float* src = level_src(b, level);
    float acc = accumulate<float, true>(__ldg(b.kernel + kmid), ld_in<NC>(src + p), 0.f);
    replay_half<float, true, int32_t, NC>(acc, p, b.codes + p, npix, nf, wsm, table, src);
    replay_half<float, true, int32_t, NC>(acc, p, b.codes + size_t((nf + 7) / 8) * npix + p,
                                          npix, kmid, wsm + nf_pad, table, src);
    level_dst(b, level)[p] = acc;
}

__global__ void __launch_bounds__(256)
batch_pass_kernel(const BatchInstance* __restrict__ insts, BatchLevel lv) {
    __shared__ int64_t starts[kMaxBatchInSmem];
    __shared__ int index[kMaxBatchInSmem];
    __shared__ __align__(16) float wsm[2 * kBatchMaxHalf];
    const int m = load_level(lv, starts, index);
    const int64_t tile = blockIdx.x;
    const int slot = find_instance(starts, m, tile);
    trace_tile<true>(insts[index[slot]], tile - starts[slot], wsm);
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
    replay_setup(b, wsm, table);
    __syncthreads();
    replay_tile<true>(b, tile - starts[slot], level, wsm, table);
}

// ------------------------------------------------- persistent work queue --
//
// One launch runs the whole batch.  Every CTA loops: it takes the next item
// number from the queue counter (the number for its following item is
// requested while the current one runs), finds the item's segment, and,
// unless the segment is a pack, waits until the segment it reads from has
// finished (thread 0 polls that segment's counter, bounded, then fences).
// Item numbers are handed out in order and an item only ever waits for items
// with smaller numbers, each held by a CTA that is already running, so the
// waits always end; the bound only guards against a fault.  Data written by
// other CTAs of the launch (the packed field, codes, the previous level's
// texture) is read with plain coherent loads after the fence, never through
// the read-only cache.

// Minimum resident CTAs per SM requested from the register allocator for
// the persistent kernel (its registers are those of its costliest path, the
// traced pass; the replays run at the same occupancy).
// 6 (at most 40 registers): measured fastest of 4 (64 registers, the
// compiler's choice), 5 and 6 on the 64-instance and 256-small-instance
// mixes (small mix 19.4 / 11.7 / 11.7 ms, 64-instance mix 199 / 105 / 102 ms).
#ifndef RLIC_BATCH_QUEUE_MIN_BLOCKS
#define RLIC_BATCH_QUEUE_MIN_BLOCKS 6
#endif

constexpr int kQueueSegSmem = 2048;          // segment starts kept in shared memory
constexpr uint32_t kQueueWaitLimit = 1u << 24;  // polls, 128 ns apart

__device__ __forceinline__ int find_segment(const int* starts, int nseg, int item) {
    int lo = 0, hi = nseg - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (starts[mid] <= item) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__global__ void __launch_bounds__(256, RLIC_BATCH_QUEUE_MIN_BLOCKS)
batch_queue_kernel(const BatchInstance* __restrict__ insts, BatchQueue q) {
    __shared__ int seg_start_s[kQueueSegSmem + 1];
    __shared__ __align__(16) float wsm[2 * kBatchMaxHalf];
    __shared__ int32_t table[16];
    __shared__ int cur_item, next_item, cur_seg, stop;
    const int tid = threadIdx.x;
    const bool in_smem = q.nseg <= kQueueSegSmem;
    if (in_smem)
        for (int k = tid; k <= q.nseg; k += blockDim.x) seg_start_s[k] = q.seg_start[k];
    if (tid == 0) {
        next_item = int(atomicAdd(q.next, 1u));
        stop = 0;
    }
    __syncthreads();
    const int* starts = in_smem ? seg_start_s : q.seg_start;
    for (;;) {
        if (tid == 0) {
            const int item = next_item;
            cur_item = item;
            if (item < q.total) {
                next_item = int(atomicAdd(q.next, 1u));  // in flight while this item runs
                const int s = find_segment(starts, q.nseg, item);
                cur_seg = s;
                const int prev = q.segs[s].prev;
                if (prev >= 0) {
                    const unsigned need = unsigned(q.segs[prev].nitems);
                    const volatile unsigned* d = q.done + prev;
                    uint32_t polls = 0;
                    while (*d < need) {
                        if (++polls > kQueueWaitLimit) {
                            atomicExch(q.timeout, 1u);
                            stop = 1;
                            break;
                        }
                        __nanosleep(128);
                    }
                    __threadfence();  // acquire: the previous level's writes are visible
                }
            }
        }
        __syncthreads();
        if (cur_item >= q.total || stop) break;
        const BatchSegment seg = q.segs[cur_seg];
        const int64_t local = cur_item - starts[cur_seg];
        const BatchInstance& b = insts[seg.inst];
        if (seg.level == 0) {
            // pack: pixels [local * chunk, (local + 1) * chunk) of the field
            const int64_t n = int64_t(b.ny) * b.nx;
            const int64_t p0 = local * kBatchPackChunk;
            const int64_t p1 = p0 + kBatchPackChunk < n ? p0 + kBatchPackChunk : n;
            float2* uv = static_cast<float2*>(b.uv);
            bool nan = false;
            for (int64_t k = p0 + tid; k < p1; k += blockDim.x) {
                const float2 v2 = make_float2(__ldg(b.u + k), __ldg(b.v + k));
                nan |= isnan(v2.x) || isnan(v2.y);
                uv[k] = v2;
            }
            if (nan) atomicOr(b.nan_flag, 1u);
        } else if (seg.level == 1) {
            trace_tile<false>(b, local, wsm);
        } else {
            replay_setup(b, wsm, table);
            __syncthreads();
            const int64_t t0 = local * b.replay_tiles;
            const int64_t t1 =
                t0 + b.replay_tiles < int64_t(b.ntiles) ? t0 + b.replay_tiles : int64_t(b.ntiles);
            for (int64_t t = t0; t < t1; ++t) replay_tile<false>(b, t, seg.level, wsm, table);
        }
        __syncthreads();  // the item's stores (and shared-memory reads) are done
        if (tid == 0) {
            __threadfence();  // release the item's stores before counting it
            atomicAdd(q.done + cur_seg, 1u);
        }
    }
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

cudaError_t launch_batch_queue(const BatchInstance* dev, const BatchQueue& q,
                               cudaStream_t stream) {
    if (q.total <= 0) return cudaSuccess;
    unsigned grid = 0;
    cudaError_t e = persistent_grid(batch_queue_kernel, 256, 0, q.total, &grid);
    if (e != cudaSuccess) return e;
    batch_queue_kernel<<<grid, 256, 0, stream>>>(dev, q);
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
