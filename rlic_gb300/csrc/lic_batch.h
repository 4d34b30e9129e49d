// lic_batch.h -- device-side tables of the batched form (lic_batch.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace rlic {

// Longest half-trace (steps) the batched kernels keep in shared memory:
// kernels of up to 2 * kBatchMaxHalf + 1 taps.
constexpr int kBatchMaxHalf = 512;

// One instance as the kernels see it (built by the host, copied to the
// device).  Buffers: `out` and `tmp` alternate between passes so that the
// last pass writes `out`; `uv` and `codes` are the packed field and the path
// cache (codes only for two or more iterations).
struct BatchInstance {
    const float* texture;
    const float* u;
    const float* v;
    const float* kernel;
    float* out;
    float* tmp;
    void* uv;
    uint32_t* codes;
    unsigned* nan_flag;  // set by the pack when the field holds a NaN sample
    int ny, nx, klen, iterations, pol;
    int bnd[4];
    int tile_x, tile_y, tiles_x, ntiles;
    int replay_tiles;  // tiles per replay work item of the persistent kernel
};

// The instances taking part in one pass level, with the first tile of each
// in the level's 1-D grid.
struct BatchLevel {
    const int64_t* tile_start;
    const int* instance;
    int count;
    int64_t total_tiles;
};

// The work queue of the persistent batched kernel.  The work of a batch is
// cut into segments, one per (instance, level): level 0 packs the instance's
// field in chunks of kBatchPackChunk pixels, level 1 traces it tile by tile,
// level L >= 2 replays it, replay_tiles tiles per work item.  Segments are
// ordered level by level (largest instances first within a level) and their
// items numbered consecutively; CTAs take item numbers from a counter in
// order, and the items of a segment wait until every item of the segment
// they read from (the same instance's previous level) has finished.
constexpr int kBatchPackChunk = 8192;

struct BatchSegment {
    int inst;     // instance
    int level;    // 0 pack, 1 traced pass, >= 2 replay
    int prev;     // segment this one reads (-1: none)
    int nitems;   // work items
};

struct BatchQueue {
    const int* seg_start;           // first item of every segment, nseg + 1 entries
    const BatchSegment* segs;
    int nseg;
    int total;                      // items of the whole batch
    unsigned* next;                 // next item to take (zeroed before the launch)
    unsigned* done;                 // finished items per segment (zeroed)
    unsigned* timeout;              // set when a wait gave up (zeroed)
};

cudaError_t launch_batch_pack(const BatchInstance* dev, int count, int64_t max_pixels,
                              cudaStream_t stream);
// One persistent launch that runs the whole queue.
cudaError_t launch_batch_queue(const BatchInstance* dev, const BatchQueue& q,
                               cudaStream_t stream);
cudaError_t launch_batch_level(const BatchInstance* dev, const BatchLevel& lv, int level,
                               cudaStream_t stream);

}  // namespace rlic
