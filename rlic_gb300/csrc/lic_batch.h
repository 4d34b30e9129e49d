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
};

// The instances taking part in one pass level, with the first tile of each
// in the level's 1-D grid.
struct BatchLevel {
    const int64_t* tile_start;
    const int* instance;
    int count;
    int64_t total_tiles;
};

cudaError_t launch_batch_pack(const BatchInstance* dev, int count, int64_t max_pixels,
                              cudaStream_t stream);
cudaError_t launch_batch_level(const BatchInstance* dev, const BatchLevel& lv, int level,
                               cudaStream_t stream);

}  // namespace rlic
