// lic_equalize.h -- histogram equalization launchers (lic_equalize.cu).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace rlic {

// Largest bin counts: tile histograms live in shared memory (4 bytes a bin);
// bins are exact in float32 up to 2^24.
constexpr int64_t kEqualizeMaxBins = int64_t(1) << 24;
constexpr int64_t kEqualizeMaxTileBins = 49152;

// Device scratch of one equalization: statistics, the bin of every pixel,
// and the global histogram or the tiles' mappings.
size_t equalize_scratch_bytes(int64_t ny, int64_t nx, int64_t nbins, int strategy, int64_t th,
                              int64_t tw, size_t elem);

cudaError_t launch_equalize(const float* x, int64_t ny, int64_t nx, int nbins, int strategy,
                            int64_t th, int64_t tw, float* out, void* scratch,
                            cudaStream_t stream);
cudaError_t launch_equalize(const double* x, int64_t ny, int64_t nx, int nbins, int strategy,
                            int64_t th, int64_t tw, double* out, void* scratch,
                            cudaStream_t stream);

}  // namespace rlic
