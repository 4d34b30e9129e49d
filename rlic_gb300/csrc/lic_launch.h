// lic_launch.h -- host-side interface between the C ABI and the kernels.
//
// One overload of each launcher per element type (float, double), defined in
// lic_kernels_f32.cu and lic_kernels_f64.cu.  All launchers are asynchronous
// on `stream` and return the launch status.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace rlic {

// Arithmetic variant: the reference's Cargo features (Cargo.toml:27-30) and
// the uv mode.
struct Variant {
    bool fma;
    bool branchless;
    bool pol;
};

// Image shape and boundary codes (x_left, x_right, y_left, y_right; 0 closed,
// 1 periodic).
struct Shape {
    int64_t ny, nx;
    int bnd[4];
    bool small_index() const { return ny * nx < (int64_t(1) << 31) - 1; }
};

// CTA shape in pixels.
struct LaunchConfig {
    int block_x, block_y;
    // traced passes only: launch the tiles [tile_begin, tile_begin +
    // tile_count) of the row-major tile grid (tile_count 0: all tiles)
    int64_t tile_begin = 0;
    int64_t tile_count = 0;
    // traced passes only: device flag that the pack kernels set when the
    // field holds a NaN sample (null: unknown, so every step checks)
    const unsigned* field_nan = nullptr;
    // traced passes only: trace each pixel's two half-streamlines on two
    // threads (lic_pass_paired_kernel), where the launch fits that form
    bool paired = false;
};

// What a traced pass does per step: sample the texture, sample and record the
// step codes, or record only (see lic_kernels.cuh).
constexpr int kPassSample = 0;
constexpr int kPassSampleRecord = 1;
constexpr int kPassRecordOnly = 2;

// Storage types of the reduced-precision form.
constexpr int kStorageFP16 = 0;
constexpr int kStorageBF16 = 1;

// Counts one kernel launch (rlic_kernel_launch_count).
void count_launch();

// Device address of a word that stays zero (lic_kernels_f32.cu), resolved
// once per device with that device current: the NaN flag of a field the
// caller promises holds no NaN sample.
const unsigned* zero_flag(cudaError_t* err);

// 32-bit words of step codes per pixel for a kernel of klen taps (8 steps of
// 4 bits per word, forward and backward halves padded separately).
inline int64_t code_words_per_pixel(int64_t klen) {
    const int64_t kmid = klen / 2;
    const int64_t nf = klen - kmid - 1;
    return (nf + 7) / 8 + (kmid + 7) / 8;
}

// Whether a traced pass over an image of npix pixels with CTAs of
// block_x x block_y pixels and a kernel of klen taps fits the paired form
// (lic_pass_paired_kernel: two threads per pixel, at most 128 threads per
// CTA, the backward samples of a CTA's pixels within 96 KiB of shared
// memory, 32-bit pixel indices, at least one tap per half).
constexpr int kPairedMaxThreadsHost = 128;
constexpr size_t kPairedSmemMax = 96 * 1024;
inline size_t paired_smem_bytes(int64_t klen, int npx, size_t elem) {
    const int64_t kmid = klen / 2;
    const int64_t nf = klen - kmid - 1;
    return elem * size_t(((nf + 7) & ~int64_t(7)) + ((kmid + 7) & ~int64_t(7))) +
           elem * size_t(kmid) * size_t(npx);
}
inline bool paired_launch_fits(int64_t npix, int block_x, int block_y, int64_t klen,
                               size_t elem) {
    const int npx = block_x * block_y;
    return npix < (int64_t(1) << 31) - 1 && klen >= 3 && klen <= (int64_t(1) << 20) &&
           npx % 16 == 0 && 2 * npx <= kPairedMaxThreadsHost &&
           paired_smem_bytes(klen, npx, elem) <= kPairedSmemMax;
}

#define RLIC_DECLARE_LAUNCHERS(T)                                                          \
    cudaError_t launch_pack(const T* u, const T* v, void* uv, int64_t n, cudaStream_t stream, \
                            unsigned* nan_flag = nullptr);                                 \
    cudaError_t launch_pass(const Variant& var, int mode, const T* tex_in, const void* uv,    \
                            const T* kernel, int klen, const Shape& sh,                    \
                            const LaunchConfig& lc, T* tex_out, uint32_t* codes,           \
                            cudaStream_t stream);                                          \
    cudaError_t launch_gather(bool fma, const T* tex_in, const uint32_t* codes,            \
                              const T* kernel, int klen, const Shape& sh,                  \
                              const LaunchConfig& lc, T* tex_out, cudaStream_t stream);    \
    cudaError_t launch_trace_cells(const Variant& var, const T* type_tag, const void* uv,  \
                                   const Shape& sh, int klen, int64_t npix,                \
                                   const int64_t* pix, int64_t* cells, cudaStream_t stream); \
    cudaError_t launch_lowp_prepare(const T* kernel, int klen, int64_t iterations,         \
                                    float* w32, float* inv_scale, double* undo,            \
                                    cudaStream_t stream);                                  \
    cudaError_t launch_to_storage(const T* src, void* dst, int storage, int64_t n,         \
                                  cudaStream_t stream);                                    \
    cudaError_t launch_from_storage(const void* src, int storage, const double* undo,      \
                                    T* dst, int64_t n, cudaStream_t stream);               \
    cudaError_t launch_check_negative(const T* x, int64_t n, unsigned* flag,               \
                                      cudaStream_t stream); /* flag zeroed by the caller */ \
    cudaError_t launch_pack_strided(const T* u, int64_t su0, int64_t su1, const T* v,      \
                                    int64_t sv0, int64_t sv1, void* uv, int64_t ny,        \
                                    int64_t nx, cudaStream_t stream,                       \
                                    unsigned* nan_flag = nullptr);                         \
    cudaError_t launch_gather_strided(const T* src, int64_t s0, int64_t s1, T* dst,        \
                                      int64_t ny, int64_t nx, cudaStream_t stream,         \
                                      unsigned* neg_flag = nullptr);                       \
    cudaError_t launch_scatter(const T* g, const uint32_t* codes, const T* kernel,         \
                               int klen, const Shape& sh, T* y, cudaStream_t stream);      \
    cudaError_t launch_kernel_grad(const T* g, const T* x, const uint32_t* codes,          \
                                   int klen, const Shape& sh, double* dw,                  \
                                   cudaStream_t stream);

RLIC_DECLARE_LAUNCHERS(float)
RLIC_DECLARE_LAUNCHERS(double)

// Reduced-precision replay (lic_lowp.cu): `tex_in`/`tex_out` hold FP16 or
// BF16 cells (`storage`), w32 the float kernel in natural order.
cudaError_t launch_gather_lowp(int storage, const void* tex_in, const uint32_t* codes,
                               const float* w32, int klen, const float* inv_scale,
                               const Shape& sh, const LaunchConfig& lc, void* tex_out,
                               cudaStream_t stream);

// Replayed pass with the texture staged in shared memory by TMA copies
// (lic_stage.cu).  Returns cudaErrorNotSupported, before launching anything,
// when the image or the kernel does not fit the staged form (rows not
// 16-byte multiples, an unaligned texture, a box beyond the copy limits,
// images of 2^31 pixels or more); the caller then uses launch_gather.
// field_nan: the packed field's NaN flag (null: unknown; codes may then
// hold stop codes).
cudaError_t launch_gather_staged(bool fma, const float* tex_in, const uint32_t* codes,
                                 const float* kernel, int klen, const Shape& sh,
                                 const unsigned* field_nan, float* tex_out, cudaStream_t stream);
cudaError_t launch_gather_staged(bool fma, const double* tex_in, const uint32_t* codes,
                                 const double* kernel, int klen, const Shape& sh,
                                 const unsigned* field_nan, double* tex_out,
                                 cudaStream_t stream);
// The reduced-precision replay (FP16/BF16 cells, FP32 compensated sums)
// with the same staging; cudaErrorNotSupported as above (rows must be a
// multiple of 16 bytes of storage cells).
cudaError_t launch_gather_staged_lowp(int storage, const void* tex_in, const uint32_t* codes,
                                      const float* w32, int klen, const float* inv_scale,
                                      const Shape& sh, const unsigned* field_nan,
                                      void* tex_out, cudaStream_t stream);
// Super-tile height of the staged replay, in pixels (a multiple of 4).
void set_stage_rows(int rows);
// Whether a staged replay ever gave up waiting for its copy.
cudaError_t stage_timeout_seen(bool* seen);

// Self-check of the screened float64 division (lic_kernels_f64.cu).
cudaError_t launch_quotient_check(const double* a, const double* b, int64_t n, double* q,
                                  int32_t* certified, cudaStream_t stream);
// Self-check of the float64 step's integer numerator (lic_kernels_f64.cu).
cudaError_t launch_numerator_check(const double* f, int64_t n, double* g, int32_t* in_range,
                                   cudaStream_t stream);

#undef RLIC_DECLARE_LAUNCHERS

}  // namespace rlic
