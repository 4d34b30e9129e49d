/*
 * rlic_gb300.h -- C ABI of the GB300 (sm_103a) line integral convolution core.
 *
 * This library replaces the native module of neutrinoceros/rlic, whose only
 * entry points are the PyO3 functions
 *
 *     rlic._core.convolve_f32(texture, (u, v, uv_mode), kernel,
 *                             ((x_left, x_right), (y_left, y_right)), iterations)
 *     rlic._core.convolve_f64(...)                        (src/lib.rs:448-485,
 *                                                          src/rlic/_core.pyi:8-29)
 *
 * The Python layer (rlic_gb300/_lib.py, mirroring src/rlic/_lib.py:37-235)
 * validates every argument before it calls into this ABI, exactly as the
 * reference validates before calling its native module.  This ABI still
 * checks its arguments and returns an error code instead of aborting.
 *
 * Conventions
 *   - Images are C-order (row-major) arrays of ny rows by nx columns:
 *     element (i, j) sits at index i * nx + j.  i runs along y (rows, v),
 *     j along x (columns, u), as in src/lib.rs:47-51.
 *   - All pointers are CUDA device pointers unless RLIC_FLAG_HOST_MEMORY is
 *     set, in which case texture, u, v, kernel and out are host pointers and
 *     the call copies them to and from the device and returns after the result
 *     is back in `out`; a NULL stream then means the calling thread's
 *     per-thread default stream, so host-memory calls from several threads
 *     overlap on the device.  Without that flag the call is asynchronous on
 *     `stream` (a cudaStream_t; NULL means the legacy default stream).
 *   - `out` must not overlap any input.  Inputs are never written.
 *   - Return value: RLIC_OK or an RLIC_ERR_* code; rlic_last_error() then
 *     describes the failure (thread-local).
 *   - Arithmetic reproduces the reference's default build (Cargo features
 *     `fma` and `branchless`, Cargo.toml:27-30) bit for bit.  The other three
 *     feature combinations are selected with RLIC_FLAG_NO_FMA and
 *     RLIC_FLAG_NO_BRANCHLESS.
 */
#ifndef RLIC_GB300_H
#define RLIC_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define RLIC_API __attribute__((visibility("default")))
#else
#define RLIC_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define RLIC_OK 0
#define RLIC_ERR_INVALID_ARGUMENT 1
#define RLIC_ERR_CUDA 2
#define RLIC_ERR_OUT_OF_MEMORY 3
#define RLIC_ERR_WORKSPACE_TOO_SMALL 4
#define RLIC_ERR_NEGATIVE_TEXTURE 5
#define RLIC_ERR_UNSUPPORTED 6

/* uv_mode: src/lib.rs:14-27 ("velocity" / "polarization") */
#define RLIC_UV_VELOCITY 0
#define RLIC_UV_POLARIZATION 1

/* boundary kinds: src/lib.rs:56-67 ("closed" / "periodic") */
#define RLIC_BOUNDARY_CLOSED 0
#define RLIC_BOUNDARY_PERIODIC 1

/* flags */
#define RLIC_FLAG_HOST_MEMORY 0x1u   /* array pointers are host memory            */
#define RLIC_FLAG_NO_FMA 0x2u        /* reference built without feature `fma`       */
#define RLIC_FLAG_NO_BRANCHLESS 0x4u /* reference built without feature `branchless` */
#define RLIC_FLAG_NO_PATH_CACHE 0x8u /* trace every streamline in every pass          */
#define RLIC_FLAG_CHECK_TEXTURE 0x20u /* with HOST_MEMORY: fail if texture has x < 0   */
#define RLIC_FLAG_FIELD_NAN_FREE 0x40u /* rlic_sweep_*: the packed field has no NaN   */

/* Library version string. */
RLIC_API const char *rlic_version(void);

/* Description of the last error raised on the calling thread ("" if none). */
RLIC_API const char *rlic_last_error(void);

/*
 * Device scratch, in bytes, that rlic_convolve_f32/_f64 need for an image of
 * ny x nx elements of `elem_bytes` (4 or 8) bytes, a kernel of klen taps,
 * `iterations` passes and the given flags: the packed (u, v) field, for two
 * or more iterations one ping-pong texture buffer, (unless
 * RLIC_FLAG_NO_PATH_CACHE) the path cache for two or more iterations, a
 * copy of the kernel and a flag that records whether the field holds a NaN
 * sample.
 * 0 on invalid arguments.
 */
RLIC_API size_t rlic_workspace_bytes(int64_t ny, int64_t nx, int64_t klen, int64_t iterations,
                                     int elem_bytes, unsigned flags);

/*
 * Bytes of the path cache of an ny x nx image and a kernel of klen taps:
 * 4 bits per streamline step, 8 steps per 32-bit word, each half of the
 * kernel padded to whole words.
 */
RLIC_API size_t rlic_path_code_bytes(int64_t ny, int64_t nx, int64_t klen);

/*
 * Line integral convolution, `iterations` passes.
 *
 * Replaces rlic._core.convolve_f32 / convolve_f64 (src/lib.rs:451-482), i.e.
 * convolve_iteratively (src/lib.rs:408-443): the texture is convolved along
 * the streamlines of (u, v) with `kernel`, and each pass feeds its output to
 * the next one.  iterations == 0 writes zeros to `out`, as the native core
 * does (src/lib.rs:425, 433); the Python layer returns a copy of the texture
 * instead, before it reaches this call (src/rlic/_lib.py:208-209).
 *
 *   texture, u, v   ny x nx, C-order
 *   kernel          klen taps; the first klen/2 weight the backward half of
 *                   the streamline, the last klen - klen/2 - 1 the forward half
 *   uv_mode         RLIC_UV_VELOCITY or RLIC_UV_POLARIZATION
 *   bx_left, bx_right, by_left, by_right
 *                   RLIC_BOUNDARY_CLOSED or RLIC_BOUNDARY_PERIODIC for each
 *                   side of each axis (x = columns, y = rows).  Any
 *                   combination is computed; the Python layer rejects a
 *                   periodic side facing a different one.
 *   out             ny x nx result
 *   flags           RLIC_FLAG_* bits.  With two or more iterations the first
 *                   pass records every streamline step (4 bits each) and the
 *                   later passes replay the record instead of re-tracing
 *                   (the path of a pixel depends on u, v and the kernel
 *                   length only); RLIC_FLAG_NO_PATH_CACHE traces every pass.
 *                   Both give identical results.
 *                   RLIC_FLAG_CHECK_TEXTURE (with RLIC_FLAG_HOST_MEMORY) tests
 *                   the texture for elements below zero on the device, as
 *                   src/rlic/_lib.py:174-179 does on the host, and returns
 *                   RLIC_ERR_NEGATIVE_TEXTURE (`out` then undefined).
 *                   With RLIC_FLAG_HOST_MEMORY on a device that can access
 *                   pageable host memory (Grace: ATS over NVLink-C2C), u and
 *                   v are read and `out` is written by the kernels in place;
 *                   only the texture is copied to the device.
 *   workspace       device scratch of at least rlic_workspace_bytes(...)
 *                   bytes, 256-byte aligned, or NULL to let the call allocate
 *                   it stream-ordered from the library's memory pool (see
 *                   rlic_release_cached_memory).
 *                   Ignored with RLIC_FLAG_HOST_MEMORY (the call allocates).
 */
RLIC_API int rlic_convolve_f32(const float *texture, const float *u, const float *v, int64_t ny,
                      int64_t nx, const float *kernel, int64_t klen, int uv_mode,
                      int bx_left, int bx_right, int by_left, int by_right,
                      int64_t iterations, float *out, void *workspace,
                      size_t workspace_bytes, void *stream, unsigned flags);

RLIC_API int rlic_convolve_f64(const double *texture, const double *u, const double *v,
                      int64_t ny, int64_t nx, const double *kernel, int64_t klen,
                      int uv_mode, int bx_left, int bx_right, int by_left, int by_right,
                      int64_t iterations, double *out, void *workspace,
                      size_t workspace_bytes, void *stream, unsigned flags);

/*
 * Batched form (float32, default arithmetic): many independent convolutions
 * of uneven sizes, kernel lengths, boundaries, uv modes and iteration counts
 * in one call.  Results are bit-identical to one rlic_convolve_f32 call per
 * item.  No counterpart in the reference.
 *
 * By default the call launches one kernel that packs every item's field,
 * then one per pass level: level 1 traces every item (recording its path
 * cache when it has two or more iterations), level L replays the items with
 * at least L iterations; each launch spreads the tiles of all its items over
 * the whole GPU.  With RLIC_FLAG_BATCH_QUEUE it makes one persistent kernel
 * launch that runs the whole batch from a work queue instead: the work is
 * cut into segments, one per (item, level) (level 0 packs), ordered level by
 * level, the largest items first; resident CTAs take work items in that
 * order from a counter, and an item waits (bounded) until the item's
 * previous level has finished.  Both give the same bits; the per-level
 * launches measured 3-8% faster on this library's benchmark mixes.  tile_x
 * (tile_y = 256 / tile_x) sets an item's CTA tile shape (0: 64);
 * replay_tiles the tiles per replay work item of the queue (0: 4).
 *
 * The per-item tables live at the start of the workspace
 * (rlic_batch_workspace_bytes_f32 bytes, 256-byte aligned).  With
 * RLIC_FLAG_BATCH_PREPARED the call assumes the workspace already holds the
 * tables of the same `items` (written by an earlier call) and issues kernel
 * launches and memsets only, with no host-to-device copy.  All pointers are
 * device memory; asynchronous on `stream`.  Limits: at most 1024 items, each
 * below 2^31 pixels, kernels of at most 1025 taps.
 */
typedef struct rlic_batch_item_f32 {
    const float *texture, *u, *v, *kernel; /* device, C-order ny x nx; klen taps */
    float *out;                            /* device, ny x nx */
    int64_t ny, nx, klen, iterations;
    int uv_mode, bx_left, bx_right, by_left, by_right;
    int tile_x;
    int replay_tiles;
} rlic_batch_item_f32;
#define RLIC_FLAG_BATCH_PREPARED 0x10u
#define RLIC_FLAG_BATCH_QUEUE 0x80u
RLIC_API size_t rlic_batch_workspace_bytes_f32(const rlic_batch_item_f32 *items, int count);
RLIC_API int rlic_convolve_batch_f32(const rlic_batch_item_f32 *items, int count,
                                     void *workspace, size_t workspace_bytes, void *stream,
                                     unsigned flags);
/* 1 if the last run of `items` on `workspace` was a work-queue run that gave
 * up waiting for a previous level (the bound guards against a fault; that
 * run's results are then incomplete), 0 if not, a negative error code on
 * bad arguments.  Synchronises the device. */
RLIC_API int rlic_batch_status_f32(const rlic_batch_item_f32 *items, int count,
                                   const void *workspace);

/*
 * Adjoint of one pass, for gradients (no counterpart in the reference).
 *
 * A pass is linear in the texture: out = A tex, with A[p, c] = sum of the
 * kernel taps with which pixel p's streamlines sample cell c.  Given codes
 * recorded by rlic_sweep_* (same ny, nx, klen):
 *
 * rlic_adjoint_*: y = A^T g (y is overwritten).  Accumulates with atomics,
 *   so the summation order, and the last bits of y, vary from run to run.
 * rlic_kernel_grad_*: dw[k] += sum_p g[p] * x[c_k(p)], the gradient of
 *   <g, A x> with respect to kernel[k]; dw (klen doubles) is accumulated
 *   into, so the caller zeroes it first.
 *
 * Device pointers, asynchronous on `stream`; `flags` must be 0.
 */
RLIC_API int rlic_adjoint_f32(const float *g, const void *codes, int64_t ny, int64_t nx,
                              const float *kernel, int64_t klen, float *y, void *stream,
                              unsigned flags);
RLIC_API int rlic_adjoint_f64(const double *g, const void *codes, int64_t ny, int64_t nx,
                              const double *kernel, int64_t klen, double *y, void *stream,
                              unsigned flags);
RLIC_API int rlic_kernel_grad_f32(const float *g, const float *x, const void *codes,
                                  int64_t ny, int64_t nx, int64_t klen, double *dw,
                                  void *stream, unsigned flags);
RLIC_API int rlic_kernel_grad_f64(const double *g, const double *x, const void *codes,
                                  int64_t ny, int64_t nx, int64_t klen, double *dw,
                                  void *stream, unsigned flags);

/*
 * Reduced-precision form of rlic_convolve_* (device pointers, asynchronous).
 *
 * Streamline cells come from a trace in the input dtype (the cell choices are
 * discontinuous in the arithmetic and need its precision); the texture and
 * every buffer between passes are then stored as FP16 (RLIC_STORAGE_FP16) or
 * BF16 (RLIC_STORAGE_BF16), each pass accumulates in FP32 with compensated
 * (Kahan) summation and stores its output divided by sum(|kernel|), and the
 * last buffer is scaled back in the input dtype into `out`.  Results are
 * approximations of rlic_convolve_*: the error is that of 16-bit storage
 * (relative 2^-11 for FP16, 2^-8 for BF16 per pass, before averaging).
 * No counterpart in the reference.
 *
 * workspace: rlic_lowp_workspace_bytes(ny, nx, klen, 4 or 8) bytes, 256-byte
 * aligned, or NULL to allocate stream-ordered.  `flags` takes the variant
 * bits only.
 */
#define RLIC_STORAGE_FP16 0
#define RLIC_STORAGE_BF16 1
RLIC_API size_t rlic_lowp_workspace_bytes(int64_t ny, int64_t nx, int64_t klen,
                                          int elem_bytes);
RLIC_API int rlic_convolve_lowp_f32(const float *texture, const float *u, const float *v,
                                    int64_t ny, int64_t nx, const float *kernel, int64_t klen,
                                    int uv_mode, int bx_left, int bx_right, int by_left,
                                    int by_right, int64_t iterations, int storage, float *out,
                                    void *workspace, size_t workspace_bytes, void *stream,
                                    unsigned flags);
RLIC_API int rlic_convolve_lowp_f64(const double *texture, const double *u, const double *v,
                                    int64_t ny, int64_t nx, const double *kernel,
                                    int64_t klen, int uv_mode, int bx_left, int bx_right,
                                    int by_left, int by_right, int64_t iterations, int storage,
                                    double *out, void *workspace, size_t workspace_bytes,
                                    void *stream, unsigned flags);

/*
 * rlic_convolve_f32 for callers that cannot allocate device memory: a plugin
 * whose host application owns the whole device-memory budget and forbids
 * its plugins from allocating, code that runs inside another library's
 * allocator callback (where calling back into the allocator would
 * deadlock), or a latency-critical loop that cannot afford the device-wide
 * synchronisation cudaMalloc and cudaFree can cause.  No counterpart in the
 * reference, whose native core allocates its own buffers on the host.
 *
 * Same arguments, results and flags as rlic_convolve_f32 with device
 * pointers, minus the workspace: the call allocates nothing (no cudaMalloc,
 * cudaMallocAsync or cudaFree) and uses a static device array of
 * RLIC_NOALLOC_SCRATCH_BYTES (64 MiB) instead.  The caller still provides
 * texture, u, v, kernel and out.  A call whose rlic_workspace_bytes(ny, nx,
 * klen, iterations, 4, flags) exceeds that size fails with
 * RLIC_ERR_WORKSPACE_TOO_SMALL before touching the GPU;
 * RLIC_FLAG_NO_PATH_CACHE shrinks the need to about 12 bytes per pixel.
 * Zero iterations only clear `out` and have no size limit.
 * RLIC_FLAG_HOST_MEMORY and RLIC_FLAG_CHECK_TEXTURE are rejected
 * (RLIC_ERR_INVALID_ARGUMENT).
 *
 * The array belongs to the library's module: once mapped on a GPU it stays
 * there until the process exits.  Under CUDA's default lazy module loading
 * it is mapped by the first call on each device, not when the library is
 * loaded, so that first call is the one that can fail for lack of device
 * memory (RLIC_ERR_OUT_OF_MEMORY, with a message saying so): make one
 * warm-up call per device up front, while memory is free.  The first call
 * on a device also looks up the array's device address
 * (cudaGetSymbolAddress) with that device current; make that first call
 * before any stream capture.  All calls
 * share the one array: calls whose work overlaps on the GPU (different
 * streams, or different host threads on one device) race and must be
 * serialised by the caller.  Each call writes every part of the array it
 * reads, so the previous call's contents never leak into a result.
 */
#define RLIC_NOALLOC_SCRATCH_BYTES (64u << 20)
RLIC_API int rlic_convolve_f32_noalloc(const float *texture, const float *u, const float *v,
                                       int64_t ny, int64_t nx, const float *kernel,
                                       int64_t klen, int uv_mode, int bx_left, int bx_right,
                                       int by_left, int by_right, int64_t iterations,
                                       float *out, void *stream, unsigned flags);

/*
 * rlic_convolve_* on strided host arrays, read in place (no host copies):
 * numpy views such as broadcasts (stride 0, as in the reference's README
 * example), transposes, reversed or sliced arrays.  strides[6] holds the
 * element strides (row, column) of texture, u and v, in that order; `out` is
 * C-contiguous.  Requires RLIC_FLAG_HOST_MEMORY and a device that can access
 * pageable host memory (rlic_host_direct_access() == 1; otherwise
 * RLIC_ERR_UNSUPPORTED).  Other arguments and flags as rlic_convolve_*; the
 * call allocates its scratch and returns once `out` holds the result.
 */
RLIC_API int rlic_convolve_strided_f32(const float *texture, const float *u, const float *v,
                                       const int64_t *strides, int64_t ny, int64_t nx,
                                       const float *kernel, int64_t klen, int uv_mode,
                                       int bx_left, int bx_right, int by_left, int by_right,
                                       int64_t iterations, float *out, void *stream,
                                       unsigned flags);
RLIC_API int rlic_convolve_strided_f64(const double *texture, const double *u,
                                       const double *v, const int64_t *strides, int64_t ny,
                                       int64_t nx, const double *kernel, int64_t klen,
                                       int uv_mode, int bx_left, int bx_right, int by_left,
                                       int by_right, int64_t iterations, double *out,
                                       void *stream, unsigned flags);

/* 1 when kernels on the current device can read and write pageable host
 * memory directly (Grace: ATS over NVLink-C2C) and RLIC_NO_HOST_DIRECT is not
 * set to 1; then host-memory calls read u, v (and strided inputs) in place
 * and write the result in place. */
RLIC_API int rlic_host_direct_access(void);

/*
 * Streamline cells, for index-for-index parity checks of the trace
 * (convole_single_pixel, src/lib.rs:305-362; advance, src/lib.rs:236-273).
 *
 * For each of the npix pixels whose linear indices (i * nx + j) are in `pix`,
 * writes klen - 1 linear cell indices to cells[p * (klen - 1) ...]: first the
 * klen - klen/2 - 1 cells reached by the forward trace, then the klen/2 cells
 * reached by the backward trace, each slot after a NaN stop set to -1.
 * Pointers follow RLIC_FLAG_HOST_MEMORY like rlic_convolve_*.
 */
RLIC_API int rlic_trace_cells_f32(const float *u, const float *v, int64_t ny, int64_t nx,
                         int64_t klen, int uv_mode, int bx_left, int bx_right, int by_left,
                         int by_right, int64_t npix, const int64_t *pix, int64_t *cells,
                         void *stream, unsigned flags);

RLIC_API int rlic_trace_cells_f64(const double *u, const double *v, int64_t ny, int64_t nx,
                         int64_t klen, int uv_mode, int bx_left, int bx_right,
                         int by_left, int by_right, int64_t npix, const int64_t *pix,
                         int64_t *cells, void *stream, unsigned flags);

/*
 * Building blocks of rlic_convolve_*, for callers that convolve many
 * textures over one field (all pointers device memory, asynchronous):
 *
 * rlic_pack_field_*: interleave u and v (ny x nx each) into `uv`, an array
 *   of ny * nx (u, v) pairs (2 * ny * nx elements, aligned to one pair), the
 *   layout every streamline step reads.  No counterpart in the reference,
 *   which reads u and v from two views (src/lib.rs:332-335).
 *
 * rlic_sweep_*: one convolution pass, `convolve` of src/lib.rs:364-406:
 *   tex_out = LIC(tex_in) along the packed field.  When `codes` is not NULL
 *   (rlic_path_code_bytes() bytes, 4-byte aligned) the pass also records
 *   every streamline step there.  `flags` takes the variant bits and
 *   RLIC_FLAG_FIELD_NAN_FREE, a promise that the packed field holds no NaN
 *   sample, which spares the steps their NaN test (the convolve entry points
 *   find this out themselves while packing; with a NaN in the field the
 *   results are then unspecified).
 *
 * rlic_replay_*: one convolution pass replayed from `codes` recorded by
 *   rlic_sweep_* on the same ny x nx image with the same klen (boundaries
 *   and uv mode are part of the record).  Identical results to
 *   rlic_sweep_*; `flags` takes RLIC_FLAG_NO_FMA and
 *   RLIC_FLAG_FIELD_NAN_FREE (the codes were recorded from a field without
 *   NaN samples, so they hold no stop code and none is tested for; codes
 *   that do hold one then give undefined results).
 */
RLIC_API int rlic_pack_field_f32(const float *u, const float *v, int64_t ny, int64_t nx,
                                 void *uv, void *stream);
RLIC_API int rlic_pack_field_f64(const double *u, const double *v, int64_t ny, int64_t nx,
                                 void *uv, void *stream);
RLIC_API int rlic_sweep_f32(const float *tex_in, const void *uv, int64_t ny, int64_t nx,
                            const float *kernel, int64_t klen, int uv_mode, int bx_left,
                            int bx_right, int by_left, int by_right, float *tex_out,
                            void *codes, void *stream, unsigned flags);
RLIC_API int rlic_sweep_f64(const double *tex_in, const void *uv, int64_t ny, int64_t nx,
                            const double *kernel, int64_t klen, int uv_mode, int bx_left,
                            int bx_right, int by_left, int by_right, double *tex_out,
                            void *codes, void *stream, unsigned flags);
RLIC_API int rlic_replay_f32(const float *tex_in, const void *codes, int64_t ny, int64_t nx,
                             const float *kernel, int64_t klen, float *tex_out, void *stream,
                             unsigned flags);
RLIC_API int rlic_replay_f64(const double *tex_in, const void *codes, int64_t ny, int64_t nx,
                             const double *kernel, int64_t klen, double *tex_out,
                             void *stream, unsigned flags);

/*
 * How replayed passes (path cache, passes 2..n) gather the texture:
 *   RLIC_REPLAY_L1      through L1 and L2 (lic_gather_kernel);
 *   RLIC_REPLAY_STAGED  from a box of cells around each 64 x stage_rows pixel
 *                       super-tile, copied into shared memory by the Tensor
 *                       Memory Accelerator together with the super-tile's
 *                       code words; super-tiles whose box crosses a
 *                       periodic edge, and images that do not fit the form
 *                       (rows not a multiple of 16 bytes, textures not in
 *                       device memory or not 16-byte aligned, boxes beyond
 *                       256 cells a side or beyond 113 KB of shared memory,
 *                       which would leave one CTA per SM, 2^31 pixels or
 *                       more), use L1;
 *   RLIC_REPLAY_AUTO    the library's default (staged, where the image fits).
 * Both give bit-identical results.  stage_rows: super-tile height, a
 * multiple of 4 in [4, 64], or 0 for 16.  Affects calls made after it on any
 * thread.  No counterpart in the reference (a tuning knob of this
 * implementation).
 */
#define RLIC_REPLAY_AUTO 0
#define RLIC_REPLAY_L1 1
#define RLIC_REPLAY_STAGED 2
RLIC_API int rlic_set_replay_mode(int mode, int stage_rows);
/*
 * Images of at most max_pixels pixels (default: 2^18 for float64 images,
 * 2^16 for float32) trace every traced pass with each pixel's two
 * half-streamlines on two threads of one warp: the forward thread
 * accumulates the centre tap and its own samples, the backward thread hands
 * its samples over through shared memory, and the forward thread adds them
 * in the reference's order.  On images too small to fill the GPU this
 * doubles the threads that run the serial streamline arithmetic.
 * Bit-identical to the one-thread-per-pixel pass; 0 turns it off and -1
 * restores the defaults.  Launches that do not fit the form (kernels of
 * fewer than 3 taps, CTA shapes of other than a multiple of 16 pixels up to
 * 64, backward samples beyond 96 KiB of shared memory, images of 2^31
 * pixels or more) keep one thread per pixel.  Affects calls made after it on
 * any thread.  No counterpart in the reference (a tuning knob of this
 * implementation).
 */
RLIC_API int rlic_set_split_pixels(int64_t max_pixels);
/*
 * 1 if a staged replay ever gave up waiting for one of its copies (each wait
 * is bounded; the CTA then returns and its remaining pixels are not written),
 * 0 if not, -1 if the device could not be queried.  Synchronises the device.
 */
RLIC_API int rlic_stage_timeouts(void);

/*
 * Launch-shape tuning for the streamline kernels: CTA width and height in
 * pixels (block_x * block_y threads, at most 256; block_x a multiple of 32
 * or a divisor of 32).  Affects calls made after it on any thread.  Until
 * it is called, traced passes use 16 x 8 (8 x 8 for images of at most 2^19
 * pixels, 4 x 4 for paired passes over images of at most 2^17 pixels: more
 * CTAs even the SMs' load when an image has few tiles) and replays through
 * L1 use 64 x 4; once called, every kernel uses the shape given.  (0, 0)
 * restores those defaults.
 */
RLIC_API int rlic_set_block_shape(int block_x, int block_y);

/*
 * Histogram equalization of an ny x nx image (float32 or float64), the
 * post-processing step commonly applied to LIC output.  The reference
 * declares these operations in its native-module stubs
 * (src/rlic/_core.pyi:30-57: equalize_histogram_*,
 * equalize_histogram_sliding_tile_*, equalize_histogram_tile_interpolation_*)
 * without implementing them; the definitions are this library's own
 * (oracle/histogram.py states them):
 *   - bins: nbins equal bins over [min, max] of the finite pixels;
 *   - RLIC_EQUALIZE_GLOBAL: cumulative histogram / finite-pixel count;
 *   - RLIC_EQUALIZE_SLIDING_TILE: the pixel's rank among the finite pixels
 *     of the tile_y x tile_x window around it (clipped to the image);
 *   - RLIC_EQUALIZE_TILE_INTERPOLATION: per-tile mappings (tiles of
 *     tile_y x tile_x) blended bilinearly between the four nearest tile
 *     centres.
 * Non-finite pixels are returned unchanged.  nbins in [1, 2^24] (tile
 * interpolation: at most 49152); tile_y, tile_x >= 1 for the tile
 * strategies.  `flags` takes RLIC_FLAG_HOST_MEMORY only.  Device pointers
 * are processed asynchronously on `stream`.
 */
#define RLIC_EQUALIZE_GLOBAL 0
#define RLIC_EQUALIZE_SLIDING_TILE 1
#define RLIC_EQUALIZE_TILE_INTERPOLATION 2
RLIC_API int rlic_equalize_histogram_f32(const float *image, int64_t ny, int64_t nx,
                                         int64_t nbins, int strategy, int64_t tile_y,
                                         int64_t tile_x, float *out, void *stream,
                                         unsigned flags);
RLIC_API int rlic_equalize_histogram_f64(const double *image, int64_t ny, int64_t nx,
                                         int64_t nbins, int strategy, int64_t tile_y,
                                         int64_t tile_x, double *out, void *stream,
                                         unsigned flags);

/*
 * Self-check of the float64 streamline step's screened division (no
 * reference counterpart).  For nonzero a[i], b[i] with binary exponents in
 * [-60, 60], sets certified[i] to 1 when the short division certified its
 * result, and q[i] to its value of |a[i] / b[i]|, which must then equal
 * the correctly rounded quotient.  Device pointers; asynchronous on
 * `stream`.
 */
RLIC_API int rlic_check_quotients_f64(const double *a, const double *b, int64_t n, double *q,
                                      int32_t *certified, void *stream);

/*
 * Self-check of the float64 streamline step's integer numerator (no
 * reference counterpart): for each f[i] sets in_range[i] to 1 when
 * 0 <= f[i] <= 1 (sign bit clear), and then g[i] to the step's value of
 * fma(2, 0.5 - f[i], f[i]) computed with integer instructions, which must
 * equal the IEEE result; otherwise in_range[i] = 0 and g[i] = 0.  Device
 * pointers; asynchronous on `stream`.
 */
RLIC_API int rlic_check_numerators_f64(const double *f, int64_t n, double *g,
                                       int32_t *in_range, void *stream);

/*
 * Number of this library's kernels launched since load (all threads).  Lets
 * a caller confirm that work ran on the device and count launches per call.
 */
RLIC_API uint64_t rlic_kernel_launch_count(void);

/*
 * Page-locked host buffers for results: rlic_host_buffer_alloc returns a
 * pinned block of `bytes` (NULL on failure), reusing a block of the same size
 * released earlier by rlic_host_buffer_free.  Host-memory calls that write
 * into such a block need no page faults and no staging copy.  At most 4 GiB
 * of released blocks are kept.
 */
RLIC_API void *rlic_host_buffer_alloc(size_t bytes);
RLIC_API void rlic_host_buffer_free(void *p);

/*
 * Calls that allocate their scratch (a NULL workspace, host-memory calls)
 * draw it from a stream-ordered memory pool owned by the library, one per
 * device, which keeps freed memory for later calls.  This returns the
 * current device's cached device memory to the driver (after a device-wide
 * synchronisation) and frees the released host buffers.
 */
RLIC_API int rlic_release_cached_memory(void);

#ifdef __cplusplus
}
#endif

#endif /* RLIC_GB300_H */
