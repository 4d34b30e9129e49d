// lic_capi.cu -- the C ABI of the rLIC convolution core (include/rlic_gb300.h).
//
// Host logic only: argument checks, workspace carving, the choice of form
// and the order of kernel launches.  The kernels live in lic_kernels.cuh.
//
// Device data layout of one rlic_convolve_* call (C-order, ny rows x nx
// columns, every region 256-byte aligned inside one workspace):
//   uv      packed (u, v) pairs, one float2/double2 per cell, so that every
//           streamline step fetches both components with a single load;
//   tmp     ping-pong texture buffer (two or more iterations);
//   codes   path cache: 4-bit step codes, 8 per 32-bit word, word-major
//           (two or more iterations, unless RLIC_FLAG_NO_PATH_CACHE);
//   kernel  a device copy of the weights (host-memory calls).
// The passes alternate between `out` and `tmp`, ordered so that the last
// one writes `out` (the reference copies output -> input and zeroes output
// between passes instead, src/lib.rs:433-440).
//
// Forms:
//   plain       every pass traces every streamline (lic_pass_kernel);
//   path cache  (default for two or more iterations) the first pass also
//               records every step's code; later passes replay the codes
//               (lic_gather_kernel).  Streamline cells do not depend on the
//               texture, so both forms give identical results.
#include "../../include/rlic_gb300.h"
#include "lic_batch.h"
#include "lic_equalize.h"
#include "lic_launch.h"

#include <algorithm>
#include <atomic>
#include <map>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

namespace rlic {

namespace {
std::atomic<uint64_t> g_launches{0};
}

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

uint64_t launches() { return g_launches.load(); }

}  // namespace rlic

namespace {

using rlic::LaunchConfig;
using rlic::Shape;
using rlic::Variant;

thread_local std::string g_last_error;
std::atomic<int> g_block_x{64};
std::atomic<int> g_block_y{4};

constexpr size_t kAlign = 256;
inline size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

constexpr unsigned kKnownFlags = RLIC_FLAG_HOST_MEMORY | RLIC_FLAG_NO_FMA |
                                 RLIC_FLAG_NO_BRANCHLESS | RLIC_FLAG_NO_PATH_CACHE |
                                 RLIC_FLAG_CHECK_TEXTURE;

int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    const int code = (e == cudaErrorMemoryAllocation) ? RLIC_ERR_OUT_OF_MEMORY : RLIC_ERR_CUDA;
    return fail(code, std::string(what) + ": " + cudaGetErrorString(e));
}

#define RLIC_CUDA_TRY(expr)                                  \
    do {                                                     \
        cudaError_t e_ = (expr);                             \
        if (e_ != cudaSuccess) return cuda_fail(e_, #expr);  \
    } while (0)

// Whether kernels may read and write the caller's pageable host memory
// directly (per device, cached).  RLIC_NO_HOST_DIRECT=1 in the environment
// turns it off.
bool host_direct_access() {
    static std::mutex mu;
    static int cache[64];
    static bool init = false;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return false;
    std::lock_guard<std::mutex> lock(mu);
    if (!init) {
        for (int& c : cache) c = -1;
        init = true;
    }
    if (cache[dev] < 0) {
        int pageable = 0, tables = 0;
        cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev);
        cudaDeviceGetAttribute(&tables, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev);
        const char* off = std::getenv("RLIC_NO_HOST_DIRECT");
        cache[dev] = (pageable && tables && !(off && off[0] == '1')) ? 1 : 0;
    }
    return cache[dev] == 1;
}

// Writes one byte per 4 KiB of [p, p + bytes) from a few host threads, so
// that every page is mapped before the GPU (or a copy) writes the result.
void touch_pages(void* p, size_t bytes) {
    constexpr size_t kPage = 4096;
    const size_t pages = (bytes + kPage - 1) / kPage;
    unsigned hw = std::thread::hardware_concurrency();
    const size_t nthreads = std::max<size_t>(1, std::min<size_t>({size_t(hw ? hw : 1), 8, pages / 256 + 1}));
    auto work = [p, bytes, pages, nthreads](size_t t) {
        volatile unsigned char* b = static_cast<unsigned char*>(p);
        for (size_t k = t; k < pages; k += nthreads) {
            const size_t off = k * kPage;
            if (off < bytes) b[off] = 0;
        }
    };
    std::vector<std::thread> pool;
    for (size_t t = 1; t < nthreads; ++t) pool.emplace_back(work, t);
    work(0);
    for (auto& th : pool) th.join();
}

// Scratch of calls that allocate (NULL workspace, host-memory calls) comes
// from a stream-ordered pool owned by this library, one per device, that
// keeps freed memory for the next call instead of returning it to the driver
// at every synchronisation (the default pool's behaviour, which made every
// call map its scratch afresh).  rlic_release_cached_memory() trims it.
cudaMemPool_t library_pool(cudaError_t* err) {
    static std::mutex mu;
    static cudaMemPool_t pools[64] = {};
    int dev = 0;
    *err = cudaGetDevice(&dev);
    if (*err != cudaSuccess) return nullptr;
    if (dev < 0 || dev >= 64) {
        *err = cudaErrorInvalidDevice;
        return nullptr;
    }
    std::lock_guard<std::mutex> lock(mu);
    if (!pools[dev]) {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.handleTypes = cudaMemHandleTypeNone;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t pool = nullptr;
        *err = cudaMemPoolCreate(&pool, &props);
        if (*err != cudaSuccess) return nullptr;
        uint64_t keep = UINT64_MAX;
        *err = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        if (*err != cudaSuccess) return nullptr;
        pools[dev] = pool;
    }
    return pools[dev];
}

// Upload chunks of a host-memory call: at most this many, each of at least
// max(K - 1, 64) rows and 2^20 pixels.  Measured end to end at 8192^2
// float32, 65 taps, 5 passes (ms per call, traced-pass groups alternating
// two streams): 6 chunks 17.23, 8 17.08, 12 16.92, 16 16.85, 20 16.81,
// 24 16.79, 32 16.76 (the first traced rows start after a smaller first
// chunk).
#ifndef RLIC_HOST_CHUNKS
#define RLIC_HOST_CHUNKS 32
#endif

// Images of at most this many pixels trace their passes with each pixel's
// two half-streamlines on two threads (lic_pass_paired_kernel) unless
// rlic_set_split_pixels chose a threshold.  Measured on GB300, calls of one
// pass on device memory (ms): float64 256^2, 65 taps 0.0957 (4 x 4-pixel
// tiles) against 0.114-0.117 with one thread per pixel, 512^2 0.336 against
// 0.375; float32 256^2 0.028 against 0.030, 512^2 0.064 against 0.058.  The
// paired form spends about 12% more FP64 instructions (the forward thread
// adds the backward samples after its own), and the float32 pass is bound
// by instruction issue, so it pays only where the image alone cannot fill
// the GPU with threads.
constexpr int64_t kPairedPixelsF64 = int64_t(1) << 18;
constexpr int64_t kPairedPixelsF32 = int64_t(1) << 16;
// Paired passes over images of at most this many pixels use 4 x 4-pixel
// tiles (one warp per CTA: with about 27 CTAs per SM the SMs' loads differ
// by one CTA in 27, against one in 7 with 8 x 8 tiles on a 256^2 image).
constexpr int64_t kPairedSmallTilePixels = int64_t(1) << 17;

// A non-blocking stream per device for the uploads of host-memory calls, at
// the greatest priority: the block scheduler then gives the upload kernels
// the SM slots that the traced pass's blocks free, instead of queueing them
// behind the whole pass.
cudaStream_t aux_stream(cudaError_t* err, bool greatest_priority = true) {
    static std::mutex mu;
    static cudaStream_t streams[2][64] = {};
    int dev = 0;
    *err = cudaGetDevice(&dev);
    if (*err != cudaSuccess) return nullptr;
    if (dev < 0 || dev >= 64) {
        *err = cudaErrorInvalidDevice;
        return nullptr;
    }
    std::lock_guard<std::mutex> lock(mu);
    cudaStream_t& s = streams[greatest_priority ? 0 : 1][dev];
    if (!s) {
        int least = 0, greatest = 0;
        *err = cudaDeviceGetStreamPriorityRange(&least, &greatest);
        if (*err != cudaSuccess) return nullptr;
        *err = cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking,
                                            greatest_priority ? greatest : least);
        if (*err != cudaSuccess) return nullptr;
    }
    return s;
}

cudaError_t scratch_alloc(void** p, size_t bytes, cudaStream_t stream) {
    cudaError_t e = cudaSuccess;
    cudaMemPool_t pool = library_pool(&e);
    if (!pool) return e;
    return cudaMallocFromPoolAsync(p, bytes, pool, stream);
}

// Cache of page-locked host buffers for results handed to Python: a result
// written into pinned memory needs no page faults and no staging copy, and a
// buffer the caller has dropped is reused by the next call of the same size.
struct HostBufferCache {
    std::mutex mu;
    std::multimap<size_t, void*> free_blocks;  // size -> block
    std::map<void*, size_t> sizes;             // every block handed out
    size_t cached_bytes = 0;
};

HostBufferCache& host_cache() {
    static HostBufferCache* c = new HostBufferCache();  // lives until exit
    return *c;
}

Variant make_variant(unsigned flags, int uv_mode) {
    return Variant{!(flags & RLIC_FLAG_NO_FMA), !(flags & RLIC_FLAG_NO_BRANCHLESS),
                   uv_mode == RLIC_UV_POLARIZATION};
}

LaunchConfig launch_config() { return LaunchConfig{g_block_x.load(), g_block_y.load()}; }

// CTA shape of the traced passes.  Unless rlic_set_block_shape chose one,
// traced passes use squarer tiles than the replay's 64 x 4: 16 x 8 pixels,
// and 8 x 8 for images of at most kSmallImagePixels pixels, whose tiles are
// too few to spread evenly over the SMs otherwise (4 x 4 for the paired
// pass on the smallest images, see kPairedSmallTilePixels).  Measured with
// one thread per pixel (ms per pass): 8192^2 float32 with recording 9.78
// against 10.18 for 64 x 4; 1024^2 float64 1.20 against 1.34; 256^2
// float64 0.117 against 0.161; 512^2 float32 0.059 against 0.062.
std::atomic<bool> g_block_custom{false};
constexpr int64_t kSmallImagePixels = int64_t(1) << 19;

int64_t split_pixels(size_t elem);

// Launch shape of the traced passes of an ny x nx image of `elem`-byte
// elements (4 or 8) and a kernel of klen taps.
LaunchConfig launch_config_for(int64_t ny, int64_t nx, size_t elem, int64_t klen) {
    LaunchConfig lc = launch_config();
    if (!g_block_custom.load()) {
        const bool small = ny * nx <= kSmallImagePixels;
        lc.block_x = small ? 8 : 16;
        lc.block_y = 8;
        if (ny * nx <= split_pixels(elem) && ny * nx <= kPairedSmallTilePixels &&
            rlic::paired_launch_fits(ny * nx, 4, 4, klen, elem)) {
            lc.block_x = 4;
            lc.block_y = 4;
        }
    }
    lc.paired = ny * nx <= split_pixels(elem);
    return lc;
}

// How replayed passes gather (rlic_set_replay_mode).
std::atomic<int> g_replay_mode{RLIC_REPLAY_AUTO};
// The staged form measured 18% faster per replay on the 8192^2 benchmark
// field (1.73 vs 2.12 ms), so it is the default where the image fits it.
constexpr bool kStagedByDefault = true;

// One replayed pass: from a texture box staged in shared memory by TMA
// copies when the mode asks for it and the image fits that form (device
// memory, 16-byte rows), otherwise through L1.
template <typename T>
cudaError_t replay_pass(bool fma, const T* src, const uint32_t* codes, const T* kernel, int klen,
                        const Shape& sh, const LaunchConfig& lc, T* dst, cudaStream_t stream) {
    const int mode = g_replay_mode.load();
    if (mode == RLIC_REPLAY_STAGED || (mode == RLIC_REPLAY_AUTO && kStagedByDefault)) {
        cudaPointerAttributes attr{};
        const bool device = cudaPointerGetAttributes(&attr, src) == cudaSuccess &&
                            attr.type == cudaMemoryTypeDevice;
        cudaGetLastError();  // a host pointer is not an error to keep
        if (device) {
            const cudaError_t e = rlic::launch_gather_staged(fma, src, codes, kernel, klen, sh,
                                                             lc.field_nan, dst, stream);
            if (e != cudaErrorNotSupported) return e;
        }
    }
    // the L1 replay keeps the library's CTA shape (64 x 4 unless set), not
    // the traced passes' squarer tiles
    LaunchConfig rl = lc;
    rl.block_x = g_block_x.load();
    rl.block_y = g_block_y.load();
    return rlic::launch_gather(fma, src, codes, kernel, klen, sh, rl, dst, stream);
}

int check_shape(int64_t ny, int64_t nx, int64_t klen) {
    if (ny <= 0 || nx <= 0)
        return fail(RLIC_ERR_INVALID_ARGUMENT, "image dimensions must be positive");
    if (ny > (int64_t(1) << 40) / nx) return fail(RLIC_ERR_INVALID_ARGUMENT, "image too large");
    if (klen <= 0) return fail(RLIC_ERR_INVALID_ARGUMENT, "kernel must have at least one tap");
    if (klen > (int64_t(1) << 20)) return fail(RLIC_ERR_INVALID_ARGUMENT, "kernel too long");
    return RLIC_OK;
}

int check_common(int64_t ny, int64_t nx, int64_t klen, int uv_mode, const int bnd[4],
                 unsigned flags) {
    int rc = check_shape(ny, nx, klen);
    if (rc) return rc;
    if (uv_mode != RLIC_UV_VELOCITY && uv_mode != RLIC_UV_POLARIZATION)
        return fail(RLIC_ERR_INVALID_ARGUMENT, "uv_mode must be 0 (velocity) or 1 (polarization)");
    for (int k = 0; k < 4; ++k)
        if (bnd[k] != RLIC_BOUNDARY_CLOSED && bnd[k] != RLIC_BOUNDARY_PERIODIC)
            return fail(RLIC_ERR_INVALID_ARGUMENT,
                        "boundaries must be 0 (closed) or 1 (periodic)");
    if (flags & ~kKnownFlags) return fail(RLIC_ERR_INVALID_ARGUMENT, "unknown flag bits");
    return RLIC_OK;
}

Shape make_shape(int64_t ny, int64_t nx, const int bnd[4]) {
    Shape sh;
    sh.ny = ny;
    sh.nx = nx;
    for (int k = 0; k < 4; ++k) sh.bnd[k] = bnd[k];
    return sh;
}

// Images of at most this many pixels trace each pass's two half-streamlines
// of a pixel on two threads of one warp (lic_pass_paired_kernel), which
// doubles the threads running the serial streamline arithmetic where an
// image's tiles alone cannot fill the GPU (rlic_set_split_pixels).
// (-1: the per-dtype defaults kPairedPixelsF32 / kPairedPixelsF64)
std::atomic<int64_t> g_split_pixels{-1};

int64_t split_pixels(size_t elem) {
    const int64_t v = g_split_pixels.load();
    if (v >= 0) return v;
    return elem == sizeof(double) ? kPairedPixelsF64 : kPairedPixelsF32;
}

bool use_path_cache(int64_t iterations, int64_t klen, unsigned flags) {
    return iterations >= 2 && klen > 1 && !(flags & RLIC_FLAG_NO_PATH_CACHE);
}

size_t code_bytes(int64_t ny, int64_t nx, int64_t klen) {
    return size_t(rlic::code_words_per_pixel(klen)) * size_t(ny) * size_t(nx) * 4;
}

struct WorkspaceLayout {
    size_t uv, tmp, codes, kernel, nan, total;
};

WorkspaceLayout workspace_layout(int64_t ny, int64_t nx, int64_t klen, int64_t iterations,
                                 size_t s, unsigned flags) {
    const size_t n = size_t(ny) * size_t(nx);
    WorkspaceLayout w{};
    size_t off = 0;
    w.uv = off;
    off += align_up(2 * n * s);
    w.tmp = off;
    if (iterations >= 2) off += align_up(n * s);
    w.codes = off;
    if (use_path_cache(iterations, klen, flags)) off += align_up(code_bytes(ny, nx, klen));
    w.kernel = off;
    off += align_up(size_t(klen) * s);
    w.nan = off;  // flag: the packed field holds a NaN sample
    off += align_up(sizeof(unsigned));
    w.total = off;
    return w;
}

struct NoHook {
    void operator()() const {}
};

// Runs `iterations` passes on device memory.  `ws` holds the workspace.
// The passes alternate between `out` and the workspace's ping-pong buffer;
// when `final_out` is given, the last pass writes it instead (and `out` is
// device scratch).  `before_last()` runs on the host just before the last
// pass is launched.
template <typename T, typename Hook = NoHook>
int run_device(const T* texture, const T* u, const T* v, int64_t ny, int64_t nx,
               const T* kernel, int64_t klen, const Variant& var, const int bnd[4],
               int64_t iterations, T* out, unsigned char* ws, unsigned flags,
               cudaStream_t stream, Hook before_last = Hook{}, T* final_out = nullptr,
               bool uv_ready = false) {
    const int64_t n = ny * nx;
    if (iterations == 0) {
        RLIC_CUDA_TRY(cudaMemsetAsync(out, 0, size_t(n) * sizeof(T), stream));
        return RLIC_OK;
    }
    const WorkspaceLayout wl = workspace_layout(ny, nx, klen, iterations, sizeof(T), flags);
    void* uv = ws + wl.uv;
    T* tmp = reinterpret_cast<T*>(ws + wl.tmp);
    uint32_t* codes = reinterpret_cast<uint32_t*>(ws + wl.codes);
    const bool cache = use_path_cache(iterations, klen, flags);
    const Shape sh = make_shape(ny, nx, bnd);
    LaunchConfig lc = launch_config_for(ny, nx, sizeof(T), klen);
    if (!uv_ready) {
        unsigned* nan_flag = reinterpret_cast<unsigned*>(ws + wl.nan);
        RLIC_CUDA_TRY(cudaMemsetAsync(nan_flag, 0, sizeof(unsigned), stream));
        RLIC_CUDA_TRY(rlic::launch_pack(u, v, uv, n, stream, nan_flag));
        lc.field_nan = nan_flag;
    }
    const T* src = texture;
    for (int64_t it = 0; it < iterations; ++it) {
        T* dst = ((iterations - 1 - it) % 2 == 0) ? out : tmp;
        if (it + 1 == iterations) {
            before_last();
            if (final_out) dst = final_out;
        }
        if (it == 0 || !cache) {
            RLIC_CUDA_TRY(rlic::launch_pass(var, cache ? rlic::kPassSampleRecord : rlic::kPassSample,
                                            src, uv, kernel, int(klen), sh, lc, dst, codes,
                                            stream));
        } else {
            RLIC_CUDA_TRY(replay_pass(var.fma, src, codes, kernel, int(klen), sh, lc,
                                              dst, stream));
        }
        src = dst;
    }
    return RLIC_OK;
}

// `strides` (host memory only): element strides (row, column) of texture,
// u and v, or NULL for C-contiguous arrays.
template <typename T>
int convolve_impl(const T* texture, const T* u, const T* v, int64_t ny, int64_t nx,
                  const T* kernel, int64_t klen, int uv_mode, int bxl, int bxr, int byl,
                  int byr, int64_t iterations, T* out, void* workspace, size_t workspace_bytes_,
                  void* stream_, unsigned flags, const int64_t* strides = nullptr) {
    g_last_error.clear();
    const int bnd[4] = {bxl, bxr, byl, byr};
    int rc = check_common(ny, nx, klen, uv_mode, bnd, flags);
    if (rc) return rc;
    if (iterations < 0) return fail(RLIC_ERR_INVALID_ARGUMENT, "iterations must be >= 0");
    if (!texture || !u || !v || !kernel || !out)
        return fail(RLIC_ERR_INVALID_ARGUMENT, "null array pointer");
    const Variant var = make_variant(flags, uv_mode);
    cudaStream_t stream = static_cast<cudaStream_t>(stream_);
    const size_t n = size_t(ny) * size_t(nx);
    const WorkspaceLayout wl = workspace_layout(ny, nx, klen, iterations, sizeof(T), flags);

    if (!(flags & RLIC_FLAG_HOST_MEMORY)) {
        unsigned char* ws = static_cast<unsigned char*>(workspace);
        bool owned = false;
        if (ws == nullptr) {
            RLIC_CUDA_TRY(scratch_alloc(reinterpret_cast<void**>(&ws), wl.total, stream));
            owned = true;
        } else {
            if (workspace_bytes_ < wl.total)
                return fail(RLIC_ERR_WORKSPACE_TOO_SMALL,
                            "workspace smaller than rlic_workspace_bytes()");
            if (reinterpret_cast<uintptr_t>(ws) % kAlign != 0)
                return fail(RLIC_ERR_INVALID_ARGUMENT, "workspace must be 256-byte aligned");
        }
        rc = run_device<T>(texture, u, v, ny, nx, kernel, klen, var, bnd, iterations, out, ws,
                           flags, stream);
        if (owned) {
            cudaError_t e = cudaFreeAsync(ws, stream);
            if (rc == RLIC_OK && e != cudaSuccess) return cuda_fail(e, "cudaFreeAsync");
        }
        return rc;
    }

    // Host memory.  With pageable-memory access (Grace: ATS over NVLink-C2C,
    // cudaDevAttrPageableMemoryAccess) the pack kernel reads u and v straight
    // from the caller's memory and the last pass stores straight into `out`;
    // only the texture, which every pass gathers from, is copied to HBM.
    // Otherwise u, v and the result go through device copies.  Either way the
    // host touches every page of `out` while the GPU runs the earlier passes,
    // so that the result lands in mapped pages.  The call returns once `out`
    // holds the result.
    const int64_t contiguous[6] = {nx, 1, nx, 1, nx, 1};
    const int64_t* st = strides ? strides : contiguous;
    const bool strided = std::memcmp(st, contiguous, sizeof(contiguous)) != 0;
    if (iterations == 0) {  // zeros, as the native core (src/lib.rs:425, 433)
        if (flags & RLIC_FLAG_CHECK_TEXTURE)
            for (int64_t i = 0; i < ny; ++i)
                for (int64_t j = 0; j < nx; ++j)
                    if (texture[i * st[0] + j * st[1]] < T(0))
                        return fail(RLIC_ERR_NEGATIVE_TEXTURE,
                                    "Found invalid texture element(s). Expected only positive values.");
        std::memset(out, 0, n * sizeof(T));
        return RLIC_OK;
    }
    // A host-memory call waits for its own work only: with no stream given
    // it runs on the calling thread's per-thread stream, so that calls from
    // several host threads overlap on the device.
    if (stream == nullptr) stream = cudaStreamPerThread;
    const bool direct = host_direct_access();
    if (strided && !direct)
        return fail(RLIC_ERR_UNSUPPORTED,
                    "strided host arrays need a device with pageable-memory access");
    const size_t a_img = align_up(n * sizeof(T));
    const size_t total = (direct ? 2 : 4) * a_img + wl.total + kAlign;
    unsigned char* d = nullptr;
    RLIC_CUDA_TRY(scratch_alloc(reinterpret_cast<void**>(&d), total, stream));
    T* d_tex = reinterpret_cast<T*>(d);
    T* d_out = reinterpret_cast<T*>(d + a_img);  // device ping-pong / result buffer
    T* d_u = direct ? const_cast<T*>(u) : reinterpret_cast<T*>(d + 2 * a_img);
    T* d_v = direct ? const_cast<T*>(v) : reinterpret_cast<T*>(d + 3 * a_img);
    unsigned char* ws = d + (direct ? 2 : 4) * a_img;
    T* d_kernel = reinterpret_cast<T*>(ws + wl.kernel);
    unsigned* d_flag = reinterpret_cast<unsigned*>(ws + wl.total);
    // page-locked output is mapped already: nothing to touch
    cudaPointerAttributes out_attr{};
    bool prefaulted = cudaPointerGetAttributes(&out_attr, out) == cudaSuccess &&
                      out_attr.type == cudaMemoryTypeHost;
    cudaGetLastError();  // a pageable pointer is not an error to keep
    auto prefault = [&]() {
        if (!prefaulted) touch_pages(out, n * sizeof(T));
        prefaulted = true;
    };
    // The inputs cross to the device in row chunks on an auxiliary stream,
    // and the first pass starts on the tile rows whose rows and halo (klen/2
    // rows, wrapped across a periodic edge) have arrived, so the upload
    // overlaps the traced pass.
    std::vector<cudaEvent_t> events;
    cudaStream_t aux = nullptr, second = nullptr;
    auto body = [&]() -> int {
        RLIC_CUDA_TRY(cudaMemcpyAsync(d_kernel, kernel, size_t(klen) * sizeof(T),
                                      cudaMemcpyHostToDevice, stream));
        cudaError_t e = cudaSuccess;
        const int64_t R = klen / 2;
        // up to RLIC_HOST_CHUNKS chunks of at least max(2R, 64) rows and
        // 2^20 pixels, for images of 4 Mpx and more
        const int nchunks =
            n < (size_t(1) << 22)
                ? 1
                : int(std::max<int64_t>(
                      1, std::min<int64_t>(std::min<int64_t>(RLIC_HOST_CHUNKS, int64_t(n >> 20)),
                                           ny / std::max<int64_t>(2 * R, 64))));
        const int64_t rows_per = (ny + nchunks - 1) / nchunks;
        const bool wraps_y = bnd[2] == RLIC_BOUNDARY_PERIODIC || bnd[3] == RLIC_BOUNDARY_PERIODIC;
        std::vector<int> order;
        if (wraps_y && nchunks > 1) order.push_back(nchunks - 1);
        for (int c = 0; c < nchunks; ++c)
            if (!(wraps_y && nchunks > 1 && c == nchunks - 1)) order.push_back(c);
        std::vector<int> arrival(nchunks, 0);
        for (int k = 0; k < nchunks; ++k) arrival[order[k]] = k;
        // one chunk (images under 4 Mpx): the upload and the passes run in
        // order on `stream`, with no second stream and no events
        const bool chunked = nchunks > 1;
        aux = chunked ? aux_stream(&e) : stream;
        if (!aux) return cuda_fail(e, "cudaStreamCreate");
        if (chunked) {
            events.resize(nchunks + 2, nullptr);
            for (auto& ev : events)
                RLIC_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        }
        // the traced pass's groups of tile rows alternate between `stream` and
        // a second stream, so that one group's last CTAs overlap the next
        // group's first ones (launches on one stream would each drain first)
        second = chunked ? aux_stream(&e, false) : nullptr;
        if (chunked && !second) return cuda_fail(e, "cudaStreamCreate");
        // the packs OR into the field's NaN flag, which the traced pass reads,
        // and the texture's uploads (or its check) into d_flag, which follows
        // it in the scratch: one memset clears both
        unsigned* nan_flag = reinterpret_cast<unsigned*>(ws + wl.nan);
        RLIC_CUDA_TRY(
            cudaMemsetAsync(nan_flag, 0, (wl.total - wl.nan) + sizeof(unsigned), stream));
        const bool check = (flags & RLIC_FLAG_CHECK_TEXTURE) != 0;
        // the scratch was allocated stream-ordered on `stream`
        if (chunked) {
            RLIC_CUDA_TRY(cudaEventRecord(events[nchunks], stream));
            RLIC_CUDA_TRY(cudaStreamWaitEvent(aux, events[nchunks], 0));
            RLIC_CUDA_TRY(cudaStreamWaitEvent(second, events[nchunks], 0));
        }
        unsigned char* uvb = ws + wl.uv;
        const bool cache = use_path_cache(iterations, klen, flags);
        const Shape sh = make_shape(ny, nx, bnd);
        const LaunchConfig lc = launch_config_for(ny, nx, sizeof(T), klen);
        const int64_t tiles_x = (nx + lc.block_x - 1) / lc.block_x;
        const int64_t tile_rows = (ny + lc.block_y - 1) / lc.block_y;
        // arrival position after which each tile row has its rows and halo
        std::vector<int> need(size_t(tile_rows), 0);
        for (int64_t tr = 0; tr < tile_rows; ++tr) {
            const int64_t lo = tr * lc.block_y - R;
            const int64_t hi = std::min(ny, (tr + 1) * lc.block_y) - 1 + R;
            for (int c = 0; c < nchunks; ++c) {
                const int64_t c0 = c * rows_per, c1 = std::min(ny, c0 + rows_per);
                bool hit = false;
                if (wraps_y && hi - lo + 1 >= ny) {
                    hit = true;
                } else if (wraps_y) {  // rows lo..hi modulo ny
                    for (int64_t shift = -ny; shift <= ny && !hit; shift += ny)
                        hit = std::max(lo, c0 + shift) <= std::min(hi, c1 - 1 + shift);
                } else {
                    hit = std::max<int64_t>(lo, c0) <= std::min<int64_t>(hi, c1 - 1);
                }
                if (hit && c0 < c1) need[tr] = std::max(need[tr], arrival[c]);
            }
        }
        uint32_t* codes = reinterpret_cast<uint32_t*>(ws + wl.codes);
        T* tmp = reinterpret_cast<T*>(ws + wl.tmp);
        T* final_dst = direct ? out : d_out;
        auto dst_of = [&](int64_t it) -> T* {
            if (it + 1 == iterations) return final_dst;
            return ((iterations - 1 - it) % 2 == 0) ? d_out : tmp;
        };
        if (iterations == 1) prefault();
        const int mode = cache ? rlic::kPassSampleRecord : rlic::kPassSample;
        for (int k = 0; k < nchunks; ++k) {
            const int64_t r0 = order[k] * rows_per, r1 = std::min(ny, r0 + rows_per);
            if (r0 < r1) {
                const size_t off = size_t(r0) * size_t(nx), cnt = size_t(r1 - r0) * size_t(nx);
                void* uv_rows = uvb + off * 2 * sizeof(T);
                if (strided || direct) {  // kernels reading the caller's memory: no host stall
                    RLIC_CUDA_TRY(rlic::launch_gather_strided(texture + r0 * st[0], st[0], st[1],
                                                              d_tex + off, r1 - r0, nx, aux,
                                                              check ? d_flag : nullptr));
                    RLIC_CUDA_TRY(rlic::launch_pack_strided(u + r0 * st[2], st[2], st[3],
                                                            v + r0 * st[4], st[4], st[5],
                                                            uv_rows, r1 - r0, nx, aux, nan_flag));
                } else {
                    RLIC_CUDA_TRY(cudaMemcpyAsync(d_tex + off, texture + off, cnt * sizeof(T),
                                                  cudaMemcpyHostToDevice, aux));
                    RLIC_CUDA_TRY(cudaMemcpyAsync(d_u + off, u + off, cnt * sizeof(T),
                                                  cudaMemcpyHostToDevice, aux));
                    RLIC_CUDA_TRY(cudaMemcpyAsync(d_v + off, v + off, cnt * sizeof(T),
                                                  cudaMemcpyHostToDevice, aux));
                    RLIC_CUDA_TRY(rlic::launch_pack(d_u + off, d_v + off, uv_rows, int64_t(cnt),
                                                    aux, nan_flag));
                }
            }
            if (chunked) RLIC_CUDA_TRY(cudaEventRecord(events[k], aux));
            // first pass over the tile rows this arrival completes, by runs,
            // on the stream of this arrival's turn
            cudaStream_t ps = (second && (k & 1)) ? second : stream;
            bool waited = false;
            for (int64_t tr = 0; tr < tile_rows;) {
                if (need[tr] != k) {
                    ++tr;
                    continue;
                }
                int64_t tr_end = tr + 1;
                while (tr_end < tile_rows && need[tr_end] == k) ++tr_end;
                if (!waited && chunked) RLIC_CUDA_TRY(cudaStreamWaitEvent(ps, events[k], 0));
                waited = true;
                LaunchConfig part = lc;
                part.tile_begin = tr * tiles_x;
                part.tile_count = (tr_end - tr) * tiles_x;
                // a NaN in a chunk that has not arrived yet cannot be reached
                // from these tile rows, so the flag's value now suffices
                part.field_nan = nan_flag;
                RLIC_CUDA_TRY(rlic::launch_pass(var, mode, d_tex, uvb, d_kernel, int(klen), sh,
                                                part, dst_of(0), codes, ps));
                tr = tr_end;
            }
        }
        if (chunked) {  // the second stream's launches and the last upload end first
            RLIC_CUDA_TRY(cudaEventRecord(events[nchunks + 1], second));
            RLIC_CUDA_TRY(cudaStreamWaitEvent(stream, events[nchunks + 1], 0));
            RLIC_CUDA_TRY(cudaStreamWaitEvent(stream, events[nchunks - 1], 0));
        }
        // copied uploads: the texture's check is a pass of its own
        if (check && !(strided || direct))
            RLIC_CUDA_TRY(rlic::launch_check_negative(d_tex, int64_t(n), d_flag, stream));
        const T* src = dst_of(0);
        // every chunk has arrived: the field's NaN flag is final
        LaunchConfig later = lc;
        later.field_nan = nan_flag;
        for (int64_t it = 1; it < iterations; ++it) {
            if (it + 1 == iterations) prefault();
            T* dst = dst_of(it);
            if (cache) {
                RLIC_CUDA_TRY(replay_pass(var.fma, src, codes, d_kernel, int(klen), sh, later,
                                          dst, stream));
            } else {
                RLIC_CUDA_TRY(rlic::launch_pass(var, rlic::kPassSample, src, uvb, d_kernel,
                                                int(klen), sh, later, dst, codes, stream));
            }
            src = dst;
        }
        prefault();
        if (!direct)
            RLIC_CUDA_TRY(cudaMemcpyAsync(out, d_out, n * sizeof(T), cudaMemcpyDeviceToHost, stream));
        return RLIC_OK;
    };
    rc = body();
    // an upload still queued after a failure must end before the scratch is released
    if (rc != RLIC_OK && aux) cudaStreamSynchronize(aux);
    if (rc != RLIC_OK && second) cudaStreamSynchronize(second);
    unsigned negative = 0;
    cudaError_t ec = cudaSuccess;
    if (rc == RLIC_OK && (flags & RLIC_FLAG_CHECK_TEXTURE))
        ec = cudaMemcpyAsync(&negative, d_flag, sizeof(unsigned), cudaMemcpyDeviceToHost, stream);
    cudaError_t ef = cudaFreeAsync(d, stream);
    cudaError_t es = cudaStreamSynchronize(stream);
    for (auto ev : events)
        if (ev) cudaEventDestroy(ev);
    if (rc) return rc;
    if (ec != cudaSuccess) return cuda_fail(ec, "cudaMemcpyAsync");
    if (ef != cudaSuccess) return cuda_fail(ef, "cudaFreeAsync");
    if (es != cudaSuccess) return cuda_fail(es, "cudaStreamSynchronize");
    if (negative)
        return fail(RLIC_ERR_NEGATIVE_TEXTURE,
                    "Found invalid texture element(s). Expected only positive values.");
    return RLIC_OK;
}

template <typename T>
int trace_cells_impl(const T* u, const T* v, int64_t ny, int64_t nx, int64_t klen, int uv_mode,
                     int bxl, int bxr, int byl, int byr, int64_t npix, const int64_t* pix,
                     int64_t* cells, void* stream_, unsigned flags) {
    g_last_error.clear();
    const int bnd[4] = {bxl, bxr, byl, byr};
    int rc = check_common(ny, nx, klen, uv_mode, bnd, flags);
    if (rc) return rc;
    if (flags & RLIC_FLAG_NO_PATH_CACHE)
        return fail(RLIC_ERR_INVALID_ARGUMENT, "unknown flag bits for this entry point");
    if (npix < 0) return fail(RLIC_ERR_INVALID_ARGUMENT, "npix must be >= 0");
    if (!u || !v || (npix > 0 && (!pix || !cells)))
        return fail(RLIC_ERR_INVALID_ARGUMENT, "null array pointer");
    if (npix == 0 || klen == 1) return RLIC_OK;
    const Variant var = make_variant(flags, uv_mode);
    cudaStream_t stream = static_cast<cudaStream_t>(stream_);
    const size_t n = size_t(ny) * size_t(nx);
    const bool host = flags & RLIC_FLAG_HOST_MEMORY;
    const size_t a_uv = align_up(2 * n * sizeof(T));
    const size_t a_img = align_up(n * sizeof(T));
    const size_t a_pix = align_up(size_t(npix) * sizeof(int64_t));
    const size_t a_cells = align_up(size_t(npix) * size_t(klen - 1) * sizeof(int64_t));
    const size_t total = a_uv + (host ? 2 * a_img + a_pix + a_cells : 0);
    unsigned char* d = nullptr;
    RLIC_CUDA_TRY(scratch_alloc(reinterpret_cast<void**>(&d), total, stream));
    void* uv = d;
    auto body = [&]() -> int {
        const T* du = u;
        const T* dv = v;
        const int64_t* dpix = pix;
        int64_t* dcells = cells;
        if (host) {
            T* hu = reinterpret_cast<T*>(d + a_uv);
            T* hv = reinterpret_cast<T*>(d + a_uv + a_img);
            int64_t* hp = reinterpret_cast<int64_t*>(d + a_uv + 2 * a_img);
            dcells = reinterpret_cast<int64_t*>(d + a_uv + 2 * a_img + a_pix);
            RLIC_CUDA_TRY(cudaMemcpyAsync(hu, u, n * sizeof(T), cudaMemcpyHostToDevice, stream));
            RLIC_CUDA_TRY(cudaMemcpyAsync(hv, v, n * sizeof(T), cudaMemcpyHostToDevice, stream));
            RLIC_CUDA_TRY(cudaMemcpyAsync(hp, pix, size_t(npix) * sizeof(int64_t),
                                          cudaMemcpyHostToDevice, stream));
            du = hu;
            dv = hv;
            dpix = hp;
        }
        RLIC_CUDA_TRY(rlic::launch_pack(du, dv, uv, int64_t(n), stream));
        RLIC_CUDA_TRY(rlic::launch_trace_cells(var, static_cast<const T*>(nullptr), uv,
                                               make_shape(ny, nx, bnd), int(klen), npix, dpix,
                                               dcells, stream));
        if (host)
            RLIC_CUDA_TRY(cudaMemcpyAsync(cells, dcells,
                                          size_t(npix) * size_t(klen - 1) * sizeof(int64_t),
                                          cudaMemcpyDeviceToHost, stream));
        return RLIC_OK;
    };
    rc = body();
    cudaError_t ef = cudaFreeAsync(d, stream);
    if (host) {
        cudaError_t es = cudaStreamSynchronize(stream);
        if (!rc && es != cudaSuccess) return cuda_fail(es, "cudaStreamSynchronize");
    }
    if (rc) return rc;
    if (ef != cudaSuccess) return cuda_fail(ef, "cudaFreeAsync");
    return RLIC_OK;
}

template <typename T>
int pack_field_impl(const T* u, const T* v, int64_t ny, int64_t nx, void* uv, void* stream_) {
    g_last_error.clear();
    if (ny <= 0 || nx <= 0)
        return fail(RLIC_ERR_INVALID_ARGUMENT, "image dimensions must be positive");
    if (!u || !v || !uv) return fail(RLIC_ERR_INVALID_ARGUMENT, "null array pointer");
    if (reinterpret_cast<uintptr_t>(uv) % (2 * sizeof(T)) != 0)
        return fail(RLIC_ERR_INVALID_ARGUMENT, "packed field must be aligned to 2 elements");
    RLIC_CUDA_TRY(rlic::launch_pack(u, v, uv, ny * nx, static_cast<cudaStream_t>(stream_)));
    return RLIC_OK;
}

template <typename T>
int sweep_impl(const T* tex_in, const void* uv, int64_t ny, int64_t nx, const T* kernel,
               int64_t klen, int uv_mode, int bxl, int bxr, int byl, int byr, T* tex_out,
               void* codes, void* stream_, unsigned flags) {
    g_last_error.clear();
    const int bnd[4] = {bxl, bxr, byl, byr};
    int rc = check_common(ny, nx, klen, uv_mode, bnd, flags & ~RLIC_FLAG_FIELD_NAN_FREE);
    if (rc) return rc;
    if (flags & (RLIC_FLAG_HOST_MEMORY | RLIC_FLAG_NO_PATH_CACHE | RLIC_FLAG_CHECK_TEXTURE))
        return fail(RLIC_ERR_INVALID_ARGUMENT,
                    "this entry point takes the variant flags and RLIC_FLAG_FIELD_NAN_FREE only");
    if (!tex_in || !uv || !kernel || !tex_out)
        return fail(RLIC_ERR_INVALID_ARGUMENT, "null array pointer");
    if (codes && reinterpret_cast<uintptr_t>(codes) % 4 != 0)
        return fail(RLIC_ERR_INVALID_ARGUMENT, "codes must be 4-byte aligned");
    const Variant var = make_variant(flags, uv_mode);
    LaunchConfig lc = launch_config_for(ny, nx, sizeof(T), klen);
    if (flags & RLIC_FLAG_FIELD_NAN_FREE) {
        cudaError_t e = cudaSuccess;
        lc.field_nan = rlic::zero_flag(&e);
        if (!lc.field_nan) return cuda_fail(e, "cudaGetSymbolAddress");
    }
    RLIC_CUDA_TRY(rlic::launch_pass(var,
                                    (codes != nullptr && klen > 1) ? rlic::kPassSampleRecord
                                                                   : rlic::kPassSample,
                                    tex_in, uv, kernel, int(klen), make_shape(ny, nx, bnd), lc,
                                    tex_out, static_cast<uint32_t*>(codes),
                                    static_cast<cudaStream_t>(stream_)));
    return RLIC_OK;
}

template <typename T>
int replay_impl(const T* tex_in, const void* codes, int64_t ny, int64_t nx, const T* kernel,
                int64_t klen, T* tex_out, void* stream_, unsigned flags) {
    g_last_error.clear();
    int rc = check_shape(ny, nx, klen);
    if (rc) return rc;
    if (flags & ~unsigned(RLIC_FLAG_NO_FMA | RLIC_FLAG_FIELD_NAN_FREE))
        return fail(RLIC_ERR_INVALID_ARGUMENT,
                    "this entry point takes RLIC_FLAG_NO_FMA and RLIC_FLAG_FIELD_NAN_FREE only");
    if (!tex_in || !kernel || !tex_out || (!codes && klen > 1))
        return fail(RLIC_ERR_INVALID_ARGUMENT, "null array pointer");
    if (codes && reinterpret_cast<uintptr_t>(codes) % 4 != 0)
        return fail(RLIC_ERR_INVALID_ARGUMENT, "codes must be 4-byte aligned");
    // the codes may hold wraps across any edge (the boundaries they were
    // recorded with are not known here): treat every side as periodic, so
    // that the staged form stages no box that crosses an edge (the L1 form
    // reads only the image size)
    const int bnd[4] = {1, 1, 1, 1};
    LaunchConfig lc = launch_config();
    if (flags & RLIC_FLAG_FIELD_NAN_FREE) {  // codes recorded from a NaN-free field
        cudaError_t e = cudaSuccess;
        lc.field_nan = rlic::zero_flag(&e);
        if (!lc.field_nan) return cuda_fail(e, "cudaGetSymbolAddress");
    }
    RLIC_CUDA_TRY(replay_pass(!(flags & RLIC_FLAG_NO_FMA), tex_in,
                              static_cast<const uint32_t*>(codes), kernel, int(klen),
                              make_shape(ny, nx, bnd), lc, tex_out,
                              static_cast<cudaStream_t>(stream_)));
    return RLIC_OK;
}

// -------------------------------------------------- reduced-precision form --

struct LowpLayout {
    size_t uv, codes, buf_a, buf_b, w32, scal, total;
};

LowpLayout lowp_layout(int64_t ny, int64_t nx, int64_t klen, size_t s) {
    const size_t n = size_t(ny) * size_t(nx);
    LowpLayout w{};
    size_t off = 0;
    w.uv = off;
    off += align_up(2 * n * s);
    w.codes = off;
    off += align_up(code_bytes(ny, nx, klen));
    w.buf_a = off;
    off += align_up(2 * n);
    w.buf_b = off;
    off += align_up(2 * n);
    w.w32 = off;
    off += align_up(size_t(klen) * 4);
    w.scal = off;  // float 1/sum(|kernel|) at +0, double undo factor at +8,
                   // NaN flag of the packed field at +16
    off += align_up(20);
    w.total = off;
    return w;
}

template <typename T>
int convolve_lowp_impl(const T* texture, const T* u, const T* v, int64_t ny, int64_t nx,
                       const T* kernel, int64_t klen, int uv_mode, int bxl, int bxr, int byl,
                       int byr, int64_t iterations, int storage, T* out, void* workspace,
                       size_t workspace_bytes_, void* stream_, unsigned flags) {
    g_last_error.clear();
    const int bnd[4] = {bxl, bxr, byl, byr};
    int rc = check_common(ny, nx, klen, uv_mode, bnd, flags);
    if (rc) return rc;
    if (flags & (RLIC_FLAG_HOST_MEMORY | RLIC_FLAG_NO_PATH_CACHE))
        return fail(RLIC_ERR_INVALID_ARGUMENT, "this entry point takes the variant flags only");
    if (storage != RLIC_STORAGE_FP16 && storage != RLIC_STORAGE_BF16)
        return fail(RLIC_ERR_INVALID_ARGUMENT, "storage must be RLIC_STORAGE_FP16 or _BF16");
    if (iterations < 0) return fail(RLIC_ERR_INVALID_ARGUMENT, "iterations must be >= 0");
    if (!texture || !u || !v || !kernel || !out)
        return fail(RLIC_ERR_INVALID_ARGUMENT, "null array pointer");
    cudaStream_t stream = static_cast<cudaStream_t>(stream_);
    const int64_t n = ny * nx;
    if (iterations == 0) {
        RLIC_CUDA_TRY(cudaMemsetAsync(out, 0, size_t(n) * sizeof(T), stream));
        return RLIC_OK;
    }
    const LowpLayout wl = lowp_layout(ny, nx, klen, sizeof(T));
    unsigned char* ws = static_cast<unsigned char*>(workspace);
    bool owned = false;
    if (ws == nullptr) {
        RLIC_CUDA_TRY(scratch_alloc(reinterpret_cast<void**>(&ws), wl.total, stream));
        owned = true;
    } else {
        if (workspace_bytes_ < wl.total)
            return fail(RLIC_ERR_WORKSPACE_TOO_SMALL,
                        "workspace smaller than rlic_lowp_workspace_bytes()");
        if (reinterpret_cast<uintptr_t>(ws) % kAlign != 0)
            return fail(RLIC_ERR_INVALID_ARGUMENT, "workspace must be 256-byte aligned");
    }
    auto body = [&]() -> int {
        const Shape sh = make_shape(ny, nx, bnd);
        const LaunchConfig lc = launch_config_for(ny, nx, sizeof(T), klen);
        void* uv = ws + wl.uv;
        uint32_t* codes = reinterpret_cast<uint32_t*>(ws + wl.codes);
        float* w32 = reinterpret_cast<float*>(ws + wl.w32);
        float* inv_scale = reinterpret_cast<float*>(ws + wl.scal);
        double* undo = reinterpret_cast<double*>(ws + wl.scal + 8);
        void* bufs[2] = {ws + wl.buf_a, ws + wl.buf_b};
        unsigned* nan_flag = reinterpret_cast<unsigned*>(ws + wl.scal + 16);
        RLIC_CUDA_TRY(cudaMemsetAsync(nan_flag, 0, sizeof(unsigned), stream));
        RLIC_CUDA_TRY(rlic::launch_pack(u, v, uv, n, stream, nan_flag));
        LaunchConfig trace_lc = lc;
        trace_lc.field_nan = nan_flag;
        RLIC_CUDA_TRY(rlic::launch_pass(make_variant(flags, uv_mode), rlic::kPassRecordOnly,
                                        static_cast<const T*>(nullptr), uv, kernel, int(klen), sh,
                                        trace_lc, static_cast<T*>(nullptr), codes, stream));
        RLIC_CUDA_TRY(rlic::launch_lowp_prepare(kernel, int(klen), iterations, w32, inv_scale,
                                                undo, stream));
        RLIC_CUDA_TRY(rlic::launch_to_storage(texture, bufs[0], storage, n, stream));
        const int mode = g_replay_mode.load();
        const bool staged =
            mode == RLIC_REPLAY_STAGED || (mode == RLIC_REPLAY_AUTO && kStagedByDefault);
        for (int64_t it = 0; it < iterations; ++it) {
            cudaError_t e = cudaErrorNotSupported;
            if (staged)
                e = rlic::launch_gather_staged_lowp(storage, bufs[it % 2], codes, w32, int(klen),
                                                    inv_scale, sh, nan_flag, bufs[(it + 1) % 2],
                                                    stream);
            if (e == cudaErrorNotSupported)
                e = rlic::launch_gather_lowp(storage, bufs[it % 2], codes, w32, int(klen),
                                             inv_scale, sh, launch_config(), bufs[(it + 1) % 2],
                                             stream);
            RLIC_CUDA_TRY(e);
        }
        RLIC_CUDA_TRY(rlic::launch_from_storage(bufs[iterations % 2], storage, undo, out, n,
                                                stream));
        return RLIC_OK;
    };
    rc = body();
    if (owned) {
        cudaError_t e = cudaFreeAsync(ws, stream);
        if (rc == RLIC_OK && e != cudaSuccess) return cuda_fail(e, "cudaFreeAsync");
    }
    return rc;
}

// --------------------------------------------------------------- adjoint --

template <typename T>
int adjoint_impl(const T* g, const void* codes, int64_t ny, int64_t nx, const T* kernel,
                 int64_t klen, T* y, void* stream_, unsigned flags) {
    g_last_error.clear();
    int rc = check_shape(ny, nx, klen);
    if (rc) return rc;
    if (flags) return fail(RLIC_ERR_INVALID_ARGUMENT, "this entry point takes no flags");
    if (!g || !kernel || !y || (!codes && klen > 1))
        return fail(RLIC_ERR_INVALID_ARGUMENT, "null array pointer");
    if (codes && reinterpret_cast<uintptr_t>(codes) % 4 != 0)
        return fail(RLIC_ERR_INVALID_ARGUMENT, "codes must be 4-byte aligned");
    const int bnd[4] = {0, 0, 0, 0};
    RLIC_CUDA_TRY(rlic::launch_scatter(g, static_cast<const uint32_t*>(codes), kernel, int(klen),
                                       make_shape(ny, nx, bnd), y,
                                       static_cast<cudaStream_t>(stream_)));
    return RLIC_OK;
}

template <typename T>
int kernel_grad_impl(const T* g, const T* x, const void* codes, int64_t ny, int64_t nx,
                     int64_t klen, double* dw, void* stream_, unsigned flags) {
    g_last_error.clear();
    int rc = check_shape(ny, nx, klen);
    if (rc) return rc;
    if (flags) return fail(RLIC_ERR_INVALID_ARGUMENT, "this entry point takes no flags");
    if (!g || !x || !dw || (!codes && klen > 1))
        return fail(RLIC_ERR_INVALID_ARGUMENT, "null array pointer");
    if (codes && reinterpret_cast<uintptr_t>(codes) % 4 != 0)
        return fail(RLIC_ERR_INVALID_ARGUMENT, "codes must be 4-byte aligned");
    const int bnd[4] = {0, 0, 0, 0};
    RLIC_CUDA_TRY(rlic::launch_kernel_grad(g, x, static_cast<const uint32_t*>(codes), int(klen),
                                           make_shape(ny, nx, bnd), dw,
                                           static_cast<cudaStream_t>(stream_)));
    return RLIC_OK;
}

// ------------------------------------------------------------ batched form --

struct BatchLayout {
    size_t insts, levels, flags, queue, counters, total;
    std::vector<size_t> uv, tmp, codes;  // per item
    int max_iterations;
    int nseg;  // segments of the persistent queue
};

int batch_replay_tiles(const rlic_batch_item_f32& it) { return it.replay_tiles ? it.replay_tiles : 4; }

// Segments of the persistent queue: one per (item, level) for levels
// 0 (pack) .. iterations.
int batch_segments(const rlic_batch_item_f32* items, int count) {
    int64_t n = 0;
    for (int k = 0; k < count; ++k)
        if (items[k].iterations > 0) n += items[k].iterations + 1;
    return int(n);
}

bool batch_tile_ok(int tx) { return tx == 8 || tx == 16 || tx == 32 || tx == 64 || tx == 128 || tx == 256; }

int batch_check(const rlic_batch_item_f32* items, int count) {
    if (count <= 0 || !items) return fail(RLIC_ERR_INVALID_ARGUMENT, "empty batch");
    if (count > 1024) return fail(RLIC_ERR_INVALID_ARGUMENT, "at most 1024 items per batch");
    for (int k = 0; k < count; ++k) {
        const auto& it = items[k];
        const int bnd[4] = {it.bx_left, it.bx_right, it.by_left, it.by_right};
        int rc = check_common(it.ny, it.nx, it.klen, it.uv_mode, bnd, 0);
        if (rc) return fail(rc, "item " + std::to_string(k) + ": " + g_last_error);
        if (it.ny * it.nx >= (int64_t(1) << 31) - 1)
            return fail(RLIC_ERR_INVALID_ARGUMENT, "item " + std::to_string(k) + ": image too large for a batch");
        if (it.klen > 2 * rlic::kBatchMaxHalf + 1)
            return fail(RLIC_ERR_INVALID_ARGUMENT, "item " + std::to_string(k) + ": kernel longer than 1025 taps");
        if (it.iterations < 0 || it.iterations > 4096)
            return fail(RLIC_ERR_INVALID_ARGUMENT, "item " + std::to_string(k) + ": iterations must be in [0, 4096]");
        if (it.tile_x != 0 && !batch_tile_ok(it.tile_x))
            return fail(RLIC_ERR_INVALID_ARGUMENT, "item " + std::to_string(k) + ": tile_x must be 0 or a power of two in [8, 256]");
        if (it.replay_tiles < 0 || it.replay_tiles > 64)
            return fail(RLIC_ERR_INVALID_ARGUMENT, "item " + std::to_string(k) + ": replay_tiles must be in [0, 64]");
        if (!it.texture || !it.u || !it.v || !it.kernel || !it.out)
            return fail(RLIC_ERR_INVALID_ARGUMENT, "item " + std::to_string(k) + ": null array pointer");
    }
    return RLIC_OK;
}

BatchLayout batch_layout(const rlic_batch_item_f32* items, int count) {
    BatchLayout L;
    size_t off = 0;
    L.insts = off;
    off += align_up(size_t(count) * sizeof(rlic::BatchInstance));
    L.max_iterations = 0;
    for (int k = 0; k < count; ++k) L.max_iterations = std::max<int>(L.max_iterations, int(items[k].iterations));
    L.levels = off;
    off += align_up(size_t(std::max(L.max_iterations, 1)) * size_t(count) * (sizeof(int64_t) + sizeof(int)));
    L.flags = off;  // one NaN flag per item
    off += align_up(size_t(count) * sizeof(unsigned));
    L.nseg = batch_segments(items, count);
    L.queue = off;  // segment starts (nseg + 1 ints), then the segments
    off += align_up(size_t(L.nseg + 1) * sizeof(int)) +
           align_up(size_t(L.nseg) * sizeof(rlic::BatchSegment));
    L.counters = off;  // next item, timeout word, then finished items per segment
    off += align_up(size_t(L.nseg + 2) * sizeof(unsigned));
    for (int k = 0; k < count; ++k) {
        const auto& it = items[k];
        const size_t n = size_t(it.ny) * size_t(it.nx);
        L.uv.push_back(off);
        off += align_up(2 * n * sizeof(float));
        L.tmp.push_back(off);
        if (it.iterations >= 2) off += align_up(n * sizeof(float));
        L.codes.push_back(off);
        if (it.iterations >= 2 && it.klen > 1) off += align_up(code_bytes(it.ny, it.nx, it.klen));
    }
    L.total = off;
    return L;
}

int convolve_batch_f32(const rlic_batch_item_f32* items, int count, void* workspace,
                       size_t workspace_bytes_, void* stream_, unsigned flags) {
    g_last_error.clear();
    int rc = batch_check(items, count);
    if (rc) return rc;
    if (flags & ~unsigned(RLIC_FLAG_BATCH_PREPARED | RLIC_FLAG_BATCH_QUEUE))
        return fail(RLIC_ERR_INVALID_ARGUMENT,
                    "this entry point takes RLIC_FLAG_BATCH_PREPARED and RLIC_FLAG_BATCH_QUEUE only");
    if (!workspace) return fail(RLIC_ERR_INVALID_ARGUMENT, "the batched form needs a workspace");
    const BatchLayout L = batch_layout(items, count);
    if (workspace_bytes_ < L.total)
        return fail(RLIC_ERR_WORKSPACE_TOO_SMALL, "workspace smaller than rlic_batch_workspace_bytes_f32()");
    if (reinterpret_cast<uintptr_t>(workspace) % kAlign != 0)
        return fail(RLIC_ERR_INVALID_ARGUMENT, "workspace must be 256-byte aligned");
    cudaStream_t stream = static_cast<cudaStream_t>(stream_);
    unsigned char* ws = static_cast<unsigned char*>(workspace);
    auto* dev_insts = reinterpret_cast<rlic::BatchInstance*>(ws + L.insts);
    auto* dev_starts = reinterpret_cast<int64_t*>(ws + L.levels);
    auto* dev_index = reinterpret_cast<int*>(ws + L.levels + size_t(std::max(L.max_iterations, 1)) *
                                                                 size_t(count) * sizeof(int64_t));
    // host tables: instances, then for every level the participating instances
    std::vector<rlic::BatchInstance> insts(count);
    std::vector<int64_t> starts(size_t(std::max(L.max_iterations, 1)) * count, 0);
    std::vector<int> index(starts.size(), 0);
    std::vector<rlic::BatchLevel> levels(L.max_iterations + 1);
    int64_t max_pixels = 0;
    for (int k = 0; k < count; ++k) {
        const auto& it = items[k];
        auto& b = insts[k];
        b.texture = it.texture;
        b.u = it.u;
        b.v = it.v;
        b.kernel = it.kernel;
        b.out = it.out;
        b.tmp = reinterpret_cast<float*>(ws + L.tmp[k]);
        b.uv = ws + L.uv[k];
        b.codes = reinterpret_cast<uint32_t*>(ws + L.codes[k]);
        b.nan_flag = reinterpret_cast<unsigned*>(ws + L.flags) + k;
        b.ny = int(it.ny);
        b.nx = int(it.nx);
        b.klen = int(it.klen);
        b.iterations = int(it.iterations);
        b.pol = it.uv_mode == RLIC_UV_POLARIZATION;
        b.bnd[0] = it.bx_left;
        b.bnd[1] = it.bx_right;
        b.bnd[2] = it.by_left;
        b.bnd[3] = it.by_right;
        b.tile_x = it.tile_x ? it.tile_x : 64;
        b.tile_y = 256 / b.tile_x;
        b.tiles_x = int((it.nx + b.tile_x - 1) / b.tile_x);
        b.ntiles = b.tiles_x * int((it.ny + b.tile_y - 1) / b.tile_y);
        b.replay_tiles = batch_replay_tiles(it);
        max_pixels = std::max<int64_t>(max_pixels, it.ny * it.nx);
    }
    for (int level = 1; level <= L.max_iterations; ++level) {
        const size_t base = size_t(level - 1) * size_t(count);
        int m = 0;
        int64_t tiles = 0;
        for (int k = 0; k < count; ++k) {
            if (insts[k].iterations < level) continue;
            starts[base + m] = tiles;
            index[base + m] = k;
            tiles += insts[k].ntiles;
            ++m;
        }
        levels[level] = rlic::BatchLevel{dev_starts + base, dev_index + base, m, tiles};
    }
    // the persistent queue: segments level by level, the largest items first
    // within a level (their previous level was taken first, so it is the
    // first to be finished)
    std::vector<int> seg_start(size_t(L.nseg) + 1, 0);
    std::vector<rlic::BatchSegment> segs(size_t(L.nseg));
    {
        std::vector<int> order(count);
        for (int k = 0; k < count; ++k) order[k] = k;
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
            return items[a].ny * items[a].nx > items[b].ny * items[b].nx;
        });
        std::vector<int> last(count, -1);  // each item's segment of the previous level
        int ns = 0;
        int64_t total = 0;
        for (int level = 0; level <= L.max_iterations; ++level) {
            for (int k : order) {
                const auto& b = insts[k];
                if (b.iterations < std::max(level, 1)) continue;
                int64_t nitems;
                if (level == 0)
                    nitems = (int64_t(b.ny) * b.nx + rlic::kBatchPackChunk - 1) / rlic::kBatchPackChunk;
                else if (level == 1)
                    nitems = b.ntiles;
                else
                    nitems = (int64_t(b.ntiles) + b.replay_tiles - 1) / b.replay_tiles;
                segs[ns] = rlic::BatchSegment{k, level, last[k], int(nitems)};
                seg_start[ns] = int(total);
                last[k] = ns;
                total += nitems;
                ++ns;
                if (total > 0x7fffffffLL)
                    return fail(RLIC_ERR_INVALID_ARGUMENT, "batch too large for one work queue");
            }
        }
        seg_start[ns] = int(total);
    }
    auto* dev_seg_start = reinterpret_cast<int*>(ws + L.queue);
    auto* dev_segs = reinterpret_cast<rlic::BatchSegment*>(
        ws + L.queue + align_up(size_t(L.nseg + 1) * sizeof(int)));
    auto* dev_counters = reinterpret_cast<unsigned*>(ws + L.counters);
    if (!(flags & RLIC_FLAG_BATCH_PREPARED)) {
        // pageable copies: the call returns once the host tables are staged
        RLIC_CUDA_TRY(cudaMemcpyAsync(dev_insts, insts.data(), insts.size() * sizeof(insts[0]),
                                      cudaMemcpyHostToDevice, stream));
        RLIC_CUDA_TRY(cudaMemcpyAsync(dev_seg_start, seg_start.data(),
                                      seg_start.size() * sizeof(int), cudaMemcpyHostToDevice,
                                      stream));
        if (!segs.empty())
            RLIC_CUDA_TRY(cudaMemcpyAsync(dev_segs, segs.data(),
                                          segs.size() * sizeof(rlic::BatchSegment),
                                          cudaMemcpyHostToDevice, stream));
        RLIC_CUDA_TRY(cudaMemcpyAsync(dev_starts, starts.data(), starts.size() * sizeof(int64_t),
                                      cudaMemcpyHostToDevice, stream));
        RLIC_CUDA_TRY(cudaMemcpyAsync(dev_index, index.data(), index.size() * sizeof(int),
                                      cudaMemcpyHostToDevice, stream));
    }
    // iterations == 0 items: zeros, as rlic_convolve_f32
    for (int k = 0; k < count; ++k)
        if (items[k].iterations == 0)
            RLIC_CUDA_TRY(cudaMemsetAsync(items[k].out, 0,
                                          size_t(items[k].ny) * size_t(items[k].nx) * 4, stream));
    if (L.max_iterations == 0) return RLIC_OK;
    RLIC_CUDA_TRY(cudaMemsetAsync(ws + L.flags, 0, size_t(count) * sizeof(unsigned), stream));
    // the queue's counters (and its timeout word, which rlic_batch_status_f32
    // reads after either form) start at zero
    RLIC_CUDA_TRY(cudaMemsetAsync(dev_counters, 0, size_t(L.nseg + 2) * sizeof(unsigned), stream));
    if (!(flags & RLIC_FLAG_BATCH_QUEUE)) {
        RLIC_CUDA_TRY(rlic::launch_batch_pack(dev_insts, count, max_pixels, stream));
        for (int level = 1; level <= L.max_iterations; ++level)
            RLIC_CUDA_TRY(rlic::launch_batch_level(dev_insts, levels[level], level, stream));
        return RLIC_OK;
    }
    rlic::BatchQueue q;
    q.seg_start = dev_seg_start;
    q.segs = dev_segs;
    q.nseg = L.nseg;
    q.total = seg_start[L.nseg];
    q.next = dev_counters;
    q.timeout = dev_counters + 1;
    q.done = dev_counters + 2;
    RLIC_CUDA_TRY(rlic::launch_batch_queue(dev_insts, q, stream));
    return RLIC_OK;
}

// 1 if a persistent batched run of these items on this workspace gave up a
// wait, 0 if not (synchronises the device).
int batch_status_f32(const rlic_batch_item_f32* items, int count, const void* workspace) {
    g_last_error.clear();
    int rc = batch_check(items, count);
    if (rc) return -rc;
    if (!workspace) return -fail(RLIC_ERR_INVALID_ARGUMENT, "null workspace");
    const BatchLayout L = batch_layout(items, count);
    unsigned v = 0;
    const cudaError_t e = cudaMemcpy(&v, static_cast<const unsigned char*>(workspace) +
                                             L.counters + sizeof(unsigned),
                                     sizeof(v), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return -cuda_fail(e, "cudaMemcpy");
    return v ? 1 : 0;
}

// ------------------------------------------------------- no-allocation path --
//
// Scratch of rlic_convolve_f32_noalloc, for callers that cannot allocate
// device memory themselves (see the header).  It is a file-scope device
// array, so the module holds it on every GPU that loads this library, for
// the life of the process.  In host code the array's name only stands for
// the symbol; its device address comes from cudaGetSymbolAddress, resolved
// once per device (with that device current) and cached.
constexpr size_t kStaticScratchBytes = size_t(RLIC_NOALLOC_SCRATCH_BYTES);
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_static_mu;
void* g_static_ptr[kMaxDevices] = {};

int static_scratch(unsigned char** ptr) {
    int dev = -1;
    RLIC_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices)
        return fail(RLIC_ERR_INVALID_ARGUMENT, "device ordinal out of range for static scratch");
    std::lock_guard<std::mutex> lock(g_static_mu);
    if (g_static_ptr[dev] == nullptr) {
        // With lazy module loading (CUDA's default) this lookup is what loads
        // the module and maps the array on this device, so it can run out of
        // memory here, once, on the first call.
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e == cudaErrorMemoryAllocation)
            return fail(RLIC_ERR_OUT_OF_MEMORY,
                        "mapping the " + std::to_string(kStaticScratchBytes >> 20) +
                            " MiB static scratch of rlic_convolve_f32_noalloc on device " +
                            std::to_string(dev) +
                            " failed: out of device memory (make the first call on each "
                            "device early, while memory is free)");
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(static scratch)");
        g_static_ptr[dev] = p;
    }
    *ptr = static_cast<unsigned char*>(g_static_ptr[dev]);
    return RLIC_OK;
}

int convolve_noalloc_f32(const float* texture, const float* u, const float* v, int64_t ny,
                         int64_t nx, const float* kernel, int64_t klen, int uv_mode, int bxl,
                         int bxr, int byl, int byr, int64_t iterations, float* out,
                         void* stream_, unsigned flags) {
    g_last_error.clear();
    const int bnd[4] = {bxl, bxr, byl, byr};
    int rc = check_common(ny, nx, klen, uv_mode, bnd, flags);
    if (rc) return rc;
    if (flags & RLIC_FLAG_HOST_MEMORY)
        return fail(RLIC_ERR_INVALID_ARGUMENT,
                    "rlic_convolve_f32_noalloc takes device pointers only");
    // the texture check belongs to host-memory calls; refusing it here keeps a
    // caller from believing a check ran
    if (flags & RLIC_FLAG_CHECK_TEXTURE)
        return fail(RLIC_ERR_INVALID_ARGUMENT,
                    "rlic_convolve_f32_noalloc does not check the texture "
                    "(RLIC_FLAG_CHECK_TEXTURE applies to host-memory calls)");
    if (iterations < 0) return fail(RLIC_ERR_INVALID_ARGUMENT, "iterations must be >= 0");
    if (!texture || !u || !v || !kernel || !out)
        return fail(RLIC_ERR_INVALID_ARGUMENT, "null array pointer");
    // zero passes only clear `out` and touch no scratch: no size limit
    if (iterations == 0)
        return run_device<float>(texture, u, v, ny, nx, kernel, klen,
                                 make_variant(flags, uv_mode), bnd, iterations, out, nullptr,
                                 flags, static_cast<cudaStream_t>(stream_));
    const WorkspaceLayout wl = workspace_layout(ny, nx, klen, iterations, sizeof(float), flags);
    if (wl.total > kStaticScratchBytes)
        return fail(RLIC_ERR_WORKSPACE_TOO_SMALL,
                    "this call needs " + std::to_string(wl.total) +
                        " bytes of scratch; the static scratch holds " +
                        std::to_string(kStaticScratchBytes) +
                        " (use a smaller image, fewer taps, or RLIC_FLAG_NO_PATH_CACHE)");
    unsigned char* ws = nullptr;
    rc = static_scratch(&ws);
    if (rc) return rc;
    // Every region of the scratch is written before it is read (packed field,
    // ping-pong buffer, path codes), so the previous call's contents need no
    // clearing; the one word that must start at zero, the field's NaN flag,
    // is zeroed by run_device on the stream before the pack kernel sets it.
    return run_device<float>(texture, u, v, ny, nx, kernel, klen, make_variant(flags, uv_mode),
                             bnd, iterations, out, ws, flags, static_cast<cudaStream_t>(stream_));
}

// Histogram equalization (lic_equalize.cu): validation, scratch, host copies.
template <typename T>
int equalize_impl(const T* image, int64_t ny, int64_t nx, int64_t nbins, int strategy,
                  int64_t tile_y, int64_t tile_x, T* out, void* stream_, unsigned flags) {
    g_last_error.clear();
    if (ny < 0 || nx < 0) return fail(RLIC_ERR_INVALID_ARGUMENT, "negative image shape");
    if (nbins < 1 || nbins > rlic::kEqualizeMaxBins)
        return fail(RLIC_ERR_INVALID_ARGUMENT, "nbins must be in [1, 2^24]");
    if (strategy != RLIC_EQUALIZE_GLOBAL && strategy != RLIC_EQUALIZE_SLIDING_TILE &&
        strategy != RLIC_EQUALIZE_TILE_INTERPOLATION)
        return fail(RLIC_ERR_INVALID_ARGUMENT, "unknown equalization strategy");
    if (strategy != RLIC_EQUALIZE_GLOBAL && (tile_y < 1 || tile_x < 1))
        return fail(RLIC_ERR_INVALID_ARGUMENT, "tile shape must be positive");
    if (strategy == RLIC_EQUALIZE_TILE_INTERPOLATION && nbins > rlic::kEqualizeMaxTileBins)
        return fail(RLIC_ERR_UNSUPPORTED, "tile interpolation takes at most 49152 bins");
    if (flags & ~RLIC_FLAG_HOST_MEMORY)
        return fail(RLIC_ERR_INVALID_ARGUMENT, "unknown flag bits for this entry point");
    const size_t n = size_t(ny) * size_t(nx);
    if (n == 0) return RLIC_OK;
    if (!image || !out) return fail(RLIC_ERR_INVALID_ARGUMENT, "null array pointer");
    cudaStream_t stream = static_cast<cudaStream_t>(stream_);
    const bool host = flags & RLIC_FLAG_HOST_MEMORY;
    if (host && stream == nullptr) stream = cudaStreamPerThread;
    const size_t scratch = rlic::equalize_scratch_bytes(ny, nx, nbins, strategy, tile_y, tile_x,
                                                        sizeof(T));
    const size_t a_img = align_up(n * sizeof(T));
    unsigned char* d = nullptr;
    RLIC_CUDA_TRY(scratch_alloc(reinterpret_cast<void**>(&d), scratch + (host ? 2 * a_img : 0),
                                stream));
    const T* src = image;
    T* dst = out;
    cudaError_t e = cudaSuccess;
    if (host) {
        T* d_in = reinterpret_cast<T*>(d + scratch);
        dst = reinterpret_cast<T*>(d + scratch + a_img);
        e = cudaMemcpyAsync(d_in, image, n * sizeof(T), cudaMemcpyHostToDevice, stream);
        src = d_in;
    }
    if (e == cudaSuccess)
        e = rlic::launch_equalize(src, ny, nx, int(nbins), strategy, tile_y, tile_x, dst, d,
                                  stream);
    if (e == cudaSuccess && host)
        e = cudaMemcpyAsync(out, dst, n * sizeof(T), cudaMemcpyDeviceToHost, stream);
    const cudaError_t ef = cudaFreeAsync(d, stream);
    if (host) {
        const cudaError_t es = cudaStreamSynchronize(stream);
        if (e == cudaSuccess) e = es;
    }
    if (e != cudaSuccess) return cuda_fail(e, "histogram equalization");
    if (ef != cudaSuccess) return cuda_fail(ef, "cudaFreeAsync");
    return RLIC_OK;
}

}  // namespace

// -------------------------------------------------------------------- C ABI --

extern "C" {

const char* rlic_version(void) { return "rlic_gb300 0.2.0 (sm_103a)"; }

const char* rlic_last_error(void) { return g_last_error.c_str(); }

size_t rlic_workspace_bytes(int64_t ny, int64_t nx, int64_t klen, int64_t iterations,
                            int elem_bytes, unsigned flags) {
    if (elem_bytes != 4 && elem_bytes != 8) return 0;
    if (ny <= 0 || nx <= 0 || klen <= 0 || iterations < 0) return 0;
    return workspace_layout(ny, nx, klen, iterations, size_t(elem_bytes), flags).total;
}

size_t rlic_path_code_bytes(int64_t ny, int64_t nx, int64_t klen) {
    if (ny <= 0 || nx <= 0 || klen <= 0) return 0;
    return code_bytes(ny, nx, klen);
}

int rlic_convolve_f32(const float* texture, const float* u, const float* v, int64_t ny,
                      int64_t nx, const float* kernel, int64_t klen, int uv_mode, int bx_left,
                      int bx_right, int by_left, int by_right, int64_t iterations, float* out,
                      void* workspace, size_t workspace_bytes, void* stream, unsigned flags) {
    return convolve_impl<float>(texture, u, v, ny, nx, kernel, klen, uv_mode, bx_left, bx_right,
                                by_left, by_right, iterations, out, workspace, workspace_bytes,
                                stream, flags);
}

int rlic_convolve_f64(const double* texture, const double* u, const double* v, int64_t ny,
                      int64_t nx, const double* kernel, int64_t klen, int uv_mode, int bx_left,
                      int bx_right, int by_left, int by_right, int64_t iterations, double* out,
                      void* workspace, size_t workspace_bytes, void* stream, unsigned flags) {
    return convolve_impl<double>(texture, u, v, ny, nx, kernel, klen, uv_mode, bx_left,
                                 bx_right, by_left, by_right, iterations, out, workspace,
                                 workspace_bytes, stream, flags);
}

int rlic_convolve_strided_f32(const float* texture, const float* u, const float* v,
                              const int64_t* strides, int64_t ny, int64_t nx,
                              const float* kernel, int64_t klen, int uv_mode, int bx_left,
                              int bx_right, int by_left, int by_right, int64_t iterations,
                              float* out, void* stream, unsigned flags) {
    if (!strides) return fail(RLIC_ERR_INVALID_ARGUMENT, "null strides");
    if (!(flags & RLIC_FLAG_HOST_MEMORY))
        return fail(RLIC_ERR_INVALID_ARGUMENT, "strided arrays are host memory only");
    return convolve_impl<float>(texture, u, v, ny, nx, kernel, klen, uv_mode, bx_left, bx_right,
                                by_left, by_right, iterations, out, nullptr, 0, stream, flags,
                                strides);
}

int rlic_convolve_strided_f64(const double* texture, const double* u, const double* v,
                              const int64_t* strides, int64_t ny, int64_t nx,
                              const double* kernel, int64_t klen, int uv_mode, int bx_left,
                              int bx_right, int by_left, int by_right, int64_t iterations,
                              double* out, void* stream, unsigned flags) {
    if (!strides) return fail(RLIC_ERR_INVALID_ARGUMENT, "null strides");
    if (!(flags & RLIC_FLAG_HOST_MEMORY))
        return fail(RLIC_ERR_INVALID_ARGUMENT, "strided arrays are host memory only");
    return convolve_impl<double>(texture, u, v, ny, nx, kernel, klen, uv_mode, bx_left,
                                 bx_right, by_left, by_right, iterations, out, nullptr, 0,
                                 stream, flags, strides);
}

int rlic_host_direct_access(void) { return host_direct_access() ? 1 : 0; }

int rlic_trace_cells_f32(const float* u, const float* v, int64_t ny, int64_t nx, int64_t klen,
                         int uv_mode, int bx_left, int bx_right, int by_left, int by_right,
                         int64_t npix, const int64_t* pix, int64_t* cells, void* stream,
                         unsigned flags) {
    return trace_cells_impl<float>(u, v, ny, nx, klen, uv_mode, bx_left, bx_right, by_left,
                                   by_right, npix, pix, cells, stream, flags);
}

int rlic_trace_cells_f64(const double* u, const double* v, int64_t ny, int64_t nx,
                         int64_t klen, int uv_mode, int bx_left, int bx_right, int by_left,
                         int by_right, int64_t npix, const int64_t* pix, int64_t* cells,
                         void* stream, unsigned flags) {
    return trace_cells_impl<double>(u, v, ny, nx, klen, uv_mode, bx_left, bx_right, by_left,
                                    by_right, npix, pix, cells, stream, flags);
}

int rlic_pack_field_f32(const float* u, const float* v, int64_t ny, int64_t nx, void* uv,
                        void* stream) {
    return pack_field_impl<float>(u, v, ny, nx, uv, stream);
}

int rlic_pack_field_f64(const double* u, const double* v, int64_t ny, int64_t nx, void* uv,
                        void* stream) {
    return pack_field_impl<double>(u, v, ny, nx, uv, stream);
}

int rlic_sweep_f32(const float* tex_in, const void* uv, int64_t ny, int64_t nx,
                   const float* kernel, int64_t klen, int uv_mode, int bx_left, int bx_right,
                   int by_left, int by_right, float* tex_out, void* codes, void* stream,
                   unsigned flags) {
    return sweep_impl<float>(tex_in, uv, ny, nx, kernel, klen, uv_mode, bx_left, bx_right,
                             by_left, by_right, tex_out, codes, stream, flags);
}

int rlic_sweep_f64(const double* tex_in, const void* uv, int64_t ny, int64_t nx,
                   const double* kernel, int64_t klen, int uv_mode, int bx_left, int bx_right,
                   int by_left, int by_right, double* tex_out, void* codes, void* stream,
                   unsigned flags) {
    return sweep_impl<double>(tex_in, uv, ny, nx, kernel, klen, uv_mode, bx_left, bx_right,
                              by_left, by_right, tex_out, codes, stream, flags);
}

int rlic_replay_f32(const float* tex_in, const void* codes, int64_t ny, int64_t nx,
                    const float* kernel, int64_t klen, float* tex_out, void* stream,
                    unsigned flags) {
    return replay_impl<float>(tex_in, codes, ny, nx, kernel, klen, tex_out, stream, flags);
}

int rlic_replay_f64(const double* tex_in, const void* codes, int64_t ny, int64_t nx,
                    const double* kernel, int64_t klen, double* tex_out, void* stream,
                    unsigned flags) {
    return replay_impl<double>(tex_in, codes, ny, nx, kernel, klen, tex_out, stream, flags);
}

size_t rlic_lowp_workspace_bytes(int64_t ny, int64_t nx, int64_t klen, int elem_bytes) {
    if (elem_bytes != 4 && elem_bytes != 8) return 0;
    if (ny <= 0 || nx <= 0 || klen <= 0) return 0;
    return lowp_layout(ny, nx, klen, size_t(elem_bytes)).total;
}

int rlic_convolve_lowp_f32(const float* texture, const float* u, const float* v, int64_t ny,
                           int64_t nx, const float* kernel, int64_t klen, int uv_mode,
                           int bx_left, int bx_right, int by_left, int by_right,
                           int64_t iterations, int storage, float* out, void* workspace,
                           size_t workspace_bytes, void* stream, unsigned flags) {
    return convolve_lowp_impl<float>(texture, u, v, ny, nx, kernel, klen, uv_mode, bx_left,
                                     bx_right, by_left, by_right, iterations, storage, out,
                                     workspace, workspace_bytes, stream, flags);
}

int rlic_convolve_lowp_f64(const double* texture, const double* u, const double* v, int64_t ny,
                           int64_t nx, const double* kernel, int64_t klen, int uv_mode,
                           int bx_left, int bx_right, int by_left, int by_right,
                           int64_t iterations, int storage, double* out, void* workspace,
                           size_t workspace_bytes, void* stream, unsigned flags) {
    return convolve_lowp_impl<double>(texture, u, v, ny, nx, kernel, klen, uv_mode, bx_left,
                                      bx_right, by_left, by_right, iterations, storage, out,
                                      workspace, workspace_bytes, stream, flags);
}

int rlic_adjoint_f32(const float* g, const void* codes, int64_t ny, int64_t nx,
                     const float* kernel, int64_t klen, float* y, void* stream, unsigned flags) {
    return adjoint_impl<float>(g, codes, ny, nx, kernel, klen, y, stream, flags);
}

int rlic_adjoint_f64(const double* g, const void* codes, int64_t ny, int64_t nx,
                     const double* kernel, int64_t klen, double* y, void* stream,
                     unsigned flags) {
    return adjoint_impl<double>(g, codes, ny, nx, kernel, klen, y, stream, flags);
}

int rlic_kernel_grad_f32(const float* g, const float* x, const void* codes, int64_t ny,
                         int64_t nx, int64_t klen, double* dw, void* stream, unsigned flags) {
    return kernel_grad_impl<float>(g, x, codes, ny, nx, klen, dw, stream, flags);
}

int rlic_kernel_grad_f64(const double* g, const double* x, const void* codes, int64_t ny,
                         int64_t nx, int64_t klen, double* dw, void* stream, unsigned flags) {
    return kernel_grad_impl<double>(g, x, codes, ny, nx, klen, dw, stream, flags);
}

size_t rlic_batch_workspace_bytes_f32(const rlic_batch_item_f32* items, int count) {
    if (!items || count <= 0) return 0;
    return batch_layout(items, count).total;
}

int rlic_convolve_batch_f32(const rlic_batch_item_f32* items, int count, void* workspace,
                            size_t workspace_bytes, void* stream, unsigned flags) {
    return convolve_batch_f32(items, count, workspace, workspace_bytes, stream, flags);
}

int rlic_batch_status_f32(const rlic_batch_item_f32* items, int count, const void* workspace) {
    return batch_status_f32(items, count, workspace);
}

int rlic_convolve_f32_noalloc(const float* texture, const float* u, const float* v,
                              int64_t ny, int64_t nx, const float* kernel, int64_t klen,
                              int uv_mode, int bx_left, int bx_right, int by_left, int by_right,
                              int64_t iterations, float* out, void* stream, unsigned flags) {
    return convolve_noalloc_f32(texture, u, v, ny, nx, kernel, klen, uv_mode, bx_left, bx_right,
                                by_left, by_right, iterations, out, stream, flags);
}

int rlic_set_replay_mode(int mode, int stage_rows) {
    g_last_error.clear();
    if (mode != RLIC_REPLAY_AUTO && mode != RLIC_REPLAY_L1 && mode != RLIC_REPLAY_STAGED)
        return fail(RLIC_ERR_INVALID_ARGUMENT, "mode must be RLIC_REPLAY_AUTO, _L1 or _STAGED");
    if (stage_rows != 0 && (stage_rows < 4 || stage_rows > 64 || stage_rows % 4 != 0))
        return fail(RLIC_ERR_INVALID_ARGUMENT, "stage_rows must be 0 or a multiple of 4 in [4, 64]");
    g_replay_mode.store(mode);
    rlic::set_stage_rows(stage_rows ? stage_rows : 16);
    return RLIC_OK;
}

int rlic_set_split_pixels(int64_t max_pixels) {
    g_last_error.clear();
    if (max_pixels < -1) return fail(RLIC_ERR_INVALID_ARGUMENT, "max_pixels must be >= -1");
    g_split_pixels.store(max_pixels);
    return RLIC_OK;
}

int rlic_stage_timeouts(void) {
    bool seen = false;
    if (rlic::stage_timeout_seen(&seen) != cudaSuccess) return -1;
    return seen ? 1 : 0;
}

int rlic_set_block_shape(int block_x, int block_y) {
    g_last_error.clear();
    if (block_x == 0 && block_y == 0) {  // the defaults
        g_block_x.store(64);
        g_block_y.store(4);
        g_block_custom.store(false);
        return RLIC_OK;
    }
    if (block_x <= 0 || block_y <= 0 || block_x * block_y > 256)
        return fail(RLIC_ERR_INVALID_ARGUMENT, "block shape must have 1..256 threads");
    g_block_x.store(block_x);
    g_block_y.store(block_y);
    g_block_custom.store(true);
    return RLIC_OK;
}

int rlic_check_quotients_f64(const double* a, const double* b, int64_t n, double* q,
                             int32_t* certified, void* stream) {
    g_last_error.clear();
    if (n < 0) return fail(RLIC_ERR_INVALID_ARGUMENT, "n must be >= 0");
    if (n > 0 && (!a || !b || !q || !certified))
        return fail(RLIC_ERR_INVALID_ARGUMENT, "null array pointer");
    RLIC_CUDA_TRY(rlic::launch_quotient_check(a, b, n, q, certified,
                                              static_cast<cudaStream_t>(stream)));
    return RLIC_OK;
}

int rlic_check_numerators_f64(const double* f, int64_t n, double* g, int32_t* in_range,
                              void* stream) {
    g_last_error.clear();
    if (n < 0) return fail(RLIC_ERR_INVALID_ARGUMENT, "n must be >= 0");
    if (n > 0 && (!f || !g || !in_range))
        return fail(RLIC_ERR_INVALID_ARGUMENT, "null array pointer");
    RLIC_CUDA_TRY(rlic::launch_numerator_check(f, n, g, in_range,
                                               static_cast<cudaStream_t>(stream)));
    return RLIC_OK;
}

uint64_t rlic_kernel_launch_count(void) { return rlic::launches(); }

void* rlic_host_buffer_alloc(size_t bytes) {
    g_last_error.clear();
    if (bytes == 0) bytes = 1;
    auto& c = host_cache();
    {
        std::lock_guard<std::mutex> lock(c.mu);
        auto it = c.free_blocks.find(bytes);
        if (it != c.free_blocks.end()) {
            void* p = it->second;
            c.free_blocks.erase(it);
            c.cached_bytes -= bytes;
            return p;
        }
    }
    void* p = nullptr;
    cudaError_t e = cudaHostAlloc(&p, bytes, cudaHostAllocPortable);
    if (e != cudaSuccess) {
        cuda_fail(e, "cudaHostAlloc");
        return nullptr;
    }
    std::lock_guard<std::mutex> lock(c.mu);
    c.sizes[p] = bytes;
    return p;
}

void rlic_host_buffer_free(void* p) {
    if (!p) return;
    auto& c = host_cache();
    std::lock_guard<std::mutex> lock(c.mu);
    auto it = c.sizes.find(p);
    if (it == c.sizes.end()) return;
    c.free_blocks.emplace(it->second, p);
    c.cached_bytes += it->second;
    // keep at most 4 GiB of idle pinned memory
    while (c.cached_bytes > (size_t(4) << 30) && !c.free_blocks.empty()) {
        auto victim = std::prev(c.free_blocks.end());
        c.cached_bytes -= victim->first;
        c.sizes.erase(victim->second);
        cudaFreeHost(victim->second);
        c.free_blocks.erase(victim);
    }
}

int rlic_release_cached_memory(void) {
    g_last_error.clear();
    {
        auto& c = host_cache();
        std::lock_guard<std::mutex> lock(c.mu);
        for (auto& kv : c.free_blocks) {
            c.sizes.erase(kv.second);
            cudaFreeHost(kv.second);
        }
        c.free_blocks.clear();
        c.cached_bytes = 0;
    }
    cudaError_t e = cudaSuccess;
    cudaMemPool_t pool = library_pool(&e);
    if (!pool) return cuda_fail(e, "cudaMemPoolCreate");
    RLIC_CUDA_TRY(cudaDeviceSynchronize());
    RLIC_CUDA_TRY(cudaMemPoolTrimTo(pool, 0));
    return RLIC_OK;
}

int rlic_equalize_histogram_f32(const float* image, int64_t ny, int64_t nx, int64_t nbins,
                                int strategy, int64_t tile_y, int64_t tile_x, float* out,
                                void* stream, unsigned flags) {
    return equalize_impl<float>(image, ny, nx, nbins, strategy, tile_y, tile_x, out, stream,
                                flags);
}

int rlic_equalize_histogram_f64(const double* image, int64_t ny, int64_t nx, int64_t nbins,
                                int strategy, int64_t tile_y, int64_t tile_x, double* out,
                                void* stream, unsigned flags) {
    return equalize_impl<double>(image, ny, nx, nbins, strategy, tile_y, tile_x, out, stream,
                                 flags);
}

}  // extern "C"
