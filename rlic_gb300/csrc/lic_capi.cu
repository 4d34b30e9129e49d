// lic_capi.cu -- CUDA kernels and the C ABI of the rLIC convolution core.
//
// Device data layout for one call (all C-order, ny rows x nx columns):
//   uv      packed (u, v) pairs, one float2/double2 per cell, built once per
//           call by pack_uv_kernel so that every streamline step fetches both
//           velocity components with a single 8/16-byte load;
//   tex     the caller's texture, read by the first pass only;
//   out/tmp ping-pong buffers across iterations, ordered so that the last
//           pass writes `out` (the reference copies output -> input and
//           zeroes output between passes instead, src/lib.rs:433-440).
//
// The streamline sweep runs one thread per output pixel.  Each thread
// performs the centre tap, the forward trace and the backward trace of
// src/lib.rs:364-406 in that order, accumulating in a register, so the
// summation order (and hence every rounding) matches the reference.
#include "lic_device.cuh"
#include "../../include/rlic_gb300.h"

#include <atomic>
#include <cstring>
#include <string>

namespace {

thread_local std::string g_last_error;
std::atomic<uint64_t> g_launches{0};
std::atomic<int> g_block_x{32};
std::atomic<int> g_block_y{8};

constexpr size_t kAlign = 256;
inline size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

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

// ---------------------------------------------------------------- kernels --

template <typename T>
__global__ void pack_uv_kernel(const T* __restrict__ u, const T* __restrict__ v,
                               typename rlic::Vec2<T>::type* __restrict__ uv, int64_t n) {
    const int64_t stride = int64_t(gridDim.x) * blockDim.x;
    for (int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; k < n; k += stride) {
        typename rlic::Vec2<T>::type p;
        p.x = u[k];
        p.y = v[k];
        uv[k] = p;
    }
}

// One convolution pass (src/lib.rs:364-406).  CTAs tile the image in
// block_x x block_y pixel tiles, numbered row-major along a 1-D grid.
template <typename T, bool FMA, bool BRANCHLESS, bool POL, typename I>
__global__ void __launch_bounds__(256)
lic_sweep_kernel(const T* __restrict__ tex_in, const typename rlic::Vec2<T>::type* __restrict__ uv,
                 const T* __restrict__ weights_g, int klen, int weights_in_smem, I ny, I nx,
                 I tiles_x, rlic::Axis<I> ax, rlic::Axis<I> ay, T* __restrict__ tex_out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const T* w = weights_g;
    if (weights_in_smem) {
        T* ws = reinterpret_cast<T*>(smem_raw);
        const int nthreads = blockDim.x * blockDim.y;
        for (int k = threadIdx.y * blockDim.x + threadIdx.x; k < klen; k += nthreads)
            ws[k] = weights_g[k];
        __syncthreads();
        w = ws;
    }
    const I tile = I(blockIdx.x);
    const I ty = tile / tiles_x;
    const I tx = tile - ty * tiles_x;
    const I j = tx * I(blockDim.x) + I(threadIdx.x);
    const I i = ty * I(blockDim.y) + I(threadIdx.y);
    if (i >= ny || j >= nx) return;

    const int kmid = klen / 2;
    const I cell = i * nx + j;
    T acc;
    if constexpr (FMA) {
        acc = rlic::fma_rn(w[kmid], tex_in[cell], T(0));
    } else {
        acc = rlic::add_rn(T(0), rlic::mul_rn(w[kmid], tex_in[cell]));
    }
    rlic::trace_half<T, FMA, BRANCHLESS, POL, false, false>(
        acc, i, j, nx, uv, tex_in, w, kmid + 1, klen - kmid - 1, ax, ay, rlic::NoRecord{});
    rlic::trace_half<T, FMA, BRANCHLESS, POL, true, false>(
        acc, i, j, nx, uv, tex_in, w, kmid - 1, kmid, ax, ay, rlic::NoRecord{});
    tex_out[cell] = acc;
}

// Cells visited by the streamlines of selected pixels (path parity checks).
template <typename T, bool FMA, bool BRANCHLESS, bool POL>
__global__ void trace_cells_kernel(const typename rlic::Vec2<T>::type* __restrict__ uv,
                                   int64_t ny, int64_t nx, int klen, rlic::Axis<int64_t> ax,
                                   rlic::Axis<int64_t> ay, int64_t npix,
                                   const int64_t* __restrict__ pix, int64_t* __restrict__ cells) {
    const int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    const int steps = klen - 1;
    const int kmid = klen / 2;
    const int nf = klen - kmid - 1;
    int64_t* dst = cells + p * steps;
    for (int s = 0; s < steps; ++s) dst[s] = -1;
    const int64_t lin = pix[p];
    if (lin < 0 || lin >= ny * nx) return;  // invalid pixel: row stays -1
    const int64_t i = lin / nx;
    const int64_t j = lin - i * nx;
    T acc = T(0);
    auto rec_f = [dst](int s, int64_t c) { dst[s] = c; };
    auto rec_b = [dst, nf](int s, int64_t c) { dst[nf + s] = c; };
    rlic::trace_half<T, FMA, BRANCHLESS, POL, false, true>(
        acc, i, j, nx, uv, static_cast<const T*>(nullptr), static_cast<const T*>(nullptr),
        kmid + 1, nf, ax, ay, rec_f);
    rlic::trace_half<T, FMA, BRANCHLESS, POL, true, true>(
        acc, i, j, nx, uv, static_cast<const T*>(nullptr), static_cast<const T*>(nullptr),
        kmid - 1, kmid, ax, ay, rec_b);
}

// --------------------------------------------------------------- launchers --

struct Variant {
    bool fma;
    bool branchless;
    bool pol;
};

Variant make_variant(unsigned flags, int uv_mode) {
    return Variant{!(flags & RLIC_FLAG_NO_FMA), !(flags & RLIC_FLAG_NO_BRANCHLESS),
                   uv_mode == RLIC_UV_POLARIZATION};
}

template <typename T>
int launch_pack(const T* u, const T* v, typename rlic::Vec2<T>::type* uv, int64_t n,
                cudaStream_t stream) {
    int64_t blocks = (n + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (blocks < 1) blocks = 1;
    pack_uv_kernel<T><<<unsigned(blocks), 256, 0, stream>>>(u, v, uv, n);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    RLIC_CUDA_TRY(cudaGetLastError());
    return RLIC_OK;
}

template <typename T, bool FMA, bool BRANCHLESS, bool POL, typename I>
int launch_sweep_t(const T* tex_in, const typename rlic::Vec2<T>::type* uv, const T* weights,
                   int klen, int64_t ny, int64_t nx, const int bnd[4], T* tex_out,
                   cudaStream_t stream) {
    const int bx = g_block_x.load(), by = g_block_y.load();
    const int64_t tiles_x = (nx + bx - 1) / bx;
    const int64_t tiles_y = (ny + by - 1) / by;
    const int64_t tiles = tiles_x * tiles_y;
    if (tiles > 0x7fffffffLL) return fail(RLIC_ERR_INVALID_ARGUMENT, "image too large for grid");
    const size_t wbytes = size_t(klen) * sizeof(T);
    const bool in_smem = wbytes <= 48 * 1024;
    const auto ax = rlic::make_axis<I>(I(nx), bnd[0], bnd[1]);
    const auto ay = rlic::make_axis<I>(I(ny), bnd[2], bnd[3]);
    lic_sweep_kernel<T, FMA, BRANCHLESS, POL, I>
        <<<unsigned(tiles), dim3(bx, by), in_smem ? wbytes : 0, stream>>>(
            tex_in, uv, weights, klen, in_smem ? 1 : 0, I(ny), I(nx), I(tiles_x), ax, ay,
            tex_out);
    g_launches.fetch_add(1, std::memory_order_relaxed);
    RLIC_CUDA_TRY(cudaGetLastError());
    return RLIC_OK;
}

template <typename T, typename I>
int launch_sweep(const Variant& var, const T* tex_in, const typename rlic::Vec2<T>::type* uv,
                 const T* weights, int klen, int64_t ny, int64_t nx, const int bnd[4],
                 T* tex_out, cudaStream_t stream) {
    const int code = (var.fma ? 4 : 0) | (var.branchless ? 2 : 0) | (var.pol ? 1 : 0);
#define RLIC_SWEEP_CASE(C, F, B, P) \
    case C:                         \
        return launch_sweep_t<T, F, B, P, I>(tex_in, uv, weights, klen, ny, nx, bnd, tex_out, stream);
    switch (code) {
        RLIC_SWEEP_CASE(0, false, false, false)
        RLIC_SWEEP_CASE(1, false, false, true)
        RLIC_SWEEP_CASE(2, false, true, false)
        RLIC_SWEEP_CASE(3, false, true, true)
        RLIC_SWEEP_CASE(4, true, false, false)
        RLIC_SWEEP_CASE(5, true, false, true)
        RLIC_SWEEP_CASE(6, true, true, false)
        RLIC_SWEEP_CASE(7, true, true, true)
    }
#undef RLIC_SWEEP_CASE
    return fail(RLIC_ERR_INVALID_ARGUMENT, "bad variant");
}

template <typename T>
int launch_trace_cells(const Variant& var, const typename rlic::Vec2<T>::type* uv, int64_t ny,
                       int64_t nx, int klen, const int bnd[4], int64_t npix, const int64_t* pix,
                       int64_t* cells, cudaStream_t stream) {
    const auto ax = rlic::make_axis<int64_t>(nx, bnd[0], bnd[1]);
    const auto ay = rlic::make_axis<int64_t>(ny, bnd[2], bnd[3]);
    const unsigned blocks = unsigned((npix + 127) / 128);
    const int code = (var.fma ? 4 : 0) | (var.branchless ? 2 : 0) | (var.pol ? 1 : 0);
#define RLIC_TRACE_CASE(C, F, B, P)                                                         \
    case C:                                                                                 \
        trace_cells_kernel<T, F, B, P><<<blocks, 128, 0, stream>>>(uv, ny, nx, klen, ax, ay, \
                                                                    npix, pix, cells);      \
        break;
    switch (code) {
        RLIC_TRACE_CASE(0, false, false, false)
        RLIC_TRACE_CASE(1, false, false, true)
        RLIC_TRACE_CASE(2, false, true, false)
        RLIC_TRACE_CASE(3, false, true, true)
        RLIC_TRACE_CASE(4, true, false, false)
        RLIC_TRACE_CASE(5, true, false, true)
        RLIC_TRACE_CASE(6, true, true, false)
        RLIC_TRACE_CASE(7, true, true, true)
    }
#undef RLIC_TRACE_CASE
    g_launches.fetch_add(1, std::memory_order_relaxed);
    RLIC_CUDA_TRY(cudaGetLastError());
    return RLIC_OK;
}

// ------------------------------------------------------------- host logic --

int check_common(int64_t ny, int64_t nx, int64_t klen, int uv_mode, const int bnd[4],
                 unsigned flags) {
    if (ny <= 0 || nx <= 0)
        return fail(RLIC_ERR_INVALID_ARGUMENT, "image dimensions must be positive");
    if (ny > (int64_t(1) << 40) / nx)
        return fail(RLIC_ERR_INVALID_ARGUMENT, "image too large");
    if (klen <= 0) return fail(RLIC_ERR_INVALID_ARGUMENT, "kernel must have at least one tap");
    if (klen > (int64_t(1) << 30)) return fail(RLIC_ERR_INVALID_ARGUMENT, "kernel too long");
    if (uv_mode != RLIC_UV_VELOCITY && uv_mode != RLIC_UV_POLARIZATION)
        return fail(RLIC_ERR_INVALID_ARGUMENT, "uv_mode must be 0 (velocity) or 1 (polarization)");
    for (int k = 0; k < 4; ++k)
        if (bnd[k] != RLIC_BOUNDARY_CLOSED && bnd[k] != RLIC_BOUNDARY_PERIODIC)
            return fail(RLIC_ERR_INVALID_ARGUMENT,
                        "boundaries must be 0 (closed) or 1 (periodic)");
    if (flags & ~(RLIC_FLAG_HOST_MEMORY | RLIC_FLAG_NO_FMA | RLIC_FLAG_NO_BRANCHLESS))
        return fail(RLIC_ERR_INVALID_ARGUMENT, "unknown flag bits");
    return RLIC_OK;
}

size_t workspace_bytes(int64_t ny, int64_t nx, int64_t klen, int64_t iterations, size_t s) {
    if (ny <= 0 || nx <= 0 || klen <= 0 || iterations < 0) return 0;
    const size_t n = size_t(ny) * size_t(nx);
    size_t b = align_up(2 * n * s);             // packed (u, v)
    if (iterations >= 2) b += align_up(n * s);  // ping-pong texture
    b += align_up(size_t(klen) * s);            // kernel weights (host-memory calls)
    return b;
}

// Runs `iterations` passes on device memory.  `ws` holds the workspace.
template <typename T>
int run_device(const T* texture, const T* u, const T* v, int64_t ny, int64_t nx,
               const T* kernel, int64_t klen, const Variant& var, const int bnd[4],
               int64_t iterations, T* out, unsigned char* ws, cudaStream_t stream) {
    using V2 = typename rlic::Vec2<T>::type;
    const int64_t n = ny * nx;
    if (iterations == 0) {
        RLIC_CUDA_TRY(cudaMemsetAsync(out, 0, size_t(n) * sizeof(T), stream));
        return RLIC_OK;
    }
    V2* uv = reinterpret_cast<V2*>(ws);
    T* tmp = reinterpret_cast<T*>(ws + align_up(2 * size_t(n) * sizeof(T)));
    int rc = launch_pack<T>(u, v, uv, n, stream);
    if (rc) return rc;
    const bool small = n < (int64_t(1) << 31) - 1;
    const T* src = texture;
    for (int64_t it = 0; it < iterations; ++it) {
        T* dst = ((iterations - 1 - it) % 2 == 0) ? out : tmp;
        rc = small ? launch_sweep<T, int32_t>(var, src, uv, kernel, int(klen), ny, nx, bnd, dst,
                                              stream)
                   : launch_sweep<T, int64_t>(var, src, uv, kernel, int(klen), ny, nx, bnd, dst,
                                              stream);
        if (rc) return rc;
        src = dst;
    }
    return RLIC_OK;
}

template <typename T>
int convolve_impl(const T* texture, const T* u, const T* v, int64_t ny, int64_t nx,
                  const T* kernel, int64_t klen, int uv_mode, int bxl, int bxr, int byl,
                  int byr, int64_t iterations, T* out, void* workspace, size_t workspace_bytes_,
                  void* stream_, unsigned flags) {
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
    const size_t need = workspace_bytes(ny, nx, klen, iterations, sizeof(T));

    if (!(flags & RLIC_FLAG_HOST_MEMORY)) {
        unsigned char* ws = static_cast<unsigned char*>(workspace);
        bool owned = false;
        if (ws == nullptr) {
            RLIC_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&ws), need, stream));
            owned = true;
        } else {
            if (workspace_bytes_ < need)
                return fail(RLIC_ERR_WORKSPACE_TOO_SMALL,
                            "workspace smaller than rlic_workspace_bytes()");
            if (reinterpret_cast<uintptr_t>(ws) % kAlign != 0)
                return fail(RLIC_ERR_INVALID_ARGUMENT, "workspace must be 256-byte aligned");
        }
        rc = run_device<T>(texture, u, v, ny, nx, kernel, klen, var, bnd, iterations, out, ws,
                           stream);
        if (owned) {
            cudaError_t e = cudaFreeAsync(ws, stream);
            if (rc == RLIC_OK && e != cudaSuccess) return cuda_fail(e, "cudaFreeAsync");
        }
        return rc;
    }

    // Host memory: one stream-ordered device block holds the inputs, the
    // output and the workspace; the call returns once `out` holds the result.
    const size_t a_img = align_up(n * sizeof(T));
    const size_t total = 4 * a_img + need;
    unsigned char* d = nullptr;
    RLIC_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&d), total, stream));
    T* d_tex = reinterpret_cast<T*>(d);
    T* d_u = reinterpret_cast<T*>(d + a_img);
    T* d_v = reinterpret_cast<T*>(d + 2 * a_img);
    T* d_out = reinterpret_cast<T*>(d + 3 * a_img);
    unsigned char* ws = d + 4 * a_img;
    T* d_kernel = reinterpret_cast<T*>(ws + need - align_up(size_t(klen) * sizeof(T)));
    auto body = [&]() -> int {
        RLIC_CUDA_TRY(cudaMemcpyAsync(d_tex, texture, n * sizeof(T), cudaMemcpyHostToDevice, stream));
        RLIC_CUDA_TRY(cudaMemcpyAsync(d_u, u, n * sizeof(T), cudaMemcpyHostToDevice, stream));
        RLIC_CUDA_TRY(cudaMemcpyAsync(d_v, v, n * sizeof(T), cudaMemcpyHostToDevice, stream));
        RLIC_CUDA_TRY(cudaMemcpyAsync(d_kernel, kernel, size_t(klen) * sizeof(T),
                                      cudaMemcpyHostToDevice, stream));
        int r = run_device<T>(d_tex, d_u, d_v, ny, nx, d_kernel, klen, var, bnd, iterations,
                              d_out, ws, stream);
        if (r) return r;
        RLIC_CUDA_TRY(cudaMemcpyAsync(out, d_out, n * sizeof(T), cudaMemcpyDeviceToHost, stream));
        return RLIC_OK;
    };
    rc = body();
    cudaError_t ef = cudaFreeAsync(d, stream);
    cudaError_t es = cudaStreamSynchronize(stream);
    if (rc) return rc;
    if (ef != cudaSuccess) return cuda_fail(ef, "cudaFreeAsync");
    if (es != cudaSuccess) return cuda_fail(es, "cudaStreamSynchronize");
    return RLIC_OK;
}

template <typename T>
int trace_cells_impl(const T* u, const T* v, int64_t ny, int64_t nx, int64_t klen, int uv_mode,
                     int bxl, int bxr, int byl, int byr, int64_t npix, const int64_t* pix,
                     int64_t* cells, void* stream_, unsigned flags) {
    using V2 = typename rlic::Vec2<T>::type;
    g_last_error.clear();
    const int bnd[4] = {bxl, bxr, byl, byr};
    int rc = check_common(ny, nx, klen, uv_mode, bnd, flags);
    if (rc) return rc;
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
    RLIC_CUDA_TRY(cudaMallocAsync(reinterpret_cast<void**>(&d), total, stream));
    V2* uv = reinterpret_cast<V2*>(d);
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
        int r = launch_pack<T>(du, dv, uv, int64_t(n), stream);
        if (r) return r;
        r = launch_trace_cells<T>(var, uv, ny, nx, int(klen), bnd, npix, dpix, dcells, stream);
        if (r) return r;
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
    if (ny <= 0 || nx <= 0) return fail(RLIC_ERR_INVALID_ARGUMENT, "image dimensions must be positive");
    if (!u || !v || !uv) return fail(RLIC_ERR_INVALID_ARGUMENT, "null array pointer");
    if (reinterpret_cast<uintptr_t>(uv) % (2 * sizeof(T)) != 0)
        return fail(RLIC_ERR_INVALID_ARGUMENT, "packed field must be aligned to 2 elements");
    return launch_pack<T>(u, v, static_cast<typename rlic::Vec2<T>::type*>(uv), ny * nx,
                          static_cast<cudaStream_t>(stream_));
}

template <typename T>
int sweep_impl(const T* tex_in, const void* uv, int64_t ny, int64_t nx, const T* kernel,
               int64_t klen, int uv_mode, int bxl, int bxr, int byl, int byr, T* tex_out,
               void* stream_, unsigned flags) {
    g_last_error.clear();
    const int bnd[4] = {bxl, bxr, byl, byr};
    int rc = check_common(ny, nx, klen, uv_mode, bnd, flags);
    if (rc) return rc;
    if (flags & RLIC_FLAG_HOST_MEMORY)
        return fail(RLIC_ERR_INVALID_ARGUMENT, "this entry point takes device pointers only");
    if (!tex_in || !uv || !kernel || !tex_out)
        return fail(RLIC_ERR_INVALID_ARGUMENT, "null array pointer");
    const Variant var = make_variant(flags, uv_mode);
    const auto* p = static_cast<const typename rlic::Vec2<T>::type*>(uv);
    cudaStream_t stream = static_cast<cudaStream_t>(stream_);
    const bool small = ny * nx < (int64_t(1) << 31) - 1;
    return small ? launch_sweep<T, int32_t>(var, tex_in, p, kernel, int(klen), ny, nx, bnd,
                                            tex_out, stream)
                 : launch_sweep<T, int64_t>(var, tex_in, p, kernel, int(klen), ny, nx, bnd,
                                            tex_out, stream);
}

}  // namespace

// -------------------------------------------------------------------- C ABI --

extern "C" {

const char* rlic_version(void) { return "rlic_gb300 0.1.0 (sm_103a)"; }

const char* rlic_last_error(void) { return g_last_error.c_str(); }

size_t rlic_workspace_bytes(int64_t ny, int64_t nx, int64_t klen, int64_t iterations,
                            int elem_bytes) {
    if (elem_bytes != 4 && elem_bytes != 8) return 0;
    return workspace_bytes(ny, nx, klen, iterations, size_t(elem_bytes));
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
                   int by_left, int by_right, float* tex_out, void* stream, unsigned flags) {
    return sweep_impl<float>(tex_in, uv, ny, nx, kernel, klen, uv_mode, bx_left, bx_right,
                             by_left, by_right, tex_out, stream, flags);
}

int rlic_sweep_f64(const double* tex_in, const void* uv, int64_t ny, int64_t nx,
                   const double* kernel, int64_t klen, int uv_mode, int bx_left, int bx_right,
                   int by_left, int by_right, double* tex_out, void* stream, unsigned flags) {
    return sweep_impl<double>(tex_in, uv, ny, nx, kernel, klen, uv_mode, bx_left, bx_right,
                              by_left, by_right, tex_out, stream, flags);
}

int rlic_set_block_shape(int block_x, int block_y) {
    if (block_x <= 0 || block_y <= 0 || block_x * block_y > 256)
        return fail(RLIC_ERR_INVALID_ARGUMENT, "block shape must have 1..256 threads");
    g_block_x.store(block_x);
    g_block_y.store(block_y);
    return RLIC_OK;
}

uint64_t rlic_kernel_launch_count(void) { return g_launches.load(); }

}  // extern "C"
