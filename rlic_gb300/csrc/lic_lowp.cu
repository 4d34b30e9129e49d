// lic_lowp.cu -- the reduced-precision form of the replayed pass.
//
// The texture and the buffers between passes are stored as FP16 or BF16; each
// pass replays the recorded streamline cells (the cells come from a trace in
// the input dtype, so the discontinuous cell choices are those of the exact
// path), accumulates kernel * texture in FP32 with compensated (Kahan)
// summation, and stores the pass's output divided by sum(|kernel|).  Without
// that normalisation every pass multiplies magnitudes by about sum(kernel)
// and FP16's range (65504) is exceeded after a few passes; the scale is
// re-applied once, in the input dtype, when the last buffer is converted
// back (lic_kernels.cuh: from_storage_kernel).
#include "lic_launch.h"
#include "lic_lowp.cuh"

namespace rlic {

template <typename S, typename I>
__global__ void __launch_bounds__(256)
lic_gather_lowp_kernel(const S* __restrict__ tex_in, const uint32_t* __restrict__ codes,
                       const float* __restrict__ kernel, int klen,
                       const float* __restrict__ inv_scale, I ny, I nx, I tiles_x, I ntiles,
                       int bx, int by, int words_f, S* __restrict__ tex_out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* wsm = reinterpret_cast<float*>(smem_raw);
    const int kmid = klen / 2;
    const int nf = klen - kmid - 1;
    const int nf_pad = (nf + 7) & ~7;
    const int nb_pad = (kmid + 7) & ~7;
    I* table = reinterpret_cast<I*>(smem_raw + sizeof(float) * size_t(nf_pad + nb_pad));
    {
        const int nthreads = blockDim.x * blockDim.y;
        const int tid = threadIdx.y * blockDim.x + threadIdx.x;
        for (int s = tid; s < nf; s += nthreads) wsm[s] = kernel[kmid + 1 + s];
        for (int s = tid; s < kmid; s += nthreads) wsm[nf_pad + s] = kernel[kmid - 1 - s];
        if (tid == 0) fill_delta_table(table, nx, ny);
    }
    __syncthreads();
    const float wmid = __ldg(kernel + kmid);
    const float scale = __ldg(inv_scale);
    const int64_t npix = int64_t(ny) * int64_t(nx);
    const uint32_t* codes_b = codes + size_t(words_f) * size_t(npix);
    for (I tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const I ti = tile / tiles_x;
        const I tj = tile - ti * tiles_x;
        const I i = ti * by + I(threadIdx.y);
        const I j = tj * bx + I(threadIdx.x);
        if (i >= ny || j >= nx) continue;
        const I p = i * nx + j;
        float sum = 0.f, comp = 0.f;
        kahan_add(sum, comp, wmid, StorageTraits<S>::load(tex_in + p));
        replay_half_lowp<S, I>(sum, comp, p, codes + p, npix, nf, wsm, table, tex_in);
        replay_half_lowp<S, I>(sum, comp, p, codes_b + p, npix, kmid, wsm + nf_pad, table, tex_in);
        tex_out[p] = StorageTraits<S>::from_float(__fmul_rn(sum, scale));
    }
}

template <typename S, typename I>
cudaError_t launch_gather_lowp_t(const void* tex_in, const uint32_t* codes, const float* w32,
                                 int klen, const float* inv_scale, const Shape& sh,
                                 const LaunchConfig& lc, void* tex_out, cudaStream_t stream) {
    const int bx = lc.block_x, by = lc.block_y;
    const int64_t tiles_x = (sh.nx + bx - 1) / bx;
    const int64_t ntiles = tiles_x * ((sh.ny + by - 1) / by);
    const int kmid = klen / 2;
    const int nf = klen - kmid - 1;
    const size_t smem =
        sizeof(float) * size_t(((nf + 7) & ~7) + ((kmid + 7) & ~7)) + 16 * sizeof(I);
    auto kfn = lic_gather_lowp_kernel<S, I>;
    int dev = 0, sms = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess && smem > 48 * 1024)
        e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kfn, bx * by, smem);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    int64_t grid = int64_t(sms) * per_sm;
    if (grid > ntiles) grid = ntiles;
    kfn<<<unsigned(grid), dim3(bx, by), smem, stream>>>(
        static_cast<const S*>(tex_in), codes, w32, klen, inv_scale, I(sh.ny), I(sh.nx),
        I(tiles_x), I(ntiles), bx, by, int((nf + 7) / 8), static_cast<S*>(tex_out));
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_gather_lowp(int storage, const void* tex_in, const uint32_t* codes,
                               const float* w32, int klen, const float* inv_scale,
                               const Shape& sh, const LaunchConfig& lc, void* tex_out,
                               cudaStream_t stream) {
    const bool small = sh.small_index();
    if (storage == kStorageFP16)
        return small ? launch_gather_lowp_t<__half, int32_t>(tex_in, codes, w32, klen, inv_scale,
                                                             sh, lc, tex_out, stream)
                     : launch_gather_lowp_t<__half, int64_t>(tex_in, codes, w32, klen, inv_scale,
                                                             sh, lc, tex_out, stream);
    if (storage == kStorageBF16)
        return small ? launch_gather_lowp_t<__nv_bfloat16, int32_t>(
                           tex_in, codes, w32, klen, inv_scale, sh, lc, tex_out, stream)
                     : launch_gather_lowp_t<__nv_bfloat16, int64_t>(
                           tex_in, codes, w32, klen, inv_scale, sh, lc, tex_out, stream);
    return cudaErrorInvalidValue;
}

}  // namespace rlic
