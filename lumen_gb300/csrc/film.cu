// Film measurement: RMSE of an RGBA32F film against a reference film.
//
// Lumen computes its on-screen error in three compute passes (src/shaders/rmse/calc_rmse.comp:20-42,
// reduce_rmse.comp:22-49, output_rmse.comp:22-25). Two details of those passes make the reported number
// something other than an RMSE: the per-workgroup combine uses subgroupMin instead of subgroupAdd
// (calc_rmse.comp:37), and the final value is sqrt(sum) / (3 N) instead of sqrt(sum / (3 N)).
// lgb_film_rmse offers both: mode 0 is the true RMSE over the RGB channels, mode 1 reproduces Lumen's
// reported value (per 1024-pixel group, the minimum over its 32-pixel warps of their squared-error sums;
// groups summed; sqrt(sum) / (3 N)). Both reductions are two-pass and deterministic: per-block partial sums
// in double precision, then one block adds the partials in a fixed order.
#include <cuda_runtime.h>

#include <vector>

#include "lgb_internal.cuh"

namespace lgb {
namespace {

constexpr int kRmseThreads = 1024;

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// One block per 1024 pixels. mode 0: partial = sum of squared errors of the block.
// mode 1: partial = min over the block's warps (those holding at least one pixel) of the warp's FP32 sum.
__global__ void __launch_bounds__(kRmseThreads) k_rmse_partial(const float4* __restrict__ a, const float4* __restrict__ b,
                                                               uint32_t npix, int mode, double* partial) {
    __shared__ double wsum[32];
    __shared__ int wvalid[32];
    const uint32_t idx = blockIdx.x * kRmseThreads + threadIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    float val = 0.0f;
    if (idx < npix) {
        const float4 x = a[idx], y = b[idx];
        const float dx = y.x - x.x, dy = y.y - x.y, dz = y.z - x.z;
        val = dx * dx + dy * dy + dz * dz;
    }
    double s;
    if (mode == 1) {
        float f = val;
        for (int o = 16; o > 0; o >>= 1) f += __shfl_xor_sync(0xffffffffu, f, o);
        s = (double)f;
    } else {
        s = warp_sum((double)val);
    }
    if (lane == 0) {
        wsum[warp] = s;
        wvalid[warp] = (blockIdx.x * kRmseThreads + warp * 32u) < npix;
    }
    __syncthreads();
    if (warp == 0) {
        double v = wsum[lane];
        const int ok = wvalid[lane];
        if (mode == 1) {
            double m = ok ? v : 1e300;
            for (int o = 16; o > 0; o >>= 1) m = fmin(m, __shfl_xor_sync(0xffffffffu, m, o));
            if (lane == 0) partial[blockIdx.x] = m;
        } else {
            v = warp_sum(ok ? v : 0.0);
            if (lane == 0) partial[blockIdx.x] = v;
        }
    }
}

__global__ void __launch_bounds__(kRmseThreads) k_rmse_final(const double* __restrict__ partial, uint32_t n,
                                                             double* out) {
    __shared__ double wsum[32];
    double v = 0.0;
    for (uint32_t i = threadIdx.x; i < n; i += kRmseThreads) v += partial[i];
    v = warp_sum(v);
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = warp_sum(wsum[threadIdx.x]);
        if (threadIdx.x == 0) *out = v;
    }
}

}  // namespace
}  // namespace lgb

extern "C" LGB_API lgb_status lgb_film_rmse(lgb_ctx* ctx, const float* d_film, const float* d_reference, uint32_t npix,
                                            uint32_t mode, double* out_rmse, void* stream) {
    using namespace lgb;
    if (!ctx) return LGB_ERR_INVALID_ARGUMENT;
    if (!d_film || !d_reference || !out_rmse || npix == 0 || mode > 1)
        return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "lgb_film_rmse: null pointer, empty film or unknown mode");
    if ((reinterpret_cast<uintptr_t>(d_film) | reinterpret_cast<uintptr_t>(d_reference)) & 15u)
        return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "films must be 16-byte aligned");
    cudaSetDevice(ctx->device);
    const cudaStream_t st = (cudaStream_t)stream;
    const uint32_t blocks = (npix + kRmseThreads - 1) / kRmseThreads;
    double* buf = nullptr;
    LGB_CUDA_TRY(ctx, cudaMallocAsync((void**)&buf, sizeof(double) * (blocks + 1), st));
    k_rmse_partial<<<blocks, kRmseThreads, 0, st>>>(reinterpret_cast<const float4*>(d_film),
                                                    reinterpret_cast<const float4*>(d_reference), npix, (int)mode, buf + 1);
    k_rmse_final<<<1, kRmseThreads, 0, st>>>(buf + 1, blocks, buf);
    double sum = 0.0;
    cudaError_t e = cudaMemcpyAsync(&sum, buf, sizeof(double), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFreeAsync(buf, st);
    if (e != cudaSuccess) return cuda_error(ctx, e, "lgb_film_rmse");
    *out_rmse = mode == 0 ? sqrt(sum / (3.0 * (double)npix)) : sqrt(sum) / (3.0 * (double)npix);
    return LGB_OK;
}
