// Measurement helpers for roofline accounting (not part of the ray-tracing path).
#include <cuda_runtime.h>

#include "lgb_internal.cuh"

namespace lgb {
namespace {

// Every thread streams 16-byte loads over the buffer `reps` times, starting at a block-dependent offset so
// that blocks spread over all L2 slices; the XOR of everything read is written once per thread so the
// loads cannot be dropped.
__global__ void __launch_bounds__(512) k_l2_read(const uint4* __restrict__ buf, size_t n16, int reps, uint32_t* sink) {
    const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    uint32_t acc = 0;
    for (int r = 0; r < reps; r++) {
        for (size_t i = tid; i < n16; i += stride) {
            const uint4 v = __ldcg(&buf[i]);
            acc ^= v.x ^ v.y ^ v.z ^ v.w;
        }
    }
    if (acc == 0x9e3779b9u) sink[tid & 1023] = acc;
}

__global__ void k_fill(uint4* buf, size_t n16) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += (size_t)gridDim.x * blockDim.x)
        buf[i] = make_uint4((uint32_t)i, (uint32_t)(i >> 7), 1u, 2u);
}

}  // namespace
}  // namespace lgb

extern "C" LGB_API lgb_status lgb_measure_l2_read_gbs(int device, uint64_t bytes, uint32_t reps, double* out_gbs) {
    using namespace lgb;
    if (!out_gbs || bytes < 1024 || reps == 0) return LGB_ERR_INVALID_ARGUMENT;
    if (cudaSetDevice(device) != cudaSuccess) return LGB_ERR_CUDA;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const size_t n16 = bytes / 16;
    uint4* buf = nullptr;
    uint32_t* sink = nullptr;
    if (cudaMalloc(&buf, n16 * 16) != cudaSuccess) return LGB_ERR_OUT_OF_MEMORY;
    if (cudaMalloc(&sink, 4096) != cudaSuccess) { cudaFree(buf); return LGB_ERR_OUT_OF_MEMORY; }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_fill<<<sms * 4, 512>>>(buf, n16);
    const int grid = sms * 4;
    k_l2_read<<<grid, 512>>>(buf, n16, 2, sink);  // warm L2
    double best = 0.0;
    for (int trial = 0; trial < 5; trial++) {
        cudaEventRecord(e0);
        k_l2_read<<<grid, 512>>>(buf, n16, (int)reps, sink);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        const double gbs = (double)n16 * 16.0 * reps / (ms * 1e-3) / 1e9;
        if (gbs > best) best = gbs;
    }
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    cudaFree(sink);
    if (err != cudaSuccess) return LGB_ERR_CUDA;
    *out_gbs = best;
    return LGB_OK;
}
