// Ray-query kernels over caller-owned ray/hit buffers (lgb_trace_closest / lgb_trace_any).
#include <cuda_runtime.h>

#include <algorithm>

#include "lgb_internal.cuh"
#include "traverse.cuh"

namespace lgb {
namespace {

constexpr int kTraceThreads = 128;
// Register budget for 9 resident blocks per SM (56 registers, a few bytes of spill). Measured on GB300 with
// the 1M-triangle, 4M incoherent-ray workload: 862 Mrays/s unbounded (79 registers, 6 blocks), 1085 at
// 8 blocks (64), 1133 at 9 (56), 1087 at 10 (48); 256-thread blocks were slower.
constexpr int kTraceMinBlocks = 9;

// Bottom entries of each thread's traversal stack kept in shared memory (8 KB per block). Measured on GB300,
// 4M incoherent rays / 1M triangles, closest / any Mrays/s: 0 entries 1133 / 2280, 4: 1137 / 2318,
// 8: 1142 / 2335, 12: 1142 / 2323.
constexpr int kTraceSharedStack = 8;
// Idle lanes a warp waits for before fetching new rays. Measured with the approximate box-test reciprocal,
// closest / any Mrays/s: refill at 1 idle lane 1176 / 2350, at 8: 1185 / 2680, at 16: 1047 / 2485.
constexpr int kTraceRefill = 8;
template <bool ANY, bool COUNT>
__global__ void __launch_bounds__(kTraceThreads, kTraceMinBlocks) k_trace(const WideNode* __restrict__ nodes, const WideTri* __restrict__ tris,
                                                         const lgb_ray* __restrict__ rays, lgb_hit* __restrict__ hits,
                                                         uint32_t* __restrict__ bits, uint32_t n, uint32_t* ray_counter,
                                                         uint32_t* status, unsigned long long* counters) {
    __shared__ uint2 s_stack[kTraceSharedStack * kTraceThreads];
    trace_persistent<ANY, COUNT, true, kTraceSharedStack, kTraceThreads, kTraceRefill>(
        nodes, tris, rays, hits, bits, n, nullptr, ray_counter, status, counters, nullptr, s_stack);
}

template <bool ANY, bool COUNT> int persistent_grid(Ctx* ctx, uint32_t n) {
    static int blocks_per_sm = 0;
    if (blocks_per_sm == 0) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, k_trace<ANY, COUNT>, kTraceThreads, 0);
        if (blocks_per_sm <= 0) blocks_per_sm = 1;
    }
    const int sms = ctx->sm_count > 0 ? ctx->sm_count : 1;
    const uint32_t need = (n + kTraceThreads - 1) / kTraceThreads;
    return (int)std::min<uint32_t>(need, (uint32_t)(sms * blocks_per_sm));
}

}  // namespace

lgb_status launch_trace_closest(Scene* s, const lgb_ray* rays, lgb_hit* hits, uint32_t n, cudaStream_t st,
                                uint64_t* counters) {
    if (n == 0) return LGB_OK;
    LGB_CUDA_TRY(s->ctx, cudaMemsetAsync(s->d_ray_counter, 0, sizeof(uint32_t), st));
    if (counters)
        k_trace<false, true><<<persistent_grid<false, true>(s->ctx, n), kTraceThreads, 0, st>>>(
            s->bvh.nodes, s->bvh.tris, rays, hits, nullptr, n, s->d_ray_counter, s->d_status,
            reinterpret_cast<unsigned long long*>(counters));
    else
        k_trace<false, false><<<persistent_grid<false, false>(s->ctx, n), kTraceThreads, 0, st>>>(
            s->bvh.nodes, s->bvh.tris, rays, hits, nullptr, n, s->d_ray_counter, s->d_status, nullptr);
    LGB_CUDA_TRY(s->ctx, cudaGetLastError());
    return LGB_OK;
}

lgb_status launch_trace_any(Scene* s, const lgb_ray* rays, uint32_t* bits, uint32_t n, cudaStream_t st) {
    if (n == 0) return LGB_OK;
    LGB_CUDA_TRY(s->ctx, cudaMemsetAsync(s->d_ray_counter, 0, sizeof(uint32_t), st));
    LGB_CUDA_TRY(s->ctx, cudaMemsetAsync(bits, 0, sizeof(uint32_t) * ((n + 31) / 32), st));
    k_trace<true, false><<<persistent_grid<true, false>(s->ctx, n), kTraceThreads, 0, st>>>(
        s->bvh.nodes, s->bvh.tris, rays, nullptr, bits, n, s->d_ray_counter, s->d_status, nullptr);
    LGB_CUDA_TRY(s->ctx, cudaGetLastError());
    return LGB_OK;
}

}  // namespace lgb
