// Ray-query kernels over caller-owned ray/hit buffers (lgb_trace_closest / lgb_trace_any).
#include <cuda_runtime.h>

#include "lgb_internal.cuh"
#include "traverse.cuh"

namespace lgb {
namespace {

constexpr int kTraceThreads = 128;

template <bool COUNT>
__global__ void __launch_bounds__(kTraceThreads) k_trace_closest(const WideNode* __restrict__ nodes,
                                                                 const WideTri* __restrict__ tris,
                                                                 const lgb_ray* __restrict__ rays, lgb_hit* __restrict__ hits,
                                                                 uint32_t n, uint32_t* status,
                                                                 unsigned long long* counters) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t nn = 0, nt = 0;
    if (i < n) {
        const float4 r0 = ldg4f(&rays[i].ox);
        const float4 r1 = ldg4f(&rays[i].dx);
        const RayQ r = make_rayq(r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w);
        float t, u, v;
        const uint32_t prim = trace_closest_dev<COUNT>(nodes, tris, r, t, u, v, status, nn, nt);
        uint4 out;
        out.x = prim;
        out.y = __float_as_uint(prim == LGB_NO_HIT ? 0.0f : t);
        out.z = __float_as_uint(u);
        out.w = __float_as_uint(v);
        reinterpret_cast<uint4*>(hits)[i] = out;
    }
    if (COUNT) {
        unsigned long long a = nn, b = nt;
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, o);
            b += __shfl_xor_sync(0xffffffffu, b, o);
        }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&counters[0], a);
            atomicAdd(&counters[1], b);
        }
    }
}

__global__ void __launch_bounds__(kTraceThreads) k_trace_any(const WideNode* __restrict__ nodes,
                                                             const WideTri* __restrict__ tris,
                                                             const lgb_ray* __restrict__ rays, uint32_t* __restrict__ bits,
                                                             uint32_t n, uint32_t* status) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    bool occ = false;
    if (i < n) {
        const float4 r0 = ldg4f(&rays[i].ox);
        const float4 r1 = ldg4f(&rays[i].dx);
        const RayQ r = make_rayq(r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w);
        occ = trace_any_dev(nodes, tris, r, status);
    }
    const uint32_t word = __ballot_sync(0xffffffffu, occ);
    if ((threadIdx.x & 31) == 0 && i < n) bits[i >> 5] = word;
}

}  // namespace

lgb_status launch_trace_closest(Scene* s, const lgb_ray* rays, lgb_hit* hits, uint32_t n, cudaStream_t st,
                                uint64_t* counters) {
    if (n == 0) return LGB_OK;
    const uint32_t grid = (n + kTraceThreads - 1) / kTraceThreads;
    if (counters)
        k_trace_closest<true><<<grid, kTraceThreads, 0, st>>>(s->bvh.nodes, s->bvh.tris, rays, hits, n, s->d_status,
                                                              reinterpret_cast<unsigned long long*>(counters));
    else
        k_trace_closest<false><<<grid, kTraceThreads, 0, st>>>(s->bvh.nodes, s->bvh.tris, rays, hits, n, s->d_status,
                                                               nullptr);
    LGB_CUDA_TRY(s->ctx, cudaGetLastError());
    return LGB_OK;
}

lgb_status launch_trace_any(Scene* s, const lgb_ray* rays, uint32_t* bits, uint32_t n, cudaStream_t st) {
    if (n == 0) return LGB_OK;
    const uint32_t grid = (n + kTraceThreads - 1) / kTraceThreads;
    k_trace_any<<<grid, kTraceThreads, 0, st>>>(s->bvh.nodes, s->bvh.tris, rays, bits, n, s->d_status);
    LGB_CUDA_TRY(s->ctx, cudaGetLastError());
    return LGB_OK;
}

}  // namespace lgb
