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
#ifdef LGB_TRACE_SK
constexpr int kTraceSharedStack = LGB_TRACE_SK;
#else
constexpr int kTraceSharedStack = 8;
#endif
// Idle lanes a warp waits for before fetching new rays. Measured with the approximate box-test reciprocal and
// mixed iterations, closest / any Mrays/s: refill at 1 idle lane 1176 / 2350, at 8: 1185 / 2680, at 16: 1047 /
// 2485. With warp-uniform triangle iterations (below) and one triangle per leaf slot: at 8: 1317 / 3048, at 4:
// 1370 / 3013, at 3: 1368 / 2939, at 2: 1356 / 2765.
constexpr int kTraceRefill = 4;
// Warp-uniform triangle and node iterations (TRI_MIN of trace_persistent): a triangle iteration once a fifth
// of the active lanes have a pending leaf triangle. Measured on GB300, 4M incoherent rays / 1M triangles,
// closest / any Mrays/s (hits bit-identical), refill at 8 and three triangles per leaf slot: mixed iterations
// 1182 / 2664; fixed thresholds 2: 1170 / 2463, 4: 1244 / 2724, 6: 1247 / 2814, 8: 1219 / 2814, 12: 1110 / 2699,
// 20: 803 / 2186; a third of the active lanes 1208 / 2853; a quarter 1252 / 2866; a fifth 1267 / 2853. With the
// refill at 4 and one triangle per leaf slot: a quarter 1370 / 3013, a fifth 1386 / 2995.
constexpr int kTraceTriMin = -5;
#ifdef LGB_TRACE_TRI_MIN
#define LGB_TRACE_TRI_MIN_ LGB_TRACE_TRI_MIN
#else
#define LGB_TRACE_TRI_MIN_ kTraceTriMin
#endif
#ifdef LGB_TRACE_MIN_BLOCKS
#define LGB_TRACE_MIN_BLOCKS_ LGB_TRACE_MIN_BLOCKS
#else
#define LGB_TRACE_MIN_BLOCKS_ kTraceMinBlocks
#endif
#ifdef LGB_TRACE_REFILL
#define LGB_TRACE_REFILL_ LGB_TRACE_REFILL
#else
#define LGB_TRACE_REFILL_ kTraceRefill
#endif
template <bool ANY, bool COUNT>
__global__ void __launch_bounds__(kTraceThreads, LGB_TRACE_MIN_BLOCKS_) k_trace(const WideNode* __restrict__ nodes, const WideTri* __restrict__ tris,
                                                         const lgb_ray* __restrict__ rays, lgb_hit* __restrict__ hits,
                                                         uint32_t* __restrict__ bits, uint32_t n, uint32_t* ray_counter,
                                                         uint32_t* status, unsigned long long* counters,
                                                         uint32_t max_visits) {
    __shared__ uint2 s_stack[kTraceSharedStack * kTraceThreads];
    trace_persistent<ANY, COUNT, true, kTraceSharedStack, kTraceThreads, LGB_TRACE_REFILL_, LGB_TRACE_TRI_MIN_>(
        nodes, tris, rays, hits, bits, n, nullptr, ray_counter, status, counters, nullptr, s_stack, max_visits);
}

uint32_t visit_budget(const Scene* s) { return s->visit_limit ? s->visit_limit : kMaxVisits; }

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
            reinterpret_cast<unsigned long long*>(counters), visit_budget(s));
    else
        k_trace<false, false><<<persistent_grid<false, false>(s->ctx, n), kTraceThreads, 0, st>>>(
            s->bvh.nodes, s->bvh.tris, rays, hits, nullptr, n, s->d_ray_counter, s->d_status, nullptr, visit_budget(s));
    LGB_CUDA_TRY(s->ctx, cudaGetLastError());
    return LGB_OK;
}

namespace {
constexpr uint32_t kHostChunks = 8;           // chunks of one host-buffer query
constexpr uint32_t kHostChunkMin = 1u << 18;  // rays in a chunk, at least
}  // namespace

// Device address of a pinned (page-locked, mapped) host buffer, or null for pageable memory.
static const void* mapped_host(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// Pinned host buffers: the persistent kernel loads each ray (32 B, once) from host memory and, for closest hits,
// stores each hit (16 B) there, over the CPU-GPU link; the link latency is hidden among the rays in flight and
// nothing else crosses it. Any-hit sets its bits with atomics, so they are gathered in device memory and copied
// out once (n / 8 bytes). Pageable buffers: the rays are cut into up to kHostChunks chunks (multiples of 32 rays,
// so any-hit bit words never straddle two chunks); chunk c is copied in on the library's upload stream, traced on
// the caller's stream once it has arrived, and its results are copied out on the download stream once traced.
// Either way the caller's stream ends after the results are in host memory, so the call is stream-ordered like
// the device-buffer queries.
lgb_status trace_host(Scene* s, const lgb_ray* h_rays, void* h_out, uint32_t n, bool any, cudaStream_t st) {
    Ctx* ctx = s->ctx;
    const lgb_ray* m_rays = reinterpret_cast<const lgb_ray*>(mapped_host(h_rays));
    void* m_out = any ? nullptr : const_cast<void*>(mapped_host(h_out));
    if (m_rays && (any || m_out) && !(reinterpret_cast<uintptr_t>(m_rays) & 15u) &&
        !(reinterpret_cast<uintptr_t>(m_out) & 15u)) {
        if (!any) return launch_trace_closest(s, m_rays, reinterpret_cast<lgb_hit*>(m_out), n, st, nullptr);
        const size_t words = (n + 31) / 32;
        if (s->stage_bytes < sizeof(uint32_t) * words) {
            cudaFree(s->stage_buf);  // waits for any query still using it
            s->stage_buf = nullptr;
            s->stage_bytes = 0;
            LGB_CUDA_TRY(ctx, cudaMalloc(&s->stage_buf, sizeof(uint32_t) * words));
            s->stage_bytes = sizeof(uint32_t) * words;
        }
        uint32_t* bits = reinterpret_cast<uint32_t*>(s->stage_buf);
        const lgb_status ls = launch_trace_any(s, m_rays, bits, n, st);
        if (ls != LGB_OK) return ls;
        LGB_CUDA_TRY(ctx, cudaMemcpyAsync(h_out, bits, sizeof(uint32_t) * words, cudaMemcpyDeviceToHost, st));
        return LGB_OK;
    }
    const size_t ray_bytes = sizeof(lgb_ray) * (size_t)n;
    const size_t out_bytes = any ? sizeof(uint32_t) * (size_t)((n + 31) / 32) : sizeof(lgb_hit) * (size_t)n;
    const size_t out_off = (ray_bytes + 255) & ~(size_t)255;
    if (s->stage_bytes < out_off + out_bytes) {
        cudaFree(s->stage_buf);  // waits for any query still using it
        s->stage_buf = nullptr;
        s->stage_bytes = 0;
        LGB_CUDA_TRY(ctx, cudaMalloc(&s->stage_buf, out_off + out_bytes));
        s->stage_bytes = out_off + out_bytes;
    }
    if (!s->stream_h2d) LGB_CUDA_TRY(ctx, cudaStreamCreateWithFlags((cudaStream_t*)&s->stream_h2d, cudaStreamNonBlocking));
    if (!s->stream_d2h) LGB_CUDA_TRY(ctx, cudaStreamCreateWithFlags((cudaStream_t*)&s->stream_d2h, cudaStreamNonBlocking));
    while (s->stage_events.size() < 2 * kHostChunks + 2) {
        cudaEvent_t e;
        LGB_CUDA_TRY(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        s->stage_events.push_back(e);
    }
    const cudaStream_t up = (cudaStream_t)s->stream_h2d, down = (cudaStream_t)s->stream_d2h;
    cudaEvent_t* ev = reinterpret_cast<cudaEvent_t*>(s->stage_events.data());
    lgb_ray* d_rays = reinterpret_cast<lgb_ray*>(s->stage_buf);
    char* d_out = reinterpret_cast<char*>(s->stage_buf) + out_off;
    uint32_t chunk = (n + kHostChunks - 1) / kHostChunks;
    chunk = std::max(chunk, kHostChunkMin);
    chunk = (chunk + 31u) & ~31u;
    // the staging buffer is free once the caller's stream reaches this point (earlier queries joined it)
    LGB_CUDA_TRY(ctx, cudaEventRecord(ev[0], st));
    LGB_CUDA_TRY(ctx, cudaStreamWaitEvent(up, ev[0], 0));
    LGB_CUDA_TRY(ctx, cudaStreamWaitEvent(down, ev[0], 0));
    uint32_t c = 0;
    for (uint32_t off = 0; off < n; off += chunk, c++) {
        const uint32_t cnt = std::min(chunk, n - off);
        cudaEvent_t arrived = ev[1 + 2 * c], traced = ev[2 + 2 * c];
        LGB_CUDA_TRY(ctx, cudaMemcpyAsync(d_rays + off, h_rays + off, sizeof(lgb_ray) * (size_t)cnt,
                                          cudaMemcpyHostToDevice, up));
        LGB_CUDA_TRY(ctx, cudaEventRecord(arrived, up));
        LGB_CUDA_TRY(ctx, cudaStreamWaitEvent(st, arrived, 0));
        size_t o_off, o_len;
        if (any) {
            uint32_t* bits = reinterpret_cast<uint32_t*>(d_out);
            const lgb_status ls = launch_trace_any(s, d_rays + off, bits + off / 32, cnt, st);
            if (ls != LGB_OK) return ls;
            o_off = sizeof(uint32_t) * (size_t)(off / 32);
            o_len = sizeof(uint32_t) * (size_t)((cnt + 31) / 32);
        } else {
            lgb_hit* hits = reinterpret_cast<lgb_hit*>(d_out);
            const lgb_status ls = launch_trace_closest(s, d_rays + off, hits + off, cnt, st, nullptr);
            if (ls != LGB_OK) return ls;
            o_off = sizeof(lgb_hit) * (size_t)off;
            o_len = sizeof(lgb_hit) * (size_t)cnt;
        }
        LGB_CUDA_TRY(ctx, cudaEventRecord(traced, st));
        LGB_CUDA_TRY(ctx, cudaStreamWaitEvent(down, traced, 0));
        LGB_CUDA_TRY(ctx, cudaMemcpyAsync(reinterpret_cast<char*>(h_out) + o_off, d_out + o_off, o_len,
                                          cudaMemcpyDeviceToHost, down));
    }
    cudaEvent_t done = ev[2 * kHostChunks + 1];
    LGB_CUDA_TRY(ctx, cudaEventRecord(done, down));
    LGB_CUDA_TRY(ctx, cudaStreamWaitEvent(st, done, 0));
    return LGB_OK;
}

lgb_status launch_trace_any(Scene* s, const lgb_ray* rays, uint32_t* bits, uint32_t n, cudaStream_t st) {
    if (n == 0) return LGB_OK;
    LGB_CUDA_TRY(s->ctx, cudaMemsetAsync(s->d_ray_counter, 0, sizeof(uint32_t), st));
    LGB_CUDA_TRY(s->ctx, cudaMemsetAsync(bits, 0, sizeof(uint32_t) * ((n + 31) / 32), st));
    k_trace<true, false><<<persistent_grid<true, false>(s->ctx, n), kTraceThreads, 0, st>>>(
        s->bvh.nodes, s->bvh.tris, rays, nullptr, bits, n, s->d_ray_counter, s->d_status, nullptr, visit_budget(s));
    LGB_CUDA_TRY(s->ctx, cudaGetLastError());
    return LGB_OK;
}

}  // namespace lgb
