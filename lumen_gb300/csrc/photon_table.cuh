// The photon table shared by the photon integrators (VCM, SPPM): grid cells and their hash slot
// (vcm_commons.glsl:17-23, utils.glsl:62-65, with get_grid_idx's discarded clamp kept), the grid resolution of
// VCM.cpp:144-147, and the table itself made deterministic: every photon slot is keyed by its hash slot (unused
// slots by the table size, below 2^31, so 32-bit keys), a stable radix sort orders (slot, photon id), and two
// run-boundary kernels write per
// slot the number of photons and the highest photon id, which is the photon a sequential writer leaves last.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "lgb_internal.cuh"
#include "path_common.cuh"
#include "radix_sort.cuh"

namespace lgb {
namespace {

__device__ __forceinline__ int3 grid_idx(v3 p, const float* mn, const float* mx, const int* res) {
    const float nx = (p.x - mn[0]) / (mx[0] - mn[0]), ny = (p.y - mn[1]) / (mx[1] - mn[1]), nz = (p.z - mn[2]) / (mx[2] - mn[2]);
    return make_int3(__float2int_rz(nx * (float)res[0]), __float2int_rz(ny * (float)res[1]), __float2int_rz(nz * (float)res[2]));
}
// utils.glsl:62-65 with the products wrapping as 32-bit integers
__device__ __forceinline__ uint32_t grid_hash(int3 p, uint32_t screen) {
    const uint32_t h = ((uint32_t)p.x * 73856093u) ^ ((uint32_t)p.y * 19349663u) ^ ((uint32_t)p.z * 83492791u);
    return h % (10u * screen);
}

// Run starts: rep[slot] = first sorted position (temporarily).
__global__ void k_table_run_first(const uint32_t* __restrict__ keys, uint32_t n, uint32_t table, uint32_t* rep) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t k = keys[i];
        if (k >= table) continue;
        if (i == 0 || keys[i - 1] != k) rep[k] = i;
    }
}
// Run ends: count = length of the run, rep = its last vertex id.
__global__ void k_table_run_last(const uint32_t* __restrict__ keys, const uint32_t* __restrict__ vals, uint32_t n,
                               uint32_t table, uint32_t* count, uint32_t* rep) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t k = keys[i];
        if (k >= table) continue;
        if (i == n - 1 || keys[i + 1] != k) {
            count[k] = i - rep[k] + 1u;
            rep[k] = vals[i];
        }
    }
}

inline int to_int_rz_host(float x) {
    if (x != x) return 0;
    if (x >= 2147483648.0f) return INT32_MAX;
    if (x <= -2147483648.0f) return INT32_MIN;
    return (int)x;
}


// VCM.cpp:144-147
inline void grid_resolution(const float* mn, const float* mx, float radius, int* res) {
    const float d[3] = {mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2]};
    const float max_comp = std::max(d[0], std::max(d[1], d[2]));
    const int base = to_int_rz_host(max_comp / radius);
    for (int k = 0; k < 3; k++) res[k] = std::max(to_int_rz_host(d[k] * (float)base / max_comp), 1);
}

inline int sort_passes(uint32_t table) {
    int bits = 0;
    while (bits < 32 && (uint64_t)table >= (1ull << bits)) bits++;
    return (bits + 7) / 8;
}

inline int table_grid_blocks(Ctx* ctx, uint64_t n) {
    const int sms = ctx->sm_count > 0 ? ctx->sm_count : 1;
    return (int)std::max<uint64_t>(1, std::min<uint64_t>((n + 255) / 256, (uint64_t)sms * 16));
}

// Sorts (keys, vals) in place (k0/v0 end up holding the result) and writes the table (count and rep zeroed first).
inline lgb_status build_table(Ctx* ctx, uint32_t*& k0, uint32_t*& v0, uint32_t*& k1, uint32_t*& v1, uint32_t* sort_counts, uint32_t n,
                       uint32_t table, uint32_t* count, uint32_t* rep, cudaStream_t st) {
    LGB_CUDA_TRY(ctx, cudaMemsetAsync(count, 0, sizeof(uint32_t) * table, st));
    LGB_CUDA_TRY(ctx, cudaMemsetAsync(rep, 0, sizeof(uint32_t) * table, st));
    LGB_CUDA_TRY(ctx, radix_sort_pairs(k0, v0, k1, v1, sort_counts, n, sort_passes(table), st));
    const int g = table_grid_blocks(ctx, n);
    k_table_run_first<<<g, 256, 0, st>>>(k0, n, table, rep);
    k_table_run_last<<<g, 256, 0, st>>>(k0, v0, n, table, count, rep);
    LGB_CUDA_TRY(ctx, cudaGetLastError());
    return LGB_OK;
}

}  // namespace
}  // namespace lgb
