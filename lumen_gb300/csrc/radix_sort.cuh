// LSD radix sort of (32- or 64-bit key, 32-bit value) pairs, 8 bits per pass, stable: per-block digit histograms,
// one exclusive scan over all (digit, block) counts, and a scatter that ranks equal digits within each warp
// with __match_any_sync so that equal keys keep their input order. Shared by the BVH builder (Morton codes)
// and the photon grid (hash slots). The scan runs in three steps over tiles of 4096 counts (tile sums, a scan of
// the sums, each tile scanned in shared memory from its offset), all with coalesced loads and stores.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <utility>

namespace lgb {
namespace {

constexpr int RS_THREADS = 256;
constexpr int RS_ITEMS = 8;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;
constexpr int SCAN_THREADS = 512;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

// Words of scratch radix_sort_pairs needs for n pairs: the (digit, block) counts and one sum per scan tile.
inline size_t radix_sort_scratch_words(uint32_t n) {
    const size_t m = 256 * (size_t)((n + RS_TILE - 1) / RS_TILE);
    return m + (m + SCAN_TILE - 1) / SCAN_TILE;
}

template <class KeyT>
__global__ void __launch_bounds__(RS_THREADS) k_rs_hist(const KeyT* __restrict__ keys, uint32_t n, int shift,
                                                        uint32_t* counts, uint32_t nblocks) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    size_t base = (size_t)blockIdx.x * RS_TILE;
    for (int k = 0; k < RS_ITEMS; k++) {
        size_t idx = base + (size_t)k * RS_THREADS + threadIdx.x;
        if (idx < n) atomicAdd(&h[(uint32_t)(keys[idx] >> shift) & 0xffu], 1u);
    }
    __syncthreads();
    counts[(size_t)threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan of m counts in place, one block of 1024 threads.
__global__ void __launch_bounds__(1024) k_scan_single(uint32_t* data, uint32_t m) {
    __shared__ uint32_t warp_sums[32];
    const uint32_t per = (m + 1023) / 1024;
    const uint32_t b = threadIdx.x * per, e = min(m, b + per);
    uint32_t sum = 0;
    for (uint32_t i = b; i < e; i++) sum += data[i];
    // block exclusive scan of sum
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = sum;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = warp_sums[lane];
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        warp_sums[lane] = w;
    }
    __syncthreads();
    uint32_t excl = x - sum + (warp > 0 ? warp_sums[warp - 1] : 0u);
    for (uint32_t i = b; i < e; i++) {
        uint32_t c = data[i];
        data[i] = excl;
        excl += c;
    }
}

// Sum of each SCAN_TILE-count tile of data[0, m) into sums[tile].
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tile_sums(const uint32_t* __restrict__ data, uint32_t m,
                                                                 uint32_t* __restrict__ sums) {
    __shared__ uint32_t ws[SCAN_THREADS / 32];
    const size_t base = (size_t)blockIdx.x * SCAN_TILE;
    uint32_t s = 0;
    for (int k = 0; k < SCAN_ITEMS; k++) {
        const size_t i = base + (size_t)k * SCAN_THREADS + threadIdx.x;
        if (i < m) s += data[i];
    }
    s = __reduce_add_sync(0xffffffffu, s);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        uint32_t v = threadIdx.x < SCAN_THREADS / 32 ? ws[threadIdx.x] : 0u;
        v = __reduce_add_sync(0xffffffffu, v);
        if (threadIdx.x == 0) sums[blockIdx.x] = v;
    }
}

// Exclusive scan of one tile of data[0, m) in place, starting from sums[tile] (0 when sums is null): the tile is
// staged in shared memory, each thread scans SCAN_ITEMS consecutive counts, and the thread totals are scanned
// across the block.
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tile_apply(uint32_t* __restrict__ data, uint32_t m,
                                                                  const uint32_t* __restrict__ sums) {
    __shared__ uint32_t tile[SCAN_TILE];
    __shared__ uint32_t ws[SCAN_THREADS / 32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const size_t base = (size_t)blockIdx.x * SCAN_TILE;
    for (int k = 0; k < SCAN_ITEMS; k++) {
        const int i = k * SCAN_THREADS + tid;
        tile[i] = base + i < m ? data[base + i] : 0u;
    }
    __syncthreads();
    uint32_t v[SCAN_ITEMS];
    uint32_t sum = 0;
    for (int j = 0; j < SCAN_ITEMS; j++) {
        v[j] = tile[tid * SCAN_ITEMS + j];
        sum += v[j];
    }
    uint32_t x = sum;  // inclusive scan of the thread totals within the warp
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < SCAN_THREADS / 32 ? ws[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < SCAN_THREADS / 32) ws[lane] = w;
    }
    __syncthreads();
    uint32_t excl = x - sum + (warp > 0 ? ws[warp - 1] : 0u) + (sums ? sums[blockIdx.x] : 0u);
    for (int j = 0; j < SCAN_ITEMS; j++) {
        tile[tid * SCAN_ITEMS + j] = excl;
        excl += v[j];
    }
    __syncthreads();
    for (int k = 0; k < SCAN_ITEMS; k++) {
        const int i = k * SCAN_THREADS + tid;
        if (base + i < m) data[base + i] = tile[i];
    }
}

// Exclusive scan of data[0, m) in place; data must have room for the tile sums after the m counts.
inline void scan_exclusive(uint32_t* data, uint32_t m, cudaStream_t st) {
    const uint32_t nt = (m + SCAN_TILE - 1) / SCAN_TILE;
    if (nt <= 1) {
        k_scan_tile_apply<<<1, SCAN_THREADS, 0, st>>>(data, m, nullptr);
        return;
    }
    uint32_t* sums = data + m;
    k_scan_tile_sums<<<nt, SCAN_THREADS, 0, st>>>(data, m, sums);
    k_scan_single<<<1, 1024, 0, st>>>(sums, nt);
    k_scan_tile_apply<<<nt, SCAN_THREADS, 0, st>>>(data, m, sums);
}

template <class KeyT>
__global__ void __launch_bounds__(RS_THREADS) k_rs_scatter(const KeyT* __restrict__ kin, const uint32_t* __restrict__ vin,
                                                           KeyT* __restrict__ kout, uint32_t* __restrict__ vout,
                                                           uint32_t n, int shift, const uint32_t* __restrict__ offsets,
                                                           uint32_t nblocks) {
    __shared__ uint32_t base_off[256];
    __shared__ uint32_t warp_cnt[RS_THREADS / 32][256];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    base_off[tid] = offsets[(size_t)tid * nblocks + blockIdx.x];
    const uint32_t lanemask_lt = (1u << lane) - 1u;
    const size_t tile = (size_t)blockIdx.x * RS_TILE;
    for (int r = 0; r < RS_ITEMS; r++) {
        for (int w = 0; w < RS_THREADS / 32; w++) warp_cnt[w][tid] = 0;
        __syncthreads();
        const size_t idx = tile + (size_t)r * RS_THREADS + tid;
        const bool valid = idx < n;
        KeyT key = valid ? kin[idx] : KeyT(0);
        uint32_t val = valid ? vin[idx] : 0u;
        uint32_t digit = valid ? ((uint32_t)(key >> shift) & 0xffu) : (256u + lane);
        uint32_t peers = __match_any_sync(0xffffffffu, digit);
        uint32_t rank = __popc(peers & lanemask_lt);
        int leader = __ffs(peers) - 1;
        if (valid && lane == leader) warp_cnt[warp][digit] = __popc(peers);
        __syncthreads();
        uint32_t running = 0;
        for (int w = 0; w < RS_THREADS / 32; w++) {
            uint32_t c = warp_cnt[w][tid];
            warp_cnt[w][tid] = running;
            running += c;
        }
        __syncthreads();
        if (valid) {
            uint32_t pos = base_off[digit] + warp_cnt[warp][digit] + rank;
            kout[pos] = key;
            vout[pos] = val;
        }
        __syncthreads();
        base_off[tid] += running;
        __syncthreads();
    }
}

// Sorts n pairs by the low 8 * passes bits of the keys (KeyT uint32_t or uint64_t); counts must hold
// radix_sort_scratch_words(n) words. The result ends in (k0, v0) or (k1, v1): the function swaps the pointers so
// that k0 / v0 name the sorted arrays.
template <class KeyT>
inline cudaError_t radix_sort_pairs(KeyT*& k0, uint32_t*& v0, KeyT*& k1, uint32_t*& v1, uint32_t* counts,
                                    uint32_t n, int passes, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    const uint32_t nblocks = (n + RS_TILE - 1) / RS_TILE;
    for (int pass = 0; pass < passes; pass++) {
        const int shift = pass * 8;
        k_rs_hist<KeyT><<<nblocks, RS_THREADS, 0, st>>>(k0, n, shift, counts, nblocks);
        scan_exclusive(counts, 256 * nblocks, st);
        k_rs_scatter<KeyT><<<nblocks, RS_THREADS, 0, st>>>(k0, v0, k1, v1, n, shift, counts, nblocks);
        std::swap(k0, k1);
        std::swap(v0, v1);
    }
    return cudaGetLastError();
}

}  // namespace
}  // namespace lgb
