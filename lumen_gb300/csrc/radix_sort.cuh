// LSD radix sort of (32- or 64-bit key, 32-bit value) pairs, 8 bits per pass, stable, reduce-then-scan over a
// persistent grid: each block owns one contiguous range of tiles for the whole pass. Per pass, a histogram kernel
// counts each block's digits (one read of the keys) and adds them into the pass's digit totals, one warp per digit
// scans that digit's block counts from the digit's start (the totals of the digits below it), which gives every
// block the output position of its first key of each digit, and the scatter kernel walks the block's tiles in
// order, advancing its per-digit positions tile by tile in shared memory. Within a tile the keys are ranked per
// warp with __match_any_sync, staged in digit order in shared memory and written out with consecutive threads on
// consecutive keys, so each digit's run of the tile lands contiguously. Blocks never wait for one another, and
// the count array has 256 entries per block of the grid rather than per tile. Shared by the BVH builder (Morton
// codes) and the photon tables (hash slots).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <utility>

namespace lgb {
namespace {

constexpr int RS_THREADS = 256;
#ifdef LGB_RS_ITEMS
constexpr int RS_ITEMS = LGB_RS_ITEMS;
#else
constexpr int RS_ITEMS = 8;
#endif
// Register budget of the 32-bit-key scatter: 3 blocks per SM (85 registers; 109 unbounded). On the VCM's 11.5 M
// keys, per pass under ncu (histogram + scatter): 13.4 + 46.7 us against 16.5 + 49.2 unbounded and 12.3 + 60.5 at
// 4 blocks (64 registers, spilling); the grid, and so the histogram's, follows the scatter's occupancy. 64-bit keys
// keep the unbounded budget (they would spill).
#ifdef LGB_RS_MIN_BLOCKS
constexpr int RS_MIN_BLOCKS = LGB_RS_MIN_BLOCKS;
#else
constexpr int RS_MIN_BLOCKS = 3;
#endif
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;
// Threads of a histogram block (the histogram's grid is the scatter's). On the VCM's 11.5 M 32-bit keys, per pass
// under ncu: 256 threads 12.0 us, 512 11.3, 1024 13.0 (two blocks per SM instead of three).
#ifdef LGB_RS_HIST_THREADS
constexpr int RS_HIST_THREADS = LGB_RS_HIST_THREADS;
#else
constexpr int RS_HIST_THREADS = 512;
#endif
constexpr int RS_MAX_BLOCKS = 1024;  // blocks of the persistent grid: a bound on the (digit, block) counts

inline uint32_t rs_tiles(uint32_t n) { return (n + RS_TILE - 1) / RS_TILE; }

// Words of scratch radix_sort_pairs needs: the (digit, block) counts, then two sets of digit totals (one per pass,
// alternating).
inline size_t radix_sort_scratch_words(uint32_t n) {
    (void)n;
    return 256 * (size_t)RS_MAX_BLOCKS + 512;
}

// Tiles [t0, t1) of block b of a grid of g blocks over `tiles` tiles.
__device__ __forceinline__ void rs_range(uint32_t tiles, uint32_t b, uint32_t g, uint32_t& t0, uint32_t& t1) {
    t0 = (uint32_t)((uint64_t)tiles * b / g);
    t1 = (uint32_t)((uint64_t)tiles * (b + 1) / g);
}

// Digit counts of each block's range: one shared-memory histogram per warp (fewer collisions on skewed keys, such
// as the hash slots of clustered photons), summed into counts[digit * gridDim.x + block] and added into the
// pass's digit totals (zeroed before the launch).
template <class KeyT>
__global__ void __launch_bounds__(RS_HIST_THREADS) k_rs_hist(const KeyT* __restrict__ keys, uint32_t n, int shift,
                                                             uint32_t tiles, uint32_t* __restrict__ counts,
                                                             uint32_t* __restrict__ totals) {
    constexpr int T = RS_HIST_THREADS;
    __shared__ uint32_t h[T / 32][256];
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int i = tid; i < T / 32 * 256; i += T) (&h[0][0])[i] = 0;
    __syncthreads();
    uint32_t t0, t1;
    rs_range(tiles, blockIdx.x, gridDim.x, t0, t1);
    const size_t e = min((size_t)t1 * RS_TILE, (size_t)n);
    size_t i0 = (size_t)t0 * RS_TILE;
    if constexpr (sizeof(KeyT) == 4) {
        if ((reinterpret_cast<uintptr_t>(keys) & 15u) == 0) {
            // four keys per load (a range starts on a tile, so on a 16-byte boundary)
            const uint4* kv = reinterpret_cast<const uint4*>(keys + i0);
            const size_t nv = i0 < e ? (e - i0) / 4 : 0;
#pragma unroll 4
            for (size_t j = tid; j < nv; j += T) {
                const uint4 k = kv[j];
                atomicAdd(&h[warp][(k.x >> shift) & 0xffu], 1u);
                atomicAdd(&h[warp][(k.y >> shift) & 0xffu], 1u);
                atomicAdd(&h[warp][(k.z >> shift) & 0xffu], 1u);
                atomicAdd(&h[warp][(k.w >> shift) & 0xffu], 1u);
            }
            i0 += nv * 4;
        }
    }
#pragma unroll 8
    for (size_t i = i0 + tid; i < e; i += T)
        atomicAdd(&h[warp][(uint32_t)(keys[i] >> shift) & 0xffu], 1u);
    __syncthreads();
    if (tid < 256) {
        uint32_t c = 0;
        for (int w = 0; w < T / 32; w++) c += h[w][tid];
        counts[(size_t)tid * gridDim.x + blockIdx.x] = c;
        if (c) atomicAdd(&totals[tid], c);
    }
}

// Output positions of every (digit, block): block d scans digit d's g block counts in place (each thread up to
// RS_MAX_BLOCKS / 256 consecutive counts, held in registers), starting from the digit's start, the sum of the
// totals of the digits below it. Replaces a general scan of all 256 x g counts. Also zeroes the other set of
// totals, which the next pass's histogram accumulates into.
__global__ void __launch_bounds__(256) k_rs_digit_offsets(uint32_t* __restrict__ counts, const uint32_t* __restrict__ totals,
                                                          uint32_t* __restrict__ next_totals, uint32_t g) {
    constexpr int PER = RS_MAX_BLOCKS / 256;
    __shared__ uint32_t ws[8];
    __shared__ uint32_t wb[8];
    const uint32_t d = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    uint32_t* row = counts + (size_t)d * g;
    uint32_t c[PER];
    uint32_t sum = 0;
#pragma unroll
    for (int k = 0; k < PER; k++) {
        const uint32_t i = (uint32_t)tid * PER + k;
        c[k] = i < g ? row[i] : 0u;
        sum += c[k];
    }
    uint32_t below = (uint32_t)tid < d ? totals[tid] : 0u;
    below = __reduce_add_sync(0xffffffffu, below);
    uint32_t x = sum;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[warp] = x;
    if (lane == 0) wb[warp] = below;
    __syncthreads();
    if (tid == 0) next_totals[d] = 0u;
    uint32_t run = x - sum;
    for (int w = 0; w < 8; w++) {
        run += w < warp ? ws[w] : 0u;
        run += wb[w];
    }
#pragma unroll
    for (int k = 0; k < PER; k++) {
        const uint32_t i = (uint32_t)tid * PER + k;
        if (i < g) row[i] = run;
        run += c[k];
    }
}

// The scatter of each block's range of tiles (see the header comment). offsets: the scanned (digit, block) counts.
template <class KeyT>
__global__ void __launch_bounds__(RS_THREADS, sizeof(KeyT) == 4 ? RS_MIN_BLOCKS : 1) k_rs_scatter(const KeyT* __restrict__ kin, const uint32_t* __restrict__ vin,
                                                           KeyT* __restrict__ kout, uint32_t* __restrict__ vout,
                                                           uint32_t n, int shift, uint32_t tiles,
                                                           const uint32_t* __restrict__ offsets) {
    constexpr int WARPS = RS_THREADS / 32;
    __shared__ uint32_t out_off[256];     // output position of the next key of each digit
    __shared__ uint32_t tile_start[256];  // position of each digit's first key in the sorted tile
    __shared__ uint32_t wcnt[WARPS][256]; // per-warp digit counts, then each warp's first position within a digit
    __shared__ KeyT skey[RS_TILE];
    __shared__ uint32_t sval[RS_TILE];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t lanemask_lt = (1u << lane) - 1u;
    out_off[tid] = offsets[(size_t)tid * gridDim.x + blockIdx.x];
    uint32_t t0, t1;
    rs_range(tiles, blockIdx.x, gridDim.x, t0, t1);
    const uint32_t wbase = (uint32_t)warp * (RS_ITEMS * 32);  // each warp owns RS_TILE / 8 consecutive keys
    // The pairs of the block's next tile are loaded into registers while the current one is ranked and written.
    KeyT key[RS_ITEMS];
    uint32_t val[RS_ITEMS];
    auto load = [&](uint32_t t, KeyT* k, uint32_t* v) {
        const size_t tile = (size_t)t * RS_TILE;
        const uint32_t tn = (uint32_t)min((size_t)RS_TILE, (size_t)n - tile);
#pragma unroll
        for (int r = 0; r < RS_ITEMS; r++) {
            const uint32_t i = wbase + (uint32_t)r * 32 + lane;
            const bool valid = i < tn;
            k[r] = valid ? kin[tile + i] : KeyT(0);
            v[r] = valid ? vin[tile + i] : 0u;
        }
    };
    if (t0 < t1) load(t0, key, val);
    for (uint32_t t = t0; t < t1; t++) {
        KeyT nkey[RS_ITEMS];
        uint32_t nval[RS_ITEMS];
        if (t + 1 < t1) load(t + 1, nkey, nval);
        for (int w = 0; w < WARPS; w++) wcnt[w][tid] = 0;
        __syncthreads();
        const size_t tile = (size_t)t * RS_TILE;
        const uint32_t tile_n = (uint32_t)min((size_t)RS_TILE, (size_t)n - tile);
        uint32_t slot[RS_ITEMS];
        // ranks within the warp, round after round (input order)
#pragma unroll
        for (int r = 0; r < RS_ITEMS; r++) {
            const uint32_t i = wbase + (uint32_t)r * 32 + lane;
            const bool valid = i < tile_n;
            const uint32_t digit = valid ? ((uint32_t)(key[r] >> shift) & 0xffu) : (256u + lane);
            const uint32_t peers = __match_any_sync(0xffffffffu, digit);
            const uint32_t before = valid ? wcnt[warp][digit] : 0u;
            slot[r] = before + __popc(peers & lanemask_lt);
            __syncwarp();
            if (valid && (__ffs(peers) - 1) == lane) wcnt[warp][digit] = before + __popc(peers);
            __syncwarp();
        }
        __syncthreads();
        // digit tid: the warps' counts in warp order and the tile's count
        uint32_t cnt = 0;
        for (int w = 0; w < WARPS; w++) {
            const uint32_t c = wcnt[w][tid];
            wcnt[w][tid] = cnt;
            cnt += c;
        }
        tile_start[tid] = cnt;
        __syncthreads();
        if (warp == 0) {  // the tile's digit starts: exclusive scan of the 256 counts, 8 per lane
            uint32_t v[8], sum = 0;
            for (int j = 0; j < 8; j++) { v[j] = tile_start[lane * 8 + j]; sum += v[j]; }
            uint32_t x = sum;
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            uint32_t e = x - sum;
            for (int j = 0; j < 8; j++) { tile_start[lane * 8 + j] = e; e += v[j]; }
        }
        __syncthreads();
        // the tile in digit order in shared memory (stable: warp-major, as the input) ...
#pragma unroll
        for (int r = 0; r < RS_ITEMS; r++) {
            const uint32_t i = wbase + (uint32_t)r * 32 + lane;
            if (i < tile_n) {
                const uint32_t digit = (uint32_t)(key[r] >> shift) & 0xffu;
                const uint32_t pos = tile_start[digit] + wcnt[warp][digit] + slot[r];
                skey[pos] = key[r];
                sval[pos] = val[r];
            }
        }
        __syncthreads();
        // ... and each digit's run of it to its place in the output
        for (uint32_t i = tid; i < tile_n; i += RS_THREADS) {
            const KeyT k = skey[i];
            const uint32_t digit = (uint32_t)(k >> shift) & 0xffu;
            const uint32_t pos = out_off[digit] + (i - tile_start[digit]);
            kout[pos] = k;
            vout[pos] = sval[i];
        }
        __syncthreads();
        out_off[tid] += cnt;
#pragma unroll
        for (int r = 0; r < RS_ITEMS; r++) {
            key[r] = nkey[r];
            val[r] = nval[r];
        }
    }
}

// Blocks of the persistent grid: as many as stay resident at once (at most RS_MAX_BLOCKS, at most one per tile).
template <class KeyT>
inline uint32_t rs_grid(uint32_t tiles) {
    static int per_sm = 0;  // resident blocks of the scatter kernel per SM (the same on every device of a build)
    if (per_sm <= 0) {
        int v = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, k_rs_scatter<KeyT>, RS_THREADS, 0);
        per_sm = std::max(v, 1);
    }
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint32_t g = (uint32_t)std::max(sms, 1) * (uint32_t)per_sm;
    return std::max(1u, std::min({g, tiles, (uint32_t)RS_MAX_BLOCKS}));
}

// Sorts n pairs by the low 8 * passes bits of the keys (KeyT uint32_t or uint64_t); counts must hold
// radix_sort_scratch_words(n) words. The result ends in (k0, v0) or (k1, v1): the function swaps the pointers so
// that k0 / v0 name the sorted arrays.
template <class KeyT>
inline cudaError_t radix_sort_pairs(KeyT*& k0, uint32_t*& v0, KeyT*& k1, uint32_t*& v1, uint32_t* counts,
                                    uint32_t n, int passes, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    const uint32_t tiles = rs_tiles(n);
    const uint32_t g = rs_grid<KeyT>(tiles);
    uint32_t* totals = counts + 256 * (size_t)RS_MAX_BLOCKS;
    const cudaError_t e = cudaMemsetAsync(totals, 0, 256 * sizeof(uint32_t), st);
    if (e != cudaSuccess) return e;
    for (int pass = 0; pass < passes; pass++) {
        const int shift = pass * 8;
        uint32_t* cur = totals + 256 * (pass & 1);
        uint32_t* next = totals + 256 * ((pass + 1) & 1);
        k_rs_hist<KeyT><<<g, RS_HIST_THREADS, 0, st>>>(k0, n, shift, tiles, counts, cur);
        k_rs_digit_offsets<<<256, 256, 0, st>>>(counts, cur, next, g);
        k_rs_scatter<KeyT><<<g, RS_THREADS, 0, st>>>(k0, v0, k1, v1, n, shift, tiles, counts);
        std::swap(k0, k1);
        std::swap(v0, v1);
    }
    return cudaGetLastError();
}

}  // namespace
}  // namespace lgb
