// GPU BVH construction for the 8-wide quantised BVH.
//
// Replaces the driver-side BLAS/TLAS build that Lumen requests through vk::build_blas / vk::build_tlas
// (src/Framework/AccelerationStructure.cpp:171-315, called from src/RayTracer/Integrator.cpp:137-160).
// All meshes are flattened into one tree over global triangle ids.
//
// Pipeline (one stream, all on the device):
//   1. triangle bounds + centroid bounds (ordered-integer atomics)
//   2. 63-bit Morton codes of triangle centroids
//   3. LSD radix sort of (code, triangle) pairs, 8 passes of 8 bits, stable block-local ranking
//   4. binary radix tree over the sorted codes (Karras, HPG 2012), ties broken by position
//   5. bottom-up node boxes, SAH costs and triangle counts (first arrival stops, second merges)
//   5b. treelet restructuring rounds: 7-leaf treelets re-topologised for minimum SAH cost (Karras and
//       Aila, HPG 2013)
//   6. top-down collapse to 8-wide nodes, one level per launch: each binary node becomes a wide node
//      by repeatedly opening its largest-area internal child; children are placed in octant slots, boxes
//      quantised to 8 bits with outward rounding, and leaf triangles copied into leaf order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <vector>

#include "lgb_internal.cuh"
#include "radix_sort.cuh"

namespace lgb {
namespace {

constexpr uint32_t kLeafFlag = 0x80000000u;

__device__ __forceinline__ uint32_t f2o(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float o2f(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// bounds[0..2] = centroid min (ordered), [3..5] = centroid max
__global__ void k_centroid_bounds(const float* __restrict__ tv, uint32_t n, uint32_t* bounds) {
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float* v = tv + 9 * (size_t)i;
        for (int a = 0; a < 3; a++) {
            float mn = fminf(fminf(v[a], v[3 + a]), v[6 + a]);
            float mx = fmaxf(fmaxf(v[a], v[3 + a]), v[6 + a]);
            float c = 0.5f * (mn + mx);
            lo[a] = fminf(lo[a], c);
            hi[a] = fmaxf(hi[a], c);
        }
    }
    for (int a = 0; a < 3; a++) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
            hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
        }
    }
    if ((threadIdx.x & 31) == 0) {
        for (int a = 0; a < 3; a++) {
            atomicMin(&bounds[a], f2o(lo[a]));
            atomicMax(&bounds[3 + a], f2o(hi[a]));
        }
    }
}

__device__ __forceinline__ uint64_t split3(uint32_t a) {
    uint64_t x = a & 0x1fffffu;
    x = (x | x << 32) & 0x1f00000000ffffull;
    x = (x | x << 16) & 0x1f0000ff0000ffull;
    x = (x | x << 8) & 0x100f00f00f00f00full;
    x = (x | x << 4) & 0x10c30c30c30c30c3ull;
    x = (x | x << 2) & 0x1249249249249249ull;
    return x;
}

__global__ void k_morton(const float* __restrict__ tv, uint32_t n, const uint32_t* bounds, uint64_t* keys,
                         uint32_t* vals, float* tri_box /* 6 per tri: lo xyz, hi xyz */) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* v = tv + 9 * (size_t)i;
    uint32_t q[3];
    for (int a = 0; a < 3; a++) {
        float mn = fminf(fminf(v[a], v[3 + a]), v[6 + a]);
        float mx = fmaxf(fmaxf(v[a], v[3 + a]), v[6 + a]);
        tri_box[6 * (size_t)i + a] = mn;
        tri_box[6 * (size_t)i + 3 + a] = mx;
        float c = 0.5f * (mn + mx);
        float clo = o2f(bounds[a]), chi = o2f(bounds[3 + a]);
        float ext = chi - clo;
        float t = ext > 0.0f ? (c - clo) / ext : 0.0f;
        float s = t * 2097152.0f;
        s = fminf(fmaxf(s, 0.0f), 2097151.0f);
        q[a] = (uint32_t)s;
    }
    keys[i] = (split3(q[0]) << 2) | (split3(q[1]) << 1) | split3(q[2]);
    vals[i] = i;
}

// ---------------- binary radix tree (Karras 2012) ----------------
__device__ __forceinline__ int delta(const uint64_t* keys, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    uint64_t a = keys[i], b = keys[j];
    if (a == b) return 64 + __clz((uint32_t)(i ^ j));
    return __clzll(a ^ b);
}

__global__ void k_radix_tree(const uint64_t* __restrict__ keys, int n, uint32_t* left, uint32_t* right,
                             uint32_t* parent_int, uint32_t* parent_leaf, uint32_t* range_lo, uint32_t* range_hi) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = delta(keys, n, i, i - d);
    int lmax = 2;
    while (delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = delta(keys, n, i, j);
    int s = 0, t = l;
    do {
        t = (t + 1) >> 1;
        if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    int gamma = i + s * d + min(d, 0);
    int lo = min(i, j), hi = max(i, j);
    uint32_t lc = (lo == gamma) ? ((uint32_t)gamma | kLeafFlag) : (uint32_t)gamma;
    uint32_t rc = (hi == gamma + 1) ? ((uint32_t)(gamma + 1) | kLeafFlag) : (uint32_t)(gamma + 1);
    left[i] = lc;
    right[i] = rc;
    range_lo[i] = lo;
    range_hi[i] = hi;
    if (lc & kLeafFlag) parent_leaf[lc & ~kLeafFlag] = i; else parent_int[lc] = i;
    if (rc & kLeafFlag) parent_leaf[rc & ~kLeafFlag] = i; else parent_int[rc] = i;
}

// Bottom-up boxes. node_box: 6 floats per internal node; leaf boxes come from tri_box via sorted vals.
// SAH constants of the binary tree the treelet pass optimises: cost of an internal node and of a triangle.
constexpr float kCostNode = 1.2f;
constexpr float kCostTri = 1.0f;

__device__ __forceinline__ float box_half_area(const float* b) {
    const float dx = fmaxf(b[3] - b[0], 0.0f), dy = fmaxf(b[4] - b[1], 0.0f), dz = fmaxf(b[5] - b[2], 0.0f);
    return dx * dy + dy * dz + dz * dx;
}

__global__ void k_bottom_up(int n, const uint32_t* __restrict__ vals, const float* __restrict__ tri_box,
                            const uint32_t* __restrict__ left, const uint32_t* __restrict__ right,
                            const uint32_t* __restrict__ parent_int, const uint32_t* __restrict__ parent_leaf,
                            float* node_box, float* node_cost, uint32_t* node_count, uint32_t* flags) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    uint32_t node = parent_leaf[k];
    // A radix tree over n keys is at most n - 1 levels deep; the bound only guards against a malformed tree.
    for (int steps = 0; steps < n; steps++) {
        __threadfence();
        if (atomicAdd(&flags[node], 1u) == 0u) return;
        __threadfence();
        float b[6];
        uint32_t cl = left[node], cr = right[node];
        const float* A = (cl & kLeafFlag) ? &tri_box[6 * (size_t)vals[cl & ~kLeafFlag]] : &node_box[6 * (size_t)cl];
        const float* B = (cr & kLeafFlag) ? &tri_box[6 * (size_t)vals[cr & ~kLeafFlag]] : &node_box[6 * (size_t)cr];
        for (int a = 0; a < 3; a++) {
            b[a] = fminf(__ldcg(&A[a]), __ldcg(&B[a]));
            b[3 + a] = fmaxf(__ldcg(&A[3 + a]), __ldcg(&B[3 + a]));
        }
        for (int a = 0; a < 6; a++) __stcg(&node_box[6 * (size_t)node + a], b[a]);
        const float cl_cost = (cl & kLeafFlag) ? kCostTri * box_half_area(A) : __ldcg(&node_cost[cl]);
        const float cr_cost = (cr & kLeafFlag) ? kCostTri * box_half_area(B) : __ldcg(&node_cost[cr]);
        const uint32_t cl_cnt = (cl & kLeafFlag) ? 1u : __ldcg(&node_count[cl]);
        const uint32_t cr_cnt = (cr & kLeafFlag) ? 1u : __ldcg(&node_count[cr]);
        __stcg(&node_cost[node], kCostNode * box_half_area(b) + cl_cost + cr_cost);
        __stcg(&node_count[node], cl_cnt + cr_cnt);
        if (node == 0) return;
        node = parent_int[node];
    }
}

// ---------------- treelet restructuring (Karras and Aila, HPG 2013) ----------------
// A bottom-up pass like k_bottom_up. When the second child of a node with at least `gamma` triangles has
// finished, the arriving thread grows a treelet of up to 7 leaves under it (always splitting the
// largest-area leaf), finds the binary topology over those leaves with minimum SAH cost by dynamic
// programming over all 127 leaf subsets, and rebuilds the treelet's internal nodes in place when that
// lowers the cost. Treelets of different threads are disjoint: a node's descendants are final before the
// node is processed, and its ancestors are untouched until it is done.
constexpr int kTreeletLeaves = 7;

struct TreeArgs {
    uint32_t* left;
    uint32_t* right;
    uint32_t* parent_int;
    uint32_t* parent_leaf;
    float* node_box;
    float* node_cost;
    uint32_t* node_count;
    const float* tri_box;
    const uint32_t* vals;
    uint32_t* flags;
};

__device__ __forceinline__ void load_ref_box(const TreeArgs& T, uint32_t ref, float* b) {
    if (ref & kLeafFlag) {
        const float* src = &T.tri_box[6 * (size_t)T.vals[ref & ~kLeafFlag]];
        for (int a = 0; a < 6; a++) b[a] = src[a];
    } else {
        for (int a = 0; a < 6; a++) b[a] = __ldcg(&T.node_box[6 * (size_t)ref + a]);
    }
}

// Shared-memory DP tables of one warp.
struct TreeletSmem {
    float cost[1 << kTreeletLeaves];
    float area[1 << kTreeletLeaves];
    uint8_t part[1 << kTreeletLeaves];
};

// Optimises the treelet under `root` with the whole warp (all 32 lanes call it with the same root). Every lane
// grows the same treelet from the same loads; the subsets' box areas and then their optimal partitions are
// computed one subset per lane, subset sizes in increasing order; lane 0 rewrites the nodes. Each subset's
// partitions are tried in the order of a sequential search with the same arithmetic, so the tree is the one a
// single-thread search would build.
__device__ void optimise_treelet_warp(const TreeArgs& T, uint32_t root, TreeletSmem& sm) {
    const int lane = threadIdx.x & 31;
    uint32_t leaves[kTreeletLeaves];
    uint32_t inner[kTreeletLeaves - 1];
    float lbox[kTreeletLeaves][6];
    float larea[kTreeletLeaves];
    int nl = 2, ni = 1;
    inner[0] = root;
    leaves[0] = __ldcg(&T.left[root]);
    leaves[1] = __ldcg(&T.right[root]);
    load_ref_box(T, leaves[0], lbox[0]);
    load_ref_box(T, leaves[1], lbox[1]);
    larea[0] = box_half_area(lbox[0]);
    larea[1] = box_half_area(lbox[1]);
    while (nl < kTreeletLeaves) {
        int best = -1;
        float ba = -1.0f;
        for (int k = 0; k < nl; k++)
            if (!(leaves[k] & kLeafFlag) && larea[k] > ba) { ba = larea[k]; best = k; }
        if (best < 0) break;
        const uint32_t r = leaves[best];
        inner[ni++] = r;
        leaves[best] = __ldcg(&T.left[r]);
        leaves[nl] = __ldcg(&T.right[r]);
        load_ref_box(T, leaves[best], lbox[best]);
        load_ref_box(T, leaves[nl], lbox[nl]);
        larea[best] = box_half_area(lbox[best]);
        larea[nl] = box_half_area(lbox[nl]);
        nl++;
    }
    if (nl < 3) return;  // the same on every lane
    const uint32_t full = (1u << nl) - 1u;
    // singletons and the union areas of the larger subsets
    for (uint32_t sset = 1u + (uint32_t)lane; sset <= full; sset += 32u) {
        if ((sset & (sset - 1u)) == 0u) {
            const int k = __ffs(sset) - 1;
            sm.cost[sset] = (leaves[k] & kLeafFlag) ? kCostTri * larea[k] : __ldcg(&T.node_cost[leaves[k]]);
            sm.part[sset] = 0;
            continue;
        }
        float b[6] = {FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX};
        for (int k = 0; k < nl; k++)
            if (sset & (1u << k))
                for (int a = 0; a < 3; a++) { b[a] = fminf(b[a], lbox[k][a]); b[3 + a] = fmaxf(b[3 + a], lbox[k][3 + a]); }
        sm.area[sset] = box_half_area(b);
    }
    __syncwarp();
    for (int size = 2; size <= nl; size++) {
        for (uint32_t sset = 1u + (uint32_t)lane; sset <= full; sset += 32u) {
            if (__popc(sset) != size) continue;
            const uint32_t low = sset & (0u - sset);
            float bc = FLT_MAX;
            uint32_t bp = low;
            for (uint32_t q = (sset - 1u) & sset; q; q = (q - 1u) & sset) {
                if (!(q & low)) continue;  // each unordered split once
                const float c = sm.cost[q] + sm.cost[sset ^ q];
                if (c < bc) { bc = c; bp = q; }
            }
            sm.cost[sset] = kCostNode * sm.area[sset] + bc;
            sm.part[sset] = (uint8_t)bp;
        }
        __syncwarp();
    }
    const bool better = sm.cost[full] < __ldcg(&T.node_cost[root]) * 0.9999f;
    if (better && lane == 0) {
        // rebuild top-down, reusing the treelet's internal nodes
        uint32_t st_set[kTreeletLeaves], st_node[kTreeletLeaves];
        int sp = 0, next = 1;
        st_set[sp] = full;
        st_node[sp] = root;
        sp++;
        while (sp > 0) {
            sp--;
            const uint32_t sset = st_set[sp], node = st_node[sp];
            const uint32_t sub[2] = {sm.part[sset], sset ^ sm.part[sset]};
            uint32_t ref[2];
            for (int c = 0; c < 2; c++) {
                if ((sub[c] & (sub[c] - 1u)) == 0u) {
                    ref[c] = leaves[__ffs(sub[c]) - 1];
                } else {
                    ref[c] = inner[next++];
                    st_set[sp] = sub[c];
                    st_node[sp] = ref[c];
                    sp++;
                }
                if (ref[c] & kLeafFlag) __stcg(&T.parent_leaf[ref[c] & ~kLeafFlag], node);
                else __stcg(&T.parent_int[ref[c]], node);
            }
            __stcg(&T.left[node], ref[0]);
            __stcg(&T.right[node], ref[1]);
            float b[6] = {FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX};
            uint32_t cnt = 0;
            for (int k = 0; k < nl; k++) {
                if (!(sset & (1u << k))) continue;
                for (int a = 0; a < 3; a++) { b[a] = fminf(b[a], lbox[k][a]); b[3 + a] = fmaxf(b[3 + a], lbox[k][3 + a]); }
                cnt += (leaves[k] & kLeafFlag) ? 1u : __ldcg(&T.node_count[leaves[k]]);
            }
            for (int a = 0; a < 6; a++) __stcg(&T.node_box[6 * (size_t)node + a], b[a]);
            __stcg(&T.node_cost[node], sm.cost[sset]);
            __stcg(&T.node_count[node], cnt);
        }
        __threadfence();  // the rewrite is visible before any lane of the warp signals the parent
    }
    __syncwarp();
}

constexpr int kTreeletThreads = 128;

// Bottom-up pass, warp-synchronous: in each step every lane still climbing takes the next node on its path
// (the first of the two children to finish stops there), refreshes that node's cost from its children, and
// the warp then optimises, one after another, the treelets of the lanes whose node has at least `gamma`
// triangles. The step count is bounded by the number of triangles (a path from a leaf to the root is shorter).
__global__ void __launch_bounds__(kTreeletThreads) k_treelet(TreeArgs T, int n, uint32_t gamma) {
    __shared__ TreeletSmem smem[kTreeletThreads / 32];
    TreeletSmem& sm = smem[threadIdx.x >> 5];
    const unsigned FULL = 0xffffffffu;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    bool climbing = k < n;
    uint32_t node = climbing ? __ldcg(&T.parent_leaf[k]) : 0u;
    for (int steps = 0; steps <= n && __any_sync(FULL, climbing); steps++) {
        bool ready = false;
        if (climbing) {
            __threadfence();
            if (atomicAdd(&T.flags[node], 1u) == 0u) {
                climbing = false;
            } else {
                __threadfence();
                ready = true;
                // children are final: refresh this node's cost
                const uint32_t cl = __ldcg(&T.left[node]), cr = __ldcg(&T.right[node]);
                float bl[6], br[6];
                load_ref_box(T, cl, bl);
                load_ref_box(T, cr, br);
                const float ccl = (cl & kLeafFlag) ? kCostTri * box_half_area(bl) : __ldcg(&T.node_cost[cl]);
                const float ccr = (cr & kLeafFlag) ? kCostTri * box_half_area(br) : __ldcg(&T.node_cost[cr]);
                float nb[6];
                for (int a = 0; a < 3; a++) { nb[a] = fminf(bl[a], br[a]); nb[3 + a] = fmaxf(bl[3 + a], br[3 + a]); }
                __stcg(&T.node_cost[node], kCostNode * box_half_area(nb) + ccl + ccr);
            }
        }
        uint32_t todo = __ballot_sync(FULL, ready && __ldcg(&T.node_count[node]) >= gamma);
        while (todo) {
            const int src = __ffs(todo) - 1;
            todo &= todo - 1u;
            optimise_treelet_warp(T, __shfl_sync(FULL, node, src), sm);
        }
        if (ready) {
            __threadfence();
            if (node == 0) climbing = false;
            else node = __ldcg(&T.parent_int[node]);
        }
    }
}

// ---------------- collapse to 8-wide ----------------
struct CollapseArgs {
    const uint32_t* left;
    const uint32_t* right;
    const uint32_t* node_count;
    const float* node_box;
    const float* tri_box;
    const uint32_t* vals;   // sorted position -> original triangle
    const float* tri_verts;
    WideNode* nodes;
    WideTri* tris;
    uint32_t* counters;     // [0] = nodes allocated, [1] = triangles written, [2] = next queue size
    float* sah;             // accumulated SAH numerator
    int leaf_max;
    int e_min[3];           // minimum biased-less exponent per axis
    float inv_root_area;
};

__device__ __forceinline__ void ref_box(const CollapseArgs& A, uint32_t ref, float* b) {
    const float* src = (ref & kLeafFlag) ? &A.tri_box[6 * (size_t)A.vals[ref & ~kLeafFlag]] : &A.node_box[6 * (size_t)ref];
    for (int a = 0; a < 6; a++) b[a] = src[a];
}
__device__ __forceinline__ uint32_t ref_count(const CollapseArgs& A, uint32_t ref) {
    return (ref & kLeafFlag) ? 1u : A.node_count[ref];
}
// Sorted-order positions of the (at most 3) triangles under a small subtree.
__device__ __forceinline__ int gather_leaves(const CollapseArgs& A, uint32_t ref, uint32_t* out) {
    uint32_t st[4];
    int sp = 0, n = 0;
    st[sp++] = ref;
    while (sp > 0 && n < 3) {
        const uint32_t r = st[--sp];
        if (r & kLeafFlag) {
            out[n++] = r & ~kLeafFlag;
        } else if (sp + 2 <= 4) {
            st[sp++] = A.right[r];
            st[sp++] = A.left[r];
        }
    }
    return n;
}
__device__ __forceinline__ float half_area(const float* b) {
    float dx = fmaxf(b[3] - b[0], 0.0f), dy = fmaxf(b[4] - b[1], 0.0f), dz = fmaxf(b[5] - b[2], 0.0f);
    return dx * dy + dy * dz + dz * dx;
}

__global__ void k_collapse(CollapseArgs A, const uint2* __restrict__ qin, uint32_t nin, uint2* __restrict__ qout) {
    uint32_t qi = blockIdx.x * blockDim.x + threadIdx.x;
    if (qi >= nin) return;
    const uint32_t bref = qin[qi].x, widx = qin[qi].y;
    uint32_t ch[8];
    int nc = 0;
    if (bref & kLeafFlag) {
        ch[nc++] = bref;
    } else {
        ch[nc++] = A.left[bref];
        ch[nc++] = A.right[bref];
        while (nc < 8) {
            int best = -1;
            float best_area = -1.0f;
            for (int c = 0; c < nc; c++) {
                if (ch[c] & kLeafFlag) continue;
                float b[6];
                ref_box(A, ch[c], b);
                float ar = half_area(b);
                if (ar > best_area) { best_area = ar; best = c; }
            }
            if (best < 0) break;
            uint32_t r = ch[best];
            ch[best] = A.left[r];
            ch[nc++] = A.right[r];
        }
    }
    // node box = union of children
    float nb[6] = {FLT_MAX, FLT_MAX, FLT_MAX, -FLT_MAX, -FLT_MAX, -FLT_MAX};
    float cb[8][6];
    for (int c = 0; c < nc; c++) {
        ref_box(A, ch[c], cb[c]);
        for (int a = 0; a < 3; a++) { nb[a] = fminf(nb[a], cb[c][a]); nb[3 + a] = fmaxf(nb[3 + a], cb[c][3 + a]); }
    }
    // slot assignment: greedy on alignment of the child centre offset with each octant direction
    float pc[3] = {0.5f * (nb[0] + nb[3]), 0.5f * (nb[1] + nb[4]), 0.5f * (nb[2] + nb[5])};
    int child_in_slot[8];
    for (int s = 0; s < 8; s++) child_in_slot[s] = -1;
    bool assigned[8] = {false, false, false, false, false, false, false, false};
    for (int it = 0; it < nc; it++) {
        float best = -FLT_MAX;
        int bc = -1, bs = -1;
        for (int c = 0; c < nc; c++) {
            if (assigned[c]) continue;
            float off[3];
            for (int a = 0; a < 3; a++) off[a] = 0.5f * (cb[c][a] + cb[c][3 + a]) - pc[a];
            for (int s = 0; s < 8; s++) {
                if (child_in_slot[s] >= 0) continue;
                float score = ((s & 1) ? off[0] : -off[0]) + ((s & 2) ? off[1] : -off[1]) + ((s & 4) ? off[2] : -off[2]);
                if (score > best) { best = score; bc = c; bs = s; }
            }
        }
        if (bc < 0) {  // non-finite boxes: take the first free child and slot
            for (int c = 0; c < nc && bc < 0; c++) if (!assigned[c]) bc = c;
            for (int s2 = 0; s2 < 8 && bs < 0; s2++) if (child_in_slot[s2] < 0) bs = s2;
        }
        assigned[bc] = true;
        child_in_slot[bs] = bc;
    }
    // classify, allocate
    const int leaf_max = A.leaf_max;
    uint32_t imask = 0, n_int = 0, n_tri = 0;
    for (int s = 0; s < 8; s++) {
        int c = child_in_slot[s];
        if (c < 0) continue;
        uint32_t cnt = ref_count(A, ch[c]);
        if ((int)cnt > leaf_max) { imask |= 1u << s; n_int++; }
        else n_tri += cnt;
    }
    uint32_t child_base = n_int ? atomicAdd(&A.counters[0], n_int) : 0u;
    uint32_t tri_base = n_tri ? atomicAdd(&A.counters[1], n_tri) : 0u;
    uint32_t qbase = n_int ? atomicAdd(&A.counters[2], n_int) : 0u;
    // quantisation frame
    WideNode node;
    float scale[3];
    int eb[3];
    for (int a = 0; a < 3; a++) {
        float ext = nb[3 + a] - nb[a];
        int e;
        if (ext > 0.0f) {
            frexpf(ext / 252.0f, &e);  // 2^e >= ext / 252
        } else {
            e = A.e_min[a];
        }
        e = max(e, A.e_min[a]);
        eb[a] = e;
        scale[a] = ldexpf(1.0f, e);
    }
    node.px = nb[0] - scale[0];
    node.py = nb[1] - scale[1];
    node.pz = nb[2] - scale[2];
    const float p[3] = {node.px, node.py, node.pz};
    node.e_imask = (uint32_t)(eb[0] + 127) | ((uint32_t)(eb[1] + 127) << 8) | ((uint32_t)(eb[2] + 127) << 16) | (imask << 24);
    node.child_base = child_base;
    node.tri_base = tri_base;
    uint8_t meta[8];
    uint8_t qlo[3][8], qhi[3][8];
    uint32_t int_rank = 0, tri_off = 0;
    float sah = half_area(nb) * A.inv_root_area;
    for (int s = 0; s < 8; s++) {
        int c = child_in_slot[s];
        if (c < 0) {
            meta[s] = 0;
            for (int a = 0; a < 3; a++) { qlo[a][s] = 255; qhi[a][s] = 0; }
            continue;
        }
        for (int a = 0; a < 3; a++) {
            float lo = floorf((cb[c][a] - p[a]) / scale[a]) - 1.0f;
            float hi = ceilf((cb[c][3 + a] - p[a]) / scale[a]) + 1.0f;
            qlo[a][s] = (uint8_t)fminf(fmaxf(lo, 0.0f), 255.0f);
            qhi[a][s] = (uint8_t)fminf(fmaxf(hi, 0.0f), 255.0f);
        }
        uint32_t cnt = ref_count(A, ch[c]);
        if (imask & (1u << s)) {
            meta[s] = 0;
            qout[qbase + int_rank] = make_uint2(ch[c], child_base + int_rank);
            int_rank++;
        } else {
            meta[s] = (uint8_t)((((1u << cnt) - 1u) << 5) | tri_off);
            uint32_t pos[3];
            gather_leaves(A, ch[c], pos);
            for (uint32_t k = 0; k < cnt; k++) {
                uint32_t prim = A.vals[pos[k]];
                const float* v = A.tri_verts + 9 * (size_t)prim;
                WideTri t;
                t.a = make_float4(v[0], v[1], v[2], __uint_as_float(prim));
                t.b = make_float4(v[3], v[4], v[5], 0.0f);
                t.c = make_float4(v[6], v[7], v[8], 0.0f);
                A.tris[tri_base + tri_off + k] = t;
            }
            sah += half_area(cb[c]) * A.inv_root_area * (float)cnt;
            tri_off += cnt;
        }
    }
    node.meta_lo = meta[0] | (meta[1] << 8) | (meta[2] << 16) | ((uint32_t)meta[3] << 24);
    node.meta_hi = meta[4] | (meta[5] << 8) | (meta[6] << 16) | ((uint32_t)meta[7] << 24);
    for (int s = 0; s < 8; s++) {
        node.qlo_x[s] = qlo[0][s]; node.qlo_y[s] = qlo[1][s]; node.qlo_z[s] = qlo[2][s];
        node.qhi_x[s] = qhi[0][s]; node.qhi_y[s] = qhi[1][s]; node.qhi_z[s] = qhi[2][s];
    }
    A.nodes[widx] = node;
    atomicAdd(A.sah, sah);
}

template <class T> cudaError_t dalloc(T** p, size_t count) { return cudaMalloc((void**)p, sizeof(T) * (count ? count : 1)); }

}  // namespace

lgb_status build_bvh(Scene* s, const lgb_build_opts* opts, lgb_build_stats* stats) {
    Ctx* ctx = s->ctx;
    const uint32_t n = s->num_tris;
    // Default leaf size (triangles per leaf slot) by scene size. Large scenes trace faster with one triangle per
    // slot (more, smaller nodes, fewer triangle tests); small scenes with three (fewer node visits). Measured on
    // GB300 (Mrays/s or ms, leaf size 3 / 2 / 1): the 1M-triangle scene's 4M incoherent rays 1301 / 1350 / 1370;
    // the 200k-triangle caustics VCM iteration 7.96 / 7.92 / 8.07 ms; the 36-triangle Cornell path tracer
    // 563 / 563 / 486 Msamples/s and its differentiable primal 16.3 / 16.3 / 17.8 ms.
#ifdef LGB_BVH_DEFAULT_LEAF
    const int leaf_default = LGB_BVH_DEFAULT_LEAF;
#else
    const int leaf_default = n >= (1u << 19) ? 1 : (n >= (1u << 15) ? 2 : 3);
#endif
    int leaf_max = (opts && opts->leaf_max) ? (int)opts->leaf_max : leaf_default;
    int treelet_rounds = 3;
    if (opts && opts->treelet_rounds)
        treelet_rounds = opts->treelet_rounds == 0xFFFFFFFFu ? 0 : (int)std::min(opts->treelet_rounds, 16u);
    if (leaf_max < 1 || leaf_max > 3) return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "leaf_max must be 1..3");
    if (n == 0) return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "scene has no triangles");
    cudaStream_t st = 0;
    cudaEvent_t e0, e1;
    LGB_CUDA_TRY(ctx, cudaEventCreate(&e0));
    LGB_CUDA_TRY(ctx, cudaEventCreate(&e1));
    LGB_CUDA_TRY(ctx, cudaEventRecord(e0, st));

    // scratch
    uint64_t *keys = nullptr, *keys2 = nullptr;
    uint32_t *vals = nullptr, *vals2 = nullptr, *counts = nullptr, *bounds = nullptr;
    uint32_t *left = nullptr, *right = nullptr, *pint = nullptr, *pleaf = nullptr, *rlo = nullptr, *rhi = nullptr, *flags = nullptr;
    float *tri_box = nullptr, *node_box = nullptr, *sah = nullptr, *node_cost = nullptr;
    uint32_t* node_count = nullptr;
    uint2 *qa = nullptr, *qb = nullptr;
    uint32_t* counters = nullptr;
    WideNode* nodes = nullptr;
    WideTri* tris = nullptr;
    const uint32_t nint = n > 1 ? n - 1 : 1;
    lgb_status status = LGB_OK;
    auto fail = [&](cudaError_t e, const char* what) { status = cuda_error(ctx, e, what); };
#define STEP(expr)                       \
    do {                                 \
        cudaError_t _e = (expr);         \
        if (_e != cudaSuccess) { fail(_e, #expr); goto cleanup; } \
    } while (0)
    {
        STEP(dalloc(&keys, n)); STEP(dalloc(&keys2, n)); STEP(dalloc(&vals, n)); STEP(dalloc(&vals2, n));
        STEP(dalloc(&counts, radix_sort_scratch_words(n))); STEP(dalloc(&bounds, 6));
        STEP(dalloc(&left, nint)); STEP(dalloc(&right, nint)); STEP(dalloc(&pint, nint)); STEP(dalloc(&pleaf, n));
        STEP(dalloc(&rlo, nint)); STEP(dalloc(&rhi, nint)); STEP(dalloc(&flags, nint));
        STEP(dalloc(&tri_box, 6 * (size_t)n)); STEP(dalloc(&node_box, 6 * (size_t)nint)); STEP(dalloc(&sah, 1));
        STEP(dalloc(&node_cost, nint)); STEP(dalloc(&node_count, nint));
        STEP(dalloc(&qa, nint + 1)); STEP(dalloc(&qb, nint + 1)); STEP(dalloc(&counters, 4));
        STEP(dalloc(&nodes, nint)); STEP(dalloc(&tris, n));

        uint32_t binit[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
        STEP(cudaMemcpyAsync(bounds, binit, sizeof(binit), cudaMemcpyHostToDevice, st));
        int grid = std::min<uint32_t>((n + 255) / 256, (uint32_t)ctx->sm_count * 8);
        k_centroid_bounds<<<grid, 256, 0, st>>>(s->d_tri_verts, n, bounds);
        k_morton<<<(n + 255) / 256, 256, 0, st>>>(s->d_tri_verts, n, bounds, keys, vals, tri_box);
        STEP(cudaGetLastError());
        STEP(radix_sort_pairs(keys, vals, keys2, vals2, counts, n, 8, st));
        uint32_t root_ref;
        if (n > 1) {
            k_radix_tree<<<(n - 1 + 255) / 256, 256, 0, st>>>(keys, (int)n, left, right, pint, pleaf, rlo, rhi);
            STEP(cudaMemsetAsync(flags, 0, sizeof(uint32_t) * nint, st));
            k_bottom_up<<<(n + 255) / 256, 256, 0, st>>>((int)n, vals, tri_box, left, right, pint, pleaf, node_box,
                                                         node_cost, node_count, flags);
            STEP(cudaGetLastError());
            TreeArgs T{left, right, pint, pleaf, node_box, node_cost, node_count, tri_box, vals, flags};
            for (int round = 0; round < treelet_rounds; round++) {
                STEP(cudaMemsetAsync(flags, 0, sizeof(uint32_t) * nint, st));
                k_treelet<<<(n + kTreeletThreads - 1) / kTreeletThreads, kTreeletThreads, 0, st>>>(T, (int)n, (uint32_t)kTreeletLeaves);
                STEP(cudaGetLastError());
            }
            root_ref = 0;
        } else {
            root_ref = kLeafFlag;
        }
        // root area for SAH statistics
        float rb[6];
        if (n > 1) {
            STEP(cudaMemcpyAsync(rb, node_box, sizeof(rb), cudaMemcpyDeviceToHost, st));
        } else {
            STEP(cudaMemcpyAsync(rb, tri_box, sizeof(rb), cudaMemcpyDeviceToHost, st));
        }
        STEP(cudaStreamSynchronize(st));
        float ra = fmaxf(rb[3] - rb[0], 0.f) * fmaxf(rb[4] - rb[1], 0.f) + fmaxf(rb[4] - rb[1], 0.f) * fmaxf(rb[5] - rb[2], 0.f) +
                   fmaxf(rb[5] - rb[2], 0.f) * fmaxf(rb[3] - rb[0], 0.f);

        CollapseArgs A;
        A.left = left; A.right = right; A.node_count = node_count; A.node_box = node_box; A.tri_box = tri_box;
        A.vals = vals; A.tri_verts = s->d_tri_verts; A.nodes = nodes; A.tris = tris; A.counters = counters; A.sah = sah;
        A.leaf_max = leaf_max;
        A.inv_root_area = ra > 0.0f ? 1.0f / ra : 0.0f;
        // The minimum quantisation step keeps one step of margin above FP32 rounding of ray distances
        // measured across the whole scene (about 2^-18 of the scene's largest extent).
        float ext = fmaxf(fmaxf(s->bmax.x - s->bmin.x, s->bmax.y - s->bmin.y), s->bmax.z - s->bmin.z);
        float mag = fmaxf(fmaxf(fmaxf(fabsf(s->bmin.x), fabsf(s->bmax.x)), fmaxf(fabsf(s->bmin.y), fabsf(s->bmax.y))),
                          fmaxf(fabsf(s->bmin.z), fabsf(s->bmax.z)));
        float ref = fmaxf(fmaxf(ext, mag), 1e-30f);
        int eref;
        frexpf(ref, &eref);
        for (int a = 0; a < 3; a++) A.e_min[a] = std::max(eref - 18, -100);

        uint32_t zero4[4] = {1u, 0u, 0u, 0u};  // node 0 = root already allocated
        STEP(cudaMemcpyAsync(counters, zero4, sizeof(zero4), cudaMemcpyHostToDevice, st));
        STEP(cudaMemsetAsync(sah, 0, sizeof(float), st));
        uint2 root = make_uint2(root_ref, 0u);
        STEP(cudaMemcpyAsync(qa, &root, sizeof(root), cudaMemcpyHostToDevice, st));
        uint32_t qn = 1, depth = 0;
        while (qn > 0) {
            depth++;
            if (depth > (uint32_t)kStackSize + 1u) {
                status = set_error(ctx, LGB_ERR_UNSUPPORTED, "8-wide BVH deeper than the traversal stack");
                goto cleanup;
            }
            STEP(cudaMemsetAsync(counters + 2, 0, sizeof(uint32_t), st));
            k_collapse<<<(qn + 127) / 128, 128, 0, st>>>(A, qa, qn, qb);
            STEP(cudaGetLastError());
            STEP(cudaMemcpyAsync(&qn, counters + 2, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
            STEP(cudaStreamSynchronize(st));
            std::swap(qa, qb);
        }
        uint32_t hc[4];
        float hsah = 0.0f;
        STEP(cudaMemcpy(hc, counters, sizeof(hc), cudaMemcpyDeviceToHost));
        STEP(cudaMemcpy(&hsah, sah, sizeof(float), cudaMemcpyDeviceToHost));
        if (hc[1] != n) {
            status = set_error(ctx, LGB_ERR_DEVICE_STATUS, "BVH collapse wrote an unexpected triangle count");
            goto cleanup;
        }
        // shrink the node array to its used size
        WideNode* tight = nullptr;
        STEP(dalloc(&tight, hc[0]));
        STEP(cudaMemcpyAsync(tight, nodes, sizeof(WideNode) * hc[0], cudaMemcpyDeviceToDevice, st));
        STEP(cudaEventRecord(e1, st));
        STEP(cudaEventSynchronize(e1));
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaFree(nodes);
        nodes = nullptr;
        if (s->bvh.nodes) cudaFree(s->bvh.nodes);
        if (s->bvh.tris) cudaFree(s->bvh.tris);
        s->bvh.nodes = tight;
        s->bvh.tris = tris;
        tris = nullptr;
        s->bvh.num_nodes = hc[0];
        s->bvh.num_tris = n;
        s->bvh.max_depth = depth;
        s->bvh.generation++;
        if (stats) {
            std::memset(stats, 0, sizeof(*stats));
            stats->build_ms = ms;
            stats->num_tris = n;
            stats->num_nodes = hc[0];
            stats->max_depth = depth;
            stats->node_bytes = (uint64_t)hc[0] * sizeof(WideNode);
            stats->tri_bytes = (uint64_t)n * sizeof(WideTri);
            stats->sah_cost = hsah;
        }
    }
cleanup:
#undef STEP
    cudaFree(keys); cudaFree(keys2); cudaFree(vals); cudaFree(vals2); cudaFree(counts); cudaFree(bounds);
    cudaFree(left); cudaFree(right); cudaFree(pint); cudaFree(pleaf); cudaFree(rlo); cudaFree(rhi); cudaFree(flags);
    cudaFree(tri_box); cudaFree(node_box); cudaFree(sah); cudaFree(qa); cudaFree(qb); cudaFree(counters);
    cudaFree(node_cost); cudaFree(node_count);
    if (nodes) cudaFree(nodes);
    if (tris) cudaFree(tris);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return status;
}

}  // namespace lgb
