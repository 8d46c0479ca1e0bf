// Device-side ray queries over the 8-wide quantised BVH.
//
// Stands in for traceRayEXT (src/shaders/integrators/path/path.rgen:48, pt_commons.glsl:21,32) whose
// traversal runs in the Vulkan driver on RT cores. Contract:
//   closest: smallest watertight t in [tmin, tmax]; equal t -> lowest global primitive id
//   any:     true iff some triangle passes the watertight test with t in [tmin, tmax]
// The triangle test (Woop, Benthin and Wald, JCGT 2013) uses explicitly rounded FP32 intrinsics so that
// no multiply-add is fused and the result is bit-identical to the CPU oracle's FP32 sequence. Box tests
// may fuse freely: quantised boxes carry one step of outward margin, so pruning stays conservative.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "lgb_internal.cuh"

namespace lgb {

struct RayQ {
    float ox, oy, oz, tmin, tmax;
    float Sx, Sy, Sz;
    int kx, ky, kz;
    float ix, iy, iz;  // inverse direction for box tests (zero components replaced by +-1e-20), approximate
    uint32_t oct;      // bit a set when the guarded direction component a is positive
};

__device__ __forceinline__ float comp(float x, float y, float z, int k) { return k == 0 ? x : (k == 1 ? y : z); }

__device__ __forceinline__ RayQ make_rayq(float ox, float oy, float oz, float tmin, float dx, float dy, float dz,
                                          float tmax) {
    RayQ r;
    r.ox = ox; r.oy = oy; r.oz = oz; r.tmin = tmin; r.tmax = tmax;
    float ax = fabsf(dx), ay = fabsf(dy), az = fabsf(dz);
    int kz = 0;
    if (ay > ax) kz = 1;
    if (az > (kz == 0 ? ax : ay)) kz = 2;
    int kx = kz + 1; if (kx == 3) kx = 0;
    int ky = kx + 1; if (ky == 3) ky = 0;
    float dkz = comp(dx, dy, dz, kz);
    if (dkz < 0.0f) { int t = kx; kx = ky; ky = t; }
    r.kx = kx; r.ky = ky; r.kz = kz;
    r.Sx = __fdiv_rn(comp(dx, dy, dz, kx), dkz);
    r.Sy = __fdiv_rn(comp(dx, dy, dz, ky), dkz);
    r.Sz = __fdiv_rn(1.0f, dkz);
    const float tiny = 1e-20f;
    float gx = ax < tiny ? copysignf(tiny, dx) : dx;
    float gy = ay < tiny ? copysignf(tiny, dy) : dy;
    float gz = az < tiny ? copysignf(tiny, dz) : dz;
    // Box tests only: rcp.approx is within a few ulps, far inside the one quantisation step of outward margin of
    // every box (the triangle test above keeps IEEE divisions). |g| >= 1e-20, so no result is denormal.
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r.ix) : "f"(gx));
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r.iy) : "f"(gy));
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r.iz) : "f"(gz));
    // The octant follows the sign of the guarded inverse, so near/far plane selection always agrees with it.
    r.oct = (gx > 0.0f ? 1u : 0u) | (gy > 0.0f ? 2u : 0u) | (gz > 0.0f ? 4u : 0u);
    return r;
}

// Watertight test. Returns true with t, u, v (u weights v1, v weights v2) when t lies in [tmin, tlim].
__device__ __forceinline__ bool tri_intersect(const RayQ& r, float4 a, float4 b, float4 c, float tlim, float& t_out,
                                              float& u_out, float& v_out) {
    const float A0 = __fsub_rn(a.x, r.ox), A1 = __fsub_rn(a.y, r.oy), A2 = __fsub_rn(a.z, r.oz);
    const float B0 = __fsub_rn(b.x, r.ox), B1 = __fsub_rn(b.y, r.oy), B2 = __fsub_rn(b.z, r.oz);
    const float C0 = __fsub_rn(c.x, r.ox), C1 = __fsub_rn(c.y, r.oy), C2 = __fsub_rn(c.z, r.oz);
    const float Akx = comp(A0, A1, A2, r.kx), Aky = comp(A0, A1, A2, r.ky), Akz = comp(A0, A1, A2, r.kz);
    const float Bkx = comp(B0, B1, B2, r.kx), Bky = comp(B0, B1, B2, r.ky), Bkz = comp(B0, B1, B2, r.kz);
    const float Ckx = comp(C0, C1, C2, r.kx), Cky = comp(C0, C1, C2, r.ky), Ckz = comp(C0, C1, C2, r.kz);
    const float Ax = __fsub_rn(Akx, __fmul_rn(r.Sx, Akz));
    const float Ay = __fsub_rn(Aky, __fmul_rn(r.Sy, Akz));
    const float Bx = __fsub_rn(Bkx, __fmul_rn(r.Sx, Bkz));
    const float By = __fsub_rn(Bky, __fmul_rn(r.Sy, Bkz));
    const float Cx = __fsub_rn(Ckx, __fmul_rn(r.Sx, Ckz));
    const float Cy = __fsub_rn(Cky, __fmul_rn(r.Sy, Ckz));
    float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
    float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
    float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        // Edge case: the products of two FP32 values are exact in double, so the difference is rounded once.
        U = __double2float_rn(__dsub_rn(__dmul_rn((double)Cx, (double)By), __dmul_rn((double)Cy, (double)Bx)));
        V = __double2float_rn(__dsub_rn(__dmul_rn((double)Ax, (double)Cy), __dmul_rn((double)Ay, (double)Cx)));
        W = __double2float_rn(__dsub_rn(__dmul_rn((double)Bx, (double)Ay), __dmul_rn((double)By, (double)Ax)));
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = __fadd_rn(__fadd_rn(U, V), W);
    if (det == 0.0f) return false;
    const float Az = __fmul_rn(r.Sz, Akz);
    const float Bz = __fmul_rn(r.Sz, Bkz);
    const float Cz = __fmul_rn(r.Sz, Ckz);
    const float T = __fadd_rn(__fadd_rn(__fmul_rn(U, Az), __fmul_rn(V, Bz)), __fmul_rn(W, Cz));
    const float t = __fdiv_rn(T, det);
    if (!(t >= r.tmin && t <= tlim)) return false;
    t_out = t;
    u_out = __fdiv_rn(V, det);
    v_out = __fdiv_rn(W, det);
    return true;
}

__device__ __forceinline__ uint4 ldg4(const void* p) { return __ldg(reinterpret_cast<const uint4*>(p)); }
__device__ __forceinline__ float4 ldg4f(const void* p) { return __ldg(reinterpret_cast<const float4*>(p)); }

__device__ __forceinline__ float fmax3(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float fmin3(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// Packed FP32 pairs (Blackwell f32x2 datapath): one instruction handles two children.
__device__ __forceinline__ unsigned long long pk(float lo, float hi) {
    return ((unsigned long long)__float_as_uint(hi) << 32) | __float_as_uint(lo);
}
__device__ __forceinline__ float lo_f(unsigned long long v) { return __uint_as_float((uint32_t)v); }
__device__ __forceinline__ float hi_f(unsigned long long v) { return __uint_as_float((uint32_t)(v >> 32)); }
__device__ __forceinline__ unsigned long long fma2(unsigned long long a, unsigned long long b, unsigned long long c) {
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
// Bytes K and K+1 of w as the float pair (2^23 + byte): each byte goes under the exponent of 2^23 with one PRMT
// (cheaper than an integer-to-float conversion, which runs on a quarter-rate pipe).
template <int K> __device__ __forceinline__ unsigned long long byte_pair(uint32_t w) {
    const uint32_t a = __byte_perm(w, 0x4B000000u, 0x7440u | K);
    const uint32_t b = __byte_perm(w, 0x4B000000u, 0x7440u | (K + 1));
    return ((unsigned long long)b << 32) | a;
}

// Children K, K+1 (K even) of one 4-child half: their slab entry/exit distances and hit bits.
template <int I>
__device__ __forceinline__ uint32_t child_pair(const RayQ& r, float tlim, uint32_t nx, uint32_t ny, uint32_t nz,
                                               uint32_t fx, uint32_t fy, uint32_t fz, unsigned long long sx,
                                               unsigned long long sy, unsigned long long sz, unsigned long long ax,
                                               unsigned long long ay, unsigned long long az) {
    constexpr int K = I & 3;
    // The byte pairs are 2^23 + q; the node offsets ax/ay/az already subtract 2^23 steps (see intersect_node).
    const unsigned long long tnx = fma2(byte_pair<K>(nx), sx, ax);
    const unsigned long long tny = fma2(byte_pair<K>(ny), sy, ay);
    const unsigned long long tnz = fma2(byte_pair<K>(nz), sz, az);
    const unsigned long long tfx = fma2(byte_pair<K>(fx), sx, ax);
    const unsigned long long tfy = fma2(byte_pair<K>(fy), sy, ay);
    const unsigned long long tfz = fma2(byte_pair<K>(fz), sz, az);
    const float tn0 = fmaxf(fmax3(lo_f(tnx), lo_f(tny), lo_f(tnz)), r.tmin);
    const float tf0 = fminf(fmin3(lo_f(tfx), lo_f(tfy), lo_f(tfz)), tlim);
    const float tn1 = fmaxf(fmax3(hi_f(tnx), hi_f(tny), hi_f(tnz)), r.tmin);
    const float tf1 = fminf(fmin3(hi_f(tfx), hi_f(tfy), hi_f(tfz)), tlim);
    return (tn0 <= tf0 ? (1u << I) : 0u) | (tn1 <= tf1 ? (2u << I) : 0u);
}

// Tests the 8 children of a node. Internal-child hits go to bit (slot ^ oct) of int_hits (bits 0-7), leaf
// hits to tri_hits relative to tri_base (bits 0-23). Empty slots carry inverted boxes and meta 0, so they
// never contribute.
__device__ __forceinline__ void intersect_node(const RayQ& r, const WideNode* __restrict__ node, float tlim,
                                               uint32_t& child_base, uint32_t& imask, uint32_t& int_hits,
                                               uint32_t& tri_base, uint32_t& tri_hits) {
    const uint4 c0 = ldg4(reinterpret_cast<const char*>(node) + 0);
    const uint4 c1 = ldg4(reinterpret_cast<const char*>(node) + 16);
    const uint4 c2 = ldg4(reinterpret_cast<const char*>(node) + 32);
    const uint4 c3 = ldg4(reinterpret_cast<const char*>(node) + 48);
    const uint4 c4 = ldg4(reinterpret_cast<const char*>(node) + 64);
    const uint32_t e = c0.w;
    imask = e >> 24;
    child_base = c1.x;
    tri_base = c1.y;
    const float fsx = __uint_as_float((e & 0xffu) << 23) * r.ix;
    const float fsy = __uint_as_float(((e >> 8) & 0xffu) << 23) * r.iy;
    const float fsz = __uint_as_float(((e >> 16) & 0xffu) << 23) * r.iz;
    // Plane distance of byte q: (origin + q * step - o) * inv_dir = (2^23 + q) * fs + (fa - 2^23 * fs), so the
    // byte decode needs no bias subtraction. Rounding fa - 2^23 * fs once costs at most half a quantisation
    // step, inside the one step of outward margin every quantised box carries (+1.3 % closest-hit on GB300,
    // identical hits).
    const float fax = fmaf(-8388608.0f, fsx, (__uint_as_float(c0.x) - r.ox) * r.ix);
    const float fay = fmaf(-8388608.0f, fsy, (__uint_as_float(c0.y) - r.oy) * r.iy);
    const float faz = fmaf(-8388608.0f, fsz, (__uint_as_float(c0.z) - r.oz) * r.iz);
    const unsigned long long sx = pk(fsx, fsx), sy = pk(fsy, fsy), sz = pk(fsz, fsz);
    const unsigned long long ax = pk(fax, fax), ay = pk(fay, fay), az = pk(faz, faz);
    // near and far byte planes per axis: qlo is near for a positive direction component
    const bool px = r.oct & 1u, py = r.oct & 2u, pz = r.oct & 4u;
    const uint32_t nx0 = px ? c2.x : c3.z, nx1 = px ? c2.y : c3.w, fx0 = px ? c3.z : c2.x, fx1 = px ? c3.w : c2.y;
    const uint32_t ny0 = py ? c2.z : c4.x, ny1 = py ? c2.w : c4.y, fy0 = py ? c4.x : c2.z, fy1 = py ? c4.y : c2.w;
    const uint32_t nz0 = pz ? c3.x : c4.z, nz1 = pz ? c3.y : c4.w, fz0 = pz ? c4.z : c3.x, fz1 = pz ? c4.w : c3.y;
    const uint32_t hits = child_pair<0>(r, tlim, nx0, ny0, nz0, fx0, fy0, fz0, sx, sy, sz, ax, ay, az) |
                          child_pair<2>(r, tlim, nx0, ny0, nz0, fx0, fy0, fz0, sx, sy, sz, ax, ay, az) |
                          child_pair<4>(r, tlim, nx1, ny1, nz1, fx1, fy1, fz1, sx, sy, sz, ax, ay, az) |
                          child_pair<6>(r, tlim, nx1, ny1, nz1, fx1, fy1, fz1, sx, sy, sz, ax, ay, az);
    // internal hits, bit i moved to bit i ^ oct (front-to-back rank)
    uint32_t x = hits & imask;
    if (r.oct & 1u) x = ((x & 0x55u) << 1) | ((x >> 1) & 0x55u);
    if (r.oct & 2u) x = ((x & 0x33u) << 2) | ((x >> 2) & 0x33u);
    if (r.oct & 4u) x = ((x & 0x0Fu) << 4) | ((x >> 4) & 0x0Fu);
    int_hits = x;
    // leaf hits: unary triangle counts at their offsets
    uint32_t lh = hits & ~imask, th = 0;
    const unsigned long long meta = ((unsigned long long)c1.w << 32) | c1.z;
    while (lh) {
        const int i = __ffs(lh) - 1;
        lh &= lh - 1u;
        const uint32_t m = (uint32_t)(meta >> (8 * i)) & 0xffu;
        th |= ((m >> 5) & 7u) << (m & 31u);
    }
    tri_hits = th;
}

// Persistent ray queries. Every warp loops until the ray list is exhausted: lanes whose ray has finished take
// a new ray index from a global counter (one atomic per warp per refill), so short rays do not leave lanes
// idle while the longest ray of a warp finishes. POSTPONE = true: each loop iteration either tests one leaf
// triangle left by the previous node or visits one node, so lanes in different phases stay converged (incoherent
// rays). POSTPONE = false: a node's leaf triangles are tested in the iteration that visits it (short coherent
// rays, fewer loop trips). Both give the same hits.
//   ANY = false: closest hit into hits[id]; ANY = true: occlusion bit id of occ_bits (which must be zeroed).
//   COUNT adds the nodes and triangles fetched into counters[0..1].
//   SK > 0: the bottom SK stack entries of each thread live in shared memory (`sstack`, SK x THREADS entries,
//   slot-major so that a warp's lanes at different depths hit different banks); deeper entries stay in the
//   per-thread local array.
//   REFILL: a warp fetches new rays once at least REFILL of its lanes are idle (a warp whose lanes are all idle
//   always refills, so every ray is fetched and the loop ends); fewer, fuller refills cost fewer atomics.
// The ray count is read from *count_ptr when it is non-null, else n. A ray that visits more than max_visits nodes
// ends with what it has found so far and sets STATUS_VISIT_LIMIT.
//   TRI_MIN > 0 (with POSTPONE): every loop iteration of a warp is either a triangle iteration (the lanes with a
//   pending leaf triangle test one, the others wait) or a node iteration (the lanes without one visit a node, the
//   others wait), never both. A warp runs a triangle iteration once at least TRI_MIN of its lanes have a
//   pending triangle, or when every active lane has one. Each lane still tests and visits in its own order, so
//   hits are unchanged; what changes is that a warp no longer issues both code paths in one iteration.
//   TRI_MIN < 0: the same with a relative threshold, a triangle iteration once at least 1 / -TRI_MIN of the
//   active lanes have a pending triangle.
template <bool ANY, bool COUNT, bool POSTPONE = true, int SK = 0, int THREADS = 128, int REFILL = 1, int TRI_MIN = 0>
__device__ __forceinline__ void trace_persistent(const WideNode* __restrict__ nodes, const WideTri* __restrict__ tris,
                                                 const lgb_ray* __restrict__ rays, lgb_hit* __restrict__ hits,
                                                 uint32_t* __restrict__ occ_bits, uint32_t n, const uint32_t* count_ptr,
                                                 uint32_t* ray_counter, uint32_t* status,
                                                 unsigned long long* counters,
                                                 const uint32_t* __restrict__ roots = nullptr,
                                                 uint2* sstack = nullptr, uint32_t max_visits = kMaxVisits) {
    static_assert(SK >= 0 && SK < kStackSize, "shared stack entries");
    static_assert(REFILL >= 1 && REFILL <= 32, "refill threshold");
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const uint32_t lanemask_lt = (1u << lane) - 1u;
    if (count_ptr) n = *count_ptr;
    // A warp whose first thread's index is at or past the ray count could take no ray in its first fetch: it leaves
    // at once, so a short queue (a bounce's tail, the BSDF-MIS rays) costs its launch, not one atomic per warp.
    if (blockIdx.x * blockDim.x + (threadIdx.x & ~31u) >= n) return;
    RayQ r;
    uint2 stack[kStackSize - SK];
    uint2* const my_stack = SK > 0 ? sstack + threadIdx.x : nullptr;
    int sp = 0;
    uint32_t ray_id = 0, g_base = 0, g_hm = 0, best = LGB_NO_HIT, visits = 0;
    float t_best = 0.0f, u_best = 0.0f, v_best = 0.0f;
    uint32_t n_nodes = 0, n_tris = 0;
    uint32_t p_base = 0, p_hits = 0;  // leaf triangles of the last node visited that are still to be tested
    bool active = false, exhausted = false;
    while (true) {
        if (!exhausted) {
            const uint32_t need = __ballot_sync(FULL, !active);
            if (__popc(need) >= REFILL) {
                uint32_t base = 0;
                if (lane == 0) base = atomicAdd(ray_counter, (uint32_t)__popc(need));
                base = __shfl_sync(FULL, base, 0);
                if (base + (uint32_t)__popc(need) >= n) exhausted = true;
                if (!active) {
                    const uint32_t id = base + (uint32_t)__popc(need & lanemask_lt);
                    if (id < n) {
                        const float4 r0 = ldg4f(&rays[id].ox), r1 = ldg4f(&rays[id].dx);
                        r = make_rayq(r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w);
                        ray_id = id;
                        sp = 0;
                        g_base = roots ? roots[id] : 0u;  // per-ray root node when several BVHs share the arrays
                        // virtual parent of the root: slot 0 internal and hit; an empty interval visits nothing
                        g_hm = r.tmin <= r.tmax ? (((1u << (0u ^ r.oct)) << 8) | 1u) : 1u;
                        best = LGB_NO_HIT;
                        t_best = r.tmax;
                        u_best = v_best = 0.0f;
                        visits = 0;
                        p_hits = 0u;
                        active = true;
                    }
                }
            }
        }
        bool tri_phase = false;
        if (POSTPONE && TRI_MIN != 0) {
            const uint32_t act = __ballot_sync(FULL, active);
            if (act == 0u) break;
            const uint32_t tri = __ballot_sync(FULL, active && p_hits != 0u);
            const bool enough = TRI_MIN > 0 ? __popc(tri) >= TRI_MIN : __popc(tri) * (-TRI_MIN) >= __popc(act);
            tri_phase = tri != 0u && (enough || tri == act);
        } else if (!__any_sync(FULL, active)) {
            break;
        }
        const bool do_tri = POSTPONE && p_hits != 0u && (TRI_MIN == 0 || tri_phase);
        const bool do_node = !(POSTPONE && p_hits != 0u) && (TRI_MIN == 0 || !tri_phase);
        if (active && (do_tri || do_node)) {
            bool done = false, occluded = false;
            if (do_tri) {
                // One postponed leaf triangle per iteration: a lane whose node hit many leaf triangles no longer
                // holds its warp for all of them in one iteration (+9 % closest-hit on GB300). The triangles are
                // tested before the next node, in the same order as an inner loop would, so hits are identical.
                const int k = __ffs(p_hits) - 1;
                p_hits &= p_hits - 1u;
                const WideTri* tp = tris + p_base + k;
                const float4 a = ldg4f(&tp->a), b = ldg4f(&tp->b), c = ldg4f(&tp->c);
                if (COUNT) n_tris++;
                float t, u, v;
                if (tri_intersect(r, a, b, c, ANY ? r.tmax : t_best, t, u, v)) {
                    if (ANY) {
                        occluded = true;
                        done = true;
                    } else {
                        const uint32_t prim = __float_as_uint(a.w);
                        if (t < t_best || prim < best) {
                            t_best = t;
                            best = prim;
                            u_best = u;
                            v_best = v;
                        }
                    }
                }
            } else {
                uint32_t hm = g_hm >> 8;
                if (hm == 0u) {
                    if (sp == 0) {
                        done = true;
                    } else {
                        --sp;
                        uint2 g;
                        if (SK > 0 && sp < SK) {
                            g = my_stack[sp * THREADS];
                        } else {
                            g = stack[sp - SK];
                        }
                        g_base = g.x;
                        g_hm = g.y;
                        hm = g_hm >> 8;
                    }
                }
                if (!done) {
                    const uint32_t imask = g_hm & 0xffu;
                    const int pos = 31 - __clz(hm);
                    hm &= ~(1u << pos);
                    const uint32_t slot = (uint32_t)pos ^ r.oct;
                    const uint32_t node_idx = g_base + __popc(imask & ((1u << slot) - 1u));
                    if (hm) {
                        if (sp >= kStackSize) {
                            atomicOr(status, STATUS_STACK_OVERFLOW);
                            done = true;
                        } else {
                            const uint2 g = make_uint2(g_base, (hm << 8) | imask);
                            if (SK > 0 && sp < SK) {
                                my_stack[sp * THREADS] = g;
                            } else {
                                stack[sp - SK] = g;
                            }
                            ++sp;
                        }
                    }
                    if (++visits > max_visits) {
                        atomicOr(status, STATUS_VISIT_LIMIT);
                        done = true;
                    }
                    if (!done) {
                        uint32_t nb, nimask, nhits;
                        intersect_node(r, nodes + node_idx, ANY ? r.tmax : t_best, nb, nimask, nhits, p_base, p_hits);
                        if (COUNT) n_nodes++;
                        g_base = nb;
                        g_hm = (nhits << 8) | nimask;
                        if (!POSTPONE) {  // all of the node's leaf triangles in this iteration
                            while (p_hits) {
                                const int k = __ffs(p_hits) - 1;
                                p_hits &= p_hits - 1u;
                                const WideTri* tp = tris + p_base + k;
                                const float4 a = ldg4f(&tp->a), b = ldg4f(&tp->b), c = ldg4f(&tp->c);
                                if (COUNT) n_tris++;
                                float t, u, v;
                                if (tri_intersect(r, a, b, c, ANY ? r.tmax : t_best, t, u, v)) {
                                    if (ANY) {
                                        occluded = true;
                                        done = true;
                                        break;
                                    }
                                    const uint32_t prim = __float_as_uint(a.w);
                                    if (t < t_best || prim < best) {
                                        t_best = t;
                                        best = prim;
                                        u_best = u;
                                        v_best = v;
                                    }
                                }
                            }
                        }
                    }
                }
            }
            if (done) {
                if (ANY) {
                    if (occluded) atomicOr(&occ_bits[ray_id >> 5], 1u << (ray_id & 31u));
                } else {
                    uint4 out = make_uint4(best, __float_as_uint(best == LGB_NO_HIT ? 0.0f : t_best),
                                           __float_as_uint(u_best), __float_as_uint(v_best));
                    reinterpret_cast<uint4*>(hits)[ray_id] = out;
                }
                active = false;
            }
        }
    }
    if (COUNT) {
        unsigned long long a = n_nodes, b = n_tris;
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_xor_sync(FULL, a, o);
            b += __shfl_xor_sync(FULL, b, o);
        }
        if (lane == 0) {
            atomicAdd(&counters[0], a);
            atomicAdd(&counters[1], b);
        }
    }
}

// Single-ray queries for kernels that trace one ray per thread inside a larger loop (path-per-thread
// megakernels). Same node and triangle tests and the same closest/any contract as trace_persistent.
__device__ __forceinline__ uint32_t trace_closest_single(const WideNode* __restrict__ nodes, const WideTri* __restrict__ tris,
                                                         const RayQ& r, float& t_best, float& u_best, float& v_best,
                                                         uint32_t* status) {
    uint2 stack[kStackSize];
    int sp = 0;
    uint32_t best = LGB_NO_HIT, visits = 0;
    t_best = r.tmax;
    u_best = v_best = 0.0f;
    uint32_t g_base = 0u, g_hm = r.tmin <= r.tmax ? (((1u << (0u ^ r.oct)) << 8) | 1u) : 1u;
    while (true) {
        uint32_t hm = g_hm >> 8;
        if (hm == 0u) {
            if (sp == 0) break;
            const uint2 g = stack[--sp];
            g_base = g.x;
            g_hm = g.y;
            hm = g_hm >> 8;
        }
        const uint32_t imask = g_hm & 0xffu;
        const int pos = 31 - __clz(hm);
        hm &= ~(1u << pos);
        const uint32_t slot = (uint32_t)pos ^ r.oct;
        const uint32_t node_idx = g_base + __popc(imask & ((1u << slot) - 1u));
        if (hm) {
            if (sp >= kStackSize) { atomicOr(status, STATUS_STACK_OVERFLOW); break; }
            stack[sp++] = make_uint2(g_base, (hm << 8) | imask);
        } else {
            g_hm = imask;  // this group is exhausted
        }
        if (++visits > kMaxVisits) { atomicOr(status, STATUS_VISIT_LIMIT); break; }
        uint32_t nb, nimask, nhits, tri_base, tri_hits;
        intersect_node(r, nodes + node_idx, t_best, nb, nimask, nhits, tri_base, tri_hits);
        g_base = nb;
        g_hm = (nhits << 8) | nimask;
        while (tri_hits) {
            const int k = __ffs(tri_hits) - 1;
            tri_hits &= tri_hits - 1u;
            const WideTri* tp = tris + tri_base + k;
            const float4 a = ldg4f(&tp->a), b = ldg4f(&tp->b), c = ldg4f(&tp->c);
            float t, u, v;
            if (tri_intersect(r, a, b, c, t_best, t, u, v)) {
                const uint32_t prim = __float_as_uint(a.w);
                if (t < t_best || prim < best) { t_best = t; best = prim; u_best = u; v_best = v; }
            }
        }
    }
    return best;
}

__device__ __forceinline__ bool trace_any_single(const WideNode* __restrict__ nodes, const WideTri* __restrict__ tris,
                                                 const RayQ& r, uint32_t* status) {
    uint2 stack[kStackSize];
    int sp = 0;
    uint32_t visits = 0;
    uint32_t g_base = 0u, g_hm = r.tmin <= r.tmax ? (((1u << (0u ^ r.oct)) << 8) | 1u) : 1u;
    while (true) {
        uint32_t hm = g_hm >> 8;
        if (hm == 0u) {
            if (sp == 0) return false;
            const uint2 g = stack[--sp];
            g_base = g.x;
            g_hm = g.y;
            hm = g_hm >> 8;
        }
        const uint32_t imask = g_hm & 0xffu;
        const int pos = 31 - __clz(hm);
        hm &= ~(1u << pos);
        const uint32_t slot = (uint32_t)pos ^ r.oct;
        const uint32_t node_idx = g_base + __popc(imask & ((1u << slot) - 1u));
        if (hm) {
            if (sp >= kStackSize) { atomicOr(status, STATUS_STACK_OVERFLOW); return false; }
            stack[sp++] = make_uint2(g_base, (hm << 8) | imask);
        }
        if (++visits > kMaxVisits) { atomicOr(status, STATUS_VISIT_LIMIT); return false; }
        uint32_t nb, nimask, nhits, tri_base, tri_hits;
        intersect_node(r, nodes + node_idx, r.tmax, nb, nimask, nhits, tri_base, tri_hits);
        g_base = nb;
        g_hm = (nhits << 8) | nimask;
        while (tri_hits) {
            const int k = __ffs(tri_hits) - 1;
            tri_hits &= tri_hits - 1u;
            const WideTri* tp = tris + tri_base + k;
            const float4 a = ldg4f(&tp->a), b = ldg4f(&tp->b), c = ldg4f(&tp->c);
            float t, u, v;
            if (tri_intersect(r, a, b, c, r.tmax, t, u, v)) return true;
        }
    }
}

}  // namespace lgb
