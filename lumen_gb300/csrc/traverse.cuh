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
    float ix, iy, iz;  // inverse direction for box tests (zero components replaced by +-1e-20)
    uint32_t oct;      // bit a set when d_a >= 0
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
    r.ix = 1.0f / gx; r.iy = 1.0f / gy; r.iz = 1.0f / gz;
    r.oct = (dx >= 0.0f ? 1u : 0u) | (dy >= 0.0f ? 2u : 0u) | (dz >= 0.0f ? 4u : 0u);
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

__device__ __forceinline__ float qbyte(uint32_t lo4, uint32_t hi4, int i) {
    uint32_t w = i < 4 ? lo4 : hi4;
    return (float)((w >> (8 * (i & 3))) & 0xffu);
}

// Tests the 8 children of a node. Returns the hit mask of internal children placed at bit (slot ^ oct)
// (bits 0-7) and the triangle hit mask relative to tri_base (bits 0-23).
__device__ __forceinline__ void intersect_node(const RayQ& r, const WideNode* __restrict__ node, float tlim,
                                               uint32_t& child_base, uint32_t& imask, uint32_t& int_hits,
                                               uint32_t& tri_base, uint32_t& tri_hits) {
    const uint4 c0 = ldg4(reinterpret_cast<const char*>(node) + 0);
    const uint4 c1 = ldg4(reinterpret_cast<const char*>(node) + 16);
    const uint4 c2 = ldg4(reinterpret_cast<const char*>(node) + 32);
    const uint4 c3 = ldg4(reinterpret_cast<const char*>(node) + 48);
    const uint4 c4 = ldg4(reinterpret_cast<const char*>(node) + 64);
    const float px = __uint_as_float(c0.x), py = __uint_as_float(c0.y), pz = __uint_as_float(c0.z);
    const uint32_t e = c0.w;
    imask = e >> 24;
    child_base = c1.x;
    tri_base = c1.y;
    const uint32_t meta_lo = c1.z, meta_hi = c1.w;
    const float sx = __uint_as_float((e & 0xffu) << 23) * r.ix;
    const float sy = __uint_as_float(((e >> 8) & 0xffu) << 23) * r.iy;
    const float sz = __uint_as_float(((e >> 16) & 0xffu) << 23) * r.iz;
    const float ax = (px - r.ox) * r.ix;
    const float ay = (py - r.oy) * r.iy;
    const float az = (pz - r.oz) * r.iz;
    // near/far byte planes per axis
    const bool fx = r.ix >= 0.0f, fy = r.iy >= 0.0f, fz = r.iz >= 0.0f;
    const uint32_t nx0 = fx ? c2.x : c3.z, nx1 = fx ? c2.y : c3.w, fx0 = fx ? c3.z : c2.x, fx1 = fx ? c3.w : c2.y;
    const uint32_t ny0 = fy ? c2.z : c4.x, ny1 = fy ? c2.w : c4.y, fy0 = fy ? c4.x : c2.z, fy1 = fy ? c4.y : c2.w;
    const uint32_t nz0 = fz ? c3.x : c4.z, nz1 = fz ? c3.y : c4.w, fz0 = fz ? c4.z : c3.x, fz1 = fz ? c4.w : c3.y;
    uint32_t ih = 0, th = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const uint32_t meta = ((i < 4 ? meta_lo : meta_hi) >> (8 * (i & 3))) & 0xffu;
        const bool is_int = (imask >> i) & 1u;
        if (!is_int && meta == 0u) continue;
        const float tnx = fmaf(qbyte(nx0, nx1, i), sx, ax);
        const float tny = fmaf(qbyte(ny0, ny1, i), sy, ay);
        const float tnz = fmaf(qbyte(nz0, nz1, i), sz, az);
        const float tfx = fmaf(qbyte(fx0, fx1, i), sx, ax);
        const float tfy = fmaf(qbyte(fy0, fy1, i), sy, ay);
        const float tfz = fmaf(qbyte(fz0, fz1, i), sz, az);
        const float tn = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, r.tmin));
        const float tf = fminf(fminf(tfx, tfy), fminf(tfz, tlim));
        if (tn <= tf) {
            if (is_int) ih |= 1u << (i ^ r.oct);
            else th |= ((meta >> 5) & 7u) << (meta & 31u);
        }
    }
    int_hits = ih;
    tri_hits = th;
}

// Closest-hit traversal. Returns prim (LGB_NO_HIT on a miss). COUNT adds node and triangle fetches.
template <bool COUNT>
__device__ __forceinline__ uint32_t trace_closest_dev(const WideNode* __restrict__ nodes, const WideTri* __restrict__ tris,
                                                       const RayQ& r, float& t_best, float& u_best, float& v_best,
                                                       uint32_t* status, uint32_t& n_nodes, uint32_t& n_tris) {
    uint2 stack[kStackSize];
    int sp = 0;
    t_best = r.tmax;
    uint32_t best = LGB_NO_HIT;
    u_best = 0.0f; v_best = 0.0f;
    // virtual parent of the root: child_base 0, slot 0 internal
    uint32_t g_base = 0u, g_hits = 1u << (0u ^ r.oct), g_imask = 1u;
    uint32_t visits = 0;
    while (true) {
        while (g_hits) {
            const int pos = 31 - __clz(g_hits);
            g_hits &= ~(1u << pos);
            const uint32_t slot = (uint32_t)pos ^ r.oct;
            const uint32_t node_idx = g_base + __popc(g_imask & ((1u << slot) - 1u));
            if (++visits > kMaxVisits) { atomicOr(status, STATUS_VISIT_LIMIT); return best; }
            if (g_hits) {
                if (sp >= kStackSize) { atomicOr(status, STATUS_STACK_OVERFLOW); return best; }
                stack[sp++] = make_uint2(g_base, (g_hits << 8) | g_imask);
            }
            uint32_t tri_base, tri_hits;
            intersect_node(r, nodes + node_idx, t_best, g_base, g_imask, g_hits, tri_base, tri_hits);
            if (COUNT) n_nodes++;
            while (tri_hits) {
                const int k = __ffs(tri_hits) - 1;
                tri_hits &= tri_hits - 1u;
                const WideTri* tp = tris + tri_base + k;
                const float4 a = ldg4f(&tp->a), b = ldg4f(&tp->b), c = ldg4f(&tp->c);
                if (COUNT) n_tris++;
                float t, u, v;
                if (tri_intersect(r, a, b, c, t_best, t, u, v)) {
                    const uint32_t prim = __float_as_uint(a.w);
                    if (t < t_best || prim < best) {
                        t_best = t; best = prim; u_best = u; v_best = v;
                    }
                }
            }
        }
        if (sp == 0) break;
        const uint2 g = stack[--sp];
        g_base = g.x;
        g_hits = g.y >> 8;
        g_imask = g.y & 0xffu;
    }
    return best;
}

// Any-hit traversal: true on the first triangle hit in [tmin, tmax].
__device__ __forceinline__ bool trace_any_dev(const WideNode* __restrict__ nodes, const WideTri* __restrict__ tris,
                                              const RayQ& r, uint32_t* status) {
    uint2 stack[kStackSize];
    int sp = 0;
    uint32_t g_base = 0u, g_hits = 1u << (0u ^ r.oct), g_imask = 1u;
    uint32_t visits = 0;
    while (true) {
        while (g_hits) {
            const int pos = 31 - __clz(g_hits);
            g_hits &= ~(1u << pos);
            const uint32_t slot = (uint32_t)pos ^ r.oct;
            const uint32_t node_idx = g_base + __popc(g_imask & ((1u << slot) - 1u));
            if (++visits > kMaxVisits) { atomicOr(status, STATUS_VISIT_LIMIT); return false; }
            if (g_hits) {
                if (sp >= kStackSize) { atomicOr(status, STATUS_STACK_OVERFLOW); return false; }
                stack[sp++] = make_uint2(g_base, (g_hits << 8) | g_imask);
            }
            uint32_t tri_base, tri_hits;
            intersect_node(r, nodes + node_idx, r.tmax, g_base, g_imask, g_hits, tri_base, tri_hits);
            while (tri_hits) {
                const int k = __ffs(tri_hits) - 1;
                tri_hits &= tri_hits - 1u;
                const WideTri* tp = tris + tri_base + k;
                const float4 a = ldg4f(&tp->a), b = ldg4f(&tp->b), c = ldg4f(&tp->c);
                float t, u, v;
                if (tri_intersect(r, a, b, c, r.tmax, t, u, v)) return true;
            }
        }
        if (sp == 0) break;
        const uint2 g = stack[--sp];
        g_base = g.x;
        g_hits = g.y >> 8;
        g_imask = g.y & 0xffu;
    }
    return false;
}

}  // namespace lgb
