// SPPM: stochastic progressive photon mapping, Lumen's SPPM integrator (src/RayTracer/SPPM.cpp:78-184).
//
//   k_sppm_eye       sppm_eye.rgen:44-127: per pixel, the path tracer's loop (emission, light sampling with the
//                    shadow and BSDF-MIS rays of pt_commons.glsl:3-42, BSDF sampling, Russian roulette) until the
//                    first diffuse hit, which becomes the pixel's visible point
//   k_sppm_bounds    min.comp / max.comp / reduce_*.comp / calc_bounds.comp: the bounds of the visible points
//                    grown by their radii, the largest radius, and the grid resolution from them
//   k_sppm_light     sppm_light.rgen:44-113: one light subpath per launch point; its hits from the second one on
//                    are photons
//   photon table     the hash table of sppm_light.rgen:86-93 built by sort and scan (photon_table.cuh): per slot
//                    the number of photons and the last one in photon order, deterministic
//   k_sppm_gather    gather.comp:43-86: every photon slot of the cells the pixel's radius covers
//   k_sppm_composite composite.comp:33-60: radius and flux update, progressive film
//
// Kept from the reference: pixel and light-path indices are column-major (x * height + y); the eye and light
// passes of a pixel share one RNG stream seed; the eye pass adds the sky for every escaping path, also after the
// visible point was recorded; a pixel with no diffuse hit this frame keeps its previous visible point; tau is
// reset after every composite, so each frame's flux stands alone; the bounds include pixels that never recorded
// a visible point (at the origin); a gathered slot counts its photon once per covered cell that hashes to it.
// Deviations: the seed is a parameter (the reference draws it with host rand()); the photon table keeps the
// last photon in photon order (the reference's last writer is whichever thread wrote last); a pixel whose
// cell range exceeds 16 cells per axis does not gather.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "bsdf_vcm.cuh"
#include "light_sample.cuh"
#include "path_common.cuh"
#include "photon_table.cuh"
#include "radix_sort.cuh"

namespace lgb {
namespace {
using namespace sh;

constexpr int kSppmThreads = 128;
constexpr int kMaxGatherCells = 16;
constexpr float kTMinS = 0.001f, kTMaxS = 10000.0f, kEpsS = 0.001f;  // sppm_eye.rgen:26-27, utils.glsl:8
constexpr int kRRMinDepthS = 3;                                      // sppm_eye.rgen:28
constexpr int kPointF4 = 8;   // visible point (SPPMData) = 8 x float4
constexpr int kPhotonF4 = 4;  // photon = 4 x float4

// SPPMData (sppm_commons.h:31-46) as 8 float4 per pixel:
//   0: p, radius   1: wo, N   2: n_s, uv.x   3: throughput, uv.y   4: col, M (int bits)
//   5: phi, material (bits)   6: tau, path_len (bits)   7: side (bits)
// Photon (PhotonHash, sppm_commons.h:48-55, one per light subpath and bounce) as 4 float4:
//   0: pos, path_len (bits, 0 = no photon)   1: wi   2: throughput   3: n_s
struct SppmArgs {
    float iv[16], ip[16];
    uint32_t W, H, screen;
    float sky[3];
    int max_depth;
    LightSet lights;
    float base_radius;
    uint32_t seed_frame;  // frame_num ^ seed
    uint32_t frame_num;
    float4* vp;           // screen * kPointF4
    float4* photons;      // screen * max_depth * kPhotonF4
    float* bounds;        // min xyz, max xyz, max radius
    int* grid_res;        // 3
    const uint32_t* g_count;
    const uint32_t* g_rep;
    float4* film;         // RGBA32F, row-major
};

// sample_light_Li (commons.glsl:224-300) as the path tracer's light sampling uses it: the light and triangle,
// the direction and distance to the sampled point, its solid-angle and area pdfs.
struct LiSample {
    v3 Le, wi;
    float wi_len, pdf_w, pdf_a;
    uint32_t flags, prim, lio, lvo;  // sampled triangle (area lights) and where its indices are
};
__device__ LiSample sample_light_Li_pt(const SceneView& S, const LightSet& Ls, float q0, float q1, float q2, float q3,
                                       v3 p) {
    LiSample r;
    const uint32_t li = (uint32_t)(q0 * (float)Ls.num_lights);
    const lgb_light* L = &S.lights[li];
    r.flags = L->light_flags;
    r.prim = LGB_NO_HIT;
    r.lio = r.lvo = 0u;
    r.Le = V3(0.0f); r.wi = V3(0.0f); r.wi_len = 0.0f; r.pdf_w = 0.0f; r.pdf_a = 0.0f;
    const uint32_t type = L->light_flags & 7u;
    if (type == LGB_LIGHT_AREA) {
        const lgb_mesh pm = S.meshes[L->prim_mesh_idx];
        const uint32_t tri = (uint32_t)(q1 * (float)L->num_triangles);
        r.prim = S.mesh_first[L->prim_mesh_idx] + tri;
        r.lio = pm.index_offset + 3u * tri;
        r.lvo = pm.vertex_offset;
        v3 lpos, ln;
        float tri_pdf;
        sample_tri(S, pm, tri, q2, q3, lpos, ln, tri_pdf);
        const lgb_material* lm = &S.mats[pm.material_index];
        r.Le = V3(lm->emissive_factor[0], lm->emissive_factor[1], lm->emissive_factor[2]);
        v3 wi = lpos - p;
        const float l2 = dot(wi, wi);
        r.wi_len = sqrtf(l2);
        r.wi = wi / r.wi_len;
        const float cfl = fabsf(dot(ln, -r.wi));
        r.pdf_a = tri_pdf;
        r.pdf_w = tri_pdf * l2 / cfl;
    } else if (type == LGB_LIGHT_SPOT) {
        const v3 lp = V3(L->pos[0], L->pos[1], L->pos[2]);
        v3 wi = lp - p;
        const float l2 = dot(wi, wi);
        r.wi_len = sqrtf(l2);
        r.wi = wi / r.wi_len;
        const v3 ldir = normalize(V3(L->to[0], L->to[1], L->to[2]) - lp);
        const float cfl = dot(-r.wi, ldir);
        const float cw = Ls.spot_cos_width, cf = Ls.spot_cos_falloff;
        float fall;
        if (cfl < cw) fall = 0.0f;
        else if (cfl >= cf) fall = 1.0f;
        else { const float d = (cfl - cw) / (cf - cw); fall = (d * d) * (d * d); }
        r.pdf_a = 1.0f;
        r.pdf_w = l2;
        r.Le = V3(L->L[0], L->L[1], L->L[2]) * fall;
    }
    return r;
}

// uniform_sample_light (pt_commons.glsl:3-42): light sample with its shadow ray, and for area lights the BSDF
// sample whose ray must hit the sampled triangle (a miss keeps the shading point's payload, ray.rmiss:13). A
// BSDF-MIS ray that fails the watertight test against the sampled triangle cannot count and is not traced.
__device__ v3 uniform_sample_light(const SceneView& S, const LightSet& Ls, uint4& seed, const Mat& m, v3 pos,
                                   bool side, v3 n_s, v3 wo, uint32_t prim, v3 payload_ns) {
    const float q0 = rnd(seed), q1 = rnd(seed), q2 = rnd(seed), q3 = rnd(seed);
    const LiSample ls = sample_light_Li_pt(S, Ls, q0, q1, q2, q3, pos);
    const v3 p = offset_ray2(pos, n_s);
    float bsdf_pdf;
    const float cos_x = dot(n_s, ls.wi);
    const v3 f = eval_bsdf(n_s, wo, m, side, ls.wi, bsdf_pdf);
    v3 res = V3(0.0f);
    const RayQ sq = make_rayq(p.x, p.y, p.z, 0.0f, ls.wi.x, ls.wi.y, ls.wi.z, ls.wi_len - kEpsS);
    const bool visible = !trace_any_single(S.nodes, S.tris, sq, S.status);
    if (visible && ls.pdf_w > 0.0f) {
        const float mis = ((ls.flags >> 5) & 1u) ? 1.0f : 1.0f / (1.0f + bsdf_pdf / ls.pdf_w);
        res = res + mis * f * fabsf(cos_x) * ls.Le / ls.pdf_w;
    }
    if ((ls.flags & 7u) == LGB_LIGHT_AREA) {
        const float b0 = rnd(seed), b1 = rnd(seed), b2 = rnd(seed);
        v3 wi2;
        float pdf2, cos2;
        const v3 f2 = sample_bsdf(n_s, wo, m, side, wi2, pdf2, cos2, V3(b0, b1, b2));
        if (pdf2 != 0.0f) {
            const RayQ mq = make_rayq(p.x, p.y, p.z, kTMinS, wi2.x, wi2.y, wi2.z, kTMaxS);
            bool may_count = true;
            if (ls.prim != prim) {
                const DevVertex a = S.verts[S.idx[ls.lio] + ls.lvo];
                const DevVertex b = S.verts[S.idx[ls.lio + 1] + ls.lvo];
                const DevVertex c = S.verts[S.idx[ls.lio + 2] + ls.lvo];
                float tt, tu, tv;
                may_count = tri_intersect(mq, make_float4(a.px, a.py, a.pz, 0.0f), make_float4(b.px, b.py, b.pz, 0.0f),
                                          make_float4(c.px, c.py, c.pz, 0.0f), mq.tmax, tt, tu, tv);
            }
            if (may_count) {
                float t, bu, bv;
                const uint32_t mprim = trace_closest_single(S.nodes, S.tris, mq, t, bu, bv, S.status);
                const uint32_t pl_prim = mprim == LGB_NO_HIT ? prim : mprim;
                if (pl_prim == ls.prim) {
                    v3 pl_pos = pos, pl_ns = payload_ns;
                    if (mprim != LGB_NO_HIT) {
                        const HitAttr mh = resolve_hit(S, mprim, bu, bv);
                        pl_pos = mh.pos;
                        pl_ns = mh.n_s;
                    }
                    const float wl = length(pl_pos - pos);
                    const float g = fabsf(dot(pl_ns, -wi2)) / (wl * wl);
                    const float mis = 1.0f / (1.0f + ls.pdf_a / (g * pdf2));
                    res = res + f2 * mis * fabsf(cos2) * ls.Le / pdf2;
                }
            }
        }
    }
    return res;
}

__device__ __forceinline__ uint32_t fbits(float x) { return __float_as_uint(x); }
__device__ __forceinline__ bool all_zero(v3 a) { return a.x == 0.0f && a.y == 0.0f && a.z == 0.0f; }  // f == vec3(0)
__device__ __forceinline__ float bitsf(uint32_t x) { return __uint_as_float(x); }

// sppm_eye.rgen:44-127
__global__ void __launch_bounds__(kSppmThreads) k_sppm_eye(SceneView S, SppmArgs A) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < A.screen; i += gridDim.x * blockDim.x) {
        const uint32_t x = i / A.H, y = i % A.H;
        float4* vp = A.vp + (size_t)i * kPointF4;
        uint4 seed = make_uint4(x, y, A.seed_frame, 0u);
        const float px = (float)x + 0.5f, py = (float)y + 0.5f;
        const float u = px / (float)A.W, v = py / (float)A.H;
        const float dx = u * 2.0f - 1.0f, dy = v * 2.0f - 1.0f;
        const float4 o4 = mat_vec(A.iv, 0.0f, 0.0f, 0.0f, 1.0f);
        const float4 t4 = mat_vec(A.ip, dx, dy, 1.0f, 1.0f);
        const v3 tn = normalize(V3(t4.x, t4.y, t4.z));
        const float4 d4 = mat_vec(A.iv, tn.x, tn.y, tn.z, 0.0f);
        v3 origin = V3(o4.x, o4.y, o4.z), dir = V3(d4.x, d4.y, d4.z);
        v3 T = V3(1.0f), col = f3(vp[4]);
        bool specular = false, recorded = false;
        for (int d = 0;; d++) {
            float t, bu, bv;
            const RayQ q = make_rayq(origin.x, origin.y, origin.z, kTMinS, dir.x, dir.y, dir.z, kTMaxS);
            const uint32_t prim = trace_closest_single(S.nodes, S.tris, q, t, bu, bv, S.status);
            if (prim == LGB_NO_HIT) {
                col = col + T * V3(A.sky[0], A.sky[1], A.sky[2]);
                break;
            }
            if (d >= A.max_depth - 1) break;
            const HitAttr h = resolve_hit(S, prim, bu, bv);
            const Mat m = load_material(S, h.mat, h.u, h.v);
            if (d == 0 || (specular && !recorded)) col = col + T * m.emissive;
            const v3 wo = -dir;
            v3 n_s = h.n_s, n_g = h.n_g;
            bool side = true;
            if (dot(h.n_g, wo) < 0.0f) n_g = -n_g;
            if (dot(n_g, h.n_s) < 0.0f) { n_s = -n_s; side = false; }
            origin = offset_ray(h.pos, n_g);
            specular = (m.props & LGB_FLAG_SPECULAR) != 0u;
            if (!recorded && !specular) {
                const float light_pick_pdf = 1.0f / (float)A.lights.light_tri_count;
                col = col + T * uniform_sample_light(S, A.lights, seed, m, h.pos, side, n_s, wo, prim, h.n_s) /
                                light_pick_pdf;
            }
            if (!recorded && (m.type & LGB_BSDF_DIFFUSE) != 0u) {
                recorded = true;
                vp[0] = make_float4(h.pos.x, h.pos.y, h.pos.z, vp[0].w);
                vp[1] = make_float4(wo.x, wo.y, wo.z, vp[1].w);
                vp[2] = make_float4(n_s.x, n_s.y, n_s.z, h.u);
                vp[3] = make_float4(T.x, T.y, T.z, h.v);
                const float4 v5 = vp[5];
                vp[5] = make_float4(v5.x, v5.y, v5.z, bitsf(h.mat));
                const float4 v6 = vp[6];
                vp[6] = make_float4(v6.x, v6.y, v6.z, bitsf((uint32_t)d));
                vp[7] = make_float4(bitsf(side ? 1u : 0u), 0.0f, 0.0f, 0.0f);
            }
            float pdf, cos_t;
            const float c0 = rnd(seed), c1 = rnd(seed), c2 = rnd(seed);
            const v3 f = sample_bsdf(n_s, wo, m, side, dir, pdf, cos_t, V3(c0, c1, c2));
            if (pdf < 1e-20f || dot(f, f) < 1e-20f) break;
            T = T * (f * fabsf(cos_t) / pdf);
            if (d > kRRMinDepthS) {
                const float rr = luminance(T);
                if (rr < rnd(seed)) break;
                T = T / rr;
            }
        }
        const float4 v4 = vp[4];
        vp[4] = make_float4(col.x, col.y, col.z, v4.w);
        if (A.frame_num == 0u) {
            const float4 v0 = vp[0];
            vp[0] = make_float4(v0.x, v0.y, v0.z, A.base_radius);
        }
    }
}

// Order-preserving float <-> uint map for atomicMax / atomicMin on floats (NaN-free inputs).
__device__ __forceinline__ uint32_t ordered(float f) {
    const uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float unordered(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// min.comp / max.comp and their reductions: min of p - radius, max of p + radius over every pixel, and the
// largest radius, into ob[0..2], ob[3..5], ob[6] as ordered integers (ob initialised to the identities). Max and
// min are exact, so the result does not depend on the reduction order.
__global__ void __launch_bounds__(256) k_sppm_bounds(SppmArgs A, uint32_t* ob) {
    uint32_t mn[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, mx[4] = {0u, 0u, 0u, 0u};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < A.screen; i += gridDim.x * blockDim.x) {
        const float4 p = A.vp[(size_t)i * kPointF4];
        const float lo[3] = {p.x - p.w, p.y - p.w, p.z - p.w}, hi[3] = {p.x + p.w, p.y + p.w, p.z + p.w};
        for (int k = 0; k < 3; k++) {
            mn[k] = min(mn[k], ordered(lo[k]));
            mx[k] = max(mx[k], ordered(hi[k]));
        }
        mx[3] = max(mx[3], ordered(p.w));
    }
    for (int k = 0; k < 3; k++) {
        mn[k] = __reduce_min_sync(0xffffffffu, mn[k]);
        mx[k] = __reduce_max_sync(0xffffffffu, mx[k]);
    }
    mx[3] = __reduce_max_sync(0xffffffffu, mx[3]);
    if ((threadIdx.x & 31) == 0) {
        for (int k = 0; k < 3; k++) {
            atomicMin(&ob[k], mn[k]);
            atomicMax(&ob[3 + k], mx[k]);
        }
        atomicMax(&ob[6], mx[3]);
    }
}

// calc_bounds.comp: the grid resolution from the bounds and the largest radius (0 when either is degenerate).
__global__ void k_sppm_grid(SppmArgs A, const uint32_t* ob) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    float b[7];
    for (int k = 0; k < 7; k++) b[k] = unordered(ob[k]);
    for (int k = 0; k < 7; k++) A.bounds[k] = b[k];
    const float max_radius = b[6];
    const float d[3] = {b[3] - b[0], b[4] - b[1], b[5] - b[2]};
    const float max_comp = fmaxf(d[0], fmaxf(d[1], d[2]));
    const int base = __float2int_rz(max_comp / max_radius);
    for (int k = 0; k < 3; k++)
        A.grid_res[k] = (max_comp > 0.0f && max_radius > 0.0f) ? max(__float2int_rz((float)base * d[k] / max_comp), 1) : 0;
}

// sppm_light.rgen:44-113
__global__ void __launch_bounds__(kSppmThreads) k_sppm_light(SceneView S, SppmArgs A) {
    const uint32_t per = (uint32_t)A.max_depth;
    for (uint32_t li = blockIdx.x * blockDim.x + threadIdx.x; li < A.screen; li += gridDim.x * blockDim.x) {
        const uint32_t x = li / A.H, y = li % A.H;
        float4* ph = A.photons + (size_t)li * per * kPhotonF4;
        for (uint32_t k = 0; k < per; k++) ph[(size_t)k * kPhotonF4] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        uint4 seed = make_uint4(x, y, A.seed_frame, 0u);
        const float r0 = rnd(seed), r1 = rnd(seed), r2 = rnd(seed), r3 = rnd(seed);
        const float d0 = rnd(seed), d1 = rnd(seed);
        const Emission e = sample_light_Le(S, A.lights, r0, r1, r2, r3, d0, d1);
        const float abs_cos_light = fabsf(dot(e.n, e.wi));
        v3 thr = (abs_cos_light == 0.0f || e.pdf_dir_w <= 0.0f)
                     ? V3(0.0f)
                     : e.L * abs_cos_light / (e.pdf_dir_w * e.pdf_pos_a);
        v3 pos = e.pos, wi = e.wi;
        for (int d = 0; d < A.max_depth; d++) {
            float t, bu, bv;
            const RayQ q = make_rayq(pos.x, pos.y, pos.z, kTMinS, wi.x, wi.y, wi.z, kTMaxS);
            const uint32_t prim = trace_closest_single(S.nodes, S.tris, q, t, bu, bv, S.status);
            if (prim == LGB_NO_HIT) break;
            const HitAttr h = resolve_hit(S, prim, bu, bv);
            const v3 wo = -wi;
            v3 n_s = h.n_s, n_g = h.n_g;
            bool side = true;
            if (dot(h.n_g, wo) < 0.0f) n_g = -n_g;
            if (dot(n_g, h.n_s) < 0.0f) { n_s = -n_s; side = false; }
            const Mat m = load_material(S, h.mat, h.u, h.v);
            if (d > 0) {  // the first hit is left to the eye pass's light sampling
                float4* p = ph + (size_t)d * kPhotonF4;
                p[0] = make_float4(h.pos.x, h.pos.y, h.pos.z, bitsf((uint32_t)d + 1u));
                p[1] = make_float4(wo.x, wo.y, wo.z, 0.0f);
                p[2] = make_float4(thr.x, thr.y, thr.z, 0.0f);
                p[3] = make_float4(n_s.x, n_s.y, n_s.z, 0.0f);
            }
            pos = offset_ray(h.pos, n_g);
            float pdf_dir, cos_t;
            const float c0 = rnd(seed), c1 = rnd(seed), c2 = rnd(seed);
            const v3 f = sample_bsdf_mode(n_s, wo, m, 0u, side, wi, pdf_dir, cos_t, V3(c0, c1, c2));
            thr = thr * (f * fabsf(cos_t) / pdf_dir);
            if (all_zero(f) || pdf_dir == 0.0f) break;
            if (d > kRRMinDepthS) {
                const float rr = fminf(0.95f, luminance(thr));
                if (rr < rnd(seed)) break;
                thr = thr / rr;
            }
        }
    }
}

// Table keys: the hash slot of every photon slot that holds a photon, the table size for the others.
__global__ void k_sppm_keys(SppmArgs A, uint32_t table, uint32_t* keys, uint32_t* vals) {
    const uint32_t n = A.screen * (uint32_t)A.max_depth;
    const float mn[3] = {A.bounds[0], A.bounds[1], A.bounds[2]}, mx[3] = {A.bounds[3], A.bounds[4], A.bounds[5]};
    const int res[3] = {A.grid_res[0], A.grid_res[1], A.grid_res[2]};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 p = A.photons[(size_t)i * kPhotonF4];
        keys[i] = __float_as_uint(p.w) == 0u ? table : grid_hash(grid_idx(V3(p.x, p.y, p.z), mn, mx, res), A.screen);
        vals[i] = i;
    }
}

// gather.comp:43-86
__global__ void __launch_bounds__(kSppmThreads) k_sppm_gather(SceneView S, SppmArgs A) {
    const float mn[3] = {A.bounds[0], A.bounds[1], A.bounds[2]}, mx[3] = {A.bounds[3], A.bounds[4], A.bounds[5]};
    const int res[3] = {A.grid_res[0], A.grid_res[1], A.grid_res[2]};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < A.screen; i += gridDim.x * blockDim.x) {
        float4* vp = A.vp + (size_t)i * kPointF4;
        const float4 v0 = vp[0];
        const v3 p = V3(v0.x, v0.y, v0.z);
        float r = v0.w;
        if (r < kEpsS) r = kEpsS;
        const float r_sqr = r * r;
        const int3 lo = grid_idx(p - V3(r), mn, mx, res);
        const int3 hi = grid_idx(p + V3(r), mn, mx, res);
        if ((long long)hi.x - lo.x >= kMaxGatherCells || (long long)hi.y - lo.y >= kMaxGatherCells ||
            (long long)hi.z - lo.z >= kMaxGatherCells)
            continue;
        const float4 v1 = vp[1], v2 = vp[2], v3_ = vp[3], v5 = vp[5], v6 = vp[6], v7 = vp[7];
        const v3 wo = V3(v1.x, v1.y, v1.z), n_s = V3(v2.x, v2.y, v2.z), vthr = V3(v3_.x, v3_.y, v3_.z);
        const uint32_t mat_idx = fbits(v5.w), vlen = fbits(v6.w);
        const bool side = fbits(v7.x) == 1u;
        v3 phi = V3(v5.x, v5.y, v5.z);
        int M = (int)fbits(vp[4].w);
        for (int cx = lo.x; cx <= hi.x; cx++)
            for (int cy = lo.y; cy <= hi.y; cy++)
                for (int cz = lo.z; cz <= hi.z; cz++) {
                    const uint32_t h = grid_hash(make_int3(cx, cy, cz), A.screen);
                    const uint32_t cnt = A.g_count[h];
                    if (cnt == 0u) continue;
                    const float4* ph = A.photons + (size_t)A.g_rep[h] * kPhotonF4;
                    const float4 p0 = ph[0];
                    const v3 pp = p - V3(p0.x, p0.y, p0.z);
                    const float dist_sqr = dot(pp, pp);
                    if (dist_sqr > r_sqr) continue;
                    if (A.max_depth < (int)(fbits(p0.w) + vlen + 1u)) continue;
                    const Mat m = load_material(S, mat_idx, v2.w, v3_.w);
                    const float4 p1 = ph[1], p2 = ph[2];
                    float pdf;
                    const v3 f = eval_bsdf(n_s, wo, m, side, V3(p1.x, p1.y, p1.z), pdf);
                    phi = phi + (float)cnt * V3(p2.x, p2.y, p2.z) * f * vthr;
                    M += 1;
                }
        vp[5] = make_float4(phi.x, phi.y, phi.z, v5.w);
        const float4 v4 = vp[4];
        vp[4] = make_float4(v4.x, v4.y, v4.z, bitsf((uint32_t)M));
    }
}

// composite.comp:33-60
__global__ void __launch_bounds__(256) k_sppm_composite(SppmArgs A) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < A.screen; i += gridDim.x * blockDim.x) {
        float4* vp = A.vp + (size_t)i * kPointF4;
        const uint32_t x = i / A.H, y = i % A.H;
        const float4 v0 = vp[0], v1 = vp[1], v4 = vp[4], v5 = vp[5], v6 = vp[6];
        v3 col = V3(v4.x, v4.y, v4.z);
        const int M = (int)fbits(v4.w);
        if (M > 0) {
            const float gamma = 2.0f / 3.0f;
            const float N = v1.w, radius = v0.w;
            const float n_new = N + gamma * (float)M;
            const float r_new = radius * sqrtf(n_new / (N + (float)M));
            const v3 tau = (V3(v6.x, v6.y, v6.z) + V3(v5.x, v5.y, v5.z)) * r_new * r_new / (radius * radius);
            vp[1] = make_float4(v1.x, v1.y, v1.z, n_new);
            vp[0] = make_float4(v0.x, v0.y, v0.z, r_new);
            vp[5] = make_float4(0.0f, 0.0f, 0.0f, v5.w);  // phi = 0
            col = col + tau / ((float)A.screen * LGB_PI * r_new * r_new);
        }
        vp[4] = make_float4(0.0f, 0.0f, 0.0f, bitsf(0u));  // col = 0 and, after a gather, M = 0
        vp[6] = make_float4(0.0f, 0.0f, 0.0f, v6.w);         // tau = 0
        float4& px = A.film[(size_t)y * A.W + x];
        if (A.frame_num > 0u) {
            const float w = 1.0f / (float)(A.frame_num + 1u);
            const float4 old = px;
            px = make_float4(mixf(old.x, col.x, w), mixf(old.y, col.y, w), mixf(old.z, col.z, w), 1.0f);
        } else {
            px = make_float4(col.x, col.y, col.z, 1.0f);
        }
    }
}

size_t align256s(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

lgb_status sppm_iteration(Scene* s, const lgb_camera* cam, const lgb_sppm_params* p, float* d_film, cudaStream_t st) {
    Ctx* ctx = s->ctx;
    const uint64_t screen64 = (uint64_t)cam->width * cam->height;
    const uint32_t per = (uint32_t)p->max_depth;
    if (screen64 * per >= 0x80000000ull || screen64 * 10u >= 0x80000000ull)
        return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "width * height * max_depth must stay below 2^31");
    const uint32_t screen = (uint32_t)screen64, nph = screen * per, table = 10u * screen;
    size_t off = 0;
    auto take = [&](size_t bytes) { const size_t o = off; off += align256s(bytes); return o; };
    const size_t o_vp = take(sizeof(float4) * kPointF4 * (size_t)screen);
    const size_t o_ph = take(sizeof(float4) * kPhotonF4 * (size_t)nph);
    const size_t o_gc = take(4ull * table), o_gr = take(4ull * table);
    const size_t o_k0 = take(4ull * nph), o_k1 = take(4ull * nph), o_v0 = take(4ull * nph), o_v1 = take(4ull * nph);
    const size_t o_sc = take(4ull * radix_sort_scratch_words(nph));
    const size_t o_bd = take(4ull * 8), o_ob = take(4ull * 8), o_gres = take(4ull * 4);
    const bool fresh = !s->sppm_buf || s->sppm_w != cam->width || s->sppm_h != cam->height || s->sppm_depth != per ||
                       s->sppm_buf_bytes < off;
    if (fresh) {
        cudaFree(s->sppm_buf);
        s->sppm_buf = nullptr;
        s->sppm_buf_bytes = 0;
        LGB_CUDA_TRY(ctx, cudaMalloc(&s->sppm_buf, off));
        s->sppm_buf_bytes = off;
        s->sppm_w = cam->width; s->sppm_h = cam->height; s->sppm_depth = per;
    }
    char* base = (char*)s->sppm_buf;
    // SPPM.cpp:149: the visible points are cleared at frame 0 (and whenever the buffers are new)
    if (fresh || p->frame_num == 0u) LGB_CUDA_TRY(ctx, cudaMemsetAsync(base + o_vp, 0, sizeof(float4) * kPointF4 * (size_t)screen, st));
    SppmArgs A;
    std::memset(&A, 0, sizeof(A));
    for (int i = 0; i < 16; i++) { A.iv[i] = cam->inv_view[i]; A.ip[i] = cam->inv_projection[i]; }
    A.W = cam->width; A.H = cam->height; A.screen = screen;
    for (int k = 0; k < 3; k++) A.sky[k] = p->sky_col[k];
    A.max_depth = p->max_depth;
    A.lights.num_lights = p->num_lights;
    A.lights.light_tri_count = p->light_triangle_count;
    spot_cone(p->spot_angle, A.lights.spot_cos_width, A.lights.spot_cos_falloff);
    A.base_radius = std::max(p->base_radius, 1e-7f);  // SPPM.cpp:87-89
    A.seed_frame = p->frame_num ^ p->seed;
    A.frame_num = p->frame_num;
    A.vp = reinterpret_cast<float4*>(base + o_vp);
    A.photons = reinterpret_cast<float4*>(base + o_ph);
    A.bounds = reinterpret_cast<float*>(base + o_bd);
    A.grid_res = reinterpret_cast<int*>(base + o_gres);
    uint32_t* gc = reinterpret_cast<uint32_t*>(base + o_gc);
    uint32_t* gr = reinterpret_cast<uint32_t*>(base + o_gr);
    A.g_count = gc;
    A.g_rep = gr;
    A.film = reinterpret_cast<float4*>(d_film);
    const SceneView S = scene_view(s);
    const int sms = ctx->sm_count > 0 ? ctx->sm_count : 1;
    const int grid = (int)std::min<uint32_t>((screen + kSppmThreads - 1) / kSppmThreads, (uint32_t)sms * 16u);
    k_sppm_eye<<<grid, kSppmThreads, 0, st>>>(S, A);
    uint32_t* ob = reinterpret_cast<uint32_t*>(base + o_ob);
    const uint32_t init[8] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u, 0u, 0u};
    LGB_CUDA_TRY(ctx, cudaMemcpyAsync(ob, init, sizeof(init), cudaMemcpyHostToDevice, st));
    k_sppm_bounds<<<(int)std::min<uint32_t>((screen + 255) / 256, (uint32_t)sms * 8u), 256, 0, st>>>(A, ob);
    k_sppm_grid<<<1, 32, 0, st>>>(A, ob);
    k_sppm_light<<<grid, kSppmThreads, 0, st>>>(S, A);
    uint32_t* k0 = reinterpret_cast<uint32_t*>(base + o_k0);
    uint32_t* k1 = reinterpret_cast<uint32_t*>(base + o_k1);
    uint32_t* v0 = reinterpret_cast<uint32_t*>(base + o_v0);
    uint32_t* v1 = reinterpret_cast<uint32_t*>(base + o_v1);
    k_sppm_keys<<<table_grid_blocks(ctx, nph), 256, 0, st>>>(A, table, k0, v0);
    LGB_CUDA_TRY(ctx, cudaGetLastError());
    const lgb_status ts = build_table(ctx, k0, v0, k1, v1, reinterpret_cast<uint32_t*>(base + o_sc), nph, table, gc, gr, st);
    if (ts != LGB_OK) return ts;
    k_sppm_gather<<<grid, kSppmThreads, 0, st>>>(S, A);
    k_sppm_composite<<<(int)std::min<uint32_t>((screen + 255) / 256, (uint32_t)sms * 8u), 256, 0, st>>>(A);
    LGB_CUDA_TRY(ctx, cudaGetLastError());
    return LGB_OK;
}

}  // namespace lgb

extern "C" {

LGB_API lgb_status lgb_sppm_iteration(lgb_scene* scene, const lgb_camera* cam, const lgb_sppm_params* p, float* d_film,
                                      void* stream) {
    using namespace lgb;
    Scene* s = scene;
    if (!s) return LGB_ERR_INVALID_ARGUMENT;
    Ctx* ctx = s->ctx;
    if (!cam || !p || !d_film || cam->width == 0 || cam->height == 0 || (reinterpret_cast<uintptr_t>(d_film) & 15u))
        return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "null camera / params, empty image or misaligned film");
    if (!s->bvh.nodes) return set_error(ctx, LGB_ERR_NOT_READY, "lgb_bvh_build has not been called");
    if (p->max_depth < 1 || p->max_depth > 64) return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "max_depth must be in [1, 64]");
    if (p->num_lights < 1 || (uint32_t)p->num_lights > s->num_lights || p->light_triangle_count <= 0)
        return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "SPPM needs 1..num_lights lights and a positive light_triangle_count");
    if (p->dir_light_idx != 0xFFFFFFFFu || s->num_directional > 0)
        return set_error(ctx, LGB_ERR_UNSUPPORTED, "SPPM supports area and spot lights only");
    if (!(p->base_radius >= 0.0f) || !std::isfinite(p->base_radius))
        return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "base_radius must be finite and non-negative");
    if (!(p->spot_angle >= 0.0f && p->spot_angle < 90.0f))
        return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "spot_angle must be in [0, 90) degrees");
    cudaSetDevice(ctx->device);
    return sppm_iteration(s, cam, p, d_film, (cudaStream_t)stream);
}

}  // extern "C"
