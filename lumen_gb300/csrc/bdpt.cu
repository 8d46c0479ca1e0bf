// BDPT: Lumen's bidirectional path tracer (src/RayTracer/BDPT.cpp:55-88, src/shaders/integrators/bdpt/bdpt.rgen,
// src/shaders/integrators/bdpt_commons.glsl) on the library's traversal, BSDFs and light sampling.
//
// The reference runs one ray-generation invocation per pixel that traces both subpaths into per-pixel buffers and
// then loops over every (s, t) connection strategy. Here the frame is three kernels:
//
//   k_bdpt_subpaths  one thread per pixel: the light subpath (bdpt_generate_light_subpath, bdpt_random_walk_light,
//                    bdpt_commons.glsl:13-105, 199-240) and the camera subpath (bdpt_generate_camera_subpath,
//                    bdpt_random_walk_eye, 107-197, 242-267); vertices stored vertex-major across pixels
//   k_bdpt_connect   one thread per (strategy, pixel): a warp shares its (s, t), so the connection code
//                    (bdpt_connect_cam 473-526, bdpt_connect 528-639) and the MIS weight (calc_mis_weight 269-471)
//                    run without divergence on the strategy; t = 1 strategies splat with float atomics, the others
//                    write their contribution to a per-strategy slot
//   k_bdpt_resolve   one thread per pixel: the t >= 2 contributions summed in the reference's loop order (t outer,
//                    s inner), the frame's splat added, the NaN guard and the progressive film (bdpt.rgen:56-89)
//
// The strategy threads need the RNG state the reference's loop would have: only the s = 1 strategies draw (four
// numbers each, in increasing t), so strategy (1, t) starts from the counter after the subpaths plus 4 (t - 2).
// Kept from the reference: the path buffers read as cleared each frame (an escaped camera ray leaves a vertex that
// is zero but for its throughput and pdf_fwd, so its s = 0 strategy adds material 0's emission); calc_mis_weight's
// s = 1 branches read the flags of the light subpath's first vertex. Deviations: splats are summed with atomics and
// all of a frame's splats land in that frame (the reference's unsynchronised `+=` and same-pass read leave that
// order undefined); the RNG frame value is frame_num ^ seed (the reference's seed is a host rand()); the spot cone
// of light_pdf follows the cone parameter (30 degrees by default, as in commons.glsl:82).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "bsdf_vcm.cuh"
#include "light_sample.cuh"
#include "path_common.cuh"

namespace lgb {
namespace {

constexpr int kBdptThreads = 128;
constexpr float kTMinB = 0.001f, kTMaxWalk = 1e6f, kEpsB = 0.001f;
constexpr uint32_t kBdptLobesDG = LGB_BSDF_DIFFUSE | LGB_BSDF_MIRROR | LGB_BSDF_GLASS | LGB_BSDF_DIELECTRIC;
constexpr uint32_t kBdptLobesDGC = kBdptLobesDG | LGB_BSDF_CONDUCTOR;

struct BdptArgs {
    float iv[16], ip[16], view[16], proj[16];
    uint32_t W, H, screen;
    int max_depth, light_tri_count;
    LightSet lights;
    uint32_t seed_frame, frame_num;
    uint32_t n_strat;   // strategies per pixel: max_depth - 1 with t = 1, then max_depth (max_depth + 1) / 2
    uint32_t first_t2;  // index of the first t >= 2 strategy (max_depth - 1)
    float4* lv;         // light vertices, 4 float4 each, [vertex][component][pixel]
    float4* cv;         // camera vertices, same layout
    uint2* meta;        // per pixel: (light vertices | camera vertices << 8, RNG counter after the subpaths)
    float4* contrib;    // t >= 2 strategies: [strategy - first_t2][pixel]
    float* splat;       // the frame's splats, 3 floats per row-major pixel
    float4* film;       // RGBA32F, row-major
};

// Path vertex (bdpt_commons.h:19-34 without `dir`, which only the subpath generators read), 64 bytes:
//   (pos, pdf_fwd) (n_s, pdf_rev) (throughput, area) (u, v, material, delta | side << 1 | mode << 2 | light_flags << 8)
struct PV {
    v3 pos, n_s, thr;
    float u, v, area, pdf_fwd, pdf_rev;
    uint32_t mat, flags;
};
__device__ __forceinline__ uint32_t pv_delta(uint32_t f) { return f & 1u; }
__device__ __forceinline__ bool pv_side(uint32_t f) { return ((f >> 1) & 1u) != 0u; }
__device__ __forceinline__ uint32_t pv_light_flags(uint32_t f) { return f >> 8; }

__device__ __forceinline__ const float4* vq(const float4* b, int v, int c, uint32_t screen, uint32_t p) {
    return b + ((size_t)(v * 4 + c) * screen + p);
}
__device__ __forceinline__ float4* vq(float4* b, int v, int c, uint32_t screen, uint32_t p) {
    return b + ((size_t)(v * 4 + c) * screen + p);
}
__device__ __forceinline__ void store_pv(float4* b, int v, uint32_t screen, uint32_t p, const PV& x) {
    *vq(b, v, 0, screen, p) = f4(x.pos, x.pdf_fwd);
    *vq(b, v, 1, screen, p) = f4(x.n_s, x.pdf_rev);
    *vq(b, v, 2, screen, p) = f4(x.thr, x.area);
    *vq(b, v, 3, screen, p) = make_float4(x.u, x.v, __uint_as_float(x.mat), __uint_as_float(x.flags));
}
__device__ __forceinline__ PV load_pv(const float4* b, int v, uint32_t screen, uint32_t p) {
    const float4 a = *vq(b, v, 0, screen, p), c = *vq(b, v, 1, screen, p), d = *vq(b, v, 2, screen, p),
                 e = *vq(b, v, 3, screen, p);
    PV x;
    x.pos = V3(a.x, a.y, a.z); x.pdf_fwd = a.w;
    x.n_s = V3(c.x, c.y, c.z); x.pdf_rev = c.w;
    x.thr = V3(d.x, d.y, d.z); x.area = d.w;
    x.u = e.x; x.v = e.y; x.mat = __float_as_uint(e.z); x.flags = __float_as_uint(e.w);
    return x;
}
__device__ __forceinline__ PV zero_pv() {
    PV x;
    x.pos = x.n_s = x.thr = V3(0.0f);
    x.u = x.v = x.area = x.pdf_fwd = x.pdf_rev = 0.0f;
    x.mat = x.flags = 0u;
    return x;
}

__device__ __forceinline__ bool is_zero3(v3 a) { return a.x == 0.0f && a.y == 0.0f && a.z == 0.0f; }
__device__ __forceinline__ bool light_finite(uint32_t f) { return ((f >> 4) & 1u) != 0u; }
__device__ __forceinline__ bool light_delta(uint32_t f) { return ((f >> 5) & 1u) != 0u; }
__device__ __forceinline__ float remap0(float x) { return x != 0.0f ? x : 1.0f; }

struct CamB {
    v3 pos, nrm;
    float area;
};
__device__ __forceinline__ CamB cam_setup(const BdptArgs& A) {
    CamB c;
    const float4 o = mat_vec(A.iv, 0.0f, 0.0f, 0.0f, 1.0f);
    const float4 f = mat_vec(A.iv, 0.0f, 0.0f, 1.0f, 0.0f);
    c.pos = V3(o.x, o.y, o.z);
    c.nrm = V3(-f.x, -f.y, -f.z);
    const float4 a = mat_vec(A.ip, 2.0f / (float)A.W, 2.0f / (float)A.H, 0.0f, 1.0f);
    c.area = fabsf((a.x / a.w) * (a.y / a.w));
    return c;
}

// bdpt_random_walk_light (CAMERA = false) / bdpt_random_walk_eye (CAMERA = true). Vertex 0 of the subpath is
// already stored (its position and normal are o_pos / o_n); the walk writes vertices 1.. and each vertex's
// pdf_rev once the next direction has been sampled. Returns the number of vertices written.
template <uint32_t MASK, bool CAMERA>
__device__ int random_walk(const SceneView& S, float4* buf, uint32_t screen, uint32_t p, v3 o_pos, v3 o_n,
                           bool finite_light, int max_depth, v3 thr, float pdf, v3 wi, uint4& seed) {
    if (max_depth == 0) return 0;
    int b = 0;
    v3 ray_pos = o_pos;
    v3 prev_pos = o_pos, prev_n = o_n;
    float pdf_fwd = pdf;
    const uint32_t mode = CAMERA ? 1u : 0u;
    while (true) {
        const int prev = b - 1;
        float t, bu, bv;
        const RayQ q = make_rayq(ray_pos.x, ray_pos.y, ray_pos.z, kTMinB, wi.x, wi.y, wi.z, kTMaxWalk);
        const uint32_t prim = trace_closest_single(S.nodes, S.tris, q, t, bu, bv, S.status);
        if (prim == LGB_NO_HIT) {
            if (CAMERA) {  // bdpt_commons.glsl:126-131: the escape vertex keeps the cleared fields
                PV e = zero_pv();
                e.thr = thr;
                e.pdf_fwd = pdf_fwd;
                store_pv(buf, 1 + b, screen, p, e);
                b++;
            }
            break;
        }
        const HitAttr h = resolve_hit(S, prim, bu, bv);
        v3 wo = prev_pos - h.pos;
        const float wo_len = length(wo);
        wo = wo / wo_len;
        v3 n_s = h.n_s, n_g = h.n_g;
        bool side = true;
        if (dot(h.n_g, wo) < 0.0f) n_g = -n_g;
        if (dot(n_g, n_s) < 0.0f) { n_s = -n_s; side = false; }
        const Mat mat = load_material(S, h.mat, h.u, h.v);
        const bool spec = (mat.props & LGB_FLAG_SPECULAR) == LGB_FLAG_SPECULAR;
        const bool trans = (mat.props & LGB_FLAG_TRANSMISSION) == LGB_FLAG_TRANSMISSION;
        PV V;
        V.pos = h.pos; V.pdf_fwd = pdf_fwd * fabsf(dot(wo, n_s)) / (wo_len * wo_len);
        V.n_s = n_s; V.pdf_rev = 0.0f;
        V.thr = thr; V.area = h.area;
        V.u = h.u; V.v = h.v; V.mat = h.mat;
        V.flags = (spec ? 1u : 0u) | ((side ? 1u : 0u) << 1) | (mode << 2);
        store_pv(buf, 1 + b, screen, p, V);
        if (++b >= max_depth) break;
        const float c0 = rnd(seed), c1 = rnd(seed), c2 = rnd(seed);
        float cos_t;
        const v3 f = sample_bsdf_mode<MASK>(n_s, wo, mat, mode, side, wi, pdf_fwd, cos_t, V3(c0, c1, c2));
        const bool same_hem = dot(wi, n_s) > 0.0f && dot(wo, n_s) > 0.0f;
        if (is_zero3(f) || pdf_fwd == 0.0f || (!same_hem && !trans)) break;
        thr = thr * (f * fabsf(cos_t) / pdf_fwd);
        float pdf_rev = pdf_fwd;
        if (!spec) pdf_rev = bsdf_pdf<MASK>(mat, n_s, wi, wo, side);
        if (CAMERA || prev > -1 || finite_light) pdf_rev *= fabsf(dot(prev_n, wo)) / (wo_len * wo_len);
        reinterpret_cast<float*>(vq(buf, 1 + prev, 1, screen, p))[3] = pdf_rev;
        ray_pos = offset_ray(h.pos, n_g);
        prev_pos = h.pos;
        prev_n = n_s;
    }
    return b;
}

// bdpt.rgen main, first half: both subpaths of pixel p = y * W + x and the RNG counter after them.
template <uint32_t MASK>
__global__ void __launch_bounds__(kBdptThreads) k_bdpt_subpaths(SceneView S, BdptArgs A) {
    const CamB cam = cam_setup(A);
    const float screen_f = (float)A.screen;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < A.screen; p += gridDim.x * blockDim.x) {
        const uint32_t x = p % A.W, y = p / A.W;
        uint4 seed = make_uint4(x, y, A.seed_frame, 0u);
        // bdpt_generate_light_subpath(max_depth + 1)
        int nl = 0;
        const float r0 = rnd(seed), r1 = rnd(seed), r2 = rnd(seed), r3 = rnd(seed);
        const float d0 = rnd(seed), d1 = rnd(seed);
        const Emission e = sample_light_Le(S, A.lights, r0, r1, r2, r3, d0, d1);
        if (e.pdf_dir_w > 0.0f) {
            PV L0 = zero_pv();
            L0.pos = e.pos;
            L0.pdf_fwd = e.pdf_pos_a;
            L0.n_s = e.n;
            L0.thr = e.L;
            // side = 1; bdpt_commons.glsl:258 sets this vertex's mode to 1 (never read)
            L0.flags = (1u << 1) | (1u << 2) | (e.flags << 8);
            if (light_delta(e.flags)) L0.pdf_fwd = 0.0f;  // set after the walk in the reference; the walk does not read it
            store_pv(A.lv, 0, A.screen, p, L0);
            const v3 thr = e.L * e.cos_from_light / (e.pdf_dir_w * e.pdf_pos_a);
            nl = random_walk<MASK, false>(S, A.lv, A.screen, p, e.pos, e.n, light_finite(e.flags), A.max_depth, thr,
                                          e.pdf_dir_w, e.wi, seed) + 1;
        }
        // bdpt_generate_camera_subpath(d, origin, max_depth + 1, cam_area)
        const float u = ((float)x + 0.5f) / (float)A.W, v = ((float)y + 0.5f) / (float)A.H;
        const float dx = u * 2.0f - 1.0f, dy = v * 2.0f - 1.0f;
        const float4 t4 = mat_vec(A.ip, dx, dy, 1.0f, 1.0f);
        const v3 tn = normalize(V3(t4.x, t4.y, t4.z));
        const float4 d4 = mat_vec(A.iv, tn.x, tn.y, tn.z, 0.0f);
        const v3 dir = V3(d4.x, d4.y, d4.z);
        PV C0 = zero_pv();
        C0.pos = cam.pos;
        C0.area = cam.area;
        C0.thr = V3(1.0f);
        C0.n_s = cam.nrm;
        C0.flags = 1u << 1;
        store_pv(A.cv, 0, A.screen, p, C0);
        const float cos_theta = dot(dir, cam.nrm);
        const float pdf = 1.0f / (cam.area * screen_f * cos_theta * cos_theta * cos_theta);
        const int nc = random_walk<MASK, true>(S, A.cv, A.screen, p, cam.pos, cam.nrm, false, A.max_depth, V3(1.0f), pdf,
                                               dir, seed) + 1;
        A.meta[p] = make_uint2((uint32_t)nl | ((uint32_t)nc << 8), seed.w);
    }
}

struct Sampled {
    v3 pos, n_s;
    float pdf_fwd;
};

// light_pdf (commons.glsl:81-95), area and spot lights
__device__ __forceinline__ float light_pdf_dir(const BdptArgs& A, uint32_t flags, v3 n_s, v3 wi) {
    const uint32_t type = flags & 7u;
    if (type == LGB_LIGHT_AREA) return fmaxf(dot(n_s, wi) / LGB_PI, 0.0f);
    if (type == LGB_LIGHT_SPOT) return 1.0f / (LGB_TWO_PI * (1.0f - A.lights.spot_cos_width));
    return 0.0f;
}

// calc_mis_weight (bdpt_commons.glsl:269-471). The reference patches the path buffers and restores them; here the
// four patched pdf_rev values, the two cleared delta flags and (s = 1) the sampled light point are overrides on
// top of the stored subpaths. Ls1 / Ls2 / Ct1 / Ct2 are light vertices s-1, s-2 and camera vertices t-1, t-2 as
// stored (those that exist); l0_flags are the light flags of light vertex 0.
template <uint32_t MASK>
__device__ float mis_weight(const SceneView& S, const BdptArgs& A, uint32_t p, int s, int t, const Sampled& sm, PV Ls1,
                            const PV& Ls2, const PV& Ct1, const PV& Ct2, uint32_t l0_flags) {
    if (s + t == 2) return 1.0f;
    if (s == 1) { Ls1.pdf_fwd = sm.pdf_fwd; Ls1.pos = sm.pos; Ls1.n_s = sm.n_s; }
    // t == 1: camera vertex 0 takes the sampled camera point, which is its own; its pdf_fwd is never read
    float r1, r2 = 0.0f, r3 = 0.0f, r4 = 0.0f;
    if (s > 0) {
        v3 dir = Ct1.pos - Ls1.pos;
        const float dir_len = length(dir);
        dir = dir / dir_len;
        float pdf_rev;
        if (s >= 2) {
            const Mat mat = load_material(S, Ls1.mat, Ls1.u, Ls1.v);
            const v3 wo = normalize(Ls2.pos - Ls1.pos);
            pdf_rev = bsdf_pdf<MASK>(mat, Ls1.n_s, wo, dir, pv_side(Ls1.flags));
        } else {
            pdf_rev = light_pdf_dir(A, l0_flags, Ls1.n_s, dir);
        }
        pdf_rev *= fabsf(dot(dir, Ct1.n_s)) / (dir_len * dir_len);
        r1 = pdf_rev;
    } else {
        r1 = 1.0f / ((float)A.light_tri_count * Ct1.area);
    }
    if (t > 1) {
        v3 dir = Ct2.pos - Ct1.pos;
        const float dir_len = length(dir);
        dir = dir / dir_len;
        if (s > 0) {
            const Mat mat = load_material(S, Ct1.mat, Ct1.u, Ct1.v);
            const v3 wo = normalize(Ls1.pos - Ct1.pos);
            r2 = bsdf_pdf<MASK>(mat, Ct1.n_s, wo, dir, pv_side(Ct1.flags));
            if (r2 != 0.0f) r2 *= fabsf(dot(dir, Ct2.n_s)) / (dir_len * dir_len);
        } else {
            const float cos_x = dot(Ct1.n_s, dir);
            const float cos_y = dot(Ct2.n_s, dir);
            r2 = fabsf(cos_x * cos_y) / (LGB_PI * dir_len * dir_len);
        }
    }
    if (s > 0) {
        v3 dir = Ls1.pos - Ct1.pos;
        const float dir_len = length(dir);
        dir = dir / dir_len;
        if (t == 1) {
            const float cos_theta = dot(Ct1.n_s, dir);
            float pdf = 1.0f / (Ct1.area * (float)A.screen * cos_theta * cos_theta * cos_theta);
            pdf *= fabsf(dot(dir, Ls1.n_s)) / (dir_len * dir_len);
            r3 = pdf;
        } else {
            const v3 wo = normalize(Ct2.pos - Ct1.pos);
            const Mat mat = load_material(S, Ct1.mat, Ct1.u, Ct1.v);
            r3 = bsdf_pdf<MASK>(mat, Ct1.n_s, wo, dir, pv_side(Ct1.flags));
            if ((s == 1 && light_finite(l0_flags)) || s > 1) r3 *= fabsf(dot(dir, Ls1.n_s)) / (dir_len * dir_len);
        }
    }
    if (s > 1) {
        v3 dir = Ls2.pos - Ls1.pos;
        const v3 wo = normalize(Ct1.pos - Ls1.pos);
        const float dir_len = length(dir);
        dir = dir / dir_len;
        const Mat mat = load_material(S, Ls1.mat, Ls1.u, Ls1.v);
        r4 = bsdf_pdf<MASK>(mat, Ls1.n_s, wo, dir, pv_side(Ls1.flags));
        if ((s == 2 && light_finite(l0_flags)) || s > 2) r4 *= fabsf(dot(dir, Ls2.n_s)) / (dir_len * dir_len);
    }
    float sum_ri = 0.0f, weight = 1.0f;
    for (int i = t - 1; i > 0; i--) {
        const float pr = i == t - 1 ? r1 : (i == t - 2 ? r2 : vq(A.cv, i, 1, A.screen, p)->w);
        const float pf = vq(A.cv, i, 0, A.screen, p)->w;
        const uint32_t di = i == t - 1 ? 0u : pv_delta(__float_as_uint(vq(A.cv, i, 3, A.screen, p)->w));
        const uint32_t dp = pv_delta(__float_as_uint(vq(A.cv, i - 1, 3, A.screen, p)->w));
        weight *= remap0(pr) / remap0(pf);
        if (di == 0u && dp == 0u) sum_ri += weight;
    }
    weight = 1.0f;
    for (int i = s - 1; i >= 0; i--) {
        const float pr = i == s - 1 ? r3 : (i == s - 2 ? r4 : vq(A.lv, i, 1, A.screen, p)->w);
        const float pf = i == s - 1 ? Ls1.pdf_fwd : vq(A.lv, i, 0, A.screen, p)->w;
        const uint32_t di = i == s - 1 ? 0u : pv_delta(__float_as_uint(vq(A.lv, i, 3, A.screen, p)->w));
        const bool delta_prev = i > 0 ? pv_delta(__float_as_uint(vq(A.lv, i - 1, 3, A.screen, p)->w)) == 1u
                                      : light_delta(l0_flags);
        weight *= remap0(pr) / remap0(pf);
        if (di == 0u && !delta_prev) sum_ri += weight;
    }
    return 1.0f / (1.0f + sum_ri);
}

// bdpt_connect_cam (bdpt_commons.glsl:473-526), s >= 2: the splat of light vertex s-1 and its pixel
template <uint32_t MASK>
__device__ v3 connect_cam(const SceneView& S, const BdptArgs& A, uint32_t p, int s, uint32_t& pidx, bool& have) {
    have = false;
    const PV Ls1 = load_pv(A.lv, s - 1, A.screen, p), Ls2 = load_pv(A.lv, s - 2, A.screen, p);
    const PV C0 = load_pv(A.cv, 0, A.screen, p);
    Sampled sm{V3(0.0f), V3(0.0f), 0.0f};
    v3 Lo = V3(0.0f);
    v3 dir = C0.pos - Ls1.pos;
    const float len = length(dir);
    dir = dir / len;
    const float cos_y = dot(dir, Ls1.n_s);
    const float cos_theta = dot(C0.n_s, -dir);
    if (cos_theta <= 0.0f) return V3(0.0f);
    const float cos_3_theta = cos_theta * cos_theta * cos_theta;
    const float cam_pdf_ratio = fabsf(cos_y) / (C0.area * cos_3_theta * len * len);
    const v3 origin = offset_ray2(Ls1.pos, Ls1.n_s);
    const Mat mat = load_material(S, Ls1.mat, Ls1.u, Ls1.v);
    const v3 wo = normalize(Ls2.pos - Ls1.pos);
    float pdf, pdf_rev;
    const v3 f = eval_bsdf_rev<MASK>(Ls1.n_s, wo, mat, pv_side(Ls1.flags), dir, pdf, pdf_rev, false);
    if (is_zero3(f)) return Lo;
    if (cam_pdf_ratio > 0.0f) {
        const RayQ q = make_rayq(origin.x, origin.y, origin.z, 0.0f, dir.x, dir.y, dir.z, len - kEpsB);
        if (!trace_any_single(S.nodes, S.tris, q, S.status)) {
            sm.pos = C0.pos;
            sm.n_s = C0.n_s;
            Lo = Ls1.thr * cam_pdf_ratio * f / (float)A.screen;
        }
    }
    dir = -dir;
    float4 tg = mat_vec(A.view, dir.x, dir.y, dir.z, 0.0f);
    tg = make_float4(tg.x / tg.z, tg.y / tg.z, tg.z / tg.z, tg.w / tg.z);
    tg = mat_vec(A.proj, tg.x, tg.y, tg.z, tg.w);
    tg = make_float4(-tg.x, -tg.y, -tg.z, -tg.w);
    const int cx = __float2int_rz(0.5f * (1.0f + tg.x) * (float)A.W - 0.5f);
    const int cy = __float2int_rz(0.5f * (1.0f + tg.y) * (float)A.H - 0.5f);
    if (cx < 0 || cx >= (int)A.W || cy < 0 || cy >= (int)A.H || dot(dir, C0.n_s) < 0.0f) return V3(0.0f);
    have = true;
    pidx = (uint32_t)cy * A.W + (uint32_t)cx;
    float mis = 1.0f;
    if (luminance(Lo) != 0.0f) {
        const uint32_t l0_flags = pv_light_flags(__float_as_uint(vq(A.lv, 0, 3, A.screen, p)->w));
        mis = mis_weight<MASK>(S, A, p, s, 1, sm, Ls1, Ls2, C0, C0, l0_flags);
    }
    return mis * Lo;
}

// bdpt_connect (bdpt_commons.glsl:528-639), t >= 2
template <uint32_t MASK>
__device__ v3 connect(const SceneView& S, const BdptArgs& A, uint32_t p, int s, int t, uint4 seed) {
    const PV Ct1 = load_pv(A.cv, t - 1, A.screen, p), Ct2 = load_pv(A.cv, t - 2, A.screen, p);
    PV Ls1 = zero_pv(), Ls2 = zero_pv();
    if (s >= 1) Ls1 = load_pv(A.lv, s - 1, A.screen, p);
    if (s >= 2) Ls2 = load_pv(A.lv, s - 2, A.screen, p);
    Sampled sm{V3(0.0f), V3(0.0f), 0.0f};
    v3 Lo = V3(0.0f);
    if (s == 0) {
        const lgb_material* m = &S.mats[Ct1.mat];  // an escape vertex reads material 0
        Lo = V3(m->emissive_factor[0], m->emissive_factor[1], m->emissive_factor[2]) * Ct1.thr;
    } else if (s == 1) {
        const float q0 = rnd(seed), q1 = rnd(seed), q2 = rnd(seed), q3 = rnd(seed);
        const Incidence li = sample_light_Li_pos(S, A.lights, q0, q1, q2, q3, Ct1.pos);
        const float cos_x = fabsf(dot(li.wi, Ct1.n_s));
        const v3 origin = offset_ray2(Ct1.pos, Ct1.n_s);
        const v3 wo = normalize(Ct2.pos - Ct1.pos);
        const Mat mat = load_material(S, Ct1.mat, Ct1.u, Ct1.v);
        float pdf, pdf_rev;
        const v3 f = eval_bsdf_rev<MASK>(Ct1.n_s, wo, mat, pv_side(Ct1.flags), li.wi, pdf, pdf_rev, false);
        if (!is_zero3(f)) {
            const RayQ q = make_rayq(origin.x, origin.y, origin.z, 0.0f, li.wi.x, li.wi.y, li.wi.z, li.wi_len - kEpsB);
            if (!trace_any_single(S.nodes, S.tris, q, S.status)) {
                const float ltc = (float)A.light_tri_count;
                const uint32_t type = li.flags & 7u;
                const float l2 = li.wi_len * li.wi_len;
                // light_pdf_a_to_w (commons.glsl:64-79)
                const float pdf_a_to_w = type == LGB_LIGHT_AREA ? li.pdf_pos_a * l2 / li.cos_y
                                         : type == LGB_LIGHT_SPOT ? l2 / li.cos_y
                                         : type == LGB_LIGHT_DIRECTIONAL ? 1.0f
                                                                         : 0.0f;
                const float pdf_light_w = pdf_a_to_w / ltc;
                sm.pdf_fwd = li.pdf_pos_a / ltc;
                sm.pos = li.pos;
                sm.n_s = li.n;
                Lo = Ct1.thr * f * cos_x * li.L / pdf_light_w;
            }
        }
    } else {
        const v3 n_s = Ls1.n_s, n_t = Ct1.n_s;
        v3 d = Ls1.pos - Ct1.pos;
        const float len = length(d);
        d = d / len;
        const float G = dot(n_s, -d) * dot(n_t, d) / (len * len);
        if (G > 0.0f) {
            const Mat mat_1 = load_material(S, Ct1.mat, Ct1.u, Ct1.v);
            const Mat mat_2 = load_material(S, Ls1.mat, Ls1.u, Ls1.v);
            const v3 wo_1 = normalize(Ct2.pos - Ct1.pos);
            const v3 wo_2 = normalize(Ls2.pos - Ls1.pos);
            float p0, p1;
            const v3 brdf1 = eval_bsdf_rev<MASK>(n_t, wo_1, mat_1, pv_side(Ct1.flags), d, p0, p1, false);
            const v3 brdf2 = eval_bsdf_rev<MASK>(n_s, wo_2, mat_2, pv_side(Ls1.flags), -d, p0, p1, false);
            if (!is_zero3(brdf1) && !is_zero3(brdf2)) {
                const v3 origin = offset_ray2(Ct1.pos, Ct1.n_s);
                const RayQ q = make_rayq(origin.x, origin.y, origin.z, 0.0f, d.x, d.y, d.z, len - kEpsB);
                if (!trace_any_single(S.nodes, S.tris, q, S.status)) Lo = Ls1.thr * G * brdf1 * brdf2 * Ct1.thr;
            }
        }
    }
    if (luminance(Lo) != 0.0f) {
        const uint32_t l0_flags = s >= 1 ? pv_light_flags(__float_as_uint(vq(A.lv, 0, 3, A.screen, p)->w)) : 0u;
        Lo = Lo * mis_weight<MASK>(S, A, p, s, t, sm, Ls1, Ls2, Ct1, Ct2, l0_flags);
    }
    return Lo;
}

// Strategy k of a pixel: k < max_depth - 1 are (s = k + 2, t = 1); then blocks t = 2 .. max_depth + 1 of
// max_depth + 2 - t strategies each, s = 0 .. max_depth + 1 - t (bdpt.rgen:52-58: s + t <= max_depth + 1).
__device__ __forceinline__ void strategy(uint32_t k, int D, int& s, int& t) {
    if (k < (uint32_t)(D - 1)) { s = (int)k + 2; t = 1; return; }
    int j = (int)k - (D - 1);
    t = 2;
    while (j >= D + 2 - t) { j -= D + 2 - t; t++; }
    s = j;
}

// One thread per (strategy, pixel), strategy-major: the threads of a warp share (s, t).
template <uint32_t MASK>
__global__ void __launch_bounds__(kBdptThreads) k_bdpt_connect(SceneView S, BdptArgs A) {
    const uint64_t total = (uint64_t)A.n_strat * A.screen;
    for (uint64_t idx = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t k = (uint32_t)(idx / A.screen), p = (uint32_t)(idx % A.screen);
        int s, t;
        strategy(k, A.max_depth, s, t);
        const uint2 m = A.meta[p];
        const int nl = (int)(m.x & 0xffu), nc = (int)((m.x >> 8) & 0xffu);
        const bool live = s <= nl && t <= nc;
        if (t == 1) {
            if (!live) continue;
            uint32_t pidx = 0;
            bool have = false;
            const v3 L = connect_cam<MASK>(S, A, p, s, pidx, have);
            if (luminance(L) > 0.0f && have) {
                atomicAdd(&A.splat[3 * (size_t)pidx], L.x);
                atomicAdd(&A.splat[3 * (size_t)pidx + 1], L.y);
                atomicAdd(&A.splat[3 * (size_t)pidx + 2], L.z);
            }
        } else {
            v3 L = V3(0.0f);
            if (live) {
                const uint32_t x = p % A.W, y = p / A.W;
                const uint4 seed = make_uint4(x, y, A.seed_frame, m.y + 4u * (uint32_t)(t - 2));
                L = connect<MASK>(S, A, p, s, t, seed);
            }
            A.contrib[(size_t)(k - A.first_t2) * A.screen + p] = f4(L, 0.0f);
        }
    }
}

// bdpt.rgen:56-89: the pixel's t >= 2 contributions in loop order, its splat, the NaN guard and the film.
__global__ void __launch_bounds__(256) k_bdpt_resolve(BdptArgs A) {
    const uint32_t n2 = A.n_strat - A.first_t2;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < A.screen; p += gridDim.x * blockDim.x) {
        v3 col = V3(0.0f);
        for (uint32_t j = 0; j < n2; j++) {
            const float4 c = A.contrib[(size_t)j * A.screen + p];
            col = col + V3(c.x, c.y, c.z);
        }
        col = col + V3(A.splat[3 * (size_t)p], A.splat[3 * (size_t)p + 1], A.splat[3 * (size_t)p + 2]);
        if (isnan(luminance(col))) continue;
        float4& px = A.film[p];
        if (A.frame_num > 0u) {
            const float w = 1.0f / (float)(A.frame_num + 1u);
            const float4 old = px;
            px = make_float4(mixf(old.x, col.x, w), mixf(old.y, col.y, w), mixf(old.z, col.z, w), 1.0f);
        } else {
            px = make_float4(col.x, col.y, col.z, 1.0f);
        }
    }
}

size_t align256b(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

lgb_status bdpt_iteration(Scene* s, const lgb_camera* cam, const lgb_bdpt_params* p, float* d_film, cudaStream_t st) {
    Ctx* ctx = s->ctx;
    const uint64_t screen64 = (uint64_t)cam->width * cam->height;
    const int D = p->max_depth;
    const uint64_t n_strat = (uint64_t)(D - 1) + (uint64_t)D * (D + 1) / 2, n2 = (uint64_t)D * (D + 1) / 2;
    const uint32_t per = (uint32_t)D + 1u;
    if (screen64 * n_strat >= 0x80000000ull || screen64 * per * 4u >= 0x80000000ull)
        return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "width * height * strategies must stay below 2^31");
    const uint32_t screen = (uint32_t)screen64;
    size_t off = 0;
    auto take = [&](size_t bytes) { const size_t o = off; off += align256b(bytes); return o; };
    const size_t o_lv = take(sizeof(float4) * 4 * per * (size_t)screen);
    const size_t o_cv = take(sizeof(float4) * 4 * per * (size_t)screen);
    const size_t o_meta = take(sizeof(uint2) * (size_t)screen);
    const size_t o_con = take(sizeof(float4) * n2 * (size_t)screen);
    const size_t o_spl = take(sizeof(float) * 3 * (size_t)screen);
    if (!s->bdpt_buf || s->bdpt_buf_bytes < off) {
        cudaFree(s->bdpt_buf);
        s->bdpt_buf = nullptr;
        s->bdpt_buf_bytes = 0;
        LGB_CUDA_TRY(ctx, cudaMalloc(&s->bdpt_buf, off));
        s->bdpt_buf_bytes = off;
    }
    char* base = (char*)s->bdpt_buf;
    BdptArgs A;
    std::memset(&A, 0, sizeof(A));
    for (int i = 0; i < 16; i++) { A.iv[i] = cam->inv_view[i]; A.ip[i] = cam->inv_projection[i]; }
    if (lgb_camera_forward(cam, A.view, A.proj) != LGB_OK)
        return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "the camera's inverse matrices are singular");
    A.W = cam->width; A.H = cam->height; A.screen = screen;
    A.max_depth = D;
    A.light_tri_count = p->light_triangle_count;
    A.lights.num_lights = p->num_lights;
    A.lights.light_tri_count = p->light_triangle_count;
    spot_cone(p->spot_angle, A.lights.spot_cos_width, A.lights.spot_cos_falloff);
    A.seed_frame = p->frame_num ^ p->seed;
    A.frame_num = p->frame_num;
    A.n_strat = (uint32_t)n_strat;
    A.first_t2 = (uint32_t)(D - 1);
    A.lv = reinterpret_cast<float4*>(base + o_lv);
    A.cv = reinterpret_cast<float4*>(base + o_cv);
    A.meta = reinterpret_cast<uint2*>(base + o_meta);
    A.contrib = reinterpret_cast<float4*>(base + o_con);
    A.splat = reinterpret_cast<float*>(base + o_spl);
    A.film = reinterpret_cast<float4*>(d_film);
    LGB_CUDA_TRY(ctx, cudaMemsetAsync(A.splat, 0, sizeof(float) * 3 * (size_t)screen, st));
    const SceneView S = scene_view(s);
    const int sms = ctx->sm_count > 0 ? ctx->sm_count : 1;
    const int grid_px = (int)std::min<uint32_t>((screen + kBdptThreads - 1) / kBdptThreads, (uint32_t)sms * 16u);
    const uint64_t total = n_strat * screen;
    const int grid_st = (int)std::min<uint64_t>((total + kBdptThreads - 1) / kBdptThreads, (uint64_t)sms * 64u);
    // kernels instantiated per set of BSDF types in the scene, as for VCM
    const uint32_t used = s->bsdf_mask;
    const uint32_t lobes = (used & ~kBdptLobesDG) == 0u ? kBdptLobesDG : ((used & ~kBdptLobesDGC) == 0u ? kBdptLobesDGC : kAllBsdfs);
    if (lobes == kBdptLobesDG) k_bdpt_subpaths<kBdptLobesDG><<<grid_px, kBdptThreads, 0, st>>>(S, A);
    else if (lobes == kBdptLobesDGC) k_bdpt_subpaths<kBdptLobesDGC><<<grid_px, kBdptThreads, 0, st>>>(S, A);
    else k_bdpt_subpaths<kAllBsdfs><<<grid_px, kBdptThreads, 0, st>>>(S, A);
    LGB_CUDA_TRY(ctx, cudaGetLastError());
    if (lobes == kBdptLobesDG) k_bdpt_connect<kBdptLobesDG><<<grid_st, kBdptThreads, 0, st>>>(S, A);
    else if (lobes == kBdptLobesDGC) k_bdpt_connect<kBdptLobesDGC><<<grid_st, kBdptThreads, 0, st>>>(S, A);
    else k_bdpt_connect<kAllBsdfs><<<grid_st, kBdptThreads, 0, st>>>(S, A);
    LGB_CUDA_TRY(ctx, cudaGetLastError());
    k_bdpt_resolve<<<(int)std::min<uint32_t>((screen + 255) / 256, (uint32_t)sms * 8u), 256, 0, st>>>(A);
    LGB_CUDA_TRY(ctx, cudaGetLastError());
    return LGB_OK;
}

}  // namespace lgb

extern "C" {

LGB_API lgb_status lgb_bdpt_iteration(lgb_scene* scene, const lgb_camera* cam, const lgb_bdpt_params* p, float* d_film,
                                      void* stream) {
    using namespace lgb;
    Scene* s = scene;
    if (!s) return LGB_ERR_INVALID_ARGUMENT;
    Ctx* ctx = s->ctx;
    if (!cam || !p || !d_film || cam->width == 0 || cam->height == 0 || (reinterpret_cast<uintptr_t>(d_film) & 15u))
        return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "null camera / params, empty image or misaligned film");
    if (!s->bvh.nodes) return set_error(ctx, LGB_ERR_NOT_READY, "lgb_bvh_build has not been called");
    if (p->max_depth < 1 || p->max_depth > 32) return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "max_depth must be in [1, 32]");
    if (p->num_lights < 1 || (uint32_t)p->num_lights > s->num_lights || p->light_triangle_count <= 0)
        return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "BDPT needs 1..num_lights lights and a positive light_triangle_count");
    if (p->dir_light_idx != 0xFFFFFFFFu || s->num_directional > 0)
        return set_error(ctx, LGB_ERR_UNSUPPORTED, "BDPT supports area and spot lights only");
    if (s->num_materials == 0)  // an escaped camera ray reads material 0 (bdpt_commons.glsl:536-537)
        return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "BDPT needs at least one material");
    if (!(p->spot_angle >= 0.0f && p->spot_angle < 90.0f))
        return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "spot_angle must be in [0, 90) degrees");
    cudaSetDevice(ctx->device);
    return bdpt_iteration(s, cam, p, d_film, (cudaStream_t)stream);
}

}  // extern "C"
