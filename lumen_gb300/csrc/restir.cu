// ReSTIR DI: Lumen's ReSTIR integrator for direct lighting (src/RayTracer/ReSTIR.cpp:74-157,
// src/shaders/integrators/restir/di/*) on the library's traversal and light sampling.
//
//   k_restir_temporal  temporal_pass.rgen:7-233: camera ray to the first hit (the G-buffer), up to 32 light
//                      candidates resampled into one reservoir, a visibility test of the chosen candidate, and
//                      the merge with the pixel's reservoir of the previous frame
//   k_restir_spatial   spatial_pass.rgen:5-47: five random neighbours within 10 pixels merged in
//   k_restir_output    output.rgen:6-35: the reservoir's light sample with a visibility ray, progressive film,
//                      and the reservoir kept for the next frame's temporal pass
//
// Kept from the reference: pixel indices are column-major (x * height + y); a candidate's pdf is multiplied by the
// integer division 1 / num_lights (1 for one light, 0 otherwise); the previous frame's reservoir is read at the
// pixel itself whenever the hit reprojects inside the image; the spatial pass starts its sample count at 1; the
// output is the resampled direct light alone (the temporal pass's path-traced colour is never added, output.rgen:12
// is commented out in the reference, so it is not computed here); the spatial and temporal passes of a pixel start
// from the same RNG seed; the spatial pass counts the pixel's own reservoir as one sample (LGB_RESTIR_SPATIAL_COUNT_FIX
// counts its m instead). Deviations: the seed is a parameter (the reference draws it with host rand()).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "light_sample.cuh"
#include "path_common.cuh"

namespace lgb {
namespace {
using namespace sh;

constexpr int kRestirThreads = 128;
constexpr float kTMinR = 0.001f, kTMaxR = 10000.0f, kEpsR = 0.001f;

// G-buffer (RestirGBufferData, restirdi_commons.h:34-43) as 3 float4: pos, material (bits) | normal, uv.x | uv.y.
// Reservoir (RestirReservoir, restirdi_commons.h:27-33) as 3 float4: w_sum, W, m (bits), light (bits) |
// triangle (bits), seed.x, seed.y, seed.z (bits) | seed.w (bits).
struct Reservoir {
    float w_sum, W;
    uint32_t m, light, tri;
    uint4 seed;
};

struct RestirArgs {
    float iv[16], ip[16], prev_view[16], prev_proj[16];
    uint32_t W, H, screen;
    LightSet lights;
    uint32_t seed_frame;  // frame_num ^ seed
    uint32_t frame_num;
    uint32_t do_spatiotemporal, enable_accumulation, flags;
    float4* gbuf;         // screen * 3
    float4* passthrough;  // screen * 3 each
    float4* temporal;
    float4* spatial;
    float4* film;         // RGBA32F, row-major
};

__device__ __forceinline__ uint32_t ub(float x) { return __float_as_uint(x); }
__device__ __forceinline__ float fu(uint32_t x) { return __uint_as_float(x); }

__device__ __forceinline__ Reservoir load_res(const float4* p) {
    const float4 a = p[0], b = p[1], c = p[2];
    Reservoir r;
    r.w_sum = a.x; r.W = a.y; r.m = ub(a.z); r.light = ub(a.w);
    r.tri = ub(b.x);
    r.seed = make_uint4(ub(b.y), ub(b.z), ub(b.w), ub(c.x));
    return r;
}
__device__ __forceinline__ void store_res(float4* p, const Reservoir& r) {
    p[0] = make_float4(r.w_sum, r.W, fu(r.m), fu(r.light));
    p[1] = make_float4(fu(r.tri), fu(r.seed.x), fu(r.seed.y), fu(r.seed.z));
    p[2] = make_float4(fu(r.seed.w), 0.0f, 0.0f, 0.0f);
}
__device__ __forceinline__ Reservoir empty_res() {
    Reservoir r;
    r.w_sum = 0.0f; r.W = 0.0f; r.m = 0u; r.light = 0u; r.tri = 0u;
    r.seed = make_uint4(0u, 0u, 0u, 0u);
    return r;
}

// The shading point every reservoir is evaluated at (load_g_buffer, restirdi_commons.glsl:26-32).
struct GPoint {
    v3 pos, normal, origin;
    float u, v;
    uint32_t mat;
};

// restirdi_commons.glsl:34-40
__device__ __forceinline__ void update_reservoir(Reservoir& r, uint32_t light, uint32_t tri, uint4 s, float w_i, uint4& seed) {
    r.w_sum += w_i;
    r.m++;
    if (rnd(seed) < w_i / r.w_sum) {
        r.light = light;
        r.tri = tri;
        r.seed = s;
    }
}

// sample_light_with_idx (commons.glsl:417-455) for area and spot lights: emission, position and normal of the
// light sample of light `li`, triangle `tri` with the given draws.
__device__ v3 sample_light_with_idx(const SceneView& S, const LightSet& Ls, float r0, float r1, float r2, float r3, v3 p,
                                    uint32_t li, uint32_t tri, v3& lpos, v3& ln) {
    (void)r0; (void)r1;
    const lgb_light* L = &S.lights[li];
    const uint32_t type = L->light_flags & 7u;
    v3 Le = V3(0.0f);
    lpos = V3(0.0f);
    ln = V3(0.0f);
    if (type == LGB_LIGHT_AREA) {
        const lgb_mesh pm = S.meshes[L->prim_mesh_idx];
        float tri_pdf;
        sample_tri(S, pm, tri, r2, r3, lpos, ln, tri_pdf);
        const lgb_material* lm = &S.mats[pm.material_index];
        Le = V3(lm->emissive_factor[0], lm->emissive_factor[1], lm->emissive_factor[2]);
    } else if (type == LGB_LIGHT_SPOT) {
        const v3 lp = V3(L->pos[0], L->pos[1], L->pos[2]);
        const v3 dir = normalize(p - lp);
        const v3 ldir = normalize(V3(L->to[0], L->to[1], L->to[2]) - lp);
        const float ct = dot(dir, ldir);
        float fall;
        if (ct < Ls.spot_cos_width) fall = 0.0f;
        else if (ct >= Ls.spot_cos_falloff) fall = 1.0f;
        else { const float d = (ct - Ls.spot_cos_width) / (Ls.spot_cos_falloff - Ls.spot_cos_width); fall = (d * d) * (d * d); }
        lpos = lp;
        ln = dir;
        Le = V3(L->L[0], L->L[1], L->L[2]) * fall;
    }
    return Le;
}

// calc_L (restirdi_commons.glsl:42-67) and, with `visibility`, calc_L_with_visibility_check (:69-100).
__device__ v3 calc_L(const SceneView& S, const LightSet& Ls, const GPoint& g, const Reservoir& r, bool visibility) {
    const Mat m = load_material(S, g.mat, g.u, g.v);
    const v3 wo = normalize(g.origin - g.pos);
    uint4 rs = r.seed;
    const float a = rnd(rs), b = rnd(rs), c = rnd(rs), d = rnd(rs);
    v3 lpos, ln;
    const v3 Le = sample_light_with_idx(S, Ls, a, b, c, d, g.pos, r.light, r.tri, lpos, ln);
    v3 wi = lpos - g.pos;
    const float wi_len = length(wi);
    wi = wi / wi_len;
    float pdf;
    const v3 f = eval_bsdf(g.normal, wo, m, true, wi, pdf);
    const float cos_x = dot(g.normal, wi);
    const float gt = fabsf(dot(ln, -wi)) / (wi_len * wi_len);
    if (visibility) {
        const v3 o = offset_ray(g.pos, g.normal);
        const RayQ q = make_rayq(o.x, o.y, o.z, 0.0f, wi.x, wi.y, wi.z, wi_len - kEpsR);
        if (trace_any_single(S.nodes, S.tris, q, S.status)) return V3(0.0f);
    }
    return f * Le * fabsf(cos_x) * gt;
}

// combine_reservoir (restirdi_commons.glsl:104-110)
__device__ void combine_reservoir(const SceneView& S, const LightSet& Ls, const GPoint& g, Reservoir& r1, const Reservoir& r2,
                                  uint4& seed) {
    float fac = r2.W * (float)r2.m;
    if (fac > 0.0f) fac *= length(calc_L(S, Ls, g, r2, false));
    update_reservoir(r1, r2.light, r2.tri, r2.seed, fac, seed);
}

// temporal_pass.rgen:7-233 (without the path-traced colour, which the output pass never reads)
// Registers for 4 blocks per SM (144 unbounded): a 256 x 256 frame's 512 blocks then fit one wave on 152 SMs.
__global__ void __launch_bounds__(kRestirThreads, 4) k_restir_temporal(SceneView S, RestirArgs A) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < A.screen; i += gridDim.x * blockDim.x) {
        const uint32_t x = i / A.H, y = i % A.H;
        uint4 seed = make_uint4(x, y, A.seed_frame, 0u);
        const float u = ((float)x + 0.5f) / (float)A.W, v = ((float)y + 0.5f) / (float)A.H;
        const float dx = u * 2.0f - 1.0f, dy = v * 2.0f - 1.0f;
        const float4 o4 = mat_vec(A.iv, 0.0f, 0.0f, 0.0f, 1.0f);
        const float4 t4 = mat_vec(A.ip, dx, dy, 1.0f, 1.0f);
        const v3 tn = normalize(V3(t4.x, t4.y, t4.z));
        const float4 d4 = mat_vec(A.iv, tn.x, tn.y, tn.z, 0.0f);
        GPoint g;
        g.origin = V3(o4.x, o4.y, o4.z);
        Reservoir r_new = empty_res(), r_prev = empty_res(), r = empty_res();
        r.seed = seed;
        r_new.seed = seed;
        float t, bu, bv;
        const RayQ q = make_rayq(g.origin.x, g.origin.y, g.origin.z, kTMinR, d4.x, d4.y, d4.z, kTMaxR);
        const uint32_t prim = trace_closest_single(S.nodes, S.tris, q, t, bu, bv, S.status);
        if (prim != LGB_NO_HIT) {
            const HitAttr h = resolve_hit(S, prim, bu, bv);
            g.pos = h.pos;
            g.u = h.u;
            g.v = h.v;
            g.mat = h.mat;
            const v3 wo = normalize(g.origin - g.pos);
            v3 n_s = h.n_s, n_g = h.n_g;
            bool side = true;
            if (dot(h.n_g, wo) < 0.0f) n_g = -n_g;
            if (dot(n_g, h.n_s) < 0.0f) { n_s = -n_s; side = false; }
            g.normal = n_s;
            const Mat m = load_material(S, g.mat, g.u, g.v);
            const uint32_t light_samples = (uint32_t)min(A.lights.light_tri_count, 32);
            if (A.do_spatiotemporal == 1u && (m.props & LGB_FLAG_SPECULAR) == 0u) {
                float4 pp = mat_vec(A.prev_view, g.pos.x, g.pos.y, g.pos.z, 1.0f);
                pp = make_float4(pp.x / pp.z, pp.y / pp.z, pp.z / pp.z, pp.w / pp.z);
                const float4 pj = mat_vec(A.prev_proj, pp.x, pp.y, pp.z, pp.w);
                const int cx = __float2int_rz(0.5f * (1.0f + -pj.x) * (float)A.W);
                const int cy = __float2int_rz(0.5f * (1.0f + -pj.y) * (float)A.H);
                if (cx < (int)A.W && cx >= 0 && cy < (int)A.H && cy >= 0) r_prev = load_res(A.temporal + (size_t)i * 3);
            }
            const int num_lights_int = A.lights.num_lights;
            const float light_pick = (float)(1 / num_lights_int);  // GLSL integer division
            for (uint32_t k = 0; k < light_samples; k++) {
                const uint4 light_seed = seed;
                const float q0 = rnd(seed), q1 = rnd(seed), q2 = rnd(seed), q3 = rnd(seed);
                const uint32_t li = (uint32_t)(q0 * (float)A.lights.num_lights);
                const lgb_light* L = &S.lights[li];
                const uint32_t type = L->light_flags & 7u;
                v3 Le = V3(0.0f), wi = V3(0.0f);
                float wi_len = 0.0f, pdf_light = 0.0f, cos_from_light = 0.0f;
                uint32_t tri = 0u;
                if (type == LGB_LIGHT_AREA) {
                    const lgb_mesh pm = S.meshes[L->prim_mesh_idx];
                    tri = (uint32_t)(q1 * (float)L->num_triangles);
                    v3 lpos, ln;
                    float tri_pdf;
                    sample_tri(S, pm, tri, q2, q3, lpos, ln, tri_pdf);
                    const lgb_material* lm = &S.mats[pm.material_index];
                    Le = V3(lm->emissive_factor[0], lm->emissive_factor[1], lm->emissive_factor[2]);
                    wi = lpos - h.pos;
                    const float l2 = dot(wi, wi);
                    wi_len = sqrtf(l2);
                    wi = wi / wi_len;
                    cos_from_light = fabsf(dot(ln, -wi));
                    pdf_light = tri_pdf;
                } else if (type == LGB_LIGHT_SPOT) {
                    const v3 lp = V3(L->pos[0], L->pos[1], L->pos[2]);
                    wi = lp - h.pos;
                    const float l2 = dot(wi, wi);
                    wi_len = sqrtf(l2);
                    wi = wi / wi_len;
                    const v3 ldir = normalize(V3(L->to[0], L->to[1], L->to[2]) - lp);
                    cos_from_light = dot(-wi, ldir);
                    float fall;
                    if (cos_from_light < A.lights.spot_cos_width) fall = 0.0f;
                    else if (cos_from_light >= A.lights.spot_cos_falloff) fall = 1.0f;
                    else {
                        const float d = (cos_from_light - A.lights.spot_cos_width) /
                                        (A.lights.spot_cos_falloff - A.lights.spot_cos_width);
                        fall = (d * d) * (d * d);
                    }
                    pdf_light = 1.0f;
                    Le = V3(L->L[0], L->L[1], L->L[2]) * fall;
                }
                float bsdf_pdf;
                const float cos_x = dot(g.normal, wi);
                const float gt = fabsf(cos_from_light) / (wi_len * wi_len);
                const v3 f = eval_bsdf(g.normal, wo, m, side, wi, bsdf_pdf);
                pdf_light *= light_pick;
                const float p_hat = length(f * Le * fabsf(cos_x) * gt);
                update_reservoir(r_new, li, tri, light_seed, p_hat / pdf_light, seed);
            }
            if (r_new.w_sum > 0.0f) {  // visibility of the chosen candidate
                uint4 rs = r_new.seed;
                const float a = rnd(rs), b = rnd(rs), c = rnd(rs), d = rnd(rs);
                v3 lpos, ln;
                const v3 Le = sample_light_with_idx(S, A.lights, a, b, c, d, h.pos, r_new.light, r_new.tri, lpos, ln);
                v3 wi = lpos - h.pos;
                const float wi_len = length(wi);
                wi = wi / wi_len;
                const v3 o = offset_ray2(g.pos, g.normal);
                const RayQ sq = make_rayq(o.x, o.y, o.z, 0.0f, wi.x, wi.y, wi.z, wi_len - kEpsR);
                const bool hit = trace_any_single(S.nodes, S.tris, sq, S.status);
                float pdf;
                const v3 f = eval_bsdf(g.normal, wo, m, side, wi, pdf);
                const float cos_x = dot(g.normal, wi);
                const float gt = fabsf(dot(ln, -wi)) / (wi_len * wi_len);
                const bool visible = !hit && !(f.x == 0.0f && f.y == 0.0f && f.z == 0.0f);
                r_new.W = 0.0f;
                if (visible) {
                    const float p_hat = length(f * Le * fabsf(cos_x) * gt);
                    r_new.W = p_hat == 0.0f ? 0.0f : r_new.w_sum / (p_hat * (float)r_new.m);
                }
            }
            combine_reservoir(S, A.lights, g, r, r_new, seed);
            uint32_t num_samples = r_new.m;
            if (A.do_spatiotemporal == 1u) {
                r_prev.m = min(20u * r.m, r_prev.m);
                combine_reservoir(S, A.lights, g, r, r_prev, seed);
                num_samples += r_prev.m;
            }
            r.m = num_samples;
            if (r_new.W > 0.0f || r_prev.W > 0.0f) {
                const float phat = length(calc_L(S, A.lights, g, r, false)) * (float)r.m;
                r.W = phat == 0.0f ? 0.0f : r.w_sum / phat;
            } else {
                r.W = 0.0f;
            }
            float4* gb = A.gbuf + (size_t)i * 3;
            gb[0] = make_float4(g.pos.x, g.pos.y, g.pos.z, fu(g.mat));
            gb[1] = make_float4(g.normal.x, g.normal.y, g.normal.z, g.u);
            gb[2] = make_float4(g.v, 0.0f, 0.0f, 0.0f);
        }
        store_res(A.passthrough + (size_t)i * 3, r);
    }
}

__device__ __forceinline__ GPoint load_gpoint(const RestirArgs& A, uint32_t i) {
    const float4* gb = A.gbuf + (size_t)i * 3;
    const float4 a = gb[0], b = gb[1], c = gb[2];
    GPoint g;
    g.pos = V3(a.x, a.y, a.z);
    g.mat = ub(a.w);
    g.normal = V3(b.x, b.y, b.z);
    g.u = b.w;
    g.v = c.x;
    const float4 o4 = mat_vec(A.iv, 0.0f, 0.0f, 0.0f, 1.0f);
    g.origin = V3(o4.x, o4.y, o4.z);
    return g;
}

// spatial_pass.rgen:5-47
__global__ void __launch_bounds__(kRestirThreads) k_restir_spatial(SceneView S, RestirArgs A) {
    const float max_r = 10.0f;
    const int num_neighbor_samples = 5;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < A.screen; i += gridDim.x * blockDim.x) {
        const uint32_t x = i / A.H, y = i % A.H;
        uint4 seed = make_uint4(x, y, A.seed_frame, 0u);
        const GPoint g = load_gpoint(A, i);
        const Reservoir curr = load_res(A.passthrough + (size_t)i * 3);
        Reservoir r = empty_res();
        if (curr.W != 0.0f) {
            combine_reservoir(S, A.lights, g, r, curr, seed);
            uint32_t num_samples = (A.flags & LGB_RESTIR_SPATIAL_COUNT_FIX) ? curr.m : r.m;
            for (int k = 0; k < num_neighbor_samples; k++) {
                const float randa = rnd(seed) * 2.0f * LGB_PI;
                const float randr = sqrtf(rnd(seed)) * max_r;
                const int ox = (int)floorf(cosf(randa) * randr), oy = (int)floorf(sinf(randa) * randr);
                const int cx = min(max((int)x + ox, 0), (int)A.W - 1), cy = min(max((int)y + oy, 0), (int)A.H - 1);
                const uint32_t n = (uint32_t)cx * A.H + (uint32_t)cy;
                const Reservoir rn = load_res(A.passthrough + (size_t)n * 3);
                combine_reservoir(S, A.lights, g, r, rn, seed);
                num_samples += rn.m;
            }
            r.m = num_samples;
            r.W = r.w_sum / ((float)r.m * length(calc_L(S, A.lights, g, r, false)));
        }
        store_res(A.spatial + (size_t)i * 3, r);
    }
}

// output.rgen:6-35
__global__ void __launch_bounds__(kRestirThreads) k_restir_output(SceneView S, RestirArgs A) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < A.screen; i += gridDim.x * blockDim.x) {
        const uint32_t x = i / A.H, y = i % A.H;
        const GPoint g = load_gpoint(A, i);
        const Reservoir r = load_res(A.spatial + (size_t)i * 3);
        v3 col = V3(0.0f);
        if (r.W > 0.0f) {
            col = col + r.W * calc_L(S, A.lights, g, r, true) * (float)A.lights.light_tri_count;
            store_res(A.temporal + (size_t)i * 3, r);
        }
        float4& px = A.film[(size_t)y * A.W + x];
        if (A.frame_num == 0u || A.enable_accumulation == 0u) {
            px = make_float4(col.x, col.y, col.z, 1.0f);
        } else {
            const float w = 1.0f / (float)(A.frame_num + 1u);
            const float4 old = px;
            px = make_float4(mixf(old.x, col.x, w), mixf(old.y, col.y, w), mixf(old.z, col.z, w), 1.0f);
        }
    }
}

size_t align256r(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

lgb_status restir_iteration(Scene* s, const lgb_camera* cam, const lgb_camera* prev, const lgb_restir_params* p,
                            float* d_film, cudaStream_t st) {
    Ctx* ctx = s->ctx;
    const uint64_t screen64 = (uint64_t)cam->width * cam->height;
    if (screen64 * 3u >= 0x80000000ull) return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "image too large");
    const uint32_t screen = (uint32_t)screen64;
    size_t off = 0;
    auto take = [&](size_t bytes) { const size_t o = off; off += align256r(bytes); return o; };
    const size_t per = sizeof(float4) * 3 * (size_t)screen;
    const size_t o_g = take(per), o_p = take(per), o_t = take(per), o_s = take(per);
    const bool fresh = !s->restir_buf || s->restir_w != cam->width || s->restir_h != cam->height || s->restir_buf_bytes < off;
    if (fresh) {
        cudaFree(s->restir_buf);
        s->restir_buf = nullptr;
        s->restir_buf_bytes = 0;
        LGB_CUDA_TRY(ctx, cudaMalloc(&s->restir_buf, off));
        s->restir_buf_bytes = off;
        s->restir_w = cam->width; s->restir_h = cam->height;
    }
    char* base = (char*)s->restir_buf;
    // ReSTIR.cpp:116-119: the G-buffer and the spatial reservoirs are cleared every frame, the temporal ones
    // while spatiotemporal reuse is off (and whenever the buffers are new)
    LGB_CUDA_TRY(ctx, cudaMemsetAsync(base + o_g, 0, per, st));
    LGB_CUDA_TRY(ctx, cudaMemsetAsync(base + o_s, 0, per, st));
    if (fresh || p->do_spatiotemporal == 0u) LGB_CUDA_TRY(ctx, cudaMemsetAsync(base + o_t, 0, per, st));
    RestirArgs A;
    std::memset(&A, 0, sizeof(A));
    for (int i = 0; i < 16; i++) { A.iv[i] = cam->inv_view[i]; A.ip[i] = cam->inv_projection[i]; }
    LGB_CUDA_TRY(ctx, lgb_camera_forward(prev ? prev : cam, A.prev_view, A.prev_proj) == LGB_OK ? cudaSuccess
                                                                                             : cudaErrorInvalidValue);
    A.W = cam->width; A.H = cam->height; A.screen = screen;
    A.lights.num_lights = p->num_lights;
    A.lights.light_tri_count = p->light_triangle_count;
    spot_cone(p->spot_angle, A.lights.spot_cos_width, A.lights.spot_cos_falloff);
    A.seed_frame = p->frame_num ^ p->seed;
    A.frame_num = p->frame_num;
    A.do_spatiotemporal = p->do_spatiotemporal ? 1u : 0u;
    A.enable_accumulation = p->enable_accumulation ? 1u : 0u;
    A.flags = p->flags;
    A.gbuf = reinterpret_cast<float4*>(base + o_g);
    A.passthrough = reinterpret_cast<float4*>(base + o_p);
    A.temporal = reinterpret_cast<float4*>(base + o_t);
    A.spatial = reinterpret_cast<float4*>(base + o_s);
    A.film = reinterpret_cast<float4*>(d_film);
    const SceneView S = scene_view(s);
    const int sms = ctx->sm_count > 0 ? ctx->sm_count : 1;
    const int grid = (int)std::min<uint32_t>((screen + kRestirThreads - 1) / kRestirThreads, (uint32_t)sms * 16u);
    k_restir_temporal<<<grid, kRestirThreads, 0, st>>>(S, A);
    k_restir_spatial<<<grid, kRestirThreads, 0, st>>>(S, A);
    k_restir_output<<<grid, kRestirThreads, 0, st>>>(S, A);
    LGB_CUDA_TRY(ctx, cudaGetLastError());
    return LGB_OK;
}

}  // namespace lgb

extern "C" {

LGB_API lgb_status lgb_restir_di_iteration(lgb_scene* scene, const lgb_camera* cam, const lgb_camera* prev_cam,
                                           const lgb_restir_params* p, float* d_film, void* stream) {
    using namespace lgb;
    Scene* s = scene;
    if (!s) return LGB_ERR_INVALID_ARGUMENT;
    Ctx* ctx = s->ctx;
    if (!cam || !p || !d_film || cam->width == 0 || cam->height == 0 || (reinterpret_cast<uintptr_t>(d_film) & 15u))
        return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "null camera / params, empty image or misaligned film");
    if (prev_cam && (prev_cam->width != cam->width || prev_cam->height != cam->height))
        return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "the previous camera must have the same image size");
    if (!s->bvh.nodes) return set_error(ctx, LGB_ERR_NOT_READY, "lgb_bvh_build has not been called");
    if (p->num_lights < 1 || (uint32_t)p->num_lights > s->num_lights || p->light_triangle_count <= 0)
        return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "ReSTIR needs 1..num_lights lights and a positive light_triangle_count");
    if (p->dir_light_idx != 0xFFFFFFFFu || s->num_directional > 0)
        return set_error(ctx, LGB_ERR_UNSUPPORTED, "ReSTIR DI supports area and spot lights only");
    if (!(p->spot_angle >= 0.0f && p->spot_angle < 90.0f))
        return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "spot_angle must be in [0, 90) degrees");
    cudaSetDevice(ctx->device);
    return restir_iteration(s, cam, prev_cam, p, d_film, (cudaStream_t)stream);
}

}  // extern "C"
