// Oracle (test infrastructure only): CPU restatement of Lumen's ReSTIR DI integrator, one frame of
// ReSTIR::render (src/RayTracer/ReSTIR.cpp:74-151):
//   temporal pass  src/shaders/integrators/restir/di/temporal_pass.rgen:7-233 with restirdi_commons.glsl:34-110
//   spatial pass   spatial_pass.rgen:5-47
//   output         output.rgen:6-35
// The temporal pass's path-traced colour is not computed: the output pass never reads it (output.rgen:12). The
// seed is a parameter (the reference draws it with host rand()). State layouts are the library's: G-buffer 3
// float4 (pos, material | normal, u | v), reservoir 3 float4 (w_sum, W, m, light | triangle, seed.xyz | seed.w),
// integer fields stored as their bits.
#include <cstdint>
#include <cstring>

#include "photon_common.h"
#include "scene_internal.h"

namespace {
using namespace orc;
using namespace orc::detail;
using namespace orc::photon;

inline uint32_t fb(float x) { uint32_t u; std::memcpy(&u, &x, 4); return u; }
inline float bf(uint32_t u) { float x; std::memcpy(&x, &u, 4); return x; }

struct Res {
    float w_sum = 0.0f, W = 0.0f;
    uint32_t m = 0, light = 0, tri = 0;
    U4 seed{0, 0, 0, 0};
};
Res load_res(const float* p) {
    Res r;
    r.w_sum = p[0]; r.W = p[1]; r.m = fb(p[2]); r.light = fb(p[3]); r.tri = fb(p[4]);
    r.seed = U4{fb(p[5]), fb(p[6]), fb(p[7]), fb(p[8])};
    return r;
}
void store_res(float* p, const Res& r) {
    p[0] = r.w_sum; p[1] = r.W; p[2] = bf(r.m); p[3] = bf(r.light);
    p[4] = bf(r.tri); p[5] = bf(r.seed.x); p[6] = bf(r.seed.y); p[7] = bf(r.seed.z);
    p[8] = bf(r.seed.w); p[9] = p[10] = p[11] = 0.0f;
}

struct GPt {
    V3<float> pos, normal, origin;
    V2<float> uv;
    uint32_t mat = 0;
};

struct Ctx {
    const Scene& s;
    const orc_restir_params* p;
    Cone cone;
};

void update_reservoir(Res& r, uint32_t light, uint32_t tri, U4 s, float w_i, U4& seed) {
    r.w_sum += w_i;
    r.m++;
    if (rand(seed) < w_i / r.w_sum) {
        r.light = light;
        r.tri = tri;
        r.seed = s;
    }
}

// sample_light_with_idx (commons.glsl:417-455), area and spot lights.
V3<float> sample_light_with_idx(const Ctx& c, V4<float> rands, V3<float> p, uint32_t li, uint32_t tri, V3<float>& lpos,
                                V3<float>& ln) {
    const orc_light& light = c.s.lights[li];
    const uint32_t type = light.light_flags & 0x7u;
    V3<float> L(0.0f);
    lpos = V3<float>(0.0f);
    ln = V3<float>(0.0f);
    if (type == LIGHT_AREA) {
        const orc_mesh& pm = c.s.meshes[light.prim_mesh_idx];
        float tri_pdf;
        V2<float> bary;
        sample_triangle<float>(c.s, pm, V2<float>(rands.z, rands.w), tri, lpos, ln, tri_pdf, bary);
        L = load_material<float>(c.s, pm.material_index, bary).emissive_factor;
    } else if (type == LIGHT_SPOT) {
        const V3<float> lp(light.pos[0], light.pos[1], light.pos[2]), to(light.to[0], light.to[1], light.to[2]);
        const V3<float> dir = normalize(p - lp);
        const V3<float> light_dir = normalize(to - lp);
        const float ct = dot(dir, light_dir);
        float fall;
        if (ct < c.cone.cos_width) fall = 0.0f;
        else if (ct >= c.cone.cos_falloff) fall = 1.0f;
        else { const float d = (ct - c.cone.cos_width) / (c.cone.cos_falloff - c.cone.cos_width); fall = (d * d) * (d * d); }
        lpos = lp;
        ln = dir;
        L = V3<float>(light.L[0], light.L[1], light.L[2]) * fall;
    }
    return L;
}

// calc_L / calc_L_with_visibility_check (restirdi_commons.glsl:42-100)
V3<float> calc_L(const Ctx& c, const GPt& g, const Res& r, bool visibility) {
    const Mat<float> mat = load_material<float>(c.s, g.mat, g.uv);
    const V3<float> wo = normalize(g.origin - g.pos);
    U4 rs = r.seed;
    const float a = rand(rs), b = rand(rs), cc = rand(rs), d = rand(rs);
    V3<float> lpos, ln;
    const V3<float> Le = sample_light_with_idx(c, V4<float>(a, b, cc, d), g.pos, r.light, r.tri, lpos, ln);
    V3<float> wi = lpos - g.pos;
    const float wi_len = length(wi);
    wi /= wi_len;
    float pdf, unused_rev;
    const V3<float> f = eval_bsdf(g.normal, wo, mat, 1u, true, wi, pdf, unused_rev, false);
    const float cos_x = dot(g.normal, wi);
    const float gt = std::fabs(dot(ln, -wi)) / (wi_len * wi_len);
    if (visibility) {
        const V3<float> o = offset_ray(g.pos, g.normal);
        float of[3] = {o.x, o.y, o.z}, wf[3] = {wi.x, wi.y, wi.z};
        if (bvh_any(c.s.bvh, of, wf, 0.0f, wi_len - EPS)) return V3<float>(0.0f);
    }
    return f * Le * std::fabs(cos_x) * gt;
}

void combine_reservoir(const Ctx& c, const GPt& g, Res& r1, const Res& r2, U4& seed) {
    float fac = r2.W * (float)r2.m;
    if (fac > 0.0f) fac *= length(calc_L(c, g, r2, false));
    update_reservoir(r1, r2.light, r2.tri, r2.seed, fac, seed);
}

void temporal(const Ctx& c, const M4<float>& iv, const M4<float>& ip, const M4<float>& pv, const M4<float>& pp,
              uint32_t x, uint32_t y, uint32_t W, uint32_t H, float* gbuf, float* pass, const float* temp) {
    U4 seed{x, y, c.p->frame_num ^ c.p->seed, 0u};
    const V2<float> in_uv(((float)x + 0.5f) / (float)W, ((float)y + 0.5f) / (float)H);
    const V2<float> d(in_uv.x * 2.0f - 1.0f, in_uv.y * 2.0f - 1.0f);
    GPt g;
    g.origin = (iv * V4<float>(0.0f, 0.0f, 0.0f, 1.0f)).xyz();
    const V3<float> direction = sample_camera(iv, ip, d);
    Res r_new, r_prev, r;
    r.seed = seed;
    r_new.seed = seed;
    Payload<float> payload;
    payload.material_idx = -1; payload.triangle_idx = 0xFFFFFFFFu; payload.instance_idx = 0xFFFFFFFFu;
    trace_closest<float>(c.s, g.origin, direction, TMIN, TMAX, payload);
    if (payload.material_idx != -1) {
        g.pos = payload.pos;
        g.uv = payload.uv;
        g.mat = (uint32_t)payload.material_idx;
        const V3<float> wo = normalize(g.origin - g.pos);
        V3<float> n_s = payload.n_s, n_g = payload.n_g;
        bool side = true;
        if (dot(payload.n_g, wo) < 0.0f) n_g = -n_g;
        if (dot(n_g, payload.n_s) < 0.0f) { n_s = -n_s; side = false; }
        g.normal = n_s;
        const Mat<float> mat = load_material<float>(c.s, g.mat, g.uv);
        const uint32_t light_samples = (uint32_t)std::min(c.p->light_triangle_count, 32);
        if (c.p->do_spatiotemporal == 1u && (mat.bsdf_props & BSDF_FLAG_SPECULAR) == 0) {
            V4<float> prev_pos = pv * V4<float>(g.pos.x, g.pos.y, g.pos.z, 1.0f);
            const float z = prev_pos.z;
            prev_pos = V4<float>(prev_pos.x / z, prev_pos.y / z, prev_pos.z / z, prev_pos.w / z);
            const V4<float> pj = pp * prev_pos;
            const int cx = to_int_rz(0.5f * (1.0f + -pj.x) * (float)W);
            const int cy = to_int_rz(0.5f * (1.0f + -pj.y) * (float)H);
            if (cx < (int)W && cx >= 0 && cy < (int)H && cy >= 0) r_prev = load_res(temp + 12 * (size_t)(x * H + y));
        }
        const float light_pick = (float)(1 / c.p->num_lights);  // GLSL integer division
        for (uint32_t k = 0; k < light_samples; k++) {
            const U4 light_seed = seed;
            const float q0 = rand(seed), q1 = rand(seed), q2 = rand(seed), q3 = rand(seed);
            const uint32_t li = (uint32_t)(q0 * (float)c.p->num_lights);
            const orc_light& light = c.s.lights[li];
            const uint32_t type = light.light_flags & 0x7u;
            V3<float> Le(0.0f), wi(0.0f);
            float wi_len = 0.0f, pdf_light = 0.0f, cos_from_light = 0.0f;
            uint32_t tri = 0;
            if (type == LIGHT_AREA) {
                const orc_mesh& pm = c.s.meshes[light.prim_mesh_idx];
                tri = (uint32_t)(q1 * (float)light.num_triangles);
                V3<float> lpos, ln;
                float tri_pdf;
                V2<float> bary;
                sample_triangle<float>(c.s, pm, V2<float>(q2, q3), tri, lpos, ln, tri_pdf, bary);
                Le = load_material<float>(c.s, pm.material_index, bary).emissive_factor;
                wi = lpos - payload.pos;
                const float l2 = dot(wi, wi);
                wi_len = std::sqrt(l2);
                wi /= wi_len;
                cos_from_light = std::fabs(dot(ln, -wi));
                pdf_light = tri_pdf;
            } else if (type == LIGHT_SPOT) {
                const V3<float> lp(light.pos[0], light.pos[1], light.pos[2]), to(light.to[0], light.to[1], light.to[2]);
                wi = lp - payload.pos;
                const float l2 = dot(wi, wi);
                wi_len = std::sqrt(l2);
                wi /= wi_len;
                const V3<float> light_dir = normalize(to - lp);
                cos_from_light = dot(-wi, light_dir);
                float fall;
                if (cos_from_light < c.cone.cos_width) fall = 0.0f;
                else if (cos_from_light >= c.cone.cos_falloff) fall = 1.0f;
                else {
                    const float dd = (cos_from_light - c.cone.cos_width) / (c.cone.cos_falloff - c.cone.cos_width);
                    fall = (dd * dd) * (dd * dd);
                }
                pdf_light = 1.0f;
                Le = V3<float>(light.L[0], light.L[1], light.L[2]) * fall;
            }
            float bsdf_pdf, unused_rev;
            const float cos_x = dot(g.normal, wi);
            const float gt = std::fabs(cos_from_light) / (wi_len * wi_len);
            const V3<float> f = eval_bsdf(g.normal, wo, mat, 1u, side, wi, bsdf_pdf, unused_rev, false);
            pdf_light *= light_pick;
            const float p_hat = length(f * Le * std::fabs(cos_x) * gt);
            update_reservoir(r_new, li, tri, light_seed, p_hat / pdf_light, seed);
        }
        if (r_new.w_sum > 0.0f) {
            U4 rs = r_new.seed;
            const float a = rand(rs), b = rand(rs), cc = rand(rs), dd = rand(rs);
            V3<float> lpos, ln;
            const V3<float> Le = sample_light_with_idx(c, V4<float>(a, b, cc, dd), payload.pos, r_new.light, r_new.tri, lpos, ln);
            V3<float> wi = lpos - payload.pos;
            const float wi_len = length(wi);
            wi /= wi_len;
            const V3<float> o = offset_ray2(g.pos, g.normal);
            float of[3] = {o.x, o.y, o.z}, wf[3] = {wi.x, wi.y, wi.z};
            const bool hit = bvh_any(c.s.bvh, of, wf, 0.0f, wi_len - EPS);
            float pdf, unused_rev;
            const V3<float> f = eval_bsdf(g.normal, wo, mat, 1u, side, wi, pdf, unused_rev, false);
            const float cos_x = dot(g.normal, wi);
            const float gt = std::fabs(dot(ln, -wi)) / (wi_len * wi_len);
            const bool visible = !hit && !(f.x == 0.0f && f.y == 0.0f && f.z == 0.0f);
            r_new.W = 0.0f;
            if (visible) {
                const float p_hat = length(f * Le * std::fabs(cos_x) * gt);
                r_new.W = p_hat == 0.0f ? 0.0f : r_new.w_sum / (p_hat * (float)r_new.m);
            }
        }
        combine_reservoir(c, g, r, r_new, seed);
        uint32_t num_samples = r_new.m;
        if (c.p->do_spatiotemporal == 1u) {
            r_prev.m = std::min(20u * r.m, r_prev.m);
            combine_reservoir(c, g, r, r_prev, seed);
            num_samples += r_prev.m;
        }
        r.m = num_samples;
        if (r_new.W > 0.0f || r_prev.W > 0.0f) {
            const float phat = length(calc_L(c, g, r, false)) * (float)r.m;
            r.W = phat == 0.0f ? 0.0f : r.w_sum / phat;
        } else {
            r.W = 0.0f;
        }
        float* gb = gbuf + 12 * (size_t)(x * H + y);
        gb[0] = g.pos.x; gb[1] = g.pos.y; gb[2] = g.pos.z; gb[3] = bf(g.mat);
        gb[4] = g.normal.x; gb[5] = g.normal.y; gb[6] = g.normal.z; gb[7] = g.uv.x;
        gb[8] = g.uv.y; gb[9] = gb[10] = gb[11] = 0.0f;
    }
    store_res(pass + 12 * (size_t)(x * H + y), r);
}

GPt load_gpt(const float* gb, V3<float> origin) {
    GPt g;
    g.pos = V3<float>(gb[0], gb[1], gb[2]);
    g.mat = fb(gb[3]);
    g.normal = V3<float>(gb[4], gb[5], gb[6]);
    g.uv = V2<float>(gb[7], gb[8]);
    g.origin = origin;
    return g;
}

void spatial(const Ctx& c, V3<float> origin, uint32_t x, uint32_t y, uint32_t W, uint32_t H, const float* gbuf,
             const float* pass, float* spat) {
    const float max_r = 10.0f;
    U4 seed{x, y, c.p->frame_num ^ c.p->seed, 0u};
    const uint32_t i = x * H + y;
    const GPt g = load_gpt(gbuf + 12 * (size_t)i, origin);
    const Res curr = load_res(pass + 12 * (size_t)i);
    Res r;
    if (curr.W != 0.0f) {
        combine_reservoir(c, g, r, curr, seed);
        uint32_t num_samples = (c.p->flags & 1u) ? curr.m : r.m;
        for (int k = 0; k < 5; k++) {
            const float randa = rand(seed) * 2.0f * K<float>::PI();
            const float randr = std::sqrt(rand(seed)) * max_r;
            const int ox = (int)std::floor(std::cos(randa) * randr), oy = (int)std::floor(std::sin(randa) * randr);
            const int cx = std::min(std::max((int)x + ox, 0), (int)W - 1), cy = std::min(std::max((int)y + oy, 0), (int)H - 1);
            const Res rn = load_res(pass + 12 * (size_t)((uint32_t)cx * H + (uint32_t)cy));
            combine_reservoir(c, g, r, rn, seed);
            num_samples += rn.m;
        }
        r.m = num_samples;
        r.W = r.w_sum / ((float)r.m * length(calc_L(c, g, r, false)));
    }
    store_res(spat + 12 * (size_t)i, r);
}

void output(const Ctx& c, V3<float> origin, uint32_t x, uint32_t y, uint32_t W, uint32_t H, const float* gbuf,
            const float* spat, float* temp, float* film) {
    const uint32_t i = x * H + y;
    const GPt g = load_gpt(gbuf + 12 * (size_t)i, origin);
    const Res r = load_res(spat + 12 * (size_t)i);
    V3<float> col(0.0f);
    if (r.W > 0.0f) {
        col += r.W * calc_L(c, g, r, true) * (float)c.p->light_triangle_count;
        store_res(temp + 12 * (size_t)i, r);
    }
    float* px = film + 4 * ((size_t)y * W + x);
    if (c.p->frame_num == 0u || c.p->enable_accumulation == 0u) {
        px[0] = col.x; px[1] = col.y; px[2] = col.z; px[3] = 1.0f;
    } else {
        const float w = 1.0f / (float)(c.p->frame_num + 1u);
        const V3<float> m = mix(V3<float>(px[0], px[1], px[2]), col, w);
        px[0] = m.x; px[1] = m.y; px[2] = m.z; px[3] = 1.0f;
    }
}

}  // namespace

extern "C" {

void orc_restir_di_iteration(void* scene, const float inv_view[16], const float inv_proj[16], const float prev_view[16],
                             const float prev_proj[16], uint32_t width, uint32_t height, const orc_restir_params* p,
                             float* gbuf, float* passthrough, float* temporal_res, float* spatial_res, float* film,
                             int nthreads) {
    const Scene& s = *(const Scene*)scene;
    const M4<float> iv = load_m4<float>(inv_view), ip = load_m4<float>(inv_proj);
    const M4<float> pv = load_m4<float>(prev_view), pp = load_m4<float>(prev_proj);
    const uint32_t screen = width * height;
    const Ctx c{s, p, spot_cone(p->spot_angle)};
    std::memset(gbuf, 0, sizeof(float) * 12 * (size_t)screen);
    std::memset(spatial_res, 0, sizeof(float) * 12 * (size_t)screen);
    if (p->do_spatiotemporal == 0u) std::memset(temporal_res, 0, sizeof(float) * 12 * (size_t)screen);
    const V3<float> origin = (iv * V4<float>(0.0f, 0.0f, 0.0f, 1.0f)).xyz();
    parallel_for(screen, nthreads, [&](uint32_t i) {
        temporal(c, iv, ip, pv, pp, i / height, i % height, width, height, gbuf, passthrough, temporal_res);
    });
    parallel_for(screen, nthreads, [&](uint32_t i) {
        spatial(c, origin, i / height, i % height, width, height, gbuf, passthrough, spatial_res);
    });
    parallel_for(screen, nthreads, [&](uint32_t i) {
        output(c, origin, i / height, i % height, width, height, gbuf, spatial_res, temporal_res, film);
    });
}

}  // extern "C"
