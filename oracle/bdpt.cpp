// Oracle (test infrastructure only): CPU restatement of Lumen's BDPT integrator.
//
// Follows src/shaders/integrators/bdpt/bdpt.rgen:39-90 (per-pixel main: subpaths, strategy loop, splat read,
// progressive film), src/shaders/integrators/bdpt_commons.glsl (bdpt_random_walk_light 13-105,
// bdpt_random_walk_eye 107-197, bdpt_generate_light_subpath 199-240, bdpt_generate_camera_subpath 242-267,
// calc_mis_weight 269-471, bdpt_connect_cam 473-526, bdpt_connect 528-639), src/RayTracer/BDPT.cpp:55-88 (buffers
// zeroed each frame) and src/shaders/commons.glsl (sample_light_Li 224-300, sample_light_Le 335-406, light_pdf
// 81-95, light_pdf_a_to_w 64-79).
//
// Semantics kept from the reference: the path buffers are cleared every frame, so a camera ray that escapes
// leaves a vertex whose fields are zero except its throughput and pdf_fwd (its s = 0 strategy adds material 0's
// emission); calc_mis_weight's s == 1 branches read the light flags of the light subpath's vertex 0, not those of
// the light that bdpt_connect sampled; the spot cone pdf of light_pdf follows the cone parameter (30 degrees by
// default, as in commons.glsl:82). Made deterministic here: the reference adds camera splats into a shared image
// with unsynchronised `+=` and each pixel reads its splat slot while other pixels may still write it; here every
// splat of a frame is summed (in source pixel order, row-major, then strategy order) before any pixel reads its
// slot, so a frame's splats land in that frame. The RNG frame value is frame_num ^ seed (the reference's seed
// is a host rand()). Directional lights are refused by the library, as for VCM and SPPM.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "photon_common.h"
#include "scene_internal.h"

namespace {
using namespace orc;
using namespace orc::detail;
using namespace orc::photon;

const float kTMaxWalk = 1e6f;  // bdpt_commons.glsl:25, 118

// PathVertex (bdpt_commons.h:19-34) minus `dir`, which only the subpath generators read.
struct PV {
    V3<float> pos, n_s, thr;
    V2<float> uv;
    float area, pdf_fwd, pdf_rev;
    uint32_t light_flags, material_idx, delta, side, mode;
};
inline PV zero_pv() {
    PV v;
    v.pos = v.n_s = v.thr = V3<float>(0.0f);
    v.uv = V2<float>(0.0f, 0.0f);
    v.area = v.pdf_fwd = v.pdf_rev = 0.0f;
    v.light_flags = v.material_idx = v.delta = v.side = v.mode = 0u;
    return v;
}

inline bool is_zero(V3<float> v) { return v.x == 0.0f && v.y == 0.0f && v.z == 0.0f; }
inline float remap0(float x) { return x != 0.0f ? x : 1.0f; }

struct Cam {
    M4<float> iv, ip, view, proj;
    V3<float> pos, nrm;
    float area;
    uint32_t W, H;
};

struct Ctx {
    const Scene& s;
    const orc_bdpt_params* p;
    const Cam& c;
    Cone cone;
    float screen;
};

// light_pdf (commons.glsl:81-95): area and spot lights
inline float light_pdf(const Ctx& X, uint32_t flags, V3<float> n_s, V3<float> wi) {
    switch (flags & 0x7u) {
        case LIGHT_AREA: return std::max(dot(n_s, wi) / K<float>::PI(), 0.0f);
        case LIGHT_SPOT: return uniform_cone_pdf(X.cone.cos_width);
        default: return 0.0f;
    }
}
// light_pdf_a_to_w (commons.glsl:64-79)
inline float light_pdf_a_to_w(uint32_t flags, float pdf_a, float wi_len_sqr, float cos_from_light) {
    switch (flags & 0x7u) {
        case LIGHT_AREA: return pdf_a * wi_len_sqr / cos_from_light;
        case LIGHT_SPOT: return wi_len_sqr / cos_from_light;
        case LIGHT_DIRECTIONAL: return 1.0f;
        default: return 0.0f;
    }
}

// bdpt_random_walk_light / bdpt_random_walk_eye: v[0] is the subpath's origin vertex, the walk writes v[1 + b].
int random_walk(const Ctx& X, PV* v, int max_depth, V3<float> thr, float pdf, V3<float> wi, bool camera, U4& seed) {
    if (max_depth == 0) return 0;
    int b = 0;
    V3<float> ray_pos = v[0].pos;
    float pdf_fwd = pdf;
    const bool finite_light = light_finite(v[0].light_flags);
    const uint32_t mode = camera ? 1u : 0u;
    while (true) {
        const int prev = b - 1;
        Payload<float> pl;
        pl.material_idx = -1;
        trace_closest<float>(X.s, ray_pos, wi, TMIN, kTMaxWalk, pl);
        if (pl.material_idx == -1) {
            if (camera) {  // bdpt_commons.glsl:126-131: the escape vertex keeps the cleared fields
                v[1 + b] = zero_pv();
                v[1 + b].thr = thr;
                v[1 + b].pdf_fwd = pdf_fwd;
                b++;
            }
            break;
        }
        V3<float> wo = v[1 + prev].pos - pl.pos;
        const float wo_len = length(wo);
        wo /= wo_len;
        V3<float> n_s = pl.n_s;
        bool side = true;
        V3<float> n_g = pl.n_g;
        if (dot(pl.n_g, wo) < 0.0f) n_g = -n_g;
        if (dot(n_g, n_s) < 0.0f) { n_s = -n_s; side = false; }
        PV& V = v[1 + b];
        V = zero_pv();
        V.pdf_fwd = pdf_fwd * std::fabs(dot(wo, n_s)) / (wo_len * wo_len);
        V.n_s = n_s;
        V.area = pl.area;
        V.pos = pl.pos;
        V.uv = pl.uv;
        V.material_idx = (uint32_t)pl.material_idx;
        V.thr = thr;
        V.side = side ? 1u : 0u;
        V.mode = mode;
        const Mat<float> mat = load_material<float>(X.s, (uint32_t)pl.material_idx, pl.uv);
        const bool spec = (mat.bsdf_props & BSDF_FLAG_SPECULAR) == BSDF_FLAG_SPECULAR;
        const bool trans = (mat.bsdf_props & BSDF_FLAG_TRANSMISSION) == BSDF_FLAG_TRANSMISSION;
        V.delta = spec ? 1u : 0u;
        if (++b >= max_depth) break;
        float cos_theta;
        const float r0 = rand(seed), r1 = rand(seed), r2 = rand(seed);
        const V3<float> f = sample_bsdf<float>(n_s, wo, mat, mode, side, wi, pdf_fwd, cos_theta, V3<float>(r0, r1, r2));
        const bool same_hem = dot(wi, n_s) > 0.0f && dot(wo, n_s) > 0.0f;
        if (is_zero(f) || pdf_fwd == 0.0f || (!same_hem && !trans)) break;
        thr *= f * std::fabs(cos_theta) / pdf_fwd;
        float pdf_rev = pdf_fwd;
        if (!spec) pdf_rev = bsdf_pdf<float>(mat, n_s, wi, wo, side);
        if (camera || prev > -1 || finite_light) pdf_rev *= std::fabs(dot(v[1 + prev].n_s, wo)) / (wo_len * wo_len);
        v[1 + prev].pdf_rev = pdf_rev;
        ray_pos = offset_ray(pl.pos, n_g);
    }
    return b;
}

// bdpt_generate_light_subpath(max_depth + 1)
int light_subpath(const Ctx& X, PV* L, U4& seed) {
    const float r0 = rand(seed), r1 = rand(seed), r2 = rand(seed), r3 = rand(seed);
    const float d0 = rand(seed), d1 = rand(seed);
    const Emission<float> e = sample_light_Le<float>(X.s, V4<float>(r0, r1, r2, r3), V2<float>(d0, d1), X.p->num_lights,
                                                     X.p->light_triangle_count, X.cone);
    if (e.pdf_dir_w <= 0.0f) return 0;
    L[0] = zero_pv();
    L[0].pos = e.pos;
    L[0].light_flags = e.flags;
    L[0].pdf_fwd = e.pdf_pos_a;
    L[0].n_s = e.n;
    L[0].side = 1u;
    const V3<float> thr = e.L * e.cos_from_light / (e.pdf_dir_w * L[0].pdf_fwd);
    L[0].thr = e.L;
    const int n = random_walk(X, L, X.p->max_depth, thr, e.pdf_dir_w, e.wi, false, seed) + 1;
    if (light_delta(e.flags)) L[0].pdf_fwd = 0.0f;
    return n;
}

// bdpt_generate_camera_subpath(d, origin, max_depth + 1, cam_area)
int camera_subpath(const Ctx& X, PV* C, PV* L, V2<float> d, U4& seed) {
    C[0] = zero_pv();
    C[0].pos = X.c.pos;
    const V3<float> dir = sample_camera(X.c.iv, X.c.ip, d);
    C[0].area = X.c.area;
    C[0].thr = V3<float>(1.0f);
    C[0].n_s = X.c.nrm;
    C[0].side = 1u;
    L[0].mode = 1u;  // bdpt_commons.glsl:258 writes the light vertex's mode (never read)
    const float cos_theta = dot(dir, C[0].n_s);
    const float pdf = 1.0f / (X.c.area * X.screen * cos_theta * cos_theta * cos_theta);
    return random_walk(X, C, X.p->max_depth, V3<float>(1.0f), pdf, dir, true, seed) + 1;
}

struct Sampled {
    V3<float> pos, n_s;
    float pdf_fwd;
};

// calc_mis_weight (bdpt_commons.glsl:269-471) on copies of the two subpaths: the reference patches the
// path buffers in place and restores them afterwards.
float mis_weight(const Ctx& X, int s, int t, const Sampled& sampled, const PV* Lp, const PV* Cp) {
    if (s + t == 2 || (X.p->check_flags & 2u)) return 1.0f;
    PV L[130], C[130];
    for (int i = 0; i < s; i++) L[i] = Lp[i];
    for (int i = 0; i < t; i++) C[i] = Cp[i];
    if (s == 1) { L[0].pdf_fwd = sampled.pdf_fwd; L[0].pos = sampled.pos; L[0].n_s = sampled.n_s; }
    if (t == 1) { C[0].pdf_fwd = sampled.pdf_fwd; C[0].pos = sampled.pos; C[0].n_s = sampled.n_s; }
    if (t > 0) C[t - 1].delta = 0u;
    if (s > 0) L[s - 1].delta = 0u;
    if (t > 0) {
        if (s > 0) {
            V3<float> dir = C[t - 1].pos - L[s - 1].pos;
            const float dir_len = length(dir);
            dir /= dir_len;
            float pdf_rev = 0.0f;
            if (s >= 2) {
                const Mat<float> mat = load_material<float>(X.s, L[s - 1].material_idx, L[s - 1].uv);
                const V3<float> wo = normalize(L[s - 2].pos - L[s - 1].pos);
                pdf_rev = bsdf_pdf<float>(mat, L[s - 1].n_s, wo, dir, L[s - 1].side == 1u);
                pdf_rev *= std::fabs(dot(dir, C[t - 1].n_s)) / (dir_len * dir_len);
            } else {  // s == 1; finite lights only (directional lights are refused)
                pdf_rev = light_pdf(X, L[0].light_flags, L[0].n_s, dir);
                pdf_rev *= std::fabs(dot(dir, C[t - 1].n_s)) / (dir_len * dir_len);
            }
            C[t - 1].pdf_rev = pdf_rev;
        } else {
            C[t - 1].pdf_rev = 1.0f / ((float)X.p->light_triangle_count * C[t - 1].area);
        }
    }
    if (t > 1) {
        V3<float> dir = C[t - 2].pos - C[t - 1].pos;
        const float dir_len = length(dir);
        dir /= dir_len;
        if (s > 0) {
            const Mat<float> mat = load_material<float>(X.s, C[t - 1].material_idx, C[t - 1].uv);
            const V3<float> wo = normalize(L[s - 1].pos - C[t - 1].pos);
            C[t - 2].pdf_rev = bsdf_pdf<float>(mat, C[t - 1].n_s, wo, dir, C[t - 1].side == 1u);
            if (C[t - 2].pdf_rev != 0.0f) C[t - 2].pdf_rev *= std::fabs(dot(dir, C[t - 2].n_s)) / (dir_len * dir_len);
        } else {
            const float cos_x = dot(C[t - 1].n_s, dir);
            const float cos_y = dot(C[t - 2].n_s, dir);
            C[t - 2].pdf_rev = std::fabs(cos_x * cos_y) / (K<float>::PI() * dir_len * dir_len);
        }
    }
    if (s > 0) {
        V3<float> dir = L[s - 1].pos - C[t - 1].pos;
        const float dir_len = length(dir);
        dir /= dir_len;
        if (t == 1) {
            const float cos_theta = dot(C[0].n_s, dir);
            float pdf = 1.0f / (C[0].area * X.screen * cos_theta * cos_theta * cos_theta);
            pdf *= std::fabs(dot(dir, L[s - 1].n_s)) / (dir_len * dir_len);
            L[s - 1].pdf_rev = pdf;
        } else {
            const V3<float> wo = normalize(C[t - 2].pos - C[t - 1].pos);
            const Mat<float> mat = load_material<float>(X.s, C[t - 1].material_idx, C[t - 1].uv);
            L[s - 1].pdf_rev = bsdf_pdf<float>(mat, C[t - 1].n_s, wo, dir, C[t - 1].side == 1u);
            if ((s == 1 && light_finite(L[0].light_flags)) || s > 1)
                L[s - 1].pdf_rev *= std::fabs(dot(dir, L[s - 1].n_s)) / (dir_len * dir_len);
        }
    }
    if (s > 1) {
        V3<float> dir = L[s - 2].pos - L[s - 1].pos;
        const V3<float> wo = normalize(C[t - 1].pos - L[s - 1].pos);
        const float dir_len = length(dir);
        dir /= dir_len;
        const Mat<float> mat = load_material<float>(X.s, L[s - 1].material_idx, L[s - 1].uv);
        L[s - 2].pdf_rev = bsdf_pdf<float>(mat, L[s - 1].n_s, wo, dir, L[s - 1].side == 1u);
        if ((s == 2 && light_finite(L[0].light_flags)) || s > 2)
            L[s - 2].pdf_rev *= std::fabs(dot(dir, L[s - 2].n_s)) / (dir_len * dir_len);
    }
    float sum_ri = 0.0f;
    float weight = 1.0f;
    for (int i = t - 1; i > 0; i--) {
        weight *= remap0(C[i].pdf_rev) / remap0(C[i].pdf_fwd);
        if (C[i].delta == 0u && C[i - 1].delta == 0u) sum_ri += weight;
    }
    weight = 1.0f;
    for (int i = s - 1; i >= 0; i--) {
        weight *= remap0(L[i].pdf_rev) / remap0(L[i].pdf_fwd);
        const bool delta_prev = i > 0 ? L[i - 1].delta == 1u : light_delta(L[0].light_flags);
        if (L[i].delta == 0u && !delta_prev) sum_ri += weight;
    }
    return 1.0f / (1.0f + sum_ri);
}

bool occluded(const Scene& s, V3<float> o, V3<float> d, float tmax) {
    const float of[3] = {o.x, o.y, o.z}, df[3] = {d.x, d.y, d.z};
    return bvh_any(s.bvh, of, df, 0.0f, tmax);
}

// bdpt_connect_cam (bdpt_commons.glsl:473-526): the splat of light vertex s - 1 and its pixel (have = false: none)
V3<float> connect_cam(const Ctx& X, int s, const PV* L, const PV* C, int32_t& cx, int32_t& cy, bool& have) {
    have = false;
    Sampled sampled{V3<float>(0.0f), V3<float>(0.0f), 0.0f};
    V3<float> Lo(0.0f);
    V3<float> dir = C[0].pos - L[s - 1].pos;
    const float len = length(dir);
    dir /= len;
    const float cos_y = dot(dir, L[s - 1].n_s);
    const float cos_theta = dot(C[0].n_s, -dir);
    if (cos_theta <= 0.0f) return V3<float>(0.0f);
    const float cos_3_theta = cos_theta * cos_theta * cos_theta;
    const float cam_pdf_ratio = std::fabs(cos_y) / (C[0].area * cos_3_theta * len * len);
    const V3<float> ray_origin = offset_ray2(L[s - 1].pos, L[s - 1].n_s);
    const Mat<float> mat = load_material<float>(X.s, L[s - 1].material_idx, L[s - 1].uv);
    const V3<float> wo = normalize(L[s - 2].pos - L[s - 1].pos);
    float pdf, pdf_rev;
    const V3<float> f = eval_bsdf<float>(L[s - 1].n_s, wo, mat, L[s - 1].mode, L[s - 1].side == 1u, dir, pdf, pdf_rev, false);
    if (is_zero(f)) return Lo;
    if (cam_pdf_ratio > 0.0f) {
        if (!occluded(X.s, ray_origin, dir, len - EPS)) {
            sampled.pos = C[0].pos;
            sampled.n_s = C[0].n_s;
            Lo = L[s - 1].thr * cam_pdf_ratio * f / X.screen;
        }
    }
    dir = -dir;
    V4<float> t = X.c.view * V4<float>(dir.x, dir.y, dir.z, 0.0f);
    t = V4<float>(t.x / t.z, t.y / t.z, t.z / t.z, t.w / t.z);
    t = X.c.proj * t;
    t = V4<float>(-t.x, -t.y, -t.z, -t.w);
    cx = to_int_rz(0.5f * (1.0f + t.x) * (float)X.c.W - 0.5f);
    cy = to_int_rz(0.5f * (1.0f + t.y) * (float)X.c.H - 0.5f);
    if (cx < 0 || cx >= (int32_t)X.c.W || cy < 0 || cy >= (int32_t)X.c.H || dot(dir, C[0].n_s) < 0.0f)
        return V3<float>(0.0f);
    have = true;
    float mis = 1.0f;
    if (luminance(Lo) != 0.0f) mis = mis_weight(X, s, 1, sampled, L, C);
    return mis * Lo;
}

// bdpt_connect (bdpt_commons.glsl:528-639), t >= 2
V3<float> connect(const Ctx& X, int s, int t, const PV* L, const PV* C, U4& seed) {
    V3<float> Lo(0.0f);
    Sampled sampled{V3<float>(0.0f), V3<float>(0.0f), 0.0f};
    if (s == 0) {
        const uint32_t mat_idx = C[t - 1].material_idx;  // never -1: an escape vertex reads material 0
        const orc_material& m = X.s.mats[mat_idx];
        Lo = V3<float>(m.emissive_factor[0], m.emissive_factor[1], m.emissive_factor[2]) * C[t - 1].thr;
    } else if (s == 1) {
        const float q0 = rand(seed), q1 = rand(seed), q2 = rand(seed), q3 = rand(seed);
        const Incidence<float> li = sample_light_Li_pos<float>(X.s, V4<float>(q0, q1, q2, q3), C[t - 1].pos,
                                                                X.p->num_lights, X.cone);
        const float cos_x = std::fabs(dot(li.wi, C[t - 1].n_s));
        const V3<float> ray_origin = offset_ray2(C[t - 1].pos, C[t - 1].n_s);
        const V3<float> wo = normalize(C[t - 2].pos - C[t - 1].pos);
        const Mat<float> mat = load_material<float>(X.s, C[t - 1].material_idx, C[t - 1].uv);
        float pdf, pdf_rev;
        const V3<float> f = eval_bsdf<float>(C[t - 1].n_s, wo, mat, C[t - 1].mode, C[t - 1].side == 1u, li.wi, pdf, pdf_rev,
                                             false);
        if (!is_zero(f)) {
            if (!occluded(X.s, ray_origin, li.wi, li.wi_len - EPS)) {
                const float ltc = (float)X.p->light_triangle_count;
                const float pdf_light_w = light_pdf_a_to_w(li.flags, li.pdf_pos_a, li.wi_len * li.wi_len, li.cos_y) / ltc;
                sampled.pdf_fwd = li.pdf_pos_a / ltc;
                sampled.pos = li.pos;
                sampled.n_s = li.n;
                Lo = C[t - 1].thr * f * cos_x * li.L / pdf_light_w;
            }
        }
    } else {
        const V3<float> n_s = L[s - 1].n_s, n_t = C[t - 1].n_s;
        V3<float> d = L[s - 1].pos - C[t - 1].pos;
        const float len = length(d);
        d /= len;
        const float G = dot(n_s, -d) * dot(n_t, d) / (len * len);
        if (G > 0.0f) {
            const Mat<float> mat_1 = load_material<float>(X.s, C[t - 1].material_idx, C[t - 1].uv);
            const Mat<float> mat_2 = load_material<float>(X.s, L[s - 1].material_idx, L[s - 1].uv);
            const V3<float> wo_1 = normalize(C[t - 2].pos - C[t - 1].pos);
            const V3<float> wo_2 = normalize(L[s - 2].pos - L[s - 1].pos);
            float p0, p1;
            const V3<float> brdf1 = eval_bsdf<float>(n_t, wo_1, mat_1, C[t - 1].mode, C[t - 1].side == 1u, d, p0, p1, false);
            const V3<float> brdf2 = eval_bsdf<float>(n_s, wo_2, mat_2, L[s - 1].mode, L[s - 1].side == 1u, -d, p0, p1, false);
            if (!is_zero(brdf1) && !is_zero(brdf2)) {
                const V3<float> ray_origin = offset_ray2(C[t - 1].pos, C[t - 1].n_s);
                if (!occluded(X.s, ray_origin, d, len - EPS)) Lo = L[s - 1].thr * G * brdf1 * brdf2 * C[t - 1].thr;
            }
        }
    }
    if (luminance(Lo) != 0.0f) {
        const float mis = mis_weight(X, s, t, sampled, L, C);
        Lo *= mis;
    }
    return Lo;
}

struct PixelOut {
    V3<float> col;
    std::vector<std::pair<uint32_t, V3<float>>> splats;  // (row-major pixel, value) in strategy order
};

// bdpt.rgen main for pixel (x, y), without the splat read and the film write
void pixel(const Ctx& X, uint32_t x, uint32_t y, PixelOut& out) {
    const uint32_t per = (uint32_t)X.p->max_depth + 1u;
    std::vector<PV> Lv(per), Cv(per);
    U4 seed{x, y, X.p->frame_num ^ X.p->seed, 0u};
    const V2<float> px((float)x + 0.5f, (float)y + 0.5f);
    const V2<float> in_uv(px.x / (float)X.c.W, px.y / (float)X.c.H);
    const V2<float> d(in_uv.x * 2.0f - 1.0f, in_uv.y * 2.0f - 1.0f);
    const int nl = light_subpath(X, Lv.data(), seed);
    const int nc = camera_subpath(X, Cv.data(), Lv.data(), d, seed);
    out.col = V3<float>(0.0f);
    out.splats.clear();
    for (int t = 1; t <= nc; t++) {
        for (int s = 0; s <= nl; s++) {
            const int depth = s + t - 2;
            if (depth > X.p->max_depth - 1 || depth < 0 || (s == 1 && t == 1)) continue;
            if ((X.p->check_flags & 1u) &&
                (s + t - 1 != X.p->check_len || (X.p->check_s >= 0 && s != X.p->check_s))) {
                if (s == 1 && t >= 2) seed.w += 4u;  // the draws of bdpt_connect's light sample
                continue;
            }
            if (t == 1) {
                int32_t cx = 0, cy = 0;
                bool have = false;
                const V3<float> sc = connect_cam(X, s, Lv.data(), Cv.data(), cx, cy, have);
                if (luminance(sc) > 0.0f && have) out.splats.push_back({(uint32_t)cy * X.c.W + (uint32_t)cx, sc});
            } else {
                out.col += connect(X, s, t, Lv.data(), Cv.data(), seed);
            }
        }
    }
}

}  // namespace

extern "C" void orc_bdpt_iteration(void* scene, const float inv_view[16], const float inv_proj[16], const float view[16],
                                   const float proj[16], uint32_t width, uint32_t height, const orc_bdpt_params* p,
                                   float* film, float* splat, int nthreads) {
    const Scene& s = *static_cast<const Scene*>(scene);
    Cam c;
    c.iv = load_m4<float>(inv_view); c.ip = load_m4<float>(inv_proj); c.view = load_m4<float>(view); c.proj = load_m4<float>(proj);
    c.W = width; c.H = height;
    c.pos = (c.iv * V4<float>(0.0f, 0.0f, 0.0f, 1.0f)).xyz();
    const V4<float> fwd = c.iv * V4<float>(0.0f, 0.0f, 1.0f, 0.0f);
    c.nrm = V3<float>(-fwd.x, -fwd.y, -fwd.z);
    V4<float> a = c.ip * V4<float>(2.0f / (float)width, 2.0f / (float)height, 0.0f, 1.0f);
    a = V4<float>(a.x / a.w, a.y / a.w, a.z / a.w, a.w / a.w);
    c.area = std::fabs(a.x * a.y);
    const uint32_t screen = width * height;
    const Ctx X{s, p, c, spot_cone(p->spot_angle), (float)screen};
    std::vector<PixelOut> outs(screen);
    parallel_for(screen, nthreads, [&](uint32_t i) { pixel(X, i % width, i / width, outs[i]); });
    std::memset(splat, 0, sizeof(float) * 3 * (size_t)screen);
    for (uint32_t i = 0; i < screen; i++)
        for (const auto& sp : outs[i].splats) {
            float* q = splat + 3 * (size_t)sp.first;
            q[0] += sp.second.x; q[1] += sp.second.y; q[2] += sp.second.z;
        }
    for (uint32_t i = 0; i < screen; i++) {
        const float* q = splat + 3 * (size_t)i;
        const V3<float> col = outs[i].col + V3<float>(q[0], q[1], q[2]);
        if (std::isnan(luminance(col))) continue;  // bdpt.rgen:77-79: the film keeps its value
        float* px = film + 4 * (size_t)i;
        if (p->frame_num > 0u) {
            const float w = 1.0f / (float)(p->frame_num + 1u);
            const V3<float> m = mix(V3<float>(px[0], px[1], px[2]), col, w);
            px[0] = m.x; px[1] = m.y; px[2] = m.z; px[3] = 1.0f;
        } else {
            px[0] = col.x; px[1] = col.y; px[2] = col.z; px[3] = 1.0f;
        }
    }
}
