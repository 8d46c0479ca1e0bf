// Oracle (test infrastructure only): CPU restatement of Lumen's unidirectional MIS path integrator.
//
// Follows src/shaders/integrators/path/path.rgen:22-113 (camera ray, bounce loop, RR, film),
// src/shaders/integrators/pt_commons.glsl:3-48 (uniform_sample_light: NEE + BSDF-MIS),
// src/shaders/commons.glsl:30-33 (sample_camera), 112-149 (sample_triangle), 173-215 (sample_area_light),
// 224-300 (sample_light_Li), 156-168 (shade_atmosphere, sky colour only),
// src/shaders/ray.rchit:24-84 (hit attributes) and ray.rmiss:13 (miss marks material_idx = -1 only).
//
// Payload semantics are kept: a miss of the BSDF-MIS ray (pt_commons.glsl:32-33) leaves the previous
// closest-hit payload in place, so its triangle/instance ids and position are the ones compared and used.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "oracle.h"
#include "shading.h"

#include "scene_internal.h"

namespace {
using namespace orc;
using namespace orc::detail;

// One invocation of path.rgen main() for pixel (x, y) at frame params.frame_num. Returns col.
template <class T>
V3<T> path_sample(const Scene& s, const M4<T>& inv_view, const M4<T>& inv_proj, const orc_path_params& pc, uint32_t x,
                  uint32_t y) {
    U4 seed{x, y, pc.frame_num, 0u};  // init_rng (utils.glsl:142)
    const V2<T> pixel(T(x) + T(0.5f), T(y) + T(0.5f));
    float r0 = rand(seed);
    float r1 = rand(seed);
    V2<T> rands(T(r0) - T(0.5f), T(r1) - T(0.5f));
    const V2<T> in_uv((pixel.x + rands.x) / T(pc.size_x), (pixel.y + rands.y) / T(pc.size_y));
    V2<T> d(in_uv.x * T(2) - T(1), in_uv.y * T(2) - T(1));
    V4<T> origin = inv_view * V4<T>(T(0), T(0), T(0), T(1));
    V3<T> direction = sample_camera(inv_view, inv_proj, d);
    V3<T> col(0);
    bool last_specular = false;
    V3<T> throughput(1);
    Payload<T> payload;
    payload.material_idx = -1; payload.triangle_idx = 0xFFFFFFFFu; payload.instance_idx = 0xFFFFFFFFu;
    const V3<T> sky(pc.sky_col[0], pc.sky_col[1], pc.sky_col[2]);
    for (int depth = 0;; depth++) {
        trace_closest<T>(s, origin.xyz(), direction, TMIN, TMAX, payload);
        const bool found_isect = payload.material_idx != -1;
        if (!found_isect) {
            // shade_atmosphere with dir_light_idx == -1 returns sky_col (commons.glsl:157-159)
            if (depth > 0 || pc.direct_lighting == 1) col += throughput * sky;
            break;
        }
        const Mat<T> hit_mat = load_material<T>(s, (uint32_t)payload.material_idx, payload.uv);
        if ((depth == 0 && pc.direct_lighting == 1) || last_specular) col += throughput * hit_mat.emissive_factor;
        if (depth >= pc.max_depth - 1) break;
        const V3<T> wo = -direction;
        V3<T> n_s = payload.n_s;
        bool side = true;
        V3<T> n_g = payload.n_g;
        if (dot(payload.n_g, wo) < T(0)) n_g = -n_g;
        if (dot(n_g, payload.n_s) < T(0)) { n_s = -n_s; side = false; }
        {
            V3<float> pf((float)payload.pos.x, (float)payload.pos.y, (float)payload.pos.z);
            V3<float> nf((float)n_g.x, (float)n_g.y, (float)n_g.z);
            V3<float> of = offset_ray(pf, nf);
            origin = V4<T>(T(of.x), T(of.y), T(of.z), origin.w);
        }
        last_specular = (hit_mat.bsdf_props & BSDF_FLAG_SPECULAR) != 0;
        if (!last_specular) {
            const T light_pick_pdf = T(1) / T(pc.light_triangle_count);
            if ((depth > 0 || pc.direct_lighting == 1) && pc.num_lights <= 0) {
                // No light to sample (Lumen would read past its light buffer): consume the four draws only.
                for (int k = 0; k < 4; k++) (void)rand(seed);
            } else if (depth > 0 || pc.direct_lighting == 1) {
                // uniform_sample_light (pt_commons.glsl:3-42)
                const V3<T> pos = payload.pos;
                V3<T> res(0);
                float q0 = rand(seed), q1 = rand(seed), q2 = rand(seed), q3 = rand(seed);
                LightSample<T> ls = sample_light_Li<T>(s, V4<T>(T(q0), T(q1), T(q2), T(q3)), pos, pc.num_lights);
                const V3<T> p = offset_ray2(pos, n_s);
                T bsdf_pdf, unused_rev;
                T cos_x = dot(n_s, ls.wi);
                V3<T> f = eval_bsdf(n_s, wo, hit_mat, 1u, side, ls.wi, bsdf_pdf, unused_rev, false);
                float pf[3] = {(float)p.x, (float)p.y, (float)p.z};
                float wf[3] = {(float)ls.wi.x, (float)ls.wi.y, (float)ls.wi.z};
                bool visible = !bvh_any(s.bvh, pf, wf, 0.0f, (float)(ls.wi_len - T(EPS)));
                if (visible && ls.pdf_pos_w > T(0)) {
                    const T mis_weight = ((ls.flags >> 5) & 1u) ? T(1) : T(1) / (T(1) + bsdf_pdf / ls.pdf_pos_w);
                    res += mis_weight * f * std::fabs(cos_x) * ls.L / ls.pdf_pos_w;
                }
                if ((ls.flags & 0x7) == LIGHT_AREA) {
                    V3<T> wi;
                    float b0 = rand(seed), b1 = rand(seed), b2 = rand(seed);
                    f = sample_bsdf(n_s, wo, hit_mat, 1u, side, wi, bsdf_pdf, cos_x, V3<T>(T(b0), T(b1), T(b2)));
                    if (bsdf_pdf != T(0)) {
                        trace_closest<T>(s, p, wi, TMIN, TMAX, payload);
                        if (payload.triangle_idx == ls.triangle_idx && payload.instance_idx == ls.instance_idx) {
                            const T wl = length(payload.pos - pos);
                            const T g = std::fabs(dot(payload.n_s, -wi)) / (wl * wl);
                            const T mis_weight = T(1) / (T(1) + ls.pdf_pos_a / (g * bsdf_pdf));
                            res += f * mis_weight * std::fabs(cos_x) * ls.L / bsdf_pdf;
                        }
                    }
                }
                col += throughput * res / light_pick_pdf;
            }
        }
        T pdf, cos_theta;
        float c0 = rand(seed), c1 = rand(seed), c2 = rand(seed);
        const V3<T> f = sample_bsdf(n_s, wo, hit_mat, 1u, side, direction, pdf, cos_theta, V3<T>(T(c0), T(c1), T(c2)));
        if (pdf == T(0)) break;
        throughput *= f * std::fabs(cos_theta) / pdf;
        T rr_scale = T(1);
        if (bsdf_has_property(hit_mat.bsdf_props, BSDF_FLAG_TRANSMISSION)) rr_scale *= side ? T(1) / hit_mat.ior : hit_mat.ior;
        if (depth > RR_MIN_DEPTH) {
            T rr_prob = gmin(T(0.95f), luminance(throughput) * rr_scale);
            if (rr_prob == T(0) || rr_prob < T(rand(seed))) break;
            else throughput /= rr_prob;
        }
    }
    return col;
}

// ---------------- differentiable estimator (test support for the adjoint kernels) ----------------
// The path estimator with sampling detached from the parameters: directions, pdfs, MIS weights and Russian
// roulette use the scene's materials; BSDF values and emission use the parameter arrays (texels of one
// texture, roughness per material, RGB emission per material). Used to take central finite differences with
// common random numbers.
struct DiffParams {
    int tex_id;
    const float* texels;  // W*H*4 or null
    uint32_t tex_w, tex_h;
    const float* rough;   // per material or null
    const float* emis;    // 3 per material or null
};

template <class T> V3<T> bilinear_param(const DiffParams& dp, V2<T> uv) {
    if (!std::isfinite(uv.x) || !std::isfinite(uv.y)) uv = V2<T>(0, 0);
    T x = uv.x * T(dp.tex_w) - T(0.5f), y = uv.y * T(dp.tex_h) - T(0.5f);
    T x0 = std::floor(x), y0 = std::floor(y);
    T fx = x - x0, fy = y - y0;
    auto wrap = [](long long i, uint32_t n) { long long m = i % (long long)n; return (uint32_t)(m < 0 ? m + n : m); };
    uint32_t i0 = wrap((long long)x0, dp.tex_w), i1 = wrap((long long)x0 + 1, dp.tex_w);
    uint32_t j0 = wrap((long long)y0, dp.tex_h), j1 = wrap((long long)y0 + 1, dp.tex_h);
    auto texel = [&](uint32_t i, uint32_t j) {
        const float* p = &dp.texels[4 * ((size_t)j * dp.tex_w + i)];
        return V3<T>(p[0], p[1], p[2]);
    };
    V3<T> c00 = texel(i0, j0), c10 = texel(i1, j0), c01 = texel(i0, j1), c11 = texel(i1, j1);
    T w00 = (T(1) - fx) * (T(1) - fy), w10 = fx * (T(1) - fy), w01 = (T(1) - fx) * fy, w11 = fx * fy;
    return c00 * w00 + c10 * w10 + c01 * w01 + c11 * w11;
}

template <class T> V3<T> eval_value(const Mat<T>& me, V3<T> n_s, V3<T> wo, V3<T> wi, V3<T> fallback, bool from_sample) {
    V3<T> Tt, B;
    branchless_onb(n_s, Tt, B);
    V3<T> wol = to_local(wo, Tt, B, n_s), wil = to_local(wi, Tt, B, n_s);
    if (me.bsdf_type == BSDF_TYPE_DIFFUSE) {
        T pdf, rev;
        V3<T> f = eval_diffuse(me, wol, wil, pdf, rev);
        return (from_sample && fallback.x == T(0) && fallback.y == T(0) && fallback.z == T(0)) ? V3<T>(0) : f;
    }
    if (me.bsdf_type == BSDF_TYPE_CONDUCTOR && !bsdf_is_effectively_delta(me.roughness * me.roughness)) {
        T pdf, rev;
        return eval_conductor(me, wol, wil, pdf, rev, false);
    }
    return fallback;
}

template <class T>
V3<T> diff_sample(const Scene& s, const M4<T>& inv_view, const M4<T>& inv_proj, const orc_path_params& pc,
                  const DiffParams& dp, uint32_t x, uint32_t y) {
    U4 seed{x, y, pc.frame_num, 0u};
    const V2<T> pixel(T(x) + T(0.5f), T(y) + T(0.5f));
    float r0 = rand(seed);
    float r1 = rand(seed);
    V2<T> rands(T(r0) - T(0.5f), T(r1) - T(0.5f));
    const V2<T> in_uv((pixel.x + rands.x) / T(pc.size_x), (pixel.y + rands.y) / T(pc.size_y));
    V2<T> d(in_uv.x * T(2) - T(1), in_uv.y * T(2) - T(1));
    V4<T> origin = inv_view * V4<T>(T(0), T(0), T(0), T(1));
    V3<T> direction = sample_camera(inv_view, inv_proj, d);
    V3<T> L(0), Tv(1), Tc(1);
    bool last_spec = false;
    Payload<T> payload;
    payload.material_idx = -1; payload.triangle_idx = 0xFFFFFFFFu; payload.instance_idx = 0xFFFFFFFFu;
    const V3<T> sky(pc.sky_col[0], pc.sky_col[1], pc.sky_col[2]);
    for (int depth = 0; depth < 16; depth++) {
        trace_closest<T>(s, origin.xyz(), direction, TMIN, TMAX, payload);
        if (payload.material_idx == -1) {
            if (depth > 0 || pc.direct_lighting == 1) L += Tv * sky;
            break;
        }
        const uint32_t mi = (uint32_t)payload.material_idx;
        const Mat<T> ms = load_material<T>(s, mi, payload.uv);
        Mat<T> me = ms;
        if (dp.texels && s.mats[mi].texture_id >= 0 && s.mats[mi].texture_id == dp.tex_id)
            me.albedo = V3<T>(s.mats[mi].albedo[0], s.mats[mi].albedo[1], s.mats[mi].albedo[2]) * bilinear_param<T>(dp, payload.uv);
        if (dp.rough) me.roughness = T(dp.rough[mi]);
        if (dp.emis) me.emissive_factor = V3<T>(dp.emis[3 * mi], dp.emis[3 * mi + 1], dp.emis[3 * mi + 2]);
        if ((depth == 0 && pc.direct_lighting == 1) || last_spec) L += Tv * me.emissive_factor;
        if (depth >= pc.max_depth - 1) break;
        const V3<T> wo = -direction;
        V3<T> n_s = payload.n_s;
        bool side = true;
        V3<T> n_g = payload.n_g;
        if (dot(payload.n_g, wo) < T(0)) n_g = -n_g;
        if (dot(n_g, payload.n_s) < T(0)) { n_s = -n_s; side = false; }
        const uint32_t shade_tri = payload.triangle_idx, shade_inst = payload.instance_idx;
        const V3<T> shade_pos = payload.pos, shade_ns = payload.n_s;
        {
            V3<float> pf((float)payload.pos.x, (float)payload.pos.y, (float)payload.pos.z);
            V3<float> nf((float)n_g.x, (float)n_g.y, (float)n_g.z);
            V3<float> of = offset_ray(pf, nf);
            origin = V4<T>(T(of.x), T(of.y), T(of.z), origin.w);
        }
        const bool spec = (ms.bsdf_props & BSDF_FLAG_SPECULAR) != 0;
        if (!spec && (depth > 0 || pc.direct_lighting == 1)) {
            if (pc.num_lights <= 0) {
                for (int k = 0; k < 4; k++) (void)rand(seed);
            } else {
                const T lpp = T(1) / T(pc.light_triangle_count);
                float q0 = rand(seed), q1 = rand(seed), q2 = rand(seed), q3 = rand(seed);
                LightSample<T> ls = sample_light_Li<T>(s, V4<T>(T(q0), T(q1), T(q2), T(q3)), shade_pos, pc.num_lights);
                const orc_light& lt = s.lights[(uint32_t)(T(q0) * T(pc.num_lights))];
                V3<T> Le = ls.L;
                if ((ls.flags & 0x7) == LIGHT_AREA && dp.emis) {
                    const uint32_t lm = s.meshes[lt.prim_mesh_idx].material_index;
                    Le = V3<T>(dp.emis[3 * lm], dp.emis[3 * lm + 1], dp.emis[3 * lm + 2]);
                }
                const V3<T> p = offset_ray2(shade_pos, n_s);
                T bsdf_pdf, unused_rev;
                T cos_x = dot(n_s, ls.wi);
                V3<T> fs1 = eval_bsdf(n_s, wo, ms, 1u, side, ls.wi, bsdf_pdf, unused_rev, false);
                V3<T> fe1 = eval_value(me, n_s, wo, ls.wi, fs1, false);
                V3<T> res(0);
                float pf[3] = {(float)p.x, (float)p.y, (float)p.z};
                float wf[3] = {(float)ls.wi.x, (float)ls.wi.y, (float)ls.wi.z};
                if (ls.pdf_pos_w > T(0) && !bvh_any(s.bvh, pf, wf, 0.0f, (float)(ls.wi_len - T(EPS)))) {
                    const T mis = ((ls.flags >> 5) & 1u) ? T(1) : T(1) / (T(1) + bsdf_pdf / ls.pdf_pos_w);
                    res += mis * fe1 * std::fabs(cos_x) / ls.pdf_pos_w * Le;
                }
                if ((ls.flags & 0x7) == LIGHT_AREA) {
                    V3<T> wi;
                    float b0 = rand(seed), b1 = rand(seed), b2 = rand(seed);
                    V3<T> fs2 = sample_bsdf(n_s, wo, ms, 1u, side, wi, bsdf_pdf, cos_x, V3<T>(T(b0), T(b1), T(b2)));
                    if (bsdf_pdf != T(0)) {
                        trace_closest<T>(s, p, wi, TMIN, TMAX, payload);
                        uint32_t hit_tri = payload.triangle_idx, hit_inst = payload.instance_idx;
                        V3<T> hpos = payload.pos, hns = payload.n_s;
                        if (payload.material_idx == -1) { hit_tri = shade_tri; hit_inst = shade_inst; hpos = shade_pos; hns = shade_ns; }
                        if (hit_tri == ls.triangle_idx && hit_inst == ls.instance_idx) {
                            const T wl = length(hpos - shade_pos);
                            const T g = std::fabs(dot(hns, -wi)) / (wl * wl);
                            const T mis = T(1) / (T(1) + ls.pdf_pos_a / (g * bsdf_pdf));
                            V3<T> fe2 = eval_value(me, n_s, wo, wi, fs2, true);
                            res += fe2 * mis * std::fabs(cos_x) / bsdf_pdf * Le;
                        }
                    }
                }
                L += Tv * res / lpp;
            }
        }
        T pdf, cos_theta;
        float c0 = rand(seed), c1 = rand(seed), c2 = rand(seed);
        V3<T> dnext;
        const V3<T> fs = sample_bsdf(n_s, wo, ms, 1u, side, dnext, pdf, cos_theta, V3<T>(T(c0), T(c1), T(c2)));
        if (pdf == T(0)) break;
        const V3<T> fe = eval_value(me, n_s, wo, dnext, fs, true);
        Tv *= fe * std::fabs(cos_theta) / pdf;
        Tc *= fs * std::fabs(cos_theta) / pdf;
        T rr_scale = T(1);
        if (bsdf_has_property(ms.bsdf_props, BSDF_FLAG_TRANSMISSION)) rr_scale *= side ? T(1) / ms.ior : ms.ior;
        if (depth > RR_MIN_DEPTH) {
            // Russian roulette on the FP32 detached throughput in both precisions, so that the same paths survive
            float rr = std::fmin(0.95f, (float)luminance(Tc) * (float)rr_scale);
            if (rr == 0.0f || rr < rand(seed)) break;
            Tv /= T(rr);
            Tc /= T(rr);
        }
        direction = dnext;
        last_spec = spec;
    }
    return L;
}

}  // namespace

extern "C" {

void* orc_scene_create(const orc_scene_desc* d) {
    Scene* s = new Scene();
    s->pos.assign(d->positions, d->positions + 3 * (size_t)d->num_vertices);
    s->nrm.assign(d->normals, d->normals + 3 * (size_t)d->num_vertices);
    s->uv.assign(d->uvs, d->uvs + 2 * (size_t)d->num_vertices);
    s->idx.assign(d->indices, d->indices + d->num_indices);
    s->meshes.assign(d->meshes, d->meshes + d->num_meshes);
    s->mats.assign(d->materials, d->materials + d->num_materials);
    s->lights.assign(d->lights, d->lights + d->num_lights);
    for (uint32_t i = 0; i < d->num_textures; i++) {
        Scene::Tex t;
        t.w = d->textures[i].width; t.h = d->textures[i].height;
        t.rgba.assign(d->textures[i].rgba, d->textures[i].rgba + 4 * (size_t)t.w * t.h);
        s->texs.push_back(std::move(t));
    }
    // Flatten: global triangle g of mesh m has index triple at index_offset + 3 * local.
    std::vector<float> tv;
    for (uint32_t m = 0; m < d->num_meshes; m++) {
        s->mesh_first_tri.push_back((uint32_t)s->tri_mesh.size());
        const orc_mesh& pm = d->meshes[m];
        for (uint32_t t = 0; t < pm.tri_count; t++) {
            s->tri_mesh.push_back(m);
            for (int k = 0; k < 3; k++) {
                uint32_t v = d->indices[pm.index_offset + 3 * t + k] + pm.vertex_offset;
                tv.push_back(d->positions[3 * v]); tv.push_back(d->positions[3 * v + 1]); tv.push_back(d->positions[3 * v + 2]);
            }
        }
    }
    s->bvh = orc::bvh_build_internal(tv.data(), (uint32_t)s->tri_mesh.size());
    return s;
}

void orc_bvh_free(void* bvh);
void orc_scene_free(void* h) {
    Scene* s = (Scene*)h;
    if (s->bvh) orc_bvh_free(s->bvh);
    delete s;
}

void orc_render_samples(void* h, const float inv_view[16], const float inv_proj[16], const orc_path_params* params,
                        const uint32_t* pixels, uint32_t n_pixels, float* out_rgb, uint8_t* out_nan, int fp64,
                        int nthreads) {
    const Scene& s = *(Scene*)h;
    parallel_for(n_pixels, nthreads, [&](uint32_t i) {
        uint32_t pix = pixels[i];
        uint32_t x = pix % params->size_x, y = pix / params->size_x;
        double c[3];
        if (fp64) {
            V3<double> col = path_sample<double>(s, load_m4<double>(inv_view), load_m4<double>(inv_proj), *params, x, y);
            c[0] = col.x; c[1] = col.y; c[2] = col.z;
            out_nan[i] = std::isnan(luminance(col)) ? 1 : 0;
        } else {
            V3<float> col = path_sample<float>(s, load_m4<float>(inv_view), load_m4<float>(inv_proj), *params, x, y);
            c[0] = col.x; c[1] = col.y; c[2] = col.z;
            out_nan[i] = std::isnan(luminance(col)) ? 1 : 0;
        }
        out_rgb[3 * i] = (float)c[0]; out_rgb[3 * i + 1] = (float)c[1]; out_rgb[3 * i + 2] = (float)c[2];
    });
}

// Converged reference renders: the plain FP64 mean of the samples of frames [frame0, frame0 + spp) per pixel
// (NaN samples skipped), into out (npix * 3 doubles). Unlike the progressive film it does not assume the frames
// start at 0, so a reference can use frames the renders it is compared with do not.
void orc_render_mean_f64(void* h, const float inv_view[16], const float inv_proj[16], const orc_path_params* params,
                         uint32_t frame0, uint32_t spp, double* out, int nthreads) {
    const Scene& s = *(Scene*)h;
    const uint32_t n = params->size_x * params->size_y;
    parallel_for(n, nthreads, [&](uint32_t pix) {
        const uint32_t x = pix % params->size_x, y = pix / params->size_x;
        orc_path_params pc = *params;
        double sum[3] = {0.0, 0.0, 0.0};
        uint32_t valid = 0;
        for (uint32_t f = frame0; f < frame0 + spp; f++) {
            pc.frame_num = f;
            const V3<double> col = path_sample<double>(s, load_m4<double>(inv_view), load_m4<double>(inv_proj), pc, x, y);
            if (std::isnan(luminance(col))) continue;
            sum[0] += col.x; sum[1] += col.y; sum[2] += col.z;
            valid++;
        }
        for (int k = 0; k < 3; k++) out[3 * (size_t)pix + k] = valid ? sum[k] / valid : 0.0;
    });
}

void orc_render_film(void* h, const float inv_view[16], const float inv_proj[16], const orc_path_params* params,
                     uint32_t frame0, uint32_t spp, float* film, int fp64, int nthreads) {
    const Scene& s = *(Scene*)h;
    uint32_t n = params->size_x * params->size_y;
    parallel_for(n, nthreads, [&](uint32_t pix) {
        uint32_t x = pix % params->size_x, y = pix / params->size_x;
        orc_path_params pc = *params;
        for (uint32_t f = frame0; f < frame0 + spp; f++) {
            pc.frame_num = f;
            float* px = &film[4 * (size_t)pix];
            if (fp64) {
                V3<double> col = path_sample<double>(s, load_m4<double>(inv_view), load_m4<double>(inv_proj), pc, x, y);
                if (std::isnan(luminance(col))) continue;
                if (f > 0) {
                    double w = 1.0 / double(f + 1);
                    for (int k = 0; k < 3; k++) px[k] = (float)(px[k] * (1.0 - w) + (&col.x)[k] * w);
                } else {
                    px[0] = (float)col.x; px[1] = (float)col.y; px[2] = (float)col.z;
                }
                px[3] = 1.0f;
            } else {
                V3<float> col = path_sample<float>(s, load_m4<float>(inv_view), load_m4<float>(inv_proj), pc, x, y);
                if (std::isnan(luminance(col))) continue;
                if (f > 0) {
                    // path.rgen:107-109: w = 1 / float(frame + 1); mix(old, col, w)
                    float w = 1.0f / float(f + 1);
                    V3<float> old(px[0], px[1], px[2]);
                    V3<float> m = mix(old, col, w);
                    px[0] = m.x; px[1] = m.y; px[2] = m.z;
                } else {
                    px[0] = col.x; px[1] = col.y; px[2] = col.z;
                }
                px[3] = 1.0f;
            }
        }
    });
}

// Mean image of the differentiable estimator over frames [frame0, frame0 + spp): film_rgb gets npix * 3
// doubles. texels (W*H*4 floats of texture tex_id), rough (per material), emis (3 per material) may be null.
void orc_render_diff(void* h, const float inv_view[16], const float inv_proj[16], const orc_path_params* params,
                     int tex_id, const float* texels, const float* rough, const float* emis, uint32_t frame0, uint32_t spp,
                     double* film_rgb, int fp64, int nthreads) {
    const Scene& s = *(Scene*)h;
    DiffParams dp;
    dp.tex_id = texels ? tex_id : -1;
    dp.texels = texels;
    dp.tex_w = (texels && tex_id >= 0) ? s.texs[tex_id].w : 0;
    dp.tex_h = (texels && tex_id >= 0) ? s.texs[tex_id].h : 0;
    dp.rough = rough;
    dp.emis = emis;
    uint32_t n = params->size_x * params->size_y;
    parallel_for(n, nthreads, [&](uint32_t pix) {
        uint32_t x = pix % params->size_x, y = pix / params->size_x;
        orc_path_params pc = *params;
        double acc[3] = {0, 0, 0};
        for (uint32_t f = frame0; f < frame0 + spp; f++) {
            pc.frame_num = f;
            if (fp64) {
                V3<double> c = diff_sample<double>(s, load_m4<double>(inv_view), load_m4<double>(inv_proj), pc, dp, x, y);
                acc[0] += c.x; acc[1] += c.y; acc[2] += c.z;
            } else {
                V3<float> c = diff_sample<float>(s, load_m4<float>(inv_view), load_m4<float>(inv_proj), pc, dp, x, y);
                acc[0] += c.x; acc[1] += c.y; acc[2] += c.z;
            }
        }
        for (int k = 0; k < 3; k++) film_rgb[3 * (size_t)pix + k] = acc[k] / (double)spp;
    });
}

void orc_pcg4d(const uint32_t* in, uint32_t* out, uint32_t n) {
    for (uint32_t i = 0; i < n; i++) {
        U4 v{in[4 * i], in[4 * i + 1], in[4 * i + 2], in[4 * i + 3]};
        U4 r = pcg4d(v);
        out[4 * i] = r.x; out[4 * i + 1] = r.y; out[4 * i + 2] = r.z; out[4 * i + 3] = r.w;
    }
}

void orc_offset_ray(const float* p, const float* nrm, float* out, uint32_t n) {
    for (uint32_t i = 0; i < n; i++) {
        V3<float> r = offset_ray(V3<float>(p[3 * i], p[3 * i + 1], p[3 * i + 2]), V3<float>(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]));
        out[3 * i] = r.x; out[3 * i + 1] = r.y; out[3 * i + 2] = r.z;
    }
}

}  // extern "C"
