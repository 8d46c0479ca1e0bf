// Oracle (test infrastructure only): CPU restatement of Lumen's SPPM integrator, one frame of SPPM::render
// (src/RayTracer/SPPM.cpp:78-184) with its passes in order:
//   eye pass      src/shaders/integrators/sppm/sppm_eye.rgen:44-127 (light sampling of pt_commons.glsl:3-42)
//   grid bounds   min.comp / max.comp / reduce_*.comp (min of p - r, max of p + r over every pixel, max r) and
//                 calc_bounds.comp (the grid resolution)
//   light pass    sppm_light.rgen:44-113 (photons from the second hit on)
//   photon table  sppm_light.rgen:86-93, written sequentially in photon order (light path * max_depth + bounce):
//                 per hash slot the photon count and the last photon
//   gather        gather.comp:43-86
//   composite     composite.comp:33-60
// Semantics kept and deviations are those of the library's kernels: the seed is a parameter, the photon table
// keeps the last photon in photon order, and a pixel whose cell range exceeds 16 cells per axis does not gather.
// The state layouts are the library's: a visible point is 8 float4 (p, radius | wo, N | n_s, u | throughput, v |
// col, M | phi, material | tau, path_len | side), a photon 4 float4 (pos, path_len | wi | throughput | n_s).
#include <cstdint>
#include <cstring>
#include <vector>

#include "photon_common.h"
#include "scene_internal.h"

namespace {
using namespace orc;
using namespace orc::detail;
using namespace orc::photon;

constexpr int kMaxGatherCells = 16;

inline uint32_t fb(float x) { uint32_t u; std::memcpy(&u, &x, 4); return u; }
inline float bf(uint32_t u) { float x; std::memcpy(&x, &u, 4); return x; }

// uniform_sample_light (pt_commons.glsl:3-42); `payload` holds the shading point's hit and is overwritten by the
// BSDF-MIS ray as in the shader (a miss leaves it in place).
V3<float> uniform_sample_light(const Scene& s, U4& seed, const Mat<float>& mat, V3<float> pos, bool side, V3<float> n_s,
                               V3<float> wo, Payload<float>& payload, int num_lights, Cone cone) {
    V3<float> res(0);
    const float q0 = rand(seed), q1 = rand(seed), q2 = rand(seed), q3 = rand(seed);
    const LightSample<float> ls =
        sample_light_Li<float>(s, V4<float>(q0, q1, q2, q3), pos, num_lights, cone.cos_width, cone.cos_falloff);
    const V3<float> p = offset_ray2(pos, n_s);
    float bsdf_pdf, unused_rev;
    float cos_x = dot(n_s, ls.wi);
    V3<float> f = eval_bsdf(n_s, wo, mat, 1u, side, ls.wi, bsdf_pdf, unused_rev, false);
    float pf[3] = {p.x, p.y, p.z};
    float wf[3] = {ls.wi.x, ls.wi.y, ls.wi.z};
    const bool visible = !bvh_any(s.bvh, pf, wf, 0.0f, ls.wi_len - EPS);
    if (visible && ls.pdf_pos_w > 0.0f) {
        const float mis = ((ls.flags >> 5) & 1u) ? 1.0f : 1.0f / (1.0f + bsdf_pdf / ls.pdf_pos_w);
        res += mis * f * std::fabs(cos_x) * ls.L / ls.pdf_pos_w;
    }
    if ((ls.flags & 0x7u) == LIGHT_AREA) {
        V3<float> wi;
        const float b0 = rand(seed), b1 = rand(seed), b2 = rand(seed);
        f = sample_bsdf(n_s, wo, mat, 1u, side, wi, bsdf_pdf, cos_x, V3<float>(b0, b1, b2));
        if (bsdf_pdf != 0.0f) {
            trace_closest<float>(s, p, wi, TMIN, TMAX, payload);
            if (payload.triangle_idx == ls.triangle_idx && payload.instance_idx == ls.instance_idx) {
                const float wl = length(payload.pos - pos);
                const float g = std::fabs(dot(payload.n_s, -wi)) / (wl * wl);
                const float mis = 1.0f / (1.0f + ls.pdf_pos_a / (g * bsdf_pdf));
                res += f * mis * std::fabs(cos_x) * ls.L / bsdf_pdf;
            }
        }
    }
    return res;
}

// sppm_eye.rgen:44-127 for pixel (x, y); vp is that pixel's 32 floats.
void eye_path(const Scene& s, const M4<float>& iv, const M4<float>& ip, const orc_sppm_params* p, Cone cone, uint32_t x,
              uint32_t y, uint32_t W, uint32_t H, float* vp) {
    U4 seed{x, y, p->frame_num ^ p->seed, 0u};
    const V2<float> pixel((float)x + 0.5f, (float)y + 0.5f);
    const V2<float> in_uv(pixel.x / (float)W, pixel.y / (float)H);
    const V2<float> d(in_uv.x * 2.0f - 1.0f, in_uv.y * 2.0f - 1.0f);
    V3<float> origin = (iv * V4<float>(0.0f, 0.0f, 0.0f, 1.0f)).xyz();
    V3<float> direction = sample_camera(iv, ip, d);
    V3<float> throughput(1.0f), col(vp[16], vp[17], vp[18]);
    const V3<float> sky(p->sky_col[0], p->sky_col[1], p->sky_col[2]);
    bool specular = false, recorded = false;
    Payload<float> payload;
    payload.material_idx = -1; payload.triangle_idx = 0xFFFFFFFFu; payload.instance_idx = 0xFFFFFFFFu;
    for (int dd = 0;; dd++) {
        trace_closest<float>(s, origin, direction, TMIN, TMAX, payload);
        if (payload.material_idx == -1) {
            col += throughput * sky;
            break;
        }
        if (dd >= p->max_depth - 1) break;
        const uint32_t mat_idx = (uint32_t)payload.material_idx;
        const V2<float> mat_uv = payload.uv;
        const Mat<float> hit_mat = load_material<float>(s, mat_idx, mat_uv);
        if (dd == 0 || (specular && !recorded)) col += throughput * hit_mat.emissive_factor;
        const V3<float> wo = -direction;
        V3<float> n_s = payload.n_s, n_g = payload.n_g;
        bool side = true;
        if (dot(payload.n_g, wo) < 0.0f) n_g = -n_g;
        if (dot(n_g, payload.n_s) < 0.0f) { n_s = -n_s; side = false; }
        const V3<float> pos = payload.pos;
        origin = offset_ray(pos, n_g);
        specular = (hit_mat.bsdf_props & BSDF_FLAG_SPECULAR) != 0;
        if (!recorded && !specular) {
            const float light_pick_pdf = 1.0f / (float)p->light_triangle_count;
            col += throughput * uniform_sample_light(s, seed, hit_mat, pos, side, n_s, wo, payload, p->num_lights, cone) /
                   light_pick_pdf;
        }
        if (!recorded && (hit_mat.bsdf_type & BSDF_TYPE_DIFFUSE) != 0) {
            recorded = true;
            vp[0] = pos.x; vp[1] = pos.y; vp[2] = pos.z;
            vp[4] = wo.x; vp[5] = wo.y; vp[6] = wo.z;
            vp[8] = n_s.x; vp[9] = n_s.y; vp[10] = n_s.z; vp[11] = mat_uv.x;
            vp[12] = throughput.x; vp[13] = throughput.y; vp[14] = throughput.z; vp[15] = mat_uv.y;
            vp[23] = bf(mat_idx);
            vp[27] = bf((uint32_t)dd);
            vp[28] = bf(side ? 1u : 0u); vp[29] = 0.0f; vp[30] = 0.0f; vp[31] = 0.0f;
        }
        float pdf, cos_theta;
        const float c0 = rand(seed), c1 = rand(seed), c2 = rand(seed);
        const V3<float> f = sample_bsdf(n_s, wo, hit_mat, 1u, side, direction, pdf, cos_theta, V3<float>(c0, c1, c2));
        if (pdf < 1e-20f || dot(f, f) < 1e-20f) break;
        throughput *= f * std::fabs(cos_theta) / pdf;
        if (dd > RR_MIN_DEPTH) {
            const float rr = luminance(throughput);
            if (rr < rand(seed)) break;
            throughput /= rr;
        }
    }
    vp[16] = col.x; vp[17] = col.y; vp[18] = col.z;
    if (p->frame_num == 0u) vp[3] = std::max(p->base_radius, 1e-7f);
}

// sppm_light.rgen:44-113 for light path li = x * H + y; ph is its max_depth photon slots (16 floats each).
void light_path(const Scene& s, const orc_sppm_params* p, Cone cone, uint32_t x, uint32_t y, float* ph) {
    for (int k = 0; k < p->max_depth; k++) std::memset(ph + 16 * k, 0, 4 * sizeof(float));
    U4 seed{x, y, p->frame_num ^ p->seed, 0u};
    const float r0 = rand(seed), r1 = rand(seed), r2 = rand(seed), r3 = rand(seed);
    const float d0 = rand(seed), d1 = rand(seed);
    const Emission<float> e = sample_light_Le<float>(s, V4<float>(r0, r1, r2, r3), V2<float>(d0, d1), p->num_lights,
                                                     p->light_triangle_count, cone);
    const float abs_cos_light = std::fabs(dot(e.n, e.wi));
    V3<float> thr = (abs_cos_light == 0.0f || e.pdf_dir_w <= 0.0f) ? V3<float>(0.0f)
                                                                     : e.L * abs_cos_light / (e.pdf_dir_w * e.pdf_pos_a);
    V3<float> pos = e.pos, wi = e.wi;
    Payload<float> payload;
    payload.material_idx = -1; payload.triangle_idx = 0xFFFFFFFFu; payload.instance_idx = 0xFFFFFFFFu;
    for (int d = 0; d < p->max_depth; d++) {
        trace_closest<float>(s, pos, wi, TMIN, TMAX, payload);
        if (payload.material_idx == -1) break;
        const V3<float> wo = -wi;
        V3<float> n_s = payload.n_s, n_g = payload.n_g;
        bool side = true;
        if (dot(payload.n_g, wo) < 0.0f) n_g = -n_g;
        if (dot(n_g, payload.n_s) < 0.0f) { n_s = -n_s; side = false; }
        const Mat<float> hit_mat = load_material<float>(s, (uint32_t)payload.material_idx, payload.uv);
        if (d > 0) {
            float* q = ph + 16 * d;
            q[0] = payload.pos.x; q[1] = payload.pos.y; q[2] = payload.pos.z; q[3] = bf((uint32_t)d + 1u);
            q[4] = wo.x; q[5] = wo.y; q[6] = wo.z; q[7] = 0.0f;
            q[8] = thr.x; q[9] = thr.y; q[10] = thr.z; q[11] = 0.0f;
            q[12] = n_s.x; q[13] = n_s.y; q[14] = n_s.z; q[15] = 0.0f;
        }
        pos = offset_ray(payload.pos, n_g);
        float pdf_dir, cos_theta;
        const float c0 = rand(seed), c1 = rand(seed), c2 = rand(seed);
        const V3<float> f = sample_bsdf(n_s, wo, hit_mat, 0u, side, wi, pdf_dir, cos_theta, V3<float>(c0, c1, c2));
        thr *= f * std::fabs(cos_theta) / pdf_dir;
        if ((f.x == 0.0f && f.y == 0.0f && f.z == 0.0f) || pdf_dir == 0.0f) break;
        if (d > RR_MIN_DEPTH) {
            const float rr = gmin(0.95f, luminance(thr));
            if (rr < rand(seed)) break;
            thr /= rr;
        }
    }
}

struct SGrid {
    float mn[3], mx[3];
    int32_t res[3];
};

// gather.comp:43-86 for pixel i.
void gather(const Scene& s, const orc_sppm_params* p, const SGrid& g, uint32_t screen, const float* photons,
            const uint32_t* count, const uint32_t* rep, float* vp) {
    const V3<float> pos(vp[0], vp[1], vp[2]);
    float r = vp[3];
    if (r < EPS) r = EPS;
    const float r_sqr = r * r;
    const I3 lo = grid_idx(pos - V3<float>(r), g.mn, g.mx, g.res);
    const I3 hi = grid_idx(pos + V3<float>(r), g.mn, g.mx, g.res);
    if ((int64_t)hi.x - lo.x >= kMaxGatherCells || (int64_t)hi.y - lo.y >= kMaxGatherCells ||
        (int64_t)hi.z - lo.z >= kMaxGatherCells)
        return;
    const V3<float> wo(vp[4], vp[5], vp[6]), n_s(vp[8], vp[9], vp[10]), vthr(vp[12], vp[13], vp[14]);
    const V2<float> uv(vp[11], vp[15]);
    const uint32_t mat_idx = fb(vp[23]), vlen = fb(vp[27]);
    const bool side = fb(vp[28]) == 1u;
    V3<float> phi(vp[20], vp[21], vp[22]);
    int M = (int)fb(vp[19]);
    for (int x = lo.x; x <= hi.x; x++)
        for (int y = lo.y; y <= hi.y; y++)
            for (int z = lo.z; z <= hi.z; z++) {
                const uint32_t h = grid_hash(I3{x, y, z}, screen);
                if (count[h] == 0u) continue;
                const float* q = photons + 16 * (size_t)rep[h];
                const V3<float> pp = pos - V3<float>(q[0], q[1], q[2]);
                const float dist_sqr = dot(pp, pp);
                if (dist_sqr > r_sqr) continue;
                if (p->max_depth < (int)(fb(q[3]) + vlen + 1u)) continue;
                const Mat<float> mat = load_material<float>(s, mat_idx, uv);
                float pdf, unused_rev;
                const V3<float> f = eval_bsdf(n_s, wo, mat, 1u, side, V3<float>(q[4], q[5], q[6]), pdf, unused_rev, false);
                phi += (float)count[h] * V3<float>(q[8], q[9], q[10]) * f * vthr;
                M += 1;
            }
    vp[20] = phi.x; vp[21] = phi.y; vp[22] = phi.z;
    vp[19] = bf((uint32_t)M);
}

// composite.comp:33-60 for pixel i = x * H + y.
void composite(const orc_sppm_params* p, uint32_t screen, uint32_t W, uint32_t x, uint32_t y, float* vp, float* film) {
    V3<float> col(vp[16], vp[17], vp[18]);
    const int M = (int)fb(vp[19]);
    if (M > 0) {
        const float gamma = 2.0f / 3.0f;
        const float N = vp[7], radius = vp[3];
        const float n_new = N + gamma * (float)M;
        const float r_new = radius * std::sqrt(n_new / (N + (float)M));
        const V3<float> tau = (V3<float>(vp[24], vp[25], vp[26]) + V3<float>(vp[20], vp[21], vp[22])) * r_new * r_new /
                              (radius * radius);
        vp[7] = n_new;
        vp[3] = r_new;
        vp[20] = vp[21] = vp[22] = 0.0f;
        col += tau / ((float)screen * K<float>::PI() * r_new * r_new);
    }
    vp[16] = vp[17] = vp[18] = 0.0f;
    vp[19] = bf(0u);
    vp[24] = vp[25] = vp[26] = 0.0f;
    float* px = film + 4 * ((size_t)y * W + x);
    if (p->frame_num > 0u) {
        const float w = 1.0f / (float)(p->frame_num + 1u);
        const V3<float> old(px[0], px[1], px[2]);
        const V3<float> m = mix(old, col, w);
        px[0] = m.x; px[1] = m.y; px[2] = m.z; px[3] = 1.0f;
    } else {
        px[0] = col.x; px[1] = col.y; px[2] = col.z; px[3] = 1.0f;
    }
}

}  // namespace

extern "C" {

void orc_sppm_iteration(void* scene, const float inv_view[16], const float inv_proj[16], uint32_t width,
                        uint32_t height, const orc_sppm_params* p, float* vp, float* photons, uint32_t* grid_count,
                        uint32_t* grid_rep, float* film, int nthreads) {
    const Scene& s = *(const Scene*)scene;
    const M4<float> iv = load_m4<float>(inv_view), ip = load_m4<float>(inv_proj);
    const uint32_t screen = width * height, per = (uint32_t)p->max_depth;
    const Cone cone = spot_cone(p->spot_angle);
    parallel_for(screen, nthreads, [&](uint32_t i) {
        eye_path(s, iv, ip, p, cone, i / height, i % height, width, height, vp + 32 * (size_t)i);
    });
    // min / max / calc_bounds (exact, so order-free)
    SGrid g;
    float mx_r = -INFINITY;
    for (int k = 0; k < 3; k++) { g.mn[k] = INFINITY; g.mx[k] = -INFINITY; }
    for (uint32_t i = 0; i < screen; i++) {
        const float* v = vp + 32 * (size_t)i;
        for (int k = 0; k < 3; k++) {
            g.mn[k] = std::min(g.mn[k], v[k] - v[3]);
            g.mx[k] = std::max(g.mx[k], v[k] + v[3]);
        }
        mx_r = std::max(mx_r, v[3]);
    }
    const float dd[3] = {g.mx[0] - g.mn[0], g.mx[1] - g.mn[1], g.mx[2] - g.mn[2]};
    const float max_comp = std::max(dd[0], std::max(dd[1], dd[2]));
    const int base = to_int_rz(max_comp / mx_r);
    for (int k = 0; k < 3; k++)
        g.res[k] = (max_comp > 0.0f && mx_r > 0.0f) ? std::max(to_int_rz((float)base * dd[k] / max_comp), 1) : 0;
    parallel_for(screen, nthreads, [&](uint32_t li) {
        light_path(s, p, cone, li / height, li % height, photons + 16 * (size_t)li * per);
    });
    // the photon table, written in photon order
    std::memset(grid_count, 0, sizeof(uint32_t) * 10u * screen);
    std::memset(grid_rep, 0, sizeof(uint32_t) * 10u * screen);
    for (uint32_t i = 0; i < screen * per; i++) {
        const float* q = photons + 16 * (size_t)i;
        if (fb(q[3]) == 0u) continue;
        const uint32_t slot = grid_hash(grid_idx(V3<float>(q[0], q[1], q[2]), g.mn, g.mx, g.res), screen);
        grid_count[slot]++;
        grid_rep[slot] = i;
    }
    parallel_for(screen, nthreads, [&](uint32_t i) {
        gather(s, p, g, screen, photons, grid_count, grid_rep, vp + 32 * (size_t)i);
    });
    for (uint32_t i = 0; i < screen; i++) composite(p, screen, width, i / height, i % height, vp + 32 * (size_t)i, film);
}

}  // extern "C"
