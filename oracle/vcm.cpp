// Oracle (test infrastructure only): CPU restatement of Lumen's VCM integrator (vertex connection and merging).
//
// Follows src/shaders/integrators/vcm_commons.glsl (get_grid_idx 17-23, vcm_connect_cam 24-75,
// vcm_generate_light_sample 77-130, vcm_get_light_radiance 132-144, vcm_connect_light 146-204,
// vcm_connect_light_vertices 206-251, vcm_merge_light_vertices 254-296, vcm_fill_light 302-474,
// vcm_trace_eye 477-631), src/shaders/integrators/vcm/vcm_light.rgen:123-166 and vcm_eye.rgen:42-97,
// src/shaders/commons.glsl (sample_light_Li 224-300, sample_light_Le 335-415, light pdfs 40-110),
// src/shaders/utils.glsl (hash 62-65, quaternions 157-175) and src/RayTracer/VCM.cpp:131-147 (radius, grid).
//
// Semantics kept from the reference: every connection and merge loop assigns (`res =`), so only the last
// contributing light vertex / cell counts (flags bit 0 accumulates instead); the photon table holds one photon per hash slot (the last one
// written) and its count. Made deterministic here: the last writer of a slot is the photon with the highest
// index (light path index * (max_depth + 1) + vertex), and camera splats are summed in light-path order.
// The reference's host rand() seeds become explicit light and eye seeds. A pdf_rev that vcm_trace_eye passes
// uninitialised (last bounce) is zero; a light path whose emission sample has a zero direction pdf gets zero
// vertices (the reference keeps the previous iteration's count); and a merge whose cell range exceeds 16 cells
// per axis (only possible with a radius far larger than a grid cell) is skipped; the random light subpath index
// uint(rand * screen) is clamped to the last subpath (it can round up to screen for large images).
#include <cstdint>
#include <vector>

#include "photon_common.h"
#include "scene_internal.h"

namespace {
using namespace orc;
using namespace orc::detail;
using namespace orc::photon;

constexpr int kMaxMergeCells = 16;

struct Cam {
    M4<float> iv, ip, view, proj;
    V3<float> pos, nrm;
    float area;
    uint32_t W, H;
};

Cam make_cam(const float* iv, const float* ip, const float* view, const float* proj, uint32_t W, uint32_t H) {
    Cam c;
    c.iv = load_m4<float>(iv); c.ip = load_m4<float>(ip); c.view = load_m4<float>(view); c.proj = load_m4<float>(proj);
    c.W = W; c.H = H;
    c.pos = (c.iv * V4<float>(0.0f, 0.0f, 0.0f, 1.0f)).xyz();
    const V4<float> fwd = c.iv * V4<float>(0.0f, 0.0f, 1.0f, 0.0f);
    c.nrm = V3<float>(-fwd.x, -fwd.y, -fwd.z);
    V4<float> a = c.ip * V4<float>(2.0f / (float)W, 2.0f / (float)H, 0.0f, 1.0f);
    a = V4<float>(a.x / a.w, a.y / a.w, a.z / a.w, a.w / a.w);
    c.area = std::fabs(a.x * a.y);
    return c;
}

struct Etas { float vcm, vc, vm, radius; };
Etas make_etas(const orc_vcm_params* p, uint32_t screen) {
    const float r2 = p->radius * p->radius;
    Etas e;
    e.vcm = K<float>::PI() * r2 * (float)screen;
    e.vc = p->use_vc == 1 ? 1.0f / e.vcm : 0.0f;
    e.vm = p->use_vm == 1 ? K<float>::PI() * r2 * (float)screen : 0.0f;
    e.radius = p->radius;
    return e;
}

struct VState {
    V3<float> pos, wi, throughput;
    float d_vcm, d_vc, d_vm;
};

inline bool is_zero(V3<float> v) { return v.x == 0.0f && v.y == 0.0f && v.z == 0.0f; }

struct Splat { uint32_t idx; V3<float> L; };

// vcm_connect_cam (vcm_commons.glsl:24-75): light vertex -> camera, returns the splat and its pixel.
V3<float> connect_cam(const Scene& s, const Cam& c, V3<float> n_s, V3<float> payload_ns, V3<float> pos, const VState& st,
                      float eta_vm, V3<float> wo, const Mat<float>& mat, int32_t& cx, int32_t& cy, bool& have_coords) {
    have_coords = false;
    V3<float> L(0.0f);
    V3<float> dir = c.pos - pos;
    const float len = length(dir);
    dir /= len;
    const float cos_y = dot(dir, n_s);
    const float cos_theta = dot(c.nrm, -dir);
    if (cos_theta <= 0.0f) return L;
    const float cos3 = cos_theta * cos_theta * cos_theta;
    const float screen = (float)(c.W * c.H);
    const float ratio = std::fabs(cos_y) / (c.area * cos3 * len * len);
    const V3<float> origin = offset_ray2(pos, n_s);
    float pdf_rev, pdf_fwd;
    const V3<float> f = eval_bsdf(n_s, wo, mat, 0u, dot(payload_ns, wo) > 0.0f, dir, pdf_fwd, pdf_rev, true);
    if (is_zero(f)) return L;
    if (ratio > 0.0f) {
        const float o[3] = {origin.x, origin.y, origin.z}, d[3] = {dir.x, dir.y, dir.z};
        if (!bvh_any(s.bvh, o, d, 0.0f, len - EPS)) {
            const float w_light = (ratio / screen) * (eta_vm + st.d_vcm + pdf_rev * st.d_vc);
            const float mis = 1.0f / (1.0f + w_light);
            L = mis * st.throughput * ratio * f / screen;
        }
    }
    dir = -dir;
    V4<float> t = c.view * V4<float>(dir.x, dir.y, dir.z, 0.0f);
    t = V4<float>(t.x / t.z, t.y / t.z, t.z / t.z, t.w / t.z);
    t = c.proj * t;
    t = V4<float>(-t.x, -t.y, -t.z, -t.w);
    cx = to_int_rz(0.5f * (1.0f + t.x) * (float)c.W - 0.5f);
    cy = to_int_rz(0.5f * (1.0f + t.y) * (float)c.H - 0.5f);
    if (cx < 0 || cx >= (int32_t)c.W || cy < 0 || cy >= (int32_t)c.H || dot(dir, c.nrm) < 0.0f) return V3<float>(0.0f);
    have_coords = true;
    return L;
}

void store_vertex(orc_vcm_vertex& v, const VState& st, V3<float> wo, V3<float> n_s, const Payload<float>& pl, uint32_t depth,
                  bool side) {
    v.wi[0] = st.wi.x; v.wi[1] = st.wi.y; v.wi[2] = st.wi.z;
    v.wo[0] = wo.x; v.wo[1] = wo.y; v.wo[2] = wo.z;
    v.n_s[0] = n_s.x; v.n_s[1] = n_s.y; v.n_s[2] = n_s.z;
    v.pos[0] = pl.pos.x; v.pos[1] = pl.pos.y; v.pos[2] = pl.pos.z;
    v.uv[0] = pl.uv.x; v.uv[1] = pl.uv.y;
    v.material_idx = (uint32_t)pl.material_idx;
    v.area = pl.area;
    v.throughput[0] = st.throughput.x; v.throughput[1] = st.throughput.y; v.throughput[2] = st.throughput.z;
    v.d_vcm = st.d_vcm; v.d_vc = st.d_vc; v.d_vm = st.d_vm;
    v.path_len = depth + 1;
    v.side = side ? 1u : 0u;
    v.coords = 0;
}

// vcm_light.rgen main + vcm_generate_light_sample + vcm_fill_light for light path (x, y).
void light_path(const Scene& s, const Cam& c, const orc_vcm_params* p, const Etas& eta, uint32_t x, uint32_t y,
                orc_vcm_vertex* verts, uint32_t* counts, std::vector<Splat>& splats) {
    const uint32_t li = x * c.H + y;  // vcm_light.rgen: launch x * height + y
    orc_vcm_vertex* lv = verts + (size_t)li * (uint32_t)(p->max_depth + 1);
    U4 seed{x, y, p->light_seed, 0u};
    const float r0 = rand(seed), r1 = rand(seed), r2 = rand(seed), r3 = rand(seed);
    const float r4 = rand(seed), r5 = rand(seed);
    const Emission<float> e = sample_light_Le<float>(s, V4<float>(r0, r1, r2, r3), V2<float>(r4, r5), p->num_lights,
                                                     p->light_triangle_count, spot_cone(p->spot_angle));
    if (e.pdf_dir_w <= 0.0f) {  // the reference returns here and leaves the previous iteration's count
        counts[li] = 0;
        return;
    }
    VState st;
    const float pdf_emit = e.pdf_pos_a * e.pdf_dir_w;
    st.pos = e.pos;
    st.wi = e.wi;
    st.throughput = e.L * e.cos_from_light / (e.pdf_dir_w * e.pdf_pos_a);
    st.d_vcm = e.pdf_pos_a / pdf_emit;
    const bool finite = light_finite(e.flags);
    st.d_vc = light_delta(e.flags) ? 0.0f : (finite ? e.cos_from_light : 1.0f) / (e.pdf_dir_w * e.pdf_pos_a);
    st.d_vm = st.d_vc * eta.vc;

    uint32_t path_idx = 0;
    lv[0].path_len = 0;
    Payload<float> pl;
    pl.material_idx = -1;
    for (int depth = 1;; depth++) {
        trace_closest<float>(s, st.pos, st.wi, TMIN, TMAX, pl);
        if (pl.material_idx == -1) break;
        V3<float> wo = st.pos - pl.pos;
        V3<float> n_s = pl.n_s, n_g = pl.n_g;
        bool side = true;
        if (dot(pl.n_g, wo) <= 0.0f) n_g = -n_g;
        if (dot(n_g, n_s) < 0.0f) { n_s = -n_s; side = false; }
        const float dist = length(pl.pos - st.pos);
        const float dist_sqr = dist * dist;
        wo /= dist;
        const Mat<float> mat = load_material<float>(s, (uint32_t)pl.material_idx, pl.uv);
        const bool spec = (mat.bsdf_props & BSDF_FLAG_SPECULAR) == BSDF_FLAG_SPECULAR;
        const float cos_wo = std::fabs(dot(wo, n_s));
        if (depth > 1 || finite) st.d_vcm *= dist_sqr;
        st.d_vcm /= cos_wo;
        st.d_vc /= cos_wo;
        st.d_vm /= cos_wo;
        if (!spec && (p->use_vc == 1 || p->use_vm == 1)) store_vertex(lv[path_idx++], st, wo, n_s, pl, (uint32_t)depth, side);
        if (depth >= p->max_depth) break;
        if (!spec && p->use_vc == 1 && depth < p->max_depth) {
            int32_t cx = 0, cy = 0;
            bool have = false;
            const V3<float> L = connect_cam(s, c, n_s, pl.n_s, pl.pos, st, eta.vm, wo, mat, cx, cy, have);
            if (luminance(L) > 0.0f && have) splats.push_back(Splat{(uint32_t)cx * c.H + (uint32_t)cy, L});
        }
        const float c0 = rand(seed), c1 = rand(seed), c2 = rand(seed);
        float pdf_dir, cos_theta;
        V3<float> wi;
        const V3<float> f = sample_bsdf(n_s, wo, mat, 0u, side, wi, pdf_dir, cos_theta, V3<float>(c0, c1, c2));
        st.wi = wi;
        const bool same = dot(st.wi, n_s) > 0.0f && dot(wo, n_s) > 0.0f;
        const bool trans = (mat.bsdf_props & BSDF_FLAG_TRANSMISSION) == BSDF_FLAG_TRANSMISSION;
        if (is_zero(f) || pdf_dir == 0.0f || (!same && !trans)) break;
        float pdf_rev = pdf_dir;
        if (!spec) pdf_rev = bsdf_pdf(mat, n_s, st.wi, wo, side);
        const float ac = std::fabs(cos_theta);
        st.pos = offset_ray(pl.pos, n_g);
        if (!spec) {
            st.d_vc = (ac / pdf_dir) * (eta.vm + st.d_vcm + pdf_rev * st.d_vc);
            st.d_vm = (ac / pdf_dir) * (1.0f + st.d_vcm * eta.vc + pdf_rev * st.d_vm);
            st.d_vcm = 1.0f / pdf_dir;
        } else {
            st.d_vcm = 0.0f;
            st.d_vc *= ac;
            st.d_vm *= ac;
        }
        st.throughput *= f * ac / pdf_dir;
    }
    counts[li] = path_idx;
}

struct Grid {
    const uint32_t* count;
    const uint32_t* rep;
    int32_t res[3];
    float mn[3], mx[3];
};

struct EyeHit {
    V3<float> pos, n_s_payload;
    float area;
};

// vcm_connect_light (vcm_commons.glsl:146-204)
V3<float> connect_light(const Scene& s, const orc_vcm_params* p, U4& seed, const EyeHit& h, V3<float> n_s, V3<float> wo,
                        const Mat<float>& mat, bool side, float eta_vm, const VState& cs, float& pdf_rev) {
    V3<float> res(0.0f);
    const float q0 = rand(seed), q1 = rand(seed), q2 = rand(seed), q3 = rand(seed);
    const Incidence<float> li = sample_light_Li_pos<float>(s, V4<float>(q0, q1, q2, q3), h.pos, p->num_lights,
                                                              spot_cone(p->spot_angle));
    const float cos_x = dot(li.wi, n_s);
    const V3<float> origin = offset_ray2(h.pos, n_s);
    float pdf_fwd;
    const V3<float> f = eval_bsdf(n_s, wo, mat, 1u, side, li.wi, pdf_fwd, pdf_rev, true);
    if (!is_zero(f)) {
        const float o[3] = {origin.x, origin.y, origin.z}, d[3] = {li.wi.x, li.wi.y, li.wi.z};
        if (!bvh_any(s.bvh, o, d, 0.0f, li.wi_len - EPS)) {
            if (light_delta(li.flags)) pdf_fwd = 0.0f;
            const float ltc = (float)p->light_triangle_count;
            const float w_light = pdf_fwd / (li.pdf_pos_w / ltc);
            const float w_cam = li.pdf_pos_dir_w * std::fabs(cos_x) / (li.pdf_pos_w * li.cos_y) *
                                (eta_vm + cs.d_vcm + cs.d_vc * pdf_rev);
            const float mis = 1.0f / (1.0f + w_light + w_cam);
            if (mis > 0.0f) res = mis * std::fabs(cos_x) * f * cs.throughput * li.L / (li.pdf_pos_w / ltc);
        }
    }
    return res;
}

V3<float> f3v(const float* a) { return V3<float>(a[0], a[1], a[2]); }

// vcm_connect_light_vertices (vcm_commons.glsl:206-251)
V3<float> connect_light_vertices(const Scene& s, const orc_vcm_params* p, const orc_vcm_vertex* lv, uint32_t len_path,
                                 int depth, const EyeHit& h, V3<float> n_s, V3<float> wo, const Mat<float>& mat, bool side,
                                 float eta_vm, const VState& cs, float pdf_rev) {
    V3<float> res(0.0f);
    for (uint32_t i = 0; i < len_path; i++) {
        const orc_vcm_vertex& v = lv[i];
        const uint32_t mdepth = v.path_len + (uint32_t)depth - 1u;
        if (mdepth >= (uint32_t)p->max_depth) break;
        V3<float> dir = f3v(v.pos) - h.pos;
        const float len = length(dir);
        const float len_sqr = len * len;
        dir /= len;
        const float cos_cam = dot(n_s, dir);
        const float cos_light = dot(f3v(v.n_s), -dir);
        const float G = cos_light * cos_cam / len_sqr;
        if (!(G > 0.0f)) continue;
        float cam_pdf_fwd, unused, light_pdf_fwd, light_pdf_rev;
        const V3<float> f_cam = eval_bsdf(n_s, wo, mat, 1u, side, dir, cam_pdf_fwd, unused, false);
        const Mat<float> lm = load_material<float>(s, v.material_idx, V2<float>(v.uv[0], v.uv[1]));
        const V3<float> f_light = eval_bsdf(f3v(v.n_s), f3v(v.wo), lm, 0u, v.side == 1u, -dir, light_pdf_fwd, light_pdf_rev, true);
        if (is_zero(f_light) || is_zero(f_cam)) continue;
        cam_pdf_fwd *= std::fabs(cos_light) / len_sqr;
        light_pdf_fwd *= std::fabs(cos_cam) / len_sqr;
        const float w_light = cam_pdf_fwd * (eta_vm + v.d_vcm + light_pdf_rev * v.d_vc);
        const float w_camera = light_pdf_fwd * (eta_vm + cs.d_vcm + pdf_rev * cs.d_vc);
        const float mis = 1.0f / (1.0f + w_camera + w_light);
        const V3<float> origin = offset_ray2(h.pos, n_s);
        const float o[3] = {origin.x, origin.y, origin.z}, d[3] = {dir.x, dir.y, dir.z};
        if (!bvh_any(s.bvh, o, d, 0.0f, len - EPS)) {
            const V3<float> c = mis * G * cs.throughput * f3v(v.throughput) * f_cam * f_light;
            res = (p->flags & 1u) ? res + c : c;
        }
    }
    return res;
}

// vcm_merge_light_vertices (vcm_commons.glsl:254-296) over the slot table: count and representative photon.
V3<float> merge(const orc_vcm_params* p, const orc_vcm_vertex* verts, const Grid& g, uint32_t screen, int depth,
                const EyeHit& h, V3<float> n_s, V3<float> wo, const Mat<float>& mat, bool side, float eta_vc,
                const VState& cs, float radius, float norm) {
    const float r_sqr = radius * radius;
    V3<float> res(0.0f);
    const I3 lo = grid_idx(h.pos - V3<float>(radius), g.mn, g.mx, g.res);
    const I3 hi = grid_idx(h.pos + V3<float>(radius), g.mn, g.mx, g.res);
    if ((int64_t)hi.x - lo.x >= kMaxMergeCells || (int64_t)hi.y - lo.y >= kMaxMergeCells ||
        (int64_t)hi.z - lo.z >= kMaxMergeCells)
        return res;
    for (int32_t x = lo.x; x <= hi.x; x++)
        for (int32_t y = lo.y; y <= hi.y; y++)
            for (int32_t z = lo.z; z <= hi.z; z++) {
                const uint32_t slot = grid_hash(I3{x, y, z}, screen);
                const uint32_t count = g.count[slot];
                if (count == 0) continue;
                const orc_vcm_vertex& ph = verts[g.rep[slot]];
                const V3<float> pp = h.pos - f3v(ph.pos);
                const float dist_sqr = dot(pp, pp);
                if (dist_sqr > r_sqr) continue;
                if (ph.path_len + (uint32_t)depth - 1u > (uint32_t)p->max_depth) continue;
                const V3<float> pwi = -f3v(ph.wi);
                float cam_pdf_fwd, cam_pdf_rev;
                const V3<float> f = eval_bsdf(n_s, wo, mat, 1u, side, pwi, cam_pdf_fwd, cam_pdf_rev, true);
                if (is_zero(f)) continue;
                const float w_light = ph.d_vcm * eta_vc + ph.d_vm * cam_pdf_fwd;
                const float w_cam = cs.d_vcm * eta_vc + cs.d_vm * cam_pdf_rev;
                const float mis = 1.0f / (1.0f + w_light + w_cam);
                const float cos_nrm = dot(f3v(ph.n_s), n_s);
                if (cos_nrm > EPS) {
                    const float w = 1.0f - std::sqrt(dist_sqr) / radius;
                    const V3<float> cc = w * mis * (float)(int32_t)count * f3v(ph.throughput) * f * cs.throughput * norm * 3.0f;
                    res = (p->flags & 1u) ? res + cc : cc;
                }
            }
    return res;
}

// vcm_eye.rgen main + vcm_trace_eye for pixel (x, y); writes film[y * W + x] and consumes the pixel's splat.
void eye_path(const Scene& s, const Cam& c, const orc_vcm_params* p, const Etas& eta, uint32_t x, uint32_t y,
              const orc_vcm_vertex* verts, const uint32_t* counts, const Grid& g, float* splat, float* film) {
    const uint32_t screen = c.W * c.H;
    U4 seed{x, y, p->eye_seed, 0u};
    const float j0 = rand(seed), j1 = rand(seed);
    const float px = (float)x + 0.5f, py = (float)y + 0.5f;
    const float u = (px + (j0 - 0.5f)) / (float)c.W, v = (py + (j1 - 0.5f)) / (float)c.H;
    const V2<float> d(u * 2.0f - 1.0f, v * 2.0f - 1.0f);
    VState cs;
    cs.wi = sample_camera(c.iv, c.ip, d);
    cs.pos = c.pos;
    cs.throughput = V3<float>(1.0f);
    const float cos_theta0 = std::fabs(dot(c.nrm, cs.wi));
    cs.d_vcm = c.area * (float)screen * cos_theta0 * cos_theta0 * cos_theta0;
    cs.d_vc = 0.0f;
    cs.d_vm = 0.0f;
    const float radius = eta.radius;
    const float norm = 1.0f / (K<float>::PI() * radius * radius * (float)screen);

    const uint32_t lp = std::min((uint32_t)(rand(seed) * (float)screen), screen - 1u);  // can round up to screen
    const uint32_t lp_len = counts[lp];
    const orc_vcm_vertex* lv = verts + (size_t)lp * (uint32_t)(p->max_depth + 1);
    V3<float> col(0.0f);
    Payload<float> pl;
    pl.material_idx = -1;
    for (int depth = 1;; depth++) {
        trace_closest<float>(s, cs.pos, cs.wi, TMIN, TMAX, pl);
        if (pl.material_idx == -1) {
            col += cs.throughput * V3<float>(p->sky_col[0], p->sky_col[1], p->sky_col[2]);
            break;
        }
        V3<float> wo = cs.pos - pl.pos;
        const float dist = length(pl.pos - cs.pos);
        const float dist_sqr = dist * dist;
        wo /= dist;
        V3<float> n_s = pl.n_s, n_g = pl.n_g;
        bool side = true;
        if (dot(pl.n_g, wo) < 0.0f) n_g = -n_g;
        if (dot(n_g, n_s) < 0.0f) { n_s = -n_s; side = false; }
        const float cos_wo = std::fabs(dot(wo, n_s));
        const Mat<float> mat = load_material<float>(s, (uint32_t)pl.material_idx, pl.uv);
        const bool spec = (mat.bsdf_props & BSDF_FLAG_SPECULAR) == BSDF_FLAG_SPECULAR;
        cs.d_vcm *= dist_sqr;
        cs.d_vcm /= cos_wo;
        cs.d_vc /= cos_wo;
        cs.d_vm /= cos_wo;
        const EyeHit h{pl.pos, pl.n_s, pl.area};
        if (luminance(mat.emissive_factor) > 0.0f) {  // vcm_get_light_radiance
            V3<float> Le = mat.emissive_factor;
            if (depth != 1) {
                const float pdf_light_pos = 1.0f / (h.area * (float)p->light_triangle_count);
                const float pdf_light_dir = std::fabs(dot(h.n_s_payload, -cs.wi)) / K<float>::PI();
                const float w_camera = pdf_light_pos * cs.d_vcm +
                                       ((p->use_vc == 1 || p->use_vm == 1) ? (pdf_light_pos * pdf_light_dir) * cs.d_vc : 0.0f);
                Le = (1.0f / (1.0f + w_camera)) * mat.emissive_factor;
            }
            col += cs.throughput * Le;
        }
        float pdf_rev = 0.0f;
        if (!spec && depth < p->max_depth) col += connect_light(s, p, seed, h, n_s, wo, mat, side, eta.vm, cs, pdf_rev);
        if (!spec) col += connect_light_vertices(s, p, lv, lp_len, depth, h, n_s, wo, mat, side, eta.vm, cs, pdf_rev);
        if (!spec && p->use_vm == 1)
            col += merge(p, verts, g, screen, depth, h, n_s, wo, mat, side, eta.vc, cs, radius, norm);
        if (depth >= p->max_depth) break;
        const float c0 = rand(seed), c1 = rand(seed), c2 = rand(seed);
        float pdf_dir, cos_theta;
        V3<float> wi;
        const V3<float> f = sample_bsdf(n_s, wo, mat, 1u, side, wi, pdf_dir, cos_theta, V3<float>(c0, c1, c2));
        cs.wi = wi;
        const bool trans = (mat.bsdf_props & BSDF_FLAG_TRANSMISSION) == BSDF_FLAG_TRANSMISSION;
        const bool same = dot(cs.wi, n_s) > 0.0f && dot(wo, n_s) > 0.0f;
        if (is_zero(f) || pdf_dir == 0.0f || (!same && !trans)) break;
        pdf_rev = pdf_dir;
        if (!spec) pdf_rev = bsdf_pdf(mat, n_s, cs.wi, wo, side);
        const float ac = std::fabs(cos_theta);
        cs.pos = offset_ray(pl.pos, n_g);
        if (!spec) {
            cs.d_vc = (ac / pdf_dir) * (eta.vm + cs.d_vcm + pdf_rev * cs.d_vc);
            cs.d_vm = (ac / pdf_dir) * (1.0f + cs.d_vcm * eta.vc + pdf_rev * cs.d_vm);
            cs.d_vcm = 1.0f / pdf_dir;
        } else {
            cs.d_vcm = 0.0f;
            cs.d_vc *= ac;
            cs.d_vm *= ac;
        }
        cs.throughput *= f * ac / pdf_dir;
    }
    if (std::isnan(luminance(col))) return;  // vcm_eye.rgen:80-83: no film write, the splat stays
    const uint32_t pidx = x * c.H + y;
    col += V3<float>(splat[3 * pidx], splat[3 * pidx + 1], splat[3 * pidx + 2]);
    splat[3 * pidx] = splat[3 * pidx + 1] = splat[3 * pidx + 2] = 0.0f;
    float* out = film + 4 * ((size_t)y * c.W + x);
    if (p->frame_num > 0) {
        const float w = 1.0f / (float)(p->frame_num + 1);
        out[0] = out[0] * (1.0f - w) + col.x * w;
        out[1] = out[1] * (1.0f - w) + col.y * w;
        out[2] = out[2] * (1.0f - w) + col.z * w;
    } else {
        out[0] = col.x; out[1] = col.y; out[2] = col.z;
    }
    out[3] = 1.0f;
}

}  // namespace

extern "C" {

void orc_vcm_grid_res(const float scene_min[3], const float scene_max[3], float radius, int32_t res[3]) {
    grid_resolution(scene_min, scene_max, radius, res);
}

// The photon table of vcm_fill_light (vcm_commons.glsl:455-469) written sequentially in photon order: per
// slot the number of photons and the index of the last one. pos4: x, y, z and w < 0 for an unused entry.
void orc_vcm_grid(const float* pos4, uint32_t n, const float scene_min[3], const float scene_max[3], float radius,
                  uint32_t screen_size, uint32_t* count, uint32_t* rep) {
    int32_t res[3];
    grid_resolution(scene_min, scene_max, radius, res);
    std::memset(count, 0, sizeof(uint32_t) * 10u * screen_size);
    std::memset(rep, 0, sizeof(uint32_t) * 10u * screen_size);
    for (uint32_t i = 0; i < n; i++) {
        if (pos4[4 * i + 3] < 0.0f) continue;
        const I3 g = grid_idx(V3<float>(pos4[4 * i], pos4[4 * i + 1], pos4[4 * i + 2]), scene_min, scene_max, res);
        const uint32_t slot = grid_hash(g, screen_size);
        count[slot]++;
        rep[slot] = i;
    }
}

// One VCM iteration (VCM::render, VCM.cpp:131-265, without the reservoir passes): light subpaths with camera
// splats, the photon table (when use_vm), eye subpaths and the progressive film. verts (W*H*(max_depth+1)),
// counts (W*H) and splat (W*H*3, pixel x*H+y) persist across iterations as the reference's buffers do;
// grid_count / grid_rep (10*W*H) receive the table.
void orc_vcm_iteration(void* scene, const float inv_view[16], const float inv_proj[16], const float view[16],
                       const float proj[16], uint32_t width, uint32_t height, const orc_vcm_params* p,
                       orc_vcm_vertex* verts, uint32_t* counts, float* splat, uint32_t* grid_count, uint32_t* grid_rep,
                       float* film, int nthreads) {
    const Scene& s = *(const Scene*)scene;
    const Cam c = make_cam(inv_view, inv_proj, view, proj, width, height);
    const uint32_t screen = width * height;
    const Etas eta = make_etas(p, screen);
    std::vector<std::vector<Splat>> splats(screen);
    parallel_for(screen, nthreads, [&](uint32_t i) {
        const uint32_t x = i / height, y = i % height;
        light_path(s, c, p, eta, x, y, verts, counts, splats[i]);
    });
    for (uint32_t i = 0; i < screen; i++)  // light path order (x * height + y)
        for (const Splat& sp : splats[i]) {
            splat[3 * sp.idx] += sp.L.x;
            splat[3 * sp.idx + 1] += sp.L.y;
            splat[3 * sp.idx + 2] += sp.L.z;
        }
    Grid g;
    std::memcpy(g.mn, p->scene_min, sizeof(g.mn));
    std::memcpy(g.mx, p->scene_max, sizeof(g.mx));
    grid_resolution(g.mn, g.mx, p->radius, g.res);
    std::memset(grid_count, 0, sizeof(uint32_t) * 10u * screen);
    std::memset(grid_rep, 0, sizeof(uint32_t) * 10u * screen);
    if (p->use_vm == 1) {
        const uint32_t per = (uint32_t)(p->max_depth + 1);
        for (uint32_t li = 0; li < screen; li++)
            for (uint32_t k = 0; k < counts[li]; k++) {
                const uint32_t vid = li * per + k;
                const I3 gi = grid_idx(f3v(verts[vid].pos), g.mn, g.mx, g.res);
                const uint32_t slot = grid_hash(gi, screen);
                grid_count[slot]++;
                grid_rep[slot] = vid;
            }
    }
    g.count = grid_count;
    g.rep = grid_rep;
    parallel_for(screen, nthreads, [&](uint32_t i) {
        const uint32_t x = i / height, y = i % height;
        eye_path(s, c, p, eta, x, y, verts, counts, g, splat, film);
    });
}

}  // extern "C"
