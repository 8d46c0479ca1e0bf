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

// Everything below is templated on the arithmetic type T: float is the shader's FP32 sequence (the parity
// oracle), double the converged FP64 reference renders. Ray queries, random numbers, pixel indices of camera
// splats and the photon table's cell keys stay FP32 in both, as the traversal boundary of the path oracle does.
template <class T> struct VertexOf { using type = orc_vcm_vertex; };
struct VertexF64 {
    double wi[3], wo[3], n_s[3], pos[3], uv[2], throughput[3];
    uint32_t material_idx, path_len;
    double area, d_vcm, d_vc, d_vm;
    uint32_t side, coords;
};
template <> struct VertexOf<double> { using type = VertexF64; };
template <class T> using Vertex = typename VertexOf<T>::type;

template <class T> V3<float> to_f(V3<T> v) { return V3<float>((float)v.x, (float)v.y, (float)v.z); }
template <class T> V3<T> from_f(V3<float> v) { return V3<T>(T(v.x), T(v.y), T(v.z)); }
template <class T> V3<T> offset_ray_t(V3<T> p, V3<T> n) { return from_f<T>(offset_ray(to_f(p), to_f(n))); }
template <class T, class S> V3<T> f3v(const S* a) { return V3<T>(T(a[0]), T(a[1]), T(a[2])); }

template <class T> struct Cam {
    M4<T> iv, ip, view, proj;
    V3<T> pos, nrm;
    T area;
    uint32_t W, H;
};

template <class T>
Cam<T> make_cam(const float* iv, const float* ip, const float* view, const float* proj, uint32_t W, uint32_t H) {
    Cam<T> c;
    c.iv = load_m4<T>(iv); c.ip = load_m4<T>(ip); c.view = load_m4<T>(view); c.proj = load_m4<T>(proj);
    c.W = W; c.H = H;
    c.pos = (c.iv * V4<T>(T(0), T(0), T(0), T(1))).xyz();
    const V4<T> fwd = c.iv * V4<T>(T(0), T(0), T(1), T(0));
    c.nrm = V3<T>(-fwd.x, -fwd.y, -fwd.z);
    V4<T> a = c.ip * V4<T>(T(2) / (T)W, T(2) / (T)H, T(0), T(1));
    a = V4<T>(a.x / a.w, a.y / a.w, a.z / a.w, a.w / a.w);
    c.area = std::fabs(a.x * a.y);
    return c;
}

template <class T> struct Etas { T vcm, vc, vm, radius; };
template <class T> Etas<T> make_etas(const orc_vcm_params* p, uint32_t screen) {
    const T r2 = T(p->radius) * T(p->radius);
    Etas<T> e;
    e.vcm = K<T>::PI() * r2 * (T)screen;
    e.vc = p->use_vc == 1 ? T(1) / e.vcm : T(0);
    e.vm = p->use_vm == 1 ? K<T>::PI() * r2 * (T)screen : T(0);
    e.radius = T(p->radius);
    return e;
}

template <class T> struct VState {
    V3<T> pos, wi, throughput;
    T d_vcm, d_vc, d_vm;
};

template <class T> inline bool is_zero(V3<T> v) { return v.x == T(0) && v.y == T(0) && v.z == T(0); }

template <class T> struct Splat { uint32_t idx; V3<T> L; };

// vcm_connect_cam (vcm_commons.glsl:24-75): light vertex -> camera, returns the splat and its pixel.
template <class T>
V3<T> connect_cam(const Scene& s, const Cam<T>& c, V3<T> n_s, V3<T> payload_ns, V3<T> pos, const VState<T>& st,
                      T eta_vm, V3<T> wo, const Mat<T>& mat, int32_t& cx, int32_t& cy, bool& have_coords) {
    have_coords = false;
    V3<T> L(T(0));
    V3<T> dir = c.pos - pos;
    const T len = length(dir);
    dir /= len;
    const T cos_y = dot(dir, n_s);
    const T cos_theta = dot(c.nrm, -dir);
    if (cos_theta <= T(0)) return L;
    const T cos3 = cos_theta * cos_theta * cos_theta;
    const T screen = (T)(c.W * c.H);
    const T ratio = std::fabs(cos_y) / (c.area * cos3 * len * len);
    const V3<T> origin = offset_ray2(pos, n_s);
    T pdf_rev, pdf_fwd;
    const V3<T> f = eval_bsdf(n_s, wo, mat, 0u, dot(payload_ns, wo) > T(0), dir, pdf_fwd, pdf_rev, true);
    if (is_zero(f)) return L;
    if (ratio > T(0)) {
        const float o[3] = {(float)origin.x, (float)origin.y, (float)origin.z};
        const float d[3] = {(float)dir.x, (float)dir.y, (float)dir.z};
        if (!bvh_any(s.bvh, o, d, 0.0f, (float)(len - EPS))) {
            const T w_light = (ratio / screen) * (eta_vm + st.d_vcm + pdf_rev * st.d_vc);
            const T mis = T(1) / (T(1) + w_light);
            L = mis * st.throughput * ratio * f / screen;
        }
    }
    dir = -dir;
    V4<T> t = c.view * V4<T>(dir.x, dir.y, dir.z, T(0));
    t = V4<T>(t.x / t.z, t.y / t.z, t.z / t.z, t.w / t.z);
    t = c.proj * t;
    t = V4<T>(-t.x, -t.y, -t.z, -t.w);
    cx = to_int_rz((float)(T(0.5) * (T(1) + t.x) * (T)c.W - T(0.5)));
    cy = to_int_rz((float)(T(0.5) * (T(1) + t.y) * (T)c.H - T(0.5)));
    if (cx < 0 || cx >= (int32_t)c.W || cy < 0 || cy >= (int32_t)c.H || dot(dir, c.nrm) < T(0)) return V3<T>(T(0));
    have_coords = true;
    return L;
}

template <class T>
void store_vertex(Vertex<T>& v, const VState<T>& st, V3<T> wo, V3<T> n_s, const Payload<T>& pl, uint32_t depth,
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
template <class T>
void light_path(const Scene& s, const Cam<T>& c, const orc_vcm_params* p, const Etas<T>& eta, uint32_t x, uint32_t y,
                Vertex<T>* verts, uint32_t* counts, std::vector<Splat<T>>& splats) {
    const uint32_t li = x * c.H + y;  // vcm_light.rgen: launch x * height + y
    Vertex<T>* lv = verts + (size_t)li * (uint32_t)(p->max_depth + 1);
    U4 seed{x, y, p->light_seed, 0u};
    const T r0 = T(rand(seed)), r1 = T(rand(seed)), r2 = T(rand(seed)), r3 = T(rand(seed));
    const T r4 = rand(seed), r5 = rand(seed);
    const Emission<T> e = sample_light_Le<T>(s, V4<T>(r0, r1, r2, r3), V2<T>(r4, r5), p->num_lights,
                                                     p->light_triangle_count, spot_cone(p->spot_angle));
    if (e.pdf_dir_w <= T(0)) {  // the reference returns here and leaves the previous iteration's count
        counts[li] = 0;
        return;
    }
    VState<T> st;
    const T pdf_emit = e.pdf_pos_a * e.pdf_dir_w;
    st.pos = e.pos;
    st.wi = e.wi;
    st.throughput = e.L * e.cos_from_light / (e.pdf_dir_w * e.pdf_pos_a);
    st.d_vcm = e.pdf_pos_a / pdf_emit;
    const bool finite = light_finite(e.flags);
    st.d_vc = light_delta(e.flags) ? T(0) : (finite ? e.cos_from_light : T(1)) / (e.pdf_dir_w * e.pdf_pos_a);
    st.d_vm = st.d_vc * eta.vc;

    uint32_t path_idx = 0;
    lv[0].path_len = 0;
    Payload<T> pl;
    pl.material_idx = -1;
    for (int depth = 1;; depth++) {
        trace_closest<T>(s, st.pos, st.wi, TMIN, TMAX, pl);
        if (pl.material_idx == -1) break;
        V3<T> wo = st.pos - pl.pos;
        V3<T> n_s = pl.n_s, n_g = pl.n_g;
        bool side = true;
        if (dot(pl.n_g, wo) <= T(0)) n_g = -n_g;
        if (dot(n_g, n_s) < T(0)) { n_s = -n_s; side = false; }
        const T dist = length(pl.pos - st.pos);
        const T dist_sqr = dist * dist;
        wo /= dist;
        const Mat<T> mat = load_material<T>(s, (uint32_t)pl.material_idx, pl.uv);
        const bool spec = (mat.bsdf_props & BSDF_FLAG_SPECULAR) == BSDF_FLAG_SPECULAR;
        const T cos_wo = std::fabs(dot(wo, n_s));
        if (depth > 1 || finite) st.d_vcm *= dist_sqr;
        st.d_vcm /= cos_wo;
        st.d_vc /= cos_wo;
        st.d_vm /= cos_wo;
        if (!spec && (p->use_vc == 1 || p->use_vm == 1)) store_vertex<T>(lv[path_idx++], st, wo, n_s, pl, (uint32_t)depth, side);
        if (depth >= p->max_depth) break;
        if (!spec && p->use_vc == 1 && depth < p->max_depth) {
            int32_t cx = 0, cy = 0;
            bool have = false;
            const V3<T> L = connect_cam(s, c, n_s, pl.n_s, pl.pos, st, eta.vm, wo, mat, cx, cy, have);
            if (luminance(L) > T(0) && have) splats.push_back(Splat<T>{(uint32_t)cx * c.H + (uint32_t)cy, L});
        }
        const T c0 = rand(seed), c1 = rand(seed), c2 = rand(seed);
        T pdf_dir, cos_theta;
        V3<T> wi;
        const V3<T> f = sample_bsdf(n_s, wo, mat, 0u, side, wi, pdf_dir, cos_theta, V3<T>(c0, c1, c2));
        st.wi = wi;
        const bool same = dot(st.wi, n_s) > T(0) && dot(wo, n_s) > T(0);
        const bool trans = (mat.bsdf_props & BSDF_FLAG_TRANSMISSION) == BSDF_FLAG_TRANSMISSION;
        if (is_zero(f) || pdf_dir == T(0) || (!same && !trans)) break;
        T pdf_rev = pdf_dir;
        if (!spec) pdf_rev = bsdf_pdf(mat, n_s, st.wi, wo, side);
        const T ac = std::fabs(cos_theta);
        st.pos = offset_ray_t(pl.pos, n_g);
        if (!spec) {
            st.d_vc = (ac / pdf_dir) * (eta.vm + st.d_vcm + pdf_rev * st.d_vc);
            st.d_vm = (ac / pdf_dir) * (T(1) + st.d_vcm * eta.vc + pdf_rev * st.d_vm);
            st.d_vcm = T(1) / pdf_dir;
        } else {
            st.d_vcm = T(0);
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

template <class T> struct EyeHit {
    V3<T> pos, n_s_payload;
    T area;
};

// vcm_connect_light (vcm_commons.glsl:146-204)
template <class T>
V3<T> connect_light(const Scene& s, const orc_vcm_params* p, U4& seed, const EyeHit<T>& h, V3<T> n_s, V3<T> wo,
                    const Mat<T>& mat, bool side, T eta_vm, const VState<T>& cs, T& pdf_rev) {
    V3<T> res(T(0));
    const T q0 = rand(seed), q1 = rand(seed), q2 = rand(seed), q3 = rand(seed);
    const Incidence<T> li = sample_light_Li_pos<T>(s, V4<T>(q0, q1, q2, q3), h.pos, p->num_lights,
                                                              spot_cone(p->spot_angle));
    const T cos_x = dot(li.wi, n_s);
    const V3<T> origin = offset_ray2(h.pos, n_s);
    T pdf_fwd;
    const V3<T> f = eval_bsdf(n_s, wo, mat, 1u, side, li.wi, pdf_fwd, pdf_rev, true);
    if (!is_zero(f)) {
        const float o[3] = {(float)origin.x, (float)origin.y, (float)origin.z};
        const float d[3] = {(float)li.wi.x, (float)li.wi.y, (float)li.wi.z};
        if (!bvh_any(s.bvh, o, d, 0.0f, (float)(li.wi_len - EPS))) {
            if (light_delta(li.flags)) pdf_fwd = T(0);
            const T ltc = (T)p->light_triangle_count;
            const T w_light = pdf_fwd / (li.pdf_pos_w / ltc);
            const T w_cam = li.pdf_pos_dir_w * std::fabs(cos_x) / (li.pdf_pos_w * li.cos_y) *
                                (eta_vm + cs.d_vcm + cs.d_vc * pdf_rev);
            const T mis = T(1) / (T(1) + w_light + w_cam);
            if (mis > T(0)) res = mis * std::fabs(cos_x) * f * cs.throughput * li.L / (li.pdf_pos_w / ltc);
        }
    }
    return res;
}


// vcm_connect_light_vertices (vcm_commons.glsl:206-251)
template <class T>
V3<T> connect_light_vertices(const Scene& s, const orc_vcm_params* p, const Vertex<T>* lv, uint32_t len_path,
                             int depth, const EyeHit<T>& h, V3<T> n_s, V3<T> wo, const Mat<T>& mat, bool side,
                             T eta_vm, const VState<T>& cs, T pdf_rev) {
    V3<T> res(T(0));
    for (uint32_t i = 0; i < len_path; i++) {
        const Vertex<T>& v = lv[i];
        const uint32_t mdepth = v.path_len + (uint32_t)depth - 1u;
        if (mdepth >= (uint32_t)p->max_depth) break;
        V3<T> dir = f3v<T>(v.pos) - h.pos;
        const T len = length(dir);
        const T len_sqr = len * len;
        dir /= len;
        const T cos_cam = dot(n_s, dir);
        const T cos_light = dot(f3v<T>(v.n_s), -dir);
        const T G = cos_light * cos_cam / len_sqr;
        if (!(G > T(0))) continue;
        T cam_pdf_fwd, unused, light_pdf_fwd, light_pdf_rev;
        const V3<T> f_cam = eval_bsdf(n_s, wo, mat, 1u, side, dir, cam_pdf_fwd, unused, false);
        const Mat<T> lm = load_material<T>(s, v.material_idx, V2<T>(v.uv[0], v.uv[1]));
        const V3<T> f_light = eval_bsdf(f3v<T>(v.n_s), f3v<T>(v.wo), lm, 0u, v.side == 1u, -dir, light_pdf_fwd, light_pdf_rev, true);
        if (is_zero(f_light) || is_zero(f_cam)) continue;
        cam_pdf_fwd *= std::fabs(cos_light) / len_sqr;
        light_pdf_fwd *= std::fabs(cos_cam) / len_sqr;
        const T w_light = cam_pdf_fwd * (eta_vm + v.d_vcm + light_pdf_rev * v.d_vc);
        const T w_camera = light_pdf_fwd * (eta_vm + cs.d_vcm + pdf_rev * cs.d_vc);
        const T mis = T(1) / (T(1) + w_camera + w_light);
        const V3<T> origin = offset_ray2(h.pos, n_s);
        const float o[3] = {(float)origin.x, (float)origin.y, (float)origin.z};
        const float d[3] = {(float)dir.x, (float)dir.y, (float)dir.z};
        if (!bvh_any(s.bvh, o, d, 0.0f, (float)(len - EPS))) {
            const V3<T> c = mis * G * cs.throughput * f3v<T>(v.throughput) * f_cam * f_light;
            res = (p->flags & 1u) ? res + c : c;
        }
    }
    return res;
}

// vcm_merge_light_vertices (vcm_commons.glsl:254-296) over the slot table: count and representative photon.
template <class T>
V3<T> merge(const orc_vcm_params* p, const Vertex<T>* verts, const Grid& g, uint32_t screen, int depth,
            const EyeHit<T>& h, V3<T> n_s, V3<T> wo, const Mat<T>& mat, bool side, T eta_vc,
            const VState<T>& cs, T radius, T norm) {
    const T r_sqr = radius * radius;
    V3<T> res(T(0));
    const I3 lo = grid_idx(to_f(h.pos - V3<T>(radius)), g.mn, g.mx, g.res);
    const I3 hi = grid_idx(to_f(h.pos + V3<T>(radius)), g.mn, g.mx, g.res);
    if ((int64_t)hi.x - lo.x >= kMaxMergeCells || (int64_t)hi.y - lo.y >= kMaxMergeCells ||
        (int64_t)hi.z - lo.z >= kMaxMergeCells)
        return res;
    for (int32_t x = lo.x; x <= hi.x; x++)
        for (int32_t y = lo.y; y <= hi.y; y++)
            for (int32_t z = lo.z; z <= hi.z; z++) {
                const uint32_t slot = grid_hash(I3{x, y, z}, screen);
                const uint32_t count = g.count[slot];
                if (count == 0) continue;
                const Vertex<T>& ph = verts[g.rep[slot]];
                const V3<T> pp = h.pos - f3v<T>(ph.pos);
                const T dist_sqr = dot(pp, pp);
                if (dist_sqr > r_sqr) continue;
                if (ph.path_len + (uint32_t)depth - 1u > (uint32_t)p->max_depth) continue;
                const V3<T> pwi = -f3v<T>(ph.wi);
                T cam_pdf_fwd, cam_pdf_rev;
                const V3<T> f = eval_bsdf(n_s, wo, mat, 1u, side, pwi, cam_pdf_fwd, cam_pdf_rev, true);
                if (is_zero(f)) continue;
                const T w_light = ph.d_vcm * eta_vc + ph.d_vm * cam_pdf_fwd;
                const T w_cam = cs.d_vcm * eta_vc + cs.d_vm * cam_pdf_rev;
                const T mis = T(1) / (T(1) + w_light + w_cam);
                const T cos_nrm = dot(f3v<T>(ph.n_s), n_s);
                if (cos_nrm > EPS) {
                    const T w = T(1) - std::sqrt(dist_sqr) / radius;
                    const V3<T> cc = w * mis * (T)(int32_t)count * f3v<T>(ph.throughput) * f * cs.throughput * norm * T(3);
                    res = (p->flags & 1u) ? res + cc : cc;
                }
            }
    return res;
}

// vcm_eye.rgen main + vcm_trace_eye for pixel (x, y); writes film[y * W + x] and consumes the pixel's splat.
template <class T>
void eye_path(const Scene& s, const Cam<T>& c, const orc_vcm_params* p, const Etas<T>& eta, uint32_t x, uint32_t y,
              const Vertex<T>* verts, const uint32_t* counts, const Grid& g, T* splat, T* film) {
    const uint32_t screen = c.W * c.H;
    U4 seed{x, y, p->eye_seed, 0u};
    const T j0 = rand(seed), j1 = rand(seed);
    const T px = (T)x + T(0.5), py = (T)y + T(0.5);
    const T u = (px + (j0 - T(0.5))) / (T)c.W, v = (py + (j1 - T(0.5))) / (T)c.H;
    const V2<T> d(u * T(2) - T(1), v * T(2) - T(1));
    VState<T> cs;
    cs.wi = sample_camera(c.iv, c.ip, d);
    cs.pos = c.pos;
    cs.throughput = V3<T>(T(1));
    const T cos_theta0 = std::fabs(dot(c.nrm, cs.wi));
    cs.d_vcm = c.area * (T)screen * cos_theta0 * cos_theta0 * cos_theta0;
    cs.d_vc = T(0);
    cs.d_vm = T(0);
    const T radius = eta.radius;
    const T norm = T(1) / (K<T>::PI() * radius * radius * (T)screen);

    const uint32_t lp = std::min((uint32_t)(rand(seed) * (float)screen), screen - 1u);  // can round up to screen
    const uint32_t lp_len = counts[lp];
    const Vertex<T>* lv = verts + (size_t)lp * (uint32_t)(p->max_depth + 1);
    V3<T> col(T(0));
    Payload<T> pl;
    pl.material_idx = -1;
    for (int depth = 1;; depth++) {
        trace_closest<T>(s, cs.pos, cs.wi, TMIN, TMAX, pl);
        if (pl.material_idx == -1) {
            col += cs.throughput * V3<T>(p->sky_col[0], p->sky_col[1], p->sky_col[2]);
            break;
        }
        V3<T> wo = cs.pos - pl.pos;
        const T dist = length(pl.pos - cs.pos);
        const T dist_sqr = dist * dist;
        wo /= dist;
        V3<T> n_s = pl.n_s, n_g = pl.n_g;
        bool side = true;
        if (dot(pl.n_g, wo) < T(0)) n_g = -n_g;
        if (dot(n_g, n_s) < T(0)) { n_s = -n_s; side = false; }
        const T cos_wo = std::fabs(dot(wo, n_s));
        const Mat<T> mat = load_material<T>(s, (uint32_t)pl.material_idx, pl.uv);
        const bool spec = (mat.bsdf_props & BSDF_FLAG_SPECULAR) == BSDF_FLAG_SPECULAR;
        cs.d_vcm *= dist_sqr;
        cs.d_vcm /= cos_wo;
        cs.d_vc /= cos_wo;
        cs.d_vm /= cos_wo;
        const EyeHit<T> h{pl.pos, pl.n_s, pl.area};
        if (luminance(mat.emissive_factor) > T(0)) {  // vcm_get_light_radiance
            V3<T> Le = mat.emissive_factor;
            if (depth != 1) {
                const T pdf_light_pos = T(1) / (h.area * (T)p->light_triangle_count);
                const T pdf_light_dir = std::fabs(dot(h.n_s_payload, -cs.wi)) / K<T>::PI();
                const T w_camera = pdf_light_pos * cs.d_vcm +
                                       ((p->use_vc == 1 || p->use_vm == 1) ? (pdf_light_pos * pdf_light_dir) * cs.d_vc : T(0));
                Le = (T(1) / (T(1) + w_camera)) * mat.emissive_factor;
            }
            col += cs.throughput * Le;
        }
        T pdf_rev = T(0);
        if (!spec && depth < p->max_depth) col += connect_light(s, p, seed, h, n_s, wo, mat, side, eta.vm, cs, pdf_rev);
        if (!spec) col += connect_light_vertices(s, p, lv, lp_len, depth, h, n_s, wo, mat, side, eta.vm, cs, pdf_rev);
        if (!spec && p->use_vm == 1)
            col += merge(p, verts, g, screen, depth, h, n_s, wo, mat, side, eta.vc, cs, radius, norm);
        if (depth >= p->max_depth) break;
        const T c0 = rand(seed), c1 = rand(seed), c2 = rand(seed);
        T pdf_dir, cos_theta;
        V3<T> wi;
        const V3<T> f = sample_bsdf(n_s, wo, mat, 1u, side, wi, pdf_dir, cos_theta, V3<T>(c0, c1, c2));
        cs.wi = wi;
        const bool trans = (mat.bsdf_props & BSDF_FLAG_TRANSMISSION) == BSDF_FLAG_TRANSMISSION;
        const bool same = dot(cs.wi, n_s) > T(0) && dot(wo, n_s) > T(0);
        if (is_zero(f) || pdf_dir == T(0) || (!same && !trans)) break;
        pdf_rev = pdf_dir;
        if (!spec) pdf_rev = bsdf_pdf(mat, n_s, cs.wi, wo, side);
        const T ac = std::fabs(cos_theta);
        cs.pos = offset_ray_t(pl.pos, n_g);
        if (!spec) {
            cs.d_vc = (ac / pdf_dir) * (eta.vm + cs.d_vcm + pdf_rev * cs.d_vc);
            cs.d_vm = (ac / pdf_dir) * (T(1) + cs.d_vcm * eta.vc + pdf_rev * cs.d_vm);
            cs.d_vcm = T(1) / pdf_dir;
        } else {
            cs.d_vcm = T(0);
            cs.d_vc *= ac;
            cs.d_vm *= ac;
        }
        cs.throughput *= f * ac / pdf_dir;
    }
    if (std::isnan(luminance(col))) return;  // vcm_eye.rgen:80-83: no film write, the splat stays
    const uint32_t pidx = x * c.H + y;
    col += V3<T>(splat[3 * pidx], splat[3 * pidx + 1], splat[3 * pidx + 2]);
    splat[3 * pidx] = splat[3 * pidx + 1] = splat[3 * pidx + 2] = T(0);
    T* out = film + 4 * ((size_t)y * c.W + x);
    if (p->frame_num > 0) {
        const T w = T(1) / (T)(p->frame_num + 1);
        out[0] = out[0] * (T(1) - w) + col.x * w;
        out[1] = out[1] * (T(1) - w) + col.y * w;
        out[2] = out[2] * (T(1) - w) + col.z * w;
    } else {
        out[0] = col.x; out[1] = col.y; out[2] = col.z;
    }
    out[3] = T(1);
}

}  // namespace

namespace {

// One VCM iteration (VCM::render, VCM.cpp:131-265, without the reservoir passes) in arithmetic type T.
template <class T>
void vcm_iteration(const Scene& s, const Cam<T>& c, const orc_vcm_params* p, Vertex<T>* verts, uint32_t* counts,
                   T* splat, uint32_t* grid_count, uint32_t* grid_rep, T* film, int nthreads) {
    const uint32_t width = c.W, height = c.H;
    const uint32_t screen = width * height;
    const Etas<T> eta = make_etas<T>(p, screen);
    std::vector<std::vector<Splat<T>>> splats(screen);
    parallel_for(screen, nthreads, [&](uint32_t i) {
        const uint32_t x = i / height, y = i % height;
        light_path<T>(s, c, p, eta, x, y, verts, counts, splats[i]);
    });
    for (uint32_t i = 0; i < screen; i++)  // light path order (x * height + y)
        for (const Splat<T>& sp : splats[i]) {
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
                const I3 gi = grid_idx(to_f(f3v<T>(verts[vid].pos)), g.mn, g.mx, g.res);
                const uint32_t slot = grid_hash(gi, screen);
                grid_count[slot]++;
                grid_rep[slot] = vid;
            }
    }
    g.count = grid_count;
    g.rep = grid_rep;
    parallel_for(screen, nthreads, [&](uint32_t i) {
        const uint32_t x = i / height, y = i % height;
        eye_path<T>(s, c, p, eta, x, y, verts, counts, g, splat, film);
    });
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

// One VCM iteration in FP32 (the shader's arithmetic). verts (W*H*(max_depth+1)), counts (W*H) and splat
// (W*H*3, pixel x*H+y) persist across iterations as the reference's buffers do; grid_count / grid_rep (10*W*H)
// receive the table.
void orc_vcm_iteration(void* scene, const float inv_view[16], const float inv_proj[16], const float view[16],
                       const float proj[16], uint32_t width, uint32_t height, const orc_vcm_params* p,
                       orc_vcm_vertex* verts, uint32_t* counts, float* splat, uint32_t* grid_count, uint32_t* grid_rep,
                       float* film, int nthreads) {
    const Cam<float> c = make_cam<float>(inv_view, inv_proj, view, proj, width, height);
    vcm_iteration<float>(*(const Scene*)scene, c, p, verts, counts, splat, grid_count, grid_rep, film, nthreads);
}

// `n_iters` VCM iterations in FP64 (converged reference renders): iteration i runs with params[i] (radius, seeds
// and frame number per iteration), the state kept in double between iterations; film is RGBA, W*H*4 doubles,
// the progressive mean of the iterations.
void orc_vcm_render_f64(void* scene, const float inv_view[16], const float inv_proj[16], const float view[16],
                        const float proj[16], uint32_t width, uint32_t height, const orc_vcm_params* params,
                        uint32_t n_iters, double* film, int nthreads) {
    const Cam<double> c = make_cam<double>(inv_view, inv_proj, view, proj, width, height);
    const size_t screen = (size_t)width * height;
    if (n_iters == 0) return;
    const uint32_t per = (uint32_t)(params[0].max_depth + 1);
    std::vector<VertexF64> verts(screen * per);
    std::vector<uint32_t> counts(screen, 0u), gc(10 * screen), gr(10 * screen);
    std::vector<double> splat(3 * screen, 0.0);
    for (uint32_t i = 0; i < n_iters; i++)
        vcm_iteration<double>(*(const Scene*)scene, c, &params[i], verts.data(), counts.data(), splat.data(), gc.data(),
                              gr.data(), film, nthreads);
}

}  // extern "C"
