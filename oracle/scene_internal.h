// Oracle (test infrastructure only): scene data and the helpers every CPU integrator of the oracle shares:
// hit attributes (ray.rchit:24-84), materials and textures (bsdf_commons.glsl:16-22), triangle and light
// sampling (commons.glsl:112-149, 173-215, 224-300), the camera ray (commons.glsl:30-33) and a thread pool.
#pragma once
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "oracle.h"
#include "shading.h"

namespace orc {
void* bvh_build_internal(const float* tri_verts, uint32_t n);
bool bvh_closest(void* bvh, const float* o, const float* d, float tmin, float tmax, uint32_t& prim, float& t, float& u,
                 float& v);
bool bvh_any(void* bvh, const float* o, const float* d, float tmin, float tmax);
}  // namespace orc

namespace orc {
namespace detail {




struct Scene {
    std::vector<float> pos, nrm, uv;
    std::vector<uint32_t> idx;
    std::vector<orc_mesh> meshes;
    std::vector<orc_material> mats;
    std::vector<orc_light> lights;
    struct Tex { uint32_t w, h; std::vector<float> rgba; };
    std::vector<Tex> texs;
    std::vector<uint32_t> tri_mesh;   // global triangle -> mesh
    std::vector<uint32_t> mesh_first_tri;
    void* bvh = nullptr;
};

const float EPS = 0.001f;          // utils.glsl:8
const float TMIN = 0.001f;         // path.rgen:19
const float TMAX = 10000.0f;       // path.rgen:20
const int RR_MIN_DEPTH = 3;        // path.rgen:21

template <class T> struct Payload {
    V3<T> n_g, n_s, pos;
    V2<T> uv;
    T area;  // world-space area of the hit triangle (ray.rchit:81)
    int32_t material_idx;
    uint32_t triangle_idx, instance_idx;
};

// Bilinear REPEAT lookup at LOD 0 in linear FP32 (stands in for texture() on the sampled image).
template <class T> V3<T> tex_lookup(const Scene& s, int id, V2<T> uv) {
    const Scene::Tex& t = s.texs[id];
    if (!std::isfinite(uv.x) || !std::isfinite(uv.y)) uv = V2<T>(0, 0);
    T x = uv.x * T(t.w) - T(0.5f), y = uv.y * T(t.h) - T(0.5f);
    T x0 = std::floor(x), y0 = std::floor(y);
    T fx = x - x0, fy = y - y0;
    auto wrap = [](long long i, uint32_t n) { long long m = i % (long long)n; return (uint32_t)(m < 0 ? m + n : m); };
    uint32_t i0 = wrap((long long)x0, t.w), i1 = wrap((long long)x0 + 1, t.w);
    uint32_t j0 = wrap((long long)y0, t.h), j1 = wrap((long long)y0 + 1, t.h);
    auto texel = [&](uint32_t i, uint32_t j) {
        const float* p = &t.rgba[4 * ((size_t)j * t.w + i)];
        return V3<T>(p[0], p[1], p[2]);
    };
    V3<T> c00 = texel(i0, j0), c10 = texel(i1, j0), c01 = texel(i0, j1), c11 = texel(i1, j1);
    T w00 = (T(1) - fx) * (T(1) - fy), w10 = fx * (T(1) - fy), w01 = (T(1) - fx) * fy, w11 = fx * fy;
    return c00 * w00 + c10 * w10 + c01 * w01 + c11 * w11;
}

template <class T> Mat<T> load_material(const Scene& s, uint32_t idx, V2<T> uv) {
    Mat<T> m = to_mat<T>(s.mats[idx]);
    if (m.texture_id > -1) m.albedo *= tex_lookup<T>(s, m.texture_id, uv);
    return m;
}

template <class T> V3<T> vtx_pos(const Scene& s, uint32_t v) { return V3<T>(s.pos[3 * v], s.pos[3 * v + 1], s.pos[3 * v + 2]); }
template <class T> V3<T> vtx_nrm(const Scene& s, uint32_t v) { return V3<T>(s.nrm[3 * v], s.nrm[3 * v + 1], s.nrm[3 * v + 2]); }
template <class T> V2<T> vtx_uv(const Scene& s, uint32_t v) { return V2<T>(s.uv[2 * v], s.uv[2 * v + 1]); }

// traceRayEXT closest + ray.rchit / ray.rmiss. Origins and directions are FP32 at the traversal boundary.
template <class T> void trace_closest(const Scene& s, V3<T> o, V3<T> d, float tmin, float tmax, Payload<T>& pl) {
    float of[3] = {(float)o.x, (float)o.y, (float)o.z}, df[3] = {(float)d.x, (float)d.y, (float)d.z};
    uint32_t prim; float t, bu, bv;
    if (!bvh_closest(s.bvh, of, df, tmin, tmax, prim, t, bu, bv)) {
        pl.material_idx = -1;  // ray.rmiss:13; every other payload field keeps its value
        return;
    }
    uint32_t mesh = s.tri_mesh[prim];
    const orc_mesh& pm = s.meshes[mesh];
    uint32_t local = prim - s.mesh_first_tri[mesh];
    uint32_t io = pm.index_offset + 3 * local;
    uint32_t i0 = s.idx[io] + pm.vertex_offset, i1 = s.idx[io + 1] + pm.vertex_offset, i2 = s.idx[io + 2] + pm.vertex_offset;
    V3<T> v0 = vtx_pos<T>(s, i0), v1 = vtx_pos<T>(s, i1), v2 = vtx_pos<T>(s, i2);
    V3<T> n0 = vtx_nrm<T>(s, i0), n1 = vtx_nrm<T>(s, i1), n2 = vtx_nrm<T>(s, i2);
    V2<T> uv0 = vtx_uv<T>(s, i0), uv1 = vtx_uv<T>(s, i1), uv2 = vtx_uv<T>(s, i2);
    V3<T> bary(T(1) - T(bu) - T(bv), T(bu), T(bv));
    V3<T> p = v0 * bary.x + v1 * bary.y + v2 * bary.z;
    V3<T> nrm = normalize(n0 * bary.x + n1 * bary.y + n2 * bary.z);
    // Object-to-world is the identity for every mesh Lumen's loader produces (LumenScene.cpp:328), so the
    // matrix products in ray.rchit:60,65,74 reduce to their arguments; the second normalize stays.
    V3<T> world_nrm = normalize(nrm);
    V2<T> uv = uv0 * bary.x + uv1 * bary.y + uv2 * bary.z;
    V3<T> e0 = v2 - v0, e1 = v1 - v0;
    pl.n_g = normalize(cross(e0, e1));
    pl.area = T(0.5f) * length(cross(e0, e1));
    pl.n_s = world_nrm;
    pl.pos = p;
    pl.uv = uv;
    pl.material_idx = (int32_t)pm.material_index;
    pl.triangle_idx = local;
    pl.instance_idx = mesh;
}

// commons.glsl:112-149 with an identity world matrix.
template <class T> void sample_triangle(const Scene& s, const orc_mesh& pm, V2<T> rands, uint32_t tri, V3<T>& pos, V3<T>& n_s,
                                        T& tri_pdf, V2<T>& uv) {
    uint32_t io = pm.index_offset + 3 * tri;
    uint32_t i0 = s.idx[io] + pm.vertex_offset, i1 = s.idx[io + 1] + pm.vertex_offset, i2 = s.idx[io + 2] + pm.vertex_offset;
    V3<T> v0 = vtx_pos<T>(s, i0), v1 = vtx_pos<T>(s, i1), v2 = vtx_pos<T>(s, i2);
    V3<T> n0 = vtx_nrm<T>(s, i0), n1 = vtx_nrm<T>(s, i1), n2 = vtx_nrm<T>(s, i2);
    uv = V2<T>(T(1) - std::sqrt(rands.x), rands.y * std::sqrt(rands.x));
    V3<T> b(T(1) - uv.x - uv.y, uv.x, uv.y);
    V3<T> et0 = v1 - v0, et1 = v2 - v0;
    V3<T> p = v0 * b.x + v1 * b.y + v2 * b.z;
    V3<T> nrm = normalize(n0 * b.x + n1 * b.y + n2 * b.z);
    n_s = normalize(nrm);
    tri_pdf = T(2) / length(cross(et0, et1));
    pos = p;
}

template <class T> struct LightSample {
    V3<T> L, wi;
    T wi_len, pdf_pos_w, pdf_pos_a, cos_from_light;
    uint32_t flags, triangle_idx, instance_idx;
};

// commons.glsl:224-300. A spot cone given by its two cosines replaces the fixed 30 / 25 degrees of
// commons.glsl:264-265 when cone_cos_width >= -1.
template <class T> LightSample<T> sample_light_Li(const Scene& s, V4<T> rands, V3<T> p, int num_lights,
                                                 T cone_cos_width = T(-2), T cone_cos_falloff = T(-2)) {
    LightSample<T> r;
    uint32_t light_idx = (uint32_t)(rands.x * T(num_lights));
    const orc_light& light = s.lights[light_idx];
    uint32_t light_type = light.light_flags & 0x7;
    r.L = V3<T>(0); r.flags = light.light_flags; r.pdf_pos_w = T(0); r.wi = V3<T>(0); r.wi_len = T(0);
    r.pdf_pos_a = T(0); r.cos_from_light = T(0); r.triangle_idx = 0; r.instance_idx = 0;
    if (light_type == LIGHT_AREA) {
        const orc_mesh& pm = s.meshes[light.prim_mesh_idx];
        uint32_t tri = (uint32_t)(rands.y * T(light.num_triangles));
        V3<T> lpos, ln; T tri_pdf; V2<T> bary;
        sample_triangle<T>(s, pm, V2<T>(rands.z, rands.w), tri, lpos, ln, tri_pdf, bary);
        Mat<T> light_mat = load_material<T>(s, pm.material_index, bary);
        V3<T> wi = lpos - p;
        T wi_len_sqr = dot(wi, wi);
        r.wi_len = std::sqrt(wi_len_sqr);
        wi /= r.wi_len;
        r.wi = wi;
        r.cos_from_light = std::fabs(dot(ln, -wi));
        r.L = light_mat.emissive_factor;
        r.pdf_pos_a = tri_pdf;
        r.pdf_pos_w = r.pdf_pos_a * wi_len_sqr / r.cos_from_light;
        r.triangle_idx = tri;
        r.instance_idx = light.prim_mesh_idx;
    } else if (light_type == LIGHT_SPOT) {
        V3<T> lp(light.pos[0], light.pos[1], light.pos[2]);
        V3<T> wi = lp - p;
        T wi_len_sqr = dot(wi, wi);
        r.wi_len = std::sqrt(wi_len_sqr);
        wi /= r.wi_len;
        r.wi = wi;
        V3<T> to(light.to[0], light.to[1], light.to[2]);
        const V3<T> light_dir = normalize(to - lp);
        r.cos_from_light = dot(-wi, light_dir);
        const T cos_width = cone_cos_width >= T(-1) ? cone_cos_width : std::cos(K<T>::PI() / T(6));
        const T cos_faloff = cone_cos_width >= T(-1) ? cone_cos_falloff : std::cos(T(25) * K<T>::PI() / T(180));
        T faloff;
        if (r.cos_from_light < cos_width) faloff = T(0);
        else if (r.cos_from_light >= cos_faloff) faloff = T(1);
        else {
            T dd = (r.cos_from_light - cos_width) / (cos_faloff - cos_width);
            faloff = (dd * dd) * (dd * dd);
        }
        r.pdf_pos_a = T(1);
        r.pdf_pos_w = wi_len_sqr;
        r.L = V3<T>(light.L[0], light.L[1], light.L[2]) * faloff;
    } else if (light_type == LIGHT_DIRECTIONAL) {
        V3<T> lp(light.pos[0], light.pos[1], light.pos[2]), to(light.to[0], light.to[1], light.to[2]);
        const V3<T> dir = normalize(lp - to);
        const V3<T> light_p = p + dir * (T(2) * T(light.world_radius));
        V3<T> wi = light_p - p;
        r.wi_len = length(wi);
        wi /= r.wi_len;
        r.wi = wi;
        r.pdf_pos_a = T(1);
        r.pdf_pos_w = T(1);
        r.L = V3<T>(light.L[0], light.L[1], light.L[2]);
        r.cos_from_light = T(1);
    }
    return r;
}

template <class T> V3<T> sample_camera(const M4<T>& inv_view, const M4<T>& inv_proj, V2<T> d) {
    V4<T> target = inv_proj * V4<T>(d.x, d.y, T(1), T(1));
    V3<T> n = normalize(target.xyz());
    V4<T> r = inv_view * V4<T>(n.x, n.y, n.z, T(0));
    return r.xyz();
}

template <class T> M4<T> load_m4(const float* m) {
    M4<T> r;
    for (int c = 0; c < 4; c++)
        for (int k = 0; k < 4; k++) r.m[c][k] = T(m[4 * c + k]);
    return r;
}

template <class F> void parallel_for(uint32_t n, int nthreads, F f) {
    if (nthreads <= 1 || n < 64) {
        for (uint32_t i = 0; i < n; i++) f(i);
        return;
    }
    std::atomic<uint32_t> next(0);
    std::vector<std::thread> th;
    for (int k = 0; k < nthreads; k++) {
        th.emplace_back([&]() {
            for (;;) {
                uint32_t b = next.fetch_add(64);
                if (b >= n) break;
                uint32_t e = std::min(n, b + 64);
                for (uint32_t i = b; i < e; i++) f(i);
            }
        });
    }
    for (auto& t : th) t.join();
}


}  // namespace detail
}  // namespace orc
