// Oracle (test infrastructure only): pieces shared by the CPU restatements of Lumen's photon integrators (VCM in
// vcm.cpp, SPPM in sppm.cpp): the photon grid's cell and hash (vcm_commons.glsl:17-23, utils.glsl:62-65) and
// resolution (VCM.cpp:144-147, SPPM.cpp:93-96), quaternion helpers (utils.glsl:157-175), light emission
// sampling (sample_light_Le, commons.glsl:335-406) and the positional-directional incidence sample
// (sample_light_Li, commons.glsl:224-300), area and spot lights.
#pragma once
#include <cstdint>

#include "scene_internal.h"

namespace orc {
namespace photon {
using namespace orc::detail;

// float -> int as GLSL int() / CUDA __float2int_rz: truncation, saturating, NaN -> 0.
inline int32_t to_int_rz(float x) {
    if (x != x) return 0;
    if (x >= 2147483648.0f) return INT32_MAX;
    if (x <= -2147483648.0f) return INT32_MIN;
    return (int32_t)x;
}

struct I3 { int32_t x, y, z; };

// utils.glsl:62-65: the products wrap as 32-bit integers.
inline uint32_t grid_hash(I3 p, uint32_t size) {
    const uint32_t h = ((uint32_t)p.x * 73856093u) ^ ((uint32_t)p.y * 19349663u) ^ ((uint32_t)p.z * 83492791u);
    return h % (10u * size);
}

// vcm_commons.glsl:17-23 (the clamp's result is discarded there, so cells outside the grid are possible).
inline I3 grid_idx(V3<float> p, const float* mn, const float* mx, const int32_t* res) {
    const float nx = (p.x - mn[0]) / (mx[0] - mn[0]), ny = (p.y - mn[1]) / (mx[1] - mn[1]), nz = (p.z - mn[2]) / (mx[2] - mn[2]);
    return I3{to_int_rz(nx * (float)res[0]), to_int_rz(ny * (float)res[1]), to_int_rz(nz * (float)res[2])};
}

// VCM.cpp:144-147
inline void grid_resolution(const float* mn, const float* mx, float radius, int32_t* res) {
    const float d[3] = {mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2]};
    const float max_comp = std::max(d[0], std::max(d[1], d[2]));
    const int base = to_int_rz(max_comp / radius);
    for (int k = 0; k < 3; k++) res[k] = std::max(to_int_rz(d[k] * (float)base / max_comp), 1);
}

template <class T> struct V4q { T x, y, z, w; };

template <class T> V4q<T> to_local_quat(V3<T> v) {  // utils.glsl:157-160
    if (v.z < T(-0.99999f)) return V4q<T>{T(1), T(0), T(0), T(0)};
    V4q<T> q{v.y, -v.x, T(0), T(1) + v.z};
    const T len = std::sqrt(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
    return V4q<T>{q.x / len, q.y / len, q.z / len, q.w / len};
}
template <class T> V3<T> rot_quat(V4q<T> q, V3<T> v) {  // utils.glsl:169-172
    const V3<T> a(q.x, q.y, q.z);
    return T(2) * dot(a, v) * a + (q.w * q.w - dot(a, a)) * v + T(2) * q.w * cross(a, v);
}
template <class T> V3<T> uniform_sample_cone(V2<T> uv, T cos_max) {  // commons.glsl:217-222
    const T cos_theta = (T(1) - uv.x) + uv.x * cos_max;
    const T sin_theta = std::sqrt(T(1) - cos_theta * cos_theta);
    const T phi = uv.y * K<T>::TWO_PI();
    return V3<T>(std::cos(phi) * sin_theta, std::sin(phi) * sin_theta, cos_theta);
}
template <class T> T uniform_cone_pdf(T cos_max) { return T(1) / (K<T>::TWO_PI() * (T(1) - cos_max)); }

inline bool light_finite(uint32_t f) { return ((f >> 4) & 1u) != 0; }
inline bool light_delta(uint32_t f) { return ((f >> 5) & 1u) != 0; }

// Light emission sample, commons.glsl:335-406 (area and spot lights; directional lights are refused upstream).
template <class T> struct Emission {
    V3<T> L, pos, wi, n;
    T cos_from_light, pdf_pos_a, pdf_dir_w;
    uint32_t flags;
};
// Spot cone: half-angle `angle` degrees, falloff from 25/30 of it; 0 gives commons.glsl:264-265's fixed 30 and
// 25 degrees. Computed in double and rounded once, as the library's host code does.
struct Cone { float cos_width, cos_falloff; };
inline Cone spot_cone(float angle) {
    const double a = angle > 0.0f ? (double)angle : 30.0;
    const double deg = 3.14159265358979323846 / 180.0;
    return Cone{(float)std::cos(a * deg), (float)std::cos(a * (25.0 / 30.0) * deg)};
}

template <class T> Emission<T> sample_light_Le(const Scene& s, V4<T> rp, V2<T> rd, int num_lights, int total_light,
                                              Cone cone) {
    Emission<T> e;
    const uint32_t light_idx = (uint32_t)(rp.x * T(num_lights));
    const orc_light& light = s.lights[light_idx];
    e.L = V3<T>(0); e.pos = V3<T>(0); e.wi = V3<T>(0); e.n = V3<T>(0);
    e.cos_from_light = T(0); e.pdf_pos_a = T(0); e.pdf_dir_w = T(0);
    e.flags = light.light_flags;
    const uint32_t type = light.light_flags & 0x7u;
    if (type == LIGHT_AREA) {
        const orc_mesh& pm = s.meshes[light.prim_mesh_idx];
        const uint32_t tri = (uint32_t)(rp.y * T(light.num_triangles));
        V3<T> pos, n; T tri_pdf; V2<T> bary;
        sample_triangle<T>(s, pm, V2<T>(rp.z, rp.w), tri, pos, n, tri_pdf, bary);
        const Mat<T> lm = load_material<T>(s, pm.material_index, bary);
        e.pos = pos;
        V3<T> Tt, B;
        branchless_onb(n, Tt, B);
        e.wi = to_world(sample_hemisphere(rd), Tt, B, n);  // sampling_commons.glsl:149-161
        e.L = lm.emissive_factor;
        e.cos_from_light = std::max(dot(n, e.wi), T(0));
        e.pdf_pos_a = tri_pdf;
        e.pdf_dir_w = dot(e.wi, n) / K<T>::PI();
        e.n = n;
    } else if (type == LIGHT_SPOT) {
        const T cos_width = T(cone.cos_width), cos_faloff = T(cone.cos_falloff);
        const V3<T> lp(light.pos[0], light.pos[1], light.pos[2]), to(light.to[0], light.to[1], light.to[2]);
        const V3<T> light_dir = normalize(to - lp);
        V4q<T> q = to_local_quat(light_dir);
        q = V4q<T>{-q.x, -q.y, -q.z, q.w};  // invert_quat
        e.wi = rot_quat(q, uniform_sample_cone(rd, cos_width));
        e.pos = lp;
        e.cos_from_light = dot(e.wi, light_dir);
        T faloff;
        if (e.cos_from_light < cos_width) faloff = T(0);
        else if (e.cos_from_light >= cos_faloff) faloff = T(1);
        else { const T d = (e.cos_from_light - cos_width) / (cos_faloff - cos_width); faloff = (d * d) * (d * d); }
        e.L = V3<T>(light.L[0], light.L[1], light.L[2]) * faloff;
        e.pdf_pos_a = T(1);
        e.pdf_dir_w = uniform_cone_pdf(cos_width);
        e.n = e.wi;
    }
    e.pdf_pos_a /= T(total_light);
    return e;
}

// sample_light_Li with the positional-directional pdf (commons.glsl:224-300, area and spot lights).
template <class T> struct Incidence {
    V3<T> L, wi, pos, n;  // pos, n: the light point and its normal (-wi for a spot light)
    T wi_len, pdf_pos_w, pdf_pos_dir_w, cos_y, pdf_pos_a;
    uint32_t flags;
};
template <class T> Incidence<T> sample_light_Li_pos(const Scene& s, V4<T> rp, V3<T> p, int num_lights, Cone cone) {
    Incidence<T> r;
    const uint32_t light_idx = (uint32_t)(rp.x * T(num_lights));
    const orc_light& light = s.lights[light_idx];
    r.L = V3<T>(0); r.wi = V3<T>(0); r.wi_len = T(0); r.pdf_pos_w = T(0); r.pdf_pos_dir_w = T(0); r.cos_y = T(0);
    r.pos = V3<T>(0); r.n = V3<T>(0); r.pdf_pos_a = T(0);
    r.flags = light.light_flags;
    const uint32_t type = light.light_flags & 0x7u;
    if (type == LIGHT_AREA) {
        const orc_mesh& pm = s.meshes[light.prim_mesh_idx];
        const uint32_t tri = (uint32_t)(rp.y * T(light.num_triangles));
        V3<T> pos, n; T tri_pdf; V2<T> bary;
        sample_triangle<T>(s, pm, V2<T>(rp.z, rp.w), tri, pos, n, tri_pdf, bary);
        const Mat<T> lm = load_material<T>(s, pm.material_index, bary);
        V3<T> wi = pos - p;
        const T l2 = dot(wi, wi);
        r.wi_len = std::sqrt(l2);
        wi /= r.wi_len;
        r.wi = wi;
        r.cos_y = std::fabs(dot(n, -wi));
        r.L = lm.emissive_factor;
        r.pdf_pos_w = tri_pdf * l2 / r.cos_y;
        r.pdf_pos_dir_w = r.cos_y * K<T>::INV_PI() * tri_pdf;
        r.pdf_pos_a = tri_pdf;
        r.n = n;
        r.pos = pos;
    } else if (type == LIGHT_SPOT) {
        const V3<T> lp(light.pos[0], light.pos[1], light.pos[2]), to(light.to[0], light.to[1], light.to[2]);
        V3<T> wi = lp - p;
        const T l2 = dot(wi, wi);
        r.wi_len = std::sqrt(l2);
        wi /= r.wi_len;
        r.wi = wi;
        const V3<T> light_dir = normalize(to - lp);
        r.cos_y = dot(-wi, light_dir);
        const T cos_width = T(cone.cos_width), cos_faloff = T(cone.cos_falloff);
        T faloff;
        if (r.cos_y < cos_width) faloff = T(0);
        else if (r.cos_y >= cos_faloff) faloff = T(1);
        else { const T d = (r.cos_y - cos_width) / (cos_faloff - cos_width); faloff = (d * d) * (d * d); }
        r.pdf_pos_w = l2;
        r.pdf_pos_dir_w = uniform_cone_pdf(cos_width);
        r.L = V3<T>(light.L[0], light.L[1], light.L[2]) * faloff;
        r.pdf_pos_a = T(1);
        r.n = -wi;
        r.pos = lp;
    }
    return r;
}

}  // namespace photon
}  // namespace orc
