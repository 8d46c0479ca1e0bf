// Oracle (test infrastructure only): line-by-line CPU restatement of Lumen's shading library, templated on
// the arithmetic type (float reproduces the shader's FP32 operation sequence; double gives FP64 references).
//
// Sources restated (paths inside the reference project):
//   src/shaders/utils.glsl            offset_ray 73-84, offset_ray2 90-93, luminance 99, pcg4d 121-133,
//                                     uint_to_float 136, init_rng/rand 138-154, branchless_onb 185-191,
//                                     to_world/to_local 193-195, concentric_sample_disk 215-229
//   src/shaders/bsdf/sampling_commons.glsl   all (SAMPLING_MODE 1 = concentric-disk hemisphere sampling)
//   src/shaders/bsdf/microfacet_commons.glsl all
//   src/shaders/bsdf/diffuse.glsl     Lambertian mode (DIFFUSE_BSDF_MODE 0)
//   src/shaders/bsdf/mirror.glsl, glass.glsl, dielectric.glsl, conductor.glsl, principled.glsl (ANISOTROPIC 1)
//   src/shaders/bsdf_commons.glsl     load_material 16-22, sample_bsdf 68-121, eval_bsdf 123-177
#pragma once
#include "glsl.h"
#include "oracle.h"

namespace orc {

template <class T> struct K;
template <> struct K<float> {
    static float PI() { return 3.14159265359f; }
    static float TWO_PI() { return 6.28318530718f; }
    static float INV_PI() { return 1.0f / 3.14159265359f; }
};
template <> struct K<double> {
    static double PI() { return 3.14159265359; }
    static double TWO_PI() { return 6.28318530718; }
    static double INV_PI() { return 1.0 / 3.14159265359; }
};

// commons.h:13-38
enum : uint32_t {
    BSDF_TYPE_DIFFUSE = 1u << 0, BSDF_TYPE_MIRROR = 1u << 1, BSDF_TYPE_GLASS = 1u << 2,
    BSDF_TYPE_DIELECTRIC = 1u << 3, BSDF_TYPE_CONDUCTOR = 1u << 4, BSDF_TYPE_PRINCIPLED = 1u << 5,
    BSDF_FLAG_DIFFUSE = 1u << 0, BSDF_FLAG_SPECULAR = 1u << 1, BSDF_FLAG_GLOSSY = 1u << 2,
    BSDF_FLAG_REFLECTION = 1u << 3, BSDF_FLAG_TRANSMISSION = 1u << 4,
    LIGHT_SPOT = 1, LIGHT_AREA = 2, LIGHT_DIRECTIONAL = 3,
};

template <class T> struct Mat {
    V3<T> albedo; T ior; V3<T> emissive_factor; uint32_t bsdf_type; uint32_t bsdf_props; V3<T> k; int32_t texture_id;
    T roughness, diffuse_trans, spec_trans, metallic, specular_tint, sheen_tint, clearcoat, clearcoat_gloss, sheen,
        subsurface, flatness, anisotropy;
    uint32_t thin;
};

template <class T> inline Mat<T> to_mat(const orc_material& m) {
    Mat<T> r;
    r.albedo = V3<T>(m.albedo[0], m.albedo[1], m.albedo[2]);
    r.ior = m.ior;
    r.emissive_factor = V3<T>(m.emissive_factor[0], m.emissive_factor[1], m.emissive_factor[2]);
    r.bsdf_type = m.bsdf_type; r.bsdf_props = m.bsdf_props;
    r.k = V3<T>(m.k[0], m.k[1], m.k[2]);
    r.texture_id = m.texture_id;
    r.roughness = m.roughness; r.diffuse_trans = m.diffuse_trans; r.spec_trans = m.spec_trans;
    r.metallic = m.metallic; r.specular_tint = m.specular_tint; r.sheen_tint = m.sheen_tint;
    r.clearcoat = m.clearcoat; r.clearcoat_gloss = m.clearcoat_gloss; r.sheen = m.sheen;
    r.subsurface = m.subsurface; r.flatness = m.flatness; r.anisotropy = m.anisotropy; r.thin = m.thin;
    return r;
}

inline bool bsdf_has_property(uint32_t props, uint32_t flag) { return (props & flag) != 0; }

// ---------------- utils.glsl ----------------
struct U4 { uint32_t x, y, z, w; };

inline U4 pcg4d(U4 v) {
    v.x = v.x * 1664525u + 1013904223u; v.y = v.y * 1664525u + 1013904223u;
    v.z = v.z * 1664525u + 1013904223u; v.w = v.w * 1664525u + 1013904223u;
    v.x += v.y * v.w; v.y += v.z * v.x; v.z += v.x * v.y; v.w += v.y * v.z;
    v.x ^= v.x >> 16u; v.y ^= v.y >> 16u; v.z ^= v.z >> 16u; v.w ^= v.w >> 16u;
    v.x += v.y * v.w; v.y += v.z * v.x; v.z += v.x * v.y; v.w += v.y * v.z;
    return v;
}
// uint_to_float: [1,2) mantissa trick minus one, computed in FP32 (the draw is FP32 in both precisions).
inline float uint_to_float(uint32_t x) { return u2f(0x3f800000u | (x >> 9)) - 1.0f; }
inline float rand(U4& s) { s.w++; return uint_to_float(pcg4d(s).x); }

inline V3<float> offset_ray(V3<float> p, V3<float> n) {
    const float origin = 1.0f / 32.0f, float_scale = 1.0f / 65536.0f, int_scale = 256.0f;
    int32_t ox = (int32_t)(int_scale * n.x), oy = (int32_t)(int_scale * n.y), oz = (int32_t)(int_scale * n.z);
    V3<float> pi(i2f(f2i(p.x) + ((p.x < 0) ? -ox : ox)), i2f(f2i(p.y) + ((p.y < 0) ? -oy : oy)),
                 i2f(f2i(p.z) + ((p.z < 0) ? -oz : oz)));
    return V3<float>(std::fabs(p.x) < origin ? p.x + float_scale * n.x : pi.x,
                     std::fabs(p.y) < origin ? p.y + float_scale * n.y : pi.y,
                     std::fabs(p.z) < origin ? p.z + float_scale * n.z : pi.z);
}
template <class T> inline V3<T> offset_ray2(V3<T> p, V3<T> n) {
    const T float_scale = T(2.0f / 65536.0f);
    return p + float_scale * n;
}
template <class T> inline T luminance(V3<T> rgb) { return dot(rgb, V3<T>(T(0.2126f), T(0.7152f), T(0.0722f))); }

template <class T> inline void branchless_onb(V3<T> n, V3<T>& b1, V3<T>& b2) {
    T sgn = n.z >= T(0) ? T(1) : T(-1);
    T a = T(-1) / (sgn + n.z);
    T b = n.x * n.y * a;
    b1 = V3<T>(T(1) + sgn * n.x * n.x * a, sgn * b, -sgn * n.x);
    b2 = V3<T>(b, sgn + n.y * n.y * a, -n.y);
}
template <class T> inline V3<T> to_world(V3<T> v, V3<T> Tt, V3<T> B, V3<T> N) { return v.x * Tt + v.y * B + v.z * N; }
template <class T> inline V3<T> to_local(V3<T> v, V3<T> Tt, V3<T> B, V3<T> N) {
    return V3<T>(dot(v, Tt), dot(v, B), dot(v, N));
}
template <class T> inline V2<T> concentric_sample_disk(V2<T> rands) {
    V2<T> offset = T(2) * rands - T(1);
    if (offset.x == T(0) && offset.y == T(0)) return V2<T>(0, 0);
    T theta, r;
    if (std::fabs(offset.x) > std::fabs(offset.y)) {
        r = offset.x;
        theta = T(0.25f) * K<T>::PI() * offset.y / offset.x;
    } else {
        r = offset.y;
        theta = K<T>::PI() * (T(0.5f) - T(0.25f) * offset.x / offset.y);
    }
    return r * V2<T>(std::cos(theta), std::sin(theta));
}

// ---------------- sampling_commons.glsl ----------------
template <class T> inline T schlick_w(T u) { T m = clamp(T(1) - u, T(0), T(1)); T m2 = m * m; return m2 * m2 * m; }
template <class T> inline bool bsdf_is_effectively_delta(T alpha) { return alpha <= T(0.0064f); }
template <class T> inline bool bsdf_is_effectively_delta(V2<T> a) { return gmin(a.x, a.y) <= T(0.0064f); }

template <class T>
inline bool refract(V3<T> n_s, V3<T> wo, bool forward_facing, T eta, uint32_t mode, V3<T>& wi, V3<T>& f, T& inv_eta) {
    wi = V3<T>(0); f = V3<T>(0);
    T cos_i = dot(n_s, wo);
    inv_eta = forward_facing ? T(1) / eta : eta;
    const T sin2_t = inv_eta * inv_eta * (T(1) - cos_i * cos_i);
    if (sin2_t >= T(1)) {
        wi = reflect(-wo, n_s);
    } else {
        const T cos_t = std::sqrt(T(1) - sin2_t);
        wi = -inv_eta * wo + (inv_eta * cos_i - cos_t) * n_s;
    }
    f = mode == 1 ? V3<T>(inv_eta * inv_eta) : V3<T>(1);
    return true;
}
template <class T> inline bool refract(V3<T> n_s, V3<T> wo, bool ff, T eta, uint32_t mode, V3<T>& wi, V3<T>& f) {
    T unused; return refract(n_s, wo, ff, eta, mode, wi, f, unused);
}

template <class T> inline T fresnel_dielectric(T cos_i, T eta, bool forward_facing) {
    cos_i = clamp(cos_i, T(-1), T(1));
    if (!forward_facing) eta = T(1) / eta;
    if (cos_i < T(0)) { eta = T(1) / eta; cos_i = -cos_i; }
    T sin2_i = T(1) - cos_i * cos_i;
    T sin2_t = sin2_i / (eta * eta);
    if (sin2_t >= T(1)) return T(1);
    T cos_t = std::sqrt(T(1) - sin2_t);
    T r_parallel = (eta * cos_i - cos_t) / (eta * cos_i + cos_t);
    T r_perp = (cos_i - eta * cos_t) / (cos_i + eta * cos_t);
    return T(0.5f) * (r_parallel * r_parallel + r_perp * r_perp);
}

template <class T> inline T fresnel_conductor(T cos_i, T eta, T k) {
    T cos_sqr = cos_i * cos_i;
    T sin_sqr = gmax(T(1) - cos_sqr, T(0));
    T sin_4 = sin_sqr * sin_sqr;
    T inner_term = eta * eta - k * k - sin_sqr;
    T a_sq_p_b_sq = std::sqrt(gmax(inner_term * inner_term + T(4) * eta * eta * k * k, T(0)));
    T a = std::sqrt(gmax((a_sq_p_b_sq + inner_term) * T(0.5f), T(0)));
    T rs = ((a_sq_p_b_sq + cos_sqr) - (T(2) * a * cos_i)) / ((a_sq_p_b_sq + cos_sqr) + (T(2) * a * cos_i));
    T rp = ((cos_sqr * a_sq_p_b_sq + sin_4) - (T(2) * a * cos_i * sin_sqr)) /
           ((cos_sqr * a_sq_p_b_sq + sin_4) + (T(2) * a * cos_i * sin_sqr));
    return T(0.5f) * (rs + rs * rp);
}
template <class T> inline V3<T> fresnel_conductor(T cos_i, V3<T> eta, V3<T> k) {
    return V3<T>(fresnel_conductor(cos_i, eta.x, k.x), fresnel_conductor(cos_i, eta.y, k.y),
                 fresnel_conductor(cos_i, eta.z, k.z));
}
template <class T> inline T fresnel_schlick(T f0, T f90, T ns) {
    return f0 + (f90 - f0) * std::pow(gmax(T(1) - ns, T(0)), T(5));
}
template <class T> inline V3<T> fresnel_schlick(V3<T> f0, V3<T> f90, T ns) {
    T p = std::pow(gmax(T(1) - ns, T(0)), T(5));
    return f0 + (f90 - f0) * p;
}
template <class T> inline T eta_to_schlick_R0(T eta) { T val = (eta - T(1)) / (eta + T(1)); return val * val; }

template <class T> inline T disney_fresnel(V3<T> wi, V3<T> wo, T roughness, T& f_wi, T& f_wo) {
    V3<T> h = normalize(wi + wo);
    T wo_dot_h = dot(wo, h);
    T fd90 = T(0.5f) + T(2) * wo_dot_h * wo_dot_h * roughness;
    T fd0 = T(1);
    f_wi = fresnel_schlick(fd0, fd90, wi.z);
    f_wo = fresnel_schlick(fd0, fd90, wo.z);
    return f_wi * f_wo;
}
template <class T> inline V3<T> calc_tint(V3<T> albedo) {
    T lum = luminance(albedo);
    return lum > T(0) ? albedo / lum : V3<T>(1);
}
template <class T> inline V3<T> disney_fresnel(const Mat<T>& mat, V3<T> wo, V3<T> h, V3<T> wi, T eta) {
    T wo_dot_h = dot(wo, h);
    V3<T> R0 = eta_to_schlick_R0(eta) * mix(V3<T>(1), calc_tint(mat.albedo), mat.specular_tint);
    R0 = mix(R0, mat.albedo, mat.metallic);
    T fr_dielectric = fresnel_dielectric(wo_dot_h, eta, true);
    V3<T> fr_metallic = fresnel_schlick(R0, V3<T>(1), wo_dot_h);
    return mix(V3<T>(fr_dielectric), fr_metallic, mat.metallic);
}

// sample_hemisphere, local frame, SAMPLING_MODE_CONCENTRIC_DISK_MAPPING (sampling_commons.glsl:169-179)
template <class T> inline V3<T> sample_hemisphere(V2<T> xi) {
    V2<T> d = concentric_sample_disk(xi);
    T z = std::sqrt(gmax(T(0), T(1) - dot(d, d)));
    return V3<T>(d.x, d.y, z);
}

// ---------------- microfacet_commons.glsl ----------------
template <class T> inline T Smith_lambda_isotropic(T alpha_sqr, T cos_theta) {
    if (cos_theta == T(0)) return T(0);
    T cos_sqr = cos_theta * cos_theta;
    T tan_sqr = gmax(T(1) - cos_sqr, T(0)) / cos_sqr;
    return T(0.5f) * (std::sqrt(T(1) + alpha_sqr * tan_sqr) - T(1));
}
template <class T> inline T Smith_lambda_anisotropic(V3<T> w, V2<T> alpha) {
    T cos_sqr = w.z * w.z;
    T sin_sqr = gmax(T(1) - cos_sqr, T(0));
    T tan_sqr = sin_sqr / cos_sqr;
    if (std::isinf(tan_sqr)) return T(0);
    V2<T> cos_phi_sqr = sin_sqr == T(0) ? V2<T>(1, 0)
                                        : V2<T>(clamp(w.x * w.x, T(0), T(1)) / sin_sqr, clamp(w.y * w.y, T(0), T(1)) / sin_sqr);
    T alpha_sqr = dot(cos_phi_sqr, V2<T>(alpha.x * alpha.x, alpha.y * alpha.y));
    return T(0.5f) * (std::sqrt(T(1) + alpha_sqr * tan_sqr) - T(1));
}
template <class T> inline T G1_GGX_anisotropic(V3<T> w, V2<T> alpha) { return T(1) / (T(1) + Smith_lambda_anisotropic(w, alpha)); }
template <class T> inline T G_GGX_correlated_isotropic(T alpha, V3<T> wo, V3<T> wi) {
    T alpha_sqr = alpha * alpha;
    return T(1) / (T(1) + Smith_lambda_isotropic(alpha_sqr, wo.z) + Smith_lambda_isotropic(alpha_sqr, wi.z));
}
template <class T> inline T G_GGX_correlated_anisotropic(V2<T> alpha, V3<T> wo, V3<T> wi) {
    return T(1) / (T(1) + Smith_lambda_anisotropic(wo, alpha) + Smith_lambda_anisotropic(wi, alpha));
}
template <class T> inline T D_GGX_anisotropic(V2<T> alpha, V3<T> h) {
    T cos_sqr = h.z * h.z;
    T sin_sqr = gmax(T(1) - cos_sqr, T(0));
    T tan_sqr = sin_sqr / cos_sqr;
    if (std::isinf(tan_sqr)) return T(0);
    T cos_4 = cos_sqr * cos_sqr;
    if (cos_4 < T(1e-16f)) return T(0);
    V2<T> phi_sqr = sin_sqr == T(0) ? V2<T>(1, 0)
                                    : V2<T>(clamp(h.x * h.x, T(0), T(1)) / sin_sqr, clamp(h.y * h.y, T(0), T(1)) / sin_sqr);
    V2<T> alpha_sqr(phi_sqr.x / (alpha.x * alpha.x), phi_sqr.y / (alpha.y * alpha.y));
    T e = tan_sqr * (alpha_sqr.x + alpha_sqr.y);
    return T(1) / (K<T>::PI() * alpha.x * alpha.y * cos_4 * (T(1) + e) * (T(1) + e));
}
template <class T> inline T D_GGX_isotropic(T alpha_sqr, T cos_theta) {
    T d = ((cos_theta * alpha_sqr - cos_theta) * cos_theta + T(1));
    return alpha_sqr / (d * d * K<T>::PI());
}
template <class T> inline T G1_GGX_isotropic(T alpha_sqr, T cos_theta) {
    T cos_sqr = cos_theta * cos_theta;
    T tan_sqr = gmax(T(1) - cos_sqr, T(0)) / cos_sqr;
    return T(2) / (T(1) + std::sqrt(T(1) + alpha_sqr * tan_sqr));
}
template <class T> inline T eval_vndf_pdf_isotropic(T alpha, V3<T> wo, V3<T> h, T& D) {
    D = T(0);
    if (wo.z <= T(0)) return T(0);
    T alpha_sqr = alpha * alpha;
    T G1 = G1_GGX_isotropic(alpha_sqr, wo.z);
    D = D_GGX_isotropic(alpha_sqr, h.z);
    return G1 * D * gmax(T(0), dot(wo, h)) / std::fabs(wo.z);
}
template <class T> inline T eval_vndf_pdf_isotropic(T alpha, V3<T> wo, V3<T> h) { T D; return eval_vndf_pdf_isotropic(alpha, wo, h, D); }
template <class T> inline T eval_vndf_pdf_anisotropic(V2<T> alpha, V3<T> wo, V3<T> h, T& D) {
    D = T(0);
    if (wo.z <= T(0)) return T(0);
    T G1 = G1_GGX_anisotropic(wo, alpha);
    D = D_GGX_anisotropic(alpha, h);
    return G1 * D * gmax(T(0), dot(wo, h)) / std::fabs(wo.z);
}
template <class T> inline T eval_vndf_pdf_anisotropic(V2<T> alpha, V3<T> wo, V3<T> h) { T D; return eval_vndf_pdf_anisotropic(alpha, wo, h, D); }

template <class T> inline V3<T> sample_ggx_vndf_common(V2<T> alpha, V3<T> wo, V2<T> xi) {
    V3<T> wo_hemisphere = normalize(V3<T>(alpha.x * wo.x, alpha.y * wo.y, wo.z));
    T phi = T(2) * K<T>::PI() * xi.x;
    T z = ((T(1) - xi.y) * (T(1) + wo_hemisphere.z)) - wo_hemisphere.z;
    T sin_theta = std::sqrt(clamp(T(1) - z * z, T(0), T(1)));
    T x = sin_theta * std::cos(phi);
    T y = sin_theta * std::sin(phi);
    V3<T> n_h = V3<T>(x, y, z) + wo_hemisphere;
    return normalize(V3<T>(alpha.x * n_h.x, alpha.y * n_h.y, gmax(T(0), n_h.z)));
}
template <class T> inline V3<T> sample_ggx_vndf_isotropic(V2<T> alpha, V3<T> wo, V2<T> xi, T& pdf, T& D) {
    V3<T> h = sample_ggx_vndf_common(alpha, wo, xi);
    pdf = eval_vndf_pdf_isotropic(alpha.x, wo, h, D);
    return h;
}
template <class T> inline V3<T> sample_ggx_vndf_anisotropic(V2<T> alpha, V3<T> wo, V2<T> xi, T& pdf, T& D) {
    V3<T> h = sample_ggx_vndf_common(alpha, wo, xi);
    pdf = eval_vndf_pdf_anisotropic(alpha, wo, h, D);
    return h;
}

// ---------------- diffuse.glsl (Lambertian) ----------------
template <class T> inline V3<T> sample_diffuse(const Mat<T>& mat, V3<T> wo, V3<T>& wi, T& pdf_w, T& cos_theta, V2<T> xi) {
    pdf_w = T(0);
    wi = sample_hemisphere(xi);
    cos_theta = wi.z;
    pdf_w = cos_theta * K<T>::INV_PI();
    if (gmin(wi.z, wo.z) <= T(0)) return V3<T>(0);
    return mat.albedo * K<T>::INV_PI();
}
template <class T> inline V3<T> eval_diffuse(const Mat<T>& mat, V3<T> wo, V3<T> wi, T& pdf_w, T& pdf_rev_w) {
    pdf_w = T(0); pdf_rev_w = T(0);
    if (gmin(wi.z, wo.z) <= T(0)) return V3<T>(0);
    pdf_w = wi.z * K<T>::INV_PI();
    pdf_rev_w = pdf_w;
    return mat.albedo * K<T>::INV_PI();
}
template <class T> inline T eval_diffuse_pdf(V3<T> wo, V3<T> wi) {
    if (gmin(wi.z, wo.z) <= T(0)) return T(0);
    return wi.z * K<T>::INV_PI();
}

// ---------------- mirror.glsl / glass.glsl ----------------
template <class T> inline V3<T> sample_mirror(V3<T> n_s, V3<T> wo, V3<T>& wi, T& pdf_w, T& cos_theta) {
    if (dot(wo, n_s) <= T(0)) { pdf_w = T(0); cos_theta = T(0); wi = V3<T>(0); return V3<T>(0); }
    wi = reflect(-wo, n_s);
    cos_theta = dot(wi, n_s);
    pdf_w = T(1);
    return V3<T>(1) / V3<T>(cos_theta);
}
template <class T>
inline V3<T> sample_glass(const Mat<T>& mat, V3<T> n_s, V3<T> wo, V3<T>& wi, T& pdf_w, T& cos_theta, uint32_t mode, bool ff) {
    wi = V3<T>(0); pdf_w = T(0); cos_theta = T(0);
    V3<T> f;
    if (!refract(n_s, wo, ff, mat.ior, mode, wi, f)) return V3<T>(0);
    cos_theta = dot(n_s, wi);
    pdf_w = T(1);
    f /= std::fabs(cos_theta);
    return f;
}

// ---------------- conductor.glsl ----------------
template <class T> inline V3<T> sample_conductor(const Mat<T>& mat, V3<T> wo, V3<T>& wi, T& pdf_w, T& cos_theta, V2<T> xi) {
    wi = V3<T>(0); pdf_w = T(0); cos_theta = T(0);
    if (wo.z <= T(0)) return V3<T>(0);
    T alpha = mat.roughness * mat.roughness;
    bool has_reflection = bsdf_has_property(mat.bsdf_props, BSDF_FLAG_REFLECTION);
    if (!has_reflection) return V3<T>(0);
    if (bsdf_is_effectively_delta(alpha)) {
        wi = V3<T>(-wo.x, -wo.y, wo.z);
        pdf_w = T(1);
        cos_theta = wi.z;
        V3<T> F = fresnel_conductor(cos_theta, mat.albedo, mat.k);
        return F / std::fabs(cos_theta);
    }
    T D;
    V3<T> h = sample_ggx_vndf_isotropic(V2<T>(alpha, alpha), wo, xi, pdf_w, D);
    V3<T> F = fresnel_conductor(dot(wo, h), mat.albedo, mat.k);
    wi = reflect(-wo, h);
    if (wo.z * wi.z < T(0)) return V3<T>(0);
    pdf_w /= (T(4) * dot(wo, h));
    cos_theta = wi.z;
    return T(0.25f) * D * F * G_GGX_correlated_isotropic(alpha, wo, wi) / (wi.z * wo.z);
}
template <class T> inline V3<T> eval_conductor(const Mat<T>& mat, V3<T> wo, V3<T> wi, T& pdf_w, T& pdf_rev_w, bool eval_reverse_pdf) {
    pdf_w = T(0); pdf_rev_w = T(0);
    T alpha = mat.roughness * mat.roughness;
    if (bsdf_is_effectively_delta(alpha)) return V3<T>(0);
    if (wo.z * wi.z < T(0)) return V3<T>(0);
    if (wo.z == T(0) || wi.z == T(0)) return V3<T>(0);
    V3<T> h = normalize(wo + wi);
    h *= T(sign(h.z));
    T jacobian = T(1) / (T(4) * dot(wo, h));
    T D;
    pdf_w = eval_vndf_pdf_isotropic(alpha, wo, h, D) * jacobian;
    if (eval_reverse_pdf) pdf_rev_w = eval_vndf_pdf_isotropic(alpha, wi, h) * jacobian;
    V3<T> F = fresnel_conductor(dot(wo, h), mat.albedo, mat.k);
    return T(0.25f) * D * F * G_GGX_correlated_isotropic(alpha, wo, wi) / (wi.z * wo.z);
}

// ---------------- dielectric.glsl ----------------
template <class T> inline T modify_thin_roughness(T ior, T roughness) {
    return clamp((T(0.65f) * ior - T(0.35f)) * roughness, T(0), T(1));
}
template <class T>
inline V3<T> sample_dielectric(const Mat<T>& mat, V3<T> wo, V3<T>& wi, uint32_t mode, bool ff, T& pdf_w, T& cos_theta, V2<T> xi) {
    wi = V3<T>(0); pdf_w = T(0); cos_theta = T(0);
    if (wo.z <= T(0)) return V3<T>(0);
    T roughness = mat.thin == 1 ? modify_thin_roughness(mat.ior, mat.roughness) : mat.roughness;
    T alpha = roughness * roughness;
    bool has_reflection = bsdf_has_property(mat.bsdf_props, BSDF_FLAG_REFLECTION);
    bool has_transmission = bsdf_has_property(mat.bsdf_props, BSDF_FLAG_TRANSMISSION);
    if ((mat.ior == T(1) && mat.thin == 0) || bsdf_is_effectively_delta(alpha)) {
        T F = fresnel_dielectric(wo.z, mat.ior, ff);
        if (!has_reflection && !has_transmission) return V3<T>(0);
        T pr = F, pt = T(1) - F;
        if (!has_reflection) pr = T(0);
        if (!has_transmission) pt = T(0);
        bool is_reflection = ((pr + pt) * xi.x) < pr;
        V3<T> f;
        if (is_reflection) {
            wi = V3<T>(-wo.x, -wo.y, wo.z);
            cos_theta = wi.z;
            f = V3<T>(F) / V3<T>(std::fabs(cos_theta));
            pdf_w = pr / (pr + pt);
        } else {
            if (!refract(V3<T>(0, 0, 1), wo, ff, mat.ior, mode, wi, f)) return V3<T>(0);
            cos_theta = wi.z;
            f = f * (T(1) - F) / std::fabs(cos_theta);
            pdf_w = pt / (pr + pt);
        }
        return f;
    }
    if (!has_reflection && !has_transmission) return V3<T>(0);
    T D;
    V3<T> h = sample_ggx_vndf_isotropic(V2<T>(alpha, alpha), wo, xi, pdf_w, D);
    T F = fresnel_dielectric(dot(wo, h), mat.ior, ff);
    T pr = has_reflection ? F : T(0);
    T pt = has_transmission ? (T(1) - F) : T(0);
    bool is_reflection = ((pr + pt) * xi.x) < pr;
    V3<T> f;
    if (is_reflection) {
        wi = reflect(-wo, h);
        if (wo.z * wi.z < T(0)) return V3<T>(0);
        pdf_w = pdf_w * (pr / (pr + pt)) / (T(4) * std::fabs(dot(wo, h)));
        f = V3<T>(T(0.25f) * D * F * G_GGX_correlated_isotropic(alpha, wo, wi) / (wi.z * wo.z));
    } else {
        V3<T> base_col;
        T possibly_modified_inv_eta;
        bool tir = false;
        if (mat.thin == 1) {
            wi = reflect(-wo, h);
            base_col = vsqrt(mat.albedo);
            possibly_modified_inv_eta = mat.ior;
        } else {
            tir = !refract(h, wo, ff, mat.ior, mode, wi, f, possibly_modified_inv_eta);
            base_col = mat.albedo;
        }
        if (wo.z * wi.z > T(0) || wi.z > T(0) || tir) return V3<T>(0);
        T jacobian_denom = dot(wi, h) + dot(wo, h) * possibly_modified_inv_eta;
        jacobian_denom = jacobian_denom * jacobian_denom;
        T jacobian = std::fabs(dot(wi, h)) / jacobian_denom;
        pdf_w = pdf_w * (pt / (pr + pt)) * jacobian;
        f = base_col * f * (T(1) - F) * D * G_GGX_correlated_isotropic(alpha, wo, wi) *
            std::fabs(dot(wi, h) * dot(wo, h) / (wi.z * wo.z * jacobian_denom));
    }
    cos_theta = wi.z;
    return f;
}

template <class T>
inline V3<T> eval_dielectric(const Mat<T>& mat, V3<T> wo, V3<T> wi, T& pdf_w, T& pdf_rev_w, bool ff, uint32_t mode, bool eval_reverse_pdf) {
    pdf_w = T(0); pdf_rev_w = T(0);
    T roughness = mat.thin == 1 ? modify_thin_roughness(mat.ior, mat.roughness) : mat.roughness;
    T alpha = roughness * roughness;
    if (alpha == T(0) || mat.ior == T(1)) return V3<T>(0);
    bool has_reflection = bsdf_has_property(mat.bsdf_props, BSDF_FLAG_REFLECTION);
    bool has_transmission = bsdf_has_property(mat.bsdf_props, BSDF_FLAG_TRANSMISSION);
    if (!has_reflection && !has_transmission) return V3<T>(0);
    T eta = T(1);
    bool is_reflection = wi.z * wo.z > T(0);
    if (!is_reflection) eta = ff ? mat.ior : T(1) / mat.ior;
    V3<T> h = normalize(wo + wi * eta);
    h *= T(sign(h.z));
    if (wi.z == T(0) || wo.z == T(0) || dot(h, h) == T(0)) return V3<T>(0);
    if (dot(wi, h) * wi.z < T(0) || dot(wo, h) * wo.z < T(0)) return V3<T>(0);
    T F = fresnel_dielectric(dot(wo, h), mat.ior, ff);
    T pr = has_reflection ? F : T(0);
    T pt = has_transmission ? (T(1) - F) : T(0);
    T D;
    if (eval_reverse_pdf) pdf_rev_w = eval_vndf_pdf_isotropic(alpha, wi, -h, D);
    pdf_w = eval_vndf_pdf_isotropic(alpha, wo, h, D);
    T G = G_GGX_correlated_isotropic(alpha, wo, wi);
    V3<T> f;
    if (is_reflection) {
        T jacobian = T(1) / (T(4) * std::fabs(dot(wo, h)));
        T prob_reflection = pr / (pr + pt);
        pdf_w = pdf_w * jacobian * prob_reflection;
        if (eval_reverse_pdf) {
            T jacobian_reverse = T(1) / (T(4) * std::fabs(dot(wi, h)));
            pdf_rev_w = pdf_rev_w * jacobian_reverse * prob_reflection;
        }
        f = V3<T>(T(0.25f) * D * G * F / std::fabs(wo.z * wi.z));
    } else {
        T jacobian_denom = dot(wi, h) + dot(wo, h) / eta;
        jacobian_denom = jacobian_denom * jacobian_denom;
        T jacobian = std::fabs(dot(wi, h)) / jacobian_denom;
        V3<T> base_col = mat.thin == 1 ? vsqrt(mat.albedo) : mat.albedo;
        // Quirk kept from dielectric.glsl:171: this declaration shadows the outer f, so the refraction
        // branch returns the outer, uninitialised-in-GLSL f. The shader's `vec3 f;` is zero in practice
        // (SPIR-V OpVariable without initialiser is undefined); we restate it as zero.
        V3<T> f_inner = base_col * D * G * (T(1) - F) * std::fabs(dot(wi, h) * dot(wo, h) / (wi.z * wo.z * jacobian_denom));
        if (mode == 1) f_inner = f_inner / (eta * eta);
        (void)f_inner;
        f = V3<T>(0);
        T prob_refraction = pt / (pr + pt);
        pdf_w = pdf_w * jacobian * prob_refraction;
        if (eval_reverse_pdf) {
            h *= T(-1);
            jacobian_denom = eta * dot(wi, h) + dot(wo, h);
            jacobian_denom *= jacobian_denom;
            T jacobian_reverse = std::fabs(dot(wo, h)) / jacobian_denom;
            pdf_rev_w = pdf_rev_w * jacobian_reverse * prob_refraction;
        }
    }
    return f;
}
template <class T> inline T eval_dielectric_pdf(const Mat<T>& mat, V3<T> wo, V3<T> wi, bool ff) {
    T roughness = mat.thin == 1 ? modify_thin_roughness(mat.ior, mat.roughness) : mat.roughness;
    T alpha = roughness * roughness;
    if (alpha == T(0) || mat.ior == T(1)) return T(0);
    bool has_reflection = bsdf_has_property(mat.bsdf_props, BSDF_FLAG_REFLECTION);
    bool has_transmission = bsdf_has_property(mat.bsdf_props, BSDF_FLAG_TRANSMISSION);
    if (!has_reflection && !has_transmission) return T(0);
    bool is_reflection = wi.z * wo.z > T(0);
    T eta = T(1);
    if (!is_reflection) eta = ff ? mat.ior : T(1) / mat.ior;
    V3<T> h = normalize(wo + wi * eta);
    h *= T(sign(h.z));
    if (wi.z == T(0) || wo.z == T(0) || dot(h, h) == T(0)) return T(0);
    if (dot(wi, h) * wi.z < T(0) || dot(wo, h) * wo.z < T(0)) return T(0);
    T F = fresnel_dielectric(dot(wo, h), mat.ior, ff);
    T pr = has_reflection ? F : T(0);
    T pt = has_transmission ? (T(1) - F) : T(0);
    T pdf_w = eval_vndf_pdf_isotropic(alpha, wo, h);
    if (is_reflection) {
        T jacobian = T(1) / (T(4) * std::fabs(dot(wo, h)));
        pdf_w = pdf_w * jacobian * (pr / (pr + pt));
    } else {
        T jacobian_denom = dot(wi, h) + dot(wo, h) / eta;
        jacobian_denom = jacobian_denom * jacobian_denom;
        T jacobian = std::fabs(dot(wi, h)) / jacobian_denom;
        pdf_w = pdf_w * jacobian * (pt / (pr + pt));
    }
    return pdf_w;
}

// ---------------- principled.glsl (ANISOTROPIC 1) ----------------
template <class T> inline V2<T> calc_anisotropy(T roughness, T anisotropic) {
    T aspect = std::sqrt(T(1) - T(0.9f) * anisotropic);
    T roughness_sqr = roughness * roughness;
    return V2<T>(gmax(T(0.001f), roughness_sqr / aspect), gmax(T(0.001f), roughness_sqr * aspect));
}
template <class T>
inline void initialize_sampling_probs(const Mat<T>& mat, T F_dielectric, bool ff, T& p_spec_reflect, T& p_diff, T& p_clearcoat,
                                      T& p_spec_trans) {
    T brdf_weight = (T(1) - mat.spec_trans) * (T(1) - mat.metallic);
    T bsdf_weight = (T(1) - mat.metallic) * mat.spec_trans;
    p_spec_reflect = ff ? (T(1) - bsdf_weight * (T(1) - F_dielectric)) : F_dielectric;
    p_spec_trans = ff ? (bsdf_weight * (T(1) - F_dielectric)) : (T(1) - F_dielectric);
    p_diff = ff ? brdf_weight : T(0);
    p_clearcoat = ff ? T(0.25f) * clamp(mat.clearcoat, T(0), T(1)) : T(0);
    T norm = T(1) / (p_spec_reflect + p_spec_trans + p_diff + p_clearcoat);
    p_spec_reflect *= norm; p_diff *= norm; p_clearcoat *= norm; p_spec_trans *= norm;
}
template <class T> inline V3<T> calc_disney_diffuse_factor(const Mat<T>& mat, V3<T> wo, V3<T> wi) {
    V3<T> h = normalize(wi + wo);
    T f_wi, f_wo;
    (void)disney_fresnel(wi, wo, mat.roughness, f_wi, f_wo);
    T roughness_sqr = mat.roughness * mat.roughness;
    T ss = T(0);
    T rr = T(2) * roughness_sqr * wi.z * wi.z;
    T f_retro = rr * (f_wi + f_wo * f_wi * f_wo * (rr - T(1)));
    T f_diff = (T(1) - T(0.5f) * f_wi) * (T(1) - T(0.5f) * f_wo);
    if (mat.flatness > T(0)) {
        T fss90 = T(0.5f) * rr;
        T h_dot_wi_sqr = dot(h, wi);
        h_dot_wi_sqr *= h_dot_wi_sqr;
        T f_ss = mix(T(1), fss90, f_wi) * mix(T(1), fss90, f_wo);
        ss = T(1.25f) * (f_ss * (T(1) / (wi.z + wo.z) - T(0.5f)) + T(0.5f));
    }
    T ss_approx_and_diff = mix(f_diff + f_retro, ss, mat.flatness);
    return mat.albedo * ss_approx_and_diff * K<T>::INV_PI();
}
template <class T> inline T calc_clearcoat_factor(const Mat<T>& mat, V3<T> wo, V3<T> wi, V3<T> h, T& D) {
    const T alpha_2 = T(0.25f * 0.25f);
    D = D_GGX_isotropic(mix(T(0.1f), T(0.001f), mat.clearcoat_gloss), h.z);
    T F = fresnel_schlick(T(0.04f), T(1), dot(wi, h));
    T G = G1_GGX_isotropic(alpha_2, wo.z) * G1_GGX_isotropic(alpha_2, wi.z);
    return T(0.25f) * mat.clearcoat * D * F * G;
}
template <class T> inline V3<T> sample_disney_diffuse(const Mat<T>& mat, V3<T> wo, V3<T>& wi, T& pdf_w, T& cos_theta, V2<T> xi) {
    wi = sample_hemisphere(xi);
    cos_theta = wi.z;
    pdf_w = cos_theta * K<T>::INV_PI();
    if (gmin(wi.z, wo.z) <= T(0)) return V3<T>(0);
    return calc_disney_diffuse_factor(mat, wo, wi);
}
template <class T>
inline V3<T> sample_principled_brdf(const Mat<T>& mat, V3<T> wo, V3<T>& wi, T& pdf_w, T& cos_theta, V2<T> xi, T eta) {
    bool has_reflection = bsdf_has_property(mat.bsdf_props, BSDF_FLAG_REFLECTION);
    if (!has_reflection) return V3<T>(0);
    T D;
    V2<T> alpha = calc_anisotropy(mat.roughness, mat.anisotropy);
    if (bsdf_is_effectively_delta(alpha)) {
        wi = V3<T>(-wo.x, -wo.y, wo.z);
        pdf_w = T(1);
        cos_theta = wi.z;
        V3<T> F = disney_fresnel(mat, wo, V3<T>(0, 0, 1), wi, eta);
        return F / std::fabs(cos_theta);
    }
    V3<T> h = sample_ggx_vndf_anisotropic(alpha, wo, xi, pdf_w, D);
    wi = reflect(-wo, h);
    if (wo.z * wi.z < T(0)) return V3<T>(0);
    V3<T> F = disney_fresnel(mat, wo, h, wi, eta);
    pdf_w /= (T(4) * dot(wo, h));
    cos_theta = wi.z;
    return T(0.25f) * D * F * G_GGX_correlated_anisotropic(alpha, wo, wi) / (wi.z * wo.z);
}
template <class T> inline V3<T> sample_clearcoat(const Mat<T>& mat, V3<T> wo, V3<T>& wi, T& pdf_w, T& cos_theta, V2<T> xi) {
    const T alpha_2 = T(0.25f * 0.25f);
    T cos_t = std::sqrt(gmax(T(0), (T(1) - std::pow(alpha_2, T(1) - xi.x)) / (T(1) - alpha_2)));
    // Quirk kept from principled.glsl:143: sin_t uses the incoming cos_theta, not cos_t.
    T sin_t = std::sqrt(gmax(T(0), T(1) - cos_theta * cos_theta));
    T phi = K<T>::TWO_PI() * xi.y;
    V3<T> h(sin_t * std::cos(phi), sin_t * std::sin(phi), cos_t);
    if (dot(h, wo) < T(0)) h *= T(-1);
    wi = reflect(-wo, h);
    if (dot(wi, wo) < T(0)) return V3<T>(0);
    T D;
    T f_clearcoat = calc_clearcoat_factor(mat, wo, wi, h, D);
    pdf_w = D / (T(4) * dot(wo, h));
    cos_theta = wi.z;
    return V3<T>(f_clearcoat);
}
template <class T> inline V3<T> eval_clearcoat(const Mat<T>& mat, V3<T> wo, V3<T> wi, T& pdf_w, T& pdf_rev_w) {
    V3<T> h = normalize(wo + wi);
    T D;
    T f_clearcoat = calc_clearcoat_factor(mat, wo, wi, h, D);
    pdf_w = D / (T(4) * dot(wo, h));
    pdf_rev_w = pdf_w;
    return V3<T>(f_clearcoat);
}
template <class T> inline T eval_clearcoat_pdf(const Mat<T>& mat, V3<T> wo, V3<T> wi) {
    V3<T> h = normalize(wo + wi);
    T D = D_GGX_isotropic(mix(T(0.1f), T(0.001f), mat.clearcoat_gloss), h.z);
    return D / (T(4) * dot(wo, h));
}
template <class T>
inline V3<T> eval_principled_brdf(const Mat<T>& mat, V3<T> wo, V3<T> wi, T& pdf_w, T& pdf_rev_w, bool ff, uint32_t, bool eval_reverse_pdf) {
    pdf_w = T(0); pdf_rev_w = T(0);
    V2<T> alpha = calc_anisotropy(mat.roughness, mat.anisotropy);
    if (bsdf_is_effectively_delta(alpha)) return V3<T>(0);
    if (wo.z * wi.z < T(0)) return V3<T>(0);
    if (wo.z == T(0) || wi.z == T(0)) return V3<T>(0);
    V3<T> h = normalize(wo + wi);
    T jacobian = T(1) / (T(4) * dot(wo, h));
    T D;
    pdf_w = eval_vndf_pdf_anisotropic(alpha, wo, h, D) * jacobian;
    T eta = ff ? mat.ior : T(1) / mat.ior;
    if (eval_reverse_pdf) pdf_rev_w = eval_vndf_pdf_anisotropic(alpha, wi, h) * jacobian;
    V3<T> F = disney_fresnel(mat, wo, h, wi, eta);
    return T(0.25f) * D * F * G_GGX_correlated_anisotropic(alpha, wo, wi) / (wi.z * wo.z);
}
template <class T> inline T eval_principled_brdf_pdf(const Mat<T>& mat, V3<T> wo, V3<T> wi) {
    V2<T> alpha = calc_anisotropy(mat.roughness, mat.anisotropy);
    if (bsdf_is_effectively_delta(alpha)) return T(0);
    if (wo.z * wi.z < T(0)) return T(0);
    if (wo.z == T(0) || wi.z == T(0)) return T(0);
    V3<T> h = normalize(wo + wi);
    h *= T(sign(h.z));
    return eval_vndf_pdf_anisotropic(alpha, wo, h) / (T(4) * dot(wo, h));
}
template <class T>
inline V3<T> sample_principled(const Mat<T>& mat, V3<T> wo, V3<T>& wi, uint32_t mode, bool ff, T& pdf_w, T& cos_theta, V3<T> xi) {
    wi = V3<T>(0); pdf_w = T(0); cos_theta = T(0);
    if (wo.z <= T(0)) return V3<T>(0);
    T p_spec, p_diff, p_clearcoat, p_spec_trans;
    T F = fresnel_dielectric(wo.z, mat.ior, ff);
    initialize_sampling_probs(mat, F, ff, p_spec, p_diff, p_clearcoat, p_spec_trans);
    T eta = ff ? mat.ior : T(1) / mat.ior;
    V3<T> f(0);
    T p_lobe = T(0);
    V2<T> xy(xi.x, xi.y);
    if (xi.z < p_spec) {
        f = sample_principled_brdf(mat, wo, wi, pdf_w, cos_theta, xy, eta);
        p_lobe = p_spec;
    } else if (xi.z > p_spec && xi.z <= (p_spec + p_clearcoat)) {
        f = sample_clearcoat(mat, wo, wi, pdf_w, cos_theta, xy);
        p_lobe = p_clearcoat;
    } else if (xi.z > (p_spec + p_clearcoat) && xi.z <= (p_spec + p_clearcoat + p_diff)) {
        f = sample_disney_diffuse(mat, wo, wi, pdf_w, cos_theta, xy);
        p_lobe = p_diff;
    } else if (p_spec_trans >= T(0) && xi.z <= (p_spec + p_clearcoat + p_diff + p_spec_trans)) {
        f = sample_dielectric(mat, wo, wi, mode, ff, pdf_w, cos_theta, xy);
        p_lobe = p_spec_trans;
    }
    pdf_w *= p_lobe;
    return f;
}
template <class T>
inline V3<T> eval_principled(const Mat<T>& mat, V3<T> wo, V3<T> wi, T& pdf_w, T& pdf_rev_w, bool ff, uint32_t mode, bool eval_reverse_pdf) {
    pdf_w = T(0); pdf_rev_w = T(0);
    T p_spec, p_diff, p_clearcoat, p_spec_trans;
    T F = fresnel_dielectric(wo.z, mat.ior, ff);
    initialize_sampling_probs(mat, F, ff, p_spec, p_diff, p_clearcoat, p_spec_trans);
    V3<T> f(0);
    T pdf = T(0), pdf_rev = T(0);
    T brdf_weight = (T(1) - mat.spec_trans) * (T(1) - mat.metallic);
    T bsdf_weight = (T(1) - mat.metallic) * mat.spec_trans;
    if (p_spec > T(0)) {
        f += eval_principled_brdf(mat, wo, wi, pdf, pdf_rev, ff, mode, eval_reverse_pdf);
        pdf *= p_spec; pdf_rev *= p_spec;
        pdf_w += pdf; pdf_rev_w += pdf_rev;
    }
    bool upper_hemisphere = gmin(wi.z, wo.z) > T(0);
    if (upper_hemisphere) {
        if (p_diff > T(0)) {
            pdf_w += p_diff * eval_diffuse_pdf(wo, wi);
            pdf_rev_w += pdf_w;
            f += brdf_weight * calc_disney_diffuse_factor(mat, wo, wi);
        }
        if (p_clearcoat > T(0)) {
            f += eval_clearcoat(mat, wo, wi, pdf, pdf_rev);
            pdf *= p_clearcoat; pdf_rev *= p_clearcoat;
            pdf_w += pdf; pdf_rev_w += pdf_rev;
        }
    }
    if (p_spec_trans > T(0)) {
        f += bsdf_weight * eval_dielectric(mat, wo, wi, pdf, pdf_rev, ff, mode, eval_reverse_pdf);
        pdf *= p_spec_trans; pdf_rev *= p_spec_trans;
        pdf_w += pdf; pdf_rev_w += pdf_rev;
    }
    return f;
}

// ---------------- bsdf_commons.glsl ----------------
template <class T>
inline V3<T> sample_bsdf(V3<T> n_s, V3<T> wo, const Mat<T>& mat, uint32_t mode, bool ff, V3<T>& wi, T& pdf_w, T& cos_theta, V3<T> rands) {
    V3<T> f(0);
    pdf_w = T(0); cos_theta = T(0); wi = V3<T>(0);
    V3<T> Tt, B;
    branchless_onb(n_s, Tt, B);
    wo = to_local(wo, Tt, B, n_s);
    V2<T> xy(rands.x, rands.y);
    switch (mat.bsdf_type) {
        case BSDF_TYPE_DIFFUSE: f = sample_diffuse(mat, wo, wi, pdf_w, cos_theta, xy); break;
        case BSDF_TYPE_MIRROR: f = sample_mirror(V3<T>(0, 0, 1), wo, wi, pdf_w, cos_theta); break;
        case BSDF_TYPE_GLASS: f = sample_glass(mat, V3<T>(0, 0, 1), wo, wi, pdf_w, cos_theta, mode, ff); break;
        case BSDF_TYPE_DIELECTRIC: f = sample_dielectric(mat, wo, wi, mode, ff, pdf_w, cos_theta, xy); break;
        case BSDF_TYPE_CONDUCTOR: f = sample_conductor(mat, wo, wi, pdf_w, cos_theta, xy); break;
        case BSDF_TYPE_PRINCIPLED: f = sample_principled(mat, wo, wi, mode, ff, pdf_w, cos_theta, rands); break;
        default: break;
    }
    wi = to_world(wi, Tt, B, n_s);
    return f;
}
template <class T>
inline V3<T> eval_bsdf(V3<T> n_s, V3<T> wo, const Mat<T>& mat, uint32_t mode, bool ff, V3<T> wi, T& pdf_w, T& pdf_rev_w, bool eval_reverse) {
    pdf_w = T(0); pdf_rev_w = T(0);
    V3<T> f(0);
    V3<T> Tt, B;
    branchless_onb(n_s, Tt, B);
    wo = to_local(wo, Tt, B, n_s);
    wi = to_local(wi, Tt, B, n_s);
    switch (mat.bsdf_type) {
        case BSDF_TYPE_DIFFUSE: f = eval_diffuse(mat, wo, wi, pdf_w, pdf_rev_w); break;
        case BSDF_TYPE_MIRROR: pdf_w = T(0); pdf_rev_w = T(0); f = V3<T>(0); break;
        case BSDF_TYPE_GLASS: pdf_w = T(0); pdf_rev_w = T(0); f = V3<T>(0); break;
        case BSDF_TYPE_DIELECTRIC: f = eval_dielectric(mat, wo, wi, pdf_w, pdf_rev_w, ff, mode, eval_reverse); break;
        case BSDF_TYPE_CONDUCTOR: f = eval_conductor(mat, wo, wi, pdf_w, pdf_rev_w, eval_reverse); break;
        case BSDF_TYPE_PRINCIPLED: f = eval_principled(mat, wo, wi, pdf_w, pdf_rev_w, ff, mode, eval_reverse); break;
        default: break;
    }
    return f;
}

// bsdf_pdf (bsdf_commons.glsl:26-66) with the per-lobe pdf functions it calls: conductor.glsl:74-90,
// principled.glsl:338-359 (the others are above).
template <class T> inline T eval_conductor_pdf(const Mat<T>& mat, V3<T> wo, V3<T> wi) {
    T alpha = mat.roughness * mat.roughness;
    if (bsdf_is_effectively_delta(alpha)) return T(0);
    if (wo.z * wi.z < T(0)) return T(0);
    if (wo.z == T(0) || wi.z == T(0)) return T(0);
    V3<T> h = normalize(wo + wi);
    h *= T(sign(h.z));
    return eval_vndf_pdf_isotropic(alpha, wo, h) / (T(4) * dot(wo, h));
}
template <class T> inline T eval_principled_pdf(const Mat<T>& mat, V3<T> wo, V3<T> wi, bool ff) {
    T pdf = T(0);
    T p_spec, p_diff, p_clearcoat, p_spec_trans;
    T F = fresnel_dielectric(wo.z, mat.ior, ff);
    initialize_sampling_probs(mat, F, ff, p_spec, p_diff, p_clearcoat, p_spec_trans);
    if (p_spec > T(0)) pdf += p_spec * eval_principled_brdf_pdf(mat, wo, wi);
    if (gmin(wi.z, wo.z) > T(0)) {
        if (p_diff > T(0)) pdf += p_diff * eval_diffuse_pdf(wo, wi);
        if (p_clearcoat > T(0)) pdf += p_clearcoat * eval_clearcoat_pdf(mat, wo, wi);
    }
    if (p_spec_trans > T(0)) pdf += p_spec_trans * eval_dielectric_pdf(mat, wo, wi, ff);
    return pdf;
}
template <class T> inline T bsdf_pdf(const Mat<T>& mat, V3<T> n_s, V3<T> wo, V3<T> wi, bool ff) {
    V3<T> Tt, B;
    branchless_onb(n_s, Tt, B);
    wo = to_local(wo, Tt, B, n_s);
    wi = to_local(wi, Tt, B, n_s);
    switch (mat.bsdf_type) {
        case BSDF_TYPE_DIFFUSE: return eval_diffuse_pdf(wo, wi);
        case BSDF_TYPE_MIRROR: return T(0);
        case BSDF_TYPE_GLASS: return T(0);
        case BSDF_TYPE_DIELECTRIC: return eval_dielectric_pdf(mat, wo, wi, ff);
        case BSDF_TYPE_CONDUCTOR: return eval_conductor_pdf(mat, wo, wi);
        case BSDF_TYPE_PRINCIPLED: return eval_principled_pdf(mat, wo, wi, ff);
        default: return T(0);
    }
}

}  // namespace orc
