// Device BSDFs: diffuse (Lambertian), mirror, glass, dielectric, conductor and Disney principled, with the
// sample/eval dispatch of src/shaders/bsdf_commons.glsl:68-177. FP32, shader evaluation order.
#pragma once
#include "shading.cuh"

namespace lgb {
namespace sh {

struct Mat {
    v3 albedo;
    float ior;
    v3 emissive;
    uint32_t type, props;
    v3 k;
    float roughness, spec_trans, metallic, specular_tint, clearcoat, clearcoat_gloss, flatness, anisotropy;
    uint32_t thin;
};

__device__ __forceinline__ Mat load_mat(const lgb_material* __restrict__ m) {
    Mat r;
    r.albedo = V3(m->albedo[0], m->albedo[1], m->albedo[2]);
    r.ior = m->ior;
    r.emissive = V3(m->emissive_factor[0], m->emissive_factor[1], m->emissive_factor[2]);
    r.type = m->bsdf_type;
    r.props = m->bsdf_props;
    r.k = V3(m->k[0], m->k[1], m->k[2]);
    r.roughness = m->roughness;
    r.spec_trans = m->spec_trans;
    r.metallic = m->metallic;
    r.specular_tint = m->specular_tint;
    r.clearcoat = m->clearcoat;
    r.clearcoat_gloss = m->clearcoat_gloss;
    r.flatness = m->flatness;
    r.anisotropy = m->anisotropy;
    r.thin = m->thin;
    return r;
}

// ---- diffuse.glsl (Lambertian) ----
__device__ __forceinline__ v3 sample_diffuse(const Mat& m, v3 wo, v3& wi, float& pdf, float& cos_t, v2 xi) {
    wi = sample_hemisphere(xi);
    cos_t = wi.z;
    pdf = cos_t * LGB_INV_PI;
    if (fminf(wi.z, wo.z) <= 0.0f) return V3(0.0f);
    return m.albedo * LGB_INV_PI;
}
__device__ __forceinline__ v3 eval_diffuse(const Mat& m, v3 wo, v3 wi, float& pdf) {
    pdf = 0.0f;
    if (fminf(wi.z, wo.z) <= 0.0f) return V3(0.0f);
    pdf = wi.z * LGB_INV_PI;
    return m.albedo * LGB_INV_PI;
}
__device__ __forceinline__ float diffuse_pdf(v3 wo, v3 wi) {
    if (fminf(wi.z, wo.z) <= 0.0f) return 0.0f;
    return wi.z * LGB_INV_PI;
}

// ---- mirror.glsl / glass.glsl (local frame, n = +z) ----
__device__ __forceinline__ v3 sample_mirror(v3 wo, v3& wi, float& pdf, float& cos_t) {
    const v3 n = V3(0.0f, 0.0f, 1.0f);
    if (dot(wo, n) <= 0.0f) { pdf = 0.0f; cos_t = 0.0f; wi = V3(0.0f); return V3(0.0f); }
    wi = reflect(-wo, n);
    cos_t = dot(wi, n);
    pdf = 1.0f;
    return V3(1.0f / cos_t);
}
__device__ __forceinline__ v3 sample_glass(const Mat& m, v3 wo, v3& wi, float& pdf, float& cos_t, uint32_t mode, bool ff) {
    const v3 n = V3(0.0f, 0.0f, 1.0f);
    v3 f;
    float unused;
    refract(n, wo, ff, m.ior, mode, wi, f, unused);
    cos_t = dot(n, wi);
    pdf = 1.0f;
    return f / fabsf(cos_t);
}

// ---- conductor.glsl ----
__device__ __forceinline__ v3 sample_conductor(const Mat& m, v3 wo, v3& wi, float& pdf, float& cos_t, v2 xi) {
    wi = V3(0.0f); pdf = 0.0f; cos_t = 0.0f;
    if (wo.z <= 0.0f) return V3(0.0f);
    const float alpha = m.roughness * m.roughness;
    if (!has_prop(m.props, LGB_FLAG_REFLECTION)) return V3(0.0f);
    if (effectively_delta(alpha)) {
        wi = V3(-wo.x, -wo.y, wo.z);
        pdf = 1.0f;
        cos_t = wi.z;
        return fresnel_conductor(cos_t, m.albedo, m.k) / fabsf(cos_t);
    }
    float D;
    const v3 h = sample_vndf(V2(alpha, alpha), wo, xi);
    pdf = vndf_pdf_iso(alpha, wo, h, D);
    const v3 F = fresnel_conductor(dot(wo, h), m.albedo, m.k);
    wi = reflect(-wo, h);
    if (wo.z * wi.z < 0.0f) return V3(0.0f);
    pdf /= (4.0f * dot(wo, h));
    cos_t = wi.z;
    return (0.25f * D) * F * G_corr_iso(alpha, wo, wi) / (wi.z * wo.z);
}
__device__ __forceinline__ v3 eval_conductor(const Mat& m, v3 wo, v3 wi, float& pdf) {
    pdf = 0.0f;
    const float alpha = m.roughness * m.roughness;
    if (effectively_delta(alpha)) return V3(0.0f);
    if (wo.z * wi.z < 0.0f) return V3(0.0f);
    if (wo.z == 0.0f || wi.z == 0.0f) return V3(0.0f);
    v3 h = normalize(wo + wi);
    h = h * signf(h.z);
    const float jac = 1.0f / (4.0f * dot(wo, h));
    float D;
    pdf = vndf_pdf_iso(alpha, wo, h, D) * jac;
    const v3 F = fresnel_conductor(dot(wo, h), m.albedo, m.k);
    return (0.25f * D) * F * G_corr_iso(alpha, wo, wi) / (wi.z * wo.z);
}

// ---- dielectric.glsl ----
__device__ __forceinline__ float thin_roughness(float ior, float r) { return clampf((0.65f * ior - 0.35f) * r, 0.0f, 1.0f); }

__device__ __forceinline__ v3 sample_dielectric(const Mat& m, v3 wo, v3& wi, uint32_t mode, bool ff, float& pdf, float& cos_t, v2 xi) {
    wi = V3(0.0f); pdf = 0.0f; cos_t = 0.0f;
    if (wo.z <= 0.0f) return V3(0.0f);
    const float rough = m.thin == 1u ? thin_roughness(m.ior, m.roughness) : m.roughness;
    const float alpha = rough * rough;
    const bool has_r = has_prop(m.props, LGB_FLAG_REFLECTION), has_t = has_prop(m.props, LGB_FLAG_TRANSMISSION);
    if ((m.ior == 1.0f && m.thin == 0u) || effectively_delta(alpha)) {
        const float F = fresnel_dielectric(wo.z, m.ior, ff);
        if (!has_r && !has_t) return V3(0.0f);
        float pr = F, pt = 1.0f - F;
        if (!has_r) pr = 0.0f;
        if (!has_t) pt = 0.0f;
        v3 f;
        if (((pr + pt) * xi.x) < pr) {
            wi = V3(-wo.x, -wo.y, wo.z);
            cos_t = wi.z;
            f = V3(F / fabsf(cos_t));
            pdf = pr / (pr + pt);
        } else {
            float unused;
            refract(V3(0.0f, 0.0f, 1.0f), wo, ff, m.ior, mode, wi, f, unused);
            cos_t = wi.z;
            f = f * (1.0f - F) / fabsf(cos_t);
            pdf = pt / (pr + pt);
        }
        return f;
    }
    if (!has_r && !has_t) return V3(0.0f);
    float D;
    const v3 h = sample_vndf(V2(alpha, alpha), wo, xi);
    pdf = vndf_pdf_iso(alpha, wo, h, D);
    const float F = fresnel_dielectric(dot(wo, h), m.ior, ff);
    const float pr = has_r ? F : 0.0f;
    const float pt = has_t ? (1.0f - F) : 0.0f;
    v3 f = V3(0.0f);  // the thin branch below reads f before any write (dielectric.glsl:85,103)
    if (((pr + pt) * xi.x) < pr) {
        wi = reflect(-wo, h);
        if (wo.z * wi.z < 0.0f) return V3(0.0f);
        pdf = pdf * (pr / (pr + pt)) / (4.0f * fabsf(dot(wo, h)));
        f = V3(0.25f * D * F * G_corr_iso(alpha, wo, wi) / (wi.z * wo.z));
    } else {
        v3 base;
        float inv_eta;
        if (m.thin == 1u) {
            wi = reflect(-wo, h);
            base = sqrt3(m.albedo);
            inv_eta = m.ior;
        } else {
            refract(h, wo, ff, m.ior, mode, wi, f, inv_eta);
            base = m.albedo;
        }
        // refract() never reports total internal reflection (sampling_commons.glsl:29-34 reflects instead)
        if (wo.z * wi.z > 0.0f || wi.z > 0.0f) return V3(0.0f);
        float jd = dot(wi, h) + dot(wo, h) * inv_eta;
        jd = jd * jd;
        const float jac = fabsf(dot(wi, h)) / jd;
        pdf = pdf * (pt / (pr + pt)) * jac;
        f = base * f * (1.0f - F) * D * G_corr_iso(alpha, wo, wi) * fabsf(dot(wi, h) * dot(wo, h) / (wi.z * wo.z * jd));
    }
    cos_t = wi.z;
    return f;
}

// eval_dielectric (dielectric.glsl:110-189). The refraction branch assigns a shadowed local (line 171), so
// the value returned for transmission is the outer, never-written f, restated as zero.
__device__ __forceinline__ v3 eval_dielectric(const Mat& m, v3 wo, v3 wi, float& pdf, bool ff) {
    pdf = 0.0f;
    const float rough = m.thin == 1u ? thin_roughness(m.ior, m.roughness) : m.roughness;
    const float alpha = rough * rough;
    if (alpha == 0.0f || m.ior == 1.0f) return V3(0.0f);
    const bool has_r = has_prop(m.props, LGB_FLAG_REFLECTION), has_t = has_prop(m.props, LGB_FLAG_TRANSMISSION);
    if (!has_r && !has_t) return V3(0.0f);
    float eta = 1.0f;
    const bool is_refl = wi.z * wo.z > 0.0f;
    if (!is_refl) eta = ff ? m.ior : 1.0f / m.ior;
    v3 h = normalize(wo + wi * eta);
    h = h * signf(h.z);
    if (wi.z == 0.0f || wo.z == 0.0f || dot(h, h) == 0.0f) return V3(0.0f);
    if (dot(wi, h) * wi.z < 0.0f || dot(wo, h) * wo.z < 0.0f) return V3(0.0f);
    const float F = fresnel_dielectric(dot(wo, h), m.ior, ff);
    const float pr = has_r ? F : 0.0f;
    const float pt = has_t ? (1.0f - F) : 0.0f;
    float D;
    pdf = vndf_pdf_iso(alpha, wo, h, D);
    const float G = G_corr_iso(alpha, wo, wi);
    if (is_refl) {
        const float jac = 1.0f / (4.0f * fabsf(dot(wo, h)));
        pdf = pdf * jac * (pr / (pr + pt));
        return V3(0.25f * D * G * F / fabsf(wo.z * wi.z));
    }
    float jd = dot(wi, h) + dot(wo, h) / eta;
    jd = jd * jd;
    const float jac = fabsf(dot(wi, h)) / jd;
    pdf = pdf * jac * (pt / (pr + pt));
    return V3(0.0f);
}
__device__ __forceinline__ float dielectric_pdf(const Mat& m, v3 wo, v3 wi, bool ff) {
    float pdf;
    (void)eval_dielectric(m, wo, wi, pdf, ff);
    return pdf;
}

// ---- principled.glsl (ANISOTROPIC 1) ----
__device__ __forceinline__ v2 calc_anisotropy(float r, float an) {
    const float aspect = sqrtf(1.0f - 0.9f * an);
    const float r2 = r * r;
    return V2(fmaxf(0.001f, r2 / aspect), fmaxf(0.001f, r2 * aspect));
}
__device__ __forceinline__ void sampling_probs(const Mat& m, float Fd, bool ff, float& ps, float& pd, float& pc, float& pt) {
    const float brdf_w = (1.0f - m.spec_trans) * (1.0f - m.metallic);
    const float bsdf_w = (1.0f - m.metallic) * m.spec_trans;
    ps = ff ? (1.0f - bsdf_w * (1.0f - Fd)) : Fd;
    pt = ff ? (bsdf_w * (1.0f - Fd)) : (1.0f - Fd);
    pd = ff ? brdf_w : 0.0f;
    pc = ff ? 0.25f * clampf(m.clearcoat, 0.0f, 1.0f) : 0.0f;
    const float norm = 1.0f / (ps + pt + pd + pc);
    ps *= norm; pd *= norm; pc *= norm; pt *= norm;
}
__device__ __forceinline__ v3 disney_fresnel_m(const Mat& m, v3 wo, v3 h, float eta) {
    const float wo_h = dot(wo, h);
    v3 R0 = eta_to_schlick_R0(eta) * mix3(V3(1.0f), calc_tint(m.albedo), m.specular_tint);
    R0 = mix3(R0, m.albedo, m.metallic);
    const float frd = fresnel_dielectric(wo_h, eta, true);
    const v3 frm = fresnel_schlick3(R0, V3(1.0f), wo_h);
    return mix3(V3(frd), frm, m.metallic);
}
__device__ __forceinline__ v3 disney_diffuse_factor(const Mat& m, v3 wo, v3 wi) {
    const v3 h = normalize(wi + wo);
    const v3 hh = normalize(wi + wo);
    const float wo_h = dot(wo, hh);
    const float fd90 = 0.5f + 2.0f * wo_h * wo_h * m.roughness;
    const float f_wi = fresnel_schlick(1.0f, fd90, wi.z);
    const float f_wo = fresnel_schlick(1.0f, fd90, wo.z);
    const float r2 = m.roughness * m.roughness;
    float ss = 0.0f;
    const float rr = 2.0f * r2 * wi.z * wi.z;
    const float f_retro = rr * (f_wi + f_wo * f_wi * f_wo * (rr - 1.0f));
    const float f_diff = (1.0f - 0.5f * f_wi) * (1.0f - 0.5f * f_wo);
    if (m.flatness > 0.0f) {
        const float fss90 = 0.5f * rr;
        float hwi = dot(h, wi);
        hwi *= hwi;
        const float f_ss = mixf(1.0f, fss90, f_wi) * mixf(1.0f, fss90, f_wo);
        ss = 1.25f * (f_ss * (1.0f / (wi.z + wo.z) - 0.5f) + 0.5f);
    }
    const float sd = mixf(f_diff + f_retro, ss, m.flatness);
    return m.albedo * sd * LGB_INV_PI;
}
__device__ __forceinline__ float clearcoat_factor(const Mat& m, v3 wo, v3 wi, v3 h, float& D) {
    const float a2 = 0.25f * 0.25f;
    D = D_iso(mixf(0.1f, 0.001f, m.clearcoat_gloss), h.z);
    const float F = fresnel_schlick(0.04f, 1.0f, dot(wi, h));
    const float G = G1_iso(a2, wo.z) * G1_iso(a2, wi.z);
    return 0.25f * m.clearcoat * D * F * G;
}
__device__ __forceinline__ v3 sample_principled_brdf(const Mat& m, v3 wo, v3& wi, float& pdf, float& cos_t, v2 xi, float eta) {
    if (!has_prop(m.props, LGB_FLAG_REFLECTION)) return V3(0.0f);
    const v2 alpha = calc_anisotropy(m.roughness, m.anisotropy);
    if (fminf(alpha.x, alpha.y) <= 0.0064f) {
        wi = V3(-wo.x, -wo.y, wo.z);
        pdf = 1.0f;
        cos_t = wi.z;
        return disney_fresnel_m(m, wo, V3(0.0f, 0.0f, 1.0f), eta) / fabsf(cos_t);
    }
    float D;
    const v3 h = sample_vndf(alpha, wo, xi);
    pdf = vndf_pdf_aniso(alpha, wo, h, D);
    wi = reflect(-wo, h);
    if (wo.z * wi.z < 0.0f) return V3(0.0f);
    const v3 F = disney_fresnel_m(m, wo, h, eta);
    pdf /= (4.0f * dot(wo, h));
    cos_t = wi.z;
    return (0.25f * D) * F * G_corr_aniso(alpha, wo, wi) / (wi.z * wo.z);
}
__device__ __forceinline__ v3 sample_clearcoat(const Mat& m, v3 wo, v3& wi, float& pdf, float& cos_t, v2 xi) {
    const float a2 = 0.25f * 0.25f;
    const float ct = sqrtf(fmaxf(0.0f, (1.0f - powf(a2, 1.0f - xi.x)) / (1.0f - a2)));
    // principled.glsl:143 takes sin_t from the incoming cos_theta (0 here), not from cos_t.
    const float st = sqrtf(fmaxf(0.0f, 1.0f - cos_t * cos_t));
    const float phi = LGB_TWO_PI * xi.y;
    v3 h = V3(st * cosf(phi), st * sinf(phi), ct);
    if (dot(h, wo) < 0.0f) h = h * -1.0f;
    wi = reflect(-wo, h);
    if (dot(wi, wo) < 0.0f) return V3(0.0f);
    float D;
    const float fc = clearcoat_factor(m, wo, wi, h, D);
    pdf = D / (4.0f * dot(wo, h));
    cos_t = wi.z;
    return V3(fc);
}
__device__ __forceinline__ v3 eval_principled_brdf(const Mat& m, v3 wo, v3 wi, float& pdf, bool ff) {
    pdf = 0.0f;
    const v2 alpha = calc_anisotropy(m.roughness, m.anisotropy);
    if (fminf(alpha.x, alpha.y) <= 0.0064f) return V3(0.0f);
    if (wo.z * wi.z < 0.0f) return V3(0.0f);
    if (wo.z == 0.0f || wi.z == 0.0f) return V3(0.0f);
    const v3 h = normalize(wo + wi);
    const float jac = 1.0f / (4.0f * dot(wo, h));
    float D;
    pdf = vndf_pdf_aniso(alpha, wo, h, D) * jac;
    const float eta = ff ? m.ior : 1.0f / m.ior;
    const v3 F = disney_fresnel_m(m, wo, h, eta);
    return (0.25f * D) * F * G_corr_aniso(alpha, wo, wi) / (wi.z * wo.z);
}
__device__ __forceinline__ v3 sample_principled(const Mat& m, v3 wo, v3& wi, uint32_t mode, bool ff, float& pdf, float& cos_t, v3 xi) {
    wi = V3(0.0f); pdf = 0.0f; cos_t = 0.0f;
    if (wo.z <= 0.0f) return V3(0.0f);
    float ps, pd, pc, pt;
    const float F = fresnel_dielectric(wo.z, m.ior, ff);
    sampling_probs(m, F, ff, ps, pd, pc, pt);
    const float eta = ff ? m.ior : 1.0f / m.ior;
    v3 f = V3(0.0f);
    float pl = 0.0f;
    const v2 xy = V2(xi.x, xi.y);
    if (xi.z < ps) {
        f = sample_principled_brdf(m, wo, wi, pdf, cos_t, xy, eta);
        pl = ps;
    } else if (xi.z > ps && xi.z <= (ps + pc)) {
        f = sample_clearcoat(m, wo, wi, pdf, cos_t, xy);
        pl = pc;
    } else if (xi.z > (ps + pc) && xi.z <= (ps + pc + pd)) {
        wi = sample_hemisphere(xy);
        cos_t = wi.z;
        pdf = cos_t * LGB_INV_PI;
        f = fminf(wi.z, wo.z) <= 0.0f ? V3(0.0f) : disney_diffuse_factor(m, wo, wi);
        pl = pd;
    } else if (pt >= 0.0f && xi.z <= (ps + pc + pd + pt)) {
        f = sample_dielectric(m, wo, wi, mode, ff, pdf, cos_t, xy);
        pl = pt;
    }
    pdf *= pl;
    return f;
}
__device__ __forceinline__ v3 eval_principled(const Mat& m, v3 wo, v3 wi, float& pdf_w, bool ff) {
    pdf_w = 0.0f;
    float ps, pd, pc, pt;
    const float F = fresnel_dielectric(wo.z, m.ior, ff);
    sampling_probs(m, F, ff, ps, pd, pc, pt);
    v3 f = V3(0.0f);
    float pdf = 0.0f;
    const float brdf_w = (1.0f - m.spec_trans) * (1.0f - m.metallic);
    const float bsdf_w = (1.0f - m.metallic) * m.spec_trans;
    if (ps > 0.0f) {
        f = f + eval_principled_brdf(m, wo, wi, pdf, ff);
        pdf *= ps;
        pdf_w += pdf;
    }
    if (fminf(wi.z, wo.z) > 0.0f) {
        if (pd > 0.0f) {
            pdf_w += pd * diffuse_pdf(wo, wi);
            f = f + brdf_w * disney_diffuse_factor(m, wo, wi);
        }
        if (pc > 0.0f) {
            const v3 h = normalize(wo + wi);
            float D;
            const float fc = clearcoat_factor(m, wo, wi, h, D);
            pdf = D / (4.0f * dot(wo, h));
            f = f + V3(fc);
            pdf *= pc;
            pdf_w += pdf;
        }
    }
    if (pt > 0.0f) {
        f = f + bsdf_w * eval_dielectric(m, wo, wi, pdf, ff);
        pdf *= pt;
        pdf_w += pdf;
    }
    return f;
}

// ---- bsdf_commons.glsl dispatch (radiance transport, mode 1) ----
// MASK (LGB_BSDF_* bits) limits the lobes compiled into a caller; a type outside it evaluates to zero, so a
// kernel instantiated for a scene's own type set gives the same results with fewer registers.
constexpr uint32_t kAllBsdfs = 0x3Fu;

template <uint32_t MASK = kAllBsdfs>
__device__ __forceinline__ v3 sample_bsdf(v3 n_s, v3 wo, const Mat& m, bool ff, v3& wi, float& pdf, float& cos_t, v3 r) {
    v3 f = V3(0.0f);
    pdf = 0.0f; cos_t = 0.0f; wi = V3(0.0f);
    v3 T, B;
    branchless_onb(n_s, T, B);
    wo = to_local(wo, T, B, n_s);
    const v2 xy = V2(r.x, r.y);
    switch (m.type & MASK) {
        case LGB_BSDF_DIFFUSE:
            if constexpr ((MASK & LGB_BSDF_DIFFUSE) != 0) f = sample_diffuse(m, wo, wi, pdf, cos_t, xy);
            break;
        case LGB_BSDF_MIRROR:
            if constexpr ((MASK & LGB_BSDF_MIRROR) != 0) f = sample_mirror(wo, wi, pdf, cos_t);
            break;
        case LGB_BSDF_GLASS:
            if constexpr ((MASK & LGB_BSDF_GLASS) != 0) f = sample_glass(m, wo, wi, pdf, cos_t, 1u, ff);
            break;
        case LGB_BSDF_DIELECTRIC:
            if constexpr ((MASK & LGB_BSDF_DIELECTRIC) != 0) f = sample_dielectric(m, wo, wi, 1u, ff, pdf, cos_t, xy);
            break;
        case LGB_BSDF_CONDUCTOR:
            if constexpr ((MASK & LGB_BSDF_CONDUCTOR) != 0) f = sample_conductor(m, wo, wi, pdf, cos_t, xy);
            break;
        case LGB_BSDF_PRINCIPLED:
            if constexpr ((MASK & LGB_BSDF_PRINCIPLED) != 0) f = sample_principled(m, wo, wi, 1u, ff, pdf, cos_t, r);
            break;
        default: break;
    }
    wi = to_world(wi, T, B, n_s);
    return f;
}
template <uint32_t MASK = kAllBsdfs>
__device__ __forceinline__ v3 eval_bsdf(v3 n_s, v3 wo, const Mat& m, bool ff, v3 wi, float& pdf) {
    pdf = 0.0f;
    v3 T, B;
    branchless_onb(n_s, T, B);
    wo = to_local(wo, T, B, n_s);
    wi = to_local(wi, T, B, n_s);
    switch (m.type & MASK) {
        case LGB_BSDF_DIFFUSE:
            if constexpr ((MASK & LGB_BSDF_DIFFUSE) != 0) return eval_diffuse(m, wo, wi, pdf);
            break;
        case LGB_BSDF_DIELECTRIC:
            if constexpr ((MASK & LGB_BSDF_DIELECTRIC) != 0) return eval_dielectric(m, wo, wi, pdf, ff);
            break;
        case LGB_BSDF_CONDUCTOR:
            if constexpr ((MASK & LGB_BSDF_CONDUCTOR) != 0) return eval_conductor(m, wo, wi, pdf);
            break;
        case LGB_BSDF_PRINCIPLED:
            if constexpr ((MASK & LGB_BSDF_PRINCIPLED) != 0) return eval_principled(m, wo, wi, pdf, ff);
            break;
        default: break;
    }
    return V3(0.0f);
}

}  // namespace sh
}  // namespace lgb
