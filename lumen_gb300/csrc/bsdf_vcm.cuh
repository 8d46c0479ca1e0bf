// BSDF evaluation with reverse pdfs and transport mode, the stand-alone pdf and a mode-aware sampler: what
// bidirectional estimators (VCM) need beyond the path tracer's radiance-only dispatch in bsdf.cuh.
// Restates src/shaders/bsdf_commons.glsl:26-66 (bsdf_pdf), 68-121 (sample_bsdf with mode), 123-177
// (eval_bsdf with pdf_rev) and the lobes' reverse pdfs: diffuse.glsl (pdf_rev = pdf), conductor.glsl:58-72,
// dielectric.glsl:110-189, principled.glsl:300-336 (including its quirk that the diffuse lobe adds the
// accumulated forward pdf to the reverse one).
#pragma once
#include "bsdf.cuh"

namespace lgb {
namespace sh {

__device__ __forceinline__ v3 eval_conductor_rev(const Mat& m, v3 wo, v3 wi, float& pdf, float& pdf_rev, bool rev) {
    pdf = 0.0f; pdf_rev = 0.0f;
    const float alpha = m.roughness * m.roughness;
    if (effectively_delta(alpha)) return V3(0.0f);
    if (wo.z * wi.z < 0.0f) return V3(0.0f);
    if (wo.z == 0.0f || wi.z == 0.0f) return V3(0.0f);
    v3 h = normalize(wo + wi);
    h = h * signf(h.z);
    const float jac = 1.0f / (4.0f * dot(wo, h));
    float D;
    pdf = vndf_pdf_iso(alpha, wo, h, D) * jac;
    if (rev) { float Dr; pdf_rev = vndf_pdf_iso(alpha, wi, h, Dr) * jac; }
    const v3 F = fresnel_conductor(dot(wo, h), m.albedo, m.k);
    return (0.25f * D) * F * G_corr_iso(alpha, wo, wi) / (wi.z * wo.z);
}

// The transmission value is the shadowed inner one of dielectric.glsl:171, restated as zero (see bsdf.cuh).
__device__ __forceinline__ v3 eval_dielectric_rev(const Mat& m, v3 wo, v3 wi, float& pdf, float& pdf_rev, bool ff, bool rev) {
    pdf = 0.0f; pdf_rev = 0.0f;
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
    if (rev) pdf_rev = vndf_pdf_iso(alpha, wi, -h, D);
    pdf = vndf_pdf_iso(alpha, wo, h, D);
    const float G = G_corr_iso(alpha, wo, wi);
    if (is_refl) {
        const float jac = 1.0f / (4.0f * fabsf(dot(wo, h)));
        const float prob = pr / (pr + pt);
        pdf = pdf * jac * prob;
        if (rev) pdf_rev = pdf_rev * (1.0f / (4.0f * fabsf(dot(wi, h)))) * prob;
        return V3(0.25f * D * G * F / fabsf(wo.z * wi.z));
    }
    float jd = dot(wi, h) + dot(wo, h) / eta;
    jd = jd * jd;
    const float jac = fabsf(dot(wi, h)) / jd;
    const float prob = pt / (pr + pt);
    pdf = pdf * jac * prob;
    if (rev) {
        const v3 hr = -h;
        float jr = eta * dot(wi, hr) + dot(wo, hr);
        jr = jr * jr;
        pdf_rev = pdf_rev * (fabsf(dot(wo, hr)) / jr) * prob;
    }
    return V3(0.0f);
}

__device__ __forceinline__ v3 eval_principled_brdf_rev(const Mat& m, v3 wo, v3 wi, float& pdf, float& pdf_rev, bool ff, bool rev) {
    pdf = 0.0f; pdf_rev = 0.0f;
    const v2 alpha = calc_anisotropy(m.roughness, m.anisotropy);
    if (fminf(alpha.x, alpha.y) <= 0.0064f) return V3(0.0f);
    if (wo.z * wi.z < 0.0f) return V3(0.0f);
    if (wo.z == 0.0f || wi.z == 0.0f) return V3(0.0f);
    const v3 h = normalize(wo + wi);
    const float jac = 1.0f / (4.0f * dot(wo, h));
    float D;
    pdf = vndf_pdf_aniso(alpha, wo, h, D) * jac;
    const float eta = ff ? m.ior : 1.0f / m.ior;
    if (rev) { float Dr; pdf_rev = vndf_pdf_aniso(alpha, wi, h, Dr) * jac; }
    const v3 F = disney_fresnel_m(m, wo, h, eta);
    return (0.25f * D) * F * G_corr_aniso(alpha, wo, wi) / (wi.z * wo.z);
}

__device__ __forceinline__ v3 eval_principled_rev(const Mat& m, v3 wo, v3 wi, float& pdf_w, float& pdf_rev_w, bool ff, bool rev) {
    pdf_w = 0.0f; pdf_rev_w = 0.0f;
    float ps, pd, pc, pt;
    const float F = fresnel_dielectric(wo.z, m.ior, ff);
    sampling_probs(m, F, ff, ps, pd, pc, pt);
    v3 f = V3(0.0f);
    float pdf = 0.0f, pdf_rev = 0.0f;
    const float brdf_w = (1.0f - m.spec_trans) * (1.0f - m.metallic);
    const float bsdf_w = (1.0f - m.metallic) * m.spec_trans;
    if (ps > 0.0f) {
        f = f + eval_principled_brdf_rev(m, wo, wi, pdf, pdf_rev, ff, rev);
        pdf *= ps; pdf_rev *= ps;
        pdf_w += pdf; pdf_rev_w += pdf_rev;
    }
    if (fminf(wi.z, wo.z) > 0.0f) {
        if (pd > 0.0f) {
            pdf_w += pd * diffuse_pdf(wo, wi);
            pdf_rev_w += pdf_w;
            f = f + brdf_w * disney_diffuse_factor(m, wo, wi);
        }
        if (pc > 0.0f) {
            const v3 h = normalize(wo + wi);
            float D;
            const float fc = clearcoat_factor(m, wo, wi, h, D);
            pdf = D / (4.0f * dot(wo, h));
            pdf_rev = pdf;
            f = f + V3(fc);
            pdf *= pc; pdf_rev *= pc;
            pdf_w += pdf; pdf_rev_w += pdf_rev;
        }
    }
    if (pt > 0.0f) {
        f = f + bsdf_w * eval_dielectric_rev(m, wo, wi, pdf, pdf_rev, ff, rev);
        pdf *= pt; pdf_rev *= pt;
        pdf_w += pdf; pdf_rev_w += pdf_rev;
    }
    return f;
}

// eval_bsdf(n_s, wo, mat, mode, ff, wi, pdf_w, pdf_rev_w, eval_reverse): the mode only changes the unused
// inner transmission value, so it is not a parameter here. MASK (LGB_BSDF_* bits) limits the lobes compiled in,
// as in bsdf.cuh: a type outside it evaluates to zero.
template <uint32_t MASK = kAllBsdfs>
__device__ __forceinline__ v3 eval_bsdf_rev(v3 n_s, v3 wo, const Mat& m, bool ff, v3 wi, float& pdf, float& pdf_rev, bool rev) {
    pdf = 0.0f; pdf_rev = 0.0f;
    v3 T, B;
    branchless_onb(n_s, T, B);
    wo = to_local(wo, T, B, n_s);
    wi = to_local(wi, T, B, n_s);
    switch (m.type & MASK) {
        case LGB_BSDF_DIFFUSE:
            if constexpr ((MASK & LGB_BSDF_DIFFUSE) != 0) {
                const v3 f = eval_diffuse(m, wo, wi, pdf);
                pdf_rev = pdf;
                return f;
            }
            break;
        case LGB_BSDF_DIELECTRIC:
            if constexpr ((MASK & LGB_BSDF_DIELECTRIC) != 0) return eval_dielectric_rev(m, wo, wi, pdf, pdf_rev, ff, rev);
            break;
        case LGB_BSDF_CONDUCTOR:
            if constexpr ((MASK & LGB_BSDF_CONDUCTOR) != 0) return eval_conductor_rev(m, wo, wi, pdf, pdf_rev, rev);
            break;
        case LGB_BSDF_PRINCIPLED:
            if constexpr ((MASK & LGB_BSDF_PRINCIPLED) != 0) return eval_principled_rev(m, wo, wi, pdf, pdf_rev, ff, rev);
            break;
        default: break;
    }
    return V3(0.0f);
}

__device__ __forceinline__ float conductor_pdf(const Mat& m, v3 wo, v3 wi) {
    const float alpha = m.roughness * m.roughness;
    if (effectively_delta(alpha)) return 0.0f;
    if (wo.z * wi.z < 0.0f) return 0.0f;
    if (wo.z == 0.0f || wi.z == 0.0f) return 0.0f;
    v3 h = normalize(wo + wi);
    h = h * signf(h.z);
    float D;
    return vndf_pdf_iso(alpha, wo, h, D) / (4.0f * dot(wo, h));
}

// eval_dielectric_pdf (dielectric.glsl:191-240)
__device__ __forceinline__ float dielectric_pdf_only(const Mat& m, v3 wo, v3 wi, bool ff) {
    const float rough = m.thin == 1u ? thin_roughness(m.ior, m.roughness) : m.roughness;
    const float alpha = rough * rough;
    if (alpha == 0.0f || m.ior == 1.0f) return 0.0f;
    const bool has_r = has_prop(m.props, LGB_FLAG_REFLECTION), has_t = has_prop(m.props, LGB_FLAG_TRANSMISSION);
    if (!has_r && !has_t) return 0.0f;
    const bool is_refl = wi.z * wo.z > 0.0f;
    float eta = 1.0f;
    if (!is_refl) eta = ff ? m.ior : 1.0f / m.ior;
    v3 h = normalize(wo + wi * eta);
    h = h * signf(h.z);
    if (wi.z == 0.0f || wo.z == 0.0f || dot(h, h) == 0.0f) return 0.0f;
    if (dot(wi, h) * wi.z < 0.0f || dot(wo, h) * wo.z < 0.0f) return 0.0f;
    const float F = fresnel_dielectric(dot(wo, h), m.ior, ff);
    const float pr = has_r ? F : 0.0f;
    const float pt = has_t ? (1.0f - F) : 0.0f;
    float D;
    float pdf = vndf_pdf_iso(alpha, wo, h, D);
    if (is_refl) return pdf * (1.0f / (4.0f * fabsf(dot(wo, h)))) * (pr / (pr + pt));
    float jd = dot(wi, h) + dot(wo, h) / eta;
    jd = jd * jd;
    return pdf * (fabsf(dot(wi, h)) / jd) * (pt / (pr + pt));
}

// eval_principled_brdf_pdf (principled.glsl:226-236) and eval_clearcoat_pdf (principled.glsl:177-181)
__device__ __forceinline__ float principled_brdf_pdf(const Mat& m, v3 wo, v3 wi) {
    const v2 alpha = calc_anisotropy(m.roughness, m.anisotropy);
    if (fminf(alpha.x, alpha.y) <= 0.0064f) return 0.0f;
    if (wo.z * wi.z < 0.0f) return 0.0f;
    if (wo.z == 0.0f || wi.z == 0.0f) return 0.0f;
    v3 h = normalize(wo + wi);
    h = h * signf(h.z);
    float D;
    return vndf_pdf_aniso(alpha, wo, h, D) / (4.0f * dot(wo, h));
}
__device__ __forceinline__ float clearcoat_pdf(const Mat& m, v3 wo, v3 wi) {
    const v3 h = normalize(wo + wi);
    const float D = D_iso(mixf(0.1f, 0.001f, m.clearcoat_gloss), h.z);
    return D / (4.0f * dot(wo, h));
}

template <uint32_t MASK = kAllBsdfs>
__device__ __forceinline__ float bsdf_pdf(const Mat& m, v3 n_s, v3 wo, v3 wi, bool ff) {
    v3 T, B;
    branchless_onb(n_s, T, B);
    wo = to_local(wo, T, B, n_s);
    wi = to_local(wi, T, B, n_s);
    switch (m.type & MASK) {
        case LGB_BSDF_DIFFUSE:
            if constexpr ((MASK & LGB_BSDF_DIFFUSE) != 0) return diffuse_pdf(wo, wi);
            break;
        case LGB_BSDF_DIELECTRIC:
            if constexpr ((MASK & LGB_BSDF_DIELECTRIC) != 0) return dielectric_pdf_only(m, wo, wi, ff);
            break;
        case LGB_BSDF_CONDUCTOR:
            if constexpr ((MASK & LGB_BSDF_CONDUCTOR) != 0) return conductor_pdf(m, wo, wi);
            break;
        case LGB_BSDF_PRINCIPLED:
            if constexpr ((MASK & LGB_BSDF_PRINCIPLED) != 0) {
            float pdf = 0.0f, ps, pd, pc, pt;
            const float F = fresnel_dielectric(wo.z, m.ior, ff);
            sampling_probs(m, F, ff, ps, pd, pc, pt);
            if (ps > 0.0f) pdf += ps * principled_brdf_pdf(m, wo, wi);
            if (fminf(wi.z, wo.z) > 0.0f) {
                if (pd > 0.0f) pdf += pd * diffuse_pdf(wo, wi);
                if (pc > 0.0f) pdf += pc * clearcoat_pdf(m, wo, wi);
            }
            if (pt > 0.0f) pdf += pt * dielectric_pdf_only(m, wo, wi, ff);
            return pdf;
            }
            break;
        default: break;
    }
    return 0.0f;
}

// sample_bsdf with an explicit transport mode (0 = importance, light subpaths; 1 = radiance).
template <uint32_t MASK = kAllBsdfs>
__device__ __forceinline__ v3 sample_bsdf_mode(v3 n_s, v3 wo, const Mat& m, uint32_t mode, bool ff, v3& wi, float& pdf,
                                               float& cos_t, v3 r) {
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
            if constexpr ((MASK & LGB_BSDF_GLASS) != 0) f = sample_glass(m, wo, wi, pdf, cos_t, mode, ff);
            break;
        case LGB_BSDF_DIELECTRIC:
            if constexpr ((MASK & LGB_BSDF_DIELECTRIC) != 0) f = sample_dielectric(m, wo, wi, mode, ff, pdf, cos_t, xy);
            break;
        case LGB_BSDF_CONDUCTOR:
            if constexpr ((MASK & LGB_BSDF_CONDUCTOR) != 0) f = sample_conductor(m, wo, wi, pdf, cos_t, xy);
            break;
        case LGB_BSDF_PRINCIPLED:
            if constexpr ((MASK & LGB_BSDF_PRINCIPLED) != 0) f = sample_principled(m, wo, wi, mode, ff, pdf, cos_t, r);
            break;
        default: break;
    }
    wi = to_world(wi, T, B, n_s);
    return f;
}

}  // namespace sh
}  // namespace lgb
