// Device shading library: FP32 restatement of Lumen's GLSL shading code for the wavefront kernels.
//
// Sources (paths inside the reference project):
//   src/shaders/utils.glsl        pcg4d/rand 121-154, offset_ray 73-84, offset_ray2 90-93, luminance 99,
//                                 branchless_onb 185-191, to_world/to_local 193-195,
//                                 concentric_sample_disk 215-229
//   src/shaders/bsdf/*.glsl       sampling_commons, microfacet_commons, diffuse (Lambertian), mirror,
//                                 glass, dielectric, conductor, principled (ANISOTROPIC 1)
//   src/shaders/bsdf_commons.glsl sample_bsdf / eval_bsdf dispatch
// Every expression keeps the shader's evaluation order; this translation unit is compiled with
// -fmad=false, so products and sums round separately exactly as the FP32 CPU oracle does. Only the
// transcendental functions (sinf, cosf, powf) may differ from the host C library by a few ULP.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "lgb.h"

namespace lgb {
namespace sh {

#define LGB_PI 3.14159265359f
#define LGB_TWO_PI 6.28318530718f
#define LGB_INV_PI (1.0f / 3.14159265359f)

struct v3 { float x, y, z; };
struct v2 { float x, y; };

__device__ __forceinline__ v3 V3(float a, float b, float c) { v3 r; r.x = a; r.y = b; r.z = c; return r; }
__device__ __forceinline__ v3 V3(float a) { return V3(a, a, a); }
__device__ __forceinline__ v2 V2(float a, float b) { v2 r; r.x = a; r.y = b; return r; }
__device__ __forceinline__ v3 operator+(v3 a, v3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ v3 operator-(v3 a, v3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ v3 operator*(v3 a, v3 b) { return V3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ v3 operator*(v3 a, float s) { return V3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ v3 operator*(float s, v3 a) { return V3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ v3 operator/(v3 a, float s) { return V3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ v3 operator-(v3 a) { return V3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ v3 cross(v3 a, v3 b) {
    return V3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
__device__ __forceinline__ float length(v3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ v3 normalize(v3 a) { float l = length(a); return V3(a.x / l, a.y / l, a.z / l); }
__device__ __forceinline__ float mixf(float x, float y, float a) { return x * (1.0f - a) + y * a; }
__device__ __forceinline__ v3 mix3(v3 x, v3 y, float a) { return V3(mixf(x.x, y.x, a), mixf(x.y, y.y, a), mixf(x.z, y.z, a)); }
__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
__device__ __forceinline__ v3 reflect(v3 I, v3 N) { return I - (2.0f * dot(N, I)) * N; }
__device__ __forceinline__ float signf(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
__device__ __forceinline__ v3 sqrt3(v3 a) { return V3(sqrtf(a.x), sqrtf(a.y), sqrtf(a.z)); }
__device__ __forceinline__ bool has_prop(uint32_t props, uint32_t flag) { return (props & flag) != 0u; }

// ---------------- RNG (utils.glsl:121-154) ----------------
__device__ __forceinline__ uint4 pcg4d(uint4 v) {
    v.x = v.x * 1664525u + 1013904223u; v.y = v.y * 1664525u + 1013904223u;
    v.z = v.z * 1664525u + 1013904223u; v.w = v.w * 1664525u + 1013904223u;
    v.x += v.y * v.w; v.y += v.z * v.x; v.z += v.x * v.y; v.w += v.y * v.z;
    v.x ^= v.x >> 16; v.y ^= v.y >> 16; v.z ^= v.z >> 16; v.w ^= v.w >> 16;
    v.x += v.y * v.w; v.y += v.z * v.x; v.z += v.x * v.y; v.w += v.y * v.z;
    return v;
}
// rand(): w is incremented first, then pcg4d(state).x is mapped into [0, 1).
__device__ __forceinline__ float rnd(uint4& s) {
    s.w++;
    return __uint_as_float(0x3f800000u | (pcg4d(s).x >> 9)) - 1.0f;
}

__device__ __forceinline__ v3 offset_ray(v3 p, v3 n) {
    const float origin = 1.0f / 32.0f, float_scale = 1.0f / 65536.0f, int_scale = 256.0f;
    const int ox = (int)(int_scale * n.x), oy = (int)(int_scale * n.y), oz = (int)(int_scale * n.z);
    const float pix = __int_as_float(__float_as_int(p.x) + ((p.x < 0.0f) ? -ox : ox));
    const float piy = __int_as_float(__float_as_int(p.y) + ((p.y < 0.0f) ? -oy : oy));
    const float piz = __int_as_float(__float_as_int(p.z) + ((p.z < 0.0f) ? -oz : oz));
    return V3(fabsf(p.x) < origin ? p.x + float_scale * n.x : pix, fabsf(p.y) < origin ? p.y + float_scale * n.y : piy,
              fabsf(p.z) < origin ? p.z + float_scale * n.z : piz);
}
__device__ __forceinline__ v3 offset_ray2(v3 p, v3 n) { return p + (2.0f / 65536.0f) * n; }
__device__ __forceinline__ float luminance(v3 c) { return dot(c, V3(0.2126f, 0.7152f, 0.0722f)); }

__device__ __forceinline__ void branchless_onb(v3 n, v3& b1, v3& b2) {
    const float sgn = n.z >= 0.0f ? 1.0f : -1.0f;
    const float a = -1.0f / (sgn + n.z);
    const float b = n.x * n.y * a;
    b1 = V3(1.0f + sgn * n.x * n.x * a, sgn * b, -sgn * n.x);
    b2 = V3(b, sgn + n.y * n.y * a, -n.y);
}
__device__ __forceinline__ v3 to_world(v3 v, v3 T, v3 B, v3 N) { return v.x * T + v.y * B + v.z * N; }
__device__ __forceinline__ v3 to_local(v3 v, v3 T, v3 B, v3 N) { return V3(dot(v, T), dot(v, B), dot(v, N)); }

__device__ __forceinline__ v2 concentric_sample_disk(v2 r) {
    const v2 o = V2(2.0f * r.x - 1.0f, 2.0f * r.y - 1.0f);
    if (o.x == 0.0f && o.y == 0.0f) return V2(0.0f, 0.0f);
    float theta, rad;
    if (fabsf(o.x) > fabsf(o.y)) {
        rad = o.x;
        theta = 0.25f * LGB_PI * o.y / o.x;
    } else {
        rad = o.y;
        theta = LGB_PI * (0.5f - 0.25f * o.x / o.y);
    }
    return V2(rad * cosf(theta), rad * sinf(theta));
}
__device__ __forceinline__ v3 sample_hemisphere(v2 xi) {
    const v2 d = concentric_sample_disk(xi);
    const float z = sqrtf(fmaxf(0.0f, 1.0f - (d.x * d.x + d.y * d.y)));
    return V3(d.x, d.y, z);
}

// ---------------- sampling_commons.glsl ----------------
__device__ __forceinline__ bool effectively_delta(float a) { return a <= 0.0064f; }

__device__ __forceinline__ void refract(v3 n_s, v3 wo, bool ff, float eta, uint32_t mode, v3& wi, v3& f, float& inv_eta) {
    const float cos_i = dot(n_s, wo);
    inv_eta = ff ? 1.0f / eta : eta;
    const float sin2_t = inv_eta * inv_eta * (1.0f - cos_i * cos_i);
    if (sin2_t >= 1.0f) {
        wi = reflect(-wo, n_s);
    } else {
        const float cos_t = sqrtf(1.0f - sin2_t);
        wi = -inv_eta * wo + (inv_eta * cos_i - cos_t) * n_s;
    }
    f = mode == 1u ? V3(inv_eta * inv_eta) : V3(1.0f);
}

__device__ __forceinline__ float fresnel_dielectric(float cos_i, float eta, bool ff) {
    cos_i = clampf(cos_i, -1.0f, 1.0f);
    if (!ff) eta = 1.0f / eta;
    if (cos_i < 0.0f) { eta = 1.0f / eta; cos_i = -cos_i; }
    const float sin2_i = 1.0f - cos_i * cos_i;
    const float sin2_t = sin2_i / (eta * eta);
    if (sin2_t >= 1.0f) return 1.0f;
    const float cos_t = sqrtf(1.0f - sin2_t);
    const float rpa = (eta * cos_i - cos_t) / (eta * cos_i + cos_t);
    const float rpe = (cos_i - eta * cos_t) / (cos_i + eta * cos_t);
    return 0.5f * (rpa * rpa + rpe * rpe);
}

__device__ __forceinline__ float fresnel_conductor1(float cos_i, float eta, float k) {
    const float cos_sqr = cos_i * cos_i;
    const float sin_sqr = fmaxf(1.0f - cos_sqr, 0.0f);
    const float sin_4 = sin_sqr * sin_sqr;
    const float inner = eta * eta - k * k - sin_sqr;
    const float ab = sqrtf(fmaxf(inner * inner + 4.0f * eta * eta * k * k, 0.0f));
    const float a = sqrtf(fmaxf((ab + inner) * 0.5f, 0.0f));
    const float rs = ((ab + cos_sqr) - (2.0f * a * cos_i)) / ((ab + cos_sqr) + (2.0f * a * cos_i));
    const float rp = ((cos_sqr * ab + sin_4) - (2.0f * a * cos_i * sin_sqr)) / ((cos_sqr * ab + sin_4) + (2.0f * a * cos_i * sin_sqr));
    return 0.5f * (rs + rs * rp);
}
__device__ __forceinline__ v3 fresnel_conductor(float cos_i, v3 eta, v3 k) {
    return V3(fresnel_conductor1(cos_i, eta.x, k.x), fresnel_conductor1(cos_i, eta.y, k.y), fresnel_conductor1(cos_i, eta.z, k.z));
}
__device__ __forceinline__ float fresnel_schlick(float f0, float f90, float ns) {
    return f0 + (f90 - f0) * powf(fmaxf(1.0f - ns, 0.0f), 5.0f);
}
__device__ __forceinline__ v3 fresnel_schlick3(v3 f0, v3 f90, float ns) {
    const float p = powf(fmaxf(1.0f - ns, 0.0f), 5.0f);
    return f0 + (f90 - f0) * p;
}
__device__ __forceinline__ float eta_to_schlick_R0(float eta) { const float v = (eta - 1.0f) / (eta + 1.0f); return v * v; }
__device__ __forceinline__ v3 calc_tint(v3 albedo) {
    const float lum = luminance(albedo);
    return lum > 0.0f ? albedo / lum : V3(1.0f);
}

// ---------------- microfacet_commons.glsl ----------------
__device__ __forceinline__ float smith_lambda_iso(float a2, float c) {
    if (c == 0.0f) return 0.0f;
    const float cs = c * c;
    const float ts = fmaxf(1.0f - cs, 0.0f) / cs;
    return 0.5f * (sqrtf(1.0f + a2 * ts) - 1.0f);
}
__device__ __forceinline__ float smith_lambda_aniso(v3 w, v2 alpha) {
    const float cs = w.z * w.z;
    const float ss = fmaxf(1.0f - cs, 0.0f);
    const float ts = ss / cs;
    if (isinf(ts)) return 0.0f;
    v2 cp = ss == 0.0f ? V2(1.0f, 0.0f) : V2(clampf(w.x * w.x, 0.0f, 1.0f) / ss, clampf(w.y * w.y, 0.0f, 1.0f) / ss);
    const float a2 = cp.x * (alpha.x * alpha.x) + cp.y * (alpha.y * alpha.y);
    return 0.5f * (sqrtf(1.0f + a2 * ts) - 1.0f);
}
__device__ __forceinline__ float G1_aniso(v3 w, v2 alpha) { return 1.0f / (1.0f + smith_lambda_aniso(w, alpha)); }
__device__ __forceinline__ float G_corr_iso(float alpha, v3 wo, v3 wi) {
    const float a2 = alpha * alpha;
    return 1.0f / (1.0f + smith_lambda_iso(a2, wo.z) + smith_lambda_iso(a2, wi.z));
}
__device__ __forceinline__ float G_corr_aniso(v2 alpha, v3 wo, v3 wi) {
    return 1.0f / (1.0f + smith_lambda_aniso(wo, alpha) + smith_lambda_aniso(wi, alpha));
}
__device__ __forceinline__ float D_aniso(v2 alpha, v3 h) {
    const float cs = h.z * h.z;
    const float ss = fmaxf(1.0f - cs, 0.0f);
    const float ts = ss / cs;
    if (isinf(ts)) return 0.0f;
    const float c4 = cs * cs;
    if (c4 < 1e-16f) return 0.0f;
    v2 ps = ss == 0.0f ? V2(1.0f, 0.0f) : V2(clampf(h.x * h.x, 0.0f, 1.0f) / ss, clampf(h.y * h.y, 0.0f, 1.0f) / ss);
    const v2 a2 = V2(ps.x / (alpha.x * alpha.x), ps.y / (alpha.y * alpha.y));
    const float e = ts * (a2.x + a2.y);
    return 1.0f / (LGB_PI * alpha.x * alpha.y * c4 * (1.0f + e) * (1.0f + e));
}
__device__ __forceinline__ float D_iso(float a2, float c) {
    const float d = ((c * a2 - c) * c + 1.0f);
    return a2 / (d * d * LGB_PI);
}
__device__ __forceinline__ float G1_iso(float a2, float c) {
    const float cs = c * c;
    const float ts = fmaxf(1.0f - cs, 0.0f) / cs;
    return 2.0f / (1.0f + sqrtf(1.0f + a2 * ts));
}
__device__ __forceinline__ float vndf_pdf_iso(float alpha, v3 wo, v3 h, float& D) {
    D = 0.0f;
    if (wo.z <= 0.0f) return 0.0f;
    const float a2 = alpha * alpha;
    const float G1 = G1_iso(a2, wo.z);
    D = D_iso(a2, h.z);
    return G1 * D * fmaxf(0.0f, dot(wo, h)) / fabsf(wo.z);
}
__device__ __forceinline__ float vndf_pdf_aniso(v2 alpha, v3 wo, v3 h, float& D) {
    D = 0.0f;
    if (wo.z <= 0.0f) return 0.0f;
    const float G1 = G1_aniso(wo, alpha);
    D = D_aniso(alpha, h);
    return G1 * D * fmaxf(0.0f, dot(wo, h)) / fabsf(wo.z);
}
__device__ __forceinline__ v3 sample_vndf(v2 alpha, v3 wo, v2 xi) {
    const v3 wh = normalize(V3(alpha.x * wo.x, alpha.y * wo.y, wo.z));
    const float phi = 2.0f * LGB_PI * xi.x;
    const float z = ((1.0f - xi.y) * (1.0f + wh.z)) - wh.z;
    const float sin_theta = sqrtf(clampf(1.0f - z * z, 0.0f, 1.0f));
    const float x = sin_theta * cosf(phi);
    const float y = sin_theta * sinf(phi);
    const v3 nh = V3(x, y, z) + wh;
    return normalize(V3(alpha.x * nh.x, alpha.y * nh.y, fmaxf(0.0f, nh.z)));
}

}  // namespace sh
}  // namespace lgb
