// Light sampling shared by the photon integrators (VCM and SPPM): emission sampling for light subpaths
// (sample_light_Le, commons.glsl:335-406) and the positional-directional incidence sample (sample_light_Li,
// commons.glsl:224-300), area and spot lights, with an identity world matrix (Lumen's loaders set no other).
#pragma once
#include "lgb_internal.cuh"
#include "path_common.cuh"
#include "shading.cuh"

namespace lgb {
namespace {

// The light list as the kernels sample it: lights picked uniformly, the emission pdf divided by the light
// triangle count (a non-area light counts as one), spot cones given by their two cosines.
struct LightSet {
    int num_lights, light_tri_count;
    float spot_cos_width, spot_cos_falloff;
};

// commons.glsl:112-149 with an identity world matrix
__device__ __forceinline__ void sample_tri(const SceneView& S, const lgb_mesh& pm, uint32_t tri, float rx, float ry, v3& pos,
                                           v3& n, float& tri_pdf) {
    const uint32_t io = pm.index_offset + 3u * tri;
    const DevVertex a = S.verts[S.idx[io] + pm.vertex_offset];
    const DevVertex b = S.verts[S.idx[io + 1] + pm.vertex_offset];
    const DevVertex c = S.verts[S.idx[io + 2] + pm.vertex_offset];
    const float su = 1.0f - sqrtf(rx), sv = ry * sqrtf(rx);
    const float b0 = 1.0f - su - sv;
    const v3 v0 = V3(a.px, a.py, a.pz), v1 = V3(b.px, b.py, b.pz), v2 = V3(c.px, c.py, c.pz);
    pos = v0 * b0 + v1 * su + v2 * sv;
    n = normalize(normalize(V3(a.nx, a.ny, a.nz) * b0 + V3(b.nx, b.ny, b.nz) * su + V3(c.nx, c.ny, c.nz) * sv));
    tri_pdf = 2.0f / length(cross(v1 - v0, v2 - v0));
}

struct Emission {
    v3 L, pos, wi, n;  // n: the emitter's normal (area), or wi itself (spot), as sample_light_Le returns it
    float cos_from_light, pdf_pos_a, pdf_dir_w;
    uint32_t flags;
};

// sample_light_Le (commons.glsl:335-406), area and spot lights
__device__ Emission sample_light_Le(const SceneView& S, const LightSet& A, float r0, float r1, float r2, float r3, float d0, float d1) {
    Emission e;
    const uint32_t li = (uint32_t)(r0 * (float)A.num_lights);
    const lgb_light* L = &S.lights[li];
    e.L = V3(0.0f); e.pos = V3(0.0f); e.wi = V3(0.0f); e.n = V3(0.0f);
    e.cos_from_light = 0.0f; e.pdf_pos_a = 0.0f; e.pdf_dir_w = 0.0f;
    e.flags = L->light_flags;
    const uint32_t type = L->light_flags & 7u;
    if (type == LGB_LIGHT_AREA) {
        const lgb_mesh pm = S.meshes[L->prim_mesh_idx];
        const uint32_t tri = (uint32_t)(r1 * (float)L->num_triangles);
        v3 n;
        float tri_pdf;
        sample_tri(S, pm, tri, r2, r3, e.pos, n, tri_pdf);
        const lgb_material* lm = &S.mats[pm.material_index];
        v3 T, B;
        branchless_onb(n, T, B);
        e.wi = to_world(sample_hemisphere(V2(d0, d1)), T, B, n);
        e.L = V3(lm->emissive_factor[0], lm->emissive_factor[1], lm->emissive_factor[2]);
        e.n = n;
        e.cos_from_light = fmaxf(dot(n, e.wi), 0.0f);
        e.pdf_pos_a = tri_pdf;
        e.pdf_dir_w = dot(e.wi, n) / LGB_PI;
    } else if (type == LGB_LIGHT_SPOT) {
        const float cos_width = A.spot_cos_width, cos_faloff = A.spot_cos_falloff;
        const v3 lp = V3(L->pos[0], L->pos[1], L->pos[2]);
        const v3 ldir = normalize(V3(L->to[0], L->to[1], L->to[2]) - lp);
        // to_local_quat (utils.glsl:157-160), then invert_quat and rot_quat (utils.glsl:167-172)
        float qx = 1.0f, qy = 0.0f, qz = 0.0f, qw = 0.0f;
        if (!(ldir.z < -0.99999f)) {
            qx = ldir.y; qy = -ldir.x; qz = 0.0f; qw = 1.0f + ldir.z;
            const float len = sqrtf(qx * qx + qy * qy + qz * qz + qw * qw);
            qx = qx / len; qy = qy / len; qz = qz / len; qw = qw / len;
        }
        const v3 a = V3(-qx, -qy, -qz);
        const float ct = (1.0f - d0) + d0 * cos_width;
        const float st = sqrtf(1.0f - ct * ct);
        const float phi = d1 * LGB_TWO_PI;
        const v3 cone = V3(cosf(phi) * st, sinf(phi) * st, ct);
        e.wi = 2.0f * dot(a, cone) * a + (qw * qw - dot(a, a)) * cone + 2.0f * qw * cross(a, cone);
        e.n = e.wi;
        e.pos = lp;
        e.cos_from_light = dot(e.wi, ldir);
        float fall;
        if (e.cos_from_light < cos_width) fall = 0.0f;
        else if (e.cos_from_light >= cos_faloff) fall = 1.0f;
        else { const float d = (e.cos_from_light - cos_width) / (cos_faloff - cos_width); fall = (d * d) * (d * d); }
        e.L = V3(L->L[0], L->L[1], L->L[2]) * fall;
        e.pdf_pos_a = 1.0f;
        e.pdf_dir_w = 1.0f / (LGB_TWO_PI * (1.0f - cos_width));
    }
    e.pdf_pos_a = e.pdf_pos_a / (float)A.light_tri_count;
    return e;
}

struct Incidence {
    v3 L, wi, pos, n;  // pos, n: the light point and its normal (-wi for a spot light)
    float wi_len, pdf_pos_w, pdf_pos_dir_w, cos_y, pdf_pos_a;
    uint32_t flags;
};

// sample_light_Li with the positional-directional pdf (commons.glsl:224-300), area and spot lights
__device__ Incidence sample_light_Li_pos(const SceneView& S, const LightSet& A, float r0, float r1, float r2, float r3, v3 p) {
    Incidence r;
    const uint32_t li = (uint32_t)(r0 * (float)A.num_lights);
    const lgb_light* L = &S.lights[li];
    r.L = V3(0.0f); r.wi = V3(0.0f); r.wi_len = 0.0f; r.pdf_pos_w = 0.0f; r.pdf_pos_dir_w = 0.0f; r.cos_y = 0.0f;
    r.pos = V3(0.0f); r.n = V3(0.0f); r.pdf_pos_a = 0.0f;
    r.flags = L->light_flags;
    const uint32_t type = L->light_flags & 7u;
    if (type == LGB_LIGHT_AREA) {
        const lgb_mesh pm = S.meshes[L->prim_mesh_idx];
        const uint32_t tri = (uint32_t)(r1 * (float)L->num_triangles);
        v3 pos, n;
        float tri_pdf;
        sample_tri(S, pm, tri, r2, r3, pos, n, tri_pdf);
        const lgb_material* lm = &S.mats[pm.material_index];
        v3 wi = pos - p;
        const float l2 = dot(wi, wi);
        r.wi_len = sqrtf(l2);
        wi = wi / r.wi_len;
        r.wi = wi;
        r.cos_y = fabsf(dot(n, -wi));
        r.L = V3(lm->emissive_factor[0], lm->emissive_factor[1], lm->emissive_factor[2]);
        r.pdf_pos_w = tri_pdf * l2 / r.cos_y;
        r.pdf_pos_dir_w = r.cos_y * LGB_INV_PI * tri_pdf;
        r.pdf_pos_a = tri_pdf;
        r.n = n;
        r.pos = pos;
    } else if (type == LGB_LIGHT_SPOT) {
        const v3 lp = V3(L->pos[0], L->pos[1], L->pos[2]);
        v3 wi = lp - p;
        const float l2 = dot(wi, wi);
        r.wi_len = sqrtf(l2);
        wi = wi / r.wi_len;
        r.wi = wi;
        const v3 ldir = normalize(V3(L->to[0], L->to[1], L->to[2]) - lp);
        r.cos_y = dot(-wi, ldir);
        const float cos_width = A.spot_cos_width, cos_faloff = A.spot_cos_falloff;
        float fall;
        if (r.cos_y < cos_width) fall = 0.0f;
        else if (r.cos_y >= cos_faloff) fall = 1.0f;
        else { const float d = (r.cos_y - cos_width) / (cos_faloff - cos_width); fall = (d * d) * (d * d); }
        r.pdf_pos_w = l2;
        r.pdf_pos_dir_w = 1.0f / (LGB_TWO_PI * (1.0f - cos_width));
        r.L = V3(L->L[0], L->L[1], L->L[2]) * fall;
        r.pdf_pos_a = 1.0f;
        r.n = -wi;
        r.pos = lp;
    }
    return r;
}

// Spot cone of sample_light_Le / sample_light_Li (commons.glsl:264-265 fixes the half-angle at 30 degrees and
// the falloff start at 25): half-angle `angle` degrees with the falloff from 25/30 of it, 0 for the fixed cone.
// Evaluated in double on the host so the oracle gets the same two floats.
inline void spot_cone(float angle, float& cos_width, float& cos_falloff) {
    const double a = angle > 0.0f ? (double)angle : 30.0;
    const double deg = 3.14159265358979323846 / 180.0;
    cos_width = (float)std::cos(a * deg);
    cos_falloff = (float)std::cos(a * (25.0 / 30.0) * deg);
}

}  // namespace
}  // namespace lgb
