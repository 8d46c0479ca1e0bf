// Helpers shared by the path-tracing kernels (path.cu) and the differentiable path kernels (adjoint.cu):
// scene view, hit attribute reconstruction (ray.rchit:24-84), texture lookup, camera matrix products.
#pragma once
#include "bsdf.cuh"
#include "lgb_internal.cuh"
#include "traverse.cuh"

namespace lgb {
namespace {
using namespace sh;

struct SceneView {
    const WideNode* nodes;
    const WideTri* tris;
    const DevVertex* verts;
    const uint32_t* idx;
    const uint32_t* tri_mesh;
    const uint8_t* tri_class;  // shading class per triangle (shade_class of its material)
    const lgb_mesh* meshes;
    const uint32_t* mesh_first;
    const lgb_material* mats;
    const lgb_light* lights;
    const DevTexture* texs;
    uint32_t* status;
};

__device__ __forceinline__ uint32_t agg_slot(uint32_t* ctr, bool pred) {
    const uint32_t m = __ballot_sync(0xffffffffu, pred);
    const int lane = threadIdx.x & 31;
    uint32_t base = 0;
    if (lane == 0 && m) base = atomicAdd(ctr, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    return base + (uint32_t)__popc(m & ((1u << lane) - 1u));
}

__device__ __forceinline__ v3 f3(float4 a) { return V3(a.x, a.y, a.z); }
__device__ __forceinline__ float4 f4(v3 a, float w) { return make_float4(a.x, a.y, a.z, w); }
__device__ __forceinline__ lgb_ray make_ray(v3 o, float tmin, v3 d, float tmax) {
    lgb_ray r;
    r.ox = o.x; r.oy = o.y; r.oz = o.z; r.tmin = tmin;
    r.dx = d.x; r.dy = d.y; r.dz = d.z; r.tmax = tmax;
    return r;
}
__device__ __forceinline__ void store_ray(lgb_ray* dst, const lgb_ray& r) {
    float4* p = reinterpret_cast<float4*>(dst);
    p[0] = make_float4(r.ox, r.oy, r.oz, r.tmin);
    p[1] = make_float4(r.dx, r.dy, r.dz, r.tmax);
}
__device__ __forceinline__ uint4 seed_of(uint32_t pix, uint32_t width, uint32_t frame, uint32_t w) {
    return make_uint4(pix % width, pix / width, frame, w);
}

// GLSL mat4 * vec4 on column-major storage, summed over columns in order.
__device__ __forceinline__ float4 mat_vec(const float* m, float x, float y, float z, float w) {
    float r[4];
#pragma unroll
    for (int row = 0; row < 4; row++) r[row] = m[row] * x + m[4 + row] * y + m[8 + row] * z + m[12 + row] * w;
    return make_float4(r[0], r[1], r[2], r[3]);
}

// Bilinear REPEAT lookup at LOD 0 in linear FP32.
__device__ __forceinline__ v3 tex_lookup(const DevTexture& t, float u, float v) {
    if (!isfinite(u) || !isfinite(v)) { u = 0.0f; v = 0.0f; }  // keep the wrap arithmetic in range
    const float x = u * (float)t.width - 0.5f, y = v * (float)t.height - 0.5f;
    const float x0 = floorf(x), y0 = floorf(y);
    const float fx = x - x0, fy = y - y0;
    const long long W = t.width, H = t.height;
    long long ix = (long long)x0 % W; if (ix < 0) ix += W;
    long long iy = (long long)y0 % H; if (iy < 0) iy += H;
    const long long ix1 = (ix + 1) % W, iy1 = (iy + 1) % H;
    const float4 c00 = t.texels[iy * W + ix], c10 = t.texels[iy * W + ix1];
    const float4 c01 = t.texels[iy1 * W + ix], c11 = t.texels[iy1 * W + ix1];
    const float w00 = (1.0f - fx) * (1.0f - fy), w10 = fx * (1.0f - fy), w01 = (1.0f - fx) * fy, w11 = fx * fy;
    return f3(c00) * w00 + f3(c10) * w10 + f3(c01) * w01 + f3(c11) * w11;
}

// ray.rchit:24-84 for an identity object-to-world transform: the matrix products reduce to their
// arguments while the second normalisation of the shading normal is kept.
struct HitAttr {
    v3 n_g, n_s, pos;
    float u, v;
    uint32_t mat;
    float area;  // world-space triangle area (ray.rchit:81)
};
__device__ __forceinline__ HitAttr resolve_hit(const SceneView& S, uint32_t prim, float bu, float bv) {
    HitAttr h;
    const uint32_t mesh = S.tri_mesh[prim];
    const lgb_mesh pm = S.meshes[mesh];
    const uint32_t local = prim - S.mesh_first[mesh];
    const uint32_t io = pm.index_offset + 3u * local;
    const DevVertex a = S.verts[S.idx[io] + pm.vertex_offset];
    const DevVertex b = S.verts[S.idx[io + 1] + pm.vertex_offset];
    const DevVertex c = S.verts[S.idx[io + 2] + pm.vertex_offset];
    const float b0 = 1.0f - bu - bv, b1 = bu, b2 = bv;
    const v3 v0 = V3(a.px, a.py, a.pz), v1 = V3(b.px, b.py, b.pz), v2 = V3(c.px, c.py, c.pz);
    const v3 n0 = V3(a.nx, a.ny, a.nz), n1 = V3(b.nx, b.ny, b.nz), n2 = V3(c.nx, c.ny, c.nz);
    h.pos = v0 * b0 + v1 * b1 + v2 * b2;
    h.n_s = normalize(normalize(n0 * b0 + n1 * b1 + n2 * b2));
    h.u = a.u * b0 + b.u * b1 + c.u * b2;
    h.v = a.v * b0 + b.v * b1 + c.v * b2;
    const v3 cr = cross(v2 - v0, v1 - v0);
    h.n_g = normalize(cr);
    h.area = 0.5f * length(cr);
    h.mat = pm.material_index;
    return h;
}

__device__ __forceinline__ Mat load_material(const SceneView& S, uint32_t idx, float u, float v) {
    Mat m = load_mat(&S.mats[idx]);
    const int tid = S.mats[idx].texture_id;
    if (tid > -1) m.albedo = m.albedo * tex_lookup(S.texs[tid], u, v);
    return m;
}


inline SceneView scene_view(Scene* s) {
    SceneView S;
    S.nodes = s->bvh.nodes; S.tris = s->bvh.tris; S.verts = s->d_vertices; S.idx = s->d_indices;
    S.tri_mesh = s->d_tri_mesh; S.tri_class = s->d_tri_class; S.meshes = s->d_meshes; S.mesh_first = s->d_mesh_first_tri; S.mats = s->d_materials;
    S.lights = s->d_lights; S.texs = s->d_textures; S.status = s->d_status;
    return S;
}

}  // namespace
}  // namespace lgb
