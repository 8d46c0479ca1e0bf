// C ABI of liblgb: contexts, scene upload, and the entry points declared in include/lgb.h.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "lgb_internal.cuh"

namespace lgb {

lgb_status set_error(Ctx* ctx, lgb_status st, const std::string& msg) {
    if (ctx) ctx->last_error = msg;
    return st;
}

lgb_status cuda_error(Ctx* ctx, cudaError_t e, const char* what) {
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    return set_error(ctx, e == cudaErrorMemoryAllocation ? LGB_ERR_OUT_OF_MEMORY : LGB_ERR_CUDA, m);
}

void ctx_retain(Ctx* c) { c->users++; }
void ctx_release(Ctx* c) {
    if (c->users > 0) c->users--;
    if (c->users == 0 && c->released) delete static_cast<lgb_ctx*>(c);
}

namespace {

void free_scene(Scene* s) {
    cudaFree(s->d_tri_verts);
    cudaFree(s->d_vertices);
    cudaFree(s->d_indices);
    cudaFree(s->d_tri_mesh);
    cudaFree(s->d_tri_class);
    cudaFree(s->d_meshes);
    cudaFree(s->d_mesh_first_tri);
    cudaFree(s->d_materials);
    cudaFree(s->d_lights);
    cudaFree(s->d_textures);
    for (void* p : s->texture_buffers) cudaFree(p);
    cudaFree(s->bvh.nodes);
    cudaFree(s->bvh.tris);
    cudaFree(s->d_status);
    cudaFree(s->d_ray_counter);
    cudaFree(s->pt_buf);
    cudaFree(s->diff_buf);
    cudaFree(s->diffw_buf);
    cudaFree(s->vcm_buf);
    cudaFree(s->sppm_buf);
    cudaFree(s->bdpt_buf);
    cudaFree(s->restir_buf);
    if (s->pt_graph) cudaGraphExecDestroy((cudaGraphExec_t)s->pt_graph);
    if (s->capture_stream) cudaStreamDestroy((cudaStream_t)s->capture_stream);
    cudaFree(s->stage_buf);
    if (s->stream_h2d) cudaStreamDestroy((cudaStream_t)s->stream_h2d);
    if (s->stream_d2h) cudaStreamDestroy((cudaStream_t)s->stream_d2h);
    for (void* e : s->stage_events) cudaEventDestroy((cudaEvent_t)e);
}

template <class T> cudaError_t upload(T** dst, const T* src, size_t count) {
    *dst = nullptr;
    cudaError_t e = cudaMalloc((void**)dst, sizeof(T) * (count ? count : 1));
    if (e != cudaSuccess) return e;
    if (count) e = cudaMemcpy(*dst, src, sizeof(T) * count, cudaMemcpyHostToDevice);
    return e;
}

bool is_identity(const float* m) {
    for (int c = 0; c < 4; c++)
        for (int r = 0; r < 4; r++)
            if (m[4 * c + r] != (c == r ? 1.0f : 0.0f)) return false;
    return true;
}

void invert4(const double m[16], double out[16]) {
    // Inverse by Gauss-Jordan elimination with partial pivoting (column-major storage m[4*c + r]).
    double a[4][8];
    for (int r = 0; r < 4; r++) {
        for (int c = 0; c < 4; c++) a[r][c] = m[4 * c + r];
        for (int c = 0; c < 4; c++) a[r][4 + c] = (r == c) ? 1.0 : 0.0;
    }
    for (int col = 0; col < 4; col++) {
        int piv = col;
        for (int r = col + 1; r < 4; r++)
            if (std::fabs(a[r][col]) > std::fabs(a[piv][col])) piv = r;
        if (piv != col)
            for (int c = 0; c < 8; c++) std::swap(a[piv][c], a[col][c]);
        double d = a[col][col];
        for (int c = 0; c < 8; c++) a[col][c] /= d;
        for (int r = 0; r < 4; r++) {
            if (r == col) continue;
            double f = a[r][col];
            if (f == 0.0) continue;
            for (int c = 0; c < 8; c++) a[r][c] -= f * a[col][c];
        }
    }
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) out[4 * c + r] = a[r][4 + c];
}

}  // namespace
}  // namespace lgb

using namespace lgb;

extern "C" {

LGB_API uint32_t lgb_abi_version(void) { return 2u; }

LGB_API lgb_status lgb_create(lgb_ctx** out, int device, const char* tuning_cache_path) {
    if (!out) return LGB_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return LGB_ERR_CUDA;
    if (device < 0 || device >= count) return LGB_ERR_INVALID_ARGUMENT;
    if (cudaSetDevice(device) != cudaSuccess) return LGB_ERR_CUDA;
    lgb_ctx* c = new (std::nothrow) lgb_ctx();
    if (!c) return LGB_ERR_OUT_OF_MEMORY;
    c->device = device;
    if (tuning_cache_path) c->tuning_cache = tuning_cache_path;
    cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
    *out = c;
    return LGB_OK;
}

LGB_API void lgb_destroy(lgb_ctx* ctx) {
    if (!ctx) return;
    if (ctx->users == 0) delete ctx;
    else ctx->released = true;
}

LGB_API const char* lgb_last_error(const lgb_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "null context"; }

LGB_API lgb_status lgb_scene_create(lgb_ctx* ctx, const lgb_scene_desc* d, lgb_scene** out) {
    if (!ctx) return LGB_ERR_INVALID_ARGUMENT;
    if (!d || !out) return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "null scene description or output");
    *out = nullptr;
    cudaSetDevice(ctx->device);
    if ((d->num_vertices && (!d->positions || !d->normals || !d->uvs)) || (d->num_indices && !d->indices) ||
        (d->num_meshes && !d->meshes) || (d->num_materials && !d->materials) || (d->num_lights && !d->lights) ||
        (d->num_textures && !d->textures))
        return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "scene array pointer is null for a non-zero count");
    // validate meshes and flatten triangles
    std::vector<uint32_t> first_tri(d->num_meshes);
    uint64_t ntri64 = 0;
    for (uint32_t m = 0; m < d->num_meshes; m++) {
        const lgb_mesh& pm = d->meshes[m];
        first_tri[m] = (uint32_t)ntri64;
        if ((uint64_t)pm.index_offset + 3ull * pm.tri_count > d->num_indices)
            return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "mesh " + std::to_string(m) + " indexes past the index array");
        if (pm.material_index >= d->num_materials)
            return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "mesh " + std::to_string(m) + " has an invalid material");
        ntri64 += pm.tri_count;
    }
    if (ntri64 >= 0x7fffffffull) return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "too many triangles");
    const uint32_t ntri = (uint32_t)ntri64;
    for (uint32_t i = 0; i < d->num_materials; i++) {
        int tid = d->materials[i].texture_id;
        if (tid >= (int)d->num_textures) return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "material texture id out of range");
    }
    for (uint32_t i = 0; i < d->num_lights; i++) {
        const lgb_light& l = d->lights[i];
        uint32_t type = l.light_flags & 7u;
        if (type != LGB_LIGHT_AREA && type != LGB_LIGHT_SPOT && type != LGB_LIGHT_DIRECTIONAL)
            return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "light " + std::to_string(i) + " has an unknown type");
        if (type == LGB_LIGHT_AREA) {
            if (l.prim_mesh_idx >= d->num_meshes || l.num_triangles == 0 ||
                l.num_triangles > d->meshes[l.prim_mesh_idx].tri_count)
                return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "area light " + std::to_string(i) + " has a bad mesh");
            if (!is_identity(l.world_matrix))
                return set_error(ctx, LGB_ERR_UNSUPPORTED, "area light world_matrix must be the identity");
        }
    }
    std::vector<float> tv(9 * (size_t)ntri);
    std::vector<uint32_t> tri_mesh(ntri);
    std::vector<uint8_t> tri_class(ntri);
    float bmin[3] = {INFINITY, INFINITY, INFINITY}, bmax[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t m = 0; m < d->num_meshes; m++) {
        const lgb_mesh& pm = d->meshes[m];
        for (uint32_t t = 0; t < pm.tri_count; t++) {
            uint32_t g = first_tri[m] + t;
            tri_mesh[g] = m;
            tri_class[g] = (uint8_t)shade_class(d->materials[pm.material_index].bsdf_type);
            for (int k = 0; k < 3; k++) {
                uint64_t v = (uint64_t)d->indices[pm.index_offset + 3 * t + k] + pm.vertex_offset;
                if (v >= d->num_vertices)
                    return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "index out of range in mesh " + std::to_string(m));
                for (int a = 0; a < 3; a++) {
                    float x = d->positions[3 * v + a];
                    if (!std::isfinite(x))
                        return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "non-finite vertex position");
                    tv[9 * (size_t)g + 3 * k + a] = x;
                    bmin[a] = std::fmin(bmin[a], x);
                    bmax[a] = std::fmax(bmax[a], x);
                }
            }
        }
    }
    lgb_scene* s = new (std::nothrow) lgb_scene();
    if (!s) return set_error(ctx, LGB_ERR_OUT_OF_MEMORY, "host allocation failed");
    s->ctx = ctx;
    s->num_tris = ntri;
    s->num_vertices = d->num_vertices;
    s->num_meshes = d->num_meshes;
    s->num_materials = d->num_materials;
    for (uint32_t i = 0; i < d->num_materials; i++) {
        s->bsdf_mask |= d->materials[i].bsdf_type;
        s->shade_classes |= 1u << shade_class(d->materials[i].bsdf_type);
    }
    s->num_lights = d->num_lights;
    for (uint32_t i = 0; i < d->num_lights; i++)
        if ((d->lights[i].light_flags & 7u) == LGB_LIGHT_DIRECTIONAL) s->num_directional++;
    s->num_textures = d->num_textures;
    s->bmin = make_float3(bmin[0], bmin[1], bmin[2]);
    s->bmax = make_float3(bmax[0], bmax[1], bmax[2]);
    if (ntri == 0) { s->bmin = make_float3(0, 0, 0); s->bmax = make_float3(0, 0, 0); }
    s->h_mesh_first_tri = first_tri;
    s->h_meshes.assign(d->meshes, d->meshes + d->num_meshes);
    std::vector<DevVertex> verts(d->num_vertices);
    for (uint32_t v = 0; v < d->num_vertices; v++) {
        DevVertex& o = verts[v];
        o.px = d->positions[3 * v]; o.py = d->positions[3 * v + 1]; o.pz = d->positions[3 * v + 2];
        o.nx = d->normals[3 * v]; o.ny = d->normals[3 * v + 1]; o.nz = d->normals[3 * v + 2];
        o.u = d->uvs[2 * v]; o.v = d->uvs[2 * v + 1];
    }
    std::vector<DevTexture> texs(d->num_textures);
    cudaError_t e = cudaSuccess;
    const char* what = "";
#define UP(dst, src, cnt) \
    if (e == cudaSuccess) { e = upload(dst, src, cnt); what = #dst; }
    UP(&s->d_tri_verts, tv.data(), tv.size());
    UP(&s->d_vertices, verts.data(), verts.size());
    UP(&s->d_indices, d->indices, d->num_indices);
    UP(&s->d_tri_mesh, tri_mesh.data(), tri_mesh.size());
    UP(&s->d_tri_class, tri_class.data(), tri_class.size());
    UP(&s->d_meshes, d->meshes, d->num_meshes);
    UP(&s->d_mesh_first_tri, first_tri.data(), first_tri.size());
    UP(&s->d_materials, d->materials, d->num_materials);
    UP(&s->d_lights, d->lights, d->num_lights);
    for (uint32_t i = 0; i < d->num_textures && e == cudaSuccess; i++) {
        const lgb_texture& t = d->textures[i];
        float4* buf = nullptr;
        size_t texels = (size_t)t.width * t.height;
        if (texels == 0 || !t.rgba) { e = cudaErrorInvalidValue; what = "texture"; break; }
        e = upload(&buf, reinterpret_cast<const float4*>(t.rgba), texels);
        what = "texture";
        if (buf) s->texture_buffers.push_back(buf);
        texs[i].width = t.width; texs[i].height = t.height; texs[i].texels = buf;
    }
    UP(&s->d_textures, texs.data(), texs.size());
    uint32_t zero = 0;
    UP(&s->d_status, &zero, 1);
    UP(&s->d_ray_counter, &zero, 1);
#undef UP
    if (e != cudaSuccess) {
        lgb_status st = cuda_error(ctx, e, what);
        free_scene(s);
        delete s;
        return st;
    }
    *out = s;
    ctx_retain(ctx);
    return LGB_OK;
}

LGB_API lgb_status lgb_scene_set_visit_limit(lgb_scene* s, uint32_t max_visits) {
    if (!s) return LGB_ERR_INVALID_ARGUMENT;
    s->visit_limit = max_visits;
    return LGB_OK;
}

LGB_API void lgb_scene_destroy(lgb_scene* s) {
    if (!s) return;
    Ctx* c = s->ctx;
    cudaSetDevice(c->device);
    free_scene(s);
    delete s;
    ctx_release(c);
}

LGB_API lgb_status lgb_bvh_build(lgb_scene* s, const lgb_build_opts* opts, lgb_build_stats* stats) {
    if (!s) return LGB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->ctx->device);
    lgb_status st = build_bvh(s, opts, stats);
    if (st == LGB_OK && s->bvh.max_depth > (uint32_t)kStackSize + 1u)
        return set_error(s->ctx, LGB_ERR_UNSUPPORTED, "BVH deeper than the traversal stack");
    return st;
}

static lgb_status check_trace(lgb_scene* s, const void* rays, const void* out, uint32_t n) {
    if (!s) return LGB_ERR_INVALID_ARGUMENT;
    if (n == 0) return LGB_OK;
    if (!rays || !out) return set_error(s->ctx, LGB_ERR_INVALID_ARGUMENT, "null ray or result buffer");
    if (n >= 0x80000000u) return set_error(s->ctx, LGB_ERR_INVALID_ARGUMENT, "at most 2^31 - 1 rays per call");
    if ((reinterpret_cast<uintptr_t>(rays) & 15u) || (reinterpret_cast<uintptr_t>(out) & 3u))
        return set_error(s->ctx, LGB_ERR_INVALID_ARGUMENT, "ray buffer must be 16-byte aligned");
    if (!s->bvh.nodes) return set_error(s->ctx, LGB_ERR_NOT_READY, "lgb_bvh_build has not been called");
    return LGB_OK;
}

LGB_API lgb_status lgb_trace_closest(lgb_scene* s, const lgb_ray* rays, lgb_hit* hits, uint32_t n, void* stream) {
    lgb_status st = check_trace(s, rays, hits, n);
    if (st != LGB_OK || n == 0) return st;
    if (reinterpret_cast<uintptr_t>(hits) & 15u)
        return set_error(s->ctx, LGB_ERR_INVALID_ARGUMENT, "hit buffer must be 16-byte aligned");
    return launch_trace_closest(s, rays, hits, n, (cudaStream_t)stream, nullptr);
}

LGB_API lgb_status lgb_trace_closest_counted(lgb_scene* s, const lgb_ray* rays, lgb_hit* hits, uint32_t n,
                                             uint64_t* d_counters, void* stream) {
    lgb_status st = check_trace(s, rays, hits, n);
    if (st != LGB_OK || n == 0) return st;
    if (!d_counters || (reinterpret_cast<uintptr_t>(d_counters) & 7u) || (reinterpret_cast<uintptr_t>(hits) & 15u))
        return set_error(s->ctx, LGB_ERR_INVALID_ARGUMENT, "bad counter or hit buffer");
    return launch_trace_closest(s, rays, hits, n, (cudaStream_t)stream, d_counters);
}

LGB_API lgb_status lgb_trace_any(lgb_scene* s, const lgb_ray* rays, uint32_t* bits, uint32_t n, void* stream) {
    lgb_status st = check_trace(s, rays, bits, n);
    if (st != LGB_OK || n == 0) return st;
    return launch_trace_any(s, rays, bits, n, (cudaStream_t)stream);
}

static lgb_status check_trace_host(lgb_scene* s, const void* rays, const void* out, uint32_t n) {
    if (!s) return LGB_ERR_INVALID_ARGUMENT;
    if (n == 0) return LGB_OK;
    if (!rays || !out) return set_error(s->ctx, LGB_ERR_INVALID_ARGUMENT, "null ray or result buffer");
    if (n >= 0x80000000u) return set_error(s->ctx, LGB_ERR_INVALID_ARGUMENT, "at most 2^31 - 1 rays per call");
    if (!s->bvh.nodes) return set_error(s->ctx, LGB_ERR_NOT_READY, "lgb_bvh_build has not been called");
    return LGB_OK;
}

LGB_API lgb_status lgb_trace_closest_host(lgb_scene* s, const lgb_ray* h_rays, lgb_hit* h_hits, uint32_t n,
                                          void* stream) {
    lgb_status st = check_trace_host(s, h_rays, h_hits, n);
    if (st != LGB_OK || n == 0) return st;
    cudaSetDevice(s->ctx->device);
    return trace_host(s, h_rays, h_hits, n, false, (cudaStream_t)stream);
}

LGB_API lgb_status lgb_trace_any_host(lgb_scene* s, const lgb_ray* h_rays, uint32_t* h_occluded_bits, uint32_t n,
                                      void* stream) {
    lgb_status st = check_trace_host(s, h_rays, h_occluded_bits, n);
    if (st != LGB_OK || n == 0) return st;
    cudaSetDevice(s->ctx->device);
    return trace_host(s, h_rays, h_occluded_bits, n, true, (cudaStream_t)stream);
}

LGB_API lgb_status lgb_sync(lgb_scene* s, void* stream) {
    if (!s) return LGB_ERR_INVALID_ARGUMENT;
    LGB_CUDA_TRY(s->ctx, cudaStreamSynchronize((cudaStream_t)stream));
    uint32_t status = 0;
    LGB_CUDA_TRY(s->ctx, cudaMemcpy(&status, s->d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    if (status) {
        uint32_t zero = 0;
        cudaMemcpy(s->d_status, &zero, sizeof(uint32_t), cudaMemcpyHostToDevice);
        char buf[96];
        snprintf(buf, sizeof(buf), "device status word 0x%x (bit 0: traversal stack overflow, bit 1: bad index, bit 2: visit limit)", status);
        return set_error(s->ctx, LGB_ERR_DEVICE_STATUS, buf);
    }
    return LGB_OK;
}

// Projection of Camera.h:109-116 (column-major; it starts from the identity, so [3][3] stays 1).
static void lumen_projection(float fov_deg, uint32_t width, uint32_t height, double P[16]) {
    const float cam_near = 0.01f, cam_far = 1000.0f;
    const float aspect = (float)width / (float)height;
    const float half = fov_deg / 2.0f * (3.14159265358979323846f / 180.0f);
    for (int i = 0; i < 16; i++) P[i] = (i % 5 == 0) ? 1.0 : 0.0;
    P[0] = 1.0f / (aspect * tanf(half));
    P[5] = -1.0f / tanf(half);
    P[10] = cam_far / (cam_near - cam_far);
    P[11] = -1.0;
    P[14] = cam_near * cam_far / (cam_near - cam_far);
}

LGB_API lgb_status lgb_camera_from_matrix(const float camera_to_world[16], float fov_deg, uint32_t width,
                                          uint32_t height, lgb_camera* out) {
    if (!camera_to_world || !out || width == 0 || height == 0 || !(fov_deg > 0.0f && fov_deg < 180.0f))
        return LGB_ERR_INVALID_ARGUMENT;
    for (int i = 0; i < 16; i++)
        if (!std::isfinite(camera_to_world[i])) return LGB_ERR_INVALID_ARGUMENT;
    double P[16], ip[16];
    lumen_projection(fov_deg, width, height, P);
    invert4(P, ip);
    for (int i = 0; i < 16; i++) { out->inv_view[i] = camera_to_world[i]; out->inv_projection[i] = (float)ip[i]; }
    out->width = width;
    out->height = height;
    return LGB_OK;
}

LGB_API lgb_status lgb_camera_lookat(const float pos[3], const float dir[3], float fov_deg, uint32_t width,
                                     uint32_t height, lgb_camera* out) {
    if (!pos || !dir || !out || width == 0 || height == 0 || !(fov_deg > 0.0f && fov_deg < 180.0f))
        return LGB_ERR_INVALID_ARGUMENT;
    double P[16];
    lumen_projection(fov_deg, width, height, P);
    // View: left-handed look-at with up (0, 1, 0) (Camera.h:74).
    double f[3] = {dir[0], dir[1], dir[2]};
    double fl = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    if (!(fl > 0.0)) return LGB_ERR_INVALID_ARGUMENT;
    for (double& x : f) x /= fl;
    double sx = f[2], sy = 0.0, sz = -f[0];  // cross((0,1,0), f)
    double sl = std::sqrt(sx * sx + sy * sy + sz * sz);
    if (!(sl > 0.0)) return LGB_ERR_INVALID_ARGUMENT;  // looking straight up or down
    sx /= sl; sy /= sl; sz /= sl;
    double ux = f[1] * sz - f[2] * sy, uy = f[2] * sx - f[0] * sz, uz = f[0] * sy - f[1] * sx;
    double V[16] = {sx, ux, f[0], 0, sy, uy, f[1], 0, sz, uz, f[2], 0, 0, 0, 0, 1};
    V[12] = -(sx * pos[0] + sy * pos[1] + sz * pos[2]);
    V[13] = -(ux * pos[0] + uy * pos[1] + uz * pos[2]);
    V[14] = -(f[0] * pos[0] + f[1] * pos[1] + f[2] * pos[2]);
    double iv[16], ip[16];
    invert4(V, iv);
    invert4(P, ip);
    for (int i = 0; i < 16; i++) { out->inv_view[i] = (float)iv[i]; out->inv_projection[i] = (float)ip[i]; }
    out->width = width;
    out->height = height;
    return LGB_OK;
}

LGB_API lgb_status lgb_render_path(lgb_scene* s, const lgb_camera* cam, const lgb_path_params* p, uint32_t frame0,
                                   uint32_t spp, float* d_film, void* stream) {
    if (!s) return LGB_ERR_INVALID_ARGUMENT;
    if (!cam || !p || !d_film || cam->width == 0 || cam->height == 0)
        return set_error(s->ctx, LGB_ERR_INVALID_ARGUMENT, "null camera, params or film");
    if (reinterpret_cast<uintptr_t>(d_film) & 15u) return set_error(s->ctx, LGB_ERR_INVALID_ARGUMENT, "film must be 16-byte aligned");
    if (!s->bvh.nodes) return set_error(s->ctx, LGB_ERR_NOT_READY, "lgb_bvh_build has not been called");
    if (p->num_lights < 0 || (uint32_t)p->num_lights > s->num_lights)
        return set_error(s->ctx, LGB_ERR_INVALID_ARGUMENT, "num_lights exceeds the scene's light count");
    if (p->num_lights > 0 && p->light_triangle_count <= 0)
        return set_error(s->ctx, LGB_ERR_INVALID_ARGUMENT, "light_triangle_count must be positive");
    if (p->dir_light_idx != 0xFFFFFFFFu)
        return set_error(s->ctx, LGB_ERR_UNSUPPORTED, "atmosphere shading for directional lights is not supported");
    if (spp == 0) return LGB_OK;
    cudaSetDevice(s->ctx->device);
    return render_path(s, cam, p, frame0, spp, d_film, (cudaStream_t)stream);
}

}  // extern "C"
