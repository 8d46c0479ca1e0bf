// Oracle (test infrastructure only): CPU restatement of Lumen's path-tracing core.
//
// This library is the checker for the CUDA path. Only the test suite, the smoke check and the
// CPU-baseline leg of the benchmark load it; the product never links or calls it.
//
// What it restates, with the reference file each part follows:
//   * scene data layouts              src/shaders/commons.h:194-234 (Vertex, Light, Material)
//   * closest/any-hit ray queries      src/shaders/integrators/path/path.rgen:18-20,48 and
//                                     src/shaders/integrators/pt_commons.glsl:20-23,32 (the queries);
//                                     the intersection itself lives in the closed Vulkan driver, so the
//                                     contract is ours: watertight FP32 triangle test (Woop, Benthin and
//                                     Wald, JCGT 2013) with the lowest primitive id winning ties in t.
//   * hit attribute reconstruction    src/shaders/ray.rchit:24-84
//   * shading and sampling            src/shaders/utils.glsl, commons.glsl, bsdf_commons.glsl, bsdf/*.glsl
//   * the path integrator             src/shaders/integrators/path/path.rgen:22-113 and pt_commons.glsl:3-48
//
// Parity status: Lumen has no tests, golden vectors or fixtures for this path and cannot run here (Vulkan
// ray tracing), so this oracle is pinned only by its own known-answer tests; see the test suite.
#pragma once
#include <cstdint>

extern "C" {

// Material, 104 bytes, scalar layout of src/shaders/commons.h:212-234.
struct orc_material {
    float albedo[3];
    float ior;
    float emissive_factor[3];
    uint32_t bsdf_type;
    uint32_t bsdf_props;
    float k[3];
    int32_t texture_id;
    float roughness, diffuse_trans, spec_trans, metallic, specular_tint, sheen_tint, clearcoat,
        clearcoat_gloss, sheen, subsurface, flatness, anisotropy;
    uint32_t thin;
};

// Light, 128 bytes, src/shaders/commons.h:200-210.
struct orc_light {
    float world_matrix[16];
    float pos[3];
    uint32_t prim_mesh_idx;
    float to[3];
    uint32_t num_triangles;
    float L[3];
    uint32_t light_flags;
    float world_center[3];
    float world_radius;
};

// Per-mesh record (the fields of PrimMeshInfo, src/shaders/commons.h:333-340, that the path reads).
struct orc_mesh {
    uint32_t index_offset;   // first index of the mesh in the index array
    uint32_t vertex_offset;  // added to every index of the mesh
    uint32_t material_index;
    uint32_t tri_count;
};

struct orc_texture {
    uint32_t width, height;
    const float* rgba;  // width*height*4 floats, linear
};

struct orc_scene_desc {
    const float* positions;  // 3 per vertex
    const float* normals;    // 3 per vertex
    const float* uvs;        // 2 per vertex
    uint32_t num_vertices;
    const uint32_t* indices;
    uint32_t num_indices;
    const orc_mesh* meshes;
    uint32_t num_meshes;
    const orc_material* materials;
    uint32_t num_materials;
    const orc_light* lights;
    uint32_t num_lights;
    const orc_texture* textures;
    uint32_t num_textures;
};

// PCPath, src/shaders/integrators/path/path_commons.h:3-15 (the fields the path reads).
struct orc_path_params {
    float sky_col[3];
    uint32_t frame_num;
    uint32_t size_x, size_y;
    int32_t num_lights;
    int32_t max_depth;
    int32_t light_triangle_count;
    uint32_t dir_light_idx;
    uint32_t direct_lighting;
};

struct orc_ray { float o[3]; float tmin; float d[3]; float tmax; };
struct orc_hit { uint32_t prim; float t, u, v; };

// ---- triangle BVH (binned SAH, binary) over flattened triangles ----
// tri_verts: 9 floats per triangle (v0, v1, v2 in world space), n triangles.
void* orc_bvh_build(const float* tri_verts, uint32_t n);
void orc_bvh_free(void* bvh);
uint32_t orc_bvh_num_nodes(void* bvh);
void orc_trace_closest(void* bvh, const orc_ray* rays, orc_hit* hits, uint32_t n, int nthreads);
void orc_trace_any(void* bvh, const orc_ray* rays, uint8_t* occluded, uint32_t n, int nthreads);
// Exhaustive test of every triangle (small meshes only).
void orc_brute_closest(const float* tri_verts, uint32_t ntri, const orc_ray* rays, orc_hit* hits, uint32_t n);
void orc_brute_any(const float* tri_verts, uint32_t ntri, const orc_ray* rays, uint8_t* occluded, uint32_t n);
// Single watertight ray/triangle test; returns 1 on hit and writes t, u, v.
int orc_intersect_tri(const float* ray8, const float* v9, float* tuv);

// ---- camera (src/framework Camera.h:67-123, Integrator.cpp:60-72) ----
// Writes inv_view and inv_projection (column-major 4x4) for a camera at pos looking along dir.
void orc_camera_matrices(const float pos[3], const float dir[3], float fov_deg, uint32_t width, uint32_t height,
                         float inv_view[16], float inv_proj[16]);

// ---- the path integrator ----
// Renders one sample (frame params->frame_num) for each listed pixel and writes its radiance (3 floats) to
// out_rgb and a flag (1 = the sample is NaN and path.rgen:102-104 drops it) to out_nan.
// fp64 != 0 evaluates shading in double precision (intersection stays FP32).
void* orc_scene_create(const orc_scene_desc* desc);
void orc_scene_free(void* scene);
void orc_render_samples(void* scene, const float inv_view[16], const float inv_proj[16],
                        const orc_path_params* params, const uint32_t* pixels, uint32_t n_pixels,
                        float* out_rgb, uint8_t* out_nan, int fp64, int nthreads);
// Progressive film exactly as path.rgen:102-112 writes it: frames [frame0, frame0+spp) into film (RGBA32F).
void orc_render_mean_f64(void* h, const float inv_view[16], const float inv_proj[16], const orc_path_params* params,
                         uint32_t frame0, uint32_t spp, double* out, int nthreads);
void orc_render_film(void* scene, const float inv_view[16], const float inv_proj[16],
                     const orc_path_params* params, uint32_t frame0, uint32_t spp, float* film, int fp64,
                     int nthreads);
// Mean image of the detached differentiable estimator (sampling from the scene's materials, values from
// the parameter arrays; see path.cpp). Used for finite-difference checks of the adjoint kernels.
void orc_render_diff(void* scene, const float inv_view[16], const float inv_proj[16], const orc_path_params* params,
                     int tex_id, const float* texels, const float* rough, const float* emis, uint32_t frame0,
                     uint32_t spp, double* film_rgb, int fp64, int nthreads);
// ---- VCM (vcm_commons.glsl, vcm_light.rgen, vcm_eye.rgen, VCM.cpp) ----
struct orc_vcm_params {
    float sky_col[3];
    int32_t max_depth;
    int32_t num_lights;
    int32_t light_triangle_count;
    float radius;             // merge radius of this iteration
    int32_t use_vm, use_vc;
    uint32_t light_seed, eye_seed;  // the reference's host rand() values
    uint32_t frame_num;
    float scene_min[3], scene_max[3];
    uint32_t flags;  // bit 0: accumulate every connection and merge instead of keeping the last (`res =`)
    float spot_angle;  // spot cone half-angle in degrees (falloff from 25/30 of it); 0: fixed 30 and 25 degrees
};
// VCMVertex, vcm_commons.h:89-104 (104 bytes).
struct orc_vcm_vertex {
    float wi[3], wo[3], n_s[3], pos[3], uv[2], throughput[3];
    uint32_t material_idx, path_len;
    float area, d_vcm, d_vc, d_vm;
    uint32_t side, coords;
};
void orc_vcm_grid_res(const float scene_min[3], const float scene_max[3], float radius, int32_t res[3]);
void orc_vcm_grid(const float* pos4, uint32_t n, const float scene_min[3], const float scene_max[3], float radius,
                  uint32_t screen_size, uint32_t* count, uint32_t* rep);
void orc_vcm_iteration(void* scene, const float inv_view[16], const float inv_proj[16], const float view[16],
                       const float proj[16], uint32_t width, uint32_t height, const orc_vcm_params* p,
                       orc_vcm_vertex* verts, uint32_t* counts, float* splat, uint32_t* grid_count, uint32_t* grid_rep,
                       float* film, int nthreads);
void orc_vcm_render_f64(void* scene, const float inv_view[16], const float inv_proj[16], const float view[16],
                        const float proj[16], uint32_t width, uint32_t height, const orc_vcm_params* params,
                        uint32_t n_iters, double* film, int nthreads);
// SPPM (SPPM.cpp:78-184): one frame. vp (W*H*32 floats), photons (W*H*max_depth*16 floats), grid_count and
// grid_rep (10*W*H) and film (W*H*4, row-major) persist across frames; vp must be zero before frame 0. The
// visible-point and photon layouts are the library's (8 and 4 float4, integer fields stored as their bits).
struct orc_sppm_params {
    float sky_col[3];
    int32_t max_depth;
    int32_t num_lights;
    int32_t light_triangle_count;
    float base_radius;
    uint32_t seed;       // RNG frame value = frame_num ^ seed
    uint32_t frame_num;
    float spot_angle;    // degrees, 0 = the fixed 30 / 25 degree cone
};
void orc_sppm_iteration(void* scene, const float inv_view[16], const float inv_proj[16], uint32_t width,
                        uint32_t height, const orc_sppm_params* p, float* vp, float* photons, uint32_t* grid_count,
                        uint32_t* grid_rep, float* film, int nthreads);
// ReSTIR DI (ReSTIR.cpp:74-151): one frame. gbuf, passthrough, temporal_res and spatial_res (W*H*12 floats each)
// and film (W*H*4, row-major) persist across frames; prev_view / prev_proj are the previous camera's forward
// matrices (column-major). Layouts are the library's.
struct orc_restir_params {
    int32_t num_lights;
    int32_t light_triangle_count;
    uint32_t seed;                 // RNG frame value = frame_num ^ seed
    uint32_t frame_num;
    uint32_t do_spatiotemporal;
    uint32_t enable_accumulation;
    float spot_angle;
    uint32_t flags;  // bit 0: the spatial pass counts the pixel's reservoir with its m (LGB_RESTIR_SPATIAL_COUNT_FIX)
};
void orc_restir_di_iteration(void* scene, const float inv_view[16], const float inv_proj[16], const float prev_view[16],
                             const float prev_proj[16], uint32_t width, uint32_t height, const orc_restir_params* p,
                             float* gbuf, float* passthrough, float* temporal_res, float* spatial_res, float* film,
                             int nthreads);
// BDPT (BDPT.cpp:55-88, bdpt.rgen, bdpt_commons.glsl): one frame. Light and camera subpaths per pixel, every
// connection strategy with its MIS weight, the light-tracing splats of the frame and the progressive film
// (W*H*4, row-major). splat (W*H*3, row-major) receives the frame's splats (diagnostic). Area and spot lights.
struct orc_bdpt_params {
    int32_t max_depth;             // path_length
    int32_t num_lights;
    int32_t light_triangle_count;
    uint32_t seed;                 // RNG frame value = frame_num ^ seed
    uint32_t frame_num;
    float spot_angle;              // degrees, 0 = the fixed 30 / 25 degree cone
    // Consistency checks of the restatement (0 = the integrator as the reference runs it). Bit 0: only the
    // strategies with path length s + t - 1 == check_len (and s == check_s when check_s >= 0) contribute; a
    // skipped s = 1 strategy still draws its four random numbers, so the others see the same ones. Bit 1: every
    // MIS weight is 1 (each strategy's own unweighted estimate).
    uint32_t check_flags;
    int32_t check_len, check_s;
};
void orc_bdpt_iteration(void* scene, const float inv_view[16], const float inv_proj[16], const float view[16],
                        const float proj[16], uint32_t width, uint32_t height, const orc_bdpt_params* p, float* film,
                        float* splat, int nthreads);
// PCG4D (utils.glsl:121-133) applied to n state vectors; for known-answer tests.
void orc_pcg4d(const uint32_t* in, uint32_t* out, uint32_t n);
// offset_ray (utils.glsl:73-84) applied to n (p, n) pairs.
void orc_offset_ray(const float* p, const float* nrm, float* out, uint32_t n);
}
