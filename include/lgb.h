/* lgb.h -- C ABI of the GB300-native ray-tracing core (BVH build, traversal, MIS path tracer).
 *
 * This header is the drop-in boundary. Lumen has no FFI of its own: its path is one C++ class per
 * integrator (src/RayTracer/Integrator.h:14-33) that records Vulkan ray-tracing passes, with the BVH built
 * and traversed inside the driver. Each entry point below replaces one piece of that path; the comment on
 * each names the reference code it stands in for.
 *
 * Conventions
 *   - Plain C types and pointers only; no CUDA or C++ types in signatures. A `stream` argument is a
 *     cudaStream_t passed as void* (NULL = the legacy default stream).
 *   - Pointers named d_* are device pointers owned by the caller. Every other pointer is a host pointer
 *     that the library reads during the call only.
 *   - Every entry point returns an lgb_status; on failure lgb_last_error() describes it. No exception or
 *     longjmp crosses this boundary.
 *   - A context is externally synchronised: one host thread at a time per context. Work is stream-ordered;
 *     the queries of one scene share a device work counter, so issue them on one stream at a time.
 */
#ifndef LGB_H
#define LGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define LGB_API __attribute__((visibility("default")))
#else
#define LGB_API
#endif

typedef int32_t lgb_status;
#define LGB_OK 0
#define LGB_ERR_INVALID_ARGUMENT 1 /* bad pointer, size or scene content */
#define LGB_ERR_CUDA 2             /* a CUDA runtime call failed */
#define LGB_ERR_OUT_OF_MEMORY 3
#define LGB_ERR_NOT_READY 4        /* e.g. a trace before lgb_bvh_build */
#define LGB_ERR_DEVICE_STATUS 5    /* a kernel reported a fault through the device status word */
#define LGB_ERR_UNSUPPORTED 6      /* scene feature outside the supported subset */

typedef struct lgb_ctx lgb_ctx;
typedef struct lgb_scene lgb_scene;

/* Ray, 32 bytes: origin, tmin, direction, tmax (the arguments of traceRayEXT, path.rgen:48). */
typedef struct lgb_ray {
    float ox, oy, oz, tmin;
    float dx, dy, dz, tmax;
} lgb_ray;

/* Closest hit, 16 bytes. prim is the global triangle id (LGB_NO_HIT on a miss); u, v are the Vulkan
 * barycentrics (hitAttributeEXT, ray.rchit:13,57): u weights vertex 1, v weights vertex 2. */
typedef struct lgb_hit {
    uint32_t prim;
    float t, u, v;
} lgb_hit;
#define LGB_NO_HIT 0xFFFFFFFFu

/* Material, 104 bytes, the scalar layout of src/shaders/commons.h:212-234. */
typedef struct lgb_material {
    float albedo[3];
    float ior;
    float emissive_factor[3];
    uint32_t bsdf_type;  /* LGB_BSDF_* (commons.h:13-18) */
    uint32_t bsdf_props; /* LGB_FLAG_* (commons.h:22-26) */
    float k[3];
    int32_t texture_id; /* -1 = none */
    float roughness, diffuse_trans, spec_trans, metallic, specular_tint, sheen_tint, clearcoat, clearcoat_gloss,
        sheen, subsurface, flatness, anisotropy;
    uint32_t thin;
} lgb_material;

#define LGB_BSDF_DIFFUSE (1u << 0)
#define LGB_BSDF_MIRROR (1u << 1)
#define LGB_BSDF_GLASS (1u << 2)
#define LGB_BSDF_DIELECTRIC (1u << 3)
#define LGB_BSDF_CONDUCTOR (1u << 4)
#define LGB_BSDF_PRINCIPLED (1u << 5)
#define LGB_FLAG_DIFFUSE (1u << 0)
#define LGB_FLAG_SPECULAR (1u << 1)
#define LGB_FLAG_GLOSSY (1u << 2)
#define LGB_FLAG_REFLECTION (1u << 3)
#define LGB_FLAG_TRANSMISSION (1u << 4)

/* Light, 128 bytes, src/shaders/commons.h:200-210. light_flags: bits 0-2 type (LGB_LIGHT_*),
 * bit 4 finite, bit 5 delta (LumenScene.cpp:89-91,500-509). world_matrix must be the identity: Lumen's
 * loaders never set anything else (LumenScene.cpp:328). */
typedef struct lgb_light {
    float world_matrix[16];
    float pos[3];
    uint32_t prim_mesh_idx;
    float to[3];
    uint32_t num_triangles;
    float L[3];
    uint32_t light_flags;
    float world_center[3];
    float world_radius;
} lgb_light;
#define LGB_LIGHT_SPOT 1u
#define LGB_LIGHT_AREA 2u
#define LGB_LIGHT_DIRECTIONAL 3u

/* One mesh (the PrimMeshInfo fields of commons.h:333-340 that the path reads, plus its triangle count). */
typedef struct lgb_mesh {
    uint32_t index_offset;  /* first index of the mesh in indices[] (a multiple of 3) */
    uint32_t vertex_offset; /* added to every index of the mesh */
    uint32_t material_index;
    uint32_t tri_count;
} lgb_mesh;

/* Linear FP32 RGBA texture, sampled bilinearly with REPEAT at LOD 0. */
typedef struct lgb_texture {
    uint32_t width, height;
    const float* rgba; /* host, width*height*4 floats, row-major from v = 0 */
} lgb_texture;

/* Host scene arrays (LumenScene::load_scene's output, LumenScene.cpp:52-229). The library copies them;
 * the caller keeps ownership. Global triangle g of mesh m is local triangle g - first_tri(m), where meshes
 * are numbered in order and first_tri is the running sum of tri_count. */
typedef struct lgb_scene_desc {
    const float* positions; /* 3 floats per vertex */
    const float* normals;   /* 3 floats per vertex */
    const float* uvs;       /* 2 floats per vertex */
    uint32_t num_vertices;
    const uint32_t* indices;
    uint32_t num_indices;
    const lgb_mesh* meshes;
    uint32_t num_meshes;
    const lgb_material* materials;
    uint32_t num_materials;
    const lgb_light* lights;
    uint32_t num_lights;
    const lgb_texture* textures;
    uint32_t num_textures;
} lgb_scene_desc;

typedef struct lgb_build_opts {
    uint32_t leaf_max;        /* triangles per 8-wide leaf slot, 1..3 (0 = by scene size: 1 from 2^19 triangles,
                                 2 from 2^15, else 3) */
    uint32_t treelet_rounds;  /* SAH treelet restructuring passes (0 = default 3, 0xFFFFFFFF = none) */
    uint32_t reserved[6];
} lgb_build_opts;

typedef struct lgb_build_stats {
    float build_ms;           /* device time of the whole build */
    uint32_t num_tris;
    uint32_t num_nodes;       /* 8-wide nodes */
    uint32_t max_depth;       /* deepest 8-wide level (root = 1) */
    uint64_t node_bytes;
    uint64_t tri_bytes;
    float sah_cost;           /* SAH cost of the 8-wide tree (node cost 1, triangle cost 1) */
    uint32_t reserved[5];
} lgb_build_stats;

/* Camera for the path integrator: the two matrices path.rgen:36-38 and commons.glsl:30-33 read
 * (column-major, as glm stores them) and the launch size. */
typedef struct lgb_camera {
    float inv_view[16];
    float inv_projection[16];
    uint32_t width, height;
} lgb_camera;

/* PCPath (src/shaders/integrators/path/path_commons.h:3-15), minus the per-frame fields. */
typedef struct lgb_path_params {
    float sky_col[3];
    int32_t max_depth;             /* path_length (SceneConfig.h:16, default 6) */
    int32_t num_lights;
    int32_t light_triangle_count;  /* LumenScene::total_light_triangle_cnt */
    uint32_t dir_light_idx;        /* 0xFFFFFFFF = none; the atmosphere model is not supported */
    uint32_t direct_lighting;      /* 1 = default (Path.h:18) */
    uint32_t film_mode;            /* 0 = progressive mean as path.rgen:106-112; 1 = write each frame's raw sample */
    uint32_t reserved[3];
} lgb_path_params;

/* ---- context (stands in for the Vulkan device/context, VulkanBase.cpp) ----
 * tuning_cache_path: a text file in which lgb_batch_tune keeps its choices, keyed by the device (name, SM count,
 * compute capability), the library's ABI version and the shape of the tuned batch, so that later processes on
 * the same kind of device skip the timing runs; null = no cache. The file is created when missing; a cache that
 * cannot be read or written is ignored (tuning then times the candidates as without one). Lumen keeps its
 * compiled pipelines in a cache keyed by pass name and shader macros (RenderGraph.h:241-284); this is the
 * counterpart for the choices of the autotuner. */
LGB_API lgb_status lgb_create(lgb_ctx** out, int device, const char* tuning_cache_path);
LGB_API void lgb_destroy(lgb_ctx* ctx);
LGB_API const char* lgb_last_error(const lgb_ctx* ctx);
LGB_API uint32_t lgb_abi_version(void);

/* ---- scene upload (LumenScene::load_scene's GPU buffers, LumenScene.cpp:146-190) ---- */
LGB_API lgb_status lgb_scene_create(lgb_ctx* ctx, const lgb_scene_desc* desc, lgb_scene** out);
LGB_API void lgb_scene_destroy(lgb_scene* scene);

/* ---- acceleration structure (Integrator::create_accel, Integrator.cpp:137-160; vk::build_blas/build_tlas,
 *      AccelerationStructure.cpp:171-315). One 8-wide BVH over all meshes' triangles. ---- */
LGB_API lgb_status lgb_bvh_build(lgb_scene* scene, const lgb_build_opts* opts, lgb_build_stats* stats);

/* ---- ray queries (traceRayEXT: closest, path.rgen:48 / pt_commons.glsl:32; any-hit shadow,
 *      pt_commons.glsl:20-23 with ray.rahit:18-21 and ray_shadow.rmiss:12). ----
 * Closest: the triangle with the smallest watertight t in [tmin, tmax]; equal t goes to the lowest prim.
 * Any: bit i of d_occluded_bits[i / 32] is set iff some triangle is hit in [tmin, tmax]. */
LGB_API lgb_status lgb_trace_closest(lgb_scene* scene, const lgb_ray* d_rays, lgb_hit* d_hits, uint32_t n,
                                     void* stream);
LGB_API lgb_status lgb_trace_any(lgb_scene* scene, const lgb_ray* d_rays, uint32_t* d_occluded_bits, uint32_t n,
                                 void* stream);
/* Node-visit budget of one ray in this scene's lgb_trace_closest / lgb_trace_any queries (device, host-buffer and
 * counted forms). 0 restores the default, 2^22 visits, which no well-formed tree reaches. A ray that runs out of
 * budget ends with what it has found so far and sets bit 2 of the scene's device status word; the next lgb_sync
 * returns LGB_ERR_DEVICE_STATUS and clears the word. No counterpart in Lumen (the driver bounds its own
 * traversal): it lets a caller exercise that error path on a sound tree, with nothing faulting or hanging. */
LGB_API lgb_status lgb_scene_set_visit_limit(lgb_scene* scene, uint32_t max_visits);
/* Same query as lgb_trace_closest, also adding the 8-wide nodes and triangles each ray fetched into
 * d_counters[0] and d_counters[1] (device uint64). For bytes-per-ray accounting. */
LGB_API lgb_status lgb_trace_closest_counted(lgb_scene* scene, const lgb_ray* d_rays, lgb_hit* d_hits, uint32_t n,
                                             uint64_t* d_counters, void* stream);
/* The same two queries on HOST buffers (a caller whose rays live in host memory). Pinned buffers (cudaHostAlloc
 * or cudaHostRegister, 16-byte aligned) are read and written by the traversal kernel itself over the CPU-GPU
 * link, each ray and hit crossing it once; pageable buffers are copied in and out in up to eight chunks that
 * overlap the traversal. Stream-ordered: the results are in h_hits / h_occluded_bits once `stream` has
 * finished. */
LGB_API lgb_status lgb_trace_closest_host(lgb_scene* scene, const lgb_ray* h_rays, lgb_hit* h_hits, uint32_t n,
                                          void* stream);
LGB_API lgb_status lgb_trace_any_host(lgb_scene* scene, const lgb_ray* h_rays, uint32_t* h_occluded_bits, uint32_t n,
                                      void* stream);

/* ---- camera helper (Camera.h:67-123, Integrator.cpp:60-72): fills out->inv_view/inv_projection ---- */
LGB_API lgb_status lgb_camera_lookat(const float pos[3], const float dir[3], float fov_deg, uint32_t width,
                                     uint32_t height, lgb_camera* out);

/* The same camera from a camera-to-world matrix (column-major, as glm stores Lumen's Camera::camera after
 * Camera::update_view_matrix, Camera.h:27-39): inv_view = camera_to_world, the projection as above. For cameras
 * given by a matrix rather than a position and direction (Mitsuba sensors, LumenScene.cpp:64-68). */
LGB_API lgb_status lgb_camera_from_matrix(const float camera_to_world[16], float fov_deg, uint32_t width,
                                          uint32_t height, lgb_camera* out);

/* ---- the Path integrator (Path::render, Path.cpp:27-59, i.e. path.rgen for frames frame0..frame0+spp-1).
 *      d_film is RGBA32F width*height (float4 per pixel), updated in place. Scenes of 2^15 triangles or more
 *      trace their ray queues with the incoherent traversal variant (see lgb_batch_opts.traversal). ---- */
LGB_API lgb_status lgb_render_path(lgb_scene* scene, const lgb_camera* camera, const lgb_path_params* params,
                                   uint32_t frame0, uint32_t spp, float* d_film, void* stream);

/* The Path integrator without any device allocation. No counterpart in Lumen: it exists for callers that
 * cannot let a library call cudaMalloc while they render (a host that budgets all device memory up front,
 * or one that cannot afford the device-wide synchronisation of cudaFree in its frame loop). Same arguments
 * and results as lgb_render_path; its work arena is a fixed 6 MiB device array that every GPU loading the
 * library holds until exit, so images are limited to 16384 pixels (e.g. 128 x 128) and larger ones are
 * rejected with LGB_ERR_INVALID_ARGUMENT. All calls share that array: calls that overlap on the GPU race,
 * so order them on one stream. The first call on a device looks the array up; make it before any stream
 * capture. The address is looked up once per device for the life of the process: after cudaDeviceReset (or
 * anything else that destroys and recreates the device's primary context) it is stale, so do not call this
 * entry point again in that process. */
LGB_API lgb_status lgb_render_path_noalloc(lgb_scene* scene, const lgb_camera* camera, const lgb_path_params* params,
                                           uint32_t frame0, uint32_t spp, float* d_film, void* stream);

/* ---- differentiable rendering (no counterpart in Lumen) ----
 * The estimator of lgb_render_path with every sampling decision detached from the parameters: directions,
 * pdfs, MIS weights and Russian roulette use the scene's materials, while BSDF values and emission use the
 * parameter buffers below. Parameters: the texels of one texture (albedo multipliers of the materials that use
 * it), roughness per material (rough GGX conductors), emission per material (RGB). Null pointers keep the
 * scene's values. With LGB_DIFF_SAMPLE_PARAMS the sampling decisions use the parameter values instead of the
 * scene's (still detached: the gradient is that of f / p with p held fixed, which is exact when p follows the
 * current values); an optimiser wants this, since sampling a lobe far from the one evaluated is noisy, while a
 * finite-difference check with common random numbers wants it off.
 * The image is the plain mean of the spp samples of each pixel (frames frame0..frame0+spp-1, seeded as
 * lgb_render_path seeds them); a sample whose radiance is not finite counts as zero and has no gradient
 * (Lumen's film drops it). Path depth is limited to 16. */
#define LGB_DIFF_SAMPLE_PARAMS 1u /* sample with the parameter values too (still detached from them) */

typedef struct lgb_diff_params {
    int32_t texture_id;      /* texture whose texels are parameters */
    uint32_t flags;          /* LGB_DIFF_* */
    const float* texels;     /* device, width*height RGBA of that texture (alpha ignored); null = no texel params */
    const float* roughness;  /* device, one per material */
    const float* emission;   /* device, three per material */
} lgb_diff_params;

typedef struct lgb_diff_grads {  /* device gradient accumulators, same layouts; the library adds into them */
    float* texels;
    float* roughness;
    float* emission;
} lgb_diff_grads;

/* Primal image of the differentiable estimator into d_film (RGBA32F, width*height). If d_samples is not null
 * it receives the radiance of every sample (RGBA32F, [spp][width*height], 16 bytes each), which
 * lgb_adjoint_path can replay from; otherwise the samples go to a scene-owned buffer. */
LGB_API lgb_status lgb_diff_render(lgb_scene* scene, const lgb_camera* camera, const lgb_path_params* params,
                                   const lgb_diff_params* diff, uint32_t frame0, uint32_t spp, float* d_film,
                                   float* d_samples, void* stream);
/* Adjoint path replay: adds d loss / d parameter into grads, given d loss / d image (RGBA32F per pixel, alpha
 * ignored) for the image lgb_diff_render produces with the same arguments. Each path is re-traced from its
 * counter-based RNG stream; no path vertex is stored. With d_primal_samples (the d_samples that
 * lgb_diff_render wrote for the same arguments and parameter values) every path is traced once more;
 * with null it is traced twice (primal, then replay). Gradients are accumulated with float atomics, so their
 * low bits depend on the order of the additions. */
LGB_API lgb_status lgb_adjoint_path(lgb_scene* scene, const lgb_camera* camera, const lgb_path_params* params,
                                    const lgb_diff_params* diff, uint32_t frame0, uint32_t spp,
                                    const float* d_dloss_dimage, const float* d_primal_samples, lgb_diff_grads* grads,
                                    void* stream);

/* Waits for `stream` and reports any fault a kernel recorded in the scene's device status word. */
LGB_API lgb_status lgb_sync(lgb_scene* scene, void* stream);

/* ---- VCM: vertex connection and merging (src/RayTracer/VCM.cpp, src/shaders/integrators/vcm*) ---- */
#define LGB_VCM_ACCUMULATE 1u /* sum every light-vertex connection and merge (the reference keeps the last) */

typedef struct lgb_vcm_params {
    float sky_col[3];
    int32_t max_depth;             /* path_length */
    int32_t num_lights;
    int32_t light_triangle_count;  /* LumenScene::total_light_triangle_cnt: a non-area light counts as one */
    uint32_t dir_light_idx;        /* must be 0xFFFFFFFF */
    float radius;                  /* merge radius of this iteration, see lgb_vcm_radius */
    float scene_min[3];            /* photon grid bounds: the scene's bounding box (LumenScene::m_dimensions) */
    float scene_max[3];
    int32_t use_vm, use_vc;        /* vertex merging / vertex connection (VCM.cpp uses VC always) */
    uint32_t light_seed, eye_seed; /* per-iteration seeds; the reference draws them with host rand() */
    uint32_t frame_num;            /* progressive film frame: 0 overwrites, k mixes with weight 1/(k+1) */
    uint32_t flags;                /* LGB_VCM_* */
    float spot_angle;              /* spot cone half-angle in degrees, (0, 90); the falloff starts at 25/30 of it.
                                      0 keeps the reference's fixed 30 and 25 degrees (commons.glsl:264-265) */
    uint32_t reserved;
} lgb_vcm_params;

/* Merge radius of iteration `iteration` (VCM.cpp:137-138): scene_radius * radius_factor / 100 shrunk by
 * (iteration + 1)^(0.5 (1 - alpha)); the reference fixes alpha = 2/3. */
LGB_API float lgb_vcm_radius(float scene_radius, float radius_factor, uint32_t iteration, float alpha);

/* One VCM iteration into d_film (RGBA32F, width*height): light subpaths with camera splats, the photon table,
 * eye subpaths. Light vertices, per-path counts and the splat image live in the scene between iterations, as
 * the reference's buffers do (reallocated and zeroed when the image size or max_depth changes). Area and spot
 * lights only. */
LGB_API lgb_status lgb_vcm_iteration(lgb_scene* scene, const lgb_camera* camera, const lgb_vcm_params* params,
                                     float* d_film, void* stream);

/* The photon table alone (vcm_commons.glsl:455-469, made deterministic): for n positions (float4, w < 0 marks
 * an unused entry) the slot hash(cell(p)) mod 10 * screen_size over the grid of (scene_min, scene_max, radius)
 * (VCM.cpp:144-147); writes, per slot, the number of positions and the index of the last one. Built by radix
 * sort and scan; waits for `stream`. */
LGB_API lgb_status lgb_vcm_grid(lgb_ctx* ctx, const float* d_pos4, uint32_t n, const float scene_min[3],
                                const float scene_max[3], float radius, uint32_t screen_size, uint32_t* d_count,
                                uint32_t* d_rep, void* stream);

/* The VCM state a scene keeps between iterations, as device pointers owned by the scene (valid until the next
 * lgb_vcm_iteration with another image size or max_depth, or lgb_scene_destroy). Lumen keeps the same data in
 * its "VCM Light Vertices", "Light Path Count" and "Photon Buffer" buffers (VCM.cpp:11-31). For inspection
 * and tests: read them after the iteration's stream has finished. */
typedef struct lgb_vcm_state {
    const float* vertices;          /* 6 float4 per light vertex, vertex k of light subpath i at i * per_path + k;
                                       the first float4 holds the position */
    const uint32_t* path_counts;    /* stored vertices per light subpath (screen entries) */
    const uint32_t* table_count;    /* photons per hash slot (table_size entries) */
    const uint32_t* table_rep;      /* per slot, the index of the last vertex in vertex order */
    uint32_t screen, per_path, table_size;
    int32_t grid_res[3];            /* cells per axis of the last iteration's grid */
    float radius;                   /* merge radius of the last iteration */
    float scene_min[3], scene_max[3];
    uint32_t reserved;
} lgb_vcm_state;
LGB_API lgb_status lgb_vcm_state_get(const lgb_scene* scene, lgb_vcm_state* out);

/* The forward matrices of a camera (view and projection, column-major), inverted in double from the camera's
 * inverse matrices and rounded to float: what lgb_vcm_iteration projects light vertices with. */
LGB_API lgb_status lgb_camera_forward(const lgb_camera* camera, float view[16], float projection[16]);

/* ---- SPPM: stochastic progressive photon mapping (src/RayTracer/SPPM.cpp:78-184,
 *      src/shaders/integrators/sppm/{sppm_eye.rgen, sppm_light.rgen, gather.comp, composite.comp, min/max/
 *      calc_bounds.comp}) on the same traversal and the same sort-and-scan photon table as VCM. ---- */
typedef struct lgb_sppm_params {
    float sky_col[3];
    int32_t max_depth;             /* path_length */
    int32_t num_lights;
    int32_t light_triangle_count;  /* LumenScene::total_light_triangle_cnt */
    uint32_t dir_light_idx;        /* must be 0xFFFFFFFF */
    float base_radius;             /* SPPMConfig::base_radius (default 0.03): every pixel's radius at frame 0 */
    uint32_t seed;                 /* the RNG's frame value is frame_num ^ seed (the reference draws seed with rand()) */
    uint32_t frame_num;            /* 0 restarts (per-pixel state cleared); k mixes the film with weight 1/(k+1) */
    float spot_angle;              /* spot cone half-angle as lgb_vcm_params; 0 = Lumen's fixed 30 / 25 degrees */
    uint32_t reserved[5];
} lgb_sppm_params;

/* One SPPM frame into d_film (RGBA32F, width*height): eye pass (visible points at the first diffuse hit, direct
 * light by the path tracer's light sampling), grid bounds from the visible points, light pass (photons from the
 * second bounce on), photon table, gather and progressive radius / flux update, film. The per-pixel state and the
 * photons live in the scene between frames. Area and spot lights only. */
LGB_API lgb_status lgb_sppm_iteration(lgb_scene* scene, const lgb_camera* camera, const lgb_sppm_params* params,
                                      float* d_film, void* stream);

/* ---- BDPT: bidirectional path tracing (src/RayTracer/BDPT.cpp:55-88, src/shaders/integrators/bdpt/bdpt.rgen,
 *      src/shaders/integrators/bdpt_commons.glsl) on the library's traversal, BSDFs and light sampling. ---- */
typedef struct lgb_bdpt_params {
    float sky_col[3];              /* PCBDPT::sky_col: set by the reference, never read by bdpt.rgen; kept for the layout */
    int32_t max_depth;             /* path_length: subpaths of up to max_depth + 1 vertices, strategies s + t <= max_depth + 1 */
    int32_t num_lights;
    int32_t light_triangle_count;  /* LumenScene::total_light_triangle_cnt */
    uint32_t dir_light_idx;        /* must be 0xFFFFFFFF */
    uint32_t seed;                 /* the RNG's frame value is frame_num ^ seed (the reference draws seed with rand()) */
    uint32_t frame_num;            /* 0 writes the frame; k mixes the film with weight 1/(k+1) */
    float spot_angle;              /* spot cone half-angle as lgb_vcm_params; 0 = Lumen's fixed 30 / 25 degrees */
    uint32_t reserved[6];
} lgb_bdpt_params;

/* One BDPT frame into d_film (RGBA32F, width*height, row-major): per pixel a light subpath and a camera subpath
 * through the pixel centre, every connection strategy (s light vertices, t camera vertices) with the reference's
 * MIS weight, the light-tracing (t = 1) strategies splatted into the frame's image, the progressive film. The
 * reference's per-frame path buffers live in the scene (reused between frames). A frame's splats all land in that
 * frame (the reference's unsynchronised splat image leaves the order undefined). max_depth in [1, 32]; area and
 * spot lights only. */
LGB_API lgb_status lgb_bdpt_iteration(lgb_scene* scene, const lgb_camera* camera, const lgb_bdpt_params* params,
                                      float* d_film, void* stream);

/* ---- ReSTIR DI (src/RayTracer/ReSTIR.cpp:74-157, src/shaders/integrators/restir/di/*): resampled direct
 *      lighting with temporal and spatial reuse, on the library's traversal and light sampling. ---- */
typedef struct lgb_restir_params {
    float sky_col[3];              /* PCReSTIR fields of the temporal pass's path-traced colour, which the output */
    int32_t max_depth;             /* pass never reads (output.rgen:12): kept for the layout, not used */
    int32_t num_lights;
    int32_t light_triangle_count;  /* LumenScene::total_light_triangle_cnt */
    uint32_t dir_light_idx;        /* must be 0xFFFFFFFF */
    uint32_t seed;                 /* the RNG's frame value is frame_num ^ seed (the reference draws seed with rand()) */
    uint32_t frame_num;
    uint32_t do_spatiotemporal;    /* 0 on the first frame (the temporal reservoirs are cleared), then 1 */
    uint32_t enable_accumulation;  /* 1: progressive mean over frames, 0: each frame alone */
    float spot_angle;              /* spot cone half-angle as lgb_vcm_params; 0 = Lumen's fixed 30 / 25 degrees */
    uint32_t flags;                /* LGB_RESTIR_* */
    uint32_t reserved[3];
} lgb_restir_params;
/* The spatial pass of the reference counts the pixel's own reservoir as one sample (spatial_pass.rgen:16-17, the
 * count is read after one combine), so W is too large by (m + neighbours) / (1 + neighbours), and the temporal
 * reuse feeds that back: the image brightens frame after frame. With this flag the count starts at the
 * reservoir's own m, and the estimate stays put. */
#define LGB_RESTIR_SPATIAL_COUNT_FIX 1u

/* One ReSTIR DI frame into d_film (RGBA32F, width*height): temporal pass (G-buffer, up to 32 light candidates,
 * visibility, merge with the previous frame's reservoir), spatial pass (5 neighbours), output. prev_camera is the
 * previous frame's camera for the temporal reprojection test (null: the same camera). The G-buffer and the
 * reservoirs live in the scene between frames. Area and spot lights only. */
LGB_API lgb_status lgb_restir_di_iteration(lgb_scene* scene, const lgb_camera* camera, const lgb_camera* prev_camera,
                                           const lgb_restir_params* params, float* d_film, void* stream);

/* ---- batched rendering (no counterpart in Lumen) ----
 * Many scenes and camera views of uneven size rendered by one wavefront: the paths of every job share the
 * queues, the traversal and shading launches and one captured bounce loop, instead of each image issuing its
 * own sequence. Every path is seeded and computed exactly as lgb_render_path computes it, so each job's film
 * is the one lgb_render_path would produce. */
typedef struct lgb_batch lgb_batch;

typedef struct lgb_batch_job {
    uint32_t scene;          /* index into the scene list given to lgb_batch_create */
    uint32_t frame0;         /* first frame (progressive film, as lgb_render_path) */
    uint32_t spp;            /* frames to add; 0 = nothing for this job */
    uint32_t reserved;
    lgb_camera camera;
    lgb_path_params params;
    float* d_film;           /* RGBA32F, width * height, 16-byte aligned; the films of one call must not overlap */
} lgb_batch_job;

typedef struct lgb_batch_opts {
    uint32_t path_capacity;        /* paths in flight per chunk (the queue size); 0 = 2^21 */
    uint32_t work_blocks_per_sm;   /* grid of the camera, shading and film kernels; 0 = 8 */
    uint32_t trace_blocks_per_sm;  /* grid of the persistent traversal kernels; 0 = as many as fit */
    uint32_t stack_placement;      /* traversal stack: LGB_STACK_LOCAL (0) per-thread local memory, or
                                      LGB_STACK_SHARED: its bottom 8 entries in shared memory */
    uint32_t from_cache;           /* written by lgb_batch_tune: 1 when the choice came from the tuning cache */
    uint32_t chunk_paths;          /* path regeneration: paths per chunk, run through the path_capacity slots
                                      (an ended path's slot takes the chunk's next path); 0 = 16 x path_capacity
                                      (at most 2^27), 1 = no regeneration (chunks of at most path_capacity) */
    uint32_t traversal;            /* traversal variant of the path tracer's ray queues: LGB_TRAVERSAL_AUTO (0) by
                                      the batch's triangle count (incoherent from 2^15), _COHERENT (a node's leaf
                                      triangles tested when it is visited) or _INCOHERENT (one postponed leaf
                                      triangle per lane and iteration); every variant gives the same hits */
    uint32_t reserved[1];
} lgb_batch_opts;
#define LGB_STACK_LOCAL 0u
#define LGB_STACK_SHARED 1u
#define LGB_TRAVERSAL_AUTO 0u
#define LGB_TRAVERSAL_COHERENT 1u
#define LGB_TRAVERSAL_INCOHERENT 2u

/* Copies the BVHs of `scenes` (each built with lgb_bvh_build) into one forest. The scenes must outlive the
 * batch; rebuilding a scene's BVH afterwards makes lgb_batch_render refuse the batch (LGB_ERR_NOT_READY). */
LGB_API lgb_status lgb_batch_create(lgb_ctx* ctx, lgb_scene* const* scenes, uint32_t num_scenes, lgb_batch** out);
LGB_API void lgb_batch_destroy(lgb_batch* batch);
/* Renders up to 128 jobs. opts null = the options lgb_batch_tune chose, else the defaults. Jobs are cut into
 * chunks of whole frames; a chunk holds frames of several jobs. With path regeneration (the default) a chunk
 * holds up to chunk_paths paths and runs through path_capacity slots: a slot whose path ended takes the chunk's
 * next path, and each job's film receives its frames in order once the chunk's last path has ended. Every path is
 * computed as lgb_render_path computes it, so films are bit-identical to rendering each job alone. A call is one
 * launch of the batch's own CUDA graph; on a stream that the caller is capturing it returns LGB_ERR_UNSUPPORTED. */
LGB_API lgb_status lgb_batch_render(lgb_batch* batch, const lgb_batch_job* jobs, uint32_t num_jobs,
                                    const lgb_batch_opts* opts, void* stream);
/* Autotuner: screens lgb_batch_render over candidate queue sizes and grids on a reduced copy of `jobs` (a quarter
 * of each job's frames), times the three fastest on `jobs` themselves, then the best of them with the other stack
 * placement and without path regeneration (films untouched throughout), keeps the fastest for later renders and
 * writes it to *best.
 * With a tuning cache (lgb_create) a batch of the same shape on the same kind of device takes the cached choice
 * without timing anything (best->from_cache = 1); a new choice is added to the cache. Waits for `stream`. */
LGB_API lgb_status lgb_batch_tune(lgb_batch* batch, const lgb_batch_job* jobs, uint32_t num_jobs,
                                  lgb_batch_opts* best, void* stream);
/* Waits for `stream` and reports faults recorded by the batch's traversal or by any of its scenes. */
LGB_API lgb_status lgb_batch_sync(lgb_batch* batch, void* stream);

/* Film error (src/shaders/rmse/*.comp, RayTracer.cpp:215-241): RMSE of d_film against d_reference, both RGBA32F
 * with npix pixels; alpha is ignored. mode 0 = sqrt(sum of squared RGB errors / (3 npix)); mode 1 = the value
 * Lumen reports (per 1024-pixel group the minimum of its warps' sums, calc_rmse.comp:37, then
 * sqrt(sum) / (3 npix), output_rmse.comp:23). Waits for `stream` and writes the result to *out_rmse. */
LGB_API lgb_status lgb_film_rmse(lgb_ctx* ctx, const float* d_film, const float* d_reference, uint32_t npix,
                                 uint32_t mode, double* out_rmse, void* stream);

/* Measurement helper with no counterpart in Lumen: best-of-5 read bandwidth (GB/s) of an L2-resident
 * buffer of `bytes` read `reps` times by all SMs, used as the roofline denominator of L2-bound traversal. */
LGB_API lgb_status lgb_measure_l2_read_gbs(int device, uint64_t bytes, uint32_t reps, double* out_gbs);

#ifdef __cplusplus
}
#endif
#endif /* LGB_H */
