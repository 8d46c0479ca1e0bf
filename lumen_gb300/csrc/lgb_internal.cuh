// Internal definitions shared by the CUDA translation units of liblgb.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "lgb.h"

namespace lgb {

// Entries of the per-thread traversal stack; a tree deeper than kStackSize + 1 levels is rejected.
constexpr int kStackSize = 48;

// ---------------------------------------------------------------------------------------------
// 8-wide BVH node, 80 bytes = five 16-byte loads.
//   chunk 0: px, py, pz (quantisation origin), e_imask = ex | ey << 8 | ez << 16 | imask << 24
//            (exponent bytes are biased by 127: the step along axis a is 2^(e_a - 127))
//   chunk 1: child_base, tri_base, meta[0..3], meta[4..7]
//   chunk 2: qlo_x[8], qlo_y[8]
//   chunk 3: qlo_z[8], qhi_x[8]
//   chunk 4: qhi_y[8], qhi_z[8]
// Slot s holds the child whose centre lies in octant s of the node (bit a of s set = positive side on
// axis a), so a ray visits children front to back by ranking slots with s ^ octant mask.
// imask bit s: slot s is an internal node, at child_base + popc(imask & ((1 << s) - 1)).
// meta[s] of a leaf slot: bits 0-4 = first triangle offset from tri_base, bits 5-7 = unary count
// (1 -> 0b001, 2 -> 0b011, 3 -> 0b111). Empty slots have meta 0 and an inverted box (qlo 255, qhi 0).
// Quantised boxes are rounded outwards with one extra step on every side, so they strictly contain the
// exact child boxes.
// ---------------------------------------------------------------------------------------------
struct __align__(16) WideNode {
    float px, py, pz;
    uint32_t e_imask;
    uint32_t child_base, tri_base;
    uint32_t meta_lo, meta_hi;
    uint8_t qlo_x[8], qlo_y[8], qlo_z[8];
    uint8_t qhi_x[8], qhi_y[8], qhi_z[8];
};
static_assert(sizeof(WideNode) == 80, "WideNode must be 80 bytes");

// Triangle in leaf order, 48 bytes = three 16-byte loads: (v0, prim), (v1, 0), (v2, 0).
struct __align__(16) WideTri {
    float4 a, b, c;
};
static_assert(sizeof(WideTri) == 48, "WideTri must be 48 bytes");

// Vertex as ray.rchit reads it (commons.h:194-198): position, normal, uv.
struct DevVertex {
    float px, py, pz;
    float nx, ny, nz;
    float u, v;
};

struct DevTexture {
    uint32_t width, height;
    const float4* texels;
};

// Device status word bits.
enum : uint32_t {
    STATUS_STACK_OVERFLOW = 1u << 0,
    STATUS_BAD_INDEX = 1u << 1,
    STATUS_VISIT_LIMIT = 1u << 2,  // a ray visited more nodes than any well-formed tree allows
};

// Upper bound on node visits of one ray: far above any real query, it only stops a malformed tree from
// looping.
constexpr uint32_t kMaxVisits = 1u << 22;

struct Scene;

struct Ctx {
    int device = 0;
    std::string last_error;
    std::string tuning_cache;  // lgb_batch_tune's cache file, empty = none
    int sm_count = 0;
    uint32_t users = 0;     // scenes and batches made with this context and not destroyed yet
    bool released = false;  // lgb_destroy was called while users > 0: freed with the last user
};
// A scene or batch holds its context: lgb_destroy of a context still in use only marks it, and the last
// lgb_scene_destroy / lgb_batch_destroy frees it, so the order of the destroy calls does not matter.
void ctx_retain(Ctx* c);
void ctx_release(Ctx* c);

struct BvhDevice {
    WideNode* nodes = nullptr;
    WideTri* tris = nullptr;
    uint32_t num_nodes = 0;
    uint32_t num_tris = 0;
    uint32_t max_depth = 0;
    uint32_t generation = 0;  // incremented by every build
};

struct Scene {
    Ctx* ctx = nullptr;
    uint32_t num_tris = 0;
    uint32_t num_vertices = 0;
    float3 bmin, bmax;           // scene bounds
    float* d_tri_verts = nullptr;  // 9 floats per global triangle (world space)
    DevVertex* d_vertices = nullptr;
    uint32_t* d_indices = nullptr;
    uint32_t* d_tri_mesh = nullptr;  // global triangle -> mesh
    uint8_t* d_tri_class = nullptr;  // global triangle -> shading class of its material (shade_class)
    lgb_mesh* d_meshes = nullptr;
    uint32_t* d_mesh_first_tri = nullptr;
    lgb_material* d_materials = nullptr;
    lgb_light* d_lights = nullptr;
    DevTexture* d_textures = nullptr;
    std::vector<void*> texture_buffers;
    uint32_t num_meshes = 0, num_materials = 0, num_lights = 0, num_textures = 0;
    uint32_t bsdf_mask = 0;  // union of the materials' LGB_BSDF_* types
    uint32_t shade_classes = 0;  // bit per shading class of the path tracer some material falls in (shade_class)
    std::vector<uint32_t> h_mesh_first_tri;
    std::vector<lgb_mesh> h_meshes;
    BvhDevice bvh;
    uint32_t* d_status = nullptr;  // device status word
    uint32_t visit_limit = 0;      // node visits per ray of the public queries; 0 = kMaxVisits
    uint32_t* d_ray_counter = nullptr;  // work counter of the persistent trace kernels
    // path-tracer work buffers (grown on demand)
    void* pt_buf = nullptr;
    size_t pt_buf_bytes = 0;
    void* pt_graph = nullptr;        // cudaGraphExec_t of the captured bounce loop
    uint64_t pt_graph_key[6] = {};   // what the captured graph depends on
    void* capture_stream = nullptr;  // private stream used only to record graphs
    void* diff_buf = nullptr;        // per-sample radiance of the differentiable renderer
    size_t diff_buf_bytes = 0;
    void* diffw_buf = nullptr;       // wavefront state of the differentiable renderer (paths, queues, rays)
    size_t diffw_buf_bytes = 0;
    void* vcm_buf = nullptr;         // VCM state kept between iterations (light vertices, counts, splats, table)
    size_t vcm_buf_bytes = 0;
    uint32_t vcm_w = 0, vcm_h = 0, vcm_per = 0;
    size_t vcm_o_verts = 0, vcm_o_counts = 0, vcm_o_gc = 0, vcm_o_gr = 0;  // offsets into vcm_buf
    float vcm_radius = 0.0f, vcm_mn[3] = {}, vcm_mx[3] = {};                 // grid of the last iteration
    int vcm_res[3] = {};
    void* bdpt_buf = nullptr;        // BDPT path buffers, strategy contributions and splat image (per frame)
    size_t bdpt_buf_bytes = 0;
    void* sppm_buf = nullptr;        // SPPM state kept between frames (visible points, photons, table, bounds)
    size_t sppm_buf_bytes = 0;
    uint32_t sppm_w = 0, sppm_h = 0, sppm_depth = 0;
    void* restir_buf = nullptr;      // ReSTIR DI state kept between frames (G-buffer, reservoirs)
    size_t restir_buf_bytes = 0;
    uint32_t restir_w = 0, restir_h = 0;
    uint32_t num_directional = 0;    // directional lights (not supported by VCM)
    // queries on host buffers: device copies of the rays and results, two copy streams and chunk events
    void* stage_buf = nullptr;
    size_t stage_bytes = 0;
    void* stream_h2d = nullptr;
    void* stream_d2h = nullptr;
    std::vector<void*> stage_events;
};

// Several scenes rendered as one wavefront: their BVHs copied into one forest (node and triangle indices
// relocated, each scene rooted at its first node), plus the batch's own work arena and captured graph.
struct Batch {
    Ctx* ctx = nullptr;
    std::vector<Scene*> scenes;
    std::vector<uint32_t> roots;            // root node of every scene in the forest
    std::vector<uint32_t> bvh_generation;   // each scene's BVH build at creation, to detect a rebuild
    WideNode* nodes = nullptr;
    WideTri* tris = nullptr;
    uint32_t num_nodes = 0, num_tris = 0;
    uint32_t* d_status = nullptr;
    void* buf = nullptr;
    size_t buf_bytes = 0;
    void* graph = nullptr;
    uint64_t graph_key[10] = {};
    void* capture_stream = nullptr;
    void* staging = nullptr;        // pinned host copy of the job table
    void* staging_event = nullptr;  // recorded after the table's upload, before the staging is reused
    // the render's chunk records in device memory, walked by the graph's device-driven loop
    void* d_chunks = nullptr;       // BatchChunk[chunk_cap]
    void* chunk_staging = nullptr;  // pinned host copy of them
    uint32_t chunk_cap = 0;
    uint32_t* d_loop = nullptr;     // [0] index of the chunk being rendered, [1] chunk count
    void* col_out = nullptr;        // float4 per path of the largest chunk: path regeneration's radiance output
    uint64_t col_out_paths = 0;
    bool regen_refused = false;     // the device refused the nested loop graph of path regeneration
    bool tuned = false;
    lgb_batch_opts tuned_opts{};
};

// Shading class of a material type in the wavefront path tracer: 0 diffuse, 1 conductor, 3 principled, 2 every
// other type (mirror, glass, dielectric, and types no BSDF handles, which still add their emission).
__host__ __device__ inline int shade_class(uint32_t bsdf_type) {
    return bsdf_type == LGB_BSDF_DIFFUSE ? 0 : bsdf_type == LGB_BSDF_CONDUCTOR ? 1 : bsdf_type == LGB_BSDF_PRINCIPLED ? 3 : 2;
}

// Error helpers: record a message on the context and return a status.
lgb_status set_error(Ctx* ctx, lgb_status st, const std::string& msg);
lgb_status cuda_error(Ctx* ctx, cudaError_t e, const char* what);

#define LGB_CUDA_TRY(ctx, expr)                                          \
    do {                                                                 \
        cudaError_t _e = (expr);                                         \
        if (_e != cudaSuccess) return ::lgb::cuda_error((ctx), _e, #expr); \
    } while (0)

// Entry points implemented per translation unit.
lgb_status build_bvh(Scene* s, const lgb_build_opts* opts, lgb_build_stats* stats);
lgb_status launch_trace_closest(Scene* s, const lgb_ray* rays, lgb_hit* hits, uint32_t n, cudaStream_t st,
                                uint64_t* counters);
lgb_status launch_trace_any(Scene* s, const lgb_ray* rays, uint32_t* bits, uint32_t n, cudaStream_t st);
// Queries on host buffers (out = lgb_hit[n] or occlusion bits), copies and traversal pipelined in chunks.
lgb_status trace_host(Scene* s, const lgb_ray* h_rays, void* h_out, uint32_t n, bool any, cudaStream_t st);
lgb_status render_path(Scene* s, const lgb_camera* cam, const lgb_path_params* p, uint32_t frame0, uint32_t spp,
                       float* film, cudaStream_t st);

}  // namespace lgb

// The opaque handles of include/lgb.h.
struct lgb_ctx : public lgb::Ctx {};
struct lgb_batch : public lgb::Batch {};
struct lgb_scene : public lgb::Scene {};
