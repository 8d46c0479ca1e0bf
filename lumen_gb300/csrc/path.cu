// Wavefront unidirectional MIS path tracer (the Path integrator).
//
// Restates src/shaders/integrators/path/path.rgen:22-113 and pt_commons.glsl:3-48 as a sequence of
// kernels over path state kept as structure-of-arrays in HBM:
//   k_camera          path.rgen:28-46   one path per (pixel, frame), jittered camera ray
//   k_q_trace_closest path.rgen:48      continuation rays of the live queue
//   k_classify        path.rgen:49-55   misses add the sky and end; hits are binned by material class (a
//                                       scene of one class skips it: its shading kernel takes the queue)
//   k_shade<CLASS>    path.rgen:56-100  ray.rchit hit resolve, emission, NEE light sample + shadow ray,
//                                       BSDF-MIS ray, BSDF sample, throughput, Russian roulette, enqueue
//   k_q_trace_nee     pt_commons.glsl:21,32  BSDF-MIS rays (closest) and shadow rays (any) in one launch
//   k_nee_resolve     pt_commons.glsl:20-41 combination of the two light-sampling strategies
//   k_film            path.rgen:102-112 NaN drop and progressive mean, frames in order
// Every kernel reads its work count from device memory, so one render issues no host synchronisation.
// Queues are compacted with warp-aggregated atomics. RNG state is the counter-based PCG4D seed
// (x, y, frame, w): a path carries only w. Compiled with -fmad=false to keep the shader's FP32 sequence.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <unistd.h>

#include "path_common.cuh"

namespace lgb {
namespace {
using namespace sh;

constexpr float kTMin = 0.001f;    // path.rgen:19
constexpr float kTMax = 10000.0f;  // path.rgen:20
constexpr float kEps = 0.001f;     // utils.glsl:8
constexpr int kRRMinDepth = 3;     // path.rgen:21
constexpr uint32_t kMaxPaths = 1u << 21;
constexpr int kThreads = 128;

enum MatClass { CLS_DIFFUSE = 0, CLS_CONDUCTOR = 1, CLS_SPECULAR = 2, CLS_PRINCIPLED = 3, NUM_CLS = 4 };

// NEE record: the light-sampling state that pt_commons.glsl keeps in registers across its two traces, 80 bytes.
// Both terms already carry the throughput and the light pick pdf (T * x / light_pick_pdf, path.rgen:76-78), so
// the resolve adds the light sample's term when its shadow ray is unoccluded and the BSDF-MIS term times its MIS
// weight 1 / (1 + pdf_pos_a / (g * pdf)) when the MIS ray hits the sampled light triangle.
struct __align__(16) NeeRec {
    float4 light;   // xyz: T * mis * f * |cos| * Le / pdf_w / light_pick_pdf (0 when pdf_w is 0); w: path id (bits)
    float4 bsdf;    // xyz: T * f2 * |cos2| * Le / pdf2 / light_pick_pdf; w: pdf_pos_a / pdf2, or -1 without a MIS term
    float4 pos;     // xyz: shading position; w: shading prim (bits)
    float4 ns;      // xyz: shading normal as the hit payload holds it (not face-forwarded); w: slot of the BSDF-MIS
                    // ray in the MIS queue (bits), 0xFFFFFFFF when no ray was queued
    float4 wi2;     // xyz: BSDF-MIS direction; w: sampled light prim (bits)
};

struct Params {
    float iv[16], ip[16];
    uint32_t width, height, npix;
    float sky[3];
    int max_depth, num_lights, light_tri_count;
    uint32_t direct_lighting, film_mode;
    uint32_t frame0;   // first frame of this chunk
    uint32_t nframes;  // frames in this chunk
    uint32_t cap;      // path capacity of the buffers
    float4* film;      // RGBA32F output
};

struct JobRec;
struct BatchChunk;

struct Buffers {
    uint32_t* pix;      // pixel index
    uint32_t* frame;
    uint32_t* w;        // RNG counter
    uint32_t* flags;    // bits 0-15 depth, bit 16 last_specular
    float4* T;          // throughput
    float4* col;        // radiance
    uint32_t* q_cur;
    uint32_t* q_next;
    uint32_t* q_cls;    // NUM_CLS * cap: queue positions binned by material class
    lgb_ray* rays;       // rays of the current queue
    lgb_ray* rays_next;  // continuation rays being enqueued
    lgb_hit* hits;
    NeeRec* nee;
    lgb_ray* srays;
    lgb_ray* mrays;
    lgb_hit* mhits;
    uint32_t* sbits;
    uint32_t* counters; // [0] cur, [1] next, [2] nee, [3..6] class counts, [8..10] trace work counters,
                        // [11] queued BSDF-MIS rays; batched only: [12] paths ended this bounce, [13] paths of
                        // the chunk started so far
    Params* params;     // per-chunk parameters in device memory, so that a captured graph can be replayed
    uint32_t cap;       // path capacity of the arena
    // batched rendering only (null otherwise)
    uint32_t* job;       // job of each path
    uint32_t* root;      // BVH root node of each ray of the current queue
    uint32_t* root_next; // ... of the continuation rays being enqueued
    uint32_t* nroot;     // ... of the shadow rays
    uint32_t* mroot;     // ... of the queued BSDF-MIS rays
    const JobRec* jobs;
    const BatchChunk* chunk;
    // batched rendering with path regeneration: a slot freed by an ended path takes the chunk's next path
    uint32_t* pid;       // chunk path (segment-major, as path_off + frame * npix + pixel) held by each slot
    uint32_t* done;      // slots whose path ended this bounce
    float4* col_out;     // final radiance of every path of the chunk, by chunk path
    const float4* film_src;  // what the film kernel reads by chunk path: col (one slot per path) or col_out
};

// Batched rendering: several scenes and cameras share one wavefront. Every job (a scene, a camera, path
// parameters, a film and a frame range) has a record in device memory; a chunk of paths is a list of segments,
// each holding whole frames of one job, so that the film of every job still receives its frames in order.
constexpr uint32_t kMaxBatchJobs = 128;

struct JobRec {
    Params P;       // camera, image and path parameters, film (frame0, nframes and cap unused)
    SceneView S;    // the job's scene arrays (traversal uses the batch's BVH forest instead)
    uint32_t root;  // root node of the job's BVH in the forest
    uint32_t pad[3];
};

struct Segment {
    uint32_t job, frame0, nframes, path_off, pix_off, npix;
};

struct BatchChunk {
    uint32_t nseg, npaths, npix_total, write_film;
    Segment seg[kMaxBatchJobs];
};

// Segment holding element `i` of a prefix-offset field (path_off or pix_off): binary search, nseg <= 128.
template <bool PIX>
__device__ __forceinline__ uint32_t find_segment(const BatchChunk& C, uint32_t i) {
    uint32_t lo = 0, hi = C.nseg - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        const uint32_t off = PIX ? C.seg[mid].pix_off : C.seg[mid].path_off;
        if (off <= i) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}




// ---------------- kernels ----------------

// path.rgen:22-46: the seed is (x, y, frame, 0); two draws jitter the pixel. Starts chunk path `id` (batched:
// segment-major over the chunk's segments; else frame-major over the chunk's frames) in arena slot `slot`, with
// its camera ray at position q of a ray queue (rays, slots and, batched, BVH roots).
template <bool BATCH>
__device__ __forceinline__ void start_path(const Params* __restrict__ Pp, const Buffers& B, uint32_t id, uint32_t slot,
                                           lgb_ray* rays, uint32_t* qlist, uint32_t* roots, uint32_t q) {
    uint32_t local = id, frame0 = 0u, job = 0u;
    if (BATCH) {
        const Segment& sg = B.chunk->seg[find_segment<false>(*B.chunk, id)];
        local = id - sg.path_off;
        frame0 = sg.frame0;
        job = sg.job;
    } else {
        frame0 = Pp->frame0;
    }
    const Params& P = BATCH ? B.jobs[job].P : *Pp;
    const uint32_t pix = local % P.npix, f = frame0 + local / P.npix;
    const uint32_t x = pix % P.width, y = pix / P.width;
    uint4 seed = make_uint4(x, y, f, 0u);
    const float px = (float)x + 0.5f, py = (float)y + 0.5f;
    const float r0 = rnd(seed) - 0.5f;
    const float r1 = rnd(seed) - 0.5f;
    const float u = (px + r0) / (float)P.width, v = (py + r1) / (float)P.height;
    const float dx = u * 2.0f - 1.0f, dy = v * 2.0f - 1.0f;
    const float4 origin = mat_vec(P.iv, 0.0f, 0.0f, 0.0f, 1.0f);
    const float4 target = mat_vec(P.ip, dx, dy, 1.0f, 1.0f);
    const v3 tn = normalize(V3(target.x, target.y, target.z));
    const float4 dir = mat_vec(P.iv, tn.x, tn.y, tn.z, 0.0f);
    B.pix[slot] = pix;
    B.frame[slot] = f;
    B.w[slot] = seed.w;
    B.flags[slot] = 0u;
    B.T[slot] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
    B.col[slot] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    qlist[q] = slot;
    if (BATCH) {
        B.job[slot] = job;
        B.pid[slot] = id;
        roots[q] = B.jobs[job].root;
    }
    store_ray(&rays[q], make_ray(V3(origin.x, origin.y, origin.z), kTMin, V3(dir.x, dir.y, dir.z), kTMax));
}

// The chunk's first paths, path i in slot i: every path of a chunk that fits the arena; batched, the first
// `cap` paths of a larger chunk, whose other paths start as slots free up (k_regen).
template <bool BATCH>
__global__ void __launch_bounds__(kThreads) k_camera(const Params* __restrict__ Pp, Buffers B) {
    const uint32_t n = BATCH ? min(B.chunk->npaths, B.cap) : Pp->npix * Pp->nframes;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        start_path<BATCH>(Pp, B, i, i, B.rays, B.q_cur, B.root, i);
}

// Closest-hit / any-hit over a device-counted queue of rays, persistent with dynamic fetch; `roots` gives each
// ray's BVH root in a batch forest (null: one BVH rooted at node 0). Registers are sized for 9 blocks per SM.
// Two traversal variants (INC):
//  - coherent (false): a node's leaf triangles are tested in the iteration that reaches it and a warp refetches
//    once all its lanes are idle; best for small scenes whose short rays stay together (Cornell box 256x256x16
//    spp: 694 Msamples/s, 672 refetching at 16 idle lanes, 659 and 635 with the incoherent settings below);
//  - incoherent (true): the headline trace kernel's settings, one postponed leaf triangle per lane and iteration
//    with warp-uniform triangle iterations once a fifth of the active lanes hold one, and a refetch at 8 idle lanes;
//    for large scenes whose secondary rays diverge (the 32-scene batch's scenes rendered one by one: 417 against
//    413 Msamples/s; the tuned batch itself lands within its run-to-run spread either way).
// The single-scene renderer takes the incoherent variant from kIncoherentTris triangles; the batch tuner times
// both. SK: bottom stack entries per thread in shared memory (0: the whole stack in local memory); the batch
// autotuner tries both placements.
#ifdef LGB_QUEUE_POSTPONE
constexpr bool kQueuePostpone = LGB_QUEUE_POSTPONE != 0;
#else
constexpr bool kQueuePostpone = false;
#endif
#ifdef LGB_QUEUE_TRI_MIN
constexpr int kQueueTriMin = LGB_QUEUE_TRI_MIN;
#else
constexpr int kQueueTriMin = 0;
#endif
#ifdef LGB_QUEUE_REFILL
constexpr int kQueueRefill = LGB_QUEUE_REFILL;
#else
constexpr int kQueueRefill = 32;
#endif
constexpr int kQueueTraceMinBlocks = 9;
constexpr int kQueueSharedStack = 8;  // entries when the stack placement is LGB_STACK_SHARED
constexpr uint32_t kIncoherentTris = 1u << 15;
template <bool INC> struct QueueTrace {  // coherent
    static constexpr bool postpone = kQueuePostpone;
    static constexpr int tri_min = kQueueTriMin, refill = kQueueRefill;
};
#ifndef LGB_QUEUE_INC_REFILL
#define LGB_QUEUE_INC_REFILL 8  // the 32-scene batch: 550-554 Msamples/s at 8 idle lanes, 542-548 at 4, 540-545 at 16
#endif
template <> struct QueueTrace<true> {  // incoherent
    static constexpr bool postpone = true;
    static constexpr int tri_min = -5, refill = LGB_QUEUE_INC_REFILL;
};
template <int SK, bool INC>
__global__ void __launch_bounds__(kThreads, kQueueTraceMinBlocks)
    k_q_trace_closest(SceneView S, const lgb_ray* __restrict__ rays, lgb_hit* __restrict__ hits,
                      const uint32_t* count_ptr, uint32_t* ray_counter, const uint32_t* __restrict__ roots) {
    using Q = QueueTrace<INC>;
    __shared__ uint2 s_stack[SK > 0 ? SK * kThreads : 1];
    trace_persistent<false, false, Q::postpone, SK, kThreads, Q::refill, Q::tri_min>(
        S.nodes, S.tris, rays, hits, nullptr, 0u, count_ptr, ray_counter, S.status, nullptr, roots, s_stack);
}
// A bounce's two NEE queries in one launch: the queued BSDF-MIS rays (closest hit) first, then the shadow rays
// (any hit). The MIS queue is short but its rays are long, so the warps that take them start at once and then
// join the shadow rays, whose queue the other warps are already draining; as two launches, the MIS trace ran alone
// at the end of every bounce, bound by the latency of its few rays (Cornell box: 17 us of each 180-330 us bounce).
template <int SK, bool INC>
__global__ void __launch_bounds__(kThreads, kQueueTraceMinBlocks)
    k_q_trace_nee(SceneView S, const lgb_ray* __restrict__ srays, uint32_t* __restrict__ sbits,
                  const uint32_t* scount, uint32_t* sctr, const uint32_t* __restrict__ sroots,
                  const lgb_ray* __restrict__ mrays, lgb_hit* __restrict__ mhits, const uint32_t* mcount,
                  uint32_t* mctr, const uint32_t* __restrict__ mroots) {
    using Q = QueueTrace<INC>;
    __shared__ uint2 s_stack[SK > 0 ? SK * kThreads : 1];
    trace_persistent<false, false, Q::postpone, SK, kThreads, Q::refill, Q::tri_min>(
        S.nodes, S.tris, mrays, mhits, nullptr, 0u, mcount, mctr, S.status, nullptr, mroots, s_stack);
    trace_persistent<true, false, Q::postpone, SK, kThreads, Q::refill, Q::tri_min>(
        S.nodes, S.tris, srays, nullptr, sbits, 0u, scount, sctr, S.status, nullptr, sroots, s_stack);
}

// path.rgen:49-55: a miss adds the sky colour (shade_atmosphere without a directional light returns
// sky_col, commons.glsl:157-159) and ends the path.
__device__ __forceinline__ void miss_sky(const Params& P, const Buffers& B, uint32_t p) {
    const uint32_t depth = B.flags[p] & 0xffffu;
    if (depth > 0 || P.direct_lighting == 1u) {
        const float4 T = B.T[p];
        float4 c = B.col[p];
        c.x = c.x + T.x * P.sky[0];
        c.y = c.y + T.y * P.sky[1];
        c.z = c.z + T.z * P.sky[2];
        B.col[p] = c;
    }
}

// Misses end their paths (miss_sky); hits are binned by material class.
template <bool BATCH>
__global__ void __launch_bounds__(kThreads) k_classify(SceneView S0, const Params* __restrict__ Pp, Buffers B) {
    const uint32_t n = B.counters[0];
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t i = base + threadIdx.x;
        int cls = -1;
        bool ended = false;
        uint32_t p = 0u;
        if (i < n) {
            const uint32_t prim = B.hits[i].prim;
            p = B.q_cur[i];
            const uint32_t job = BATCH ? B.job[p] : 0u;
            if (prim == LGB_NO_HIT) {
                ended = true;
                miss_sky(BATCH ? B.jobs[job].P : *Pp, B, p);
            } else {
                const SceneView S = BATCH ? B.jobs[job].S : S0;
                cls = S.tri_class[prim];
            }
        }
#pragma unroll
        for (int c = 0; c < NUM_CLS; c++) {
            const uint32_t slot = agg_slot(&B.counters[3 + c], cls == c);
            if (cls == c) B.q_cls[(size_t)c * B.cap + slot] = i;
        }
        if (BATCH) {  // a missed path ends here; its slot is listed for regeneration
            const uint32_t dslot = agg_slot(&B.counters[12], ended);
            if (ended) B.done[dslot] = p;
        }
    }
}

// Restricted BSDF dispatch per material class, so each shading kernel compiles only its own lobes.
template <int CLS>
__device__ __forceinline__ v3 cls_sample(v3 n_s, v3 wo, const Mat& m, bool ff, v3& wi, float& pdf, float& cos_t, v3 r) {
    if (CLS == CLS_DIFFUSE) {
        v3 T, B;
        branchless_onb(n_s, T, B);
        const v3 wl = to_local(wo, T, B, n_s);
        v3 wil;
        const v3 f = sample_diffuse(m, wl, wil, pdf, cos_t, V2(r.x, r.y));
        wi = to_world(wil, T, B, n_s);
        return f;
    }
    return sample_bsdf(n_s, wo, m, ff, wi, pdf, cos_t, r);
}
template <int CLS>
__device__ __forceinline__ v3 cls_eval(v3 n_s, v3 wo, const Mat& m, bool ff, v3 wi, float& pdf) {
    if (CLS == CLS_DIFFUSE) {
        v3 T, B;
        branchless_onb(n_s, T, B);
        return eval_diffuse(m, to_local(wo, T, B, n_s), to_local(wi, T, B, n_s), pdf);
    }
    return eval_bsdf(n_s, wo, m, ff, wi, pdf);
}

// One bounce of path.rgen:56-100 for the hits of one material class. SOLE (a scene whose materials all fall in
// this class): the kernel takes the whole queue in place of k_classify, a miss ending its path as there.
// Registers capped for 4 blocks per SM (128): the diffuse kernel reads and writes ~400 B of path state per path
// and wants occupancy (Cornell / batch scene 550 / 354 Msamples/s against 549 / 349 uncapped at 140 registers).
#ifdef LGB_SHADE_MIN_BLOCKS
constexpr int kShadeMinBlocks = LGB_SHADE_MIN_BLOCKS;
#else
constexpr int kShadeMinBlocks = 4;
#endif
template <int CLS, bool BATCH, bool SOLE = false>
__global__ void __launch_bounds__(kThreads, kShadeMinBlocks) k_shade(SceneView S0, const Params* __restrict__ Pp, Buffers B, int bounce) {
    const uint32_t n = SOLE ? B.counters[0] : B.counters[3 + CLS];
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t* list = B.q_cls + (size_t)CLS * B.cap;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t k = base + threadIdx.x;
        bool cont = false, nee = false;
        uint32_t p = 0, root = 0;
        lgb_ray next_ray, sray, mray;
        NeeRec rec;
        if (k < n) {
            const uint32_t qi = SOLE ? k : list[k];
            p = B.q_cur[qi];
            const uint32_t job = BATCH ? B.job[p] : 0u;
            const Params& P = BATCH ? B.jobs[job].P : *Pp;
            const SceneView S = BATCH ? B.jobs[job].S : S0;
            if (BATCH) root = B.jobs[job].root;
            const lgb_hit hit = B.hits[qi];
            if (SOLE && hit.prim == LGB_NO_HIT) {
                miss_sky(P, B, p);
            } else {
                const lgb_ray ray = B.rays[qi];
                const uint32_t pix = B.pix[p], frame = B.frame[p];
                uint4 seed = seed_of(pix, P.width, frame, B.w[p]);
                const uint32_t fl = B.flags[p];
                // batched, paths of different depths share a bounce (regeneration): each path's own depth
                const int depth = BATCH ? (int)(fl & 0xffffu) : bounce;
                const bool last_specular = (fl >> 16) & 1u;
                v3 T = f3(B.T[p]);
                v3 col = f3(B.col[p]);
                const HitAttr h = resolve_hit(S, hit.prim, hit.u, hit.v);
                const Mat m = load_material(S, h.mat, h.u, h.v);
                if ((depth == 0 && P.direct_lighting == 1u) || last_specular) col = col + T * m.emissive;
                if (depth < P.max_depth - 1) {
                    const v3 direction = V3(ray.dx, ray.dy, ray.dz);
                    const v3 wo = -direction;
                    v3 n_s = h.n_s;
                    bool side = true;
                    v3 n_g = h.n_g;
                    if (dot(h.n_g, wo) < 0.0f) n_g = -n_g;
                    if (dot(n_g, h.n_s) < 0.0f) { n_s = -n_s; side = false; }
                    const v3 origin = offset_ray(h.pos, n_g);
                    const bool spec = has_prop(m.props, LGB_FLAG_SPECULAR);
                    if (!spec && (depth > 0 || P.direct_lighting == 1u) && P.num_lights <= 0) {
                        // No light to sample: Lumen would read past its light buffer; here the four draws are
                        // consumed and nothing is added.
                        for (int k = 0; k < 4; k++) (void)rnd(seed);
                    } else if (!spec && (depth > 0 || P.direct_lighting == 1u)) {
                        // uniform_sample_light (pt_commons.glsl:3-42) and sample_light_Li (commons.glsl:224-300)
                        nee = true;
                        const float lpp = 1.0f / (float)P.light_tri_count;
                        const float q0 = rnd(seed), q1 = rnd(seed), q2 = rnd(seed), q3 = rnd(seed);
                        const uint32_t li = (uint32_t)(q0 * (float)P.num_lights);
                        const lgb_light* L = &S.lights[li];
                        const uint32_t lflags = L->light_flags, ltype = lflags & 7u;
                        v3 Le = V3(0.0f), wi = V3(0.0f);
                        float wi_len = 0.0f, pdf_w = 0.0f, pdf_a = 0.0f;
                        uint32_t lprim = LGB_NO_HIT, lio = 0u, lvo = 0u;
                        if (ltype == LGB_LIGHT_AREA) {
                            const lgb_mesh pm = S.meshes[L->prim_mesh_idx];
                            const uint32_t tri = (uint32_t)(q1 * (float)L->num_triangles);
                            lprim = S.mesh_first[L->prim_mesh_idx] + tri;
                            const uint32_t io = pm.index_offset + 3u * tri;
                            lio = io;
                            lvo = pm.vertex_offset;
                            const DevVertex a = S.verts[S.idx[io] + pm.vertex_offset];
                            const DevVertex b = S.verts[S.idx[io + 1] + pm.vertex_offset];
                            const DevVertex c = S.verts[S.idx[io + 2] + pm.vertex_offset];
                            const float su = 1.0f - sqrtf(q2), sv = q3 * sqrtf(q2);
                            const float b0 = 1.0f - su - sv;
                            const v3 v0 = V3(a.px, a.py, a.pz), v1 = V3(b.px, b.py, b.pz), v2 = V3(c.px, c.py, c.pz);
                            const v3 et0 = v1 - v0, et1 = v2 - v0;
                            const v3 lpos = v0 * b0 + v1 * su + v2 * sv;
                            const v3 ln = normalize(normalize(V3(a.nx, a.ny, a.nz) * b0 + V3(b.nx, b.ny, b.nz) * su +
                                                              V3(c.nx, c.ny, c.nz) * sv));
                            const float tri_pdf = 2.0f / length(cross(et0, et1));
                            const lgb_material* lm = &S.mats[pm.material_index];
                            Le = V3(lm->emissive_factor[0], lm->emissive_factor[1], lm->emissive_factor[2]);
                            wi = lpos - h.pos;
                            const float l2 = dot(wi, wi);
                            wi_len = sqrtf(l2);
                            wi = wi / wi_len;
                            const float cfl = fabsf(dot(ln, -wi));
                            pdf_a = tri_pdf;
                            pdf_w = pdf_a * l2 / cfl;
                        } else if (ltype == LGB_LIGHT_SPOT) {
                            const v3 lp = V3(L->pos[0], L->pos[1], L->pos[2]);
                            wi = lp - h.pos;
                            const float l2 = dot(wi, wi);
                            wi_len = sqrtf(l2);
                            wi = wi / wi_len;
                            const v3 ldir = normalize(V3(L->to[0], L->to[1], L->to[2]) - lp);
                            const float cfl = dot(-wi, ldir);
                            const float cw = cosf(LGB_PI / 6.0f), cf = cosf(25.0f * LGB_PI / 180.0f);
                            float fall;
                            if (cfl < cw) fall = 0.0f;
                            else if (cfl >= cf) fall = 1.0f;
                            else { const float d = (cfl - cw) / (cf - cw); fall = (d * d) * (d * d); }
                            pdf_a = 1.0f;
                            pdf_w = l2;
                            Le = V3(L->L[0], L->L[1], L->L[2]) * fall;
                        } else {
                            const v3 dir = normalize(V3(L->pos[0], L->pos[1], L->pos[2]) - V3(L->to[0], L->to[1], L->to[2]));
                            const v3 lp = h.pos + dir * (2.0f * L->world_radius);
                            wi = lp - h.pos;
                            wi_len = length(wi);
                            wi = wi / wi_len;
                            pdf_a = 1.0f;
                            pdf_w = 1.0f;
                            Le = V3(L->L[0], L->L[1], L->L[2]);
                        }
                        const v3 sp = offset_ray2(h.pos, n_s);
                        float bsdf_pdf;
                        const float cos_x = dot(n_s, wi);
                        const v3 f = cls_eval<CLS>(n_s, wo, m, side, wi, bsdf_pdf);
                        v3 term1 = V3(0.0f);
                        if (pdf_w > 0.0f) {
                            const float mis = ((lflags >> 5) & 1u) ? 1.0f : 1.0f / (1.0f + bsdf_pdf / pdf_w);
                            term1 = mis * f * fabsf(cos_x) * Le / pdf_w;
                        }
                        // The shadow ray only matters when the light sample can contribute.
                        sray = make_ray(sp, 0.0f, wi, pdf_w > 0.0f ? wi_len - kEps : -1.0f);
                        v3 f2 = V3(0.0f), wi2 = V3(0.0f);
                        float pdf2 = 0.0f, cos2 = 0.0f;
                        if (ltype == LGB_LIGHT_AREA) {
                            const float b0r = rnd(seed), b1r = rnd(seed), b2r = rnd(seed);
                            f2 = cls_sample<CLS>(n_s, wo, m, side, wi2, pdf2, cos2, V3(b0r, b1r, b2r));
                        }
                        mray = make_ray(sp, kTMin, wi2, pdf2 != 0.0f ? kTMax : -1.0f);
                        // The MIS ray only counts when its closest hit is the sampled light triangle. Unless the
                        // shading point is on that triangle (a miss then reuses the shading point's own payload), a
                        // ray that fails the traversal's watertight test against it (same ray, same vertices) cannot
                        // count: it gets an empty interval, which the trace kernel ends at once as a miss, and a miss
                        // resolves to no contribution exactly as the traced ray would have.
                        if (pdf2 != 0.0f && lprim != hit.prim) {
                            const DevVertex a = S.verts[S.idx[lio] + lvo];
                            const DevVertex b = S.verts[S.idx[lio + 1] + lvo];
                            const DevVertex c = S.verts[S.idx[lio + 2] + lvo];
                            const RayQ rq = make_rayq(mray.ox, mray.oy, mray.oz, mray.tmin, mray.dx, mray.dy, mray.dz,
                                                      mray.tmax);
                            float tt, tu, tv;
                            if (!tri_intersect(rq, make_float4(a.px, a.py, a.pz, 0.0f), make_float4(b.px, b.py, b.pz, 0.0f),
                                               make_float4(c.px, c.py, c.pz, 0.0f), rq.tmax, tt, tu, tv))
                                mray.tmax = -1.0f;
                        }
                        const bool mis_term = ltype == LGB_LIGHT_AREA && pdf2 != 0.0f;
                        rec.light = f4(T * term1 / lpp, __uint_as_float(p));
                        rec.bsdf = mis_term ? f4(T * (f2 * fabsf(cos2) * Le / pdf2) / lpp, pdf_a / pdf2)
                                            : make_float4(0.0f, 0.0f, 0.0f, -1.0f);
                        rec.pos = f4(h.pos, __uint_as_float(hit.prim));
                        rec.ns = f4(h.n_s, __uint_as_float(0xFFFFFFFFu));
                        rec.wi2 = f4(wi2, __uint_as_float(lprim));
                    }
                    float pdf, cos_t;
                    v3 dir_next;
                    const float c0 = rnd(seed), c1 = rnd(seed), c2 = rnd(seed);
                    const v3 f = cls_sample<CLS>(n_s, wo, m, side, dir_next, pdf, cos_t, V3(c0, c1, c2));
                    if (pdf != 0.0f) {
                        T = T * (f * fabsf(cos_t) / pdf);
                        float rr_scale = 1.0f;
                        if (has_prop(m.props, LGB_FLAG_TRANSMISSION)) rr_scale *= side ? 1.0f / m.ior : m.ior;
                        cont = true;
                        if (depth > kRRMinDepth) {
                            const float rr = fminf(0.95f, luminance(T) * rr_scale);
                            if (rr == 0.0f || rr < rnd(seed)) cont = false;
                            else T = T / rr;
                        }
                        next_ray = make_ray(origin, kTMin, dir_next, kTMax);
                    }
                    B.flags[p] = (uint32_t)(depth + 1) | (spec ? (1u << 16) : 0u);
                }
                B.w[p] = seed.w;
                B.T[p] = f4(T, 0.0f);
                B.col[p] = f4(col, 0.0f);
            }
        }
        const uint32_t cslot = agg_slot(&B.counters[1], cont);
        if (cont) {
            B.q_next[cslot] = p;
            store_ray(&B.rays_next[cslot], next_ray);
            if (BATCH) B.root_next[cslot] = root;
        }
        if (BATCH) {  // an ended path's slot is listed for regeneration (its NEE record still resolves first)
            const bool ended = k < n && !cont;
            const uint32_t dslot = agg_slot(&B.counters[12], ended);
            if (ended) B.done[dslot] = p;
        }
        // Only BSDF-MIS rays with a non-empty interval are queued (those the pre-test above did not end); the NEE
        // record keeps the ray's queue slot. A record without a queued ray resolves as a miss, as its empty ray
        // would have.
        const bool mis_ray = nee && mray.tmax >= mray.tmin;
        const uint32_t mslot = agg_slot(&B.counters[11], mis_ray);
        if (mis_ray) {
            store_ray(&B.mrays[mslot], mray);
            if (BATCH) B.mroot[mslot] = root;
            rec.ns.w = __uint_as_float(mslot);
        }
        const uint32_t nslot = agg_slot(&B.counters[2], nee);
        if (nee) {
            B.nee[nslot] = rec;
            store_ray(&B.srays[nslot], sray);
            if (BATCH) B.nroot[nslot] = root;
            // The shadow ray's occlusion word starts at zero: every record's writer clears its word (the lanes
            // of a warp write the same one or two words), before the any-hit launch sets the bits.
            B.sbits[nslot >> 5] = 0u;
        }
    }
}

// pt_commons.glsl:20-41 after both traces: combine the light sample (if unoccluded) with the BSDF-MIS
// sample (if it hit the sampled light triangle), then col += T * res / light_pick_pdf (path.rgen:78).
// A missed MIS ray leaves the previous closest-hit payload in place (ray.rmiss:13 only marks the
// material), so the comparison then uses the shading point's own triangle, position and normal.
template <bool BATCH>
__global__ void __launch_bounds__(kThreads) k_nee_resolve(SceneView S0, Buffers B) {
    const uint32_t n = B.counters[2];
    for (uint32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        const NeeRec rec = B.nee[r];
        const uint32_t p = __float_as_uint(rec.light.w);
        const SceneView S = BATCH ? B.jobs[B.job[p]].S : S0;
        const bool occluded = (B.sbits[r >> 5] >> (r & 31)) & 1u;
        v3 add = V3(0.0f);
        if (!occluded) add = f3(rec.light);
        if (rec.bsdf.w >= 0.0f) {
            const uint32_t mslot = __float_as_uint(rec.ns.w);
            const lgb_hit mh = mslot != 0xFFFFFFFFu ? B.mhits[mslot] : lgb_hit{LGB_NO_HIT, 0.0f, 0.0f, 0.0f};
            const uint32_t lprim = __float_as_uint(rec.wi2.w);
            const uint32_t pl_prim = mh.prim == LGB_NO_HIT ? __float_as_uint(rec.pos.w) : mh.prim;
            if (pl_prim == lprim) {
                v3 pl_pos, pl_ns;
                if (mh.prim == LGB_NO_HIT) {
                    pl_pos = f3(rec.pos);
                    pl_ns = f3(rec.ns);
                } else {
                    const HitAttr h = resolve_hit(S, mh.prim, mh.u, mh.v);
                    pl_pos = h.pos;
                    pl_ns = h.n_s;
                }
                const v3 wi2 = f3(rec.wi2);
                const float wl = length(pl_pos - f3(rec.pos));
                const float g = fabsf(dot(pl_ns, -wi2)) / (wl * wl);
                const float mis = 1.0f / (1.0f + rec.bsdf.w / g);
                add = add + f3(rec.bsdf) * mis;
            }
        }
        float4 c = B.col[p];
        c.x = c.x + add.x; c.y = c.y + add.y; c.z = c.z + add.z;
        B.col[p] = c;
    }
}

// Queue rotation between bounces: the enqueued continuation count becomes the live count.
__global__ void k_rotate(uint32_t* counters) {
    if (threadIdx.x == 0) {
        counters[0] = counters[1];
        counters[1] = 0u;
        counters[2] = 0u;
        for (int c = 0; c < NUM_CLS; c++) counters[3 + c] = 0u;
        counters[8] = counters[9] = counters[10] = counters[11] = counters[12] = 0u;
    }
}

// Path regeneration (batched): after the bounce's NEE records have resolved, every slot on the ended list hands its
// path's radiance to col_out, and the first of them take the chunk's next paths, whose camera rays are appended
// to the continuation queue behind the continuing paths. k_rotate_regen then makes both the next bounce's queue.
__global__ void __launch_bounds__(kThreads) k_regen(Buffers B) {
    const uint32_t nd = B.counters[12], base = B.counters[1], next = B.counters[13];
    const uint32_t nn = min(nd, B.chunk->npaths - next);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nd; i += gridDim.x * blockDim.x) {
        const uint32_t slot = B.done[i];
        B.col_out[B.pid[slot]] = B.col[slot];
        if (i < nn) start_path<true>(nullptr, B, next + i, slot, B.rays_next, B.q_next, B.root_next, base + i);
    }
}
__global__ void k_rotate_regen(uint32_t* counters, const BatchChunk* __restrict__ chunk, cudaGraphConditionalHandle h) {
    if (threadIdx.x == 0) {
        const uint32_t next = counters[13];
        const uint32_t nn = min(counters[12], chunk->npaths - next);
        const uint32_t live = counters[1] + nn;
        counters[0] = live;
        counters[13] = next + nn;
        counters[1] = 0u;
        counters[2] = 0u;
        for (int c = 0; c < NUM_CLS; c++) counters[3 + c] = 0u;
        counters[8] = counters[9] = counters[10] = counters[11] = counters[12] = 0u;
        cudaGraphSetConditional(h, live > 0u ? 1u : 0u);
    }
}

// path.rgen:102-112 applied to the chunk's frames in order.
__device__ __forceinline__ void film_frames(const Params& P, const Buffers& B, float4* __restrict__ film, uint32_t pix,
                                            uint32_t frame0, uint32_t nframes, uint32_t path_off) {
    float4 px = film[pix];
    for (uint32_t k = 0; k < nframes; k++) {
        const uint32_t f = frame0 + k;
        const float4 c4 = B.film_src[path_off + (size_t)k * P.npix + pix];
        const v3 col = f3(c4);
        if (P.film_mode == 1u) {
            px = make_float4(col.x, col.y, col.z, 1.0f);
            continue;
        }
        if (isnan(luminance(col))) continue;
        if (f > 0u) {
            const float w = 1.0f / (float)(f + 1u);
            px = make_float4(mixf(px.x, col.x, w), mixf(px.y, col.y, w), mixf(px.z, col.z, w), 1.0f);
        } else {
            px = make_float4(col.x, col.y, col.z, 1.0f);
        }
    }
    film[pix] = px;
}

template <bool BATCH>
__global__ void __launch_bounds__(kThreads) k_film(const Params* __restrict__ Pp, Buffers B) {
    if (BATCH) {
        const BatchChunk& C = *B.chunk;
        if (!C.write_film) return;
        for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < C.npix_total; i += gridDim.x * blockDim.x) {
            const Segment& sg = C.seg[find_segment<true>(C, i)];
            const Params& P = B.jobs[sg.job].P;
            film_frames(P, B, P.film, i - sg.pix_off, sg.frame0, sg.nframes, sg.path_off);
        }
    } else {
        const Params& P = *Pp;
        for (uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x; pix < P.npix; pix += gridDim.x * blockDim.x)
            film_frames(P, B, P.film, pix, P.frame0, P.nframes, 0u);
    }
}

template <bool BATCH>
__global__ void k_init_counters(Buffers B, const Params* __restrict__ Pp) {
    const uint32_t n = BATCH ? min(B.chunk->npaths, B.cap) : Pp->npix * Pp->nframes;
    if (threadIdx.x < 16) B.counters[threadIdx.x] = threadIdx.x == 0 || (BATCH && threadIdx.x == 13) ? n : 0u;
}

__global__ void k_set_params(Params P, Params* dst) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *dst = P;
}

size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

// Carves the work arena for `cap` paths (with the per-path job and per-ray root arrays when `batch`); returns
// the byte size when base is null.
size_t carve(char* base, uint32_t cap, Buffers& B, bool batch = false) {
    size_t off = 0;
    auto take = [&](size_t bytes) { char* p = base ? base + off : nullptr; off += align_up(bytes); return p; };
    B.pix = (uint32_t*)take(4ull * cap);
    B.frame = (uint32_t*)take(4ull * cap);
    B.w = (uint32_t*)take(4ull * cap);
    B.flags = (uint32_t*)take(4ull * cap);
    B.T = (float4*)take(16ull * cap);
    B.col = (float4*)take(16ull * cap);
    B.q_cur = (uint32_t*)take(4ull * cap);
    B.q_next = (uint32_t*)take(4ull * cap);
    B.q_cls = (uint32_t*)take(4ull * NUM_CLS * cap);
    B.rays = (lgb_ray*)take(sizeof(lgb_ray) * (size_t)cap);
    B.rays_next = (lgb_ray*)take(sizeof(lgb_ray) * (size_t)cap);
    B.hits = (lgb_hit*)take(sizeof(lgb_hit) * (size_t)cap);
    B.nee = (NeeRec*)take(sizeof(NeeRec) * (size_t)cap);
    B.srays = (lgb_ray*)take(sizeof(lgb_ray) * (size_t)cap);
    B.mrays = (lgb_ray*)take(sizeof(lgb_ray) * (size_t)cap);
    B.mhits = (lgb_hit*)take(sizeof(lgb_hit) * (size_t)cap);
    B.sbits = (uint32_t*)take(4ull * ((cap + 31) / 32));
    B.counters = (uint32_t*)take(64);
    B.params = (Params*)take(sizeof(Params));
    B.cap = cap;
    B.job = B.root = B.root_next = B.nroot = B.mroot = nullptr;
    B.jobs = nullptr;
    B.chunk = nullptr;
    B.pid = B.done = nullptr;
    B.col_out = nullptr;
    B.film_src = B.col;
    if (batch) {
        B.job = (uint32_t*)take(4ull * cap);
        B.root = (uint32_t*)take(4ull * cap);
        B.root_next = (uint32_t*)take(4ull * cap);
        B.nroot = (uint32_t*)take(4ull * cap);
        B.mroot = (uint32_t*)take(4ull * cap);
        B.jobs = (const JobRec*)take(sizeof(JobRec) * kMaxBatchJobs);
        B.chunk = (const BatchChunk*)take(sizeof(BatchChunk));
        B.pid = (uint32_t*)take(4ull * cap);
        B.done = (uint32_t*)take(4ull * cap);
    }
    return off;
}

// Blocks per SM of the grid-stride path kernels. Cornell box: 674 Msamples/s at 8, 662 at 4, 511 at 2; the
// 32-scene batch prefers 4 (550 against 500 at 8 and 16), which its tuner finds.
#ifdef LGB_WORK_BLOCKS
constexpr int kWorkBlocksPerSm = LGB_WORK_BLOCKS;
#else
constexpr int kWorkBlocksPerSm = 8;
#endif
struct Grids {
    int work, trace;
    bool shared_stack;  // the traversal kernels keep the bottom of their stack in shared memory
    bool incoherent;    // the traversal kernels' incoherent variant (QueueTrace<true>)
};

Grids path_grids(Ctx* ctx, bool shared_stack, bool incoherent) {
    int trace_blocks = 0;  // the same register budget for every variant
    if (shared_stack)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&trace_blocks, k_q_trace_closest<kQueueSharedStack, false>, kThreads, 0);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&trace_blocks, k_q_trace_closest<0, false>, kThreads, 0);
    const int sms = ctx->sm_count > 0 ? ctx->sm_count : 1;
    return Grids{sms * kWorkBlocksPerSm, sms * std::max(trace_blocks, 1), shared_stack, incoherent};
}

template <int SK, bool INC>
void launch_queue_traces(const SceneView& S, const Buffers& B, Grids g, cudaStream_t st, bool first) {
    if (first) {
        k_q_trace_closest<SK, INC><<<g.trace, kThreads, 0, st>>>(S, B.rays, B.hits, B.counters + 0, B.counters + 8, B.root);
    } else {
        k_q_trace_nee<SK, INC><<<g.trace, kThreads, 0, st>>>(S, B.srays, B.sbits, B.counters + 2, B.counters + 9, B.nroot,
                                                             B.mrays, B.mhits, B.counters + 11, B.counters + 10, B.mroot);
    }
}
// first: the continuation rays' closest hits; else the shadow rays and the BSDF-MIS rays of the bounce.
void queue_traces(const SceneView& S, const Buffers& B, Grids g, cudaStream_t st, bool first) {
    if (g.shared_stack) {
        if (g.incoherent) launch_queue_traces<kQueueSharedStack, true>(S, B, g, st, first);
        else launch_queue_traces<kQueueSharedStack, false>(S, B, g, st, first);
    } else {
        if (g.incoherent) launch_queue_traces<0, true>(S, B, g, st, first);
        else launch_queue_traces<0, false>(S, B, g, st, first);
    }
}

// One bounce over the live queue: closest hits, classification, shading per class, shadow and BSDF-MIS traces,
// NEE resolve. `classes` (bit c: shading class c) names the classes the scene's materials fall in; the shading
// kernels of the other classes would always find an empty list and are not launched.
template <bool BATCH>
void launch_bounce(const SceneView& S, const Buffers& B, int depth, Grids g, uint32_t classes, cudaStream_t st) {
    queue_traces(S, B, g, st, true);
    bool sole = false;
    if constexpr (!BATCH) {
        // One shading class (the Cornell box: all diffuse): its kernel takes the queue without k_classify.
        sole = true;
        if (classes == (1u << CLS_DIFFUSE)) k_shade<CLS_DIFFUSE, false, true><<<g.work, kThreads, 0, st>>>(S, B.params, B, depth);
        else if (classes == (1u << CLS_CONDUCTOR)) k_shade<CLS_CONDUCTOR, false, true><<<g.work, kThreads, 0, st>>>(S, B.params, B, depth);
        else if (classes == (1u << CLS_SPECULAR)) k_shade<CLS_SPECULAR, false, true><<<g.work, kThreads, 0, st>>>(S, B.params, B, depth);
        else if (classes == (1u << CLS_PRINCIPLED)) k_shade<CLS_PRINCIPLED, false, true><<<g.work, kThreads, 0, st>>>(S, B.params, B, depth);
        else sole = false;
    }
    if (!sole) {
        k_classify<BATCH><<<g.work, kThreads, 0, st>>>(S, B.params, B);
        if (classes & (1u << CLS_DIFFUSE)) k_shade<CLS_DIFFUSE, BATCH><<<g.work, kThreads, 0, st>>>(S, B.params, B, depth);
        if (classes & (1u << CLS_CONDUCTOR)) k_shade<CLS_CONDUCTOR, BATCH><<<g.work, kThreads, 0, st>>>(S, B.params, B, depth);
        if (classes & (1u << CLS_SPECULAR)) k_shade<CLS_SPECULAR, BATCH><<<g.work, kThreads, 0, st>>>(S, B.params, B, depth);
        if (classes & (1u << CLS_PRINCIPLED)) k_shade<CLS_PRINCIPLED, BATCH><<<g.work, kThreads, 0, st>>>(S, B.params, B, depth);
    }
    queue_traces(S, B, g, st, false);
    k_nee_resolve<BATCH><<<g.work, kThreads, 0, st>>>(S, B);
}

void swap_queues(Buffers& B) {
    std::swap(B.rays, B.rays_next);
    std::swap(B.q_cur, B.q_next);
    std::swap(B.root, B.root_next);
}

// One chunk of frames that fits the arena: camera rays, `bounces` bounces, film. Every kernel reads its
// parameters from device memory (B.params, or the job table and chunk record when batched), so this sequence can
// be captured once and replayed with new parameters.
template <bool BATCH>
cudaError_t launch_chunk(const SceneView& S, Buffers B, int bounces, Grids g, uint32_t classes, cudaStream_t st) {
    k_init_counters<BATCH><<<1, 32, 0, st>>>(B, B.params);
    k_camera<BATCH><<<g.work, kThreads, 0, st>>>(B.params, B);
    for (int depth = 0; depth < bounces; depth++) {
        launch_bounce<BATCH>(S, B, depth, g, classes, st);
        k_rotate<<<1, 32, 0, st>>>(B.counters);
        swap_queues(B);
    }
    k_film<BATCH><<<g.work, kThreads, 0, st>>>(B.params, B);
    return cudaGetLastError();
}

// The body of a regenerating chunk's bounce loop: two bounces (the ray queues alternate between them), each
// followed by regeneration and the queue rotation that sets the loop's condition (some path still live). A
// bounce over an empty queue finds every count zero and does nothing.
cudaError_t launch_regen_bounces(const SceneView& S, Buffers B, Grids g, uint32_t classes,
                                 cudaGraphConditionalHandle h, cudaStream_t st) {
    for (int k = 0; k < 2; k++) {
        launch_bounce<true>(S, B, 0, g, classes, st);
        k_regen<<<g.work, kThreads, 0, st>>>(B);
        k_rotate_regen<<<1, 32, 0, st>>>(B.counters, B.chunk, h);
        swap_queues(B);
    }
    return cudaGetLastError();
}


uint32_t batch_classes(const Batch* b) {
    uint32_t c = 0;
    for (const Scene* s : b->scenes) c |= s->shade_classes;
    return c;
}

Params make_params(const lgb_camera* cam, const lgb_path_params* pp, uint32_t cap, float* film) {
    Params P;
    for (int i = 0; i < 16; i++) { P.iv[i] = cam->inv_view[i]; P.ip[i] = cam->inv_projection[i]; }
    P.width = cam->width; P.height = cam->height; P.npix = cam->width * cam->height;
    for (int i = 0; i < 3; i++) P.sky[i] = pp->sky_col[i];
    P.max_depth = pp->max_depth; P.num_lights = pp->num_lights; P.light_tri_count = pp->light_triangle_count;
    P.direct_lighting = pp->direct_lighting; P.film_mode = pp->film_mode;
    P.cap = cap;
    P.film = reinterpret_cast<float4*>(film);
    P.frame0 = 0;
    P.nframes = 0;
    return P;
}

}  // namespace

lgb_status render_path(Scene* s, const lgb_camera* cam, const lgb_path_params* pp, uint32_t frame0, uint32_t spp,
                       float* film, cudaStream_t st) {
    Ctx* ctx = s->ctx;
    const uint32_t npix = cam->width * cam->height;
    if ((uint64_t)cam->width * cam->height > kMaxPaths)
        return set_error(ctx, LGB_ERR_UNSUPPORTED, "image larger than the path capacity (2^21 pixels)");
    const uint32_t frames_per_chunk = std::max(1u, std::min(spp, kMaxPaths / npix));
    const uint32_t cap = npix * frames_per_chunk;
    Buffers B;
    const size_t bytes = carve(nullptr, cap, B);
    if (s->pt_buf_bytes < bytes) {
        if (s->pt_graph) { cudaGraphExecDestroy((cudaGraphExec_t)s->pt_graph); s->pt_graph = nullptr; }
        cudaFree(s->pt_buf);
        s->pt_buf = nullptr;
        s->pt_buf_bytes = 0;
        LGB_CUDA_TRY(ctx, cudaMalloc(&s->pt_buf, bytes));
        s->pt_buf_bytes = bytes;
    }
    carve((char*)s->pt_buf, cap, B);
    const SceneView S = scene_view(s);
    Params P = make_params(cam, pp, cap, film);
    const Grids g = path_grids(ctx, false, s->num_tris >= kIncoherentTris);
    const int bounces = std::max(pp->max_depth, 1);
    // The bounce loop of a chunk is captured once into a CUDA graph and replayed; the graph depends only on the
    // arena layout, the scene's device arrays and the bounce count, while everything per call travels in
    // B.params. If the caller is itself capturing this stream, the kernels are issued directly into its capture.
    cudaStreamCaptureStatus cap_status = cudaStreamCaptureStatusNone;
    LGB_CUDA_TRY(ctx, cudaStreamIsCapturing(st, &cap_status));
    const bool use_graph = cap_status == cudaStreamCaptureStatusNone;
    const uint64_t key[6] = {(uint64_t)(uintptr_t)s->pt_buf, cap,
                             (uint64_t)bounces | ((uint64_t)g.incoherent << 32) | ((uint64_t)s->shade_classes << 40),
                             (uint64_t)(uintptr_t)S.nodes,
                             (uint64_t)(uintptr_t)S.tris, ((uint64_t)g.work << 32) | (uint32_t)g.trace};
    if (use_graph && (!s->pt_graph || std::memcmp(key, s->pt_graph_key, sizeof(key)) != 0)) {
        if (s->pt_graph) { cudaGraphExecDestroy((cudaGraphExec_t)s->pt_graph); s->pt_graph = nullptr; }
        if (!s->capture_stream) LGB_CUDA_TRY(ctx, cudaStreamCreateWithFlags((cudaStream_t*)&s->capture_stream, cudaStreamNonBlocking));
        const cudaStream_t cs = (cudaStream_t)s->capture_stream;
        cudaGraph_t graph = nullptr;
        LGB_CUDA_TRY(ctx, cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
        const cudaError_t le = launch_chunk<false>(S, B, bounces, g, s->shade_classes, cs);
        const cudaError_t ce = cudaStreamEndCapture(cs, &graph);
        if (le != cudaSuccess) { if (graph) cudaGraphDestroy(graph); return cuda_error(ctx, le, "capturing the bounce loop"); }
        if (ce != cudaSuccess) return cuda_error(ctx, ce, "cudaStreamEndCapture");
        cudaGraphExec_t exec = nullptr;
        const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) return cuda_error(ctx, ie, "cudaGraphInstantiate");
        s->pt_graph = exec;
        std::memcpy(s->pt_graph_key, key, sizeof(key));
    }
    for (uint32_t done = 0; done < spp; done += frames_per_chunk) {
        P.frame0 = frame0 + done;
        P.nframes = std::min(frames_per_chunk, spp - done);
        k_set_params<<<1, 1, 0, st>>>(P, B.params);
        if (use_graph) {
            LGB_CUDA_TRY(ctx, cudaGraphLaunch((cudaGraphExec_t)s->pt_graph, st));
        } else {
            LGB_CUDA_TRY(ctx, launch_chunk<false>(S, B, bounces, g, s->shade_classes, st));
        }
    }
    LGB_CUDA_TRY(ctx, cudaGetLastError());
    return LGB_OK;
}

}  // namespace lgb

// ---------------------------------------------------------------------------------------------------------
// lgb_render_path_noalloc: the same path integrator with its work arena in a fixed device array.
//
// Who needs it: callers that cannot call cudaMalloc while they render. A real-time host that budgets all
// device memory up front (its own pool, a fixed VRAM budget) cannot let a library allocate in the middle of
// a frame, where an allocation can fail or stall; cudaFree also synchronises the whole device, which would
// stall the caller's other streams. lgb_render_path grows its arena with cudaMalloc on first use; this entry
// point never allocates and instead uses the static array below.
//
// Limit: at most kNoAllocPaths paths in flight, so images of at most 16384 pixels (for example 128 x 128);
// more samples per pixel are rendered in successive chunks of whole frames.
// Every GPU that loads the library holds the array (6 MiB) until the process exits. All calls share it, so
// calls that overlap on the GPU (another stream, another thread) race on it; order them on one stream.
// The first call on a device takes the array's address there (cudaGetSymbolAddress); make that first call
// before any stream capture. The address is kept for the life of the process, so it is stale after a
// cudaDeviceReset that recreates the device's primary context.
// ---------------------------------------------------------------------------------------------------------
namespace lgb {
namespace {

constexpr uint32_t kNoAllocPaths = 16384;
constexpr size_t kNoAllocBytes = (size_t)6 << 20;
static __device__ __align__(256) unsigned char g_noalloc_arena[kNoAllocBytes];

constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_ptr[kMaxDevices] = {};

// Host address of g_noalloc_arena on `device` (current), looked up once per device.
lgb_status noalloc_arena(Ctx* ctx, int device, char** out) {
    if (device < 0 || device >= kMaxDevices)
        return set_error(ctx, LGB_ERR_UNSUPPORTED, "device index too large for the no-alloc arena table");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_arena);
        if (e != cudaSuccess) return cuda_error(ctx, e, "cudaGetSymbolAddress(g_noalloc_arena)");
        g_noalloc_ptr[device] = p;
    }
    *out = (char*)g_noalloc_ptr[device];
    return LGB_OK;
}

lgb_status render_path_noalloc(Scene* s, const lgb_camera* cam, const lgb_path_params* pp, uint32_t frame0,
                               uint32_t spp, float* film, cudaStream_t st) {
    Ctx* ctx = s->ctx;
    const uint64_t npix64 = (uint64_t)cam->width * cam->height;
    if (npix64 > kNoAllocPaths)
        return set_error(ctx, LGB_ERR_INVALID_ARGUMENT,
                         "lgb_render_path_noalloc renders at most 16384 pixels per image (its fixed arena holds "
                         "16384 paths); use lgb_render_path for larger images");
    const uint32_t npix = (uint32_t)npix64;
    const uint32_t frames_per_chunk = std::max(1u, std::min(spp, kNoAllocPaths / npix));
    const uint32_t cap = npix * frames_per_chunk;
    Buffers B;
    if (carve(nullptr, cap, B) > kNoAllocBytes)
        return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "no-alloc arena too small for this launch");
    char* arena = nullptr;
    lgb_status ast = noalloc_arena(ctx, ctx->device, &arena);
    if (ast != LGB_OK) return ast;
    carve(arena, cap, B);
    const SceneView S = scene_view(s);
    Params P = make_params(cam, pp, cap, film);
    const Grids g = path_grids(ctx, false, s->num_tris >= kIncoherentTris);
    const int bounces = std::max(pp->max_depth, 1);
    for (uint32_t done = 0; done < spp; done += frames_per_chunk) {
        P.frame0 = frame0 + done;
        P.nframes = std::min(frames_per_chunk, spp - done);
        // The arena keeps the previous call's contents: the parameters and counters are rewritten here, the
        // occlusion bits before every shadow query, and every other array is written before it is read.
        k_set_params<<<1, 1, 0, st>>>(P, B.params);
        LGB_CUDA_TRY(ctx, launch_chunk<false>(S, B, bounces, g, s->shade_classes, st));
    }
    return LGB_OK;
}

}  // namespace
}  // namespace lgb

extern "C" LGB_API lgb_status lgb_render_path_noalloc(lgb_scene* s, const lgb_camera* cam, const lgb_path_params* p,
                                                      uint32_t frame0, uint32_t spp, float* d_film, void* stream) {
    using namespace lgb;
    if (!s) return LGB_ERR_INVALID_ARGUMENT;
    if (!cam || !p || !d_film || cam->width == 0 || cam->height == 0)
        return set_error(s->ctx, LGB_ERR_INVALID_ARGUMENT, "null camera, params or film");
    if (reinterpret_cast<uintptr_t>(d_film) & 15u)
        return set_error(s->ctx, LGB_ERR_INVALID_ARGUMENT, "film must be 16-byte aligned");
    if (!s->bvh.nodes) return set_error(s->ctx, LGB_ERR_NOT_READY, "lgb_bvh_build has not been called");
    if (p->num_lights < 0 || (uint32_t)p->num_lights > s->num_lights)
        return set_error(s->ctx, LGB_ERR_INVALID_ARGUMENT, "num_lights exceeds the scene's light count");
    if (p->num_lights > 0 && p->light_triangle_count <= 0)
        return set_error(s->ctx, LGB_ERR_INVALID_ARGUMENT, "light_triangle_count must be positive");
    if (p->dir_light_idx != 0xFFFFFFFFu)
        return set_error(s->ctx, LGB_ERR_UNSUPPORTED, "atmosphere shading for directional lights is not supported");
    if (spp == 0) return LGB_OK;
    if (cudaSetDevice(s->ctx->device) != cudaSuccess) return set_error(s->ctx, LGB_ERR_CUDA, "cudaSetDevice failed");
    return render_path_noalloc(s, cam, p, frame0, spp, d_film, (cudaStream_t)stream);
}

// ---------------------------------------------------------------------------------------------------------
// Batched rendering (lgb_batch_*): the path integrator above over many jobs at once. The BVHs of the batch's
// scenes are copied into one forest with relocated node and triangle indices, so the traversal kernels keep
// one node array and one triangle array and each ray carries only its root node; the shading kernels find
// their scene, camera and film through the job of the path.
// ---------------------------------------------------------------------------------------------------------
namespace lgb {
namespace {

constexpr uint32_t kBatchDefaultCap = 1u << 21;
constexpr uint32_t kBatchMaxCap = 1u << 24;
#ifdef LGB_BATCH_CHUNK_PATHS
constexpr uint64_t kBatchChunkPaths = LGB_BATCH_CHUNK_PATHS;
#else
constexpr uint64_t kBatchChunkPaths = 16;             // default regenerating chunk: 16 x the path capacity
#endif
constexpr uint64_t kBatchMaxChunkPaths = 1ull << 27;  // 2 GB of radiance output

__global__ void k_relocate(const WideNode* __restrict__ src, uint32_t n, uint32_t node_off, uint32_t tri_off,
                           WideNode* __restrict__ dst) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        WideNode w = src[i];
        w.child_base += node_off;
        w.tri_base += tri_off;
        dst[i] = w;
    }
}

// The device-driven chunk loop of a batch render: the body of the graph's WHILE node starts by copying chunk
// loop[0] of the uploaded records into the chunk record the kernels read, and ends by advancing loop[0] and
// setting the loop condition to loop[0] < loop[1]. loop[0] grows by one per iteration and loop[1] is the
// chunk count of the call, so the loop runs exactly that many times.
__global__ void k_next_chunk(const BatchChunk* __restrict__ chunks, const uint32_t* __restrict__ loop, BatchChunk* dst) {
    const uint32_t* src = reinterpret_cast<const uint32_t*>(chunks + loop[0]);
    uint32_t* d = reinterpret_cast<uint32_t*>(dst);
    constexpr uint32_t words = sizeof(BatchChunk) / 4;
    static_assert(sizeof(BatchChunk) % 4 == 0, "chunk record of whole words");
    for (uint32_t i = threadIdx.x; i < words; i += blockDim.x) d[i] = src[i];
}
__global__ void k_loop_next(cudaGraphConditionalHandle h, uint32_t* loop) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const uint32_t next = loop[0] + 1u;
        loop[0] = next;
        cudaGraphSetConditional(h, next < loop[1] ? 1u : 0u);
    }
}
__global__ void k_loop_init(uint32_t* loop, uint32_t n) {
    if (threadIdx.x == 0 && blockIdx.x == 0) { loop[0] = 0u; loop[1] = n; }
}
// Enters a regenerating chunk's bounce loop while it has live paths.
__global__ void k_bounce_loop_begin(cudaGraphConditionalHandle h, const uint32_t* counters) {
    if (threadIdx.x == 0 && blockIdx.x == 0) cudaGraphSetConditional(h, counters[0] > 0u ? 1u : 0u);
}

// Adds a WHILE node with handle `h` (created on `g`) to graph `g` after `deps`; returns its body graph.
cudaError_t add_while(cudaGraph_t g, const cudaGraphNode_t* deps, size_t ndeps, cudaGraphConditionalHandle h,
                      cudaGraphNode_t* node, cudaGraph_t* body) {
    cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};  // the remaining fields zero
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    const cudaError_t e = cudaGraphAddNode(node, g, deps, nullptr, ndeps, &np);
    if (e == cudaSuccess) *body = np.conditional.phGraph_out[0];
    return e;
}

// The graph of one batch render: a WHILE loop over the call's chunk records. Without regeneration its body is
// k_next_chunk, the captured fixed bounce loop of launch_chunk and k_loop_next. With regeneration (B.col_out
// set) the body starts the chunk's first paths, runs a nested WHILE loop of bounces with regeneration until no
// path is live, then writes the films.
cudaError_t build_batch_graph(Batch* b, const SceneView& F, const Buffers& B, int bounces, Grids g, uint32_t classes,
                              cudaStream_t cs, cudaGraphExec_t* out) {
    cudaStream_t cs2 = nullptr;  // captures the nested loop's body while cs captures the outer body
    cudaError_t e = B.col_out ? cudaStreamCreateWithFlags(&cs2, cudaStreamNonBlocking) : cudaSuccess;
    if (e != cudaSuccess) return e;
    cudaGraph_t top = nullptr;
    e = cudaGraphCreate(&top, 0);
    if (e != cudaSuccess) { if (cs2) cudaStreamDestroy(cs2); return e; }
    cudaGraphConditionalHandle cond;
    cudaGraphNode_t loop_node = nullptr;
    cudaGraph_t body = nullptr;
    e = cudaGraphConditionalHandleCreate(&cond, top, 1u, cudaGraphCondAssignDefault);
    if (e == cudaSuccess) e = add_while(top, nullptr, 0, cond, &loop_node, &body);
    if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        cudaGraphDestroy(top);
        if (cs2) cudaStreamDestroy(cs2);
        return e;
    }
    cudaGraph_t captured = nullptr;
    k_next_chunk<<<1, 256, 0, cs>>>(reinterpret_cast<const BatchChunk*>(b->d_chunks), b->d_loop,
                                    const_cast<BatchChunk*>(B.chunk));
    if (!B.col_out) {
        e = launch_chunk<true>(F, B, bounces, g, classes, cs);
    } else {
        k_init_counters<true><<<1, 32, 0, cs>>>(B, B.params);
        k_camera<true><<<g.work, kThreads, 0, cs>>>(B.params, B);
        // the nested bounce loop, added to the body after what has been captured so far
        cudaGraphConditionalHandle inner;
        cudaStreamCaptureStatus cst;
        cudaGraph_t cg = nullptr;
        const cudaGraphNode_t* deps = nullptr;
        size_t nd = 0;
        cudaGraphNode_t inner_node = nullptr;
        cudaGraph_t inner_body = nullptr;
        e = cudaStreamGetCaptureInfo(cs, &cst, nullptr, &cg, &deps, nullptr, &nd);
        if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&inner, cg, 0u, 0u);
        if (e == cudaSuccess) {
            k_bounce_loop_begin<<<1, 32, 0, cs>>>(inner, B.counters);
            e = cudaStreamGetCaptureInfo(cs, &cst, nullptr, &cg, &deps, nullptr, &nd);
        }
        if (e == cudaSuccess) e = add_while(cg, deps, nd, inner, &inner_node, &inner_body);
        if (e == cudaSuccess) e = cudaStreamUpdateCaptureDependencies(cs, &inner_node, nullptr, 1, cudaStreamSetCaptureDependencies);
        if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(cs2, inner_body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            const cudaError_t le = launch_regen_bounces(F, B, g, classes, inner, cs2);
            cudaGraph_t ig = nullptr;
            const cudaError_t ce = cudaStreamEndCapture(cs2, &ig);
            e = le != cudaSuccess ? le : ce;
        }
        if (e == cudaSuccess) {
            k_film<true><<<g.work, kThreads, 0, cs>>>(B.params, B);
            e = cudaGetLastError();
        }
    }
    k_loop_next<<<1, 32, 0, cs>>>(cond, b->d_loop);
    if (e == cudaSuccess) e = cudaGetLastError();
    const cudaError_t ce = cudaStreamEndCapture(cs, &captured);
    if (e == cudaSuccess) e = ce;
    if (cs2) cudaStreamDestroy(cs2);
    cudaGraphExec_t exec = nullptr;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, top, 0);
    cudaGraphDestroy(top);
    if (e == cudaSuccess) *out = exec;
    return e;
}

void free_batch(Batch* b) {
    cudaSetDevice(b->ctx->device);
    if (b->graph) cudaGraphExecDestroy((cudaGraphExec_t)b->graph);
    if (b->capture_stream) cudaStreamDestroy((cudaStream_t)b->capture_stream);
    if (b->staging_event) {
        cudaEventSynchronize((cudaEvent_t)b->staging_event);
        cudaEventDestroy((cudaEvent_t)b->staging_event);
    }
    if (b->staging) cudaFreeHost(b->staging);
    if (b->chunk_staging) cudaFreeHost(b->chunk_staging);
    cudaFree(b->d_chunks);
    cudaFree(b->d_loop);
    cudaFree(b->col_out);
    cudaFree(b->buf);
    cudaFree(b->nodes);
    cudaFree(b->tris);
    cudaFree(b->d_status);
}

lgb_status batch_create(Ctx* ctx, Scene* const* scenes, uint32_t n, Batch* b) {
    b->ctx = ctx;
    uint64_t nodes = 0, tris = 0;
    for (uint32_t i = 0; i < n; i++) {
        Scene* s = scenes[i];
        if (!s || s->ctx != ctx) return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "scene " + std::to_string(i) + " is null or of another context");
        if (!s->bvh.nodes || s->bvh.num_nodes == 0)
            return set_error(ctx, LGB_ERR_NOT_READY, "scene " + std::to_string(i) + " has no BVH (lgb_bvh_build)");
        b->scenes.push_back(s);
        b->roots.push_back((uint32_t)nodes);
        b->bvh_generation.push_back(s->bvh.generation);
        nodes += s->bvh.num_nodes;
        tris += s->bvh.num_tris;
    }
    if (nodes >= 0x7fffffffull || tris >= 0x7fffffffull)
        return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "the batch's BVHs exceed 2^31 nodes or triangles");
    b->num_nodes = (uint32_t)nodes;
    b->num_tris = (uint32_t)tris;
    LGB_CUDA_TRY(ctx, cudaMalloc(&b->nodes, sizeof(WideNode) * std::max<uint64_t>(nodes, 1)));
    LGB_CUDA_TRY(ctx, cudaMalloc(&b->tris, sizeof(WideTri) * std::max<uint64_t>(tris, 1)));
    LGB_CUDA_TRY(ctx, cudaMalloc(&b->d_status, sizeof(uint32_t)));
    LGB_CUDA_TRY(ctx, cudaMemset(b->d_status, 0, sizeof(uint32_t)));
    uint32_t tri_off = 0;
    const int sms = ctx->sm_count > 0 ? ctx->sm_count : 1;
    for (uint32_t i = 0; i < n; i++) {
        const Scene* s = b->scenes[i];
        const uint32_t nn = s->bvh.num_nodes, nt = s->bvh.num_tris;
        if (nn) k_relocate<<<std::min<uint32_t>((nn + 255) / 256, sms * 8), 256>>>(s->bvh.nodes, nn, b->roots[i], tri_off,
                                                                             b->nodes + b->roots[i]);
        if (nt) LGB_CUDA_TRY(ctx, cudaMemcpy(b->tris + tri_off, s->bvh.tris, sizeof(WideTri) * nt, cudaMemcpyDeviceToDevice));
        tri_off += nt;
    }
    LGB_CUDA_TRY(ctx, cudaGetLastError());
    LGB_CUDA_TRY(ctx, cudaDeviceSynchronize());
    LGB_CUDA_TRY(ctx, cudaMallocHost(&b->staging, sizeof(JobRec) * kMaxBatchJobs));
    LGB_CUDA_TRY(ctx, cudaMalloc(&b->d_loop, 2 * sizeof(uint32_t)));
    cudaEvent_t ev;
    LGB_CUDA_TRY(ctx, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    b->staging_event = ev;
    LGB_CUDA_TRY(ctx, cudaEventRecord(ev, 0));
    return LGB_OK;
}

lgb_status check_jobs(Batch* b, const lgb_batch_job* jobs, uint32_t n) {
    Ctx* ctx = b->ctx;
    if (!jobs || n == 0 || n > kMaxBatchJobs)
        return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "between 1 and 128 jobs per batch call");
    for (size_t i = 0; i < b->scenes.size(); i++)
        if (b->scenes[i]->bvh.generation != b->bvh_generation[i])
            return set_error(ctx, LGB_ERR_NOT_READY, "scene " + std::to_string(i) + " was rebuilt after lgb_batch_create");
    for (uint32_t i = 0; i < n; i++) {
        const lgb_batch_job& j = jobs[i];
        const std::string id = "job " + std::to_string(i) + ": ";
        if (j.scene >= b->scenes.size()) return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, id + "scene index out of range");
        const Scene* s = b->scenes[j.scene];
        const lgb_path_params& p = j.params;
        if (!j.d_film || (reinterpret_cast<uintptr_t>(j.d_film) & 15u) || j.camera.width == 0 || j.camera.height == 0)
            return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, id + "null or misaligned film, or empty image");
        if ((uint64_t)j.camera.width * j.camera.height > kBatchMaxCap)
            return set_error(ctx, LGB_ERR_UNSUPPORTED, id + "image larger than 2^24 pixels");
        if (p.num_lights < 0 || (uint32_t)p.num_lights > s->num_lights)
            return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, id + "num_lights exceeds the scene's light count");
        if (p.num_lights > 0 && p.light_triangle_count <= 0)
            return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, id + "light_triangle_count must be positive");
        if (p.dir_light_idx != 0xFFFFFFFFu)
            return set_error(ctx, LGB_ERR_UNSUPPORTED, id + "atmosphere shading for directional lights is not supported");
    }
    return LGB_OK;
}

// Cuts the jobs into chunks of at most `cap` paths, each a list of whole-frame segments. A job's frames are
// taken in order, as many as fit; a chunk that cannot take one more frame of the current job is closed, so
// a job appears at most once per chunk and its chunks run in frame order.
void plan_chunks(const lgb_batch_job* jobs, uint32_t n, uint32_t cap, bool write_film, std::vector<BatchChunk>& out) {
    BatchChunk C;
    std::memset(&C, 0, sizeof(C));
    C.write_film = write_film ? 1u : 0u;
    auto flush = [&]() {
        if (C.nseg) out.push_back(C);
        std::memset(&C, 0, sizeof(C));
        C.write_film = write_film ? 1u : 0u;
    };
    for (uint32_t j = 0; j < n; j++) {
        const uint32_t npix = jobs[j].camera.width * jobs[j].camera.height;
        uint32_t f = jobs[j].frame0, left = jobs[j].spp;
        while (left > 0) {
            const uint32_t k = std::min(left, (cap - C.npaths) / npix);
            if (k == 0) { flush(); continue; }
            Segment& sg = C.seg[C.nseg++];
            sg.job = j; sg.frame0 = f; sg.nframes = k; sg.path_off = C.npaths; sg.pix_off = C.npix_total; sg.npix = npix;
            C.npaths += k * npix;
            C.npix_total += npix;
            f += k;
            left -= k;
            if (C.nseg == kMaxBatchJobs) flush();
        }
    }
    flush();
}

lgb_status batch_render(Batch* b, const lgb_batch_job* jobs, uint32_t n, const lgb_batch_opts& o, bool write_film,
                        cudaStream_t st) {
    Ctx* ctx = b->ctx;
    // A call is one launch of the batch's own graph, whose job table and chunk records are uploaded from pinned
    // staging on the stream; inside a caller's capture those uploads would replay whatever the staging holds then.
    cudaStreamCaptureStatus cap_status = cudaStreamCaptureStatusNone;
    LGB_CUDA_TRY(ctx, cudaStreamIsCapturing(st, &cap_status));
    if (cap_status != cudaStreamCaptureStatusNone)
        return set_error(ctx, LGB_ERR_UNSUPPORTED, "lgb_batch_render cannot be captured: each call is one launch of its own graph");
    uint32_t max_npix = 1;
    int bounces = 1;
    for (uint32_t j = 0; j < n; j++) {
        max_npix = std::max(max_npix, jobs[j].camera.width * jobs[j].camera.height);
        bounces = std::max(bounces, jobs[j].params.max_depth);
    }
    uint32_t cap = o.path_capacity ? o.path_capacity : kBatchDefaultCap;
    cap = std::min(std::max(cap, max_npix), kBatchMaxCap);
    Buffers B;
    const size_t bytes = carve(nullptr, cap, B, true);
    if (b->buf_bytes < bytes) {
        if (b->graph) { cudaGraphExecDestroy((cudaGraphExec_t)b->graph); b->graph = nullptr; }
        cudaFree(b->buf);
        b->buf = nullptr;
        b->buf_bytes = 0;
        LGB_CUDA_TRY(ctx, cudaMalloc(&b->buf, bytes));
        b->buf_bytes = bytes;
    }
    carve((char*)b->buf, cap, B, true);
    const int sms = ctx->sm_count > 0 ? ctx->sm_count : 1;
    if (o.stack_placement > LGB_STACK_SHARED)
        return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "stack_placement must be LGB_STACK_LOCAL or LGB_STACK_SHARED");
    if (o.traversal > LGB_TRAVERSAL_INCOHERENT)
        return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "traversal must be LGB_TRAVERSAL_AUTO, _COHERENT or _INCOHERENT");
    const bool incoherent = o.traversal == LGB_TRAVERSAL_AUTO ? b->num_tris >= kIncoherentTris
                                                               : o.traversal == LGB_TRAVERSAL_INCOHERENT;
    Grids g = path_grids(ctx, o.stack_placement == LGB_STACK_SHARED, incoherent);
    if (o.work_blocks_per_sm) g.work = sms * (int)std::min(o.work_blocks_per_sm, 64u);
    if (o.trace_blocks_per_sm) g.trace = std::min(g.trace, sms * (int)o.trace_blocks_per_sm);

    // Job table: staged in pinned memory (after the previous upload has left it) and copied on the stream.
    LGB_CUDA_TRY(ctx, cudaEventSynchronize((cudaEvent_t)b->staging_event));
    JobRec* stage = reinterpret_cast<JobRec*>(b->staging);
    for (uint32_t j = 0; j < n; j++) {
        std::memset(&stage[j], 0, sizeof(JobRec));
        stage[j].P = make_params(&jobs[j].camera, &jobs[j].params, cap, jobs[j].d_film);
        stage[j].S = scene_view(b->scenes[jobs[j].scene]);
        stage[j].root = b->roots[jobs[j].scene];
    }
    LGB_CUDA_TRY(ctx, cudaMemcpyAsync(const_cast<JobRec*>(B.jobs), stage, sizeof(JobRec) * n, cudaMemcpyHostToDevice, st));
    // Path regeneration (in the call's own graph): chunks of up to chunk_paths paths run through the arena's `cap`
    // slots, each ended path's slot taking the chunk's next path, so the queues stay full until the chunk's last
    // paths; the radiance of every path goes to col_out for the film.
    const bool regen = !b->regen_refused && o.chunk_paths != 1u;
    uint64_t chunk_limit = cap;
    if (regen) {
        const uint64_t want = o.chunk_paths > 1u ? o.chunk_paths : kBatchChunkPaths * (uint64_t)cap;
        chunk_limit = std::max<uint64_t>(cap, std::min<uint64_t>(want, kBatchMaxChunkPaths));
    }
    std::vector<BatchChunk> chunks;
    plan_chunks(jobs, n, (uint32_t)chunk_limit, write_film, chunks);
    const uint32_t nch = (uint32_t)chunks.size();
    if (regen) {
        uint64_t most = 0;
        for (const BatchChunk& C : chunks) most = std::max<uint64_t>(most, C.npaths);
        if (b->col_out_paths < most) {
            if (b->graph) { cudaGraphExecDestroy((cudaGraphExec_t)b->graph); b->graph = nullptr; }
            cudaFree(b->col_out);
            b->col_out = nullptr;
            b->col_out_paths = 0;
            LGB_CUDA_TRY(ctx, cudaMalloc(&b->col_out, sizeof(float4) * most));
            b->col_out_paths = most;
        }
        B.col_out = reinterpret_cast<float4*>(b->col_out);
        B.film_src = B.col_out;
    }
    if (nch > 0) {
        // The chunk records, staged in pinned memory (free once the previous call's uploads are done, which the
        // staging event waited for above) and uploaded on the stream for the graph's device-driven loop.
        if (nch > b->chunk_cap) {
            if (b->graph) { cudaGraphExecDestroy((cudaGraphExec_t)b->graph); b->graph = nullptr; }
            if (b->chunk_staging) cudaFreeHost(b->chunk_staging);
            b->chunk_staging = nullptr;
            cudaFree(b->d_chunks);
            b->d_chunks = nullptr;
            b->chunk_cap = 0;
            const uint32_t want = std::max(nch, 16u);
            LGB_CUDA_TRY(ctx, cudaMalloc(&b->d_chunks, sizeof(BatchChunk) * want));
            LGB_CUDA_TRY(ctx, cudaMallocHost(&b->chunk_staging, sizeof(BatchChunk) * want));
            b->chunk_cap = want;
        }
        std::memcpy(b->chunk_staging, chunks.data(), sizeof(BatchChunk) * nch);
        LGB_CUDA_TRY(ctx, cudaMemcpyAsync(b->d_chunks, b->chunk_staging, sizeof(BatchChunk) * nch, cudaMemcpyHostToDevice, st));
    }
    LGB_CUDA_TRY(ctx, cudaEventRecord((cudaEvent_t)b->staging_event, st));

    SceneView F;
    std::memset(&F, 0, sizeof(F));
    F.nodes = b->nodes;
    F.tris = b->tris;
    F.status = b->d_status;
    if (nch == 0) return LGB_OK;
    // One graph renders every chunk of the call (build_batch_graph). It depends on the arena, the forest, the
    // bounce count, the grids, the chunk-record array and the regeneration output, not on the jobs.
    const uint64_t key[10] = {(uint64_t)(uintptr_t)b->buf, cap,
                              (uint64_t)bounces | ((uint64_t)g.shared_stack << 32) | ((uint64_t)g.incoherent << 33) |
                                  ((uint64_t)batch_classes(b) << 40),
                              (uint64_t)(uintptr_t)b->nodes, (uint64_t)(uintptr_t)b->tris,
                              ((uint64_t)g.work << 32) | (uint32_t)g.trace, (uint64_t)(uintptr_t)b->d_chunks,
                              (uint64_t)(uintptr_t)b->d_loop, (uint64_t)(uintptr_t)B.col_out, regen ? 1u : 0u};
    if (!b->graph || std::memcmp(key, b->graph_key, sizeof(key)) != 0) {
        if (b->graph) { cudaGraphExecDestroy((cudaGraphExec_t)b->graph); b->graph = nullptr; }
        if (!b->capture_stream) LGB_CUDA_TRY(ctx, cudaStreamCreateWithFlags((cudaStream_t*)&b->capture_stream, cudaStreamNonBlocking));
        cudaGraphExec_t exec = nullptr;
        cudaError_t e = build_batch_graph(b, F, B, bounces, g, batch_classes(b), (cudaStream_t)b->capture_stream, &exec);
        if (e != cudaSuccess && regen) {
            // A device or driver without nested conditional loops: render this and later calls without
            // regeneration (the chunks are re-planned to fit the arena).
            cudaGetLastError();
            b->regen_refused = true;
            return batch_render(b, jobs, n, o, write_film, st);
        }
        if (e != cudaSuccess) return cuda_error(ctx, e, "building the batch render graph");
        b->graph = exec;
        std::memcpy(b->graph_key, key, sizeof(key));
    }
    k_loop_init<<<1, 1, 0, st>>>(b->d_loop, nch);
    LGB_CUDA_TRY(ctx, cudaGraphLaunch((cudaGraphExec_t)b->graph, st));
    LGB_CUDA_TRY(ctx, cudaGetLastError());
    return LGB_OK;
}

// ---- the tuning cache (lgb_create's tuning_cache_path) ----
// One line per choice: "<key> <path_capacity> <work_blocks_per_sm> <trace_blocks_per_sm> <stack_placement>
// <chunk_paths> <traversal>". The
// key names the device (name, SM count, compute capability), the ABI version and the batch's shape: job count,
// and the powers of two of its samples, of its largest image and of its triangles, its deepest path and the union
// of its scenes' BSDF types. A later line replaces an earlier one with the same key.
std::string tune_key(const Batch* b, const lgb_batch_job* jobs, uint32_t n) {
    cudaDeviceProp prop;
    std::memset(&prop, 0, sizeof(prop));
    cudaGetDeviceProperties(&prop, b->ctx->device);
    std::string dev = prop.name;
    for (char& ch : dev)
        if (ch == ' ' || ch == '\t' || ch == ';') ch = '_';
    uint64_t samples = 0, tris = 0;
    uint32_t max_npix = 1, depth = 0, bsdf = 0;
    std::vector<bool> seen(b->scenes.size(), false);
    for (uint32_t i = 0; i < n; i++) {
        const lgb_batch_job& j = jobs[i];
        const uint64_t npix = (uint64_t)j.camera.width * j.camera.height;
        samples += npix * j.spp;
        max_npix = std::max<uint32_t>(max_npix, (uint32_t)npix);
        depth = std::max<uint32_t>(depth, (uint32_t)std::max(j.params.max_depth, 0));
        const Scene* s = b->scenes[j.scene];
        bsdf |= s->bsdf_mask;
        if (!seen[j.scene]) { seen[j.scene] = true; tris += s->num_tris; }
    }
    auto lg = [](uint64_t v) { int k = 0; while (v > 1) { v >>= 1; k++; } return k; };
    std::ostringstream k;
    k << "dev=" << dev << ";sm=" << prop.multiProcessorCount << ";cc=" << prop.major << "." << prop.minor
      << ";abi=" << lgb_abi_version() << ";jobs=" << n << ";samples=2^" << lg(samples) << ";pix=2^" << lg(max_npix)
      << ";tris=2^" << lg(tris) << ";depth=" << depth << ";bsdf=" << bsdf;
    return k.str();
}

std::map<std::string, lgb_batch_opts> read_tune_cache(const std::string& path) {
    std::map<std::string, lgb_batch_opts> m;
    std::ifstream f(path);
    std::string line;
    while (std::getline(f, line)) {
        std::istringstream ls(line);
        std::string key;
        lgb_batch_opts o{};
        if (ls >> key >> o.path_capacity >> o.work_blocks_per_sm >> o.trace_blocks_per_sm >> o.stack_placement) {
            uint32_t chunk = 0, traversal = 0;
            if (ls >> chunk) o.chunk_paths = chunk;  // absent in lines written before path regeneration
            if (ls >> traversal) o.traversal = traversal;  // absent in lines written before the traversal variants
            m[key] = o;
        }
    }
    return m;
}

// Adds or replaces one entry: the file is rewritten through a temporary file renamed over it, so a reader never
// sees half a file.
void write_tune_cache(const std::string& path, const std::string& key, const lgb_batch_opts& o) {
    std::map<std::string, lgb_batch_opts> m = read_tune_cache(path);
    m[key] = o;
    const std::string tmp = path + ".tmp." + std::to_string((long)getpid());
    {
        std::ofstream f(tmp, std::ios::trunc);
        if (!f) return;
        for (const auto& e : m)
            f << e.first << ' ' << e.second.path_capacity << ' ' << e.second.work_blocks_per_sm << ' '
              << e.second.trace_blocks_per_sm << ' ' << e.second.stack_placement << ' ' << e.second.chunk_paths << ' '
              << e.second.traversal << '\n';
        if (!f) { std::remove(tmp.c_str()); return; }
    }
    if (std::rename(tmp.c_str(), path.c_str()) != 0) std::remove(tmp.c_str());
}

// Screens every candidate (queue size x shading grid, stack in local memory, path regeneration) on a quarter of
// each job's frames, then times the three fastest on the full jobs, then the best of those with the stack bottom
// in shared memory, with the other traversal variant and without path regeneration; films untouched throughout. The first run of a candidate
// records its graph, the second is timed.
lgb_status batch_tune(Batch* b, const lgb_batch_job* jobs, uint32_t n, lgb_batch_opts* best, cudaStream_t st) {
    Ctx* ctx = b->ctx;
    std::string key;
    if (!ctx->tuning_cache.empty()) {
        key = tune_key(b, jobs, n);
        const auto cache = read_tune_cache(ctx->tuning_cache);
        const auto it = cache.find(key);
        if (it != cache.end()) {
            b->tuned = true;
            b->tuned_opts = it->second;
            b->tuned_opts.from_cache = 0;
            if (best) { *best = it->second; best->from_cache = 1; }
            return LGB_OK;
        }
    }
    std::vector<lgb_batch_job> reduced(jobs, jobs + n);
    uint32_t max_npix = 1;
    for (auto& j : reduced) {
        if (j.spp) j.spp = std::max(1u, (j.spp + 3u) / 4u);
        max_npix = std::max(max_npix, j.camera.width * j.camera.height);
    }
    const uint32_t caps[] = {1u << 20, 1u << 21, 1u << 22, 1u << 23};
    const uint32_t works[] = {2u, 4u, 8u, 16u};
    cudaEvent_t e0, e1;
    LGB_CUDA_TRY(ctx, cudaEventCreate(&e0));
    LGB_CUDA_TRY(ctx, cudaEventCreate(&e1));
    lgb_status result = LGB_OK;
    // One candidate on a job list: the first run records its graph, the second is timed.
    auto trial = [&](const lgb_batch_opts& o, const lgb_batch_job* js) {
        float ms = 0.0f;
        for (int rep = 0; rep < 2 && result == LGB_OK; rep++) {
            cudaEventRecord(e0, st);
            result = batch_render(b, js, n, o, false, st);
            cudaEventRecord(e1, st);
            if (result == LGB_OK && cudaEventSynchronize(e1) != cudaSuccess) result = cuda_error(ctx, cudaGetLastError(), "batch tuning");
            if (result == LGB_OK) cudaEventElapsedTime(&ms, e0, e1);
        }
        return ms;
    };
    // Screen: every queue size x shading grid on the reduced jobs.
    std::vector<std::pair<float, lgb_batch_opts>> screened;
    for (uint32_t c : caps) {
        if (c < max_npix && c != caps[3]) continue;  // smaller than one frame: the larger candidates cover it
        for (uint32_t w : works) {
            lgb_batch_opts o{};
            o.path_capacity = c;
            o.work_blocks_per_sm = w;
            o.stack_placement = LGB_STACK_LOCAL;
            const float ms = trial(o, reduced.data());
            if (result != LGB_OK) break;
            screened.push_back({ms, o});
        }
        if (result != LGB_OK) break;
    }
    // Confirm on the full jobs: the three fastest of the screen (a quarter of the frames favours smaller queues
    // than the whole batch does), then the best of them with the stack bottom in shared memory and without
    // path regeneration.
    float best_ms = 0.0f;
    lgb_batch_opts best_o{};
    bool have = false;
    auto confirm = [&](const lgb_batch_opts& o) {
        const float ms = trial(o, jobs);
        if (result == LGB_OK && (!have || ms < best_ms)) { best_ms = ms; best_o = o; have = true; }
    };
    std::sort(screened.begin(), screened.end(),
              [](const std::pair<float, lgb_batch_opts>& x, const std::pair<float, lgb_batch_opts>& y) { return x.first < y.first; });
    for (size_t i = 0; i < screened.size() && i < 3 && result == LGB_OK; i++) confirm(screened[i].second);
    if (result == LGB_OK && have) {
        lgb_batch_opts o = best_o;
        o.stack_placement = LGB_STACK_SHARED;
        confirm(o);
    }
    if (result == LGB_OK && have) {  // the other traversal variant than the scene size picks
        lgb_batch_opts o = best_o;
        o.traversal = b->num_tris >= kIncoherentTris ? LGB_TRAVERSAL_COHERENT : LGB_TRAVERSAL_INCOHERENT;
        confirm(o);
    }
    if (result == LGB_OK && have && !b->regen_refused) {
        lgb_batch_opts o = best_o;
        o.chunk_paths = 1u;
        confirm(o);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (result != LGB_OK) return result;
    b->tuned = true;
    b->tuned_opts = best_o;
    if (best) *best = best_o;
    if (!key.empty()) write_tune_cache(ctx->tuning_cache, key, best_o);
    return LGB_OK;
}

}  // namespace
}  // namespace lgb

extern "C" {

LGB_API lgb_status lgb_batch_create(lgb_ctx* ctx, lgb_scene* const* scenes, uint32_t num_scenes, lgb_batch** out) {
    using namespace lgb;
    if (!ctx) return LGB_ERR_INVALID_ARGUMENT;
    if (!out || !scenes || num_scenes == 0) return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "null output or empty scene list");
    *out = nullptr;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return set_error(ctx, LGB_ERR_CUDA, "cudaSetDevice failed");
    lgb_batch* b = new (std::nothrow) lgb_batch();
    if (!b) return set_error(ctx, LGB_ERR_OUT_OF_MEMORY, "host allocation failed");
    std::vector<Scene*> list(scenes, scenes + num_scenes);
    const lgb_status st = batch_create(ctx, list.data(), num_scenes, b);
    if (st != LGB_OK) {
        free_batch(b);
        delete b;
        return st;
    }
    *out = b;
    ctx_retain(ctx);
    return LGB_OK;
}

LGB_API void lgb_batch_destroy(lgb_batch* b) {
    if (!b) return;
    lgb::Ctx* c = b->ctx;
    lgb::free_batch(b);
    delete b;
    lgb::ctx_release(c);
}

LGB_API lgb_status lgb_batch_render(lgb_batch* b, const lgb_batch_job* jobs, uint32_t num_jobs, const lgb_batch_opts* opts,
                                    void* stream) {
    using namespace lgb;
    if (!b) return LGB_ERR_INVALID_ARGUMENT;
    lgb_status st = check_jobs(b, jobs, num_jobs);
    if (st != LGB_OK) return st;
    if (cudaSetDevice(b->ctx->device) != cudaSuccess) return set_error(b->ctx, LGB_ERR_CUDA, "cudaSetDevice failed");
    const lgb_batch_opts o = opts ? *opts : (b->tuned ? b->tuned_opts : lgb_batch_opts{});
    return batch_render(b, jobs, num_jobs, o, true, (cudaStream_t)stream);
}

LGB_API lgb_status lgb_batch_tune(lgb_batch* b, const lgb_batch_job* jobs, uint32_t num_jobs, lgb_batch_opts* best,
                                  void* stream) {
    using namespace lgb;
    if (!b) return LGB_ERR_INVALID_ARGUMENT;
    lgb_status st = check_jobs(b, jobs, num_jobs);
    if (st != LGB_OK) return st;
    if (cudaSetDevice(b->ctx->device) != cudaSuccess) return set_error(b->ctx, LGB_ERR_CUDA, "cudaSetDevice failed");
    return batch_tune(b, jobs, num_jobs, best, (cudaStream_t)stream);
}

LGB_API lgb_status lgb_batch_sync(lgb_batch* b, void* stream) {
    using namespace lgb;
    if (!b) return LGB_ERR_INVALID_ARGUMENT;
    LGB_CUDA_TRY(b->ctx, cudaStreamSynchronize((cudaStream_t)stream));
    uint32_t status = 0;
    LGB_CUDA_TRY(b->ctx, cudaMemcpy(&status, b->d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    for (Scene* s : b->scenes) {
        uint32_t v = 0;
        LGB_CUDA_TRY(b->ctx, cudaMemcpy(&v, s->d_status, sizeof(uint32_t), cudaMemcpyDeviceToHost));
        status |= v;
    }
    if (status) {
        const uint32_t zero = 0;
        cudaMemcpy(b->d_status, &zero, sizeof(uint32_t), cudaMemcpyHostToDevice);
        for (Scene* s : b->scenes) cudaMemcpy(s->d_status, &zero, sizeof(uint32_t), cudaMemcpyHostToDevice);
        return set_error(b->ctx, LGB_ERR_DEVICE_STATUS,
                         "device status word 0x" + std::to_string(status) + " (bit 0: traversal stack overflow, bit 1: bad index, bit 2: visit limit)");
    }
    return LGB_OK;
}

}  // extern "C"
