// VCM: vertex connection and merging, Lumen's VCM integrator (src/RayTracer/VCM.cpp:131-265 without the
// reservoir passes, which Lumen disables: RAY_GUIDE = 0 in vcm_light.rgen:34).
//
//   k_vcm_light    vcm_light.rgen:123-166, vcm_generate_light_sample and vcm_fill_light
//                  (vcm_commons.glsl:77-130, 302-454): one light subpath per launch point, its non-specular
//                  vertices stored, each connected to the camera and splatted (atomics into the splat image)
//   photon table   vcm_commons.glsl:455-469 built by sort and scan: a slot key per stored vertex, a stable LSD
//                  radix sort of (slot, vertex id), then per slot the count and the last vertex in id order,
//                  which is the photon the reference's last writer leaves (deterministic here)
//   k_vcm_eye      vcm_eye.rgen:42-97 and vcm_trace_eye (vcm_commons.glsl:477-631): eye subpath with emission
//                  MIS, light connection, connections to one random light subpath, merging, progressive film
//
// Kept from the reference: the connection and merge loops assign rather than accumulate (`res =`), unless
// LGB_VCM_ACCUMULATE is set; splat and light-path indices are column-major (x * height + y). Deviations: the
// seeds are parameters (the reference draws them with host rand()); a light subpath whose emission sample has
// a zero direction pdf stores no vertex (the reference keeps the previous iteration's count); an eye vertex
// whose merge range exceeds 16 cells per axis does not merge; the uninitialised pdf_rev of the last eye
// bounce is zero; the random light subpath index is clamped to the last subpath.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "bsdf_vcm.cuh"
#include "light_sample.cuh"
#include "path_common.cuh"
#include "photon_table.cuh"
#include "radix_sort.cuh"

namespace lgb {
namespace {

constexpr int kVcmThreads = 128;
// The step kernels' register budget: 4 blocks per SM (eye step 128 registers instead of 166): caustics iteration
// 7.43 against 7.58 ms on the same GPU.
#ifdef LGB_VCM_STEP_MIN_BLOCKS
constexpr int kVcmStepMinBlocks = LGB_VCM_STEP_MIN_BLOCKS;
#else
constexpr int kVcmStepMinBlocks = 4;
#endif
// The light step alone at 6 blocks per SM (80 registers, a few bytes of spill; 104 at 4): caustics iteration 7.27
// against 7.39 ms (5 blocks: 7.32; 7 or 8: 7.27). The eye step spills heavily below 128 registers.
#ifdef LGB_VCM_LIGHT_STEP_MIN_BLOCKS
constexpr int kVcmLightStepMinBlocks = LGB_VCM_LIGHT_STEP_MIN_BLOCKS;
#else
constexpr int kVcmLightStepMinBlocks = 6;
#endif
constexpr int kMaxMergeCells = 16;
constexpr float kTMinV = 0.001f, kTMaxV = 10000.0f, kEpsV = 0.001f;
constexpr int kVertexF4 = 6;  // light vertex = 6 x float4 (96 bytes)
// BSDF type sets the subpath kernels are compiled for: diffuse, mirror, glass and dielectric; those and conductor.
constexpr uint32_t kVcmLobesDG = LGB_BSDF_DIFFUSE | LGB_BSDF_MIRROR | LGB_BSDF_GLASS | LGB_BSDF_DIELECTRIC;
constexpr uint32_t kVcmLobesDGC = kVcmLobesDG | LGB_BSDF_CONDUCTOR;

struct VcmArgs {
    float iv[16], ip[16], view[16], proj[16];
    uint32_t W, H, screen;
    float sky[3];
    int max_depth, num_lights, light_tri_count;
    int use_vm, use_vc;
    uint32_t light_seed, eye_seed, frame_num, accumulate;
    float spot_cos_width, spot_cos_falloff;  // cosines of the spot cone and of its falloff start
    float radius;
    float mn[3], mx[3];
    int res[3];
    float4* verts;           // screen * (max_depth + 1) vertices
    uint32_t* counts;        // stored vertices per light subpath
    float* splat;            // screen * 3, pixel x * H + y
    const uint32_t* g_count; // 10 * screen slots
    const uint32_t* g_rep;
    float4* film;            // RGBA32F, row-major
};

__device__ __forceinline__ LightSet lights_of(const VcmArgs& A) {
    return LightSet{A.num_lights, A.light_tri_count, A.spot_cos_width, A.spot_cos_falloff};
}

struct CamV {
    v3 pos, nrm;
    float area;
};
__device__ __forceinline__ CamV cam_setup(const VcmArgs& A) {
    CamV c;
    const float4 o = mat_vec(A.iv, 0.0f, 0.0f, 0.0f, 1.0f);
    const float4 f = mat_vec(A.iv, 0.0f, 0.0f, 1.0f, 0.0f);
    c.pos = V3(o.x, o.y, o.z);
    c.nrm = V3(-f.x, -f.y, -f.z);
    const float4 a = mat_vec(A.ip, 2.0f / (float)A.W, 2.0f / (float)A.H, 0.0f, 1.0f);
    c.area = fabsf((a.x / a.w) * (a.y / a.w));
    return c;
}

struct Etas { float vcm, vc, vm; };
__device__ __forceinline__ Etas etas(const VcmArgs& A) {
    const float r2 = A.radius * A.radius;
    Etas e;
    e.vcm = LGB_PI * r2 * (float)A.screen;
    e.vc = A.use_vc == 1 ? 1.0f / e.vcm : 0.0f;
    e.vm = A.use_vm == 1 ? LGB_PI * r2 * (float)A.screen : 0.0f;
    return e;
}


// Light vertex: (pos, area) (wi, d_vcm) (wo, d_vc) (n_s, d_vm) (throughput, u) (v, material, path_len, side)
struct LVert {
    v3 pos, wi, wo, n_s, thr;
    float area, d_vcm, d_vc, d_vm, u, v;
    uint32_t mat, path_len, side;
};
__device__ __forceinline__ void store_lvert(float4* p, const LVert& v) {
    p[0] = f4(v.pos, v.area);
    p[1] = f4(v.wi, v.d_vcm);
    p[2] = f4(v.wo, v.d_vc);
    p[3] = f4(v.n_s, v.d_vm);
    p[4] = f4(v.thr, v.u);
    p[5] = make_float4(v.v, __uint_as_float(v.mat), __uint_as_float(v.path_len), __uint_as_float(v.side));
}
__device__ __forceinline__ LVert load_lvert(const float4* p) {
    LVert v;
    const float4 a = p[0], b = p[1], c = p[2], d = p[3], e = p[4], g = p[5];
    v.pos = V3(a.x, a.y, a.z); v.area = a.w;
    v.wi = V3(b.x, b.y, b.z); v.d_vcm = b.w;
    v.wo = V3(c.x, c.y, c.z); v.d_vc = c.w;
    v.n_s = V3(d.x, d.y, d.z); v.d_vm = d.w;
    v.thr = V3(e.x, e.y, e.z); v.u = e.w;
    v.v = g.x; v.mat = __float_as_uint(g.y); v.path_len = __float_as_uint(g.z); v.side = __float_as_uint(g.w);
    return v;
}

__device__ __forceinline__ bool is_zero3(v3 a) { return a.x == 0.0f && a.y == 0.0f && a.z == 0.0f; }
__device__ __forceinline__ bool light_finite(uint32_t f) { return ((f >> 4) & 1u) != 0u; }
__device__ __forceinline__ bool light_delta(uint32_t f) { return ((f >> 5) & 1u) != 0u; }


struct VState {
    v3 pos, wi, thr;
    float d_vcm, d_vc, d_vm;
};

// vcm_connect_cam (vcm_commons.glsl:24-75) with its visibility test deferred: the shadow ray towards the camera
// and the splat it adds to pixel pidx (x * H + y) when not occluded; false when the vertex adds nothing (the
// camera behind it, a zero BSDF value, a zero pdf ratio, a pixel outside the image, a zero contribution).
template <uint32_t MASK>
__device__ bool connect_cam(const VcmArgs& A, const CamV& c, v3 n_s, v3 payload_ns, v3 pos, const VState& st, float eta_vm,
                            v3 wo, const Mat& mat, float4 (&ray)[2], v3& L, uint32_t& pidx) {
    v3 dir = c.pos - pos;
    const float len = length(dir);
    dir = dir / len;
    const float cos_y = dot(dir, n_s);
    const float cos_theta = dot(c.nrm, -dir);
    if (cos_theta <= 0.0f) return false;
    const float cos3 = cos_theta * cos_theta * cos_theta;
    const float screen = (float)A.screen;
    const float ratio = fabsf(cos_y) / (c.area * cos3 * len * len);
    const v3 origin = offset_ray2(pos, n_s);
    float pdf_fwd, pdf_rev;
    const v3 f = eval_bsdf_rev<MASK>(n_s, wo, mat, dot(payload_ns, wo) > 0.0f, dir, pdf_fwd, pdf_rev, true);
    if (is_zero3(f) || !(ratio > 0.0f)) return false;
    const float w_light = (ratio / screen) * (eta_vm + st.d_vcm + pdf_rev * st.d_vc);
    const float mis = 1.0f / (1.0f + w_light);
    L = mis * st.thr * ratio * f / screen;
    ray[0] = make_float4(origin.x, origin.y, origin.z, 0.0f);
    ray[1] = make_float4(dir.x, dir.y, dir.z, len - kEpsV);
    dir = -dir;
    float4 t = mat_vec(A.view, dir.x, dir.y, dir.z, 0.0f);
    t = make_float4(t.x / t.z, t.y / t.z, t.z / t.z, t.w / t.z);
    t = mat_vec(A.proj, t.x, t.y, t.z, t.w);
    t = make_float4(-t.x, -t.y, -t.z, -t.w);
    const int cx = __float2int_rz(0.5f * (1.0f + t.x) * (float)A.W - 0.5f);
    const int cy = __float2int_rz(0.5f * (1.0f + t.y) * (float)A.H - 0.5f);
    if (cx < 0 || cx >= (int)A.W || cy < 0 || cy >= (int)A.H || dot(dir, c.nrm) < 0.0f) return false;
    pidx = (uint32_t)cx * A.H + (uint32_t)cy;
    return luminance(L) > 0.0f;
}

// Wavefront form of the subpath loops: per bounce, the closest hits of a queue of rays come from the persistent
// traversal kernel (lanes whose ray is done fetch the next one), then a step kernel runs one iteration of the
// reference's loop body per queued path and appends the paths that continue, with their next rays, to the next
// queue. Path state lives in path-indexed SoA buffers, with the RNG counter, so a path's arithmetic and random
// numbers are the loop's; only the order of the camera splats' atomics changes.
struct Wave {
    float4* ls;        // light path state, 4 float4 per path: (pos, d_vcm) (wi, d_vc) (thr, d_vm) (rng, stored, finite, -)
    float4* es;        // eye path state, 5 float4 per pixel: the same three, (col, rng), (lp, lp_len, -, -)
    lgb_ray* rays[2];  // ray queues of consecutive bounces
    uint32_t* qidx[2]; // path of each queued ray
    lgb_hit* hits;
    uint32_t* qcount;  // [2 * (max_depth + 1)]: queue lengths per bounce, light pass then eye pass
    uint32_t* tcount;  // [2 * (max_depth + 1)]: fetch counters of the traversal launches, then the shadow queue's
    lgb_ray* srays;    // camera connections of the light pass: shadow rays,
    float4* spay;      // their splats (value, pixel) and
    uint32_t* sbits;   // occlusion bits
    uint32_t* scount;  // [2]: shadow queue length and fetch counter
};
__device__ __forceinline__ float4* sq(float4* b, int c, uint32_t screen, uint32_t i) { return b + ((size_t)c * screen + i); }

// One slot of a queue for each calling lane: one atomic per group of converged lanes.
__device__ __forceinline__ uint32_t warp_append(uint32_t* counter) {
    const uint32_t mask = __activemask();
    const int leader = __ffs(mask) - 1;
    const int lane = (int)(threadIdx.x & 31u);
    uint32_t first = 0;
    if (lane == leader) first = atomicAdd(counter, (uint32_t)__popc(mask));
    first = __shfl_sync(mask, first, leader);
    return first + (uint32_t)__popc(mask & ((1u << lane) - 1u));
}
__device__ __forceinline__ void push_ray(const Wave& W, int q, uint32_t* counter, uint32_t path, v3 o, float tmin, v3 d,
                                         float tmax) {
    const uint32_t j = warp_append(counter);
    (q ? W.qidx[1] : W.qidx[0])[j] = path;  // selects, not an indexed copy of the pointer arrays in local memory
    float4* r = reinterpret_cast<float4*>(&(q ? W.rays[1] : W.rays[0])[j]);
    r[0] = make_float4(o.x, o.y, o.z, tmin);
    r[1] = make_float4(d.x, d.y, d.z, tmax);
}

constexpr int kWaveTraceMinBlocks = 9;
// Idle lanes a warp waits for before fetching new rays: caustics iteration 7.64 ms at 16, 7.48 at 8, 7.49 at 4.
#ifdef LGB_WAVE_REFILL
constexpr int kWaveRefill = LGB_WAVE_REFILL;
#else
constexpr int kWaveRefill = 8;
#endif
// Leaf triangles postponed one per loop iteration, with warp-uniform triangle and node iterations once a quarter
// of the active lanes hold a pending triangle (trace_persistent's TRI_MIN): the caustics configuration's VCM
// iteration 8.29 -> 8.01 ms on GB300 against a node's leaf triangles tested in the iteration that visits it.
#ifdef LGB_WAVE_POSTPONE
constexpr bool kWavePostpone = LGB_WAVE_POSTPONE != 0;
#else
constexpr bool kWavePostpone = true;
#endif
#ifdef LGB_WAVE_TRI_MIN
constexpr int kWaveTriMin = LGB_WAVE_TRI_MIN;
#else
constexpr int kWaveTriMin = -4;
#endif
// Bottom traversal-stack entries in shared memory: none. 4 or 8 entries measured 7.46 against 7.40 ms per caustics
// iteration on GB300 (the headline query, whose warps stay longer on one ray, gains 0.8 % from 8).
#ifdef LGB_WAVE_SK
constexpr int kWaveSharedStack = LGB_WAVE_SK;
#else
constexpr int kWaveSharedStack = 0;
#endif
__global__ void __launch_bounds__(kVcmThreads, kWaveTraceMinBlocks)
    k_vcm_trace(SceneView S, const lgb_ray* __restrict__ rays, lgb_hit* __restrict__ hits, const uint32_t* count,
                uint32_t* fetch) {
    __shared__ uint2 s_stack[kWaveSharedStack > 0 ? kWaveSharedStack * kVcmThreads : 1];
    trace_persistent<false, false, kWavePostpone, kWaveSharedStack, kVcmThreads, kWaveRefill, kWaveTriMin>(
        S.nodes, S.tris, rays, hits, nullptr, 0u, count, fetch, S.status, nullptr, nullptr, s_stack);
}
__global__ void __launch_bounds__(kVcmThreads, kWaveTraceMinBlocks)
    k_vcm_trace_any(SceneView S, const lgb_ray* __restrict__ rays, uint32_t* __restrict__ bits, const uint32_t* count,
                    uint32_t* fetch) {
    __shared__ uint2 s_stack[kWaveSharedStack > 0 ? kWaveSharedStack * kVcmThreads : 1];
    trace_persistent<true, false, kWavePostpone, kWaveSharedStack, kVcmThreads, kWaveRefill, kWaveTriMin>(
        S.nodes, S.tris, rays, nullptr, bits, 0u, count, fetch, S.status, nullptr, nullptr, s_stack);
}

// The camera splats of the light pass whose shadow rays are not occluded.
__global__ void __launch_bounds__(256) k_vcm_splat(VcmArgs A, Wave W) {
    const uint32_t n = W.scount[0];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if ((W.sbits[i >> 5] >> (i & 31u)) & 1u) continue;
        const float4 c = W.spay[i];
        const uint32_t pidx = __float_as_uint(c.w);
        atomicAdd(&A.splat[3 * pidx], c.x);
        atomicAdd(&A.splat[3 * pidx + 1], c.y);
        atomicAdd(&A.splat[3 * pidx + 2], c.z);
    }
}

// vcm_light.rgen main and vcm_generate_light_sample: one light subpath per launch point (x, y), path x * H + y;
// its first ray goes to queue 0.
__global__ void __launch_bounds__(kVcmThreads) k_vcm_light_init(SceneView S, VcmArgs A, Wave W) {
    const Etas eta = etas(A);
    for (uint32_t li = blockIdx.x * blockDim.x + threadIdx.x; li < A.screen; li += gridDim.x * blockDim.x) {
        const uint32_t x = li / A.H, y = li % A.H;
        uint4 seed = make_uint4(x, y, A.light_seed, 0u);
        const float r0 = rnd(seed), r1 = rnd(seed), r2 = rnd(seed), r3 = rnd(seed);
        const float d0 = rnd(seed), d1 = rnd(seed);
        const Emission e = sample_light_Le(S, lights_of(A), r0, r1, r2, r3, d0, d1);
        if (e.pdf_dir_w <= 0.0f) {
            A.counts[li] = 0u;
            continue;
        }
        const float pdf_emit = e.pdf_pos_a * e.pdf_dir_w;
        const v3 thr = e.L * e.cos_from_light / (e.pdf_dir_w * e.pdf_pos_a);
        const float d_vcm = e.pdf_pos_a / pdf_emit;
        const bool finite = light_finite(e.flags);
        const float d_vc = light_delta(e.flags) ? 0.0f : (finite ? e.cos_from_light : 1.0f) / (e.pdf_dir_w * e.pdf_pos_a);
        const float d_vm = d_vc * eta.vc;
        *sq(W.ls, 0, A.screen, li) = f4(e.pos, d_vcm);
        *sq(W.ls, 1, A.screen, li) = f4(e.wi, d_vc);
        *sq(W.ls, 2, A.screen, li) = f4(thr, d_vm);
        *sq(W.ls, 3, A.screen, li) = make_float4(__uint_as_float(seed.w), __uint_as_float(0u), __uint_as_float(finite ? 1u : 0u), 0.0f);
        push_ray(W, 0, W.qcount, li, e.pos, kTMinV, e.wi, kTMaxV);
    }
}

// vcm_fill_light, one bounce (depth) of the queued light subpaths: vertex store, camera connection, the next
// direction; a subpath that ends writes its vertex count.
template <uint32_t MASK>
__global__ void __launch_bounds__(kVcmThreads, kVcmLightStepMinBlocks) k_vcm_light_step(SceneView S, VcmArgs A, Wave W, int depth) {
    const CamV cam = cam_setup(A);
    const Etas eta = etas(A);
    const uint32_t per = (uint32_t)(A.max_depth + 1);
    const int cur = (depth - 1) & 1;
    const uint32_t n = W.qcount[depth - 1];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t li = (cur ? W.qidx[1] : W.qidx[0])[i];
        const lgb_hit hit = W.hits[i];
        const float4 s0 = *sq(W.ls, 0, A.screen, li), s1 = *sq(W.ls, 1, A.screen, li), s2 = *sq(W.ls, 2, A.screen, li),
                     s3 = *sq(W.ls, 3, A.screen, li);
        VState st;
        st.pos = V3(s0.x, s0.y, s0.z); st.d_vcm = s0.w;
        st.wi = V3(s1.x, s1.y, s1.z); st.d_vc = s1.w;
        st.thr = V3(s2.x, s2.y, s2.z); st.d_vm = s2.w;
        uint4 seed = make_uint4(li / A.H, li % A.H, A.light_seed, __float_as_uint(s3.x));
        uint32_t path_idx = __float_as_uint(s3.y);
        const bool finite = __float_as_uint(s3.z) != 0u;
        float4* lv = A.verts + (size_t)li * per * kVertexF4;
        bool done = true;
        if (hit.prim != LGB_NO_HIT) {
            const HitAttr h = resolve_hit(S, hit.prim, hit.u, hit.v);
            v3 wo = st.pos - h.pos;
            v3 n_s = h.n_s, n_g = h.n_g;
            bool side = true;
            if (dot(h.n_g, wo) <= 0.0f) n_g = -n_g;
            if (dot(n_g, n_s) < 0.0f) { n_s = -n_s; side = false; }
            const float dist = length(h.pos - st.pos);
            const float dist_sqr = dist * dist;
            wo = wo / dist;
            const Mat mat = load_material(S, h.mat, h.u, h.v);
            const bool spec = (mat.props & LGB_FLAG_SPECULAR) == LGB_FLAG_SPECULAR;
            const float cos_wo = fabsf(dot(wo, n_s));
            if (depth > 1 || finite) st.d_vcm *= dist_sqr;
            st.d_vcm /= cos_wo;
            st.d_vc /= cos_wo;
            st.d_vm /= cos_wo;
            if (!spec && (A.use_vc == 1 || A.use_vm == 1)) {
                LVert v;
                v.pos = h.pos; v.area = h.area; v.wi = st.wi; v.d_vcm = st.d_vcm; v.wo = wo; v.d_vc = st.d_vc;
                v.n_s = n_s; v.d_vm = st.d_vm; v.thr = st.thr; v.u = h.u; v.v = h.v; v.mat = h.mat;
                v.path_len = (uint32_t)depth + 1u; v.side = side ? 1u : 0u;
                store_lvert(lv + (size_t)path_idx * kVertexF4, v);
                path_idx++;
            }
            if (depth < A.max_depth) {
                if (!spec && A.use_vc == 1) {
                    float4 ray[2];
                    v3 L;
                    uint32_t pidx;
                    if (connect_cam<MASK>(A, cam, n_s, h.n_s, h.pos, st, eta.vm, wo, mat, ray, L, pidx)) {
                        const uint32_t j = warp_append(W.scount);
                        float4* r = reinterpret_cast<float4*>(&W.srays[j]);
                        r[0] = ray[0];
                        r[1] = ray[1];
                        W.spay[j] = make_float4(L.x, L.y, L.z, __uint_as_float(pidx));
                    }
                }
                const float c0 = rnd(seed), c1 = rnd(seed), c2 = rnd(seed);
                float pdf_dir, cos_t;
                v3 wi;
                const v3 f = sample_bsdf_mode<MASK>(n_s, wo, mat, 0u, side, wi, pdf_dir, cos_t, V3(c0, c1, c2));
                st.wi = wi;
                const bool same = dot(st.wi, n_s) > 0.0f && dot(wo, n_s) > 0.0f;
                const bool trans = (mat.props & LGB_FLAG_TRANSMISSION) == LGB_FLAG_TRANSMISSION;
                if (!(is_zero3(f) || pdf_dir == 0.0f || (!same && !trans))) {
                    float pdf_rev = pdf_dir;
                    if (!spec) pdf_rev = bsdf_pdf<MASK>(mat, n_s, st.wi, wo, side);
                    const float ac = fabsf(cos_t);
                    st.pos = offset_ray(h.pos, n_g);
                    if (!spec) {
                        st.d_vc = (ac / pdf_dir) * (eta.vm + st.d_vcm + pdf_rev * st.d_vc);
                        st.d_vm = (ac / pdf_dir) * (1.0f + st.d_vcm * eta.vc + pdf_rev * st.d_vm);
                        st.d_vcm = 1.0f / pdf_dir;
                    } else {
                        st.d_vcm = 0.0f;
                        st.d_vc *= ac;
                        st.d_vm *= ac;
                    }
                    st.thr = st.thr * (f * ac / pdf_dir);
                    done = false;
                }
            }
        }
        if (done) {
            A.counts[li] = path_idx;
        } else {
            *sq(W.ls, 0, A.screen, li) = f4(st.pos, st.d_vcm);
            *sq(W.ls, 1, A.screen, li) = f4(st.wi, st.d_vc);
            *sq(W.ls, 2, A.screen, li) = f4(st.thr, st.d_vm);
            *sq(W.ls, 3, A.screen, li) = make_float4(__uint_as_float(seed.w), __uint_as_float(path_idx), s3.z, 0.0f);
            push_ray(W, depth & 1, W.qcount + depth, li, st.pos, kTMinV, st.wi, kTMaxV);
        }
    }
}

struct EyeHit {
    v3 pos, ns_payload;
    float area;
};

// Eye-pass connections with their visibility deferred: each candidate is a shadow ray and the radiance it adds
// when not occluded. A vertex's candidates take consecutive slots of the shadow queue (the light connection
// first, then one per light-subpath vertex in order); k_vcm_eye_resolve combines them once the any-hit launch has
// traced them. An unused slot keeps an empty ray and the marker kNoCandidate.
constexpr uint32_t kNoCandidate = 0xFFFFFFFFu;
__device__ __forceinline__ void put_candidate(const Wave& W, uint32_t slot, v3 origin, v3 dir, float tmax, v3 c) {
    float4* r = reinterpret_cast<float4*>(&W.srays[slot]);
    r[0] = make_float4(origin.x, origin.y, origin.z, 0.0f);
    r[1] = make_float4(dir.x, dir.y, dir.z, tmax);
    W.spay[slot] = make_float4(c.x, c.y, c.z, 0.0f);
    W.sbits[slot >> 5] = 0u;  // the lanes of a warp clear their words before the any-hit launch sets bits
}
__device__ __forceinline__ void put_empty(const Wave& W, uint32_t slot) {
    float4* r = reinterpret_cast<float4*>(&W.srays[slot]);
    r[0] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    r[1] = make_float4(0.0f, 0.0f, 1.0f, -1.0f);
    W.spay[slot] = make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(kNoCandidate));
    W.sbits[slot >> 5] = 0u;
}

// vcm_connect_light (vcm_commons.glsl:146-204), the visibility test deferred: the candidate goes to `slot`.
template <uint32_t MASK>
__device__ void connect_light(const SceneView& S, const VcmArgs& A, const Wave& W, uint32_t slot, uint4& seed,
                              const EyeHit& h, v3 n_s, v3 wo, const Mat& mat, bool side, float eta_vm, const VState& cs,
                              float& pdf_rev) {
    const float q0 = rnd(seed), q1 = rnd(seed), q2 = rnd(seed), q3 = rnd(seed);
    const Incidence li = sample_light_Li_pos(S, lights_of(A), q0, q1, q2, q3, h.pos);
    const float cos_x = dot(li.wi, n_s);
    const v3 origin = offset_ray2(h.pos, n_s);
    float pdf_fwd;
    const v3 f = eval_bsdf_rev<MASK>(n_s, wo, mat, side, li.wi, pdf_fwd, pdf_rev, true);
    if (!is_zero3(f)) {
        if (light_delta(li.flags)) pdf_fwd = 0.0f;
        const float ltc = (float)A.light_tri_count;
        const float w_light = pdf_fwd / (li.pdf_pos_w / ltc);
        const float w_cam = li.pdf_pos_dir_w * fabsf(cos_x) / (li.pdf_pos_w * li.cos_y) *
                            (eta_vm + cs.d_vcm + cs.d_vc * pdf_rev);
        const float mis = 1.0f / (1.0f + w_light + w_cam);
        const v3 c = mis > 0.0f ? mis * fabsf(cos_x) * f * cs.thr * li.L / (li.pdf_pos_w / ltc) : V3(0.0f);
        put_candidate(W, slot, origin, li.wi, li.wi_len - kEpsV, c);
    } else {
        put_empty(W, slot);
    }
}

// vcm_connect_light_vertices (vcm_commons.glsl:206-251), the visibility tests deferred: candidate i goes to slot
// first + i (slots first .. first + len_path - 1, unused ones left empty).
template <uint32_t MASK>
__device__ void connect_light_vertices(const SceneView& S, const VcmArgs& A, const Wave& W, uint32_t first,
                                       const float4* lv, uint32_t len_path, int depth, const EyeHit& h, v3 n_s, v3 wo,
                                       const Mat& mat, bool side, float eta_vm, const VState& cs, float pdf_rev) {
    uint32_t i = 0;
    for (; i < len_path; i++) {
        const LVert v = load_lvert(lv + (size_t)i * kVertexF4);
        if (v.path_len + (uint32_t)depth - 1u >= (uint32_t)A.max_depth) break;
        v3 dir = v.pos - h.pos;
        const float len = length(dir);
        const float len_sqr = len * len;
        dir = dir / len;
        const float cos_cam = dot(n_s, dir);
        const float cos_light = dot(v.n_s, -dir);
        const float G = cos_light * cos_cam / len_sqr;
        if (!(G > 0.0f)) { put_empty(W, first + i); continue; }
        float cam_pdf_fwd, unused, light_pdf_fwd, light_pdf_rev;
        const v3 f_cam = eval_bsdf_rev<MASK>(n_s, wo, mat, side, dir, cam_pdf_fwd, unused, false);
        const Mat lm = load_material(S, v.mat, v.u, v.v);
        const v3 f_light = eval_bsdf_rev<MASK>(v.n_s, v.wo, lm, v.side == 1u, -dir, light_pdf_fwd, light_pdf_rev, true);
        if (is_zero3(f_light) || is_zero3(f_cam)) { put_empty(W, first + i); continue; }
        cam_pdf_fwd *= fabsf(cos_light) / len_sqr;
        light_pdf_fwd *= fabsf(cos_cam) / len_sqr;
        const float w_light = cam_pdf_fwd * (eta_vm + v.d_vcm + light_pdf_rev * v.d_vc);
        const float w_camera = light_pdf_fwd * (eta_vm + cs.d_vcm + pdf_rev * cs.d_vc);
        const float mis = 1.0f / (1.0f + w_camera + w_light);
        const v3 origin = offset_ray2(h.pos, n_s);
        put_candidate(W, first + i, origin, dir, len - kEpsV, mis * G * cs.thr * v.thr * f_cam * f_light);
    }
    for (; i < len_path; i++) put_empty(W, first + i);
}

// vcm_merge_light_vertices (vcm_commons.glsl:254-296) over the slot table (count, representative photon)
template <uint32_t MASK>
__device__ v3 merge(const VcmArgs& A, int depth, const EyeHit& h, v3 n_s, v3 wo, const Mat& mat, bool side, float eta_vc,
                    const VState& cs, float norm) {
    const float radius = A.radius;
    const float r_sqr = radius * radius;
    v3 res = V3(0.0f);
    const int3 lo = grid_idx(h.pos - V3(radius), A.mn, A.mx, A.res);
    const int3 hi = grid_idx(h.pos + V3(radius), A.mn, A.mx, A.res);
    if ((long long)hi.x - lo.x >= kMaxMergeCells || (long long)hi.y - lo.y >= kMaxMergeCells ||
        (long long)hi.z - lo.z >= kMaxMergeCells)
        return res;
    for (int x = lo.x; x <= hi.x; x++)
        for (int y = lo.y; y <= hi.y; y++)
            for (int z = lo.z; z <= hi.z; z++) {
                const uint32_t slot = grid_hash(make_int3(x, y, z), A.screen);
                const uint32_t count = A.g_count[slot];
                if (count == 0u) continue;
                const LVert ph = load_lvert(A.verts + (size_t)A.g_rep[slot] * kVertexF4);
                const v3 pp = h.pos - ph.pos;
                const float dist_sqr = dot(pp, pp);
                if (dist_sqr > r_sqr) continue;
                if (ph.path_len + (uint32_t)depth - 1u > (uint32_t)A.max_depth) continue;
                const v3 pwi = -ph.wi;
                float cam_pdf_fwd, cam_pdf_rev;
                const v3 f = eval_bsdf_rev<MASK>(n_s, wo, mat, side, pwi, cam_pdf_fwd, cam_pdf_rev, true);
                if (is_zero3(f)) continue;
                const float w_light = ph.d_vcm * eta_vc + ph.d_vm * cam_pdf_fwd;
                const float w_cam = cs.d_vcm * eta_vc + cs.d_vm * cam_pdf_rev;
                const float mis = 1.0f / (1.0f + w_light + w_cam);
                if (dot(ph.n_s, n_s) > kEpsV) {
                    const float w = 1.0f - sqrtf(dist_sqr) / radius;
                    const v3 c = w * mis * (float)(int)count * ph.thr * f * cs.thr * norm * 3.0f;
                    res = A.accumulate ? res + c : c;
                }
            }
    return res;
}

// vcm_eye.rgen main: the camera ray of pixel (x, y) (path y * W + x), the random light subpath it connects to
// (vcm_commons.glsl:518) and its first ray in queue 0 of the eye pass.
__global__ void __launch_bounds__(kVcmThreads) k_vcm_eye_init(VcmArgs A, Wave W) {
    const CamV cam = cam_setup(A);
    uint32_t* const qc = W.qcount + (A.max_depth + 1);
    if (blockIdx.x == 0 && threadIdx.x == 0) {  // the shadow queue, read by the light pass's splats, starts empty
        W.scount[0] = 0u;
        W.scount[1] = 0u;
    }
    for (uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x; pix < A.screen; pix += gridDim.x * blockDim.x) {
        const uint32_t x = pix % A.W, y = pix / A.W;
        uint4 seed = make_uint4(x, y, A.eye_seed, 0u);
        const float j0 = rnd(seed), j1 = rnd(seed);
        const float u = ((float)x + 0.5f + (j0 - 0.5f)) / (float)A.W, v = ((float)y + 0.5f + (j1 - 0.5f)) / (float)A.H;
        const float dx = u * 2.0f - 1.0f, dy = v * 2.0f - 1.0f;
        const float4 t4 = mat_vec(A.ip, dx, dy, 1.0f, 1.0f);
        const v3 tn = normalize(V3(t4.x, t4.y, t4.z));
        const float4 d4 = mat_vec(A.iv, tn.x, tn.y, tn.z, 0.0f);
        const v3 wi = V3(d4.x, d4.y, d4.z);
        const float ct0 = fabsf(dot(cam.nrm, wi));
        const float d_vcm = cam.area * (float)A.screen * ct0 * ct0 * ct0;
        // uint(rand * screen) can round up to screen for large images: clamped
        const uint32_t lp = min((uint32_t)(rnd(seed) * (float)A.screen), A.screen - 1u);
        *sq(W.es, 0, A.screen, pix) = f4(cam.pos, d_vcm);
        *sq(W.es, 1, A.screen, pix) = f4(wi, 0.0f);
        *sq(W.es, 2, A.screen, pix) = f4(V3(1.0f), 0.0f);
        *sq(W.es, 3, A.screen, pix) = make_float4(0.0f, 0.0f, 0.0f, __uint_as_float(seed.w));
        *sq(W.es, 4, A.screen, pix) = make_float4(__uint_as_float(lp), __uint_as_float(A.counts[lp]), 0.0f, 0.0f);
        push_ray(W, 0, qc, pix, cam.pos, kTMinV, wi, kTMaxV);
    }
}

// Slots of the shadow queue for each lane's count k, consecutive per lane: an exclusive scan over the warp and one
// atomic per warp. Every lane of the warp calls it.
__device__ __forceinline__ uint32_t warp_alloc(uint32_t* counter, uint32_t k) {
    const int lane = (int)(threadIdx.x & 31u);
    uint32_t x = k;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    uint32_t first = 0;
    if (lane == 31 && x) first = atomicAdd(counter, x);
    first = __shfl_sync(0xffffffffu, first, 31);
    return first + x - k;
}

// vcm_trace_eye, one bounce (depth) of the queued eye subpaths: emission, the light connection and the connections
// to the light subpath's vertices (queued as shadow-ray candidates), merging, the next direction. The radiance so
// far goes to the path state with the candidates' slots; k_vcm_eye_resolve adds the visible candidates and writes
// the pixel of a subpath that ends (vcm_eye.rgen:80-97).
template <uint32_t MASK>
__global__ void __launch_bounds__(kVcmThreads, kVcmStepMinBlocks) k_vcm_eye_step(SceneView S, VcmArgs A, Wave W, int depth) {
    const Etas eta = etas(A);
    const float norm = 1.0f / (LGB_PI * A.radius * A.radius * (float)A.screen);
    const uint32_t per = (uint32_t)(A.max_depth + 1);
    const int cur = (depth - 1) & 1;
    uint32_t* const qc = W.qcount + (A.max_depth + 1);
    const uint32_t n = qc[depth - 1];
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        const bool valid = i < n;
        uint32_t pix = 0u, kl = 0u, kv = 0u;
        lgb_hit hit{LGB_NO_HIT, 0.0f, 0.0f, 0.0f};
        float4 s4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (valid) {
            pix = (cur ? W.qidx[1] : W.qidx[0])[i];
            hit = W.hits[i];
            s4 = *sq(W.es, 4, A.screen, pix);
            if (hit.prim != LGB_NO_HIT) {
                // at most one light connection and max_depth - depth vertex connections: the i-th stored vertex of
                // a light subpath has path_len >= i + 2, so connect_light_vertices stops before that many
                kl = depth < A.max_depth ? 1u : 0u;
                kv = min(__float_as_uint(s4.y), (uint32_t)(A.max_depth - depth));
            }
        }
        const uint32_t first = warp_alloc(W.scount, kl + kv);
        if (!valid) continue;
        const float4 s0 = *sq(W.es, 0, A.screen, pix), s1 = *sq(W.es, 1, A.screen, pix), s2 = *sq(W.es, 2, A.screen, pix),
                     s3 = *sq(W.es, 3, A.screen, pix);
        VState cs;
        cs.pos = V3(s0.x, s0.y, s0.z); cs.d_vcm = s0.w;
        cs.wi = V3(s1.x, s1.y, s1.z); cs.d_vc = s1.w;
        cs.thr = V3(s2.x, s2.y, s2.z); cs.d_vm = s2.w;
        v3 col = V3(s3.x, s3.y, s3.z);
        const uint32_t x = pix % A.W, y = pix / A.W;
        uint4 seed = make_uint4(x, y, A.eye_seed, __float_as_uint(s3.w));
        const uint32_t lp = __float_as_uint(s4.x);
        const float4* lv = A.verts + (size_t)lp * per * kVertexF4;
        bool done = true;
        if (hit.prim == LGB_NO_HIT) {
            col = col + cs.thr * V3(A.sky[0], A.sky[1], A.sky[2]);
        } else {
            const HitAttr h = resolve_hit(S, hit.prim, hit.u, hit.v);
            v3 wo = cs.pos - h.pos;
            const float dist = length(h.pos - cs.pos);
            const float dist_sqr = dist * dist;
            wo = wo / dist;
            v3 n_s = h.n_s, n_g = h.n_g;
            bool side = true;
            if (dot(h.n_g, wo) < 0.0f) n_g = -n_g;
            if (dot(n_g, n_s) < 0.0f) { n_s = -n_s; side = false; }
            const float cos_wo = fabsf(dot(wo, n_s));
            const Mat mat = load_material(S, h.mat, h.u, h.v);
            const bool spec = (mat.props & LGB_FLAG_SPECULAR) == LGB_FLAG_SPECULAR;
            cs.d_vcm *= dist_sqr;
            cs.d_vcm /= cos_wo;
            cs.d_vc /= cos_wo;
            cs.d_vm /= cos_wo;
            const EyeHit eh{h.pos, h.n_s, h.area};
            if (luminance(mat.emissive) > 0.0f) {  // vcm_get_light_radiance (vcm_commons.glsl:132-144)
                v3 Le = mat.emissive;
                if (depth != 1) {
                    const float pdf_light_pos = 1.0f / (eh.area * (float)A.light_tri_count);
                    const float pdf_light_dir = fabsf(dot(eh.ns_payload, -cs.wi)) / LGB_PI;
                    const float w_camera = pdf_light_pos * cs.d_vcm +
                                           ((A.use_vc == 1 || A.use_vm == 1) ? (pdf_light_pos * pdf_light_dir) * cs.d_vc : 0.0f);
                    Le = (1.0f / (1.0f + w_camera)) * mat.emissive;
                }
                col = col + cs.thr * Le;
            }
            float pdf_rev = 0.0f;
            if (kl) {
                if (!spec) connect_light<MASK>(S, A, W, first, seed, eh, n_s, wo, mat, side, eta.vm, cs, pdf_rev);
                else put_empty(W, first);
            }
            if (!spec) {
                connect_light_vertices<MASK>(S, A, W, first + kl, lv, kv, depth, eh, n_s, wo, mat, side, eta.vm, cs, pdf_rev);
            } else {
                for (uint32_t j = 0; j < kv; j++) put_empty(W, first + kl + j);
            }
            if (!spec && A.use_vm == 1) col = col + merge<MASK>(A, depth, eh, n_s, wo, mat, side, eta.vc, cs, norm);
            if (depth < A.max_depth) {
                const float c0 = rnd(seed), c1 = rnd(seed), c2 = rnd(seed);
                float pdf_dir, cos_t;
                v3 wi;
                const v3 f = sample_bsdf_mode<MASK>(n_s, wo, mat, 1u, side, wi, pdf_dir, cos_t, V3(c0, c1, c2));
                cs.wi = wi;
                const bool trans = (mat.props & LGB_FLAG_TRANSMISSION) == LGB_FLAG_TRANSMISSION;
                const bool same = dot(cs.wi, n_s) > 0.0f && dot(wo, n_s) > 0.0f;
                if (!(is_zero3(f) || pdf_dir == 0.0f || (!same && !trans))) {
                    pdf_rev = pdf_dir;
                    if (!spec) pdf_rev = bsdf_pdf<MASK>(mat, n_s, cs.wi, wo, side);
                    const float ac = fabsf(cos_t);
                    cs.pos = offset_ray(h.pos, n_g);
                    if (!spec) {
                        cs.d_vc = (ac / pdf_dir) * (eta.vm + cs.d_vcm + pdf_rev * cs.d_vc);
                        cs.d_vm = (ac / pdf_dir) * (1.0f + cs.d_vcm * eta.vc + pdf_rev * cs.d_vm);
                        cs.d_vcm = 1.0f / pdf_dir;
                    } else {
                        cs.d_vcm = 0.0f;
                        cs.d_vc *= ac;
                        cs.d_vm *= ac;
                    }
                    cs.thr = cs.thr * (f * ac / pdf_dir);
                    done = false;
                }
            }
        }
        *sq(W.es, 3, A.screen, pix) = make_float4(col.x, col.y, col.z, __uint_as_float(seed.w));
        *sq(W.es, 4, A.screen, pix) = make_float4(s4.x, s4.y, __uint_as_float(first),
                                                  __uint_as_float(kv | (kl << 16) | (done ? 0x80000000u : 0u)));
        if (!done) {
            *sq(W.es, 0, A.screen, pix) = f4(cs.pos, cs.d_vcm);
            *sq(W.es, 1, A.screen, pix) = f4(cs.wi, cs.d_vc);
            *sq(W.es, 2, A.screen, pix) = f4(cs.thr, cs.d_vm);
            push_ray(W, depth & 1, qc + depth, pix, cs.pos, kTMinV, cs.wi, kTMaxV);
        }
    }
}

// After the any-hit launch over a bounce's candidates: the light connection when visible, then the vertex
// connections in order (vcm_commons.glsl:247: each visible one adds to the result, or, Lumen's default, replaces
// it), added to the eye subpath's radiance; a subpath that ended this bounce writes its pixel (vcm_eye.rgen:80-97).
// Block 0 also resets the shadow queue's counters for the next bounce (nothing here reads them).
__global__ void __launch_bounds__(kVcmThreads) k_vcm_eye_resolve(VcmArgs A, Wave W, int depth) {
    const int cur = (depth - 1) & 1;
    const uint32_t n = (W.qcount + (A.max_depth + 1))[depth - 1];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        W.scount[0] = 0u;
        W.scount[1] = 0u;
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t pix = (cur ? W.qidx[1] : W.qidx[0])[i];
        const float4 s3 = *sq(W.es, 3, A.screen, pix), s4 = *sq(W.es, 4, A.screen, pix);
        const uint32_t first = __float_as_uint(s4.z), kw = __float_as_uint(s4.w);
        const uint32_t kl = (kw >> 16) & 1u, kv = kw & 0xffffu;
        v3 col = V3(s3.x, s3.y, s3.z);
        v3 res = V3(0.0f);
        for (uint32_t j = 0; j < kl + kv; j++) {
            const uint32_t slot = first + j;
            const float4 pay = W.spay[slot];
            if (__float_as_uint(pay.w) == kNoCandidate || ((W.sbits[slot >> 5] >> (slot & 31u)) & 1u)) continue;
            const v3 c = V3(pay.x, pay.y, pay.z);
            if (j < kl) col = col + c;  // the light connection
            else res = A.accumulate ? res + c : c;
        }
        col = col + res;
        if (!(kw & 0x80000000u)) {
            *sq(W.es, 3, A.screen, pix) = make_float4(col.x, col.y, col.z, s3.w);
            continue;
        }
        if (isnan(luminance(col))) continue;  // vcm_eye.rgen:80-83: no film write, the splat stays
        const uint32_t x = pix % A.W, y = pix / A.W;
        const uint32_t sidx = x * A.H + y;
        col = col + V3(A.splat[3 * sidx], A.splat[3 * sidx + 1], A.splat[3 * sidx + 2]);
        A.splat[3 * sidx] = 0.0f;
        A.splat[3 * sidx + 1] = 0.0f;
        A.splat[3 * sidx + 2] = 0.0f;
        float4 px = A.film[pix];
        if (A.frame_num > 0u) {
            const float w = 1.0f / (float)(A.frame_num + 1u);
            px = make_float4(mixf(px.x, col.x, w), mixf(px.y, col.y, w), mixf(px.z, col.z, w), 1.0f);
        } else {
            px = make_float4(col.x, col.y, col.z, 1.0f);
        }
        A.film[pix] = px;
    }
}

// Photon table by sort and scan. Keys: the slot of every stored light vertex; unused vertex slots get the
// table size and sort after every real slot. Values: the vertex id, so the stable sort keeps id order inside
// a slot and the run's last element is the highest id (the sequential last writer).
__global__ void k_vcm_keys(VcmArgs A, uint32_t table, uint32_t* keys, uint32_t* vals) {
    const uint32_t per = (uint32_t)(A.max_depth + 1);
    const uint32_t n = A.screen * per;
    for (uint32_t vid = blockIdx.x * blockDim.x + threadIdx.x; vid < n; vid += gridDim.x * blockDim.x) {
        const uint32_t li = vid / per, k = vid % per;
        uint32_t key = table;
        if (k < A.counts[li]) {
            const float4 p = A.verts[(size_t)vid * kVertexF4];
            key = grid_hash(grid_idx(V3(p.x, p.y, p.z), A.mn, A.mx, A.res), A.screen);
        }
        keys[vid] = key;
        vals[vid] = vid;
    }
}

// Keys of n photon positions (w < 0: unused), for the stand-alone table builder.
__global__ void k_vcm_keys_pos(const float4* __restrict__ pos, uint32_t n, float mn0, float mn1, float mn2, float mx0,
                               float mx1, float mx2, int r0, int r1, int r2, uint32_t screen, uint32_t* keys, uint32_t* vals) {
    const float mn[3] = {mn0, mn1, mn2}, mx[3] = {mx0, mx1, mx2};
    const int res[3] = {r0, r1, r2};
    const uint32_t table = 10u * screen;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 p = pos[i];
        keys[i] = p.w < 0.0f ? table : grid_hash(grid_idx(V3(p.x, p.y, p.z), mn, mx, res), screen);
        vals[i] = i;
    }
}



size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// Inverts a column-major 4x4 matrix in double (Gauss-Jordan with partial pivoting); false if singular.
bool invert4(const float* in, double* out) {
    double a[4][8];
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) { a[r][c] = in[4 * c + r]; a[r][4 + c] = r == c ? 1.0 : 0.0; }
    for (int c = 0; c < 4; c++) {
        int piv = c;
        for (int r = c + 1; r < 4; r++) if (std::fabs(a[r][c]) > std::fabs(a[piv][c])) piv = r;
        if (a[piv][c] == 0.0) return false;
        if (piv != c) for (int k = 0; k < 8; k++) std::swap(a[c][k], a[piv][k]);
        const double inv = 1.0 / a[c][c];
        for (int k = 0; k < 8; k++) a[c][k] *= inv;
        for (int r = 0; r < 4; r++) {
            if (r == c) continue;
            const double f = a[r][c];
            for (int k = 0; k < 8; k++) a[r][k] -= f * a[c][k];
        }
    }
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++) out[4 * c + r] = a[r][4 + c];
    return true;
}

}  // namespace
}  // namespace lgb

using namespace lgb;

extern "C" {

LGB_API float lgb_vcm_radius(float scene_radius, float radius_factor, uint32_t iteration, float alpha) {
    float r = scene_radius * radius_factor / 100.0f;
    r /= (float)std::pow((double)iteration + 1.0, 0.5 * (1.0 - (double)alpha));
    return r;
}

LGB_API lgb_status lgb_camera_forward(const lgb_camera* cam, float view[16], float projection[16]) {
    if (!cam || !view || !projection) return LGB_ERR_INVALID_ARGUMENT;
    double v[16], p[16];
    if (!invert4(cam->inv_view, v) || !invert4(cam->inv_projection, p)) return LGB_ERR_INVALID_ARGUMENT;
    for (int i = 0; i < 16; i++) { view[i] = (float)v[i]; projection[i] = (float)p[i]; }
    return LGB_OK;
}

LGB_API lgb_status lgb_vcm_grid(lgb_ctx* ctx, const float* d_pos4, uint32_t n, const float scene_min[3],
                                const float scene_max[3], float radius, uint32_t screen_size, uint32_t* d_count,
                                uint32_t* d_rep, void* stream) {
    if (!ctx) return LGB_ERR_INVALID_ARGUMENT;
    if (!scene_min || !scene_max || !d_count || !d_rep || (n > 0 && !d_pos4) || (reinterpret_cast<uintptr_t>(d_pos4) & 15u))
        return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "null or misaligned argument");
    if (screen_size == 0 || screen_size > 0x0CCCCCCCu || !(radius > 0.0f) || !std::isfinite(radius))
        return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "screen_size must be in [1, 2^32 / 20) and radius positive");
    for (int k = 0; k < 3; k++)
        if (!(scene_max[k] > scene_min[k])) return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "scene bounds are not a volume");
    cudaSetDevice(ctx->device);
    const cudaStream_t st = (cudaStream_t)stream;
    const uint32_t table = 10u * screen_size;
    int res[3];
    grid_resolution(scene_min, scene_max, radius, res);
    uint32_t *k0 = nullptr, *k1 = nullptr;
    uint32_t *v0 = nullptr, *v1 = nullptr, *cnt = nullptr;
    const uint32_t nb = std::max<uint32_t>(1u, (n + RS_TILE - 1) / RS_TILE);
    lgb_status result = LGB_OK;
    const size_t m = std::max<uint32_t>(n, 1u);
    if (cudaMalloc(&k0, 4 * m) != cudaSuccess || cudaMalloc(&k1, 4 * m) != cudaSuccess || cudaMalloc(&v0, 4 * m) != cudaSuccess ||
        cudaMalloc(&v1, 4 * m) != cudaSuccess || cudaMalloc(&cnt, sizeof(uint32_t) * radix_sort_scratch_words(n)) != cudaSuccess) {
        result = set_error(ctx, LGB_ERR_OUT_OF_MEMORY, "photon table scratch");
    } else {
        if (n > 0)
            k_vcm_keys_pos<<<table_grid_blocks(ctx, n), 256, 0, st>>>(reinterpret_cast<const float4*>(d_pos4), n, scene_min[0],
                                                                 scene_min[1], scene_min[2], scene_max[0], scene_max[1],
                                                                 scene_max[2], res[0], res[1], res[2], screen_size, k0, v0);
        result = build_table(ctx, k0, v0, k1, v1, cnt, n, table, d_count, d_rep, st);
        if (result == LGB_OK && cudaStreamSynchronize(st) != cudaSuccess)
            result = cuda_error(ctx, cudaGetLastError(), "lgb_vcm_grid");
    }
    cudaFree(k0); cudaFree(k1); cudaFree(v0); cudaFree(v1); cudaFree(cnt);
    return result;
}

LGB_API lgb_status lgb_vcm_iteration(lgb_scene* s, const lgb_camera* cam, const lgb_vcm_params* p, float* d_film,
                                     void* stream) {
    if (!s) return LGB_ERR_INVALID_ARGUMENT;
    Ctx* ctx = s->ctx;
    if (!cam || !p || !d_film || (reinterpret_cast<uintptr_t>(d_film) & 15u) || cam->width == 0 || cam->height == 0)
        return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "null camera / params, empty image or misaligned film");
    if (!s->bvh.nodes) return set_error(ctx, LGB_ERR_NOT_READY, "lgb_bvh_build has not been called");
    if (p->max_depth < 1 || p->max_depth > 64) return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "max_depth must be in [1, 64]");
    if (p->num_lights < 1 || (uint32_t)p->num_lights > s->num_lights || p->light_triangle_count <= 0)
        return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "VCM needs 1..num_lights lights and a positive light_triangle_count");
    if (p->dir_light_idx != 0xFFFFFFFFu || s->num_directional > 0)
        return set_error(ctx, LGB_ERR_UNSUPPORTED, "VCM supports area and spot lights only");
    if (!(p->radius > 0.0f) || !std::isfinite(p->radius)) return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "radius must be positive");
    for (int k = 0; k < 3; k++)
        if (!(p->scene_max[k] > p->scene_min[k])) return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "scene bounds are not a volume");
    if (!(p->spot_angle >= 0.0f && p->spot_angle < 90.0f))
        return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "spot_angle must be in [0, 90) degrees");
    const uint64_t screen64 = (uint64_t)cam->width * cam->height;
    const uint32_t per = (uint32_t)p->max_depth + 1u;
    if (screen64 * per >= 0x80000000ull || screen64 * 10u >= 0x80000000ull)
        return set_error(ctx, LGB_ERR_INVALID_ARGUMENT, "width * height * (max_depth + 1) must stay below 2^31");
    const uint32_t screen = (uint32_t)screen64, nv = screen * per, table = 10u * screen;
    cudaSetDevice(ctx->device);
    const cudaStream_t st = (cudaStream_t)stream;
    // state: vertices, counts, splats, table, sort scratch
    const uint32_t nb = std::max<uint32_t>(1u, (nv + RS_TILE - 1) / RS_TILE);
    size_t off = 0;
    auto take = [&](size_t bytes) { const size_t o = off; off += align256(bytes); return o; };
    const size_t o_verts = take(sizeof(float4) * kVertexF4 * (size_t)nv), o_counts = take(4ull * screen),
                 o_splat = take(12ull * screen), o_gc = take(4ull * table), o_gr = take(4ull * table), o_k0 = take(4ull * nv),
                 o_k1 = take(4ull * nv), o_v0 = take(4ull * nv), o_v1 = take(4ull * nv), o_sc = take(4ull * radix_sort_scratch_words(nv));
    // wavefront: path states, two ray queues with their path indices, hits, queue and fetch counters
    const size_t o_ls = take(sizeof(float4) * 4 * (size_t)screen), o_es = take(sizeof(float4) * 5 * (size_t)screen),
                 o_r0 = take(sizeof(lgb_ray) * (size_t)screen), o_r1 = take(sizeof(lgb_ray) * (size_t)screen),
                 o_q0 = take(4ull * screen), o_q1 = take(4ull * screen), o_hits = take(sizeof(lgb_hit) * (size_t)screen),
                 o_cnt = take(4ull * (4 * per + 2)), o_sr = take(sizeof(lgb_ray) * (size_t)nv),
                 o_sp = take(sizeof(float4) * (size_t)nv), o_sb = take(4ull * ((nv + 31) / 32));
    if (!s->vcm_buf || s->vcm_w != cam->width || s->vcm_h != cam->height || s->vcm_per != per || s->vcm_buf_bytes < off) {
        cudaFree(s->vcm_buf);
        s->vcm_buf = nullptr;
        s->vcm_buf_bytes = 0;
        LGB_CUDA_TRY(ctx, cudaMalloc(&s->vcm_buf, off));
        LGB_CUDA_TRY(ctx, cudaMemsetAsync(s->vcm_buf, 0, off, st));
        s->vcm_buf_bytes = off;
        s->vcm_w = cam->width; s->vcm_h = cam->height; s->vcm_per = per;
    }
    char* base = (char*)s->vcm_buf;
    VcmArgs A;
    std::memset(&A, 0, sizeof(A));
    for (int i = 0; i < 16; i++) { A.iv[i] = cam->inv_view[i]; A.ip[i] = cam->inv_projection[i]; }
    LGB_CUDA_TRY(ctx, lgb_camera_forward(cam, A.view, A.proj) == LGB_OK ? cudaSuccess : cudaErrorInvalidValue);
    A.W = cam->width; A.H = cam->height; A.screen = screen;
    for (int k = 0; k < 3; k++) { A.sky[k] = p->sky_col[k]; A.mn[k] = p->scene_min[k]; A.mx[k] = p->scene_max[k]; }
    A.max_depth = p->max_depth; A.num_lights = p->num_lights; A.light_tri_count = p->light_triangle_count;
    A.use_vm = p->use_vm; A.use_vc = p->use_vc;
    A.light_seed = p->light_seed; A.eye_seed = p->eye_seed; A.frame_num = p->frame_num;
    A.accumulate = (p->flags & LGB_VCM_ACCUMULATE) ? 1u : 0u;
    spot_cone(p->spot_angle, A.spot_cos_width, A.spot_cos_falloff);
    A.radius = p->radius;
    grid_resolution(A.mn, A.mx, A.radius, A.res);
    s->vcm_o_verts = o_verts; s->vcm_o_counts = o_counts; s->vcm_o_gc = o_gc; s->vcm_o_gr = o_gr;
    s->vcm_radius = A.radius;
    for (int k = 0; k < 3; k++) { s->vcm_mn[k] = A.mn[k]; s->vcm_mx[k] = A.mx[k]; s->vcm_res[k] = A.res[k]; }
    A.verts = reinterpret_cast<float4*>(base + o_verts);
    A.counts = reinterpret_cast<uint32_t*>(base + o_counts);
    A.splat = reinterpret_cast<float*>(base + o_splat);
    uint32_t* gc = reinterpret_cast<uint32_t*>(base + o_gc);
    uint32_t* gr = reinterpret_cast<uint32_t*>(base + o_gr);
    A.g_count = gc;
    A.g_rep = gr;
    A.film = reinterpret_cast<float4*>(d_film);
    Wave W;
    W.ls = reinterpret_cast<float4*>(base + o_ls);
    W.es = reinterpret_cast<float4*>(base + o_es);
    W.rays[0] = reinterpret_cast<lgb_ray*>(base + o_r0);
    W.rays[1] = reinterpret_cast<lgb_ray*>(base + o_r1);
    W.qidx[0] = reinterpret_cast<uint32_t*>(base + o_q0);
    W.qidx[1] = reinterpret_cast<uint32_t*>(base + o_q1);
    W.hits = reinterpret_cast<lgb_hit*>(base + o_hits);
    W.qcount = reinterpret_cast<uint32_t*>(base + o_cnt);
    W.tcount = W.qcount + 2 * per;
    W.scount = W.qcount + 4 * per;
    W.srays = reinterpret_cast<lgb_ray*>(base + o_sr);
    W.spay = reinterpret_cast<float4*>(base + o_sp);
    W.sbits = reinterpret_cast<uint32_t*>(base + o_sb);
    LGB_CUDA_TRY(ctx, cudaMemsetAsync(W.qcount, 0, 4ull * (4 * per + 2), st));
    LGB_CUDA_TRY(ctx, cudaMemsetAsync(W.sbits, 0, 4ull * ((nv + 31) / 32), st));
    const SceneView S = scene_view(s);
    const int sms = ctx->sm_count > 0 ? ctx->sm_count : 1;
    const uint32_t blocks_needed = (screen + kVcmThreads - 1) / kVcmThreads;
// Blocks per SM of the grid-stride step kernels: caustics iteration 7.49 ms at 16, 7.42 at 32, 7.38 at 64 and 256,
// 7.60 at 8 (the step kernels hold 4 blocks per SM; more blocks in line keep the SMs fed to the end).
#ifndef LGB_VCM_GRID
#define LGB_VCM_GRID 64u
#endif
    const int grid = (int)std::min<uint32_t>(blocks_needed, (uint32_t)sms * LGB_VCM_GRID);
    int trace_bps = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&trace_bps, k_vcm_trace, kVcmThreads, 0) != cudaSuccess || trace_bps < 1)
        trace_bps = 1;
    const int trace_grid = (int)std::min<uint32_t>(blocks_needed, (uint32_t)trace_bps * (uint32_t)sms);
    // The step kernels are instantiated per set of BSDF types (the caustics scene needs only diffuse and
    // dielectric lobes): fewer inlined lobes keep them inside the instruction cache.
    const uint32_t used = s->bsdf_mask;
    const uint32_t lobes = (used & ~kVcmLobesDG) == 0u ? kVcmLobesDG : ((used & ~kVcmLobesDGC) == 0u ? kVcmLobesDGC : kAllBsdfs);
    // bounce d of a pass: queue d - 1 traced, then stepped into queue d
    auto bounce = [&](int pass, int d) {
        const int q = (d - 1) & 1;
        k_vcm_trace<<<trace_grid, kVcmThreads, 0, st>>>(S, W.rays[q], W.hits, W.qcount + pass * per + (d - 1),
                                                         W.tcount + pass * per + (d - 1));
        if (pass == 0) {
            if (lobes == kVcmLobesDG) k_vcm_light_step<kVcmLobesDG><<<grid, kVcmThreads, 0, st>>>(S, A, W, d);
            else if (lobes == kVcmLobesDGC) k_vcm_light_step<kVcmLobesDGC><<<grid, kVcmThreads, 0, st>>>(S, A, W, d);
            else k_vcm_light_step<kAllBsdfs><<<grid, kVcmThreads, 0, st>>>(S, A, W, d);
        } else {
            if (lobes == kVcmLobesDG) k_vcm_eye_step<kVcmLobesDG><<<grid, kVcmThreads, 0, st>>>(S, A, W, d);
            else if (lobes == kVcmLobesDGC) k_vcm_eye_step<kVcmLobesDGC><<<grid, kVcmThreads, 0, st>>>(S, A, W, d);
            else k_vcm_eye_step<kAllBsdfs><<<grid, kVcmThreads, 0, st>>>(S, A, W, d);
            // the bounce's connection candidates: one any-hit launch, then their sums into the subpaths
            k_vcm_trace_any<<<trace_grid, kVcmThreads, 0, st>>>(S, W.srays, W.sbits, W.scount, W.scount + 1);
            k_vcm_eye_resolve<<<grid, kVcmThreads, 0, st>>>(A, W, d);
        }
    };
    k_vcm_light_init<<<grid, kVcmThreads, 0, st>>>(S, A, W);
    for (int d = 1; d <= A.max_depth; d++) bounce(0, d);
    // the light pass's camera connections: one any-hit launch over all of them, then the visible splats
    k_vcm_trace_any<<<trace_grid, kVcmThreads, 0, st>>>(S, W.srays, W.sbits, W.scount, W.scount + 1);
    k_vcm_splat<<<(int)std::min<uint32_t>((nv + 255) / 256, (uint32_t)sms * 8u), 256, 0, st>>>(A, W);
    LGB_CUDA_TRY(ctx, cudaGetLastError());
    if (p->use_vm == 1) {
        uint32_t* k0 = reinterpret_cast<uint32_t*>(base + o_k0);
        uint32_t* k1 = reinterpret_cast<uint32_t*>(base + o_k1);
        uint32_t* v0 = reinterpret_cast<uint32_t*>(base + o_v0);
        uint32_t* v1 = reinterpret_cast<uint32_t*>(base + o_v1);
        k_vcm_keys<<<table_grid_blocks(ctx, nv), 256, 0, st>>>(A, table, k0, v0);
        LGB_CUDA_TRY(ctx, cudaGetLastError());
        const lgb_status ts = build_table(ctx, k0, v0, k1, v1, reinterpret_cast<uint32_t*>(base + o_sc), nv, table, gc, gr, st);
        if (ts != LGB_OK) return ts;
    } else {
        LGB_CUDA_TRY(ctx, cudaMemsetAsync(gc, 0, 4ull * table, st));
    }
    k_vcm_eye_init<<<grid, kVcmThreads, 0, st>>>(A, W);
    for (int d = 1; d <= A.max_depth; d++) bounce(1, d);
    LGB_CUDA_TRY(ctx, cudaGetLastError());
    return LGB_OK;
}

LGB_API lgb_status lgb_vcm_state_get(const lgb_scene* s, lgb_vcm_state* out) {
    if (!s || !out) return LGB_ERR_INVALID_ARGUMENT;
    if (!s->vcm_buf) return set_error(s->ctx, LGB_ERR_NOT_READY, "lgb_vcm_iteration has not run on this scene");
    const char* base = static_cast<const char*>(s->vcm_buf);
    std::memset(out, 0, sizeof(*out));
    out->vertices = reinterpret_cast<const float*>(base + s->vcm_o_verts);
    out->path_counts = reinterpret_cast<const uint32_t*>(base + s->vcm_o_counts);
    out->table_count = reinterpret_cast<const uint32_t*>(base + s->vcm_o_gc);
    out->table_rep = reinterpret_cast<const uint32_t*>(base + s->vcm_o_gr);
    out->screen = s->vcm_w * s->vcm_h;
    out->per_path = s->vcm_per;
    out->table_size = 10u * out->screen;
    out->radius = s->vcm_radius;
    for (int k = 0; k < 3; k++) {
        out->grid_res[k] = s->vcm_res[k];
        out->scene_min[k] = s->vcm_mn[k];
        out->scene_max[k] = s->vcm_mx[k];
    }
    return LGB_OK;
}

}  // extern "C"
