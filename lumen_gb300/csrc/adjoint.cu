// Differentiable path tracing: primal and adjoint path replay for gradients of an image loss with respect to
// albedo texels, conductor roughness and emission. No counterpart in Lumen; built on the Path integrator's
// estimator (src/shaders/integrators/path/path.rgen:22-113, pt_commons.glsl:3-48).
//
// Estimator. Every discrete or sampling decision is detached from the parameters: directions, pdfs, MIS
// weights and Russian roulette come from the scene's own materials, while the BSDF values and emission that
// multiply the path come from the parameter buffers. With the parameters equal to the scene's values this is
// the ordinary estimator; for fixed random numbers it is a smooth function of the parameters (visibility held
// fixed), so its gradient can be checked by central finite differences with common random numbers.
//
// Adjoint. Each thread renders one sample of one pixel twice. The primal pass records the radiance collected
// at each depth; the replay pass re-runs the same path from the same counter-based RNG stream (nothing about
// the path is stored) and, at every vertex, adds
//   * for the BSDF value f at the continuation direction:   d loss / d ln f = delta * (radiance collected after it)
//   * for the BSDF values in the two light-sampling terms:  d loss / d ln f = delta * (that term's contribution)
//   * for emission: the throughput-weighted factors multiplying it,
// where delta = d loss / d sample = d loss / d image / spp. These are turned into parameter gradients with
// d f / d texel (bilinear weights) and d ln f / d roughness (GGX D and Smith G). Texel gradients go straight
// to global atomics; roughness and emission gradients are kept per thread and reduced per warp before one
// atomic per parameter.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "path_common.cuh"

namespace lgb {
namespace {

constexpr int kDiffMaxDepth = 16;
constexpr int kDiffRegMaterials = 8;  // roughness/emission gradients held in registers for materials 0..7
#ifndef LGB_DIFF_THREADS
#define LGB_DIFF_THREADS 128
#endif
#ifndef LGB_DIFF_MIN_BLOCKS
#define LGB_DIFF_MIN_BLOCKS 1
#endif
constexpr int kDiffThreads = LGB_DIFF_THREADS;      // threads per block of the path kernels
constexpr int kDiffMinBlocks = LGB_DIFF_MIN_BLOCKS; // resident blocks per SM the register budget is sized for
// The wave kernels' register budget: 4 blocks per SM (128 registers, a few spilled) against 1 (163 registers):
// 512x512x32 primal / replay 13.6 / 19.1 ms against 14.8 / 21.0.
#ifndef LGB_DIFF_WAVE_MIN_BLOCKS
#define LGB_DIFF_WAVE_MIN_BLOCKS 4
#endif
constexpr int kDiffWaveMinBlocks = LGB_DIFF_WAVE_MIN_BLOCKS;
// The completion kernels at 5 blocks per SM (96 registers, some spilled): primal 13.63 -> 13.31 ms (117-127
// registers at 4; 6 blocks, 80 registers: 13.28), replay 19.13 -> 18.79 ms (128 registers at 4; 3 blocks without
// spills: 21.07). The rays kernels (64-72 registers) stay at 4 (the primal measured 0.8 % slower at 5).
#ifndef LGB_DIFF_PRIMAL_MIN_BLOCKS
#define LGB_DIFF_PRIMAL_MIN_BLOCKS 5
#endif
#ifndef LGB_DIFF_REPLAY_MIN_BLOCKS
#define LGB_DIFF_REPLAY_MIN_BLOCKS 5
#endif
constexpr float kTMinD = 0.001f, kTMaxD = 10000.0f, kEpsD = 0.001f;

#ifndef LGB_DIFF_OUTLINE
#define LGB_DIFF_OUTLINE 0
#endif
// Code size: the path loop calls closest-hit traversal twice, any-hit once and the BSDF sampler twice, and the
// inlined body stalls on instruction fetch while a warp's paths sit at different bounces. Calling them out of
// line (1 = traversal, 2 = traversal and BSDF dispatch) keeps one copy of each but measured slower on GB300
// (call overhead and more registers: 46-55 against 69 Msamples/s at 512^2 x 32 spp), so the default inlines.
#if LGB_DIFF_OUTLINE >= 1
#define LGB_DIFF_TRACE_FN __noinline__
#else
#define LGB_DIFF_TRACE_FN __forceinline__
#endif
#if LGB_DIFF_OUTLINE >= 2
#define LGB_DIFF_BSDF_FN __noinline__
#else
#define LGB_DIFF_BSDF_FN __forceinline__
#endif

struct DiffHit {
    uint32_t prim;
    float t, u, v;
};

__device__ LGB_DIFF_TRACE_FN DiffHit diff_closest(const WideNode* __restrict__ nodes, const WideTri* __restrict__ tris,
                                                  RayQ rq, uint32_t* status) {
    DiffHit h;
    h.prim = trace_closest_single(nodes, tris, rq, h.t, h.u, h.v, status);
    return h;
}

__device__ LGB_DIFF_TRACE_FN bool diff_any(const WideNode* __restrict__ nodes, const WideTri* __restrict__ tris, RayQ rq,
                                           uint32_t* status) {
    return trace_any_single(nodes, tris, rq, status);
}

struct BsdfSample {
    v3 f, wi;
    float pdf, cos_t;
};

template <uint32_t MASK>
__device__ LGB_DIFF_BSDF_FN BsdfSample diff_sample_bsdf(v3 n_s, v3 wo, Mat m, bool side, v3 r) {
    BsdfSample b;
    b.f = sample_bsdf<MASK>(n_s, wo, m, side, b.wi, b.pdf, b.cos_t, r);
    return b;
}

template <uint32_t MASK>
__device__ LGB_DIFF_BSDF_FN float4 diff_eval_bsdf(v3 n_s, v3 wo, Mat m, bool side, v3 wi) {
    float pdf;
    const v3 f = eval_bsdf<MASK>(n_s, wo, m, side, wi, pdf);
    return make_float4(f.x, f.y, f.z, pdf);
}

struct DiffArgs {
    float iv[16], ip[16];
    uint32_t width, height, npix;
    float sky[3];
    int max_depth, num_lights, light_tri_count;
    uint32_t direct_lighting, frame0, spp, num_materials;
    int tex_id;                 // texture whose texels are parameters (-1 = none)
    uint32_t sample_params;     // sampling uses the evaluation material too
    const float4* texels;       // its evaluation texels, tex_w * tex_h
    uint32_t tex_w, tex_h;
    const float* rough;         // evaluation roughness per material (null = scene values)
    const float* emis;          // evaluation emission per material, RGB (null = scene values)
    float4* samples;            // primal: radiance per sample, [spp][npix]
    const float4* dimage;       // adjoint: d loss / d image per pixel
    const float4* primal;       // adjoint: radiance per sample from the primal, [spp][npix] (null = recompute)
    float4* g_tex;              // adjoint outputs
    float* g_rough;
    float* g_emis;
};

struct EvalMat {
    Mat m;              // evaluation material
    bool textured;      // albedo = base * parameter texture
    v3 base;            // untextured albedo
    float tex_w[4];     // bilinear weights and texel indices of the lookup
    uint32_t tex_i[4];
    v3 texc;            // interpolated texel colour
};

__device__ __forceinline__ v3 bilinear(const float4* __restrict__ t, uint32_t W, uint32_t H, float u, float v, float* w,
                                       uint32_t* idx) {
    if (!isfinite(u) || !isfinite(v)) { u = 0.0f; v = 0.0f; }
    const float x = u * (float)W - 0.5f, y = v * (float)H - 0.5f;
    const float x0 = floorf(x), y0 = floorf(y);
    const float fx = x - x0, fy = y - y0;
    const long long Wl = W, Hl = H;
    long long ix = (long long)x0 % Wl; if (ix < 0) ix += Wl;
    long long iy = (long long)y0 % Hl; if (iy < 0) iy += Hl;
    const long long ix1 = (ix + 1) % Wl, iy1 = (iy + 1) % Hl;
    idx[0] = (uint32_t)(iy * Wl + ix); idx[1] = (uint32_t)(iy * Wl + ix1);
    idx[2] = (uint32_t)(iy1 * Wl + ix); idx[3] = (uint32_t)(iy1 * Wl + ix1);
    w[0] = (1.0f - fx) * (1.0f - fy); w[1] = fx * (1.0f - fy); w[2] = (1.0f - fx) * fy; w[3] = fx * fy;
    return f3(t[idx[0]]) * w[0] + f3(t[idx[1]]) * w[1] + f3(t[idx[2]]) * w[2] + f3(t[idx[3]]) * w[3];
}

__device__ __forceinline__ EvalMat eval_material(const SceneView& S, const DiffArgs& A, const Mat& ms, uint32_t mat_idx,
                                                 float u, float v) {
    EvalMat e;
    e.m = ms;
    e.textured = false;
    const lgb_material* src = &S.mats[mat_idx];
    e.base = V3(src->albedo[0], src->albedo[1], src->albedo[2]);
    if (A.texels && src->texture_id >= 0 && src->texture_id == A.tex_id) {
        e.textured = true;
        e.texc = bilinear(A.texels, A.tex_w, A.tex_h, u, v, e.tex_w, e.tex_i);
        e.m.albedo = e.base * e.texc;
    }
    if (A.rough) e.m.roughness = A.rough[mat_idx];
    if (A.emis) e.m.emissive = V3(A.emis[3 * mat_idx], A.emis[3 * mat_idx + 1], A.emis[3 * mat_idx + 2]);
    return e;
}

// Value of the evaluation BSDF for (wo, wi) in world space. Diffuse and rough conductors depend on the
// parameters; every other lobe keeps the detached value `fallback`.
__device__ __forceinline__ v3 eval_value(const EvalMat& e, v3 n_s, v3 wo, v3 wi, v3 fallback, bool from_sample) {
    v3 T, B;
    branchless_onb(n_s, T, B);
    const v3 wol = to_local(wo, T, B, n_s), wil = to_local(wi, T, B, n_s);
    if (e.m.type == LGB_BSDF_DIFFUSE) {
        float pdf;
        const v3 f = eval_diffuse(e.m, wol, wil, pdf);
        return from_sample && fallback.x == 0.0f && fallback.y == 0.0f && fallback.z == 0.0f ? V3(0.0f) : f;
    }
    if (e.m.type == LGB_BSDF_CONDUCTOR && !effectively_delta(e.m.roughness * e.m.roughness)) {
        float pdf;
        return eval_conductor(e.m, wol, wil, pdf);
    }
    return fallback;
}

// d ln(D G) / d roughness of the isotropic GGX conductor (D_iso and the height-correlated Smith G of
// microfacet_commons.glsl, alpha = roughness^2, so alpha^2 = roughness^4).
__device__ __forceinline__ float conductor_dlog_dr(float r, v3 wol, v3 wil) {
    const float alpha = r * r, a2 = alpha * alpha;
    v3 h = normalize(wol + wil);
    h = h * signf(h.z);
    const float c2 = h.z * h.z;
    const float d = c2 * (a2 - 1.0f) + 1.0f;
    const float dlnD = 1.0f / a2 - 2.0f * c2 / d;
    auto lam = [&](float c, float& dl) {
        const float cs = c * c;
        const float ts = fmaxf(1.0f - cs, 0.0f) / cs;
        const float q = sqrtf(1.0f + a2 * ts);
        dl = c == 0.0f ? 0.0f : 0.25f * ts / q;
        return c == 0.0f ? 0.0f : 0.5f * (q - 1.0f);
    };
    float dlo, dli;
    const float lo = lam(wol.z, dlo), li = lam(wil.z, dli);
    const float G = 1.0f / (1.0f + lo + li);
    const float dlnG = -(dlo + dli) * G;
    return (dlnD + dlnG) * 4.0f * r * r * r;
}

// Roughness and emission gradients of materials 0..kDiffRegMaterials-1 are summed in shared memory per block
// and pushed with one global atomic per parameter at the end; other materials go straight to global memory.
struct GradAcc {
    float* rough;  // shared, kDiffRegMaterials
    float* emis;   // shared, 3 * kDiffRegMaterials
};

__device__ __forceinline__ void add_emis(const DiffArgs& A, GradAcc& g, uint32_t m, v3 v) {
    if (!(isfinite(v.x) && isfinite(v.y) && isfinite(v.z))) return;
    if (m < kDiffRegMaterials) {
        atomicAdd(&g.emis[3 * m], v.x); atomicAdd(&g.emis[3 * m + 1], v.y); atomicAdd(&g.emis[3 * m + 2], v.z);
    } else {
        atomicAdd(&A.g_emis[3 * m], v.x); atomicAdd(&A.g_emis[3 * m + 1], v.y); atomicAdd(&A.g_emis[3 * m + 2], v.z);
    }
}

// sf = d loss / d ln f per channel for the rough-conductor value f(wo, wi) of evaluation material e.
__device__ __forceinline__ void add_rough_grad(const DiffArgs& A, GradAcc& g, const EvalMat& e, uint32_t m, v3 sf,
                                               v3 n_s, v3 wo, v3 wi) {
    if (e.m.type != LGB_BSDF_CONDUCTOR || !A.rough || effectively_delta(e.m.roughness * e.m.roughness)) return;
    v3 T, B;
    branchless_onb(n_s, T, B);
    const float q = conductor_dlog_dr(e.m.roughness, to_local(wo, T, B, n_s), to_local(wi, T, B, n_s));
    const float v = (sf.x + sf.y + sf.z) * q;
    if (!isfinite(v)) return;
    atomicAdd(m < kDiffRegMaterials ? &g.rough[m] : &A.g_rough[m], v);
}

// Warp-aggregated float4 reduction into base[idx]: the active lanes with the same index form one group
// (__match_any_sync); its lowest lane sums the group's values, taken from each member by shuffles within the
// group, and issues the one 16-byte reduction. Neighbouring pixels of a coherent bounce land on the same texels,
// so most groups hold several lanes; a lane alone in its group reduces directly.
__device__ __forceinline__ void red_add_f4_aggregated(float4* base, uint32_t idx, float4 v) {
    const unsigned active = __activemask();
    const unsigned peers = __match_any_sync(active, idx);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    unsigned rest = peers & ~(1u << leader);
    while (rest) {  // every member runs the same iterations: the group shares `peers`
        const int m = __ffs(rest) - 1;
        rest &= rest - 1u;
        const float x = __shfl_sync(peers, v.x, m), y = __shfl_sync(peers, v.y, m), z = __shfl_sync(peers, v.z, m);
        if (lane == leader) { v.x += x; v.y += y; v.z += z; }
    }
    if (lane == leader) atomicAdd(base + idx, v);
}

// Texel gradients of one vertex. All BSDF values of a textured diffuse vertex share the texture lookup, so
// their d loss / d ln f add up first: f_c = base_c * tex_c / pi gives d loss / d texel_{i,c} = sf_c * w_i / tex_c,
// one warp-aggregated float4 reduction per bilinear tap.
__device__ __forceinline__ void flush_texel_grad(const DiffArgs& A, const EvalMat& e, v3 sf) {
    if (!e.textured || e.m.type != LGB_BSDF_DIFFUSE) return;
    if (sf.x == 0.0f && sf.y == 0.0f && sf.z == 0.0f) return;
    const v3 s = V3(e.texc.x > 0.0f ? sf.x / e.texc.x : 0.0f, e.texc.y > 0.0f ? sf.y / e.texc.y : 0.0f,
                    e.texc.z > 0.0f ? sf.z / e.texc.z : 0.0f);
    if (!(isfinite(s.x) && isfinite(s.y) && isfinite(s.z))) return;
    for (int k = 0; k < 4; k++) {
        const float w = e.tex_w[k];
        if (w == 0.0f) continue;
        red_add_f4_aggregated(A.g_tex, e.tex_i[k], make_float4(s.x * w, s.y * w, s.z * w, 0.0f));
    }
}

// Replay modes of diff_path.
enum : int {
    kPrimal = 0,       // radiance only
    kReplaySuffix = 1, // contrib holds, per depth, the radiance collected after that depth
    kReplayTotal = 2,  // total holds the sample's radiance; the radiance after each depth is what remains
    kRecord = 3,       // radiance, and the radiance collected at each depth written to contrib
};

// State of one sample's path between bounces.
struct DPath {
    uint4 seed;
    v3 origin, dir;
    v3 Tv, Tc;       // throughput with the evaluation values / with the sampler's values (Russian roulette)
    v3 L, rem;       // radiance so far; radiance still to come (kReplayTotal)
    bool last_spec;
};

// The camera ray of one sample of pixel `pix` at `frame` (path.rgen:23-38).
__device__ __forceinline__ DPath diff_begin(const DiffArgs& A, uint32_t pix, uint32_t frame, v3 total) {
    DPath P;
    const uint32_t x = pix % A.width, y = pix / A.width;
    P.seed = make_uint4(x, y, frame, 0u);
    const float r0 = rnd(P.seed) - 0.5f;
    const float r1 = rnd(P.seed) - 0.5f;
    const float pu = ((float)x + 0.5f + r0) / (float)A.width, pv = ((float)y + 0.5f + r1) / (float)A.height;
    const float dx = pu * 2.0f - 1.0f, dy = pv * 2.0f - 1.0f;
    const float4 o4 = mat_vec(A.iv, 0.0f, 0.0f, 0.0f, 1.0f);
    const float4 t4 = mat_vec(A.ip, dx, dy, 1.0f, 1.0f);
    const v3 tn = normalize(V3(t4.x, t4.y, t4.z));
    const float4 d4 = mat_vec(A.iv, tn.x, tn.y, tn.z, 0.0f);
    P.origin = V3(o4.x, o4.y, o4.z);
    P.dir = V3(d4.x, d4.y, d4.z);
    P.Tv = V3(1.0f); P.Tc = V3(1.0f); P.L = V3(0.0f); P.rem = total;
    P.last_spec = false;
    return P;
}

// How a vertex gets its two secondary traversals: inline (the loop below), or in a wavefront as two passes over
// the same code, the first recording the NEE shadow ray and the BSDF-MIS ray, the second taking their results.
enum : int { kPhaseInline = 0, kPhaseRays = 1, kPhaseResults = 2 };
struct VertexIO {
    float4 sray[2], mray[2];  // kPhaseRays: the rays to trace as (origin, tmin) (direction, tmax); tmin > tmax: none
    bool occluded;      // kPhaseResults: the shadow ray's result
    DiffHit mhit;       // kPhaseResults: the BSDF-MIS ray's closest hit
};
enum : int { kStepContinue = 0, kStepEnd = 1 };

// One bounce (depth) of the path at the closest hit ph of its current ray (the body of path.rgen's loop):
// emission, next-event estimation with both MIS strategies, the continuation sample and Russian roulette, and in
// the replay modes the gradients of the vertex. Returns kStepEnd when the path ends here.
template <int MODE, uint32_t MASK, int PHASE>
__device__ int diff_vertex(const SceneView& S, const DiffArgs& A, DPath& P, int depth, const DiffHit& ph, v3* contrib,
                           v3 delta, GradAcc& g, VertexIO& io) {
    constexpr bool ADJ = MODE == kReplaySuffix || MODE == kReplayTotal;
    uint4& seed = P.seed;
    v3& origin = P.origin;
    v3& dir = P.dir;
    v3& Tv = P.Tv;
    v3& Tc = P.Tc;
    v3& L = P.L;
    v3& rem = P.rem;
    bool& last_spec = P.last_spec;
    const v3 sky = V3(A.sky[0], A.sky[1], A.sky[2]);
    v3 Cd = V3(0.0f);
    const uint32_t prim = ph.prim;
    const float bu = ph.u, bv = ph.v;
    if (prim == LGB_NO_HIT) {
        if (depth > 0 || A.direct_lighting == 1u) Cd = Tv * sky;
        if (MODE == kRecord) contrib[depth] = Cd;
        L = L + Cd;
        return kStepEnd;
    }
    const HitAttr h = resolve_hit(S, prim, bu, bv);
    Mat ms = load_material(S, h.mat, h.u, h.v);
    const EvalMat em = eval_material(S, A, ms, h.mat, h.u, h.v);
    if (A.sample_params) ms = em.m;  // then every BSDF value below is the sampler's own
    if ((depth == 0 && A.direct_lighting == 1u) || last_spec) {
        Cd = Cd + Tv * em.m.emissive;
        if (ADJ && PHASE != kPhaseRays && A.emis) add_emis(A, g, h.mat, delta * Tv);
    }
    if (depth >= A.max_depth - 1) {
        if (MODE == kRecord) contrib[depth] = Cd;
        L = L + Cd;
        return kStepEnd;
    }
    const v3 wo = -dir;
    v3 n_s = h.n_s;
    bool side = true;
    v3 n_g = h.n_g;
    if (dot(h.n_g, wo) < 0.0f) n_g = -n_g;
    if (dot(n_g, h.n_s) < 0.0f) { n_s = -n_s; side = false; }
    const v3 next_origin = offset_ray(h.pos, n_g);
    const bool spec = has_prop(ms.props, LGB_FLAG_SPECULAR);
    v3 sf_tex = V3(0.0f);  // d loss / d ln f summed over this vertex's BSDF values (texel gradients)
    if (!spec && (depth > 0 || A.direct_lighting == 1u)) {
        if (A.num_lights <= 0) {
            for (int k = 0; k < 4; k++) (void)rnd(seed);
        } else {
            const float lpp = 1.0f / (float)A.light_tri_count;
            const float q0 = rnd(seed), q1 = rnd(seed), q2 = rnd(seed), q3 = rnd(seed);
            const uint32_t li = (uint32_t)(q0 * (float)A.num_lights);
            const lgb_light* Lt = &S.lights[li];
            const uint32_t ltype = Lt->light_flags & 7u;
            v3 Le = V3(0.0f), wi = V3(0.0f);
            float wi_len = 0.0f, pdf_w = 0.0f, pdf_a = 0.0f;
            uint32_t lprim = LGB_NO_HIT, lmat = 0xFFFFFFFFu, lio = 0u, lvo = 0u;
            if (ltype == LGB_LIGHT_AREA) {
                const lgb_mesh pm = S.meshes[Lt->prim_mesh_idx];
                const uint32_t tri = (uint32_t)(q1 * (float)Lt->num_triangles);
                lprim = S.mesh_first[Lt->prim_mesh_idx] + tri;
                const uint32_t io = pm.index_offset + 3u * tri;
                lio = io;
                lvo = pm.vertex_offset;
                const DevVertex a = S.verts[S.idx[io] + pm.vertex_offset];
                const DevVertex b = S.verts[S.idx[io + 1] + pm.vertex_offset];
                const DevVertex c = S.verts[S.idx[io + 2] + pm.vertex_offset];
                const float su = 1.0f - sqrtf(q2), sv = q3 * sqrtf(q2);
                const float b0 = 1.0f - su - sv;
                const v3 v0 = V3(a.px, a.py, a.pz), v1 = V3(b.px, b.py, b.pz), v2 = V3(c.px, c.py, c.pz);
                const v3 lpos = v0 * b0 + v1 * su + v2 * sv;
                const v3 ln = normalize(normalize(V3(a.nx, a.ny, a.nz) * b0 + V3(b.nx, b.ny, b.nz) * su +
                                                  V3(c.nx, c.ny, c.nz) * sv));
                const float tri_pdf = 2.0f / length(cross(v1 - v0, v2 - v0));
                lmat = pm.material_index;
                const lgb_material* lm = &S.mats[lmat];
                Le = A.emis ? V3(A.emis[3 * lmat], A.emis[3 * lmat + 1], A.emis[3 * lmat + 2])
                            : V3(lm->emissive_factor[0], lm->emissive_factor[1], lm->emissive_factor[2]);
                wi = lpos - h.pos;
                const float l2 = dot(wi, wi);
                wi_len = sqrtf(l2);
                wi = wi / wi_len;
                const float cfl = fabsf(dot(ln, -wi));
                pdf_a = tri_pdf;
                pdf_w = pdf_a * l2 / cfl;
            } else if (ltype == LGB_LIGHT_SPOT) {
                const v3 lp = V3(Lt->pos[0], Lt->pos[1], Lt->pos[2]);
                wi = lp - h.pos;
                const float l2 = dot(wi, wi);
                wi_len = sqrtf(l2);
                wi = wi / wi_len;
                const v3 ldir = normalize(V3(Lt->to[0], Lt->to[1], Lt->to[2]) - lp);
                const float cfl = dot(-wi, ldir);
                const float cw = cosf(LGB_PI / 6.0f), cf = cosf(25.0f * LGB_PI / 180.0f);
                float fall;
                if (cfl < cw) fall = 0.0f;
                else if (cfl >= cf) fall = 1.0f;
                else { const float dd = (cfl - cw) / (cf - cw); fall = (dd * dd) * (dd * dd); }
                pdf_a = 1.0f;
                pdf_w = l2;
                Le = V3(Lt->L[0], Lt->L[1], Lt->L[2]) * fall;
            } else {
                const v3 ddir = normalize(V3(Lt->pos[0], Lt->pos[1], Lt->pos[2]) - V3(Lt->to[0], Lt->to[1], Lt->to[2]));
                const v3 lp = h.pos + ddir * (2.0f * Lt->world_radius);
                wi = lp - h.pos;
                wi_len = length(wi);
                wi = wi / wi_len;
                pdf_a = 1.0f;
                pdf_w = 1.0f;
                Le = V3(Lt->L[0], Lt->L[1], Lt->L[2]);
            }
            const v3 sp = offset_ray2(h.pos, n_s);
            const float cos_x = dot(n_s, wi);
            const float4 fp1 = diff_eval_bsdf<MASK>(n_s, wo, ms, side, wi);
            const v3 fs1 = V3(fp1.x, fp1.y, fp1.z);
            const float bsdf_pdf = fp1.w;
            const v3 fe1 = A.sample_params ? fs1 : eval_value(em, n_s, wo, wi, fs1, false);
            v3 term1 = V3(0.0f), k1 = V3(0.0f);
            if (pdf_w > 0.0f) {
                const RayQ sq = make_rayq(sp.x, sp.y, sp.z, 0.0f, wi.x, wi.y, wi.z, wi_len - kEpsD);
                bool visible = false;
                if constexpr (PHASE == kPhaseInline) visible = !diff_any(S.nodes, S.tris, sq, S.status);
                else if constexpr (PHASE == kPhaseRays) {
                    io.sray[0] = make_float4(sp.x, sp.y, sp.z, 0.0f);
                    io.sray[1] = make_float4(wi.x, wi.y, wi.z, wi_len - kEpsD);
                }
                else visible = !io.occluded;
                if (visible) {
                    const float mis = ((Lt->light_flags >> 5) & 1u) ? 1.0f : 1.0f / (1.0f + bsdf_pdf / pdf_w);
                    k1 = mis * fe1 * fabsf(cos_x) / pdf_w;  // term1 = k1 * Le
                    term1 = k1 * Le;
                }
            }
            v3 term2 = V3(0.0f), k2 = V3(0.0f), wi2 = V3(0.0f);
            if (ltype == LGB_LIGHT_AREA) {
                const float b0r = rnd(seed), b1r = rnd(seed), b2r = rnd(seed);
                const BsdfSample bs2 = diff_sample_bsdf<MASK>(n_s, wo, ms, side, V3(b0r, b1r, b2r));
                const v3 fs2 = bs2.f;
                const float pdf2 = bs2.pdf, cos2 = bs2.cos_t;
                wi2 = bs2.wi;
                const RayQ mq = make_rayq(sp.x, sp.y, sp.z, kTMinD, wi2.x, wi2.y, wi2.z, kTMaxD);
                bool may_count = pdf2 != 0.0f;
                if (may_count && lprim != prim) {
                    // Only a closest hit on the sampled light triangle counts (a miss reuses the shading
                    // triangle, which differs here): a ray that fails the traversal's own watertight test
                    // against that triangle cannot count, so it is not traced.
                    const DevVertex a = S.verts[S.idx[lio] + lvo];
                    const DevVertex b = S.verts[S.idx[lio + 1] + lvo];
                    const DevVertex c = S.verts[S.idx[lio + 2] + lvo];
                    float tt, tu, tv;
                    may_count = tri_intersect(mq, make_float4(a.px, a.py, a.pz, 0.0f),
                                              make_float4(b.px, b.py, b.pz, 0.0f),
                                              make_float4(c.px, c.py, c.pz, 0.0f), mq.tmax, tt, tu, tv);
                }
                if constexpr (PHASE == kPhaseRays) {
                    if (may_count) {
                        io.mray[0] = make_float4(sp.x, sp.y, sp.z, kTMinD);
                        io.mray[1] = make_float4(wi2.x, wi2.y, wi2.z, kTMaxD);
                    }
                    may_count = false;
                }
                if (may_count) {
                    DiffHit mhit;
                    if constexpr (PHASE == kPhaseInline) mhit = diff_closest(S.nodes, S.tris, mq, S.status);
                    else mhit = io.mhit;
                    const uint32_t mprim = mhit.prim;
                    const float mu = mhit.u, mv = mhit.v;
                    // a missed MIS ray leaves the previous payload (ray.rmiss:13): compare the shading triangle
                    const uint32_t pl_prim = mprim == LGB_NO_HIT ? prim : mprim;
                    if (pl_prim == lprim) {
                        v3 pl_pos = h.pos, pl_ns = h.n_s;
                        if (mprim != LGB_NO_HIT) {
                            const HitAttr mh = resolve_hit(S, mprim, mu, mv);
                            pl_pos = mh.pos;
                            pl_ns = mh.n_s;
                        }
                        const float wl = length(pl_pos - h.pos);
                        const float gg = fabsf(dot(pl_ns, -wi2)) / (wl * wl);
                        const float mis = 1.0f / (1.0f + pdf_a / (gg * pdf2));
                        const v3 fe2 = A.sample_params ? fs2 : eval_value(em, n_s, wo, wi2, fs2, true);
                        k2 = fe2 * mis * fabsf(cos2) / pdf2;
                        term2 = k2 * Le;
                    }
                }
            }
            const v3 res = term1 + term2;
            Cd = Cd + Tv * res / lpp;
            if (ADJ && PHASE != kPhaseRays) {
                if (A.emis && lmat != 0xFFFFFFFFu) add_emis(A, g, lmat, delta * Tv * (k1 + k2) / lpp);
                const v3 sf1 = delta * (Tv * term1 / lpp), sf2 = delta * (Tv * term2 / lpp);
                sf_tex = sf1 + sf2;
                add_rough_grad(A, g, em, h.mat, sf1, n_s, wo, wi);
                if (ltype == LGB_LIGHT_AREA) add_rough_grad(A, g, em, h.mat, sf2, n_s, wo, wi2);
            }
        }
    }
    if constexpr (PHASE == kPhaseRays) return kStepContinue;  // the vertex's rays are recorded
    const float c0 = rnd(seed), c1 = rnd(seed), c2 = rnd(seed);
    const BsdfSample bs = diff_sample_bsdf<MASK>(n_s, wo, ms, side, V3(c0, c1, c2));
    const v3 fs = bs.f, dnext = bs.wi;
    const float pdf = bs.pdf, cos_t = bs.cos_t;
    if (MODE == kRecord) contrib[depth] = Cd;
    L = L + Cd;
    v3 after = V3(0.0f);  // radiance collected after this depth
    if (MODE == kReplaySuffix) after = contrib[depth];
    if (MODE == kReplayTotal) { rem = rem - Cd; after = rem; }
    if (pdf == 0.0f) {
        if (ADJ) flush_texel_grad(A, em, sf_tex);
        return kStepEnd;
    }
    const v3 fe = A.sample_params ? fs : eval_value(em, n_s, wo, dnext, fs, true);
    if (ADJ) {
        const v3 sf3 = delta * after;
        add_rough_grad(A, g, em, h.mat, sf3, n_s, wo, dnext);
        flush_texel_grad(A, em, sf_tex + sf3);
    }
    Tv = Tv * (fe * fabsf(cos_t) / pdf);
    Tc = Tc * (fs * fabsf(cos_t) / pdf);
    float rr_scale = 1.0f;
    if (has_prop(ms.props, LGB_FLAG_TRANSMISSION)) rr_scale *= side ? 1.0f / ms.ior : ms.ior;
    if (depth > 3) {
        const float rr = fminf(0.95f, luminance(Tc) * rr_scale);
        if (rr == 0.0f || rr < rnd(seed)) return kStepEnd;
        Tv = Tv / rr;
        Tc = Tc / rr;
    }
    origin = next_origin;
    dir = dnext;
    last_spec = spec;
    return kStepContinue;
}

// One sample of pixel `pix` at `frame`; returns its radiance. The replay modes accumulate gradients.
template <int MODE, uint32_t MASK>
__device__ v3 diff_path(const SceneView& S, const DiffArgs& A, uint32_t pix, uint32_t frame, v3* contrib, v3 total,
                        v3 delta, GradAcc& g) {
    DPath P = diff_begin(A, pix, frame, total);
    VertexIO io;
    for (int depth = 0; depth < kDiffMaxDepth; depth++) {
        const RayQ rq = make_rayq(P.origin.x, P.origin.y, P.origin.z, kTMinD, P.dir.x, P.dir.y, P.dir.z, kTMaxD);
        const DiffHit ph = diff_closest(S.nodes, S.tris, rq, S.status);
        if (diff_vertex<MODE, MASK, kPhaseInline>(S, A, P, depth, ph, contrib, delta, g, io) == kStepEnd) break;
    }
    return P.L;
}

// The loop form, one thread per sample. MODE kPrimal writes each sample's radiance; kReplaySuffix re-runs the
// primal in the thread (kRecord, keeping the per-depth radiance in local memory) and then replays; kReplayTotal
// replays once from the stored radiance of each sample. The library runs kPrimal and kReplayTotal as wavefronts
// (diff_wave below) and this kernel for kReplaySuffix, the replay without stored samples.
template <int MODE, uint32_t MASK>
__global__ void __launch_bounds__(kDiffThreads, kDiffMinBlocks) k_diff(SceneView S, DiffArgs A) {
    __shared__ float sh_grad[4 * kDiffRegMaterials];
    constexpr bool ADJ = MODE != kPrimal;
    GradAcc g{sh_grad, sh_grad + kDiffRegMaterials};
    if (ADJ) {
        for (int i = threadIdx.x; i < 4 * kDiffRegMaterials; i += blockDim.x) sh_grad[i] = 0.0f;
        __syncthreads();
    }
    const uint32_t n = A.npix * A.spp;
    const uint32_t stride = gridDim.x * blockDim.x;
    const float inv = 1.0f / (float)A.spp;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint32_t pix = i % A.npix, k = i / A.npix;
        if (MODE == kPrimal) {
            // a sample whose radiance is not finite counts as zero and is marked (w = 0) so the replay skips it;
            // Lumen's film drops such samples (path.rgen:102-104)
            const v3 L = diff_path<kPrimal, MASK>(S, A, pix, A.frame0 + k, nullptr, V3(0.0f), V3(0.0f), g);
            const bool ok = isfinite(L.x) && isfinite(L.y) && isfinite(L.z);
            A.samples[(size_t)k * A.npix + pix] = ok ? make_float4(L.x, L.y, L.z, 1.0f) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        } else {
            const float4 di = A.dimage[pix];
            const v3 delta = V3(di.x * inv, di.y * inv, di.z * inv);
            if (delta.x == 0.0f && delta.y == 0.0f && delta.z == 0.0f) continue;
            if (MODE == kReplayTotal) {
                const float4 tot = A.primal[(size_t)k * A.npix + pix];
                if (tot.w == 0.0f) continue;
                (void)diff_path<kReplayTotal, MASK>(S, A, pix, A.frame0 + k, nullptr, V3(tot.x, tot.y, tot.z), delta, g);
            } else {
                v3 contrib[kDiffMaxDepth];
                for (int d = 0; d < kDiffMaxDepth; d++) contrib[d] = V3(0.0f);
                const v3 L = diff_path<kRecord, MASK>(S, A, pix, A.frame0 + k, contrib, V3(0.0f), V3(0.0f), g);
                if (!(isfinite(L.x) && isfinite(L.y) && isfinite(L.z))) continue;
                v3 acc = V3(0.0f);  // per-depth radiance into suffix sums, summed back to front
                for (int d = kDiffMaxDepth - 1; d >= 0; d--) {
                    const v3 c = contrib[d];
                    contrib[d] = acc;
                    acc = acc + c;
                }
                (void)diff_path<kReplaySuffix, MASK>(S, A, pix, A.frame0 + k, contrib, V3(0.0f), delta, g);
            }
        }
    }
    if (ADJ) {
        __syncthreads();
        const uint32_t nm = min(A.num_materials, (uint32_t)kDiffRegMaterials);
        for (uint32_t j = threadIdx.x; j < nm; j += blockDim.x) {
            if (A.rough && sh_grad[j] != 0.0f) atomicAdd(&A.g_rough[j], sh_grad[j]);
            if (A.emis) {
                for (int c = 0; c < 3; c++) {
                    const float e = sh_grad[kDiffRegMaterials + 3 * j + c];
                    if (e != 0.0f) atomicAdd(&A.g_emis[3 * j + c], e);
                }
            }
        }
    }
}

// Kernel instantiation for a scene's BSDF types: diffuse + conductor scenes get a kernel without the
// dielectric and principled lobes.
template <int MODE>
void launch_diff(Scene* s, const DiffArgs& A, int grid, cudaStream_t cs) {
    constexpr uint32_t kDC = LGB_BSDF_DIFFUSE | LGB_BSDF_CONDUCTOR;
    if ((s->bsdf_mask & ~kDC) == 0) k_diff<MODE, kDC><<<grid, kDiffThreads, 0, cs>>>(scene_view(s), A);
    else k_diff<MODE, sh::kAllBsdfs><<<grid, kDiffThreads, 0, cs>>>(scene_view(s), A);
}

// Wavefront form of the sample loop for kPrimal and kReplayTotal. Per bounce: the closest hits of the queued rays
// (the persistent traversal kernel, lanes whose ray is done fetch the next), a pass over the vertices that records
// each one's shadow ray and BSDF-MIS ray, their traversals, and a pass that completes the vertices with those
// results and queues the continuation rays. Both passes run diff_vertex on the same state (the RNG counter is part
// of it), so a sample's arithmetic and random numbers are the loop's; the instruction footprint of each kernel is a
// fraction of the loop's.
struct DiffWave {
    float4* st;        // sample state, 6 consecutive float4 per sample: (origin, rng) (dir, last_spec) (Tv) (Tc) (L) (rem)
    lgb_ray* rays[2];  // ray queues of consecutive bounces
    uint32_t* qidx[2]; // sample of each queued ray
    lgb_hit* hits;
    lgb_ray* srays;    // per queue slot: the vertex's shadow ray (tmin > tmax: none)
    uint32_t* sbits;   // their occlusion bits
    lgb_ray* mrays;    // per queue slot: the vertex's BSDF-MIS ray
    lgb_hit* mhits;
    uint32_t* counts;  // queue lengths per bounce [kDiffMaxDepth + 1], then 3 fetch counters per bounce, then
                       // the lengths of the 3 BSDF-class lists per bounce
    uint32_t* cls[3];  // per BSDF class: the queue slots of the bounce's vertices in that class
    uint32_t n;        // samples: npix * spp, sample i = frame (i / npix), pixel (i % npix)
};
constexpr int kDiffCountWords = (kDiffMaxDepth + 1) + 3 * kDiffMaxDepth + 3 * kDiffMaxDepth;
__device__ __forceinline__ uint32_t* cls_list(const DiffWave& W, int c) {
    return c == 0 ? W.cls[0] : (c == 1 ? W.cls[1] : W.cls[2]);
}
__device__ __forceinline__ uint32_t* class_counts(const DiffWave& W, int depth) {
    return W.counts + (kDiffMaxDepth + 1) + 3 * kDiffMaxDepth + 3 * depth;
}
// A sample's 96 B of state are contiguous: the completion passes visit samples out of queue order (per-class
// lists), and a scattered sample then costs three full 32 B sectors.
__device__ __forceinline__ float4* wst(const DiffWave& W, int c, uint32_t i) { return W.st + ((size_t)i * 6 + c); }
__device__ __forceinline__ void store_dpath(const DiffWave& W, uint32_t i, const DPath& P) {
    *wst(W, 0, i) = f4(P.origin, __uint_as_float(P.seed.w));
    *wst(W, 1, i) = f4(P.dir, __uint_as_float(P.last_spec ? 1u : 0u));
    *wst(W, 2, i) = f4(P.Tv, 0.0f);
    *wst(W, 3, i) = f4(P.Tc, 0.0f);
    *wst(W, 4, i) = f4(P.L, 0.0f);
    *wst(W, 5, i) = f4(P.rem, 0.0f);
}
__device__ __forceinline__ DPath load_dpath(const DiffWave& W, const DiffArgs& A, uint32_t i) {
    const uint32_t pix = i % A.npix, frame = A.frame0 + i / A.npix;
    const float4 a = *wst(W, 0, i), b = *wst(W, 1, i), c = *wst(W, 2, i), d = *wst(W, 3, i), e = *wst(W, 4, i),
                 f = *wst(W, 5, i);
    DPath P;
    P.seed = make_uint4(pix % A.width, pix / A.width, frame, __float_as_uint(a.w));
    P.origin = V3(a.x, a.y, a.z);
    P.dir = V3(b.x, b.y, b.z);
    P.last_spec = __float_as_uint(b.w) != 0u;
    P.Tv = V3(c.x, c.y, c.z); P.Tc = V3(d.x, d.y, d.z); P.L = V3(e.x, e.y, e.z); P.rem = V3(f.x, f.y, f.z);
    return P;
}
__device__ __forceinline__ uint32_t diff_append(uint32_t* counter) {
    const uint32_t mask = __activemask();
    const int leader = __ffs(mask) - 1;
    const int lane = (int)(threadIdx.x & 31u);
    uint32_t first = 0;
    if (lane == leader) first = atomicAdd(counter, (uint32_t)__popc(mask));
    first = __shfl_sync(mask, first, leader);
    return first + (uint32_t)__popc(mask & ((1u << lane) - 1u));
}
// One slot of list `c` (of three, counters at `counters`) for each calling lane; lanes with the same list share
// one atomic.
__device__ __forceinline__ uint32_t diff_append_to(uint32_t* counters, int c) {
    const uint32_t mask = __activemask();
    const uint32_t peers = __match_any_sync(mask, c);
    const int leader = __ffs(peers) - 1;
    const int lane = (int)(threadIdx.x & 31u);
    uint32_t first = 0;
    if (lane == leader) first = atomicAdd(counters + c, (uint32_t)__popc(peers));
    first = __shfl_sync(peers, first, leader);
    return first + (uint32_t)__popc(peers & ((1u << lane) - 1u));
}
__device__ __forceinline__ void push_diff_ray(const DiffWave& W, int q, uint32_t* counter, uint32_t i, const DPath& P) {
    const uint32_t j = diff_append(counter);
    (q ? W.qidx[1] : W.qidx[0])[j] = i;  // selects: an indexed pointer array would be copied to local memory
    float4* r = reinterpret_cast<float4*>(&(q ? W.rays[1] : W.rays[0])[j]);
    r[0] = make_float4(P.origin.x, P.origin.y, P.origin.z, kTMinD);
    r[1] = make_float4(P.dir.x, P.dir.y, P.dir.z, kTMaxD);
}

constexpr int kDiffTraceMinBlocks = 9;
// A warp refetches rays once all its lanes are idle: 512x512x32 primal / replay 15.8 / 22.7 ms at 16 idle lanes,
// 16.2 / 23.0 at 8, 15.4 / 22.2 at 32.
#ifdef LGB_DIFF_REFILL
constexpr int kDiffRefill = LGB_DIFF_REFILL;
#else
constexpr int kDiffRefill = 32;
#endif
#ifdef LGB_DIFF_POSTPONE
constexpr bool kDiffPostpone = LGB_DIFF_POSTPONE != 0;
#else
constexpr bool kDiffPostpone = false;
#endif
#ifdef LGB_DIFF_TRI_MIN
constexpr int kDiffTriMin = LGB_DIFF_TRI_MIN;
#else
constexpr int kDiffTriMin = 0;
#endif
__global__ void __launch_bounds__(kDiffThreads, kDiffTraceMinBlocks)
    k_diff_trace(SceneView S, const lgb_ray* __restrict__ rays, lgb_hit* __restrict__ hits, const uint32_t* count,
                 uint32_t* fetch) {
    trace_persistent<false, false, kDiffPostpone, 0, kDiffThreads, kDiffRefill, kDiffTriMin>(S.nodes, S.tris, rays, hits, nullptr, 0u, count,
                                                                      fetch, S.status, nullptr, nullptr, nullptr);
}
// A bounce's BSDF-MIS rays (closest hit) and shadow rays (any hit) in one launch, the MIS rays first: warps move on
// to the shadow rays as the MIS queue runs dry, so neither trace ends the bounce alone on its last few rays.
__global__ void __launch_bounds__(kDiffThreads, kDiffTraceMinBlocks)
    k_diff_trace_nee(SceneView S, const lgb_ray* __restrict__ mrays, lgb_hit* __restrict__ mhits,
                     const lgb_ray* __restrict__ srays, uint32_t* __restrict__ sbits, const uint32_t* count,
                     uint32_t* mfetch, uint32_t* sfetch) {
    trace_persistent<false, false, kDiffPostpone, 0, kDiffThreads, kDiffRefill, kDiffTriMin>(S.nodes, S.tris, mrays, mhits, nullptr, 0u, count,
                                                                      mfetch, S.status, nullptr, nullptr, nullptr);
    trace_persistent<true, false, kDiffPostpone, 0, kDiffThreads, kDiffRefill, kDiffTriMin>(S.nodes, S.tris, srays, nullptr, sbits, 0u, count,
                                                                     sfetch, S.status, nullptr, nullptr, nullptr);
}

// The camera rays of every sample into queue 0; the replay skips the samples the loop form skips (zero d loss /
// d pixel, a primal sample marked not finite).
template <int MODE>
__global__ void __launch_bounds__(kDiffThreads) k_diff_wave_init(DiffArgs A, DiffWave W) {
    const float inv = 1.0f / (float)A.spp;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < W.n; i += gridDim.x * blockDim.x) {
        const uint32_t pix = i % A.npix;
        v3 total = V3(0.0f);
        if (MODE == kReplayTotal) {
            const float4 di = A.dimage[pix];
            if (di.x * inv == 0.0f && di.y * inv == 0.0f && di.z * inv == 0.0f) continue;
            const float4 tot = A.primal[i];
            if (tot.w == 0.0f) continue;
            total = V3(tot.x, tot.y, tot.z);
        }
        const DPath P = diff_begin(A, pix, A.frame0 + i / A.npix, total);
        store_dpath(W, i, P);
        push_diff_ray(W, 0, W.counts, i, P);
    }
}

// One pass over the vertices of bounce `depth`: PHASE kPhaseRays records their rays and sorts the vertices into
// three lists by the class of their material's BSDF type (diffuse, conductor, the rest; a miss or a type without
// lobes goes to class miss_cls), kPhaseResults completes the vertices of one class (cls). MASK keeps only that
// class's lobes in the completion kernel, so each launch's code is a fraction of the loop's (the pass stalls on
// instruction fetch otherwise).
template <int MODE, uint32_t MASK, int PHASE>
__global__ void __launch_bounds__(kDiffThreads, PHASE != kPhaseResults ? kDiffWaveMinBlocks
                                                : MODE == kPrimal       ? LGB_DIFF_PRIMAL_MIN_BLOCKS
                                                                        : LGB_DIFF_REPLAY_MIN_BLOCKS)
    k_diff_wave(SceneView S, DiffArgs A, DiffWave W, int depth, int cls, int miss_cls) {
    __shared__ float sh_grad[4 * kDiffRegMaterials];
    constexpr bool GRAD = MODE != kPrimal && PHASE == kPhaseResults;
    GradAcc g{sh_grad, sh_grad + kDiffRegMaterials};
    if (GRAD) {
        for (int t = threadIdx.x; t < 4 * kDiffRegMaterials; t += blockDim.x) sh_grad[t] = 0.0f;
        __syncthreads();
    }
    const uint32_t n = PHASE == kPhaseResults ? class_counts(W, depth)[cls] : W.counts[depth];
    const int q = depth & 1;
    const float inv = 1.0f / (float)A.spp;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const uint32_t j = PHASE == kPhaseResults ? cls_list(W, cls)[t] : t;
        const lgb_hit hh = W.hits[j];
        const uint32_t i = (q ? W.qidx[1] : W.qidx[0])[j];
        DPath P = load_dpath(W, A, i);
        const DiffHit ph{hh.prim, hh.t, hh.u, hh.v};
        v3 delta = V3(0.0f);
        if (MODE != kPrimal) {
            const float4 di = A.dimage[i % A.npix];
            delta = V3(di.x * inv, di.y * inv, di.z * inv);
        }
        VertexIO io;
        if (PHASE == kPhaseRays) {
            io.sray[0] = io.mray[0] = make_float4(0.0f, 0.0f, 0.0f, 1.0f);  // tmin > tmax: no ray
            io.sray[1] = io.mray[1] = make_float4(0.0f, 0.0f, 1.0f, 0.0f);
        } else {
            io.occluded = ((W.sbits[j >> 5] >> (j & 31u)) & 1u) != 0u;
            const lgb_hit mh = W.mhits[j];
            io.mhit = DiffHit{mh.prim, mh.t, mh.u, mh.v};
        }
        const int r = diff_vertex<MODE, MASK, PHASE>(S, A, P, depth, ph, nullptr, delta, g, io);
        if (PHASE == kPhaseRays) {
            float4* sr = reinterpret_cast<float4*>(&W.srays[j]);
            float4* mr = reinterpret_cast<float4*>(&W.mrays[j]);
            sr[0] = io.sray[0]; sr[1] = io.sray[1];
            mr[0] = io.mray[0]; mr[1] = io.mray[1];
            const uint32_t ty = hh.prim == LGB_NO_HIT ? 0u : S.mats[S.meshes[S.tri_mesh[hh.prim]].material_index].bsdf_type;
            const int c = (ty & LGB_BSDF_DIFFUSE) ? 0 : ((ty & LGB_BSDF_CONDUCTOR) ? 1 : ((ty & sh::kAllBsdfs) ? 2 : miss_cls));
            cls_list(W, c)[diff_append_to(class_counts(W, depth), c)] = j;
        } else if (r == kStepContinue) {
            store_dpath(W, i, P);
            push_diff_ray(W, q ^ 1, W.counts + depth + 1, i, P);
        } else if (MODE == kPrimal) {
            // a sample whose radiance is not finite counts as zero and is marked (w = 0) so the replay skips it;
            // Lumen's film drops such samples (path.rgen:102-104)
            const v3 L = P.L;
            const bool ok = isfinite(L.x) && isfinite(L.y) && isfinite(L.z);
            A.samples[i] = ok ? make_float4(L.x, L.y, L.z, 1.0f) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
    }
    if (GRAD) {
        __syncthreads();
        const uint32_t nm = min(A.num_materials, (uint32_t)kDiffRegMaterials);
        for (uint32_t t = threadIdx.x; t < nm; t += blockDim.x) {
            if (A.rough && sh_grad[t] != 0.0f) atomicAdd(&A.g_rough[t], sh_grad[t]);
            if (A.emis) {
                for (int c = 0; c < 3; c++) {
                    const float e = sh_grad[kDiffRegMaterials + 3 * t + c];
                    if (e != 0.0f) atomicAdd(&A.g_emis[3 * t + c], e);
                }
            }
        }
    }
}

// Film = mean of the spp samples of each pixel, summed in frame order.
__global__ void k_mean(const float4* __restrict__ samples, uint32_t npix, uint32_t spp, float4* __restrict__ film) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x) {
        float sx = 0.0f, sy = 0.0f, sz = 0.0f;
        for (uint32_t k = 0; k < spp; k++) {
            const float4 v = samples[(size_t)k * npix + p];
            sx += v.x; sy += v.y; sz += v.z;
        }
        const float inv = 1.0f / (float)spp;
        film[p] = make_float4(sx * inv, sy * inv, sz * inv, 1.0f);
    }
}

}  // namespace
}  // namespace lgb

using namespace lgb;

namespace {

lgb_status make_diff_args(lgb_scene* s, const lgb_camera* cam, const lgb_path_params* p, const lgb_diff_params* dp,
                          uint32_t frame0, uint32_t spp, DiffArgs& A) {
    if (!cam || !p || !dp || cam->width == 0 || cam->height == 0 || spp == 0)
        return set_error(s->ctx, LGB_ERR_INVALID_ARGUMENT, "null camera/params/diff params or zero spp");
    if (!s->bvh.nodes) return set_error(s->ctx, LGB_ERR_NOT_READY, "lgb_bvh_build has not been called");
    if (p->max_depth > kDiffMaxDepth) return set_error(s->ctx, LGB_ERR_UNSUPPORTED, "differentiable path depth is limited to 16");
    if (p->num_lights < 0 || (uint32_t)p->num_lights > s->num_lights || (p->num_lights > 0 && p->light_triangle_count <= 0))
        return set_error(s->ctx, LGB_ERR_INVALID_ARGUMENT, "bad light counts");
    if (p->dir_light_idx != 0xFFFFFFFFu) return set_error(s->ctx, LGB_ERR_UNSUPPORTED, "directional-light atmosphere unsupported");
    if ((uint64_t)cam->width * cam->height * spp >= 0x80000000ull)
        return set_error(s->ctx, LGB_ERR_INVALID_ARGUMENT, "width * height * spp must stay below 2^31");
    if (dp->texels) {
        if (dp->texture_id < 0 || (uint32_t)dp->texture_id >= s->num_textures)
            return set_error(s->ctx, LGB_ERR_INVALID_ARGUMENT, "texture_id of the texel parameters is out of range");
        if (reinterpret_cast<uintptr_t>(dp->texels) & 15u)
            return set_error(s->ctx, LGB_ERR_INVALID_ARGUMENT, "texel parameters must be 16-byte aligned");
    }
    if ((reinterpret_cast<uintptr_t>(dp->roughness) & 3u) || (reinterpret_cast<uintptr_t>(dp->emission) & 3u))
        return set_error(s->ctx, LGB_ERR_INVALID_ARGUMENT, "roughness/emission parameters must be 4-byte aligned");
    std::memset(&A, 0, sizeof(A));
    for (int i = 0; i < 16; i++) { A.iv[i] = cam->inv_view[i]; A.ip[i] = cam->inv_projection[i]; }
    A.width = cam->width; A.height = cam->height; A.npix = cam->width * cam->height;
    for (int i = 0; i < 3; i++) A.sky[i] = p->sky_col[i];
    A.max_depth = p->max_depth; A.num_lights = p->num_lights; A.light_tri_count = p->light_triangle_count;
    A.direct_lighting = p->direct_lighting; A.frame0 = frame0; A.spp = spp; A.num_materials = s->num_materials;
    A.tex_id = dp->texels ? dp->texture_id : -1;
    A.sample_params = (dp->flags & LGB_DIFF_SAMPLE_PARAMS) ? 1u : 0u;
    A.texels = reinterpret_cast<const float4*>(dp->texels);
    if (dp->texels) {
        DevTexture t;
        LGB_CUDA_TRY(s->ctx, cudaMemcpy(&t, s->d_textures + dp->texture_id, sizeof(t), cudaMemcpyDeviceToHost));
        A.tex_w = t.width; A.tex_h = t.height;
    }
    A.rough = dp->roughness;
    A.emis = dp->emission;
    return LGB_OK;
}

int diff_grid(Ctx* ctx, uint32_t n) {
    const int sms = ctx->sm_count > 0 ? ctx->sm_count : 1;
// Blocks per SM of the grid-stride wave kernels (512x512x32 primal / replay): 15.4 / 22.2 ms at 16, 14.9 / 21.4 at
// 32, 14.8 / 21.1 at 64, 14.8 / 21.0 at 256.
#ifndef LGB_DIFF_GRID
#define LGB_DIFF_GRID 256u
#endif
    return (int)std::min<uint32_t>((n + kDiffThreads - 1) / kDiffThreads, (uint32_t)sms * LGB_DIFF_GRID);
}

size_t align256d(size_t x) { return (x + 255) & ~(size_t)255; }

// BSDF classes of the completion pass: diffuse, conductor, and the other types together.
constexpr uint32_t kDiffClsD = LGB_BSDF_DIFFUSE, kDiffClsC = LGB_BSDF_CONDUCTOR;
constexpr uint32_t kDiffClsRest = sh::kAllBsdfs & ~(LGB_BSDF_DIFFUSE | LGB_BSDF_CONDUCTOR);

template <int MODE, uint32_t MASK>
cudaError_t diff_wave_passes(Scene* s, const DiffArgs& A, const DiffWave& W, int bounces, int grid, int trace_grid,
                             cudaStream_t cs) {
    const SceneView S = scene_view(s);
    const uint32_t used = s->bsdf_mask;
    // misses and types without lobes are completed with the first class the scene has (no BSDF code is reached)
    const int miss_cls = (used & kDiffClsD) ? 0 : ((used & kDiffClsC) ? 1 : 2);
    const bool has[3] = {(used & kDiffClsD) != 0u || miss_cls == 0, (used & kDiffClsC) != 0u || miss_cls == 1,
                         (used & kDiffClsRest) != 0u || miss_cls == 2};
    for (int d = 0; d < bounces; d++) {
        uint32_t* f = W.counts + (kDiffMaxDepth + 1) + 3 * d;  // fetch counters of the bounce's three traversals
        k_diff_trace<<<trace_grid, kDiffThreads, 0, cs>>>(S, W.rays[d & 1], W.hits, W.counts + d, f);
        k_diff_wave<MODE, MASK, kPhaseRays><<<grid, kDiffThreads, 0, cs>>>(S, A, W, d, -1, miss_cls);
        const cudaError_t me = cudaMemsetAsync(W.sbits, 0, 4ull * ((W.n + 31) / 32), cs);
        if (me != cudaSuccess) return me;
        k_diff_trace_nee<<<trace_grid, kDiffThreads, 0, cs>>>(S, W.mrays, W.mhits, W.srays, W.sbits, W.counts + d, f + 2,
                                                              f + 1);
        if (has[0]) k_diff_wave<MODE, kDiffClsD, kPhaseResults><<<grid, kDiffThreads, 0, cs>>>(S, A, W, d, 0, miss_cls);
        if (has[1]) k_diff_wave<MODE, kDiffClsC, kPhaseResults><<<grid, kDiffThreads, 0, cs>>>(S, A, W, d, 1, miss_cls);
        if (has[2]) k_diff_wave<MODE, kDiffClsRest, kPhaseResults><<<grid, kDiffThreads, 0, cs>>>(S, A, W, d, 2, miss_cls);
        const cudaError_t le = cudaGetLastError();
        if (le != cudaSuccess) return le;
    }
    return cudaSuccess;
}

// The wavefront form (kPrimal or kReplayTotal) of one lgb_diff_render / lgb_adjoint_path call.
template <int MODE>
lgb_status diff_wave(Scene* s, const DiffArgs& A, cudaStream_t cs) {
    Ctx* ctx = s->ctx;
    DiffWave W;
    W.n = A.npix * A.spp;
    const size_t n = W.n;
    size_t off = 0;
    auto take = [&](size_t bytes) { const size_t o = off; off += align256d(bytes); return o; };
    const size_t o_st = take(sizeof(float4) * 6 * n), o_r0 = take(sizeof(lgb_ray) * n), o_r1 = take(sizeof(lgb_ray) * n),
                 o_q0 = take(4 * n), o_q1 = take(4 * n), o_h = take(sizeof(lgb_hit) * n), o_sr = take(sizeof(lgb_ray) * n),
                 o_sb = take(4 * ((n + 31) / 32)), o_mr = take(sizeof(lgb_ray) * n), o_mh = take(sizeof(lgb_hit) * n),
                 o_c = take(4 * (size_t)kDiffCountWords), o_l0 = take(4 * n), o_l1 = take(4 * n), o_l2 = take(4 * n);
    if (s->diffw_buf_bytes < off) {
        cudaFree(s->diffw_buf);
        s->diffw_buf = nullptr;
        s->diffw_buf_bytes = 0;
        LGB_CUDA_TRY(ctx, cudaMalloc(&s->diffw_buf, off));
        s->diffw_buf_bytes = off;
    }
    char* b = (char*)s->diffw_buf;
    W.st = reinterpret_cast<float4*>(b + o_st);
    W.rays[0] = reinterpret_cast<lgb_ray*>(b + o_r0);
    W.rays[1] = reinterpret_cast<lgb_ray*>(b + o_r1);
    W.qidx[0] = reinterpret_cast<uint32_t*>(b + o_q0);
    W.qidx[1] = reinterpret_cast<uint32_t*>(b + o_q1);
    W.hits = reinterpret_cast<lgb_hit*>(b + o_h);
    W.srays = reinterpret_cast<lgb_ray*>(b + o_sr);
    W.sbits = reinterpret_cast<uint32_t*>(b + o_sb);
    W.mrays = reinterpret_cast<lgb_ray*>(b + o_mr);
    W.mhits = reinterpret_cast<lgb_hit*>(b + o_mh);
    W.counts = reinterpret_cast<uint32_t*>(b + o_c);
    W.cls[0] = reinterpret_cast<uint32_t*>(b + o_l0);
    W.cls[1] = reinterpret_cast<uint32_t*>(b + o_l1);
    W.cls[2] = reinterpret_cast<uint32_t*>(b + o_l2);
    LGB_CUDA_TRY(ctx, cudaMemsetAsync(W.counts, 0, 4 * (size_t)kDiffCountWords, cs));
    const int sms = ctx->sm_count > 0 ? ctx->sm_count : 1;
    const int grid = diff_grid(ctx, W.n);
    int tb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&tb, k_diff_trace, kDiffThreads, 0) != cudaSuccess || tb < 1) tb = 1;
    const int trace_grid = (int)std::min<uint64_t>((n + kDiffThreads - 1) / kDiffThreads, (uint64_t)tb * sms);
    // a path ends at depth max_depth - 1 at the latest (path.rgen:60)
    const int bounces = std::max(1, std::min(A.max_depth, kDiffMaxDepth));
    k_diff_wave_init<MODE><<<grid, kDiffThreads, 0, cs>>>(A, W);
    constexpr uint32_t kDC = LGB_BSDF_DIFFUSE | LGB_BSDF_CONDUCTOR;
    if ((s->bsdf_mask & ~kDC) == 0) LGB_CUDA_TRY(ctx, (diff_wave_passes<MODE, kDC>(s, A, W, bounces, grid, trace_grid, cs)));
    else LGB_CUDA_TRY(ctx, (diff_wave_passes<MODE, sh::kAllBsdfs>(s, A, W, bounces, grid, trace_grid, cs)));
    LGB_CUDA_TRY(ctx, cudaGetLastError());
    return LGB_OK;
}

}  // namespace

extern "C" LGB_API lgb_status lgb_diff_render(lgb_scene* s, const lgb_camera* cam, const lgb_path_params* p,
                                              const lgb_diff_params* dp, uint32_t frame0, uint32_t spp, float* d_film,
                                              float* d_samples, void* stream) {
    if (!s) return LGB_ERR_INVALID_ARGUMENT;
    if (!d_film || (reinterpret_cast<uintptr_t>(d_film) & 15u) || (reinterpret_cast<uintptr_t>(d_samples) & 15u))
        return set_error(s->ctx, LGB_ERR_INVALID_ARGUMENT, "film and samples must be 16-byte aligned device pointers");
    cudaSetDevice(s->ctx->device);
    DiffArgs A;
    lgb_status st = make_diff_args(s, cam, p, dp, frame0, spp, A);
    if (st != LGB_OK) return st;
    if (d_samples) {
        A.samples = reinterpret_cast<float4*>(d_samples);
    } else {
        const size_t bytes = sizeof(float4) * (size_t)A.npix * spp;
        if (s->diff_buf_bytes < bytes) {
            cudaFree(s->diff_buf);
            s->diff_buf = nullptr;
            s->diff_buf_bytes = 0;
            LGB_CUDA_TRY(s->ctx, cudaMalloc(&s->diff_buf, bytes));
            s->diff_buf_bytes = bytes;
        }
        A.samples = reinterpret_cast<float4*>(s->diff_buf);
    }
    const cudaStream_t cs = (cudaStream_t)stream;
    st = diff_wave<kPrimal>(s, A, cs);
    if (st != LGB_OK) return st;
    k_mean<<<diff_grid(s->ctx, A.npix), kDiffThreads, 0, cs>>>(A.samples, A.npix, spp, reinterpret_cast<float4*>(d_film));
    LGB_CUDA_TRY(s->ctx, cudaGetLastError());
    return LGB_OK;
}

extern "C" LGB_API lgb_status lgb_adjoint_path(lgb_scene* s, const lgb_camera* cam, const lgb_path_params* p,
                                               const lgb_diff_params* dp, uint32_t frame0, uint32_t spp,
                                               const float* d_dloss_dimage, const float* d_primal_samples,
                                               lgb_diff_grads* grads, void* stream) {
    if (!s) return LGB_ERR_INVALID_ARGUMENT;
    if (!d_dloss_dimage || !grads || (reinterpret_cast<uintptr_t>(d_dloss_dimage) & 15u) ||
        (reinterpret_cast<uintptr_t>(d_primal_samples) & 15u))
        return set_error(s->ctx, LGB_ERR_INVALID_ARGUMENT, "null or misaligned d_dloss_dimage / samples / grads");
    if ((dp && dp->texels && !grads->texels) || (dp && dp->roughness && !grads->roughness) ||
        (dp && dp->emission && !grads->emission))
        return set_error(s->ctx, LGB_ERR_INVALID_ARGUMENT, "a gradient buffer is missing for a parameter set");
    if ((reinterpret_cast<uintptr_t>(grads->texels) & 15u) || (reinterpret_cast<uintptr_t>(grads->roughness) & 3u) ||
        (reinterpret_cast<uintptr_t>(grads->emission) & 3u))
        return set_error(s->ctx, LGB_ERR_INVALID_ARGUMENT, "misaligned gradient buffer");
    cudaSetDevice(s->ctx->device);
    DiffArgs A;
    lgb_status st = make_diff_args(s, cam, p, dp, frame0, spp, A);
    if (st != LGB_OK) return st;
    A.dimage = reinterpret_cast<const float4*>(d_dloss_dimage);
    A.primal = reinterpret_cast<const float4*>(d_primal_samples);
    A.g_tex = reinterpret_cast<float4*>(grads->texels);
    A.g_rough = grads->roughness;
    A.g_emis = grads->emission;
    const cudaStream_t cs = (cudaStream_t)stream;
    const int grid = diff_grid(s->ctx, A.npix * spp);
    if (A.primal) {
        st = diff_wave<kReplayTotal>(s, A, cs);
        if (st != LGB_OK) return st;
    } else {
        launch_diff<kReplaySuffix>(s, A, grid, cs);
    }
    LGB_CUDA_TRY(s->ctx, cudaGetLastError());
    return LGB_OK;
}
