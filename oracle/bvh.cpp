// Oracle (test infrastructure only): CPU triangle BVH and ray queries.
//
// Stands in for the closed driver traversal behind traceRayEXT (src/shaders/integrators/path/path.rgen:48,
// src/shaders/integrators/pt_commons.glsl:21,32). The answer is defined independently of any tree:
//   closest hit = the triangle with the smallest watertight-test t in [tmin, tmax], the lowest primitive
//                 id winning equal t;
//   any hit     = whether any triangle passes the test in [tmin, tmax].
// The BVH (binned SAH, binary, up to 4 triangles per leaf) only prunes; its box tests run in double
// precision with a relative slack so that no triangle that could win is ever culled.
#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

namespace {

// Watertight ray/triangle intersection, Woop, Benthin and Wald, "Watertight Ray/Triangle Intersection",
// JCGT 2(1) 2013. The operation order below is the contract shared with the CUDA traversal kernels:
// every product and sum is a separately rounded FP32 operation (built with -ffp-contract=off).
struct RayPre {
    float o[3];
    float tmin, tmax;
    int kx, ky, kz;
    float Sx, Sy, Sz;
};

inline RayPre precompute(const float* o, const float* d, float tmin, float tmax) {
    RayPre r;
    r.o[0] = o[0]; r.o[1] = o[1]; r.o[2] = o[2];
    r.tmin = tmin; r.tmax = tmax;
    float ax = std::fabs(d[0]), ay = std::fabs(d[1]), az = std::fabs(d[2]);
    int kz = 0;
    if (ay > ax) kz = 1;
    if (az > (kz == 0 ? ax : ay)) kz = 2;
    int kx = kz + 1; if (kx == 3) kx = 0;
    int ky = kx + 1; if (ky == 3) ky = 0;
    if (d[kz] < 0.0f) std::swap(kx, ky);
    r.kx = kx; r.ky = ky; r.kz = kz;
    r.Sx = d[kx] / d[kz];
    r.Sy = d[ky] / d[kz];
    r.Sz = 1.0f / d[kz];
    return r;
}

// Returns true and t, u, v (Vulkan barycentrics: u weights v1, v weights v2) on a hit with t in [tmin, tmax].
inline bool intersect(const RayPre& r, const float* v, float& t_out, float& u_out, float& v_out) {
    const float Ax_ = v[0] - r.o[0], Ay_ = v[1] - r.o[1], Az_ = v[2] - r.o[2];
    const float Bx_ = v[3] - r.o[0], By_ = v[4] - r.o[1], Bz_ = v[5] - r.o[2];
    const float Cx_ = v[6] - r.o[0], Cy_ = v[7] - r.o[1], Cz_ = v[8] - r.o[2];
    const float A[3] = {Ax_, Ay_, Az_}, B[3] = {Bx_, By_, Bz_}, C[3] = {Cx_, Cy_, Cz_};
    const float Ax = A[r.kx] - r.Sx * A[r.kz];
    const float Ay = A[r.ky] - r.Sy * A[r.kz];
    const float Bx = B[r.kx] - r.Sx * B[r.kz];
    const float By = B[r.ky] - r.Sy * B[r.kz];
    const float Cx = C[r.kx] - r.Sx * C[r.kz];
    const float Cy = C[r.ky] - r.Sy * C[r.kz];
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        // Edge case: redo the three 2D edge functions in double precision (exact for FP32 inputs).
        double CxBy = (double)Cx * (double)By, CyBx = (double)Cy * (double)Bx;
        double AxCy = (double)Ax * (double)Cy, AyCx = (double)Ay * (double)Cx;
        double BxAy = (double)Bx * (double)Ay, ByAx = (double)By * (double)Ax;
        U = (float)(CxBy - CyBx);
        V = (float)(AxCy - AyCx);
        W = (float)(BxAy - ByAx);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = U + V + W;
    if (det == 0.0f) return false;
    const float Az = r.Sz * A[r.kz];
    const float Bz = r.Sz * B[r.kz];
    const float Cz = r.Sz * C[r.kz];
    const float T = U * Az + V * Bz + W * Cz;
    const float t = T / det;
    if (!(t >= r.tmin && t <= r.tmax)) return false;
    t_out = t;
    u_out = V / det;
    v_out = W / det;
    return true;
}

struct Box {
    float lo[3], hi[3];
    void reset() {
        for (int i = 0; i < 3; i++) { lo[i] = std::numeric_limits<float>::max(); hi[i] = -std::numeric_limits<float>::max(); }
    }
    void grow(const float* p) {
        for (int i = 0; i < 3; i++) { lo[i] = std::min(lo[i], p[i]); hi[i] = std::max(hi[i], p[i]); }
    }
    void grow(const Box& b) {
        for (int i = 0; i < 3; i++) { lo[i] = std::min(lo[i], b.lo[i]); hi[i] = std::max(hi[i], b.hi[i]); }
    }
    double area() const {
        double dx = (double)hi[0] - lo[0], dy = (double)hi[1] - lo[1], dz = (double)hi[2] - lo[2];
        if (dx < 0 || dy < 0 || dz < 0) return 0.0;
        return 2.0 * (dx * dy + dy * dz + dz * dx);
    }
};

struct Node {
    Box box;
    uint32_t left_or_first;  // internal: left child index; leaf: first index into order[]
    uint32_t count;          // 0 = internal (right child = left + 1 is NOT assumed; see right)
    uint32_t right;
};

struct Bvh {
    std::vector<Node> nodes;
    std::vector<uint32_t> order;
    std::vector<float> verts;  // 9 per triangle, original order
};

struct BuildItem { Box box; float c[3]; };

uint32_t build_rec(Bvh& bvh, std::vector<BuildItem>& items, uint32_t first, uint32_t count, int depth) {
    uint32_t idx = (uint32_t)bvh.nodes.size();
    bvh.nodes.push_back(Node());
    Box box; box.reset();
    Box cbox; cbox.reset();
    for (uint32_t i = first; i < first + count; i++) {
        box.grow(items[bvh.order[i]].box);
        cbox.grow(items[bvh.order[i]].c);
    }
    bvh.nodes[idx].box = box;
    if (count <= 4 || depth > 60) {
        bvh.nodes[idx].left_or_first = first;
        bvh.nodes[idx].count = count;
        return idx;
    }
    // binned SAH over the centroid box, 16 bins per axis
    const int NB = 16;
    double best_cost = std::numeric_limits<double>::max();
    int best_axis = -1, best_split = -1;
    for (int axis = 0; axis < 3; axis++) {
        double ext = (double)cbox.hi[axis] - cbox.lo[axis];
        if (ext <= 0.0) continue;
        Box bb[NB]; uint32_t bc[NB];
        for (int b = 0; b < NB; b++) { bb[b].reset(); bc[b] = 0; }
        for (uint32_t i = first; i < first + count; i++) {
            const BuildItem& it = items[bvh.order[i]];
            int b = (int)(NB * ((double)it.c[axis] - cbox.lo[axis]) / ext);
            b = std::min(std::max(b, 0), NB - 1);
            bb[b].grow(it.box); bc[b]++;
        }
        double right_area[NB]; uint32_t right_cnt[NB];
        Box acc; acc.reset(); uint32_t cnt = 0;
        for (int b = NB - 1; b > 0; b--) {
            acc.grow(bb[b]); cnt += bc[b];
            right_area[b] = acc.area(); right_cnt[b] = cnt;
        }
        acc.reset(); cnt = 0;
        for (int b = 0; b < NB - 1; b++) {
            acc.grow(bb[b]); cnt += bc[b];
            if (cnt == 0 || right_cnt[b + 1] == 0) continue;
            double cost = acc.area() * cnt + right_area[b + 1] * right_cnt[b + 1];
            if (cost < best_cost) { best_cost = cost; best_axis = axis; best_split = b; }
        }
    }
    uint32_t mid;
    if (best_axis < 0) {
        mid = first + count / 2;  // all centroids coincide: split by count
    } else {
        double lo = cbox.lo[best_axis], ext = (double)cbox.hi[best_axis] - lo;
        auto it = std::partition(bvh.order.begin() + first, bvh.order.begin() + first + count, [&](uint32_t p) {
            int b = (int)(NB * ((double)items[p].c[best_axis] - lo) / ext);
            b = std::min(std::max(b, 0), NB - 1);
            return b <= best_split;
        });
        mid = (uint32_t)(it - bvh.order.begin());
        if (mid == first || mid == first + count) mid = first + count / 2;
    }
    uint32_t l = build_rec(bvh, items, first, mid - first, depth + 1);
    uint32_t r = build_rec(bvh, items, mid, first + count - mid, depth + 1);
    bvh.nodes[idx].left_or_first = l;
    bvh.nodes[idx].right = r;
    bvh.nodes[idx].count = 0;
    return idx;
}

// Double-precision slab test with relative slack: returns false only when the box certainly cannot
// contain a hit with t in [tmin, tlimit].
struct RayBox {
    double o[3], inv[3];
};
inline RayBox make_raybox(const float* o, const float* d) {
    RayBox rb;
    for (int i = 0; i < 3; i++) {
        double di = d[i];
        if (di == 0.0) di = 1e-300;  // parallel axis: a huge slab distance keeps min/max ordering valid
        rb.o[i] = o[i];
        rb.inv[i] = 1.0 / di;
    }
    return rb;
}
inline bool box_hit(const RayBox& rb, const Box& b, double tmin, double tlimit, double& tnear) {
    double t0 = -std::numeric_limits<double>::infinity(), t1 = std::numeric_limits<double>::infinity();
    for (int i = 0; i < 3; i++) {
        double a = ((double)b.lo[i] - rb.o[i]) * rb.inv[i];
        double c = ((double)b.hi[i] - rb.o[i]) * rb.inv[i];
        if (a > c) std::swap(a, c);
        t0 = std::max(t0, a);
        t1 = std::min(t1, c);
    }
    const double slack = 1.0 / 4096.0;
    double lo_lim = tmin - std::fabs(tmin) * slack - 1e-30;
    double hi_lim = tlimit + std::fabs(tlimit) * slack + 1e-30;
    tnear = t0;
    return t0 <= t1 + std::fabs(t1) * slack + 1e-30 && t1 >= lo_lim && t0 <= hi_lim;
}

void closest_one(const Bvh& bvh, const orc_ray& ray, orc_hit& hit) {
    RayPre rp = precompute(ray.o, ray.d, ray.tmin, ray.tmax);
    RayBox rb = make_raybox(ray.o, ray.d);
    float best_t = ray.tmax;
    uint32_t best = 0xFFFFFFFFu;
    float bu = 0, bv = 0;
    uint32_t stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const Node& n = bvh.nodes[stack[--sp]];
        double tn;
        if (!box_hit(rb, n.box, ray.tmin, best_t, tn)) continue;
        if (n.count > 0) {
            for (uint32_t i = 0; i < n.count; i++) {
                uint32_t p = bvh.order[n.left_or_first + i];
                float t, u, v;
                if (intersect(rp, &bvh.verts[9 * (size_t)p], t, u, v)) {
                    if (t < best_t || (t == best_t && p < best)) { best_t = t; best = p; bu = u; bv = v; }
                }
            }
        } else {
            double tl, tr;
            bool hl = box_hit(rb, bvh.nodes[n.left_or_first].box, ray.tmin, best_t, tl);
            bool hr = box_hit(rb, bvh.nodes[n.right].box, ray.tmin, best_t, tr);
            if (hl && hr) {
                if (tl <= tr) { stack[sp++] = n.right; stack[sp++] = n.left_or_first; }
                else { stack[sp++] = n.left_or_first; stack[sp++] = n.right; }
            } else if (hl) stack[sp++] = n.left_or_first;
            else if (hr) stack[sp++] = n.right;
        }
    }
    hit.prim = best;
    hit.t = best == 0xFFFFFFFFu ? 0.0f : best_t;
    hit.u = bu; hit.v = bv;
}

bool any_one(const Bvh& bvh, const orc_ray& ray) {
    RayPre rp = precompute(ray.o, ray.d, ray.tmin, ray.tmax);
    RayBox rb = make_raybox(ray.o, ray.d);
    uint32_t stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const Node& n = bvh.nodes[stack[--sp]];
        double tn;
        if (!box_hit(rb, n.box, ray.tmin, ray.tmax, tn)) continue;
        if (n.count > 0) {
            for (uint32_t i = 0; i < n.count; i++) {
                uint32_t p = bvh.order[n.left_or_first + i];
                float t, u, v;
                if (intersect(rp, &bvh.verts[9 * (size_t)p], t, u, v)) return true;
            }
        } else {
            stack[sp++] = n.right;
            stack[sp++] = n.left_or_first;
        }
    }
    return false;
}

template <class F> void parallel_for(uint32_t n, int nthreads, F f) {
    if (nthreads <= 1 || n < 256) {
        for (uint32_t i = 0; i < n; i++) f(i);
        return;
    }
    std::atomic<uint32_t> next(0);
    std::vector<std::thread> th;
    for (int k = 0; k < nthreads; k++) {
        th.emplace_back([&]() {
            for (;;) {
                uint32_t b = next.fetch_add(1024);
                if (b >= n) break;
                uint32_t e = std::min(n, b + 1024);
                for (uint32_t i = b; i < e; i++) f(i);
            }
        });
    }
    for (auto& t : th) t.join();
}

}  // namespace

// Shared with the path integrator (path.cpp).
namespace orc {
void* bvh_build_internal(const float* tri_verts, uint32_t n);
bool bvh_closest(void* bvh, const float* o, const float* d, float tmin, float tmax, uint32_t& prim, float& t,
                 float& u, float& v);
bool bvh_any(void* bvh, const float* o, const float* d, float tmin, float tmax);
}

void* orc::bvh_build_internal(const float* tri_verts, uint32_t n) {
    Bvh* bvh = new Bvh();
    bvh->verts.assign(tri_verts, tri_verts + 9 * (size_t)n);
    std::vector<BuildItem> items(n);
    for (uint32_t i = 0; i < n; i++) {
        items[i].box.reset();
        for (int k = 0; k < 3; k++) items[i].box.grow(&tri_verts[9 * (size_t)i + 3 * k]);
        for (int a = 0; a < 3; a++) items[i].c[a] = 0.5f * (items[i].box.lo[a] + items[i].box.hi[a]);
    }
    bvh->order.resize(n);
    for (uint32_t i = 0; i < n; i++) bvh->order[i] = i;
    if (n == 0) {
        Node leaf; leaf.box.reset(); leaf.left_or_first = 0; leaf.count = 0; leaf.right = 0;
        // an empty leaf: box_hit fails on the inverted box
        bvh->nodes.push_back(leaf);
        bvh->nodes[0].count = 0;
        bvh->nodes[0].left_or_first = 0;
        return bvh;
    }
    bvh->nodes.reserve(2 * (size_t)n / 3 + 16);
    build_rec(*bvh, items, 0, n, 0);
    return bvh;
}

bool orc::bvh_closest(void* h, const float* o, const float* d, float tmin, float tmax, uint32_t& prim, float& t,
                      float& u, float& v) {
    Bvh* bvh = (Bvh*)h;
    orc_ray r;
    std::memcpy(r.o, o, 12); std::memcpy(r.d, d, 12); r.tmin = tmin; r.tmax = tmax;
    orc_hit hit;
    if (bvh->order.empty()) { prim = 0xFFFFFFFFu; return false; }
    closest_one(*bvh, r, hit);
    prim = hit.prim; t = hit.t; u = hit.u; v = hit.v;
    return hit.prim != 0xFFFFFFFFu;
}

bool orc::bvh_any(void* h, const float* o, const float* d, float tmin, float tmax) {
    Bvh* bvh = (Bvh*)h;
    if (bvh->order.empty()) return false;
    orc_ray r;
    std::memcpy(r.o, o, 12); std::memcpy(r.d, d, 12); r.tmin = tmin; r.tmax = tmax;
    return any_one(*bvh, r);
}

extern "C" {

void* orc_bvh_build(const float* tri_verts, uint32_t n) { return orc::bvh_build_internal(tri_verts, n); }
void orc_bvh_free(void* bvh) { delete (Bvh*)bvh; }
uint32_t orc_bvh_num_nodes(void* bvh) { return (uint32_t)((Bvh*)bvh)->nodes.size(); }

void orc_trace_closest(void* h, const orc_ray* rays, orc_hit* hits, uint32_t n, int nthreads) {
    Bvh* bvh = (Bvh*)h;
    parallel_for(n, nthreads, [&](uint32_t i) {
        if (bvh->order.empty()) { hits[i].prim = 0xFFFFFFFFu; hits[i].t = hits[i].u = hits[i].v = 0; return; }
        closest_one(*bvh, rays[i], hits[i]);
    });
}

void orc_trace_any(void* h, const orc_ray* rays, uint8_t* occ, uint32_t n, int nthreads) {
    Bvh* bvh = (Bvh*)h;
    parallel_for(n, nthreads, [&](uint32_t i) { occ[i] = (!bvh->order.empty() && any_one(*bvh, rays[i])) ? 1 : 0; });
}

void orc_brute_closest(const float* tv, uint32_t ntri, const orc_ray* rays, orc_hit* hits, uint32_t n) {
    for (uint32_t i = 0; i < n; i++) {
        RayPre rp = precompute(rays[i].o, rays[i].d, rays[i].tmin, rays[i].tmax);
        float best_t = rays[i].tmax; uint32_t best = 0xFFFFFFFFu; float bu = 0, bv = 0;
        for (uint32_t p = 0; p < ntri; p++) {
            float t, u, v;
            if (intersect(rp, &tv[9 * (size_t)p], t, u, v) && (t < best_t || (t == best_t && p < best))) {
                best_t = t; best = p; bu = u; bv = v;
            }
        }
        hits[i].prim = best; hits[i].t = best == 0xFFFFFFFFu ? 0.0f : best_t; hits[i].u = bu; hits[i].v = bv;
    }
}

void orc_brute_any(const float* tv, uint32_t ntri, const orc_ray* rays, uint8_t* occ, uint32_t n) {
    for (uint32_t i = 0; i < n; i++) {
        RayPre rp = precompute(rays[i].o, rays[i].d, rays[i].tmin, rays[i].tmax);
        occ[i] = 0;
        for (uint32_t p = 0; p < ntri; p++) {
            float t, u, v;
            if (intersect(rp, &tv[9 * (size_t)p], t, u, v)) { occ[i] = 1; break; }
        }
    }
}

int orc_intersect_tri(const float* ray8, const float* v9, float* tuv) {
    RayPre rp = precompute(ray8, ray8 + 4, ray8[3], ray8[7]);
    float t, u, v;
    if (!intersect(rp, v9, t, u, v)) return 0;
    tuv[0] = t; tuv[1] = u; tuv[2] = v;
    return 1;
}

}  // extern "C"
