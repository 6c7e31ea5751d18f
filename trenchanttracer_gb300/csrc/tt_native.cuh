// Device-side structures of the native wavefront path tracer, shared by the shading
// (tt_render_native.cu) and the traversal (tt_render_extend.cu) translation units.
//
// Path index space. A render covers one or more camera views; view k owns the contiguous range
// [first_k, first_k + npix_k * spp_k) of a batch-global path index space, sample-major inside
// the view (index = sample * npix + pixel). A wave is a contiguous range of that space, so it can
// span several views and partial samples; every kernel maps an index back to its view with a
// binary search over the view table. A path's PCG32 stream is its view-local index
// (sample_offset * npix + index - first), so a view renders the same bits whether it is drawn
// alone or inside any batch.
//
// Queues. Queue slot q of bounce parity c holds the path index queue[c][q] and that path's next
// ray ray[c][2q], ray[c][2q + 1] = (o.xyz, d.x), (d.y, d.z, tmin, tmax): the traversal kernels
// read rays contiguously, in queue order. Hit records are indexed by queue slot.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "tt_device.h"
#include "tt_ptmath.cuh"
#include "tt_reorder.h"

namespace tt {

struct EnvView {
    const float4 *tex;  // w*h radiance
    const float *marg;  // h+1 marginal CDF over rows
    const float *cond;  // h*(w+1) conditional CDFs per row
    // Guide tables (gm, gc powers of two): guide_m[k] is the marginal search's answer for
    // u = k / gm, and guide_c[y * (gc + 1) + k] row y's for u = k / gc. The answer for any u lies
    // between the entries of the two grid points around it, so the search runs on that range
    // only and returns the index the full search would.
    const int *guide_m, *guide_c;
    int gm, gc;
    int w, h;
    float scale;
};

// One camera view of a render.
struct ViewRec {
    long long first;      // batch-global index of the view's first path
    long long paths;      // npix * spp
    long long accum;      // element offset of the view's npix * 3 accumulation block
    long long stream0;    // sample_offset * npix: PCG32 stream index of the view's first path
    uint64_t seed_state;  // PCG32 initial state of the view's seed
    int width, height, npix, pad;
    float pos[3], view[3], up[3];
    float tanx, tany;
    float aperture, focal;  // thin lens (aperture <= 1e-5: pinhole)
};

struct PathSoA {
    float *beta, *L;     // 3 per path
    uint64_t *rng;       // PCG32 state
    uint64_t *rng_inc;   // PCG32 stream increment
    float *last_pdf;
    int *depth, *flags;
    int *queue[2];       // path index per queue slot, by bounce parity
    float4 *ray[2];      // 2 float4 per queue slot, by bounce parity
    float *hit_t, *hit_u, *hit_v;  // per slot of the queue being shaded
    int *hit_prim;       // triangle slot >= 0, -(geometry+2) for analytic objects, -1 = miss
    int *counts;         // [0] [1] queue lengths by parity, [2] shadow queue length,
                         // [3] extend work counter, [4] shadow work counter
    int *shadow_path;
    float4 *shadow_ray;  // 2 float4 per shadow ray
    float *shadow_val;   // 3 per shadow ray
    float *a0;           // radiance cache: pixel footprint of the path at its first vertex
    float *spread;       // radiance cache: running sum of sqrt(t^2 / (pdf cos)) over the bounces
};

// The radiance cache's side of a render (enabled = 0: the plain tracer).
struct CacheView {
    int enabled;
    int train;                // training paths are selected
    float spread_c;           // termination threshold (< 0: never)
    unsigned train_stride;    // a path trains when (stream index + phase) % stride == 0
    unsigned train_phase;
    int train_cap;            // capacity of the training records
    float *q_rec;             // queries: kRec floats per query
    int *q_path;
    float *q_beta;            // 3 per query: throughput arriving at the query vertex
    float *q_rgb;             // 3 per query: the cache's radiance
    float *t_rec;             // training records, compacted in slot order (k_cache_compact)
    int *t_path;
    float *t_L;               // 3 per record: the path's radiance up to the record vertex
    float *t_beta;            // 3 per record: throughput arriving at the record vertex
    float *t_target;          // 3 per record: measured radiance leaving the vertex
    int *counts;              // [0] queries, [1] training records
    // Each training path of a wave owns slot (stream index + phase) / stride - train_slot0 of the
    // slot arrays (path -1: no record), so the records' order does not depend on scheduling.
    long long train_slot0;
    int train_slots;
    float *s_rec;
    int *s_path;
    float *s_L, *s_beta;
    int *block_counts;        // filled slots per 1024-slot block
};

// Ordering of an extension queue (tt_reorder.cu): when order_built(state), k_extend reads the
// ordered copy of the queue's first *n_sorted rays and writes their hits by ordered slot, and
// k_order_gather_hits moves each of those hits back to its queue slot (pos: the ordered slot of
// each queue slot). The rest of the queue (a streamed render's new camera rays, coherent as they
// are) is traced in place.
struct OrderView {
    const float4 *sorted;  // nullptr: ordering off
    float *hit_t, *hit_u, *hit_v;
    int *hit_prim;
    const int *pos;
    const unsigned long long *state;
    const int *n_sorted;
};

// Ordering of the shadow queue: when order_built(state), k_shadow traces the queue in the order of
// `sorted` and takes each ray's path and value from its original slot src[p].
struct ShadowOrderView {
    const float4 *sorted;  // nullptr: ordering off
    const int *src;
    const unsigned long long *state;
};

// Path state by index: the state slot of a path in waves, the queue slot in a streamed render.
struct PathState {
    float *beta, *L;  // 3 per path
    float *last_pdf;
    uint64_t *rng, *rng_inc;
    int *depth, *flags;
    long long *g;     // streamed renders: the path's index
};

// Streamed render: a pool of wave_paths queue slots that is refilled with the next paths of the
// index space as paths end, so every bounce launch works on a full pool and the few long paths
// at the end of a wave no longer hold the GPU half idle. The path state lives in queue order, one
// copy per queue parity: shade writes each survivor's state next to its ray in the next queue,
// and the refill writes new paths' state behind the survivors, so every state access is
// coalesced. An ended path's radiance goes to a ring of ring_n entries at (path index mod
// ring_n), where it waits until every path below it has ended; an accumulate pass then adds that
// range in sample order, exactly as the wave scheme does, so the image bits do not change.
// ring_n = max_depth * pool holds every path still in flight plus one refill.
struct StreamPlan {
    long long next;                 // the next path of the index space to start
    long long frontier;             // every path below it has been accumulated
    unsigned long long min_alive;   // smallest path index among the last shade's survivors
    long long acc_lo, acc_hi;       // the range the next accumulate pass adds
    long long new_first;            // the paths the next refill starts: [new_first, + new_n)
    int new_n, new_at;              // how many, and their first slot in the extension queue
};

struct StreamView {
    long long total;    // paths of the render
    long long ring_n;   // entries of the radiance ring
    float *ring;        // 3 floats per entry
    PathState st[2];    // path state by queue slot, by queue parity
    StreamPlan *plan;
};

struct NativeArgs {
    BvhView bvh;
    const MaterialRec *materials;
    int num_materials;
    const GeomRec *geoms;
    int num_geoms;
    EnvView env;
    PathSoA ps;
    tt_render_params p;
    const ViewRec *views;  // device view table (nullptr: the single view `view0`)
    int n_views;
    ViewRec view0;
    long long wave_first;  // batch-global index of the wave's first path
    int wave_paths;
    unsigned int *err;
    unsigned long long *stats;  // [0] extension rays, [1] shadow rays, [2] paths
    CacheView cache;
    StreamView stream;  // a streamed render's state (ring == nullptr: waves)
    const struct GeomNode *gnodes;  // box hierarchy over the analytic objects, or nullptr
    const int *gidx;
    OrderView order;
    ShadowOrderView shadow_order;
};

__device__ __forceinline__ int find_view(const NativeArgs &a, long long g) {
    if (!a.views) return 0;
    int lo = 0, hi = a.n_views - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(&a.views[mid].first) <= g) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ ViewRec view_of(const NativeArgs &a, int v) { return a.views ? a.views[v] : a.view0; }

// A node of the box hierarchy over the analytic objects: an inner node (count = -1 - split axis)
// has its children at `first` (lower centroids along the axis) and `first + 1`; a leaf holds
// objects gidx[first .. first + count).
struct GeomNode {
    float lo[3];
    int first;
    float hi[3];
    int count;
};
static_assert(sizeof(GeomNode) == 32, "GeomNode must stay 32 B");
constexpr int kGeomStack = 64;

// The exact test of analytic object i (the reference's Plane / Sphere tests); a hit nearer than
// t replaces the current one, and an equally near one replaces it only when it is an analytic
// object of higher index, so any visiting order gives the result of the reference's loop over
// the objects in index order.
__device__ __forceinline__ void analytic_one(const NativeArgs &a, int i, const V3 &o, const V3 &d, float tmin,
                                             float &t, int &prim, float &hu, float &hv) {
    using namespace pt;
    const GeomRec g = a.geoms[i];
    float th, u = 0.f, v = 0.f;
    if (g.kind == GEOM_PLANE) {
        const V3 p0(g.p0[0], g.p0[1], g.p0[2]);
        const V3 e1 = sub(V3(g.p1[0], g.p1[1], g.p1[2]), p0), e2 = sub(V3(g.p2[0], g.p2[1], g.p2[2]), p0);
        const V3 P = cross(d, e2);
        const float det = dot(e1, P);
        if (det > -1e-12f && det < 1e-12f) return;
        const float inv = PT_DIV(1.0f, det);
        const V3 T = sub(o, p0);
        u = PT_MUL(dot(T, P), inv);
        if (u < 0.f || u > 1.f) return;
        const V3 Q = cross(T, e1);
        v = PT_MUL(dot(d, Q), inv);
        if (v < 0.f || v > 1.f) return;
        th = PT_MUL(dot(e2, Q), inv);
    } else if (g.kind == GEOM_SPHERE) {
        const V3 c(g.p0[0], g.p0[1], g.p0[2]);
        const V3 oc = sub(c, o);
        const float bq = dot(oc, d);
        const float disc = PT_FMA(g.radius, g.radius, PT_FMA(bq, bq, -dot(oc, oc)));
        if (disc < 0.0f) return;
        const float sq = PT_SQRT(disc);
        th = PT_SUB(bq, sq);
        if (!(th > tmin)) th = PT_ADD(bq, sq);
    } else {
        return;
    }
    if (th > tmin && (th < t || (th == t && prim <= -2 && i < -prim - 2))) {
        t = th;
        prim = -(i + 2);
        hu = u;
        hv = v;
    }
}

// Hits among the analytic objects for the lanes of `mask` (every lane of `mask` calls this
// together; `live` lanes want the test): the closest one, or with any_hit whether there is one
// below t (prim != -1 afterwards). Without a box hierarchy, the reference's loop over all objects.
// With one, the warp walks the hierarchy together: it enters a node when the node's box passes
// the box test of any live lane, so node and object reads are the same address across the warp,
// and each lane tests a leaf's objects only when its own ray passes the leaf's box. The boxes
// are padded on the host so that no hit the exact tests accept is culled; a warp never tests
// more objects than the loop would, and a stack that would overflow falls back to the loop.
__device__ __forceinline__ void analytic_hit(const NativeArgs &a, unsigned mask, bool live, const V3 &o,
                                             const V3 &d, float tmin, float &t, int &prim, float &hu, float &hv,
                                             bool any_hit) {
    if (!a.gnodes) {
        if (!live) return;
        for (int i = 0; i < a.num_geoms; i++) {
            analytic_one(a, i, o, d, tmin, t, prim, hu, hv);
            if (any_hit && prim != -1) return;
        }
        return;
    }
    const unsigned live_m = __ballot_sync(mask, live);
    if (!live_m) return;
    // the warp's near-first order: per axis, whether most live rays point towards -axis
    const int half = __popc(live_m);
    const int order = (2 * __popc(__ballot_sync(mask, live && d.x < 0.0f)) > half ? 1 : 0) |
                      (2 * __popc(__ballot_sync(mask, live && d.y < 0.0f)) > half ? 2 : 0) |
                      (2 * __popc(__ballot_sync(mask, live && d.z < 0.0f)) > half ? 4 : 0);
    const float ix = 1.0f / (fabsf(d.x) > 1e-20f ? d.x : copysignf(1e-20f, d.x));
    const float iy = 1.0f / (fabsf(d.y) > 1e-20f ? d.y : copysignf(1e-20f, d.y));
    const float iz = 1.0f / (fabsf(d.z) > 1e-20f ? d.z : copysignf(1e-20f, d.z));
    const float4 *nodes = reinterpret_cast<const float4 *>(a.gnodes);
    int stack[kGeomStack];  // the same contents in every lane
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const int ni = stack[--sp];
        const float4 n0 = __ldg(nodes + 2 * ni), n1 = __ldg(nodes + 2 * ni + 1);
        bool h = false;
        if (live) {
            const float tx0 = (n0.x - o.x) * ix, tx1 = (n1.x - o.x) * ix;
            const float ty0 = (n0.y - o.y) * iy, ty1 = (n1.y - o.y) * iy;
            const float tz0 = (n0.z - o.z) * iz, tz1 = (n1.z - o.z) * iz;
            const float entry = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fminf(tz0, tz1));
            const float exit = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fmaxf(tz0, tz1));
            const float slack = 1e-4f * fmaxf(fabsf(entry), fabsf(exit)) + 1e-6f;
            h = entry <= exit + slack && exit + slack >= tmin && entry - slack <= t;
        }
        if (!__any_sync(mask, h)) continue;
        const int first = __float_as_int(n0.w), count = __float_as_int(n1.w);
        if (count > 0) {
            if (h)
                for (int k = 0; k < count; k++) analytic_one(a, __ldg(a.gidx + first + k), o, d, tmin, t, prim, hu, hv);
            if (any_hit) {
                live = live && prim == -1;
                if (!__any_sync(mask, live)) return;
            }
        } else if (sp + 2 <= kGeomStack) {
            const int far_first = (order >> (-1 - count)) & 1;  // the warp travels towards -axis
            stack[sp++] = first + 1 - far_first;
            stack[sp++] = first + far_first;
        } else {  // deeper than the stack: every object, as the reference does
            if (live)
                for (int i = 0; i < a.num_geoms; i++) analytic_one(a, i, o, d, tmin, t, prim, hu, hv);
            return;
        }
    }
}

// Kernels of one traversal launch shape (threads per block, shared-memory stack entries).
struct TraceKernels {
    void (*extend)(NativeArgs, int);
    void (*extend_prefix)(NativeArgs, int);  // for queues ordered only up to *order.n_sorted
    void (*shadow)(NativeArgs);
};
// Moves the hits of an ordered extension queue back to their queue slots (nothing when the
// queue was not ordered).
__global__ void k_order_gather_hits(NativeArgs a, int cur);
// Block sizes and shared stack depths the traversal kernels are built for.
constexpr int kNumBlockShapes = 3;
constexpr int kBlockShapes[kNumBlockShapes] = {64, 128, 256};
constexpr int kNumStackShapes = 3;
constexpr int kStackShapes[kNumStackShapes] = {0, 8, 16};
static_assert(sizeof(tt_renderer::occ_trace) == sizeof(int) * kNumBlockShapes * kNumStackShapes &&
                  sizeof(tt_renderer::occ_shade) == sizeof(int) * kNumBlockShapes,
              "occupancy cache shape");
// nullptr if (block, stack_shared) is not one of the built shapes.
TraceKernels trace_kernels(int block, int stack_shared);

}  // namespace tt
