// Two-wide SBVH traversal for sm_103a over the reference's compact layout.
//
// Semantics follow intersect() of the reference (include/geometry/IntersectKernel.cuh:78-296)
// so that hit triangle ids and distances are bit-identical:
//   - inverse direction with the 2^-80 guard (:92-101), per-axis slab values
//     fma(bound, idir, -orig*idir) (:126-143);
//   - entry/exit spans from float min/max for x and y and SIGNED-INTEGER min/max on the float
//     bits for z and the tmin / hit-distance operand (the Kepler video min/max, :22-60);
//   - a child is entered iff entry <= exit, entry >= tmin and entry <= 1e20 (:145-147);
//     near-first order, the far child pushed, swap only when c1 entry < c0 entry (:149-167);
//   - one postponed leaf per lane (:169-178); the reference's warp vote (:180-203) is available
//     as an option, but by default a lane processes its leaf without visiting further nodes, so
//     the result is the per-ray result of the reference's algorithm whatever the other lanes do;
//   - Moller-Trumbore on the three raw float4 vertices, accepting only det > 1e-5 with
//     u in [0,1], v >= 0, u+v <= 1; the det < -1e-5 branch keeps the reference's comparisons
//     (which reject every finite u) (:209-271); a hit needs tmin < t < current distance;
//   - any-hit stops at the first accepted triangle in traversal order (:265-269).
// Every floating-point product/sum is written with explicit round-to-nearest intrinsics in
// the contraction pattern that nvcc applies to the reference's source, so the result does not
// depend on how this file happens to be optimised. The pattern is pinned by the tests against
// the reference kernel's own outputs.
//
// GB300 choices: all BVH and triangle reads are 16-byte read-only vector loads
// (ld.global.nc.v4) so they go through the L1/tex path without texture objects; the traversal
// stack keeps its lower entries in a per-thread column of shared memory (conflict-free: lane i
// of entry k sits at k*blockDim + i) and spills only entries beyond that into local memory, so
// stack traffic does not evict BVH nodes from L1; every loop carries an iteration cap and the
// stack a bounds check, both reported through an error word instead of faulting or hanging.
#pragma once

#include <cstdint>

namespace tt {

constexpr int kEntrypointSentinel = 0x76543210;
constexpr int kStackSize = 68;          // depth <= 64 pushes + sentinel, with slack
constexpr uint32_t kErrStack = 1u;      // traversal stack would overflow
constexpr uint32_t kErrIter = 2u;       // iteration cap reached (corrupt BVH)
constexpr uint32_t kMaxIterations = 1u << 22;

struct BvhView {
    const float4 *__restrict__ nodes;
    const float4 *__restrict__ verts;
    const float4 *__restrict__ norms;
    const int32_t *__restrict__ tri_idx;
    const uint32_t *__restrict__ mat_idx;
};

__device__ __forceinline__ float4 ldg4(const float4 *p) { return __ldg(p); }

// ---- arithmetic in the reference's contraction pattern --------------------------------------
// x * y - z  ->  fma(x, y, -z)
__device__ __forceinline__ float slab(float b, float idir, float ood) { return __fmaf_rn(b, idir, -ood); }
// a.y*b.z - a.z*b.y  ->  fma(a.y, b.z, -(a.z*b.y))
__device__ __forceinline__ float cross_c(float ay, float bz, float az, float by) {
    return __fmaf_rn(ay, bz, -__fmul_rn(az, by));
}
// a.x*b.x + a.y*b.y + a.z*b.z  ->  fma(a.z, b.z, fma(a.x, b.x, a.y*b.y))
__device__ __forceinline__ float dot_c(float ax, float ay, float az, float bx, float by, float bz) {
    return __fmaf_rn(az, bz, __fmaf_rn(ax, bx, __fmul_rn(ay, by)));
}
// n0*(1-u-v) + n1*u + n2*v per component  ->  fma(n2, v, fma(n0, w, n1*u))
__device__ __forceinline__ float interp_c(float n0, float n1, float n2, float w, float u, float v) {
    return __fmaf_rn(n2, v, __fmaf_rn(n0, w, __fmul_rn(n1, u)));
}

// Signed-integer min/max on float bit patterns (the reference's vmin/vmax).
__device__ __forceinline__ int imin(int a, int b) { return a < b ? a : b; }
__device__ __forceinline__ int imax(int a, int b) { return a > b ? a : b; }
__device__ __forceinline__ float span_begin(float a0, float a1, float b0, float b1, float c0, float c1, float d) {
    int x = imax(__float_as_int(fminf(a0, a1)), __float_as_int(fminf(b0, b1)));
    int y = imax(imin(__float_as_int(c0), __float_as_int(c1)), __float_as_int(d));
    return __int_as_float(imax(x, y));
}
__device__ __forceinline__ float span_end(float a0, float a1, float b0, float b1, float c0, float c1, float d) {
    int x = imin(__float_as_int(fmaxf(a0, a1)), __float_as_int(fmaxf(b0, b1)));
    int y = imin(imax(__float_as_int(c0), __float_as_int(c1)), __float_as_int(d));
    return __int_as_float(imin(x, y));
}

// ---- traversal stack ---------------------------------------------------------------------------
// Entries [0, kSh) live in shared memory at sh[i * kStride]; the rest in a local array.
template <int kSh, int kStride>
struct TravStack {
    int *sh;
    int loc[kStackSize - kSh + 1];
    __device__ __forceinline__ int get(int i) const {
        if (kSh > 0 && i < kSh) return sh[i * kStride];
        return loc[i - kSh];
    }
    __device__ __forceinline__ void set(int i, int v) {
        if (kSh > 0 && i < kSh) sh[i * kStride] = v;
        else loc[i - kSh] = v;
    }
};

// Resumable per-ray traversal state.
struct TravState {
    float ox, oy, oz, dx, dy, dz, tmin;
    float idirx, idiry, idirz, oodx, oody, oodz;
    float t, u, v;  // current hit distance (tmax until a hit) and barycentrics of the hit
    int addr;       // float4 slot of the hit triangle, -1 = none yet
    int node, leaf, sp;
    uint32_t iter;
};

template <class Stack>
__device__ __forceinline__ void trav_init(TravState &s, Stack &stack, float4 r0, float4 r1) {
    s.ox = r0.x;
    s.oy = r0.y;
    s.oz = r0.z;
    s.dx = r0.w;
    s.dy = r1.x;
    s.dz = r1.y;
    s.tmin = r1.z;
    s.t = r1.w;
    const float ooeps = 8.27180612553027674871e-25f;  // exp2f(-80), exact
    s.idirx = __fdiv_rn(1.0f, fabsf(s.dx) > ooeps ? s.dx : copysignf(ooeps, s.dx));
    s.idiry = __fdiv_rn(1.0f, fabsf(s.dy) > ooeps ? s.dy : copysignf(ooeps, s.dy));
    s.idirz = __fdiv_rn(1.0f, fabsf(s.dz) > ooeps ? s.dz : copysignf(ooeps, s.dz));
    s.oodx = __fmul_rn(s.ox, s.idirx);
    s.oody = __fmul_rn(s.oy, s.idiry);
    s.oodz = __fmul_rn(s.oz, s.idirz);
    s.u = 0.f;
    s.v = 0.f;
    s.addr = -1;
    s.node = 0;
    s.leaf = 0;
    s.sp = 0;
    s.iter = 0;
    stack.set(0, kEntrypointSentinel);
}

__device__ __forceinline__ void trav_fail(TravState &s, uint32_t &err, uint32_t code, float tmax) {
    err |= code;
    s.addr = -1;
    s.t = tmax;
    s.node = kEntrypointSentinel;
    s.leaf = kEntrypointSentinel;
}

// One inner-node visit of the reference's inner loop (IntersectKernel.cuh:112-178).
// Returns false if the ray failed (stack / iteration bound).
template <class Stack>
__device__ __forceinline__ bool trav_node_step(TravState &s, Stack &stack, const BvhView &bvh, uint32_t &err,
                                               float tmax) {
    const float4 n0xy = ldg4(bvh.nodes + s.node);
    const float4 n1xy = ldg4(bvh.nodes + s.node + 1);
    const float4 nz = ldg4(bvh.nodes + s.node + 2);
    const float4 tmp = ldg4(bvh.nodes + s.node + 3);
    const float c0lox = slab(n0xy.x, s.idirx, s.oodx);
    const float c0hix = slab(n0xy.y, s.idirx, s.oodx);
    const float c0loy = slab(n0xy.z, s.idiry, s.oody);
    const float c0hiy = slab(n0xy.w, s.idiry, s.oody);
    const float c0loz = slab(nz.x, s.idirz, s.oodz);
    const float c0hiz = slab(nz.y, s.idirz, s.oodz);
    const float c1loz = slab(nz.z, s.idirz, s.oodz);
    const float c1hiz = slab(nz.w, s.idirz, s.oodz);
    const float c0min = span_begin(c0lox, c0hix, c0loy, c0hiy, c0loz, c0hiz, s.tmin);
    const float c0max = span_end(c0lox, c0hix, c0loy, c0hiy, c0loz, c0hiz, s.t);
    const float c1lox = slab(n1xy.x, s.idirx, s.oodx);
    const float c1hix = slab(n1xy.y, s.idirx, s.oodx);
    const float c1loy = slab(n1xy.z, s.idiry, s.oody);
    const float c1hiy = slab(n1xy.w, s.idiry, s.oody);
    const float c1min = span_begin(c1lox, c1hix, c1loy, c1hiy, c1loz, c1hiz, s.tmin);
    const float c1max = span_end(c1lox, c1hix, c1loy, c1hiy, c1loz, c1hiz, s.t);
    const bool t0 = (c0min <= c0max) && (c0min >= s.tmin) && (c0min <= 1e20f);
    const bool t1 = (c1min <= c1max) && (c1min >= s.tmin) && (c1min <= 1e20f);
    if (!t0 && !t1) {
        s.node = stack.get(s.sp--);
    } else {
        int far_child = __float_as_int(tmp.y);
        s.node = t0 ? __float_as_int(tmp.x) : far_child;
        if (t0 && t1) {
            if (c1min < c0min) {
                const int sw = s.node;
                s.node = far_child;
                far_child = sw;
            }
            if (s.sp + 1 >= kStackSize) {
                trav_fail(s, err, kErrStack, tmax);
                return false;
            }
            stack.set(++s.sp, far_child);
        }
    }
    if (s.node < 0 && s.leaf >= 0) {
        s.leaf = s.node;
        s.node = stack.get(s.sp--);
    }
    if (++s.iter > kMaxIterations) {
        trav_fail(s, err, kErrIter, tmax);
        return false;
    }
    return true;
}

// The reference's leaf loop (IntersectKernel.cuh:209-281) for a lane holding a postponed leaf:
// that leaf, then every leaf popped right after it. Returns false if the ray failed.
template <bool kClosest, class Stack>
__device__ __forceinline__ bool trav_leaf_phase(TravState &s, Stack &stack, const BvhView &bvh, uint32_t &err,
                                                float tmax) {
    bool stop = false;  // any hit: a triangle was accepted
    while (s.leaf < 0) {
        for (int tri = ~s.leaf;; tri += 3) {
            const float4 v0 = ldg4(bvh.verts + tri);
            // The any-hit stop is taken here, with the leaf terminator (the slot after an accepted
            // triangle is another triangle or the terminator): a break at the acceptance itself
            // made the any-hit build issue 10 % more warp instructions than the closest-hit one.
            if (__float_as_int(v0.x) == (int)0x80000000 || (!kClosest && stop)) break;
            const float4 v1 = ldg4(bvh.verts + tri + 1);
            const float4 v2 = ldg4(bvh.verts + tri + 2);
            if (++s.iter > kMaxIterations) {
                trav_fail(s, err, kErrIter, tmax);
                return false;
            }
            const float e1x = __fsub_rn(v1.x, v0.x), e1y = __fsub_rn(v1.y, v0.y), e1z = __fsub_rn(v1.z, v0.z);
            const float e2x = __fsub_rn(v2.x, v0.x), e2y = __fsub_rn(v2.y, v0.y), e2z = __fsub_rn(v2.z, v0.z);
            const float tvx = __fsub_rn(s.ox, v0.x), tvy = __fsub_rn(s.oy, v0.y), tvz = __fsub_rn(s.oz, v0.z);
            const float px = cross_c(s.dy, e2z, s.dz, e2y);
            const float py = cross_c(s.dz, e2x, s.dx, e2z);
            const float pz = cross_c(s.dx, e2y, s.dy, e2x);
            const float det = dot_c(e1x, e1y, e1z, px, py, pz);
            const float inv_det = __fdiv_rn(1.0f, det);
            const float u = __fmul_rn(dot_c(tvx, tvy, tvz, px, py, pz), inv_det);
            const float qx = cross_c(tvy, e1z, tvz, e1y);
            const float qy = cross_c(tvz, e1x, tvx, e1z);
            const float qz = cross_c(tvx, e1y, tvy, e1x);
            const float v = __fmul_rn(dot_c(s.dx, s.dy, s.dz, qx, qy, qz), inv_det);
            const float kEps = 0.00001f;
            if (det > kEps) {
                if (u < 0.0f || u > 1.0f) continue;
                if (v < 0.0f || __fadd_rn(u, v) > 1.0f) continue;
            } else if (det < -kEps) {
                if (u > 0.0f || u < 1.0f) continue;
                if (v > 0.0f || __fadd_rn(u, v) < 1.0f) continue;
            } else {
                continue;
            }
            const float t = __fmul_rn(dot_c(e2x, e2y, e2z, qx, qy, qz), inv_det);
            if (s.tmin < t && t < s.t) {
                s.t = t;
                s.addr = tri;
                s.u = u;
                s.v = v;
                if (!kClosest) {
                    s.node = kEntrypointSentinel;
                    stop = true;
                }
            }
        }
        s.leaf = s.node;
        if (s.node < 0) s.node = stack.get(s.sp--);
    }
    return true;
}

// One pass of the reference's outer loop: inner nodes until a leaf is postponed and the next
// entry is found (kSpec = false: this lane alone decides, so the result depends on nothing but
// the ray; kSpec = true: continue speculatively until a warp vote says every active lane holds a
// leaf, as the reference kernel does), then the pending leaves. Returns true when the ray is
// finished. tmax is needed only to report a failed ray as a miss.
template <bool kClosest, bool kSpec, class Stack>
__device__ __forceinline__ bool trav_iterate(TravState &s, Stack &stack, const BvhView &bvh, uint32_t &err,
                                             float tmax) {
    while (s.node >= 0 && s.node != kEntrypointSentinel) {
        if (!trav_node_step(s, stack, bvh, err, tmax)) return true;
        if (kSpec) {
            if (__ballot_sync(__activemask(), s.leaf >= 0) == 0u) break;
        } else {
            if (s.leaf < 0) break;
        }
    }
    if (!trav_leaf_phase<kClosest>(s, stack, bvh, err, tmax)) return true;
    return s.node == kEntrypointSentinel;
}

struct TraceResult {
    int addr;  // float4 slot of the hit triangle, -1 = miss
    float t;   // hit distance; tmax on a miss
    float u, v;
};

// One ray through the BVH, start to finish, on the given stack.
template <bool kClosest, class Stack>
__device__ __forceinline__ TraceResult traverse_on(Stack &stack, const BvhView &bvh, float4 r0, float4 r1,
                                                   uint32_t &err) {
    TravState s;
    trav_init(s, stack, r0, r1);
    while (!trav_iterate<kClosest, false>(s, stack, bvh, err, r1.w)) {
    }
    TraceResult res;
    res.addr = s.addr;
    res.t = s.t;
    res.u = s.u;
    res.v = s.v;
    return res;
}

// One ray through the BVH, start to finish, with its whole stack in local memory.
template <bool kClosest>
__device__ __forceinline__ TraceResult traverse(const BvhView &bvh, float4 r0, float4 r1, uint32_t &err) {
    TravStack<0, 1> stack;
    TravState s;
    trav_init(s, stack, r0, r1);
    while (!trav_iterate<kClosest, false>(s, stack, bvh, err, r1.w)) {
    }
    TraceResult res;
    res.addr = s.addr;
    res.t = s.t;
    res.u = s.u;
    res.v = s.v;
    return res;
}

// The remaining fields of the reference's Hit for a hit slot: material index, original
// triangle id and the interpolated (unnormalised) shading normal (IntersectKernel.cuh:260-264,
// :285-290).
__device__ __forceinline__ void hit_normal(const BvhView &bvh, int addr, float u, float v, float &nx, float &ny,
                                           float &nz) {
    const float4 n0 = ldg4(bvh.norms + addr);
    const float4 n1 = ldg4(bvh.norms + addr + 1);
    const float4 n2 = ldg4(bvh.norms + addr + 2);
    const float w = __fsub_rn(__fsub_rn(1.0f, u), v);
    nx = interp_c(n0.x, n1.x, n2.x, w, u, v);
    ny = interp_c(n0.y, n1.y, n2.y, w, u, v);
    nz = interp_c(n0.z, n1.z, n2.z, w, u, v);
}

}  // namespace tt
