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
//   - one postponed leaf per lane and a warp vote that ends the inner-node loop once every
//     active lane holds a leaf (:169-203);
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
// (ld.global.nc.v4) so they go through the L1/tex path without texture objects; the
// traversal stack lives in a per-thread local array that stays in L1; every loop carries an
// iteration cap and the stack a bounds check, both reported through an error word instead of
// faulting or hanging.
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

struct TraceResult {
    int addr;  // float4 slot of the hit triangle, -1 = miss
    float t;   // hit distance; tmax on a miss
    float u, v;
};

// One ray through the BVH. kClosest selects closest-hit vs any-hit.
template <bool kClosest>
__device__ __forceinline__ TraceResult traverse(const BvhView &bvh, float ox, float oy, float oz, float dx, float dy,
                                                float dz, float tmin, float tmax, uint32_t &err) {
    const float ooeps = 8.27180612553027674871e-25f;  // exp2f(-80), exact
    const float idirx = __fdiv_rn(1.0f, fabsf(dx) > ooeps ? dx : copysignf(ooeps, dx));
    const float idiry = __fdiv_rn(1.0f, fabsf(dy) > ooeps ? dy : copysignf(ooeps, dy));
    const float idirz = __fdiv_rn(1.0f, fabsf(dz) > ooeps ? dz : copysignf(ooeps, dz));
    const float oodx = __fmul_rn(ox, idirx);
    const float oody = __fmul_rn(oy, idiry);
    const float oodz = __fmul_rn(oz, idirz);

    int stack[kStackSize];
    int sp = 0;
    stack[0] = kEntrypointSentinel;
    int leaf_addr = 0;
    int node_addr = 0;
    TraceResult res;
    res.addr = -1;
    res.t = tmax;
    res.u = 0.f;
    res.v = 0.f;
    uint32_t iter = 0;

    while (node_addr != kEntrypointSentinel) {
        while (node_addr >= 0 && node_addr != kEntrypointSentinel) {
            const float4 n0xy = ldg4(bvh.nodes + node_addr);
            const float4 n1xy = ldg4(bvh.nodes + node_addr + 1);
            const float4 nz = ldg4(bvh.nodes + node_addr + 2);
            const float4 tmp = ldg4(bvh.nodes + node_addr + 3);

            const float c0lox = slab(n0xy.x, idirx, oodx);
            const float c0hix = slab(n0xy.y, idirx, oodx);
            const float c0loy = slab(n0xy.z, idiry, oody);
            const float c0hiy = slab(n0xy.w, idiry, oody);
            const float c0loz = slab(nz.x, idirz, oodz);
            const float c0hiz = slab(nz.y, idirz, oodz);
            const float c1loz = slab(nz.z, idirz, oodz);
            const float c1hiz = slab(nz.w, idirz, oodz);
            const float c0min = span_begin(c0lox, c0hix, c0loy, c0hiy, c0loz, c0hiz, tmin);
            const float c0max = span_end(c0lox, c0hix, c0loy, c0hiy, c0loz, c0hiz, res.t);
            const float c1lox = slab(n1xy.x, idirx, oodx);
            const float c1hix = slab(n1xy.y, idirx, oodx);
            const float c1loy = slab(n1xy.z, idiry, oody);
            const float c1hiy = slab(n1xy.w, idiry, oody);
            const float c1min = span_begin(c1lox, c1hix, c1loy, c1hiy, c1loz, c1hiz, tmin);
            const float c1max = span_end(c1lox, c1hix, c1loy, c1hiy, c1loz, c1hiz, res.t);

            const bool t0 = (c0min <= c0max) && (c0min >= tmin) && (c0min <= 1e20f);
            const bool t1 = (c1min <= c1max) && (c1min >= tmin) && (c1min <= 1e20f);

            if (!t0 && !t1) {
                node_addr = stack[sp--];
            } else {
                int far_child = __float_as_int(tmp.y);
                node_addr = t0 ? __float_as_int(tmp.x) : far_child;
                if (t0 && t1) {
                    if (c1min < c0min) {
                        const int s = node_addr;
                        node_addr = far_child;
                        far_child = s;
                    }
                    if (sp + 1 >= kStackSize) {
                        err |= kErrStack;
                        res.addr = -1;
                        res.t = tmax;
                        return res;
                    }
                    stack[++sp] = far_child;
                }
            }
            if (node_addr < 0 && leaf_addr >= 0) {
                leaf_addr = node_addr;
                node_addr = stack[sp--];
            }
            if (++iter > kMaxIterations) {
                err |= kErrIter;
                res.addr = -1;
                res.t = tmax;
                return res;
            }
            if (__ballot_sync(__activemask(), leaf_addr >= 0) == 0u) break;
        }

        while (leaf_addr < 0) {
            for (int tri = ~leaf_addr;; tri += 3) {
                const float4 v0 = ldg4(bvh.verts + tri);
                if (__float_as_int(v0.x) == (int)0x80000000) break;
                const float4 v1 = ldg4(bvh.verts + tri + 1);
                const float4 v2 = ldg4(bvh.verts + tri + 2);
                if (++iter > kMaxIterations) {
                    err |= kErrIter;
                    res.addr = -1;
                    res.t = tmax;
                    return res;
                }

                const float e1x = __fsub_rn(v1.x, v0.x), e1y = __fsub_rn(v1.y, v0.y), e1z = __fsub_rn(v1.z, v0.z);
                const float e2x = __fsub_rn(v2.x, v0.x), e2y = __fsub_rn(v2.y, v0.y), e2z = __fsub_rn(v2.z, v0.z);
                const float tvx = __fsub_rn(ox, v0.x), tvy = __fsub_rn(oy, v0.y), tvz = __fsub_rn(oz, v0.z);
                const float px = cross_c(dy, e2z, dz, e2y);
                const float py = cross_c(dz, e2x, dx, e2z);
                const float pz = cross_c(dx, e2y, dy, e2x);
                const float det = dot_c(e1x, e1y, e1z, px, py, pz);
                const float inv_det = __fdiv_rn(1.0f, det);
                const float u = __fmul_rn(dot_c(tvx, tvy, tvz, px, py, pz), inv_det);
                const float qx = cross_c(tvy, e1z, tvz, e1y);
                const float qy = cross_c(tvz, e1x, tvx, e1z);
                const float qz = cross_c(tvx, e1y, tvy, e1x);
                const float v = __fmul_rn(dot_c(dx, dy, dz, qx, qy, qz), inv_det);

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
                if (tmin < t && t < res.t) {
                    res.t = t;
                    res.addr = tri;
                    res.u = u;
                    res.v = v;
                    if (!kClosest) {
                        node_addr = kEntrypointSentinel;
                        break;
                    }
                }
            }
            leaf_addr = node_addr;
            if (node_addr < 0) node_addr = stack[sp--];
        }
    }
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
