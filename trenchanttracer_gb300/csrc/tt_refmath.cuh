// Float3 arithmetic in the reference's rounding: each helper is one Vec3f expression of the
// reference (include/math/LinearMath.h) written with explicit round-to-nearest intrinsics in the
// FMA contraction nvcc applies to it on sm_103a (a product is fused into the add/sub that
// consumes it, the left operand first), so the path tracer reproduces the reference kernel's
// bits without depending on this file's own optimisation.
#pragma once

#include "tt_vec.h"

namespace tt {

__device__ __forceinline__ V3 r_add(const V3 &a, const V3 &b) {
    return V3(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z));
}
__device__ __forceinline__ V3 r_sub(const V3 &a, const V3 &b) {
    return V3(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z));
}
__device__ __forceinline__ V3 r_mul(const V3 &a, float s) {
    return V3(__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s));
}
__device__ __forceinline__ V3 r_mul(const V3 &a, const V3 &b) {
    return V3(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y), __fmul_rn(a.z, b.z));
}
// c + a * s  (Vec3f + Vec3f * float)
__device__ __forceinline__ V3 r_madd(const V3 &a, float s, const V3 &c) {
    return V3(__fmaf_rn(a.x, s, c.x), __fmaf_rn(a.y, s, c.y), __fmaf_rn(a.z, s, c.z));
}
// c + a * b  (Vec3f += Vec3f * Vec3f)
__device__ __forceinline__ V3 r_madd(const V3 &a, const V3 &b, const V3 &c) {
    return V3(__fmaf_rn(a.x, b.x, c.x), __fmaf_rn(a.y, b.y, c.y), __fmaf_rn(a.z, b.z, c.z));
}
// c - a * s  (Vec3f - Vec3f * float)
__device__ __forceinline__ V3 r_msub(const V3 &c, const V3 &a, float s) {
    return V3(__fmaf_rn(-a.x, s, c.x), __fmaf_rn(-a.y, s, c.y), __fmaf_rn(-a.z, s, c.z));
}
// dot: x*x' + y*y' + z*z'  ->  fma(z, z', fma(x, x', y*y'))
__device__ __forceinline__ float r_dot(const V3 &a, const V3 &b) {
    return __fmaf_rn(a.z, b.z, __fmaf_rn(a.x, b.x, __fmul_rn(a.y, b.y)));
}
// cross: each component p*q - r*s  ->  fma(p, q, -(r*s))
__device__ __forceinline__ V3 r_cross(const V3 &a, const V3 &b) {
    return V3(__fmaf_rn(a.y, b.z, -__fmul_rn(a.z, b.y)), __fmaf_rn(a.z, b.x, -__fmul_rn(a.x, b.z)),
              __fmaf_rn(a.x, b.y, -__fmul_rn(a.y, b.x)));
}
// Vec3f::normalize: sqrtf(x*x + y*y + z*z), then three IEEE divides
__device__ __forceinline__ V3 r_normalize(const V3 &a) {
    const float n = __fsqrt_rn(__fmaf_rn(a.z, a.z, __fmaf_rn(a.x, a.x, __fmul_rn(a.y, a.y))));
    return V3(__fdiv_rn(a.x, n), __fdiv_rn(a.y, n), __fdiv_rn(a.z, n));
}
// The same two Vec3f expressions where nvcc contracts them the other way round, as it does inside
// the reference's refrSample (measured on interactions recorded in the reference's own kernel):
// dot(n, d) in `d - n * 2.0f * dot(n, d)` -> fma(y, y', x*x') + z*z' (the last product unfused),
// and Vec3f::normalize -> sqrtf(fma(z, z, fma(y, y, x*x))).
__device__ __forceinline__ float r_dot_yx(const V3 &a, const V3 &b) {
    return __fadd_rn(__fmaf_rn(a.y, b.y, __fmul_rn(a.x, b.x)), __fmul_rn(a.z, b.z));
}
__device__ __forceinline__ V3 r_normalize_yx(const V3 &a) {
    const float n = __fsqrt_rn(__fmaf_rn(a.z, a.z, __fmaf_rn(a.y, a.y, __fmul_rn(a.x, a.x))));
    return V3(__fdiv_rn(a.x, n), __fdiv_rn(a.y, n), __fdiv_rn(a.z, n));
}
// Vec3f::length
__device__ __forceinline__ float r_length(const V3 &a) {
    return __fsqrt_rn(__fmaf_rn(a.z, a.z, __fmaf_rn(a.x, a.x, __fmul_rn(a.y, a.y))));
}

}  // namespace tt
