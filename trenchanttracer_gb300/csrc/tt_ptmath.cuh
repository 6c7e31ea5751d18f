// Math of the native path tracer, for device and host alike.
//
// Everything here is built from IEEE-754 basic operations (add, sub, mul, div, sqrt, fma) with
// the rounding of every step written out, so the integrator is a deterministic function of its
// inputs: the same on every GPU and reproducible by a CPU restatement. In particular the
// trigonometric functions are this file's own (not a math library's):
//   sin / cos: Cody & Waite's argument reduction by pi/2 with a two-part pi/2 (Cody & Waite,
//              "Software Manual for the Elementary Functions", 1980), then the Taylor series to
//              x^9 / x^8 on [-pi/4, pi/4] (truncation error below 3e-8);
//   atan:      atan(x) = pi/2 - atan(1/x) for x > 1 and two applications of the half-angle
//              identity atan(x) = 2 atan(x / (1 + sqrt(1 + x^2))), leaving |x| <= tan(pi/16),
//              then the Taylor series to x^13 (truncation error below 1e-11);
//   atan2 / acos from atan.
// PCG32 is M. O'Neill's permuted congruential generator (pcg-random.org, pcg32_random_r).
#pragma once

#include <cstdint>

#include "tt_vec.h"

#if defined(__CUDA_ARCH__)
#define PT_FMA(a, b, c) __fmaf_rn((a), (b), (c))
#define PT_MUL(a, b) __fmul_rn((a), (b))
#define PT_ADD(a, b) __fadd_rn((a), (b))
#define PT_SUB(a, b) __fsub_rn((a), (b))
#define PT_DIV(a, b) __fdiv_rn((a), (b))
#define PT_SQRT(a) __fsqrt_rn((a))
#define PT_RINT(a) rintf((a))
#else
#include <cmath>
#define PT_FMA(a, b, c) std::fma((float)(a), (float)(b), (float)(c))
#define PT_MUL(a, b) ((float)(a) * (float)(b))
#define PT_ADD(a, b) ((float)(a) + (float)(b))
#define PT_SUB(a, b) ((float)(a) - (float)(b))
#define PT_DIV(a, b) ((float)(a) / (float)(b))
#define PT_SQRT(a) std::sqrt((float)(a))
#define PT_RINT(a) std::nearbyint((float)(a))
#endif

namespace tt {
namespace pt {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kTwoPi = 6.28318530717958647692f;
constexpr float kInvPi = 0.318309886183790671538f;
constexpr float kPiOver2Hi = 1.57079637050628662109375f;   // float(pi/2)
constexpr float kPiOver2Lo = -4.37113900018624283e-8f;     // pi/2 - float(pi/2)
constexpr float kTwoOverPi = 0.636619772367581343076f;

// ---- trigonometry ------------------------------------------------------------------------------
TT_HD void sincos(float x, float &s, float &c) {
    const float k = PT_RINT(PT_MUL(x, kTwoOverPi));
    float r = PT_FMA(-k, kPiOver2Hi, x);
    r = PT_FMA(-k, kPiOver2Lo, r);
    const float r2 = PT_MUL(r, r);
    // sin r = r + r^3 (-1/6 + r^2 (1/120 + r^2 (-1/5040 + r^2 / 362880)))
    float ps = PT_FMA(r2, 2.75573192239858906526e-6f, -1.98412698412698412698e-4f);
    ps = PT_FMA(ps, r2, 8.33333333333333333333e-3f);
    ps = PT_FMA(ps, r2, -1.66666666666666666667e-1f);
    const float sr = PT_FMA(PT_MUL(ps, r2), r, r);
    // cos r = 1 + r^2 (-1/2 + r^2 (1/24 + r^2 (-1/720 + r^2 / 40320)))
    float pc = PT_FMA(r2, 2.48015873015873015873e-5f, -1.38888888888888888889e-3f);
    pc = PT_FMA(pc, r2, 4.16666666666666666667e-2f);
    pc = PT_FMA(pc, r2, -0.5f);
    const float cr = PT_FMA(pc, r2, 1.0f);
    const int q = ((int)k) & 3;
    switch (q) {
        case 0: s = sr; c = cr; break;
        case 1: s = cr; c = -sr; break;
        case 2: s = -sr; c = -cr; break;
        default: s = -cr; c = sr; break;
    }
}

// atan on [0, inf)
TT_HD float atan_pos(float x) {
    bool inv = false;
    if (x > 1.0f) {
        x = PT_DIV(1.0f, x);
        inv = true;
    }
    // two half-angle steps: x <- x / (1 + sqrt(1 + x^2))
    x = PT_DIV(x, PT_ADD(1.0f, PT_SQRT(PT_FMA(x, x, 1.0f))));
    x = PT_DIV(x, PT_ADD(1.0f, PT_SQRT(PT_FMA(x, x, 1.0f))));
    const float x2 = PT_MUL(x, x);
    // x - x^3/3 + x^5/5 - x^7/7 + x^9/9 - x^11/11 + x^13/13
    float p = PT_FMA(x2, 7.69230769230769230769e-2f, -9.09090909090909090909e-2f);
    p = PT_FMA(p, x2, 1.11111111111111111111e-1f);
    p = PT_FMA(p, x2, -1.42857142857142857143e-1f);
    p = PT_FMA(p, x2, 2.0e-1f);
    p = PT_FMA(p, x2, -3.33333333333333333333e-1f);
    float a = PT_FMA(PT_MUL(p, x2), x, x);
    a = PT_MUL(a, 4.0f);
    if (inv) a = PT_SUB(PT_ADD(kPiOver2Hi, kPiOver2Lo), a);
    return a;
}

TT_HD float atan2(float y, float x) {
    const float ax = x < 0.0f ? -x : x;
    const float ay = y < 0.0f ? -y : y;
    float a;
    if (ax == 0.0f && ay == 0.0f) a = 0.0f;
    else if (ax >= ay) a = atan_pos(PT_DIV(ay, ax));
    else a = PT_SUB(PT_ADD(kPiOver2Hi, kPiOver2Lo), atan_pos(PT_DIV(ax, ay)));
    if (x < 0.0f) a = PT_SUB(kPi, a);
    return y < 0.0f ? -a : a;
}

TT_HD float acos(float y) {
    if (y > 1.0f) y = 1.0f;
    if (y < -1.0f) y = -1.0f;
    const float s = PT_SQRT(PT_MUL(PT_SUB(1.0f, y), PT_ADD(1.0f, y)));
    return atan2(s, y);
}

// ---- PCG32 -------------------------------------------------------------------------------------
struct Rng {
    uint64_t state;
    uint64_t inc;
};

TT_HD uint32_t pcg32(Rng &g) {
    const uint64_t old = g.state;
    g.state = old * 6364136223846793005ull + g.inc;
    const uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    const uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((0u - rot) & 31u));
}

TT_HD Rng pcg32_seed(uint64_t initstate, uint64_t initseq) {
    Rng g;
    g.state = 0u;
    g.inc = (initseq << 1u) | 1u;
    pcg32(g);
    g.state += initstate;
    pcg32(g);
    return g;
}

// [0, 1) with 24 random bits
TT_HD float uniform(Rng &g) { return (float)(pcg32(g) >> 8) * (1.0f / 16777216.0f); }

// ---- vectors -----------------------------------------------------------------------------------
TT_HD float dot(const V3 &a, const V3 &b) { return PT_FMA(a.z, b.z, PT_FMA(a.y, b.y, PT_MUL(a.x, b.x))); }
TT_HD V3 add(const V3 &a, const V3 &b) { return V3(PT_ADD(a.x, b.x), PT_ADD(a.y, b.y), PT_ADD(a.z, b.z)); }
TT_HD V3 sub(const V3 &a, const V3 &b) { return V3(PT_SUB(a.x, b.x), PT_SUB(a.y, b.y), PT_SUB(a.z, b.z)); }
TT_HD V3 mul(const V3 &a, float s) { return V3(PT_MUL(a.x, s), PT_MUL(a.y, s), PT_MUL(a.z, s)); }
TT_HD V3 mul(const V3 &a, const V3 &b) { return V3(PT_MUL(a.x, b.x), PT_MUL(a.y, b.y), PT_MUL(a.z, b.z)); }
// a * s + c
TT_HD V3 madd(const V3 &a, float s, const V3 &c) {
    return V3(PT_FMA(a.x, s, c.x), PT_FMA(a.y, s, c.y), PT_FMA(a.z, s, c.z));
}
TT_HD V3 cross(const V3 &a, const V3 &b) {
    return V3(PT_FMA(a.y, b.z, -PT_MUL(a.z, b.y)), PT_FMA(a.z, b.x, -PT_MUL(a.x, b.z)),
              PT_FMA(a.x, b.y, -PT_MUL(a.y, b.x)));
}
TT_HD V3 normalize(const V3 &a) {
    const float inv = PT_DIV(1.0f, PT_SQRT(dot(a, a)));
    return mul(a, inv);
}
TT_HD float maxc(const V3 &a) {
    const float m = a.x > a.y ? a.x : a.y;
    return m > a.z ? m : a.z;
}
TT_HD float luminance(float r, float g, float b) {
    return PT_FMA(0.0722f, b, PT_FMA(0.7152f, g, PT_MUL(0.2126f, r)));
}

// Orthonormal basis around unit n (Duff et al. 2017, "Building an Orthonormal Basis, Revisited").
TT_HD void onb(const V3 &n, V3 &t, V3 &b) {
    const float sgn = n.z >= 0.0f ? 1.0f : -1.0f;
    const float a = PT_DIV(-1.0f, PT_ADD(sgn, n.z));
    const float bb = PT_MUL(PT_MUL(n.x, n.y), a);
    t = V3(PT_FMA(PT_MUL(sgn, n.x), PT_MUL(n.x, a), 1.0f), PT_MUL(sgn, bb), PT_MUL(-sgn, n.x));
    b = V3(bb, PT_FMA(PT_MUL(n.y, n.y), a, sgn), -n.y);
}
TT_HD V3 to_world(const V3 &l, const V3 &t, const V3 &b, const V3 &n) {
    return madd(n, l.z, madd(b, l.y, mul(t, l.x)));
}

// Equirectangular mapping of the reference (include/hdr/HDRKernel.cuh:18-28):
// u = atan2(x, z) / 2pi in [0, 1), v = acos(y) / pi.
TT_HD void dir_to_uv(const V3 &d, float &u, float &v) {
    float lx = atan2(d.x, d.z);
    if (lx < 0.0f) lx = PT_ADD(lx, kTwoPi);
    u = PT_DIV(lx, kTwoPi);
    v = PT_DIV(acos(d.y), kPi);
}
TT_HD V3 uv_to_dir(float u, float v, float &sin_theta) {
    float st, ct, sp, cp;
    sincos(PT_MUL(v, kPi), st, ct);
    sincos(PT_MUL(u, kTwoPi), sp, cp);
    sin_theta = st;
    return V3(PT_MUL(st, sp), ct, PT_MUL(st, cp));
}

}  // namespace pt
}  // namespace tt
