// Small float vector helpers shared by host C++ and device CUDA code.
//
// Expression shapes follow the reference's LinearMath (include/math/LinearMath.h:
// cross :260-262, dot :264-266, normalize :101-107, min3f/max3f :252-258). The host
// library is compiled with -ffp-contract=off so that every product and sum is rounded
// on its own, as the reference's x86 host build does (SSE, no FMA); that keeps the
// SBVH build and the scene transforms bit-identical across x86 and Arm.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define TT_HD __host__ __device__ __forceinline__
#else
#define TT_HD inline
#endif

namespace tt {

struct V3 {
    float x, y, z;
    TT_HD V3() : x(0.f), y(0.f), z(0.f) {}
    TT_HD V3(float a, float b, float c) : x(a), y(b), z(c) {}
    TT_HD float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    TT_HD float &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
};

TT_HD V3 operator+(const V3 &a, const V3 &b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
TT_HD V3 operator-(const V3 &a, const V3 &b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
TT_HD V3 operator*(const V3 &a, const V3 &b) { return V3(a.x * b.x, a.y * b.y, a.z * b.z); }
TT_HD V3 operator*(const V3 &a, float s) { return V3(a.x * s, a.y * s, a.z * s); }
TT_HD V3 operator/(const V3 &a, float s) { return V3(a.x / s, a.y / s, a.z / s); }
TT_HD V3 operator-(const V3 &a) { return V3(-a.x, -a.y, -a.z); }

TT_HD float dot3(const V3 &a, const V3 &b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
TT_HD V3 cross3(const V3 &a, const V3 &b) {
    return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
// normalize as the reference does it: one sqrt of the squared length, then three divides.
TT_HD V3 normalized(const V3 &a) {
    float n = sqrtf(a.x * a.x + a.y * a.y + a.z * a.z);
    return V3(a.x / n, a.y / n, a.z / n);
}
TT_HD V3 vmin3(const V3 &a, const V3 &b) {
    return V3(a.x < b.x ? a.x : b.x, a.y < b.y ? a.y : b.y, a.z < b.z ? a.z : b.z);
}
TT_HD V3 vmax3(const V3 &a, const V3 &b) {
    return V3(a.x > b.x ? a.x : b.x, a.y > b.y ? a.y : b.y, a.z > b.z ? a.z : b.z);
}

TT_HD uint32_t f2u(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}
TT_HD float u2f(uint32_t u) {
    float f;
    memcpy(&f, &u, 4);
    return f;
}

}  // namespace tt
