// Host stand-ins for the device intrinsics the reference's intersect() uses, so that the
// reference's own traversal source compiles for the CPU: a texture object is the address of
// its linear buffer (see cudart_stub.cpp), and the float/int reinterpretations are memcpy.
// The two inline-PTX sites of IntersectKernel.cuh (video min/max, warp ballot) are rewritten
// by oracle/build_ref.py in a temporary copy of that one header.
//
// Test infrastructure only.
#pragma once

#include <cuda_runtime_api.h>

#include <cstdint>
#include <cstring>

template <class T>
inline T tex1Dfetch(cudaTextureObject_t obj, int i) {
    return reinterpret_cast<const T *>(static_cast<uintptr_t>(obj))[i];
}

inline int __float_as_int(float f) {
    int i;
    memcpy(&i, &f, 4);
    return i;
}

inline float __int_as_float(int i) {
    float f;
    memcpy(&f, &i, 4);
    return f;
}
