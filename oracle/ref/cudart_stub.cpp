// Host-only stand-ins for the handful of CUDA runtime calls the reference's builder and
// scene code make (BVHCompact.cpp:196-317, HDRImage.cpp:16-52, Renderer-free paths), so that
// the reference's own SBVH builder can run on a machine without a GPU. "Device" memory is
// host memory; a texture object is the address of its linear buffer.
//
// Test infrastructure only: linked into oracle/_ref/libttref_host.so, never into libtt.so.
#include <cuda_runtime_api.h>

#include <cstdlib>
#include <cstdint>
#include <cstring>

extern "C" {

cudaError_t cudaMalloc(void **p, size_t n) {
    *p = malloc(n ? n : 1);
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}

cudaError_t cudaFree(void *p) {
    free(p);
    return cudaSuccess;
}

cudaError_t cudaMemcpy(void *dst, const void *src, size_t n, enum cudaMemcpyKind) {
    if (n) memmove(dst, src, n);
    return cudaSuccess;
}

cudaError_t cudaMemset(void *p, int v, size_t n) {
    memset(p, v, n);
    return cudaSuccess;
}

cudaError_t cudaCreateTextureObject(cudaTextureObject_t *tex, const struct cudaResourceDesc *res,
                                    const struct cudaTextureDesc *, const struct cudaResourceViewDesc *) {
    *tex = (cudaTextureObject_t)(uintptr_t)res->res.linear.devPtr;
    return cudaSuccess;
}

cudaError_t cudaDestroyTextureObject(cudaTextureObject_t) { return cudaSuccess; }

}  // extern "C"
