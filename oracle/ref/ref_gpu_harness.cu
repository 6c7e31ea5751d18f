// Harness kernel around the reference's OWN device intersect(), compiled by
// oracle/build_ref.py (with the one-line ballot shim the reference needs on sm_70+) into
// oracle/_ref/ref_intersect.cubin. It runs one ray per thread, 256 threads per block, over
// texture objects created exactly as BVHCompact::createTexture does
// (src/bvh/BVHCompact.cpp:276-317), and writes every field of the returned Hit.
//
// Test infrastructure only: the device oracle that pins hit ids and distances bit for bit.
#include <geometry/IntersectKernel.cuh>

extern "C" __global__ void ref_trace_kernel(const float *rays, int n, cudaTextureObject_t nodes,
                                            cudaTextureObject_t vertices, cudaTextureObject_t normals,
                                            cudaTextureObject_t tri_indices, cudaTextureObject_t mat_indices,
                                            int closest, int *idx, int *mat, float *t, float *normal) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    alignas(16) unsigned char storage[sizeof(BVHCompact)];
    BVHCompact *bvh = reinterpret_cast<BVHCompact *>(storage);
    bvh->nodesTexture = nodes;
    bvh->verticesTexture = vertices;
    bvh->normalsTexture = normals;
    bvh->triIndicesTexture = tri_indices;
    bvh->matIndicesTexture = mat_indices;
    const float *r = rays + 8 * (long long)i;
    Ray ray(Vec3f(r[0], r[1], r[2]), Vec3f(r[3], r[4], r[5]), r[6], r[7]);
    Hit h = intersect(ray, bvh, closest != 0);
    idx[i] = h.index;
    t[i] = h.distance;
    mat[i] = h.index != -1 ? h.matIndex : -1;
    normal[3 * (long long)i + 0] = h.normal.x;
    normal[3 * (long long)i + 1] = h.normal.y;
    normal[3 * (long long)i + 2] = h.normal.z;
}
