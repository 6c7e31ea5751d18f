// Probe build of the reference's OWN path tracer (src/core/RenderKernel.cu, pathTracingKernel):
// the same translation unit as ref_render_harness.cu, except that each of the five material
// samplers (include/material/{Diff,Metal,Spec,Refr,Coat}Impl.cuh) is called through a wrapper that
// records one interaction per call: the incoming ray, the hit record that renderKernel built
// (raw normal and distance, then n, nl and point from normalize() / hitPoint(),
// include/geometry/IntersectKernel.cuh:62-76), the throughput mask, the curand XORWOW state and the
// first uniform it will draw, and what the sampler returned (next ray, mask, curand state); and
// every environment lookup (hdrSample) at a path's miss with the radiance it returned.
//
// The wrappers only copy values in and out around the unchanged reference sampler, so the
// frame this kernel accumulates must equal ref_render.cubin's bit for bit (tests check that
// before trusting a record). The records are the reference's own single interactions, inside its
// own kernel, that tt_compat_replay re-runs through the compatible renderer's samplers.
//
// Record layout: 64 x 32-bit words, the same as tt_compat_interaction in include/tt.h.
// Test infrastructure only: compiled by oracle/build_ref.py into oracle/_ref/ref_render_probe.cubin.
#include <core/Renderer.h>
#include <curand_kernel.h>
#include <hdr/HDRImage.h>
#include <hdr/HDRKernel.cuh>
#include <math/CutilMath.h>
#include <geometry/IntersectKernel.cuh>
#include <geometry/Ray.h>
#include <geometry/GeometryCompact.h>
#include <geometry/SphereImpl.cuh>
#include <geometry/PlaneImpl.cuh>
#include <material/CoatImpl.cuh>
#include <material/DiffImpl.cuh>
#include <material/MetalImpl.cuh>
#include <material/SpecImpl.cuh>
#include <material/RefrImpl.cuh>

static_assert(sizeof(curandState) == 48, "curand XORWOW state is 12 words");

struct ProbeRecord {
    int kind, thread, material, seq;
    float o[3], d[3], tmin, tmax;
    float normal[3], distance;
    float n[3], nl[3], point[3];
    float mask[3];
    unsigned rng[12];
    float out_o[3], out_d[3], out_mask[3];
    unsigned out_rng[12];
    float u0;
    int pad[2];
};
static_assert(sizeof(ProbeRecord) == 256, "one record is 64 words");

__device__ ProbeRecord *g_probe_records;
__device__ unsigned long long g_probe_capacity;
__device__ unsigned long long g_probe_count;

// capacity >= 1
extern "C" __global__ void ref_probe_setup(ProbeRecord *records, unsigned long long capacity) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    g_probe_records = records;
    g_probe_capacity = capacity;
    g_probe_count = 0;
}

extern "C" __global__ void ref_probe_count(unsigned long long *out) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *out = g_probe_count;
}

__device__ __forceinline__ void put3(float *dst, const Vec3f &v) {
    dst[0] = v.x;
    dst[1] = v.y;
    dst[2] = v.z;
}

// Straight-line code only: a branch here would split renderKernel's basic blocks, and nvcc decides
// which products it fuses into adds within a block, so the reference's own rounding would change.
__device__ __forceinline__ void probe_begin(int kind, const void *m, curandState *rs, const Ray &ray, const Hit &hit,
                                            const Vec3f &mask, ProbeRecord &r) {
    r.kind = kind;
    r.thread = (int)((blockIdx.x + blockIdx.y * gridDim.x) * (blockDim.x * blockDim.y) + threadIdx.y * blockDim.x +
                     threadIdx.x);
    r.material = (int)reinterpret_cast<const Material *>(m)->index;
    r.seq = (int)rs->d;  // the XORWOW counter advances with every draw: orders a thread's records
    put3(r.o, ray.origin);
    put3(r.d, ray.direction);
    r.tmin = ray.tMin;
    r.tmax = ray.tMax;
    put3(r.normal, hit.normal);
    r.distance = hit.distance;
    put3(r.n, hit.n);
    put3(r.nl, hit.nl);
    put3(r.point, hit.point);
    put3(r.mask, mask);
    memcpy(r.rng, rs, 48);
    curandState copy = *rs;
    r.u0 = curand_uniform(&copy);
}

__device__ __forceinline__ void probe_end(ProbeRecord &r, const Ray &next, const curandState *rs, const Vec3f &mask) {
    put3(r.out_o, next.origin);
    put3(r.out_d, next.direction);
    put3(r.out_mask, mask);
    memcpy(r.out_rng, rs, 48);
    const unsigned long long slot = atomicAdd(&g_probe_count, 1ull);
    // past the capacity every record lands in the last slot (a select, not a branch)
    g_probe_records[slot < g_probe_capacity ? slot : g_probe_capacity - 1] = r;
}

// Each wrapper calls the reference sampler directly, so it is inlined into renderKernel as in
// the plain build.
#define TT_PROBE_WRAPPER(name, Type, sampler, KIND)                                                 \
    __device__ __inline__ Ray name(Type *m, curandState *rs, const Ray &ray, const Hit &hit, Vec3f &mask) { \
        ProbeRecord r;                                                                              \
        probe_begin(KIND, m, rs, ray, hit, mask, r);                                               \
        const Ray next = sampler(m, rs, ray, hit, mask);                                           \
        probe_end(r, next, rs, mask);                                                              \
        return next;                                                                                \
    }
TT_PROBE_WRAPPER(probe_diff, Diff, diffSample, DIFF)
TT_PROBE_WRAPPER(probe_metal, Metal, metalSample, METAL)
TT_PROBE_WRAPPER(probe_spec, Spec, specSample, SPEC)
TT_PROBE_WRAPPER(probe_refr, Refr, refrSample, REFR)
TT_PROBE_WRAPPER(probe_coat, Coat, coatSample, COAT)

// hdrSample (include/hdr/HDRKernel.cuh:6-42) at a path's miss: recorded as kind 5 with the ray
// that missed, the mask, and the returned radiance in out_mask; the curand fields are unused.
__device__ __inline__ Vec3f probe_hdr(const HDRImage *img, const Ray &ray, RenderMeta *meta) {
    ProbeRecord r;
    r.kind = 5;
    r.thread = (int)((blockIdx.x + blockIdx.y * gridDim.x) * (blockDim.x * blockDim.y) + threadIdx.y * blockDim.x +
                     threadIdx.x);
    r.material = -1;
    r.seq = 0;
    put3(r.o, ray.origin);
    put3(r.d, ray.direction);
    r.tmin = ray.tMin;
    r.tmax = ray.tMax;
    const Vec3f c = hdrSample(img, ray, meta);
    put3(r.out_mask, c);
    const unsigned long long slot = atomicAdd(&g_probe_count, 1ull);
    g_probe_records[slot < g_probe_capacity ? slot : g_probe_capacity - 1] = r;
    return c;
}

// renderKernel's calls go to the wrappers; the samplers' own headers are already included above,
// so RenderKernel.cu's includes of them are no-ops and the definitions keep their names.
// TT_PROBE_KINDS (bit k: MaterialType k, bit 5: hdrSample; default all) picks which calls are
// recorded, so that a build recording fewer of them can be checked against the plain frame.
#ifndef TT_PROBE_KINDS
#define TT_PROBE_KINDS 0x3F
#endif
#if TT_PROBE_KINDS & 1
#define diffSample probe_diff
#endif
#if TT_PROBE_KINDS & 2
#define metalSample probe_metal
#endif
#if TT_PROBE_KINDS & 4
#define specSample probe_spec
#endif
#if TT_PROBE_KINDS & 8
#define refrSample probe_refr
#endif
#if TT_PROBE_KINDS & 16
#define coatSample probe_coat
#endif
#if TT_PROBE_KINDS & 32
#define hdrSample probe_hdr
#endif
#include "ref_render_harness.cu"
