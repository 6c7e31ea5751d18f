// Internal glue between the CUDA translation units of libtt.so (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>

#include "tt_internal.h"
#include "tt_traverse.cuh"

namespace tt {

// The device arrays of an uploaded BVH (tt_trace.cu owns the handle's layout), and its scene
// bounds from the root's boxes (the ray-ordering grid).
BvhView dbvh_view(const tt_dbvh *bvh);
void dbvh_bounds(const tt_dbvh *bvh, float lo[3], float hi[3]);

}  // namespace tt

// Renderer state shared by the compatible (tt_render_compat.cu) and native
// (tt_render_native.cu) path tracers.
struct tt_renderer {
    tt::BvhView bvh{};
    tt::MaterialRec *materials = nullptr;
    int num_materials = 0;
    tt::GeomRec *geoms = nullptr;
    int num_geoms = 0;
    // the native tracer's bounding-box hierarchy over the analytic objects (more than a few):
    // num_geom_nodes GeomNode records followed by num_geoms object indices, one allocation
    void *geom_tree = nullptr;
    int num_geom_nodes = 0;
    float4 *env = nullptr;  // env_w * env_h radiance texels (w = 0: no environment)
    int env_w = 0, env_h = 0;
    unsigned int *err = nullptr;  // 256 bytes: error word at 0, native ray counters at byte 64
    // native path tracer
    float *env_marg = nullptr;  // env_h + 1
    float *env_cond = nullptr;  // env_h * (env_w + 1)
    // guide tables of the CDFs: env_gm + 1 entries for the marginal, then env_gc + 1 per row
    int *env_guide = nullptr;
    int env_gm = 0, env_gc = 0;
    void *paths = nullptr;      // path state, queues and shadow rays for path_capacity paths
    size_t paths_bytes = 0;
    int path_capacity = 0;
    unsigned long long paths_gen = 0;  // bumped whenever `paths` is reallocated
    int num_sms = 0;
    // launch shape of the native kernels (tt_renderer_set_launch, tt_batch_autotune)
    int launch_block = 128, launch_stack = 16, launch_wave = 1 << 22;
    int launch_order = 0;  // order each extension queue by origin and direction cell before tracing
    int launch_stream = 1; // stream renders of more paths than one wave through a refilled pool
    unsigned long long launches = 0;  // path-tracer kernels issued (launched or captured)
    float order_lo[3] = {-1.f, -1.f, -1.f}, order_hi[3] = {1.f, 1.f, 1.f};  // scene bounds
    size_t order_off = 0;       // byte offset of the ordering scratch inside `paths` (0: none)
    size_t order_state_at = 0;  // its state block, relative to the scratch
    int occ_trace[3][3] = {};  // resident blocks per SM by (block shape, stack shape); 0 = unknown
    int occ_shade[3] = {};
    // radiance-cache queries and training records of cached renders
    void *cache_mem = nullptr;
    size_t cache_bytes = 0;
    long long cache_queries = 0, cache_records = 0;
    // streamed renders (more paths than one wave, refilled as paths end): the radiance ring, the
    // second copy of the path state, both copies' path indices and the plan record, one allocation
    void *stream_mem = nullptr;
    size_t stream_bytes = 0;
};

namespace tt {
// Error-word bit of the renderer: a streamed render ended with paths unfinished.
constexpr uint32_t kErrStream = 16u;
// [0] extension rays, [1] shadow rays, [2] paths traced by the native path tracer
inline unsigned long long *renderer_stats(tt_renderer *r) {
    return reinterpret_cast<unsigned long long *>(reinterpret_cast<char *>(r->err) + 64);
}
}  // namespace tt

namespace tt {
// Builds the environment's sampling tables and the analytic objects' box hierarchy (called by
// tt_renderer_create with the scene's objects) / frees native state.
tt_status native_setup(tt_renderer *r, const std::vector<GeomRec> &geoms);
void native_release(tt_renderer *r);
}  // namespace tt
