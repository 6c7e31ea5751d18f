// Internal glue between the CUDA translation units of libtt.so (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>

#include "tt_internal.h"
#include "tt_traverse.cuh"

namespace tt {

// The device arrays of an uploaded BVH (tt_trace.cu owns the handle's layout).
BvhView dbvh_view(const tt_dbvh *bvh);

}  // namespace tt

// Renderer state shared by the compatible (tt_render_compat.cu) and native
// (tt_render_native.cu) path tracers.
struct tt_renderer {
    tt::BvhView bvh{};
    tt::MaterialRec *materials = nullptr;
    int num_materials = 0;
    tt::GeomRec *geoms = nullptr;
    int num_geoms = 0;
    float4 *env = nullptr;  // env_w * env_h radiance texels (w = 0: no environment)
    int env_w = 0, env_h = 0;
    unsigned int *err = nullptr;
    // native path tracer
    float *env_marg = nullptr;  // env_h + 1
    float *env_cond = nullptr;  // env_h * (env_w + 1)
    void *paths = nullptr;      // path state, queues and shadow rays for path_capacity paths
    size_t paths_bytes = 0;
    int path_capacity = 0;
    int num_sms = 0;
};

namespace tt {
// Builds the environment's sampling tables (called by tt_renderer_create) / frees native state.
tt_status native_setup(tt_renderer *r);
void native_release(tt_renderer *r);
}  // namespace tt
