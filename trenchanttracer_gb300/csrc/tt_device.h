// Internal glue between the CUDA translation units of libtt.so (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>

#include "tt_internal.h"
#include "tt_traverse.cuh"

namespace tt {

// The device arrays of an uploaded BVH (tt_trace.cu owns the handle's layout).
BvhView dbvh_view(const tt_dbvh *bvh);

}  // namespace tt
