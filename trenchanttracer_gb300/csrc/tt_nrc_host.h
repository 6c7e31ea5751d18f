// Host-side entry points of the radiance cache used by the path tracer (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>

#include "../../include/tt.h"

namespace tt {
namespace nrc {

// Radiance of the first min(*n_dev, cap) records (kRec floats each) into rgb (3 floats each); a
// tensor-core wait that runs out sets the flag 8 in `err` (the cache's own error word when null).
tt_status cache_infer_device(tt_cache *c, const float *rec, const int *n_dev, long long cap, float *rgb, int use_ema,
                             unsigned *err, cudaStream_t s);
// params.steps Adam steps over consecutive slices of params.batch of the first *n_dev records.
tt_status cache_train_device(tt_cache *c, const float *rec, const float *target, const int *n_dev, cudaStream_t s);
const tt_cache_params &cache_params(const tt_cache *c);

}  // namespace nrc
}  // namespace tt
