// Ray ordering before traversal (tt_reorder.cu); internal to libtt.so.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "../../include/tt.h"

namespace tt {

constexpr int kOrderBits = 21;  // direction octant (3) + Morton code of a 64^3 origin grid (18)

// Device scratch for ordering n rays: keys, permutation, 2^21 counts and the scan's block sums.
size_t reorder_scratch_bytes(int64_t n);
// Writes to *perm_out a device array of n ray indices grouped by key (launch only, on stream s).
// scene bounds lo < hi per axis.
tt_status reorder_rays(const float4 *rays, int64_t n, const float lo[3], const float hi[3], void *scratch,
                       int num_sms, cudaStream_t s, const int **perm_out);

}  // namespace tt
