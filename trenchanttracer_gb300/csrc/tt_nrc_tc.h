// The radiance cache's tcgen05 inference path (tt_nrc_tc.cu); internal to libtt.so.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>

#include "tt_internal.h"

namespace tt {
namespace nrc {

tt_status tc_setup();
// BF16 elements of the weights in the tcgen05 operand layout
size_t tc_weight_elems();
// compact FP32 [out][in] weights -> the operand layout (launch only)
void tc_relayout(const float *w_f32, uint16_t *w_tc, cudaStream_t s);
// radiance of min(*n_dev, cap) records (n_dev set) or n_host records; flag 8 in the error word on a wait
// that ran out; wait_cycles: the budget of each wait in clock cycles (<= 0: about a second) (launch
// only)
tt_status tc_infer(const uint16_t *w_tc, const float *rec, long long n_host, const int *n_dev, long long cap,
                   const float lo[3], const float inv_ext[3], float *rgb, unsigned *err, int num_sms,
                   long long wait_cycles, cudaStream_t s);

}  // namespace nrc
}  // namespace tt
