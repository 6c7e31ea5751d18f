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

// BF16 elements of the transposed operand layout of layers 1..5 (the backward pass's B operand)
size_t tcT_weight_elems();
void tcT_relayout(const float *w_f32, uint16_t *w_tcT, cudaStream_t s);
// chunks (partial gradients) of a weight-gradient pass over `rows` rows
int tc_wgrad_chunks(long long rows, int num_sms);

// One training pass on the tensor cores over rows [0, rows) of the call (rows = clamp(*n_dev - off,
// 0, cap) with n_dev set, else n_host): forward (storing each layer's input H_l and the raw
// outputs y), backward (dZ_l, the loss) and the weight gradients, one partial per chunk of rows.
struct TcTrainArgs {
    const uint16_t *w_tc, *w_tcT;
    const float *rec, *target;  // the pass's first row
    long long n_host;
    const int *n_dev;
    long long off, cap;
    float lo[3], inv_ext[3];
    float *y;
    uint16_t *h[6], *dz[6];
    float *loss;
    float *partial;
    unsigned *err;
    int num_sms;
    long long wait_cycles;
};
tt_status tc_train(const TcTrainArgs &t, cudaStream_t s);

}  // namespace nrc
}  // namespace tt
