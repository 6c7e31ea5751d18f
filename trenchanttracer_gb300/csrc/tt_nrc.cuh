// Learned radiance cache: network shape, feature records and parameter layouts, shared by the
// MLP kernels (tt_nrc.cu) and the path tracer that queries and trains it (tt_render_native.cu).
//
// Network: encoded input (160) -> 64 -> 64 -> 64 -> 64 -> 64 -> 3, ReLU on the hidden layers, no
// biases (the encoding carries a constant-1 feature), RGB radiance = exp(output). BF16 weights and
// activations, FP32 accumulation on the tensor cores (tcgen05 with TMEM accumulators by default,
// mma.sync m16n8k16 as the alternative kind), FP32 master weights and Adam state.
//
// Layers l = 0..5: Z_l = W_l H_l, H_{l+1} = relu(Z_l) for l < 5, Y = W_5 H_5. W_l is stored
// [out][in]; the output layer is padded from 3 to 8 rows that stay zero.
#pragma once

#include <cstdint>

#ifdef __CUDACC__
#include <cuda_bf16.h>
#endif

namespace tt {
namespace nrc {

constexpr int kIn = 160;      // encoded input width
constexpr int kHidden = 64;   // hidden width
constexpr int kLayers = 6;
constexpr int kOut = 3;       // RGB
constexpr int kOutPad = 8;    // output rows of W_5 (rows 3..7 are zero)
constexpr int kRowPad = 8;    // bf16 padding of every weight row in the padded layout
constexpr int kRec = 16;      // floats per raw feature record

// Raw feature record of a cache query (16 floats):
//   [0..2] position, [3..5] direction towards the previous vertex (wo), [6..8] shading normal
//   (facing wo), [9] roughness, [10..12] albedo (Lambert colour, GGX F0, 1 for smooth
//   dielectrics and mirrors), [13] material kind / 8, [14..15] 0.
// Encoding (160 values):
//   [0, 72)    position: p_hat = (p - lo) / (hi - lo); for axis i and frequency k < 12:
//              sin(pi 2^k p_hat_i), cos(pi 2^k p_hat_i) at 24 i + 2 k, 24 i + 2 k + 1
//   [72, 108)  direction: x_i = (wo_i + 1) / 2, frequencies k < 6, at 72 + 12 i + 2 k (+1)
//   [108, 144) normal: the same as direction, at 108 + 12 i + 2 k (+1)
//   [144, 160) roughness, albedo (3), 1, wo (3), normal (3), p_hat (3), kind / 8, 0
constexpr int kPosFreq = 12;
constexpr int kDirFreq = 6;

__host__ __device__ constexpr int layer_in(int l) { return l == 0 ? kIn : kHidden; }
__host__ __device__ constexpr int layer_out(int l) { return l == kLayers - 1 ? kOutPad : kHidden; }
// offsets of W_l in the compact FP32 layout ([out][in]) and the padded BF16 layout ([out][in + 8])
__host__ __device__ constexpr int w_offset(int l) { return l == 0 ? 0 : w_offset(l - 1) + layer_in(l - 1) * layer_out(l - 1); }
__host__ __device__ constexpr int p_offset(int l) {
    return l == 0 ? 0 : p_offset(l - 1) + (layer_in(l - 1) + kRowPad) * layer_out(l - 1);
}
constexpr int kParams = w_offset(kLayers);     // 27136
constexpr int kPadded = p_offset(kLayers);     // 29760 bf16 = 59520 bytes
static_assert(kParams == 160 * 64 + 4 * 64 * 64 + 8 * 64, "parameter count");

// The tcgen05 operand layout of the weights (tt_nrc_tc.cu): layer l as N = tc_out(l) rows of K =
// layer_in(l) BF16 values in 8 x 8 core matrices, K-major; rows beyond the layer's outputs are 0.
__host__ __device__ constexpr int tc_out(int l) { return l == kLayers - 1 ? 16 : kHidden; }
__host__ __device__ constexpr int tc_offset(int l) { return l == 0 ? 0 : tc_offset(l - 1) + layer_in(l - 1) * tc_out(l - 1); }
constexpr int kTcWeights = tc_offset(kLayers);  // 27648 bf16
__host__ __device__ inline int tc_index(int l, int n, int k) {
    const int ng = tc_out(l) / 8;
    return tc_offset(l) + ((k / 8) * ng + n / 8) * 64 + (n % 8) * 8 + (k % 8);
}
// The transposed operand layout the backward pass multiplies by: layer l >= 1 as N = layer_in(l)
// rows of K = tc_out(l) values, element (n, k) = W_l[k][n] (k beyond the layer's outputs: 0), in 8 x
// 8 core matrices, K-major.
__host__ __device__ constexpr int tcT_offset(int l) { return l <= 1 ? 0 : tcT_offset(l - 1) + layer_in(l - 1) * tc_out(l - 1); }
constexpr int kTcTWeights = tcT_offset(kLayers);  // 17408 bf16
static_assert(kTcTWeights == 4 * 64 * 64 + 64 * 16, "transposed weights of layers 1..5");
__host__ __device__ inline int tcT_index(int l, int n, int k) {
    const int ng = layer_in(l) / 8;
    return tcT_offset(l) + ((k / 8) * ng + n / 8) * 64 + (n % 8) * 8 + (k % 8);
}


#ifdef __CUDACC__
// sin(pi x) and cos(pi x): the argument reduced exactly to r = x - 2 rint(x / 2) in [-1, 1],
// then the hardware approximations of sin and cos of pi r (absolute error ~4e-7, far below the
// BF16 step of the encoding).
__device__ __forceinline__ void sincospi_fast(float x, float &s, float &c) {
    const float r = x - 2.0f * rintf(0.5f * x);
    __sincosf(r * 3.14159265358979f, &s, &c);
}

// The per-record inputs of the encoding: normalised position, (wo + 1) / 2, (n + 1) / 2.
struct EncInputs {
    float ph[3], xd[3], xn[3];
};

__device__ __forceinline__ EncInputs enc_inputs(const float *rec, const float lo[3], const float inv_ext[3]) {
    EncInputs in;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        in.ph[i] = (rec[i] - lo[i]) * inv_ext[i];
        in.xd[i] = (rec[3 + i] + 1.0f) * 0.5f;
        in.xn[i] = (rec[6 + i] + 1.0f) * 0.5f;
    }
    return in;
}

__device__ __forceinline__ uint32_t enc_pack(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t *>(&v);
}

// Encoding values [8 c, 8 c + 8) as four packed BF16 pairs (c = 0..19; with c a compile-time
// constant after unrolling, the index arithmetic folds away).
__device__ __forceinline__ uint4 enc_chunk(const EncInputs &in, const float *rec, int c) {
    uint32_t w[4];
    if (c < 18) {
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int idx = 8 * c + 2 * j;
            float src;
            int k;
            if (idx < 72) {
                src = in.ph[idx / 24];
                k = (idx % 24) / 2;
            } else if (idx < 108) {
                src = in.xd[(idx - 72) / 12];
                k = ((idx - 72) % 12) / 2;
            } else {
                src = in.xn[(idx - 108) / 12];
                k = ((idx - 108) % 12) / 2;
            }
            float sv, cv;
            sincospi_fast(src * (float)(1 << k), sv, cv);
            w[j] = enc_pack(sv, cv);
        }
    } else if (c == 18) {  // roughness, albedo, 1, wo
        w[0] = enc_pack(rec[9], rec[10]);
        w[1] = enc_pack(rec[11], rec[12]);
        w[2] = enc_pack(1.0f, rec[3]);
        w[3] = enc_pack(rec[4], rec[5]);
    } else {  // normal, p_hat, kind, 0
        w[0] = enc_pack(rec[6], rec[7]);
        w[1] = enc_pack(rec[8], in.ph[0]);
        w[2] = enc_pack(in.ph[1], in.ph[2]);
        w[3] = enc_pack(rec[13], 0.0f);
    }
    return make_uint4(w[0], w[1], w[2], w[3]);
}
#endif

}  // namespace nrc
}  // namespace tt
