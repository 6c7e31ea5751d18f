// Learned radiance cache: network shape, feature records and parameter layouts, shared by the
// MLP kernels (tt_nrc.cu) and the path tracer that queries and trains it (tt_render_native.cu).
//
// Network: encoded input (160) -> 64 -> 64 -> 64 -> 64 -> 64 -> 3, ReLU on the hidden layers, no
// biases (the encoding carries a constant-1 feature), RGB radiance = exp(output). BF16 weights and
// activations, FP32 accumulation (mma.sync m16n8k16 bf16 tensor-core instructions), FP32 master
// weights and Adam state.
//
// Layers l = 0..5: Z_l = W_l H_l, H_{l+1} = relu(Z_l) for l < 5, Y = W_5 H_5. W_l is stored
// [out][in]; the output layer is padded from 3 to 8 rows that stay zero.
#pragma once

#include <cstdint>

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

}  // namespace nrc
}  // namespace tt
