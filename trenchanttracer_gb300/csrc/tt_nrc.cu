// Learned radiance cache: the cache object and its C ABI, the Adam kernel, and the mma.sync kind
// of the MLP's encoding, forward, backward and weight-gradient kernels (BF16 m16n8k16, FP32
// accumulation; mma_kind = 1). The default kind runs the network on tcgen05 + TMEM
// (tt_nrc_tc.cu); both write the same scratch layouts and partial gradients, which Adam sums.
//
// Fused forward / backward: each warp owns tiles of 16 rows. The encoding of a tile is built in
// shared memory; every later activation stays in registers, because the FP32 accumulator
// fragment of an m16n8 product, rounded to BF16 in pairs, is exactly the A-operand fragment of
// the next m16n8k16 product (two n-tiles make one k-tile). All weights of the network (59.5 KB
// as padded BF16) sit in shared memory; a padded row stride (in + 8 elements) makes every
// fragment load conflict-free. Training also stores each layer's BF16 activations and
// pre-activation gradients for the weight gradients.
//
// Weight gradients dW_l = dZ_l^T H_l are split over row chunks (one CTA per chunk and layer):
// each CTA stages transposed 32-row tiles of dZ_l and H_l in shared memory and accumulates
// its partial product with the same mma instruction; Adam sums the partials in chunk order, so a
// training step is deterministic.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "tt_internal.h"
#include "tt_nrc.cuh"
#include "tt_nrc_host.h"
#include "tt_nrc_tc.h"

namespace tt {
namespace nrc {

constexpr int kWarps = 4;
constexpr int kThreads = 32 * kWarps;
constexpr int kEncStride = kIn + kRowPad;  // bf16 per row of a warp's encoding tile
constexpr int kWeightBytes = kPadded * 2;
constexpr int kFwdSmem = kWeightBytes + kWarps * 16 * kEncStride * 2;
constexpr int kChunkRows = 128;            // rows per weight-gradient CTA (128 CTAs x 6 layers per 16K batch)

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t *>(&v);
}
__device__ __forceinline__ uint32_t pack_u16(uint16_t lo, uint16_t hi) { return (uint32_t)lo | ((uint32_t)hi << 16); }
__device__ __forceinline__ bool bf16_positive(uint32_t bits16) { return bits16 != 0u && !(bits16 & 0x8000u); }

// D += A B, m16n8k16, A row-major BF16, B column-major BF16, FP32 accumulators.
__device__ __forceinline__ void mma(float c[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

struct Encoding {
    float lo[3], inv_ext[3];
};

// Values of record `rec` into one encoding row (16-byte aligned): part 0 = chunks 0..8 (the
// position block [0, 72)), part 1 = chunks 9..19 (everything else).
__device__ __forceinline__ void encode_part(const float *rec, const Encoding &e, __nv_bfloat16 *dst, int part) {
    const EncInputs in = enc_inputs(rec, e.lo, e.inv_ext);
    uint4 *d4 = reinterpret_cast<uint4 *>(dst);
    if (part == 0) {
#pragma unroll
        for (int c = 0; c < 9; c++) d4[c] = enc_chunk(in, rec, c);
    } else {
#pragma unroll
        for (int c = 9; c < 20; c++) d4[c] = enc_chunk(in, rec, c);
    }
}

struct MlpArgs {
    const uint16_t *w;   // padded BF16 weights
    const float *rec;    // records (row 0 of this call)
    const float *target; // backward: n x 3 target radiance
    long long n_host;    // rows when n_dev is null
    const int *n_dev;    // device row count of the buffer (rows = clamp(*n_dev - off, 0, cap))
    long long off, cap;
    Encoding enc;
    float *rgb;          // inference output: n x 3 radiance
    float *y;            // training: n x 3 raw outputs
    uint16_t *h[kLayers];   // training: H_0 (n x 160), H_1..H_5 (n x 64)
    uint16_t *dz[kLayers];  // backward: dZ_0..dZ_4 (n x 64), dY (n x 8)
    float *loss;         // backward: loss sum (atomic, for monitoring)
};

__device__ __forceinline__ long long rows_of(const MlpArgs &a) {
    if (!a.n_dev) return a.n_host;
    long long n = (long long)*a.n_dev - a.off;
    return n < 0 ? 0 : (n > a.cap ? a.cap : n);
}

__device__ __forceinline__ void load_weights(uint8_t *smem, const uint16_t *w) {
    const uint4 *src = reinterpret_cast<const uint4 *>(w);
    uint4 *dst = reinterpret_cast<uint4 *>(smem);
    for (int i = threadIdx.x; i < kWeightBytes / 16; i += blockDim.x) dst[i] = src[i];
}

// relu, round to BF16 and re-pack an m16n64 accumulator as the four A fragments of a k = 64
// operand
__device__ __forceinline__ void relu_pack(const float acc[8][4], uint32_t hf[4][4]) {
#pragma unroll
    for (int kt = 0; kt < 4; kt++) {
        hf[kt][0] = pack2(fmaxf(acc[2 * kt][0], 0.f), fmaxf(acc[2 * kt][1], 0.f));
        hf[kt][1] = pack2(fmaxf(acc[2 * kt][2], 0.f), fmaxf(acc[2 * kt][3], 0.f));
        hf[kt][2] = pack2(fmaxf(acc[2 * kt + 1][0], 0.f), fmaxf(acc[2 * kt + 1][1], 0.f));
        hf[kt][3] = pack2(fmaxf(acc[2 * kt + 1][2], 0.f), fmaxf(acc[2 * kt + 1][3], 0.f));
    }
}

// stores A fragments (16 x 64) into a row-major n x 64 BF16 matrix, rows below n only
__device__ __forceinline__ void store_frag64(uint16_t *m, long long r0, long long n, const uint32_t f[4][4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const long long ra = r0 + g, rb = r0 + g + 8;
#pragma unroll
    for (int kt = 0; kt < 4; kt++) {
        if (ra < n) {
            *reinterpret_cast<uint32_t *>(m + ra * 64 + 16 * kt + 2 * t) = f[kt][0];
            *reinterpret_cast<uint32_t *>(m + ra * 64 + 16 * kt + 8 + 2 * t) = f[kt][2];
        }
        if (rb < n) {
            *reinterpret_cast<uint32_t *>(m + rb * 64 + 16 * kt + 2 * t) = f[kt][1];
            *reinterpret_cast<uint32_t *>(m + rb * 64 + 16 * kt + 8 + 2 * t) = f[kt][3];
        }
    }
}

// acc += A (16 x 64, fragments) * W^T for a 64-input layer with `kOutTiles` n-tiles of 8 outputs
template <int kOutTiles>
__device__ __forceinline__ void layer64(float acc[][4], const uint32_t af[4][4], const uint16_t *ws) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    constexpr int stride = kHidden + kRowPad;
#pragma unroll
    for (int kt = 0; kt < 4; kt++) {
#pragma unroll
        for (int j = 0; j < kOutTiles; j++) {
            const uint16_t *br = ws + (8 * j + g) * stride + 16 * kt + 2 * t;
            mma(acc[j], af[kt], *reinterpret_cast<const uint32_t *>(br), *reinterpret_cast<const uint32_t *>(br + 8));
        }
    }
}

template <bool kTrain>
__global__ void __launch_bounds__(kThreads) k_mlp_forward(MlpArgs a) {
    extern __shared__ __align__(16) uint8_t smem[];
    const uint16_t *ws = reinterpret_cast<const uint16_t *>(smem);
    load_weights(smem, a.w);
    __syncthreads();
    const long long n = rows_of(a);
    const float *rec = a.rec + a.off * kRec;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    uint16_t *tile = reinterpret_cast<uint16_t *>(smem + kWeightBytes) + warp * 16 * kEncStride;
    const long long ntiles = (n + 15) / 16;
    for (long long ti = (long long)blockIdx.x * kWarps + warp; ti < ntiles; ti += (long long)gridDim.x * kWarps) {
        const long long r0 = ti * 16;
        {
            const int row = lane & 15, part = lane >> 4;
            __nv_bfloat16 *dst = reinterpret_cast<__nv_bfloat16 *>(tile + row * kEncStride);
            if (r0 + row < n) {
                encode_part(rec + (r0 + row) * kRec, a.enc, dst, part);
            } else {
                const int b = part == 0 ? 0 : 72, e = part == 0 ? 72 : kIn;
                for (int c = b; c < e; c++) dst[c] = __float2bfloat16_rn(0.0f);
            }
        }
        __syncwarp();
        if (kTrain) {
            // H_0: 16 rows x 160 bf16 = 16 x 20 vectors of 16 bytes
            for (int v = lane; v < 16 * 20; v += 32) {
                const int row = v / 20, col = (v % 20) * 8;
                if (r0 + row < n)
                    *reinterpret_cast<uint4 *>(a.h[0] + (r0 + row) * kIn + col) =
                        *reinterpret_cast<const uint4 *>(tile + row * kEncStride + col);
            }
        }
        float acc[8][4];
#pragma unroll
        for (int j = 0; j < 8; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
#pragma unroll
        for (int kt = 0; kt < kIn / 16; kt++) {
            const uint16_t *ar = tile + g * kEncStride + 16 * kt + 2 * t;
            uint32_t af[4];
            af[0] = *reinterpret_cast<const uint32_t *>(ar);
            af[1] = *reinterpret_cast<const uint32_t *>(ar + 8 * kEncStride);
            af[2] = *reinterpret_cast<const uint32_t *>(ar + 8);
            af[3] = *reinterpret_cast<const uint32_t *>(ar + 8 * kEncStride + 8);
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const uint16_t *br = ws + p_offset(0) + (8 * j + g) * (kIn + kRowPad) + 16 * kt + 2 * t;
                mma(acc[j], af, *reinterpret_cast<const uint32_t *>(br), *reinterpret_cast<const uint32_t *>(br + 8));
            }
        }
        uint32_t hf[4][4];
        relu_pack(acc, hf);
        if (kTrain) store_frag64(a.h[1], r0, n, hf);
#pragma unroll
        for (int l = 1; l < kLayers - 1; l++) {
#pragma unroll
            for (int j = 0; j < 8; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
            layer64<8>(acc, hf, ws + p_offset(l));
            relu_pack(acc, hf);
            if (kTrain) store_frag64(a.h[l + 1], r0, n, hf);
        }
        float out[1][4] = {{0.f, 0.f, 0.f, 0.f}};
        layer64<1>(out, hf, ws + p_offset(kLayers - 1));
        // out: (row g, cols 2t, 2t+1) and (row g + 8, cols 2t, 2t+1); columns 0..2 are RGB
        if (t < 2) {
#pragma unroll
            for (int half = 0; half < 2; half++) {
                const long long r = r0 + g + 8 * half;
                if (r >= n) continue;
#pragma unroll
                for (int e = 0; e < 2; e++) {
                    const int c = 2 * t + e;
                    if (c >= kOut) continue;
                    const float v = out[0][2 * half + e];
                    if (kTrain) a.y[r * 3 + c] = v;
                    else a.rgb[r * 3 + c] = expf(fminf(v, 20.0f));
                }
            }
        }
        __syncwarp();
    }
}

// dZ = dH * [H > 0] for an accumulator of 16 x 64 (H: row-major n x 64 BF16); stores dZ and
// returns it as A fragments
__device__ __forceinline__ void mask_store(float acc[8][4], const uint16_t *H, uint16_t *dz, long long r0, long long n,
                                           uint32_t za[4][4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const long long ra = r0 + g, rb = r0 + g + 8;
#pragma unroll
    for (int j = 0; j < 8; j++) {
        const uint32_t ha = ra < n ? *reinterpret_cast<const uint32_t *>(H + ra * 64 + 8 * j + 2 * t) : 0u;
        const uint32_t hb = rb < n ? *reinterpret_cast<const uint32_t *>(H + rb * 64 + 8 * j + 2 * t) : 0u;
        if (!bf16_positive(ha & 0xffffu)) acc[j][0] = 0.f;
        if (!bf16_positive(ha >> 16)) acc[j][1] = 0.f;
        if (!bf16_positive(hb & 0xffffu)) acc[j][2] = 0.f;
        if (!bf16_positive(hb >> 16)) acc[j][3] = 0.f;
    }
#pragma unroll
    for (int kt = 0; kt < 4; kt++) {
        za[kt][0] = pack2(acc[2 * kt][0], acc[2 * kt][1]);
        za[kt][1] = pack2(acc[2 * kt][2], acc[2 * kt][3]);
        za[kt][2] = pack2(acc[2 * kt + 1][0], acc[2 * kt + 1][1]);
        za[kt][3] = pack2(acc[2 * kt + 1][2], acc[2 * kt + 1][3]);
    }
    store_frag64(dz, r0, n, za);
}

// relative L2 loss sum_c (p - t)^2 / (p^2 + 0.01) with p = exp(y) (p not differentiated in the
// denominator); gradients scaled by 1 / rows
__global__ void __launch_bounds__(kThreads) k_mlp_backward(MlpArgs a) {
    extern __shared__ __align__(16) uint8_t smem[];
    const uint16_t *ws = reinterpret_cast<const uint16_t *>(smem);
    load_weights(smem, a.w);
    __syncthreads();
    const long long n = rows_of(a);
    if (n <= 0) return;
    const float inv_n = 1.0f / (float)n;
    const float *target = a.target + a.off * 3;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const long long ntiles = (n + 15) / 16;
    float loss = 0.0f;
    for (long long ti = (long long)blockIdx.x * kWarps + warp; ti < ntiles; ti += (long long)gridDim.x * kWarps) {
        const long long r0 = ti * 16;
        float dy[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
        for (int half = 0; half < 2; half++) {
            const long long r = r0 + g + 8 * half;
#pragma unroll
            for (int e = 0; e < 2; e++) {
                const int c = 2 * t + e;
                if (c >= kOut || r >= n) continue;
                const float yv = a.y[r * 3 + c];
                const float p = expf(fminf(yv, 20.0f));
                const float diff = p - target[r * 3 + c];
                const float den = p * p + 0.01f;
                loss += diff * diff / den;
                dy[2 * half + e] = yv < 20.0f ? 2.0f * diff / den * p * inv_n : 0.0f;
            }
        }
        uint32_t ya[4] = {pack2(dy[0], dy[1]), pack2(dy[2], dy[3]), 0u, 0u};
        {
            const long long ra = r0 + g, rb = r0 + g + 8;
            if (ra < n) *reinterpret_cast<uint32_t *>(a.dz[kLayers - 1] + ra * kOutPad + 2 * t) = ya[0];
            if (rb < n) *reinterpret_cast<uint32_t *>(a.dz[kLayers - 1] + rb * kOutPad + 2 * t) = ya[1];
        }
        // dH_5 = dY W_5: B[k = out][n = in] = W_5[out][in]; k rows 8..15 are zero
        float acc[8][4];
        const uint16_t *w5 = ws + p_offset(kLayers - 1);
        constexpr int stride = kHidden + kRowPad;
#pragma unroll
        for (int j = 0; j < 8; j++) {
            acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
            const uint32_t b0 = pack_u16(w5[(2 * t) * stride + 8 * j + g], w5[(2 * t + 1) * stride + 8 * j + g]);
            mma(acc[j], ya, b0, 0u);
        }
        uint32_t za[4][4];
        mask_store(acc, a.h[kLayers - 1], a.dz[kLayers - 2], r0, n, za);
#pragma unroll
        for (int l = kLayers - 2; l >= 1; l--) {
            const uint16_t *wl = ws + p_offset(l);
#pragma unroll
            for (int j = 0; j < 8; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
#pragma unroll
            for (int kt = 0; kt < 4; kt++) {
#pragma unroll
                for (int j = 0; j < 8; j++) {
                    const int col = 8 * j + g, k0 = 16 * kt + 2 * t;
                    const uint32_t b0 = pack_u16(wl[k0 * stride + col], wl[(k0 + 1) * stride + col]);
                    const uint32_t b1 = pack_u16(wl[(k0 + 8) * stride + col], wl[(k0 + 9) * stride + col]);
                    mma(acc[j], za[kt], b0, b1);
                }
            }
            mask_store(acc, a.h[l], a.dz[l - 1], r0, n, za);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
    if (lane == 0 && a.loss) atomicAdd(a.loss, loss * inv_n);
}

struct WgradArgs {
    const uint16_t *h[kLayers];
    const uint16_t *dz[kLayers];
    const int *n_dev;
    long long n_host, off, cap;
    float *partial;  // [chunk][kParams]
};

// Partial dW_l = dZ_l^T H_l over this CTA's chunk of kChunkRows rows. kInW = in width, kOutW =
// out width. The chunk's rows of dZ_l and H_l are copied into shared memory as they are (16-byte
// cp.async; rows padded by 16 bytes so that the eight row addresses of an ldmatrix fall in
// different banks), and ldmatrix .trans turns them into the fragments of dZ^T (the A operand) and
// of H read along its rows (the B operand): no transposing stores.
constexpr int wg_out_cols(int out_w) { return out_w < 16 ? 16 : out_w; }  // A tiles are 16 rows high
template <int kInW, int kOutW>
constexpr int wgrad_smem_bytes() {
    return kChunkRows * ((wg_out_cols(kOutW) + 8) + (kInW + 8)) * 2;
}

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(smem)),
                 "l"(gmem)
                 : "memory");
}
__device__ __forceinline__ void ldsm_x4_trans(uint32_t r[4], const void *smem_row) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"((uint32_t)__cvta_generic_to_shared(smem_row))
                 : "memory");
}

template <int kInW, int kOutW>
__device__ __forceinline__ void wgrad_layer(const WgradArgs &a, int l, long long n, uint16_t *sm) {
    constexpr int kOutCols = wg_out_cols(kOutW);
    constexpr int kZS = kOutCols + 8, kHS = kInW + 8;  // row strides (bf16) of the two tiles
    uint16_t *dzs = sm;                                 // [kChunkRows][kZS]: dZ rows
    uint16_t *hs = sm + kChunkRows * kZS;               // [kChunkRows][kHS]: H rows
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    constexpr int kNT = kInW / 8;
    static_assert(kNT % 2 == 0, "B fragments are loaded two n-tiles at a time");
    const long long c0 = (long long)blockIdx.x * kChunkRows;
    const long long c1 = c0 + kChunkRows < n ? c0 + kChunkRows : n;
    const uint16_t *H = a.h[l];  // the pass's activations start at row 0 of the scratch
    const uint16_t *DZ = a.dz[l];
    // stage: 16-byte pieces of each row; rows past the chunk's end and the output layer's columns
    // 8..15 are zero
    constexpr int kZP = kOutW / 8, kHP = kInW / 8;  // 16-byte pieces per row
    for (int i = threadIdx.x; i < kChunkRows * (kZP + kHP); i += blockDim.x) {
        const int r = i / (kZP + kHP), q = i % (kZP + kHP);
        const long long row = c0 + r;
        uint16_t *dst = q < kZP ? dzs + r * kZS + 8 * q : hs + r * kHS + 8 * (q - kZP);
        if (row < c1) {
            const uint16_t *src = q < kZP ? DZ + row * kOutW + 8 * q : H + row * kInW + 8 * (q - kZP);
            cp_async16(dst, src);
        } else {
            *reinterpret_cast<uint4 *>(dst) = make_uint4(0u, 0u, 0u, 0u);
        }
    }
    if (kOutCols > kOutW)
        for (int r = threadIdx.x; r < kChunkRows; r += blockDim.x)
            *reinterpret_cast<uint4 *>(dzs + r * kZS + kOutW) = make_uint4(0u, 0u, 0u, 0u);
    asm volatile("cp.async.wait_all;" ::: "memory");
    __syncthreads();
    if (warp * 16 >= kOutCols) return;  // no output rows for this warp
    float acc[kNT][4];
#pragma unroll
    for (int j = 0; j < kNT; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
    const int m0 = 16 * warp, qm = lane >> 3, qi = lane & 7;
#pragma unroll 2
    for (int k0 = 0; k0 < kChunkRows; k0 += 16) {
        // A = dZ^T (m = output, k = row): matrices (m0-7, k0-7), (m8-15, k0-7), (m0-7, k8-15), (m8-15, k8-15)
        uint32_t af[4];
        ldsm_x4_trans(af, dzs + (k0 + 8 * (qm >> 1) + qi) * kZS + m0 + 8 * (qm & 1));
#pragma unroll
        for (int j = 0; j < kNT; j += 2) {
            // B = H (k = row, n = input): n-tiles j and j + 1, rows k0-7 and k8-15 of each
            uint32_t bf[4];
            ldsm_x4_trans(bf, hs + (k0 + 8 * (qm & 1) + qi) * kHS + 8 * j + 8 * (qm >> 1));
            mma(acc[j], af, bf[0], bf[1]);
            mma(acc[j + 1], af, bf[2], bf[3]);
        }
    }
    float *P = a.partial + (size_t)blockIdx.x * kParams + w_offset(l);
    const int ra = m0 + g, rb = ra + 8;
#pragma unroll
    for (int j = 0; j < kNT; j++) {
        const int col = 8 * j + 2 * t;
        if (ra < kOutW) {
            P[ra * kInW + col] = acc[j][0];
            P[ra * kInW + col + 1] = acc[j][1];
        }
        if (rb < kOutW) {
            P[rb * kInW + col] = acc[j][2];
            P[rb * kInW + col + 1] = acc[j][3];
        }
    }
}

constexpr int kWgradSmem = wgrad_smem_bytes<kIn, kHidden>();  // the largest (layer 0)
static_assert(wgrad_smem_bytes<kHidden, kHidden>() <= kWgradSmem &&
                  wgrad_smem_bytes<kHidden, kOutPad>() <= kWgradSmem, "layer 0 needs the most");

__global__ void __launch_bounds__(kThreads) k_mlp_wgrad(WgradArgs a) {
    extern __shared__ __align__(16) uint16_t sm[];
    long long n = a.n_host;
    if (a.n_dev) {
        n = (long long)*a.n_dev - a.off;
        n = n < 0 ? 0 : (n > a.cap ? a.cap : n);
    }
    const int l = blockIdx.y;
    if (l == 0) wgrad_layer<kIn, kHidden>(a, 0, n, sm);
    else if (l < kLayers - 1) wgrad_layer<kHidden, kHidden>(a, l, n, sm);
    else wgrad_layer<kHidden, kOutPad>(a, l, n, sm);
}

struct AdamArgs {
    const float *partial;
    int chunks;  // partial rows to sum (chunks with no rows hold zeros)
    float *grad;  // optional: the summed gradient
    float *master, *m, *v, *ema;
    uint16_t *w_train, *w_ema;
    uint16_t *w_tc_train, *w_tc_ema;  // the same in the tcgen05 operand layout
    uint16_t *w_tcT_train;            // layers 1..5 in the transposed operand layout
    int *step;   // [0] device step counter, advanced by the last block; [1] blocks done
    const int *n_dev;
    long long n_host, off;
    float lr, beta1, beta2, eps, ema_f;
    int update;  // 0: only sum the gradient
};

__device__ __forceinline__ int padded_index(int i) {
    int l = 0;
    while (l + 1 < kLayers && i >= w_offset(l + 1)) l++;
    const int in = layer_in(l);
    const int local = i - w_offset(l);
    return p_offset(l) + (local / in) * (in + kRowPad) + local % in;
}

__device__ __forceinline__ void k_adam_body(const AdamArgs &a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kParams) return;
    long long n = a.n_host;
    if (a.n_dev) n = (long long)*a.n_dev - a.off;
    float g = 0.0f;
    for (int c = 0; c < a.chunks; c++) g += a.partial[(size_t)c * kParams + i];
    if (a.grad) a.grad[i] = g;
    if (!a.update || n <= 0) return;
    const int t = a.step[0] + 1;
    const float m = a.beta1 * a.m[i] + (1.0f - a.beta1) * g;
    const float v = a.beta2 * a.v[i] + (1.0f - a.beta2) * g * g;
    a.m[i] = m;
    a.v[i] = v;
    const float mh = m / (1.0f - powf(a.beta1, (float)t));
    const float vh = v / (1.0f - powf(a.beta2, (float)t));
    const float w = a.master[i] - a.lr * mh / (sqrtf(vh) + a.eps);
    a.master[i] = w;
    const float e = t == 1 ? w : a.ema_f * a.ema[i] + (1.0f - a.ema_f) * w;
    a.ema[i] = e;
    const int pi = padded_index(i);
    const __nv_bfloat16 wb = __float2bfloat16_rn(w), eb = __float2bfloat16_rn(e);
    a.w_train[pi] = *reinterpret_cast<const uint16_t *>(&wb);
    a.w_ema[pi] = *reinterpret_cast<const uint16_t *>(&eb);
    int l = 0;
    while (l + 1 < kLayers && i >= w_offset(l + 1)) l++;
    const int local = i - w_offset(l);
    const int ti = tc_index(l, local / layer_in(l), local % layer_in(l));
    a.w_tc_train[ti] = *reinterpret_cast<const uint16_t *>(&wb);
    a.w_tc_ema[ti] = *reinterpret_cast<const uint16_t *>(&eb);
    if (l >= 1) a.w_tcT_train[tcT_index(l, local % layer_in(l), local / layer_in(l))] = *reinterpret_cast<const uint16_t *>(&wb);
}

__global__ void k_adam(AdamArgs a) { k_adam_body(a); }

// k_adam with the step counter advanced by its last block to finish, once every block has read it
__global__ void k_adam_update(AdamArgs a) {
    k_adam_body(a);
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(a.step + 1, 1) == (int)gridDim.x - 1) {
            long long n = a.n_host;
            if (a.n_dev) n = (long long)*a.n_dev - a.off;
            if (n > 0) a.step[0] += 1;
            a.step[1] = 0;
            __threadfence();
        }
    }
}

}  // namespace nrc
}  // namespace tt

// ---- the cache object ----------------------------------------------------------------------------
using namespace tt;
using namespace tt::nrc;

struct tt_cache {
    tt_cache_params p{};
    int num_sms = 0;
    float *master = nullptr, *m = nullptr, *v = nullptr, *ema = nullptr, *grad = nullptr;
    uint16_t *w_train = nullptr, *w_ema = nullptr;
    uint16_t *w_tc_train = nullptr, *w_tc_ema = nullptr;  // the same in the tcgen05 operand layout
    uint16_t *w_tcT_train = nullptr;                        // layers 1..5 transposed (tcgen05 backward)
    unsigned *err = nullptr;                                // error word of the tcgen05 kernels
    int *step = nullptr;
    float *loss = nullptr;
    // training scratch for `p.batch` rows
    uint16_t *h[kLayers] = {};
    uint16_t *dz[kLayers] = {};
    float *y = nullptr;
    float *partial = nullptr;
    int chunks = 0;
    void *block = nullptr;  // one allocation for all of the above
};

namespace {

tt_status cuda_fail_c(cudaError_t e, const char *what) {
    return fail(TT_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define TT_CUDA_C(call)                                       \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return cuda_fail_c(e_, #call); \
    } while (0)

Encoding encoding_of(const tt_cache_params &p) {
    Encoding e;
    for (int i = 0; i < 3; i++) {
        e.lo[i] = p.bbox_lo[i];
        const float ext = p.bbox_hi[i] - p.bbox_lo[i];
        e.inv_ext[i] = ext > 0.0f ? 1.0f / ext : 1.0f;
    }
    return e;
}

int fwd_grid(const tt_cache *c, long long rows) {
    const long long tiles = (rows + 15) / 16;
    const long long blocks = (tiles + kWarps - 1) / kWarps;
    const long long cap = 2ll * c->num_sms;
    return (int)(blocks < 1 ? 1 : (blocks < cap ? blocks : cap));
}

// He-uniform initial weights from a PCG32 stream (the output layer scaled by 0.1, its padding 0)
void init_weights(uint32_t seed, std::vector<float> &w) {
    uint64_t state = 0x853c49e6748fea9bull ^ ((uint64_t)seed << 1), inc = 0xda3e39cb94b95bdbull;
    auto next = [&]() {
        const uint64_t old = state;
        state = old * 6364136223846793005ull + inc;
        const uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        const uint32_t rot = (uint32_t)(old >> 59u);
        const uint32_t r = (xs >> rot) | (xs << ((32u - rot) & 31u));
        return (float)(r >> 8) * (1.0f / 16777216.0f);
    };
    w.assign(kParams, 0.0f);
    for (int l = 0; l < kLayers; l++) {
        const int in = layer_in(l), out = layer_out(l);
        const float s = std::sqrt(6.0f / (float)in) * (l == kLayers - 1 ? 0.1f : 1.0f);
        for (int o = 0; o < out; o++)
            for (int k = 0; k < in; k++) {
                const float u = next();
                w[w_offset(l) + o * in + k] = (l == kLayers - 1 && o >= kOut) ? 0.0f : (2.0f * u - 1.0f) * s;
            }
    }
}

tt_status upload_weights(tt_cache *c, const std::vector<float> &w) {
    std::vector<uint16_t> pad(kPadded, 0);
    for (int l = 0; l < kLayers; l++) {
        const int in = layer_in(l), out = layer_out(l);
        for (int o = 0; o < out; o++)
            for (int k = 0; k < in; k++) {
                const __nv_bfloat16 b = __float2bfloat16_rn(w[w_offset(l) + o * in + k]);
                pad[p_offset(l) + o * (in + kRowPad) + k] = *reinterpret_cast<const uint16_t *>(&b);
            }
    }
    TT_CUDA_C(cudaMemcpy(c->master, w.data(), sizeof(float) * kParams, cudaMemcpyHostToDevice));
    TT_CUDA_C(cudaMemcpy(c->ema, w.data(), sizeof(float) * kParams, cudaMemcpyHostToDevice));
    TT_CUDA_C(cudaMemset(c->m, 0, sizeof(float) * kParams));
    TT_CUDA_C(cudaMemset(c->v, 0, sizeof(float) * kParams));
    TT_CUDA_C(cudaMemcpy(c->w_train, pad.data(), 2 * kPadded, cudaMemcpyHostToDevice));
    TT_CUDA_C(cudaMemcpy(c->w_ema, pad.data(), 2 * kPadded, cudaMemcpyHostToDevice));
    TT_CUDA_C(cudaMemset(c->step, 0, sizeof(int)));
    tc_relayout(c->master, c->w_tc_train, nullptr);
    tc_relayout(c->ema, c->w_tc_ema, nullptr);
    tcT_relayout(c->master, c->w_tcT_train, nullptr);
    TT_CUDA_C(cudaDeviceSynchronize());
    return TT_OK;
}

MlpArgs train_args(tt_cache *c, const float *rec, const float *target, long long n_host, const int *n_dev,
                   long long off, long long cap) {
    MlpArgs a;
    std::memset(&a, 0, sizeof(a));
    a.w = c->w_train;
    a.rec = rec;
    a.target = target;
    a.n_host = n_host;
    a.n_dev = n_dev;
    a.off = off;
    a.cap = cap;
    a.enc = encoding_of(c->p);
    a.y = c->y;
    for (int l = 0; l < kLayers; l++) {
        a.h[l] = c->h[l];
        a.dz[l] = c->dz[l];
    }
    a.loss = c->loss;
    return a;
}

// One forward + backward + weight gradient pass over rows [off, off + cap) of the buffer
// (device count n_dev, or n_host rows), then Adam (update = 1) or only the summed gradient.
tt_status train_pass(tt_cache *c, const float *rec, const float *target, long long n_host, const int *n_dev,
                     long long off, int update, cudaStream_t s) {
    const long long cap = c->p.batch;
    const long long rows = n_dev ? cap : (n_host - off < cap ? n_host - off : cap);
    MlpArgs a = train_args(c, rec, target, n_dev ? 0 : rows, n_dev, off, cap);
    if (!n_dev) a.off = 0, a.rec = rec + off * kRec, a.target = target + off * 3;
    int chunks = c->chunks;
    if (c->p.mma_kind == 0) {  // tcgen05 + TMEM: forward, backward, weight gradients
        TcTrainArgs t;
        std::memset(&t, 0, sizeof(t));
        t.w_tc = c->w_tc_train;
        t.w_tcT = c->w_tcT_train;
        t.rec = rec + off * kRec;  // the pass's first row
        t.target = target + off * 3;
        t.n_host = a.n_host;
        t.n_dev = n_dev;
        t.off = n_dev ? off : 0;  // rows = clamp(*n_dev - off, 0, cap), or n_host
        t.cap = cap;
        for (int i = 0; i < 3; i++) {
            t.lo[i] = a.enc.lo[i];
            t.inv_ext[i] = a.enc.inv_ext[i];
        }
        t.y = c->y;
        for (int l = 0; l < kLayers; l++) {
            t.h[l] = c->h[l];
            t.dz[l] = c->dz[l];
        }
        t.loss = c->loss;
        t.partial = c->partial;
        t.err = c->err;
        t.num_sms = c->num_sms;
        t.wait_cycles = c->p.wait_limit;
        const tt_status st = tc_train(t, s);
        if (st != TT_OK) return st;
        chunks = tc_wgrad_chunks(rows, c->num_sms);
    } else {  // mma.sync
        const int grid = fwd_grid(c, rows);
        k_mlp_forward<true><<<grid, kThreads, kFwdSmem, s>>>(a);
        k_mlp_backward<<<grid, kThreads, kWeightBytes, s>>>(a);
        WgradArgs w;
        std::memset(&w, 0, sizeof(w));
        for (int l = 0; l < kLayers; l++) {
            w.h[l] = c->h[l];
            w.dz[l] = c->dz[l];
        }
        w.n_dev = n_dev;  // rows = clamp(*n_dev - off, 0, cap), or n_host
        w.n_host = a.n_host;
        w.off = n_dev ? off : 0;
        w.cap = cap;
        w.partial = c->partial;
        k_mlp_wgrad<<<dim3(c->chunks, kLayers), kThreads, kWgradSmem, s>>>(w);
    }
    AdamArgs ad;
    std::memset(&ad, 0, sizeof(ad));
    ad.partial = c->partial;
    ad.chunks = chunks;
    ad.grad = c->grad;
    ad.master = c->master;
    ad.m = c->m;
    ad.v = c->v;
    ad.ema = c->ema;
    ad.w_train = c->w_train;
    ad.w_ema = c->w_ema;
    ad.w_tc_train = c->w_tc_train;
    ad.w_tc_ema = c->w_tc_ema;
    ad.w_tcT_train = c->w_tcT_train;
    ad.step = c->step;
    ad.n_dev = n_dev;
    ad.n_host = a.n_host;
    ad.off = n_dev ? off : 0;
    ad.lr = c->p.lr;
    ad.beta1 = c->p.beta1;
    ad.beta2 = c->p.beta2;
    ad.eps = c->p.eps;
    ad.ema_f = c->p.ema;
    ad.update = update;
    if (update) k_adam_update<<<(kParams + 255) / 256, 256, 0, s>>>(ad);  // also the tcgen05-layout copies
    else k_adam<<<(kParams + 255) / 256, 256, 0, s>>>(ad);
    TT_CUDA_C(cudaGetLastError());
    return TT_OK;
}

}  // namespace

namespace tt {
namespace nrc {

tt_status cache_infer_device(tt_cache *c, const float *rec, const int *n_dev, long long cap, float *rgb, int use_ema,
                             unsigned *err, cudaStream_t s) {
    if (c->p.mma_kind == 0) {
        const Encoding e = encoding_of(c->p);
        return tc_infer(use_ema ? c->w_tc_ema : c->w_tc_train, rec, 0, n_dev, cap, e.lo, e.inv_ext, rgb,
                        err ? err : c->err, c->num_sms, c->p.wait_limit, s);
    }
    MlpArgs a;
    std::memset(&a, 0, sizeof(a));
    a.w = use_ema ? c->w_ema : c->w_train;
    a.rec = rec;
    a.n_dev = n_dev;
    a.cap = cap;
    a.enc = encoding_of(c->p);
    a.rgb = rgb;
    k_mlp_forward<false><<<fwd_grid(c, cap), kThreads, kFwdSmem, s>>>(a);
    TT_CUDA_C(cudaGetLastError());
    return TT_OK;
}

tt_status cache_train_device(tt_cache *c, const float *rec, const float *target, const int *n_dev, cudaStream_t s) {
    for (int k = 0; k < c->p.steps; k++) {
        const tt_status st = train_pass(c, rec, target, 0, n_dev, (long long)k * c->p.batch, 1, s);
        if (st != TT_OK) return st;
    }
    return TT_OK;
}

const tt_cache_params &cache_params(const tt_cache *c) { return c->p; }

}  // namespace nrc
}  // namespace tt

extern "C" {

tt_status tt_cache_params_default(tt_cache_params *p) {
    if (!p) return fail(TT_ERR_INVALID, "null argument");
    std::memset(p, 0, sizeof(*p));
    p->lr = 1e-2f;
    p->beta1 = 0.9f;
    p->beta2 = 0.99f;
    p->eps = 1e-10f;
    p->ema = 0.95f;
    p->batch = 16384;
    p->steps = 4;
    p->train_paths = 65536;
    p->spread_c = 0.01f;
    p->seed = 1;
    p->use_ema = 1;
    p->mma_kind = 0;
    p->wait_limit = 0;
    for (int i = 0; i < 3; i++) {
        p->bbox_lo[i] = -1.0f;
        p->bbox_hi[i] = 1.0f;
    }
    return TT_OK;
}

tt_status tt_cache_create(const tt_cache_params *p, tt_cache **out) {
    if (!p || !out) return fail(TT_ERR_INVALID, "null argument");
    *out = nullptr;
    if (p->mma_kind < 0 || p->mma_kind > 1) return fail(TT_ERR_INVALID, "cache: mma_kind must be 0 or 1");
    if (p->batch < 16 || p->batch > (1 << 22) || p->steps < 1 || p->train_paths < 1 || p->train_paths > (1 << 24))
        return fail(TT_ERR_INVALID, "cache: batch must be in 16..2^22, steps >= 1, train_paths in 1..2^24");
    if (!(p->lr > 0.0f) || !(p->beta1 >= 0.0f && p->beta1 < 1.0f) || !(p->beta2 >= 0.0f && p->beta2 < 1.0f) ||
        !(p->ema >= 0.0f && p->ema < 1.0f))
        return fail(TT_ERR_INVALID, "cache: bad optimiser parameters");
    tt_cache *c = new tt_cache();
    c->p = *p;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_mlp_forward<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, kFwdSmem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_mlp_forward<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, kFwdSmem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_mlp_backward, cudaFuncAttributeMaxDynamicSharedMemorySize, kWeightBytes);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_mlp_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize, kWgradSmem);
    if (e != cudaSuccess) {
        delete c;
        return cuda_fail_c(e, "cache setup");
    }
    if (tc_setup() != TT_OK) {
        delete c;
        return TT_ERR_CUDA;
    }
    const size_t B = (size_t)p->batch;
    c->chunks = (int)((B + kChunkRows - 1) / kChunkRows);
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    std::vector<size_t> sizes = {4 * kParams, 4 * kParams, 4 * kParams, 4 * kParams, 4 * kParams, 2 * kPadded,
                                 2 * kPadded, 256, 256, 2 * B * kIn};
    for (int l = 1; l < kLayers; l++) sizes.push_back(2 * B * kHidden);  // H_1..H_5
    for (int l = 0; l < kLayers - 1; l++) sizes.push_back(2 * B * kHidden);  // dZ_0..dZ_4
    sizes.push_back(2 * B * kOutPad);                                       // dY
    sizes.push_back(4 * B * 3);                                             // y
    sizes.push_back(4 * (size_t)c->chunks * kParams);                       // partials
    sizes.push_back(2 * tc_weight_elems());                                 // operand-layout weights
    sizes.push_back(2 * tc_weight_elems());
    sizes.push_back(256);                                                   // error word
    sizes.push_back(2 * tcT_weight_elems());                                // transposed operand layout
    size_t total = 0;
    for (size_t s : sizes) total += al(s);
    e = cudaMalloc(&c->block, total);
    if (e != cudaSuccess) {
        delete c;
        return fail(TT_ERR_OOM, std::string("cache buffers: ") + cudaGetErrorString(e));
    }
    cudaMemset(c->block, 0, total);
    char *q = static_cast<char *>(c->block);
    size_t k = 0;
    auto take = [&]() {
        char *r = q;
        q += al(sizes[k++]);
        return r;
    };
    c->master = (float *)take();
    c->m = (float *)take();
    c->v = (float *)take();
    c->ema = (float *)take();
    c->grad = (float *)take();
    c->w_train = (uint16_t *)take();
    c->w_ema = (uint16_t *)take();
    c->step = (int *)take();
    c->loss = (float *)take();
    for (int l = 0; l < kLayers; l++) c->h[l] = (uint16_t *)take();
    for (int l = 0; l < kLayers; l++) c->dz[l] = (uint16_t *)take();
    c->y = (float *)take();
    c->partial = (float *)take();
    c->w_tc_train = (uint16_t *)take();
    c->w_tc_ema = (uint16_t *)take();
    c->err = (unsigned *)take();
    c->w_tcT_train = (uint16_t *)take();
    std::vector<float> w;
    init_weights(p->seed, w);
    const tt_status st = upload_weights(c, w);
    if (st != TT_OK) {
        tt_cache_free(c);
        return st;
    }
    *out = c;
    return TT_OK;
}

tt_status tt_cache_free(tt_cache *c) {
    if (!c) return TT_OK;
    if (c->block) cudaFree(c->block);
    delete c;
    return TT_OK;
}

tt_status tt_cache_param_count(int32_t *n) {
    if (!n) return fail(TT_ERR_INVALID, "null argument");
    *n = kParams;
    return TT_OK;
}

tt_status tt_cache_get_weights(const tt_cache *c, float *w, int32_t which) {
    if (!c || !w) return fail(TT_ERR_INVALID, "null argument");
    const float *src = which == 1 ? c->ema : (which == 2 ? c->grad : c->master);
    TT_CUDA_C(cudaMemcpy(w, src, sizeof(float) * kParams, cudaMemcpyDeviceToHost));
    return TT_OK;
}

tt_status tt_cache_set_weights(tt_cache *c, const float *w) {
    if (!c || !w) return fail(TT_ERR_INVALID, "null argument");
    std::vector<float> v(w, w + kParams);
    for (int l = 0; l < kLayers; l++)  // the padding rows of the output layer stay zero
        for (int o = kOut; o < layer_out(l) && l == kLayers - 1; o++)
            for (int k = 0; k < layer_in(l); k++) v[w_offset(l) + o * layer_in(l) + k] = 0.0f;
    return upload_weights(c, v);
}

tt_status tt_cache_encode(tt_cache *c, const float *d_records, int64_t n, void *d_encoded, void *stream) {
    if (!c || (n > 0 && (!d_records || !d_encoded))) return fail(TT_ERR_INVALID, "null argument");
    if (n < 0 || n > c->p.batch) return fail(TT_ERR_BOUNDS, "cache: n must be in 0..batch");
    if (n == 0) return TT_OK;
    MlpArgs a = train_args(c, d_records, nullptr, n, nullptr, 0, n);
    a.h[0] = static_cast<uint16_t *>(d_encoded);
    k_mlp_forward<true><<<fwd_grid(c, n), kThreads, kFwdSmem, (cudaStream_t)stream>>>(a);
    TT_CUDA_C(cudaGetLastError());
    return TT_OK;
}

tt_status tt_cache_infer(tt_cache *c, const float *d_records, int64_t n, float *d_rgb, int32_t use_ema,
                         void *stream) {
    if (!c || (n > 0 && (!d_records || !d_rgb))) return fail(TT_ERR_INVALID, "null argument");
    if (n <= 0) return n == 0 ? TT_OK : fail(TT_ERR_INVALID, "negative count");
    if (c->p.mma_kind == 0) {
        if (reinterpret_cast<uintptr_t>(d_records) & 15)
            return fail(TT_ERR_INVALID, "cache: records must be 16-byte aligned");
        const Encoding e = encoding_of(c->p);
        return tc_infer(use_ema ? c->w_tc_ema : c->w_tc_train, d_records, n, nullptr, 0, e.lo, e.inv_ext, d_rgb,
                        c->err, c->num_sms, c->p.wait_limit, (cudaStream_t)stream);
    }
    MlpArgs a;
    std::memset(&a, 0, sizeof(a));
    a.w = use_ema ? c->w_ema : c->w_train;
    a.rec = d_records;
    a.n_host = n;
    a.enc = encoding_of(c->p);
    a.rgb = d_rgb;
    k_mlp_forward<false><<<fwd_grid(c, n), kThreads, kFwdSmem, (cudaStream_t)stream>>>(a);
    TT_CUDA_C(cudaGetLastError());
    return TT_OK;
}

tt_status tt_cache_check(tt_cache *c, void *stream) {
    if (!c) return fail(TT_ERR_INVALID, "null cache");
    unsigned w = 0;
    TT_CUDA_C(cudaMemcpyAsync(&w, c->err, sizeof(w), cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    TT_CUDA_C(cudaStreamSynchronize((cudaStream_t)stream));
    if (w) {
        TT_CUDA_C(cudaMemset(c->err, 0, sizeof(w)));
        return fail(TT_ERR_TIMEOUT, "cache: a tensor-core wait ran out");
    }
    return TT_OK;
}

tt_status tt_cache_gradient(tt_cache *c, const float *d_records, const float *d_targets, int64_t n, float *h_grad,
                            float *h_loss, void *stream) {
    if (!c || !d_records || !d_targets || !h_grad) return fail(TT_ERR_INVALID, "null argument");
    if (n < 1 || n > c->p.batch) return fail(TT_ERR_BOUNDS, "cache: n must be in 1..batch");
    cudaStream_t s = (cudaStream_t)stream;
    TT_CUDA_C(cudaMemsetAsync(c->loss, 0, sizeof(float), s));
    TT_CUDA_C(cudaMemsetAsync(c->partial, 0, sizeof(float) * (size_t)c->chunks * kParams, s));
    tt_status st = train_pass(c, d_records, d_targets, n, nullptr, 0, 0, s);
    if (st != TT_OK) return st;
    TT_CUDA_C(cudaStreamSynchronize(s));
    TT_CUDA_C(cudaMemcpy(h_grad, c->grad, sizeof(float) * kParams, cudaMemcpyDeviceToHost));
    if (h_loss) TT_CUDA_C(cudaMemcpy(h_loss, c->loss, sizeof(float), cudaMemcpyDeviceToHost));
    return TT_OK;
}

tt_status tt_cache_train(tt_cache *c, const float *d_records, const float *d_targets, int64_t n, int32_t steps,
                         float *h_loss, void *stream) {
    if (!c || !d_records || !d_targets) return fail(TT_ERR_INVALID, "null argument");
    if (n < 1 || steps < 1) return fail(TT_ERR_INVALID, "cache: n and steps must be positive");
    cudaStream_t s = (cudaStream_t)stream;
    TT_CUDA_C(cudaMemsetAsync(c->loss, 0, sizeof(float), s));
    for (int k = 0; k < steps; k++) {
        const long long off = ((long long)k * c->p.batch) % n;
        // every partial that Adam sums is written by the weight-gradient kernel (zeros for chunks
        // without rows), so the partials need no clearing
        const tt_status st = train_pass(c, d_records, d_targets, n, nullptr, off, 1, s);
        if (st != TT_OK) return st;
    }
    if (h_loss) {
        TT_CUDA_C(cudaStreamSynchronize(s));
        TT_CUDA_C(cudaMemcpy(h_loss, c->loss, sizeof(float), cudaMemcpyDeviceToHost));
        *h_loss /= (float)steps;
    }
    return TT_OK;
}

tt_status tt_cache_steps(const tt_cache *c, int32_t *steps) {
    if (!c || !steps) return fail(TT_ERR_INVALID, "null argument");
    TT_CUDA_C(cudaMemcpy(steps, c->step, sizeof(int), cudaMemcpyDeviceToHost));
    return TT_OK;
}

}  // extern "C"
