// The radiance cache's network on 5th-generation tensor cores: tcgen05.mma with the FP32
// accumulator in tensor memory (TMEM), operands in shared memory, weights and feature records
// brought in by bulk asynchronous copies (cp.async.bulk) that signal an mbarrier. Inference is
// described here; training (the same forward kernel storing each layer's input, a backward kernel
// and a weight-gradient kernel) further down.
//
// One CTA per SM, six warpgroups of 128 threads (kTcGroups) sharing one copy of the network's
// weights (55.3 KB, loaded once per CTA). Each warpgroup owns its own stream of tiles of 128 rows
// (row r = thread r of the group = TMEM lane r), its own 16 KB operand buffer, its own 64 TMEM
// columns and one record buffer (kRecBufs), so six tiles are in flight per SM and a tile's
// records arrive while the previous tile's later layers compute:
//   records  cp.async.bulk of the next tile's 128 x 64 B, issued once the current tile's records
//            are encoded
//   layer 0  the 160 encoded inputs go through the operand buffer as a ring of two 32-column
//            slots: each thread encodes its row's 32 BF16 values of one slot, one thread issues
//            that slot's two products (K = 16 each) and commits them to the slot's mbarrier, and
//            the next slot is encoded while they run; a slot is refilled once its products have
//            read it
//   layers   one thread of the group issues the layer's tcgen05.mma (M = 128, N = 64 or 16, K = 16
//            each) and a tcgen05.commit to the group's mbarrier; after the wait every warp of the
//            group reads its 32 TMEM lanes (tcgen05.ld 32x32b), applies ReLU, rounds to BF16 and
//            writes the next layer's A (the 64 hidden columns fill the whole buffer)
//   output   exp of the first three columns of the last layer
// A warpgroup synchronises on its own named barrier, so the groups advance independently.
//
// Operand layout: no swizzle, K-major, 8 x 16-byte core matrices. A (128 x K): core (m8, k8) at
// byte (k8 * 16 + m8) * 128, so the stride between 8-row groups (SBO) is 128 and between the two
// K halves of one instruction (LBO) 2048; a ring slot holds k8 = 0..3 of its 32 columns. Weights
// W_l (N x K): core (n8, k8) at (k8 * N/8 + n8) * 128 from the layer's base: SBO 128, LBO N/8 *
// 128. Shared memory holds the groups' operand buffers first, then the weights, the records and
// the barriers, so that every operand address the descriptors can form (with either of the two
// byte offsets applied along either dimension) lies inside the CTA's own allocation.
//
// Every wait is bounded (a clock budget of about a second): one thread waits, the outcome goes
// to all threads through shared memory and a block barrier, so a failure is uniform; it is
// reported in the error word, and the TMEM columns are freed on every path.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>

#include "tt_nrc.cuh"
#include "tt_nrc_tc.h"

namespace tt {
namespace nrc {

constexpr int kTcRows = 128;
constexpr int kTcGroups = 6;                         // warpgroups (tiles in flight) per CTA
constexpr int kTcThreads = 128 * kTcGroups;
constexpr int kTmemCols = 512;                       // 64 per group, allocated as a power of two
constexpr int kFillCols = 32;                        // encoded columns per ring slot (two K = 16 steps)
constexpr int kFills = kIn / kFillCols;              // 5 slot fills per tile
constexpr int kSlotBytes = kTcRows * kFillCols * 2;  // 8192
constexpr int kABytes = 2 * kSlotBytes;              // 16384: the ring, later the hidden activations
constexpr int kRecBytes = kTcRows * kRec * 4;        // 8192
constexpr int kRecBufs = 1;                          // record buffers per group
constexpr long long kWaitCycles = 2000000000ll;      // ~1 s at 2 GHz
constexpr unsigned kErrMlpWait = 8u;                 // error word bit: a tensor-core wait ran out
static_assert(kIn % kFillCols == 0 && kFillCols % 8 == 0, "whole encoding chunks per slot");
static_assert(kABytes == kTcRows * kHidden * 2, "the hidden activations fill the operand buffer");

constexpr int kTcWeightBytes = kTcWeights * 2;        // 55296
// weights barrier; per group 2 record, 2 ring-slot and 1 product barriers; TMEM slot; flags
constexpr int kTcBarBytes = 512;
// Shared memory and TMEM columns of a CTA of g warpgroups (inference: kTcGroups; training, whose
// batches are a few hundred tiles: one, so that the tiles spread over every SM).
__host__ __device__ constexpr int tc_smem(int g) {
    return g * (kABytes + kRecBufs * kRecBytes) + kTcWeightBytes + kTcBarBytes;
}
__host__ __device__ constexpr int tc_tmem_cols(int g) {
    return 64 * g <= 32 ? 32 : (64 * g <= 64 ? 64 : (64 * g <= 128 ? 128 : (64 * g <= 256 ? 256 : 512)));
}
constexpr int kTcSmem = tc_smem(kTcGroups);
static_assert(kTcSmem <= 232448, "fits the 227 KB a CTA may use");
static_assert(kTcWeightBytes % 16 == 0 && kABytes % 16 == 0 && kRecBytes % 16 == 0, "bulk copy sizes");
static_assert(kTmemCols >= 64 * kTcGroups, "64 accumulator columns per group");


// ---- PTX helpers ------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(saddr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait for the phase of the given parity (budget in clock cycles)
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, long long budget = kWaitCycles) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > budget) return false;
    return true;
}
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     saddr(dst)),
                 "l"(src), "r"(bytes), "r"(saddr(bar))
                 : "memory");
}
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t cols) {  // whole warp
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(slot)), "r"(cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t cols) {  // whole warp
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols) : "memory");
}

// shared-memory matrix descriptor: no swizzle, version 1 (bits 46-47), LBO / SBO in bytes
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}
// instruction descriptor, kind::f16: D = F32 (bits 4-5), A = B = BF16 (bits 7-9, 10-12),
// both K-major, N >> 3 at bit 17, M >> 4 at bit 24
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}
__device__ __forceinline__ void umma(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            dtmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(bar))
                 : "memory");
}
// 16 consecutive 32-bit TMEM columns of this thread's lane
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float v[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// ---- the A operand ----------------------------------------------------------------------------
__device__ __forceinline__ int a_offset(int r, int k) {  // bf16 element index in the A buffer
    return ((k >> 3) * 16 + (r >> 3)) * 64 + (r & 7) * 8 + (k & 7);
}
// bf16 index of element (r, k) of a K-major operand of R rows (R a multiple of 8)
__device__ __forceinline__ int kmajor_offset(int r, int k, int R) {
    return ((k >> 3) * (R >> 3) + (r >> 3)) * 64 + (r & 7) * 8 + (k & 7);
}

struct TcEncoding {
    float lo[3], inv_ext[3];
};

// Encoding values [32 f, 32 f + 32) of one row (tt_nrc.cuh) into ring slot S: four chunks of 8
// BF16 values, each one 16-byte store (the 32 rows of a warp write 512 contiguous bytes per
// chunk). f must be a compile-time constant after unrolling.
// gout (training): the row of H_0 in global memory, which gets the same values.
__device__ __forceinline__ void encode_fill(const EncInputs &in, const float *rec, __nv_bfloat16 *S, int r, int f,
                                            uint4 *gout) {
#pragma unroll
    for (int j = 0; j < kFillCols / 8; j++) {
        const uint4 v = enc_chunk(in, rec, f * (kFillCols / 8) + j);
        *reinterpret_cast<uint4 *>(S + a_offset(r, 8 * j)) = v;
        if (gout) gout[f * (kFillCols / 8) + j] = v;
    }
}

// ReLU of this thread's 64 accumulator columns, rounded to BF16, into its row of the next A (and,
// training, into the row of that layer's input H in global memory, gout).
__device__ __forceinline__ void relu_to_operand(uint32_t lane_addr, __nv_bfloat16 *A, int r, uint4 *gout = nullptr) {
#pragma unroll
    for (int c = 0; c < kHidden; c += 16) {
        float v[16];
        tmem_ld16(lane_addr + c, v);
        tmem_wait_ld();
        uint32_t w[8];
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const __nv_bfloat162 b = __floats2bfloat162_rn(fmaxf(v[2 * j], 0.f), fmaxf(v[2 * j + 1], 0.f));
            w[j] = *reinterpret_cast<const uint32_t *>(&b);
        }
        *reinterpret_cast<uint4 *>(A + a_offset(r, c)) = make_uint4(w[0], w[1], w[2], w[3]);
        *reinterpret_cast<uint4 *>(A + a_offset(r, c + 8)) = make_uint4(w[4], w[5], w[6], w[7]);
        if (gout) {
            gout[c / 8] = make_uint4(w[0], w[1], w[2], w[3]);
            gout[c / 8 + 1] = make_uint4(w[4], w[5], w[6], w[7]);
        }
    }
}

struct TcArgs {
    const uint16_t *w;  // weights in the operand layout (kTcWeights bf16)
    const float *rec;   // the call's first record
    long long n_host;
    const int *n_dev;   // rows = clamp(*n_dev - off, 0, cap) when set
    long long off, cap;
    TcEncoding enc;
    float *rgb;         // inference: radiance, 3 per row
    float *y;           // training: the raw outputs, 3 per row
    uint16_t *h[kLayers];  // training: each layer's input H_l (BF16 rows of 160 or 64)
    unsigned *err;
    long long wait_cycles;  // budget of the waits in the main path (the drain at exit keeps ~1 s)
};

__device__ __forceinline__ long long tc_rows(long long n_host, const int *n_dev, long long off, long long cap) {
    if (!n_dev) return n_host;
    const long long n = (long long)*n_dev - off;
    return n < 0 ? 0 : (n > cap ? cap : n);
}

__device__ __forceinline__ void group_sync(int group) {  // the 128 threads of one warpgroup
    asm volatile("bar.sync %0, 128;" ::"r"(1 + group) : "memory");
}

// kTrain: also writes every layer's input H_l and the raw outputs, for the backward pass.
template <bool kTrain, int kG>
__global__ void __launch_bounds__(128 * kG, 1) k_mlp_forward_tc(TcArgs a) {
    extern __shared__ __align__(128) uint8_t smem[];
    const int tid = threadIdx.x, group = tid >> 7, gt = tid & 127, warp_in_group = gt >> 5;
    __nv_bfloat16 *A = reinterpret_cast<__nv_bfloat16 *>(smem + group * kABytes);
    uint16_t *W = reinterpret_cast<uint16_t *>(smem + kG * kABytes);
    float *R = reinterpret_cast<float *>(smem + kG * kABytes + kTcWeightBytes) +
               (size_t)group * kRecBufs * kTcRows * kRec;  // this group's record buffers
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + kG * (kABytes + kRecBufs * kRecBytes) + kTcWeightBytes);
    uint64_t *bar_w = bars;                        // weights
    uint64_t *bar_rec = bars + 1 + 5 * group;      // [0] [1]: the group's record buffers
    uint64_t *bar_ring = bar_rec + 2;              // [0] [1]: the products that read each ring slot
    uint64_t *bar_mma = bar_rec + 4;               // the group's hidden and output layers
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 1 + 5 * kG);
    int *ok_w = reinterpret_cast<int *>(tmem_slot + 1);  // the weights arrived
    int *ok = ok_w + 1 + group;                          // this group's waits all ended
    static_assert(8 * (1 + 5 * kG) + 4 + 4 * (1 + kG) <= kTcBarBytes, "barrier block");

    const long long n = tc_rows(a.n_host, a.n_dev, a.off, a.cap);
    const long long ntiles = (n + kTcRows - 1) / kTcRows;
    if ((long long)blockIdx.x * kG >= ntiles) return;  // uniform per block: nothing allocated yet

    if (tid == 0) {
        mbar_init(bar_w, 1);
        for (int g = 0; g < kG; g++) {
            for (int k = 0; k < 5; k++) mbar_init(bars + 1 + 5 * g + k, 1);
            ok_w[1 + g] = 1;
        }
        *ok_w = 1;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (tid < 32) tmem_alloc(tmem_slot, tc_tmem_cols(kG));
    // Asynchronous operations of this group, counted by its issuing thread (gt == 0): the k-th
    // completion of a barrier is awaited with parity k & 1, and whatever was issued and not yet
    // awaited is drained (bounded) before the block exits.
    int rec_issued[2] = {0, 0}, rec_done[2] = {0, 0}, ring_issued[2] = {0, 0}, ring_done[2] = {0, 0};
    int mma_issued = 0, mma_done = 0;
    const long long tstride = (long long)gridDim.x * kG;
    const long long first = (long long)blockIdx.x * kG + group;
    if (gt == 0 && first < ntiles) {  // the group's first records, while the weights come in
        const long long r0 = first * kTcRows;
        const uint32_t bytes = (uint32_t)((n - r0) < kTcRows ? (n - r0) : kTcRows) * kRec * 4;
        mbar_expect_tx(bar_rec, bytes);
        bulk_load(R, a.rec + r0 * kRec, bytes, bar_rec);
        rec_issued[0]++;
    }
    bool w_pending = false;  // tid 0: the weights copy was issued and not seen complete
    if (tid == 0) {
        mbar_expect_tx(bar_w, kTcWeightBytes);
        bulk_load(W, a.w, kTcWeightBytes, bar_w);
        if (!mbar_wait(bar_w, 0, a.wait_cycles)) {
            *ok_w = 0;
            w_pending = true;
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot + (uint32_t)(group * 64);
    const uint32_t lane_addr = tmem + ((uint32_t)(warp_in_group * 32) << 16);
    // *ok_w is not written after the block barrier above; *ok is read by the group only right after
    // a group barrier that follows the issuing thread's write and precedes its next one
    const bool weights_ok = *ok_w != 0;
    if (!weights_ok && gt == 0) *ok = 0;
    group_sync(group);
    int buf = 0;
    for (long long tile = first; weights_ok && tile < ntiles; tile += tstride) {
        const long long r0 = tile * kTcRows;
        const int rows = (int)((n - r0) < kTcRows ? (n - r0) : kTcRows);
        const float *rec = R + buf * kTcRows * kRec + gt * kRec;
        if (gt == 0) {
            if (mbar_wait(bar_rec + buf, (uint32_t)(rec_done[buf] & 1), a.wait_cycles)) rec_done[buf]++;
            else *ok = 0;
        }
        group_sync(group);
        if (!*ok) break;
        // layer 0 through the ring: encode a slot, issue its products, encode the other slot meanwhile
        EncInputs in{};
        if (gt < rows) in = enc_inputs(rec, a.enc.lo, a.enc.inv_ext);
        bool failed = false;
#pragma unroll
        for (int f = 0; f < kFills; f++) {
            const int slot = f & 1;
            __nv_bfloat16 *S = A + slot * (kSlotBytes / 2);
            if (f >= 2) {  // the slot's previous products have read it
                if (gt == 0) {
                    if (mbar_wait(bar_ring + slot, (uint32_t)(ring_done[slot] & 1), a.wait_cycles)) ring_done[slot]++;
                    else *ok = 0;
                }
                group_sync(group);
                if (!*ok) {
                    failed = true;
                    break;
                }
            }
            if (gt < rows) {
                encode_fill(in, rec, S, gt, f, kTrain ? reinterpret_cast<uint4 *>(a.h[0] + (r0 + gt) * kIn) : nullptr);
            } else {
                for (int k = 0; k < kFillCols; k += 8)
                    *reinterpret_cast<uint4 *>(S + a_offset(gt, k)) = make_uint4(0u, 0u, 0u, 0u);
            }
            fence_async_smem();
            tc_fence_before();
            group_sync(group);  // the slot is encoded (after the last fill the records are free too)
            tc_fence_after();
            if (gt == 0) {
                const uint32_t s0 = saddr(S), b0 = saddr(W + tc_offset(0));
                constexpr int N = tc_out(0);
                for (int k = 0; k < kFillCols / 16; k++) {
                    const int ks = f * (kFillCols / 16) + k;  // K = 16 step of the layer
                    umma(tmem, sdesc(s0 + k * 2 * 2048, 2048, 128), sdesc(b0 + ks * 2 * (N / 8) * 128, (N / 8) * 128, 128),
                         idesc_bf16(kTcRows, N), ks > 0 ? 1u : 0u);
                }
                umma_commit(bar_ring + slot);
                ring_issued[slot]++;
            }
        }
        if (failed) break;
        if (gt == 0) {
            if (tile + tstride < ntiles) {  // the next tile's records (every encoding read is done)
                const int nb = (buf + 1) % kRecBufs;
                const long long nr0 = (tile + tstride) * kTcRows;
                const uint32_t bytes = (uint32_t)((n - nr0) < kTcRows ? (n - nr0) : kTcRows) * kRec * 4;
                mbar_expect_tx(bar_rec + nb, bytes);
                bulk_load(R + nb * kTcRows * kRec, a.rec + nr0 * kRec, bytes, bar_rec + nb);
                rec_issued[nb]++;
            }
            // layer 0 is complete when the last fill of each slot is
            for (int b = 0; b < 2; b++) {
                if (ring_done[b] < ring_issued[b]) {
                    if (mbar_wait(bar_ring + b, (uint32_t)(ring_done[b] & 1), a.wait_cycles)) ring_done[b]++;
                    else *ok = 0;
                }
            }
        }
        group_sync(group);
        tc_fence_after();
        if (!*ok) break;
        // the whole buffer: the ring is no longer read
        relu_to_operand(lane_addr, A, gt,
                        kTrain && gt < rows ? reinterpret_cast<uint4 *>(a.h[1] + (r0 + gt) * kHidden) : nullptr);
        fence_async_smem();
        tc_fence_before();
        group_sync(group);
        tc_fence_after();
        for (int l = 1; l < kLayers; l++) {
            const int K = layer_in(l), N = tc_out(l);
            if (gt == 0) {
                const uint32_t a0 = saddr(A), b0 = saddr(W + tc_offset(l));
                const uint32_t idesc = idesc_bf16(kTcRows, N);
                for (int s = 0; s < K / 16; s++)
                    umma(tmem, sdesc(a0 + s * 2 * 2048, 2048, 128), sdesc(b0 + s * 2 * (N / 8) * 128, (N / 8) * 128, 128),
                         idesc, s > 0 ? 1u : 0u);
                umma_commit(bar_mma);
                mma_issued++;
                if (mbar_wait(bar_mma, (uint32_t)(mma_done & 1), a.wait_cycles)) mma_done++;
                else *ok = 0;
            }
            group_sync(group);
            tc_fence_after();
            if (!*ok) break;
            if (l < kLayers - 1) {
                relu_to_operand(lane_addr, A, gt,
                                kTrain && gt < rows ? reinterpret_cast<uint4 *>(a.h[l + 1] + (r0 + gt) * kHidden) : nullptr);
                fence_async_smem();
            } else {
                float v[16];
                tmem_ld16(lane_addr, v);
                tmem_wait_ld();
                if (gt < rows) {
                    if (kTrain) {
                        float *o = a.y + (r0 + gt) * 3;
                        o[0] = v[0];
                        o[1] = v[1];
                        o[2] = v[2];
                    } else {
                        float *o = a.rgb + (r0 + gt) * 3;
                        o[0] = expf(fminf(v[0], 20.0f));
                        o[1] = expf(fminf(v[1], 20.0f));
                        o[2] = expf(fminf(v[2], 20.0f));
                    }
                }
            }
            tc_fence_before();
            group_sync(group);
            tc_fence_after();
        }
        buf = (buf + 1) % kRecBufs;
    }
    if (gt == 0) {
        if (!*ok) atomicOr(a.err, kErrMlpWait);
        // drain what this group issued and did not see complete (bounded again), before TMEM is freed
        for (int b = 0; b < 2; b++) {
            while (rec_done[b] < rec_issued[b] && mbar_wait(bar_rec + b, (uint32_t)(rec_done[b] & 1))) rec_done[b]++;
            while (ring_done[b] < ring_issued[b] && mbar_wait(bar_ring + b, (uint32_t)(ring_done[b] & 1)))
                ring_done[b]++;
        }
        while (mma_done < mma_issued && mbar_wait(bar_mma, (uint32_t)(mma_done & 1))) mma_done++;
    }
    if (tid == 0 && w_pending) mbar_wait(bar_w, 0);  // the weights copy, if its wait ran out
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (tid < 32) tmem_free(*tmem_slot, tc_tmem_cols(kG));
}

__global__ void k_tc_layout(const float *w, uint16_t *out) {
    // compact [out][in] FP32 weights -> operand layout BF16 (rows beyond the layer's outputs: 0)
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kTcWeights) return;
    int l = 0;
    while (l + 1 < kLayers && i >= tc_offset(l + 1)) l++;
    const int local = i - tc_offset(l);
    const int ng = tc_out(l) / 8;
    const int core = local / 64, within = local % 64;
    const int k8 = core / ng, n8 = core % ng;
    const int n = n8 * 8 + within / 8, k = k8 * 8 + within % 8;
    const float v = n < layer_out(l) ? w[w_offset(l) + n * layer_in(l) + k] : 0.0f;
    const __nv_bfloat16 b = __float2bfloat16_rn(v);
    out[i] = *reinterpret_cast<const uint16_t *>(&b);
}

__global__ void k_tcT_layout(const float *w, uint16_t *out) {
    // compact [out][in] FP32 weights of layers 1..5 -> the transposed operand layout BF16
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kTcTWeights) return;
    int l = 1;
    while (l + 1 < kLayers && i >= tcT_offset(l + 1)) l++;
    const int local = i - tcT_offset(l);
    const int ng = layer_in(l) / 8;
    const int core = local / 64, within = local % 64;
    const int k8 = core / ng, n8 = core % ng;
    const int n = n8 * 8 + within / 8, k = k8 * 8 + within % 8;  // n: input, k: output
    const float v = k < layer_out(l) ? w[w_offset(l) + k * layer_in(l) + n] : 0.0f;
    const __nv_bfloat16 b = __float2bfloat16_rn(v);
    out[i] = *reinterpret_cast<const uint16_t *>(&b);
}

// ---- training: backward pass ---------------------------------------------------------------------
// One warpgroup per tile of 128 rows (six per CTA, as in the forward kernel). Row r of the tile is
// thread r and TMEM lane r. The loss gradient of the row's three outputs (relative L2 loss
// sum_c (p - t)^2 / (p^2 + 0.01), p = exp(y), the denominator not differentiated, scaled by
// 1 / rows) is the K = 16 operand dZ_5 (columns 3..15 zero). Then for l = 5 .. 1 one product
// dH_l = dZ_l W_l (M = 128, N = 64, K = 16 or 64, B = the transposed weights), and the epilogue
// reads the row's 64 columns, keeps those where H_l > 0 (the forward pass's stored BF16 input of
// layer l, i.e. relu(Z_{l-1})), rounds to BF16 and writes dZ_{l-1} to global memory and, but for
// l = 1, into the operand buffer for the next product. Every dZ row is stored as the weight
// gradient needs it.
struct TcBackArgs {
    const uint16_t *wT;  // transposed operand-layout weights of layers 1..5 (kTcTWeights bf16)
    const float *y, *target;
    const uint16_t *h[kLayers];
    uint16_t *dz[kLayers];
    float *loss;  // loss sum over the rows / rows (atomic), or nullptr
    long long n_host;
    const int *n_dev;
    long long off, cap;
    unsigned *err;
    long long wait_cycles;
};
constexpr int kTcTWeightBytes = kTcTWeights * 2;  // 34816
__host__ __device__ constexpr int tc_back_smem(int g) { return g * kABytes + kTcTWeightBytes + kTcBarBytes; }
static_assert(tc_back_smem(kTcGroups) <= 232448 && kTcTWeightBytes % 16 == 0, "backward shared memory");
constexpr int kTrainGroups = 1;  // warpgroups per CTA of the training passes

__device__ __forceinline__ bool bf16_pos(uint32_t bits16) { return bits16 != 0u && !(bits16 & 0x8000u); }

// dZ = dH * [H > 0] for this thread's 64 accumulator columns; H: the row's 64 BF16 values in
// global memory (nullptr: a row past the end, all zero). Into the operand buffer (A != nullptr)
// and to gout (!= nullptr).
__device__ __forceinline__ void mask_to_operand(uint32_t lane_addr, const uint16_t *H, __nv_bfloat16 *A, int r,
                                                uint4 *gout) {
#pragma unroll
    for (int c = 0; c < kHidden; c += 16) {
        float v[16];
        tmem_ld16(lane_addr + c, v);
        tmem_wait_ld();
        uint4 hv[2] = {make_uint4(0u, 0u, 0u, 0u), make_uint4(0u, 0u, 0u, 0u)};
        if (H) {
            hv[0] = *reinterpret_cast<const uint4 *>(H + c);
            hv[1] = *reinterpret_cast<const uint4 *>(H + c + 8);
        }
        const uint32_t hw[8] = {hv[0].x, hv[0].y, hv[0].z, hv[0].w, hv[1].x, hv[1].y, hv[1].z, hv[1].w};
        uint32_t w[8];
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const float lo = bf16_pos(hw[j] & 0xffffu) ? v[2 * j] : 0.0f;
            const float hi = bf16_pos(hw[j] >> 16) ? v[2 * j + 1] : 0.0f;
            const __nv_bfloat162 b = __floats2bfloat162_rn(lo, hi);
            w[j] = *reinterpret_cast<const uint32_t *>(&b);
        }
        if (A) {
            *reinterpret_cast<uint4 *>(A + a_offset(r, c)) = make_uint4(w[0], w[1], w[2], w[3]);
            *reinterpret_cast<uint4 *>(A + a_offset(r, c + 8)) = make_uint4(w[4], w[5], w[6], w[7]);
        }
        if (gout) {
            gout[c / 8] = make_uint4(w[0], w[1], w[2], w[3]);
            gout[c / 8 + 1] = make_uint4(w[4], w[5], w[6], w[7]);
        }
    }
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat162 b = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t *>(&b);
}

template <int kG>
__global__ void __launch_bounds__(128 * kG, 1) k_mlp_backward_tc(TcBackArgs a) {
    extern __shared__ __align__(128) uint8_t smem[];
    const int tid = threadIdx.x, group = tid >> 7, gt = tid & 127, warp_in_group = gt >> 5;
    __nv_bfloat16 *A = reinterpret_cast<__nv_bfloat16 *>(smem + group * kABytes);
    uint16_t *W = reinterpret_cast<uint16_t *>(smem + kG * kABytes);
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + kG * kABytes + kTcTWeightBytes);
    uint64_t *bar_w = bars;                  // weights
    uint64_t *bar_mma = bars + 1 + group;    // the group's products
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 1 + kG);
    int *ok_w = reinterpret_cast<int *>(tmem_slot + 1);
    int *ok = ok_w + 1 + group;
    static_assert(8 * (1 + kG) + 4 + 4 * (1 + kG) <= kTcBarBytes, "barrier block");

    const long long n = tc_rows(a.n_host, a.n_dev, a.off, a.cap);
    const long long ntiles = (n + kTcRows - 1) / kTcRows;
    if ((long long)blockIdx.x * kG >= ntiles) return;  // uniform per block: nothing allocated yet
    if (tid == 0) {
        mbar_init(bar_w, 1);
        for (int g = 0; g < kG; g++) {
            mbar_init(bars + 1 + g, 1);
            ok_w[1 + g] = 1;
        }
        *ok_w = 1;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (tid < 32) tmem_alloc(tmem_slot, tc_tmem_cols(kG));
    bool w_pending = false;
    if (tid == 0) {
        mbar_expect_tx(bar_w, kTcTWeightBytes);
        bulk_load(W, a.wT, kTcTWeightBytes, bar_w);
        if (!mbar_wait(bar_w, 0, a.wait_cycles)) {
            *ok_w = 0;
            w_pending = true;
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot + (uint32_t)(group * 64);
    const uint32_t lane_addr = tmem + ((uint32_t)(warp_in_group * 32) << 16);
    const bool weights_ok = *ok_w != 0;
    if (!weights_ok && gt == 0) *ok = 0;
    group_sync(group);
    const float inv_n = 1.0f / (float)n;
    float loss = 0.0f;
    int mma_issued = 0, mma_done = 0;
    const long long tstride = (long long)gridDim.x * kG;
    for (long long tile = (long long)blockIdx.x * kG + group; weights_ok && tile < ntiles; tile += tstride) {
        const long long r0 = tile * kTcRows, row = r0 + gt;
        const bool own = row < n;
        float dy[3] = {0.f, 0.f, 0.f};
        if (own) {
#pragma unroll
            for (int c = 0; c < kOut; c++) {
                const float yv = a.y[row * 3 + c];
                const float p = expf(fminf(yv, 20.0f));
                const float diff = p - a.target[row * 3 + c];
                const float den = p * p + 0.01f;
                loss += diff * diff / den;
                dy[c] = yv < 20.0f ? 2.0f * diff / den * p * inv_n : 0.0f;
            }
        }
        const uint4 d5 = make_uint4(pack_bf16(dy[0], dy[1]), pack_bf16(dy[2], 0.0f), 0u, 0u);
        *reinterpret_cast<uint4 *>(A + a_offset(gt, 0)) = d5;
        *reinterpret_cast<uint4 *>(A + a_offset(gt, 8)) = make_uint4(0u, 0u, 0u, 0u);
        if (own) *reinterpret_cast<uint4 *>(a.dz[kLayers - 1] + row * kOutPad) = d5;
        fence_async_smem();
        tc_fence_before();
        group_sync(group);
        tc_fence_after();
        bool failed = false;
        for (int l = kLayers - 1; l >= 1; l--) {
            const int K = tc_out(l), N = layer_in(l);
            if (gt == 0) {
                const uint32_t a0 = saddr(A), b0 = saddr(W + tcT_offset(l));
                const uint32_t idesc = idesc_bf16(kTcRows, N);
                for (int s2 = 0; s2 < K / 16; s2++)
                    umma(tmem, sdesc(a0 + s2 * 2 * 2048, 2048, 128), sdesc(b0 + s2 * 2 * (N / 8) * 128, (N / 8) * 128, 128),
                         idesc, s2 > 0 ? 1u : 0u);
                umma_commit(bar_mma);
                mma_issued++;
                if (mbar_wait(bar_mma, (uint32_t)(mma_done & 1), a.wait_cycles)) mma_done++;
                else *ok = 0;
            }
            group_sync(group);
            tc_fence_after();
            if (!*ok) {
                failed = true;
                break;
            }
            mask_to_operand(lane_addr, own ? a.h[l] + row * kHidden : nullptr, l > 1 ? A : nullptr, gt,
                            own ? reinterpret_cast<uint4 *>(a.dz[l - 1] + row * kHidden) : nullptr);
            fence_async_smem();
            tc_fence_before();
            group_sync(group);
            tc_fence_after();
        }
        if (failed) break;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xffffffffu, loss, o);
    if ((tid & 31) == 0 && a.loss) atomicAdd(a.loss, loss * inv_n);
    if (gt == 0) {
        if (!*ok) atomicOr(a.err, kErrMlpWait);
        while (mma_done < mma_issued && mbar_wait(bar_mma, (uint32_t)(mma_done & 1))) mma_done++;
    }
    if (tid == 0 && w_pending) mbar_wait(bar_w, 0);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (tid < 32) tmem_free(*tmem_slot, tc_tmem_cols(kG));
}

// ---- training: weight gradients ------------------------------------------------------------------
// dW_l = dZ_l^T H_l over the batch's rows: one CTA per chunk of rows and layer, a product with
// M = 128 (the layer's outputs, zero beyond them), N = the layer's inputs (160 or 64) and K = the
// chunk's rows, 128 at a time. Both operands are MN-major (the transpose bits of the instruction
// descriptor): a core matrix is 8 consecutive rows of the batch x 16 bytes of consecutive columns,
// which is a 16-byte piece of each of 8 rows of the row-major H and dZ that the forward and
// backward passes wrote, so staging is 16-byte asynchronous copies (cp.async) with no
// transposition. Core (c8, k8) of an operand of R columns sits at c8 * 128 + k8 * (R / 8) * 128
// bytes: the descriptor's LBO is the stride between K-adjacent core matrices and SBO between
// column-adjacent ones, as in the K-major layout. The sums stay in TMEM across the chunk, and each
// CTA writes its partial gradient, which Adam sums over the chunks in chunk order (deterministic).
constexpr int kWgMinRows = 256;  // rows per chunk: at least this, more for large batches (tc_wgrad_rows)
constexpr int kWgABytes = kTcRows * kTcRows * 2;  // 128 outputs x 128 rows
constexpr int kWgBBytes = kIn * kTcRows * 2;      // up to 160 inputs x 128 rows
constexpr int kWgSmem = kWgABytes + kWgBBytes + 256;
// requested per CTA, so that at most two CTAs share an SM and their 256 TMEM columns each fit
constexpr int kWgSmemReq = 80 * 1024;
static_assert(kWgSmem <= kWgSmemReq && 3 * kWgSmemReq > 232448, "at most two CTAs per SM");
constexpr int kWgTmemCols = 256;
constexpr int kWgThreads = 512;  // staging threads; warps 0-3 also read the sums out of TMEM

struct TcWgradArgs {
    const uint16_t *h[kLayers];
    const uint16_t *dz[kLayers];
    int chunk_rows;  // a multiple of 128
    long long n_host;
    const int *n_dev;
    long long off, cap;
    float *partial;  // [chunk][kParams]
    unsigned *err;
    long long wait_cycles;
};

__global__ void __launch_bounds__(kWgThreads, 1) k_mlp_wgrad_tc(TcWgradArgs a) {
    extern __shared__ __align__(128) uint8_t smem[];
    uint16_t *As = reinterpret_cast<uint16_t *>(smem);
    uint16_t *Bs = reinterpret_cast<uint16_t *>(smem + kWgABytes);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + kWgABytes + kWgBBytes);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bar + 1);
    int *ok = reinterpret_cast<int *>(tmem_slot + 1);
    const int l = blockIdx.y, tid = threadIdx.x, warp = tid >> 5;
    const int in = layer_in(l), out = layer_out(l);
    const long long n = tc_rows(a.n_host, a.n_dev, a.off, a.cap);
    const long long c0 = (long long)blockIdx.x * a.chunk_rows, c1 = c0 + a.chunk_rows < n ? c0 + a.chunk_rows : n;
    float *P = a.partial + (size_t)blockIdx.x * kParams + w_offset(l);
    if (c0 >= n) {  // a chunk without rows adds nothing
        for (int i = tid; i < out * in; i += kWgThreads) P[i] = 0.0f;
        return;
    }
    if (tid == 0) {
        mbar_init(bar, 1);
        *ok = 1;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int i = tid; i < kWgABytes / 16; i += kWgThreads)  // A columns beyond the outputs stay zero
        reinterpret_cast<uint4 *>(As)[i] = make_uint4(0u, 0u, 0u, 0u);
    __syncthreads();
    if (tid < 32) tmem_alloc(tmem_slot, kWgTmemCols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    int issued = 0, done = 0;
    for (long long k0 = c0; k0 < c1; k0 += kTcRows) {
        const int nk = (int)(c1 - k0 < kTcRows ? c1 - k0 : kTcRows);  // rows past the chunk are zero
        // one 16-byte piece per item: row r of the tile, columns 8 p .. 8 p + 7 (consecutive items
        // are consecutive pieces of a row, so each row is read whole by neighbouring threads)
        const int pa = out / 8, pb = in / 8;
        for (int it = tid; it < kTcRows * (pa + pb); it += kWgThreads) {
            const bool is_a = it < kTcRows * pa;
            const int np = is_a ? pa : pb, j = is_a ? it : it - kTcRows * pa;
            const int r = j / np, p = j % np;
            const int R = is_a ? kTcRows : in;  // columns of the operand in shared memory
            uint8_t *dst = reinterpret_cast<uint8_t *>(is_a ? As : Bs) + p * 128 + (r >> 3) * (R / 8) * 128 + (r & 7) * 16;
            if (r < nk) {
                const uint16_t *src = (is_a ? a.dz[l] + (k0 + r) * out : a.h[l] + (k0 + r) * in) + 8 * p;
                asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(saddr(dst)), "l"(src) : "memory");
            } else {
                *reinterpret_cast<uint4 *>(dst) = make_uint4(0u, 0u, 0u, 0u);
            }
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
            const uint32_t a0 = saddr(As), b0 = saddr(Bs);
            const uint32_t idesc = idesc_bf16(kTcRows, in) | (1u << 15) | (1u << 16);  // A and B MN-major
            for (int s2 = 0; s2 < kTcRows / 16; s2++)
                umma(tmem, sdesc(a0 + s2 * 2 * (kTcRows / 8) * 128, (kTcRows / 8) * 128, 128),
                     sdesc(b0 + s2 * 2 * (in / 8) * 128, (in / 8) * 128, 128), idesc, (k0 > c0 || s2 > 0) ? 1u : 0u);
            umma_commit(bar);
            issued++;
            if (mbar_wait(bar, (uint32_t)(done & 1), a.wait_cycles)) done++;
            else *ok = 0;
        }
        __syncthreads();
        tc_fence_after();
        if (!*ok) break;  // the products may still read the operands: stage nothing more
    }
    if (*ok && warp < 4) {  // row m of the sums = TMEM lane m; warp w reads lanes 32w .. 32w + 31
        const int m = warp * 32 + (tid & 31);
        const uint32_t la = tmem + ((uint32_t)(warp * 32) << 16);
        for (int c = 0; c < in; c += 16) {
            float v[16];
            tmem_ld16(la + c, v);
            tmem_wait_ld();
            if (m < out)
#pragma unroll
                for (int j = 0; j < 16; j++) P[m * in + c + j] = v[j];
        }
    }
    if (tid == 0) {
        if (!*ok) atomicOr(a.err, kErrMlpWait);
        while (done < issued && mbar_wait(bar, (uint32_t)(done & 1))) done++;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (tid < 32) tmem_free(*tmem_slot, kWgTmemCols);
}

tt_status tc_setup() {
    cudaError_t e = cudaFuncSetAttribute(k_mlp_forward_tc<false, kTcGroups>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_mlp_forward_tc<true, kTrainGroups>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 tc_smem(kTrainGroups));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_mlp_forward_tc<true, kTcGroups>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 tc_smem(kTcGroups));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_mlp_backward_tc<kTrainGroups>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 tc_back_smem(kTrainGroups));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_mlp_backward_tc<kTcGroups>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 tc_back_smem(kTcGroups));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_mlp_wgrad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kWgSmemReq);
    if (e != cudaSuccess) return fail(TT_ERR_CUDA, std::string("tensor-core MLP setup: ") + cudaGetErrorString(e));
    return TT_OK;
}

size_t tc_weight_elems() { return kTcWeights; }
size_t tcT_weight_elems() { return kTcTWeights; }

void tc_relayout(const float *w_f32, uint16_t *w_tc, cudaStream_t s) {
    k_tc_layout<<<(kTcWeights + 255) / 256, 256, 0, s>>>(w_f32, w_tc);
}

void tcT_relayout(const float *w_f32, uint16_t *w_tcT, cudaStream_t s) {
    k_tcT_layout<<<(kTcTWeights + 255) / 256, 256, 0, s>>>(w_f32, w_tcT);
}

// rows per weight-gradient chunk: about two chunks per SM for each layer, 256 .. 4096 rows (each
// chunk's tiles run one after another, so more, shorter chunks finish sooner: 512-row chunks, one
// round of CTAs at 16K rows, took 28 us against 22)
static int tc_wgrad_rows(long long rows, int num_sms) {
    int c = kWgMinRows;
    while (c < 4096 && (long long)c * 2 * num_sms < rows) c *= 2;
    return c;
}

int tc_wgrad_chunks(long long rows, int num_sms) {
    const int c = tc_wgrad_rows(rows, num_sms);
    return (int)((rows + c - 1) / c);
}

// blocks of g groups for the tiles of `rows`, at most `per_sm` resident blocks per SM
static int tc_grid(long long rows, int g, int num_sms, int per_sm) {
    const long long tiles = (rows + kTcRows - 1) / kTcRows;
    const long long want = (tiles + g - 1) / g;
    const long long most = (long long)num_sms * per_sm;
    return (int)(want < 1 ? 1 : (want < most ? want : most));
}

tt_status tc_train(const TcTrainArgs &t, cudaStream_t s) {
    const long long rows = t.n_dev ? t.cap : t.n_host;
    const long long wc = t.wait_cycles > 0 ? t.wait_cycles : kWaitCycles;
    TcArgs f;
    std::memset(&f, 0, sizeof(f));
    f.w = t.w_tc;
    f.rec = t.rec;
    f.n_host = t.n_host;
    f.n_dev = t.n_dev;
    f.off = t.off;
    f.cap = t.cap;
    for (int i = 0; i < 3; i++) {
        f.enc.lo[i] = t.lo[i];
        f.enc.inv_ext[i] = t.inv_ext[i];
    }
    f.y = t.y;
    for (int l = 0; l < kLayers; l++) f.h[l] = t.h[l];
    f.err = t.err;
    f.wait_cycles = wc;
    // A batch of fewer tiles than six per SM: one group per block, so that the tiles spread over
    // every SM (two blocks fit an SM); larger ones: six groups per block, as inference runs.
    const bool wide = (rows + kTcRows - 1) / kTcRows >= (long long)kTcGroups * t.num_sms;
    const int grid = wide ? tc_grid(rows, kTcGroups, t.num_sms, 1) : tc_grid(rows, kTrainGroups, t.num_sms, 2);
    if (wide) k_mlp_forward_tc<true, kTcGroups><<<grid, 128 * kTcGroups, tc_smem(kTcGroups), s>>>(f);
    else k_mlp_forward_tc<true, kTrainGroups><<<grid, 128 * kTrainGroups, tc_smem(kTrainGroups), s>>>(f);
    TcBackArgs b;
    std::memset(&b, 0, sizeof(b));
    b.wT = t.w_tcT;
    b.y = t.y;
    b.target = t.target;
    for (int l = 0; l < kLayers; l++) {
        b.h[l] = t.h[l];
        b.dz[l] = t.dz[l];
    }
    b.loss = t.loss;
    b.n_host = t.n_host;
    b.n_dev = t.n_dev;
    b.off = t.off;
    b.cap = t.cap;
    b.err = t.err;
    b.wait_cycles = wc;
    if (wide) k_mlp_backward_tc<kTcGroups><<<grid, 128 * kTcGroups, tc_back_smem(kTcGroups), s>>>(b);
    else k_mlp_backward_tc<kTrainGroups><<<grid, 128 * kTrainGroups, tc_back_smem(kTrainGroups), s>>>(b);
    TcWgradArgs w;
    std::memset(&w, 0, sizeof(w));
    for (int l = 0; l < kLayers; l++) {
        w.h[l] = t.h[l];
        w.dz[l] = t.dz[l];
    }
    w.n_host = t.n_host;
    w.n_dev = t.n_dev;
    w.off = t.off;
    w.cap = t.cap;
    w.partial = t.partial;
    w.err = t.err;
    w.wait_cycles = wc;
    w.chunk_rows = tc_wgrad_rows(rows, t.num_sms);
    k_mlp_wgrad_tc<<<dim3(tc_wgrad_chunks(rows, t.num_sms), kLayers), kWgThreads, kWgSmemReq, s>>>(w);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(TT_ERR_CUDA, std::string("tensor-core MLP training: ") + cudaGetErrorString(e));
    return TT_OK;
}

tt_status tc_infer(const uint16_t *w_tc, const float *rec, long long n_host, const int *n_dev, long long cap,
                   const float lo[3], const float inv_ext[3], float *rgb, unsigned *err, int num_sms,
                   long long wait_cycles, cudaStream_t s) {
    TcArgs a;
    std::memset(&a, 0, sizeof(a));
    a.wait_cycles = wait_cycles > 0 ? wait_cycles : kWaitCycles;
    a.w = w_tc;
    a.rec = rec;
    a.n_host = n_host;
    a.n_dev = n_dev;
    a.cap = cap;
    for (int i = 0; i < 3; i++) {
        a.enc.lo[i] = lo[i];
        a.enc.inv_ext[i] = inv_ext[i];
    }
    a.rgb = rgb;
    a.err = err;
    const long long rows = n_dev ? cap : n_host;
    const int grid = tc_grid(rows, kTcGroups, num_sms, 1);
    k_mlp_forward_tc<false, kTcGroups><<<grid, kTcThreads, kTcSmem, s>>>(a);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(TT_ERR_CUDA, std::string("tensor-core MLP: ") + cudaGetErrorString(e));
    return TT_OK;
}

}  // namespace nrc
}  // namespace tt
