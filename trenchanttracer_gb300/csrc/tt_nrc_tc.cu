// The radiance cache's inference on 5th-generation tensor cores: tcgen05.mma with the FP32
// accumulator in tensor memory (TMEM), operands in shared memory, weights and feature records
// brought in by bulk asynchronous copies (cp.async.bulk) that signal an mbarrier.
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
constexpr int kTcSmem = kTcGroups * (kABytes + kRecBufs * kRecBytes) + kTcWeightBytes + kTcBarBytes;
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

struct TcEncoding {
    float lo[3], inv_ext[3];
};

// Encoding values [32 f, 32 f + 32) of one row (tt_nrc.cuh) into ring slot S: four chunks of 8
// BF16 values, each one 16-byte store (the 32 rows of a warp write 512 contiguous bytes per
// chunk). f must be a compile-time constant after unrolling.
__device__ __forceinline__ void encode_fill(const EncInputs &in, const float *rec, __nv_bfloat16 *S, int r, int f) {
#pragma unroll
    for (int j = 0; j < kFillCols / 8; j++)
        *reinterpret_cast<uint4 *>(S + a_offset(r, 8 * j)) = enc_chunk(in, rec, f * (kFillCols / 8) + j);
}

// ReLU of this thread's 64 accumulator columns, rounded to BF16, into its row of the next A.
__device__ __forceinline__ void relu_to_operand(uint32_t lane_addr, __nv_bfloat16 *A, int r) {
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
    }
}

struct TcArgs {
    const uint16_t *w;  // weights in the operand layout (kTcWeights bf16)
    const float *rec;
    long long n_host;
    const int *n_dev;   // rows = min(*n_dev, cap) when set
    long long cap;
    TcEncoding enc;
    float *rgb;
    unsigned *err;
    long long wait_cycles;  // budget of the waits in the main path (the drain at exit keeps ~1 s)
};

__device__ __forceinline__ void group_sync(int group) {  // the 128 threads of one warpgroup
    asm volatile("bar.sync %0, 128;" ::"r"(1 + group) : "memory");
}

__global__ void __launch_bounds__(kTcThreads, 1) k_mlp_forward_tc(TcArgs a) {
    extern __shared__ __align__(128) uint8_t smem[];
    const int tid = threadIdx.x, group = tid >> 7, gt = tid & 127, warp_in_group = gt >> 5;
    __nv_bfloat16 *A = reinterpret_cast<__nv_bfloat16 *>(smem + group * kABytes);
    uint16_t *W = reinterpret_cast<uint16_t *>(smem + kTcGroups * kABytes);
    float *R = reinterpret_cast<float *>(smem + kTcGroups * kABytes + kTcWeightBytes) +
               (size_t)group * kRecBufs * kTcRows * kRec;  // this group's record buffers
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + kTcGroups * (kABytes + kRecBufs * kRecBytes) + kTcWeightBytes);
    uint64_t *bar_w = bars;                        // weights
    uint64_t *bar_rec = bars + 1 + 5 * group;      // [0] [1]: the group's record buffers
    uint64_t *bar_ring = bar_rec + 2;              // [0] [1]: the products that read each ring slot
    uint64_t *bar_mma = bar_rec + 4;               // the group's hidden and output layers
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 1 + 5 * kTcGroups);
    int *ok_w = reinterpret_cast<int *>(tmem_slot + 1);  // the weights arrived
    int *ok = ok_w + 1 + group;                          // this group's waits all ended
    static_assert(8 * (1 + 5 * kTcGroups) + 4 + 4 * (1 + kTcGroups) <= kTcBarBytes, "barrier block");

    long long n = a.n_host;
    if (a.n_dev) {
        n = *a.n_dev;
        n = n < 0 ? 0 : (n > a.cap ? a.cap : n);
    }
    const long long ntiles = (n + kTcRows - 1) / kTcRows;
    if ((long long)blockIdx.x * kTcGroups >= ntiles) return;  // uniform per block: nothing allocated yet

    if (tid == 0) {
        mbar_init(bar_w, 1);
        for (int g = 0; g < kTcGroups; g++) {
            for (int k = 0; k < 5; k++) mbar_init(bars + 1 + 5 * g + k, 1);
            ok_w[1 + g] = 1;
        }
        *ok_w = 1;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (tid < 32) tmem_alloc(tmem_slot, kTmemCols);
    // Asynchronous operations of this group, counted by its issuing thread (gt == 0): the k-th
    // completion of a barrier is awaited with parity k & 1, and whatever was issued and not yet
    // awaited is drained (bounded) before the block exits.
    int rec_issued[2] = {0, 0}, rec_done[2] = {0, 0}, ring_issued[2] = {0, 0}, ring_done[2] = {0, 0};
    int mma_issued = 0, mma_done = 0;
    const long long tstride = (long long)gridDim.x * kTcGroups;
    const long long first = (long long)blockIdx.x * kTcGroups + group;
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
                encode_fill(in, rec, S, gt, f);
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
        relu_to_operand(lane_addr, A, gt);  // the whole buffer: the ring is no longer read
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
                relu_to_operand(lane_addr, A, gt);
                fence_async_smem();
            } else {
                float v[16];
                tmem_ld16(lane_addr, v);
                tmem_wait_ld();
                if (gt < rows) {
                    float *o = a.rgb + (r0 + gt) * 3;
                    o[0] = expf(fminf(v[0], 20.0f));
                    o[1] = expf(fminf(v[1], 20.0f));
                    o[2] = expf(fminf(v[2], 20.0f));
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
    if (tid < 32) tmem_free(*tmem_slot, kTmemCols);
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

tt_status tc_setup() {
    const cudaError_t e =
        cudaFuncSetAttribute(k_mlp_forward_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
    if (e != cudaSuccess) return fail(TT_ERR_CUDA, std::string("tensor-core MLP setup: ") + cudaGetErrorString(e));
    return TT_OK;
}

size_t tc_weight_elems() { return kTcWeights; }

void tc_relayout(const float *w_f32, uint16_t *w_tc, cudaStream_t s) {
    k_tc_layout<<<(kTcWeights + 255) / 256, 256, 0, s>>>(w_f32, w_tc);
}

tt_status tc_infer(const uint16_t *w_tc, const float *rec, long long n_host, const int *n_dev, long long cap,
                   const float lo[3], const float inv_ext[3], float *rgb, unsigned *err, int num_sms,
                   long long wait_cycles, cudaStream_t s) {
    TcArgs a;
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
    const long long tiles = (rows + kTcRows - 1) / kTcRows;
    const long long want = (tiles + kTcGroups - 1) / kTcGroups;  // blocks, each with kTcGroups groups
    const int grid = (int)(want < 1 ? 1 : (want < num_sms ? want : num_sms));
    k_mlp_forward_tc<<<grid, kTcThreads, kTcSmem, s>>>(a);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(TT_ERR_CUDA, std::string("tensor-core MLP: ") + cudaGetErrorString(e));
    return TT_OK;
}

}  // namespace nrc
}  // namespace tt
