// Ray ordering before traversal (tt_reorder.cu); internal to libtt.so.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstddef>
#include <cstdint>

#include "../../include/tt.h"

namespace tt {

// the origin's cell (up to 13 bits: Morton-like code of a grid over the scene bounds whose bits go
// to the longest remaining cell side first; fewer bits for fewer rays, about 2^(origin bits + 9)
// rays each) above the direction's cell (8 bits: 16 x 16 octahedral grid)
constexpr int kOrderDirBits = 8;
constexpr int kOrderOriginBits = 13;
constexpr int kOrderMinOriginBits = 6;
constexpr int kOrderBits = kOrderDirBits + kOrderOriginBits;  // the largest key
static_assert(kOrderDirBits % 2 == 0 && kOrderBits <= 21, "direction cells square; counts for 2^21 keys at most");
// Fewer rays than this are traced in their own order: ordering them cannot pay for the scan of
// the 2^21 key counts.
constexpr int64_t kOrderMinRays = 1 << 15;
// Error-word bit: a sorted slot came out of range (the ray's hit is then left unwritten).
constexpr uint32_t kErrOrder = 4u;

// The origin grid: q_k = clamp((o_k - lo_k) * scale_k, 0, cells_k - 1), and bit j of q_k goes to
// the j-th lowest set bit of mask_k in the origin code.
struct OrderGrid {
    float3 lo, scale, qmax;
    unsigned mask[3];
    int origin_bits;
};

__host__ __device__ inline unsigned deposit(unsigned q, unsigned mask) {
    unsigned r = 0;
    for (unsigned m = mask; m; m &= m - 1u) {
        if (q & 1u) r |= m & (0u - m);
        q >>= 1;
    }
    return r;
}

__host__ __device__ inline unsigned order_key(const float4 r0, const float4 r1, const OrderGrid &g) {
    // direction: octahedral map (x, z over |x| + |y| + |z|, the lower hemisphere folded out),
    // kOrderDirBits / 2 bits per map axis, interleaved; non-finite or zero directions go to cell 0
    const float dx = r0.w, dy = r1.x, dz = r1.y;
    const float s = fabsf(dx) + fabsf(dy) + fabsf(dz);
    unsigned dcell = 0;
    if (s > 0.0f && s < INFINITY) {
        float u = dx / s, v = dz / s;
        if (dy < 0.0f) {
            const float fu = (1.0f - fabsf(v)) * (u < 0.0f ? -1.0f : 1.0f);
            v = (1.0f - fabsf(u)) * (v < 0.0f ? -1.0f : 1.0f);
            u = fu;
        }
        constexpr float kCells = (float)(1 << (kOrderDirBits / 2));  // per map axis
        constexpr unsigned kMask = (1u << kOrderDirBits) - 1u;
        const unsigned qu = (unsigned)fminf(fmaxf((u + 1.0f) * (0.5f * kCells), 0.0f), kCells - 1.0f);
        const unsigned qv = (unsigned)fminf(fmaxf((v + 1.0f) * (0.5f * kCells), 0.0f), kCells - 1.0f);
        dcell = deposit(qu, 0xAAAAAAAAu & kMask) | deposit(qv, 0x55555555u & kMask);
    }
    // origin (NaN coordinates clamp to cell 0: fmaxf returns the non-NaN operand)
    const unsigned qx = (unsigned)fminf(fmaxf((r0.x - g.lo.x) * g.scale.x, 0.0f), g.qmax.x);
    const unsigned qy = (unsigned)fminf(fmaxf((r0.y - g.lo.y) * g.scale.y, 0.0f), g.qmax.y);
    const unsigned qz = (unsigned)fminf(fmaxf((r0.z - g.lo.z) * g.scale.z, 0.0f), g.qmax.z);
    const unsigned ocell = deposit(qx, g.mask[0]) | deposit(qy, g.mask[1]) | deposit(qz, g.mask[2]);
    return (ocell << kOrderDirBits) | dcell;
}

// Origin bits of the key for n rays, and the grid they index (host).
int order_origin_bits(int64_t n);
OrderGrid order_grid(const float lo[3], const float hi[3], int origin_bits);

// Whether 64 warps of 32 consecutive rays (8 floats each, host memory), evenly spaced over the n,
// are mostly uniform in key (six lanes of each compared with its first): the host-side twin of
// the device probe, for callers that still hold the rays on the host.
bool host_rays_coherent(const float *rays, int64_t n, const float lo[3], const float hi[3]);

// Device scratch for ordering n rays: key + rank, sorted slot of each ray, sorted ray copy, sorted
// hit records (up to 24 B), 2^21 counts, the scan's chunk totals and the 256-byte state block
// (which must be zero when the scratch is new).
size_t reorder_scratch_bytes(int64_t n);
// Byte offset of the state block inside the scratch (to clear it on allocation).
size_t reorder_state_offset(int64_t n);

struct OrderOut {
    const int *pos;                   // sorted slot of each ray
    const float4 *sorted;             // 2 float4 per sorted slot
    void *sorted_hits;                // hit record per sorted slot, written by the trace kernel
    const unsigned long long *state;  // order_built(state): whether pos / sorted were built
    const int *src;                   // with_src: the ray slot of each sorted slot (in sorted_hits)
};

// Launches (on stream s) the ordering of n rays (or of min(*n_dev, n) when n_dev is set: a count
// that lives on the device) within scene bounds lo < hi per axis. The scratch holds at least
// reorder_scratch_bytes(n); its 256-byte state block sits at byte state_at, zeroed when the
// scratch was made and fixed for its life (reorder_state_offset of the size it was made for).
// Calls on one scratch must be ordered (one stream). Launches only, no allocation, so a call can
// be captured in a CUDA graph. Device-side errors go to *err as kErrOrder. with_src: the scatter
// also writes the inverse permutation (out->src, over the sorted_hits region), for a pass that
// reads the rays in sorted order and their other records by original slot.
tt_status reorder_rays(const float4 *rays, int64_t n, const int *n_dev, const float lo[3], const float hi[3],
                       void *scratch, size_t state_at, unsigned *err, cudaStream_t s, OrderOut *out, bool with_src = false);

// After the trace kernel wrote hits of hit_bytes (8 or 24) per sorted slot into out.sorted_hits:
// moves each ray's hit to hits[ray] (launch only; nothing to do when the order was not built).
tt_status reorder_unpermute(const OrderOut &out, int64_t n, void *hits, size_t hit_bytes, unsigned *err,
                            cudaStream_t s);

// Whether this call's rays were ordered: false when more than half of the sampled warps held 32
// equal keys (the rays are coherent already: camera rays share one origin cell and neighbouring
// pixels one direction cell) or fewer than kOrderMinRays rays came; they are then traced in their
// own order.
__device__ __forceinline__ bool order_built(const unsigned long long *state) { return state[3] == 1ull; }

}  // namespace tt
