// Ray ordering before traversal: a counting sort of the rays by a key of up to 21 bits. The key's
// high bits (13 for 4M rays, 2 fewer per quartering of the count, 6 at least) are the origin's
// cell in a grid over the scene bounds, in an order that halves the longest remaining cell side
// first (13 bits on a 16 x 1.8 x 16 terrain: 6, 2 and 5 per axis); its low 8 bits are the ray
// direction's cell in a 16 x 16 octahedral map of the sphere. Rays that leave the same region in
// nearly the same direction then share a warp, so their lanes fetch the same nodes and diverge
// less (on 4M cosine-distributed terrain rays the direction cell is worth 11 % of traversal time
// over the direction octant alone, and origin-major order 2.4 % over direction-major). Each ray's
// hit still goes to its own slot, and traversal has per-ray semantics, so the results do not
// depend on the order.
//
// Kernels, in stream order: (1) clear the key counts and probe every 16th warp of rays (a
// warp is uniform when its 32 keys are equal); when more than half of the sampled warps are
// uniform the rays are already coherent and every later kernel returns at once, leaving the rays
// in their own order. (2) Keys, and for each ray its rank among the rays of its key, from one
// atomic per group of equal keys in a warp (__match_any_sync). (3) Exclusive scan of the counts in
// 2048-entry chunks, chunk totals aside. (4) Every block scans the 1024 chunk totals in shared
// memory; each ray goes to slot chunk offset + count offset + rank, where the kernel writes the
// ray itself (the trace kernel then reads rays and writes hits contiguously, in sorted order); the
// slot is kept per ray, and after the trace a gather pass moves every hit to its own ray's place,
// reading the sorted hits (32 MB for 4M rays: L2-resident) at random and writing the output in
// order. Slots are bounds-checked. The order inside a key is whatever the atomics give; only the
// grouping matters. Plain launches on the caller's stream, so copies on other streams keep
// overlapping them.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <string>

#include "tt_internal.h"
#include "tt_reorder.h"

namespace tt {

constexpr int kOrderBlock = 256;
constexpr int kScanChunk = 2048;  // counts per scan chunk: 256 threads x 8
constexpr int kNumChunks = (1 << kOrderBits) / kScanChunk;
constexpr int kProbeStride = 16;  // the coherence probe looks at every 16th warp of rays
static_assert(kScanChunk == 8 * kOrderBlock && kNumChunks == 4 * kOrderBlock, "scan shapes");
static_assert(((1 << (kOrderDirBits + kOrderMinOriginBits)) / kScanChunk) % 4 == 0, "whole uint4 of chunk totals");

// State block (64-bit words): [0] sampled uniform warps, [1] sampled full warps, [2] probe blocks
// done, [3] the decision (1: ordered). The probe's last block to finish writes the decision and
// clears [0..2] for the next call, so calls need no other bookkeeping (and replay in a graph).
struct OrderArgs {
    const float4 *rays;
    int64_t n;         // rays, or the capacity when n_dev is set
    const int *n_dev;  // rays = min(*n_dev, n) when set
    OrderGrid g;
    uint2 *kr;         // per ray: key, rank within the key
    int *pos;          // per ray: its sorted slot
    int *src;          // per sorted slot: its ray (nullptr: not wanted)
    float4 *sorted;    // per sorted slot: the ray
    unsigned *counts;  // 2^key_bits
    unsigned *sums;    // chunk totals
    int key_bits;
    unsigned long long *state;
    unsigned *err;
};

__device__ __forceinline__ int64_t order_rays(const OrderArgs &a) {
    if (!a.n_dev) return a.n;
    const int64_t m = *a.n_dev;
    return m < 0 ? 0 : (m > a.n ? a.n : m);
}

// inclusive scan of one value per lane
__device__ __forceinline__ unsigned warp_scan(unsigned x) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    return x;
}

// Exclusive scan of one value per thread over the block; the block total to *total.
__device__ __forceinline__ unsigned block_exclusive_scan(unsigned x, unsigned *s_warp, unsigned *total) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const unsigned incl = warp_scan(x);
    if (lane == 31) s_warp[w] = incl;
    __syncthreads();
    if (w == 0) {
        const unsigned v = lane < kOrderBlock / 32 ? s_warp[lane] : 0u;
        const unsigned vi = warp_scan(v);
        if (lane < kOrderBlock / 32) s_warp[lane] = vi;
    }
    __syncthreads();
    const unsigned excl = incl - x + (w ? s_warp[w - 1] : 0u);
    *total = s_warp[kOrderBlock / 32 - 1];
    __syncthreads();  // s_warp is reused by the next call
    return excl;
}

// (1) clear the counts; probe; the last block decides
__global__ void __launch_bounds__(kOrderBlock) k_order_probe(OrderArgs a) {
    __shared__ unsigned s_probe[2];
    const int lane = threadIdx.x & 31;
    const int64_t tid = (int64_t)blockIdx.x * kOrderBlock + threadIdx.x;
    const int64_t nthreads = (int64_t)gridDim.x * kOrderBlock;
    const int64_t n = order_rays(a);
    for (int64_t j = tid; j < (1 << a.key_bits) / 4; j += nthreads)
        reinterpret_cast<uint4 *>(a.counts)[j] = make_uint4(0u, 0u, 0u, 0u);
    if (threadIdx.x < 2) s_probe[threadIdx.x] = 0u;
    __syncthreads();
    const int64_t warps = (n + 31) / 32;
    unsigned uniform = 0, full = 0;
    for (int64_t w = (tid >> 5) * kProbeStride; w < warps; w += (nthreads >> 5) * kProbeStride) {
        if (w * 32 + 32 > n) continue;  // only full warps count; w is the same in every lane
        const int64_t i = w * 32 + lane;
        const unsigned key = order_key(__ldg(a.rays + 2 * i), __ldg(a.rays + 2 * i + 1), a.g);
        full++;
        if (__match_any_sync(0xffffffffu, key) == 0xffffffffu) uniform++;
    }
    if (lane == 0 && full) {
        atomicAdd(&s_probe[0], uniform);
        atomicAdd(&s_probe[1], full);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (s_probe[1]) {
            atomicAdd(a.state + 0, (unsigned long long)s_probe[0]);
            atomicAdd(a.state + 1, (unsigned long long)s_probe[1]);
        }
        __threadfence();
        if (atomicAdd(a.state + 2, 1ull) == (unsigned long long)gridDim.x - 1) {  // every block's counts are in
            const unsigned long long u = atomicAdd(a.state + 0, 0ull), f = atomicAdd(a.state + 1, 0ull);
            // ordered unless mostly uniform; fewer than kOrderMinRays stay in their own order
            a.state[3] = (f > 0 && 2 * u <= f && n >= kOrderMinRays) ? 1ull : 0ull;
            a.state[0] = 0ull;
            a.state[1] = 0ull;
            a.state[2] = 0ull;
            __threadfence();
        }
    }
}

// (2) keys and ranks
__global__ void __launch_bounds__(kOrderBlock) k_order_keys(OrderArgs a) {
    if (!order_built(a.state)) return;
    const int lane = threadIdx.x & 31;
    const int64_t nthreads = (int64_t)gridDim.x * kOrderBlock;
    const int64_t n = order_rays(a);
    for (int64_t base = ((int64_t)blockIdx.x * kOrderBlock + threadIdx.x) & ~int64_t(31); base < n;
         base += nthreads) {
        const int64_t i = base + lane;
        const bool valid = i < n;
        unsigned key = 0xffffffffu;  // no real key has bit 31 set
        if (valid) key = order_key(__ldg(a.rays + 2 * i), __ldg(a.rays + 2 * i + 1), a.g);
        const unsigned peers = __match_any_sync(0xffffffffu, key);
        const int leader = __ffs(peers) - 1;
        unsigned first = 0;
        if (valid && lane == leader) first = atomicAdd(a.counts + key, (unsigned)__popc(peers));
        first = __shfl_sync(0xffffffffu, first, leader);
        if (valid) a.kr[i] = make_uint2(key, first + __popc(peers & ((1u << lane) - 1u)));
    }
}

// (3) exclusive scan of each chunk of counts (one chunk per block); chunk totals to sums
__global__ void __launch_bounds__(kOrderBlock) k_order_scan(OrderArgs a) {
    if (!order_built(a.state)) return;
    __shared__ unsigned s_warp[kOrderBlock / 32];
    uint4 *blk = reinterpret_cast<uint4 *>(a.counts + (size_t)blockIdx.x * kScanChunk);
    const uint4 v0 = blk[2 * threadIdx.x], v1 = blk[2 * threadIdx.x + 1];
    const unsigned x[8] = {v0.x, v0.y, v0.z, v0.w, v1.x, v1.y, v1.z, v1.w};
    unsigned t = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) t += x[k];
    unsigned total;
    unsigned run = block_exclusive_scan(t, s_warp, &total);
    unsigned o[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
        o[k] = run;
        run += x[k];
    }
    blk[2 * threadIdx.x] = make_uint4(o[0], o[1], o[2], o[3]);
    blk[2 * threadIdx.x + 1] = make_uint4(o[4], o[5], o[6], o[7]);
    if (threadIdx.x == 0) a.sums[blockIdx.x] = total;
}

// (4) chunk offsets (every block), then each ray and its slot
__global__ void __launch_bounds__(kOrderBlock) k_order_scatter(OrderArgs a) {
    if (!order_built(a.state)) return;
    __shared__ unsigned s_warp[kOrderBlock / 32];
    __shared__ unsigned s_prefix[kNumChunks];
    {
        const int nchunks = (1 << a.key_bits) / kScanChunk;
        const uint4 v = 4 * (int)threadIdx.x < nchunks ? reinterpret_cast<const uint4 *>(a.sums)[threadIdx.x]
                                                     : make_uint4(0u, 0u, 0u, 0u);
        unsigned total;
        unsigned run = block_exclusive_scan(v.x + v.y + v.z + v.w, s_warp, &total);
        s_prefix[4 * threadIdx.x] = run;
        run += v.x;
        s_prefix[4 * threadIdx.x + 1] = run;
        run += v.y;
        s_prefix[4 * threadIdx.x + 2] = run;
        run += v.z;
        s_prefix[4 * threadIdx.x + 3] = run;
    }
    __syncthreads();
    unsigned bad = 0;
    const int64_t n = order_rays(a);
    for (int64_t i = (int64_t)blockIdx.x * kOrderBlock + threadIdx.x; i < n; i += (int64_t)gridDim.x * kOrderBlock) {
        const uint2 kr = a.kr[i];
        if (kr.x >= (1u << a.key_bits)) {
            a.pos[i] = -1;
            bad = 1;
            continue;
        }
        const uint64_t pos = (uint64_t)s_prefix[kr.x / kScanChunk] + a.counts[kr.x] + kr.y;
        if (pos < (uint64_t)n) {
            a.sorted[2 * pos] = __ldg(a.rays + 2 * i);
            a.sorted[2 * pos + 1] = __ldg(a.rays + 2 * i + 1);
            a.pos[i] = (int)pos;
            if (a.src) a.src[pos] = (int)i;
        } else {
            a.pos[i] = -1;
            bad = 1;
        }
    }
    if (bad) atomicOr(a.err, kErrOrder);
}

// Origin bits by axis: each of the kOrderOriginBits bits, from the most significant down, halves
// the axis whose cell side is then the longest (ties to the lower axis); an axis without a
// positive finite extent gets none.
OrderGrid order_grid(const float lo[3], const float hi[3], int origin_bits) {
    OrderGrid g;
    g.origin_bits = origin_bits;
    double side[3];
    int bits[3] = {0, 0, 0};
    int axis_of[kOrderOriginBits];
    for (int k = 0; k < 3; k++) {
        const double e = (double)hi[k] - (double)lo[k];
        side[k] = (std::isfinite(e) && e > 0.0) ? e : 0.0;
    }
    for (int b = 0; b < origin_bits; b++) {
        int best = 0;
        for (int k = 1; k < 3; k++)
            if (side[k] > side[best]) best = k;
        axis_of[b] = best;
        bits[best]++;
        side[best] *= 0.5;
    }
    // an axis's first assignment is its most significant bit, so its bits fill its mask from the top
    for (int k = 0; k < 3; k++) g.mask[k] = 0;
    for (int b = 0; b < origin_bits; b++) g.mask[axis_of[b]] |= 1u << (origin_bits - 1 - b);
    float scale[3], qmax[3];
    for (int k = 0; k < 3; k++) {
        const double e = (double)hi[k] - (double)lo[k];
        const double cells = (double)(1u << bits[k]);
        scale[k] = (bits[k] > 0) ? (float)(cells / e) : 0.0f;
        qmax[k] = (float)(cells - 1.0);
    }
    g.lo = make_float3(lo[0], lo[1], lo[2]);
    g.scale = make_float3(scale[0], scale[1], scale[2]);
    g.qmax = make_float3(qmax[0], qmax[1], qmax[2]);
    return g;
}

int order_origin_bits(int64_t n) {
    int ob = kOrderOriginBits;  // 13 at 2^22 rays and above, 2 fewer per quartering
    while (ob > kOrderMinOriginBits && ((int64_t)1 << (ob + 9)) > n) ob -= 2;
    return ob < kOrderMinOriginBits ? kOrderMinOriginBits : ob;
}

bool host_rays_coherent(const float *rays, int64_t n, const float lo[3], const float hi[3]) {
    const int64_t warps = n / 32;
    if (warps <= 0) return true;
    const OrderGrid g = order_grid(lo, hi, order_origin_bits(n));
    const int64_t samples = warps < 64 ? warps : 64;
    int uniform = 0;
    for (int64_t k = 0; k < samples; k++) {
        const float *w = rays + 8 * 32 * (k * warps / samples);
        auto key = [&](int lane) {
            const float *r = w + 8 * lane;
            return order_key(make_float4(r[0], r[1], r[2], r[3]), make_float4(r[4], r[5], r[6], r[7]), g);
        };
        // lanes 1, 7, 13, 19, 25 and 31 against lane 0: enough to choose a schedule
        const unsigned k0 = key(0);
        int lane = 1;
        while (lane < 32 && key(lane) == k0) lane += 6;
        uniform += lane >= 32;
    }
    return 2 * uniform > samples;
}

static size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

size_t reorder_state_offset(int64_t n) {
    return al256(8ull * n) + al256(4ull * n) + al256(32ull * n) + al256(24ull * n) + al256(4ull << kOrderBits) +
           al256(4ull * kNumChunks);
}

size_t reorder_scratch_bytes(int64_t n) { return reorder_state_offset(n) + 256; }

static std::atomic<int> g_order_sms[64];  // SMs per device (0 = not yet known)

tt_status reorder_rays(const float4 *rays, int64_t n, const int *n_dev, const float lo[3], const float hi[3],
                       void *scratch, size_t state_at, unsigned *err, cudaStream_t s, OrderOut *out, bool with_src) {
    if (n <= 0 || n >= ((int64_t)1 << 31)) return fail(TT_ERR_INVALID, "ray ordering: n must be in 1..2^31-1");
    if (state_at < reorder_state_offset(n) || (state_at & 255))
        return fail(TT_ERR_INVALID, "ray ordering: scratch too small for this many rays");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(TT_ERR_CUDA, std::string("ray ordering: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= 64) return fail(TT_ERR_INVALID, "ray ordering: device ordinal out of range");
    int sms = g_order_sms[dev].load();
    if (sms <= 0) {
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return fail(TT_ERR_CUDA, std::string("ray ordering: ") + cudaGetErrorString(e));
        g_order_sms[dev].store(sms);
    }
    char *p = static_cast<char *>(scratch);
    OrderArgs a;
    a.rays = rays;
    a.n = n;
    a.n_dev = n_dev;
    const int ob = order_origin_bits(n);
    a.g = order_grid(lo, hi, ob);
    a.key_bits = kOrderDirBits + ob;
    a.kr = reinterpret_cast<uint2 *>(p);
    p += al256(8ull * n);
    a.pos = reinterpret_cast<int *>(p);
    p += al256(4ull * n);
    a.sorted = reinterpret_cast<float4 *>(p);
    p += al256(32ull * n);
    void *sorted_hits = p;
    a.src = with_src ? static_cast<int *>(sorted_hits) : nullptr;
    p += al256(24ull * n);
    a.counts = reinterpret_cast<unsigned *>(p);
    p += al256(4ull << kOrderBits);
    a.sums = reinterpret_cast<unsigned *>(p);
    a.state = reinterpret_cast<unsigned long long *>(static_cast<char *>(scratch) + state_at);
    a.err = err;
    const int64_t want = (n + kOrderBlock - 1) / kOrderBlock;
    const unsigned grid = (unsigned)(want < (int64_t)sms * 8 ? want : (int64_t)sms * 8);
    k_order_probe<<<(unsigned)sms * 4, kOrderBlock, 0, s>>>(a);
    k_order_keys<<<grid, kOrderBlock, 0, s>>>(a);
    k_order_scan<<<(1u << a.key_bits) / kScanChunk, kOrderBlock, 0, s>>>(a);
    k_order_scatter<<<grid, kOrderBlock, 0, s>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(TT_ERR_CUDA, std::string("ray ordering: ") + cudaGetErrorString(e));
    out->pos = a.pos;
    out->sorted = a.sorted;
    out->sorted_hits = sorted_hits;
    out->state = a.state;
    out->src = a.src;
    return TT_OK;
}

// hits[i] = sorted_hits[pos[i]], one record of Rec per ray
template <typename Rec>
__global__ void __launch_bounds__(256) k_order_unpermute(Rec *hits, const Rec *sorted_hits, const int *pos, int64_t n,
                                                         const unsigned long long *state, unsigned *err) {
    if (!order_built(state)) return;
    unsigned bad = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int p = __ldcs(pos + i);
        if ((uint64_t)(int64_t)p < (uint64_t)n) hits[i] = sorted_hits[p];
        else bad = 1;
    }
    if (bad) atomicOr(err, kErrOrder);
}

struct HitExtRec {  // tt_hit_ext as three 8-byte words
    uint2 w[3];
};

tt_status reorder_unpermute(const OrderOut &out, int64_t n, void *hits, size_t hit_bytes, unsigned *err,
                            cudaStream_t s) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(TT_ERR_CUDA, std::string("ray ordering: ") + cudaGetErrorString(e));
    const int sms = (dev >= 0 && dev < 64) ? g_order_sms[dev].load() : 0;
    const int64_t want = (n + 255) / 256;
    const int64_t cap = (int64_t)(sms > 0 ? sms : 132) * 8;
    const unsigned grid = (unsigned)(want < cap ? want : cap);
    if (hit_bytes == 8)
        k_order_unpermute<uint2><<<grid, 256, 0, s>>>(static_cast<uint2 *>(hits),
                                                       static_cast<const uint2 *>(out.sorted_hits), out.pos, n,
                                                       out.state, err);
    else if (hit_bytes == 24)
        k_order_unpermute<HitExtRec><<<grid, 256, 0, s>>>(static_cast<HitExtRec *>(hits),
                                                           static_cast<const HitExtRec *>(out.sorted_hits), out.pos,
                                                           n, out.state, err);
    else
        return fail(TT_ERR_INVALID, "ray ordering: hit records are 8 or 24 bytes");
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(TT_ERR_CUDA, std::string("ray ordering: ") + cudaGetErrorString(e));
    return TT_OK;
}

// tt_ray_order_keys_device: the key of every ray, as the ordering kernels compute it
__global__ void __launch_bounds__(kOrderBlock) k_order_keys_only(const float4 *rays, int64_t n, OrderGrid g,
                                                                unsigned *keys) {
    for (int64_t i = (int64_t)blockIdx.x * kOrderBlock + threadIdx.x; i < n; i += (int64_t)gridDim.x * kOrderBlock)
        keys[i] = order_key(__ldg(rays + 2 * i), __ldg(rays + 2 * i + 1), g);
}

}  // namespace tt

extern "C" tt_status tt_ray_order_keys_device(const tt_ray *d_rays, int64_t n, const float lo[3], const float hi[3],
                                              uint32_t *d_keys, int32_t *key_bits, void *stream) {
    if (n < 0 || n >= ((int64_t)1 << 31)) return tt::fail(TT_ERR_INVALID, "tt_ray_order_keys_device: n out of range");
    if (!lo || !hi || !key_bits || (n > 0 && (!d_rays || !d_keys)))
        return tt::fail(TT_ERR_INVALID, "tt_ray_order_keys_device: null argument");
    if (reinterpret_cast<uintptr_t>(d_rays) & 15)
        return tt::fail(TT_ERR_INVALID, "tt_ray_order_keys_device: rays must be 16-byte aligned");
    const int ob = tt::order_origin_bits(n);
    *key_bits = tt::kOrderDirBits + ob;
    if (n == 0) return TT_OK;
    const tt::OrderGrid g = tt::order_grid(lo, hi, ob);
    const int64_t blocks = std::min<int64_t>((n + tt::kOrderBlock - 1) / tt::kOrderBlock, 152 * 8);
    tt::k_order_keys_only<<<(unsigned)blocks, tt::kOrderBlock, 0, (cudaStream_t)stream>>>(
        reinterpret_cast<const float4 *>(d_rays), n, g, d_keys);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return tt::fail(TT_ERR_CUDA, std::string("tt_ray_order_keys_device: ") + cudaGetErrorString(e));
    return TT_OK;
}

extern "C" tt_status tt_ray_order_keys(const tt_ray *rays, int64_t n, const float lo[3], const float hi[3],
                                       uint32_t *keys, int32_t *key_bits) {
    if (n < 0) return tt::fail(TT_ERR_INVALID, "tt_ray_order_keys: n < 0");
    if (!lo || !hi || !key_bits || (n > 0 && (!rays || !keys)))
        return tt::fail(TT_ERR_INVALID, "tt_ray_order_keys: null argument");
    const int ob = tt::order_origin_bits(n);
    *key_bits = tt::kOrderDirBits + ob;
    const tt::OrderGrid g = tt::order_grid(lo, hi, ob);
    const float *r = reinterpret_cast<const float *>(rays);
    for (int64_t i = 0; i < n; i++, r += 8)
        keys[i] = tt::order_key(make_float4(r[0], r[1], r[2], r[3]), make_float4(r[4], r[5], r[6], r[7]), g);
    return TT_OK;
}
