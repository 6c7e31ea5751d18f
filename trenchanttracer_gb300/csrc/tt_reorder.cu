// Ray ordering before traversal: a counting sort of the rays by a 21-bit key — the direction's
// octant (3 bits, most significant) above the Morton code of the origin's cell in a 64^3 grid over
// the scene bounds — producing a permutation the warp-batched trace kernel reads rays through.
// Rays that leave the same region in the same octant then share a warp, so their lanes fetch the
// same nodes and diverge less. Each ray's hit still goes to its own slot, and traversal has
// per-ray semantics, so the results do not depend on the order.
//
// Passes: keys (and a count of the warps whose 32 keys are all equal), histogram (one atomic
// per group of equal keys in a warp, __match_any_sync), exclusive scan of the 2^21 counts
// (2048-element blocks, then the 1024 block sums, then the offsets added back), scatter (again
// one atomic per group of equal keys). The order inside a key is whatever the atomics give; only
// the grouping matters. When more than half of the warps are uniform the rays are already
// coherent (camera rays share one origin cell): histogram, scan and scatter then leave the
// permutation as the identity, which costs less than sorting into a handful of heavily
// contended keys and loses nothing in traversal.
#include <cuda_runtime.h>

#include <string>

#include "tt_internal.h"
#include "tt_reorder.h"

namespace tt {

constexpr int kCells = 64;  // per axis
constexpr int kScanBlock = 2048;
static_assert((1 << kOrderBits) == 8 * kCells * kCells * kCells, "key = octant x 64^3 cells");
static_assert((1 << kOrderBits) / kScanBlock == 1024, "one block scans the block sums");

// info[0]: warps of 32 equal keys, info[1]: full warps
__global__ void __launch_bounds__(256) k_order_keys(const float4 *rays, int64_t n, float3 lo, float3 scale,
                                                    unsigned *keys, unsigned long long *info) {
    const int lane = threadIdx.x & 31;
    unsigned uniform = 0, full = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float4 r0 = rays[2 * i], r1 = rays[2 * i + 1];
        const unsigned oct = (r0.w < 0.0f ? 1u : 0u) | (r1.x < 0.0f ? 2u : 0u) | (r1.y < 0.0f ? 4u : 0u);
        const unsigned qx = (unsigned)fminf(fmaxf((r0.x - lo.x) * scale.x, 0.0f), (float)(kCells - 1));
        const unsigned qy = (unsigned)fminf(fmaxf((r0.y - lo.y) * scale.y, 0.0f), (float)(kCells - 1));
        const unsigned qz = (unsigned)fminf(fmaxf((r0.z - lo.z) * scale.z, 0.0f), (float)(kCells - 1));
        unsigned code = 0;
#pragma unroll
        for (int b = 0; b < 6; b++)
            code |= (((qx >> b) & 1u) << (3 * b)) | (((qy >> b) & 1u) << (3 * b + 1)) | (((qz >> b) & 1u) << (3 * b + 2));
        const unsigned key = (oct << 18) | code;
        keys[i] = key;
        const unsigned active = __activemask();
        const unsigned peers = __match_any_sync(active, key);
        if (active == 0xffffffffu && lane == 0) {
            full++;
            if (peers == 0xffffffffu) uniform++;
        }
    }
    if (lane == 0 && full) {
        atomicAdd(info, (unsigned long long)uniform);
        atomicAdd(info + 1, (unsigned long long)full);
    }
}

__device__ __forceinline__ bool coherent(const unsigned long long *info) { return 2 * info[0] > info[1]; }

__global__ void __launch_bounds__(256) k_order_hist(const unsigned *keys, int64_t n, unsigned *counts,
                                                    const unsigned long long *info) {
    if (coherent(info)) return;
    const int lane = threadIdx.x & 31;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const unsigned key = keys[i];
        const unsigned peers = __match_any_sync(__activemask(), key);
        if (lane == __ffs(peers) - 1) atomicAdd(counts + key, (unsigned)__popc(peers));
    }
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

// exclusive scan of kScanBlock counts per block (two per thread); the block's total to sums
__global__ void __launch_bounds__(1024) k_scan_local(unsigned *v, unsigned *sums, const unsigned long long *info) {
    if (coherent(info)) return;
    __shared__ unsigned warp_tot[32];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    unsigned *blk = v + (size_t)blockIdx.x * kScanBlock;
    const unsigned a = blk[2 * t], b = blk[2 * t + 1];
    const unsigned s = a + b;
    const unsigned x = warp_scan(s);
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) warp_tot[lane] = warp_scan(warp_tot[lane]);
    __syncthreads();
    const unsigned excl = x - s + (w ? warp_tot[w - 1] : 0u);
    blk[2 * t] = excl;
    blk[2 * t + 1] = excl + a;
    if (t == 1023) sums[blockIdx.x] = excl + s;
}

// exclusive scan of the 1024 block sums, in place
__global__ void __launch_bounds__(1024) k_scan_sums(unsigned *sums, const unsigned long long *info) {
    if (coherent(info)) return;
    __shared__ unsigned warp_tot[32];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const unsigned s = sums[t];
    const unsigned x = warp_scan(s);
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) warp_tot[lane] = warp_scan(warp_tot[lane]);
    __syncthreads();
    sums[t] = x - s + (w ? warp_tot[w - 1] : 0u);
}

__global__ void __launch_bounds__(256) k_scan_add(unsigned *v, const unsigned *sums, const unsigned long long *info) {
    if (coherent(info)) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < (1 << kOrderBits)) v[i] += sums[i / kScanBlock];
}

__global__ void __launch_bounds__(256) k_order_scatter(const unsigned *keys, int64_t n, unsigned *cursor,
                                                       int *perm, const unsigned long long *info) {
    const int lane = threadIdx.x & 31;
    if (coherent(info)) {
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
            perm[i] = (int)i;
        return;
    }
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const unsigned key = keys[i];
        const unsigned peers = __match_any_sync(__activemask(), key);
        const int leader = __ffs(peers) - 1;
        unsigned base = 0;
        if (lane == leader) base = atomicAdd(cursor + key, (unsigned)__popc(peers));
        base = __shfl_sync(peers, base, leader);
        perm[base + __popc(peers & ((1u << lane) - 1u))] = (int)i;
    }
}

size_t reorder_scratch_bytes(int64_t n) {
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    return al(4ull * n) + al(4ull * n) + al(4ull << kOrderBits) + al(4ull * 1024) + 256;
}

tt_status reorder_rays(const float4 *rays, int64_t n, const float lo[3], const float hi[3], void *scratch,
                       int num_sms, cudaStream_t s, const int **perm_out) {
    if (n <= 0 || n >= ((int64_t)1 << 31)) return fail(TT_ERR_INVALID, "ray ordering: n must be in 1..2^31-1");
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    char *p = static_cast<char *>(scratch);
    unsigned *keys = reinterpret_cast<unsigned *>(p);
    p += al(4ull * n);
    int *perm = reinterpret_cast<int *>(p);
    p += al(4ull * n);
    unsigned *counts = reinterpret_cast<unsigned *>(p);
    p += al(4ull << kOrderBits);
    unsigned *sums = reinterpret_cast<unsigned *>(p);
    p += al(4ull * 1024);
    unsigned long long *info = reinterpret_cast<unsigned long long *>(p);
    const float3 flo = make_float3(lo[0], lo[1], lo[2]);
    const float3 scale = make_float3((float)kCells / (hi[0] - lo[0]), (float)kCells / (hi[1] - lo[1]),
                                     (float)kCells / (hi[2] - lo[2]));
    cudaError_t e = cudaMemsetAsync(counts, 0, 4ull << kOrderBits, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(info, 0, 16, s);
    if (e != cudaSuccess) return fail(TT_ERR_CUDA, std::string("ray ordering: ") + cudaGetErrorString(e));
    const int64_t want = (n + 255) / 256;
    const unsigned grid = (unsigned)(want < (int64_t)num_sms * 8 ? want : (int64_t)num_sms * 8);
    k_order_keys<<<grid, 256, 0, s>>>(rays, n, flo, scale, keys, info);
    k_order_hist<<<grid, 256, 0, s>>>(keys, n, counts, info);
    k_scan_local<<<(1 << kOrderBits) / kScanBlock, 1024, 0, s>>>(counts, sums, info);
    k_scan_sums<<<1, 1024, 0, s>>>(sums, info);
    k_scan_add<<<(1 << kOrderBits) / 256, 256, 0, s>>>(counts, sums, info);
    k_order_scatter<<<grid, 256, 0, s>>>(keys, n, counts, perm, info);
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(TT_ERR_CUDA, std::string("ray ordering: ") + cudaGetErrorString(e));
    *perm_out = perm;
    return TT_OK;
}

}  // namespace tt
