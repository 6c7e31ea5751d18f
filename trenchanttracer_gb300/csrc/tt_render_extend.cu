// Traversal stages of the native wavefront path tracer: closest hit of every queued path
// (extend) and any hit of every queued shadow ray (shadow).
//
// Both are persistent grids in which each warp claims 32 consecutive queue slots with one atomic
// and traces them with the per-ray traversal of tt_traverse.cuh, so the result of a ray never
// depends on the other rays of its warp. Each is built for every block size and shared-memory
// stack depth in kBlockShapes x kStackShapes; the renderer's autotuner picks one.
#include <cuda_runtime.h>

#include "tt_native.cuh"

namespace tt {

using namespace pt;

// kPrefix: the ordering covers only the queue's first *n_sorted slots (a streamed render's
// survivors); the rest is traced in place. Without it an ordered queue is ordered whole.
template <int kBlock, int kSh, bool kPrefix>
__global__ void __launch_bounds__(kBlock) k_extend(NativeArgs a, int cur) {
    __shared__ int sh_stack[(kSh > 0 ? kSh : 1) * kBlock];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.ps.counts[cur ^ 1] = 0;
        a.ps.counts[2] = 0;
        a.ps.counts[4] = 0;
    }
    const int n = a.ps.counts[cur];
    const int lane = threadIdx.x & 31;
    TravStack<kSh, kBlock> stack;
    stack.sh = sh_stack + threadIdx.x;
    uint32_t err = 0;
    // an ordered queue prefix: rays and hits by ordered slot, moved back by k_order_gather_hits
    const bool ordered = a.order.sorted && order_built(a.order.state);
    const int n_sorted = ordered ? (kPrefix ? *a.order.n_sorted : n) : 0;
    for (;;) {
        int base = 0;
        if (lane == 0) base = atomicAdd(a.ps.counts + 3, 32);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        const int q = base + lane;
        const unsigned mask = __ballot_sync(0xffffffffu, q < n);
        if (q < n) {
            const bool srt = kPrefix ? q < n_sorted : ordered;
            const float4 *rays = srt ? a.order.sorted : a.ps.ray[cur];
            const float4 r0 = rays[2 * q], r1 = rays[2 * q + 1];
            const TraceResult tr = traverse_on<true>(stack, a.bvh, r0, r1, err);
            float t = tr.t, hu = tr.u, hv = tr.v;
            int prim = tr.addr;
            if (a.num_geoms)
                analytic_hit(a, mask, true, V3(r0.x, r0.y, r0.z), V3(r0.w, r1.x, r1.y), r1.z, t, prim, hu, hv, false);
            (srt ? a.order.hit_t : a.ps.hit_t)[q] = t;
            (srt ? a.order.hit_prim : a.ps.hit_prim)[q] = prim;
            (srt ? a.order.hit_u : a.ps.hit_u)[q] = hu;
            (srt ? a.order.hit_v : a.ps.hit_v)[q] = hv;
        }
        __syncwarp();
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(a.stats + 0, (unsigned long long)n);
    if (err) atomicOr(a.err, err);
}

template <int kBlock, int kSh>
__global__ void __launch_bounds__(kBlock) k_shadow(NativeArgs a) {
    __shared__ int sh_stack[(kSh > 0 ? kSh : 1) * kBlock];
    if (blockIdx.x == 0 && threadIdx.x == 0) a.ps.counts[3] = 0;  // the next extend's work counter
    const int n = a.ps.counts[2];
    const int lane = threadIdx.x & 31;
    TravStack<kSh, kBlock> stack;
    stack.sh = sh_stack + threadIdx.x;
    uint32_t err = 0;
    // an ordered queue: rays in sorted order, each ray's path and value at its original slot
    const bool ordered = a.shadow_order.sorted && order_built(a.shadow_order.state);
    const float4 *rays = ordered ? a.shadow_order.sorted : a.ps.shadow_ray;
    for (;;) {
        int base = 0;
        if (lane == 0) base = atomicAdd(a.ps.counts + 4, 32);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n) break;
        const int j = base + lane;
        const unsigned mask = __ballot_sync(0xffffffffu, j < n);
        if (j < n) {
            const float4 r0 = rays[2 * j], r1 = rays[2 * j + 1];
            const TraceResult tr = traverse_on<false>(stack, a.bvh, r0, r1, err);
            bool blocked = tr.addr >= 0;
            if (a.num_geoms) {
                float t = r1.w, hu, hv;
                int prim = -1;
                analytic_hit(a, mask, !blocked, V3(r0.x, r0.y, r0.z), V3(r0.w, r1.x, r1.y), r1.z, t, prim, hu, hv,
                             true);
                blocked = blocked || prim != -1;
            }
            const int src = ordered ? a.shadow_order.src[j] : j;
            if ((unsigned)src >= (unsigned)n) {  // not reachable with a consistent ordering
                err |= kErrOrder;
            } else if (!blocked) {
                // a path's radiance: L[3 * t] for t >= 0, else (an ended path of a streamed
                // render) ring entry -1 - t
                const int t = a.ps.shadow_path[src];
                float *L = t >= 0 ? a.ps.L + 3ll * t : a.stream.ring + 3ll * (-1ll - t);
                const float *c = a.ps.shadow_val + 3ll * src;
                L[0] = PT_ADD(L[0], c[0]);
                L[1] = PT_ADD(L[1], c[1]);
                L[2] = PT_ADD(L[2], c[2]);
            }
        }
        __syncwarp();
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(a.stats + 1, (unsigned long long)n);
    if (err) atomicOr(a.err, err);
}

__global__ void __launch_bounds__(256) k_order_gather_hits(NativeArgs a, int cur) {
    if (!a.order.sorted || !order_built(a.order.state)) return;
    const int n = *a.order.n_sorted;
    unsigned bad = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int p = __ldcs(a.order.pos + i);
        if ((unsigned)p < (unsigned)n) {
            a.ps.hit_t[i] = a.order.hit_t[p];
            a.ps.hit_u[i] = a.order.hit_u[p];
            a.ps.hit_v[i] = a.order.hit_v[p];
            a.ps.hit_prim[i] = a.order.hit_prim[p];
        } else {  // not reachable with a consistent ordering: report, and let the path miss
            a.ps.hit_prim[i] = -1;
            bad = 1;
        }
    }
    if (bad) atomicOr(a.err, kErrOrder);
}

template <int kBlock, int kSh>
static TraceKernels kernels_of() {
    TraceKernels k;
    k.extend = k_extend<kBlock, kSh, false>;
    k.extend_prefix = k_extend<kBlock, kSh, true>;
    k.shadow = k_shadow<kBlock, kSh>;
    return k;
}

template <int kBlock>
static TraceKernels kernels_of_block(int sh) {
    switch (sh) {
        case 0: return kernels_of<kBlock, 0>();
        case 8: return kernels_of<kBlock, 8>();
        case 16: return kernels_of<kBlock, 16>();
        default: return TraceKernels{nullptr, nullptr, nullptr};
    }
}

TraceKernels trace_kernels(int block, int stack_shared) {
    switch (block) {
        case 64: return kernels_of_block<64>(stack_shared);
        case 128: return kernels_of_block<128>(stack_shared);
        case 256: return kernels_of_block<256>(stack_shared);
        default: return TraceKernels{nullptr, nullptr, nullptr};
    }
}

}  // namespace tt
