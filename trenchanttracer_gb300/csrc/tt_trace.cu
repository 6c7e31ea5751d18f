// Ray-cast kernels (closest-hit / any-hit) and the device half of the compact BVH.
//
// All kernels are persistent grids sized to fill every SM of the GB300 with resident blocks.
// Kernel shapes (tt_dbvh_set_variant; tt_dbvh_autotune times them and keeps the fastest):
//   TT_VARIANT_WARP       each warp claims 32 consecutive rays (lane i traces ray base+i, as a
//                         one-ray-per-thread launch would) and traces them with the per-ray
//                         semantics; the whole traversal stack is in local memory.
//   TT_VARIANT_WARP_SH16  as WARP, the lowest 16 stack entries in shared memory (the rest, rarely
//   TT_VARIANT_WARP_SH32  touched, in local memory), so stack traffic does not evict BVH nodes
//                         from L1; SH32 keeps 32 entries.
//   TT_VARIANT_DYNAMIC    every lane claims a new ray (one warp-aggregated atomic per claim
//                         round: ballot + popc + one atomicAdd) as soon as it finishes one.
//   TT_VARIANT_WARP_VOTE  as WARP, but a lane that has postponed a leaf keeps visiting inner
//                         nodes until a warp vote says every active lane holds one, as the
//                         reference kernel does (IntersectKernel.cuh:180-203). Which lanes are
//                         active at the vote depends on how the warp re-converges, so in float
//                         corner cases (a leaf box whose entry rounds above a nearly equal hit
//                         distance) the result can depend on the other rays of the warp.
//   TT_VARIANT_SORTED     WARP_SH16 over the rays in the order of a counting sort by origin
//                         cell and direction cell (tt_reorder.cu), or in their own order when a
//                         sample finds them coherent; each hit still goes to its own ray's slot.
//                         Compiled for 10 resident blocks per SM (48 registers, 8 bytes spilled;
//                         without that bound it takes 61 registers and 8 blocks fit).
//   TT_VARIANT_SH16_OCC,  WARP_SH16 and SORTED compiled for 12 resident blocks per SM (40
//   TT_VARIANT_SORTED_OCC registers and a few spilled values), trading spills for more warps to
//                         hide the node-fetch latency.
// All but WARP_VOTE return the per-ray result of the reference's algorithm, bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "tt_internal.h"
#include "tt_reorder.h"
#include "tt_traverse.cuh"

namespace tt {

constexpr int kTraceBlock = 128;
enum TraceVariant : int {
    VARIANT_WARP = 0,
    VARIANT_WARP_SH16 = 1,
    VARIANT_WARP_SH32 = 2,
    VARIANT_DYNAMIC = 3,
    VARIANT_WARP_VOTE = 4,
    VARIANT_SORTED = 5,
    VARIANT_SH16_OCC = 6,
    VARIANT_SORTED_OCC = 7,
    NUM_VARIANTS = 8
};
constexpr int kOccBlocks = 12;  // resident blocks per SM the *_OCC variants are compiled for
// resident blocks per SM the default (ordered) variant is compiled for: 48 registers, 8 bytes
// spilled; against 8 blocks at 61 registers it traces the terrain sets 4 % faster (9: 2 %)
constexpr int kSortedBlocks = 10;
// the node array's top levels laid out first at upload (bytes), and the default L2 persisting
// window of the trace launches over them
constexpr size_t kL2TopRegion = 16ull << 20;
constexpr size_t kL2WindowDefault = 8ull << 20;

struct DeviceBVH {
    BvhView view;
    void *base = nullptr;          // one allocation holding all five arrays
    size_t bytes = 0;
    uint32_t num_nodes = 0, num_verts = 0;
    unsigned long long *scratch = nullptr;  // [0] work counter, [1] error word (low 32 bits)
    int device = 0;
    int num_sms = 0;
    int blocks_per_sm[NUM_VARIANTS] = {1, 1, 1, 1, 1, 1, 1, 1};
    int variant = VARIANT_SORTED;
    // L2 access-policy window over the node array for the trace launches (0 bytes: none), set up
    // at the first trace launch (the persisting set-aside shrinks the L2 left to other work, so a
    // BVH that is only rendered never asks for one)
    size_t l2_window_bytes = 0;
    float l2_hit_ratio = 0.0f;
    bool l2_setup = false;
    size_t l2_top_bytes = 0;                   // the breadth-first top of the node array (upload)
    size_t l2_window_want = kL2WindowDefault;  // tt_dbvh_set_l2_window
    float lo[3] = {-1.f, -1.f, -1.f}, hi[3] = {1.f, 1.f, 1.f};  // scene bounds (root boxes)
    // ray-ordering scratch per work-counter slot (caller stream, three pipeline streams)
    void *order[4] = {nullptr, nullptr, nullptr, nullptr};
    size_t order_bytes[4] = {0, 0, 0, 0};
    size_t order_state_at[4] = {0, 0, 0, 0};  // byte offset of the ordering state block
    // device staging, streams and events for the host-buffer entry point's copy/compute pipeline
    void *d_stage = nullptr;
    size_t d_stage_bytes = 0;
    cudaStream_t pipe[3] = {nullptr, nullptr, nullptr};
    cudaEvent_t pipe_done[3] = {nullptr, nullptr, nullptr};
    cudaEvent_t pipe_start = nullptr;
};

// Scratch words (64-bit) of a DeviceBVH: [0] work counter of the caller-stream launches,
// [1] error word shared by all launches, [2..4] work counters of the three pipeline streams.
constexpr int kScratchErr = 1;
constexpr int kScratchPipe = 2;

struct TraceArgs {
    BvhView bvh;
    const float4 *rays;  // 2 float4 per ray
    int64_t n;
    void *hits;
    unsigned long long *counter;
    unsigned int *err;
    // TT_VARIANT_SORTED, when order_built(order_state): rays and hits by sorted slot (the hits
    // are moved to their rays' places afterwards)
    const float4 *sorted;
    void *sorted_hits;
    const unsigned long long *order_state;
};

template <bool kExt>
__device__ __forceinline__ void store_hit(const TraceArgs &a, void *hits, int64_t i, const TravState &s) {
    int id = -1;
    if (s.addr >= 0) id = __ldg(a.bvh.tri_idx + s.addr);
    if (!kExt) {
        reinterpret_cast<int2 *>(hits)[i] = make_int2(id, __float_as_int(s.t));
    } else {
        int mat = -1;
        float nx = 0.f, ny = 0.f, nz = 0.f;
        if (s.addr >= 0) {
            mat = (int)__ldg(a.bvh.mat_idx + s.addr);
            hit_normal(a.bvh, s.addr, s.u, s.v, nx, ny, nz);
        }
        tt_hit_ext *o = reinterpret_cast<tt_hit_ext *>(hits) + i;
        o->id = id;
        o->mat = mat;
        o->t = s.t;
        o->nx = nx;
        o->ny = ny;
        o->nz = nz;
    }
}

// Warp-batched: each warp claims 32 consecutive rays (kPerm: 32 consecutive slots of the sorted
// ray copy, when the ordering built one). kSh stack entries live in shared memory.
template <bool kClosest, bool kExt, bool kSpec, int kSh, bool kPerm = false, int kMinBlocks = 1>
__global__ void __launch_bounds__(kTraceBlock, kMinBlocks) trace_warp_kernel(TraceArgs a) {
    __shared__ int sh_stack[(kSh > 0 ? kSh : 1) * kTraceBlock];
    const int lane = threadIdx.x & 31;
    uint32_t err = 0;
    TravStack<kSh, kTraceBlock> stack;
    stack.sh = sh_stack + threadIdx.x;
    const bool use_perm = kPerm && order_built(a.order_state);
    for (;;) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(a.counter, 32ull);
        base = __shfl_sync(0xffffffffu, base, 0);
        if ((int64_t)base >= a.n) break;
        const int64_t slot = (int64_t)base + lane;
        if (slot < a.n) {
            // sorted: rays and hits by sorted slot (contiguous); else by ray
            const float4 *rays = use_perm ? a.sorted : a.rays;
            const float4 r0 = __ldg(rays + 2 * slot), r1 = __ldg(rays + 2 * slot + 1);
            TravState s;
            trav_init(s, stack, r0, r1);
            while (!trav_iterate<kClosest, kSpec>(s, stack, a.bvh, err, r1.w)) {
            }
            store_hit<kExt>(a, use_perm ? a.sorted_hits : a.hits, slot, s);
        }
        __syncwarp();
    }
    if (err) atomicOr(a.err, err);
}

// Dynamic per-lane fetch: a lane that finishes its ray claims the next one at the top of the
// following outer iteration; claims are aggregated per warp.
template <bool kClosest, bool kExt, int kSh>
__global__ void __launch_bounds__(kTraceBlock) trace_dynamic_kernel(TraceArgs a) {
    __shared__ int sh_stack[(kSh > 0 ? kSh : 1) * kTraceBlock];
    const int lane = threadIdx.x & 31;
    const unsigned lanemask_lt = (1u << lane) - 1u;
    uint32_t err = 0;
    TravStack<kSh, kTraceBlock> stack;
    stack.sh = sh_stack + threadIdx.x;
    TravState s;
    int64_t ray = -1;
    float tmax = 0.f;
    bool exhausted = false;
    for (;;) {
        const bool need = (ray < 0) && !exhausted;
        const unsigned needmask = __ballot_sync(0xffffffffu, need);
        if (needmask) {
            const int leader = __ffs(needmask) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(a.counter, (unsigned long long)__popc(needmask));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (need) {
                const int64_t idx = (int64_t)base + __popc(needmask & lanemask_lt);
                if (idx < a.n) {
                    ray = idx;
                    const float4 r0 = __ldg(a.rays + 2 * idx), r1 = __ldg(a.rays + 2 * idx + 1);
                    tmax = r1.w;
                    trav_init(s, stack, r0, r1);
                } else {
                    exhausted = true;
                }
            }
        }
        if (__all_sync(0xffffffffu, exhausted)) break;
        if (ray >= 0) {
            if (trav_iterate<kClosest, false>(s, stack, a.bvh, err, tmax)) {
                store_hit<kExt>(a, a.hits, ray, s);
                ray = -1;
            }
        }
    }
    if (err) atomicOr(a.err, err);
}

template <bool kClosest, bool kExt>
static const void *kernel_for(int variant) {
    switch (variant) {
        case VARIANT_WARP: return (const void *)trace_warp_kernel<kClosest, kExt, false, 0>;
        case VARIANT_WARP_SH16: return (const void *)trace_warp_kernel<kClosest, kExt, false, 16>;
        case VARIANT_WARP_SH32: return (const void *)trace_warp_kernel<kClosest, kExt, false, 32>;
        case VARIANT_DYNAMIC: return (const void *)trace_dynamic_kernel<kClosest, kExt, 16>;
        case VARIANT_SORTED: return (const void *)trace_warp_kernel<kClosest, kExt, false, 16, true, kSortedBlocks>;
        case VARIANT_SH16_OCC: return (const void *)trace_warp_kernel<kClosest, kExt, false, 16, false, kOccBlocks>;
        case VARIANT_SORTED_OCC: return (const void *)trace_warp_kernel<kClosest, kExt, false, 16, true, kOccBlocks>;
        default: return (const void *)trace_warp_kernel<kClosest, kExt, true, 0>;
    }
}

static tt_status cuda_fail(cudaError_t e, const char *what) {
    return fail(TT_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define TT_CUDA(call)                                       \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

// The device's node order: the top levels of the tree first (breadth first from the root, until
// they fill top_bytes), then every other inner node in the file's depth-first order. Child order,
// node contents and leaf addresses are unchanged, only inner-child addresses are renumbered, so a
// traversal visits the same nodes and leaves in the same order and returns the same hits. The
// L2 persisting window of the trace launches then covers a prefix of the array that is exactly
// the tree's top levels (the file's depth-first order scatters them over the whole array).
// Returns false, leaving `out` empty, for an array whose child addresses do not form a tree.
static bool top_first_nodes(const std::vector<I4> &nodes, size_t top_bytes, std::vector<I4> &out, size_t &top_out) {
    const size_t count = nodes.size() / 4;
    out.clear();
    top_out = 0;
    if (count == 0 || nodes.size() % 4) return false;
    std::vector<int64_t> new_index(count, -1), order;
    order.reserve(count);
    const size_t top_nodes = std::max<size_t>(1, top_bytes / 64);
    // breadth first, level by level, while the placed nodes fit in top_bytes
    new_index[0] = 0;
    order.push_back(0);
    for (size_t head = 0; head < order.size() && order.size() < top_nodes; head++) {
        const I4 &c = nodes[4 * (size_t)order[head] + 3];
        for (int32_t addr : {c.x, c.y}) {
            if (addr < 0) continue;  // a leaf
            if (addr % 4 || (size_t)addr / 4 >= count) return false;
            const size_t k = (size_t)addr / 4;
            if (new_index[k] >= 0) return false;  // not a tree
            if (order.size() >= top_nodes) break;
            new_index[k] = (int64_t)order.size();
            order.push_back((int64_t)k);
        }
    }
    top_out = 64 * order.size();
    for (size_t k = 0; k < count; k++)
        if (new_index[k] < 0) {
            new_index[k] = (int64_t)order.size();
            order.push_back((int64_t)k);
        }
    out.resize(nodes.size());
    for (size_t j = 0; j < count; j++) {
        const size_t k = (size_t)order[j];
        for (int q = 0; q < 4; q++) out[4 * j + q] = nodes[4 * k + q];
        I4 &c = out[4 * j + 3];
        for (int32_t *addr : {&c.x, &c.y}) {
            if (*addr < 0) continue;
            if (*addr % 4 || (size_t)*addr / 4 >= count) {
                out.clear();
                top_out = 0;
                return false;
            }
            *addr = (int32_t)(4 * new_index[(size_t)*addr / 4]);
        }
    }
    return true;
}

static tt_status upload(const CompactBVH &b, DeviceBVH &d) {
    int dev = 0;
    TT_CUDA(cudaGetDevice(&dev));
    d.device = dev;
    TT_CUDA(cudaDeviceGetAttribute(&d.num_sms, cudaDevAttrMultiProcessorCount, dev));
    for (int v = 0; v < NUM_VARIANTS; v++) {
        int bps = 0;
        TT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kernel_for<true, false>(v), kTraceBlock, 0));
        d.blocks_per_sm[v] = bps > 0 ? bps : 1;
    }
    const size_t nb = 16ull * b.nodes.size(), vb = 16ull * b.vertices.size(), mb = 16ull * b.normals.size();
    const size_t tb = 4ull * b.tri_idx.size(), ab = 4ull * b.mat_idx.size();
    auto align = [](size_t x) { return (x + 255) & ~size_t(255); };
    d.bytes = align(nb) + align(vb) + align(mb) + align(tb) + align(ab);
    cudaError_t e = cudaMalloc(&d.base, d.bytes);
    if (e != cudaSuccess) return fail(TT_ERR_OOM, std::string("cudaMalloc BVH: ") + cudaGetErrorString(e));
    char *p = static_cast<char *>(d.base);
    d.view.nodes = reinterpret_cast<const float4 *>(p);
    {
        std::vector<I4> reordered;
        size_t top = 0;
        if (top_first_nodes(b.nodes, kL2TopRegion, reordered, top)) {
            TT_CUDA(cudaMemcpy(p, reordered.data(), nb, cudaMemcpyHostToDevice));
            d.l2_top_bytes = top;
        } else {
            TT_CUDA(cudaMemcpy(p, b.nodes.data(), nb, cudaMemcpyHostToDevice));
            d.l2_top_bytes = nb;  // file order: only the whole array is a window over the top levels
        }
    }
    p += align(nb);
    d.view.verts = reinterpret_cast<const float4 *>(p);
    TT_CUDA(cudaMemcpy(p, b.vertices.data(), vb, cudaMemcpyHostToDevice));
    p += align(vb);
    d.view.norms = reinterpret_cast<const float4 *>(p);
    TT_CUDA(cudaMemcpy(p, b.normals.data(), mb, cudaMemcpyHostToDevice));
    p += align(mb);
    d.view.tri_idx = reinterpret_cast<const int32_t *>(p);
    TT_CUDA(cudaMemcpy(p, b.tri_idx.data(), tb, cudaMemcpyHostToDevice));
    p += align(tb);
    d.view.mat_idx = reinterpret_cast<const uint32_t *>(p);
    TT_CUDA(cudaMemcpy(p, b.mat_idx.data(), ab, cudaMemcpyHostToDevice));
    d.num_nodes = (uint32_t)b.nodes.size();
    d.num_verts = (uint32_t)b.vertices.size();
    // scene bounds from the root's two child boxes (float4 0: c0 x/y, 1: c1 x/y, 2: z of both),
    // for the ray-ordering grid; an axis without a finite, non-empty extent keeps [-1, 1]
    if (b.nodes.size() >= 3) {
        const float *n0 = reinterpret_cast<const float *>(&b.nodes[0]);
        const float *n1 = reinterpret_cast<const float *>(&b.nodes[1]);
        const float *nz = reinterpret_cast<const float *>(&b.nodes[2]);
        const float lo[3] = {std::fmin(n0[0], n1[0]), std::fmin(n0[2], n1[2]), std::fmin(nz[0], nz[2])};
        const float hi[3] = {std::fmax(n0[1], n1[1]), std::fmax(n0[3], n1[3]), std::fmax(nz[1], nz[3])};
        for (int k = 0; k < 3; k++)
            if (std::isfinite(lo[k]) && std::isfinite(hi[k]) && hi[k] > lo[k]) {
                d.lo[k] = lo[k];
                d.hi[k] = hi[k];
            }
    }
    e = cudaMalloc(&d.scratch, 256);
    if (e != cudaSuccess) return fail(TT_ERR_OOM, std::string("cudaMalloc scratch: ") + cudaGetErrorString(e));
    TT_CUDA(cudaMemset(d.scratch, 0, 256));
    return TT_OK;
}

static void release(DeviceBVH &d) {
    if (d.base) cudaFree(d.base);
    if (d.scratch) cudaFree(d.scratch);
    if (d.d_stage) cudaFree(d.d_stage);
    for (int i = 0; i < 4; i++)
        if (d.order[i]) cudaFree(d.order[i]);
    for (int i = 0; i < 3; i++) {
        if (d.pipe[i]) cudaStreamDestroy(d.pipe[i]);
        if (d.pipe_done[i]) cudaEventDestroy(d.pipe_done[i]);
    }
    if (d.pipe_start) cudaEventDestroy(d.pipe_start);
    d = DeviceBVH();
}

// Launches a variant's kernel. The node array is the launch's L2 access-policy window when the
// device allows one: node lines persist in the L2 set-aside and the rest of the window's traffic
// (rays, triangles, hits lie outside it) keeps the normal policy, so streaming triangles cannot
// push the nodes out.
template <bool kClosest, bool kExt>
static cudaError_t launch_variant(const DeviceBVH &d, int variant, unsigned blocks, cudaStream_t stream,
                                  TraceArgs a) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(kTraceBlock);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    if (d.l2_window_bytes) {
        attr[0].id = cudaLaunchAttributeAccessPolicyWindow;
        attr[0].val.accessPolicyWindow.base_ptr = const_cast<float4 *>(d.view.nodes);
        attr[0].val.accessPolicyWindow.num_bytes = d.l2_window_bytes;
        attr[0].val.accessPolicyWindow.hitRatio = d.l2_hit_ratio;
        attr[0].val.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
        attr[0].val.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
    }
    void *args[] = {&a};
    return cudaLaunchKernelExC(&cfg, kernel_for<kClosest, kExt>(variant), args);
}

// The L2 set-aside for the node array (a limit of this process's own context, which ends with it)
// and the window of the trace launches.
static void setup_l2_window(DeviceBVH &d) {
    d.l2_setup = true;
    int max_persist = 0, max_window = 0;
    if (cudaDeviceGetAttribute(&max_persist, cudaDevAttrMaxPersistingL2CacheSize, d.device) == cudaSuccess &&
        cudaDeviceGetAttribute(&max_window, cudaDevAttrMaxAccessPolicyWindowSize, d.device) == cudaSuccess &&
        max_persist > 0 && max_window > 0) {
        const size_t nb = std::min(std::min((size_t)16 * (size_t)d.num_nodes, d.l2_top_bytes), d.l2_window_want);
        size_t cur = 0;
        cudaDeviceGetLimit(&cur, cudaLimitPersistingL2CacheSize);
        const size_t want = std::min(nb, (size_t)max_persist);
        if (want > cur && cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, want) == cudaSuccess)
            cudaDeviceGetLimit(&cur, cudaLimitPersistingL2CacheSize);
        d.l2_window_bytes = (cur && nb) ? std::min(nb, (size_t)max_window) : 0;
        d.l2_hit_ratio = cur >= d.l2_window_bytes ? 1.0f : (float)cur / (float)d.l2_window_bytes;
    }
    cudaGetLastError();
}

// unordered = true traces a SORTED / SORTED_OCC variant's rays in their own order (its unsorted twin).
static tt_status launch_trace(const DeviceBVH &d, const void *d_rays, int64_t n, void *d_hits, bool closest,
                              bool ext, cudaStream_t stream, int counter_slot = 0, bool unordered = false) {
    if (n < 0 || n > ((int64_t)1 << 40)) return fail(TT_ERR_INVALID, "ray count out of range");
    if (n == 0) return TT_OK;
    if (!d_rays || !d_hits) return fail(TT_ERR_INVALID, "null ray or hit buffer");
    if ((reinterpret_cast<uintptr_t>(d_rays) & 15) || (reinterpret_cast<uintptr_t>(d_hits) & 7))
        return fail(TT_ERR_INVALID, "ray buffer must be 16-byte aligned and hit buffer 8-byte aligned");
    if (!d.l2_setup) setup_l2_window(const_cast<DeviceBVH &>(d));
    TT_CUDA(cudaMemsetAsync(d.scratch + counter_slot, 0, 8, stream));
    TraceArgs a;
    a.bvh = d.view;
    a.rays = reinterpret_cast<const float4 *>(d_rays);
    a.n = n;
    a.hits = d_hits;
    a.counter = d.scratch + counter_slot;
    a.err = reinterpret_cast<unsigned int *>(d.scratch + kScratchErr);
    a.sorted = nullptr;
    a.sorted_hits = nullptr;
    a.order_state = nullptr;
    OrderOut order{};
    int variant = d.variant;
    const bool sorted = variant == VARIANT_SORTED || variant == VARIANT_SORTED_OCC;
    // slots are int; too few rays cannot pay for the ordering
    if (sorted && (unordered || n >= ((int64_t)1 << 31) || n < kOrderMinRays))
        variant = variant == VARIANT_SORTED_OCC ? VARIANT_SH16_OCC : VARIANT_WARP_SH16;
    if (variant == VARIANT_SORTED || variant == VARIANT_SORTED_OCC) {
        // one scratch per work-counter slot, so the pipeline streams never share one
        const int k = counter_slot == 0 ? 0 : 1 + (counter_slot - kScratchPipe) % 3;
        const size_t need = reorder_scratch_bytes(n);
        DeviceBVH &dm = const_cast<DeviceBVH &>(d);
        if (dm.order_bytes[k] < need) {
            if (dm.order[k]) cudaFree(dm.order[k]);
            dm.order[k] = nullptr;
            dm.order_bytes[k] = 0;
            cudaError_t e = cudaMalloc(&dm.order[k], need);
            if (e != cudaSuccess) return fail(TT_ERR_OOM, std::string("ray ordering scratch: ") + cudaGetErrorString(e));
            dm.order_bytes[k] = need;
            dm.order_state_at[k] = reorder_state_offset(n);
            e = cudaMemsetAsync(static_cast<char *>(dm.order[k]) + dm.order_state_at[k], 0, 256, stream);
            if (e != cudaSuccess) return fail(TT_ERR_CUDA, std::string("ray ordering scratch: ") + cudaGetErrorString(e));
        }
        const tt_status st =
            reorder_rays(a.rays, n, nullptr, d.lo, d.hi, dm.order[k], dm.order_state_at[k], a.err, stream, &order);
        if (st != TT_OK) return st;
        a.sorted = order.sorted;
        a.sorted_hits = order.sorted_hits;
        a.order_state = order.state;
    }
    const int64_t warps_needed = (n + 31) / 32;
    int64_t blocks = (int64_t)d.num_sms * d.blocks_per_sm[variant];
    const int64_t max_useful = (warps_needed * 32 + kTraceBlock - 1) / kTraceBlock;
    if (blocks > max_useful) blocks = max_useful;
    if (blocks < 1) blocks = 1;
    cudaError_t le;
    if (closest) le = ext ? launch_variant<true, true>(d, variant, (unsigned)blocks, stream, a)
                          : launch_variant<true, false>(d, variant, (unsigned)blocks, stream, a);
    else le = ext ? launch_variant<false, true>(d, variant, (unsigned)blocks, stream, a)
                  : launch_variant<false, false>(d, variant, (unsigned)blocks, stream, a);
    TT_CUDA(le);
    if (a.order_state) return reorder_unpermute(order, n, d_hits, ext ? sizeof(tt_hit_ext) : sizeof(tt_hit), a.err, stream);
    return TT_OK;
}

static tt_status read_error_word(const DeviceBVH &d, cudaStream_t stream) {
    unsigned int w = 0;
    TT_CUDA(cudaMemcpyAsync(&w, d.scratch + 1, 4, cudaMemcpyDeviceToHost, stream));
    TT_CUDA(cudaStreamSynchronize(stream));
    if (w) {
        TT_CUDA(cudaMemsetAsync(d.scratch + 1, 0, 8, stream));
        TT_CUDA(cudaStreamSynchronize(stream));
        if (w & kErrStack) return fail(TT_ERR_BOUNDS, "traversal stack overflow (BVH deeper than 66 levels)");
        if (w & kErrOrder)
            return fail(TT_ERR_BOUNDS, "ray ordering: a sorted slot was out of range");
        return fail(TT_ERR_TIMEOUT, "traversal iteration cap reached (corrupt BVH?)");
    }
    return TT_OK;
}

// ---- allocation-free host-buffer tracing ----------------------------------------------------------
// A fixed staging area for tt_trace_host_noalloc: a 256-byte header (64-bit work counter, 32-bit
// error word) followed by room for kNoAllocMaxRays rays (32 B each) and their hits (8 B each),
// about 10 MiB in all. It is reserved on a GPU when this library's module is loaded there (with
// CUDA's lazy loading, at the first call that runs libtt code on that GPU) and held until the
// process exits.
constexpr int64_t kNoAllocMaxRays = 1 << 18;
constexpr size_t kNoAllocHeader = 256;
constexpr size_t kNoAllocBytes = kNoAllocHeader + (size_t)kNoAllocMaxRays * (32 + 8);
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

constexpr int kNoAllocMaxDevices = 64;
struct NoAllocDevice {
    unsigned char *scratch = nullptr;  // device address of g_noalloc_scratch on this device
    int num_sms = 0;
    int blocks_per_sm = 0;
};
static std::mutex g_noalloc_mu;
static NoAllocDevice g_noalloc_dev[kNoAllocMaxDevices];

// Once per device, with that device current: the device address of the staging array (host code
// must not hand the array's host-side name to a kernel) and the launch shape.
static tt_status noalloc_setup(NoAllocDevice &out) {
    int dev = 0;
    TT_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices) return fail(TT_ERR_INVALID, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    NoAllocDevice &d = g_noalloc_dev[dev];
    if (!d.scratch) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        int sms = 0, bps = 0;
        TT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        // one launch size for closest and any hit: the kernels claim rays from a counter, so the
        // grid only needs to fill the SMs, and the closest-hit build has the larger register count
        TT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kernel_for<true, false>(VARIANT_WARP_SH16),
                                                              kTraceBlock, 0));
        d.num_sms = sms;
        d.blocks_per_sm = bps > 0 ? bps : 1;
        d.scratch = static_cast<unsigned char *>(p);
    }
    out = d;
    return TT_OK;
}

}  // namespace tt

struct tt_dbvh {
    tt::DeviceBVH d;
};

using namespace tt;

namespace tt {
BvhView dbvh_view(const tt_dbvh *bvh) { return bvh->d.view; }
void dbvh_bounds(const tt_dbvh *bvh, float lo[3], float hi[3]) {
    for (int k = 0; k < 3; k++) {
        lo[k] = bvh->d.lo[k];
        hi[k] = bvh->d.hi[k];
    }
}
}  // namespace tt

extern "C" {

tt_status tt_bvh_upload(const tt_bvh *bvh, tt_dbvh **out) {
    if (!bvh || !out) return fail(TT_ERR_INVALID, "null argument");
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) return fail(TT_ERR_NO_DEVICE, "no CUDA device");
    auto *h = new tt_dbvh();
    tt_status st = upload(bvh->b, h->d);
    if (st != TT_OK) {
        release(h->d);
        delete h;
        return st;
    }
    *out = h;
    return TT_OK;
}

void tt_dbvh_free(tt_dbvh *dbvh) {
    if (!dbvh) return;
    release(dbvh->d);
    delete dbvh;
}

tt_status tt_dbvh_set_l2_window(tt_dbvh *bvh, int64_t bytes) {
    if (!bvh || bytes < 0) return fail(TT_ERR_INVALID, "null BVH or negative window");
    bvh->d.l2_window_want = (size_t)bytes;
    bvh->d.l2_setup = false;  // the next trace launch sets the window (and the set-aside) up again
    bvh->d.l2_window_bytes = 0;
    return TT_OK;
}

tt_status tt_dbvh_set_variant(tt_dbvh *bvh, int32_t variant) {
    if (!bvh || variant < 0 || variant >= NUM_VARIANTS) return fail(TT_ERR_INVALID, "unknown traversal variant");
    bvh->d.variant = variant;
    return TT_OK;
}

tt_status tt_dbvh_get_variant(const tt_dbvh *bvh, int32_t *variant) {
    if (!bvh || !variant) return fail(TT_ERR_INVALID, "null argument");
    *variant = bvh->d.variant;
    return TT_OK;
}

tt_status tt_dbvh_autotune(tt_dbvh *bvh, const tt_ray *d_rays, int64_t n, tt_hit *d_hits, int32_t closest,
                           int32_t include_vote, void *stream, float *ms_out) {
    if (!bvh) return fail(TT_ERR_INVALID, "null BVH");
    cudaStream_t s = (cudaStream_t)stream;
    DeviceBVH &d = bvh->d;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    TT_CUDA(cudaEventCreate(&e0));
    TT_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    int best_v = d.variant;
    tt_status st = TT_OK;
    for (int v = 0; v < NUM_VARIANTS && st == TT_OK; v++) {
        if (ms_out) ms_out[v] = 0.f;
        if (v == VARIANT_WARP_VOTE && !include_vote) continue;
        d.variant = v;
        float ms_min = 1e30f;
        for (int rep = 0; rep < 3 && st == TT_OK; rep++) {
            cudaEventRecord(e0, s);
            st = launch_trace(d, d_rays, n, d_hits, closest != 0, false, s);
            cudaEventRecord(e1, s);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (rep > 0 && ms < ms_min) ms_min = ms;  // the first launch is a warm-up
        }
        if (ms_out) ms_out[v] = ms_min;
        if (ms_min < best) {
            best = ms_min;
            best_v = v;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    d.variant = best_v;
    if (st != TT_OK) return st;
    return read_error_word(d, s);
}

tt_status tt_trace(const tt_dbvh *bvh, const tt_ray *d_rays, int64_t n, tt_hit *d_hits, int32_t closest,
                   void *stream) {
    if (!bvh) return fail(TT_ERR_INVALID, "null BVH");
    return launch_trace(bvh->d, d_rays, n, d_hits, closest != 0, false, (cudaStream_t)stream);
}

tt_status tt_trace_ext(const tt_dbvh *bvh, const tt_ray *d_rays, int64_t n, tt_hit_ext *d_hits, int32_t closest,
                       void *stream) {
    if (!bvh) return fail(TT_ERR_INVALID, "null BVH");
    return launch_trace(bvh->d, d_rays, n, d_hits, closest != 0, true, (cudaStream_t)stream);
}

// The device address of page-locked host memory mapped into the device's address space, or
// nullptr (pageable memory, device memory, or an error, which is cleared).
static const void *mapped_host_pointer(const void *p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

tt_status tt_trace_host(const tt_dbvh *bvh, const tt_ray *h_rays, int64_t n, tt_hit *h_hits, int32_t closest,
                        void *stream) {
    if (!bvh || (!h_rays && n) || (!h_hits && n)) return fail(TT_ERR_INVALID, "null argument");
    if (n == 0) return TT_OK;
    DeviceBVH &d = const_cast<tt_dbvh *>(bvh)->d;
    cudaStream_t s = (cudaStream_t)stream;
    // Coherent rays (a sample of the host buffer decides, as the device probe would) are bound by
    // the transfer in, incoherent ones by the trace.
    const bool sorted_variant = d.variant == VARIANT_SORTED || d.variant == VARIANT_SORTED_OCC;
    const bool coherent = !sorted_variant || n < (int64_t)(1 << 21) ||
                          host_rays_coherent(reinterpret_cast<const float *>(h_rays), n, d.lo, d.hi);
    // Coherent rays in page-locked, device-mapped host buffers: one trace launch that reads the rays
    // and writes the hits across the host link itself (about 208 / 192 GB/s each way on a GB300,
    // the rate the copy engines reach too), so the transfer overlaps traversal with no staging.
    if (coherent && n >= (int64_t)(1 << 21)) {
        const void *dr_mapped = mapped_host_pointer(h_rays), *dh_mapped = mapped_host_pointer(h_hits);
        if (dr_mapped && dh_mapped) {
            tt_status st = launch_trace(d, dr_mapped, n, const_cast<void *>(dh_mapped), closest != 0, false, s, 0, true);
            if (st != TT_OK) return st;
            TT_CUDA(cudaStreamSynchronize(s));
            return read_error_word(d, s);
        }
    }
    const size_t rb = 32ull * n, hb = 8ull * n;
    if (d.d_stage_bytes < rb + hb) {
        if (d.d_stage) cudaFree(d.d_stage);
        d.d_stage = nullptr;
        d.d_stage_bytes = 0;
        cudaError_t e = cudaMalloc(&d.d_stage, rb + hb);
        if (e != cudaSuccess) return fail(TT_ERR_OOM, std::string("cudaMalloc staging: ") + cudaGetErrorString(e));
        d.d_stage_bytes = rb + hb;
    }
    if (!d.pipe_start) {
        for (int i = 0; i < 3; i++) {
            TT_CUDA(cudaStreamCreateWithFlags(&d.pipe[i], cudaStreamNonBlocking));
            TT_CUDA(cudaEventCreateWithFlags(&d.pipe_done[i], cudaEventDisableTiming));
        }
        TT_CUDA(cudaEventCreateWithFlags(&d.pipe_start, cudaEventDisableTiming));
    }
    char *dr = static_cast<char *>(d.d_stage);
    char *dh = dr + rb;
    // Otherwise chunks rotate over three streams so that the copy in of chunk i+1, the trace of
    // chunk i and the copy out of chunk i-1 overlap; everything is ordered after prior work on
    // `stream`. Coherent rays: 1M-ray chunks, traced in their own order. Incoherent ones: chunks of
    // n/16, 3n/16, 6n/16 and the rest, each ordered when the variant orders, so that the trace
    // starts early and the later chunks are large enough for ordering to pay (measured on 4M
    // terrain rays: 2.04 ms against 2.32 ms for 1M chunks).
    const int64_t sched[4] = {n / 16, 3 * (n / 16), 6 * (n / 16), 0};
    // The first failing call stops the issue, but every stream used is still drained before the
    // return, so no copy of the caller's buffers is in flight once the call has returned.
    tt_status st = TT_OK;
    auto cu = [&st](cudaError_t e, const char *what) {
        if (e != cudaSuccess && st == TT_OK) st = cuda_fail(e, what);
        return e == cudaSuccess;
    };
    int used = 0;
    if (cu(cudaEventRecord(d.pipe_start, s), "cudaEventRecord(pipeline start)")) {
        for (int64_t off = 0, k = 0, m = 0; off < n; off += m, k++) {
            if (n < (int64_t)(1 << 21)) m = n;
            else if (coherent) m = (int64_t)(1 << 20);
            else m = k < 3 ? sched[k] : n - off;
            if (m > n - off) m = n - off;
            const int p = (int)(k % 3);
            cudaStream_t ps = d.pipe[p];
            if (k < 3) {
                if (!cu(cudaStreamWaitEvent(ps, d.pipe_start, 0), "cudaStreamWaitEvent(pipeline start)")) break;
                used = (int)k + 1;
            }
            if (!cu(cudaMemcpyAsync(dr + 32 * off, reinterpret_cast<const char *>(h_rays) + 32 * off, 32ull * m,
                                    cudaMemcpyHostToDevice, ps),
                    "cudaMemcpyAsync(rays to the device)"))
                break;
            st = launch_trace(d, dr + 32 * off, m, dh + 8 * off, closest != 0, false, ps, kScratchPipe + p,
                              coherent && n >= (int64_t)(1 << 21));
            if (st != TT_OK) break;
            if (!cu(cudaMemcpyAsync(reinterpret_cast<char *>(h_hits) + 8 * off, dh + 8 * off, 8ull * m,
                                    cudaMemcpyDeviceToHost, ps),
                    "cudaMemcpyAsync(hits to the host)"))
                break;
        }
    }
    for (int p = 0; p < used; p++) cu(cudaStreamSynchronize(d.pipe[p]), "cudaStreamSynchronize(pipeline)");
    cu(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    if (st != TT_OK) return st;
    return read_error_word(d, s);
}

tt_status tt_dbvh_check(const tt_dbvh *bvh, void *stream) {
    if (!bvh) return fail(TT_ERR_INVALID, "null BVH");
    return read_error_word(bvh->d, (cudaStream_t)stream);
}

// tt_trace_host for callers that must not allocate device memory: the BVH arrays are the
// caller's own device memory, and the staging of rays and hits plus the work counter and error
// word live in g_noalloc_scratch. Allocates nothing (no cudaMalloc, cudaFree or library
// allocation). The first call on a device also looks up the staging array's device address.
tt_status tt_trace_host_noalloc(const void *d_nodes, const void *d_vertices, const int32_t *d_tri_indices,
                                const tt_ray *h_rays, int64_t n, tt_hit *h_hits, int32_t closest, void *stream) {
    if (n < 0 || n > kNoAllocMaxRays)
        return fail(TT_ERR_INVALID, "tt_trace_host_noalloc: " + std::to_string(n) +
                                        " rays exceed the allocation-free staging capacity of " +
                                        std::to_string(kNoAllocMaxRays) +
                                        " rays per call; split the batch (or use tt_trace_host)");
    NoAllocDevice nd;
    if (n == 0) return noalloc_setup(nd);  // a warm-up: loads this library's device code here
    if (!d_nodes || !d_vertices || !d_tri_indices || !h_rays || !h_hits)
        return fail(TT_ERR_INVALID, "tt_trace_host_noalloc: null argument");
    if ((reinterpret_cast<uintptr_t>(d_nodes) & 15) || (reinterpret_cast<uintptr_t>(d_vertices) & 15) ||
        (reinterpret_cast<uintptr_t>(d_tri_indices) & 3))
        return fail(TT_ERR_INVALID, "tt_trace_host_noalloc: BVH arrays must be 16-byte (nodes, vertices) and "
                                    "4-byte (triangle indices) aligned");
    tt_status st = noalloc_setup(nd);
    if (st != TT_OK) return st;
    DeviceBVH d;  // a view only: nothing here is owned or freed
    d.view.nodes = static_cast<const float4 *>(d_nodes);
    d.view.verts = static_cast<const float4 *>(d_vertices);
    d.view.norms = nullptr;
    d.view.tri_idx = d_tri_indices;
    d.view.mat_idx = nullptr;
    d.scratch = reinterpret_cast<unsigned long long *>(nd.scratch);
    d.num_sms = nd.num_sms;
    d.variant = VARIANT_WARP_SH16;
    d.blocks_per_sm[VARIANT_WARP_SH16] = nd.blocks_per_sm;
    d.l2_setup = true;  // no L2 window: the call changes no limit of the context
    cudaStream_t s = (cudaStream_t)stream;
    char *dr = reinterpret_cast<char *>(nd.scratch) + kNoAllocHeader;
    char *dh = dr + 32 * (size_t)kNoAllocMaxRays;
    // the header keeps the last call's contents: the error word must start at zero (the launch
    // itself zeroes the work counter)
    TT_CUDA(cudaMemsetAsync(nd.scratch + 8, 0, 8, s));
    cudaError_t e = cudaMemcpyAsync(dr, h_rays, 32ull * n, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) st = cuda_fail(e, "cudaMemcpyAsync(rays to the device)");
    if (st == TT_OK) st = launch_trace(d, dr, n, dh, closest != 0, false, s);
    if (st == TT_OK) {
        e = cudaMemcpyAsync(h_hits, dh, 8ull * n, cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) st = cuda_fail(e, "cudaMemcpyAsync(hits to the host)");
    }
    // drained on failure too: no copy of the caller's buffers stays in flight after the return
    e = cudaStreamSynchronize(s);
    if (st != TT_OK) return st;
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
    return read_error_word(d, s);
}

}  // extern "C"
