// Ray-cast kernels (closest-hit / any-hit) and the device half of the compact BVH.
//
// Kernel shape: persistent warps. The grid is sized to fill every SM (152 on GB300) with
// resident blocks; each warp claims 32 consecutive rays with one atomic on a per-BVH work
// counter, so lane i of a warp always traces ray base+i, as in a one-ray-per-thread launch,
// while warps that finish early take more work instead of idling at the tail.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "tt_internal.h"
#include "tt_traverse.cuh"

namespace tt {

constexpr int kTraceBlock = 128;

struct DeviceBVH {
    BvhView view;
    void *base = nullptr;          // one allocation holding all five arrays
    size_t bytes = 0;
    uint32_t num_nodes = 0, num_verts = 0;
    uint32_t *scratch = nullptr;   // [0] work counter, [1] error word
    int device = 0;
    int num_sms = 0;
    int blocks_per_sm = 0;
    // pinned staging for the host-buffer entry point
    void *h_stage = nullptr;
    size_t h_stage_bytes = 0;
    void *d_stage = nullptr;
    size_t d_stage_bytes = 0;
};

struct TraceArgs {
    BvhView bvh;
    const float4 *rays;  // 2 float4 per ray
    int64_t n;
    void *hits;
    uint32_t *counter;
    uint32_t *err;
};

template <bool kClosest, bool kExt>
__global__ void __launch_bounds__(kTraceBlock) trace_kernel(TraceArgs a) {
    const int lane = threadIdx.x & 31;
    uint32_t err = 0;
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(a.counter, 32u);
        base = __shfl_sync(0xffffffffu, base, 0);
        if ((int64_t)base >= a.n) break;
        const int64_t i = (int64_t)base + lane;
        if (i < a.n) {
            const float4 r0 = __ldg(a.rays + 2 * i);
            const float4 r1 = __ldg(a.rays + 2 * i + 1);
            TraceResult h = traverse<kClosest>(a.bvh, r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w, err);
            int id = -1;
            if (h.addr >= 0) id = __ldg(a.bvh.tri_idx + h.addr);
            if (!kExt) {
                reinterpret_cast<int2 *>(a.hits)[i] = make_int2(id, __float_as_int(h.t));
            } else {
                int mat = -1;
                float nx = 0.f, ny = 0.f, nz = 0.f;
                if (h.addr >= 0) {
                    mat = (int)__ldg(a.bvh.mat_idx + h.addr);
                    hit_normal(a.bvh, h.addr, h.u, h.v, nx, ny, nz);
                }
                tt_hit_ext *o = reinterpret_cast<tt_hit_ext *>(a.hits) + i;
                o->id = id;
                o->mat = mat;
                o->t = h.t;
                o->nx = nx;
                o->ny = ny;
                o->nz = nz;
            }
        }
        __syncwarp();
    }
    if (err) atomicOr(a.err, err);
}

static tt_status cuda_fail(cudaError_t e, const char *what) {
    return fail(TT_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define TT_CUDA(call)                                   \
    do {                                                \
        cudaError_t e_ = (call);                        \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

static tt_status upload(const CompactBVH &b, DeviceBVH &d) {
    int dev = 0;
    TT_CUDA(cudaGetDevice(&dev));
    d.device = dev;
    TT_CUDA(cudaDeviceGetAttribute(&d.num_sms, cudaDevAttrMultiProcessorCount, dev));
    int bps = 0;
    TT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, trace_kernel<true, false>, kTraceBlock, 0));
    d.blocks_per_sm = bps > 0 ? bps : 1;
    const size_t nb = 16ull * b.nodes.size(), vb = 16ull * b.vertices.size(), mb = 16ull * b.normals.size();
    const size_t tb = 4ull * b.tri_idx.size(), ab = 4ull * b.mat_idx.size();
    auto align = [](size_t x) { return (x + 255) & ~size_t(255); };
    d.bytes = align(nb) + align(vb) + align(mb) + align(tb) + align(ab);
    cudaError_t e = cudaMalloc(&d.base, d.bytes);
    if (e != cudaSuccess) return fail(TT_ERR_OOM, std::string("cudaMalloc BVH: ") + cudaGetErrorString(e));
    char *p = static_cast<char *>(d.base);
    d.view.nodes = reinterpret_cast<const float4 *>(p);
    TT_CUDA(cudaMemcpy(p, b.nodes.data(), nb, cudaMemcpyHostToDevice));
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
    e = cudaMalloc(&d.scratch, 256);
    if (e != cudaSuccess) return fail(TT_ERR_OOM, std::string("cudaMalloc scratch: ") + cudaGetErrorString(e));
    TT_CUDA(cudaMemset(d.scratch, 0, 256));
    return TT_OK;
}

static void release(DeviceBVH &d) {
    if (d.base) cudaFree(d.base);
    if (d.scratch) cudaFree(d.scratch);
    if (d.h_stage) cudaFreeHost(d.h_stage);
    if (d.d_stage) cudaFree(d.d_stage);
    d = DeviceBVH();
}

static tt_status launch_trace(const DeviceBVH &d, const void *d_rays, int64_t n, void *d_hits, bool closest,
                              bool ext, cudaStream_t stream) {
    if (n < 0 || n > (int64_t)0xFFFFFFFF - 64) return fail(TT_ERR_INVALID, "ray count out of range");
    if (n == 0) return TT_OK;
    if (!d_rays || !d_hits) return fail(TT_ERR_INVALID, "null ray or hit buffer");
    if ((reinterpret_cast<uintptr_t>(d_rays) & 15) || (reinterpret_cast<uintptr_t>(d_hits) & 7))
        return fail(TT_ERR_INVALID, "ray buffer must be 16-byte aligned and hit buffer 8-byte aligned");
    TT_CUDA(cudaMemsetAsync(d.scratch, 0, 4, stream));
    TraceArgs a;
    a.bvh = d.view;
    a.rays = reinterpret_cast<const float4 *>(d_rays);
    a.n = n;
    a.hits = d_hits;
    a.counter = d.scratch;
    a.err = d.scratch + 1;
    const int64_t warps_needed = (n + 31) / 32;
    int64_t blocks = (int64_t)d.num_sms * d.blocks_per_sm;
    const int64_t max_useful = (warps_needed * 32 + kTraceBlock - 1) / kTraceBlock;
    if (blocks > max_useful) blocks = max_useful;
    if (blocks < 1) blocks = 1;
    if (closest) {
        if (ext) trace_kernel<true, true><<<(unsigned)blocks, kTraceBlock, 0, stream>>>(a);
        else trace_kernel<true, false><<<(unsigned)blocks, kTraceBlock, 0, stream>>>(a);
    } else {
        if (ext) trace_kernel<false, true><<<(unsigned)blocks, kTraceBlock, 0, stream>>>(a);
        else trace_kernel<false, false><<<(unsigned)blocks, kTraceBlock, 0, stream>>>(a);
    }
    TT_CUDA(cudaGetLastError());
    return TT_OK;
}

static tt_status read_error_word(const DeviceBVH &d, cudaStream_t stream) {
    uint32_t w = 0;
    TT_CUDA(cudaMemcpyAsync(&w, d.scratch + 1, 4, cudaMemcpyDeviceToHost, stream));
    TT_CUDA(cudaStreamSynchronize(stream));
    if (w) {
        TT_CUDA(cudaMemsetAsync(d.scratch + 1, 0, 4, stream));
        if (w & kErrStack) return fail(TT_ERR_BOUNDS, "traversal stack overflow (BVH deeper than 66 levels)");
        return fail(TT_ERR_TIMEOUT, "traversal iteration cap reached (corrupt BVH?)");
    }
    return TT_OK;
}

}  // namespace tt

struct tt_dbvh {
    tt::DeviceBVH d;
};

using namespace tt;

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

tt_status tt_trace_host(const tt_dbvh *bvh, const tt_ray *h_rays, int64_t n, tt_hit *h_hits, int32_t closest,
                        void *stream) {
    if (!bvh || (!h_rays && n) || (!h_hits && n)) return fail(TT_ERR_INVALID, "null argument");
    if (n == 0) return TT_OK;
    DeviceBVH &d = const_cast<tt_dbvh *>(bvh)->d;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t rb = 32ull * n, hb = 8ull * n;
    if (d.d_stage_bytes < rb + hb) {
        if (d.d_stage) cudaFree(d.d_stage);
        d.d_stage = nullptr;
        d.d_stage_bytes = 0;
        cudaError_t e = cudaMalloc(&d.d_stage, rb + hb);
        if (e != cudaSuccess) return fail(TT_ERR_OOM, std::string("cudaMalloc staging: ") + cudaGetErrorString(e));
        d.d_stage_bytes = rb + hb;
    }
    char *dr = static_cast<char *>(d.d_stage);
    char *dh = dr + rb;
    TT_CUDA(cudaMemcpyAsync(dr, h_rays, rb, cudaMemcpyHostToDevice, s));
    tt_status st = launch_trace(d, dr, n, dh, closest != 0, false, s);
    if (st != TT_OK) return st;
    TT_CUDA(cudaMemcpyAsync(h_hits, dh, hb, cudaMemcpyDeviceToHost, s));
    TT_CUDA(cudaStreamSynchronize(s));
    return read_error_word(d, s);
}

tt_status tt_dbvh_check(const tt_dbvh *bvh, void *stream) {
    if (!bvh) return fail(TT_ERR_INVALID, "null BVH");
    return read_error_word(bvh->d, (cudaStream_t)stream);
}

}  // extern "C"
