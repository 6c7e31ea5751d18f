// Native path tracer: a wavefront of compacted ray queues on one GB300.
//
// A render (one view, or a batch of views of any sizes and sample counts) is processed in waves
// of up to `wave_paths` paths (path = one sample of one pixel of one view; index space in
// tt_native.cuh). Per wave: raygen, then for each bounce extend (closest hit over the BVH and the
// analytic objects, tt_render_extend.cu) -> shade (emission, environment light sampling with
// MIS, BSDF sampling, Russian roulette; survivors and shadow rays are appended to queues with one
// atomic per warp) -> shadow (any hit), and finally accumulate (each pixel adds its samples in
// sample order, in float or double, so the sum does not depend on how the waves fall). Every
// kernel is a persistent grid that reads its queue length from device memory, so a wave needs no
// host round trip and a whole batch is captured once as a CUDA graph (tt_batch_render). A render
// of more paths than one wave can instead stream them through a pool of wave_paths slots that is
// refilled with new camera paths as paths end (issue_stream, StreamPlan in tt_native.cuh), with
// the same image bits. The launch shape (threads per block, shared-memory traversal stack depth,
// paths per wave, ordered queues, streamed) is a renderer setting that tt_batch_autotune picks by
// timing.
//
// The integrator (all of it built from basic IEEE operations, tt_ptmath.cuh):
//   camera     pinhole of the CameraMeta; pixel (x, y) with y = 0 at the top, jittered by two
//              PCG32 draws; tan(fov/2) evaluated on the host; with aperture > 1e-5 a thin lens
//              (two more draws: a point of the lens disc aimed at the pinhole ray's point on the
//              focal plane, which lies `focal` along the view direction, as in the reference's
//              camera, src/core/RenderKernel.cu:168-184)
//   rng        PCG32, stream = global path index (sample * pixels + pixel), state = frame seed
//   Lambert    cosine sampling (pdf cos/pi), f = albedo/pi
//   GGX        conductor: alpha = roughness^2, Trowbridge-Reitz D, separable Smith G, Schlick F
//              with F0; visible-normal sampling (Heitz 2018, "Sampling the GGX Distribution of
//              Visible Normals"), weight F * G1(wi)
//   dielectric smooth, exact unpolarised Fresnel, reflect with probability F else refract
//   reference  Metal (Phong 30 lobe), Spec (mirror), Refr (dielectric, IOR 1.4), Coat (Fresnel
//   kinds      choice between mirror and Lambert): sampled, treated as specular for MIS
//   env        nearest texel of the equirectangular map in the reference's mapping; light
//              sampling by a 2D CDF over luminance * sin(theta) (FP64 prefix sums, searched
//              between the entries of guide tables); power heuristic MIS between light and BSDF
//              sampling for Lambert and GGX vertices
//   roulette   from rr_depth on, survival max(beta) clamped to [0.05, 1]
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "tt_native.cuh"
#include "tt_nrc_host.h"

namespace tt {

using namespace pt;

constexpr int kShadeBlockMax = 256;
constexpr int kFlagSpecular = 1;  // the last bounce was specular (no light sampling was done)
constexpr int kFlagTrain = 2;     // a radiance-cache training path
constexpr int kFlagRecorded = 4;  // the training path has left its record
constexpr int kFlagsKept = kFlagTrain | kFlagRecorded;  // carried from bounce to bounce

// ---- small helpers ------------------------------------------------------------------------------
__device__ __forceinline__ int warp_append(int *counter, bool pred) {
    const unsigned mask = __ballot_sync(0xffffffffu, pred);
    if (!mask) return -1;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(counter, __popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    return pred ? base + __popc(mask & ((1u << lane) - 1u)) : -1;
}

__device__ __forceinline__ V3 ld3(const float *p) { return V3(p[0], p[1], p[2]); }
__device__ __forceinline__ void st3(float *p, const V3 &v) {
    p[0] = v.x;
    p[1] = v.y;
    p[2] = v.z;
}

// ---- environment ------------------------------------------------------------------------------
__device__ __forceinline__ int env_texel(const EnvView &e, const V3 &d) {
    float u, v;
    dir_to_uv(d, u, v);
    int x = (int)PT_MUL(u, (float)e.w);
    int y = (int)PT_MUL(v, (float)e.h);
    x = x < 0 ? 0 : (x >= e.w ? e.w - 1 : x);
    y = y < 0 ? 0 : (y >= e.h ? e.h - 1 : y);
    return y * e.w + x;
}

__device__ __forceinline__ V3 env_radiance(const EnvView &e, int texel) {
    const float4 c = __ldg(e.tex + texel);
    return V3(PT_MUL(c.x, e.scale), PT_MUL(c.y, e.scale), PT_MUL(c.z, e.scale));
}

// solid-angle pdf of light-sampling direction d (texel index and sin(theta) of d)
__device__ __forceinline__ float env_pdf(const EnvView &e, int texel, float sin_theta) {
    if (sin_theta <= 0.0f) return 0.0f;
    const int y = texel / e.w, x = texel - y * e.w;
    const float pr = PT_SUB(__ldg(e.marg + y + 1), __ldg(e.marg + y));
    const float pc = PT_SUB(__ldg(e.cond + (size_t)y * (e.w + 1) + x + 1), __ldg(e.cond + (size_t)y * (e.w + 1) + x));
    const float jac = PT_DIV((float)e.w * (float)e.h, PT_MUL(PT_MUL(2.0f * kPi, kPi), sin_theta));
    return PT_MUL(PT_MUL(pr, pc), jac);
}

// The smallest i in [lo, hi] with cdf[i + 1] > u, else hi: over [0, n - 1] the inverse CDF.
__device__ __forceinline__ int cdf_search_in(const float *cdf, int lo, int hi, float u) {
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(cdf + mid + 1) <= u) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ int cdf_search(const float *cdf, int n, float u) { return cdf_search_in(cdf, 0, n - 1, u); }

// The same answer, searched between the guide entries of the grid points k / g <= u < (k + 1) / g
// (g a power of two, so u * g and k / g are exact); the answer is monotone in u.
__device__ __forceinline__ int cdf_search_guided(const float *cdf, const int *guide, int g, float u) {
    int k = (int)(u * (float)g);
    k = k < 0 ? 0 : (k >= g ? g - 1 : k);
    return cdf_search_in(cdf, __ldg(guide + k), __ldg(guide + k + 1), u);
}

// Samples a direction by the 2D CDF. Returns pdf (0 = no sample), radiance, direction and the
// chosen texel (-1: a row without power).
__device__ __forceinline__ float env_sample(const EnvView &e, float u1, float u2, V3 &dir, V3 &le, int &texel) {
    const int y = cdf_search_guided(e.marg, e.guide_m, e.gm, u1);
    const float m0 = __ldg(e.marg + y), m1 = __ldg(e.marg + y + 1);
    texel = -1;
    if (!(m1 > m0)) return 0.0f;
    const float *row = e.cond + (size_t)y * (e.w + 1);
    const int x = cdf_search_guided(row, e.guide_c + (size_t)y * (e.gc + 1), e.gc, u2);
    texel = y * e.w + x;
    const float c0 = __ldg(row + x), c1 = __ldg(row + x + 1);
    if (!(c1 > c0)) return 0.0f;
    float dv = PT_DIV(PT_SUB(u1, m0), PT_SUB(m1, m0));
    float du = PT_DIV(PT_SUB(u2, c0), PT_SUB(c1, c0));
    dv = dv < 0.0f ? 0.0f : (dv > 0.99999994f ? 0.99999994f : dv);
    du = du < 0.0f ? 0.0f : (du > 0.99999994f ? 0.99999994f : du);
    const float v = PT_DIV(PT_ADD((float)y, dv), (float)e.h);
    const float u = PT_DIV(PT_ADD((float)x, du), (float)e.w);
    float st;
    dir = uv_to_dir(u, v, st);
    if (st <= 0.0f) return 0.0f;
    le = env_radiance(e, texel);
    const float jac = PT_DIV((float)e.w * (float)e.h, PT_MUL(PT_MUL(2.0f * kPi, kPi), st));
    return PT_MUL(PT_MUL(PT_SUB(m1, m0), PT_SUB(c1, c0)), jac);
}

__device__ __forceinline__ float power_heuristic(float a, float b) {
    const float a2 = PT_MUL(a, a);
    return PT_DIV(a2, PT_FMA(b, b, a2));
}

// ---- BSDFs (local frame: n = +z) ----------------------------------------------------------------
struct BsdfSample {
    V3 wi;        // world direction
    V3 weight;    // f * |cos| / pdf
    float pdf;    // solid-angle pdf, 0 for specular choices
    bool specular;
};

__device__ __forceinline__ float ggx_d(float alpha2, float cos_h) {
    const float c2 = PT_MUL(cos_h, cos_h);
    const float den = PT_FMA(c2, PT_SUB(alpha2, 1.0f), 1.0f);
    return PT_DIV(alpha2, PT_MUL(PT_MUL(kPi, den), den));
}
__device__ __forceinline__ float ggx_g1(float alpha2, float c) {
    const float c2 = PT_MUL(c, c);
    return PT_DIV(PT_MUL(2.0f, c), PT_ADD(c, PT_SQRT(PT_FMA(PT_SUB(1.0f, alpha2), c2, alpha2))));
}
__device__ __forceinline__ V3 schlick(const V3 &f0, float c) {
    const float m = PT_SUB(1.0f, c < 0.0f ? 0.0f : c);
    const float m2 = PT_MUL(m, m);
    const float m5 = PT_MUL(PT_MUL(m2, m2), m);
    return V3(PT_FMA(PT_SUB(1.0f, f0.x), m5, f0.x), PT_FMA(PT_SUB(1.0f, f0.y), m5, f0.y),
              PT_FMA(PT_SUB(1.0f, f0.z), m5, f0.z));
}

// f * cos(wi) and pdf for light sampling (Lambert and GGX only); wo, wi world, n oriented to wo
__device__ __forceinline__ V3 bsdf_eval(const MaterialRec &m, const V3 &n, const V3 &wo, const V3 &wi, float &pdf) {
    const float ci = dot(n, wi);
    pdf = 0.0f;
    if (ci <= 0.0f) return V3(0.f, 0.f, 0.f);
    if (m.kind == MAT_DIFF) {
        pdf = PT_MUL(ci, kInvPi);
        return V3(PT_MUL(PT_MUL(m.color[0], kInvPi), ci), PT_MUL(PT_MUL(m.color[1], kInvPi), ci),
                  PT_MUL(PT_MUL(m.color[2], kInvPi), ci));
    }
    // GGX conductor
    const float co = dot(n, wo);
    if (co <= 0.0f) return V3(0.f, 0.f, 0.f);
    const float alpha = PT_MUL(m.roughness, m.roughness);
    const float a2 = PT_MUL(alpha, alpha);
    const V3 h = normalize(add(wo, wi));
    const float d = ggx_d(a2, dot(n, h));
    const float g1o = ggx_g1(a2, co);
    const float g1i = ggx_g1(a2, ci);
    const V3 f = schlick(V3(m.color[0], m.color[1], m.color[2]), dot(wi, h));
    pdf = PT_DIV(PT_MUL(d, g1o), PT_MUL(4.0f, co));
    const float s = PT_DIV(PT_MUL(PT_MUL(d, g1o), g1i), PT_MUL(4.0f, co));  // D G / (4 co ci) * ci
    return mul(f, s);
}

__device__ __forceinline__ V3 reflect_about(const V3 &wo, const V3 &n) {
    // 2 (wo.n) n - wo
    return sub(mul(n, PT_MUL(2.0f, dot(wo, n))), wo);
}

__device__ __forceinline__ BsdfSample bsdf_sample(const MaterialRec &m, const V3 &n, const V3 &wo, bool entering,
                                                  float u1, float u2, float u3) {
    BsdfSample s;
    s.pdf = 0.0f;
    s.specular = true;
    s.weight = V3(0.f, 0.f, 0.f);
    V3 t, b;
    onb(n, t, b);
    switch (m.kind) {
        case MAT_DIFF: {
            const float r = PT_SQRT(u1);
            float sp, cp;
            sincos(PT_MUL(kTwoPi, u2), sp, cp);
            const V3 l(PT_MUL(r, cp), PT_MUL(r, sp), PT_SQRT(PT_SUB(1.0f, u1)));
            s.wi = to_world(l, t, b, n);
            s.pdf = PT_MUL(l.z, kInvPi);
            s.weight = V3(m.color[0], m.color[1], m.color[2]);
            s.specular = false;
            if (!(l.z > 0.0f)) s.weight = V3(0.f, 0.f, 0.f);
            break;
        }
        case MAT_GGX: {
            const float alpha = PT_MUL(m.roughness, m.roughness);
            const float a2 = PT_MUL(alpha, alpha);
            // wo in the local frame, stretched to the hemisphere configuration
            const V3 wl(dot(wo, t), dot(wo, b), dot(wo, n));
            const V3 vh = normalize(V3(PT_MUL(alpha, wl.x), PT_MUL(alpha, wl.y), wl.z));
            const float lensq = PT_FMA(vh.y, vh.y, PT_MUL(vh.x, vh.x));
            V3 t1 = lensq > 0.0f ? mul(V3(-vh.y, vh.x, 0.0f), PT_DIV(1.0f, PT_SQRT(lensq))) : V3(1.f, 0.f, 0.f);
            const V3 t2 = cross(vh, t1);
            const float r = PT_SQRT(u1);
            float sp, cp;
            sincos(PT_MUL(kTwoPi, u2), sp, cp);
            const float p1 = PT_MUL(r, cp);
            float p2 = PT_MUL(r, sp);
            const float sh = PT_MUL(0.5f, PT_ADD(1.0f, vh.z));
            p2 = PT_FMA(PT_SUB(1.0f, sh), PT_SQRT(PT_FMA(-p1, p1, 1.0f)), PT_MUL(sh, p2));
            const float p3 = PT_SQRT(fmaxf(0.0f, PT_SUB(PT_SUB(1.0f, PT_MUL(p1, p1)), PT_MUL(p2, p2))));
            const V3 nh = madd(vh, p3, madd(t2, p2, mul(t1, p1)));
            const V3 hl = normalize(V3(PT_MUL(alpha, nh.x), PT_MUL(alpha, nh.y), fmaxf(0.0f, nh.z)));
            const V3 h = to_world(hl, t, b, n);
            s.wi = reflect_about(wo, h);
            const float ci = dot(n, s.wi);
            const float co = wl.z;
            s.specular = false;
            if (ci <= 0.0f || co <= 0.0f) {
                s.weight = V3(0.f, 0.f, 0.f);
                break;
            }
            const float g1o = ggx_g1(a2, co);
            const float g1i = ggx_g1(a2, ci);
            const V3 f = schlick(V3(m.color[0], m.color[1], m.color[2]), dot(s.wi, h));
            s.weight = mul(f, g1i);
            s.pdf = PT_DIV(PT_MUL(ggx_d(a2, hl.z), g1o), PT_MUL(4.0f, co));
            break;
        }
        case MAT_DIELECTRIC:
        case MAT_REFR: {
            const float ior = m.kind == MAT_REFR ? 1.4f : m.ior;
            const float eta = entering ? PT_DIV(1.0f, ior) : ior;  // n_incident / n_transmitted
            const float ci = dot(wo, n);
            const float s2t = PT_MUL(PT_MUL(eta, eta), PT_FMA(-ci, ci, 1.0f));
            float F = 1.0f;
            float ct = 0.0f;
            if (s2t < 1.0f) {
                ct = PT_SQRT(PT_SUB(1.0f, s2t));
                const float rs = PT_DIV(PT_FMA(eta, ci, -ct), PT_FMA(eta, ci, ct));
                const float rp = PT_DIV(PT_FMA(-eta, ct, ci), PT_FMA(eta, ct, ci));
                F = PT_MUL(0.5f, PT_FMA(rs, rs, PT_MUL(rp, rp)));
            }
            if (u1 < F) {
                s.wi = reflect_about(wo, n);
            } else {
                // -eta wo + (eta ci - ct) n
                s.wi = madd(n, PT_FMA(eta, ci, -ct), mul(wo, -eta));
            }
            s.weight = V3(1.f, 1.f, 1.f);
            break;
        }
        case MAT_SPEC:
            s.wi = reflect_about(wo, n);
            s.weight = V3(m.color[0], m.color[1], m.color[2]);
            break;
        case MAT_COAT: {
            // the reference's coat: Fresnel (air 1.000293 / coat 1.291) picks mirror or Lambert
            const float ci = dot(wo, n);
            const float eta = PT_DIV(1.000293f, 1.291f);
            const float s2t = PT_MUL(PT_MUL(eta, eta), PT_FMA(-ci, ci, 1.0f));
            float F = 1.0f;
            if (s2t < 1.0f) {
                const float ct = PT_SQRT(PT_SUB(1.0f, s2t));
                const float rs = PT_DIV(PT_FMA(eta, ci, -ct), PT_FMA(eta, ci, ct));
                const float rp = PT_DIV(PT_FMA(-eta, ct, ci), PT_FMA(eta, ct, ci));
                F = PT_MUL(0.5f, PT_FMA(rs, rs, PT_MUL(rp, rp)));
            }
            if (u3 < F) {
                s.wi = reflect_about(wo, n);
                s.weight = V3(m.color2[0], m.color2[1], m.color2[2]);
            } else {
                const float r = PT_SQRT(u1);
                float sp, cp;
                sincos(PT_MUL(kTwoPi, u2), sp, cp);
                s.wi = to_world(V3(PT_MUL(r, cp), PT_MUL(r, sp), PT_SQRT(PT_SUB(1.0f, u1))), t, b, n);
                s.weight = V3(m.color[0], m.color[1], m.color[2]);
            }
            break;
        }
        default:
            break;
    }
    return s;
}

// ---- kernels ------------------------------------------------------------------------------------
// ---- radiance cache hooks ------------------------------------------------------------------------
// One slot of `counter` for each currently active lane (one atomic per converged group).
__device__ __forceinline__ int append_active(int *counter) {
    const unsigned mask = __activemask();
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(counter, __popc(mask));
    base = __shfl_sync(mask, base, leader);
    return base + __popc(mask & ((1u << lane) - 1u));
}

// The feature record of a vertex (layout in tt_nrc.cuh).
__device__ __forceinline__ void cache_record(float *r, const V3 &p, const V3 &wo, const V3 &n, const MaterialRec &m) {
    float rough = 0.0f, a0 = 1.0f, a1 = 1.0f, a2 = 1.0f;
    if (m.kind == MAT_DIFF || m.kind == MAT_GGX || m.kind == MAT_SPEC || m.kind == MAT_COAT) {
        a0 = m.color[0];
        a1 = m.color[1];
        a2 = m.color[2];
    }
    if (m.kind == MAT_DIFF) rough = 1.0f;
    else if (m.kind == MAT_GGX) rough = m.roughness;
    else if (m.kind == MAT_COAT) rough = 0.5f;
    float4 *r4 = reinterpret_cast<float4 *>(r);
    r4[0] = make_float4(p.x, p.y, p.z, wo.x);
    r4[1] = make_float4(wo.y, wo.z, n.x, n.y);
    r4[2] = make_float4(n.z, rough, a0, a1);
    r4[3] = make_float4(a2, (float)m.kind * 0.125f, 0.0f, 0.0f);
}

// The path-spread heuristic of Mueller et al. 2021 ("Real-time Neural Radiance Caching for Path
// Tracing"): at its first vertex a path records its pixel footprint a0 = t^2 / (4 pi cos); at
// vertex n >= 2 its spread is a_n = (sum over the non-specular bounces so far of
// sqrt(t^2 / (pdf cos)))^2, the running sum kept per path. At the first vertex where
// a_n > spread_c a0 a training path leaves a record (once) and goes on; any other path leaves a
// query there and ends (returns true). Records and queries are appended with one atomic per
// converged group of lanes.
__device__ __forceinline__ bool cache_vertex(const NativeArgs &a, int i, int depth, int &flags, float last_pdf, float t,
                                             const V3 &p, const V3 &wo, const V3 &nl, const MaterialRec &m,
                                             const V3 &beta, const V3 &L) {
    const float cos_o = fabsf(dot(nl, wo));
    if (depth == 0) {
        a.ps.a0[i] = cos_o > 0.0f ? PT_DIV(PT_MUL(t, t), PT_MUL(4.0f * kPi, cos_o)) : 3.0e38f;
        a.ps.spread[i] = 0.0f;
        return false;
    }
    if (a.cache.spread_c < 0.0f || (flags & kFlagRecorded)) return false;
    float s_sum = a.ps.spread[i];
    if (last_pdf > 0.0f && cos_o > 0.0f) s_sum = PT_ADD(s_sum, PT_SQRT(PT_DIV(PT_MUL(t, t), PT_MUL(last_pdf, cos_o))));
    a.ps.spread[i] = s_sum;
    if (!(PT_MUL(s_sum, s_sum) > PT_MUL(a.cache.spread_c, a.ps.a0[i]))) return false;
    if (flags & kFlagTrain) {
        flags |= kFlagRecorded;
        const long long gid = a.view0.stream0 + a.wave_first + i;  // the path's stream index
        const long long s = (gid + (long long)a.cache.train_phase) / (long long)a.cache.train_stride -
                            a.cache.train_slot0;
        if (s >= 0 && s < a.cache.train_slots) {
            cache_record(a.cache.s_rec + 16ll * s, p, wo, nl, m);
            a.cache.s_path[s] = i;
            st3(a.cache.s_L + 3ll * s, L);
            st3(a.cache.s_beta + 3ll * s, beta);
        }
        return false;
    }
    const int s = append_active(a.cache.counts + 0);
    cache_record(a.cache.q_rec + 16ll * s, p, wo, nl, m);
    a.cache.q_path[s] = i;
    st3(a.cache.q_beta + 3ll * s, beta);
    return true;
}

// Filled training slots per 1024-slot block.
__global__ void __launch_bounds__(1024) k_cache_count(NativeArgs a) {
    const int s = blockIdx.x * 1024 + threadIdx.x;
    const int filled = __syncthreads_count(s < a.cache.train_slots && a.cache.s_path[s] >= 0);
    if (threadIdx.x == 0) a.cache.block_counts[blockIdx.x] = filled;
}

// The filled training slots, in slot order, into the record arrays the targets and the training
// read; counts[1] = their number.
__global__ void __launch_bounds__(1024) k_cache_compact(NativeArgs a) {
    __shared__ int s_base, s_warp[32];
    const int s = blockIdx.x * 1024 + threadIdx.x, lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        int base = 0;
        for (int b = 0; b < (int)blockIdx.x; b++) base += a.cache.block_counts[b];
        s_base = base;
    }
    const int path = s < a.cache.train_slots ? a.cache.s_path[s] : -1;
    const unsigned ballot = __ballot_sync(0xffffffffu, path >= 0);
    if (lane == 0) s_warp[w] = __popc(ballot);
    __syncthreads();
    if (w == 0) {
        int v = s_warp[lane], x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        s_warp[lane] = x - v;  // exclusive
    }
    __syncthreads();
    const int dst = s_base + s_warp[w] + __popc(ballot & ((1u << lane) - 1u));
    if (path >= 0) {
        const float4 *src = reinterpret_cast<const float4 *>(a.cache.s_rec + 16ll * s);
        float4 *out = reinterpret_cast<float4 *>(a.cache.t_rec + 16ll * dst);
#pragma unroll
        for (int k = 0; k < 4; k++) out[k] = src[k];
        a.cache.t_path[dst] = path;
        for (int c = 0; c < 3; c++) {
            a.cache.t_L[3ll * dst + c] = a.cache.s_L[3ll * s + c];
            a.cache.t_beta[3ll * dst + c] = a.cache.s_beta[3ll * s + c];
        }
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 1023) a.cache.counts[1] = dst + (path >= 0 ? 1 : 0);
}

// Adds throughput x cache radiance of every query to its path.
__global__ void __launch_bounds__(kShadeBlockMax) k_cache_resolve(NativeArgs a) {
    const int n = a.cache.counts[0];
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        float *L = a.ps.L + 3ll * a.cache.q_path[q];
        const float *b = a.cache.q_beta + 3ll * q, *c = a.cache.q_rgb + 3ll * q;
        L[0] = PT_FMA(b[0], c[0], L[0]);
        L[1] = PT_FMA(b[1], c[1], L[1]);
        L[2] = PT_FMA(b[2], c[2], L[2]);
    }
}

// Training targets: the radiance each training path measured from its record vertex on.
__global__ void __launch_bounds__(kShadeBlockMax) k_cache_targets(NativeArgs a) {
    const int n = min(a.cache.counts[1], a.cache.train_cap);
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        const float *L = a.ps.L + 3ll * a.cache.t_path[s];
        for (int c = 0; c < 3; c++) {
            const float b = a.cache.t_beta[3ll * s + c];
            const float v = b > 0.0f ? PT_DIV(PT_SUB(L[c], a.cache.t_L[3ll * s + c]), b) : 0.0f;
            a.cache.t_target[3ll * s + c] = v > 0.0f ? v : 0.0f;
        }
    }
}

__device__ __forceinline__ void put_ray(float4 *rays, int slot, const V3 &o, const V3 &d) {
    rays[2 * slot] = make_float4(o.x, o.y, o.z, d.x);
    rays[2 * slot + 1] = make_float4(d.y, d.z, 0.0f, 1e20f);
}

// The camera ray of path g (batch-global index), its PCG32 state after the jitter (and lens)
// draws and its stream index. cc caches the last view's frame across a thread's paths.
struct CamFrame {
    int v = -1;
    ViewRec vw;
    V3 pos, view, right, up;
};

__device__ __forceinline__ void camera_path(const NativeArgs &a, long long g, CamFrame &cc, V3 &org, V3 &dir,
                                            Rng &rg, long long &gid) {
    const int v = find_view(a, g);
    if (v != cc.v) {
        cc.vw = view_of(a, v);
        cc.pos = V3(cc.vw.pos[0], cc.vw.pos[1], cc.vw.pos[2]);
        cc.view = normalize(V3(cc.vw.view[0], cc.vw.view[1], cc.vw.view[2]));
        cc.right = normalize(cross(cc.view, V3(cc.vw.up[0], cc.vw.up[1], cc.vw.up[2])));
        cc.up = cross(cc.right, cc.view);
        cc.v = v;
    }
    const ViewRec &vw = cc.vw;
    gid = vw.stream0 + (g - vw.first);
    const int pixel = (int)(gid % vw.npix);
    const int px = pixel % vw.width, py = pixel / vw.width;
    rg = pcg32_seed(vw.seed_state, (uint64_t)gid);
    const float jx = uniform(rg), jy = uniform(rg);
    const float sx = PT_SUB(PT_MUL(2.0f, PT_DIV(PT_ADD((float)px, jx), (float)vw.width)), 1.0f);
    const float sy = PT_SUB(1.0f, PT_MUL(2.0f, PT_DIV(PT_ADD((float)py, jy), (float)vw.height)));
    const V3 dp = madd(cc.up, PT_MUL(sy, vw.tany), madd(cc.right, PT_MUL(sx, vw.tanx), cc.view));
    org = cc.pos;
    if (vw.aperture > 1e-5f) {
        // thin lens: aim at the pinhole ray's point on the focal plane from a point of the lens disc
        const V3 focus = madd(dp, vw.focal, cc.pos);
        const float u1 = uniform(rg), u2 = uniform(rg);
        const float r = PT_MUL(vw.aperture, PT_SQRT(u1));
        float sp, cp;
        sincos(PT_MUL(kTwoPi, u2), sp, cp);
        org = madd(cc.up, PT_MUL(r, sp), madd(cc.right, PT_MUL(r, cp), cc.pos));
        dir = normalize(sub(focus, org));
    } else {
        dir = normalize(dp);
    }
}

__device__ __forceinline__ PathState wave_state(const PathSoA &ps) {
    return PathState{ps.beta, ps.L, ps.last_pdf, ps.rng, ps.rng_inc, ps.depth, ps.flags, nullptr};
}

// A new path in state slot i, its camera ray in slot q of `rays`.
__device__ __forceinline__ void start_path(const PathState &S, int i, float4 *rays, int q, const V3 &org,
                                           const V3 &dir, const Rng &rg, int flags) {
    put_ray(rays, q, org, dir);
    st3(S.beta + 3ll * i, V3(1.f, 1.f, 1.f));
    st3(S.L + 3ll * i, V3(0.f, 0.f, 0.f));
    S.rng[i] = rg.state;
    S.rng_inc[i] = rg.inc;
    S.last_pdf[i] = 0.0f;
    S.depth[i] = 0;
    S.flags[i] = flags;
}

// Camera rays of the wave's paths into queue 0.
__global__ void __launch_bounds__(kShadeBlockMax) k_raygen(NativeArgs a) {
    const int stride = gridDim.x * blockDim.x;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.ps.counts[0] = a.wave_paths;
        a.ps.counts[1] = 0;
        a.ps.counts[2] = 0;
        a.ps.counts[3] = 0;
        a.ps.counts[4] = 0;
        atomicAdd(a.stats + 2, (unsigned long long)a.wave_paths);
        if (a.cache.enabled) {
            a.cache.counts[0] = 0;
            a.cache.counts[1] = 0;
        }
    }
    if (a.cache.enabled)  // this wave's training slots start empty
        for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < a.cache.train_slots; s += stride) a.cache.s_path[s] = -1;
    CamFrame cc;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.wave_paths; i += stride) {
        V3 org, dir;
        Rng rg;
        long long gid;
        camera_path(a, a.wave_first + i, cc, org, dir, rg, gid);
        const bool train = a.cache.train && ((unsigned long long)gid + a.cache.train_phase) % a.cache.train_stride == 0;
        start_path(wave_state(a.ps), i, a.ps.ray[0], i, org, dir, rg, kFlagSpecular | (train ? kFlagTrain : 0));
        a.ps.queue[0][i] = i;
    }
}

// ---- streamed renders -------------------------------------------------------------------------
// Per iteration (queue parity c): k_stream_plan (one thread) -> k_accumulate_stream -> k_regen ->
// extend -> k_shade_stream -> shadow. The plan turns the last shade's survivors and ended paths
// into the frontier (all paths below it have ended), the range to accumulate and the refill.

__global__ void k_stream_init(NativeArgs a) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    StreamPlan *pl = a.stream.plan;
    pl->next = 0;
    pl->frontier = 0;
    pl->min_alive = ~0ull;
    pl->acc_lo = pl->acc_hi = 0;
    pl->new_first = 0;
    pl->new_n = pl->new_at = 0;
    for (int k = 0; k < 5; k++) a.ps.counts[k] = 0;
}

// final = 1: no refill, and the frontier must have reached the end of the index space.
__global__ void k_stream_plan(NativeArgs a, int c, int pool, int final) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    StreamPlan *pl = a.stream.plan;
    const int alive = a.ps.counts[c];
    const long long next = pl->next;
    const long long front = pl->min_alive < (unsigned long long)next ? (long long)pl->min_alive : next;
    pl->acc_lo = pl->frontier;
    pl->acc_hi = front;
    pl->frontier = front;
    long long n_new = 0;
    if (!final) {
        n_new = min((long long)(pool - alive), a.stream.total - next);
        n_new = min(n_new, front + a.stream.ring_n - next);  // ring entries not yet accumulated
        n_new = max(n_new, 0ll);
    } else if (front != a.stream.total) {
        atomicOr(a.err, kErrStream);
    }
    pl->new_first = next;
    pl->new_n = (int)n_new;
    pl->new_at = alive;
    pl->next = next + n_new;
    pl->min_alive = ~0ull;
    a.ps.counts[c] = alive + (int)n_new;
}

// The refill: new paths behind the survivors in queue c.
__global__ void __launch_bounds__(kShadeBlockMax) k_regen(NativeArgs a, int c) {
    const StreamPlan *pl = a.stream.plan;
    const int n = pl->new_n, at = pl->new_at;
    const long long first = pl->new_first;
    if (blockIdx.x == 0 && threadIdx.x == 0 && n > 0) atomicAdd(a.stats + 2, (unsigned long long)n);
    const PathState &S = a.stream.st[c];
    CamFrame cc;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const long long g = first + t;
        V3 org, dir;
        Rng rg;
        long long gid;
        camera_path(a, g, cc, org, dir, rg, gid);
        start_path(S, at + t, a.ps.ray[c], at + t, org, dir, rg, kFlagSpecular);
        S.g[at + t] = g;
    }
}

__device__ __forceinline__ float ray_eps(const NativeArgs &a, const V3 &p) {
    const float m = fmaxf(fmaxf(fabsf(p.x), fabsf(p.y)), fabsf(p.z));
    return PT_MUL(a.p.ray_eps, fmaxf(1.0f, m));
}

// kStream: a streamed render. The state is read by queue slot from copy `cur` and written for
// each survivor at its slot of the next queue in copy cur ^ 1; an ended path leaves its radiance
// in the ring, and the survivors report the smallest path index among them. In waves the state
// stays in the path's own slot.
template <bool kStream>
__device__ __forceinline__ void shade_queue(const NativeArgs &a, int cur) {
    const int n = a.ps.counts[cur];
    const int stride = gridDim.x * blockDim.x;
    const int rounds = (n + stride - 1) / stride;
    const bool use_env = a.env.w > 0;
// the state field f this queue reads (kept as kernel-parameter reads, not copied to registers)
#define TT_ST(f) (kStream ? (cur ? a.stream.st[1].f : a.stream.st[0].f) : a.ps.f)
    for (int round = 0, q = blockIdx.x * blockDim.x + threadIdx.x; round < rounds; round++, q += stride) {
        const bool live = q < n;
        bool alive = false;
        bool shadow = false;
        int i = 0;         // state slot
        long long pg = 0;  // kStream: the path's index
        V3 sh_o, sh_d, sh_val, next_o, next_d;
        // kStream: what a survivor carries to its slot of the next queue
        V3 out_beta, out_L;
        uint64_t out_rng = 0, out_inc = 0;
        int out_depth = 0, flags_next = 0;
        float pdf_next = 0.0f;
        if (live) {
            i = kStream ? q : a.ps.queue[cur][q];
            if (kStream) pg = (cur ? a.stream.st[1].g : a.stream.st[0].g)[i];
            Rng g;
            g.state = TT_ST(rng)[i];
            g.inc = TT_ST(rng_inc)[i];
            const float4 r0 = a.ps.ray[cur][2 * q], r1 = a.ps.ray[cur][2 * q + 1];
            const V3 o(r0.x, r0.y, r0.z), d(r0.w, r1.x, r1.y);
            V3 beta = ld3(TT_ST(beta) + 3ll * i), L = ld3(TT_ST(L) + 3ll * i);
            const int prim = a.ps.hit_prim[q];
            int flags = TT_ST(flags)[i];
            const float last_pdf = TT_ST(last_pdf)[i];
            int depth = TT_ST(depth)[i];
            if (prim == -1) {
                if (use_env) {
                    const int texel = env_texel(a.env, d);
                    V3 le = env_radiance(a.env, texel);
                    float w = 1.0f;
                    if (!(flags & kFlagSpecular)) {
                        const float st = PT_SQRT(fmaxf(0.0f, PT_FMA(-d.y, d.y, 1.0f)));
                        w = power_heuristic(last_pdf, env_pdf(a.env, texel, st));
                    }
                    L = madd(mul(beta, le), w, L);
                }
            } else {
                const float t = a.ps.hit_t[q];
                const V3 p = madd(d, t, o);
                V3 n;
                int mat;
                if (prim >= 0) {
                    hit_normal(a.bvh, prim, a.ps.hit_u[q], a.ps.hit_v[q], n.x, n.y, n.z);
                    mat = (int)__ldg(a.bvh.mat_idx + prim);
                } else {
                    const GeomRec g2 = a.geoms[-prim - 2];
                    mat = g2.mat;
                    if (g2.kind == GEOM_PLANE) {
                        const V3 p0(g2.p0[0], g2.p0[1], g2.p0[2]);
                        n = cross(sub(V3(g2.p1[0], g2.p1[1], g2.p1[2]), p0), sub(V3(g2.p2[0], g2.p2[1], g2.p2[2]), p0));
                    } else {
                        n = sub(p, V3(g2.p0[0], g2.p0[1], g2.p0[2]));
                    }
                }
                n = normalize(n);
                const V3 wo(-d.x, -d.y, -d.z);
                const bool entering = dot(n, wo) > 0.0f;
                const V3 nl = entering ? n : V3(-n.x, -n.y, -n.z);
                MaterialRec m;
                if (mat >= 0 && mat < a.num_materials) m = a.materials[mat];
                else memset(&m, 0, sizeof(m));
                if (m.kind == MAT_METAL) {
                    // native Metal: the reference's Phong lobe (exponent 30) as the GGX lobe of
                    // about the same width (alpha = sqrt(2 / (n + 2)) = 0.25), F0 = colour
                    m.kind = MAT_GGX;
                    m.roughness = 0.5f;
                }
                L = V3(PT_FMA(beta.x, m.emission[0], L.x), PT_FMA(beta.y, m.emission[1], L.y),
                       PT_FMA(beta.z, m.emission[2], L.z));
                bool cache_end = false;
                if (a.cache.enabled) cache_end = cache_vertex(a, i, depth, flags, last_pdf, t, p, wo, nl, m, beta, L);
                const bool nee = !cache_end && use_env && !(a.p.flags & TT_RENDER_NO_ENV_SAMPLING) &&
                                 (m.kind == MAT_DIFF || m.kind == MAT_GGX);
                const float eps = ray_eps(a, p);
                if (nee) {
                    const float u1 = uniform(g), u2 = uniform(g);
                    V3 wi, le;
                    int texel;
                    const float pl = env_sample(a.env, u1, u2, wi, le, texel);
                    if (pl > 0.0f) {
                        float pb;
                        const V3 fc = bsdf_eval(m, nl, wo, wi, pb);
                        if (maxc(fc) > 0.0f) {
                            const float w = power_heuristic(pl, pb);
                            sh_val = mul(mul(beta, mul(fc, le)), PT_DIV(w, pl));
                            sh_o = madd(nl, eps, p);
                            sh_d = wi;
                            shadow = true;
                        }
                    }
                }
                const float u1 = cache_end ? 0.0f : uniform(g), u2 = cache_end ? 0.0f : uniform(g),
                            u3 = cache_end ? 0.0f : uniform(g);
                const BsdfSample bs = bsdf_sample(m, nl, wo, entering, u1, u2, u3);
                if (!cache_end && maxc(bs.weight) > 0.0f) {
                    beta = mul(beta, bs.weight);
                    depth++;
                    alive = depth < a.p.max_depth;
                    if (alive && depth >= a.p.rr_depth) {
                        float q_surv = maxc(beta);
                        q_surv = q_surv > 1.0f ? 1.0f : (q_surv < 0.05f ? 0.05f : q_surv);
                        if (uniform(g) >= q_surv) alive = false;
                        else beta = mul(beta, PT_DIV(1.0f, q_surv));
                    }
                    if (alive) {
                        const V3 off = dot(bs.wi, nl) >= 0.0f ? nl : V3(-nl.x, -nl.y, -nl.z);
                        next_o = madd(off, eps, p);
                        next_d = bs.wi;
                        if (kStream) {
                            pdf_next = bs.pdf;
                            flags_next = (flags & kFlagsKept) | ((bs.specular || !nee) ? kFlagSpecular : 0);
                        } else {
                            st3(TT_ST(beta) + 3ll * i, beta);
                            TT_ST(last_pdf)[i] = bs.pdf;
                            TT_ST(flags)[i] = (flags & kFlagsKept) | ((bs.specular || !nee) ? kFlagSpecular : 0);
                            TT_ST(depth)[i] = depth;
                        }
                    }
                }
            }
            if (kStream) {
                out_beta = beta;
                out_L = L;
                out_rng = g.state;
                out_inc = g.inc;
                out_depth = depth;
            } else {
                st3(TT_ST(L) + 3ll * i, L);
                TT_ST(rng)[i] = g.state;
            }
        }
        const int slot = warp_append(a.ps.counts + (cur ^ 1), alive);
        if (alive) {
            if (!kStream) a.ps.queue[cur ^ 1][slot] = i;
            put_ray(a.ps.ray[cur ^ 1], slot, next_o, next_d);
            if (kStream) {
                const PathState &N = cur ? a.stream.st[0] : a.stream.st[1];
                st3(N.beta + 3ll * slot, out_beta);
                st3(N.L + 3ll * slot, out_L);
                N.rng[slot] = out_rng;
                N.rng_inc[slot] = out_inc;
                N.last_pdf[slot] = pdf_next;
                N.flags[slot] = flags_next;
                N.depth[slot] = out_depth;
                N.g[slot] = pg;
            }
        }
        long long ring_e = 0;
        if (kStream && live && !alive) {
            ring_e = pg % a.stream.ring_n;
            st3(a.stream.ring + 3 * ring_e, out_L);
        }
        const int sslot = warp_append(a.ps.counts + 2, shadow);
        if (shadow) {
            // the shadow stage adds to L[3 * t] of the state it is given for t >= 0, else to ring
            // entry -1 - t
            a.ps.shadow_path[sslot] = !kStream ? i : (alive ? slot : (int)(-1 - ring_e));
            put_ray(a.ps.shadow_ray, sslot, sh_o, sh_d);
            st3(a.ps.shadow_val + 3ll * sslot, sh_val);
        }
        if (kStream) {
            unsigned long long m = alive ? (unsigned long long)pg : ~0ull;
            for (int o = 16; o > 0; o >>= 1) {
                const unsigned long long other = __shfl_xor_sync(0xffffffffu, m, o);
                m = other < m ? other : m;
            }
            if ((threadIdx.x & 31) == 0 && m != ~0ull) atomicMin(&a.stream.plan->min_alive, m);
        }
    }
#undef TT_ST
}

__global__ void __launch_bounds__(kShadeBlockMax) k_shade(NativeArgs a, int cur) { shade_queue<false>(a, cur); }

__global__ void __launch_bounds__(kShadeBlockMax) k_shade_stream(NativeArgs a, int cur) { shade_queue<true>(a, cur); }

// Adds the radiance of paths [first, first + n) to the views' accumulation blocks. The thread of
// a pixel's first path in the range adds all of that pixel's paths in the range, in sample order,
// so the sums do not depend on how a render is cut into ranges. kRing: path g's radiance is at
// ring entry g mod ring_n, else at L[g - first].
template <typename T, bool kRing>
__device__ __forceinline__ void accumulate_range(const NativeArgs &a, T *accum, long long first, long long n,
                                                 const float *L) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const long long g = first + i;
        const ViewRec vw = view_of(a, find_view(a, g));
        const long long l = g - vw.first;
        if (l >= vw.npix && g - vw.npix >= first) continue;  // not the pixel's first path here
        const long long pixel = l % vw.npix;
        T *px = accum + vw.accum + 3 * pixel;
        T acc[3] = {px[0], px[1], px[2]};
        for (long long k = i, lk = l; k < n && lk < vw.paths; k += vw.npix, lk += vw.npix) {
            const long long e = kRing ? (first + k) % a.stream.ring_n : k;
            acc[0] += (T)L[3 * e];
            acc[1] += (T)L[3 * e + 1];
            acc[2] += (T)L[3 * e + 2];
        }
        px[0] = acc[0];
        px[1] = acc[1];
        px[2] = acc[2];
    }
}

template <typename T>
__global__ void __launch_bounds__(kShadeBlockMax) k_accumulate(NativeArgs a, T *accum) {
    accumulate_range<T, false>(a, accum, a.wave_first, a.wave_paths, a.ps.L);
}

template <typename T>
__global__ void __launch_bounds__(kShadeBlockMax) k_accumulate_stream(NativeArgs a, T *accum) {
    const long long lo = a.stream.plan->acc_lo, hi = a.stream.plan->acc_hi;
    accumulate_range<T, true>(a, accum, lo, hi - lo, a.stream.ring);
}

}  // namespace tt

// ---- sampling probe (tt_native_sample_probe) ------------------------------------------------------
namespace tt {
__global__ void k_sample_probe(const MaterialRec *materials, int num_materials, EnvView env, int what,
                               tt_sample_probe *q, long long n) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        tt_sample_probe r = q[i];
        if (what == 2) {
            Rng g = pcg32_seed(r.pcg_state, r.pcg_seq);
            for (int k = 0; k < 8; k++) r.pcg_out[k] = pcg32(g);
        } else if (what == 1) {
            V3 dir(0.f, 0.f, 0.f), le(0.f, 0.f, 0.f);
            r.texel = -1;
            r.pdf = env.w > 0 ? env_sample(env, r.u[0], r.u[1], dir, le, r.texel) : 0.0f;
            st3(r.wi, dir);
            st3(r.weight, le);
            const float st = PT_SQRT(fmaxf(0.0f, PT_FMA(-dir.y, dir.y, 1.0f)));
            r.eval_pdf = r.pdf > 0.0f ? env_pdf(env, env_texel(env, dir), st) : 0.0f;
        } else if (r.material >= 0 && r.material < num_materials) {
            const MaterialRec m = materials[r.material];
            const V3 nn = ld3(r.n), wo = ld3(r.wo);
            const BsdfSample s = bsdf_sample(m, nn, wo, r.entering != 0, r.u[0], r.u[1], r.u[2]);
            st3(r.wi, s.wi);
            st3(r.weight, s.weight);
            r.pdf = s.pdf;
            r.specular = s.specular ? 1 : 0;
            float ep = 0.0f;
            V3 ev(0.f, 0.f, 0.f);
            if (m.kind == MAT_DIFF || m.kind == MAT_GGX) ev = bsdf_eval(m, nn, wo, s.wi, ep);
            st3(r.eval, ev);
            r.eval_pdf = ep;
        }
        q[i] = r;
    }
}
}  // namespace tt

// ---- environment sampling tables (FP64 prefix sums) ----------------------------------------------
namespace tt {

// One thread per row, sequential prefix sums in double: weight = luminance * sin(theta_row).
__global__ void k_env_rows(const float4 *tex, int w, int h, float *cond, double *rowsum) {
    const int y = blockIdx.x * blockDim.x + threadIdx.x;
    if (y >= h) return;
    float st, ct;
    sincos(PT_MUL(PT_DIV(PT_ADD((float)y, 0.5f), (float)h), kPi), st, ct);
    // first pass: the row total; second pass: the same prefix sums, normalised by it
    double acc = 0.0;
    float *row = cond + (size_t)y * (w + 1);
    row[0] = 0.0f;
    for (int x = 0; x < w; x++) {
        const float4 c = tex[(size_t)y * w + x];
        const float wt = PT_MUL(luminance(c.x, c.y, c.z), st);
        acc += (double)(wt > 0.0f ? wt : 0.0f);
    }
    rowsum[y] = acc;
    double acc2 = 0.0;
    for (int x = 0; x < w; x++) {
        const float4 c = tex[(size_t)y * w + x];
        const float wt = PT_MUL(luminance(c.x, c.y, c.z), st);
        acc2 += (double)(wt > 0.0f ? wt : 0.0f);
        row[x + 1] = acc > 0.0 ? __double2float_rn(acc2 / acc) : PT_DIV((float)(x + 1), (float)w);
    }
}

// Guide entries: the full search's answer at u = k / gm (marginal) and k / gc (each row).
__global__ void k_env_guides(const float *marg, const float *cond, int w, int h, int gm, int gc, int *guide) {
    const long long n = (long long)(gm + 1) + (long long)h * (gc + 1);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        if (i <= gm) {
            guide[i] = cdf_search(marg, h, (float)i * (1.0f / (float)gm));
        } else {
            const long long j = i - (gm + 1);
            const int y = (int)(j / (gc + 1)), k = (int)(j % (gc + 1));
            guide[i] = cdf_search(cond + (size_t)y * (w + 1), w, (float)k * (1.0f / (float)gc));
        }
    }
}

__global__ void k_env_marginal(const double *rowsum, int h, float *marg) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    double total = 0.0;
    for (int y = 0; y < h; y++) total += rowsum[y];
    double acc = 0.0;
    marg[0] = 0.0f;
    for (int y = 0; y < h; y++) {
        acc += rowsum[y];
        marg[y + 1] = total > 0.0 ? __double2float_rn(acc / total) : PT_DIV((float)(y + 1), (float)h);
    }
}

static tt_status cuda_fail_n(cudaError_t e, const char *what) {
    return fail(TT_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define TT_CUDA_N(call)                                       \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return cuda_fail_n(e_, #call); \
    } while (0)

// Median-split box hierarchy over more than kGeomBrute analytic objects (leaves of at most
// kGeomLeaf; an inner node records its split axis for the warp's near-first order).
// Each box is grown by 1e-4 of its extent plus its largest coordinate, so that a hit point the
// exact float tests accept always lies inside its object's box.
// At 8 objects the loop is about 5% faster than the hierarchy, at 64 they are level, at 512 the
// hierarchy is 1.5x and at 4096 4.9x faster (512x512 pixels, 8 samples, random spheres).
constexpr int kGeomBrute = 32;
constexpr int kGeomLeaf = 4;

static void geom_box(const GeomRec &g, float lo[3], float hi[3]) {
    for (int k = 0; k < 3; k++) {
        if (g.kind == GEOM_SPHERE) {
            lo[k] = g.p0[k] - g.radius;
            hi[k] = g.p0[k] + g.radius;
        } else {  // parallelogram p0, p1, p2, p1 + p2 - p0
            const float p3 = g.p1[k] + g.p2[k] - g.p0[k];
            lo[k] = std::min(std::min(g.p0[k], g.p1[k]), std::min(g.p2[k], p3));
            hi[k] = std::max(std::max(g.p0[k], g.p1[k]), std::max(g.p2[k], p3));
        }
    }
    float ext = 0.0f, mag = 0.0f;
    for (int k = 0; k < 3; k++) {
        ext = std::max(ext, hi[k] - lo[k]);
        mag = std::max(mag, std::max(std::fabs(lo[k]), std::fabs(hi[k])));
    }
    const float pad = 1e-4f * (ext + mag) + 1e-6f;
    for (int k = 0; k < 3; k++) {
        lo[k] -= pad;
        hi[k] += pad;
    }
}

static tt_status build_geom_tree(tt_renderer *r, const std::vector<GeomRec> &geoms) {
    const int n = (int)geoms.size();
    if (n <= kGeomBrute) return TT_OK;
    std::vector<std::array<float, 6>> box(n);
    std::vector<int> idx(n);
    for (int i = 0; i < n; i++) {
        geom_box(geoms[i], box[i].data(), box[i].data() + 3);
        idx[i] = i;
    }
    std::vector<GeomNode> nodes(1);
    struct Item {
        int node, b, e;
    };
    std::vector<Item> todo{{0, 0, n}};
    while (!todo.empty()) {
        const Item it = todo.back();
        todo.pop_back();
        GeomNode nd;
        float clo[3] = {3e38f, 3e38f, 3e38f}, chi[3] = {-3e38f, -3e38f, -3e38f};
        for (int k = 0; k < 3; k++) {
            nd.lo[k] = 3e38f;
            nd.hi[k] = -3e38f;
        }
        for (int j = it.b; j < it.e; j++)
            for (int k = 0; k < 3; k++) {
                const auto &bx = box[idx[j]];
                nd.lo[k] = std::min(nd.lo[k], bx[k]);
                nd.hi[k] = std::max(nd.hi[k], bx[3 + k]);
                const float c = 0.5f * (bx[k] + bx[3 + k]);
                clo[k] = std::min(clo[k], c);
                chi[k] = std::max(chi[k], c);
            }
        if (it.e - it.b <= kGeomLeaf) {
            nd.first = it.b;
            nd.count = it.e - it.b;
        } else {
            int axis = 0;
            for (int k = 1; k < 3; k++)
                if (chi[k] - clo[k] > chi[axis] - clo[axis]) axis = k;
            const int mid = (it.b + it.e) / 2;
            std::nth_element(idx.begin() + it.b, idx.begin() + mid, idx.begin() + it.e, [&](int x, int y) {
                const float cx = box[x][axis] + box[x][3 + axis], cy = box[y][axis] + box[y][3 + axis];
                return cx < cy || (cx == cy && x < y);
            });
            nd.first = (int)nodes.size();
            nd.count = -1 - axis;
            nodes.resize(nodes.size() + 2);
            todo.push_back({nd.first + 1, mid, it.e});
            todo.push_back({nd.first, it.b, mid});
        }
        nodes[it.node] = nd;
    }
    const size_t nb = sizeof(GeomNode) * nodes.size(), ib = sizeof(int) * idx.size();
    TT_CUDA_N(cudaMalloc(&r->geom_tree, nb + ib));
    TT_CUDA_N(cudaMemcpy(r->geom_tree, nodes.data(), nb, cudaMemcpyHostToDevice));
    TT_CUDA_N(cudaMemcpy(static_cast<char *>(r->geom_tree) + nb, idx.data(), ib, cudaMemcpyHostToDevice));
    r->num_geom_nodes = (int)nodes.size();
    return TT_OK;
}

tt_status native_setup(tt_renderer *r, const std::vector<GeomRec> &geoms) {
    int dev = 0;
    TT_CUDA_N(cudaGetDevice(&dev));
    TT_CUDA_N(cudaDeviceGetAttribute(&r->num_sms, cudaDevAttrMultiProcessorCount, dev));
    const tt_status gst = build_geom_tree(r, geoms);
    if (gst != TT_OK) return gst;
    if (r->env_w <= 0) return TT_OK;
    const int w = r->env_w, h = r->env_h;
    TT_CUDA_N(cudaMalloc(&r->env_marg, sizeof(float) * (h + 1)));
    TT_CUDA_N(cudaMalloc(&r->env_cond, sizeof(float) * (size_t)h * (w + 1)));
    double *rowsum = nullptr;
    TT_CUDA_N(cudaMalloc(&rowsum, sizeof(double) * h));
    k_env_rows<<<(h + 127) / 128, 128>>>(r->env, w, h, r->env_cond, rowsum);
    k_env_marginal<<<1, 1>>>(rowsum, h, r->env_marg);
    auto pow2_at_least = [](int x) {
        int p = 1;
        while (p < x) p <<= 1;
        return p;
    };
    r->env_gm = pow2_at_least(h);
    r->env_gc = pow2_at_least(std::max(1, w / 4));
    const long long guides = (long long)(r->env_gm + 1) + (long long)h * (r->env_gc + 1);
    TT_CUDA_N(cudaMalloc(&r->env_guide, sizeof(int) * guides));
    k_env_guides<<<(unsigned)std::min<long long>((guides + 255) / 256, 4096), 256>>>(
        r->env_marg, r->env_cond, w, h, r->env_gm, r->env_gc, r->env_guide);
    cudaError_t e = cudaDeviceSynchronize();
    cudaFree(rowsum);
    if (e != cudaSuccess) return cuda_fail_n(e, "environment tables");
    return TT_OK;
}

void native_release(tt_renderer *r) {
    if (r->env_marg) cudaFree(r->env_marg);
    if (r->env_cond) cudaFree(r->env_cond);
    if (r->env_guide) cudaFree(r->env_guide);
    r->env_guide = nullptr;
    if (r->paths) cudaFree(r->paths);
    if (r->cache_mem) cudaFree(r->cache_mem);
    if (r->stream_mem) cudaFree(r->stream_mem);
    if (r->geom_tree) cudaFree(r->geom_tree);
    r->geom_tree = nullptr;
    r->num_geom_nodes = 0;
    r->env_marg = r->env_cond = nullptr;
    r->paths = nullptr;
    r->paths_bytes = 0;
    r->path_capacity = 0;
    r->cache_mem = nullptr;
    r->cache_bytes = 0;
    r->stream_mem = nullptr;
    r->stream_bytes = 0;
}

// Path state for `cap` paths, carved out of one allocation sized for the renderer's capacity (so
// the pointers, which captured graphs hold, change only when the allocation does).
static tt_status ensure_paths(tt_renderer *r, int cap, PathSoA &ps) {
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    constexpr int kArrays = 21;
    auto layout = [&](size_t n, size_t *sizes) {
        const size_t s[kArrays] = {12 * n, 12 * n, 8 * n, 8 * n,  4 * n,  4 * n, 4 * n, 4 * n, 4 * n, 32 * n, 32 * n,
                                   4 * n,  4 * n,  4 * n, 4 * n, 64,     4 * n, 32 * n, 12 * n, 4 * n, 4 * n};
        size_t total = 0;
        for (int i = 0; i < kArrays; i++) {
            sizes[i] = s[i];
            total += al(s[i]);
        }
        return total;
    };
    size_t sizes[kArrays];
    // the ordering scratch of the extension queues follows the arrays when ordering is on
    const bool want_order = r->launch_order != 0;
    if (r->path_capacity < cap || !r->paths || (want_order && !r->order_off)) {
        const int c = std::max(cap, r->path_capacity);
        const size_t arrays = layout((size_t)c, sizes);
        const size_t total = arrays + (want_order ? reorder_scratch_bytes(c) : 0);
        cap = c;
        if (r->paths) cudaFree(r->paths);
        r->paths = nullptr;
        r->paths_bytes = 0;
        r->path_capacity = 0;
        cudaError_t e = cudaMalloc(&r->paths, total);
        if (e != cudaSuccess) return fail(TT_ERR_OOM, std::string("path state: ") + cudaGetErrorString(e));
        r->paths_bytes = total;
        r->path_capacity = cap;
        r->paths_gen++;
        r->order_off = want_order ? arrays : 0;
        r->order_state_at = want_order ? reorder_state_offset(c) : 0;
        if (want_order) {  // the ordering state starts at zero
            e = cudaMemset(static_cast<char *>(r->paths) + r->order_off + r->order_state_at, 0, 256);
            if (e != cudaSuccess) return fail(TT_ERR_CUDA, std::string("path state: ") + cudaGetErrorString(e));
        }
    }
    layout((size_t)r->path_capacity, sizes);
    char *p = static_cast<char *>(r->paths);
    void *v[kArrays];
    for (int i = 0; i < kArrays; i++) {
        v[i] = p;
        p += al(sizes[i]);
    }
    ps.beta = (float *)v[0];
    ps.L = (float *)v[1];
    ps.rng = (uint64_t *)v[2];
    ps.rng_inc = (uint64_t *)v[3];
    ps.last_pdf = (float *)v[4];
    ps.depth = (int *)v[5];
    ps.flags = (int *)v[6];
    ps.queue[0] = (int *)v[7];
    ps.queue[1] = (int *)v[8];
    ps.ray[0] = (float4 *)v[9];
    ps.ray[1] = (float4 *)v[10];
    ps.hit_t = (float *)v[11];
    ps.hit_u = (float *)v[12];
    ps.hit_v = (float *)v[13];
    ps.hit_prim = (int *)v[14];
    ps.counts = (int *)v[15];
    ps.shadow_path = (int *)v[16];
    ps.shadow_ray = (float4 *)v[17];
    ps.shadow_val = (float *)v[18];
    ps.a0 = (float *)v[19];
    ps.spread = (float *)v[20];
    return TT_OK;
}

constexpr int kMaxWavePaths = 1 << 26;

static int block_index(int block) {
    for (int i = 0; i < kNumBlockShapes; i++)
        if (kBlockShapes[i] == block) return i;
    return -1;
}
static int stack_index(int sh) {
    for (int i = 0; i < kNumStackShapes; i++)
        if (kStackShapes[i] == sh) return i;
    return -1;
}

// A launch shape resolved to kernels and persistent grid sizes.
struct Launch {
    TraceKernels tk;
    int block = 0, wave = 0;
    int grid_trace = 0, grid_shade = 0, grid_gather = 0;
    bool order = false;  // order the extension queues (scratch in the path allocation)
    bool stream = true;  // stream a render of more paths than one wave (StreamPlan)
};

// Where a render's queue ordering works: the scratch inside the path allocation and the scene
// bounds of the origin grid (scratch = nullptr: the allocation has none).
struct OrderPlan {
    void *scratch = nullptr;
    size_t state_at = 0;
    const float *lo = nullptr, *hi = nullptr;
};

static OrderPlan order_plan(const tt_renderer *r) {
    OrderPlan o;
    if (r->order_off) {
        o.scratch = static_cast<char *>(r->paths) + r->order_off;
        o.state_at = r->order_state_at;
        o.lo = r->order_lo;
        o.hi = r->order_hi;
    }
    return o;
}

static tt_status resolve_launch(tt_renderer *r, int block, int sh, int wave, int order, int stream, Launch &L) {
    const int bi = block_index(block), si = stack_index(sh);
    if (bi < 0 || si < 0 || wave < 1 || wave > kMaxWavePaths || (order != 0 && order != 1) ||
        (stream != 0 && stream != 1))
        return fail(TT_ERR_INVALID, "launch shape: block must be 64/128/256, stack_shared 0/8/16, "
                                    "wave_paths 1..67108864, ordered and streamed 0 or 1");
    L.stream = stream != 0;
    L.tk = trace_kernels(block, sh);
    L.block = block;
    L.wave = wave;
    L.order = order != 0;
    if (!r->occ_trace[bi][si]) {
        int b = 0;
        TT_CUDA_N(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, (const void *)L.tk.extend, block, 0));
        int b2 = 0;
        TT_CUDA_N(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b2, (const void *)L.tk.shadow, block, 0));
        r->occ_trace[bi][si] = std::max(1, std::min(b, b2));
    }
    if (!r->occ_shade[bi]) {
        int b = 0, b2 = 0;
        TT_CUDA_N(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, (const void *)k_shade, block, 0));
        TT_CUDA_N(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b2, (const void *)k_shade_stream, block, 0));
        r->occ_shade[bi] = std::max(1, std::min(b, b2));
    }
    L.grid_trace = r->num_sms * r->occ_trace[bi][si];
    L.grid_shade = r->num_sms * r->occ_shade[bi];
    L.grid_gather = r->num_sms * 8;
    return TT_OK;
}

static ViewRec make_view(const tt_camera_meta &cam, int spp, int sample_offset, uint32_t seed, long long first,
                         long long accum) {
    ViewRec v;
    std::memset(&v, 0, sizeof(v));
    v.width = cam.width;
    v.height = cam.height;
    v.npix = cam.width * cam.height;
    v.first = first;
    v.paths = (long long)v.npix * spp;
    v.accum = accum;
    v.stream0 = (long long)sample_offset * v.npix;
    v.seed_state = (uint64_t)seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
    for (int k = 0; k < 3; k++) {
        v.pos[k] = cam.position[k];
        v.view[k] = cam.view[k];
        v.up[k] = cam.up[k];
    }
    v.tanx = (float)std::tan((double)cam.fov[0] * 0.5 * 3.14159265358979323846 / 180.0);
    v.tany = (float)std::tan((double)cam.fov[1] * 0.5 * 3.14159265358979323846 / 180.0);
    v.aperture = cam.aperture;
    v.focal = cam.focal;
    return v;
}

static tt_status check_view(const tt_camera_meta &cam, int spp, int sample_offset) {
    if (cam.width <= 0 || cam.height <= 0 || spp < 1 || sample_offset < 0)
        return fail(TT_ERR_INVALID, "bad image size, spp or sample offset");
    if ((long long)cam.width * cam.height > (1ll << 30)) return fail(TT_ERR_INVALID, "image too large");
    if ((long long)cam.width * cam.height * ((long long)sample_offset + spp) > (1ll << 62))
        return fail(TT_ERR_INVALID, "sample index out of range");
    return TT_OK;
}

static tt_status check_params(const tt_render_params &p) {
    if (p.max_depth < 1 || p.max_depth > 1024) return fail(TT_ERR_INVALID, "max_depth must be in 1..1024");
    return TT_OK;
}

static NativeArgs base_args(tt_renderer *r, const tt_render_params &p, const PathSoA &ps) {
    NativeArgs a;
    std::memset(&a, 0, sizeof(a));
    a.bvh = r->bvh;
    a.materials = r->materials;
    a.num_materials = r->num_materials;
    a.geoms = r->geoms;
    a.num_geoms = r->num_geoms;
    if (r->geom_tree) {
        a.gnodes = static_cast<const GeomNode *>(r->geom_tree);
        a.gidx = reinterpret_cast<const int *>(static_cast<const char *>(r->geom_tree) +
                                               sizeof(GeomNode) * r->num_geom_nodes);
    }
    a.env.tex = r->env;
    a.env.marg = r->env_marg;
    a.env.cond = r->env_cond;
    a.env.guide_m = r->env_guide;
    a.env.guide_c = r->env_guide ? r->env_guide + r->env_gm + 1 : nullptr;
    a.env.gm = r->env_gm;
    a.env.gc = r->env_gc;
    a.env.w = r->env_w;
    a.env.h = r->env_h;
    a.env.scale = p.env_scale;
    a.ps = ps;
    a.p = p;
    a.err = r->err;
    a.stats = renderer_stats(r);
    return a;
}

// Issues the kernels of `total` paths (waves of L.wave) on stream s. accum = nullptr: no
// accumulation (autotuning trials). cache: the radiance cache of a cached render (a.cache set up),
// queried after the second bounce and trained after every wave when `train`.
// Whether shade can queue shadow rays: they sample the environment light.
static bool has_shadows(const NativeArgs &a) { return a.env.w > 0 && !(a.p.flags & TT_RENDER_NO_ENV_SAMPLING); }

// Orders the shadow queue (a.ps.counts[2] rays of at most cap) for the shadow stage.
static tt_status order_shadows(NativeArgs &a, long long cap, const OrderPlan &plan, cudaStream_t s) {
    OrderOut so;
    const tt_status st = reorder_rays(a.ps.shadow_ray, cap, a.ps.counts + 2, plan.lo, plan.hi, plan.scratch,
                                      plan.state_at, a.err, s, &so, true);
    if (st != TT_OK) return st;
    a.shadow_order.sorted = so.sorted;
    a.shadow_order.src = so.src;
    a.shadow_order.state = so.state;
    return TT_OK;
}

static tt_status issue_waves(NativeArgs a, long long total, const Launch &L, const OrderPlan &plan, void *accum,
                             cudaStream_t s, tt_renderer *r, tt_cache *cache, bool train) {
    const bool f64 = (a.p.flags & TT_RENDER_ACCUM_F64) != 0;
    if (L.order && !plan.scratch) return fail(TT_ERR_INVALID, "queue ordering: no scratch for it");
    const long long qcap = std::min<long long>(L.wave, total);  // queue capacity: the path arrays' size
    for (long long done = 0; done < total; done += L.wave) {
        a.wave_first = done;
        a.wave_paths = (int)std::min<long long>(total - done, L.wave);
        if (cache) {
            const long long tp = nrc::cache_params(cache).train_paths;
            a.cache.train_stride = (unsigned)std::max<long long>(1, (a.wave_paths + tp - 1) / tp);
            a.cache.train_phase = (unsigned)((a.view0.stream0 / std::max(1, a.view0.npix) + done) * 7 %
                                             a.cache.train_stride);
            // slots of the wave's training paths: stream indices g with (g + phase) % stride == 0
            const long long st = (long long)a.cache.train_stride, ph = (long long)a.cache.train_phase;
            const long long g0 = a.view0.stream0 + done, g1 = g0 + a.wave_paths - 1;
            a.cache.train_slot0 = (g0 + ph + st - 1) / st;
            a.cache.train_slots = (int)std::max<long long>(0, (g1 + ph) / st - a.cache.train_slot0 + 1);
            if (a.cache.train_slots > a.cache.train_cap)
                return fail(TT_ERR_INVALID, "cache: more training paths in a wave than training slots");
        }
        k_raygen<<<L.grid_shade, L.block, 0, s>>>(a);
        r->launches += 1 + (accum ? 1 : 0) + (unsigned long long)a.p.max_depth * (L.order ? (has_shadows(a) ? 12 : 8) : 3);
        for (int b = 0; b < a.p.max_depth; b++) {
            if (L.order) {  // order the queue; the probe leaves coherent queues (camera rays) alone
                OrderOut oo;
                const tt_status st = reorder_rays(a.ps.ray[b & 1], qcap, a.ps.counts + (b & 1), plan.lo, plan.hi,
                                                  plan.scratch, plan.state_at, a.err, s, &oo);
                if (st != TT_OK) return st;
                float *h = static_cast<float *>(oo.sorted_hits);
                a.order.n_sorted = a.ps.counts + (b & 1);
                a.order.sorted = oo.sorted;
                a.order.pos = oo.pos;
                a.order.state = oo.state;
                a.order.hit_t = h;
                a.order.hit_u = h + qcap;
                a.order.hit_v = h + 2 * qcap;
                a.order.hit_prim = reinterpret_cast<int *>(h + 3 * qcap);
            }
            L.tk.extend<<<L.grid_trace, L.block, 0, s>>>(a, b & 1);
            if (L.order) k_order_gather_hits<<<L.grid_gather, 256, 0, s>>>(a, b & 1);
            k_shade<<<L.grid_shade, L.block, 0, s>>>(a, b & 1);
            if (L.order && has_shadows(a)) {  // the shadow queue too (scratch shared with the extension queue's)
                const tt_status st = order_shadows(a, qcap, plan, s);
                if (st != TT_OK) return st;
            }
            L.tk.shadow<<<L.grid_trace, L.block, 0, s>>>(a);
        }
        if (cache) {  // every path queries at most once, so all queries of the wave fit
            const tt_status st = nrc::cache_infer_device(cache, a.cache.q_rec, a.cache.counts, a.wave_paths,
                                                         a.cache.q_rgb, nrc::cache_params(cache).use_ema, a.err, s);
            if (st != TT_OK) return st;
            k_cache_resolve<<<L.grid_shade, L.block, 0, s>>>(a);
            r->launches += 1;
        }
        if (cache && train) {
            if (a.cache.train_slots > 0) {  // the records in slot order
                const unsigned nb = (unsigned)((a.cache.train_slots + 1023) / 1024);
                k_cache_count<<<nb, 1024, 0, s>>>(a);
                k_cache_compact<<<nb, 1024, 0, s>>>(a);
                r->launches += 2;
            }
            k_cache_targets<<<L.grid_shade, L.block, 0, s>>>(a);
            r->launches += 1;
        }
        if (accum) {
            if (f64) k_accumulate<double><<<L.grid_shade, L.block, 0, s>>>(a, (double *)accum);
            else k_accumulate<float><<<L.grid_shade, L.block, 0, s>>>(a, (float *)accum);
        }
        if (cache && train) {
            const tt_status st = nrc::cache_train_device(cache, a.cache.t_rec, a.cache.t_target, a.cache.counts + 1, s);
            if (st != TT_OK) return st;
        }
    }
    TT_CUDA_N(cudaGetLastError());
    return TT_OK;
}

// Radiance ring entries of a streamed render of pool slots and max_depth bounces (0: too many to
// stream; such renders run in waves).
constexpr long long kMaxRingEntries = 1ll << 29;
static long long stream_ring_entries(long long pool, int max_depth) {
    const long long n = pool * (long long)max_depth;
    return n <= kMaxRingEntries ? n : 0;
}

// The streamed render's buffers for `pool` slots and `ring` entries, carved out of one allocation
// that only grows (a reallocation bumps paths_gen, so captured graphs are rebuilt): the ring, the
// second copy of the path state (the first is the wave arrays of `ps`) and both copies' path
// indices.
static tt_status ensure_stream(tt_renderer *r, const PathSoA &ps, long long pool, long long ring, StreamView &sv) {
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    constexpr int kArrays = 11;
    const size_t P = (size_t)pool;
    const size_t sizes[kArrays] = {12ull * (size_t)ring, 12 * P, 12 * P, 4 * P, 8 * P, 8 * P, 4 * P, 4 * P,
                                   8 * P, 8 * P, sizeof(StreamPlan)};
    size_t need = 0;
    for (size_t x : sizes) need += al(x);
    if (r->stream_bytes < need) {
        if (r->stream_mem) cudaFree(r->stream_mem);
        r->stream_mem = nullptr;
        r->stream_bytes = 0;
        const cudaError_t e = cudaMalloc(&r->stream_mem, need);
        if (e != cudaSuccess) return fail(TT_ERR_OOM, std::string("streamed render: ") + cudaGetErrorString(e));
        r->stream_bytes = need;
        r->paths_gen++;
    }
    char *p = static_cast<char *>(r->stream_mem);
    void *v[kArrays];
    for (int k = 0; k < kArrays; k++) {
        v[k] = p;
        p += al(sizes[k]);
    }
    sv.ring = (float *)v[0];
    sv.ring_n = ring;
    sv.st[0] = PathState{ps.beta, ps.L, ps.last_pdf, ps.rng, ps.rng_inc, ps.depth, ps.flags, (long long *)v[8]};
    sv.st[1] = PathState{(float *)v[1], (float *)v[2], (float *)v[3], (uint64_t *)v[4], (uint64_t *)v[5],
                         (int *)v[6], (int *)v[7], (long long *)v[9]};
    sv.plan = (StreamPlan *)v[10];
    return TT_OK;
}

// A streamed render of `total` paths through a pool of L.wave slots (see StreamPlan). The
// iteration count is an upper bound fixed on the host, so the sequence can be captured. Path g
// starts by the plan of iteration floor(g / pool) * max_depth (every earlier generation of pool
// paths has ended by then, leaving it a slot and ring room) and ends within max_depth iterations,
// so ceil(total / pool) * max_depth iterations end every path; the max_depth more issued here are
// slack. Iterations after the last path ends find empty queues and return at once. The final
// plan flags the error word if any path had not ended.
static tt_status issue_stream(NativeArgs a, long long total, const Launch &L, const OrderPlan &plan, void *accum,
                              cudaStream_t s, tt_renderer *r) {
    const bool f64 = (a.p.flags & TT_RENDER_ACCUM_F64) != 0;
    if (L.order && !plan.scratch) return fail(TT_ERR_INVALID, "queue ordering: no scratch for it");
    const long long pool = L.wave;
    StreamView sv{};
    tt_status st = ensure_stream(r, a.ps, pool, stream_ring_entries(pool, a.p.max_depth), sv);
    if (st != TT_OK) return st;
    sv.total = total;
    a.stream = sv;
    const long long iters = (total + pool - 1) / pool * a.p.max_depth + a.p.max_depth;
    // init; per iteration plan, accumulate, refill, extend, shade, shadow (+ 4 ordering kernels
    // and the hit gather for the extension queue, 4 for the shadow queue); the final plan and
    // accumulate
    r->launches += 1 + (unsigned long long)iters * ((accum ? 6 : 5) + (L.order ? (has_shadows(a) ? 9 : 5) : 0)) +
                   (accum ? 2 : 1);
    k_stream_init<<<1, 32, 0, s>>>(a);
    for (long long it = 0; it <= iters; it++) {
        const int c = (int)(it & 1);
        const bool last = it == iters;
        k_stream_plan<<<1, 32, 0, s>>>(a, c, (int)pool, last ? 1 : 0);
        if (accum) {
            if (f64) k_accumulate_stream<double><<<L.grid_shade, L.block, 0, s>>>(a, (double *)accum);
            else k_accumulate_stream<float><<<L.grid_shade, L.block, 0, s>>>(a, (float *)accum);
        }
        if (last) break;
        k_regen<<<L.grid_shade, L.block, 0, s>>>(a, c);
        if (L.order) {
            // the survivors (queue slots below new_at) are ordered; the new camera rays behind
            // them are coherent already
            OrderOut oo;
            const int *n_sorted = &sv.plan->new_at;
            st = reorder_rays(a.ps.ray[c], pool, n_sorted, plan.lo, plan.hi, plan.scratch, plan.state_at, a.err, s, &oo);
            if (st != TT_OK) return st;
            float *h = static_cast<float *>(oo.sorted_hits);
            a.order.n_sorted = n_sorted;
            a.order.sorted = oo.sorted;
            a.order.pos = oo.pos;
            a.order.state = oo.state;
            a.order.hit_t = h;
            a.order.hit_u = h + pool;
            a.order.hit_v = h + 2 * pool;
            a.order.hit_prim = reinterpret_cast<int *>(h + 3 * pool);
        }
        (L.order ? L.tk.extend_prefix : L.tk.extend)<<<L.grid_trace, L.block, 0, s>>>(a, c);
        if (L.order) k_order_gather_hits<<<L.grid_gather, 256, 0, s>>>(a, c);
        k_shade_stream<<<L.grid_shade, L.block, 0, s>>>(a, c);
        if (L.order && has_shadows(a)) {
            st = order_shadows(a, pool, plan, s);
            if (st != TT_OK) return st;
        }
        NativeArgs as = a;  // shadow rays of survivors add to their state in the next queue
        as.ps.L = sv.st[c ^ 1].L;
        L.tk.shadow<<<L.grid_trace, L.block, 0, s>>>(as);
    }
    TT_CUDA_N(cudaGetLastError());
    return TT_OK;
}

// Issues the kernels of `total` paths on stream s: streamed through a pool of L.wave slots when
// they are more than one wave (plain renders), else in waves.
static bool streamed(long long total, const Launch &L, int max_depth, const tt_cache *cache) {
    return L.stream && !cache && total > L.wave && stream_ring_entries(L.wave, max_depth) > 0;
}

static tt_status issue(NativeArgs a, long long total, const Launch &L, const OrderPlan &plan, void *accum,
                       cudaStream_t s, tt_renderer *r, tt_cache *cache = nullptr, bool train = false) {
    if (streamed(total, L, a.p.max_depth, cache)) return issue_stream(a, total, L, plan, accum, s, r);
    return issue_waves(a, total, L, plan, accum, s, r, cache, train);
}

// Query and training buffers of a cached render: `queries` query slots, `records` training slots.
static tt_status ensure_cache_buffers(tt_renderer *r, long long queries, long long records, CacheView &cv) {
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t q = (size_t)queries, t = (size_t)records;
    const size_t sizes[] = {64 * q, 4 * q, 12 * q, 12 * q, 64 * t, 4 * t, 12 * t, 12 * t, 12 * t, 256,
                            64 * t, 4 * t, 12 * t, 12 * t, 4 * (t / 1024 + 1)};
    size_t total = 0;
    for (size_t s : sizes) total += al(s);
    if (r->cache_bytes < total || r->cache_queries < queries || r->cache_records < records) {
        if (r->cache_mem) cudaFree(r->cache_mem);
        r->cache_mem = nullptr;
        r->cache_bytes = 0;
        cudaError_t e = cudaMalloc(&r->cache_mem, total);
        if (e != cudaSuccess) return fail(TT_ERR_OOM, std::string("cache buffers: ") + cudaGetErrorString(e));
        r->cache_bytes = total;
        r->cache_queries = queries;
        r->cache_records = records;
    }
    char *p = static_cast<char *>(r->cache_mem);
    int k = 0;
    auto take = [&]() {
        char *x = p;
        p += al(sizes[k++]);
        return x;
    };
    cv.q_rec = (float *)take();
    cv.q_path = (int *)take();
    cv.q_beta = (float *)take();
    cv.q_rgb = (float *)take();
    cv.t_rec = (float *)take();
    cv.t_path = (int *)take();
    cv.t_L = (float *)take();
    cv.t_beta = (float *)take();
    cv.t_target = (float *)take();
    cv.counts = (int *)take();
    cv.s_rec = (float *)take();
    cv.s_path = (int *)take();
    cv.s_L = (float *)take();
    cv.s_beta = (float *)take();
    cv.block_counts = (int *)take();
    cv.train_cap = (int)records;
    return TT_OK;
}

}  // namespace tt

// A compiled batch of views: the device view table and, once rendered, the captured graph.
struct tt_batch {
    tt_renderer *r = nullptr;
    std::vector<tt::ViewRec> views;
    tt::ViewRec *d_views = nullptr;
    long long total_paths = 0;
    long long accum_elems = 0;
    tt_render_params p{};
    cudaStream_t cap = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    void *graph_accum = nullptr;
    int graph_block = 0, graph_stack = -1, graph_wave = 0, graph_order = -1, graph_stream = -1;
    unsigned long long graph_paths_gen = 0;
    int graph_kernels = 0;
};

namespace tt {

static void drop_graph(tt_batch *b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    b->graph_accum = nullptr;
}

static NativeArgs batch_args(tt_batch *b, const PathSoA &ps) {
    NativeArgs a = base_args(b->r, b->p, ps);
    a.views = b->d_views;
    a.n_views = (int)b->views.size();
    a.view0 = b->views[0];
    return a;
}

}  // namespace tt

using namespace tt;

extern "C" {

tt_status tt_render_params_default(tt_render_params *out) {
    if (!out) return fail(TT_ERR_INVALID, "null argument");
    out->spp = 1;
    out->sample_offset = 0;
    out->max_depth = 8;
    out->rr_depth = 4;
    out->seed = 1;
    out->env_scale = 1.0f;
    out->ray_eps = 1e-4f;
    out->flags = 0;
    return TT_OK;
}

tt_status tt_render_native(tt_renderer *r, const tt_camera_meta *cam, const tt_render_params *p, void *d_accum,
                           void *stream) {
    if (!r || !cam || !p || !d_accum) return fail(TT_ERR_INVALID, "null argument");
    tt_status st = check_view(*cam, p->spp, p->sample_offset);
    if (st == TT_OK) st = check_params(*p);
    if (st != TT_OK) return st;
    const ViewRec v = make_view(*cam, p->spp, p->sample_offset, p->seed, 0, 0);
    Launch L;
    st = resolve_launch(r, r->launch_block, r->launch_stack, r->launch_wave, r->launch_order, r->launch_stream, L);
    if (st != TT_OK) return st;
    PathSoA ps;
    st = ensure_paths(r, (int)std::min<long long>(v.paths, L.wave), ps);
    if (st != TT_OK) return st;
    NativeArgs a = base_args(r, *p, ps);
    a.views = nullptr;
    a.n_views = 1;
    a.view0 = v;
    return issue(a, v.paths, L, order_plan(r), d_accum, (cudaStream_t)stream, r);
}

tt_status tt_render_cached(tt_renderer *r, tt_cache *c, const tt_camera_meta *cam, const tt_render_params *p,
                           void *d_accum, int32_t train, void *stream) {
    if (!r || !c || !cam || !p || !d_accum) return fail(TT_ERR_INVALID, "null argument");
    tt_status st = check_view(*cam, p->spp, p->sample_offset);
    if (st == TT_OK) st = check_params(*p);
    if (st != TT_OK) return st;
    const tt_cache_params &cp = nrc::cache_params(c);
    const ViewRec v = make_view(*cam, p->spp, p->sample_offset, p->seed, 0, 0);
    Launch L;
    st = resolve_launch(r, r->launch_block, r->launch_stack, r->launch_wave, r->launch_order, r->launch_stream, L);
    if (st != TT_OK) return st;
    const int wave = (int)std::min<long long>(v.paths, L.wave);
    PathSoA ps;
    st = ensure_paths(r, wave, ps);
    if (st != TT_OK) return st;
    NativeArgs a = base_args(r, *p, ps);
    a.views = nullptr;
    a.n_views = 1;
    a.view0 = v;
    const long long records = std::max<long long>(cp.train_paths, (long long)cp.steps * cp.batch);
    st = ensure_cache_buffers(r, wave, records, a.cache);
    if (st != TT_OK) return st;
    a.cache.enabled = 1;
    a.cache.train = train ? 1 : 0;
    a.cache.spread_c = cp.spread_c;
    a.cache.train_stride = 1;
    return issue(a, v.paths, L, order_plan(r), d_accum, (cudaStream_t)stream, r, c, train != 0);
}

tt_status tt_renderer_set_launch(tt_renderer *r, const tt_launch_shape *shape) {
    if (!r || !shape) return fail(TT_ERR_INVALID, "null argument");
    Launch L;
    tt_status st = resolve_launch(r, shape->block, shape->stack_shared, shape->wave_paths, shape->ordered,
                                  shape->streamed, L);
    if (st != TT_OK) return st;
    r->launch_block = shape->block;
    r->launch_stack = shape->stack_shared;
    r->launch_wave = shape->wave_paths;
    r->launch_order = shape->ordered;
    r->launch_stream = shape->streamed;
    return TT_OK;
}

tt_status tt_renderer_get_launch(const tt_renderer *r, tt_launch_shape *shape) {
    if (!r || !shape) return fail(TT_ERR_INVALID, "null argument");
    shape->block = r->launch_block;
    shape->stack_shared = r->launch_stack;
    shape->wave_paths = r->launch_wave;
    shape->ordered = r->launch_order;
    shape->streamed = r->launch_stream;
    shape->ms = 0.0f;
    return TT_OK;
}

tt_status tt_renderer_launches(tt_renderer *r, uint64_t *out, int32_t reset) {
    if (!r || !out) return fail(TT_ERR_INVALID, "null argument");
    *out = r->launches;
    if (reset) r->launches = 0;
    return TT_OK;
}

tt_status tt_renderer_stats(tt_renderer *r, uint64_t *out, int reset) {
    if (!r || !out) return fail(TT_ERR_INVALID, "null argument");
    unsigned long long s[3];
    TT_CUDA_N(cudaMemcpy(s, renderer_stats(r), sizeof(s), cudaMemcpyDeviceToHost));
    for (int i = 0; i < 3; i++) out[i] = s[i];
    if (reset) TT_CUDA_N(cudaMemset(renderer_stats(r), 0, sizeof(s)));
    return TT_OK;
}

tt_status tt_batch_create(tt_renderer *r, const tt_view *views, int n, const tt_render_params *p, tt_batch **out) {
    if (!r || !views || !p || !out) return fail(TT_ERR_INVALID, "null argument");
    *out = nullptr;
    if (n < 1) return fail(TT_ERR_INVALID, "a batch needs at least one view");
    tt_status st = check_params(*p);
    if (st != TT_OK) return st;
    tt_batch *b = new tt_batch();
    b->r = r;
    b->p = *p;
    b->views.reserve(n);
    for (int k = 0; k < n; k++) {
        st = check_view(views[k].cam, views[k].spp, views[k].sample_offset);
        if (st != TT_OK) {
            delete b;
            return fail(TT_ERR_INVALID, "view " + std::to_string(k) + ": " + tt_last_error_string());
        }
        b->views.push_back(
            make_view(views[k].cam, views[k].spp, views[k].sample_offset, views[k].seed, b->total_paths, b->accum_elems));
        b->total_paths += b->views.back().paths;
        b->accum_elems += 3ll * b->views.back().npix;
    }
    cudaError_t e = cudaMalloc((void **)&b->d_views, sizeof(ViewRec) * n);
    if (e == cudaSuccess) e = cudaMemcpy(b->d_views, b->views.data(), sizeof(ViewRec) * n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        tt_batch_free(b);
        return cuda_fail_n(e, "batch view table");
    }
    *out = b;
    return TT_OK;
}

tt_status tt_batch_info(const tt_batch *b, int64_t *total_paths, int64_t *accum_elems) {
    if (!b) return fail(TT_ERR_INVALID, "null batch");
    if (total_paths) *total_paths = b->total_paths;
    if (accum_elems) *accum_elems = b->accum_elems;
    return TT_OK;
}

tt_status tt_batch_render(tt_batch *b, void *d_accum, int use_graph, void *stream) {
    if (!b || !d_accum) return fail(TT_ERR_INVALID, "null argument");
    tt_renderer *r = b->r;
    Launch L;
    tt_status st = resolve_launch(r, r->launch_block, r->launch_stack, r->launch_wave, r->launch_order, r->launch_stream, L);
    if (st != TT_OK) return st;
    PathSoA ps;
    st = ensure_paths(r, (int)std::min<long long>(b->total_paths, L.wave), ps);
    if (st != TT_OK) return st;
    if (streamed(b->total_paths, L, b->p.max_depth, nullptr)) {  // allocate before any capture
        StreamView sv;
        st = ensure_stream(r, ps, L.wave, stream_ring_entries(L.wave, b->p.max_depth), sv);
        if (st != TT_OK) return st;
    }
    const NativeArgs a = batch_args(b, ps);
    if (!use_graph) return issue(a, b->total_paths, L, order_plan(r), d_accum, (cudaStream_t)stream, r);
    const bool stale = !b->exec || b->graph_accum != d_accum || b->graph_block != L.block ||
                       b->graph_stack != r->launch_stack || b->graph_wave != L.wave || b->graph_order != r->launch_order ||
                       b->graph_stream != r->launch_stream ||
                       b->graph_paths_gen != r->paths_gen;
    if (stale) {
        drop_graph(b);
        TT_CUDA_N(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal));
        st = issue(a, b->total_paths, L, order_plan(r), d_accum, b->cap, r);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(b->cap, &g);
        if (st != TT_OK) {
            if (g) cudaGraphDestroy(g);
            return st;
        }
        if (e != cudaSuccess) return cuda_fail_n(e, "capturing the batch");
        b->graph = g;
        const cudaError_t e2 = cudaGraphInstantiate(&b->exec, g, 0);
        if (e2 != cudaSuccess) {
            drop_graph(b);
            return cuda_fail_n(e2, "instantiating the batch graph");
        }
        size_t nodes = 0;
        cudaGraphGetNodes(g, nullptr, &nodes);
        b->graph_kernels = (int)nodes;
        b->graph_accum = d_accum;
        b->graph_block = L.block;
        b->graph_stack = r->launch_stack;
        b->graph_wave = L.wave;
        b->graph_order = r->launch_order;
        b->graph_stream = r->launch_stream;
        b->graph_paths_gen = r->paths_gen;
    }
    TT_CUDA_N(cudaGraphLaunch(b->exec, (cudaStream_t)stream));
    return TT_OK;
}

tt_status tt_batch_graph_kernels(const tt_batch *b, int *kernels) {
    if (!b || !kernels) return fail(TT_ERR_INVALID, "null argument");
    *kernels = b->exec ? b->graph_kernels : 0;
    return TT_OK;
}

tt_status tt_batch_autotune(tt_batch *b, int64_t sample_paths, void *stream, tt_launch_shape *results, int max_results,
                            int *n_results) {
    if (!b) return fail(TT_ERR_INVALID, "null batch");
    tt_renderer *r = b->r;
    cudaStream_t s = (cudaStream_t)stream;
    // stage 2 times `sample` paths, stage 1 a quarter of them (at least 2^22): a wave's last bounces
    // trace few rays at the latency of the longest ones, so larger waves (or a streamed pool) pay
    // that tail less often, and the sample has to span several of the largest waves to show it
    const long long sample = std::min<long long>(b->total_paths, sample_paths > 0 ? sample_paths : (1ll << 28));
    const long long sample1 = std::min<long long>(sample, std::max<long long>(sample / 4, 1ll << 22));
    static const int kWaves[] = {1 << 20, 1 << 22, 1 << 24, 1 << 26};
    PathSoA ps;
    const int order_was = r->launch_order;
    r->launch_order = 1;  // the trials with ordered queues need its scratch
    tt_status st = ensure_paths(r, (int)std::min<long long>(sample, kWaves[3]), ps);
    r->launch_order = order_was;
    if (st != TT_OK) return st;
    NativeArgs a = batch_args(b, ps);
    const OrderPlan plan = order_plan(r);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    TT_CUDA_N(cudaEventCreate(&e0));
    TT_CUDA_N(cudaEventCreate(&e1));
    float best = 3.4e38f;
    tt_launch_shape best_shape{r->launch_block, r->launch_stack, r->launch_wave, r->launch_order, r->launch_stream, 0.0f};
    int count = 0;
    // times n paths under one shape (buffers allocated before the timed region)
    auto trial = [&](long long n, int block, int sh, int wave, int order, int strm) -> tt_status {
        Launch L;
        tt_status t = resolve_launch(r, block, sh, wave, order, strm, L);
        if (t == TT_OK && streamed(n, L, b->p.max_depth, nullptr)) {
            StreamView sv;
            t = ensure_stream(r, ps, wave, stream_ring_entries(wave, b->p.max_depth), sv);
        }
        if (t == TT_OK) t = issue(a, std::min<long long>(n, 1 << 16), L, plan, nullptr, s, r);  // warm-up
        cudaError_t e = cudaEventRecord(e0, s);
        if (t == TT_OK && e == cudaSuccess) t = issue(a, n, L, plan, nullptr, s, r);
        if (e == cudaSuccess) e = cudaEventRecord(e1, s);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (t != TT_OK) return t;
        if (e != cudaSuccess) return cuda_fail_n(e, "autotune timing");
        const tt_launch_shape shape{block, sh, wave, order, strm, ms};
        if (results && count < max_results) results[count] = shape;
        count++;
        if (ms < best) {
            best = ms;
            best_shape = shape;
        }
        return TT_OK;
    };
    // stage 1: threads per block x shared stack entries, at 2^22-path waves, ordered and streamed
    for (int bi = 0; bi < kNumBlockShapes && st == TT_OK; bi++)
        for (int si = 0; si < kNumStackShapes && st == TT_OK; si++)
            st = trial(sample1, kBlockShapes[bi], kStackShapes[si], kWaves[1], 1, 1);
    // stage 2: the fastest of those at every wave size, ordered or not, streamed or in waves (a
    // sample that fits one wave is the same either way); the renderer keeps the fastest of these
    const int bb = best_shape.block, bs = best_shape.stack_shared;
    best = 3.4e38f;
    for (int wave : kWaves)
        for (int order = 0; order < 2; order++)
            for (int strm = 0; strm < 2; strm++) {
                if (st != TT_OK) break;
                if (wave > kWaves[0] && wave / 2 >= sample) continue;  // the same as a smaller wave
                if (strm && sample <= wave) continue;
                st = trial(sample, bb, bs, wave, order, strm);
            }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != TT_OK) return st;
    r->launch_block = best_shape.block;
    r->launch_stack = best_shape.stack_shared;
    r->launch_wave = best_shape.wave_paths;
    r->launch_order = best_shape.ordered;
    r->launch_stream = best_shape.streamed;
    if (n_results) *n_results = count;
    return TT_OK;
}

tt_status tt_batch_free(tt_batch *b) {
    if (!b) return TT_OK;
    drop_graph(b);
    if (b->d_views) cudaFree(b->d_views);
    if (b->cap) cudaStreamDestroy(b->cap);
    delete b;
    return TT_OK;
}

tt_status tt_native_sample_probe(const tt_renderer *r, int32_t what, tt_sample_probe *d_q, int64_t n, void *stream) {
    static_assert(sizeof(tt_sample_probe) == 160, "tt_sample_probe is 160 bytes");
    if (!r || (n > 0 && !d_q)) return fail(TT_ERR_INVALID, "null argument");
    if (what < 0 || what > 2) return fail(TT_ERR_INVALID, "what must be 0 (BSDF), 1 (environment) or 2 (PCG32)");
    if (what == 1 && r->env_w <= 0) return fail(TT_ERR_INVALID, "the scene has no environment map");
    if (n < 0) return fail(TT_ERR_INVALID, "negative query count");
    if (n == 0) return TT_OK;
    EnvView env{};
    env.tex = r->env;
    env.marg = r->env_marg;
    env.cond = r->env_cond;
    env.guide_m = r->env_guide;
    env.guide_c = r->env_guide ? r->env_guide + r->env_gm + 1 : nullptr;
    env.gm = r->env_gm;
    env.gc = r->env_gc;
    env.w = r->env_w;
    env.h = r->env_h;
    env.scale = 1.0f;
    const long long blocks = std::min<long long>((n + 255) / 256, 152ll * 16);
    k_sample_probe<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(r->materials, r->num_materials, env, what, d_q,
                                                                       (long long)n);
    TT_CUDA_N(cudaGetLastError());
    return TT_OK;
}

tt_status tt_renderer_env_tables(const tt_renderer *r, float *marginal, float *conditional) {
    if (!r) return fail(TT_ERR_INVALID, "null renderer");
    if (r->env_w <= 0) return fail(TT_ERR_INVALID, "the scene has no environment map");
    if (marginal) TT_CUDA_N(cudaMemcpy(marginal, r->env_marg, sizeof(float) * (r->env_h + 1), cudaMemcpyDeviceToHost));
    if (conditional)
        TT_CUDA_N(cudaMemcpy(conditional, r->env_cond, sizeof(float) * (size_t)r->env_h * (r->env_w + 1),
                             cudaMemcpyDeviceToHost));
    return TT_OK;
}

}  // extern "C"
