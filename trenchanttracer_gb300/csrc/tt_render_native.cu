// Native path tracer: a wavefront of compacted ray queues on one GB300.
//
// A frame is processed in waves of up to `wave_paths` paths (path = one sample of one pixel).
// Per wave: raygen, then for each bounce extend (closest hit over the BVH and the analytic
// objects) -> shade (emission, environment light sampling with MIS, BSDF sampling, Russian
// roulette; survivors and shadow rays are appended to queues with one atomic per warp) ->
// shadow (any hit), and finally accumulate (each pixel adds its samples in a fixed order, in
// float or double). Every kernel reads its queue length from device memory, so a wave needs no
// host round trip and the whole frame can be captured as a CUDA graph (tt_render_native_graph).
//
// The integrator (all of it built from basic IEEE operations, tt_ptmath.cuh):
//   camera     pinhole of the CameraMeta; pixel (x, y) with y = 0 at the top, jittered by two
//              PCG32 draws; tan(fov/2) evaluated on the host
//   rng        PCG32, stream = global path index (sample * pixels + pixel), state = frame seed
//   Lambert    cosine sampling (pdf cos/pi), f = albedo/pi
//   GGX        conductor: alpha = roughness^2, Trowbridge-Reitz D, separable Smith G, Schlick F
//              with F0; visible-normal sampling (Heitz 2018, "Sampling the GGX Distribution of
//              Visible Normals"), weight F * G1(wi)
//   dielectric smooth, exact unpolarised Fresnel, reflect with probability F else refract
//   reference  Metal (Phong 30 lobe), Spec (mirror), Refr (dielectric, IOR 1.4), Coat (Fresnel
//   kinds      choice between mirror and Lambert): sampled, treated as specular for MIS
//   env        nearest texel of the equirectangular map in the reference's mapping; light
//              sampling by a 2D CDF over luminance * sin(theta) (FP64 prefix sums); power
//              heuristic MIS between light and BSDF sampling for Lambert and GGX vertices
//   roulette   from rr_depth on, survival max(beta) clamped to [0.05, 1]
#include <cuda_runtime.h>

#include <cstring>
#include <string>
#include <vector>

#include "tt_device.h"
#include "tt_ptmath.cuh"

namespace tt {

using namespace pt;

constexpr int kPtBlock = 128;
constexpr int kFlagSpecular = 1;  // the last bounce was specular (no light sampling was done)

struct EnvView {
    const float4 *tex;  // w*h radiance
    const float *marg;  // h+1 marginal CDF over rows
    const float *cond;  // h*(w+1) conditional CDFs per row
    int w, h;
    float scale;
};

struct PathSoA {
    float *o, *d;       // 3 per path
    float *beta, *L;    // 3 per path
    uint64_t *rng;      // PCG32 state (the stream increment is derived from the path index)
    float *last_pdf;
    int *depth, *flags;
    float *hit_t, *hit_u, *hit_v;
    int *hit_prim;      // triangle slot >= 0, -(geometry+2) for analytic objects, -1 = miss
    int *queue[2];      // path indices of the active paths
    int *counts;        // [0], [1] queue lengths by bounce parity, [2] shadow queue length
    int *shadow_path;
    float *shadow_ray;  // 8 per shadow ray
    float *shadow_val;  // 3 per shadow ray
};

struct NativeArgs {
    BvhView bvh;
    const MaterialRec *materials;
    int num_materials;
    const GeomRec *geoms;
    int num_geoms;
    EnvView env;
    PathSoA ps;
    tt_camera_meta cam;
    float tanx, tany;   // tan(fov/2)
    tt_render_params p;
    int npix;           // width * height
    long long wave_first_path;  // global index of the wave's first path
    int wave_paths;
    unsigned int *err;
};

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

__device__ __forceinline__ Rng path_rng(const NativeArgs &a, long long gid, uint64_t state) {
    Rng g;
    g.state = state;
    g.inc = ((uint64_t)gid << 1u) | 1u;
    return g;
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

__device__ __forceinline__ int cdf_search(const float *cdf, int n, float u) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(cdf + mid + 1) <= u) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Samples a direction by the 2D CDF. Returns pdf (0 = no sample), radiance and direction.
__device__ __forceinline__ float env_sample(const EnvView &e, float u1, float u2, V3 &dir, V3 &le) {
    const int y = cdf_search(e.marg, e.h, u1);
    const float m0 = __ldg(e.marg + y), m1 = __ldg(e.marg + y + 1);
    if (!(m1 > m0)) return 0.0f;
    const float *row = e.cond + (size_t)y * (e.w + 1);
    const int x = cdf_search(row, e.w, u2);
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
    const int texel = y * e.w + x;
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

// ---- analytic objects (brute force, as the reference does) --------------------------------------
__device__ __forceinline__ void analytic_hit(const NativeArgs &a, const V3 &o, const V3 &d, float tmin, float &t,
                                             int &prim, float &hu, float &hv) {
    for (int i = 0; i < a.num_geoms; i++) {
        const GeomRec g = a.geoms[i];
        if (g.kind == GEOM_PLANE) {
            const V3 p0(g.p0[0], g.p0[1], g.p0[2]);
            const V3 e1 = sub(V3(g.p1[0], g.p1[1], g.p1[2]), p0), e2 = sub(V3(g.p2[0], g.p2[1], g.p2[2]), p0);
            const V3 P = cross(d, e2);
            const float det = dot(e1, P);
            if (det > -1e-12f && det < 1e-12f) continue;
            const float inv = PT_DIV(1.0f, det);
            const V3 T = sub(o, p0);
            const float u = PT_MUL(dot(T, P), inv);
            if (u < 0.f || u > 1.f) continue;
            const V3 Q = cross(T, e1);
            const float v = PT_MUL(dot(d, Q), inv);
            if (v < 0.f || v > 1.f) continue;
            const float th = PT_MUL(dot(e2, Q), inv);
            if (th > tmin && th < t) {
                t = th;
                prim = -(i + 2);
                hu = u;
                hv = v;
            }
        } else if (g.kind == GEOM_SPHERE) {
            const V3 c(g.p0[0], g.p0[1], g.p0[2]);
            const V3 oc = sub(c, o);
            const float bq = dot(oc, d);
            const float disc = PT_FMA(g.radius, g.radius, PT_FMA(bq, bq, -dot(oc, oc)));
            if (disc < 0.0f) continue;
            const float sq = PT_SQRT(disc);
            float th = PT_SUB(bq, sq);
            if (!(th > tmin)) th = PT_ADD(bq, sq);
            if (th > tmin && th < t) {
                t = th;
                prim = -(i + 2);
                hu = 0.f;
                hv = 0.f;
            }
        }
    }
}

// ---- kernels ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kPtBlock) k_raygen(NativeArgs a) {
    const int stride = gridDim.x * blockDim.x;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.ps.counts[0] = a.wave_paths;
        a.ps.counts[1] = 0;
        a.ps.counts[2] = 0;
    }
    const V3 cam_pos(a.cam.position[0], a.cam.position[1], a.cam.position[2]);
    const V3 view = normalize(V3(a.cam.view[0], a.cam.view[1], a.cam.view[2]));
    const V3 right = normalize(cross(view, V3(a.cam.up[0], a.cam.up[1], a.cam.up[2])));
    const V3 up = cross(right, view);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.wave_paths; i += stride) {
        const long long gid = a.wave_first_path + i;
        const int pixel = (int)(gid % a.npix);
        const int px = pixel % a.cam.width, py = pixel / a.cam.width;
        Rng g = pcg32_seed((uint64_t)a.p.seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull, (uint64_t)gid);
        const float jx = uniform(g), jy = uniform(g);
        const float sx = PT_SUB(PT_MUL(2.0f, PT_DIV(PT_ADD((float)px, jx), (float)a.cam.width)), 1.0f);
        const float sy = PT_SUB(1.0f, PT_MUL(2.0f, PT_DIV(PT_ADD((float)py, jy), (float)a.cam.height)));
        const V3 dir = normalize(madd(up, PT_MUL(sy, a.tany), madd(right, PT_MUL(sx, a.tanx), view)));
        st3(a.ps.o + 3ll * i, cam_pos);
        st3(a.ps.d + 3ll * i, dir);
        st3(a.ps.beta + 3ll * i, V3(1.f, 1.f, 1.f));
        st3(a.ps.L + 3ll * i, V3(0.f, 0.f, 0.f));
        a.ps.rng[i] = g.state;
        a.ps.last_pdf[i] = 0.0f;
        a.ps.depth[i] = 0;
        a.ps.flags[i] = kFlagSpecular;
        a.ps.queue[0][i] = i;
    }
}

// closest hit of every queued path; `cur` = bounce parity
__global__ void __launch_bounds__(kPtBlock) k_extend(NativeArgs a, int cur) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        a.ps.counts[cur ^ 1] = 0;
        a.ps.counts[2] = 0;
    }
    const int n = a.ps.counts[cur];
    const int stride = gridDim.x * blockDim.x;
    uint32_t err = 0;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += stride) {
        const int i = a.ps.queue[cur][q];
        const V3 o = ld3(a.ps.o + 3ll * i), d = ld3(a.ps.d + 3ll * i);
        const float4 r0 = make_float4(o.x, o.y, o.z, d.x);
        const float4 r1 = make_float4(d.y, d.z, 0.0f, 1e20f);
        const TraceResult tr = traverse<true>(a.bvh, r0, r1, err);
        float t = tr.t, hu = tr.u, hv = tr.v;
        int prim = tr.addr;
        if (a.num_geoms) analytic_hit(a, o, d, 0.0f, t, prim, hu, hv);
        a.ps.hit_t[i] = t;
        a.ps.hit_prim[i] = prim;
        a.ps.hit_u[i] = hu;
        a.ps.hit_v[i] = hv;
    }
    if (err) atomicOr(a.err, err);
}

__device__ __forceinline__ float ray_eps(const NativeArgs &a, const V3 &p) {
    const float m = fmaxf(fmaxf(fabsf(p.x), fabsf(p.y)), fabsf(p.z));
    return PT_MUL(a.p.ray_eps, fmaxf(1.0f, m));
}

__global__ void __launch_bounds__(kPtBlock) k_shade(NativeArgs a, int cur) {
    const int n = a.ps.counts[cur];
    const int stride = gridDim.x * blockDim.x;
    const int rounds = (n + stride - 1) / stride;
    const bool use_env = a.env.w > 0;
    for (int round = 0, q = blockIdx.x * blockDim.x + threadIdx.x; round < rounds; round++, q += stride) {
        const bool live = q < n;
        bool alive = false;
        bool shadow = false;
        int i = 0;
        V3 sh_o, sh_d, sh_val;
        if (live) {
            i = a.ps.queue[cur][q];
            const long long gid = a.wave_first_path + i;
            Rng g = path_rng(a, gid, a.ps.rng[i]);
            const V3 o = ld3(a.ps.o + 3ll * i), d = ld3(a.ps.d + 3ll * i);
            V3 beta = ld3(a.ps.beta + 3ll * i), L = ld3(a.ps.L + 3ll * i);
            const int prim = a.ps.hit_prim[i];
            const int flags = a.ps.flags[i];
            const float last_pdf = a.ps.last_pdf[i];
            int depth = a.ps.depth[i];
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
                const float t = a.ps.hit_t[i];
                const V3 p = madd(d, t, o);
                V3 n;
                int mat;
                if (prim >= 0) {
                    hit_normal(a.bvh, prim, a.ps.hit_u[i], a.ps.hit_v[i], n.x, n.y, n.z);
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
                const bool nee = use_env && !(a.p.flags & TT_RENDER_NO_ENV_SAMPLING) &&
                                 (m.kind == MAT_DIFF || m.kind == MAT_GGX);
                const float eps = ray_eps(a, p);
                if (nee) {
                    const float u1 = uniform(g), u2 = uniform(g);
                    V3 wi, le;
                    const float pl = env_sample(a.env, u1, u2, wi, le);
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
                const float u1 = uniform(g), u2 = uniform(g), u3 = uniform(g);
                const BsdfSample bs = bsdf_sample(m, nl, wo, entering, u1, u2, u3);
                if (maxc(bs.weight) > 0.0f) {
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
                        st3(a.ps.o + 3ll * i, madd(off, eps, p));
                        st3(a.ps.d + 3ll * i, bs.wi);
                        st3(a.ps.beta + 3ll * i, beta);
                        a.ps.last_pdf[i] = bs.pdf;
                        a.ps.flags[i] = (bs.specular || !nee) ? kFlagSpecular : 0;
                        a.ps.depth[i] = depth;
                    }
                }
            }
            st3(a.ps.L + 3ll * i, L);
            a.ps.rng[i] = g.state;
        }
        const int slot = warp_append(a.ps.counts + (cur ^ 1), alive);
        if (alive) a.ps.queue[cur ^ 1][slot] = i;
        const int sslot = warp_append(a.ps.counts + 2, shadow);
        if (shadow) {
            a.ps.shadow_path[sslot] = i;
            float *r = a.ps.shadow_ray + 8ll * sslot;
            r[0] = sh_o.x;
            r[1] = sh_o.y;
            r[2] = sh_o.z;
            r[3] = sh_d.x;
            r[4] = sh_d.y;
            r[5] = sh_d.z;
            r[6] = 0.0f;
            r[7] = 1e20f;
            st3(a.ps.shadow_val + 3ll * sslot, sh_val);
        }
    }
}

__global__ void __launch_bounds__(kPtBlock) k_shadow(NativeArgs a) {
    const int n = a.ps.counts[2];
    const int stride = gridDim.x * blockDim.x;
    uint32_t err = 0;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride) {
        const float4 *r = reinterpret_cast<const float4 *>(a.ps.shadow_ray + 8ll * j);
        const float4 r0 = r[0], r1 = r[1];
        const TraceResult tr = traverse<false>(a.bvh, r0, r1, err);
        bool blocked = tr.addr >= 0;
        if (!blocked && a.num_geoms) {
            float t = r1.w, hu, hv;
            int prim = -1;
            analytic_hit(a, V3(r0.x, r0.y, r0.z), V3(r0.w, r1.x, r1.y), r1.z, t, prim, hu, hv);
            blocked = prim != -1;
        }
        if (!blocked) {
            const int i = a.ps.shadow_path[j];
            st3(a.ps.L + 3ll * i, add(ld3(a.ps.L + 3ll * i), ld3(a.ps.shadow_val + 3ll * j)));
        }
    }
    if (err) atomicOr(a.err, err);
}

template <typename T>
__global__ void __launch_bounds__(kPtBlock) k_accumulate(NativeArgs a, T *accum) {
    // paths of the wave are laid out sample-major: path i = (wave sample k) * npix + pixel
    const int first_pixel = (int)(a.wave_first_path % a.npix);
    const int stride = gridDim.x * blockDim.x;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.npix && i < a.wave_paths; i += stride) {
        const int pixel = (first_pixel + i) % a.npix;
        T acc[3] = {accum[3ll * pixel], accum[3ll * pixel + 1], accum[3ll * pixel + 2]};
        for (int k = i; k < a.wave_paths; k += a.npix) {
            acc[0] += (T)a.ps.L[3ll * k];
            acc[1] += (T)a.ps.L[3ll * k + 1];
            acc[2] += (T)a.ps.L[3ll * k + 2];
        }
        accum[3ll * pixel] = acc[0];
        accum[3ll * pixel + 1] = acc[1];
        accum[3ll * pixel + 2] = acc[2];
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

tt_status native_setup(tt_renderer *r) {
    int dev = 0;
    TT_CUDA_N(cudaGetDevice(&dev));
    TT_CUDA_N(cudaDeviceGetAttribute(&r->num_sms, cudaDevAttrMultiProcessorCount, dev));
    if (r->env_w <= 0) return TT_OK;
    const int w = r->env_w, h = r->env_h;
    TT_CUDA_N(cudaMalloc(&r->env_marg, sizeof(float) * (h + 1)));
    TT_CUDA_N(cudaMalloc(&r->env_cond, sizeof(float) * (size_t)h * (w + 1)));
    double *rowsum = nullptr;
    TT_CUDA_N(cudaMalloc(&rowsum, sizeof(double) * h));
    k_env_rows<<<(h + 127) / 128, 128>>>(r->env, w, h, r->env_cond, rowsum);
    k_env_marginal<<<1, 1>>>(rowsum, h, r->env_marg);
    cudaError_t e = cudaDeviceSynchronize();
    cudaFree(rowsum);
    if (e != cudaSuccess) return cuda_fail_n(e, "environment tables");
    return TT_OK;
}

void native_release(tt_renderer *r) {
    if (r->env_marg) cudaFree(r->env_marg);
    if (r->env_cond) cudaFree(r->env_cond);
    if (r->paths) cudaFree(r->paths);
    r->env_marg = r->env_cond = nullptr;
    r->paths = nullptr;
    r->paths_bytes = 0;
    r->path_capacity = 0;
}

// Carves the path state of `cap` paths out of one allocation.
static tt_status ensure_paths(tt_renderer *r, int cap, PathSoA &ps) {
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t n = (size_t)cap;
    const size_t sizes[] = {12 * n, 12 * n, 12 * n, 12 * n, 8 * n, 4 * n, 4 * n, 4 * n, 4 * n, 4 * n, 4 * n,
                            4 * n, 4 * n, 4 * n, 64, 4 * n, 32 * n, 12 * n};
    size_t total = 0;
    for (size_t s : sizes) total += al(s);
    if (r->paths_bytes < total) {
        if (r->paths) cudaFree(r->paths);
        r->paths = nullptr;
        r->paths_bytes = 0;
        cudaError_t e = cudaMalloc(&r->paths, total);
        if (e != cudaSuccess) return fail(TT_ERR_OOM, std::string("path state: ") + cudaGetErrorString(e));
        r->paths_bytes = total;
        r->path_capacity = cap;
    }
    char *p = static_cast<char *>(r->paths);
    int k = 0;
    auto take = [&](void *&dst) {
        dst = p;
        p += al(sizes[k++]);
    };
    void *v[18];
    for (int i = 0; i < 18; i++) take(v[i]);
    ps.o = (float *)v[0];
    ps.d = (float *)v[1];
    ps.beta = (float *)v[2];
    ps.L = (float *)v[3];
    ps.rng = (uint64_t *)v[4];
    ps.last_pdf = (float *)v[5];
    ps.depth = (int *)v[6];
    ps.flags = (int *)v[7];
    ps.hit_t = (float *)v[8];
    ps.hit_u = (float *)v[9];
    ps.hit_v = (float *)v[10];
    ps.hit_prim = (int *)v[11];
    ps.queue[0] = (int *)v[12];
    ps.queue[1] = (int *)v[13];
    ps.counts = (int *)v[14];
    ps.shadow_path = (int *)v[15];
    ps.shadow_ray = (float *)v[16];
    ps.shadow_val = (float *)v[17];
    return TT_OK;
}

static const int kMaxWavePaths = 1 << 22;

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
    if (cam->width <= 0 || cam->height <= 0 || p->spp < 1 || p->max_depth < 1 || p->sample_offset < 0)
        return fail(TT_ERR_INVALID, "bad image size or render parameters");
    const long long npix = (long long)cam->width * cam->height;
    if (npix > (1ll << 30)) return fail(TT_ERR_INVALID, "image too large");
    const long long total = npix * p->spp;
    int wave = (int)(total < kMaxWavePaths ? total : (kMaxWavePaths / npix > 0 ? (kMaxWavePaths / npix) * npix
                                                                                : kMaxWavePaths));
    PathSoA ps;
    tt_status st = ensure_paths(r, wave > r->path_capacity ? wave : r->path_capacity, ps);
    if (st != TT_OK) return st;
    NativeArgs a;
    a.bvh = r->bvh;
    a.materials = r->materials;
    a.num_materials = r->num_materials;
    a.geoms = r->geoms;
    a.num_geoms = r->num_geoms;
    a.env.tex = r->env;
    a.env.marg = r->env_marg;
    a.env.cond = r->env_cond;
    a.env.w = r->env_w;
    a.env.h = r->env_h;
    a.env.scale = p->env_scale;
    a.ps = ps;
    a.cam = *cam;
    a.tanx = (float)std::tan((double)cam->fov[0] * 0.5 * 3.14159265358979323846 / 180.0);
    a.tany = (float)std::tan((double)cam->fov[1] * 0.5 * 3.14159265358979323846 / 180.0);
    a.p = *p;
    a.npix = (int)npix;
    a.err = r->err;
    cudaStream_t s = (cudaStream_t)stream;
    const int grid = r->num_sms * 8;
    const long long first = (long long)p->sample_offset * npix;
    for (long long done = 0; done < total; done += wave) {
        a.wave_first_path = first + done;
        a.wave_paths = (int)((total - done) < wave ? (total - done) : wave);
        k_raygen<<<grid, kPtBlock, 0, s>>>(a);
        for (int b = 0; b < p->max_depth; b++) {
            k_extend<<<grid, kPtBlock, 0, s>>>(a, b & 1);
            k_shade<<<grid, kPtBlock, 0, s>>>(a, b & 1);
            k_shadow<<<grid, kPtBlock, 0, s>>>(a);
        }
        if (p->flags & TT_RENDER_ACCUM_F64) k_accumulate<double><<<grid, kPtBlock, 0, s>>>(a, (double *)d_accum);
        else k_accumulate<float><<<grid, kPtBlock, 0, s>>>(a, (float *)d_accum);
    }
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
