// Reference-compatible path tracer: the per-pixel megakernel semantics of the reference's
// pathTracingKernel / renderKernel (src/core/RenderKernel.cu:27-218), so that an image rendered
// here with the same camera, seed and scene equals the reference kernel's accumulation buffer.
//
// Reproduced on purpose: one thread per pixel in 16x16 blocks over a (W/16) x (H/16) grid
// (the reference truncates, :221-222); curand XORWOW seeded with hashedFrame + threadId and its
// draws in the reference's order (:117-118, :152-153, :171-172, the samplers); 10 bounces, no
// Russian roulette (:35); brute-force Plane/Sphere objects after the BVH (:38-62); on a miss the
// environment's nearest texel times 2 (include/hdr/HDRKernel.cuh:6-42); emission added at every
// hit; the five samplers Diff / Metal (Phong 30) / Spec / Refr (IOR 1.4) / Coat
// (include/material/*Impl.cuh); the accumulation accum += sum_s L / SAMPLES. Float arithmetic uses
// the reference's rounding (tt_refmath.cuh); constants the reference writes in double
// (2 * M_PI * u, fabs(w.x) > .1, u < 0.2, det bounds) stay double. The BVH hit itself is this
// project's traversal, whose per-ray results are the reference algorithm's.
#include <cuda_runtime.h>
#include <curand_kernel.h>

#include <algorithm>
#include <string>

#include "tt_device.h"
#include "tt_refmath.cuh"
#include "tt_reorder.h"

namespace tt {

struct CompatArgs {
    BvhView bvh;
    const MaterialRec *materials;
    int num_materials;
    const GeomRec *geoms;
    int num_geoms;
    const float4 *env;
    int env_w, env_h;
    tt_camera_meta cam;
    tt_render_meta meta;
    float *accum;  // W*H*3 floats (Vec3f per pixel)
    unsigned int *err;
};

struct RHit {
    int index;
    int mat;
    float distance;
    V3 normal;
    V3 n, nl, point;
};

// Hit::operator< (include/geometry/Hit.h:16-22)
__device__ __forceinline__ bool hit_less(const RHit &a, const RHit &b) {
    if (a.distance == b.distance) return false;
    if (b.distance == -1) return true;
    return a.distance < b.distance;
}

// planeIntersect (include/geometry/PlaneImpl.cuh:10-51): a two-sided parallelogram.
__device__ __forceinline__ RHit plane_hit(const GeomRec &g, const V3 &o, const V3 &d, float tmax) {
    RHit h;
    h.index = -1;
    h.mat = -1;
    h.distance = tmax;
    const V3 p0(g.p0[0], g.p0[1], g.p0[2]), p1(g.p1[0], g.p1[1], g.p1[2]), p2(g.p2[0], g.p2[1], g.p2[2]);
    const V3 e1 = r_sub(p1, p0), e2 = r_sub(p2, p0);
    const V3 P = r_cross(d, e2);
    const float det = r_dot(e1, P);
    if ((double)det > -0.00001 && (double)det < 0.00001) return h;
    const float inv = __fdiv_rn(1.f, det);
    const V3 T = r_sub(o, p0);
    const V3 Q = r_cross(T, e1);
    const float u = __fmul_rn(r_dot(T, P), inv);
    const float v = __fmul_rn(r_dot(d, Q), inv);
    if (u < 0.f || u > 1.f || v < 0.f || v > 1.f) return h;
    const float t = __fmul_rn(r_dot(e2, Q), inv);
    if ((double)t > 0.00001) {
        h.distance = t;
        h.normal = r_cross(e1, e2);
    }
    return h;
}

// sphereIntersect (include/geometry/SphereImpl.cuh:11-32)
__device__ __forceinline__ RHit sphere_hit(const GeomRec &g, const V3 &o, const V3 &d, float tmax) {
    RHit h;
    h.index = -1;
    h.mat = -1;
    h.distance = tmax;
    const V3 pos(g.p0[0], g.p0[1], g.p0[2]);
    const V3 op = r_sub(pos, o);
    const float eps = 0.01f;
    const float b = r_dot(op, d);
    // b*b - dot(op, op) + r*r  ->  fma(r, r, fma(b, b, -dot))
    float disc = __fmaf_rn(g.radius, g.radius, __fmaf_rn(b, b, -r_dot(op, op)));
    if (disc >= 0) {
        disc = __fsqrt_rn(disc);
        float t = __fsub_rn(b, disc);
        float distance;
        if (t > eps) {
            distance = t;
        } else {
            t = __fadd_rn(b, disc);
            distance = t > eps ? t : 0.0f;
        }
        if (0.01f < distance && distance < tmax) {
            h.distance = distance;
            h.point = r_madd(d, h.distance, o);
            h.normal = V3(__fsub_rn(h.point.x, pos.x), __fsub_rn(h.point.y, pos.y), __fsub_rn(h.point.z, pos.z));
        }
    }
    return h;
}

// hdrSample (include/hdr/HDRKernel.cuh:6-42): nearest texel of an equirectangular map, x 2.
__device__ __forceinline__ V3 env_lookup(const CompatArgs &a, const V3 &d) {
    if (!a.env) return V3(0.f, 0.f, 0.f);
    float lx = atan2f(d.x, d.z);
    lx = lx < 0.f ? __fadd_rn(lx, a.meta.two_pi) : lx;
    const float ly = acosf(d.y);
    const float u = __fdiv_rn(lx, a.meta.two_pi);
    const float v = __fdiv_rn(ly, a.meta.pi);
    const int u2 = (int)__fmul_rn(u, (float)a.env_w);
    const int v2 = (int)__fmul_rn(v, (float)a.env_h);
    const long long idx = (long long)u2 + (long long)v2 * a.env_w;
    // the reference's linear texture returns zero outside the array
    float4 c = make_float4(0.f, 0.f, 0.f, 0.f);
    if (idx >= 0 && idx < (long long)a.env_w * a.env_h) c = __ldg(a.env + idx);
    return V3(__fmul_rn(c.x, 2.0f), __fmul_rn(c.y, 2.0f), __fmul_rn(c.z, 2.0f));
}

__device__ __forceinline__ float two_pi_u(curandState *rs) {
    // 2 * M_PI * curand_uniform(...) in double, stored to float
    return __double2float_rn(__dmul_rn(6.283185307179586232, (double)curand_uniform(rs)));
}

__device__ __forceinline__ V3 basis_u(const V3 &w) {
    const V3 a = (double)fabsf(w.x) > .1 ? V3(0.f, 1.f, 0.f) : V3(1.f, 0.f, 0.f);
    return r_normalize(r_cross(a, w));
}

// u*cos(phi)*s + v*sin(phi)*s + w*c  ->  fma(w, c, fma(u*cos*s ... ))
__device__ __forceinline__ V3 lobe_dir(const V3 &u, const V3 &v, const V3 &w, float cphi, float sphi, float s,
                                       float c) {
    V3 r;
    r.x = __fmaf_rn(w.x, c, __fmaf_rn(__fmul_rn(u.x, cphi), s, __fmul_rn(__fmul_rn(v.x, sphi), s)));
    r.y = __fmaf_rn(w.y, c, __fmaf_rn(__fmul_rn(u.y, cphi), s, __fmul_rn(__fmul_rn(v.y, sphi), s)));
    r.z = __fmaf_rn(w.z, c, __fmaf_rn(__fmul_rn(u.z, cphi), s, __fmul_rn(__fmul_rn(v.z, sphi), s)));
    return r;
}

// `d - n * 2.0f * dot(n, d)` (MetalImpl.cuh:25, CoatImpl.cuh:12-14, RefrImpl.cuh:24,43): inside the
// reference's kernel dot(n, d) rounds as r_dot_yx in all three samplers (and in Spec's reflection); Metal and Refr fuse the
// n * 2 * k product into the subtraction, Coat's reflect() keeps it rounded (both measured on
// interactions recorded in the reference's own kernel, oracle/ref/ref_render_probe.cu).
__device__ __forceinline__ V3 reflect_ref(const V3 &d, const V3 &n) {
    const float k = r_dot_yx(n, d);
    return V3(__fmaf_rn(-__fmul_rn(n.x, 2.0f), k, d.x), __fmaf_rn(-__fmul_rn(n.y, 2.0f), k, d.y),
              __fmaf_rn(-__fmul_rn(n.z, 2.0f), k, d.z));
}
__device__ __forceinline__ V3 reflect_ref_rounded(const V3 &d, const V3 &n) {
    const float k = r_dot_yx(n, d);
    return V3(__fsub_rn(d.x, __fmul_rn(__fmul_rn(n.x, 2.0f), k)), __fsub_rn(d.y, __fmul_rn(__fmul_rn(n.y, 2.0f), k)),
              __fsub_rn(d.z, __fmul_rn(__fmul_rn(n.z, 2.0f), k)));
}

struct RRay {
    V3 o, d;
    float tmin, tmax;
};

// diffSample (include/material/DiffImpl.cuh:12-36)
__device__ __forceinline__ void diff_sample(const MaterialRec &m, curandState *rs, RRay &ray, const RHit &h, V3 &mask) {
    const float phi = two_pi_u(rs);
    const float r2 = curand_uniform(rs);
    const float r2s = __fsqrt_rn(r2);
    const V3 w = r_normalize(h.nl);
    const V3 u = basis_u(w);
    const V3 v = r_cross(w, u);
    ray.d = r_normalize(lobe_dir(u, v, w, cosf(phi), sinf(phi), r2s, __fsqrt_rn(__fsub_rn(1.f, r2))));
    ray.o = r_madd(h.nl, 0.001f, h.point);
    mask = r_mul(mask, V3(m.color[0], m.color[1], m.color[2]));
}

// metalSample (include/material/MetalImpl.cuh:13-41): Phong lobe, exponent 30
__device__ __forceinline__ void metal_sample(const MaterialRec &m, curandState *rs, RRay &ray, const RHit &h,
                                             V3 &mask) {
    const float phi = two_pi_u(rs);
    const float r2 = curand_uniform(rs);
    const float cos_t = powf(__fsub_rn(1.f, r2), 1.0f / 31.0f);
    const float sin_t = __fsqrt_rn(__fmaf_rn(-cos_t, cos_t, 1.f));
    const V3 w = r_normalize(reflect_ref(ray.d, h.n));
    const V3 u = basis_u(w);
    const V3 v = r_cross(w, u);
    ray.d = r_normalize(lobe_dir(u, v, w, cosf(phi), sinf(phi), sin_t, cos_t));
    ray.o = r_madd(h.nl, 0.0001f, h.point);
    mask = r_mul(mask, V3(m.color[0], m.color[1], m.color[2]));
}

// specSample (include/material/SpecImpl.cuh:12-25): d - n * dot(n, d) * 2.0f, with dot(n, d) rounded
// as in the other samplers' reflections (r_dot_yx; found by comparing whole frames of a scene that
// mixes every material kind, because recording Spec interactions changes how nvcc compiles the
// reference's kernel)
__device__ __forceinline__ void spec_sample(const MaterialRec &m, RRay &ray, const RHit &h, V3 &mask) {
    const float k = r_dot_yx(h.n, ray.d);
    const V3 d(__fmaf_rn(-__fmul_rn(h.n.x, k), 2.0f, ray.d.x), __fmaf_rn(-__fmul_rn(h.n.y, k), 2.0f, ray.d.y),
               __fmaf_rn(-__fmul_rn(h.n.z, k), 2.0f, ray.d.z));
    ray.d = r_normalize(d);
    ray.o = r_madd(h.nl, 0.001f, h.point);
    mask = r_mul(mask, V3(m.color[0], m.color[1], m.color[2]));
}

// refrSample (include/material/RefrImpl.cuh:12-61): IOR 1.4, Schlick weights, reflect p = 0.2.
// The rounding of every expression was pinned against interactions recorded inside the reference's
// own kernel (oracle/ref/ref_render_probe.cu): the reflected direction is normalised as
// r_normalize_yx, and so is the transmitted one the second time round.
__device__ __forceinline__ V3 refr_reflect(const V3 &d, const V3 &n) {
    return r_normalize_yx(reflect_ref(d, n));
}

__device__ __forceinline__ void refr_sample(curandState *rs, RRay &ray, const RHit &h, V3 &mask) {
    const bool into = r_dot(h.n, h.nl) > 0;
    const float nc = 1.0f, nt = 1.4f;
    const float nnt = into ? __fdiv_rn(nc, nt) : __fdiv_rn(nt, nc);
    const float ddn = r_dot(ray.d, h.nl);
    const float cos2t = __fmaf_rn(-__fmul_rn(nnt, nnt), __fmaf_rn(-ddn, ddn, 1.f), 1.0f);
    if (cos2t < 0.0f) {
        ray.d = refr_reflect(ray.d, h.n);
        ray.o = r_madd(h.nl, 0.001f, h.point);
        return;
    }
    const float k = __fmul_rn((float)(into ? 1 : -1), __fmaf_rn(ddn, nnt, __fsqrt_rn(cos2t)));
    // `tdir = d * nnt; tdir -= n * k;`: d * nnt stays rounded and n * k is fused into the subtraction
    V3 tdir(__fmaf_rn(-h.n.x, k, __fmul_rn(ray.d.x, nnt)), __fmaf_rn(-h.n.y, k, __fmul_rn(ray.d.y, nnt)),
            __fmaf_rn(-h.n.z, k, __fmul_rn(ray.d.z, nnt)));
    tdir = r_normalize(tdir);
    const float a = __fsub_rn(nt, nc);
    const float R0 = __fmul_rn(__fdiv_rn(__fmul_rn(a, a), __fadd_rn(nt, nc)), __fadd_rn(nt, nc));
    const float c = __fsub_rn(1.f, into ? -ddn : r_dot(tdir, h.n));
    const float x4 = __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(__fsub_rn(1.f, R0), c), c), c), c);
    const float Re = __fmaf_rn(x4, c, R0);
    const float Tr = __fsub_rn(1.f, Re);
    const float P = __fmaf_rn(.5f, Re, .25f);
    const float RP = __fdiv_rn(Re, P);
    const float TP = __fdiv_rn(Tr, __fsub_rn(1.f, P));
    if ((double)curand_uniform(rs) < 0.2) {
        mask = r_mul(mask, RP);
        ray.d = refr_reflect(ray.d, h.n);
    } else {
        mask = r_mul(mask, TP);
        ray.d = r_normalize_yx(tdir);  // `nextRay.direction = tdir; nextRay.direction.normalize();`
    }
    ray.o = r_madd(h.nl, 0.001f, h.point);
}

// refract() / fresnel() of include/material/CoatImpl.cuh:16-58
__device__ __forceinline__ V3 coat_refract(const RRay &ray, const RHit &h, float n1, float n2) {
    const float cos1 = r_dot(h.n, V3(-ray.d.x, -ray.d.y, -ray.d.z));
    const float n12 = __fdiv_rn(n1, n2);
    const float radicand = __fmaf_rn(-powf(n12, 2), __fsub_rn(1.f, powf(cos1, 2)), 1.f);
    if (radicand < 0) return V3(0.f, 0.f, 0.f);
    const float cos2 = __fsqrt_rn(radicand);
    const float k = cos1 > 0 ? __fmaf_rn(cos1, n12, -cos2) : __fmaf_rn(cos1, n12, cos2);
    return V3(__fmaf_rn(ray.d.x, n12, __fmul_rn(h.n.x, k)), __fmaf_rn(ray.d.y, n12, __fmul_rn(h.n.y, k)),
              __fmaf_rn(ray.d.z, n12, __fmul_rn(h.n.z, k)));
}

__device__ __forceinline__ float coat_fresnel(const RRay &ray, const RHit &h, float n1, float n2, const V3 &tdir) {
    if ((double)r_length(tdir) <= 0.12345 || r_dot(h.n, tdir) > 0) return 1;
    const float ci = r_dot(h.n, V3(-ray.d.x, -ray.d.y, -ray.d.z));
    const float ct = r_dot(V3(-h.n.x, -h.n.y, -h.n.z), tdir);
    const float rs = powf(__fdiv_rn(__fmaf_rn(n1, ci, -__fmul_rn(n2, ct)), __fmaf_rn(n1, ci, __fmul_rn(n2, ct))), 2);
    const float rp = powf(__fdiv_rn(__fmaf_rn(n1, ct, -__fmul_rn(n2, ci)), __fmaf_rn(n1, ct, __fmul_rn(n2, ci))), 2);
    return __fdiv_rn(__fadd_rn(rs, rp), 2.0f);
}

// coatSample (include/material/CoatImpl.cuh:68-116)
__device__ __forceinline__ void coat_sample(const MaterialRec &m, curandState *rs, RRay &ray, const RHit &h,
                                            V3 &mask) {
    const V3 refl = reflect_ref_rounded(ray.d, h.n);
    const float roulette = curand_uniform(rs);
    const float n_air = (float)1.000293, n_coat = (float)1.291;  // double literals, as written
    const V3 refr = coat_refract(ray, h, n_air, n_coat);
    const float threshold = coat_fresnel(ray, h, n_air, n_coat, refr);
    if (roulette < threshold) {
        mask = r_mul(mask, V3(m.color2[0], m.color2[1], m.color2[2]));
        ray.d = r_normalize(refl);
        ray.o = r_madd(h.nl, 0.001f, h.point);
    } else {
        const float r1 = two_pi_u(rs);
        const float r2 = curand_uniform(rs);
        const float r2s = __fsqrt_rn(r2);
        const V3 w = r_normalize(h.nl);
        const V3 u = basis_u(w);
        const V3 v = r_cross(w, u);
        ray.d = r_normalize(lobe_dir(u, v, w, cosf(r1), sinf(r1), r2s, __fsqrt_rn(__fsub_rn(1.f, r2))));
        ray.o = r_madd(h.nl, 0.001f, h.point);
        mask = r_mul(mask, V3(m.color[0], m.color[1], m.color[2]));
    }
}

// normalize(hit, ray) + hitPoint(hit, ray) (include/geometry/IntersectKernel.cuh:62-76)
__device__ __forceinline__ void hit_frame(RHit &hit, const RRay &ray) {
    hit.n = r_normalize(hit.normal);
    hit.nl = r_dot(hit.n, ray.d) < 0 ? hit.n : r_mul(hit.n, -1.0f);
    hit.point = r_madd(ray.d, hit.distance, ray.o);
}

// the sampler switch of renderKernel (src/core/RenderKernel.cu:75-91)
__device__ __forceinline__ void sample_material(const MaterialRec &m, int kind, curandState *rs, RRay &ray,
                                                const RHit &hit, V3 &mask) {
    switch (kind) {
        case MAT_COAT: coat_sample(m, rs, ray, hit, mask); break;
        case MAT_DIFF: diff_sample(m, rs, ray, hit, mask); break;
        case MAT_METAL: metal_sample(m, rs, ray, hit, mask); break;
        case MAT_SPEC: spec_sample(m, ray, hit, mask); break;
        case MAT_REFR: refr_sample(rs, ray, hit, mask); break;
        default: break;  // materials the reference does not know leave the ray unchanged
    }
}

// renderKernel (src/core/RenderKernel.cu:27-95)
__device__ V3 radiance(const CompatArgs &a, curandState *rs, RRay ray, uint32_t &err) {
    V3 mask(1.0f, 1.0f, 1.0f);
    V3 acc(0.0f, 0.0f, 0.0f);
    for (int bounce = 0; bounce < 10; bounce++) {
        const float4 r0 = make_float4(ray.o.x, ray.o.y, ray.o.z, ray.d.x);
        const float4 r1 = make_float4(ray.d.y, ray.d.z, ray.tmin, ray.tmax);
        const TraceResult tr = traverse<true>(a.bvh, r0, r1, err);
        RHit hit;
        hit.distance = tr.t;
        hit.index = -1;
        hit.mat = -1;
        if (tr.addr >= 0) {
            hit.index = __ldg(a.bvh.tri_idx + tr.addr);
            hit.mat = (int)__ldg(a.bvh.mat_idx + tr.addr);
            hit_normal(a.bvh, tr.addr, tr.u, tr.v, hit.normal.x, hit.normal.y, hit.normal.z);
        }
        RHit gh;
        gh.index = -1;
        gh.mat = -1;
        gh.distance = ray.tmax;
        for (int i = 0; i < a.num_geoms; i++) {
            const GeomRec g = a.geoms[i];
            if (g.kind == GEOM_SPHERE) gh = sphere_hit(g, ray.o, ray.d, ray.tmax);
            else if (g.kind == GEOM_PLANE) gh = plane_hit(g, ray.o, ray.d, ray.tmax);
            if (gh.distance < ray.tmax) {
                gh.index = i;
                if (hit_less(gh, hit)) {
                    gh.mat = g.mat;
                    hit = gh;
                }
            }
        }
        if ((double)hit.distance > 1e19) {
            acc = r_madd(mask, env_lookup(a, ray.d), acc);
            return acc;
        }
        hit_frame(hit, ray);
        if (hit.mat < 0 || hit.mat >= a.num_materials) return acc;  // no material: stop the path
        const MaterialRec m = a.materials[hit.mat];
        acc = r_madd(mask, V3(m.emission[0], m.emission[1], m.emission[2]), acc);
        sample_material(m, m.kind, rs, ray, hit, mask);
    }
    return acc;
}

// The primary ray of one sample (src/core/RenderKernel.cu:131-197): jitter and, with an aperture,
// a lens point drawn from rs; pixel_y counts from the image's bottom row.
__device__ __forceinline__ RRay camera_ray(const CompatArgs &a, int pixel_x, int pixel_y, curandState *rs) {
    const int width = a.cam.width;
    const int height = a.cam.height;
    const V3 cam_pos(a.cam.position[0], a.cam.position[1], a.cam.position[2]);
    const V3 view = r_normalize(V3(a.cam.view[0], a.cam.view[1], a.cam.view[2]));
    const V3 up = r_normalize(V3(a.cam.up[0], a.cam.up[1], a.cam.up[2]));
    const V3 haxis = r_normalize(r_cross(view, up));
    const V3 vaxis = r_normalize(r_cross(haxis, view));
    const V3 middle = r_add(cam_pos, view);
    const float deg = __fdiv_rn(a.meta.pi, 180.0f);
    const V3 horizontal = r_mul(haxis, tanf(__fmul_rn(__fmul_rn(a.cam.fov[0], 0.5f), deg)));
    const V3 vertical = r_mul(vaxis, tanf(__fmul_rn(__fmul_rn(-a.cam.fov[1], 0.5f), deg)));
    const float jx = __fsub_rn(curand_uniform(rs), 0.5f);
    const float jy = __fsub_rn(curand_uniform(rs), 0.5f);
    const float sx = __fdiv_rn(__fadd_rn(jx, (float)pixel_x), (float)(width - 1));
    const float sy = __fdiv_rn(__fadd_rn(jy, (float)pixel_y), (float)(height - 1));
    const float ax = __fmaf_rn(2.0f, sx, -1.0f);
    const float ay = __fmaf_rn(2.0f, sy, -1.0f);
    const V3 point = r_madd(vertical, ay, r_madd(horizontal, ax, middle));
    const V3 on_plane = r_madd(r_sub(point, cam_pos), a.cam.focal, cam_pos);
    V3 aperture_point = cam_pos;
    if ((double)a.cam.aperture > 0.00001) {
        const float rnd1 = curand_uniform(rs);
        const float rnd2 = curand_uniform(rs);
        const float angle = __fmul_rn(a.meta.two_pi, rnd1);
        const float dist = __fmul_rn(a.cam.aperture, __fsqrt_rn(rnd2));
        const float apx = __fmul_rn(cosf(angle), dist);
        const float apy = __fmul_rn(sinf(angle), dist);
        aperture_point = r_madd(vaxis, apy, r_madd(haxis, apx, cam_pos));
    }
    // apertureToImagePlane.normalize() rounds as r_normalize_yx, the second normalize as
    // r_normalize (measured on primary rays recorded in the reference's own kernel)
    V3 dir = r_normalize_yx(r_sub(on_plane, aperture_point));
    dir = r_normalize(dir);
    RRay ray;
    ray.o = aperture_point;
    ray.d = dir;
    ray.tmin = 0.01f;  // tMin, tMax of pathTracingKernel (:110-111)
    ray.tmax = 1e20f;
    return ray;
}

// pathTracingKernel (src/core/RenderKernel.cu:97-206): one thread per pixel, 16x16 blocks.
__global__ void __launch_bounds__(256) render_compat_kernel(CompatArgs a) {
    const unsigned x = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned y = blockIdx.y * blockDim.y + threadIdx.y;
    const int width = a.cam.width;
    const int height = a.cam.height;
    const int thread_id = (int)((blockIdx.x + blockIdx.y * gridDim.x) * (blockDim.x * blockDim.y) +
                                (threadIdx.y * blockDim.x) + threadIdx.x);
    curandState rs;
    curand_init((unsigned long long)(a.meta.hashed_frame + (unsigned)thread_id), 0, 0, &rs);
    uint32_t err = 0;
    V3 final_color(0.0f, 0.0f, 0.0f);
    const int i = (int)((unsigned)(height - (int)y - 1) * (unsigned)width + x);
    const int pixel_x = (int)x;
    const int pixel_y = height - (int)y - 1;
    for (int s = 0; s < a.meta.samples; s++) {
        const RRay ray = camera_ray(a, pixel_x, pixel_y, &rs);
        const V3 L = radiance(a, &rs, ray, err);
        final_color = r_madd(L, __fdiv_rn(1.0f, (float)a.meta.samples), final_color);
    }
    float *px = a.accum + 3ll * i;
    px[0] = __fadd_rn(px[0], final_color.x);
    px[1] = __fadd_rn(px[1], final_color.y);
    px[2] = __fadd_rn(px[2], final_color.z);
    if (err) atomicOr(a.err, err);
}

__device__ __forceinline__ V3 ld3(const float *p) { return V3(p[0], p[1], p[2]); }
__device__ __forceinline__ void st3(float *p, const V3 &v) {
    p[0] = v.x;
    p[1] = v.y;
    p[2] = v.z;
}

// tt_compat_replay: one recorded interaction per thread (grid-stride)
__global__ void compat_replay_kernel(CompatArgs a, const tt_compat_interaction *in, long long n,
                                     tt_compat_interaction *out) {
    static_assert(sizeof(curandState) == 48, "curand XORWOW state is 12 words");
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        tt_compat_interaction r = in[i];
        if (r.kind == 5) {  // environment lookup at a miss
            st3(r.out_mask, env_lookup(a, ld3(r.d)));
            out[i] = r;
            continue;
        }
        if (r.kind == 6) {  // a sample's primary ray for the pixel of thread r.thread
            const int gx = a.cam.width / 16;
            const int block = r.thread / 256, lane = r.thread % 256;
            const int x = (block % gx) * 16 + lane % 16, y = (block / gx) * 16 + lane / 16;
            curandState st;
            if (r.seq < 0)  // the thread's first sample: the state pathTracingKernel seeds
                curand_init((unsigned long long)(a.meta.hashed_frame + (unsigned)r.thread), 0, 0, &st);
            else
                memcpy(&st, r.rng, sizeof(st));
            const RRay ray = camera_ray(a, x, a.cam.height - y - 1, &st);
            st3(r.out_o, ray.o);
            st3(r.out_d, ray.d);
            r.tmin = ray.tmin;
            r.tmax = ray.tmax;
            memcpy(r.out_rng, &st, sizeof(st));
            out[i] = r;
            continue;
        }
        RRay ray;
        ray.o = ld3(r.o);
        ray.d = ld3(r.d);
        ray.tmin = r.tmin;
        ray.tmax = r.tmax;
        RHit mine;
        mine.normal = ld3(r.normal);
        mine.distance = r.distance;
        hit_frame(mine, ray);
        RHit h = mine;  // the sampler sees the recorded n / nl / point
        h.n = ld3(r.n);
        h.nl = ld3(r.nl);
        h.point = ld3(r.point);
        st3(r.n, mine.n);
        st3(r.nl, mine.nl);
        st3(r.point, mine.point);
        curandState st;
        memcpy(&st, r.rng, sizeof(st));
        {
            curandState c = st;
            r.u0 = curand_uniform(&c);
        }
        V3 mask = ld3(r.mask);
        if (r.material >= 0 && r.material < a.num_materials && r.kind >= MAT_DIFF && r.kind <= MAT_COAT) {
            sample_material(a.materials[r.material], r.kind, &st, ray, h, mask);
        } else {
            r.kind = -1;  // not a record this renderer can replay
        }
        st3(r.out_o, ray.o);
        st3(r.out_d, ray.d);
        st3(r.out_mask, mask);
        memcpy(r.out_rng, &st, sizeof(st));
        out[i] = r;
    }
}

}  // namespace tt

// ---- renderer handle (struct tt_renderer: tt_device.h) ---------------------------------------------
using namespace tt;

static tt_status cuda_fail_r(cudaError_t e, const char *what) {
    return fail(TT_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define TT_CUDA_R(call)                                       \
    do {                                                      \
        cudaError_t e_ = (call);                              \
        if (e_ != cudaSuccess) return cuda_fail_r(e_, #call); \
    } while (0)

static void renderer_release(tt_renderer *r) {
    if (!r) return;
    native_release(r);
    cudaFree(r->materials);
    cudaFree(r->geoms);
    cudaFree(r->env);
    cudaFree(r->err);
}

extern "C" {

tt_status tt_renderer_create(const tt_dbvh *bvh, const tt_scene *scene, tt_renderer **out) {
    if (!bvh || !scene || !out) return fail(TT_ERR_INVALID, "null argument");
    const Scene &sc = scene->s;
    auto *r = new tt_renderer();
    r->bvh = dbvh_view(bvh);
    dbvh_bounds(bvh, r->order_lo, r->order_hi);
    auto up = [&](void **dst, const void *src, size_t bytes) -> cudaError_t {
        if (!bytes) return cudaSuccess;
        cudaError_t e = cudaMalloc(dst, bytes);
        if (e != cudaSuccess) return e;
        return cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice);
    };
    cudaError_t e = up((void **)&r->materials, sc.materials.data(), sizeof(MaterialRec) * sc.materials.size());
    if (e == cudaSuccess) e = up((void **)&r->geoms, sc.geoms.data(), sizeof(GeomRec) * sc.geoms.size());
    std::vector<float4> env4((size_t)sc.env_w * sc.env_h);
    for (size_t i = 0; i < env4.size(); i++)
        env4[i] = make_float4(sc.env_rgb[3 * i], sc.env_rgb[3 * i + 1], sc.env_rgb[3 * i + 2], 0.f);
    if (e == cudaSuccess) e = up((void **)&r->env, env4.data(), sizeof(float4) * env4.size());
    if (e == cudaSuccess) e = cudaMalloc((void **)&r->err, 256);
    if (e == cudaSuccess) e = cudaMemset(r->err, 0, 256);
    if (e != cudaSuccess) {
        renderer_release(r);
        delete r;
        return fail(TT_ERR_OOM, std::string("renderer upload: ") + cudaGetErrorString(e));
    }
    r->num_materials = (int)sc.materials.size();
    r->num_geoms = (int)sc.geoms.size();
    r->env_w = sc.env_w;
    r->env_h = sc.env_h;
    tt_status st = native_setup(r, sc.geoms);
    if (st != TT_OK) {
        renderer_release(r);
        delete r;
        return st;
    }
    *out = r;
    return TT_OK;
}

void tt_renderer_free(tt_renderer *r) {
    renderer_release(r);
    delete r;
}

tt_status tt_render_compat(tt_renderer *r, const tt_camera_meta *cam, const tt_render_meta *meta, float *d_accum,
                           void *stream) {
    if (!r || !cam || !meta || !d_accum) return fail(TT_ERR_INVALID, "null argument");
    if (cam->width < 16 || cam->height < 16 || meta->samples < 1)
        return fail(TT_ERR_INVALID, "image must be at least 16 x 16 and samples >= 1");
    CompatArgs a;
    a.bvh = r->bvh;
    a.materials = r->materials;
    a.num_materials = r->num_materials;
    a.geoms = r->geoms;
    a.num_geoms = r->num_geoms;
    a.env = r->env_w > 0 ? r->env : nullptr;
    a.env_w = r->env_w;
    a.env_h = r->env_h;
    a.cam = *cam;
    a.meta = *meta;
    a.accum = d_accum;
    a.err = r->err;
    dim3 block(16, 16, 1);
    dim3 grid(cam->width / 16, cam->height / 16, 1);
    render_compat_kernel<<<grid, block, 0, (cudaStream_t)stream>>>(a);
    TT_CUDA_R(cudaGetLastError());
    return TT_OK;
}

tt_status tt_renderer_check(tt_renderer *r, void *stream) {
    if (!r) return fail(TT_ERR_INVALID, "null renderer");
    unsigned int w = 0;
    TT_CUDA_R(cudaMemcpyAsync(&w, r->err, 4, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    TT_CUDA_R(cudaStreamSynchronize((cudaStream_t)stream));
    if (w) {
        TT_CUDA_R(cudaMemset(r->err, 0, 4));
        if (w & kErrStack) return fail(TT_ERR_BOUNDS, "traversal stack overflow during rendering");
        if (w & kErrIter) return fail(TT_ERR_TIMEOUT, "traversal iteration cap reached during rendering");
        if (w & kErrOrder) return fail(TT_ERR_BOUNDS, "ray ordering: a slot index out of range during rendering");
        if (w & kErrStream) return fail(TT_ERR_TIMEOUT, "a streamed render ended with paths unfinished");
        return fail(TT_ERR_TIMEOUT, "a radiance-cache tensor-core wait ran out during rendering");
    }
    return TT_OK;
}

tt_status tt_compat_replay(const tt_renderer *r, const tt_camera_meta *cam, const tt_render_meta *meta,
                           const tt_compat_interaction *d_in, int64_t n, tt_compat_interaction *d_out, void *stream) {
    if (!r || !cam || !meta || (n > 0 && (!d_in || !d_out))) return fail(TT_ERR_INVALID, "null argument");
    if (cam->width < 16 || cam->height < 16) return fail(TT_ERR_INVALID, "image must be at least 16 x 16");
    if (n < 0) return fail(TT_ERR_INVALID, "negative record count");
    if (n == 0) return TT_OK;
    CompatArgs a{};
    a.materials = r->materials;
    a.num_materials = r->num_materials;
    a.env = r->env_w > 0 ? r->env : nullptr;
    a.env_w = r->env_w;
    a.env_h = r->env_h;
    a.meta = *meta;
    a.cam = *cam;
    const int threads = 256;
    const long long blocks = std::min<long long>((n + threads - 1) / threads, 152ll * 16);
    compat_replay_kernel<<<(unsigned)blocks, threads, 0, (cudaStream_t)stream>>>(a, d_in, (long long)n, d_out);
    TT_CUDA_R(cudaGetLastError());
    return TT_OK;
}

}  // extern "C"
