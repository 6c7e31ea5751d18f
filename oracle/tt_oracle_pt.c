/*
 * ORACLE — test infrastructure, not product code.
 *
 * A CPU restatement of the native path tracer (trenchanttracer_gb300/csrc/tt_render_native.cu,
 * whose documentation states the integrator), written independently in C with the same
 * sequence of IEEE operations (every fused multiply-add explicit, -ffp-contract=off), so that a
 * small image rendered here must equal the GPU's bit for bit: the same PCG32 streams, the same
 * own sin/cos/atan (Cody-Waite reduction + Taylor series; atan by the half-angle identity), the
 * same environment tables (sequential FP64 prefix sums), the same traversal (tt_oracle.c, device
 * arithmetic) and the same per-pixel accumulation order. Paths are traced one after another.
 * This file includes tt_oracle.c and is the one compiled into liboracle.so.
 */
#include "tt_oracle.c"

#include <stdlib.h>

typedef struct { float x, y, z; } V3;

#define KPI 3.14159265358979323846f
#define KTWOPI 6.28318530717958647692f
#define KINVPI 0.318309886183790671538f
#define KPIO2HI 1.57079637050628662109375f
#define KPIO2LO (-4.37113900018624283e-8f)
#define KTWOOPI 0.636619772367581343076f

static V3 v3(float x, float y, float z) { V3 r = {x, y, z}; return r; }
static float dot3(V3 a, V3 b) { return fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x)); }
static V3 add3(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static V3 sub3(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static V3 muls(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
static V3 mulv(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
static V3 madd3(V3 a, float s, V3 c) { return v3(fmaf(a.x, s, c.x), fmaf(a.y, s, c.y), fmaf(a.z, s, c.z)); }
static V3 cross3(V3 a, V3 b) {
    return v3(fmaf(a.y, b.z, -(a.z * b.y)), fmaf(a.z, b.x, -(a.x * b.z)), fmaf(a.x, b.y, -(a.y * b.x)));
}
static V3 norm3(V3 a) { return muls(a, 1.0f / sqrtf(dot3(a, a))); }
static float maxc3(V3 a) { float m = a.x > a.y ? a.x : a.y; return m > a.z ? m : a.z; }
static float lum(float r, float g, float b) { return fmaf(0.0722f, b, fmaf(0.7152f, g, 0.2126f * r)); }

static void o_sincos(float x, float *s, float *c) {
    const float k = nearbyintf(x * KTWOOPI);
    float r = fmaf(-k, KPIO2HI, x);
    r = fmaf(-k, KPIO2LO, r);
    const float r2 = r * r;
    float ps = fmaf(r2, 2.75573192239858906526e-6f, -1.98412698412698412698e-4f);
    ps = fmaf(ps, r2, 8.33333333333333333333e-3f);
    ps = fmaf(ps, r2, -1.66666666666666666667e-1f);
    const float sr = fmaf(ps * r2, r, r);
    float pc = fmaf(r2, 2.48015873015873015873e-5f, -1.38888888888888888889e-3f);
    pc = fmaf(pc, r2, 4.16666666666666666667e-2f);
    pc = fmaf(pc, r2, -0.5f);
    const float cr = fmaf(pc, r2, 1.0f);
    switch (((int)k) & 3) {
        case 0: *s = sr; *c = cr; break;
        case 1: *s = cr; *c = -sr; break;
        case 2: *s = -sr; *c = -cr; break;
        default: *s = -cr; *c = sr; break;
    }
}

static float o_atan_pos(float x) {
    int inv = 0;
    if (x > 1.0f) { x = 1.0f / x; inv = 1; }
    x = x / (1.0f + sqrtf(fmaf(x, x, 1.0f)));
    x = x / (1.0f + sqrtf(fmaf(x, x, 1.0f)));
    const float x2 = x * x;
    float p = fmaf(x2, 7.69230769230769230769e-2f, -9.09090909090909090909e-2f);
    p = fmaf(p, x2, 1.11111111111111111111e-1f);
    p = fmaf(p, x2, -1.42857142857142857143e-1f);
    p = fmaf(p, x2, 2.0e-1f);
    p = fmaf(p, x2, -3.33333333333333333333e-1f);
    float a = fmaf(p * x2, x, x);
    a = a * 4.0f;
    if (inv) a = (KPIO2HI + KPIO2LO) - a;
    return a;
}

static float o_atan2(float y, float x) {
    const float ax = x < 0.0f ? -x : x, ay = y < 0.0f ? -y : y;
    float a;
    if (ax == 0.0f && ay == 0.0f) a = 0.0f;
    else if (ax >= ay) a = o_atan_pos(ay / ax);
    else a = (KPIO2HI + KPIO2LO) - o_atan_pos(ax / ay);
    if (x < 0.0f) a = KPI - a;
    return y < 0.0f ? -a : a;
}

static float o_acos(float y) {
    if (y > 1.0f) y = 1.0f;
    if (y < -1.0f) y = -1.0f;
    return o_atan2(sqrtf((1.0f - y) * (1.0f + y)), y);
}

typedef struct { uint64_t state, inc; } Pcg;
static uint32_t o_pcg(Pcg *g) {
    const uint64_t old = g->state;
    g->state = old * 6364136223846793005ull + g->inc;
    const uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    const uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((0u - rot) & 31u));
}
static float o_unif(Pcg *g) { return (float)(o_pcg(g) >> 8) * (1.0f / 16777216.0f); }

static void o_onb(V3 n, V3 *t, V3 *b) {
    const float sgn = n.z >= 0.0f ? 1.0f : -1.0f;
    const float a = -1.0f / (sgn + n.z);
    const float bb = (n.x * n.y) * a;
    *t = v3(fmaf(sgn * n.x, n.x * a, 1.0f), sgn * bb, -sgn * n.x);
    *b = v3(bb, fmaf(n.y * n.y, a, sgn), -n.y);
}
static V3 o_world(V3 l, V3 t, V3 b, V3 n) { return madd3(n, l.z, madd3(b, l.y, muls(t, l.x))); }

/* ---- scene given to the oracle -------------------------------------------------------------- */
typedef struct {
    int32_t kind;
    float emission[3], color[3], color2[3];
    float roughness, ior, pad[4];
} Mat;
typedef struct {
    int32_t kind, mat;
    float radius, pad, p0[3], p1[3], p2[3], pad2[3];
} Geo;
typedef struct {
    int32_t width, height;
    float position[3], view[3], up[3], fov[2], aperture, focal;
} Cam;
typedef struct {
    int32_t spp, sample_offset, max_depth, rr_depth;
    uint32_t seed;
    float env_scale, ray_eps;
    int32_t flags;
} Params;

typedef struct {
    const Bvh *bvh;
    const Mat *mats;
    int nmat;
    const Geo *geos;
    int ngeo;
    const float *env; /* w*h*3 */
    int ew, eh;
    const float *marg, *cond;
    float scale;
} World;

static int o_env_texel(const World *w, V3 d) {
    float lx = o_atan2(d.x, d.z);
    if (lx < 0.0f) lx = lx + KTWOPI;
    const float u = lx / KTWOPI;
    const float v = o_acos(d.y) / KPI;
    int x = (int)(u * (float)w->ew), y = (int)(v * (float)w->eh);
    x = x < 0 ? 0 : (x >= w->ew ? w->ew - 1 : x);
    y = y < 0 ? 0 : (y >= w->eh ? w->eh - 1 : y);
    return y * w->ew + x;
}
static V3 o_env_rad(const World *w, int t) {
    return v3(w->env[3 * t] * w->scale, w->env[3 * t + 1] * w->scale, w->env[3 * t + 2] * w->scale);
}
static float o_env_pdf(const World *w, int texel, float st) {
    if (st <= 0.0f) return 0.0f;
    const int y = texel / w->ew, x = texel - y * w->ew;
    const float pr = w->marg[y + 1] - w->marg[y];
    const float pc = w->cond[(size_t)y * (w->ew + 1) + x + 1] - w->cond[(size_t)y * (w->ew + 1) + x];
    const float jac = ((float)w->ew * (float)w->eh) / (((2.0f * KPI) * KPI) * st);
    return (pr * pc) * jac;
}
static int o_cdf_search(const float *cdf, int n, float u) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (cdf[mid + 1] <= u) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}
static float o_env_sample(const World *w, float u1, float u2, V3 *dir, V3 *le) {
    const int y = o_cdf_search(w->marg, w->eh, u1);
    const float m0 = w->marg[y], m1 = w->marg[y + 1];
    if (!(m1 > m0)) return 0.0f;
    const float *row = w->cond + (size_t)y * (w->ew + 1);
    const int x = o_cdf_search(row, w->ew, u2);
    const float c0 = row[x], c1 = row[x + 1];
    if (!(c1 > c0)) return 0.0f;
    float dv = (u1 - m0) / (m1 - m0);
    float du = (u2 - c0) / (c1 - c0);
    dv = dv < 0.0f ? 0.0f : (dv > 0.99999994f ? 0.99999994f : dv);
    du = du < 0.0f ? 0.0f : (du > 0.99999994f ? 0.99999994f : du);
    const float v = ((float)y + dv) / (float)w->eh;
    const float u = ((float)x + du) / (float)w->ew;
    float st, ct, sp, cp;
    o_sincos(v * KPI, &st, &ct);
    o_sincos(u * KTWOPI, &sp, &cp);
    *dir = v3(st * sp, ct, st * cp);
    if (st <= 0.0f) return 0.0f;
    *le = o_env_rad(w, y * w->ew + x);
    const float jac = ((float)w->ew * (float)w->eh) / (((2.0f * KPI) * KPI) * st);
    return ((m1 - m0) * (c1 - c0)) * jac;
}
static float o_power(float a, float b) { const float a2 = a * a; return a2 / fmaf(b, b, a2); }

/* ---- BSDFs ------------------------------------------------------------------------------------ */
static float o_ggx_d(float a2, float ch) {
    const float c2 = ch * ch;
    const float den = fmaf(c2, a2 - 1.0f, 1.0f);
    return a2 / ((KPI * den) * den);
}
static float o_ggx_g1(float a2, float c) {
    const float c2 = c * c;
    return (2.0f * c) / (c + sqrtf(fmaf(1.0f - a2, c2, a2)));
}
static V3 o_schlick(V3 f0, float c) {
    const float m = 1.0f - (c < 0.0f ? 0.0f : c);
    const float m2 = m * m;
    const float m5 = (m2 * m2) * m;
    return v3(fmaf(1.0f - f0.x, m5, f0.x), fmaf(1.0f - f0.y, m5, f0.y), fmaf(1.0f - f0.z, m5, f0.z));
}
static V3 o_eval(const Mat *m, V3 n, V3 wo, V3 wi, float *pdf) {
    const float ci = dot3(n, wi);
    *pdf = 0.0f;
    if (ci <= 0.0f) return v3(0, 0, 0);
    if (m->kind == 0) {
        *pdf = ci * KINVPI;
        return v3((m->color[0] * KINVPI) * ci, (m->color[1] * KINVPI) * ci, (m->color[2] * KINVPI) * ci);
    }
    const float co = dot3(n, wo);
    if (co <= 0.0f) return v3(0, 0, 0);
    const float alpha = m->roughness * m->roughness;
    const float a2 = alpha * alpha;
    const V3 h = norm3(add3(wo, wi));
    const float d = o_ggx_d(a2, dot3(n, h));
    const float g1o = o_ggx_g1(a2, co), g1i = o_ggx_g1(a2, ci);
    const V3 f = o_schlick(v3(m->color[0], m->color[1], m->color[2]), dot3(wi, h));
    *pdf = (d * g1o) / (4.0f * co);
    return muls(f, ((d * g1o) * g1i) / (4.0f * co));
}
static V3 o_reflect(V3 wo, V3 n) { return sub3(muls(n, 2.0f * dot3(wo, n)), wo); }

typedef struct { V3 wi, weight; float pdf; int specular; } Bs;

static Bs o_sample(const Mat *m, V3 n, V3 wo, int entering, float u1, float u2, float u3) {
    Bs s;
    s.pdf = 0.0f;
    s.specular = 1;
    s.weight = v3(0, 0, 0);
    s.wi = v3(0, 0, 0);
    V3 t, b;
    o_onb(n, &t, &b);
    if (m->kind == 0) {
        const float r = sqrtf(u1);
        float sp, cp;
        o_sincos(KTWOPI * u2, &sp, &cp);
        const V3 l = v3(r * cp, r * sp, sqrtf(1.0f - u1));
        s.wi = o_world(l, t, b, n);
        s.pdf = l.z * KINVPI;
        s.weight = v3(m->color[0], m->color[1], m->color[2]);
        s.specular = 0;
        if (!(l.z > 0.0f)) s.weight = v3(0, 0, 0);
    } else if (m->kind == 5) {
        const float alpha = m->roughness * m->roughness;
        const float a2 = alpha * alpha;
        const V3 wl = v3(dot3(wo, t), dot3(wo, b), dot3(wo, n));
        const V3 vh = norm3(v3(alpha * wl.x, alpha * wl.y, wl.z));
        const float lensq = fmaf(vh.y, vh.y, vh.x * vh.x);
        const V3 t1 = lensq > 0.0f ? muls(v3(-vh.y, vh.x, 0.0f), 1.0f / sqrtf(lensq)) : v3(1, 0, 0);
        const V3 t2 = cross3(vh, t1);
        const float r = sqrtf(u1);
        float sp, cp;
        o_sincos(KTWOPI * u2, &sp, &cp);
        const float p1 = r * cp;
        float p2 = r * sp;
        const float sh = 0.5f * (1.0f + vh.z);
        p2 = fmaf(1.0f - sh, sqrtf(fmaf(-p1, p1, 1.0f)), sh * p2);
        const float p3 = sqrtf(fmaxf(0.0f, (1.0f - p1 * p1) - p2 * p2));
        const V3 nh = madd3(vh, p3, madd3(t2, p2, muls(t1, p1)));
        const V3 hl = norm3(v3(alpha * nh.x, alpha * nh.y, fmaxf(0.0f, nh.z)));
        const V3 h = o_world(hl, t, b, n);
        s.wi = o_reflect(wo, h);
        const float ci = dot3(n, s.wi), co = wl.z;
        s.specular = 0;
        if (ci <= 0.0f || co <= 0.0f) return s;
        const float g1o = o_ggx_g1(a2, co), g1i = o_ggx_g1(a2, ci);
        const V3 f = o_schlick(v3(m->color[0], m->color[1], m->color[2]), dot3(s.wi, h));
        s.weight = muls(f, g1i);
        s.pdf = (o_ggx_d(a2, hl.z) * g1o) / (4.0f * co);
    } else if (m->kind == 6 || m->kind == 3) {
        const float ior = m->kind == 3 ? 1.4f : m->ior;
        const float eta = entering ? 1.0f / ior : ior;
        const float ci = dot3(wo, n);
        const float s2t = (eta * eta) * fmaf(-ci, ci, 1.0f);
        float F = 1.0f, ct = 0.0f;
        if (s2t < 1.0f) {
            ct = sqrtf(1.0f - s2t);
            const float rs = fmaf(eta, ci, -ct) / fmaf(eta, ci, ct);
            const float rp = fmaf(-eta, ct, ci) / fmaf(eta, ct, ci);
            F = 0.5f * fmaf(rs, rs, rp * rp);
        }
        if (u1 < F) s.wi = o_reflect(wo, n);
        else s.wi = madd3(n, fmaf(eta, ci, -ct), muls(wo, -eta));
        s.weight = v3(1, 1, 1);
    } else if (m->kind == 2) {
        s.wi = o_reflect(wo, n);
        s.weight = v3(m->color[0], m->color[1], m->color[2]);
    } else if (m->kind == 4) {
        const float ci = dot3(wo, n);
        const float eta = 1.000293f / 1.291f;
        const float s2t = (eta * eta) * fmaf(-ci, ci, 1.0f);
        float F = 1.0f;
        if (s2t < 1.0f) {
            const float ct = sqrtf(1.0f - s2t);
            const float rs = fmaf(eta, ci, -ct) / fmaf(eta, ci, ct);
            const float rp = fmaf(-eta, ct, ci) / fmaf(eta, ct, ci);
            F = 0.5f * fmaf(rs, rs, rp * rp);
        }
        if (u3 < F) {
            s.wi = o_reflect(wo, n);
            s.weight = v3(m->color2[0], m->color2[1], m->color2[2]);
        } else {
            const float r = sqrtf(u1);
            float sp, cp;
            o_sincos(KTWOPI * u2, &sp, &cp);
            s.wi = o_world(v3(r * cp, r * sp, sqrtf(1.0f - u1)), t, b, n);
            s.weight = v3(m->color[0], m->color[1], m->color[2]);
        }
    }
    return s;
}

static void o_analytic(const World *w, V3 o, V3 d, float tmin, float *t, int *prim, float *hu, float *hv) {
    for (int i = 0; i < w->ngeo; i++) {
        const Geo *g = &w->geos[i];
        if (g->kind == 3) {
            const V3 p0 = v3(g->p0[0], g->p0[1], g->p0[2]);
            const V3 e1 = sub3(v3(g->p1[0], g->p1[1], g->p1[2]), p0), e2 = sub3(v3(g->p2[0], g->p2[1], g->p2[2]), p0);
            const V3 P = cross3(d, e2);
            const float det = dot3(e1, P);
            if (det > -1e-12f && det < 1e-12f) continue;
            const float inv = 1.0f / det;
            const V3 T = sub3(o, p0);
            const float u = dot3(T, P) * inv;
            if (u < 0.f || u > 1.f) continue;
            const V3 Q = cross3(T, e1);
            const float v = dot3(d, Q) * inv;
            if (v < 0.f || v > 1.f) continue;
            const float th = dot3(e2, Q) * inv;
            if (th > tmin && th < *t) { *t = th; *prim = -(i + 2); *hu = u; *hv = v; }
        } else if (g->kind == 0) {
            const V3 oc = sub3(v3(g->p0[0], g->p0[1], g->p0[2]), o);
            const float bq = dot3(oc, d);
            const float disc = fmaf(g->radius, g->radius, fmaf(bq, bq, -dot3(oc, oc)));
            if (disc < 0.0f) continue;
            const float sq = sqrtf(disc);
            float th = bq - sq;
            if (!(th > tmin)) th = bq + sq;
            if (th > tmin && th < *t) { *t = th; *prim = -(i + 2); *hu = 0.f; *hv = 0.f; }
        }
    }
}

static float o_eps(const Params *p, V3 q) {
    const float m = fmaxf(fmaxf(fabsf(q.x), fabsf(q.y)), fabsf(q.z));
    return p->ray_eps * fmaxf(1.0f, m);
}

/* Closest (mode 1) or any (mode 0) hit over triangles and analytic objects. */
static void o_trace(const World *w, V3 o, V3 d, float tmin, float tmax, int closest, float *t, int *prim, float *hu,
                    float *hv) {
    const float r[8] = {o.x, o.y, o.z, d.x, d.y, d.z, tmin, tmax};
    int32_t id;
    trace_one(w->bvh, r, closest, ORACLE_SLAB_FMA | ORACLE_CROSS_A | ORACLE_DOT_B | ORACLE_INTERP_B, &id, t, 0, 0, 0);
    *prim = g_hit_addr;
    *hu = g_hit_u;
    *hv = g_hit_v;
    if (!closest && *prim >= 0) return;
    if (w->ngeo) o_analytic(w, o, d, tmin, t, prim, hu, hv);
}

static V3 o_hit_normal(const World *w, int prim, float u, float v) {
    const float *n0 = w->bvh->norms + 4 * (int64_t)prim, *n1 = n0 + 4, *n2 = n0 + 8;
    const float ww = (1.0f - u) - v;
    const int ar = ORACLE_INTERP_B;
    return v3(interp_c(n0[0], n1[0], n2[0], ww, u, v, ar), interp_c(n0[1], n1[1], n2[1], ww, u, v, ar),
              interp_c(n0[2], n1[2], n2[2], ww, u, v, ar));
}

/* One path; returns its radiance. */
static V3 o_path(const World *w, const Cam *cam, float tanx, float tany, const Params *p, int64_t gid, int npix) {
    const int pixel = (int)(gid % npix);
    const int px = pixel % cam->width, py = pixel / cam->width;
    Pcg g;
    g.state = 0;
    g.inc = ((uint64_t)gid << 1u) | 1u;
    o_pcg(&g);
    g.state += (uint64_t)p->seed * 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull;
    o_pcg(&g);
    const V3 cpos = v3(cam->position[0], cam->position[1], cam->position[2]);
    const V3 view = norm3(v3(cam->view[0], cam->view[1], cam->view[2]));
    const V3 right = norm3(cross3(view, v3(cam->up[0], cam->up[1], cam->up[2])));
    const V3 up = cross3(right, view);
    const float jx = o_unif(&g), jy = o_unif(&g);
    const float sx = (2.0f * (((float)px + jx) / (float)cam->width)) - 1.0f;
    const float sy = 1.0f - 2.0f * (((float)py + jy) / (float)cam->height);
    const V3 dp = madd3(up, sy * tany, madd3(right, sx * tanx, view));
    V3 o = cpos, d;
    if (cam->aperture > 1e-5f) { /* thin lens, as the device raygen */
        const V3 focus = madd3(dp, cam->focal, cpos);
        const float u1 = o_unif(&g), u2 = o_unif(&g);
        const float r = cam->aperture * sqrtf(u1);
        float sp, cp;
        o_sincos(KTWOPI * u2, &sp, &cp);
        o = madd3(up, r * sp, madd3(right, r * cp, cpos));
        d = norm3(sub3(focus, o));
    } else {
        d = norm3(dp);
    }
    V3 beta = v3(1, 1, 1), L = v3(0, 0, 0);
    int specular = 1;
    float last_pdf = 0.0f;
    const int use_env = w->ew > 0;
    for (int depth = 0; depth < p->max_depth;) {
        float t, hu, hv;
        int prim;
        o_trace(w, o, d, 0.0f, 1e20f, 1, &t, &prim, &hu, &hv);
        if (prim == -1) {
            if (use_env) {
                const int texel = o_env_texel(w, d);
                const V3 le = o_env_rad(w, texel);
                float wt = 1.0f;
                if (!specular) {
                    const float st = sqrtf(fmaxf(0.0f, fmaf(-d.y, d.y, 1.0f)));
                    wt = o_power(last_pdf, o_env_pdf(w, texel, st));
                }
                L = madd3(mulv(beta, le), wt, L);
            }
            break;
        }
        const V3 q = madd3(d, t, o);
        V3 n;
        int mat;
        if (prim >= 0) {
            n = o_hit_normal(w, prim, hu, hv);
            mat = (int)w->bvh->mat_idx[prim];
        } else {
            const Geo *gg = &w->geos[-prim - 2];
            mat = gg->mat;
            if (gg->kind == 3) {
                const V3 p0 = v3(gg->p0[0], gg->p0[1], gg->p0[2]);
                n = cross3(sub3(v3(gg->p1[0], gg->p1[1], gg->p1[2]), p0), sub3(v3(gg->p2[0], gg->p2[1], gg->p2[2]), p0));
            } else {
                n = sub3(q, v3(gg->p0[0], gg->p0[1], gg->p0[2]));
            }
        }
        n = norm3(n);
        const V3 wo = v3(-d.x, -d.y, -d.z);
        const int entering = dot3(n, wo) > 0.0f;
        const V3 nl = entering ? n : v3(-n.x, -n.y, -n.z);
        Mat m;
        if (mat >= 0 && mat < w->nmat) m = w->mats[mat];
        else memset(&m, 0, sizeof(m));
        if (m.kind == 1) { m.kind = 5; m.roughness = 0.5f; }
        L = v3(fmaf(beta.x, m.emission[0], L.x), fmaf(beta.y, m.emission[1], L.y), fmaf(beta.z, m.emission[2], L.z));
        const int nee = use_env && !(p->flags & 2) && (m.kind == 0 || m.kind == 5);
        const float eps = o_eps(p, q);
        int shadow = 0;
        V3 sh_o = v3(0, 0, 0), sh_d = v3(0, 0, 0), sh_v = v3(0, 0, 0);
        if (nee) {
            const float u1 = o_unif(&g), u2 = o_unif(&g);
            V3 wi, le;
            const float pl = o_env_sample(w, u1, u2, &wi, &le);
            if (pl > 0.0f) {
                float pb;
                const V3 fc = o_eval(&m, nl, wo, wi, &pb);
                if (maxc3(fc) > 0.0f) {
                    const float wt = o_power(pl, pb);
                    sh_v = muls(mulv(beta, mulv(fc, le)), wt / pl);
                    sh_o = madd3(nl, eps, q);
                    sh_d = wi;
                    shadow = 1;
                }
            }
        }
        const float u1 = o_unif(&g), u2 = o_unif(&g), u3 = o_unif(&g);
        const Bs bs = o_sample(&m, nl, wo, entering, u1, u2, u3);
        int alive = 0;
        if (maxc3(bs.weight) > 0.0f) {
            beta = mulv(beta, bs.weight);
            depth++;
            alive = depth < p->max_depth;
            if (alive && depth >= p->rr_depth) {
                float qs = maxc3(beta);
                qs = qs > 1.0f ? 1.0f : (qs < 0.05f ? 0.05f : qs);
                if (o_unif(&g) >= qs) alive = 0;
                else beta = muls(beta, 1.0f / qs);
            }
            if (alive) {
                const V3 off = dot3(bs.wi, nl) >= 0.0f ? nl : v3(-nl.x, -nl.y, -nl.z);
                o = madd3(off, eps, q);
                d = bs.wi;
                last_pdf = bs.pdf;
                specular = (bs.specular || !nee) ? 1 : 0;
            }
        }
        if (shadow) {
            float st_, su, sv;
            int sp_;
            o_trace(w, sh_o, sh_d, 0.0f, 1e20f, 0, &st_, &sp_, &su, &sv);
            if (sp_ == -1) L = add3(L, sh_v);
        }
        if (!alive) break;
    }
    return L;
}

/* Environment sampling tables: sequential FP64 prefix sums of luminance * sin(theta_row). */
void oracle_env_tables(const float *env, int w, int h, float *marg, float *cond) {
    double *rowsum = (double *)malloc(sizeof(double) * (h > 0 ? h : 1));
    for (int y = 0; y < h; y++) {
        float st, ct;
        o_sincos((((float)y + 0.5f) / (float)h) * KPI, &st, &ct);
        double acc = 0.0;
        for (int x = 0; x < w; x++) {
            const float *c = env + 3 * ((size_t)y * w + x);
            const float wt = lum(c[0], c[1], c[2]) * st;
            acc += (double)(wt > 0.0f ? wt : 0.0f);
        }
        rowsum[y] = acc;
        float *row = cond + (size_t)y * (w + 1);
        row[0] = 0.0f;
        double acc2 = 0.0;
        for (int x = 0; x < w; x++) {
            const float *c = env + 3 * ((size_t)y * w + x);
            const float wt = lum(c[0], c[1], c[2]) * st;
            acc2 += (double)(wt > 0.0f ? wt : 0.0f);
            row[x + 1] = acc > 0.0 ? (float)(acc2 / acc) : (float)(x + 1) / (float)w;
        }
    }
    double total = 0.0;
    for (int y = 0; y < h; y++) total += rowsum[y];
    double acc = 0.0;
    marg[0] = 0.0f;
    for (int y = 0; y < h; y++) {
        acc += rowsum[y];
        marg[y + 1] = total > 0.0 ? (float)(acc / total) : (float)(y + 1) / (float)h;
    }
    free(rowsum);
}

/* Renders spp samples per pixel into accum (W*H*3 floats, added in sample order). */
int oracle_render_native(const void *nodes, const void *verts, const void *norms, const int32_t *tri_idx,
                         const uint32_t *mat_idx, const void *mats, int nmat, const void *geos, int ngeo,
                         const float *env, int ew, int eh, const float *marg, const float *cond, const void *cam_,
                         const void *params_, float tanx, float tany, float *accum, int threads) {
    const Cam *cam = (const Cam *)cam_;
    const Params *p = (const Params *)params_;
    Bvh b = {(const float *)nodes, (const float *)verts, (const float *)norms, tri_idx, mat_idx};
    World w = {&b, (const Mat *)mats, nmat, (const Geo *)geos, ngeo, env, ew, eh, marg, cond, p->env_scale};
    const int npix = cam->width * cam->height;
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 64)
    for (int pix = 0; pix < npix; pix++) {
        for (int s = 0; s < p->spp; s++) {
            const int64_t gid = (int64_t)(p->sample_offset + s) * npix + pix;
            const V3 L = o_path(&w, cam, tanx, tany, p, gid, npix);
            accum[3 * (size_t)pix] += L.x;
            accum[3 * (size_t)pix + 1] += L.y;
            accum[3 * (size_t)pix + 2] += L.z;
        }
    }
    return 0;
}
