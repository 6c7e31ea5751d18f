/*
 * ORACLE — test infrastructure, not product code.
 *
 * A CPU restatement of the reference's ray traversal, intersect(ray, bvh, needClosestHit)
 * (include/geometry/IntersectKernel.cuh:78-296), over the compact BVH arrays read from a
 * bvh.cache (src/bvh/BVHCompact.cpp:319-375). Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg use it, always to check results or as the reported CPU baseline.
 *
 * Per ray it follows the reference's single-lane semantics: near-first order with the far
 * child pushed (:149-167), one postponed leaf, the warp vote reduced to this lane
 * (:169-203), the Moller-Trumbore leaf loop with the det > 1e-5 / det < -1e-5 branches
 * (:209-271) and the id remap (:285-290). Closest-hit results of a warp-wide traversal differ
 * from this only in how stale the culling distance is while nodes are visited, which changes
 * nothing but float corner cases; any-hit results are identical (first accepted triangle in
 * DFS order).
 *
 * Arithmetic modes (`arith` flags): 0 rounds every product and sum separately, which is the
 * reference compiled for an x86 host (no FMA). The ORACLE_* flags select where an FMA replaces
 * a multiply + add, so that the same restatement reproduces the contraction nvcc applies to
 * the reference's device code; which combination that is gets pinned against outputs of the
 * reference kernel itself (tests/golden).
 *
 * Counters (optional, 4 x uint32 per ray): inner nodes fetched, leaves entered, triangles
 * tested, accepted hit updates — the N_node, N_leaf, N_tri and hit terms of the bytes-per-ray
 * roofline.
 */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <string.h>

#define ORACLE_SLAB_FMA 1
#define ORACLE_CROSS_A 2   /* a.y*b.z - a.z*b.y -> fma(a.y, b.z, -(a.z*b.y)) */
#define ORACLE_CROSS_B 4   /*                    -> fma(-a.z, b.y, a.y*b.z)  */
#define ORACLE_DOT_A 8     /* x*x'+y*y'+z*z'    -> fma(z, z', fma(y, y', x*x')) */
#define ORACLE_DOT_B 16    /*                    -> fma(z, z', fma(x, x', y*y')) */
#define ORACLE_INTERP_A 32 /* n0*w + n1*u + n2*v -> fma(n2, v, fma(n1, u, n0*w)) */
#define ORACLE_INTERP_B 64 /*                    -> fma(n2, v, fma(n0, w, n1*u)) */

#define SENTINEL 0x76543210
#define STACK_SIZE 128

static inline int f2i(float f) { int i; memcpy(&i, &f, 4); return i; }
static inline float i2f(int i) { float f; memcpy(&f, &i, 4); return f; }
static inline int imin(int a, int b) { return a < b ? a : b; }
static inline int imax(int a, int b) { return a > b ? a : b; }

static inline float slab(float b, float idir, float ood, int arith) {
    if (arith & ORACLE_SLAB_FMA) return fmaf(b, idir, -ood);
    float p = b * idir;
    return p - ood;
}

static inline float cross_c(float ay, float bz, float az, float by, int arith) {
    if (arith & ORACLE_CROSS_A) return fmaf(ay, bz, -(az * by));
    if (arith & ORACLE_CROSS_B) return fmaf(-az, by, ay * bz);
    float p = ay * bz;
    float q = az * by;
    return p - q;
}

static inline float dot_c(float ax, float ay, float az, float bx, float by, float bz, int arith) {
    if (arith & ORACLE_DOT_A) return fmaf(az, bz, fmaf(ay, by, ax * bx));
    if (arith & ORACLE_DOT_B) return fmaf(az, bz, fmaf(ax, bx, ay * by));
    float p = ax * bx;
    float q = ay * by;
    float r = az * bz;
    float s = p + q;
    return s + r;
}

static inline float interp_c(float n0, float n1, float n2, float w, float u, float v, int arith) {
    if (arith & ORACLE_INTERP_A) return fmaf(n2, v, fmaf(n1, u, n0 * w));
    if (arith & ORACLE_INTERP_B) return fmaf(n2, v, fmaf(n0, w, n1 * u));
    float a = n0 * w;
    float b = n1 * u;
    float c = n2 * v;
    float s = a + b;
    return s + c;
}

/* spanBeginKepler / spanEndKepler: float min/max for x, y; signed-int min/max on the float bits
 * for z and the fourth operand (IntersectKernel.cuh:22-60). */
static inline float span_begin(float a0, float a1, float b0, float b1, float c0, float c1, float d) {
    int x = imax(f2i(fminf(a0, a1)), f2i(fminf(b0, b1)));
    int y = imax(imin(f2i(c0), f2i(c1)), f2i(d));
    return i2f(imax(x, y));
}
static inline float span_end(float a0, float a1, float b0, float b1, float c0, float c1, float d) {
    int x = imin(f2i(fmaxf(a0, a1)), f2i(fmaxf(b0, b1)));
    int y = imin(imax(f2i(c0), f2i(c1)), f2i(d));
    return i2f(imin(x, y));
}

typedef struct {
    const float *nodes; /* float4 array as floats */
    const float *verts;
    const float *norms;
    const int32_t *tri_idx;
    const uint32_t *mat_idx;
} Bvh;

/* Raw hit of the last trace_one call on this thread: float4 slot (-1 = miss) and barycentrics. */
static _Thread_local int g_hit_addr;
static _Thread_local float g_hit_u, g_hit_v;

/* Returns 0, or -1 when the stack would overflow. */
static int trace_one(const Bvh *b, const float *r, int closest, int arith, int32_t *o_id, float *o_t,
                     int32_t *o_mat, float *o_n, uint32_t *cnt) {
    const float ox = r[0], oy = r[1], oz = r[2], dx = r[3], dy = r[4], dz = r[5], tmin = r[6];
    const float ooeps = 8.27180612553027674871e-25f;
    const float idirx = 1.0f / (fabsf(dx) > ooeps ? dx : copysignf(ooeps, dx));
    const float idiry = 1.0f / (fabsf(dy) > ooeps ? dy : copysignf(ooeps, dy));
    const float idirz = 1.0f / (fabsf(dz) > ooeps ? dz : copysignf(ooeps, dz));
    const float oodx = ox * idirx, oody = oy * idiry, oodz = oz * idirz;
    int stack[STACK_SIZE];
    int sp = 0;
    stack[0] = SENTINEL;
    int leaf = 0, node = 0;
    float dist = r[7];
    int hit_addr = -1;
    float hu = 0.f, hv = 0.f;
    uint32_t n_node = 0, n_leaf = 0, n_tri = 0, n_upd = 0;

    while (node != SENTINEL) {
        while (node >= 0 && node != SENTINEL) {
            const float *n0 = b->nodes + 4 * (int64_t)node;
            n_node++;
            float c0lox = slab(n0[0], idirx, oodx, arith), c0hix = slab(n0[1], idirx, oodx, arith);
            float c0loy = slab(n0[2], idiry, oody, arith), c0hiy = slab(n0[3], idiry, oody, arith);
            float c0loz = slab(n0[8], idirz, oodz, arith), c0hiz = slab(n0[9], idirz, oodz, arith);
            float c1loz = slab(n0[10], idirz, oodz, arith), c1hiz = slab(n0[11], idirz, oodz, arith);
            float c0min = span_begin(c0lox, c0hix, c0loy, c0hiy, c0loz, c0hiz, tmin);
            float c0max = span_end(c0lox, c0hix, c0loy, c0hiy, c0loz, c0hiz, dist);
            float c1lox = slab(n0[4], idirx, oodx, arith), c1hix = slab(n0[5], idirx, oodx, arith);
            float c1loy = slab(n0[6], idiry, oody, arith), c1hiy = slab(n0[7], idiry, oody, arith);
            float c1min = span_begin(c1lox, c1hix, c1loy, c1hiy, c1loz, c1hiz, tmin);
            float c1max = span_end(c1lox, c1hix, c1loy, c1hiy, c1loz, c1hiz, dist);
            int t0 = (c0min <= c0max) && (c0min >= tmin) && (c0min <= 1e20f);
            int t1 = (c1min <= c1max) && (c1min >= tmin) && (c1min <= 1e20f);
            if (!t0 && !t1) {
                node = stack[sp--];
            } else {
                int c0 = f2i(n0[12]), c1 = f2i(n0[13]);
                node = t0 ? c0 : c1;
                if (t0 && t1) {
                    if (c1min < c0min) { int s = node; node = c1; c1 = s; }
                    if (sp + 1 >= STACK_SIZE) return -1;
                    stack[++sp] = c1;
                }
            }
            if (node < 0 && leaf >= 0) {
                leaf = node;
                node = stack[sp--];
            }
            if (leaf < 0) break; /* the vote over this one lane */
        }
        while (leaf < 0) {
            n_leaf++;
            for (int tri = ~leaf;; tri += 3) {
                const float *v0 = b->verts + 4 * (int64_t)tri;
                if ((uint32_t)f2i(v0[0]) == 0x80000000u) break;
                const float *v1 = v0 + 4, *v2 = v0 + 8;
                n_tri++;
                float e1x = v1[0] - v0[0], e1y = v1[1] - v0[1], e1z = v1[2] - v0[2];
                float e2x = v2[0] - v0[0], e2y = v2[1] - v0[1], e2z = v2[2] - v0[2];
                float tvx = ox - v0[0], tvy = oy - v0[1], tvz = oz - v0[2];
                float px = cross_c(dy, e2z, dz, e2y, arith);
                float py = cross_c(dz, e2x, dx, e2z, arith);
                float pz = cross_c(dx, e2y, dy, e2x, arith);
                float det = dot_c(e1x, e1y, e1z, px, py, pz, arith);
                float inv = 1.0f / det;
                float u = dot_c(tvx, tvy, tvz, px, py, pz, arith) * inv;
                float qx = cross_c(tvy, e1z, tvz, e1y, arith);
                float qy = cross_c(tvz, e1x, tvx, e1z, arith);
                float qz = cross_c(tvx, e1y, tvy, e1x, arith);
                float v = dot_c(dx, dy, dz, qx, qy, qz, arith) * inv;
                if (det > 0.00001f) {
                    if (u < 0.0f || u > 1.0f) continue;
                    if (v < 0.0f || (u + v) > 1.0f) continue;
                } else if (det < -0.00001f) {
                    if (u > 0.0f || u < 1.0f) continue;
                    if (v > 0.0f || (u + v) < 1.0f) continue;
                } else {
                    continue;
                }
                float t = dot_c(e2x, e2y, e2z, qx, qy, qz, arith) * inv;
                if (tmin < t && t < dist) {
                    dist = t;
                    hit_addr = tri;
                    hu = u;
                    hv = v;
                    n_upd++;
                    if (!closest) {
                        node = SENTINEL;
                        break;
                    }
                }
            }
            leaf = node;
            if (node < 0) node = stack[sp--];
        }
    }
    *o_t = dist;
    g_hit_addr = hit_addr;
    g_hit_u = hu;
    g_hit_v = hv;
    if (hit_addr >= 0) {
        *o_id = b->tri_idx[hit_addr];
        if (o_mat) *o_mat = (int32_t)b->mat_idx[hit_addr];
        if (o_n) {
            const float *n0 = b->norms + 4 * (int64_t)hit_addr, *n1 = n0 + 4, *n2 = n0 + 8;
            float w = (1.0f - hu) - hv;
            o_n[0] = interp_c(n0[0], n1[0], n2[0], w, hu, hv, arith);
            o_n[1] = interp_c(n0[1], n1[1], n2[1], w, hu, hv, arith);
            o_n[2] = interp_c(n0[2], n1[2], n2[2], w, hu, hv, arith);
        }
    } else {
        *o_id = -1;
        if (o_mat) *o_mat = -1;
        if (o_n) o_n[0] = o_n[1] = o_n[2] = 0.0f;
    }
    if (cnt) {
        cnt[0] = n_node;
        cnt[1] = n_leaf;
        cnt[2] = n_tri;
        cnt[3] = n_upd;
    }
    return 0;
}

/* Traces n rays (8 floats each). Output arrays may be NULL except id and t. Returns the
 * number of rays whose traversal stack would have overflowed (reported as misses). */
int64_t oracle_intersect(const void *nodes, const void *verts, const void *norms, const int32_t *tri_idx,
                         const uint32_t *mat_idx, const float *rays, int64_t n, int closest, int arith,
                         int32_t *out_id, float *out_t, int32_t *out_mat, float *out_normal, uint32_t *counters,
                         int threads) {
    Bvh b = {(const float *)nodes, (const float *)verts, (const float *)norms, tri_idx, mat_idx};
    int64_t overflow = 0;
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 4096) reduction(+ : overflow)
    for (int64_t i = 0; i < n; i++) {
        int rc = trace_one(&b, rays + 8 * i, closest, arith, out_id + i, out_t + i, out_mat ? out_mat + i : 0,
                           out_normal ? out_normal + 3 * i : 0, counters ? counters + 4 * i : 0);
        if (rc) {
            out_id[i] = -1;
            out_t[i] = rays[8 * i + 7];
            overflow++;
        }
    }
    return overflow;
}

int oracle_max_threads(void) { return omp_get_max_threads(); }

/* WangHash::encode (src/util/WangHash.cpp:8-15), the per-frame seed hash. */
uint32_t oracle_wang_hash(uint32_t a) {
    a = (a ^ 61u) ^ (a >> 16u);
    a = a + (a << 3u);
    a = a ^ (a >> 4u);
    a = a * 0x27d4eb2du;
    a = a ^ (a >> 15u);
    return a;
}
