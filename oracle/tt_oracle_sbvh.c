/*
 * ORACLE -- test infrastructure, never part of the product. A plain, single-threaded C restatement
 * of the reference's host SBVH builder and compact emission, used to check this project's builder
 * and as the host build timed in bench.py's reference arm:
 *   BVH::BVH / buildNode / createLeaf        src/bvh/BVH.cpp:3-120
 *   findObjectSplit / performObjectSplit     src/bvh/BVH.cpp:122-164
 *   findSpatialSplit / performSpatialSplit   src/bvh/BVH.cpp:166-300
 *   splitReference / sortCompare             src/bvh/BVH.cpp:302-351
 *   AABB grow / intersect / area             src/bvh/AABB.cpp:3-39
 *   SAHHelper defaults (costs 1, batch 1)    include/bvh/SAHHelper.h:11-19, src/bvh/SAHHelper.cpp
 *   lerp                                     include/util/Sort.h:26-29
 *   BVHCompact::createCompact / getTriangle  src/bvh/BVHCompact.cpp:88-274
 *   BVHCompact::save                         src/bvh/BVHCompact.cpp:319-375
 * Like the reference, the references of the node being built are the top `num` entries of one
 * stack; a leaf pops them (so it lists them last-first) and the right child is built first.
 * Within one node every triangle appears once, so the (centroid, triangle) order is total and the
 * C library's qsort gives the permutation the reference's own quicksort (src/util/Sort.cpp) gives.
 * Compile with -ffp-contract=off: the reference's x86 host build rounds every operation.
 */
#include <float.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef struct {
    float lo[3], hi[3];
} Box;

typedef struct {
    int32_t tri;
    Box b;
} Ref;

typedef struct {
    Box b;
    int leaf;
    int child[2]; /* inner: [0] left, [1] right */
    int lo, hi;   /* leaf: range of the emitted triangle list */
} Node;

typedef struct {
    const float *v, *n;
    const int32_t *vidx, *nidx;
    const uint32_t *mat;
    int leaf_min, leaf_max;
    float min_overlap;
    Ref *refs;
    int nrefs, cap_refs;
    int32_t *tris;
    int ntris, cap_tris;
    Node *nodes;
    int nnodes, cap_nodes;
    int error;
} Builder;

enum { kMaxDepth = 64, kMaxSpatialDepth = 48, kBins = 32 };

static Box box_empty(void) {
    Box b = {{FLT_MAX, FLT_MAX, FLT_MAX}, {-FLT_MAX, -FLT_MAX, -FLT_MAX}};
    return b;
}

/* AABB::grow(Vec3f): min3f / max3f keep the current bound unless the point is beyond it */
static void grow_pt(Box *b, const float *p) {
    for (int d = 0; d < 3; d++) {
        b->lo[d] = b->lo[d] < p[d] ? b->lo[d] : p[d];
        b->hi[d] = b->hi[d] > p[d] ? b->hi[d] : p[d];
    }
}

/* AABB::grow(AABB): by both corners, so an empty box makes this one unbounded */
static void grow_box(Box *b, const Box *o) {
    grow_pt(b, o->lo);
    grow_pt(b, o->hi);
}

static void intersect_box(Box *b, const Box *o) {
    for (int d = 0; d < 3; d++) {
        b->lo[d] = b->lo[d] > o->lo[d] ? b->lo[d] : o->lo[d];
        b->hi[d] = b->hi[d] < o->hi[d] ? b->hi[d] : o->hi[d];
    }
}

static float area(const Box *b) {
    if (!(b->lo[0] <= b->hi[0] && b->lo[1] <= b->hi[1] && b->lo[2] <= b->hi[2])) return 0.0f;
    const float dx = b->hi[0] - b->lo[0], dy = b->hi[1] - b->lo[1], dz = b->hi[2] - b->lo[2];
    return (dx * dy + dy * dz + dz * dx) * 2.0f;
}

static float min1f(float a, float b) { return (a > b) ? b : a; }
static int clamp1i(int v, int lo, int hi) { return v < lo ? lo : v > hi ? hi : v; }

/* float -> int as x86's cvttss2si: NaN and out-of-range values give 0x80000000 */
static int f2i(float f) {
    if (!(f > -2147483648.0f && f < 2147483648.0f)) return INT32_MIN;
    return (int)f;
}

static const float *vert(const Builder *B, int tri, int k) { return B->v + 3 * B->vidx[3 * tri + k]; }

static void push_ref(Builder *B, Ref r) {
    if (B->nrefs == B->cap_refs) {
        B->cap_refs = B->cap_refs ? 2 * B->cap_refs : 1024;
        Ref *p = (Ref *)realloc(B->refs, sizeof(Ref) * (size_t)B->cap_refs);
        if (!p) {
            B->error = 1;
            return;
        }
        B->refs = p;
    }
    B->refs[B->nrefs++] = r;
}

static int new_node(Builder *B) {
    if (B->nnodes == B->cap_nodes) {
        B->cap_nodes = B->cap_nodes ? 2 * B->cap_nodes : 1024;
        Node *p = (Node *)realloc(B->nodes, sizeof(Node) * (size_t)B->cap_nodes);
        if (!p) {
            B->error = 1;
            return 0;
        }
        B->nodes = p;
    }
    memset(&B->nodes[B->nnodes], 0, sizeof(Node));
    return B->nnodes++;
}

/* createLeaf: the node's references popped off the stack into the triangle list */
static int create_leaf(Builder *B, int num, const Box *bounds) {
    if (B->ntris + num > B->cap_tris) {
        while (B->ntris + num > B->cap_tris) B->cap_tris = B->cap_tris ? 2 * B->cap_tris : 4096;
        int32_t *p = (int32_t *)realloc(B->tris, sizeof(int32_t) * (size_t)B->cap_tris);
        if (!p) {
            B->error = 1;
            return 0;
        }
        B->tris = p;
    }
    for (int i = 0; i < num; i++) B->tris[B->ntris++] = B->refs[--B->nrefs].tri;
    const int id = new_node(B);
    if (B->error) return 0;
    B->nodes[id].b = *bounds;
    B->nodes[id].leaf = 1;
    B->nodes[id].lo = B->ntris - num;
    B->nodes[id].hi = B->ntris;
    return id;
}

static int g_sort_dim; /* qsort has no user pointer in C11 */

static int cmp_ref(const void *pa, const void *pb) {
    const Ref *a = (const Ref *)pa, *b = (const Ref *)pb;
    const float ca = a->b.lo[g_sort_dim] + a->b.hi[g_sort_dim];
    const float cb = b->b.lo[g_sort_dim] + b->b.hi[g_sort_dim];
    return (ca < cb) ? -1 : (ca > cb) ? 1 : (a->tri < b->tri) ? -1 : (a->tri > b->tri) ? 1 : 0;
}

static void sort_top(Builder *B, int num, int dim) {
    g_sort_dim = dim;
    qsort(B->refs + B->nrefs - num, (size_t)num, sizeof(Ref), cmp_ref);
}

typedef struct {
    float sah;
    int dim, num_left;
    Box left, right;
} ObjectSplit;

typedef struct {
    float sah;
    int dim;
    float pos;
} SpatialSplit;

static ObjectSplit find_object_split(Builder *B, int num, float node_sah) {
    ObjectSplit s;
    s.sah = FLT_MAX;
    s.dim = 0;
    s.num_left = 0;
    s.left = s.right = box_empty();
    Box *rb_all = (Box *)malloc(sizeof(Box) * (size_t)(num > 1 ? num - 1 : 1));
    if (!rb_all) {
        B->error = 1;
        return s;
    }
    for (int dim = 0; dim < 3; dim++) {
        sort_top(B, num, dim);
        const Ref *r = B->refs + B->nrefs - num;
        Box rb = box_empty();
        for (int i = num - 1; i > 0; i--) {
            grow_box(&rb, &r[i].b);
            rb_all[i - 1] = rb;
        }
        Box lb = box_empty();
        for (int i = 1; i < num; i++) {
            grow_box(&lb, &r[i - 1].b);
            const float sah = node_sah + area(&lb) * (float)i + area(&rb_all[i - 1]) * (float)(num - i);
            if (sah < s.sah) {
                s.sah = sah;
                s.dim = dim;
                s.num_left = i;
                s.left = lb;
                s.right = rb_all[i - 1];
            }
        }
    }
    free(rb_all);
    return s;
}

/* splitReference: the triangle clipped against the plane x[dim] = pos */
static void split_reference(const Builder *B, Ref *left, Ref *right, const Ref *ref, int dim, float pos) {
    left->tri = right->tri = ref->tri;
    left->b = right->b = box_empty();
    const float *v1 = vert(B, ref->tri, 2);
    for (int k = 0; k < 3; k++) {
        const float *v0 = v1;
        v1 = vert(B, ref->tri, k);
        const float v0p = v0[dim], v1p = v1[dim];
        if (v0p <= pos) grow_pt(&left->b, v0);
        if (v0p >= pos) grow_pt(&right->b, v0);
        if ((v0p < pos && v1p > pos) || (v0p > pos && v1p < pos)) {
            float t = (pos - v0p) / (v1p - v0p);
            t = t < 0.0f ? 0.0f : t > 1.0f ? 1.0f : t;
            float q[3];
            for (int d = 0; d < 3; d++) q[d] = v0[d] * (1.0f - t) + v1[d] * t; /* lerp(a, b, t) */
            grow_pt(&left->b, q);
            grow_pt(&right->b, q);
        }
    }
    left->b.hi[dim] = pos;
    right->b.lo[dim] = pos;
    intersect_box(&left->b, &ref->b);
    intersect_box(&right->b, &ref->b);
}

typedef struct {
    Box b;
    int enter, exit;
} Bin;

static SpatialSplit find_spatial_split(Builder *B, int num, const Box *bounds, float node_sah) {
    float origin[3], bin_size[3], inv[3];
    for (int d = 0; d < 3; d++) {
        origin[d] = bounds->lo[d];
        bin_size[d] = (bounds->hi[d] - origin[d]) * (1.0f / (float)kBins);
        inv[d] = 1.0f / bin_size[d];
    }
    Bin bins[3][kBins];
    for (int d = 0; d < 3; d++)
        for (int i = 0; i < kBins; i++) {
            bins[d][i].b = box_empty();
            bins[d][i].enter = bins[d][i].exit = 0;
        }
    for (int r = B->nrefs - num; r < B->nrefs; r++) {
        const Ref ref = B->refs[r];
        int first[3], last[3];
        for (int d = 0; d < 3; d++) first[d] = clamp1i(f2i((ref.b.lo[d] - origin[d]) * inv[d]), 0, kBins - 1);
        for (int d = 0; d < 3; d++) last[d] = clamp1i(f2i((ref.b.hi[d] - origin[d]) * inv[d]), first[d], kBins - 1);
        for (int dim = 0; dim < 3; dim++) {
            Ref curr = ref;
            for (int i = first[dim]; i < last[dim]; i++) {
                Ref lr, rr;
                split_reference(B, &lr, &rr, &curr, dim, origin[dim] + bin_size[dim] * (float)(i + 1));
                grow_box(&bins[dim][i].b, &lr.b);
                curr = rr;
            }
            grow_box(&bins[dim][last[dim]].b, &curr.b);
            bins[dim][first[dim]].enter++;
            bins[dim][last[dim]].exit++;
        }
    }
    SpatialSplit s = {FLT_MAX, 0, 0.0f};
    Box rb_all[kBins - 1];
    for (int dim = 0; dim < 3; dim++) {
        Box rb = box_empty();
        for (int i = kBins - 1; i > 0; i--) {
            grow_box(&rb, &bins[dim][i].b);
            rb_all[i - 1] = rb;
        }
        Box lb = box_empty();
        int left_num = 0, right_num = num;
        for (int i = 1; i < kBins; i++) {
            grow_box(&lb, &bins[dim][i - 1].b);
            left_num += bins[dim][i - 1].enter;
            right_num -= bins[dim][i - 1].exit;
            const float sah = node_sah + area(&lb) * (float)left_num + area(&rb_all[i - 1]) * (float)right_num;
            if (sah < s.sah) {
                s.sah = sah;
                s.dim = dim;
                s.pos = origin[dim] + bin_size[dim] * (float)i;
            }
        }
    }
    return s;
}

static void swap_ref(Ref *a, Ref *b) {
    Ref t = *a;
    *a = *b;
    *b = t;
}

/* performSpatialSplit: left = [left_start, left_end), right = [right_start, top) of the stack */
static void perform_spatial_split(Builder *B, int num, const SpatialSplit *sp, int *left_n, Box *left_b,
                                  int *right_n, Box *right_b) {
    const int dim = sp->dim;
    const float pos = sp->pos;
    const int left_start = B->nrefs - num;
    int left_end = left_start, right_start = B->nrefs;
    *left_b = *right_b = box_empty();
    for (int i = left_end; i < right_start; i++) {
        if (B->refs[i].b.hi[dim] <= pos) {
            grow_box(left_b, &B->refs[i].b);
            swap_ref(&B->refs[i], &B->refs[left_end++]);
        } else if (B->refs[i].b.lo[dim] >= pos) {
            grow_box(right_b, &B->refs[i].b);
            swap_ref(&B->refs[i], &B->refs[--right_start]);
            i--;
        }
    }
    while (left_end < right_start && !B->error) {
        Ref lr, rr;
        split_reference(B, &lr, &rr, &B->refs[left_end], dim, pos);
        Box lub = *left_b, rub = *right_b, ldb = *left_b, rdb = *right_b;
        grow_box(&lub, &B->refs[left_end].b);
        grow_box(&rub, &B->refs[left_end].b);
        grow_box(&ldb, &lr.b);
        grow_box(&rdb, &rr.b);
        const float lac = (float)(left_end - left_start), rac = (float)(B->nrefs - right_start);
        const float lbc = (float)(left_end - left_start + 1), rbc = (float)(B->nrefs - right_start + 1);
        const float unsplit_left = area(&lub) * lbc + area(right_b) * rac;
        const float unsplit_right = area(left_b) * lac + area(&rub) * rbc;
        const float duplicate = area(&ldb) * lbc + area(&rdb) * rbc;
        const float m = min1f(min1f(unsplit_left, unsplit_right), duplicate);
        if (m == unsplit_left) {
            *left_b = lub;
            left_end++;
        } else if (m == unsplit_right) {
            *right_b = rub;
            swap_ref(&B->refs[left_end], &B->refs[--right_start]);
        } else {
            *left_b = ldb;
            *right_b = rdb;
            B->refs[left_end++] = lr;
            push_ref(B, rr);
        }
    }
    *left_n = left_end - left_start;
    *right_n = B->nrefs - right_start;
}

static int build_node(Builder *B, int num, Box bounds, int level) {
    if (B->error) return 0;
    if (num <= B->leaf_min || level >= kMaxDepth) return create_leaf(B, num, &bounds);
    const float a = area(&bounds);
    const float leaf_sah = a * (float)num;
    const float node_sah = a * 2.0f;
    ObjectSplit object = find_object_split(B, num, node_sah);
    SpatialSplit spatial = {FLT_MAX, 0, 0.0f};
    if (level < kMaxSpatialDepth) {
        Box overlap = object.left;
        intersect_box(&overlap, &object.right);
        if (area(&overlap) >= B->min_overlap) spatial = find_spatial_split(B, num, &bounds, node_sah);
    }
    const float min_sah = min1f(min1f(leaf_sah, object.sah), spatial.sah);
    if (min_sah == leaf_sah && num <= B->leaf_max) return create_leaf(B, num, &bounds);
    int left_n = 0, right_n = 0;
    Box left_b = box_empty(), right_b = box_empty();
    if (min_sah == spatial.sah) perform_spatial_split(B, num, &spatial, &left_n, &left_b, &right_n, &right_b);
    if (!left_n || !right_n) {
        sort_top(B, num, object.dim);  /* performObjectSplit */
        left_n = object.num_left;
        left_b = object.left;
        right_n = num - object.num_left;
        right_b = object.right;
    }
    const int right = build_node(B, right_n, right_b, level + 1);
    const int left = build_node(B, left_n, left_b, level + 1);
    const int id = new_node(B);
    if (B->error) return 0;
    B->nodes[id].b = bounds;
    B->nodes[id].child[0] = left;
    B->nodes[id].child[1] = right;
    return id;
}

/* ---- compact emission (BVHCompact::createCompact) --------------------------------------------- */
typedef struct {
    uint32_t *p;
    size_t n, cap; /* in 32-bit words */
} Words;

static int words_add(Words *w, const uint32_t *src, size_t k) {
    if (w->n + k > w->cap) {
        size_t c = w->cap ? w->cap : 4096;
        while (w->n + k > c) c *= 2;
        uint32_t *p = (uint32_t *)realloc(w->p, c * 4);
        if (!p) return 0;
        w->p = p;
        w->cap = c;
    }
    if (src) memcpy(w->p + w->n, src, k * 4);
    else memset(w->p + w->n, 0, k * 4);
    w->n += k;
    return 1;
}

static uint32_t fbits(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}

typedef struct {
    int node;
    size_t idx; /* float4 index of the node's record */
} Entry;

static int emit_compact(const Builder *B, int root, Words *nodes, Words *verts, Words *norms, Words *tri_idx,
                        Words *mat_idx, uint32_t *tri_count, uint32_t *leaf_count) {
    if (B->nodes[root].leaf) return 0; /* the reference asserts two children at the root */
    Entry *stack = (Entry *)malloc(sizeof(Entry) * (size_t)(B->nnodes + 1));
    if (!stack) return 0;
    int sp = 0;
    stack[sp].node = root;
    stack[sp++].idx = 0;
    if (!words_add(nodes, NULL, 16)) return free(stack), 0;
    *tri_count = *leaf_count = 0;
    while (sp) {
        const Entry e = stack[--sp];
        const Node *nd = &B->nodes[e.node];
        int32_t child_index[2];
        for (int i = 0; i < 2; i++) {
            const Node *c = &B->nodes[nd->child[i]];
            if (!c->leaf) {
                child_index[i] = (int32_t)(nodes->n / 4); /* float4 index */
                stack[sp].node = nd->child[i];
                stack[sp++].idx = nodes->n / 4;
                if (!words_add(nodes, NULL, 16)) return free(stack), 0;
                continue;
            }
            child_index[i] = ~(int32_t)(verts->n / 4);
            for (int j = c->lo; j < c->hi; j++) {
                const int t = B->tris[j];
                uint32_t vw[12], nw[12];
                for (int k = 0; k < 3; k++) {
                    const float *p = B->v + 3 * B->vidx[3 * t + k];
                    const float *q = B->n + 3 * B->nidx[3 * t + k];
                    for (int d = 0; d < 3; d++) {
                        vw[4 * k + d] = fbits(p[d]);
                        nw[4 * k + d] = fbits(q[d]);
                    }
                    vw[4 * k + 3] = nw[4 * k + 3] = 0;
                }
                if (vw[0] == 0x80000000u) vw[0] = 0; /* `if (x == 0.0f) x = 0.0f`: -0.0 becomes +0.0 */
                (*tri_count)++;
                const uint32_t ti[3] = {(uint32_t)t, 0, 0}, mi[3] = {B->mat ? B->mat[t] : 0, 0, 0};
                if (!words_add(verts, vw, 12) || !words_add(norms, nw, 12) || !words_add(tri_idx, ti, 3) ||
                    !words_add(mat_idx, mi, 3))
                    return free(stack), 0;
            }
            const uint32_t term[4] = {0x80000000u, 0, 0, 0}, zero = 0;
            if (!words_add(verts, term, 4) || !words_add(norms, term, 4) || !words_add(tri_idx, &zero, 1) ||
                !words_add(mat_idx, &zero, 1))
                return free(stack), 0;
            (*leaf_count)++;
        }
        const Box *b0 = &B->nodes[nd->child[0]].b, *b1 = &B->nodes[nd->child[1]].b;
        uint32_t *dst = nodes->p + 4 * e.idx;
        const uint32_t rec[16] = {fbits(b0->lo[0]), fbits(b0->hi[0]), fbits(b0->lo[1]), fbits(b0->hi[1]),
                                  fbits(b1->lo[0]), fbits(b1->hi[0]), fbits(b1->lo[1]), fbits(b1->hi[1]),
                                  fbits(b0->lo[2]), fbits(b0->hi[2]), fbits(b1->lo[2]), fbits(b1->hi[2]),
                                  (uint32_t)child_index[0], (uint32_t)child_index[1], 0, 0};
        memcpy(dst, rec, sizeof(rec));
    }
    free(stack);
    return 1;
}

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static int write_all(FILE *f, const void *p, size_t bytes) { return bytes == 0 || fwrite(p, 1, bytes, f) == bytes; }

/* BVH(scene, SAHHelper{leaf_min, leaf_max}, split_alpha) + BVHCompact::createCompact + save:
 * vertices / normals are xyz triples, vidx / nidx three indices per triangle, mat one material per
 * triangle (NULL = 0). Writes bvh.cache to cache_path; *seconds gets the build + emission time
 * (file writing excluded). Returns 0, or -1 on bad input, -2 when out of memory, -3 when the root
 * is a leaf (the reference cannot emit that), -4 on a write error. */
int oracle_sbvh_build(const float *v, int nv, const float *n, int nn, const int32_t *vidx, const int32_t *nidx,
                      const uint32_t *mat, int ntri, float split_alpha, int leaf_min, int leaf_max,
                      const char *cache_path, double *seconds) {
    if (!v || !n || !vidx || !nidx || ntri <= 0 || nv <= 0 || nn <= 0) return -1;
    for (long long i = 0; i < 3ll * ntri; i++)
        if (vidx[i] < 0 || vidx[i] >= nv || nidx[i] < 0 || nidx[i] >= nn) return -1;
    const double t0 = now_s();
    Builder B;
    memset(&B, 0, sizeof(B));
    B.v = v;
    B.n = n;
    B.vidx = vidx;
    B.nidx = nidx;
    B.mat = mat;
    B.leaf_min = leaf_min;
    B.leaf_max = leaf_max;
    Box root = box_empty();
    for (int i = 0; i < ntri && !B.error; i++) {
        Ref r;
        r.tri = i;
        r.b = box_empty();
        for (int k = 0; k < 3; k++) grow_pt(&r.b, vert(&B, i, k));
        grow_box(&root, &r.b);
        push_ref(&B, r);
    }
    B.min_overlap = area(&root) * split_alpha;
    const int root_id = B.error ? 0 : build_node(&B, ntri, root, 0);
    Words nodes = {0}, verts = {0}, norms = {0}, tri_idx = {0}, mat_idx = {0};
    uint32_t tri_count = 0, leaf_count = 0;
    int rc = 0;
    if (B.error) rc = -2;
    else if (B.nodes[root_id].leaf) rc = -3;
    else if (!emit_compact(&B, root_id, &nodes, &verts, &norms, &tri_idx, &mat_idx, &tri_count, &leaf_count)) rc = -2;
    if (seconds) *seconds = now_s() - t0;
    if (rc == 0) {
        FILE *f = fopen(cache_path, "wb");
        const uint32_t hdr[7] = {(uint32_t)(nodes.n / 4), tri_count, leaf_count, (uint32_t)(verts.n / 4),
                                 (uint32_t)(norms.n / 4), (uint32_t)tri_idx.n, (uint32_t)mat_idx.n};
        if (!f) rc = -4;
        else {
            if (!write_all(f, hdr, sizeof(hdr)) || !write_all(f, nodes.p, nodes.n * 4) ||
                !write_all(f, verts.p, verts.n * 4) || !write_all(f, norms.p, norms.n * 4) ||
                !write_all(f, tri_idx.p, tri_idx.n * 4) || !write_all(f, mat_idx.p, mat_idx.n * 4))
                rc = -4;
            if (fclose(f) != 0) rc = -4;
        }
    }
    free(B.refs);
    free(B.tris);
    free(B.nodes);
    free(nodes.p);
    free(verts.p);
    free(norms.p);
    free(tri_idx.p);
    free(mat_idx.p);
    return rc;
}
