// Host SBVH builder (Stich et al. 2009 spatial-split BVH) emitting the reference's compact
// two-wide layout and its bvh.cache file.
//
// The build reproduces every decision of the reference builder (src/bvh/BVH.cpp) so that the
// emitted arrays are byte-identical to what BVHCompact::createCompact writes
// (src/bvh/BVHCompact.cpp:88-250):
//   - SAH costs of SAHHelper's defaults: triangle cost n * 1, node cost 2 * 1
//     (src/bvh/SAHHelper.cpp:19-25, include/bvh/SAHHelper.h:73-81);
//   - leaf if numRef <= leaf_min or depth >= 64; spatial splits only above depth 48 and when
//     the object-split children overlap by >= alpha * rootArea (BVH.cpp:70-111, BVH.h:96-100);
//   - object splits: full sweep of the references sorted on (min+max) along each axis, ties
//     broken by triangle index (BVH.cpp:122-154, :343-351);
//   - spatial splits: 32 bins per axis, reference clipping against the split plane, and the
//     unsplit-left / unsplit-right / duplicate choice (BVH.cpp:166-341);
//   - AABB growth semantics, including that growing a box by an EMPTY box makes it unbounded
//     (src/bvh/AABB.cpp:35-39; an empty bin therefore disqualifies a spatial split);
//   - leaf triangle order: the reference pops its reference stack, so a leaf lists its
//     references in reverse partition order (BVH.cpp:113-120);
//   - compact emission: DFS from an explicit stack, inner children addressed by float4 index,
//     leaves by ~vertexIndex, -0.0 in vertex0.x rewritten to +0.0, a (0x80000000,0,0,0)
//     terminator after each leaf (BVHCompact.cpp:88-192).
// Within one node every triangle index appears at most once, so the centroid comparator is a
// strict total order and a node's order along each axis is unique. The root is sorted once per
// axis; every other node receives its three orders from its parent by stable partition (plus a
// merge of the clipped halves of a spatial split), which yields that unique order without a sort.
// Subtrees are built as OpenMP tasks; each task owns the reference lists of its node, and a leaf
// lists its triangles in the order the reference's shared stack would hold them, so the output
// does not depend on threads.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <thread>
#include <unordered_map>
#include <omp.h>

#include "tt_internal.h"

namespace tt {
namespace {

constexpr int kMaxDepth = 64;
constexpr int kMaxSpatialDepth = 48;
constexpr int kBins = 32;
constexpr int kTaskThreshold = 2048;
constexpr int kAxisThreadsMin = 1 << 16;

struct AABB {
    V3 lo{FLT_MAX, FLT_MAX, FLT_MAX};
    V3 hi{-FLT_MAX, -FLT_MAX, -FLT_MAX};
    void grow(const V3 &p) {
        lo = vmin3(lo, p);
        hi = vmax3(hi, p);
    }
    // Grows by the two corner points, as the reference does: an empty box (lo = +MAX,
    // hi = -MAX) turns this box into [-MAX, +MAX].
    void grow(const AABB &b) {
        grow(b.lo);
        grow(b.hi);
    }
    void intersect(const AABB &b) {
        lo = vmax3(lo, b.lo);
        hi = vmin3(hi, b.hi);
    }
    bool valid() const { return lo.x <= hi.x && lo.y <= hi.y && lo.z <= hi.z; }
    float area() const {
        if (!valid()) return 0.0f;
        V3 d = hi - lo;
        return (d.x * d.y + d.y * d.z + d.z * d.x) * 2.0f;
    }
};

struct Ref {
    int32_t tri;
    AABB b;
};

// What the compact emission of an inner node's subtree writes, its own four node entries not
// counted: the node entries of the inner nodes below it, and the vertex (= normal = index)
// entries of the leaves below it, three per triangle plus a terminator per leaf.
struct EmitSize {
    int64_t nodes = 0, verts = 0, tris = 0, leaves = 0;
};

struct Node {
    AABB b;
    std::unique_ptr<Node> child[2];  // [0] = left, [1] = right
    std::vector<int32_t> tris;       // leaf triangles, in emission order
    bool leaf = false;
    EmitSize below;                  // inner nodes only, filled before emission
};

struct ObjectSplit {
    float sah = FLT_MAX;
    int dim = 0;
    int num_left = 0;
    AABB left, right;
};

struct SpatialSplit {
    float sah = FLT_MAX;
    int dim = 0;
    float pos = 0.0f;
};

struct Bin {
    AABB b;
    int enter = 0, exit = 0;
};

inline float min1f(float a, float b) { return (a > b) ? b : a; }
inline int clamp1i(int v, int lo, int hi) { return v < lo ? lo : v > hi ? hi : v; }

// float -> int32 with the x86 cvttss2si result for NaN and out-of-range values (0x80000000),
// so that flat nodes (0 * inf bin coordinates) bin the same way on every host.
inline int f2i_trunc(float f) {
    if (!(f > -2147483648.0f && f < 2147483648.0f)) return INT32_MIN;
    return (int)f;
}

// The node's references sorted along each axis (centroid, then triangle index: a strict total
// order). The reference re-sorts every node along all three axes (BVH.cpp:132-164); here each
// node receives its three orders from its parent, which partitions them stably (a stable filter of
// a sorted list is sorted) and merges in the few references a spatial split clipped, so a node
// costs O(n) instead of O(n log n) and every set, order and split is the reference's.
struct NodeRefs {
    std::vector<Ref> s[3];
    size_t size() const { return s[0].size(); }
};

// Centroid order along dim, ties by triangle index.
struct ByCentroid {
    int dim;
    bool operator()(const Ref &a, const Ref &b) const {
        const float ca = a.b.lo[dim] + a.b.hi[dim];
        const float cb = b.b.lo[dim] + b.b.hi[dim];
        if (ca < cb) return true;
        if (ca > cb) return false;
        return a.tri < b.tri;
    }
};

// `refs` (in triangle order) in ByCentroid{dim} order, by a stable LSD radix sort of the
// centroid sums' bits mapped to unsigned order (-0 taken as +0, as the float comparison has it):
// stability over the triangle-ordered input breaks ties by triangle index. Centroids are never
// NaN (the build refuses non-finite vertices).
std::vector<Ref> sorted_by_centroid(const std::vector<Ref> &refs, int dim) {
    const size_t n = refs.size();
    std::vector<uint32_t> key(n), key2(n);
    std::vector<int32_t> idx(n), idx2(n);
    for (size_t i = 0; i < n; i++) {
        float c = refs[i].b.lo[dim] + refs[i].b.hi[dim];
        if (c == 0.0f) c = 0.0f;
        uint32_t u;
        memcpy(&u, &c, 4);
        key[i] = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
        idx[i] = (int32_t)i;
    }
    constexpr int kBits = 11, kDigits = 1 << kBits;
    std::vector<size_t> count(kDigits);
    for (int shift = 0; shift < 32; shift += kBits) {
        std::fill(count.begin(), count.end(), 0);
        for (size_t i = 0; i < n; i++) count[(key[i] >> shift) & (kDigits - 1)]++;
        size_t sum = 0;
        for (size_t &c : count) {
            const size_t t = c;
            c = sum;
            sum += t;
        }
        for (size_t i = 0; i < n; i++) {
            const size_t at = count[(key[i] >> shift) & (kDigits - 1)]++;
            key2[at] = key[i];
            idx2[at] = idx[i];
        }
        key.swap(key2);
        idx.swap(idx2);
    }
    std::vector<Ref> out(n);
    for (size_t i = 0; i < n; i++) out[i] = refs[idx[i]];
    return out;
}

// What the spatial partition did with one reference that straddles the plane.
enum class Straddle : uint8_t { kLeft, kRight, kBoth };

class Builder {
public:
    Builder(const Scene &s, const BuildParams &p) : sc_(s), p_(p) {}

    std::unique_ptr<Node> run(int64_t &duplicates) {
        const int n = sc_.num_tris();
        std::vector<Ref> refs(n);
        AABB root;
        for (int i = 0; i < n; i++) {
            refs[i].tri = i;
            for (int k = 0; k < 3; k++) refs[i].b.grow(sc_.vertices[sc_.vidx[3 * i + k]]);
            root.grow(refs[i].b);
        }
        min_overlap_ = root.area() * p_.split_alpha;
        int threads = p_.threads > 0 ? p_.threads : omp_get_max_threads();
        par_min_ = threads > 1 ? std::max(kAxisThreadsMin, n / 16) : INT32_MAX;
        std::unique_ptr<Node> out;
        dup_ = 0;
#pragma omp parallel num_threads(threads)
#pragma omp single
        {
            NodeRefs nr;
            for (int d = 0; d < 3; d++) {
#pragma omp task firstprivate(d) shared(nr, refs)
                nr.s[d] = sorted_by_centroid(refs, d);
            }
#pragma omp taskwait
            out = build(std::move(nr), root, 0, &refs);
        }
        duplicates = dup_;
        return out;
    }

private:
    const Scene &sc_;
    BuildParams p_;
    float min_overlap_ = 0.0f;
    int64_t dup_ = 0;
    int par_min_ = INT32_MAX;  // nodes of at least this many references split their axes over threads

    // Runs f(0), f(1), f(2); with `par`, axes 1 and 2 on threads of their own. These are plain
    // threads, not OpenMP tasks: a thread that waits for tasks may run any queued subtree task
    // first, which held a node near the root up for seconds.
    template <class F>
    static void for_axes(bool par, F &&f) {
        if (!par) {
            for (int d = 0; d < 3; d++) f(d);
            return;
        }
        std::thread t1([&] { f(1); });
        std::thread t2([&] { f(2); });
        f(0);
        t1.join();
        t2.join();
    }

    const V3 &vert(int tri, int k) const { return sc_.vertices[sc_.vidx[3 * tri + k]]; }

    // refs in the order the reference holds them at that point (it emits them reversed)
    std::unique_ptr<Node> leaf(const std::vector<Ref> &refs, const AABB &b) {
        auto nd = std::make_unique<Node>();
        nd->leaf = true;
        nd->b = b;
        nd->tris.resize(refs.size());
        for (size_t i = 0; i < refs.size(); i++) nd->tris[i] = refs[refs.size() - 1 - i].tri;
        return nd;
    }

    // The reference's sweep over one axis's sorted order (BVH.cpp:132-155): the first best split.
    static ObjectSplit object_sweep(const std::vector<Ref> &refs, int dim, float node_sah) {
        ObjectSplit split;
        const int n = (int)refs.size();
        std::vector<AABB> right_bounds(n > 1 ? n - 1 : 1);
        AABB rb;
        for (int i = n - 1; i > 0; i--) {
            rb.grow(refs[i].b);
            right_bounds[i - 1] = rb;
        }
        AABB lb;
        for (int i = 1; i < n; i++) {
            lb.grow(refs[i - 1].b);
            float sah = node_sah + lb.area() * (float)i + right_bounds[i - 1].area() * (float)(n - i);
            if (sah < split.sah) {
                split.sah = sah;
                split.dim = dim;
                split.num_left = i;
                split.left = lb;
                split.right = right_bounds[i - 1];
            }
        }
        return split;
    }

    // The reference sweeps axes 0, 1, 2 in turn, replacing its best only on a strictly lower cost:
    // the first best of each axis, taken in axis order on the same strict comparison, is that split.
    ObjectSplit find_object_split(const NodeRefs &nr, float node_sah, bool par) {
        ObjectSplit per_axis[3];
        for_axes(par, [&](int d) { per_axis[d] = object_sweep(nr.s[d], d, node_sah); });
        ObjectSplit split;
        for (int d = 0; d < 3; d++)
            if (per_axis[d].sah < split.sah) split = per_axis[d];
        return split;
    }

    void split_reference(Ref &left, Ref &right, const Ref &ref, int dim, float pos) const {
        left.tri = right.tri = ref.tri;
        left.b = right.b = AABB();
        const V3 *v1 = &vert(ref.tri, 2);
        for (int k = 0; k < 3; k++) {
            const V3 *v0 = v1;
            v1 = &vert(ref.tri, k);
            float v0p = (*v0)[dim];
            float v1p = (*v1)[dim];
            if (v0p <= pos) left.b.grow(*v0);
            if (v0p >= pos) right.b.grow(*v0);
            if ((v0p < pos && v1p > pos) || (v0p > pos && v1p < pos)) {
                float t = (pos - v0p) / (v1p - v0p);
                t = t < 0.0f ? 0.0f : (t > 1.0f ? 1.0f : t);
                V3 a = (*v0) * (1.0f - t);
                V3 b = (*v1) * t;
                V3 q = a + b;
                left.b.grow(q);
                right.b.grow(q);
            }
        }
        left.b.hi[dim] = pos;
        right.b.lo[dim] = pos;
        left.b.intersect(ref.b);
        right.b.intersect(ref.b);
    }

    // One axis's bins (BVH.cpp:184-215): each reference is clipped at the planes it crosses, in
    // order, and enters its first bin and exits its last. The axes do not share any state.
    void bin_axis(const std::vector<Ref> &refs, int dim, float origin, float bin_size, float inv_bin,
                  Bin *bins) const {
        for (const Ref &ref : refs) {
            const int first = clamp1i(f2i_trunc((ref.b.lo[dim] - origin) * inv_bin), 0, kBins - 1);
            const int last = clamp1i(f2i_trunc((ref.b.hi[dim] - origin) * inv_bin), first, kBins - 1);
            Ref curr = ref;
            for (int i = first; i < last; i++) {
                Ref lr, rr;
                split_reference(lr, rr, curr, dim, origin + bin_size * (float)(i + 1));
                bins[i].b.grow(lr.b);
                curr = rr;
            }
            bins[last].b.grow(curr.b);
            bins[first].enter++;
            bins[last].exit++;
        }
    }

    SpatialSplit find_spatial_split(const std::vector<Ref> &refs, const AABB &bounds, float node_sah, bool par) {
        const V3 origin = bounds.lo;
        const V3 bin_size = (bounds.hi - origin) * (1.0f / (float)kBins);
        const V3 inv_bin(1.0f / bin_size.x, 1.0f / bin_size.y, 1.0f / bin_size.z);
        Bin bins[3][kBins];
        for_axes(par, [&](int d) { bin_axis(refs, d, origin[d], bin_size[d], inv_bin[d], bins[d]); });
        SpatialSplit split;
        const int n = (int)refs.size();
        AABB right_bounds[kBins - 1];
        for (int dim = 0; dim < 3; dim++) {
            AABB rb;
            for (int i = kBins - 1; i > 0; i--) {
                rb.grow(bins[dim][i].b);
                right_bounds[i - 1] = rb;
            }
            AABB lb;
            int left_num = 0, right_num = n;
            for (int i = 1; i < kBins; i++) {
                lb.grow(bins[dim][i - 1].b);
                left_num += bins[dim][i - 1].enter;
                right_num -= bins[dim][i - 1].exit;
                float sah = node_sah + lb.area() * (float)left_num + right_bounds[i - 1].area() * (float)right_num;
                if (sah < split.sah) {
                    split.sah = sah;
                    split.dim = dim;
                    split.pos = origin[dim] + bin_size[dim] * (float)i;
                }
            }
        }
        return split;
    }

    // The reference's partition (BVH.cpp:266-330) of `refs` (the node's references in the order it
    // holds them: along axis 2) in place, plus appended duplicates: left = [0, left_n), right =
    // [left_n, size). `decisions` receives what became of each straddling reference.
    void perform_spatial_split(std::vector<Ref> &refs, const SpatialSplit &split, int &left_n, AABB &left_b,
                               int &right_n, AABB &right_b,
                               std::vector<std::pair<int32_t, Straddle>> &decisions) {
        const int dim = split.dim;
        const float pos = split.pos;
        int left_start = 0, left_end = 0, right_start = (int)refs.size();
        left_b = right_b = AABB();
        for (int i = left_end; i < right_start; i++) {
            if (refs[i].b.hi[dim] <= pos) {
                left_b.grow(refs[i].b);
                std::swap(refs[i], refs[left_end++]);
            } else if (refs[i].b.lo[dim] >= pos) {
                right_b.grow(refs[i].b);
                std::swap(refs[i], refs[--right_start]);
                i--;
            }
        }
        decisions.clear();
        decisions.reserve(right_start - left_end);
        while (left_end < right_start) {
            Ref lr, rr;
            split_reference(lr, rr, refs[left_end], dim, pos);
            AABB lub = left_b, rub = right_b, ldb = left_b, rdb = right_b;
            lub.grow(refs[left_end].b);
            rub.grow(refs[left_end].b);
            ldb.grow(lr.b);
            rdb.grow(rr.b);
            float lac = (float)(left_end - left_start);
            float rac = (float)((int)refs.size() - right_start);
            float lbc = (float)(left_end - left_start + 1);
            float rbc = (float)((int)refs.size() - right_start + 1);
            float unsplit_left = lub.area() * lbc + right_b.area() * rac;
            float unsplit_right = left_b.area() * lac + rub.area() * rbc;
            float duplicate = ldb.area() * lbc + rdb.area() * rbc;
            float m = min1f(min1f(unsplit_left, unsplit_right), duplicate);
            if (m == unsplit_left) {
                decisions.emplace_back(refs[left_end].tri, Straddle::kLeft);
                left_b = lub;
                left_end++;
            } else if (m == unsplit_right) {
                decisions.emplace_back(refs[left_end].tri, Straddle::kRight);
                right_b = rub;
                std::swap(refs[left_end], refs[--right_start]);
            } else {
                decisions.emplace_back(refs[left_end].tri, Straddle::kBoth);
                left_b = ldb;
                right_b = rdb;
                refs[left_end++] = lr;
                refs.push_back(rr);
            }
        }
        left_n = left_end - left_start;
        right_n = (int)refs.size() - right_start;
    }

    // Children's sorted orders after an object split: the left set is the first num_left
    // references along its axis, so membership along the other axes is a comparison with the
    // first right reference.
    static void split_object_orders(NodeRefs &nr, const ObjectSplit &os, NodeRefs &L, NodeRefs &R, bool par) {
        const int d = os.dim;
        const size_t nl = (size_t)os.num_left;
        const size_t n = nr.size();
        const Ref pivot = nr.s[d][nl];
        const ByCentroid cmp{d};
        for_axes(par, [&](int e) {
            L.s[e].reserve(nl);
            R.s[e].reserve(n - nl);
            if (e == d) {
                L.s[e].assign(nr.s[e].begin(), nr.s[e].begin() + nl);
                R.s[e].assign(nr.s[e].begin() + nl, nr.s[e].end());
            } else {
                for (const Ref &r : nr.s[e]) (cmp(r, pivot) ? L : R).s[e].push_back(r);
            }
            std::vector<Ref>().swap(nr.s[e]);
        });
    }

    // Children's sorted orders after a spatial split: each axis's order filtered by where its
    // unclipped references went, with the clipped halves (sorted on their own) merged in.
    static void split_spatial_orders(NodeRefs &nr, const SpatialSplit &sp, const std::vector<Ref> &parted, int left_n,
                                     const std::vector<std::pair<int32_t, Straddle>> &decisions, NodeRefs &L,
                                     NodeRefs &R, bool par) {
        const int dim = sp.dim;
        const float pos = sp.pos;
        std::unordered_map<int32_t, Straddle> fate(decisions.begin(), decisions.end());
        // the clipped halves: every reference of `parted` whose triangle was split on both sides
        std::vector<Ref> clipped_l, clipped_r;
        for (size_t i = 0; i < parted.size(); i++) {
            auto it = fate.find(parted[i].tri);
            if (it != fate.end() && it->second == Straddle::kBoth) ((int)i < left_n ? clipped_l : clipped_r).push_back(parted[i]);
        }
        for_axes(par, [&](int e) {
            std::vector<Ref> l, r;
            l.reserve(left_n);
            r.reserve(parted.size() - left_n);
            for (const Ref &ref : nr.s[e]) {
                if (ref.b.hi[dim] <= pos) {
                    l.push_back(ref);
                } else if (ref.b.lo[dim] >= pos) {
                    r.push_back(ref);
                } else {
                    const Straddle f = fate.at(ref.tri);
                    if (f == Straddle::kLeft) l.push_back(ref);
                    else if (f == Straddle::kRight) r.push_back(ref);
                }
            }
            std::vector<Ref>().swap(nr.s[e]);
            const ByCentroid cmp{e};
            std::vector<Ref> cl = clipped_l, cr = clipped_r;
            std::sort(cl.begin(), cl.end(), cmp);
            std::sort(cr.begin(), cr.end(), cmp);
            L.s[e].resize(l.size() + cl.size());
            std::merge(l.begin(), l.end(), cl.begin(), cl.end(), L.s[e].begin(), cmp);
            R.s[e].resize(r.size() + cr.size());
            std::merge(r.begin(), r.end(), cr.begin(), cr.end(), R.s[e].begin(), cmp);
        });
    }

    // `arrival` (may be null when the node is not small): the references in the order the
    // reference would hold them on entering this node, which only a leaf made on entry uses.
    std::unique_ptr<Node> build(NodeRefs nr, AABB bounds, int level, const std::vector<Ref> *arrival) {
        const int n = (int)nr.size();
        if (n <= p_.leaf_min || level >= kMaxDepth) return leaf(*arrival, bounds);

        const float area = bounds.area();
        const float leaf_sah = area * (float)n;
        const float node_sah = area * 2.0f;
        // the three axes of a node near the root on three threads: few subtree tasks run yet
        const bool par = n >= par_min_;
        ObjectSplit object = find_object_split(nr, node_sah, par);

        SpatialSplit spatial;
        if (level < kMaxSpatialDepth) {
            AABB overlap = object.left;
            overlap.intersect(object.right);
            if (overlap.area() >= min_overlap_) spatial = find_spatial_split(nr.s[0], bounds, node_sah, par);
        }

        const float min_sah = min1f(min1f(leaf_sah, object.sah), spatial.sah);
        // after its sorts the reference holds the references along axis 2
        if (min_sah == leaf_sah && n <= p_.leaf_max) return leaf(nr.s[2], bounds);

        int left_n = 0, right_n = 0;
        AABB left_b, right_b;
        NodeRefs L, R;
        std::vector<Ref> parted;  // the spatial partition's order (left part, then right part)
        bool spatial_done = false;
        if (min_sah == spatial.sah) {
            parted = nr.s[2];
            std::vector<std::pair<int32_t, Straddle>> decisions;
            perform_spatial_split(parted, spatial, left_n, left_b, right_n, right_b, decisions);
            if (left_n && right_n) {
                split_spatial_orders(nr, spatial, parted, left_n, decisions, L, R, par);
                spatial_done = true;
            }
        }
        if (!spatial_done) {
            // sorted along the chosen axis again, exactly as the reference does (BVH.cpp:156-164)
            left_n = object.num_left;
            left_b = object.left;
            right_n = n - object.num_left;
            right_b = object.right;
            split_object_orders(nr, object, L, R, par);
        }

        const int total = left_n + right_n;
        if (total > n) {
#pragma omp atomic
            dup_ += total - n;
        }
        // the order each child arrives in (needed only by a child that becomes a leaf on entry)
        const bool small_l = left_n <= p_.leaf_min || level + 1 >= kMaxDepth;
        const bool small_r = right_n <= p_.leaf_min || level + 1 >= kMaxDepth;
        std::vector<Ref> arrive_l, arrive_r;
        if (small_l) {
            if (spatial_done) arrive_l.assign(parted.begin(), parted.begin() + left_n);
            else arrive_l = L.s[object.dim];
        }
        if (small_r) {
            if (spatial_done) arrive_r.assign(parted.begin() + left_n, parted.end());
            else arrive_r = R.s[object.dim];
        }
        std::vector<Ref>().swap(parted);

        auto nd = std::make_unique<Node>();
        nd->b = bounds;
        if (total >= kTaskThreshold) {
            std::unique_ptr<Node> r;
#pragma omp task shared(r, R, arrive_r) firstprivate(right_b, level, small_r)
            r = build(std::move(R), right_b, level + 1, small_r ? &arrive_r : nullptr);
            nd->child[0] = build(std::move(L), left_b, level + 1, small_l ? &arrive_l : nullptr);
#pragma omp taskwait
            nd->child[1] = std::move(r);
        } else {
            nd->child[1] = build(std::move(R), right_b, level + 1, small_r ? &arrive_r : nullptr);
            nd->child[0] = build(std::move(L), left_b, level + 1, small_l ? &arrive_l : nullptr);
        }
        return nd;
    }
};

inline int32_t fbits(float f) { return (int32_t)f2u(f); }

constexpr int64_t kEmitTaskVerts = 1 << 15;  // subtrees this large are emitted as tasks

EmitSize size_subtree(Node &x, int depth) {
    for (int i = 0; i < 2; i++) {
        Node &c = *x.child[i];
        if (c.leaf) continue;
        if (depth < 10) {
#pragma omp task firstprivate(i) shared(x)
            size_subtree(*x.child[i], depth + 1);
        } else {
            size_subtree(c, depth + 1);
        }
    }
#pragma omp taskwait
    EmitSize e;
    for (int i = 0; i < 2; i++) {
        const Node &c = *x.child[i];
        if (c.leaf) {
            e.verts += 3 * (int64_t)c.tris.size() + 1;
            e.tris += (int64_t)c.tris.size();
            e.leaves += 1;
        } else {
            e.nodes += 4 + c.below.nodes;
            e.verts += c.below.verts;
            e.tris += c.below.tris;
            e.leaves += c.below.leaves;
        }
    }
    x.below = e;
    return e;
}

// A leaf's triangles at vertex entry `at`, then the terminator (BVHCompact.cpp:127-171).
void emit_leaf(const Scene &sc, const Node &leaf, CompactBVH &out, int64_t at) {
    for (int32_t id : leaf.tris) {
        V3 v[3], nrm[3];
        for (int k = 0; k < 3; k++) {
            v[k] = sc.vertices[sc.vidx[3 * id + k]];
            nrm[k] = sc.normals[sc.nidx[3 * id + k]];
        }
        if (v[0].x == 0.0f) v[0].x = 0.0f;  // -0.0 would read as the leaf terminator
        for (int k = 0; k < 3; k++) {
            out.vertices[at + k] = I4{fbits(v[k].x), fbits(v[k].y), fbits(v[k].z), 0};
            out.normals[at + k] = I4{fbits(nrm[k].x), fbits(nrm[k].y), fbits(nrm[k].z), 0};
            out.tri_idx[at + k] = k == 0 ? id : 0;
            out.mat_idx[at + k] = k == 0 ? sc.mat[id] : 0u;
        }
        at += 3;
    }
    out.vertices[at] = I4{(int32_t)0x80000000, 0, 0, 0};
    out.normals[at] = I4{(int32_t)0x80000000, 0, 0, 0};
    out.tri_idx[at] = 0;
    out.mat_idx[at] = 0;
}

// The reference emits from an explicit stack (BVHCompact.cpp:101-125): it pops a node, gives each
// inner child the next four node entries and writes each leaf child's triangles, then pushes the
// inner children, so the right child's whole subtree comes before the left child's. With every
// subtree's size known, that is a recursion whose two halves write disjoint, precomputed ranges,
// so large subtrees are written as parallel tasks. `slot`: this node's first entry; `node_at`,
// `vert_at`: where the entries this call writes begin.
void emit_subtree(const Scene &sc, const Node &x, int64_t slot, int64_t node_at, int64_t vert_at,
                  CompactBVH &out) {
    int32_t cidx[2];
    int64_t child_slot[2] = {0, 0};
    for (int i = 0; i < 2; i++) {
        const Node &c = *x.child[i];
        if (!c.leaf) {
            child_slot[i] = node_at;
            cidx[i] = (int32_t)node_at;  // float4 index = bytes / 16
            node_at += 4;
        } else {
            cidx[i] = ~(int32_t)vert_at;
            emit_leaf(sc, c, out, vert_at);
            vert_at += 3 * (int64_t)c.tris.size() + 1;
        }
    }
    const AABB *box[2] = {&x.child[0]->b, &x.child[1]->b};
    I4 *dst = &out.nodes[slot];
    dst[0] = I4{fbits(box[0]->lo.x), fbits(box[0]->hi.x), fbits(box[0]->lo.y), fbits(box[0]->hi.y)};
    dst[1] = I4{fbits(box[1]->lo.x), fbits(box[1]->hi.x), fbits(box[1]->lo.y), fbits(box[1]->hi.y)};
    dst[2] = I4{fbits(box[0]->lo.z), fbits(box[0]->hi.z), fbits(box[1]->lo.z), fbits(box[1]->hi.z)};
    dst[3] = I4{cidx[0], cidx[1], 0, 0};
    for (int i = 1; i >= 0; i--) {
        const Node &c = *x.child[i];
        if (c.leaf) continue;
        if (c.below.verts >= kEmitTaskVerts) {
#pragma omp task firstprivate(i, node_at, vert_at, child_slot) shared(sc, x, out)
            emit_subtree(sc, *x.child[i], child_slot[i], node_at, vert_at, out);
        } else {
            emit_subtree(sc, c, child_slot[i], node_at, vert_at, out);
        }
        node_at += c.below.nodes;
        vert_at += c.below.verts;
    }
#pragma omp taskwait
}

void emit_compact(const Scene &sc, Node &root, int threads, CompactBVH &out) {
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel num_threads(threads)
#pragma omp single
    size_subtree(root, 0);
    const EmitSize &e = root.below;
    out.nodes.assign(4 + e.nodes, I4{0, 0, 0, 0});
    out.vertices.resize(e.verts);
    out.normals.resize(e.verts);
    out.tri_idx.resize(e.verts);
    out.mat_idx.resize(e.verts);
    out.hdr.tri_count = (uint32_t)e.tris;
    out.hdr.leaf_count = (uint32_t)e.leaves;
#pragma omp parallel num_threads(threads)
#pragma omp single
    emit_subtree(sc, root, 0, 4, 0, out);
}

}  // namespace

tt_status build_compact(const Scene &sc, const BuildParams &p, CompactBVH &out) {
    const int n = sc.num_tris();
    if (sc.vidx.size() != (size_t)3 * n || sc.nidx.size() != (size_t)3 * n)
        return fail(TT_ERR_INVALID, "scene index arrays do not match the triangle count");
    for (int i = 0; i < 3 * n; i++) {
        if (sc.vidx[i] < 0 || (size_t)sc.vidx[i] >= sc.vertices.size())
            return fail(TT_ERR_INVALID, "vertex index out of range");
        // a NaN or infinite coordinate makes a NaN centroid, which no sort order can place
        const V3 &v = sc.vertices[sc.vidx[i]];
        if (!std::isfinite(v.x) || !std::isfinite(v.y) || !std::isfinite(v.z))
            return fail(TT_ERR_INVALID, "a triangle has a NaN or infinite vertex coordinate");
        if (sc.nidx[i] < 0 || (size_t)sc.nidx[i] >= sc.normals.size())
            return fail(TT_ERR_INVALID, "normal index out of range");
    }
    if (p.leaf_min < 0 || p.leaf_max < 1) return fail(TT_ERR_INVALID, "bad leaf size preferences");
    out = CompactBVH();
    std::unique_ptr<Node> root;
    if (n > 0) {
        Builder b(sc, p);
        int64_t dups = 0;
        root = b.run(dups);
    }
    // The reference requires an inner root (BVHCompact.cpp:104 asserts two children and
    // dereferences them). A scene that ends in a single leaf -- or has no triangles -- gets an
    // inner root whose missing child is an empty leaf with an empty box, which no ray enters.
    if (!root || root->leaf) {
        auto top = std::make_unique<Node>();
        auto empty = std::make_unique<Node>();
        empty->leaf = true;
        if (root) {
            top->b = root->b;
            top->child[0] = std::move(root);
        } else {
            auto empty0 = std::make_unique<Node>();
            empty0->leaf = true;
            top->child[0] = std::move(empty0);
        }
        top->child[1] = std::move(empty);
        root = std::move(top);
    }
    emit_compact(sc, *root, p.threads, out);
    out.hdr.nodes = (uint32_t)out.nodes.size();
    out.hdr.vertices = (uint32_t)out.vertices.size();
    out.hdr.normals = (uint32_t)out.normals.size();
    out.hdr.tri_indices = (uint32_t)out.tri_idx.size();
    out.hdr.mat_indices = (uint32_t)out.mat_idx.size();
    return TT_OK;
}

// ---- bvh.cache ------------------------------------------------------------------------
tt_status save_compact(const CompactBVH &b, const std::string &path) {
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) return fail(TT_ERR_IO, "cannot open " + path + " for writing");
    const tt_bvh_header &h = b.hdr;
    const uint32_t words[7] = {h.nodes, h.tri_count, h.leaf_count, h.vertices, h.normals, h.tri_indices,
                               h.mat_indices};
    bool ok = fwrite(words, 4, 7, f) == 7;
    ok = ok && fwrite(b.nodes.data(), 16, b.nodes.size(), f) == b.nodes.size();
    ok = ok && fwrite(b.vertices.data(), 16, b.vertices.size(), f) == b.vertices.size();
    ok = ok && fwrite(b.normals.data(), 16, b.normals.size(), f) == b.normals.size();
    ok = ok && fwrite(b.tri_idx.data(), 4, b.tri_idx.size(), f) == b.tri_idx.size();
    ok = ok && fwrite(b.mat_idx.data(), 4, b.mat_idx.size(), f) == b.mat_idx.size();
    ok = (fclose(f) == 0) && ok;
    if (!ok) return fail(TT_ERR_IO, "short write to " + path);
    return TT_OK;
}

tt_status load_compact(const std::string &path, CompactBVH &out) {
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) return fail(TT_ERR_IO, "cannot open " + path);
    uint32_t w[7];
    if (fread(w, 4, 7, f) != 7) {
        fclose(f);
        return fail(TT_ERR_FORMAT, "bvh.cache header truncated: " + path);
    }
    fseek(f, 0, SEEK_END);
    long long size = ftell(f);
    fseek(f, 28, SEEK_SET);
    const long long need = 28 + 16LL * w[0] + 16LL * w[3] + 16LL * w[4] + 4LL * w[5] + 4LL * w[6];
    if (size != need) {
        fclose(f);
        return fail(TT_ERR_FORMAT, "bvh.cache size " + std::to_string(size) + " does not match its header (" +
                                       std::to_string(need) + "): " + path);
    }
    if (w[3] != w[4] || w[3] != w[5] || w[3] != w[6] || (w[0] % 4) != 0 || w[0] == 0) {
        fclose(f);
        return fail(TT_ERR_FORMAT, "bvh.cache header is inconsistent: " + path);
    }
    out = CompactBVH();
    out.hdr = tt_bvh_header{w[0], w[1], w[2], w[3], w[4], w[5], w[6]};
    out.nodes.resize(w[0]);
    out.vertices.resize(w[3]);
    out.normals.resize(w[4]);
    out.tri_idx.resize(w[5]);
    out.mat_idx.resize(w[6]);
    bool ok = fread(out.nodes.data(), 16, w[0], f) == w[0];
    ok = ok && fread(out.vertices.data(), 16, w[3], f) == w[3];
    ok = ok && fread(out.normals.data(), 16, w[4], f) == w[4];
    ok = ok && fread(out.tri_idx.data(), 4, w[5], f) == w[5];
    ok = ok && fread(out.mat_idx.data(), 4, w[6], f) == w[6];
    fclose(f);
    if (!ok) return fail(TT_ERR_FORMAT, "bvh.cache truncated: " + path);
    // Structural validation: every child address must land inside its array, so that a
    // corrupt file is rejected here instead of steering a traversal out of bounds. A leaf is read
    // a triangle (three vertex entries) at a time, the second and third after the first was found
    // not to be the terminator, so from every leaf address the walk in steps of three must meet a
    // terminator inside the array. closed[i]: the walk from entry i does.
    std::vector<uint8_t> closed(w[3], 0);
    for (int64_t i = (int64_t)w[3] - 1; i >= 0; i--)
        closed[i] = (uint32_t)out.vertices[i].x == 0x80000000u || (i + 3 < (int64_t)w[3] && closed[i + 3]);
    for (uint32_t i = 0; i < w[0]; i += 4) {
        const I4 &c = out.nodes[i + 3];
        for (int32_t a : {c.x, c.y}) {
            if (a >= 0) {
                if ((a % 4) != 0 || (uint32_t)a + 3 >= w[0])
                    return fail(TT_ERR_FORMAT, "bvh.cache inner child address out of range");
            } else if ((uint32_t)(~a) >= w[3]) {
                return fail(TT_ERR_FORMAT, "bvh.cache leaf address out of range");
            } else if (!closed[~a]) {
                return fail(TT_ERR_FORMAT, "bvh.cache leaf runs past the vertex array without a terminator");
            }
        }
    }
    return TT_OK;
}

}  // namespace tt
