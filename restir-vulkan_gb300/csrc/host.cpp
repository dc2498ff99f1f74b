// host.cpp -- host-side preprocessing of the ReSTIR path: the binned-SAH AABB
// tree in the reference's node layout, the Vose alias table, scene-buffer
// repacking for the GPU and the CPU primary-ray G-buffer.
//
// Built with -ffp-contract=off so float arithmetic rounds after every
// operation, as the reference's host build does on x86-64.
#include <cmath>
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <deque>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "host_internal.h"
#include "rg_gbuffer.cuh"

namespace {

struct V3 { float x, y, z; };
inline V3 v3(float x, float y, float z) { V3 r; r.x = x; r.y = y; r.z = z; return r; }
// nvmath's nv_min / nv_max: (a < b) ? a : b and (a > b) ? a : b per component.
inline float nvmin(float a, float b) { return (a < b) ? a : b; }
inline float nvmax(float a, float b) { return (a > b) ? a : b; }
inline V3 vmin(V3 a, V3 b) { return v3(nvmin(a.x, b.x), nvmin(a.y, b.y), nvmin(a.z, b.z)); }
inline V3 vmax(V3 a, V3 b) { return v3(nvmax(a.x, b.x), nvmax(a.y, b.y), nvmax(a.z, b.z)); }
inline float comp(V3 a, int d) { return d == 0 ? a.x : (d == 1 ? a.y : a.z); }

// surfaceAreaHeuristic, aabbTreeBuilder.cpp:16-19
inline float surface_area(V3 mn, V3 mx) {
    const V3 s = v3(mx.x - mn.x, mx.y - mn.y, mx.z - mn.z);
    return s.x * s.y + s.x * s.z + s.y * s.z;
}

struct Leaf {
    V3 centroid, bmin, bmax;
    int32_t geom;
    size_t bucket;
};
struct Bucket {
    V3 bmin = v3(FLT_MAX, FLT_MAX, FLT_MAX);
    V3 bmax = v3(-FLT_MAX, -FLT_MAX, -FLT_MAX);
    size_t count = 0;
    float heuristic() const { return (float)count * surface_area(bmin, bmax); }
    static Bucket merge(Bucket l, const Bucket &r) {
        l.count += r.count;
        l.bmin = vmin(l.bmin, r.bmin);
        l.bmax = vmax(l.bmax, r.bmax);
        return l;
    }
};
struct Step {
    int32_t *parent;
    size_t beg, end;
};

inline void set_box(float *dst4, V3 v) { dst4[0] = v.x; dst4[1] = v.y; dst4[2] = v.z; dst4[3] = 1.0f; }

}  // namespace

// Binned SAH over 12 centroid buckets on the widest centroid axis, BFS node
// allocation, 2-wide nodes holding both child boxes, leaves as ~triangle.
// Follows the reference's AabbTree::build (src/aabbTreeBuilder.cpp:52-214)
// operation for operation so the emitted buffers are byte-identical to the
// reference's.  Inputs the reference leaves undefined (a range whose
// centroids all coincide, or with zero surface area) take the median split
// and are reported through *ref_undefined.
int host_build_bvh(const float *xyz, int32_t n, rg_aabb_tree_node *out_nodes, rg_triangle *out_tris,
                   int *ref_undefined) {
    constexpr size_t kBuckets = 12;
    if (n < 2) return RG_ERR_INVALID_ARGUMENT;
    if (ref_undefined) *ref_undefined = 0;
    std::vector<Leaf> leaves((size_t)n);
    for (int32_t i = 0; i < n; ++i) {
        // the reference transforms each vertex by the node's world matrix
        // (identity here): x*1 + y*0 + z*0 + 0 turns -0 into +0.
        V3 p[3];
        for (int k = 0; k < 3; ++k)
            p[k] = v3(xyz[9 * (size_t)i + 3 * k] + 0.0f, xyz[9 * (size_t)i + 3 * k + 1] + 0.0f,
                      xyz[9 * (size_t)i + 3 * k + 2] + 0.0f);
        rg_triangle &t = out_tris[i];
        set_box(t.p1, p[0]);
        set_box(t.p2, p[1]);
        set_box(t.p3, p[2]);
        Leaf &l = leaves[(size_t)i];
        l.bmin = l.bmax = p[0];
        l.bmin = vmin(l.bmin, p[1]);
        l.bmax = vmax(l.bmax, p[1]);
        l.bmin = vmin(l.bmin, p[2]);
        l.bmax = vmax(l.bmax, p[2]);
        l.geom = i;
        l.centroid = v3(0.5f * (l.bmin.x + l.bmax.x), 0.5f * (l.bmin.y + l.bmax.y), 0.5f * (l.bmin.z + l.bmax.z));
        l.bucket = 0;
    }
    memset(out_nodes, 0, sizeof(rg_aabb_tree_node) * (size_t)(n - 1));
    int32_t alloc = 0;
    int32_t dummy_root = -1;
    std::deque<Step> q;
    q.push_back(Step{&dummy_root, 0, (size_t)n});
    while (!q.empty()) {
        const Step step = q.front();
        q.pop_front();
        const size_t cnt = step.end - step.beg;
        if (cnt == 1) {
            *step.parent = ~leaves[step.beg].geom;
            continue;
        }
        if (cnt == 2) {
            const Leaf &l = leaves[step.beg], &r = leaves[step.beg + 1];
            const int32_t ni = alloc++;
            *step.parent = ni;
            rg_aabb_tree_node &nd = out_nodes[ni];
            nd.left_child = ~l.geom;
            nd.right_child = ~r.geom;
            set_box(nd.left_aabb_min, l.bmin);
            set_box(nd.left_aabb_max, l.bmax);
            set_box(nd.right_aabb_min, r.bmin);
            set_box(nd.right_aabb_max, r.bmax);
            continue;
        }
        V3 cmin = leaves[step.beg].centroid, cmax = cmin;
        V3 amin = leaves[step.beg].bmin, amax = leaves[step.beg].bmax;
        for (size_t i = step.beg + 1; i < step.end; ++i) {
            const Leaf &c = leaves[i];
            cmin = vmin(cmin, c.centroid);
            cmax = vmax(cmax, c.centroid);
            amin = vmin(amin, c.bmin);
            amax = vmax(amax, c.bmax);
        }
        const float outer = surface_area(amin, amax);
        const V3 span = v3(cmax.x - cmin.x, cmax.y - cmin.y, cmax.z - cmin.z);
        int dim = span.x > span.y ? 0 : 1;
        if (span.z > comp(span, dim)) dim = 2;
        const float range = comp(span, dim) / (float)kBuckets;
        const bool undefined = !(range > 0.0f) || !(outer > 0.0f);
        Bucket buckets[kBuckets];
        for (size_t i = step.beg; i < step.end; ++i) {
            Leaf &c = leaves[i];
            float u = undefined ? 0.5f : (comp(c.centroid, dim) - comp(cmin, dim)) / range;
            u = (u < 0.5f) ? 0.5f : u;
            u = (u > (float)kBuckets - 0.5f) ? (float)kBuckets - 0.5f : u;
            c.bucket = (size_t)u;
            Bucket &b = buckets[c.bucket];
            b.bmin = vmin(b.bmin, c.bmin);
            b.bmax = vmax(b.bmax, c.bmax);
            ++b.count;
        }
        Bucket cache[kBuckets - 1];
        {
            Bucket cur = buckets[kBuckets - 1];
            for (size_t i = kBuckets - 1; i > 0;) {
                cache[--i] = cur;
                cur = Bucket::merge(cur, buckets[i]);
            }
        }
        size_t opt = 0;
        V3 lmin = v3(0, 0, 0), lmax = lmin, rmin = lmin, rmax = lmin;
        bool found = false;
        {
            float best = FLT_MAX;
            Bucket left;
            for (size_t sp = 0; sp < kBuckets - 1; ++sp) {
                left = Bucket::merge(left, buckets[sp]);
                const Bucket &right = cache[sp];
                const float h = 0.125f + (left.heuristic() + right.heuristic()) / outer;
                if (h < best) {
                    best = h;
                    opt = sp;
                    lmin = left.bmin; lmax = left.bmax;
                    rmin = right.bmin; rmax = right.bmax;
                    found = true;
                }
            }
        }
        size_t pivot = step.beg;
        for (size_t i = step.beg; i < step.end; ++i)
            if (leaves[i].bucket <= opt) std::swap(leaves[i], leaves[pivot++]);
        if (pivot == step.beg || pivot == step.end || !found) {
            if (!found && ref_undefined) *ref_undefined = 1;
            pivot = (step.beg + step.end) / 2;
            lmin = leaves[step.beg].bmin;
            lmax = leaves[step.beg].bmax;
            for (size_t i = step.beg + 1; i < pivot; ++i) {
                lmin = vmin(lmin, leaves[i].bmin);
                lmax = vmax(lmax, leaves[i].bmax);
            }
            rmin = leaves[pivot].bmin;
            rmax = leaves[pivot].bmax;
            for (size_t i = pivot; i < step.end; ++i) {
                rmin = vmin(rmin, leaves[i].bmin);
                rmax = vmax(rmax, leaves[i].bmax);
            }
        }
        if (undefined && ref_undefined) *ref_undefined = 1;
        const int32_t ni = alloc++;
        *step.parent = ni;
        rg_aabb_tree_node &nd = out_nodes[ni];
        set_box(nd.left_aabb_min, lmin);
        set_box(nd.left_aabb_max, lmax);
        set_box(nd.right_aabb_min, rmin);
        set_box(nd.right_aabb_max, rmax);
        q.push_back(Step{&nd.left_child, step.beg, pivot});
        q.push_back(Step{&nd.right_child, pivot, step.end});
    }
    return alloc;
}

// Checks that the buffers form one tree rooted at node 0 in which every node
// and every triangle is reached exactly once, and returns its depth (root = 1)
// or a negative error.  Traversal relies on this to bound its stack and loop.
int host_validate_tree(const rg_aabb_tree_node *nodes, int32_t n_nodes, int32_t n_tris) {
    if (n_nodes <= 0) return n_tris <= 1 ? 0 : RG_ERR_INVALID_ARGUMENT;
    std::vector<uint8_t> seen_node((size_t)n_nodes, 0), seen_tri((size_t)n_tris, 0);
    std::vector<std::pair<int32_t, int>> st;
    st.push_back({0, 1});
    seen_node[0] = 1;
    int depth = 0;
    int32_t nodes_seen = 1, tris_seen = 0;
    while (!st.empty()) {
        auto [ni, d] = st.back();
        st.pop_back();
        depth = std::max(depth, d);
        const int32_t ch[2] = {nodes[ni].left_child, nodes[ni].right_child};
        for (int k = 0; k < 2; ++k) {
            const int32_t c = ch[k];
            if (c >= 0) {
                if (c >= n_nodes || seen_node[(size_t)c]) return RG_ERR_INVALID_ARGUMENT;
                seen_node[(size_t)c] = 1;
                ++nodes_seen;
                st.push_back({c, d + 1});
            } else {
                const int32_t t = ~c;
                if (t >= n_tris || seen_tri[(size_t)t]) return RG_ERR_INVALID_ARGUMENT;
                seen_tri[(size_t)t] = 1;
                ++tris_seen;
            }
        }
    }
    if (nodes_seen != n_nodes || tris_seen != n_tris) return RG_ERR_INVALID_ARGUMENT;
    return depth;
}

// Vose's alias method with FIFO work lists in float, as createAliasTable
// (src/misc.cpp:418-497): point lights weighted by luminance if any, else
// triangle lights by luminance * area.
int host_build_alias_table(const rg_point_light *pl, int32_t n_pl, const rg_tri_light *tl, int32_t n_tl,
                           rg_alias_table_column *out) {
    const int32_t n = n_pl > 0 ? n_pl : n_tl;
    if (n <= 0) return RG_ERR_INVALID_ARGUMENT;
    std::vector<float> p((size_t)n);
    std::deque<int32_t> big, small;
    float sum = 0.0f;
    for (int32_t i = 0; i < n; ++i) {
        const float v = n_pl > 0 ? pl[i].color_luminance[3] : tl[i].emission_luminance[3] * tl[i].normal_area[3];
        sum += v;
        p[(size_t)i] = v;
    }
    for (int32_t i = 0; i < n; ++i) {
        out[i].prob = 0.0f;
        out[i].alias = -1;
        out[i].ori_prob = p[(size_t)i] / sum;
        p[(size_t)i] = (float)n * p[(size_t)i] / sum;
        if (p[(size_t)i] >= 1.0f) big.push_back(i); else small.push_back(i);
    }
    while (!big.empty() && !small.empty()) {
        const int32_t g = big.front(), l = small.front();
        big.pop_front();
        small.pop_front();
        out[l].prob = p[(size_t)l];
        out[l].alias = g;
        p[(size_t)g] = (p[(size_t)g] + p[(size_t)l]) - 1.0f;
        if (p[(size_t)g] < 1.0f) small.push_back(g); else big.push_back(g);
    }
    while (!big.empty()) { const int32_t g = big.front(); big.pop_front(); out[g].prob = 1.0f; out[g].alias = g; }
    while (!small.empty()) { const int32_t l = small.front(); small.pop_front(); out[l].prob = 1.0f; out[l].alias = l; }
    for (int32_t i = 0; i < n; ++i) out[i].alias_ori_prob = out[out[i].alias].ori_prob;
    return RG_OK;
}

// GNode: per axis (a = x, b = y, c = z) left min, right min, left max, right
// max; d = left right.
void host_pack_nodes(const rg_aabb_tree_node *src, int32_t n, float *dst16) {
    for (int32_t i = 0; i < n; ++i) {
        const rg_aabb_tree_node &s = src[i];
        float *d = dst16 + 16 * (size_t)i;
        for (int a = 0; a < 3; ++a) {  // per axis: left min, right min, left max, right max
            d[4 * a] = s.left_aabb_min[a];
            d[4 * a + 1] = s.right_aabb_min[a];
            d[4 * a + 2] = s.left_aabb_max[a];
            d[4 * a + 3] = s.right_aabb_max[a];
        }
        memcpy(&d[12], &s.left_child, 4);
        memcpy(&d[13], &s.right_child, 4);
        const int32_t none = INT32_MIN;  // no third or fourth child (the walk shares the 4-wide code)
        memcpy(&d[14], &none, 4);
        memcpy(&d[15], &none, 4);
    }
}

// The tree renumbered in depth-first preorder (root 0, a node's left
// subtree right after it, then its right subtree), child links remapped;
// leaves keep their triangle indices.  The tree must be valid
// (host_validate_tree).
void host_tree_preorder(const rg_aabb_tree_node *src, int32_t n, rg_aabb_tree_node *dst) {
    if (n <= 0) return;
    std::vector<int32_t> order, renum((size_t)n, -1), st;
    order.reserve((size_t)n);
    st.push_back(0);
    while (!st.empty()) {
        const int32_t x = st.back();
        st.pop_back();
        renum[(size_t)x] = (int32_t)order.size();
        order.push_back(x);
        if (src[x].right_child >= 0) st.push_back(src[x].right_child);
        if (src[x].left_child >= 0) st.push_back(src[x].left_child);
    }
    for (int32_t i = 0; i < n; ++i) {
        rg_aabb_tree_node nd = src[order[(size_t)i]];
        if (nd.left_child >= 0) nd.left_child = renum[(size_t)nd.left_child];
        if (nd.right_child >= 0) nd.right_child = renum[(size_t)nd.right_child];
        dst[i] = nd;
    }
}

// As host_pack_nodes, over the preorder-renumbered tree: a walk that takes
// the left child first then mostly steps to the next node in memory.
void host_pack_nodes_preorder(const rg_aabb_tree_node *src, int32_t n, float *dst16) {
    if (n <= 0) return;
    std::vector<rg_aabb_tree_node> tmp((size_t)n);
    host_tree_preorder(src, n, tmp.data());
    host_pack_nodes(tmp.data(), n, dst16);
}

// ---------------------------------------------------------------- 4-wide copy
// The tree collapsed to four children per node for shadow rays on the
// filtered fast path.  A node of the copy holds the boxes of up to four
// descendants of one binary node, chosen by expanding, while fewer than four
// are held, the inner descendant with the largest box surface into its two
// children (descendants kept in left-to-right order); leaves keep their
// triangle links.  Every box is copied bit for bit from the reference's node
// that stores it.  Skipping the expanded boxes keeps the any-hit answer when
// each child box of a node lies inside the box its parent stores for it:
// the reference's slab test is then monotone along every path (a box that
// passes implies that every box containing it passes), so a triangle is
// tested by the collapsed walk exactly when its whole box path passes, as in
// the reference.  Returns the node count (preorder: a node's first inner
// child follows it), or -1 when some child box is not inside its parent's
// box (the copy is then not used).  Layout per node (32 floats): children 0,1
// as in host_pack_nodes (per axis lo0 lo1 hi0 hi1), child links (4 ints,
// kNoChild for empty slots, whose box repeats the last child's), children
// 2,3 the same way, 4 unused.
namespace {
struct WEntry { float lo[3], hi[3]; int32_t ref; };
constexpr int32_t kNoChild = INT32_MIN;

bool box_inside(const float *lo, const float *hi, const float *plo, const float *phi) {
    for (int a = 0; a < 3; ++a)
        if (!(lo[a] >= plo[a] && hi[a] <= phi[a])) return false;
    return true;
}
WEntry child_entry(const rg_aabb_tree_node &n, int side) {
    WEntry e;
    for (int a = 0; a < 3; ++a) {
        e.lo[a] = side == 0 ? n.left_aabb_min[a] : n.right_aabb_min[a];
        e.hi[a] = side == 0 ? n.left_aabb_max[a] : n.right_aabb_max[a];
    }
    e.ref = side == 0 ? n.left_child : n.right_child;
    return e;
}
float surface(const WEntry &e) {
    const float x = e.hi[0] - e.lo[0], y = e.hi[1] - e.lo[1], z = e.hi[2] - e.lo[2];
    return x * y + x * z + y * z;
}

// The up to four descendants of binary node x that one node of a 4-wide copy
// holds (expansion by largest surface, left-to-right order); clears ok when an
// expanded box does not contain its children's.  Returns their count.
int expand4(const rg_aabb_tree_node *src, int32_t x, WEntry e[4], bool &ok) {
    int n = 2;
    e[0] = child_entry(src[x], 0);
    e[1] = child_entry(src[x], 1);
    while (n < 4) {
        int pick = -1;
        float best = -1.0f;
        for (int k = 0; k < n; ++k)
            if (e[k].ref >= 0 && surface(e[k]) > best) { best = surface(e[k]); pick = k; }
        if (pick < 0) break;
        const rg_aabb_tree_node &y = src[e[pick].ref];
        const WEntry l = child_entry(y, 0), r = child_entry(y, 1);
        if (!box_inside(l.lo, l.hi, e[pick].lo, e[pick].hi) || !box_inside(r.lo, r.hi, e[pick].lo, e[pick].hi))
            ok = false;
        for (int k = n; k > pick + 1; --k) e[k] = e[k - 1];
        e[pick] = l;
        e[pick + 1] = r;
        ++n;
    }
    return n;
}

struct WideBuilder {
    const rg_aabb_tree_node *src;
    std::vector<float> *out;
    int max_depth = 0;
    bool ok = true;

    int32_t build(int32_t x, int depth) {
        max_depth = std::max(max_depth, depth);
        WEntry e[4];
        const int n = expand4(src, x, e, ok);
        const int32_t me = (int32_t)(out->size() / 32);
        out->resize(out->size() + 32, 0.0f);
        int32_t links[4] = {kNoChild, kNoChild, kNoChild, kNoChild};
        for (int k = 0; k < n; ++k) links[k] = e[k].ref < 0 ? e[k].ref : build(e[k].ref, depth + 1);
        float *d = out->data() + 32 * (size_t)me;
        for (int pair = 0; pair < 2; ++pair) {
            float *q = d + (pair == 0 ? 0 : 16);
            for (int a = 0; a < 3; ++a) {
                for (int j = 0; j < 2; ++j) {
                    const int k = 2 * pair + j;
                    // an empty slot repeats the last child's box (its link is kNoChild, so
                    // the result is ignored; a copy decides like its original)
                    const WEntry &src_e = e[k < n ? k : n - 1];
                    q[4 * a + j] = src_e.lo[a];
                    q[4 * a + 2 + j] = src_e.hi[a];
                }
            }
        }
        memcpy(d + 12, links, sizeof(links));
        return me;
    }
};
}  // namespace

int32_t host_pack_wide(const rg_aabb_tree_node *src, int32_t n, std::vector<float> &out, int *wide_depth) {
    out.clear();
    if (n <= 0) return 0;
    WideBuilder b;
    b.src = src;
    b.out = &out;
    out.reserve((size_t)32 * (size_t)(n / 2 + 1));
    b.build(0, 1);
    if (wide_depth) *wide_depth = b.max_depth;
    if (!b.ok) return -1;
    return (int32_t)(out.size() / 32);
}

// ---------------------------------------------------------------- quantized 4-wide copy
// The same collapse with each node's child boxes stored as 8-bit codes (64-
// byte nodes: a third of the binary tree's bytes).  Per axis a node stores a
// base c and a power of two s = 2^e; code q decodes to
//   D(q) = RN((2^23 + q) * s + c),
// one FMA on the float whose bits are 0x4B000000 | q (= 2^23 + q).  D is
// non-decreasing in q.  c is the largest float with D(0) <= the node's lower
// bound, e the smallest exponent with D(255) >= its upper bound, and per child
// the lower code is the largest q with D(q) <= the child's lower bound, the
// upper code the smallest with D(q) >= its upper bound, so the decoded box
// contains the child's box.  The host evaluates D with fmaf, which rounds like
// the device's FMA.  Leaf slots link (as ~index) to leaf records that hold the
// triangle's exact box from the reference's tree and the triangle itself
// (host_pack_tris form).
//
// The walk tests the decoded boxes only for a sure miss (a decoded box
// contains the exact one, and the slab test is monotone under containment),
// and gates each reached triangle with its exact box.  That answer equals the
// reference's when every child box of the reference's tree lies inside the
// box its parent stores for it (then a triangle's exact box passing implies
// its whole box path passes); host_tree_nested checks that.
//
// Node (16 words): bases xyz (float), biased exponents (bytes 0-2 of word 3)
// and the slot masks (byte 3: bit k child k is a leaf, bit 4+k an inner
// node), then per axis a word of lower codes and a word of upper codes (byte
// k = child k; x, y in words 4-7, z in words 8-9), s of x and y as floats
// (words 10-11), then 4 links (node index, ~leaf record index, or kNoChild).  Leaf record (16 floats):
// lo.xyz hi.xyz, p1.xyz e1.xyz e2.xyz, 0.
namespace {
inline float pow2f(int eb) {
    float s;
    const uint32_t bits = (uint32_t)eb << 23;
    memcpy(&s, &bits, 4);
    return s;
}
// D(q) for biased exponent eb and base c
inline float qdecode(int q, int eb, float c) { return fmaf(8388608.0f + (float)q, pow2f(eb), c); }

// Base and biased exponent of one axis of a node with bounds [lo, hi]; false
// when no exponent up to 246 (255 * s finite) reaches hi.
bool quant_axis(float lo, float hi, float &c, int &eb) {
    const double ext = (double)hi - (double)lo;
    eb = 1;
    if (ext > 0.0) eb = std::max(1, std::min(246, (int)std::ceil(std::log2(ext / 254.0)) + 127));
    for (; eb <= 246; ++eb) {
        const float s = pow2f(eb);
        float cc = (float)((double)lo - std::ldexp(1.0, eb - 127 + 23));
        while (fmaf(8388608.0f, s, cc) > lo) cc = std::nextafter(cc, -INFINITY);
        while (fmaf(8388608.0f, s, std::nextafter(cc, INFINITY)) <= lo) cc = std::nextafter(cc, INFINITY);
        const float top = qdecode(255, eb, cc);
        if (std::isfinite(cc) && std::isfinite(top) && top >= hi) {
            c = cc;
            return true;
        }
    }
    return false;
}

struct QuantBuilder {
    const rg_aabb_tree_node *src;
    const float *tris12;
    std::vector<uint32_t> *nodes;
    std::vector<float> *leaves;
    int max_depth = 0;
    bool ok = true;

    int32_t build(int32_t x, int depth) {
        max_depth = std::max(max_depth, depth);
        WEntry e[4];
        const int n = expand4(src, x, e, ok);
        const int32_t me = (int32_t)(nodes->size() / 16);
        nodes->resize(nodes->size() + 16, 0u);
        uint32_t w[16] = {0};
        float base[3] = {0.0f, 0.0f, 0.0f};
        int eb[3] = {1, 1, 1};
        for (int a = 0; a < 3; ++a) {
            float lo = e[0].lo[a], hi = e[0].hi[a];
            for (int k = 1; k < n; ++k) { lo = std::min(lo, e[k].lo[a]); hi = std::max(hi, e[k].hi[a]); }
            if (!std::isfinite(lo) || !std::isfinite(hi) || !quant_axis(lo, hi, base[a], eb[a])) ok = false;
            memcpy(&w[a], &base[a], 4);
        }
        uint32_t leafbits = 0, innerbits = 0;
        for (int k = 0; k < n; ++k) (e[k].ref < 0 ? leafbits : innerbits) |= 1u << k;
        w[3] = (uint32_t)eb[0] | ((uint32_t)eb[1] << 8) | ((uint32_t)eb[2] << 16) | ((leafbits | innerbits << 4) << 24);
        w[10] = (uint32_t)eb[0] << 23;  // s of x and y as floats (the walk reads them directly)
        w[11] = (uint32_t)eb[1] << 23;
        for (int k = 0; k < 4 && ok; ++k) {
            const WEntry &c = e[k < n ? k : n - 1];  // an empty slot repeats the last child (ignored)
            for (int a = 0; a < 3; ++a) {
                // start from the real-valued estimate, then step to the exact codes
                const double s = std::ldexp(1.0, eb[a] - 127), o = (double)base[a] + 8388608.0 * s;
                int ql = (int)std::max(0.0, std::min(255.0, std::floor(((double)c.lo[a] - o) / s)));
                int qh = (int)std::max(0.0, std::min(255.0, std::ceil(((double)c.hi[a] - o) / s)));
                while (ql > 0 && qdecode(ql, eb[a], base[a]) > c.lo[a]) --ql;
                while (ql < 255 && qdecode(ql + 1, eb[a], base[a]) <= c.lo[a]) ++ql;
                while (qh < 255 && qdecode(qh, eb[a], base[a]) < c.hi[a]) ++qh;
                while (qh > 0 && qdecode(qh - 1, eb[a], base[a]) >= c.hi[a]) --qh;
                if (!(qdecode(ql, eb[a], base[a]) <= c.lo[a]) || !(qdecode(qh, eb[a], base[a]) >= c.hi[a])) ok = false;
                w[4 + 2 * a] |= (uint32_t)ql << (8 * k);
                w[5 + 2 * a] |= (uint32_t)qh << (8 * k);
            }
        }
        int32_t links[4] = {kNoChild, kNoChild, kNoChild, kNoChild};
        for (int k = 0; k < n; ++k) {
            if (e[k].ref < 0) {
                const int32_t rec = (int32_t)(leaves->size() / 16);
                const float *t = tris12 + 12 * (size_t)(~e[k].ref);
                const float r[16] = {e[k].lo[0], e[k].lo[1], e[k].lo[2], e[k].hi[0], e[k].hi[1], e[k].hi[2],
                                     t[0], t[1], t[2], t[3], t[4], t[5], t[6], t[7], t[8], 0.0f};
                leaves->insert(leaves->end(), r, r + 16);
                links[k] = ~rec;
            }
        }
        for (int k = 0; k < n; ++k)
            if (e[k].ref >= 0) links[k] = build(e[k].ref, depth + 1);
        memcpy(&w[12], links, sizeof(links));
        memcpy(nodes->data() + 16 * (size_t)me, w, sizeof(w));
        return me;
    }
};
}  // namespace

// True when every child box of every inner node lies inside the box that the
// node's parent stores for it (the root's children have no enclosing box).
bool host_tree_nested(const rg_aabb_tree_node *src, int32_t n) {
    for (int32_t i = 0; i < n; ++i) {
        for (int side = 0; side < 2; ++side) {
            const WEntry c = child_entry(src[i], side);
            if (c.ref < 0) continue;
            const WEntry l = child_entry(src[c.ref], 0), r = child_entry(src[c.ref], 1);
            if (!box_inside(l.lo, l.hi, c.lo, c.hi) || !box_inside(r.lo, r.hi, c.lo, c.hi)) return false;
        }
    }
    return true;
}

int32_t host_pack_quant(const rg_aabb_tree_node *src, int32_t n, const float *tris12, std::vector<uint32_t> &nodes,
                        std::vector<float> &leaves, int *wide_depth) {
    nodes.clear();
    leaves.clear();
    if (n <= 0) return 0;
    if (!host_tree_nested(src, n)) return -1;
    QuantBuilder b;
    b.src = src;
    b.tris12 = tris12;
    b.nodes = &nodes;
    b.leaves = &leaves;
    nodes.reserve((size_t)16 * (size_t)(n / 3 + 1));
    leaves.reserve((size_t)16 * (size_t)(n + 1));
    b.build(0, 1);
    if (wide_depth) *wide_depth = b.max_depth;
    if (!b.ok) return -1;
    return (int32_t)(nodes.size() / 16);
}

// True when a child box coordinate of some node is NaN (e.g. a tree built
// over triangles with NaN vertices); the filtered slab test is then off.
bool host_boxes_have_nan(const rg_aabb_tree_node *nodes, int32_t n) {
    for (int32_t i = 0; i < n; ++i) {
        const rg_aabb_tree_node &s = nodes[i];
        for (int a = 0; a < 3; ++a)
            if (std::isnan(s.left_aabb_min[a]) || std::isnan(s.left_aabb_max[a]) || std::isnan(s.right_aabb_min[a]) ||
                std::isnan(s.right_aabb_max[a]))
                return true;
    }
    return false;
}

// GTri: p1.xyz, e1 = p2-p1, e2 = p3-p1 (float subtraction, as the reference's
// rayTriangleIntersection computes them).
void host_pack_tris(const rg_triangle *src, int32_t n, float *dst12) {
    for (int32_t i = 0; i < n; ++i) {
        const rg_triangle &t = src[i];
        float *d = dst12 + 12 * (size_t)i;
        d[0] = t.p1[0]; d[1] = t.p1[1]; d[2] = t.p1[2];
        d[3] = t.p2[0] - t.p1[0]; d[4] = t.p2[1] - t.p1[1]; d[5] = t.p2[2] - t.p1[2];
        d[6] = t.p3[0] - t.p1[0]; d[7] = t.p3[1] - t.p1[1]; d[8] = t.p3[2] - t.p1[2];
        d[9] = d[10] = d[11] = 0.0f;
    }
}

// R8G8B8A8_SRGB decode table: IEC 61966-2-1 in double, rounded to float once.
void srgb_lut_host(float *out256) {
    for (int i = 0; i < 256; ++i) {
        const double c = (double)i / 255.0;
        const double l = c <= 0.04045 ? c / 12.92 : pow((c + 0.055) / 1.055, 2.4);
        out256[i] = (float)l;
    }
}

int host_trace_gbuffer(const float *nodes16, int32_t n_nodes, const float *tris12, int32_t n_tris,
                       const rg_material *mats, int32_t n_mats, const rg_camera &cam, int32_t w, int32_t h,
                       uint8_t *albedo, uint16_t *normal, uint16_t *material, float *world_pos, float *depth) {
    rgm::TraceScene s;
    s.nodes = nodes16;
    s.n_nodes = n_nodes;
    s.tris = tris12;
    s.n_tris = n_tris;
#pragma omp parallel for schedule(dynamic, 16)
    for (int32_t y = 0; y < h; ++y) {
        for (int32_t x = 0; x < w; ++x) {
            rgm::f3 o, d;
            rgm::primary_ray(cam, x, y, w, h, o, d);
            const rgm::Hit hit = rgm::closest_hit(s, o, d);
            rgm::GTexel g;
            rgm::shade_texel(s, mats, n_mats, cam, o, d, hit, g);
            const size_t i = (size_t)y * (size_t)w + (size_t)x;
            memcpy(albedo + 4 * i, &g.albedo, 4);
            memcpy(normal + 4 * i, g.normal, 8);
            memcpy(material + 2 * i, &g.material, 4);
            memcpy(world_pos + 4 * i, g.wpos, 16);
            depth[i] = g.depth;
        }
    }
    return RG_OK;
}

// ---------------------------------------------------------------- light clusters
// Seeded k-means (Lloyd) over light positions for the learned proposal:
// initial centres are the lights at the first k positions of a seeded
// Fisher-Yates shuffle (SplitMix64), assignment to the nearest centre (ties
// to the smaller index, distances in double), centres moved to their
// members' mean; a centre that loses all members stays where it was.
namespace {
inline uint64_t splitmix64(uint64_t &s) {
    uint64_t z = (s += 0x9e3779b97f4a7c15ULL);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}
}  // namespace

int host_kmeans(const float *pos4, int32_t n, int32_t k, int32_t iterations, uint64_t seed, int32_t *cluster_of,
                float *centers3) {
    if (n <= 0 || k <= 0 || k > n) return RG_ERR_INVALID_ARGUMENT;
    std::vector<int32_t> perm((size_t)n);
    for (int32_t i = 0; i < n; ++i) perm[(size_t)i] = i;
    uint64_t st = seed;
    for (int32_t i = n - 1; i > 0; --i) {
        const int32_t j = (int32_t)(splitmix64(st) % (uint64_t)(i + 1));
        std::swap(perm[(size_t)i], perm[(size_t)j]);
    }
    std::vector<double> c((size_t)k * 3);
    for (int32_t j = 0; j < k; ++j)
        for (int d = 0; d < 3; ++d) c[(size_t)j * 3 + d] = pos4[(size_t)perm[(size_t)j] * 4 + d];
    for (int it = 0; it <= iterations; ++it) {
#pragma omp parallel for schedule(static)
        for (int32_t i = 0; i < n; ++i) {
            const double x = pos4[(size_t)i * 4], y = pos4[(size_t)i * 4 + 1], z = pos4[(size_t)i * 4 + 2];
            double best = 1e300;
            int32_t bj = 0;
            for (int32_t j = 0; j < k; ++j) {
                const double dx = x - c[(size_t)j * 3], dy = y - c[(size_t)j * 3 + 1], dz = z - c[(size_t)j * 3 + 2];
                const double dd = dx * dx + dy * dy + dz * dz;
                if (dd < best) { best = dd; bj = j; }
            }
            cluster_of[i] = bj;
        }
        if (it == iterations) break;
        std::vector<double> sum((size_t)k * 3, 0.0);
        std::vector<int64_t> cnt((size_t)k, 0);
        for (int32_t i = 0; i < n; ++i) {
            const int32_t j = cluster_of[i];
            for (int d = 0; d < 3; ++d) sum[(size_t)j * 3 + d] += pos4[(size_t)i * 4 + d];
            ++cnt[(size_t)j];
        }
        for (int32_t j = 0; j < k; ++j)
            if (cnt[(size_t)j] > 0)
                for (int d = 0; d < 3; ++d) c[(size_t)j * 3 + d] = sum[(size_t)j * 3 + d] / (double)cnt[(size_t)j];
    }
    if (centers3)
        for (size_t i = 0; i < c.size(); ++i) centers3[i] = (float)c[i];
    return RG_OK;
}

// Lights grouped by cluster (stable by light index), with one Vose alias
// table per cluster over its members' luminance, laid out in grouped order:
//   order[pos]        light at grouped position pos
//   offset[c]         first grouped position of cluster c (offset[k] = n)
//   col[pos]          {prob, alias grouped position, p(light|cluster) of the
//                      column's own light, p of the alias's light}
//   within[light]     p(light | its cluster)
int host_cluster_tables(const rg_point_light *pl, int32_t n, const int32_t *cluster_of, int32_t k, int32_t *order,
                        int32_t *offset, rg_alias_table_column *col, float *within) {
    std::vector<int32_t> cnt((size_t)k + 1, 0);
    for (int32_t i = 0; i < n; ++i) {
        if (cluster_of[i] < 0 || cluster_of[i] >= k) return RG_ERR_INVALID_ARGUMENT;
        ++cnt[(size_t)cluster_of[i] + 1];
    }
    offset[0] = 0;
    for (int32_t c = 0; c < k; ++c) offset[c + 1] = offset[c] + cnt[(size_t)c + 1];
    std::vector<int32_t> fill(offset, offset + k);
    for (int32_t i = 0; i < n; ++i) order[fill[(size_t)cluster_of[i]]++] = i;
    for (int32_t c = 0; c < k; ++c) {
        const int32_t b = offset[c], e = offset[c + 1], m = e - b;
        if (m <= 0) continue;
        std::vector<rg_point_light> sub((size_t)m);
        for (int32_t j = 0; j < m; ++j) sub[(size_t)j] = pl[order[b + j]];
        std::vector<rg_alias_table_column> t((size_t)m);
        host_build_alias_table(sub.data(), m, nullptr, 0, t.data());
        for (int32_t j = 0; j < m; ++j) {
            col[b + j] = t[(size_t)j];
            col[b + j].alias = b + t[(size_t)j].alias;
            within[order[b + j]] = t[(size_t)j].ori_prob;
        }
    }
    return RG_OK;
}

// ---------------------------------------------------------------- triangle lights
// collectTriangleLightsFromScene (src/misc.cpp:380-414), with the float
// operations of the nvmath calls it makes, in their order:
//   M * vec4(p, 1): u_r = ((M[r][0] x + M[r][1] y) + M[r][2] z) + M[r][3] 1
//                   (nvmath.inl:491-499; M column-major)
//   cross(a, b) = (a.y b.z - a.z b.y, a.z b.x - a.x b.z, a.x b.y - a.y b.x)
//                   (nvmath.inl:254-261)
//   norm() = sqrtf((x x + y y) + z z), v /= s per component (nvmath_types.h)
//   luminance = (0.2126f r + 0.7152f g) + 0.0722f b (common.glsl:7-9)
// and the emissive test sq_norm() > 1e-6 made in double, as the reference's
// float-to-double comparison does.
int64_t host_collect_tri_lights(const rg_mesh_instance *inst, int32_t n, rg_tri_light *out, int64_t capacity) {
    int64_t count = 0;
    for (int32_t k = 0; k < n; ++k) {
        const rg_mesh_instance &m = inst[k];
        const float *e = m.emissive_factor;
        const float esq = (e[0] * e[0] + e[1] * e[1]) + e[2] * e[2];
        if (!((double)esq > 1e-6)) continue;
        const float lum = (0.2126f * e[0] + 0.7152f * e[1]) + 0.0722f * e[2];
        const float *M = m.world_matrix;
        for (uint32_t i = 0; i + 2 < m.index_count; i += 3) {
            float p[3][4];
            for (int v = 0; v < 3; ++v) {
                const float *q = m.positions + 3 * (size_t)m.indices[i + v];
                for (int r = 0; r < 4; ++r) p[v][r] = ((M[r] * q[0] + M[4 + r] * q[1]) + M[8 + r] * q[2]) + M[12 + r] * 1.0f;
            }
            const float a0 = p[1][0] - p[0][0], a1 = p[1][1] - p[0][1], a2 = p[1][2] - p[0][2];
            const float b0 = p[2][0] - p[0][0], b1 = p[2][1] - p[0][1], b2 = p[2][2] - p[0][2];
            float nx = a1 * b2 - a2 * b1, ny = a2 * b0 - a0 * b2, nz = a0 * b1 - a1 * b0;
            float area = sqrtf((nx * nx + ny * ny) + nz * nz);
            nx /= area;
            ny /= area;
            nz /= area;
            area *= 0.5f;
            if (out && count < capacity) {
                rg_tri_light &t = out[count];
                for (int r = 0; r < 4; ++r) {
                    t.p1[r] = p[0][r];
                    t.p2[r] = p[1][r];
                    t.p3[r] = p[2][r];
                }
                t.emission_luminance[0] = e[0];
                t.emission_luminance[1] = e[1];
                t.emission_luminance[2] = e[2];
                t.emission_luminance[3] = lum;
                t.normal_area[0] = nx;
                t.normal_area[1] = ny;
                t.normal_area[2] = nz;
                t.normal_area[3] = area;
            }
            ++count;
        }
    }
    return count;
}
