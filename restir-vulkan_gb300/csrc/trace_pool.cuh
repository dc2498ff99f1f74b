// trace_pool.cuh -- block-cooperative shadow-ray traversal.
//
// A block first collects its shadow segments in a shared-memory pool, then
// every thread of the block traces rays from that pool: a thread that
// finishes a ray immediately takes the next one (shared-memory counter), so
// the lanes of a warp stay busy until the pool runs dry instead of idling
// while the longest ray of their batch finishes.  Each thread's traversal
// stack lives in local memory by default (RG_STACK_LOCAL, cached in L1 while
// in use; measured faster than a reserved slice of shared memory, which the
// RG_STACK_LOCAL=0 build uses, interleaved by thread so consecutive lanes hit
// consecutive banks); its depth is bounded by the validated tree depth.
//
// Results equal the reference's batched stack walk
// (src/shaders/include/softwareRaytracing.glsl:42-85): the any-hit answer is
// an OR over every triangle whose whole box path passes the slab test, which
// does not depend on the visiting order; every slab and triangle test uses
// the exact arithmetic of rg_math.cuh.  On the 4-wide copy of the tree a
// path skips the boxes that the collapse expanded; for rays on the filtered
// fast path (no zero, tiny or huge direction component, no NaN box) the
// reference's slab test is monotone under box containment (t = RN((b-o)/d)
// is monotone in b, so a contained box has a later entry and an earlier exit
// on every axis), and the upload checks that every child box lies inside its
// parent's, so a box that passes implies that the skipped boxes above it
// pass: the set of triangles tested, and the answer, are unchanged.
#pragma once
#include "rg_internal.h"
#include "rg_math.cuh"

namespace rgpool {

using rgm::f3;
using rgm::mk;

// 16-byte pool entry: segment start p1 and an owner tag chosen by the
// producer; the segment end p2 comes from the caller's endpoint(owner), so
// rays that share an end (the spatial pass: one sample per pixel) store it
// once.  The tracer forms testVisibility's offset segment itself.
struct Ray {
    float4 a;  // p1.xyz, owner (int bits)
};

__device__ __forceinline__ void put_ray(Ray *pool, int slot, f3 p1, int owner) {
    pool[slot].a = make_float4(p1.x, p1.y, p1.z, __int_as_float(owner));
}

// Warp-aggregated append to a shared counter: returns this lane's slot
// (only meaningful where `want` is true).
__device__ __forceinline__ int append_slot(int *counter, bool want) {
    const unsigned mask = __ballot_sync(0xffffffffu, want);
    if (!mask) return -1;
    const int lane = (threadIdx.x + threadIdx.y * blockDim.x) & 31;
    const int leader = __ffs(mask) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(counter, __popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    return base + __popc(mask & ((1u << lane) - 1u));
}

// Warp-aggregated append of `count` consecutive slots per lane (every lane of
// the warp calls it): returns this lane's first slot.
__device__ __forceinline__ int append_range(int *counter, int count) {
    const int lane = (threadIdx.x + threadIdx.y * blockDim.x) & 31;
    int inc = count;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    const int total = __shfl_sync(0xffffffffu, inc, 31);
    int base = 0;
    if (lane == 0 && total > 0) base = atomicAdd(counter, total);
    base = __shfl_sync(0xffffffffu, base, 0);
    return base + inc - count;
}

// Slab test of one child box (softwareRaytracing.glsl:9-14).
__device__ __forceinline__ bool box_hit(f3 o, f3 d, f3 bmin, f3 bmax) {
    const float t0x = (bmin.x - o.x) / d.x, t1x = (bmax.x - o.x) / d.x;
    const float t0y = (bmin.y - o.y) / d.y, t1y = (bmax.y - o.y) / d.y;
    const float t0z = (bmin.z - o.z) / d.z, t1z = (bmax.z - o.z) / d.z;
    const float rmin = rgm::gmax(rgm::gmin(t0x, t1x), rgm::gmax(rgm::gmin(t0y, t1y), rgm::gmin(t0z, t1z)));
    const float rmax = rgm::gmin(rgm::gmax(t0x, t1x), rgm::gmin(rgm::gmax(t0y, t1y), rgm::gmax(t0z, t1z)));
    return rmin < 1.0f && rmax >= rmin && rmax > 0.0f;
}

// Filtered slab test.  The reference computes t = RN((b-o)/d) per slab; here
// t~ = RN((b-o) * RN(1/d)) with 1/d precomputed per ray.  b-o is rounded the
// same way in both, so
//   |t~ - t| <= e|t| + a,   e = 1.5 * 2^-23, a = 2^-148,
// and where either overflows to infinity the other is at least 2^127 in
// magnitude with the same sign, so clamping both to +-2^127 restores the
// bound.  rmin and rmax are max/min compositions, which
// are monotone, and min(g(x), g(y)) = g(min(x, y)) for g(t) = t +- (e|t| + a)
// (also monotone), so rmin~ and rmax~ keep the same bound against the
// reference's rmin and rmax (clamped; clamping changes none of its three
// comparisons, since rmin and rmax beyond +-2^127 already fail rmin < 1 or
// rmax > 0).  With E = 2^-19 (about 10 e) and T = 2^-90 (far above a):
//   rmin~ < 1 - E          =>  rmin < 1       rmin~ > 1 + E   =>  rmin >= 1
//   rmax~ > T              =>  rmax > 0       rmax~ < -T      =>  rmax < 0
//   D > S                  =>  rmax > rmin    D < -S          =>  rmax < rmin
// where D = RN(rmax~ - rmin~) and S = E (|rmin~| + |rmax~|) + T (both
// rounded: their errors are 2^-24 relative, far inside the factor 10).  The
// reference hits iff rmin < 1 and rmax >= rmin and rmax > 0, so all three
// left-hand tests true decide a hit and any right-hand test true decides a
// miss; otherwise (values within the margins, infinities on both sides of a
// difference, NaN) the test is undecided and the caller repeats it with
// exact division.
//
// The fast path only runs for rays whose direction components are all
// nonzero, finite and within [2^-100, 2^100] in magnitude (ray_inverse), so
// 1/d is a normal float, and only on trees whose boxes hold no NaN
// (DevScene::box_nan), so no slab value is NaN and IEEE fminf/fmaxf select
// the same values as the GLSL min/max definitions.

// max/min of three (IEEE maxNum/minNum, as fmaxf/fminf)
__device__ __forceinline__ float max3f(float a, float b, float c) {
    float y;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(y) : "f"(a), "f"(b), "f"(c));
    return y;
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
    float y;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(y) : "f"(a), "f"(b), "f"(c));
    return y;
}

// The filtered test's decision from a box's slab distances: sets hit or miss
// when decided (never both), neither when undecided.
__device__ __forceinline__ void filtered_decision(float rmin, float rmax, bool &hit, bool &miss) {
    constexpr float kEps = 1.9073486328125e-6f;     // 2^-19
    constexpr float kTiny = 8.0779356694631609e-28f; // 2^-90
    const float dd = rmax - rmin;
    const float ss = __fmaf_rn(kEps, fabsf(rmin) + fabsf(rmax), kTiny);
    hit = rmin < 1.0f - kEps && rmax > kTiny && dd > ss;
    miss = rmin > 1.0f + kEps || rmax < -kTiny || dd < -ss;
}

// The filtered test of both children of a node at once: lane .x of every
// packed pair is the left box, lane .y the right box; each lane rounds
// exactly like the scalar t~ = RN((b - o) * RN(1/d)) (b - o is b + (-o)),
// and min/max of three is the nested min/max.  Returns false when both
// children are decided (hl, hr hold the decisions), true when either needs
// the exact test.
__device__ __forceinline__ bool boxes_filtered(f3 o, f3 inv, const float4 &na, const float4 &nb, const float4 &nc,
                                               bool &hl, bool &hr) {
    const float2 nox = make_float2(-o.x, -o.x), noy = make_float2(-o.y, -o.y), noz = make_float2(-o.z, -o.z);
    const float2 ix = make_float2(inv.x, inv.x), iy = make_float2(inv.y, inv.y), iz = make_float2(inv.z, inv.z);
    const float2 t0x = __fmul2_rn(__fadd2_rn(make_float2(na.x, na.y), nox), ix);
    const float2 t1x = __fmul2_rn(__fadd2_rn(make_float2(na.z, na.w), nox), ix);
    const float2 t0y = __fmul2_rn(__fadd2_rn(make_float2(nb.x, nb.y), noy), iy);
    const float2 t1y = __fmul2_rn(__fadd2_rn(make_float2(nb.z, nb.w), noy), iy);
    const float2 t0z = __fmul2_rn(__fadd2_rn(make_float2(nc.x, nc.y), noz), iz);
    const float2 t1z = __fmul2_rn(__fadd2_rn(make_float2(nc.z, nc.w), noz), iz);
    const float rminl = max3f(fminf(t0x.x, t1x.x), fminf(t0y.x, t1y.x), fminf(t0z.x, t1z.x));
    const float rmaxl = min3f(fmaxf(t0x.x, t1x.x), fmaxf(t0y.x, t1y.x), fmaxf(t0z.x, t1z.x));
    const float rminr = max3f(fminf(t0x.y, t1x.y), fminf(t0y.y, t1y.y), fminf(t0z.y, t1z.y));
    const float rmaxr = min3f(fmaxf(t0x.y, t1x.y), fmaxf(t0y.y, t1y.y), fmaxf(t0z.y, t1z.y));
    bool ml, mr;
    filtered_decision(rminl, rmaxl, hl, ml);
    filtered_decision(rminr, rmaxr, hr, mr);
    return !((hl || ml) && (hr || mr));
}

// The exact slab tests of both children of a node; returns bit 0 left hit,
// bit 1 right hit.  Kept out of line: it runs only for nodes with an
// undecided filtered test and for rays without the fast path, and its
// divisions inlined into the walk would cost every node visit.
__device__ __noinline__ int boxes_exact(f3 o, f3 d, float4 na, float4 nb, float4 nc) {
    const bool l = box_hit(o, d, mk(na.x, nb.x, nc.x), mk(na.z, nb.z, nc.z));
    const bool r = box_hit(o, d, mk(na.y, nb.y, nc.y), mk(na.w, nb.w, nc.w));
    return (l ? 1 : 0) | (r ? 2 : 0);
}

// Per-ray reciprocal of the direction; false when a component is zero,
// tiny, huge or NaN, for which the ray uses exact division throughout.
__device__ __forceinline__ bool ray_inverse(f3 d, f3 &inv) {
    inv = mk(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    constexpr float kLo = 7.8886090522101181e-31f;  // 2^-100
    constexpr float kHi = 1.2676506002282294e30f;   // 2^100
    const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    return ax >= kLo && ax <= kHi && ay >= kLo && ay <= kHi && az >= kLo && az <= kHi;
}

__device__ __forceinline__ bool tri_hit(const GTri *tris, int t, f3 o, f3 d) {
    const GTri *tp = tris + t;
    const float4 a = __ldg(&tp->a), b = __ldg(&tp->b), c = __ldg(&tp->c);
    return rgm::ray_tri(mk(a.x, a.y, a.z), mk(a.w, b.x, b.y), mk(b.z, b.w, c.x), o, d);
}

// Lanes of a warp share one loop and each pass through it does one warp-wide
// step: refill idle lanes with new segments (once at least RG_FETCH_MIN of
// them are idle, or the whole warp is), test deferred triangles (once at
// least RG_LEAF_MIN lanes hold some, or no lane can walk on), or walk: each
// walking lane visits up to RG_WALK_STEPS tree nodes, stopping early when it
// parks a leaf or its walk ends, so the warp-wide phase checks are paid once
// per several node visits.  A node whose hit children are leaves parks them
// (two slots) instead of testing them at once, so triangle tests and ray
// set-up run with many lanes active rather than one or two.  Defaults are the
// fastest measured on the 1080p unbiased pass (walk steps 1, 2, 3, 4, 6, 8,
// 16; leaf and fetch minimums 1 to 16; the fetch minimum was retuned from 8
// to 4 for the quantized walk, within 1 %).
#ifndef RG_FETCH_MIN
#define RG_FETCH_MIN 4
#endif
#ifndef RG_LEAF_MIN
#define RG_LEAF_MIN 2
#endif
#ifndef RG_WALK_STEPS
#define RG_WALK_STEPS 8
#endif

// RG_STACK_LOCAL: keep each lane's traversal stack in local memory (cached
// in L1 only while in use) instead of a reserved slice of shared memory.
#ifndef RG_STACK_LOCAL
#define RG_STACK_LOCAL 1
#endif

// Per-lane traversal counters, reduced per warp into the context's counters.
struct TraceStats {
    bool err = false;        // walk exceeded one visit per node or the stack (malformed tree)
    unsigned visits = 0;     // tree nodes visited
    unsigned tri_tests = 0;  // triangle tests
    unsigned skipped = 0;    // pool segments the fetch declined (answer unobservable)
};

// Traces pool slots 0..n-1 with all threads of the block; `fetch(k, p1)`
// returns slot k's owner tag and sets its segment start p1, or returns a
// negative tag to skip the slot (no trace, no emit); reports shadowed (1) /
// unoccluded (0) through `emit(owner, shadowed)`.  `stack` points at
// blockDim.x * blockDim.y * depth ints of shared memory.  Sets ts.err on a
// walk longer than one visit per node or a stack overflow (malformed tree;
// not reachable for trees validated at upload).  Every thread of the block
// must call it, and the block size must be a multiple of 32.
// (The walk over the reference's binary tree, for scenes without the 4-wide
// copy.)
template <typename Fetch, typename Endpoint, typename Emit>
__device__ void trace_binary_loop(const DevScene &s, Fetch fetch, int n, int *next, int *stack, int depth,
                             TraceStats &ts, Endpoint endpoint, Emit emit) {
    constexpr unsigned kFull = 0xffffffffu;
#if RG_STACK_LOCAL
    int local_stack[RG_MAX_TREE_DEPTH + 1];
    int *my_stack = local_stack;
    const int nthreads = 1;
    (void)stack;
#else
    const int nthreads = blockDim.x * blockDim.y;
    int *my_stack = stack + threadIdx.x + threadIdx.y * blockDim.x;
#endif
    int cur = -1;          // pool index of this lane's segment, -1: none
    bool retired = false;  // the pool has no segment left for this lane
    int owner = 0, node = 0, sp = 0, visits = 0;
    int leaf0 = -1, leaf1 = -1;  // parked triangle tests
    bool walked = false;         // tree walk finished, only parked triangles remain
    f3 o = mk(0.f, 0.f, 0.f), d = o, inv = o;
    bool fast = true;
    while (true) {
        // 1. refill idle lanes, several at a time
        const bool idle = !retired && cur < 0;
        const unsigned m_idle = __ballot_sync(kFull, idle);
        const unsigned m_busy = __ballot_sync(kFull, cur >= 0);
        if (m_idle != 0u && (__popc(m_idle) >= RG_FETCH_MIN || m_busy == 0u)) {
            if (idle) {
                const int k = atomicAdd(next, 1);
                f3 p1;
                if (k >= n) {
                    retired = true;
                } else if ((owner = fetch(k, p1)) < 0) {
                    ++ts.skipped;
                } else {
                    cur = k;
                    rgm::shadow_segment(p1, endpoint(owner), o, d);
                    fast = ray_inverse(d, inv) && !s.box_nan;
                    node = 0;
                    sp = 0;
                    visits = 0;
                    leaf0 = leaf1 = -1;
                    walked = false;
                    if (s.n_nodes <= 0) {  // single-triangle scene: no tree
                        leaf0 = s.n_tris > 0 ? 0 : -1;
                        walked = true;
                        if (leaf0 < 0) { emit(owner, false); cur = -1; }
                    }
                }
            }
        }
        if (__all_sync(kFull, retired)) break;
        // 2. parked triangle tests
        const bool has_leaf = cur >= 0 && leaf0 >= 0;
        const unsigned m_leaf = __ballot_sync(kFull, has_leaf);
        const unsigned m_walk = __ballot_sync(kFull, cur >= 0 && leaf0 < 0 && !walked);
        if (m_leaf != 0u && (__popc(m_leaf) >= RG_LEAF_MIN || m_walk == 0u)) {
            if (has_leaf) {
                bool hit = tri_hit(s.tris, leaf0, o, d);
                ++ts.tri_tests;
                if (!hit && leaf1 >= 0) {
                    hit = tri_hit(s.tris, leaf1, o, d);
                    ++ts.tri_tests;
                }
                leaf0 = leaf1 = -1;
                if (hit || walked) {
                    emit(owner, hit);
                    cur = -1;
                }
            }
            continue;
        }
        // 3. up to RG_WALK_STEPS nodes per walking lane
#pragma unroll 1
        for (int step = 0; step < RG_WALK_STEPS && cur >= 0 && leaf0 < 0 && !walked; ++step) {
            ++ts.visits;
            if (++visits > s.n_nodes) {
                ts.err = true;
                emit(owner, false);
                cur = -1;
                continue;
            }
            const GNode *np = s.nodes + node;
            const float4 na = __ldg(&np->a), nb = __ldg(&np->b), nc = __ldg(&np->c);
            const int4 ch = __ldg(&np->d);
            // both filtered tests at once, then the rare exact retests
            bool hl = false, hr = false;
            if (!fast || boxes_filtered(o, inv, na, nb, nc, hl, hr)) {
                const int e = boxes_exact(o, d, na, nb, nc);
                hl = (e & 1) != 0;
                hr = (e & 2) != 0;
            }
            if (hl && ch.x < 0) leaf0 = ~ch.x;
            if (hr && ch.y < 0) {
                if (leaf0 < 0) leaf0 = ~ch.y;
                else leaf1 = ~ch.y;
            }
            const bool il = hl && ch.x >= 0, ir = hr && ch.y >= 0;
            if (il && ir) {
                // left child first (measured faster than nearer-child-first,
                // with as many node visits; with the device copy of the tree
                // in preorder the left child is the next node in memory)
                node = ch.x;
                if (sp >= depth) {
                    ts.err = true;
                    emit(owner, false);
                    cur = -1;
                    leaf0 = leaf1 = -1;
                    continue;
                }
                my_stack[sp * nthreads] = ch.y;
                ++sp;
            } else if (il) {
                node = ch.x;
            } else if (ir) {
                node = ch.y;
            } else if (sp > 0) {
                --sp;
                node = my_stack[sp * nthreads];
            } else {
                walked = true;
                if (leaf0 < 0) {
                    emit(owner, false);
                    cur = -1;
                }
            }
        }
    }
}

// The exact any-hit walk of one segment over the reference's binary tree, for
// the rays the 4-wide walk does not take (a zero, tiny or huge direction
// component): both child boxes tested by division, leaves at once.  Kept out
// of line, so its registers do not weigh on the 4-wide loop.
__device__ __noinline__ bool trace_exact_binary(const DevScene &s, f3 o, f3 d, TraceStats &ts) {
    int stack[RG_MAX_TREE_DEPTH + 1];
    int sp = 0, node = 0, visits = 0;
    for (;;) {
        ++ts.visits;
        if (++visits > s.n_nodes) { ts.err = true; return false; }
        const GNode *np = s.nodes + node;
        const float4 na = __ldg(&np->a), nb = __ldg(&np->b), nc = __ldg(&np->c);
        const int4 ch = __ldg(&np->d);
        const int e = boxes_exact(o, d, na, nb, nc);
        int nxt = -1;
        if (e & 2) {
            if (ch.y < 0) { ++ts.tri_tests; if (tri_hit(s.tris, ~ch.y, o, d)) return true; }
            else nxt = ch.y;
        }
        if (e & 1) {
            if (ch.x < 0) { ++ts.tri_tests; if (tri_hit(s.tris, ~ch.x, o, d)) return true; }
            else {
                if (nxt >= 0) {
                    if (sp >= s.depth) { ts.err = true; return false; }
                    stack[sp++] = nxt;
                }
                nxt = ch.x;
            }
        }
        if (nxt >= 0) node = nxt;
        else if (sp > 0) node = stack[--sp];
        else return false;
    }
}

// The same loop over the 4-wide copy of the tree (DevScene::wide): a node
// visit tests its four child boxes as two packed pairs; hit leaves are parked
// as a mask over the node's links and tested in the warp's triangle phase;
// the first hit inner child is walked next (the next node in memory: the copy
// is in preorder), the others pushed.  The stack needs at most three entries
// per level of the copy, which the upload checks against its 64 entries, and
// every node is visited at most once per segment (a tree).  Rays off the
// filtered fast path take trace_exact_binary as soon as they are fetched.
template <typename Fetch, typename Endpoint, typename Emit>
__device__ void trace_wide_loop(const DevScene &s, Fetch fetch, int n, int *next, TraceStats &ts, Endpoint endpoint,
                                Emit emit) {
    constexpr unsigned kFull = 0xffffffffu;
    int my_stack[RG_MAX_TREE_DEPTH + 1];
    int cur = -1;          // pool index of this lane's segment, -1: none
    bool retired = false;  // the pool has no segment left for this lane
    int owner = 0, node = 0, sp = 0, visits = 0;
    unsigned leafmask = 0; // parked triangle tests: links of leaf_node
    int leaf_node = 0;
    bool walked = false;   // tree walk finished, only parked triangles remain
    f3 o = mk(0.f, 0.f, 0.f), d = o, inv = o;
    while (true) {
        // 1. refill idle lanes, several at a time
        const bool idle = !retired && cur < 0;
        const unsigned m_idle = __ballot_sync(kFull, idle);
        const unsigned m_busy = __ballot_sync(kFull, cur >= 0);
        if (m_idle != 0u && (__popc(m_idle) >= RG_FETCH_MIN || m_busy == 0u)) {
            if (idle) {
                const int k = atomicAdd(next, 1);
                f3 p1;
                if (k >= n) {
                    retired = true;
                } else if ((owner = fetch(k, p1)) < 0) {
                    ++ts.skipped;
                } else {
                    rgm::shadow_segment(p1, endpoint(owner), o, d);
                    if (ray_inverse(d, inv)) {
                        cur = k;
                        node = 0;
                        sp = 0;
                        visits = 0;
                        leafmask = 0u;
                        walked = false;
                    } else {
                        emit(owner, trace_exact_binary(s, o, d, ts));
                    }
                }
            }
        }
        if (__all_sync(kFull, retired)) break;
        // 2. parked triangle tests
        const bool has_leaf = cur >= 0 && leafmask != 0u;
        const unsigned m_leaf = __ballot_sync(kFull, has_leaf);
        const unsigned m_walk = __ballot_sync(kFull, cur >= 0 && leafmask == 0u && !walked);
        if (m_leaf != 0u && (__popc(m_leaf) >= RG_LEAF_MIN || m_walk == 0u)) {
            if (has_leaf) {
                const int4 ch = __ldg(&s.wide[leaf_node].d);
                bool hit = false;
                for (unsigned m = leafmask; m != 0u && !hit; m &= m - 1u) {
                    const int k = __ffs(m) - 1;
                    const int link = k == 0 ? ch.x : k == 1 ? ch.y : k == 2 ? ch.z : ch.w;
                    hit = tri_hit(s.tris, ~link, o, d);
                    ++ts.tri_tests;
                }
                leafmask = 0u;
                if (hit || walked) {
                    emit(owner, hit);
                    cur = -1;
                }
            }
            continue;
        }
        // 3. up to RG_WALK_STEPS nodes per walking lane
#pragma unroll 1
        for (int step = 0; step < RG_WALK_STEPS && cur >= 0 && leafmask == 0u && !walked; ++step) {
            ++ts.visits;
            if (++visits > s.n_wide) {
                ts.err = true;
                emit(owner, false);
                cur = -1;
                continue;
            }
            const WNode *np = s.wide + node;
            const float4 na = __ldg(&np->a), nb = __ldg(&np->b), nc = __ldg(&np->c);
            const int4 ch = __ldg(&np->d);
            const float4 ne = __ldg(&np->e), nf = __ldg(&np->f), ng = __ldg(&np->g);
            bool h0 = false, h1 = false, h2 = false, h3 = false;
            if (boxes_filtered(o, inv, na, nb, nc, h0, h1)) {
                const int e = boxes_exact(o, d, na, nb, nc);
                h0 = (e & 1) != 0;
                h1 = (e & 2) != 0;
            }
            if (boxes_filtered(o, inv, ne, nf, ng, h2, h3)) {
                const int e = boxes_exact(o, d, ne, nf, ng);
                h2 = (e & 1) != 0;
                h3 = (e & 2) != 0;
            }
            h2 = h2 && ch.z != kWideNoChild;
            h3 = h3 && ch.w != kWideNoChild;
            leafmask = (h0 && ch.x < 0 ? 1u : 0u) | (h1 && ch.y < 0 ? 2u : 0u) | (h2 && ch.z < 0 ? 4u : 0u) |
                       (h3 && ch.w < 0 ? 8u : 0u);
            if (leafmask) leaf_node = node;
            int nxt = -1;
            if (h3 && ch.w >= 0) nxt = ch.w;
            if (h2 && ch.z >= 0) {
                if (nxt >= 0) my_stack[sp++] = nxt;
                nxt = ch.z;
            }
            if (h1 && ch.y >= 0) {
                if (nxt >= 0) my_stack[sp++] = nxt;
                nxt = ch.y;
            }
            if (h0 && ch.x >= 0) {
                if (nxt >= 0) my_stack[sp++] = nxt;
                nxt = ch.x;
            }
            if (nxt >= 0) {
                node = nxt;
            } else if (sp > 0) {
                node = my_stack[--sp];
            } else {
                walked = true;
                if (leafmask == 0u) {
                    emit(owner, false);
                    cur = -1;
                }
            }
        }
    }
}

// Codes sel0, sel1 (byte selectors) of a word decoded as a packed pair:
// D(q) = RN((2^23 + q) * s + c), one FMA on the float whose bits are
// 0x4B000000 | q.
__device__ __forceinline__ float2 qdecode2(unsigned w, unsigned sel0, unsigned sel1, float2 sc, float2 base) {
    const float2 f = make_float2(__uint_as_float(__byte_perm(w, 0x4B000000u, sel0)),
                                 __uint_as_float(__byte_perm(w, 0x4B000000u, sel1)));
    return __ffma2_rn(f, sc, base);
}

// Per-ray and per-node operands of the quantized box tests.  Each axis' near
// and far code words are picked by the sign of the ray's direction (near =
// lower bounds where it is positive), so the slab distances come out ordered:
// t(near) <= t(far), because b - o and the product with 1/d round
// monotonically; they equal the min and max of the two distances.
struct QAxes {
    unsigned nx, fx, ny, fy, nz, fz;  // near / far code words
};
__device__ __forceinline__ QAxes qaxes(f3 inv, const uint4 &qa, const uint4 &qb) {
    QAxes a;
    const bool sx = inv.x < 0.0f, sy = inv.y < 0.0f, sz = inv.z < 0.0f;
    a.nx = sx ? qa.y : qa.x; a.fx = sx ? qa.x : qa.y;
    a.ny = sy ? qa.w : qa.z; a.fy = sy ? qa.z : qa.w;
    a.nz = sz ? qb.y : qb.x; a.fz = sz ? qb.x : qb.y;
    return a;
}

// The sure-miss part of the filtered decision with a constant difference
// margin: where rmin~ <= 1 + E and rmax~ >= -T, a difference below -SS
// needs rmax~ < rmin~, so both lie in [-T, 1 + E] and E (|rmin~| + |rmax~|)
// + T < 2^-17 = SS; the test is therefore never looser than
// filtered_decision's.
__device__ __forceinline__ bool filtered_miss(float rmin, float rmax) {
    constexpr float kEps = 1.9073486328125e-6f;     // 2^-19
    constexpr float kTiny = 8.0779356694631609e-28f; // 2^-90
    constexpr float kSS = 7.62939453125e-6f;         // 2^-17
    return rmin > 1.0f + kEps || rmax < -kTiny || rmax - rmin < -kSS;
}

// RG_QMISS_SIGN: the quantized walk's sure-miss test as packed differences
// and the sign of their minimum (moves compares from the ALU pipe to the FMA
// pipe; 5.88 -> 5.80 ms per 1080p unbiased pass, same decisions).
#ifndef RG_QMISS_SIGN
#define RG_QMISS_SIGN 1
#endif

// Children 2p, 2p+1 of a quantized node: bit 0 / bit 1 set when the filtered
// test does not surely miss their decoded boxes.
__device__ __forceinline__ unsigned qpair_live(f3 o, f3 inv, const float4 &base, const QAxes &w, float2 sx,
                                               float2 sy, float2 sz, int p) {
    const unsigned s0 = 0x7440u + 2u * (unsigned)p, s1 = s0 + 1u;
    const float2 cx = make_float2(base.x, base.x), cy = make_float2(base.y, base.y), cz = make_float2(base.z, base.z);
    const float2 nox = make_float2(-o.x, -o.x), noy = make_float2(-o.y, -o.y), noz = make_float2(-o.z, -o.z);
    const float2 ix = make_float2(inv.x, inv.x), iy = make_float2(inv.y, inv.y), iz = make_float2(inv.z, inv.z);
    const float2 tnx = __fmul2_rn(__fadd2_rn(qdecode2(w.nx, s0, s1, sx, cx), nox), ix);
    const float2 tfx = __fmul2_rn(__fadd2_rn(qdecode2(w.fx, s0, s1, sx, cx), nox), ix);
    const float2 tny = __fmul2_rn(__fadd2_rn(qdecode2(w.ny, s0, s1, sy, cy), noy), iy);
    const float2 tfy = __fmul2_rn(__fadd2_rn(qdecode2(w.fy, s0, s1, sy, cy), noy), iy);
    const float2 tnz = __fmul2_rn(__fadd2_rn(qdecode2(w.nz, s0, s1, sz, cz), noz), iz);
    const float2 tfz = __fmul2_rn(__fadd2_rn(qdecode2(w.fz, s0, s1, sz, cz), noz), iz);
#if RG_QMISS_SIGN
    // filtered_miss of both children as signs: RN(1 + E - rmin) < 0 iff
    // rmin > 1 + E, RN(rmax + T) < 0 iff rmax < -T, RN(RN(rmax - rmin) + SS)
    // < 0 iff RN(rmax - rmin) < -SS (no result is -0: each adds a nonzero
    // constant; a NaN difference of two infinities is dropped by the minimum,
    // as its comparison is false)
    const float2 rmin = make_float2(max3f(tnx.x, tny.x, tnz.x), max3f(tnx.y, tny.y, tnz.y));
    const float2 rmax = make_float2(min3f(tfx.x, tfy.x, tfz.x), min3f(tfx.y, tfy.y, tfz.y));
    const float2 m1 = make_float2(-1.0f, -1.0f);
    const float2 a = __ffma2_rn(rmin, m1, make_float2(1.0000019073486328125f, 1.0000019073486328125f));
    const float2 b = __fadd2_rn(rmax, make_float2(8.0779356694631609e-28f, 8.0779356694631609e-28f));
    const float2 c = __fadd2_rn(__ffma2_rn(rmin, m1, rmax), make_float2(7.62939453125e-6f, 7.62939453125e-6f));
    const unsigned ml = __float_as_uint(min3f(a.x, b.x, c.x)) >> 31, mr = __float_as_uint(min3f(a.y, b.y, c.y)) >> 31;
    return (ml ^ 1u) | ((mr ^ 1u) << 1);
#else
    const bool ml = filtered_miss(max3f(tnx.x, tny.x, tnz.x), min3f(tfx.x, tfy.x, tfz.x));
    const bool mr = filtered_miss(max3f(tnx.y, tny.y, tnz.y), min3f(tfx.y, tfy.y, tfz.y));
    return (ml ? 0u : 1u) | (mr ? 0u : 2u);
#endif
}

// The exact slab test of a leaf record's box (undecided filtered tests only).
__device__ __noinline__ bool leaf_box_exact(f3 o, f3 d, float4 a, float4 b) {
    return box_hit(o, d, mk(a.x, a.y, a.z), mk(a.w, b.x, b.y));
}

// A leaf of the quantized copy: the reference's slab test of the triangle's
// exact box (filtered, exact where undecided), then its triangle test.
__device__ __forceinline__ bool qleaf_hit(const QLeaf *lp, f3 o, f3 d, f3 inv) {
    const float4 a = __ldg(&lp->a), b = __ldg(&lp->b), c = __ldg(&lp->c), e = __ldg(&lp->d);
    const float2 tx = __fmul2_rn(__fadd2_rn(make_float2(a.x, a.w), make_float2(-o.x, -o.x)), make_float2(inv.x, inv.x));
    const float2 ty = __fmul2_rn(__fadd2_rn(make_float2(a.y, b.x), make_float2(-o.y, -o.y)), make_float2(inv.y, inv.y));
    const float2 tz = __fmul2_rn(__fadd2_rn(make_float2(a.z, b.y), make_float2(-o.z, -o.z)), make_float2(inv.z, inv.z));
    const float rmin = max3f(fminf(tx.x, tx.y), fminf(ty.x, ty.y), fminf(tz.x, tz.y));
    const float rmax = min3f(fmaxf(tx.x, tx.y), fmaxf(ty.x, ty.y), fmaxf(tz.x, tz.y));
    bool hit, miss;
    filtered_decision(rmin, rmax, hit, miss);
    if (!hit && !miss) hit = leaf_box_exact(o, d, a, b);
    return hit && rgm::ray_tri(mk(b.z, b.w, c.x), mk(c.y, c.z, c.w), mk(e.x, e.y, e.z), o, d);
}

// RG_LEAF_SLOTS: parked leaf sets a lane may hold in the quantized walk (1
// or 2).  With two, a lane that parks a node's leaves keeps walking until it
// parks a second set, so fewer lanes sit idle in the walk phase and the leaf
// phase tests more lanes at once.
#ifndef RG_LEAF_SLOTS
#define RG_LEAF_SLOTS 2
#endif
// Node visits per walking lane per pass through the quantized walk's warp
// loop (with two leaf slots lanes stop less often: 8, 12, 16, 24, 32 steps
// give 5.60, 5.49, 5.44, 5.63, 5.99 ms per 1080p unbiased pass).
#ifndef RG_QWALK_STEPS
#define RG_QWALK_STEPS 16
#endif


// RG_LEAF_COMPACT: the leaf phase lists the leaves every holding lane has
// parked and tests them with all lanes of the warp (1 KB of shared memory per
// warp), instead of each lane looping over its own.
#ifndef RG_LEAF_COMPACT
#define RG_LEAF_COMPACT 1
#endif
#ifndef RG_UNBIASED_BT
#define RG_UNBIASED_BT 128
#endif
constexpr int kLeafQueueWarps = (RG_UNBIASED_BT > 128 ? RG_UNBIASED_BT : 128) / 32;  // the largest pool block

// The parked leaves of one node ((node << 4) | mask of its leaf slots): the
// exact box gate and the triangle test of each until one hits.
__device__ __forceinline__ bool qparked_hit(const DevScene &s, unsigned e, f3 o, f3 d, f3 inv, TraceStats &ts) {
    const int4 ch = __ldg(&s.qnodes[e >> 4].d);
    bool hit = false;
    for (unsigned m = e & 15u; m != 0u && !hit; m &= m - 1u) {
        const int k = __ffs(m) - 1;
        const int link = k == 0 ? ch.x : k == 1 ? ch.y : k == 2 ? ch.z : ch.w;
        hit = qleaf_hit(s.qleaves + ~link, o, d, inv);
        ++ts.tri_tests;
    }
    return hit;
}

// The loop over the quantized 4-wide copy (DevScene::qnodes): a node visit
// decodes its four child boxes and drops those the filtered test surely
// misses (a decoded box contains the exact one, so the reference's test
// misses the exact box too); the rest are walked (inner) or parked (leaves).
// A parked leaf is tested with its exact box, then its triangle, so a
// triangle is tested exactly when the reference's test passes its box,
// which on a nested tree implies its whole box path passes, as in the
// reference's walk.  Stack and order as in trace_wide_loop.
template <typename Fetch, typename Endpoint, typename Emit>
__device__ void trace_quant_loop(const DevScene &s, Fetch fetch, int n, int *next, TraceStats &ts, Endpoint endpoint,
                                 Emit emit) {
    constexpr unsigned kFull = 0xffffffffu;
#if RG_LEAF_COMPACT
    __shared__ uint32_t s_leafq[kLeafQueueWarps][32 * 8];  // per warp: up to 8 parked leaves per lane
#endif
    int my_stack[RG_MAX_TREE_DEPTH + 1];
    int cur = -1;          // pool index of this lane's segment, -1: none
    bool retired = false;  // the pool has no segment left for this lane
    int owner = 0, node = 0, sp = 0, visits = 0;
    unsigned park0 = 0u, park1 = 0u;  // parked leaves, (node << 4) | leaf slot mask; 0: none
    bool walked = false;   // tree walk finished, only parked leaves remain
    f3 o = mk(0.f, 0.f, 0.f), d = o, inv = o;
    while (true) {
        // 1. refill idle lanes, several at a time
        const bool idle = !retired && cur < 0;
        const unsigned m_idle = __ballot_sync(kFull, idle);
        const unsigned m_busy = __ballot_sync(kFull, cur >= 0);
        if (m_idle != 0u && (__popc(m_idle) >= RG_FETCH_MIN || m_busy == 0u)) {
            if (idle) {
                ts.visits += (unsigned)visits;  // the finished segment's node visits
                visits = 0;
                const int k = atomicAdd(next, 1);
                f3 p1;
                if (k >= n) {
                    retired = true;
                } else if ((owner = fetch(k, p1)) < 0) {
                    ++ts.skipped;
                } else {
                    rgm::shadow_segment(p1, endpoint(owner), o, d);
                    if (ray_inverse(d, inv)) {
                        cur = k;
                        node = 0;
                        sp = 0;
                        visits = 0;
                        park0 = park1 = 0u;
                        walked = false;
                    } else {
                        emit(owner, trace_exact_binary(s, o, d, ts));
                    }
                }
            }
        }
        if (__all_sync(kFull, retired)) break;
        // 2. parked leaves, once enough lanes cannot walk on (walk ended or
        //    every slot taken) or none can; every lane holding some tests them
        const bool blocked = cur >= 0 && (walked || (RG_LEAF_SLOTS == 1 ? park0 : park1) != 0u);
        const unsigned m_block = __ballot_sync(kFull, blocked);
        const unsigned m_walk = __ballot_sync(kFull, cur >= 0 && !blocked);
        if (m_block != 0u && (__popc(m_block) >= RG_LEAF_MIN || m_walk == 0u)) {
#if RG_LEAF_COMPACT
            // the holders' leaves go to the warp's queue ((lane << 27) |
            // record), and every lane tests queued leaves, a chunk of 32 at a
            // time, with the owning lane's ray taken by shuffles; a ray's
            // remaining leaves are skipped once one of its leaves hits
            const int lane = (threadIdx.x + threadIdx.y * blockDim.x) & 31;
            uint32_t *q = s_leafq[(threadIdx.x + threadIdx.y * blockDim.x) >> 5];
            const bool holder = cur >= 0 && park0 != 0u;
            const int cnt = holder ? __popc(park0 & 15u) + __popc(park1 & 15u) : 0;
            int incl = cnt;
#pragma unroll
            for (int sh = 1; sh < 32; sh <<= 1) {
                const int t = __shfl_up_sync(kFull, incl, sh);
                if (lane >= sh) incl += t;
            }
            const int total = __shfl_sync(kFull, incl, 31);
            if (cnt != 0) {
                int at = incl - cnt;
#pragma unroll
                for (int slot = 0; slot < 2; ++slot) {
                    const unsigned e = slot == 0 ? park0 : park1;
                    if (e == 0u) continue;
                    const int4 ch = __ldg(&s.qnodes[e >> 4].d);
                    for (unsigned m = e & 15u; m != 0u; m &= m - 1u) {
                        const int k = __ffs(m) - 1;
                        const int link = k == 0 ? ch.x : k == 1 ? ch.y : k == 2 ? ch.z : ch.w;
                        q[at++] = ((unsigned)lane << 27) | (unsigned)(~link);
                    }
                }
            }
            __syncwarp();
            unsigned hits = 0u;  // bit l: lane l's segment is shadowed
            for (int base = 0; base < total; base += 32) {
                const int j = base + lane;
                const unsigned e = j < total ? q[j] : 0u;
                const int src = (int)(e >> 27);
                const f3 so = mk(__shfl_sync(kFull, o.x, src), __shfl_sync(kFull, o.y, src), __shfl_sync(kFull, o.z, src));
                const f3 sd = mk(__shfl_sync(kFull, d.x, src), __shfl_sync(kFull, d.y, src), __shfl_sync(kFull, d.z, src));
                const f3 si =
                    mk(__shfl_sync(kFull, inv.x, src), __shfl_sync(kFull, inv.y, src), __shfl_sync(kFull, inv.z, src));
                bool h = false;
                if (j < total && ((hits >> src) & 1u) == 0u) {
                    h = qleaf_hit(s.qleaves + (e & 0x7ffffffu), so, sd, si);
                    ++ts.tri_tests;
                }
                hits |= __reduce_or_sync(kFull, h ? 1u << src : 0u);
            }
            __syncwarp();
            if (holder) {
                const bool hit = ((hits >> lane) & 1u) != 0u;
                park0 = park1 = 0u;
                if (hit || walked) {
                    emit(owner, hit);
                    cur = -1;
                }
            }
#else
            if (cur >= 0 && park0 != 0u) {
                bool hit = qparked_hit(s, park0, o, d, inv, ts);
                if (!hit && park1 != 0u) hit = qparked_hit(s, park1, o, d, inv, ts);
                park0 = park1 = 0u;
                if (hit || walked) {
                    emit(owner, hit);
                    cur = -1;
                }
            }
#endif
            continue;
        }
        // 3. up to RG_QWALK_STEPS nodes per walking lane.  The copy is built on
        //    the host from a validated tree (a tree, stack bound checked at
        //    upload), so a walk visits each node at most once; the visit count
        //    is checked here, once per pass through this loop rather than per
        //    visit (at most RG_QWALK_STEPS visits past the limit)
        if (cur >= 0 && !walked && visits > s.n_qnodes) {
            ts.err = true;
            emit(owner, false);
            cur = -1;
            park0 = park1 = 0u;
        }
#pragma unroll 1
        for (int step = 0; step < RG_QWALK_STEPS && cur >= 0 && !walked &&
                           (RG_LEAF_SLOTS == 1 ? park0 : park1) == 0u;
             ++step) {
            ++visits;
            const QNode *np = s.qnodes + node;
            const float4 base = __ldg(&np->base);
            const uint4 qa = __ldg(&np->qxy), qb = __ldg(&np->qz);
            const int4 ch = __ldg(&np->d);
            const unsigned eb = __float_as_uint(base.w);
            const float ex = __uint_as_float(qb.z), ey = __uint_as_float(qb.w),
                        ez = __uint_as_float(((eb >> 16) & 0xffu) << 23);
            const float2 sx = make_float2(ex, ex), sy = make_float2(ey, ey), sz = make_float2(ez, ez);
            const QAxes w = qaxes(inv, qa, qb);
            const unsigned live = qpair_live(o, inv, base, w, sx, sy, sz, 0) |
                                  (qpair_live(o, inv, base, w, sx, sy, sz, 1) << 2);
            const unsigned leafmask = live & (eb >> 24) & 15u;
            if (leafmask != 0u) {
                const unsigned e = ((unsigned)node << 4) | leafmask;
                if (park0 == 0u) park0 = e;
                else park1 = e;
            }
            const unsigned im = live & (eb >> 28);
            if (im != 0u) {
                // the first inner child is walked next, the others pushed
                // (last slot first, so they pop in slot order)
                const unsigned rest = im & (im - 1u);
                if (rest & 8u) my_stack[sp++] = ch.w;
                if (rest & 4u) my_stack[sp++] = ch.z;
                if (rest & 2u) my_stack[sp++] = ch.y;
                node = (im & 1u) ? ch.x : (im & 2u) ? ch.y : (im & 4u) ? ch.z : ch.w;
            } else if (sp > 0) {
                node = my_stack[--sp];
            } else {
                walked = true;
                if (park0 == 0u) {
                    emit(owner, false);
                    cur = -1;
                }
            }
        }
    }
}

// The block's walk: over the quantized or the exact 4-wide copy when the
// upload built one, else over the reference's tree.
template <typename Fetch, typename Endpoint, typename Emit>
__device__ __forceinline__ void trace_pool_f(const DevScene &s, Fetch fetch, int n, int *next, int *stack, int depth,
                                             TraceStats &ts, Endpoint endpoint, Emit emit) {
    if (s.qnodes != nullptr) trace_quant_loop(s, fetch, n, next, ts, endpoint, emit);
    else if (s.wide != nullptr) trace_wide_loop(s, fetch, n, next, ts, endpoint, emit);
    else trace_binary_loop(s, fetch, n, next, stack, depth, ts, endpoint, emit);
}

// trace_pool_f over a pool of Ray entries (start point and owner stored).
template <typename Endpoint, typename Emit>
__device__ __forceinline__ void trace_pool(const DevScene &s, const Ray *pool, int n, int *next, int *stack,
                                           int depth, TraceStats &ts, Endpoint endpoint, Emit emit) {
    trace_pool_f(
        s,
        [&](int k, f3 &p1) {
            const float4 a = pool[k].a;
            p1 = mk(a.x, a.y, a.z);
            return __float_as_int(a.w);
        },
        n, next, stack, depth, ts, endpoint, emit);
}

}  // namespace rgpool
