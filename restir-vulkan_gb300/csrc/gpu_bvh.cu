// gpu_bvh.cu -- the reference's binned-SAH AABB tree (src/aabbTreeBuilder.cpp:
// 52-214) built on the GPU, byte-identical to host_build_bvh.
//
// The reference builds breadth-first from a FIFO queue; nodes are numbered in
// pop order.  Here each BFS level is one round of kernels over all of its
// tasks (leaf ranges), in queue order:
//   bounds   centroid and box bounds per task (min/max, order-independent:
//            the inputs hold no NaN and no negative zero), warp-aggregated
//            atomics on order-preserving integer keys;
//   buckets  12 centroid buckets per task on the widest centroid axis, same;
//   sah      one thread per task runs the reference's split sweep with the
//            same float operations;
//   permute  the reference partitions with the in-place loop
//              for i: if bucket[i] <= opt: swap(a[i], a[pivot++])
//            whose result is: the k-th left element goes to beg + k, and a
//            right element at p moves along p -> L(p - beg) (the position of
//            the (p-beg)-th left element) until it reaches [beg + nL, end);
//            the chains are resolved by pointer jumping;
//   emit     node boxes (the sweep's, or the median split's recomputed over
//            the permuted halves), child links, next level's tasks.
// Tasks of one and two leaves end their branch as in the reference.
#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>
#include <string.h>

#include "rg_internal.h"

namespace {

constexpr int kBuckets = 12;

struct GLeaf {
    float c[3], lo[3], hi[3];
    int32_t geom;
};

// float -> int key with the same order (no NaN); involution on negatives
__host__ __device__ __forceinline__ int fkey(float f) {
    int b;
    memcpy(&b, &f, 4);
    return b >= 0 ? b : b ^ 0x7fffffff;
}
__host__ __device__ __forceinline__ float kfloat(int k) {
    const int b = k >= 0 ? k : k ^ 0x7fffffff;
    float f;
    memcpy(&f, &b, 4);
    return f;
}
// nvmath nv_min / nv_max
__device__ __forceinline__ float nvmin(float a, float b) { return (a < b) ? a : b; }
__device__ __forceinline__ float nvmax(float a, float b) { return (a > b) ? a : b; }

__device__ __forceinline__ float surface_area(const float *mn, const float *mx) {
    const float sx = mx[0] - mn[0], sy = mx[1] - mn[1], sz = mx[2] - mn[2];
    return (sx * sy + sx * sz) + sy * sz;
}

// Per-task state of one level.  Keys: [0..2] centroid min, [3..5] centroid
// max, [6..8] box min, [9..11] box max; buckets: count then 3 min, 3 max keys.
struct TaskState {
    int32_t beg, end, parent;  // parent: node * 2 + side, -1 for the root
    int32_t keys[12];
    int32_t bcount[kBuckets];
    int32_t bkeys[kBuckets][6];
    int32_t dim, undefined, opt, found;
    float cmin_dim, range;
    float box[12];             // left min, left max, right min, right max
    int32_t nl, pivot, fallback;
    int32_t fkeys[12];         // median-split bounds: left min, left max, right min, right max
};

__global__ void k_leaves(const float *xyz, int n, GLeaf *leaves, rg_triangle *tris) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float p[3][3];
    for (int k = 0; k < 3; ++k)
        for (int d = 0; d < 3; ++d) p[k][d] = __fadd_rn(xyz[9 * (size_t)i + 3 * k + d], 0.0f);  // -0 -> +0
    GLeaf l;
    for (int d = 0; d < 3; ++d) {
        float lo = p[0][d], hi = p[0][d];
        lo = nvmin(lo, p[1][d]);
        hi = nvmax(hi, p[1][d]);
        lo = nvmin(lo, p[2][d]);
        hi = nvmax(hi, p[2][d]);
        l.lo[d] = lo;
        l.hi[d] = hi;
        l.c[d] = 0.5f * (lo + hi);
    }
    l.geom = i;
    leaves[i] = l;
    rg_triangle t;
    for (int d = 0; d < 3; ++d) {
        t.p1[d] = p[0][d];
        t.p2[d] = p[1][d];
        t.p3[d] = p[2][d];
    }
    t.p1[3] = t.p2[3] = t.p3[3] = 1.0f;
    tris[i] = t;
}

__global__ void k_task_init(TaskState *ts, int T) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    TaskState &s = ts[t];
    const int kmin = fkey(FLT_MAX), kmax = fkey(-FLT_MAX);
    for (int j = 0; j < 12; ++j) {
        s.keys[j] = (j % 6) < 3 ? kmin : kmax;
        s.fkeys[j] = (j % 6) < 3 ? kmin : kmax;
    }
    for (int b = 0; b < kBuckets; ++b) {
        s.bcount[b] = 0;
        for (int j = 0; j < 6; ++j) s.bkeys[b][j] = j < 3 ? kmin : kmax;
    }
}

// task holding position p among the level's tasks (ordered by position), or -1
__device__ __forceinline__ int task_of(const TaskState *ts, int T, int p) {
    int lo = 0, hi = T - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (ts[mid].beg <= p) lo = mid;
        else hi = mid - 1;
    }
    return (T > 0 && ts[lo].beg <= p && p < ts[lo].end) ? lo : -1;
}

// group reduction of an int key among the lanes of `grp`, one atomic per group
__device__ __forceinline__ void group_min(unsigned grp, bool leader, int *addr, int v) {
    const int r = __reduce_min_sync(grp, v);
    if (leader) atomicMin(addr, r);
}
__device__ __forceinline__ void group_max(unsigned grp, bool leader, int *addr, int v) {
    const int r = __reduce_max_sync(grp, v);
    if (leader) atomicMax(addr, r);
}

__global__ void k_bounds(TaskState *ts, int T, const GLeaf *leaves, int n) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    int t = p < n ? task_of(ts, T, p) : -1;
    if (t >= 0 && ts[t].end - ts[t].beg < 3) t = -1;
    const unsigned grp = __match_any_sync(0xffffffffu, t);
    if (t < 0) return;
    const bool leader = (threadIdx.x & 31) == __ffs(grp) - 1;
    const GLeaf &l = leaves[p];
    TaskState &s = ts[t];
    for (int d = 0; d < 3; ++d) {
        group_min(grp, leader, &s.keys[d], fkey(l.c[d]));
        group_max(grp, leader, &s.keys[3 + d], fkey(l.c[d]));
        group_min(grp, leader, &s.keys[6 + d], fkey(l.lo[d]));
        group_max(grp, leader, &s.keys[9 + d], fkey(l.hi[d]));
    }
}

__global__ void k_split_axis(TaskState *ts, int T) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    TaskState &s = ts[t];
    if (s.end - s.beg < 3) return;
    float cmin[3], cmax[3], amin[3], amax[3];
    for (int d = 0; d < 3; ++d) {
        cmin[d] = kfloat(s.keys[d]);
        cmax[d] = kfloat(s.keys[3 + d]);
        amin[d] = kfloat(s.keys[6 + d]);
        amax[d] = kfloat(s.keys[9 + d]);
    }
    const float outer = surface_area(amin, amax);
    const float span[3] = {cmax[0] - cmin[0], cmax[1] - cmin[1], cmax[2] - cmin[2]};
    int dim = span[0] > span[1] ? 0 : 1;
    if (span[2] > span[dim]) dim = 2;
    const float range = span[dim] / (float)kBuckets;
    s.dim = dim;
    s.range = range;
    s.cmin_dim = cmin[dim];
    s.undefined = (!(range > 0.0f) || !(outer > 0.0f)) ? 1 : 0;
    // the outer heuristic is kept in box[0] until the sweep
    s.box[0] = outer;
}

__global__ void k_buckets(TaskState *ts, int T, const GLeaf *leaves, int n, uint8_t *bucket) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    int t = p < n ? task_of(ts, T, p) : -1;
    if (t >= 0 && ts[t].end - ts[t].beg < 3) t = -1;
    int b = 0;
    if (t >= 0) {
        const TaskState &s = ts[t];
        const GLeaf &l = leaves[p];
        float u = s.undefined ? 0.5f : (l.c[s.dim] - s.cmin_dim) / s.range;
        u = (u < 0.5f) ? 0.5f : u;
        u = (u > (float)kBuckets - 0.5f) ? (float)kBuckets - 0.5f : u;
        b = (int)u;
        bucket[p] = (uint8_t)b;
    }
    const unsigned grp = __match_any_sync(0xffffffffu, t < 0 ? -1 : t * kBuckets + b);
    if (t < 0) return;
    const bool leader = (threadIdx.x & 31) == __ffs(grp) - 1;
    const GLeaf &l = leaves[p];
    TaskState &s = ts[t];
    if (leader) atomicAdd(&s.bcount[b], __popc(grp));
    for (int d = 0; d < 3; ++d) {
        group_min(grp, leader, &s.bkeys[b][d], fkey(l.lo[d]));
        group_max(grp, leader, &s.bkeys[b][3 + d], fkey(l.hi[d]));
    }
}

struct DBucket {
    float mn[3], mx[3];
    float count;  // exact: counts stay below 2^24
    __device__ float heuristic() const { return count * surface_area(mn, mx); }
};
__device__ __forceinline__ DBucket merge(DBucket l, const DBucket &r) {
    l.count += r.count;
    for (int d = 0; d < 3; ++d) {
        l.mn[d] = nvmin(l.mn[d], r.mn[d]);
        l.mx[d] = nvmax(l.mx[d], r.mx[d]);
    }
    return l;
}

// the reference's split sweep (aabbTreeBuilder.cpp:146-173)
__global__ void k_sah(TaskState *ts, int T) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    TaskState &s = ts[t];
    if (s.end - s.beg < 3) return;
    const float outer = s.box[0];
    DBucket b[kBuckets];
    for (int i = 0; i < kBuckets; ++i) {
        b[i].count = (float)s.bcount[i];
        for (int d = 0; d < 3; ++d) {
            b[i].mn[d] = kfloat(s.bkeys[i][d]);
            b[i].mx[d] = kfloat(s.bkeys[i][3 + d]);
        }
    }
    DBucket cache[kBuckets - 1];
    {
        DBucket cur = b[kBuckets - 1];
        for (int i = kBuckets - 1; i > 0;) {
            cache[--i] = cur;
            cur = merge(cur, b[i]);
        }
    }
    int opt = 0, found = 0;
    float box[12] = {0};
    float best = FLT_MAX;
    DBucket left;
    for (int d = 0; d < 3; ++d) {
        left.mn[d] = FLT_MAX;
        left.mx[d] = -FLT_MAX;
    }
    left.count = 0.0f;
    for (int sp = 0; sp < kBuckets - 1; ++sp) {
        left = merge(left, b[sp]);
        const DBucket &right = cache[sp];
        const float h = 0.125f + (left.heuristic() + right.heuristic()) / outer;
        if (h < best) {
            best = h;
            opt = sp;
            for (int d = 0; d < 3; ++d) {
                box[d] = left.mn[d];
                box[3 + d] = left.mx[d];
                box[6 + d] = right.mn[d];
                box[9 + d] = right.mx[d];
            }
            found = 1;
        }
    }
    s.opt = opt;
    s.found = found;
    for (int j = 0; j < 12; ++j) s.box[j] = box[j];
}

__global__ void k_left_flags(const TaskState *ts, int T, int n, const uint8_t *bucket, int32_t *flag) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int t = task_of(ts, T, p);
    int f = 0;
    if (t >= 0 && ts[t].end - ts[t].beg >= 3) f = bucket[p] <= ts[t].opt ? 1 : 0;
    flag[p] = f;
}

// nL and the pivot of every task from the exclusive scan S (n + 1 entries)
__global__ void k_pivot(TaskState *ts, int T, const int32_t *S, int *undefined) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    TaskState &s = ts[t];
    if (s.end - s.beg < 3) return;
    if (s.undefined || !s.found) atomicOr(undefined, 1);
    s.nl = S[s.end] - S[s.beg];
    const int pivot = s.beg + s.nl;
    s.fallback = (pivot == s.beg || pivot == s.end || !s.found) ? 1 : 0;
    s.pivot = s.fallback ? (s.beg + s.end) / 2 : pivot;  // (beg + end) / 2 as the reference's size_t division
}

// lp[beg + k] = position of the task's k-th left element; nxt = first jump
__global__ void k_chains(const TaskState *ts, int T, int n, const int32_t *flag, const int32_t *S, int32_t *lp) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    if (!flag[p]) return;
    const int t = task_of(ts, T, p);
    lp[ts[t].beg + (S[p] - S[ts[t].beg])] = p;
}
__global__ void k_jump_init(const TaskState *ts, int T, int n, const int32_t *lp, int32_t *J) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int t = task_of(ts, T, p);
    int j = p;
    if (t >= 0 && ts[t].end - ts[t].beg >= 3 && p < ts[t].beg + ts[t].nl) j = lp[p];
    J[p] = j;
}
__global__ void k_jump(const int32_t *J, int32_t *J2, int n) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < n) J2[p] = J[J[p]];
}
__global__ void k_scatter(const TaskState *ts, int T, int n, const int32_t *flag, const int32_t *S, const int32_t *J,
                          const GLeaf *in, GLeaf *out) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const int t = task_of(ts, T, p);
    int dst = p;
    if (t >= 0 && ts[t].end - ts[t].beg >= 3) dst = flag[p] ? ts[t].beg + (S[p] - S[ts[t].beg]) : J[p];
    out[dst] = in[p];
}

__global__ void k_fallback_bounds(TaskState *ts, int T, const GLeaf *leaves, int n) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    int t = p < n ? task_of(ts, T, p) : -1;
    if (t >= 0 && (ts[t].end - ts[t].beg < 3 || !ts[t].fallback)) t = -1;
    const int side = t >= 0 && p >= ts[t].pivot ? 1 : 0;
    const unsigned grp = __match_any_sync(0xffffffffu, t < 0 ? -1 : 2 * t + side);
    if (t < 0) return;
    const bool leader = (threadIdx.x & 31) == __ffs(grp) - 1;
    const GLeaf &l = leaves[p];
    TaskState &s = ts[t];
    for (int d = 0; d < 3; ++d) {
        group_min(grp, leader, &s.fkeys[6 * side + d], fkey(l.lo[d]));
        group_max(grp, leader, &s.fkeys[6 * side + 3 + d], fkey(l.hi[d]));
    }
}

// flags for the task scans: node (size >= 2) and split (size >= 3)
__global__ void k_task_flags(const TaskState *ts, int T, int32_t *node_flag, int32_t *split_flag, int *max_size) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    const int sz = ts[t].end - ts[t].beg;
    node_flag[t] = sz >= 2 ? 1 : 0;
    split_flag[t] = sz >= 3 ? 1 : 0;
    atomicMax(max_size, sz);
}

__device__ __forceinline__ void put_box(float *dst4, const float *v) {
    dst4[0] = v[0];
    dst4[1] = v[1];
    dst4[2] = v[2];
    dst4[3] = 1.0f;
}
__device__ __forceinline__ void link(rg_aabb_tree_node *nodes, int parent, int32_t value) {
    if (parent < 0) return;
    if (parent & 1) nodes[parent >> 1].right_child = value;
    else nodes[parent >> 1].left_child = value;
}

__global__ void k_emit(const TaskState *ts, int T, const GLeaf *leaves, const int32_t *node_scan,
                       const int32_t *split_scan, int node_base, rg_aabb_tree_node *nodes, TaskState *next) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    const TaskState &s = ts[t];
    const int sz = s.end - s.beg;
    if (sz == 1) {
        link(nodes, s.parent, ~leaves[s.beg].geom);
        return;
    }
    const int ni = node_base + node_scan[t];
    link(nodes, s.parent, ni);
    rg_aabb_tree_node nd;
    memset(&nd, 0, sizeof(nd));
    if (sz == 2) {
        const GLeaf &l = leaves[s.beg], &r = leaves[s.beg + 1];
        put_box(nd.left_aabb_min, l.lo);
        put_box(nd.left_aabb_max, l.hi);
        put_box(nd.right_aabb_min, r.lo);
        put_box(nd.right_aabb_max, r.hi);
        nd.left_child = ~l.geom;
        nd.right_child = ~r.geom;
        nodes[ni] = nd;
        return;
    }
    float box[12];
    if (s.fallback) {
        for (int j = 0; j < 12; ++j) box[j] = kfloat(s.fkeys[j]);
    } else {
        for (int j = 0; j < 12; ++j) box[j] = s.box[j];
    }
    put_box(nd.left_aabb_min, box);
    put_box(nd.left_aabb_max, box + 3);
    put_box(nd.right_aabb_min, box + 6);
    put_box(nd.right_aabb_max, box + 9);
    nd.left_child = 0;
    nd.right_child = 0;
    nodes[ni] = nd;
    const int c = 2 * split_scan[t];
    next[c].beg = s.beg;
    next[c].end = s.pivot;
    next[c].parent = 2 * ni;
    next[c + 1].beg = s.pivot;
    next[c + 1].end = s.end;
    next[c + 1].parent = 2 * ni + 1;
}

// ---- exclusive scan of n int32 flags into out[0..n] (out[n] = total), n <= 4M
constexpr int kScanThreads = 256, kScanPer = 8, kScanBlock = kScanThreads * kScanPer;

__global__ void k_scan_block(const int32_t *in, int n, int32_t *out, int32_t *block_sums) {
    __shared__ int32_t warp_sums[kScanThreads / 32];
    const int base = blockIdx.x * kScanBlock + threadIdx.x * kScanPer;
    int32_t v[kScanPer], s = 0;
    for (int k = 0; k < kScanPer; ++k) {
        v[k] = base + k < n ? in[base + k] : 0;
        s += v[k];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int32_t incl = s;
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int32_t w = lane < kScanThreads / 32 ? warp_sums[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < kScanThreads / 32) warp_sums[lane] = w;
    }
    __syncthreads();
    int32_t run = incl - s + (warp > 0 ? warp_sums[warp - 1] : 0);
    for (int k = 0; k < kScanPer; ++k) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
    }
    if (threadIdx.x == kScanThreads - 1) block_sums[blockIdx.x] = run;
}
__global__ void k_scan_add(int32_t *out, int n, const int32_t *block_offsets) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += block_offsets[i / kScanBlock];
}
__global__ void k_scan_total(int32_t *out, int n, const int32_t *block_offsets, const int32_t *block_sums, int nb) {
    out[n] = block_offsets[nb - 1] + block_sums[nb - 1];
}

struct Scanner {
    int32_t *sums = nullptr, *offs = nullptr, *tot = nullptr;
    int cap = 0;
    cudaError_t init(int max_n) {
        cap = (max_n + kScanBlock - 1) / kScanBlock;
        if (cap > kScanBlock) return cudaErrorInvalidValue;
        cudaError_t e = cudaMalloc(&sums, (size_t)cap * 4);
        if (e == cudaSuccess) e = cudaMalloc(&offs, ((size_t)cap + 1) * 4);
        if (e == cudaSuccess) e = cudaMalloc(&tot, 4);
        return e;
    }
    void release() {
        if (sums) cudaFree(sums);
        if (offs) cudaFree(offs);
        if (tot) cudaFree(tot);
        sums = offs = tot = nullptr;
    }
    cudaError_t run(const int32_t *in, int n, int32_t *out, cudaStream_t st) {
        const int nb = (n + kScanBlock - 1) / kScanBlock;
        if (nb < 1) {
            cudaMemsetAsync(out, 0, 4, st);
            return cudaGetLastError();
        }
        k_scan_block<<<nb, kScanThreads, 0, st>>>(in, n, out, sums);
        k_scan_block<<<1, kScanThreads, 0, st>>>(sums, nb, offs, tot);
        k_scan_add<<<(n + 255) / 256, 256, 0, st>>>(out, n, offs);
        k_scan_total<<<1, 1, 0, st>>>(out, n, offs, sums, nb);
        return cudaGetLastError();
    }
};

template <typename T> cudaError_t dalloc(T **p, size_t count) {
    return cudaMalloc(reinterpret_cast<void **>(p), (count ? count : 1) * sizeof(T));
}

}  // namespace

// Builds the tree of n triangles (9 floats each, device) into nodes[n-1] and
// tris[n] (device), synchronously on `st`.  Returns the node count or a
// negative cudaError_t (as -1000 - code); *undefined receives whether a range
// took the reference-undefined path (coincident centroids or zero area).
int gpu_build_bvh(const float *xyz, int n, rg_aabb_tree_node *nodes, rg_triangle *tris, int *undefined,
                  cudaStream_t st) {
    if (n < 2 || n > (1 << 22)) return -1;
    GLeaf *la = nullptr, *lb = nullptr;
    TaskState *ta = nullptr, *tb = nullptr;
    uint8_t *bucket = nullptr;
    int32_t *flag = nullptr, *S = nullptr, *lp = nullptr, *J = nullptr, *J2 = nullptr, *tflag = nullptr,
            *tflag2 = nullptr, *tscan = nullptr, *tscan2 = nullptr;
    int *dmax = nullptr, *dundef = nullptr;
    Scanner sc;
    const int max_tasks = n;  // a level never holds more tasks than leaves
    cudaError_t e = dalloc(&la, n);
    if (e == cudaSuccess) e = dalloc(&lb, n);
    if (e == cudaSuccess) e = dalloc(&ta, max_tasks);
    if (e == cudaSuccess) e = dalloc(&tb, max_tasks);
    if (e == cudaSuccess) e = dalloc(&bucket, n);
    if (e == cudaSuccess) e = dalloc(&flag, n);
    if (e == cudaSuccess) e = dalloc(&S, (size_t)n + 1);
    if (e == cudaSuccess) e = dalloc(&lp, n);
    if (e == cudaSuccess) e = dalloc(&J, n);
    if (e == cudaSuccess) e = dalloc(&J2, n);
    if (e == cudaSuccess) e = dalloc(&tflag, max_tasks);
    if (e == cudaSuccess) e = dalloc(&tflag2, max_tasks);
    if (e == cudaSuccess) e = dalloc(&tscan, (size_t)max_tasks + 1);
    if (e == cudaSuccess) e = dalloc(&tscan2, (size_t)max_tasks + 1);
    if (e == cudaSuccess) e = dalloc(&dmax, 1);
    if (e == cudaSuccess) e = dalloc(&dundef, 1);
    if (e == cudaSuccess) e = cudaMemset(dundef, 0, 4);
    if (e == cudaSuccess) e = sc.init(n > max_tasks ? n : max_tasks);
    int rc = 0;
    int undef = 0;
    if (e == cudaSuccess) {
        const int gb = (n + 255) / 256;
        k_leaves<<<gb, 256, 0, st>>>(xyz, n, la, tris);
        e = cudaMemsetAsync(nodes, 0, sizeof(rg_aabb_tree_node) * (size_t)(n - 1), st);
        TaskState root{};
        root.beg = 0;
        root.end = n;
        root.parent = -1;
        if (e == cudaSuccess) e = cudaMemcpyAsync(ta, &root, sizeof(root), cudaMemcpyHostToDevice, st);
        int T = 1, node_base = 0;
        while (e == cudaSuccess && T > 0) {
            const int tg = (T + 127) / 128;
            k_task_init<<<tg, 128, 0, st>>>(ta, T);
            e = cudaMemsetAsync(dmax, 0, 4, st);
            k_task_flags<<<tg, 128, 0, st>>>(ta, T, tflag, tflag2, dmax);
            if (e == cudaSuccess) e = sc.run(tflag, T, tscan, st);
            if (e == cudaSuccess) e = sc.run(tflag2, T, tscan2, st);
            int maxsz = 0, nsplit = 0, nnode = 0;
            if (e == cudaSuccess) e = cudaMemcpyAsync(&maxsz, dmax, 4, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaMemcpyAsync(&nsplit, tscan2 + T, 4, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaMemcpyAsync(&nnode, tscan + T, 4, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) break;
            if (nsplit > 0) {
                k_bounds<<<gb, 256, 0, st>>>(ta, T, la, n);
                k_split_axis<<<tg, 128, 0, st>>>(ta, T);
                k_buckets<<<gb, 256, 0, st>>>(ta, T, la, n, bucket);
                k_sah<<<tg, 128, 0, st>>>(ta, T);
                k_left_flags<<<gb, 256, 0, st>>>(ta, T, n, bucket, flag);
                e = sc.run(flag, n, S, st);
                if (e != cudaSuccess) break;
                k_pivot<<<tg, 128, 0, st>>>(ta, T, S, dundef);
                k_chains<<<gb, 256, 0, st>>>(ta, T, n, flag, S, lp);
                k_jump_init<<<gb, 256, 0, st>>>(ta, T, n, lp, J);
                int rounds = 0;
                while ((1 << rounds) < maxsz) ++rounds;
                for (int r = 0; r < rounds; ++r) {
                    k_jump<<<gb, 256, 0, st>>>(J, J2, n);
                    int32_t *tmp = J;
                    J = J2;
                    J2 = tmp;
                }
                k_scatter<<<gb, 256, 0, st>>>(ta, T, n, flag, S, J, la, lb);
                GLeaf *tmp = la;
                la = lb;
                lb = tmp;
                k_fallback_bounds<<<gb, 256, 0, st>>>(ta, T, la, n);
            }
            k_emit<<<tg, 128, 0, st>>>(ta, T, la, tscan, tscan2, node_base, nodes, tb);
            e = cudaGetLastError();
            node_base += nnode;
            T = 2 * nsplit;
            TaskState *tmp = ta;
            ta = tb;
            tb = tmp;
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(&undef, dundef, 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        rc = node_base;
    }
    if (la) cudaFree(la);
    if (lb) cudaFree(lb);
    if (ta) cudaFree(ta);
    if (tb) cudaFree(tb);
    if (bucket) cudaFree(bucket);
    if (flag) cudaFree(flag);
    if (S) cudaFree(S);
    if (lp) cudaFree(lp);
    if (J) cudaFree(J);
    if (J2) cudaFree(J2);
    if (tflag) cudaFree(tflag);
    if (tflag2) cudaFree(tflag2);
    if (tscan) cudaFree(tscan);
    if (tscan2) cudaFree(tscan2);
    if (dmax) cudaFree(dmax);
    if (dundef) cudaFree(dundef);
    sc.release();
    if (undefined) *undefined = undef;
    if (e != cudaSuccess) return -1000 - (int)e;
    return rc;
}

extern "C" int rg_build_bvh_device(rg_context *ctx, const float *tri_xyz, int32_t n_tris, rg_aabb_tree_node *nodes,
                                   rg_triangle *triangles, int32_t *ref_undefined, void *stream) {
    int device = 0;
    int rc = rg_internal_device(ctx, &device);
    if (rc) return rc;
    if (!tri_xyz || !nodes || !triangles) return rg_internal_fail(RG_ERR_INVALID_ARGUMENT, "null pointer");
    if (n_tris < 2 || n_tris > (1 << 22))
        return rg_internal_fail(RG_ERR_INVALID_ARGUMENT, "rg_build_bvh_device: 2 .. 4194304 triangles");
    if (((uintptr_t)tri_xyz & 3u) || ((uintptr_t)nodes & 15u) || ((uintptr_t)triangles & 15u))
        return rg_internal_fail(RG_ERR_INVALID_ARGUMENT, "misaligned buffer");
    int undef = 0;
    const int r = gpu_build_bvh(tri_xyz, n_tris, nodes, triangles, &undef, (cudaStream_t)stream);
    if (r < 0) return rg_internal_fail(r == -1 ? RG_ERR_INVALID_ARGUMENT : RG_ERR_CUDA, "rg_build_bvh_device failed");
    if (ref_undefined) *ref_undefined = undef;
    return r;
}
