// capi.cu -- the extern "C" entry points declared in include/restir_gb300.h.
//
// Argument checking happens here, on the host, before any launch: pointers,
// plane sizes, tree shape (every node and triangle reached once, depth within
// the traversal stack) and light/alias counts.  Kernels can then index
// without bounds checks.  Errors are returned as RG_ERR_* codes with a
// per-thread message; nothing throws or aborts.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <vector>

#include "host_internal.h"
#include "mlp.cuh"
#include "rg_internal.h"

// RG_NODE_PREORDER: the device copy of the tree is renumbered in depth-first
// preorder (host_pack_nodes_preorder); the walk's results do not depend on
// the numbering.
#ifndef RG_NODE_PREORDER
#define RG_NODE_PREORDER 1
#endif


namespace {

thread_local char g_err[512] = "";

int fail(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}
int cuda_fail(cudaError_t e, const char *what) {
    return fail(e == cudaErrorMemoryAllocation ? RG_ERR_OUT_OF_MEMORY : RG_ERR_CUDA, "%s: %s", what,
                cudaGetErrorString(e));
}
#define RG_CUDA(call, what)                          \
    do {                                             \
        cudaError_t e_ = (call);                     \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

template <typename T> cudaError_t dev_alloc(T **p, size_t count) {
    *p = nullptr;
    if (count == 0) return cudaSuccess;
    return cudaMalloc(reinterpret_cast<void **>(p), count * sizeof(T));
}
template <typename T> void dev_free(T *&p) {
    if (p) cudaFree(const_cast<void *>(static_cast<const void *>(p)));
    p = nullptr;
}

struct GBufSlot {
    int w = 0, h = 0;
    uint32_t *albedo = nullptr;
    uint2 *normal = nullptr;
    uint32_t *material = nullptr;
    float4 *wpos = nullptr;
    float *depth = nullptr;
    void release() { dev_free(albedo); dev_free(normal); dev_free(material); dev_free(wpos); dev_free(depth); w = h = 0; }
    rg_gbuffer view() const {
        rg_gbuffer g;
        memset(&g, 0, sizeof(g));  // default formats
        g.width = w; g.height = h;
        g.albedo = albedo; g.normal = normal; g.material = material; g.world_pos = wpos; g.depth = depth;
        return g;
    }
};

}  // namespace

struct rg_context {
    int device = 0;
    DevScene scene{};
    bool has_scene = false;
    GNode *nodes = nullptr;
    WNode *wide = nullptr;
    QNode *qnodes = nullptr;
    QLeaf *qleaves = nullptr;
    GTri *tris = nullptr;
    AliasLight *alias = nullptr;
    float4 *pl_color = nullptr;
    rg_tri_light *tri_lights = nullptr;
    rg_alias_table_column *tri_alias = nullptr;
    rg_material *materials = nullptr;
    unsigned long long *counters = nullptr;
    int *mma_timeouts = nullptr;
    ProposalState *proposal = nullptr;  // learned proposal (proposal.cu), tied to the uploaded lights
    int res_samples = 1, res_mis = 0;   // reservoir format (rg_set_reservoir_format)
    int tree_layout = RG_TREE_QUANT4;   // rg_set_tree_layout, applied at the next upload
    size_t frame_bytes = 0;             // bytes per pixel of the frame driver's reservoir buffers
    // frame driver
    int fw = 0, fh = 0;
    rg_reservoir *res[2] = {nullptr, nullptr};
    rg_reservoir *tmp = nullptr;
    float4 *image = nullptr;
    GBufSlot gslot[2];
    bool gslot_valid[2] = {false, false};
    // visibility cache of own-segment answers between ray passes (VisCache)
    float4 *vc_buf[2] = {nullptr, nullptr};
    size_t vc_cap = 0;        // entries per buffer
    int vc_cur = 0;           // the buffer the last ray pass wrote
    uint32_t vc_tag = 0;
    bool vc_on = true;        // rg_set_visibility_cache
    bool vc_dirty = true;     // clear before the next use (new scene, new buffers)

    void release_scene() {
        proposal_release(proposal);
        proposal = nullptr;
        dev_free(nodes); dev_free(wide); dev_free(qnodes); dev_free(qleaves); dev_free(tris); dev_free(alias); dev_free(pl_color); dev_free(tri_lights);
        dev_free(tri_alias); dev_free(materials);
        has_scene = false;
    }
    void release_frame() {
        dev_free(res[0]); dev_free(res[1]); dev_free(tmp); dev_free(image);
        gslot[0].release(); gslot[1].release();
        gslot_valid[0] = gslot_valid[1] = false;
        fw = fh = 0;
    }
};

namespace {

int check_ctx(rg_context *ctx, bool need_scene) {
    if (!ctx) return fail(RG_ERR_INVALID_ARGUMENT, "null context");
    if (need_scene && !ctx->has_scene) return fail(RG_ERR_NO_SCENE, "no scene uploaded");
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    return RG_OK;
}

int check_gbuffer(const rg_gbuffer *g, uint32_t w, uint32_t h, const char *name) {
    if (!g) return fail(RG_ERR_INVALID_ARGUMENT, "%s: null G-buffer", name);
    if (g->width <= 0 || g->height <= 0 || (uint32_t)g->width != w || (uint32_t)g->height != h)
        return fail(RG_ERR_INVALID_ARGUMENT, "%s: G-buffer is %dx%d, uniforms say %ux%u", name, g->width, g->height, w, h);
    if (!g->albedo || !g->normal || !g->material || !g->world_pos || !g->depth)
        return fail(RG_ERR_INVALID_ARGUMENT, "%s: null G-buffer plane", name);
    // formats: the reference's candidates (gBufferPass.cpp:81-101) or 0
    const int nf = g->normal_format, pf = g->world_pos_format, df = g->depth_format;
    uintptr_t n_align;
    switch (nf) {
        case 0: case RG_FORMAT_R16G16B16A16_SFLOAT: case RG_FORMAT_R16G16B16A16_SNORM: n_align = 8; break;
        case RG_FORMAT_R16G16B16_SNORM: case RG_FORMAT_R16G16B16_SFLOAT: n_align = 2; break;
        case RG_FORMAT_R32G32B32_SFLOAT: n_align = 4; break;
        default: return fail(RG_ERR_UNSUPPORTED, "%s: normal format %d is not one of the reference's", name, nf);
    }
    uintptr_t p_align;
    switch (pf) {
        case 0: case RG_FORMAT_R32G32B32A32_SFLOAT: p_align = 16; break;
        case RG_FORMAT_R32G32B32_SFLOAT: p_align = 4; break;
        default: return fail(RG_ERR_UNSUPPORTED, "%s: world-position format %d is not one of the reference's", name, pf);
    }
    if (df != 0 && df != RG_FORMAT_D32_SFLOAT && df != RG_FORMAT_D32_SFLOAT_S8_UINT && df != RG_FORMAT_D24_UNORM_S8_UINT)
        return fail(RG_ERR_UNSUPPORTED, "%s: depth format %d is not one of the reference's", name, df);
    if (g->_reserved != 0) return fail(RG_ERR_INVALID_ARGUMENT, "%s: reserved field must be 0", name);
    if (((uintptr_t)g->normal & (n_align - 1)) || ((uintptr_t)g->world_pos & (p_align - 1)) ||
        ((uintptr_t)g->albedo & 3u) || ((uintptr_t)g->material & 3u) || ((uintptr_t)g->depth & 3u))
        return fail(RG_ERR_INVALID_ARGUMENT, "%s: misaligned G-buffer plane", name);
    return RG_OK;
}

int check_res(const void *p, const char *name) {
    if (!p) return fail(RG_ERR_INVALID_ARGUMENT, "%s: null reservoir buffer", name);
    if ((uintptr_t)p & 15u) return fail(RG_ERR_INVALID_ARGUMENT, "%s: reservoir buffer not 16-byte aligned", name);
    return RG_OK;
}

int check_size(uint32_t w, uint32_t h) {
    if (w == 0 || h == 0 || w > 32768 || h > 32768) return fail(RG_ERR_INVALID_ARGUMENT, "bad screen size %ux%u", w, h);
    return RG_OK;
}

}  // namespace

extern "C" {

const char *rg_last_error(void) { return g_err; }

int rg_create(int32_t device, rg_context **out) {
    if (!out) return fail(RG_ERR_INVALID_ARGUMENT, "null output pointer");
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceCount");
    if (device < 0 || device >= n) return fail(RG_ERR_INVALID_ARGUMENT, "device %d out of range (%d devices)", device, n);
    RG_CUDA(cudaSetDevice(device), "cudaSetDevice");
    noalloc_forget_device(device);
    rg_context *ctx = new rg_context();
    ctx->device = device;
    float lut[256];
    srgb_lut_host(lut);
    e = upload_srgb_lut(lut);
    if (e == cudaSuccess) e = dev_alloc(&ctx->counters, 4);
    if (e == cudaSuccess) e = cudaMemset(ctx->counters, 0, 4 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = dev_alloc(&ctx->mma_timeouts, 1);
    if (e == cudaSuccess) e = cudaMemset(ctx->mma_timeouts, 0, sizeof(int));
    if (e != cudaSuccess) {
        dev_free(ctx->counters);
        dev_free(ctx->mma_timeouts);
        delete ctx;
        return cuda_fail(e, "rg_create");
    }
    *out = ctx;
    return RG_OK;
}

int rg_destroy(rg_context *ctx) {
    if (!ctx) return RG_OK;
    cudaSetDevice(ctx->device);
    ctx->release_scene();
    ctx->release_frame();
    dev_free(ctx->counters);
    dev_free(ctx->mma_timeouts);
    dev_free(ctx->vc_buf[0]);
    dev_free(ctx->vc_buf[1]);
    delete ctx;
    return RG_OK;
}

int rg_get_stats(rg_context *ctx, rg_stats *out, int32_t reset) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (!out) return fail(RG_ERR_INVALID_ARGUMENT, "null stats");
    unsigned long long c[4];
    RG_CUDA(cudaDeviceSynchronize(), "rg_get_stats");
    RG_CUDA(cudaMemcpy(c, ctx->counters, sizeof(c), cudaMemcpyDeviceToHost), "rg_get_stats");
    out->rays_traced = c[0];
    out->traversal_errors = c[1];
    out->node_visits = c[2];
    out->triangle_tests = c[3];
    int to = 0;
    RG_CUDA(cudaMemcpy(&to, ctx->mma_timeouts, sizeof(int), cudaMemcpyDeviceToHost), "rg_get_stats");
    out->mma_timeouts = (uint64_t)to;
    out->wide_nodes = !ctx->has_scene ? 0u : ctx->scene.qnodes ? (uint64_t)ctx->scene.n_qnodes
                                                                : (uint64_t)ctx->scene.n_wide;
    out->tree_layout = !ctx->has_scene ? RG_TREE_BINARY : ctx->scene.qnodes ? RG_TREE_QUANT4
                                                        : ctx->scene.wide ? RG_TREE_WIDE4 : RG_TREE_BINARY;
    if (reset) RG_CUDA(cudaMemset(ctx->mma_timeouts, 0, sizeof(int)), "rg_get_stats");
    if (reset) RG_CUDA(cudaMemset(ctx->counters, 0, sizeof(c)), "rg_get_stats");
    return RG_OK;
}

int64_t rg_collect_triangle_lights(const rg_mesh_instance *instances, int32_t n_instances, rg_tri_light *out,
                                   int64_t capacity) {
    if (n_instances < 0 || capacity < 0 || (n_instances > 0 && !instances))
        return fail(RG_ERR_INVALID_ARGUMENT, "rg_collect_triangle_lights: bad arguments");
    for (int32_t k = 0; k < n_instances; ++k)
        if (instances[k].index_count > 0 && (!instances[k].positions || !instances[k].indices))
            return fail(RG_ERR_INVALID_ARGUMENT, "rg_collect_triangle_lights: instance %d has no mesh", k);
    return host_collect_tri_lights(instances, n_instances, out, capacity);
}

int rg_build_bvh(const float *tri_xyz, int32_t n_tris, rg_aabb_tree_node *out_nodes, rg_triangle *out_tris) {
    if (!tri_xyz || !out_nodes || !out_tris) return fail(RG_ERR_INVALID_ARGUMENT, "null pointer");
    if (n_tris < 2) return fail(RG_ERR_INVALID_ARGUMENT, "the reference's tree needs at least 2 triangles");
    int undefined = 0;
    int rc = host_build_bvh(tri_xyz, n_tris, out_nodes, out_tris, &undefined);
    if (rc < 0) return fail(rc, "rg_build_bvh failed");
    return rc;
}

int rg_tree_depth(const rg_aabb_tree_node *nodes, int32_t n_nodes) {
    if (!nodes && n_nodes > 0) return fail(RG_ERR_INVALID_ARGUMENT, "null nodes");
    int d = host_validate_tree(nodes, n_nodes, n_nodes + 1);
    if (d < 0) return fail(d, "malformed tree");
    return d;
}

int rg_tree_preorder(const rg_aabb_tree_node *nodes, int32_t n_nodes, rg_aabb_tree_node *out) {
    if ((!nodes || !out) && n_nodes > 0) return fail(RG_ERR_INVALID_ARGUMENT, "null pointer");
    if (n_nodes < 0) return fail(RG_ERR_INVALID_ARGUMENT, "negative node count");
    if (nodes == out && n_nodes > 0) return fail(RG_ERR_INVALID_ARGUMENT, "nodes and out must differ");
    const int d = host_validate_tree(nodes, n_nodes, n_nodes + 1);
    if (d < 0) return fail(d, "malformed tree");
    host_tree_preorder(nodes, n_nodes, out);
    return n_nodes;
}

int rg_build_alias_table(const rg_point_light *pl, int32_t n_pl, const rg_tri_light *tl, int32_t n_tl,
                         rg_alias_table_column *out) {
    if (!out) return fail(RG_ERR_INVALID_ARGUMENT, "null output");
    if (n_pl > 0 && !pl) return fail(RG_ERR_INVALID_ARGUMENT, "null point lights");
    if (n_pl <= 0 && (n_tl <= 0 || !tl)) return fail(RG_ERR_INVALID_ARGUMENT, "no lights");
    return host_build_alias_table(pl, n_pl, tl, n_tl, out);
}

int rg_trace_gbuffer_host(const rg_scene_desc *sc, const rg_camera *cam, int32_t w, int32_t h, uint8_t *albedo,
                          uint16_t *normal, uint16_t *material, float *world_pos, float *depth) {
    if (!sc || !cam || !albedo || !normal || !material || !world_pos || !depth)
        return fail(RG_ERR_INVALID_ARGUMENT, "null pointer");
    if (w <= 0 || h <= 0) return fail(RG_ERR_INVALID_ARGUMENT, "bad size");
    int d = host_validate_tree(sc->nodes, sc->n_nodes, sc->n_triangles);
    if (d < 0) return fail(RG_ERR_INVALID_ARGUMENT, "malformed tree");
    if (d > RG_MAX_TREE_DEPTH) return fail(RG_ERR_TREE_TOO_DEEP, "tree depth %d > %d", d, RG_MAX_TREE_DEPTH);
    std::vector<float> n16(16 * (size_t)(sc->n_nodes > 0 ? sc->n_nodes : 1)), t12(12 * (size_t)sc->n_triangles);
    host_pack_nodes(sc->nodes, sc->n_nodes, n16.data());
    host_pack_tris(sc->triangles, sc->n_triangles, t12.data());
    return host_trace_gbuffer(n16.data(), sc->n_nodes, t12.data(), sc->n_triangles, sc->materials, sc->n_materials,
                              *cam, w, h, albedo, normal, material, world_pos, depth);
}

int rg_upload_scene(rg_context *ctx, const rg_scene_desc *sc) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (!sc) return fail(RG_ERR_INVALID_ARGUMENT, "null scene");
    if (sc->n_triangles < 0 || sc->n_nodes < 0 || sc->n_point_lights < 0 || sc->n_tri_lights < 0)
        return fail(RG_ERR_INVALID_ARGUMENT, "negative count");
    if (sc->n_triangles > 0 && !sc->triangles) return fail(RG_ERR_INVALID_ARGUMENT, "null triangles");
    if (sc->n_nodes > 0 && !sc->nodes) return fail(RG_ERR_INVALID_ARGUMENT, "null nodes");
    if (sc->n_nodes > 0 && sc->n_nodes != sc->n_triangles - 1)
        return fail(RG_ERR_INVALID_ARGUMENT, "tree has %d nodes for %d triangles", sc->n_nodes, sc->n_triangles);
    const int depth = host_validate_tree(sc->nodes, sc->n_nodes, sc->n_triangles);
    if (depth < 0) return fail(RG_ERR_INVALID_ARGUMENT, "malformed tree (every node/triangle must be reached once)");
    if (depth > RG_MAX_TREE_DEPTH) return fail(RG_ERR_TREE_TOO_DEEP, "tree depth %d > %d", depth, RG_MAX_TREE_DEPTH);
    const bool point = sc->n_point_lights > 0;
    const int32_t n_lights = point ? sc->n_point_lights : sc->n_tri_lights;
    if (n_lights <= 0) return fail(RG_ERR_INVALID_ARGUMENT, "scene has no lights");
    if (point && !sc->point_lights) return fail(RG_ERR_INVALID_ARGUMENT, "null point lights");
    if (!point && !sc->tri_lights) return fail(RG_ERR_INVALID_ARGUMENT, "null triangle lights");
    if (!sc->alias_table || sc->n_alias != n_lights)
        return fail(RG_ERR_INVALID_ARGUMENT, "alias table must have one column per light (%d vs %d)", sc->n_alias, n_lights);
    for (int32_t i = 0; i < sc->n_alias; ++i) {
        const int32_t a = sc->alias_table[i].alias;
        if (a < 0 || a >= n_lights) return fail(RG_ERR_INVALID_ARGUMENT, "alias column %d points to %d", i, a);
    }
    if (sc->n_materials > 0 && !sc->materials) return fail(RG_ERR_INVALID_ARGUMENT, "null materials");

    ctx->release_scene();
    cudaError_t e = cudaSuccess;
    std::vector<float> n16(16 * (size_t)sc->n_nodes), t12(12 * (size_t)sc->n_triangles);
#if RG_NODE_PREORDER
    host_pack_nodes_preorder(sc->nodes, sc->n_nodes, n16.data());
#else
    host_pack_nodes(sc->nodes, sc->n_nodes, n16.data());
#endif
    host_pack_tris(sc->triangles, sc->n_triangles, t12.data());
    // the 4-wide copy for fast-path shadow rays (rg_set_tree_layout)
    const bool box_nan = host_boxes_have_nan(sc->nodes, sc->n_nodes);
    std::vector<float> w32;
    int wide_depth = 0;
    int32_t n_wide = -1;
    if (ctx->tree_layout == RG_TREE_WIDE4 && sc->n_nodes > 0 && !box_nan)
        n_wide = host_pack_wide(sc->nodes, sc->n_nodes, w32, &wide_depth);
    const int wide_stack = 3 * wide_depth + 1;
    if (n_wide > 0 && wide_stack > RG_MAX_TREE_DEPTH + 1) n_wide = -1;
    std::vector<uint32_t> q16;
    std::vector<float> ql16;
    int q_depth = 0;
    int32_t n_q = -1;
    if (ctx->tree_layout == RG_TREE_QUANT4 && sc->n_nodes > 0 && !box_nan)
        n_q = host_pack_quant(sc->nodes, sc->n_nodes, t12.data(), q16, ql16, &q_depth);
    if (n_q > 0 && 3 * q_depth + 1 > RG_MAX_TREE_DEPTH + 1) n_q = -1;
    if (n_q > (1 << 27) || sc->n_triangles >= (1 << 27)) n_q = -1;  // node << 4, lane << 27 | leaf record
    e = dev_alloc(&ctx->nodes, (size_t)sc->n_nodes);
    if (e == cudaSuccess && sc->n_nodes) e = cudaMemcpy(ctx->nodes, n16.data(), n16.size() * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && n_wide > 0) {
        e = dev_alloc(&ctx->wide, (size_t)n_wide);
        if (e == cudaSuccess) e = cudaMemcpy(ctx->wide, w32.data(), w32.size() * 4, cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess && n_q > 0) {
        e = dev_alloc(&ctx->qnodes, (size_t)n_q);
        if (e == cudaSuccess) e = cudaMemcpy(ctx->qnodes, q16.data(), q16.size() * 4, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = dev_alloc(&ctx->qleaves, ql16.size() / 16);
        if (e == cudaSuccess) e = cudaMemcpy(ctx->qleaves, ql16.data(), ql16.size() * 4, cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = dev_alloc(&ctx->tris, (size_t)sc->n_triangles);
    if (e == cudaSuccess && sc->n_triangles) e = cudaMemcpy(ctx->tris, t12.data(), t12.size() * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && point) {
        std::vector<AliasLight> al((size_t)n_lights);
        std::vector<float4> col((size_t)n_lights);
        for (int32_t i = 0; i < n_lights; ++i) {
            const rg_alias_table_column &c = sc->alias_table[i];
            const rg_point_light &own = sc->point_lights[i], &ali = sc->point_lights[c.alias];
            float alias_bits;
            memcpy(&alias_bits, &c.alias, 4);
            al[(size_t)i].col = make_float4(c.prob, alias_bits, c.ori_prob, c.alias_ori_prob);
            al[(size_t)i].own_pos = make_float4(own.pos[0], own.pos[1], own.pos[2], own.color_luminance[3]);
            al[(size_t)i].alias_pos = make_float4(ali.pos[0], ali.pos[1], ali.pos[2], ali.color_luminance[3]);
            col[(size_t)i] = make_float4(own.color_luminance[0], own.color_luminance[1], own.color_luminance[2],
                                         own.color_luminance[3]);
        }
        e = dev_alloc(&ctx->alias, al.size());
        if (e == cudaSuccess) e = cudaMemcpy(ctx->alias, al.data(), al.size() * sizeof(AliasLight), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = dev_alloc(&ctx->pl_color, col.size());
        if (e == cudaSuccess) e = cudaMemcpy(ctx->pl_color, col.data(), col.size() * sizeof(float4), cudaMemcpyHostToDevice);
    } else if (e == cudaSuccess) {
        e = dev_alloc(&ctx->tri_lights, (size_t)n_lights);
        if (e == cudaSuccess)
            e = cudaMemcpy(ctx->tri_lights, sc->tri_lights, (size_t)n_lights * sizeof(rg_tri_light), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = dev_alloc(&ctx->tri_alias, (size_t)n_lights);
        if (e == cudaSuccess)
            e = cudaMemcpy(ctx->tri_alias, sc->alias_table, (size_t)n_lights * sizeof(rg_alias_table_column),
                           cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess && sc->n_materials > 0) {
        e = dev_alloc(&ctx->materials, (size_t)sc->n_materials);
        if (e == cudaSuccess)
            e = cudaMemcpy(ctx->materials, sc->materials, (size_t)sc->n_materials * sizeof(rg_material),
                           cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) {
        ctx->release_scene();
        return cuda_fail(e, "rg_upload_scene");
    }
    DevScene &s = ctx->scene;
    s.nodes = ctx->nodes;
    s.n_nodes = sc->n_nodes;
    s.depth = depth < 1 ? 1 : depth;
    s.box_nan = box_nan ? 1 : 0;
    s.wide = n_wide > 0 ? ctx->wide : nullptr;
    s.n_wide = n_wide > 0 ? n_wide : 0;
    s.wide_stack = n_wide > 0 ? wide_stack : 0;
    s.qnodes = n_q > 0 ? ctx->qnodes : nullptr;
    s.qleaves = n_q > 0 ? ctx->qleaves : nullptr;
    s.n_qnodes = n_q > 0 ? n_q : 0;
    if (n_q > 0) s.wide_stack = 3 * q_depth + 1;
    s.tris = ctx->tris;
    s.n_tris = sc->n_triangles;
    s.alias = ctx->alias;
    s.n_alias = n_lights;
    s.pl_color = ctx->pl_color;
    s.n_point_lights = point ? n_lights : 0;
    s.tri_lights = ctx->tri_lights;
    s.tri_alias = ctx->tri_alias;
    s.n_tri_lights = point ? 0 : n_lights;
    s.materials = ctx->materials;
    s.n_materials = sc->n_materials;
    s.counters = ctx->counters;
    s.mma_timeouts = ctx->mma_timeouts;
    s.res_samples = ctx->res_samples;
    s.res_mis = ctx->res_mis;
    ctx->has_scene = true;
    ctx->vc_dirty = true;  // cached answers belong to the previous scene
    return RG_OK;
}

namespace {
// The cache buffers of the next ray pass over `pixels` pixels: reads what the
// previous ray pass wrote, writes the other buffer.  Entries hold whole
// segments, so a pass never takes an answer for another segment, whatever
// ran before it; the buffers are cleared after a scene upload.
int vcache_next(rg_context *ctx, size_t pixels, cudaStream_t st, VisCache *vc) {
    *vc = VisCache{};
    const size_t entries = pixels * (size_t)ctx->res_samples;
    if (!ctx->vc_on || entries == 0) return RG_OK;
    if (entries > ctx->vc_cap) {
        dev_free(ctx->vc_buf[0]);
        dev_free(ctx->vc_buf[1]);
        ctx->vc_cap = 0;
        cudaError_t e = dev_alloc(&ctx->vc_buf[0], 2 * entries);
        if (e == cudaSuccess) e = dev_alloc(&ctx->vc_buf[1], 2 * entries);
        if (e != cudaSuccess) {
            dev_free(ctx->vc_buf[0]);
            return cuda_fail(e, "visibility cache");
        }
        ctx->vc_cap = entries;
        ctx->vc_dirty = true;
    }
    if (ctx->vc_dirty) {
        for (int b = 0; b < 2; ++b) RG_CUDA(cudaMemsetAsync(ctx->vc_buf[b], 0, ctx->vc_cap * 32, st), "visibility cache");
        ctx->vc_dirty = false;
    }
    ctx->vc_tag = ctx->vc_tag >= 0x7fffffffu ? 1u : ctx->vc_tag + 1u;  // a reused tag is harmless: it only
                                                                       // pairs an entry's two halves
    vc->in = ctx->vc_buf[ctx->vc_cur];
    vc->out = ctx->vc_buf[1 - ctx->vc_cur];
    vc->tag = ctx->vc_tag;
    vc->n = (uint32_t)pixels;
    ctx->vc_cur = 1 - ctx->vc_cur;
    return RG_OK;
}
}  // namespace

int rg_set_visibility_cache(rg_context *ctx, int32_t enable) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (enable != 0 && enable != 1) return fail(RG_ERR_INVALID_ARGUMENT, "enable must be 0 or 1");
    if (enable && !ctx->vc_on) ctx->vc_dirty = true;
    ctx->vc_on = enable != 0;
    return RG_OK;
}

int rg_initial_temporal(rg_context *ctx, const rg_gbuffer *cur, const rg_gbuffer *prev,
                        const rg_reservoir *prev_res, rg_reservoir *out, const rg_restir_uniforms *u, void *stream) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    mlp::LearnedRis learned{};
    if (u && (u->flags & RG_FLAG_LEARNED_PROPOSAL) &&
        (rc = proposal_learned_ris(ctx->proposal, (int)u->screen_size[0], (int)u->screen_size[1], u->frame,
                                   u->initial_light_sample_count, &learned)))
        return rc;
    if (!u) return fail(RG_ERR_INVALID_ARGUMENT, "null uniforms");
    if ((rc = check_size(u->screen_size[0], u->screen_size[1]))) return rc;
    if ((rc = check_gbuffer(cur, u->screen_size[0], u->screen_size[1], "current G-buffer"))) return rc;
    if ((rc = check_res(out, "out"))) return rc;
    const bool temporal = (u->flags & RG_FLAG_TEMPORAL_REUSE) != 0;
    GBufView pv;
    if (temporal) {
        if ((rc = check_gbuffer(prev, u->screen_size[0], u->screen_size[1], "previous G-buffer"))) return rc;
        if ((rc = check_res(prev_res, "previous reservoirs"))) return rc;
        pv = make_view(prev);
    }
    const GBufView cv = make_view(cur);
    VisCache vc;
    if ((rc = vcache_next(ctx, (size_t)u->screen_size[0] * u->screen_size[1], (cudaStream_t)stream, &vc))) return rc;
    RG_CUDA(launch_initial_temporal(ctx->scene, cv, temporal ? &pv : nullptr, temporal ? prev_res : nullptr, out, *u,
                                    learned.cand ? &learned : nullptr, (cudaStream_t)stream, &vc),
            "k_initial_temporal");
    return RG_OK;
}

int rg_spatial_biased(rg_context *ctx, const rg_gbuffer *g, const rg_reservoir *in, rg_reservoir *out,
                      const rg_restir_uniforms *u, int32_t iter, void *stream) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (!u) return fail(RG_ERR_INVALID_ARGUMENT, "null uniforms");
    if ((rc = check_size(u->screen_size[0], u->screen_size[1]))) return rc;
    if ((rc = check_gbuffer(g, u->screen_size[0], u->screen_size[1], "G-buffer"))) return rc;
    if ((rc = check_res(in, "in")) || (rc = check_res(out, "out"))) return rc;
    if (in == out) return fail(RG_ERR_INVALID_ARGUMENT, "in and out must differ");
    RG_CUDA(launch_spatial_biased(ctx->scene, make_view(g), in, out, *u, iter, (cudaStream_t)stream), "k_spatial_biased");
    return RG_OK;
}

int rg_spatial_unbiased(rg_context *ctx, const rg_gbuffer *g, const rg_reservoir *in, rg_reservoir *out,
                        const rg_restir_uniforms *u, int32_t num_neighbors, int32_t pass_index, void *stream) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (!u) return fail(RG_ERR_INVALID_ARGUMENT, "null uniforms");
    if ((rc = check_size(u->screen_size[0], u->screen_size[1]))) return rc;
    if ((rc = check_gbuffer(g, u->screen_size[0], u->screen_size[1], "G-buffer"))) return rc;
    if ((rc = check_res(in, "in")) || (rc = check_res(out, "out"))) return rc;
    if (in == out) return fail(RG_ERR_INVALID_ARGUMENT, "in and out must differ");
    if (num_neighbors < 0 || num_neighbors > 16) return fail(RG_ERR_INVALID_ARGUMENT, "num_neighbors must be 0..16");
    VisCache vc;
    if ((rc = vcache_next(ctx, (size_t)u->screen_size[0] * u->screen_size[1], (cudaStream_t)stream, &vc))) return rc;
    RG_CUDA(launch_spatial_unbiased(ctx->scene, make_view(g), in, out, *u, num_neighbors, pass_index,
                                    (cudaStream_t)stream, &vc),
            "k_spatial_unbiased");
    return RG_OK;
}

int rg_shade(rg_context *ctx, const rg_gbuffer *g, const rg_reservoir *res, const rg_lighting_uniforms *u,
             float *rgba_out, void *stream) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (!u) return fail(RG_ERR_INVALID_ARGUMENT, "null uniforms");
    if ((rc = check_size(u->buffer_size[0], u->buffer_size[1]))) return rc;
    if ((rc = check_gbuffer(g, u->buffer_size[0], u->buffer_size[1], "G-buffer"))) return rc;
    if ((rc = check_res(res, "reservoirs"))) return rc;
    if (!rgba_out || ((uintptr_t)rgba_out & 15u)) return fail(RG_ERR_INVALID_ARGUMENT, "bad output image");
    if (u->debug_mode != 0) return fail(RG_ERR_UNSUPPORTED, "only GBUFFER_DEBUG_NONE is computed");
    if (!(u->gamma > 0.0f)) return fail(RG_ERR_INVALID_ARGUMENT, "gamma must be > 0");
    RG_CUDA(launch_shade(ctx->scene, make_view(g), res, *u, reinterpret_cast<float4 *>(rgba_out), (cudaStream_t)stream),
            "k_shade");
    return RG_OK;
}

int rg_visibility_batch(rg_context *ctx, const float *p1, const float *p2, uint8_t *out, int32_t n, void *stream) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (n < 0) return fail(RG_ERR_INVALID_ARGUMENT, "negative count");
    if (n == 0) return RG_OK;
    if (!p1 || !p2 || !out || ((uintptr_t)p1 & 15u) || ((uintptr_t)p2 & 15u))
        return fail(RG_ERR_INVALID_ARGUMENT, "bad pointers");
    RG_CUDA(launch_visibility_batch(ctx->scene, reinterpret_cast<const float4 *>(p1), reinterpret_cast<const float4 *>(p2),
                                    out, n, (cudaStream_t)stream),
            "k_visibility_batch");
    return RG_OK;
}

int rg_trace_gbuffer(rg_context *ctx, const rg_camera *cam, const rg_gbuffer_out *out, void *stream) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (!cam || !out) return fail(RG_ERR_INVALID_ARGUMENT, "null pointer");
    if ((rc = check_size((uint32_t)out->width, (uint32_t)out->height))) return rc;
    if (!out->albedo || !out->normal || !out->material || !out->world_pos || !out->depth)
        return fail(RG_ERR_INVALID_ARGUMENT, "null plane");
    if (((uintptr_t)out->normal & 7u) || ((uintptr_t)out->world_pos & 15u))
        return fail(RG_ERR_INVALID_ARGUMENT, "misaligned plane");
    RG_CUDA(launch_trace_gbuffer(ctx->scene, *cam, *out, (cudaStream_t)stream), "k_trace_gbuffer");
    return RG_OK;
}

static size_t reservoir_bytes(int samples, int mis) { return (size_t)samples * (mis ? 64 : 48) + 16; }

static int ensure_frame_buffers(rg_context *ctx, int w, int h, cudaStream_t st) {
    const size_t rb = reservoir_bytes(ctx->res_samples, ctx->res_mis);
    if (ctx->fw == w && ctx->fh == h && ctx->res[0] && ctx->frame_bytes == rb) return RG_OK;
    ctx->release_frame();
    const size_t np = (size_t)w * (size_t)h;
    const size_t units = (np * rb + sizeof(rg_reservoir) - 1) / sizeof(rg_reservoir);
    cudaError_t e = dev_alloc(&ctx->res[0], units);
    if (e == cudaSuccess) e = dev_alloc(&ctx->res[1], units);
    if (e == cudaSuccess) e = dev_alloc(&ctx->tmp, units);
    if (e == cudaSuccess) e = dev_alloc(&ctx->image, np);
    // zero-filled at creation, as the reference's fillBuffer (src/app.h:276,283)
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) e = cudaMemsetAsync(ctx->res[k], 0, np * rb, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx->tmp, 0, np * rb, st);
    if (e != cudaSuccess) {
        ctx->release_frame();
        return cuda_fail(e, "frame buffers");
    }
    ctx->fw = w;
    ctx->fh = h;
    ctx->frame_bytes = rb;
    return RG_OK;
}

int rg_set_reservoir_format(rg_context *ctx, int32_t samples, int32_t unbiased_mis) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if ((samples != 1 && samples != 2) || (unbiased_mis != 0 && unbiased_mis != 1))
        return fail(RG_ERR_INVALID_ARGUMENT, "reservoir format: samples 1 or 2, unbiased_mis 0 or 1");
    RG_CUDA(cudaDeviceSynchronize(), "rg_set_reservoir_format");
    ctx->res_samples = samples;
    ctx->res_mis = unbiased_mis;
    ctx->scene.res_samples = samples;
    ctx->scene.res_mis = unbiased_mis;
    return RG_OK;
}

int rg_set_tree_layout(rg_context *ctx, int32_t layout) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (layout != RG_TREE_BINARY && layout != RG_TREE_WIDE4 && layout != RG_TREE_QUANT4)
        return fail(RG_ERR_INVALID_ARGUMENT, "tree layout must be RG_TREE_BINARY, RG_TREE_WIDE4 or RG_TREE_QUANT4");
    ctx->tree_layout = layout;
    return RG_OK;
}

int rg_reservoir_bytes(rg_context *ctx) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    return (int)reservoir_bytes(ctx->res_samples, ctx->res_mis);
}

int rg_render_frame(rg_context *ctx, const rg_gbuffer *cur, const rg_gbuffer *prev, int32_t slot,
                    const rg_frame_params *fp, float *rgba_out, void *stream) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (!fp) return fail(RG_ERR_INVALID_ARGUMENT, "null params");
    if (slot != 0 && slot != 1) return fail(RG_ERR_INVALID_ARGUMENT, "frame_slot must be 0 or 1");
    const rg_restir_uniforms &u = fp->uniforms;
    if ((rc = check_size(u.screen_size[0], u.screen_size[1]))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    if ((rc = ensure_frame_buffers(ctx, (int)u.screen_size[0], (int)u.screen_size[1], st))) return rc;
    rg_reservoir *cur_res = ctx->res[slot], *prev_res = ctx->res[1 - slot];
    const int passes = fp->spatial_iterations < 0 ? 0 : fp->spatial_iterations;
    if ((u.flags & RG_FLAG_LEARNED_PROPOSAL) && (rc = rg_proposal_infer(ctx, cur, &u, stream))) return rc;
    // src/app.h:212-262 and :297-334
    if (fp->unbiased) {
        // RIS -> temporary, then `passes` unbiased passes ending in the frame buffer.
        rg_reservoir *first = (passes % 2 == 1 || passes == 0) ? ctx->tmp : cur_res;
        if (passes == 0) first = cur_res;
        if ((rc = rg_initial_temporal(ctx, cur, prev, prev_res, first, &u, stream))) return rc;
        rg_reservoir *src = first;
        for (int k = 0; k < passes; ++k) {
            rg_reservoir *dst = (src == ctx->tmp) ? cur_res : ctx->tmp;
            if ((rc = rg_spatial_unbiased(ctx, cur, src, dst, &u, fp->unbiased_neighbors, k, stream))) return rc;
            src = dst;
        }
    } else {
        if ((rc = rg_initial_temporal(ctx, cur, prev, prev_res, cur_res, &u, stream))) return rc;
        for (int j = 0; j < passes; ++j) {
            if ((rc = rg_spatial_biased(ctx, cur, cur_res, prev_res, &u, 2 * j, stream))) return rc;
            if ((rc = rg_spatial_biased(ctx, cur, prev_res, cur_res, &u, 2 * j + 1, stream))) return rc;
        }
    }
    rg_lighting_uniforms lu;
    memset(&lu, 0, sizeof(lu));
    memcpy(lu.camera_pos, u.camera_pos, sizeof(lu.camera_pos));
    lu.buffer_size[0] = u.screen_size[0];
    lu.buffer_size[1] = u.screen_size[1];
    lu.debug_mode = 0;
    lu.gamma = fp->gamma > 0.0f ? fp->gamma : 1.0f;
    float *img = rgba_out ? rgba_out : reinterpret_cast<float *>(ctx->image);
    if ((rc = rg_shade(ctx, cur, cur_res, &lu, img, stream))) return rc;
    if ((u.flags & RG_FLAG_LEARNED_TRAIN) && (rc = rg_proposal_train(ctx, cur, &u, cur_res, stream))) return rc;
    return RG_OK;
}

int rg_frame_reservoirs(rg_context *ctx, int32_t slot, const rg_reservoir **out) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (!out || (slot != 0 && slot != 1)) return fail(RG_ERR_INVALID_ARGUMENT, "bad arguments");
    if (!ctx->res[slot]) return fail(RG_ERR_INVALID_ARGUMENT, "no frame rendered yet");
    *out = ctx->res[slot];
    return RG_OK;
}

int rg_render_frame_host(rg_context *ctx, int32_t w, int32_t h, const uint8_t *albedo, const uint16_t *normal,
                         const uint16_t *material, const float *world_pos, const float *depth,
                         const rg_frame_params *fp, float *rgba_out_host, void *stream) {
    int rc = check_ctx(ctx, true);
    if (rc) return rc;
    if (!fp || !albedo || !normal || !material || !world_pos || !depth || !rgba_out_host)
        return fail(RG_ERR_INVALID_ARGUMENT, "null pointer");
    if ((uint32_t)w != fp->uniforms.screen_size[0] || (uint32_t)h != fp->uniforms.screen_size[1])
        return fail(RG_ERR_INVALID_ARGUMENT, "image size does not match uniforms");
    if ((rc = check_size((uint32_t)w, (uint32_t)h))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    if ((rc = ensure_frame_buffers(ctx, w, h, st))) return rc;
    const size_t np = (size_t)w * (size_t)h;
    // G-buffer slots alternate like the reference's two GBuffers (src/app.h:116).
    const int slot = (int)(fp->uniforms.frame & 1u);
    GBufSlot &g = ctx->gslot[slot];
    if (g.w != w || g.h != h) {
        g.release();
        cudaError_t e = dev_alloc(&g.albedo, np);
        if (e == cudaSuccess) e = dev_alloc(&g.normal, np);
        if (e == cudaSuccess) e = dev_alloc(&g.material, np);
        if (e == cudaSuccess) e = dev_alloc(&g.wpos, np);
        if (e == cudaSuccess) e = dev_alloc(&g.depth, np);
        if (e != cudaSuccess) { g.release(); return cuda_fail(e, "G-buffer slot"); }
        g.w = w;
        g.h = h;
        ctx->gslot_valid[slot] = false;
    }
    RG_CUDA(cudaMemcpyAsync(g.albedo, albedo, np * 4, cudaMemcpyHostToDevice, st), "H2D albedo");
    RG_CUDA(cudaMemcpyAsync(g.normal, normal, np * 8, cudaMemcpyHostToDevice, st), "H2D normal");
    RG_CUDA(cudaMemcpyAsync(g.material, material, np * 4, cudaMemcpyHostToDevice, st), "H2D material");
    RG_CUDA(cudaMemcpyAsync(g.wpos, world_pos, np * 16, cudaMemcpyHostToDevice, st), "H2D world_pos");
    RG_CUDA(cudaMemcpyAsync(g.depth, depth, np * 4, cudaMemcpyHostToDevice, st), "H2D depth");
    ctx->gslot_valid[slot] = true;
    const rg_gbuffer cur = g.view();
    const bool have_prev = ctx->gslot_valid[1 - slot] && ctx->gslot[1 - slot].w == w && ctx->gslot[1 - slot].h == h;
    rg_frame_params p = *fp;
    if (!have_prev) p.uniforms.flags &= ~RG_FLAG_TEMPORAL_REUSE;
    const rg_gbuffer prev = have_prev ? ctx->gslot[1 - slot].view() : cur;
    if ((rc = rg_render_frame(ctx, &cur, &prev, slot, &p, reinterpret_cast<float *>(ctx->image), stream))) return rc;
    RG_CUDA(cudaMemcpyAsync(rgba_out_host, ctx->image, np * 16, cudaMemcpyDeviceToHost, st), "D2H image");
    RG_CUDA(cudaStreamSynchronize(st), "rg_render_frame_host");
    return RG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- internal accessors
// For entry points defined in other translation units (noalloc.cu): the
// per-thread error message and the uploaded scene of a context.
int rg_internal_fail(int code, const char *msg) { return fail(code, "%s", msg); }

bool rg_internal_vcache_on(rg_context *ctx) { return ctx->vc_on; }

ProposalState **rg_internal_proposal(rg_context *ctx) {
    cudaSetDevice(ctx->device);
    return &ctx->proposal;
}

int rg_internal_device(rg_context *ctx, int *device) {
    const int rc = check_ctx(ctx, false);
    if (rc) return rc;
    *device = ctx->device;
    return RG_OK;
}

int rg_internal_prepare(rg_context *ctx, const DevScene **scene, int *device) {
    const int rc = check_ctx(ctx, true);
    if (rc) return rc;
    *scene = &ctx->scene;
    *device = ctx->device;
    return RG_OK;
}

int rg_internal_check_spatial_args(const rg_gbuffer *g, const void *in, const void *out,
                                   const rg_restir_uniforms *u) {
    if (!u) return fail(RG_ERR_INVALID_ARGUMENT, "null uniforms");
    int rc = check_size(u->screen_size[0], u->screen_size[1]);
    if (rc) return rc;
    if ((rc = check_gbuffer(g, u->screen_size[0], u->screen_size[1], "G-buffer"))) return rc;
    if ((rc = check_res(in, "in")) || (rc = check_res(out, "out"))) return rc;
    if (in == out) return fail(RG_ERR_INVALID_ARGUMENT, "in and out must differ");
    return RG_OK;
}

extern "C" int rg_gemm_bf16(rg_context *ctx, const void *a, int32_t a_fp32, int64_t a_row_stride, int64_t a_k_stride,
                            int32_t m, const void *b, int32_t b_fp32, int64_t b_row_stride, int64_t b_k_stride,
                            int32_t n, int32_t k, float *d, int64_t ldd, int32_t accumulate, float alpha,
                            int32_t k_splits, void *stream) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (!a || !b || !d || m <= 0 || n <= 0 || k <= 0 || ldd < n)
        return fail(RG_ERR_INVALID_ARGUMENT, "rg_gemm_bf16: bad arguments");
    RG_CUDA(launch_gemm_tc(a, a_fp32, a_row_stride, a_k_stride, m, b, b_fp32, b_row_stride, b_k_stride, n, k, d, ldd,
                           accumulate, alpha, k_splits, ctx->mma_timeouts, (cudaStream_t)stream),
            "k_gemm_tc");
    return RG_OK;
}
