// rg_internal.h -- device-side scene layout and kernel launch interface.
//
// The reference's buffers are repacked once at upload into layouts a GB300
// reads with 128-bit loads; the repacking copies values, it never recomputes
// them, so every test the kernels evaluate sees the reference's floats.
//   GNode      64 B: both child boxes (interleaved per axis) + child links
//              of one AabbTreeNode (80 B in the reference: the vec4 w lanes
//              are dropped).
//   GTri       48 B: p1, e1 = p2-p1, e2 = p3-p1 (the same subtractions the
//              reference's rayTriangleIntersection performs per test).
//   AliasLight 48 B: one alias-table column plus the position/luminance of
//              both lights it can return, so a candidate is one gather.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/restir_gb300.h"

struct GNode {
    float4 a;  // lmin.x rmin.x lmax.x rmax.x  (per axis, so that a pair of lanes
    float4 b;  // lmin.y rmin.y lmax.y rmax.y   holds the same bound of both
    float4 c;  // lmin.z rmin.z lmax.z rmax.z   children: packed FP32x2 slab math)
    int4 d;    // left right 0 0
};
struct GTri {
    float4 a;  // p1.xyz e1.x
    float4 b;  // e1.y e1.z e2.x e2.y
    float4 c;  // e2.z 0 0 0
};
struct AliasLight {
    float4 col;        // prob, alias (int bits), ori_prob, alias_ori_prob
    float4 own_pos;    // light[column].pos.xyz, luminance
    float4 alias_pos;  // light[alias].pos.xyz, luminance
};

// WNode 128 B: the 4-wide copy of the tree (host_pack_wide) walked by shadow
// rays on the filtered fast path; the first 64 bytes have GNode's layout
// (children 0 and 1, then the links of all four children), so one walk reads
// both copies.  Links: >= 0 node, < 0 triangle ~t, kWideNoChild = empty.
struct WNode {
    float4 a, b, c;   // children 0, 1: per axis lo0 lo1 hi0 hi1
    int4 d;           // links of children 0..3
    float4 e, f, g;   // children 2, 3 as a, b, c
    float4 pad;
};
constexpr int32_t kWideNoChild = INT32_MIN;

// QNode 64 B: the quantized 4-wide copy (host_pack_quant).  Per axis a base
// c and a power of two s (biased exponent bytes in base.w); child k's bounds
// are byte k of the axis' lower and upper code words, code q decoding to
// RN((2^23 + q) * s + c), a box containing the child's exact box.  Links:
// >= 0 node, < 0 leaf record ~r, kWideNoChild = empty.
struct QNode {
    float4 base; // c.xyz, exponent bytes (x, y, z) and slot masks (leaf bits 0-3, inner bits 4-7)
    uint4 qxy;   // lo x, hi x, lo y, hi y (byte k: child k)
    uint4 qz;    // lo z, hi z, s of x, s of y (float bits)
    int4 d;      // links of children 0..3
};
// QLeaf 64 B: a leaf of the quantized copy, the triangle's exact box from
// the reference's tree and the triangle in GTri form.
struct QLeaf {
    float4 a;  // lo.xyz hi.x
    float4 b;  // hi.y hi.z p1.x p1.y
    float4 c;  // p1.z e1.xyz
    float4 d;  // e2.xyz 0
};

struct DevScene {
    const GNode *nodes;
    int32_t n_nodes;
    int32_t depth;                // validated tree depth (root = 1): traversal stack size
    int32_t box_nan;              // some node box coordinate is NaN: shadow rays use exact slab tests only
    const WNode *wide;            // 4-wide copy, or null (containment failed, NaN boxes, too deep)
    int32_t n_wide;
    int32_t wide_stack;           // stack entries the 4-wide walk may need (3 per level)
    const QNode *qnodes;          // quantized 4-wide copy, or null (not nested, NaN or huge boxes, too deep)
    const QLeaf *qleaves;
    int32_t n_qnodes;
    const GTri *tris;
    int32_t n_tris;
    const AliasLight *alias;      // point-light scenes
    int32_t n_alias;
    const float4 *pl_color;       // point light color_luminance
    int32_t n_point_lights;
    const rg_tri_light *tri_lights;
    const rg_alias_table_column *tri_alias;  // triangle-light scenes
    int32_t n_tri_lights;
    const rg_material *materials;
    int32_t n_materials;
    unsigned long long *counters; // [0] rays traced, [1] traversal errors, [2] node visits, [3] triangle tests
    int *mma_timeouts;            // tensor-core kernels whose bounded mbarrier wait ran out
    int32_t res_samples;          // reservoir format: RESERVOIR_SIZE (1 or 2)
    int32_t res_mis;              // and UNBIASED_MIS (0 or 1)
};

// G-buffer planes with their formats (rg_gbuffer's VkFormat numbers, 0 =
// default).  The typed pointers are the default layouts; the loaders in
// kernels.cu reinterpret them for the other formats.
struct GBufView {
    int32_t w, h;
    const uint32_t *albedo;  // RGBA8
    const uint2 *normal;     // RGBA16F (nfmt 0)
    const uint32_t *material;// RG16
    const float4 *wpos;      // RGBA32F (pfmt 0)
    const float *depth;      // D32F (dfmt 0)
    int32_t nfmt, pfmt, dfmt;
};
// True when every plane of g is in the default layout.
inline bool default_formats(const GBufView &g) { return g.nfmt == 0 && g.pfmt == 0 && g.dfmt == 0; }

// Answers of the pixels' own visibility segments (a pixel's world position
// to its sample's light position) kept between ray passes, keyed by the
// segment's end points: an entry is two float4, (start.xyz, tag) and
// (end.xyz, 2 * tag + shadowed), tag 0 = empty, one entry per (sample slot,
// pixel).  A pass reads the entries the previous ray pass wrote (`in`) and
// writes its own (`out`, another buffer); a segment whose end points equal
// an entry's bit for bit has that entry's answer (the answer depends on the
// scene and the two points only).  Null pointers: no cache.
struct VisCache {
    const float4 *in = nullptr;
    float4 *out = nullptr;
    uint32_t tag = 0;     // this launch's tag, 1 .. 2^31 - 1
    uint32_t n = 0;       // entries per sample slot (the pass's pixel count)
};

GBufView make_view(const rg_gbuffer *g);

// launchers (kernels.cu); return cudaGetLastError()
namespace mlp { struct LearnedRis; struct ProposalDev; }
cudaError_t launch_initial_temporal(const DevScene &s, const GBufView &cur, const GBufView *prev,
                                    const rg_reservoir *prev_res, rg_reservoir *out, const rg_restir_uniforms &u,
                                    const mlp::LearnedRis *learned, cudaStream_t st, const VisCache *vc = nullptr);
cudaError_t launch_spatial_biased(const DevScene &s, const GBufView &g, const rg_reservoir *in, rg_reservoir *out,
                                  const rg_restir_uniforms &u, int iter, cudaStream_t st);
cudaError_t launch_spatial_unbiased(const DevScene &s, const GBufView &g, const rg_reservoir *in, rg_reservoir *out,
                                    const rg_restir_uniforms &u, int num_neighbors, int pass_index, cudaStream_t st,
                                    const VisCache *vc = nullptr);
cudaError_t launch_shade(const DevScene &s, const GBufView &g, const rg_reservoir *res, const rg_lighting_uniforms &u,
                         float4 *out, cudaStream_t st);
cudaError_t launch_visibility_batch(const DevScene &s, const float4 *p1, const float4 *p2, uint8_t *out, int n,
                                    cudaStream_t st);
cudaError_t launch_trace_gbuffer(const DevScene &s, const rg_camera &cam, const rg_gbuffer_out &out, cudaStream_t st);
cudaError_t upload_srgb_lut(const float *lut256);
cudaError_t launch_gemm_tc(const void *a, int a_fp32, int64_t a_rs, int64_t a_ks, int m, const void *b, int b_fp32,
                           int64_t b_rs, int64_t b_ks, int n, int k, float *d, int64_t ldd, int accumulate,
                           float alpha, int splits, int *err, cudaStream_t st);

// host helpers (host_bvh.cpp, host_alias.cpp, host_gbuffer.cpp)
void srgb_lut_host(float *out256);

// ---- many views per launch (kernels.cu); kind 0: RIS + visibility + temporal,
// 1: spatial pass, 2: shading.  A parameter record is the single-view kernel's
// parameter block for one view.
struct ViewTiles {
    const int32_t *view_start;  // first tile of each view in the launch's tile order
    const int32_t *tiles_x;     // tiles per row of each view
    int32_t n_views;
    int32_t total;              // tiles of all views
    unsigned *counter;          // zero before the launch
};
size_t view_params_size(int kind);
void make_initial_params(void *dst, const DevScene &s, const GBufView &cur, const GBufView *prev,
                         const rg_reservoir *prev_res, rg_reservoir *out, const rg_restir_uniforms &u,
                         const mlp::LearnedRis *learned, const VisCache *vc = nullptr);
void make_spatial_params(void *dst, const DevScene &s, const GBufView &g, const rg_reservoir *in, rg_reservoir *out,
                         const rg_restir_uniforms &u, bool unbiased, int iter_or_pass, int num_neighbors,
                         const VisCache *vc = nullptr);
void make_shade_params(void *dst, const DevScene &s, const GBufView &g, const rg_reservoir *res,
                       const rg_lighting_uniforms &u, float4 *out);
// tile of pass `kind` for tuning variant `variant` (RIS: pixels per thread 1/2/4;
// unbiased spatial: tile width 8/16/32; others: 32 x 4)
void view_tile_shape(int kind, int variant, int *tw, int *th);
// Persistent grid of a pass (sets the kernel's shared-memory attribute; call
// before any stream capture), then the launch itself (stream work only).
cudaError_t views_pass_grid(int kind, int variant, bool unbiased, int num_neighbors, int depth, int total,
                            int ctas_per_sm, int *grid);
cudaError_t launch_views_pass(int kind, int variant, bool unbiased, int num_neighbors, int depth, const void *params,
                              const ViewTiles &vt, int grid, cudaStream_t st);
// Candidate-count tuning: every view's RIS candidate count; the luminance of
// the views' shaded images (mode 0: into lum at first_px[v] + pixel; mode 1:
// acc[0] += sum of squared differences to lum, acc[1] += pixels counted),
// over the shading tile map (counter zeroed before the launch).
cudaError_t launch_set_candidates(void *initial_params, int n_views, uint32_t count, cudaStream_t st);
cudaError_t launch_views_luminance(const void *shade_params, const ViewTiles &vt, const long long *first_px, float *lum,
                                   int mode, double *acc, int grid, cudaStream_t st);
// Sets every view's frame index to start_frame[v] + *runs (also into
// frame_out[v] when frame_out is not null), then adds one to *runs.
cudaError_t launch_advance_frames(void *initial_params, void *spatial_params, int n_views, int n_spatial,
                                  const uint32_t *start_frame, uint32_t *runs, uint32_t *frame_out, cudaStream_t st);

// capi.cu: error reporting and context access for other translation units.
int rg_internal_fail(int code, const char *msg);
int rg_internal_prepare(rg_context *ctx, const DevScene **scene, int *device);
// A valid context (no scene needed); makes its device current.
int rg_internal_device(rg_context *ctx, int *device);
// The argument checks of rg_spatial_unbiased (frame size, every G-buffer
// plane present and aligned for the kernels' loads, reservoir buffers
// present, 16-byte aligned and distinct), for entry points that launch the
// same kernel.
int rg_internal_check_spatial_args(const rg_gbuffer *g, const void *in, const void *out,
                                   const rg_restir_uniforms *u);
// noalloc.cu: forget the cached device address of the allocation-free
// chain's scratch array on `device` (a new context may follow a reset of the
// device's primary context, which unloads the module holding the array).
void noalloc_forget_device(int device);

// gpu_bvh.cu: the reference tree built on the device (node count, or < 0).
int gpu_build_bvh(const float *xyz, int n, rg_aabb_tree_node *nodes, rg_triangle *tris, int *undefined,
                  cudaStream_t st);

// proposal.cu: the learned proposal attached to a context.
struct ProposalState;
ProposalState **rg_internal_proposal(rg_context *ctx);
// Whether the context's visibility cache is on (rg_set_visibility_cache).
bool rg_internal_vcache_on(rg_context *ctx);
void proposal_release(ProposalState *ps);
// Learned RIS inputs for a frame of w x h with `count` candidates, or an
// RG_ERR_* code when the context's candidates do not match that frame.
int proposal_learned_ris(ProposalState *ps, int w, int h, uint32_t frame, uint32_t count, mlp::LearnedRis *out);
// The network and the learned RIS tables (cand left null) for batched views,
// and the proposal's identity: a number no other proposal of the process has.
uint64_t proposal_batch_tables(ProposalState *ps, mlp::ProposalDev *dev, mlp::LearnedRis *out);
