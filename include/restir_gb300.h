/*
 * restir_gb300.h -- C ABI of the GB300-native ReSTIR direct-lighting path.
 *
 * Drop-in for the compute half of ReSTIR-Vulkan's per-frame pass sequence
 * (reference paths relative to the reference project root):
 *
 *   reference pass (Pass::issueCommands, src/passes/pass.h:103)     entry point here
 *   ------------------------------------------------------------    -------------------------
 *   RestirPass          src/passes/restirPass.h:36-62               rg_initial_temporal
 *     -> src/shaders/restirOmni.glsl:86-212 (software RT variant)
 *   SpatialReusePass    src/passes/spatialReusePass.h:11-26         rg_spatial_biased
 *     -> src/shaders/spatialReuse.comp:30-86
 *   UnbiasedReusePass   src/passes/unbiasedReusePass.h:23-49        rg_spatial_unbiased
 *     -> src/shaders/unbiasedReuse.glsl:50-185
 *   LightingPass        src/passes/lightingPass.h:14-42             rg_shade
 *     -> src/shaders/lighting.frag:43-71,103 (GBUFFER_DEBUG_NONE)
 *   testVisibility      src/shaders/include/visibilityTest.glsl:26  rg_visibility_batch
 *   App::_recordMainCommandBuffers  src/app.h:212-262 (+ buffer     rg_render_frame
 *     wiring src/app.h:264-336, per-frame uniforms src/app.cpp:775-826)
 *   host preprocessing:
 *   AabbTree::build     src/aabbTreeBuilder.cpp:52-214              rg_build_bvh
 *   createAliasTable    src/misc.cpp:418-497                        rg_build_alias_table
 *   SceneBuffers / AabbTreeBuffers upload (sceneBuffers.h:71-273,   rg_upload_scene
 *     aabbTreeBuilder.h:25-51)
 *
 * Conventions
 *  - Every call returns RG_OK (0) or a negative RG_ERR_* code; nothing throws
 *    across the ABI and nothing aborts.  rg_last_error() gives the message of
 *    the last failure on the calling thread.
 *  - Pass entry points take DEVICE pointers owned by the caller and launch on
 *    the given CUDA stream (a cudaStream_t passed as void*; NULL = legacy
 *    default stream).  They return once the work is enqueued and allocate
 *    nothing.  Uniform structs are read on the host at call time.
 *  - Byte layouts of rg_reservoir, rg_aabb_tree_node, rg_triangle,
 *    rg_point_light, rg_tri_light, rg_alias_table_column, rg_restir_uniforms
 *    and rg_lighting_uniforms are the reference's std430/std140 layouts
 *    (src/shaderIncludes.h; src/shaders/include/structs/).
 *  - G-buffer planes are the reference's attachment formats
 *    (src/passes/gBufferPass.cpp:75-108) stored as linear row-major buffers.
 *  - A context is thread-compatible: one host thread at a time.
 */
#ifndef RESTIR_GB300_H
#define RESTIR_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RG_OK 0
#define RG_ERR_INVALID_ARGUMENT (-1)
#define RG_ERR_CUDA (-2)
#define RG_ERR_OUT_OF_MEMORY (-3)
#define RG_ERR_NO_SCENE (-4)
#define RG_ERR_TREE_TOO_DEEP (-5)
#define RG_ERR_UNSUPPORTED (-6)
#define RG_ERR_TRAVERSAL (-7)

#define RG_FLAG_VISIBILITY_REUSE 1 /* RESTIR_VISIBILITY_REUSE_FLAG, restirStructs.glsl:37 */
#define RG_FLAG_TEMPORAL_REUSE 2   /* RESTIR_TEMPORAL_REUSE_FLAG, restirStructs.glsl:38 */
/* Extension (not in the reference, off by default): after the RIS candidate
 * loop set W = sumWeights / (M * pHat), the standard RIS weight, instead of
 * keeping the value stored when the sample was selected
 * (reservoir.glsl:33-40 never refreshes it), which biases RIS upwards. */
#define RG_FLAG_FINAL_RIS_WEIGHT 256
/* Extensions of the learned light-cluster proposal (no reference counterpart):
 * LEARNED_PROPOSAL draws the initial RIS candidates from the context's
 * proposal (rg_proposal_create) instead of the alias table; in
 * rg_render_frame it also runs the proposal's inference for the frame, and
 * LEARNED_TRAIN adds one training step on the frame's final reservoirs. */
#define RG_FLAG_LEARNED_PROPOSAL 512
#define RG_FLAG_LEARNED_TRAIN 1024
/* Extension for the UNBIASED_MIS format (off by default): combineReservoirs
 * passes the merged sample's (w, sumPHat) in the order updateReservoirAt
 * declares them; the reference passes them swapped (reservoir.glsl:55-60),
 * which is what the passes do without this flag. */
#define RG_FLAG_MIS_SWAP_FIX 2048

/* Deepest BVH the traversal accepts: its stack holds depth+1 entries. */
#define RG_MAX_TREE_DEPTH 63

typedef struct rg_context rg_context;

/* Reservoir with RESERVOIR_SIZE 1 (restirStructs.glsl:19-34): 64 bytes. */
typedef struct rg_reservoir {
    float position_emission_lum[4]; /* sample position, w = emission luminance */
    float normal[4];                /* light normal; w > 0.5 => triangle light */
    int32_t light_index;            /* >= 0 point light, < 0: triangle light -1-i */
    float p_hat;
    float sum_weights;
    float w;
    uint32_t num_stream_samples;    /* M */
    uint32_t _pad[3];
} rg_reservoir;

/* AabbTreeNode (structs/aabbTree.glsl:1-8): 80 bytes.  A child < 0 is the
 * triangle ~child; the root is node 0. */
typedef struct rg_aabb_tree_node {
    float left_aabb_min[4], left_aabb_max[4];
    float right_aabb_min[4], right_aabb_max[4];
    int32_t left_child, right_child;
    int32_t _pad[2];
} rg_aabb_tree_node;

typedef struct rg_triangle { float p1[4], p2[4], p3[4]; } rg_triangle;                 /* 48 B */
typedef struct rg_point_light { float pos[4]; float color_luminance[4]; } rg_point_light; /* 32 B */
typedef struct rg_tri_light {                                                           /* 80 B */
    float p1[4], p2[4], p3[4];
    float emission_luminance[4];
    float normal_area[4];
} rg_tri_light;
typedef struct rg_alias_table_column { float prob; int32_t alias; float ori_prob; float alias_ori_prob; } rg_alias_table_column; /* 16 B */

/* RestirUniforms (restirStructs.glsl:40-56), std140: 128 bytes. */
typedef struct rg_restir_uniforms {
    float prev_frame_projection_view[16]; /* column-major */
    float camera_pos[4];
    uint32_t screen_size[2];
    uint32_t frame;
    uint32_t initial_light_sample_count;
    uint32_t temporal_sample_count_multiplier;
    float spatial_pos_threshold;
    float spatial_normal_threshold;       /* degrees */
    uint32_t spatial_neighbors;
    float spatial_radius;
    int32_t flags;
    uint32_t _pad[2];
} rg_restir_uniforms;

/* LightingPassUniforms (structs/lightingPassStructs.glsl:1-7): 96 bytes. */
typedef struct rg_lighting_uniforms {
    float prev_frame_projection_view[16];
    float camera_pos[4];
    uint32_t buffer_size[2];
    int32_t debug_mode;                   /* only GBUFFER_DEBUG_NONE (0) is computed */
    float gamma;
} rg_lighting_uniforms;

/* G-buffer attachment formats.  The reference takes the first format the
 * device supports from a list per attachment (GBuffer::Formats::initialize,
 * src/passes/gBufferPass.cpp:75-101); the values here are the VkFormat
 * numbers of those candidates, so a host passes what it selected.  0 (the
 * default) is the headless layout: RGBA16F normals, RGBA32F positions, D32F
 * depth.  Texels are tightly packed in each plane (a 3-component 16-bit
 * normal takes 6 bytes).  Decoding: SNORM16 c -> max(c / 32767, -1) (Vulkan's
 * normalized fixed-point rule, IEEE division), half and float exactly, the
 * D24 depth of D24_UNORM_S8_UINT from the low 24 bits of each 32-bit word
 * (d / 16777215, the stencil byte above it ignored); D32_SFLOAT_S8_UINT's
 * depth plane is plain float (its stencil lives in a plane of its own, which
 * no pass reads). */
#define RG_FORMAT_DEFAULT 0
#define RG_FORMAT_R16G16B16_SNORM 85
#define RG_FORMAT_R16G16B16_SFLOAT 90
#define RG_FORMAT_R16G16B16A16_SNORM 92
#define RG_FORMAT_R16G16B16A16_SFLOAT 97
#define RG_FORMAT_R32G32B32_SFLOAT 106
#define RG_FORMAT_R32G32B32A32_SFLOAT 109
#define RG_FORMAT_D32_SFLOAT 126
#define RG_FORMAT_D24_UNORM_S8_UINT 129
#define RG_FORMAT_D32_SFLOAT_S8_UINT 130

/* G-buffer planes (device pointers), width*height texels each, row-major. */
typedef struct rg_gbuffer {
    int32_t width, height;
    const void *albedo;     /* R8G8B8A8_SRGB: sRGB-encoded rgb, alpha 255 = emissive */
    const void *normal;     /* normal_format (default R16G16B16A16_SFLOAT) */
    const void *material;   /* R16G16_UNORM: roughness, metallic */
    const void *world_pos;  /* world_pos_format (default R32G32B32A32_SFLOAT) */
    const void *depth;      /* depth_format (default D32_SFLOAT): projected z/w */
    int32_t normal_format;     /* 0, R16G16B16_SNORM, R16G16B16_SFLOAT, R16G16B16A16_SNORM,
                                  R16G16B16A16_SFLOAT or R32G32B32_SFLOAT (gBufferPass.cpp:81-89) */
    int32_t world_pos_format;  /* 0, R32G32B32_SFLOAT or R32G32B32A32_SFLOAT (:98-101) */
    int32_t depth_format;      /* 0, D32_SFLOAT, D32_SFLOAT_S8_UINT or D24_UNORM_S8_UINT (:90-93) */
    int32_t _reserved;         /* 0 */
} rg_gbuffer;

/* Writable G-buffer planes, for rg_trace_gbuffer (default formats). */
typedef struct rg_gbuffer_out {
    int32_t width, height;
    void *albedo, *normal, *material, *world_pos, *depth;
} rg_gbuffer_out;

/* Per-triangle surface, indexed like the triangle buffer. */
typedef struct rg_material {
    uint8_t albedo_srgb[4];   /* rgb sRGB-encoded; a = 255 for emissive surfaces */
    uint16_t roughness_unorm; /* 0..65535 */
    uint16_t metallic_unorm;
} rg_material;

/* Pinhole camera in the reference's convention (src/camera.h:25-50). */
typedef struct rg_camera {
    float position[3];
    float right[3];           /* unitRight */
    float up[3];              /* unitUp (view y is -up) */
    float forward[3];         /* unitForward */
    float tan_half_fov_y;     /* 1/f */
    float aspect;             /* width / height */
    float projection_view[16];/* column-major P*V of this camera (depth output) */
} rg_camera;

/* Host-side scene as the reference uploads it. */
typedef struct rg_scene_desc {
    const rg_aabb_tree_node *nodes; int32_t n_nodes;
    const rg_triangle *triangles; int32_t n_triangles;
    const rg_point_light *point_lights; int32_t n_point_lights;
    const rg_tri_light *tri_lights; int32_t n_tri_lights;
    const rg_alias_table_column *alias_table; int32_t n_alias; /* one column per light */
    const rg_material *materials; int32_t n_materials;        /* optional: per triangle, for rg_trace_gbuffer */
} rg_scene_desc;

/* Frame parameters for the driver (App state, src/app.h:150-174). */
typedef struct rg_frame_params {
    rg_restir_uniforms uniforms;     /* frame, flags, counts, thresholds, camera */
    int32_t unbiased;                /* 1: UnbiasedReusePass, 0: SpatialReusePass pairs */
    int32_t spatial_iterations;      /* biased: iterations (2 dispatches each); unbiased: passes */
    int32_t unbiased_neighbors;      /* NUM_NEIGHBORS (reference: 3) */
    float gamma;
} rg_frame_params;

typedef struct rg_stats {
    uint64_t rays_traced;            /* shadow segments traced since the last reset */
    uint64_t traversal_errors;       /* traversals that hit the iteration limit */
    uint64_t node_visits;            /* tree nodes visited by those segments */
    uint64_t triangle_tests;         /* triangle tests made by those segments */
    uint64_t mma_timeouts;           /* tensor-core launches whose bounded completion wait ran out */
    uint64_t wide_nodes;             /* nodes of the uploaded tree's 4-wide copy, exact or quantized (0: not
                                        built, every ray walks the binary tree) */
    uint64_t tree_layout;            /* the layout shadow rays of the uploaded scene walk (RG_TREE_*) */
} rg_stats;

/* ---- context ---- */
int rg_create(int32_t device, rg_context **out);
int rg_destroy(rg_context *ctx);
const char *rg_last_error(void);
int rg_get_stats(rg_context *ctx, rg_stats *out, int32_t reset);

/* ---- host preprocessing (no GPU needed) ---- */
/* AabbTree::build on a flat list of n_tris triangles (9 floats each).  Writes
 * n_tris-1 nodes and n_tris triangles; returns the node count or an error. */
int rg_build_bvh(const float *tri_xyz, int32_t n_tris, rg_aabb_tree_node *out_nodes, rg_triangle *out_tris);
/* The same tree built on the GPU from device buffers: tri_xyz (9 floats per
 * triangle) in, n_tris-1 nodes and n_tris triangles out (device), with
 * contents byte-identical to rg_build_bvh's.  Synchronous on `stream`;
 * returns the node count; *ref_undefined (host, may be null) is set when a
 * range took a path the reference leaves undefined (see rg_build_bvh).
 * At most 4,194,304 triangles; coordinates must be finite.  No counterpart
 * in the reference, which builds on the host (aabbTreeBuilder.cpp:52-214). */
int rg_build_bvh_device(rg_context *ctx, const float *tri_xyz, int32_t n_tris, rg_aabb_tree_node *nodes,
                        rg_triangle *triangles, int32_t *ref_undefined, void *stream);
/* Depth of the tree (root = 1). */
int rg_tree_depth(const rg_aabb_tree_node *nodes, int32_t n_nodes);
/* The same tree with its nodes renumbered in depth-first preorder (root 0,
 * each node's left subtree right after it, then its right subtree); child
 * links remapped, leaves (~triangle index) unchanged, boxes copied bit for
 * bit.  rg_upload_scene keeps its device copy of the tree in this order, so
 * a left-first walk mostly steps to the next node in memory; traversal
 * results do not depend on the numbering.  No counterpart in the reference,
 * whose builder numbers nodes breadth first (aabbTreeBuilder.cpp:52-214).
 * Returns n_nodes or an error (malformed tree). */
int rg_tree_preorder(const rg_aabb_tree_node *nodes, int32_t n_nodes, rg_aabb_tree_node *out);
/* createAliasTable: point lights if n_point > 0, else triangle lights. */
int rg_build_alias_table(const rg_point_light *point_lights, int32_t n_point, const rg_tri_light *tri_lights,
                         int32_t n_tri, rg_alias_table_column *out);
/* CPU primary-ray G-buffer (host planes, same formats as rg_gbuffer). */
int rg_trace_gbuffer_host(const rg_scene_desc *scene, const rg_camera *cam, int32_t width, int32_t height,
                          uint8_t *albedo, uint16_t *normal, uint16_t *material, float *world_pos, float *depth);

/* ---- reservoir format ----
 * The reference's compile-time variants (restirStructs.glsl:16-17):
 * RESERVOIR_SIZE samples per reservoir (1 or 2) and UNBIASED_MIS (0 or 1,
 * a sumPHat per sample, used by the unbiased pass's normalisation).  The
 * default is the reference's (1, 0), the rg_reservoir layout.  Otherwise the
 * reservoir buffers every pass reads and writes hold rg_reservoir_bytes()
 * bytes per pixel in the std430 layout: `samples` LightSamples of 48 bytes
 * (64 with MIS: sumPHat, then 12 bytes of padding) followed by
 * numStreamSamples, padded to 16 bytes.  The frame driver reallocates its
 * buffers; the batched views, the learned proposal's training and the
 * allocation-free chain accept only the default format. */
int rg_set_reservoir_format(rg_context *ctx, int32_t samples, int32_t unbiased_mis);
int rg_reservoir_bytes(rg_context *ctx);

/* ---- device layout of the tree ----
 * No counterpart in the reference.  Shadow rays on the filtered slab test's
 * fast path (every direction component nonzero, finite, within 2^+-100; no
 * NaN box) may walk a copy of the reference's tree built at upload; the
 * others always walk the reference's own tree.  Results are unchanged: the
 * reference's slab test is monotone under box containment for those rays.
 *   RG_TREE_QUANT4 (the default): collapsed to four children per node, child
 *     boxes stored as 8-bit offsets decoding to boxes that contain the exact
 *     ones (64-byte nodes), each reached triangle tested with its exact box
 *     first.  Built when every child box of the tree lies inside the box its
 *     parent stores for it and every box is finite.  Measured fastest (1080p,
 *     1.05M triangles: 6.5 against 7.5 ms per unbiased spatial pass).
 *   RG_TREE_WIDE4: the same collapse with exact boxes (128-byte nodes; each
 *     expanded box's children checked to lie inside it): 8.2 ms.
 *   RG_TREE_BINARY: the reference's tree only.
 * Takes effect at the next upload; rg_stats.tree_layout tells which layout
 * the uploaded scene's walk uses (a copy whose checks fail is not built). */
#define RG_TREE_BINARY 0
#define RG_TREE_WIDE4 1
#define RG_TREE_QUANT4 2
int rg_set_tree_layout(rg_context *ctx, int32_t layout);

/* ---- visibility cache between ray passes ----
 * No counterpart in the reference, which traces every segment.  With the
 * cache on (the default), rg_initial_temporal and rg_spatial_unbiased record
 * the answer of each pixel's own visibility segment (its world position to
 * its sample's light) together with the segment's two end points, and the
 * next of those passes takes the answer of any segment equal to a recorded
 * one bit for bit instead of tracing it (a pixel that kept its sample meets
 * its own segment again; one that took a neighbour's sample meets that
 * neighbour's own segment).  Results are unchanged: an answer depends only on
 * the scene and the two points, and an upload clears the record.  The record
 * lives in the context (32 bytes per pixel and sample, two buffers), so
 * passes of one context must run in order: on one stream, or with the
 * caller synchronising between streams; turn the cache off otherwise.  A
 * batch created while the cache is on keeps a cache of its own
 * (rg_batch_create); the allocation-free entry point does not use it. */
int rg_set_visibility_cache(rg_context *ctx, int32_t enable);

/* ---- scene upload (host pointers; copied to device, synchronous) ---- */
int rg_upload_scene(rg_context *ctx, const rg_scene_desc *scene);

/* ---- passes (device pointers, stream-ordered) ---- */
int rg_initial_temporal(rg_context *ctx, const rg_gbuffer *cur, const rg_gbuffer *prev,
                        const rg_reservoir *prev_reservoirs, rg_reservoir *out,
                        const rg_restir_uniforms *uniforms, void *stream);
int rg_spatial_biased(rg_context *ctx, const rg_gbuffer *gbuf, const rg_reservoir *in, rg_reservoir *out,
                      const rg_restir_uniforms *uniforms, int32_t iter, void *stream);
/* num_neighbors is NUM_NEIGHBORS (reference: 3, unbiasedReuse.glsl:48).  The
 * reference seeds the pass with frame*17 (:72); pass_index p seeds it with
 * frame*17 + p so that chained passes draw fresh neighbours (0 = reference). */
int rg_spatial_unbiased(rg_context *ctx, const rg_gbuffer *gbuf, const rg_reservoir *in, rg_reservoir *out,
                        const rg_restir_uniforms *uniforms, int32_t num_neighbors, int32_t pass_index,
                        void *stream);
int rg_shade(rg_context *ctx, const rg_gbuffer *gbuf, const rg_reservoir *reservoirs,
             const rg_lighting_uniforms *uniforms, float *rgba_out, void *stream);
/* p1, p2: n float4 (xyz used).  shadowed[i] = testVisibility(p1[i], p2[i]). */
int rg_visibility_batch(rg_context *ctx, const float *p1, const float *p2, uint8_t *shadowed, int32_t n,
                        void *stream);
/* GPU primary-ray G-buffer on the uploaded scene (needs materials). */
int rg_trace_gbuffer(rg_context *ctx, const rg_camera *cam, const rg_gbuffer_out *out, void *stream);

/* ---- frame driver: the reference's pass order and reservoir ping-pong ----
 * Owns two frame reservoir buffers and one temporary buffer sized for
 * width*height (allocated on first use or size change, zero-filled, as
 * src/app.h:264-290).  frame_slot selects the current buffer (0/1), the other
 * one is the previous frame's.  Writes the shaded image (float4 rgba). */
int rg_render_frame(rg_context *ctx, const rg_gbuffer *cur, const rg_gbuffer *prev, int32_t frame_slot,
                    const rg_frame_params *params, float *rgba_out, void *stream);
/* Reservoirs of the last rendered frame in slot frame_slot (device pointer). */
int rg_frame_reservoirs(rg_context *ctx, int32_t frame_slot, const rg_reservoir **out);
/* Same as rg_render_frame with HOST planes: copies the current G-buffer in
 * (the previous frame's G-buffer is kept on the device from the last call),
 * renders, and copies the image back; returns after the copy completes. */
int rg_render_frame_host(rg_context *ctx, int32_t width, int32_t height, const uint8_t *albedo,
                         const uint16_t *normal, const uint16_t *material, const float *world_pos,
                         const float *depth, const rg_frame_params *params, float *rgba_out_host, void *stream);

/* ---- triangle lights of a loaded scene ----
 * Replaces collectTriangleLightsFromScene (src/misc.cpp:380-414), which
 * walks the glTF scene's nodes after loading.  Parsing glTF files is not part
 * of this library; the caller passes what the loaded scene holds: per node,
 * its mesh's positions and triangle indices, the node's world matrix and its
 * material's emissive factor. */
typedef struct rg_mesh_instance {
    const float *positions;    /* xyz per vertex (the mesh's vertex range) */
    const uint32_t *indices;   /* index_count indices into positions, three per triangle */
    uint32_t index_count;
    float world_matrix[16];    /* column-major (nvmath::mat4f, the glTF node world matrix) */
    float emissive_factor[3];
} rg_mesh_instance;
/* Every triangle of every instance whose emissive factor has a squared norm
 * above 1e-6 becomes one rg_tri_light, in instance and index order: vertices
 * transformed by the world matrix (w kept), normal = cross(p2 - p1, p3 - p1)
 * divided by its length, area = half that length, emission = (emissive
 * factor, its luminance).  Writes at most `capacity` lights to out (which may
 * be null to count) and returns the number of lights, or a negative
 * RG_ERR_* code. */
int64_t rg_collect_triangle_lights(const rg_mesh_instance *instances, int32_t n_instances, rg_tri_light *out,
                                   int64_t capacity);

/* ---- tensor-core GEMM (a general utility of the library) ----
 * D = alpha * A . B^T, or D += alpha * A . B^T with accumulate != 0 (always
 * atomic when k_splits > 1).  A is m x k and B is n x k, read from device
 * memory with the given element strides of (row, k), as bf16 or, with
 * *_fp32 != 0, as float rounded to bf16; accumulation is FP32 in tensor
 * memory (tcgen05); D is row-major float with leading dimension ldd. */
int rg_gemm_bf16(rg_context *ctx, const void *a, int32_t a_fp32, int64_t a_row_stride, int64_t a_k_stride, int32_t m,
                 const void *b, int32_t b_fp32, int64_t b_row_stride, int64_t b_k_stride, int32_t n, int32_t k,
                 float *d, int64_t ldd, int32_t accumulate, float alpha, int32_t k_splits, void *stream);

/* ---- allocation-free pass chain ----
 * No counterpart in the reference.  Runs num_passes (1..64) unbiased spatial
 * passes, pass index k seeding pass k exactly as rg_spatial_unbiased does,
 * reading `in` and leaving the last pass's reservoirs in `out`; the results
 * equal chaining rg_spatial_unbiased through a caller-provided temporary.
 * For callers that must not allocate device memory while a frame is
 * recorded (fixed memory budgets, frame loops where a cudaMalloc/cudaFree
 * would stall the device, memory owned by another framework's allocator): the
 * intermediate reservoirs live in a 16 MiB buffer built into the library,
 * present on every GPU that loads it until the process exits.  Frames are
 * limited to 262144 pixels (512x512); larger ones return
 * RG_ERR_INVALID_ARGUMENT.  The first call on a device after a context is
 * created there looks up that buffer's device address (rg_create drops the
 * cached one: a reset of the device's primary context unloads the module that
 * holds the buffer, and no context may be used across such a reset), so make
 * that call before any stream capture.  All calls share the buffer: calls
 * whose GPU work overlaps (other streams or host threads) race and must be
 * serialised.  Arguments are checked as rg_spatial_unbiased checks them, and
 * only the default reservoir format is accepted (RG_ERR_UNSUPPORTED
 * otherwise).  Allocates nothing. */
int rg_spatial_unbiased_chain_noalloc(rg_context *ctx, const rg_gbuffer *gbuf, const rg_reservoir *in,
                                      rg_reservoir *out, const rg_restir_uniforms *uniforms, int32_t num_neighbors,
                                      int32_t num_passes, void *stream);

/* ---- many views per launch ----
 * No counterpart in the reference (one view per frame there).  A batch runs the
 * frame driver's pass sequence (rg_render_frame) for many views of the
 * uploaded scene with one launch per pass over all views: a persistent grid
 * takes the tiles of every view from a work counter.  Each view's results
 * equal those of rg_render_frame on that view.  The parameters of every view
 * stay on the device, so a run is stream work only (no host copy, no
 * allocation) and can be captured into a CUDA graph, one per parity. */
typedef struct rg_view {
    rg_gbuffer cur;               /* device G-buffer planes of the view */
    rg_gbuffer prev;              /* previous frame's (may equal cur: a static camera) */
    rg_reservoir *reservoirs[2];  /* parity p writes reservoirs[p] and reads reservoirs[1-p] as the
                                     previous frame's */
    rg_reservoir *tmp;            /* temporary for the spatial chain */
    float *rgba_out;              /* shaded image, float4 per pixel */
    rg_restir_uniforms uniforms;  /* frame = the first run's frame index; each run adds one */
} rg_view;

/* Launch shapes; none of them changes a result. */
typedef struct rg_batch_tuning {
    int32_t ris_pixels_per_thread; /* 1, 2 or 4: RIS tiles of 32 x (4 * this) pixels */
    int32_t spatial_tile_width;    /* 8, 16 or 32: unbiased spatial tiles of w x (128 / w) pixels */
    int32_t ctas_per_sm;           /* persistent CTAs per SM; 0: as many as fit */
} rg_batch_tuning;

typedef struct rg_batch rg_batch;
/* params: unbiased, spatial_iterations, unbiased_neighbors and gamma as for
 * rg_render_frame (its uniforms are not used); tuning may be null.
 * RG_FLAG_LEARNED_PROPOSAL on the views (all or none; 1..32 candidates each)
 * batches the context's learned proposal too: each run first infers it over
 * the pixels of every view (one launch per inference pass) into the batch's
 * own candidate buffer, so each view's results equal rg_proposal_infer
 * followed by rg_render_frame's passes for that view.  The batch uses the
 * proposal's weights as they are at each run (training between runs is
 * fine); once the proposal is re-created, rg_batch_run fails and a captured
 * graph of the batch must not be replayed.  Training stays a separate call
 * (rg_proposal_train on a view's G-buffer and reservoirs).  With the
 * context's visibility cache on at creation, unbiased batches keep their own
 * cache (64 bytes per pixel of all views) with the same results. */
int rg_batch_create(rg_context *ctx, const rg_view *views, int32_t n_views, const rg_frame_params *params,
                    const rg_batch_tuning *tuning, rg_batch **out);
/* One frame of every view on `stream`. */
int rg_batch_run(rg_batch *batch, int32_t parity, void *stream);
/* The next run uses the views' starting frame indices again. */
int rg_batch_reset_frames(rg_batch *batch, void *stream);
int rg_batch_set_tuning(rg_batch *batch, const rg_batch_tuning *tuning);
int rg_batch_get_tuning(rg_batch *batch, rg_batch_tuning *tuning);
/* Times every tuning candidate over `repeats` runs (which advance the frame
 * index and overwrite the views' reservoirs), keeps the fastest and returns it
 * with its mean run time. */
int rg_batch_autotune(rg_batch *batch, int32_t repeats, rg_batch_tuning *best, float *best_ms, void *stream);
/* Chooses the views' RIS candidate count (initial_light_sample_count) among
 * counts[0..n_counts) by Monte Carlo efficiency, 1 / (time x variance): per
 * count, the mean run time over `repeats` runs and the per-pixel variance of
 * the shaded image's log(1 + luminance) (robust to firefly pixels), from two
 * runs that start from the same previous-frame reservoirs (half the mean
 * squared difference of their images).  Unlike the launch shapes, the count
 * is part of the estimator: the
 * chosen count stays set on every view (and in captured graphs of later
 * runs).  Runs advance the frame index and overwrite the views' reservoirs
 * and images.  ms_per_run and variance (n_counts each) may be null.  Counts
 * are 1..32 with the learned proposal, else 1..4096. */
int rg_batch_autotune_candidates(rg_batch *batch, const int32_t *counts, int32_t n_counts, int32_t repeats,
                                 int32_t *best_count, float *ms_per_run, double *variance, void *stream);
int rg_batch_destroy(rg_batch *batch);

/* ---- learned light-cluster proposal ----
 * No counterpart in the reference: it replaces the source pdf of the initial
 * RIS candidates (restirOmni.glsl:73-83).  Per pixel an MLP (9 features:
 * position in the normalisation box, normal, direction to the camera ->
 * 3 x 64 ReLU -> one logit per light cluster; bf16 weights and activations,
 * FP32 accumulation on the tensor cores) gives q(cluster | pixel); a candidate
 * is a cluster c ~ q with a light l ~ p(l | c) from the cluster's alias table
 * over luminance with probability `mix`, else a light drawn uniformly, and its
 * source pdf is the mixture  mix * q(c(l)) * p(l | c(l)) + (1 - mix) / N.
 * The network is trained online by Adam on the clusters of the lights that the
 * final reservoirs hold (softmax cross-entropy).  Point-light scenes only. */
typedef struct rg_proposal_config {
    int32_t clusters;      /* multiple of 128, <= number of lights */
    float mix;             /* probability of the learned branch, in (0, 1) */
    float learning_rate;   /* Adam step size */
    int32_t batch;         /* training pixels per frame */
    float box_min[3];      /* feature normalisation box (scene bounds) */
    float box_max[3];
    uint64_t seed;         /* weight initialisation */
} rg_proposal_config;

/* One learned candidate: key >= 0 is a light drawn uniformly, key < 0 the
 * cluster -1-key drawn from q; q = q(that cluster | pixel). */
typedef struct rg_proposal_candidate {
    int32_t key;
    float q;
} rg_proposal_candidate;

/* Seeded k-means (Lloyd, `iterations` rounds, first centres a seeded shuffle)
 * of the point lights' positions into k clusters; host only. */
int rg_cluster_lights(const rg_point_light *lights, int32_t n, int32_t k, int32_t iterations, uint64_t seed,
                      int32_t *cluster_of, float *centers_xyz);
/* Parameters of the network for `clusters` clusters, packed FP32 in this
 * order, matrices row-major with one row per input: W1 16x64 (rows 9..15 are
 * zero), b1, W2 64x64, b2, W3 64x64, b3, W4 64xC, b4. */
int64_t rg_proposal_param_count(int32_t clusters);
/* Creates (or replaces) the proposal of a context whose uploaded scene has
 * these n point lights; cluster_of[i] is the cluster of light i.  Initial
 * weights are seeded; b4 starts at log(cluster luminance), so that the
 * untrained proposal is close to the luminance-proportional one. */
int rg_proposal_create(rg_context *ctx, const rg_proposal_config *config, const rg_point_light *lights, int32_t n,
                       const int32_t *cluster_of);
int rg_proposal_destroy(rg_context *ctx);
/* Host copies of the FP32 parameters; set also resets Adam. */
int rg_proposal_set_params(rg_context *ctx, const float *params, int64_t n);
int rg_proposal_get_params(rg_context *ctx, float *params, int64_t n);
/* Inference over every pixel for uniforms->frame: fills the candidate buffer
 * (initial_light_sample_count <= 32 candidates per pixel) used by
 * rg_initial_temporal with RG_FLAG_LEARNED_PROPOSAL. */
int rg_proposal_infer(rg_context *ctx, const rg_gbuffer *gbuf, const rg_restir_uniforms *uniforms, void *stream);
/* Device buffers of the last inference: candidates [pixels x 32] and per-pixel
 * {log-sum-exp, most probable cluster (int bits), its probability, 0}. */
int rg_proposal_buffers(rg_context *ctx, const rg_proposal_candidate **candidates, const float **row_stats);
/* Gradient of the mean cross-entropy over n rows (pixel rows[i] of gbuf with
 * target cluster targets[i], -1 = no target, counted in the mean with zero
 * loss) w.r.t. the packed parameters, into grad (device, param_count floats);
 * *loss_sum (host, may be null) receives the summed loss.  No update. */
int rg_proposal_gradients(rg_context *ctx, const rg_gbuffer *gbuf, const float camera_pos[3], const int32_t *rows,
                          const int32_t *targets, int32_t n, float *grad, double *loss_sum, void *stream);
/* One Adam step on `batch` pixels of the frame (a strided sweep whose offset
 * changes with uniforms->frame), targets from final_reservoirs. */
int rg_proposal_train(rg_context *ctx, const rg_gbuffer *gbuf, const rg_restir_uniforms *uniforms,
                      const rg_reservoir *final_reservoirs, void *stream);
/* Mean loss over the rows with a target, and their number, of the last
 * training step (synchronises). */
int rg_proposal_last_loss(rg_context *ctx, double *mean_loss, int64_t *rows_with_target);

#ifdef __cplusplus
}
#endif
#endif
