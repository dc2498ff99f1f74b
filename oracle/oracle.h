/*
 * oracle.h -- CPU oracle for the ReSTIR direct-lighting hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: the parity tests,
 * __graft_entry__.smoke() and the CPU-baseline leg of bench.py load it to
 * compute the expected result of every pass on the same inputs the CUDA path
 * receives.  Product code never links, loads or calls it.
 *
 * It restates, in plain single-precision C with OpenMP over pixels, the
 * reference's GLSL passes (reference paths are relative to the reference
 * project root):
 *   PCG32                src/shaders/include/rand.glsl:7-32
 *   reservoir ops        src/shaders/include/reservoir.glsl:6-76
 *   BRDF / p-hat         src/shaders/include/disneyBRDF.glsl:5-90,
 *                        src/shaders/include/restirUtils.glsl:3-55
 *   BVH traversal        src/shaders/include/softwareRaytracing.glsl:3-85,
 *                        src/shaders/include/visibilityTest.glsl:1-30
 *   RIS+vis+temporal     src/shaders/restirOmni.glsl:68-212
 *   biased spatial       src/shaders/spatialReuse.comp:30-86
 *   unbiased spatial     src/shaders/unbiasedReuse.glsl:50-185
 *   shading              src/shaders/lighting.frag:43-71,103
 *   alias table (Vose)   src/misc.cpp:418-497
 * plus an FP64 brute-force judge (sum over every light with exact
 * visibility) used for image RMSE.
 *
 * The byte layouts of every struct below equal the reference's std430/std140
 * layouts (src/shaderIncludes.h, the files under src/shaders/include/structs/) and the
 * product's C ABI (include/restir_gb300.h).
 */
#ifndef RESTIR_ORACLE_H
#define RESTIR_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { float x, y, z, w; } or_f4;

/* Compile-time variants of the reference (restirStructs.glsl:16-17):
 * OR_RS = RESERVOIR_SIZE, OR_MIS = UNBIASED_MIS.  The default build is the
 * reference's configuration (1, off); oracle/Makefile builds the others as
 * separate libraries with the same symbols. */
#ifndef OR_RS
#define OR_RS 1
#endif
#ifndef OR_MIS
#define OR_MIS 0
#endif

typedef struct {             /* LightSample (std430): 48 bytes, 64 with UNBIASED_MIS */
    or_f4 pos_lum;           /* position_emissionLum */
    or_f4 normal;            /* light normal, w>0.5 => use it */
    int32_t light_index;     /* negative: triangle light -1-i */
    float p_hat;
    float sum_weights;
    float w;
#if OR_MIS
    float sum_phat;
    float pad_s[3];
#endif
} or_sample;

typedef struct {             /* Reservoir: OR_RS samples + numStreamSamples (64 bytes in the default build) */
    or_sample s[OR_RS];
    uint32_t m;              /* numStreamSamples */
    uint32_t pad[3];
} or_reservoir;

typedef struct { or_f4 lmin, lmax, rmin, rmax; int32_t left, right, pad0, pad1; } or_node;   /* 80 B */
typedef struct { or_f4 p1, p2, p3; } or_tri;                                                /* 48 B */
typedef struct { or_f4 pos, color_lum; } or_point_light;                                    /* 32 B */
typedef struct { or_f4 p1, p2, p3, emission_lum, normal_area; } or_tri_light;               /* 80 B */
typedef struct { float prob; int32_t alias; float ori_prob; float alias_ori_prob; } or_alias; /* 16 B */

typedef struct {             /* RestirUniforms: 128 bytes */
    float prev_pv[16];       /* column-major prevFrameProjectionViewMatrix */
    or_f4 camera_pos;
    uint32_t size[2];
    uint32_t frame;
    uint32_t initial_light_sample_count;
    uint32_t temporal_mult;
    float pos_threshold;
    float normal_threshold;  /* degrees */
    uint32_t spatial_neighbors;
    float spatial_radius;
    int32_t flags;
    uint32_t pad[2];
} or_uniforms;

typedef struct {             /* LightingPassUniforms: 96 bytes */
    float prev_pv[16];
    or_f4 camera_pos;
    uint32_t size[2];
    int32_t debug_mode;
    float gamma;
} or_lighting_uniforms;

#define OR_FLAG_VISIBILITY 1
#define OR_FLAG_TEMPORAL 2
#define OR_FLAG_FINAL_RIS_WEIGHT 256 /* extension: W = sumWeights / (M * pHat) after RIS */
#define OR_FLAG_MIS_SWAP_FIX 2048    /* extension (UNBIASED_MIS): combineReservoirs passes (w, sumPHat) in order */

typedef struct {
    const or_node *nodes; int32_t n_nodes;
    const or_tri *tris; int32_t n_tris;
    const or_point_light *point_lights; int32_t n_point_lights;
    const or_tri_light *tri_lights; int32_t n_tri_lights;
    const or_alias *alias; int32_t n_alias;
} or_scene;

typedef struct {             /* headless G-buffer planes, row-major, width*height texels */
    int32_t width, height;
    const uint8_t *albedo;   /* RGBA8, sRGB-encoded rgb, a = emissive flag */
    const uint16_t *normal;  /* normal_format; 0: RGBA16F bit patterns */
    const uint16_t *material;/* RG16 unorm (roughness, metallic) */
    const float *world_pos;  /* world_pos_format; 0: RGBA32F */
    const float *depth;      /* depth_format; 0: D32F */
    /* VkFormat numbers of the reference's attachment candidates
     * (gBufferPass.cpp:81-101), 0 = the default above */
    int32_t normal_format, world_pos_format, depth_format, reserved;
} or_gbuffer;

typedef struct {
    uint64_t rays;           /* shadow segments traced */
    uint64_t node_visits;    /* nodes popped */
    uint64_t box_tests;
    uint64_t tri_tests;
    uint64_t stack_overflows;
    uint64_t rays_unobservable; /* unbiased pass: neighbour segments of a sample whose own segment is
                                   shadowed (the count is then reset, so their answers never reach
                                   the output) */
} or_stats;

/* ---- primitives ---- */
void or_pcg_stream(uint64_t seed, uint64_t seq, int32_t n, uint32_t *out);
void or_rand_floats(uint64_t seed, uint64_t seq, int32_t n, float *out);
void or_sincos_batch(int32_t n, const float *x, float *s, float *c);
void or_srgb_lut(float *out256);
float or_half_to_float(uint16_t h);
/* args: 20 floats per call: worldPos3 lightPos3 camPos3 normal3 lightNormal3 useLightNormal albedoLum emissionLum roughness metallic */
void or_eval_phat_batch(int32_t n, const float *args, float *out);
/* args: 24 floats: worldPos3 lightPos3 camPos3 normal3 lightNormal3 useLightNormal albedo3 emission3 roughness metallic */
void or_eval_phat_full_batch(int32_t n, const float *args, float *out3);
void or_ray_aabb_batch(int32_t n, const float *args /*12*/, uint8_t *out);
void or_ray_tri_batch(int32_t n, const float *args /*15*/, uint8_t *out);
/* raw traversal: origin3,dir3 per ray; out 1 = unoccluded (reference raytrace() value) */
void or_raytrace_batch(const or_scene *scene, int32_t n, const float *rays, uint8_t *out, int32_t stack_size, or_stats *stats);
/* testVisibility: p1[3],p2[3] per ray; out 1 = shadowed */
void or_test_visibility_batch(const or_scene *scene, int32_t n, const float *p1, const float *p2, uint8_t *out, or_stats *stats);
void or_alias_sample_batch(const or_alias *table, int32_t count, int32_t n, const float *r, int32_t *idx, float *prob);
void or_build_alias_table(const or_point_light *pl, int32_t n_pl, const or_tri_light *tl, int32_t n_tl, or_alias *out);
/* Triangle lights of loaded meshes (collectTriangleLightsFromScene, src/misc.cpp:380-414); the instance
 * record has the layout of the product's rg_mesh_instance.  Returns the light count, writing at most cap. */
typedef struct {
    const float *positions; const uint32_t *indices; uint32_t index_count;
    float world_matrix[16]; float emissive_factor[3];
} or_mesh_instance;
int64_t or_collect_tri_lights(const or_mesh_instance *inst, int32_t n, or_tri_light *out, int64_t cap);

/* ---- passes; crop = {x0, y0, w, h} or NULL for the full frame; out is full-frame sized ---- */
typedef struct { int32_t key; float q; } or_candidate;     /* learned candidate (see or_mlp below) */
typedef struct {
    const or_candidate *cand;   /* [pixels x 32] */
    const int32_t *order, *offset;
    const or_alias *col;        /* per grouped position, alias = grouped position */
    const float *within;
    float mix, uniform_pdf;
} or_learned;
int or_initial_temporal_learned(const or_scene *scene, const or_gbuffer *cur, const or_gbuffer *prev,
                                const or_reservoir *prev_res, or_reservoir *out, const or_uniforms *u,
                                const or_learned *learned, const int32_t *crop, or_stats *stats);
int or_initial_temporal(const or_scene *scene, const or_gbuffer *cur, const or_gbuffer *prev,
                        const or_reservoir *prev_res, or_reservoir *out, const or_uniforms *u,
                        const int32_t *crop, or_stats *stats);
int or_spatial_biased(const or_scene *scene, const or_gbuffer *g, const or_reservoir *in, or_reservoir *out,
                      const or_uniforms *u, int32_t iter, const int32_t *crop);
int or_spatial_unbiased(const or_scene *scene, const or_gbuffer *g, const or_reservoir *in, or_reservoir *out,
                        const or_uniforms *u, int32_t num_neighbors, int32_t pass_index, const int32_t *crop, or_stats *stats);
int or_shade(const or_scene *scene, const or_gbuffer *g, const or_reservoir *res, const or_lighting_uniforms *u,
             float *rgba_out, const int32_t *crop);
int or_brute_force_fp64(const or_scene *scene, const or_gbuffer *g, const float *camera_pos3,
                        double *rgb_out, const int32_t *crop);

/* ---- learned light-cluster proposal (no reference counterpart; see oracle.c) ---- */
typedef struct {
    int32_t clusters;
    float mix;                   /* probability of the learned branch */
    int32_t n_lights;
    float box_center[3], box_inv_half[3];
    const float *params;         /* packed FP32 parameters */
    const uint8_t *cluster_valid;/* 1: the cluster has lights */
    const int32_t *cluster_of;   /* cluster of each light */
} or_mlp;
float or_bf16_round(float x);
int or_cluster_tables(const or_point_light *pl, int32_t n, const int32_t *cluster_of, int32_t k, int32_t *order,
                      int32_t *offset, or_alias *col, float *within);
int64_t or_mlp_param_count(int32_t clusters);
void or_mlp_features(const or_mlp *m, const or_gbuffer *g, const float cam[3], int32_t px, float x[16]);
/* rows == NULL: row r is pixel r; z_out (optional) receives [n x clusters] logits */
void or_mlp_row_stats(const or_mlp *m, const or_gbuffer *g, const float cam[3], int32_t n, const int32_t *rows,
                      double *lse, int32_t *amax, double *z_out);
void or_mlp_sample(const or_mlp *m, const or_gbuffer *g, const float cam[3], uint32_t frame, int32_t n_cand,
                   int32_t n, const int32_t *rows, int32_t *keys, float *qs);
double or_mlp_loss_grad(const or_mlp *m, const double *params64, const or_gbuffer *g, const float cam[3], int32_t n,
                        const int32_t *rows, const int32_t *target, int32_t emulate, double *grad);

/* ---- reservoir variants ---- */
void or_reservoir_layout(int32_t *reservoir_size, int32_t *unbiased_mis, int32_t *bytes);
/* newReservoir, addSampleToReservoir for each of n candidates (12 floats:
 * position xyz, normal xyzw, emission luminance, light index (int bits),
 * p-hat, source pdf, unused), then combineReservoirs(other, other_phat[OR_RS])
 * when other != NULL; PCG stream (seed, seq). */
void or_reservoir_script(const float *cand, int32_t n, const or_reservoir *other, const float *other_phat,
                         uint64_t seed, uint64_t seq, int32_t swap_fix, or_reservoir *out);

/* ---- the reference's tree builder (AabbTree::build, aabbTreeBuilder.cpp:52-214) ----
 * tri_xyz: n triangles x 9 floats.  Writes n-1 nodes and n triangles (w = 1)
 * and returns n-1; -1 for n < 2; -3 when the input takes a path the reference
 * leaves undefined (a range whose centroids all coincide, or one with no
 * finite split heuristic). */
int32_t or_build_bvh(const float *tri_xyz, int32_t n, or_node *out_nodes, or_tri *out_tris);

/* ---- primary-ray G-buffer (replaces the raster pass gBufferPass.cpp / gBuffer.frag) ---- */
typedef struct { uint8_t albedo_srgb[4]; uint16_t roughness, metallic; } or_material;   /* 8 B per triangle */
typedef struct {             /* pinhole camera (camera.h:25-50), the library's rg_camera layout */
    float position[3], right[3], up[3], forward[3];
    float tan_half_fov_y, aspect;
    float projection_view[16];   /* column-major P*V */
} or_camera;
/* One closest-hit ray through every pixel centre of the crop (NULL: the whole
 * frame); planes are full-frame, row-major, written only inside the crop.
 * Returns 0, or -2 for a bad crop, -5 for a malformed tree. */
int or_trace_gbuffer(const or_scene *scene, const or_material *mats, int32_t n_mats, const or_camera *cam,
                     int32_t width, int32_t height, const int32_t *crop, uint8_t *albedo, uint16_t *normal,
                     uint16_t *material, float *world_pos, float *depth);
uint16_t or_float_to_half(float f);

int or_max_threads(void);
void or_set_threads(int32_t n);

#ifdef __cplusplus
}
#endif
#endif
