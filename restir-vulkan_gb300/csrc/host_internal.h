// host_internal.h -- host-side preprocessing shared by the C ABI (host.cpp).
#pragma once
#include <stdint.h>

#include <vector>

#include "../../include/restir_gb300.h"

int host_build_bvh(const float *xyz, int32_t n, rg_aabb_tree_node *out_nodes, rg_triangle *out_tris,
                   int *ref_undefined);
int host_validate_tree(const rg_aabb_tree_node *nodes, int32_t n_nodes, int32_t n_tris);
int host_build_alias_table(const rg_point_light *pl, int32_t n_pl, const rg_tri_light *tl, int32_t n_tl,
                           rg_alias_table_column *out);
void host_pack_nodes(const rg_aabb_tree_node *src, int32_t n, float *dst16);
void host_pack_nodes_preorder(const rg_aabb_tree_node *src, int32_t n, float *dst16);
void host_tree_preorder(const rg_aabb_tree_node *src, int32_t n, rg_aabb_tree_node *dst);
bool host_boxes_have_nan(const rg_aabb_tree_node *nodes, int32_t n);
void host_pack_tris(const rg_triangle *src, int32_t n, float *dst12);
// The 4-wide copy of a valid tree (32 floats per node; see host.cpp): node
// count, or -1 when some child box lies outside its parent's box.
int32_t host_pack_wide(const rg_aabb_tree_node *src, int32_t n, std::vector<float> &out, int *wide_depth);
// The quantized 4-wide copy (16 words per node, 16 floats per leaf record;
// see host.cpp) over packed triangles: node count, or -1 when the tree is not
// nested (host_tree_nested) or a box cannot be quantized (non-finite bounds).
bool host_tree_nested(const rg_aabb_tree_node *src, int32_t n);
int32_t host_pack_quant(const rg_aabb_tree_node *src, int32_t n, const float *tris12, std::vector<uint32_t> &nodes,
                        std::vector<float> &leaves, int *wide_depth);
void srgb_lut_host(float *out256);
int host_trace_gbuffer(const float *nodes16, int32_t n_nodes, const float *tris12, int32_t n_tris,
                       const rg_material *mats, int32_t n_mats, const rg_camera &cam, int32_t w, int32_t h,
                       uint8_t *albedo, uint16_t *normal, uint16_t *material, float *world_pos, float *depth);
int host_kmeans(const float *pos4, int32_t n, int32_t k, int32_t iterations, uint64_t seed, int32_t *cluster_of,
                float *centers3);
int host_cluster_tables(const rg_point_light *pl, int32_t n, const int32_t *cluster_of, int32_t k, int32_t *order,
                        int32_t *offset, rg_alias_table_column *col, float *within);
// collectTriangleLightsFromScene (src/misc.cpp:380-414) on loaded meshes:
// the light count; at most `capacity` lights written to out (may be null).
int64_t host_collect_tri_lights(const rg_mesh_instance *inst, int32_t n, rg_tri_light *out, int64_t capacity);
