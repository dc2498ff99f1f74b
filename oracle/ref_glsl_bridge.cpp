// ref_glsl_bridge.cpp -- compiles the reference's own shader includes for
// BRDF / p-hat (src/shaders/include/disneyBRDF.glsl, restirUtils.glsl,
// common.glsl) and software shadow-ray traversal
// (src/shaders/include/softwareRaytracing.glsl, visibilityTest.glsl,
// structs/aabbTree.glsl) as C++ through glsl_shim.hpp, and exports them with
// a C ABI so the tests can pin the oracle's restatement against them.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/Makefile into oracle/_ref/ from
// the reference sources where they lie; nothing here is shipped.
#include <cstdint>
#include <cstring>

#include "refshim/glsl_shim.hpp"

namespace refglsl {
using namespace glsl;

struct NodeBufferView;
#define float gfloat
#include "structs/aabbTree.glsl"
#undef float

struct NodeBufferView { const AabbTreeNode *nodes; };
static thread_local NodeBufferView g_node_buffer;
static thread_local const Triangle *g_triangles;

#define float gfloat
#define NODE_BUFFER g_node_buffer
#define TRIANGLE_BUFFER g_triangles
#undef M_PI
#include "restirUtils.glsl"
#include "softwareRaytracing.glsl"
#include "visibilityTest.glsl"
#undef TRIANGLE_BUFFER
#undef NODE_BUFFER
#undef float
}  // namespace refglsl

using refglsl::gfloat;
using refglsl::vec3;
using refglsl::vec4;

static inline vec3 v3(const float *p) { return vec3(gfloat(p[0]), gfloat(p[1]), gfloat(p[2])); }

extern "C" {

// Layout of the node/triangle buffers handed in: the reference's std430
// AabbTreeNode (80 B) and Triangle (48 B).
struct ref_node { float lmin[4], lmax[4], rmin[4], rmax[4]; int32_t left, right, pad0, pad1; };
struct ref_tri { float p1[4], p2[4], p3[4]; };

static void load_nodes(const ref_node *nodes, int32_t n_nodes, const ref_tri *tris, int32_t n_tris,
                       refglsl::AabbTreeNode **out_nodes, refglsl::Triangle **out_tris) {
    auto *nn = new refglsl::AabbTreeNode[n_nodes > 0 ? n_nodes : 1];
    for (int32_t i = 0; i < n_nodes; ++i) {
        const ref_node &s = nodes[i];
        nn[i].leftAabbMin = vec4(s.lmin[0], s.lmin[1], s.lmin[2], s.lmin[3]);
        nn[i].leftAabbMax = vec4(s.lmax[0], s.lmax[1], s.lmax[2], s.lmax[3]);
        nn[i].rightAabbMin = vec4(s.rmin[0], s.rmin[1], s.rmin[2], s.rmin[3]);
        nn[i].rightAabbMax = vec4(s.rmax[0], s.rmax[1], s.rmax[2], s.rmax[3]);
        nn[i].leftChild = s.left;
        nn[i].rightChild = s.right;
    }
    auto *tt = new refglsl::Triangle[n_tris > 0 ? n_tris : 1];
    for (int32_t i = 0; i < n_tris; ++i) {
        tt[i].p1 = vec4(tris[i].p1[0], tris[i].p1[1], tris[i].p1[2], tris[i].p1[3]);
        tt[i].p2 = vec4(tris[i].p2[0], tris[i].p2[1], tris[i].p2[2], tris[i].p2[3]);
        tt[i].p3 = vec4(tris[i].p3[0], tris[i].p3[1], tris[i].p3[2], tris[i].p3[3]);
    }
    *out_nodes = nn;
    *out_tris = tt;
}

// Depth of the tree below node 0 (root depth 1); the reference's 32-entry
// traversal stack holds at most depth+1 entries.
static int tree_depth(const ref_node *nodes, int32_t idx, int32_t n_nodes, int guard) {
    if (idx < 0 || idx >= n_nodes || guard > 4096) return 0;
    int l = nodes[idx].left >= 0 ? tree_depth(nodes, nodes[idx].left, n_nodes, guard + 1) : 0;
    int r = nodes[idx].right >= 0 ? tree_depth(nodes, nodes[idx].right, n_nodes, guard + 1) : 0;
    return 1 + (l > r ? l : r);
}

int32_t ref_tree_depth(const ref_node *nodes, int32_t n_nodes) {
    return n_nodes > 0 ? tree_depth(nodes, 0, n_nodes, 0) : 0;
}

// args per call: worldPos3 lightPos3 camPos3 normal3 lightNormal3 useLightNormal albedoLum emissionLum roughness metallic
void ref_eval_phat_batch(int32_t n, const float *a, float *out) {
    for (int32_t i = 0; i < n; ++i, a += 20) {
        gfloat r = refglsl::evaluatePHat(v3(a), v3(a + 3), v3(a + 6), v3(a + 9), v3(a + 12), a[15] > 0.5f,
                                         gfloat(a[16]), gfloat(a[17]), gfloat(a[18]), gfloat(a[19]));
        out[i] = static_cast<float>(r);
    }
}

// args per call: worldPos3 lightPos3 camPos3 normal3 lightNormal3 useLightNormal albedo3 emission3 roughness metallic
void ref_eval_phat_full_batch(int32_t n, const float *a, float *out) {
    for (int32_t i = 0; i < n; ++i, a += 24) {
        vec3 r = refglsl::evaluatePHatFull(v3(a), v3(a + 3), v3(a + 6), v3(a + 9), v3(a + 12), a[15] > 0.5f,
                                           v3(a + 16), v3(a + 19), gfloat(a[22]), gfloat(a[23]));
        out[3 * i] = static_cast<float>(r.x);
        out[3 * i + 1] = static_cast<float>(r.y);
        out[3 * i + 2] = static_cast<float>(r.z);
    }
}

// args: origin3 dir3 aabbMin3 aabbMax3
void ref_ray_aabb_batch(int32_t n, const float *a, uint8_t *out) {
    for (int32_t i = 0; i < n; ++i, a += 12)
        out[i] = refglsl::rayAabIntersection(v3(a), v3(a + 3), v3(a + 6), v3(a + 9)) ? 1 : 0;
}

// args: origin3 dir3 p1 p2 p3
void ref_ray_tri_batch(int32_t n, const float *a, uint8_t *out) {
    for (int32_t i = 0; i < n; ++i, a += 15) {
        refglsl::Triangle t;
        t.p1 = vec4(a[6], a[7], a[8], 1.0f);
        t.p2 = vec4(a[9], a[10], a[11], 1.0f);
        t.p3 = vec4(a[12], a[13], a[14], 1.0f);
        out[i] = refglsl::rayTriangleIntersection(t, v3(a), v3(a + 3)) ? 1 : 0;
    }
}

// Reference raytrace(): out 1 = unoccluded.  Returns -1 (and traces nothing)
// if the tree is deep enough to overflow the reference's 32-entry stack.
int32_t ref_raytrace_batch(const ref_node *nodes, int32_t n_nodes, const ref_tri *tris, int32_t n_tris,
                           int32_t n, const float *rays, uint8_t *out) {
    if (ref_tree_depth(nodes, n_nodes) + 1 > 32) return -1;
    refglsl::AabbTreeNode *nn;
    refglsl::Triangle *tt;
    load_nodes(nodes, n_nodes, tris, n_tris, &nn, &tt);
    refglsl::g_node_buffer.nodes = nn;
    refglsl::g_triangles = tt;
    for (int32_t i = 0; i < n; ++i) out[i] = refglsl::raytrace(v3(rays + 6 * i), v3(rays + 6 * i + 3)) ? 1 : 0;
    delete[] nn;
    delete[] tt;
    return 0;
}

// Reference testVisibility(): out 1 = shadowed.
int32_t ref_test_visibility_batch(const ref_node *nodes, int32_t n_nodes, const ref_tri *tris, int32_t n_tris,
                                  int32_t n, const float *p1, const float *p2, uint8_t *out) {
    if (ref_tree_depth(nodes, n_nodes) + 1 > 32) return -1;
    refglsl::AabbTreeNode *nn;
    refglsl::Triangle *tt;
    load_nodes(nodes, n_nodes, tris, n_tris, &nn, &tt);
    refglsl::g_node_buffer.nodes = nn;
    refglsl::g_triangles = tt;
    for (int32_t i = 0; i < n; ++i) out[i] = refglsl::testVisibility(v3(p1 + 3 * i), v3(p2 + 3 * i)) ? 1 : 0;
    delete[] nn;
    delete[] tt;
    return 0;
}

}  // extern "C"
