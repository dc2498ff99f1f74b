// ref_bvh_bridge.cpp -- drives the reference's own binned-SAH BVH builder
// (src/aabbTreeBuilder.cpp:52-214, compiled unmodified from the reference
// sources against the stub headers in refshim/) on a flat triangle list, and
// returns its node and triangle buffers in the std430 layout
// (src/shaders/include/structs/aabbTree.glsl).
//
// TEST INFRASTRUCTURE ONLY: pins the product's own builder, which must emit
// byte-identical buffers.
#include <cstdint>
#include <cstring>
#include <vector>

#include "aabbTreeBuilder.h"

extern "C" {

struct ref_node { float lmin[4], lmax[4], rmin[4], rmax[4]; int32_t left, right, pad0, pad1; };
struct ref_tri { float p1[4], p2[4], p3[4]; };

// tri_xyz: n_tris * 9 floats (p1, p2, p3).  out_nodes: n_tris - 1 records,
// out_tris: n_tris records.  Returns the node count, or -1 for n_tris < 2
// (the reference sizes the node array as n-1 and needs a root node).
int32_t ref_build_bvh(const float *tri_xyz, int32_t n_tris, ref_node *out_nodes, ref_tri *out_tris) {
    if (n_tris < 2) return -1;
    nvh::GltfScene scene;
    scene.m_nodes.resize(1);
    scene.m_primMeshes.resize(1);
    scene.m_primMeshes[0].firstIndex = 0;
    scene.m_primMeshes[0].vertexOffset = 0;
    scene.m_primMeshes[0].indexCount = static_cast<uint32_t>(3 * n_tris);
    scene.m_indices.resize(3 * static_cast<size_t>(n_tris));
    scene.m_positions.resize(3 * static_cast<size_t>(n_tris));
    for (size_t i = 0; i < 3 * static_cast<size_t>(n_tris); ++i) {
        scene.m_indices[i] = static_cast<uint32_t>(i);
        scene.m_positions[i] = nvmath::vec3f(tri_xyz[3 * i], tri_xyz[3 * i + 1], tri_xyz[3 * i + 2]);
    }
    AabbTree tree = AabbTree::build(scene);
    for (size_t i = 0; i < tree.nodes.size(); ++i) {
        const shader::AabbTreeNode &s = tree.nodes[i];
        ref_node &d = out_nodes[i];
        const nvmath::vec4 *boxes[4] = {&s.leftAabbMin, &s.leftAabbMax, &s.rightAabbMin, &s.rightAabbMax};
        float *dst[4] = {d.lmin, d.lmax, d.rmin, d.rmax};
        for (int b = 0; b < 4; ++b) {
            dst[b][0] = boxes[b]->x; dst[b][1] = boxes[b]->y; dst[b][2] = boxes[b]->z; dst[b][3] = boxes[b]->w;
        }
        d.left = s.leftChild;
        d.right = s.rightChild;
        d.pad0 = d.pad1 = 0;
    }
    for (size_t i = 0; i < tree.triangles.size(); ++i) {
        const shader::Triangle &s = tree.triangles[i];
        ref_tri &d = out_tris[i];
        d.p1[0] = s.p1.x; d.p1[1] = s.p1.y; d.p1[2] = s.p1.z; d.p1[3] = s.p1.w;
        d.p2[0] = s.p2.x; d.p2[1] = s.p2.y; d.p2[2] = s.p2.z; d.p2[3] = s.p2.w;
        d.p3[0] = s.p3.x; d.p3[1] = s.p3.y; d.p3[2] = s.p3.z; d.p3[3] = s.p3.w;
    }
    return static_cast<int32_t>(tree.nodes.size());
}

}  // extern "C"
