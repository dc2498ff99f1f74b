// Stub for the reference's glTF scene type (thirdparty/gltf/gltfscene.h).
// TEST INFRASTRUCTURE ONLY: it declares exactly the members that
// src/aabbTreeBuilder.cpp:59-62 reads, so the reference's BVH builder can be
// compiled unmodified and fed triangles directly.
#pragma once
#include <cstdint>
#include <vector>
#include <nvmath.h>

namespace nvh {
struct GltfNode {
    nvmath::mat4f worldMatrix{1};
    uint32_t primMesh{0};
};
struct GltfPrimMesh {
    uint32_t firstIndex{0};
    uint32_t indexCount{0};
    uint32_t vertexOffset{0};
};
struct GltfScene {
    std::vector<GltfNode> m_nodes;
    std::vector<GltfPrimMesh> m_primMeshes;
    std::vector<uint32_t> m_indices;
    std::vector<nvmath::vec3f> m_positions;
};
}  // namespace nvh
