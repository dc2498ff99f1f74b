// ref_lights_bridge.cpp -- the triangle-light collection of the reference
// (collectTriangleLightsFromScene, src/misc.cpp:380-414) evaluated with the
// reference's own nvmath types and operators (thirdparty/nvmath: mat4f * vec4f,
// cross, norm, operator/=, sq_norm) and its luminance (common.glsl through
// src/shaderIncludes.h), on meshes handed in with the product's instance
// layout.  misc.cpp itself includes Vulkan and does not build here, so this
// bridge makes the same library calls in the same order.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/Makefile into oracle/_ref/ from
// the reference sources where they lie; nothing here is shipped.
#include <cstdint>

#include "nvmath.h"
#include "shaderIncludes.h"

extern "C" {

struct ref_mesh_instance {
    const float *positions;
    const uint32_t *indices;
    uint32_t index_count;
    float world_matrix[16];
    float emissive_factor[3];
};

// out: 20 floats per light (p1, p2, p3, emission_luminance, normalArea)
int64_t ref_collect_tri_lights(const ref_mesh_instance *inst, int32_t n, float *out, int64_t cap) {
    int64_t count = 0;
    for (int32_t k = 0; k < n; ++k) {
        const nvmath::mat4f world(inst[k].world_matrix);
        const nvmath::vec3f emissive(inst[k].emissive_factor[0], inst[k].emissive_factor[1],
                                     inst[k].emissive_factor[2]);
        if (!(emissive.sq_norm() > 1e-6)) continue;
        for (uint32_t i = 0; i + 2 < inst[k].index_count; i += 3) {
            const float *q0 = inst[k].positions + 3 * (size_t)inst[k].indices[i];
            const float *q1 = inst[k].positions + 3 * (size_t)inst[k].indices[i + 1];
            const float *q2 = inst[k].positions + 3 * (size_t)inst[k].indices[i + 2];
            const nvmath::vec4f p1 = world * nvmath::vec4f(nvmath::vec3f(q0[0], q0[1], q0[2]), 1.0f);
            const nvmath::vec4f p2 = world * nvmath::vec4f(nvmath::vec3f(q1[0], q1[1], q1[2]), 1.0f);
            const nvmath::vec4f p3 = world * nvmath::vec4f(nvmath::vec3f(q2[0], q2[1], q2[2]), 1.0f);
            const nvmath::vec3f a(p1.x, p1.y, p1.z), b(p2.x, p2.y, p2.z), c(p3.x, p3.y, p3.z);
            nvmath::vec3f normal = nvmath::cross(b - a, c - a);
            float area = normal.norm();
            normal /= area;
            area *= 0.5f;
            const float lum = shader::luminance(emissive.x, emissive.y, emissive.z);
            if (out && count < cap) {
                float *o = out + 20 * count;
                const float v[20] = {p1.x, p1.y, p1.z, p1.w, p2.x, p2.y, p2.z, p2.w, p3.x, p3.y, p3.z, p3.w,
                                     emissive.x, emissive.y, emissive.z, lum, normal.x, normal.y, normal.z, area};
                for (int j = 0; j < 20; ++j) o[j] = v[j];
            }
            ++count;
        }
    }
    return count;
}

}  // extern "C"
