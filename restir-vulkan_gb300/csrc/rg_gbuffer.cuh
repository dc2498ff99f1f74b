// rg_gbuffer.cuh -- primary-ray G-buffer, shared by the CUDA kernel and the
// host tracer so both write identical planes.
//
// Replaces the reference's raster G-buffer pass (src/passes/gBufferPass.cpp,
// src/shaders/gBuffer.frag:27-79) for headless use: one closest-hit ray per
// pixel centre through the reference's camera (src/camera.h:25-50: view rows
// right, -up, forward; clip w = view z), writing the same attachment formats
// (albedo RGBA8 sRGB with alpha = emissive flag, normal RGBA16F, material
// RG16 unorm, world position RGBA32F, depth = clip z / clip w).
#pragma once
#include "rg_math.cuh"
#include "../../include/restir_gb300.h"

namespace rgm {

struct Hit { float t; int tri; };

// Slab test for closest hit: entry/exit along o + t*d using 1/d.
RG_HD bool slab(f3 o, f3 inv, f3 bmin, f3 bmax, float tbest, float &tenter) {
    const float t0x = (bmin.x - o.x) * inv.x, t1x = (bmax.x - o.x) * inv.x;
    const float t0y = (bmin.y - o.y) * inv.y, t1y = (bmax.y - o.y) * inv.y;
    const float t0z = (bmin.z - o.z) * inv.z, t1z = (bmax.z - o.z) * inv.z;
    const float rmin = gmax(gmin(t0x, t1x), gmax(gmin(t0y, t1y), gmin(t0z, t1z)));
    const float rmax = gmin(gmax(t0x, t1x), gmin(gmax(t0y, t1y), gmax(t0z, t1z)));
    tenter = rmin;
    return rmax >= rmin && rmax > 0.0f && rmin < tbest;
}

RG_HD bool tri_t(f3 p1, f3 e1, f3 e2, f3 o, f3 d, float &t) {
    const f3 p = cross(d, e2);
    const float f = 1.0f / dot(e1, p);
    const f3 s = o - p1;
    const float bx = f * dot(s, p);
    if (!(bx >= 0.0f && bx <= 1.0f)) return false;
    const f3 q = cross(s, e1);
    const float by = f * dot(d, q);
    if (!(by >= 0.0f && by + bx <= 1.0f)) return false;
    t = f * dot(e2, q);
    return t > 0.0f;
}

// Node/triangle access as plain 16-byte vectors, layouts as GNode / GTri.
struct TraceScene {
    const float *nodes;  // 16 floats per node
    int n_nodes;
    const float *tris;   // 12 floats per triangle
    int n_tris;
};

// Closest hit: nearer child first, ties broken to the smaller triangle index.
// Returns tri = -1 on a miss or if the walk needed more than one visit per
// node or a deeper stack than RG_MAX_TREE_DEPTH+1 (malformed tree).
RG_HD Hit closest_hit(const TraceScene &s, f3 o, f3 d) {
    Hit h;
    h.t = 3.402823466e38f;
    h.tri = -1;
    if (s.n_nodes <= 0) return h;
    const f3 inv = mk(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
    int stack[RG_MAX_TREE_DEPTH + 1];
    int top = 0;
    int node = 0;
    int visits = 0;
    while (true) {
        if (++visits > s.n_nodes) { h.tri = -1; return h; }
        const float *n = s.nodes + 16 * (size_t)node;
        const int left = ((const int *)n)[12], right = ((const int *)n)[13];
        float tl, tr;
        const bool hl = slab(o, inv, mk(n[0], n[4], n[8]), mk(n[2], n[6], n[10]), h.t, tl);
        const bool hr = slab(o, inv, mk(n[1], n[5], n[9]), mk(n[3], n[7], n[11]), h.t, tr);
        int first = -1, second = -1;
        if (hl) {
            if (left < 0) {
                const float *tp = s.tris + 12 * (size_t)(~left);
                float t;
                if (tri_t(mk(tp[0], tp[1], tp[2]), mk(tp[3], tp[4], tp[5]), mk(tp[6], tp[7], tp[8]), o, d, t))
                    if (t < h.t || (t == h.t && ~left < h.tri)) { h.t = t; h.tri = ~left; }
            } else {
                first = left;
            }
        }
        if (hr) {
            if (right < 0) {
                const float *tp = s.tris + 12 * (size_t)(~right);
                float t;
                if (tri_t(mk(tp[0], tp[1], tp[2]), mk(tp[3], tp[4], tp[5]), mk(tp[6], tp[7], tp[8]), o, d, t))
                    if (t < h.t || (t == h.t && ~right < h.tri)) { h.t = t; h.tri = ~right; }
            } else if (first < 0) {
                first = right;
            } else if (tr < tl) {
                second = first;
                first = right;
            } else {
                second = right;
            }
        }
        if (second >= 0) {
            if (top > RG_MAX_TREE_DEPTH) { h.tri = -1; return h; }
            stack[top++] = second;
        }
        if (first < 0) {
            if (top == 0) return h;
            first = stack[--top];
        }
        node = first;
    }
}

struct GTexel {
    uint32_t albedo;
    uint16_t normal[4];
    uint32_t material;
    float wpos[4];
    float depth;
};

RG_HD void primary_ray(const rg_camera &c, int px, int py, int w, int h, f3 &o, f3 &d) {
    const float ndc_x = (((float)px + 0.5f) / (float)w) * 2.0f - 1.0f;
    const float ndc_y = (((float)py + 0.5f) / (float)h) * 2.0f - 1.0f;
    const float vx = ndc_x * c.aspect * c.tan_half_fov_y;
    const float vy = ndc_y * c.tan_half_fov_y;
    const f3 right = mk(c.right[0], c.right[1], c.right[2]);
    const f3 up = mk(c.up[0], c.up[1], c.up[2]);
    const f3 fwd = mk(c.forward[0], c.forward[1], c.forward[2]);
    o = mk(c.position[0], c.position[1], c.position[2]);
    d = (scale(vx, right) - scale(vy, up)) + fwd;
}

RG_HD void shade_texel(const TraceScene &s, const rg_material *mats, int n_mats, const rg_camera &c, f3 o, f3 d,
                       const Hit &hit, GTexel &g) {
    if (hit.tri < 0) {
        g.albedo = 0u;
        g.normal[0] = g.normal[1] = g.normal[2] = g.normal[3] = 0;
        g.material = 0u;
        g.wpos[0] = g.wpos[1] = g.wpos[2] = g.wpos[3] = 0.0f;
        g.depth = 1.0f;
        return;
    }
    const float *tp = s.tris + 12 * (size_t)hit.tri;
    f3 n = normalize(cross(mk(tp[3], tp[4], tp[5]), mk(tp[6], tp[7], tp[8])));
    if (dot(n, d) > 0.0f) n = mk(-n.x, -n.y, -n.z);
    const f3 p = o + scale(hit.t, d);
    if (mats && hit.tri < n_mats) {
        const rg_material &m = mats[hit.tri];
        g.albedo = (uint32_t)m.albedo_srgb[0] | ((uint32_t)m.albedo_srgb[1] << 8) | ((uint32_t)m.albedo_srgb[2] << 16) |
                   ((uint32_t)m.albedo_srgb[3] << 24);
        g.material = (uint32_t)m.roughness_unorm | ((uint32_t)m.metallic_unorm << 16);
    } else {
        g.albedo = 0x00b4b4b4u;
        g.material = 0xffffu;
    }
    g.normal[0] = float_to_half_bits(n.x);
    g.normal[1] = float_to_half_bits(n.y);
    g.normal[2] = float_to_half_bits(n.z);
    g.normal[3] = 0;
    g.wpos[0] = p.x; g.wpos[1] = p.y; g.wpos[2] = p.z; g.wpos[3] = 1.0f;
    const float *m = c.projection_view;
    const float cz = ((m[2] * p.x + m[6] * p.y) + m[10] * p.z) + m[14] * 1.0f;
    const float cw = ((m[3] * p.x + m[7] * p.y) + m[11] * p.z) + m[15] * 1.0f;
    g.depth = cz / cw;
}

}  // namespace rgm
