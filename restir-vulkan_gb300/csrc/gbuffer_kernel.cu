// gbuffer_kernel.cu -- primary-ray G-buffer on the GPU (one thread per pixel,
// closest hit on the uploaded tree).  Shares every operation with the host
// tracer through rg_gbuffer.cuh, so both write identical planes.
#include <cuda_runtime.h>

#include "rg_gbuffer.cuh"
#include "rg_internal.h"

namespace {

struct GbufParams {
    rgm::TraceScene s;
    const rg_material *mats;
    int n_mats;
    rg_camera cam;
    int w, h;
    uint32_t *albedo;
    uint2 *normal;
    uint32_t *material;
    float4 *wpos;
    float *depth;
};

__global__ void __launch_bounds__(128) k_trace_gbuffer(const GbufParams p) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= p.w || y >= p.h) return;
    rgm::f3 o, d;
    rgm::primary_ray(p.cam, x, y, p.w, p.h, o, d);
    const rgm::Hit hit = rgm::closest_hit(p.s, o, d);
    rgm::GTexel g;
    rgm::shade_texel(p.s, p.mats, p.n_mats, p.cam, o, d, hit, g);
    const size_t i = (size_t)y * (size_t)p.w + (size_t)x;
    p.albedo[i] = g.albedo;
    p.normal[i] = make_uint2((uint32_t)g.normal[0] | ((uint32_t)g.normal[1] << 16),
                             (uint32_t)g.normal[2] | ((uint32_t)g.normal[3] << 16));
    p.material[i] = g.material;
    p.wpos[i] = make_float4(g.wpos[0], g.wpos[1], g.wpos[2], g.wpos[3]);
    p.depth[i] = g.depth;
}

}  // namespace

cudaError_t launch_trace_gbuffer(const DevScene &s, const rg_camera &cam, const rg_gbuffer_out &out, cudaStream_t st) {
    GbufParams p;
    p.s.nodes = reinterpret_cast<const float *>(s.nodes);
    p.s.n_nodes = s.n_nodes;
    p.s.tris = reinterpret_cast<const float *>(s.tris);
    p.s.n_tris = s.n_tris;
    p.mats = s.materials;
    p.n_mats = s.n_materials;
    p.cam = cam;
    p.w = out.width;
    p.h = out.height;
    p.albedo = static_cast<uint32_t *>(out.albedo);
    p.normal = static_cast<uint2 *>(out.normal);
    p.material = static_cast<uint32_t *>(out.material);
    p.wpos = static_cast<float4 *>(out.world_pos);
    p.depth = static_cast<float *>(out.depth);
    const dim3 block(16, 8);
    const dim3 grid((unsigned)((out.width + 15) / 16), (unsigned)((out.height + 7) / 8));
    k_trace_gbuffer<<<grid, block, 0, st>>>(p);
    return cudaGetLastError();
}
