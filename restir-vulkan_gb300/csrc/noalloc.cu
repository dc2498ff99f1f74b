// noalloc.cu -- a chain of unbiased spatial-reuse passes that allocates no
// device memory.
//
// rg_spatial_unbiased only runs one pass, and chaining several (as the frame
// driver does) needs a temporary reservoir buffer for the intermediate
// passes.  Some callers cannot provide one on demand: a renderer whose device
// memory budget is fixed up front, a host application that forbids
// allocations inside its frame loop (cudaMalloc and cudaFree can synchronise
// the whole device), or a caller whose device memory belongs to another
// framework's allocator.  rg_spatial_unbiased_chain_noalloc serves them: its
// intermediate reservoirs live in the file-scope array below, which the CUDA
// runtime places in device memory when the library is loaded on a GPU.
//
// Costs and limits of that choice:
//  - every GPU that loads this library holds the array (16 MiB) until the
//    process exits, whether or not the entry point is used;
//  - frames are limited to kNoAllocMaxPixels pixels (512 x 512);
//  - all calls share the one array, so calls whose work overlaps on the GPU
//    (other streams, other host threads) race; serialise them;
//  - the array's device address is looked up by the first call on a device
//    after a context is created there (rg_create forgets the cached address,
//    because a reset of the device's primary context unloads the module that
//    holds the array), so that call must come before any stream capture.
#include <cuda_runtime.h>

#include <mutex>

#include "rg_internal.h"

namespace {

// Largest frame (in pixels) the chain accepts: 512 x 512.
constexpr size_t kNoAllocMaxPixels = 512u * 512u;
constexpr int kMaxDevices = 64;

// Intermediate reservoirs of the chain (64 bytes each, 16 MiB in total).
static __device__ __align__(256) rg_reservoir g_chain_scratch[kNoAllocMaxPixels];

// Device address of g_chain_scratch, looked up once per device.  Host code
// must not use the symbol itself as a pointer: on the host it only names a
// stand-in object.
rg_reservoir *g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mutex;

int scratch_for_device(int device, rg_reservoir **out) {
    if (device < 0 || device >= kMaxDevices)
        return rg_internal_fail(RG_ERR_UNSUPPORTED, "rg_spatial_unbiased_chain_noalloc: device index above 63");
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (!g_scratch_addr[device]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_chain_scratch);  // the caller made `device` current
        if (e != cudaSuccess) {
            return rg_internal_fail(RG_ERR_CUDA, "rg_spatial_unbiased_chain_noalloc: cudaGetSymbolAddress failed");
        }
        g_scratch_addr[device] = static_cast<rg_reservoir *>(p);
    }
    *out = g_scratch_addr[device];
    return RG_OK;
}

}  // namespace

void noalloc_forget_device(int device) {
    if (device < 0 || device >= kMaxDevices) return;
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    g_scratch_addr[device] = nullptr;
}

extern "C" int rg_spatial_unbiased_chain_noalloc(rg_context *ctx, const rg_gbuffer *gbuf, const rg_reservoir *in,
                                                 rg_reservoir *out, const rg_restir_uniforms *u,
                                                 int32_t num_neighbors, int32_t num_passes, void *stream) {
    const DevScene *scene = nullptr;
    int device = 0;
    int rc = rg_internal_prepare(ctx, &scene, &device);  // also makes the context's device current
    if (rc) return rc;
    // the checks of rg_spatial_unbiased: every plane present and aligned for
    // the kernel's loads, distinct 16-byte aligned reservoir buffers
    if ((rc = rg_internal_check_spatial_args(gbuf, in, out, u))) return rc;
    if (scene->res_samples != 1 || scene->res_mis)
        return rg_internal_fail(RG_ERR_UNSUPPORTED,
                                "rg_spatial_unbiased_chain_noalloc: its scratch holds the default reservoir format");
    const size_t w = u->screen_size[0], h = u->screen_size[1];
    if (w * h > kNoAllocMaxPixels)
        return rg_internal_fail(RG_ERR_INVALID_ARGUMENT,
                                "rg_spatial_unbiased_chain_noalloc: frame larger than 262144 pixels (512x512), "
                                "the size of its built-in scratch buffer");
    if (num_neighbors < 0 || num_neighbors > 16 || num_passes < 1 || num_passes > 64)
        return rg_internal_fail(RG_ERR_INVALID_ARGUMENT,
                                "rg_spatial_unbiased_chain_noalloc: num_neighbors must be 0..16, num_passes 1..64");
    rg_reservoir *scratch = nullptr;
    if ((rc = scratch_for_device(device, &scratch))) return rc;
    // Pass k reads the previous pass's reservoirs and writes all w*h of its
    // own, so the scratch is fully overwritten before it is read: nothing
    // left from an earlier call is ever used and nothing needs clearing.
    // Buffers alternate so that the last pass writes `out`.
    const GBufView g = make_view(gbuf);
    const rg_reservoir *src = in;
    for (int k = 0; k < num_passes; ++k) {
        rg_reservoir *dst = ((num_passes - 1 - k) % 2 == 0) ? out : scratch;
        const cudaError_t e = launch_spatial_unbiased(*scene, g, src, dst, *u, num_neighbors, k, (cudaStream_t)stream);
        if (e != cudaSuccess)
            return rg_internal_fail(RG_ERR_CUDA, "rg_spatial_unbiased_chain_noalloc: kernel launch failed");
        src = dst;
    }
    return RG_OK;
}
