// batch.cu -- many views through the passes with one launch per pass
// (rg_batch_* in include/restir_gb300.h).
//
// A batch keeps, in device memory, the single-view kernels' parameter block of
// every view for both frame parities (which reservoir buffer is current), the
// tile maps of each pass and one work counter per launch.  A run is then
// stream work only: zero the counters, advance every view's frame index on the
// device, and launch RIS, the spatial passes and shading once each over all
// views.  Nothing is copied from the host and nothing is allocated, so a run
// can be captured into a CUDA graph once per parity and replayed.
//
// With the learned proposal (RG_FLAG_LEARNED_PROPOSAL on the views), a run
// first infers the proposal over all views' pixels (the two k_mlp_fused
// passes, each one launch over the concatenated pixels of every view) into
// the batch's own candidate buffer, whose slice of a view its RIS records
// point at.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <vector>

#include "mlp.cuh"
#include "rg_internal.h"

namespace {

int bfail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    return rg_internal_fail(code, buf);
}
int bcuda(cudaError_t e, const char *what) {
    return bfail(e == cudaErrorMemoryAllocation ? RG_ERR_OUT_OF_MEMORY : RG_ERR_CUDA, "%s: %s", what,
                 cudaGetErrorString(e));
}
#define B_CUDA(call, what)                           \
    do {                                             \
        cudaError_t e_ = (call);                     \
        if (e_ != cudaSuccess) return bcuda(e_, what); \
    } while (0)

struct TileMap {
    int32_t *view_start = nullptr, *tiles_x = nullptr;
    int32_t total = 0;
    int grid = 0;  // persistent CTAs of the pass's launch
};

}  // namespace

struct rg_batch {
    rg_context *ctx = nullptr;
    int device = 0;
    int n = 0;
    bool unbiased = true;
    int spatial = 0;     // spatial launches per run
    int neighbors = 0;
    int depth = 1;
    rg_batch_tuning tuning{4, 32, 0};
    std::vector<rg_view> views;
    // device
    unsigned char *initial[2] = {nullptr, nullptr};  // [n] parameter records per parity
    unsigned char *spatial_p[2] = {nullptr, nullptr};  // [spatial][n]
    unsigned char *shade[2] = {nullptr, nullptr};
    float4 *vcache[2] = {nullptr, nullptr};  // visibility cache, 2 float4 per pixel of all views, per buffer
    uint32_t *start_frame = nullptr, *runs = nullptr;
    unsigned *counters = nullptr;  // 2 + spatial
    TileMap maps[3];               // RIS, spatial, shade (for the current tuning)
    // learned proposal
    bool learned = false;
    uint64_t proposal_generation = 0;
    mlp::ProposalDev pd{};
    int *err = nullptr;            // the context's tensor-core timeout counter
    int64_t rows = 0;              // pixels of all views
    mlp::ViewRows *mlp_views = nullptr;
    uint32_t *view_frame = nullptr;
    float4 *stat = nullptr;
    mlp::Candidate *cand = nullptr;

    void release_maps() {
        for (auto &m : maps) {
            if (m.view_start) cudaFree(m.view_start);
            if (m.tiles_x) cudaFree(m.tiles_x);
            m = TileMap{};
        }
    }
    void release() {
        for (int k = 0; k < 2; ++k) {
            if (initial[k]) cudaFree(initial[k]);
            if (spatial_p[k]) cudaFree(spatial_p[k]);
            if (shade[k]) cudaFree(shade[k]);
            initial[k] = spatial_p[k] = shade[k] = nullptr;
        }
        for (int k = 0; k < 2; ++k) {
            if (vcache[k]) cudaFree(vcache[k]);
            vcache[k] = nullptr;
        }
        if (start_frame) cudaFree(start_frame);
        if (runs) cudaFree(runs);
        if (counters) cudaFree(counters);
        if (mlp_views) cudaFree(mlp_views);
        if (view_frame) cudaFree(view_frame);
        if (stat) cudaFree(stat);
        if (cand) cudaFree(cand);
        start_frame = runs = view_frame = nullptr;
        counters = nullptr;
        mlp_views = nullptr;
        stat = nullptr;
        cand = nullptr;
        release_maps();
    }
};

namespace {

int build_maps(rg_batch &b) {
    b.release_maps();
    const int variants[3] = {b.tuning.ris_pixels_per_thread, b.unbiased ? b.tuning.spatial_tile_width : 32, 0};
    for (int kind = 0; kind < 3; ++kind) {
        std::vector<int32_t> start((size_t)b.n), tx((size_t)b.n);
        int64_t total = 0;
        for (int v = 0; v < b.n; ++v) {
            int tw, th;
            view_tile_shape(kind, variants[kind], &tw, &th);
            const int w = (int)b.views[(size_t)v].uniforms.screen_size[0];
            const int h = (int)b.views[(size_t)v].uniforms.screen_size[1];
            start[(size_t)v] = (int32_t)total;
            tx[(size_t)v] = (w + tw - 1) / tw;
            total += (int64_t)tx[(size_t)v] * ((h + th - 1) / th);
        }
        if (total > 0x7fffffff) return bfail(RG_ERR_INVALID_ARGUMENT, "too many tiles");
        TileMap &m = b.maps[kind];
        m.total = (int32_t)total;
        B_CUDA(views_pass_grid(kind, variants[kind], b.unbiased, b.neighbors, b.depth, m.total, b.tuning.ctas_per_sm,
                               &m.grid),
               "persistent grid");
        B_CUDA(cudaMalloc(&m.view_start, (size_t)b.n * 4), "tile map");
        B_CUDA(cudaMalloc(&m.tiles_x, (size_t)b.n * 4), "tile map");
        B_CUDA(cudaMemcpy(m.view_start, start.data(), (size_t)b.n * 4, cudaMemcpyHostToDevice), "tile map");
        B_CUDA(cudaMemcpy(m.tiles_x, tx.data(), (size_t)b.n * 4, cudaMemcpyHostToDevice), "tile map");
    }
    return RG_OK;
}

int check_tuning(const rg_batch_tuning &t) {
    if (t.ris_pixels_per_thread != 1 && t.ris_pixels_per_thread != 2 && t.ris_pixels_per_thread != 4)
        return bfail(RG_ERR_INVALID_ARGUMENT, "ris_pixels_per_thread must be 1, 2 or 4");
    if (t.spatial_tile_width != 8 && t.spatial_tile_width != 16 && t.spatial_tile_width != 32)
        return bfail(RG_ERR_INVALID_ARGUMENT, "spatial_tile_width must be 8, 16 or 32");
    if (t.ctas_per_sm < 0 || t.ctas_per_sm > 32) return bfail(RG_ERR_INVALID_ARGUMENT, "ctas_per_sm must be 0..32");
    return RG_OK;
}

__global__ void k_set_view_candidates(mlp::ViewRows *v, int n, int32_t count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i].n_cand = count;
}

int enqueue_run(rg_batch *b, int parity, cudaStream_t st) {
    const int nl = 2 + b->spatial;
    B_CUDA(cudaMemsetAsync(b->counters, 0, (size_t)nl * sizeof(unsigned), st), "rg_batch_run");
    B_CUDA(launch_advance_frames(b->initial[parity], b->spatial_p[parity], b->n, b->spatial, b->start_frame, b->runs,
                                 b->view_frame, st),
           "frame advance");
    if (b->learned) {
        int *err = b->err;
        B_CUDA(mlp::forward_lse_views(b->pd, b->mlp_views, b->n, b->view_frame, (int)b->rows, b->stat, b->cand, err, st),
               "proposal lse over views");
        B_CUDA(mlp::forward_sample_views(b->pd, b->mlp_views, b->n, b->view_frame, (int)b->rows, b->stat, b->cand, err,
                                         st),
               "proposal sampling over views");
    }
    ViewTiles vt{b->maps[0].view_start, b->maps[0].tiles_x, b->n, b->maps[0].total, b->counters};
    B_CUDA(launch_views_pass(0, b->tuning.ris_pixels_per_thread, b->unbiased, b->neighbors, b->depth, b->initial[parity],
                             vt, b->maps[0].grid, st),
           "RIS over views");
    const size_t rec = view_params_size(1);
    for (int k = 0; k < b->spatial; ++k) {
        ViewTiles vs{b->maps[1].view_start, b->maps[1].tiles_x, b->n, b->maps[1].total, b->counters + 1 + k};
        B_CUDA(launch_views_pass(1, b->tuning.spatial_tile_width, b->unbiased, b->neighbors, b->depth,
                                 b->spatial_p[parity] + (size_t)k * b->n * rec, vs, b->maps[1].grid, st),
               "spatial pass over views");
    }
    ViewTiles vh{b->maps[2].view_start, b->maps[2].tiles_x, b->n, b->maps[2].total, b->counters + 1 + b->spatial};
    B_CUDA(launch_views_pass(2, 0, b->unbiased, b->neighbors, b->depth, b->shade[parity], vh, b->maps[2].grid, st),
           "shading over views");
    return RG_OK;
}

}  // namespace

extern "C" {

int rg_batch_create(rg_context *ctx, const rg_view *views, int32_t n_views, const rg_frame_params *fp,
                    const rg_batch_tuning *tuning, rg_batch **out) {
    const DevScene *s = nullptr;
    int device = 0;
    int rc = rg_internal_prepare(ctx, &s, &device);
    if (rc) return rc;
    if (!views || !fp || !out || n_views <= 0 || n_views > 65536) return bfail(RG_ERR_INVALID_ARGUMENT, "bad arguments");
    if (s->res_samples != 1 || s->res_mis) return bfail(RG_ERR_UNSUPPORTED, "batched views need the default reservoir format");
    *out = nullptr;
    const int passes = fp->spatial_iterations < 0 ? 0 : fp->spatial_iterations;
    if (fp->unbiased && (fp->unbiased_neighbors < 0 || fp->unbiased_neighbors > 16))
        return bfail(RG_ERR_INVALID_ARGUMENT, "unbiased_neighbors must be 0..16");
    for (int v = 0; v < n_views; ++v) {
        const rg_view &w = views[v];
        const uint32_t W = w.uniforms.screen_size[0], H = w.uniforms.screen_size[1];
        if (W == 0 || H == 0 || W > 32768 || H > 32768) return bfail(RG_ERR_INVALID_ARGUMENT, "view %d: bad size", v);
        const rg_gbuffer *gs[2] = {&w.cur, &w.prev};
        for (const rg_gbuffer *g : gs) {
            if ((uint32_t)g->width != W || (uint32_t)g->height != H || !g->albedo || !g->normal || !g->material ||
                !g->world_pos || !g->depth)
                return bfail(RG_ERR_INVALID_ARGUMENT, "view %d: G-buffer does not match its uniforms", v);
            if (((uintptr_t)g->normal & 7u) || ((uintptr_t)g->world_pos & 15u) || ((uintptr_t)g->albedo & 3u) ||
                ((uintptr_t)g->material & 3u) || ((uintptr_t)g->depth & 3u))
                return bfail(RG_ERR_INVALID_ARGUMENT, "view %d: misaligned G-buffer plane", v);
            if (!default_formats(make_view(g)) || g->_reserved != 0)
                return bfail(RG_ERR_UNSUPPORTED, "view %d: batched views take the default G-buffer formats", v);
        }
        if (!w.reservoirs[0] || !w.reservoirs[1] || !w.tmp || !w.rgba_out || ((uintptr_t)w.reservoirs[0] & 15u) ||
            ((uintptr_t)w.reservoirs[1] & 15u) || ((uintptr_t)w.tmp & 15u) || ((uintptr_t)w.rgba_out & 15u))
            return bfail(RG_ERR_INVALID_ARGUMENT, "view %d: null or misaligned buffer", v);
        if (((w.uniforms.flags ^ views[0].uniforms.flags) & RG_FLAG_LEARNED_PROPOSAL) != 0)
            return bfail(RG_ERR_INVALID_ARGUMENT, "view %d: RG_FLAG_LEARNED_PROPOSAL must be set on all views or none", v);
        if ((w.uniforms.flags & RG_FLAG_LEARNED_PROPOSAL) &&
            (w.uniforms.initial_light_sample_count < 1 || w.uniforms.initial_light_sample_count > (uint32_t)mlp::kCand))
            return bfail(RG_ERR_INVALID_ARGUMENT, "view %d: the learned proposal draws 1..%d candidates per pixel", v,
                         mlp::kCand);
    }
    const bool learned = (views[0].uniforms.flags & RG_FLAG_LEARNED_PROPOSAL) != 0;
    ProposalState *ps = learned ? *rg_internal_proposal(ctx) : nullptr;
    if (learned && !ps) return bfail(RG_ERR_INVALID_ARGUMENT, "RG_FLAG_LEARNED_PROPOSAL without a proposal");
    std::vector<int64_t> first_row((size_t)n_views + 1, 0);
    for (int v = 0; v < n_views; ++v)
        first_row[(size_t)v + 1] = first_row[(size_t)v] + (int64_t)views[v].uniforms.screen_size[0] *
                                                              (int64_t)views[v].uniforms.screen_size[1];
    if (learned && first_row[(size_t)n_views] > 0x7fffffff)
        return bfail(RG_ERR_INVALID_ARGUMENT, "the learned proposal batches at most 2^31 - 1 pixels");
    mlp::LearnedRis lr{};
    std::vector<mlp::ViewRows> vrows;
    uint64_t generation = 0;
    mlp::ProposalDev pd{};
    if (learned) {
        generation = proposal_batch_tables(ps, &pd, &lr);
        vrows.resize((size_t)n_views);
        for (int v = 0; v < n_views; ++v) {
            const rg_view &w = views[v];
            vrows[(size_t)v].g = make_view(&w.cur);
            for (int d = 0; d < 3; ++d) vrows[(size_t)v].cam[d] = w.uniforms.camera_pos[d];
            vrows[(size_t)v].first_row = (uint32_t)first_row[(size_t)v];
            vrows[(size_t)v].n_cand = (int32_t)w.uniforms.initial_light_sample_count;
        }
        B_CUDA(mlp::prepare_views(), "proposal kernel attributes");
    }
    rg_batch *b = new rg_batch();
    b->ctx = ctx;
    b->device = device;
    b->n = n_views;
    b->unbiased = fp->unbiased != 0;
    b->spatial = b->unbiased ? passes : 2 * passes;
    b->neighbors = fp->unbiased_neighbors;
    b->depth = s->depth;
    b->views.assign(views, views + n_views);
    b->learned = learned;
    b->proposal_generation = generation;
    b->pd = pd;
    b->err = s->mma_timeouts;
    b->rows = first_row[(size_t)n_views];
    if (learned) {
        cudaError_t ea = cudaMalloc(&b->mlp_views, (size_t)n_views * sizeof(mlp::ViewRows));
        if (ea == cudaSuccess)
            ea = cudaMemcpy(b->mlp_views, vrows.data(), (size_t)n_views * sizeof(mlp::ViewRows), cudaMemcpyHostToDevice);
        if (ea == cudaSuccess) ea = cudaMalloc(&b->view_frame, (size_t)n_views * 4);
        if (ea == cudaSuccess) ea = cudaMalloc(&b->stat, (size_t)b->rows * sizeof(float4));
        if (ea == cudaSuccess) ea = cudaMalloc(&b->cand, (size_t)b->rows * mlp::kCand * sizeof(mlp::Candidate));
        if (ea != cudaSuccess) {
            b->release();
            delete b;
            return bcuda(ea, "learned proposal buffers");
        }
    }
    if (tuning) {
        if ((rc = check_tuning(*tuning))) {
            delete b;
            return rc;
        }
        b->tuning = *tuning;
    }
    // the visibility cache (rg_set_visibility_cache): the RIS pass writes
    // buffer 1, unbiased pass k reads buffer (k + 1) % 2 and writes k % 2, so
    // every pass reads what the pass before it wrote; each pass rewrites every
    // pixel's entry, and the tag of a pass position pairs an entry's halves
    const bool vcache = b->unbiased && rg_internal_vcache_on(ctx);
    if (vcache) {
        cudaError_t ev = cudaSuccess;
        for (int k = 0; k < 2 && ev == cudaSuccess; ++k) {
            ev = cudaMalloc(&b->vcache[k], (size_t)b->rows * 2 * sizeof(float4));
            if (ev == cudaSuccess) ev = cudaMemset(b->vcache[k], 0, (size_t)b->rows * 2 * sizeof(float4));
        }
        if (ev != cudaSuccess) {
            b->release();
            delete b;
            return bcuda(ev, "visibility cache");
        }
    }
    // parameter records: the same pointer choices as rg_render_frame
    const size_t ri = view_params_size(0), rs = view_params_size(1), rh = view_params_size(2);
    std::vector<unsigned char> hi(ri * n_views), hs(rs * n_views * (size_t)(b->spatial > 0 ? b->spatial : 1)),
        hh(rh * n_views);
    std::vector<uint32_t> start((size_t)n_views);
    cudaError_t e = cudaSuccess;
    for (int parity = 0; parity < 2 && e == cudaSuccess; ++parity) {
        for (int v = 0; v < n_views; ++v) {
            const rg_view &w = views[v];
            const GBufView cur = make_view(&w.cur), prev = make_view(&w.prev);
            rg_reservoir *cur_res = w.reservoirs[parity], *prev_res = w.reservoirs[1 - parity];
            const rg_restir_uniforms &u = w.uniforms;
            start[(size_t)v] = u.frame;
            const bool temporal = (u.flags & RG_FLAG_TEMPORAL_REUSE) != 0;
            rg_reservoir *first = cur_res;
            if (b->unbiased && passes % 2 == 1) first = w.tmp;
            mlp::LearnedRis vlr = lr;
            if (learned) vlr.cand = b->cand + (size_t)first_row[(size_t)v] * mlp::kCand;
            const size_t px = (size_t)u.screen_size[0] * u.screen_size[1];
            auto vc_of = [&](int read_buf, int write_buf, uint32_t tag) {
                VisCache c;
                if (!vcache) return c;
                const size_t off = 2 * (size_t)first_row[(size_t)v];
                c.in = read_buf < 0 ? nullptr : b->vcache[read_buf] + off;
                c.out = b->vcache[write_buf] + off;
                c.tag = tag;
                c.n = (uint32_t)px;
                return c;
            };
            const VisCache vc_ris = vc_of(-1, 1, 1u);
            make_initial_params(hi.data() + ri * v, *s, cur, temporal ? &prev : nullptr, temporal ? prev_res : nullptr,
                                first, u, learned ? &vlr : nullptr, &vc_ris);
            if (b->unbiased) {
                rg_reservoir *src = first;
                for (int k = 0; k < passes; ++k) {
                    rg_reservoir *dst = (src == w.tmp) ? cur_res : w.tmp;
                    const VisCache vc_k = vc_of((k + 1) % 2, k % 2, 2u + (uint32_t)k);
                    make_spatial_params(hs.data() + rs * ((size_t)k * n_views + v), *s, cur, src, dst, u, true, k,
                                        b->neighbors, &vc_k);
                    src = dst;
                }
            } else {
                for (int j = 0; j < passes; ++j) {
                    make_spatial_params(hs.data() + rs * ((size_t)(2 * j) * n_views + v), *s, cur, cur_res, prev_res, u,
                                        false, 2 * j, 0);
                    make_spatial_params(hs.data() + rs * ((size_t)(2 * j + 1) * n_views + v), *s, cur, prev_res,
                                        cur_res, u, false, 2 * j + 1, 0);
                }
            }
            rg_lighting_uniforms lu;
            memset(&lu, 0, sizeof(lu));
            memcpy(lu.camera_pos, u.camera_pos, sizeof(lu.camera_pos));
            lu.buffer_size[0] = u.screen_size[0];
            lu.buffer_size[1] = u.screen_size[1];
            lu.gamma = fp->gamma > 0.0f ? fp->gamma : 1.0f;
            make_shade_params(hh.data() + rh * v, *s, cur, cur_res, lu, reinterpret_cast<float4 *>(w.rgba_out));
        }
        e = cudaMalloc(&b->initial[parity], hi.size());
        if (e == cudaSuccess) e = cudaMemcpy(b->initial[parity], hi.data(), hi.size(), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMalloc(&b->spatial_p[parity], hs.size());
        if (e == cudaSuccess) e = cudaMemcpy(b->spatial_p[parity], hs.data(), hs.size(), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMalloc(&b->shade[parity], hh.size());
        if (e == cudaSuccess) e = cudaMemcpy(b->shade[parity], hh.data(), hh.size(), cudaMemcpyHostToDevice);
    }
    if (e == cudaSuccess) e = cudaMalloc(&b->start_frame, (size_t)n_views * 4);
    if (e == cudaSuccess) e = cudaMemcpy(b->start_frame, start.data(), (size_t)n_views * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&b->runs, 4);
    if (e == cudaSuccess) e = cudaMemset(b->runs, 0, 4);
    if (e == cudaSuccess) e = cudaMalloc(&b->counters, (size_t)(2 + b->spatial) * sizeof(unsigned));
    if (e != cudaSuccess) {
        b->release();
        delete b;
        return bcuda(e, "rg_batch_create");
    }
    if ((rc = build_maps(*b))) {
        b->release();
        delete b;
        return rc;
    }
    *out = b;
    return RG_OK;
}

int rg_batch_run(rg_batch *b, int32_t parity, void *stream) {
    if (!b || (parity != 0 && parity != 1)) return bfail(RG_ERR_INVALID_ARGUMENT, "bad arguments");
    if (b->learned) {
        ProposalState *ps = *rg_internal_proposal(b->ctx);
        mlp::ProposalDev pd;
        mlp::LearnedRis lr;
        if (!ps || proposal_batch_tables(ps, &pd, &lr) != b->proposal_generation)
            return bfail(RG_ERR_INVALID_ARGUMENT, "the context's proposal changed since rg_batch_create");
    }
    int cur = -1;
    B_CUDA(cudaGetDevice(&cur), "cudaGetDevice");
    if (cur != b->device) B_CUDA(cudaSetDevice(b->device), "cudaSetDevice");
    return enqueue_run(b, parity, (cudaStream_t)stream);
}

int rg_batch_reset_frames(rg_batch *b, void *stream) {
    if (!b) return bfail(RG_ERR_INVALID_ARGUMENT, "null batch");
    B_CUDA(cudaSetDevice(b->device), "cudaSetDevice");
    B_CUDA(cudaMemsetAsync(b->runs, 0, 4, (cudaStream_t)stream), "rg_batch_reset_frames");
    return RG_OK;
}

int rg_batch_set_tuning(rg_batch *b, const rg_batch_tuning *t) {
    if (!b || !t) return bfail(RG_ERR_INVALID_ARGUMENT, "bad arguments");
    int rc = check_tuning(*t);
    if (rc) return rc;
    B_CUDA(cudaSetDevice(b->device), "cudaSetDevice");
    B_CUDA(cudaDeviceSynchronize(), "sync");
    b->tuning = *t;
    return build_maps(*b);
}

int rg_batch_get_tuning(rg_batch *b, rg_batch_tuning *t) {
    if (!b || !t) return bfail(RG_ERR_INVALID_ARGUMENT, "bad arguments");
    *t = b->tuning;
    return RG_OK;
}

int rg_batch_autotune(rg_batch *b, int32_t repeats, rg_batch_tuning *best_out, float *best_ms, void *stream) {
    if (!b || repeats < 1) return bfail(RG_ERR_INVALID_ARGUMENT, "bad arguments");
    B_CUDA(cudaSetDevice(b->device), "cudaSetDevice");
    cudaStream_t st = (cudaStream_t)stream;
    const int ppts[3] = {1, 2, 4};
    const int tws[3] = {8, 16, 32};
    const int ctas[3] = {0, 4, 2};
    rg_batch_tuning best = b->tuning;
    float best_t = 1e30f;
    cudaEvent_t e0, e1;
    B_CUDA(cudaEventCreate(&e0), "event");
    B_CUDA(cudaEventCreate(&e1), "event");
    int rc = RG_OK;
    for (int a = 0; a < 3 && rc == RG_OK; ++a)
        for (int c = 0; c < (b->unbiased ? 3 : 1) && rc == RG_OK; ++c)
            for (int d = 0; d < 3 && rc == RG_OK; ++d) {
                rg_batch_tuning t{ppts[a], b->unbiased ? tws[c] : 32, ctas[d]};
                if ((rc = rg_batch_set_tuning(b, &t))) break;
                if ((rc = enqueue_run(b, 0, st))) break;  // warm (attributes, caches)
                cudaError_t e = cudaEventRecord(e0, st);
                for (int k = 0; k < repeats && rc == RG_OK; ++k) rc = enqueue_run(b, k & 1, st);
                if (e == cudaSuccess) e = cudaEventRecord(e1, st);
                if (e == cudaSuccess) e = cudaEventSynchronize(e1);
                float ms = 0.0f;
                if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
                if (e != cudaSuccess) rc = bcuda(e, "autotune timing");
                if (rc == RG_OK && ms < best_t) {
                    best_t = ms;
                    best = t;
                }
            }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if ((rc = rg_batch_set_tuning(b, &best))) return rc;
    if (best_out) *best_out = best;
    if (best_ms) *best_ms = best_t / (float)repeats;
    return RG_OK;
}

int rg_batch_autotune_candidates(rg_batch *b, const int32_t *counts, int32_t n_counts, int32_t repeats,
                                 int32_t *best_count, float *ms_per_run, double *variance, void *stream) {
    if (!b || !counts || n_counts < 1 || n_counts > 16 || repeats < 1)
        return bfail(RG_ERR_INVALID_ARGUMENT, "bad arguments");
    for (int i = 0; i < n_counts; ++i)
        if (counts[i] < 1 || counts[i] > (b->learned ? mlp::kCand : 4096))
            return bfail(RG_ERR_INVALID_ARGUMENT, "candidate count %d out of range (1..%d)", counts[i],
                         b->learned ? mlp::kCand : 4096);
    B_CUDA(cudaSetDevice(b->device), "cudaSetDevice");
    cudaStream_t st = (cudaStream_t)stream;
    // per-view first pixel in one luminance buffer over all views
    std::vector<long long> first((size_t)b->n);
    long long total = 0;
    for (int v = 0; v < b->n; ++v) {
        first[(size_t)v] = total;
        total += (long long)b->views[(size_t)v].uniforms.screen_size[0] * b->views[(size_t)v].uniforms.screen_size[1];
    }
    float *lum = nullptr;
    long long *first_d = nullptr;
    double *acc = nullptr;
    unsigned *counter = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = RG_OK;
    auto cleanup = [&]() {
        if (lum) cudaFree(lum);
        if (first_d) cudaFree(first_d);
        if (acc) cudaFree(acc);
        if (counter) cudaFree(counter);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    };
    cudaError_t e = cudaMalloc(&lum, (size_t)total * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&first_d, (size_t)b->n * sizeof(long long));
    if (e == cudaSuccess) e = cudaMemcpy(first_d, first.data(), (size_t)b->n * sizeof(long long), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMalloc(&acc, 2 * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&counter, sizeof(unsigned));
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e != cudaSuccess) {
        cleanup();
        return bcuda(e, "candidate tuning buffers");
    }
    auto set_count = [&](int32_t c) -> cudaError_t {
        cudaError_t r = launch_set_candidates(b->initial[0], b->n, (uint32_t)c, st);
        if (r == cudaSuccess) r = launch_set_candidates(b->initial[1], b->n, (uint32_t)c, st);
        if (r == cudaSuccess && b->learned) {
            k_set_view_candidates<<<(b->n + 127) / 128, 128, 0, st>>>(b->mlp_views, b->n, c);
            r = cudaGetLastError();
        }
        return r;
    };
    const ViewTiles vt{b->maps[2].view_start, b->maps[2].tiles_x, b->n, b->maps[2].total, counter};
    double best_eff = -1.0;
    int32_t best = counts[0];
    for (int i = 0; i < n_counts && rc == RG_OK; ++i) {
        if ((e = set_count(counts[i])) != cudaSuccess) { rc = bcuda(e, "candidate count"); break; }
        if ((rc = enqueue_run(b, 0, st)) || (rc = enqueue_run(b, 1, st))) break;  // settle the reservoirs
        e = cudaEventRecord(e0, st);
        for (int k = 0; k < repeats && rc == RG_OK; ++k) rc = enqueue_run(b, k & 1, st);
        if (rc) break;
        if (e == cudaSuccess) e = cudaEventRecord(e1, st);
        // two runs from the same previous-frame reservoirs (parity 0 reads
        // reservoirs[1], written before): independent estimates of one frame
        if (e == cudaSuccess) e = cudaMemsetAsync(acc, 0, 2 * sizeof(double), st);
        if (e != cudaSuccess) { rc = bcuda(e, "candidate tuning"); break; }
        if ((rc = enqueue_run(b, 1, st))) break;
        if ((rc = enqueue_run(b, 0, st))) break;
        e = cudaMemsetAsync(counter, 0, sizeof(unsigned), st);
        if (e == cudaSuccess) e = launch_views_luminance(b->shade[0], vt, first_d, lum, 0, acc, b->maps[2].grid, st);
        if (e != cudaSuccess) { rc = bcuda(e, "luminance"); break; }
        if ((rc = enqueue_run(b, 0, st))) break;
        e = cudaMemsetAsync(counter, 0, sizeof(unsigned), st);
        if (e == cudaSuccess) e = launch_views_luminance(b->shade[0], vt, first_d, lum, 1, acc, b->maps[2].grid, st);
        double h[2] = {0.0, 0.0};
        if (e == cudaSuccess) e = cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        float ms = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        if (e != cudaSuccess) { rc = bcuda(e, "candidate tuning"); break; }
        ms /= (float)repeats;
        const double var = h[1] > 0.0 ? h[0] / (2.0 * h[1]) : 0.0;  // E[(a - b)^2] / 2 per pixel
        if (ms_per_run) ms_per_run[i] = ms;
        if (variance) variance[i] = var;
        const double eff = var > 0.0 ? 1.0 / ((double)ms * var) : 1e300 / (double)ms;
        if (eff > best_eff) {
            best_eff = eff;
            best = counts[i];
        }
    }
    if (rc == RG_OK) {
        if ((e = set_count(best)) != cudaSuccess) rc = bcuda(e, "candidate count");
        else if ((e = cudaStreamSynchronize(st)) != cudaSuccess) rc = bcuda(e, "candidate tuning");
    }
    cleanup();
    if (rc) return rc;
    for (auto &v : b->views) v.uniforms.initial_light_sample_count = (uint32_t)best;
    if (best_count) *best_count = best;
    return RG_OK;
}

int rg_batch_destroy(rg_batch *b) {
    if (!b) return RG_OK;
    cudaSetDevice(b->device);
    b->release();
    delete b;
    return RG_OK;
}

}  // extern "C"
