// proposal.cu -- the learned light-cluster proposal of a context: device
// state, initialisation, inference, gradients and the Adam step behind the
// rg_proposal_* entry points of include/restir_gb300.h.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <atomic>
#include <vector>

#include "host_internal.h"
#include "mlp.cuh"
#include "rg_internal.h"

namespace {

int pfail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    return rg_internal_fail(code, buf);
}
int pcuda(cudaError_t e, const char *what) {
    return pfail(e == cudaErrorMemoryAllocation ? RG_ERR_OUT_OF_MEMORY : RG_ERR_CUDA, "%s: %s", what,
                 cudaGetErrorString(e));
}
#define PR_CUDA(call, what)                          \
    do {                                             \
        cudaError_t e_ = (call);                     \
        if (e_ != cudaSuccess) return pcuda(e_, what); \
    } while (0)

template <typename T> cudaError_t alloc(T **p, size_t count) {
    *p = nullptr;
    if (count == 0) return cudaSuccess;
    return cudaMalloc(reinterpret_cast<void **>(p), count * sizeof(T));
}
template <typename T> void release(T *&p) {
    if (p) cudaFree(const_cast<void *>(static_cast<const void *>(p)));
    p = nullptr;
}

uint64_t splitmix(uint64_t &s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
double unit(uint64_t &s) { return (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0); }

}  // namespace

struct ProposalState {
    uint64_t generation = 0;  // distinct for every proposal created in the process
    int c = 0, n_lights = 0, batch = 0;
    float mix = 0.9f, lr = 1e-3f;
    float3 box_center{}, box_inv_half{};
    size_t n_params = 0;
    int step = 0;
    float *params = nullptr, *grad = nullptr, *adam_m = nullptr, *adam_v = nullptr;
    __nv_bfloat16 *w123img = nullptr, *w4t = nullptr, *w4k = nullptr, *w123 = nullptr, *w4 = nullptr;
    float *b4e = nullptr;
    uint8_t *valid = nullptr;
    int32_t *cluster_of = nullptr, *offset = nullptr;
    mlp::LearnedCol *lcol = nullptr;
    float *within = nullptr;
    int *err = nullptr;  // the context's tensor-core timeout counter (not owned)
    // inference
    size_t inf_cap = 0;
    float4 *stat = nullptr;
    mlp::Candidate *cand = nullptr;
    int cand_w = 0, cand_h = 0;
    uint32_t cand_frame = 0, cand_count = 0;
    bool cand_ready = false;
    // training
    int train_cap = 0;
    int32_t *rows = nullptr, *target = nullptr;
    float4 *tstat = nullptr;
    __nv_bfloat16 *x = nullptr, *h1 = nullptr, *h2 = nullptr, *h3 = nullptr;
    float *dh3 = nullptr;
    float *loss = nullptr;
    int *count = nullptr;
    bool has_loss = false;

    mlp::ProposalDev dev() const {
        mlp::ProposalDev d;
        d.c = c;
        d.n_lights = n_lights;
        d.mix = mix;
        d.box_center = box_center;
        d.box_inv_half = box_inv_half;
        d.params = params;
        d.b4e = b4e;
        d.w123img = w123img;
        d.w4t = w4t;
        d.w4k = w4k;
        d.w123 = w123;
        d.w4 = w4;
        d.cluster_valid = valid;
        d.cluster_of = cluster_of;
        return d;
    }
    void release_train() {
        release(rows); release(target); release(tstat); release(x); release(h1); release(h2); release(h3);
        release(dh3);
        train_cap = 0;
    }
    void release_all() {
        release(params); release(grad); release(adam_m); release(adam_v); release(w123img); release(w4t); release(w4k);
        release(w123); release(w4); release(b4e); release(valid); release(cluster_of); release(offset); release(lcol);
        release(within); release(stat); release(cand); release(loss); release(count);
        release_train();
        inf_cap = 0;
    }
};

void proposal_release(ProposalState *ps) {
    if (!ps) return;
    ps->release_all();
    delete ps;
}

namespace {

int get_state(rg_context *ctx, ProposalState **ps, const DevScene **scene = nullptr) {
    const DevScene *s = nullptr;
    int device = 0;
    int rc = rg_internal_prepare(ctx, &s, &device);
    if (rc) return rc;
    *ps = *rg_internal_proposal(ctx);
    if (!*ps) return pfail(RG_ERR_INVALID_ARGUMENT, "no proposal (rg_proposal_create)");
    if (scene) *scene = s;
    return RG_OK;
}

cudaError_t refresh_images(ProposalState &ps, cudaStream_t st) {
    return mlp::refresh(ps.params, ps.c, ps.valid, ps.w123img, ps.w4t, ps.w4k, ps.w123, ps.w4, ps.b4e, st);
}

int ensure_train(ProposalState &ps, int n) {
    if (n <= ps.train_cap) return RG_OK;
    ps.release_train();
    const size_t nn = (size_t)n;
    cudaError_t e = alloc(&ps.rows, nn);
    if (e == cudaSuccess) e = alloc(&ps.target, nn);
    if (e == cudaSuccess) e = alloc(&ps.tstat, nn);
    if (e == cudaSuccess) e = alloc(&ps.x, nn * mlp::kIn);
    if (e == cudaSuccess) e = alloc(&ps.h1, nn * mlp::kH);
    if (e == cudaSuccess) e = alloc(&ps.h2, nn * mlp::kH);
    if (e == cudaSuccess) e = alloc(&ps.h3, nn * mlp::kH);
    if (e == cudaSuccess) e = alloc(&ps.dh3, nn * mlp::kH);
    if (e != cudaSuccess) {
        ps.release_train();
        return pcuda(e, "proposal training buffers");
    }
    ps.train_cap = n;
    return RG_OK;
}

int check_gbuf(const rg_gbuffer *g) {
    if (!g || g->width <= 0 || g->height <= 0 || !g->normal || !g->world_pos)
        return pfail(RG_ERR_INVALID_ARGUMENT, "bad G-buffer");
    if (((uintptr_t)g->normal & 7u) || ((uintptr_t)g->world_pos & 15u))
        return pfail(RG_ERR_INVALID_ARGUMENT, "misaligned G-buffer plane");
    if (!default_formats(make_view(g)))
        return pfail(RG_ERR_UNSUPPORTED, "the learned proposal takes the default G-buffer formats");
    return RG_OK;
}

// Gradient of the mean loss over ps.rows/ps.target[0..n) into ps.grad.
int gradients(ProposalState &ps, const GBufView &g, const float cam[3], int n, cudaStream_t st) {
    const mlp::ProposalDev pd = ps.dev();
    const mlp::Layout L(ps.c);
    const mlp::TrainBuffers tb{ps.x, ps.h1, ps.h2, ps.h3};
    PR_CUDA(mlp::forward_lse(pd, g, cam, ps.rows, n, ps.tstat, &tb, 0, 0, nullptr, ps.err, st), "proposal forward");
    PR_CUDA(cudaMemsetAsync(ps.loss, 0, sizeof(float), st), "memset");
    PR_CUDA(cudaMemsetAsync(ps.grad, 0, ps.n_params * sizeof(float), st), "memset");
    // dh3 = dz W4^T and the loss (dz stays on chip), then dW4 and db4
    PR_CUDA(mlp::forward_grad(pd, g, cam, ps.rows, n, ps.tstat, ps.target, 1.0f / (float)n, ps.dh3, ps.loss, ps.err, st),
            "proposal logits gradient");
    PR_CUDA(mlp::dw4(pd, ps.h3, ps.tstat, ps.target, n, 1.0f / (float)n, ps.grad + L.w4, ps.grad + L.b4, ps.err, st),
            "dW4");
    // the hidden layers: weight and bias gradients from dh3
    PR_CUDA(mlp::backward_rows(ps.w123, tb, ps.dh3, ps.grad + L.w1, ps.grad + L.w2, ps.grad + L.w3, ps.grad + L.b1,
                               ps.grad + L.b2, ps.grad + L.b3, n, st),
            "hidden backward");
    return RG_OK;
}

}  // namespace

int proposal_learned_ris(ProposalState *ps, int w, int h, uint32_t frame, uint32_t count, mlp::LearnedRis *out) {
    if (!ps) return pfail(RG_ERR_INVALID_ARGUMENT, "RG_FLAG_LEARNED_PROPOSAL without a proposal");
    if (!ps->cand_ready || ps->cand_w != w || ps->cand_h != h || ps->cand_frame != frame || ps->cand_count != count)
        return pfail(RG_ERR_INVALID_ARGUMENT,
                     "learned candidates are for %dx%d frame %u (%u per pixel), not %dx%d frame %u (%u): "
                     "run rg_proposal_infer first",
                     ps->cand_w, ps->cand_h, ps->cand_frame, ps->cand_count, w, h, frame, count);
    mlp::ProposalDev dev;
    proposal_batch_tables(ps, &dev, out);
    out->cand = ps->cand;
    return RG_OK;
}

uint64_t proposal_batch_tables(ProposalState *ps, mlp::ProposalDev *dev, mlp::LearnedRis *out) {
    *dev = ps->dev();
    out->cand = nullptr;
    out->offset = ps->offset;
    out->lcol = ps->lcol;
    out->within = ps->within;
    out->mix = ps->mix;
    out->uniform_pdf = (1.0f - ps->mix) / (float)ps->n_lights;
    return ps->generation;
}

extern "C" {

int rg_cluster_lights(const rg_point_light *lights, int32_t n, int32_t k, int32_t iterations, uint64_t seed,
                      int32_t *cluster_of, float *centers_xyz) {
    if (!lights || !cluster_of || n <= 0 || k <= 0 || k > n || iterations < 0)
        return pfail(RG_ERR_INVALID_ARGUMENT, "rg_cluster_lights: bad arguments");
    std::vector<float> pos4((size_t)n * 4);
    for (int32_t i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) pos4[(size_t)i * 4 + d] = lights[i].pos[d];
    return host_kmeans(pos4.data(), n, k, iterations, seed, cluster_of, centers_xyz);
}

int64_t rg_proposal_param_count(int32_t clusters) {
    if (clusters <= 0) return 0;
    return (int64_t)mlp::Layout(clusters).total;
}

int rg_proposal_create(rg_context *ctx, const rg_proposal_config *cfg, const rg_point_light *lights, int32_t n,
                       const int32_t *cluster_of) {
    const DevScene *s = nullptr;
    int device = 0;
    int rc = rg_internal_prepare(ctx, &s, &device);
    if (rc) return rc;
    if (!cfg || !lights || !cluster_of) return pfail(RG_ERR_INVALID_ARGUMENT, "null argument");
    if (s->n_point_lights <= 0) return pfail(RG_ERR_UNSUPPORTED, "the learned proposal needs a point-light scene");
    if (n != s->n_point_lights)
        return pfail(RG_ERR_INVALID_ARGUMENT, "%d lights given, the scene has %d", n, s->n_point_lights);
    if (cfg->clusters < mlp::kChunkN || cfg->clusters % mlp::kChunkN != 0 || cfg->clusters > n)
        return pfail(RG_ERR_INVALID_ARGUMENT, "clusters must be a multiple of %d and at most the light count",
                     mlp::kChunkN);
    if (!(cfg->mix > 0.0f && cfg->mix < 1.0f)) return pfail(RG_ERR_INVALID_ARGUMENT, "mix must be in (0, 1)");
    if (cfg->batch <= 0 || cfg->batch > (1 << 22)) return pfail(RG_ERR_INVALID_ARGUMENT, "batch must be 1..4194304");
    if (!(cfg->learning_rate > 0.0f)) return pfail(RG_ERR_INVALID_ARGUMENT, "learning rate must be > 0");
    for (int d = 0; d < 3; ++d)
        if (!(cfg->box_max[d] > cfg->box_min[d])) return pfail(RG_ERR_INVALID_ARGUMENT, "empty normalisation box");
    const int C = cfg->clusters;
    std::vector<int32_t> order((size_t)n), offset((size_t)C + 1);
    std::vector<rg_alias_table_column> col((size_t)n);
    std::vector<float> within((size_t)n);
    rc = host_cluster_tables(lights, n, cluster_of, C, order.data(), offset.data(), col.data(), within.data());
    if (rc) return pfail(rc, "cluster ids must be in [0, clusters)");
    std::vector<mlp::LearnedCol> lcol((size_t)n);
    std::vector<uint8_t> valid((size_t)C);
    std::vector<double> power((size_t)C, 0.0);
    for (int32_t i = 0; i < n; ++i) power[(size_t)cluster_of[i]] += lights[i].color_luminance[3];
    for (int c = 0; c < C; ++c) valid[(size_t)c] = offset[(size_t)c + 1] > offset[(size_t)c] ? 1 : 0;
    for (int32_t pos = 0; pos < n; ++pos) {
        const rg_alias_table_column &cc = col[(size_t)pos];
        const int32_t own = order[(size_t)pos], ali = order[(size_t)cc.alias];
        float own_bits, ali_bits;
        memcpy(&own_bits, &own, 4);
        memcpy(&ali_bits, &ali, 4);
        const rg_point_light &a = lights[own], &b = lights[ali];
        lcol[(size_t)pos].col = make_float4(cc.prob, own_bits, ali_bits, cc.ori_prob);
        lcol[(size_t)pos].own_pos = make_float4(a.pos[0], a.pos[1], a.pos[2], a.color_luminance[3]);
        lcol[(size_t)pos].alias_pos = make_float4(b.pos[0], b.pos[1], b.pos[2], b.color_luminance[3]);
    }
    // initial parameters: He-uniform hidden weights, small W4, b4 = log(cluster luminance)
    const mlp::Layout L(C);
    std::vector<float> params(L.total, 0.0f);
    uint64_t st = cfg->seed;
    auto fill = [&](size_t off, int rows, int cols, int used_rows, double bound) {
        for (int r = 0; r < rows; ++r)
            for (int c2 = 0; c2 < cols; ++c2)
                params[off + (size_t)r * cols + c2] = r < used_rows ? (float)((2.0 * unit(st) - 1.0) * bound) : 0.0f;
    };
    fill(L.w1, mlp::kIn, mlp::kH, mlp::kInUsed, sqrt(6.0 / mlp::kInUsed));
    fill(L.w2, mlp::kH, mlp::kH, mlp::kH, sqrt(6.0 / mlp::kH));
    fill(L.w3, mlp::kH, mlp::kH, mlp::kH, sqrt(6.0 / mlp::kH));
    fill(L.w4, mlp::kH, C, mlp::kH, 0.01);
    for (int c = 0; c < C; ++c) params[L.b4 + (size_t)c] = power[(size_t)c] > 0.0 ? (float)log(power[(size_t)c]) : 0.0f;

    ProposalState **slot = rg_internal_proposal(ctx);
    proposal_release(*slot);
    *slot = nullptr;
    static std::atomic<uint64_t> generations{0};  // contexts may live on different host threads
    ProposalState *ps = new ProposalState();
    ps->generation = ++generations;
    ps->c = C;
    ps->n_lights = n;
    ps->batch = cfg->batch;
    ps->mix = cfg->mix;
    ps->lr = cfg->learning_rate;
    ps->box_center = make_float3(0.5f * (cfg->box_min[0] + cfg->box_max[0]), 0.5f * (cfg->box_min[1] + cfg->box_max[1]),
                                 0.5f * (cfg->box_min[2] + cfg->box_max[2]));
    ps->box_inv_half = make_float3(2.0f / (cfg->box_max[0] - cfg->box_min[0]), 2.0f / (cfg->box_max[1] - cfg->box_min[1]),
                                   2.0f / (cfg->box_max[2] - cfg->box_min[2]));
    ps->n_params = L.total;
    ps->err = s->mma_timeouts;
    const size_t n123 = (size_t)mlp::kIn * mlp::kH + 2 * (size_t)mlp::kH * mlp::kH;
    cudaError_t e = alloc(&ps->params, L.total);
    if (e == cudaSuccess) e = alloc(&ps->grad, L.total);
    if (e == cudaSuccess) e = alloc(&ps->adam_m, L.total);
    if (e == cudaSuccess) e = alloc(&ps->adam_v, L.total);
    if (e == cudaSuccess) e = alloc(&ps->w123img, n123);
    if (e == cudaSuccess) e = alloc(&ps->w4t, (size_t)mlp::kH * C);
    if (e == cudaSuccess) e = alloc(&ps->w4k, (size_t)mlp::kH * C);
    if (e == cudaSuccess) e = alloc(&ps->w123, n123);
    if (e == cudaSuccess) e = alloc(&ps->w4, (size_t)mlp::kH * C);
    if (e == cudaSuccess) e = alloc(&ps->b4e, (size_t)C);
    if (e == cudaSuccess) e = alloc(&ps->valid, (size_t)C);
    if (e == cudaSuccess) e = alloc(&ps->cluster_of, (size_t)n);
    if (e == cudaSuccess) e = alloc(&ps->offset, (size_t)C + 1);
    if (e == cudaSuccess) e = alloc(&ps->lcol, (size_t)n);
    if (e == cudaSuccess) e = alloc(&ps->within, (size_t)n);
    if (e == cudaSuccess) e = alloc(&ps->loss, 1);
    if (e == cudaSuccess) e = alloc(&ps->count, 1);
    if (e == cudaSuccess) e = cudaMemcpy(ps->params, params.data(), L.total * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(ps->adam_m, 0, L.total * 4);
    if (e == cudaSuccess) e = cudaMemset(ps->adam_v, 0, L.total * 4);
    if (e == cudaSuccess) e = cudaMemcpy(ps->valid, valid.data(), (size_t)C, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(ps->cluster_of, cluster_of, (size_t)n * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(ps->offset, offset.data(), ((size_t)C + 1) * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(ps->lcol, lcol.data(), (size_t)n * sizeof(mlp::LearnedCol), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(ps->within, within.data(), (size_t)n * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = refresh_images(*ps, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        proposal_release(ps);
        return pcuda(e, "rg_proposal_create");
    }
    *slot = ps;
    return RG_OK;
}

int rg_proposal_destroy(rg_context *ctx) {
    if (!ctx) return RG_OK;
    ProposalState **slot = rg_internal_proposal(ctx);
    proposal_release(*slot);
    *slot = nullptr;
    return RG_OK;
}

int rg_proposal_set_params(rg_context *ctx, const float *params, int64_t n) {
    ProposalState *ps = nullptr;
    int rc = get_state(ctx, &ps);
    if (rc) return rc;
    if (!params || n != (int64_t)ps->n_params)
        return pfail(RG_ERR_INVALID_ARGUMENT, "expected %lld parameters", (long long)ps->n_params);
    const mlp::Layout L(ps->c);
    std::vector<float> p(params, params + n);
    for (size_t i = L.w1 + (size_t)mlp::kInUsed * mlp::kH; i < L.w1 + (size_t)mlp::kIn * mlp::kH; ++i) p[i] = 0.0f;
    PR_CUDA(cudaDeviceSynchronize(), "sync");
    PR_CUDA(cudaMemcpy(ps->params, p.data(), ps->n_params * 4, cudaMemcpyHostToDevice), "set params");
    PR_CUDA(cudaMemset(ps->adam_m, 0, ps->n_params * 4), "reset Adam");
    PR_CUDA(cudaMemset(ps->adam_v, 0, ps->n_params * 4), "reset Adam");
    ps->step = 0;
    PR_CUDA(refresh_images(*ps, 0), "refresh");
    PR_CUDA(cudaDeviceSynchronize(), "sync");
    ps->cand_ready = false;
    return RG_OK;
}

int rg_proposal_get_params(rg_context *ctx, float *params, int64_t n) {
    ProposalState *ps = nullptr;
    int rc = get_state(ctx, &ps);
    if (rc) return rc;
    if (!params || n != (int64_t)ps->n_params)
        return pfail(RG_ERR_INVALID_ARGUMENT, "expected %lld parameters", (long long)ps->n_params);
    PR_CUDA(cudaDeviceSynchronize(), "sync");
    PR_CUDA(cudaMemcpy(params, ps->params, ps->n_params * 4, cudaMemcpyDeviceToHost), "get params");
    return RG_OK;
}

int rg_proposal_infer(rg_context *ctx, const rg_gbuffer *g, const rg_restir_uniforms *u, void *stream) {
    ProposalState *ps = nullptr;
    int rc = get_state(ctx, &ps);
    if (rc) return rc;
    if (!u) return pfail(RG_ERR_INVALID_ARGUMENT, "null uniforms");
    if ((rc = check_gbuf(g))) return rc;
    if ((uint32_t)g->width != u->screen_size[0] || (uint32_t)g->height != u->screen_size[1])
        return pfail(RG_ERR_INVALID_ARGUMENT, "G-buffer size does not match the uniforms");
    const uint32_t count = u->initial_light_sample_count;
    if (count < 1 || count > (uint32_t)mlp::kCand)
        return pfail(RG_ERR_INVALID_ARGUMENT, "the learned proposal draws 1..%d candidates per pixel", mlp::kCand);
    const size_t np = (size_t)g->width * (size_t)g->height;
    if (np > (size_t)0x7fffffff) return pfail(RG_ERR_INVALID_ARGUMENT, "frame too large");
    if (np > ps->inf_cap) {
        release(ps->stat);
        release(ps->cand);
        ps->inf_cap = 0;
        cudaError_t e = alloc(&ps->stat, np);
        if (e == cudaSuccess) e = alloc(&ps->cand, np * mlp::kCand);
        if (e != cudaSuccess) {
            release(ps->stat);
            release(ps->cand);
            return pcuda(e, "proposal inference buffers");
        }
        ps->inf_cap = np;
    }
    cudaStream_t st = (cudaStream_t)stream;
    const GBufView gv = make_view(g);
    const mlp::ProposalDev pd = ps->dev();
    PR_CUDA(mlp::forward_lse(pd, gv, u->camera_pos, nullptr, (int)np, ps->stat, nullptr, u->frame, (int)count,
                             ps->cand, ps->err, st),
            "proposal lse");
    PR_CUDA(mlp::forward_sample(pd, gv, u->camera_pos, (int)np, ps->stat, u->frame, (int)count, ps->cand, ps->err, st),
            "proposal sample");
    ps->cand_ready = true;
    ps->cand_w = g->width;
    ps->cand_h = g->height;
    ps->cand_frame = u->frame;
    ps->cand_count = count;
    return RG_OK;
}

int rg_proposal_buffers(rg_context *ctx, const rg_proposal_candidate **candidates, const float **row_stats) {
    ProposalState *ps = nullptr;
    int rc = get_state(ctx, &ps);
    if (rc) return rc;
    if (!ps->cand_ready) return pfail(RG_ERR_INVALID_ARGUMENT, "no inference run yet");
    if (candidates) *candidates = reinterpret_cast<const rg_proposal_candidate *>(ps->cand);
    if (row_stats) *row_stats = reinterpret_cast<const float *>(ps->stat);
    return RG_OK;
}

int rg_proposal_gradients(rg_context *ctx, const rg_gbuffer *g, const float cam[3], const int32_t *rows,
                          const int32_t *targets, int32_t n, float *grad, double *loss_sum, void *stream) {
    ProposalState *ps = nullptr;
    int rc = get_state(ctx, &ps);
    if (rc) return rc;
    if ((rc = check_gbuf(g))) return rc;
    if (!cam || !rows || !targets || !grad || n <= 0) return pfail(RG_ERR_INVALID_ARGUMENT, "bad arguments");
    std::vector<int32_t> hr((size_t)n), ht((size_t)n);
    cudaStream_t st = (cudaStream_t)stream;
    PR_CUDA(cudaStreamSynchronize(st), "sync");
    PR_CUDA(cudaMemcpy(hr.data(), rows, (size_t)n * 4, cudaMemcpyDeviceToHost), "rows");
    PR_CUDA(cudaMemcpy(ht.data(), targets, (size_t)n * 4, cudaMemcpyDeviceToHost), "targets");
    const int64_t np = (int64_t)g->width * g->height;
    for (int32_t i = 0; i < n; ++i) {
        if (hr[(size_t)i] < 0 || hr[(size_t)i] >= np) return pfail(RG_ERR_INVALID_ARGUMENT, "row %d out of range", i);
        if (ht[(size_t)i] < -1 || ht[(size_t)i] >= ps->c) return pfail(RG_ERR_INVALID_ARGUMENT, "target %d out of range", i);
    }
    if ((rc = ensure_train(*ps, n))) return rc;
    PR_CUDA(cudaMemcpyAsync(ps->rows, rows, (size_t)n * 4, cudaMemcpyDeviceToDevice, st), "rows");
    PR_CUDA(cudaMemcpyAsync(ps->target, targets, (size_t)n * 4, cudaMemcpyDeviceToDevice, st), "targets");
    if ((rc = gradients(*ps, make_view(g), cam, n, st))) return rc;
    PR_CUDA(cudaMemcpyAsync(grad, ps->grad, ps->n_params * 4, cudaMemcpyDeviceToDevice, st), "grad");
    if (loss_sum) {
        float l = 0.0f;
        PR_CUDA(cudaMemcpyAsync(&l, ps->loss, 4, cudaMemcpyDeviceToHost, st), "loss");
        PR_CUDA(cudaStreamSynchronize(st), "sync");
        *loss_sum = l;
    }
    return RG_OK;
}

int rg_proposal_train(rg_context *ctx, const rg_gbuffer *g, const rg_restir_uniforms *u, const rg_reservoir *res,
                      void *stream) {
    ProposalState *ps = nullptr;
    const DevScene *scene = nullptr;
    int rc = get_state(ctx, &ps, &scene);
    if (rc) return rc;
    if (scene->res_samples != 1 || scene->res_mis)
        return pfail(RG_ERR_UNSUPPORTED, "training reads the default reservoir format");
    if (!u || !res || ((uintptr_t)res & 15u)) return pfail(RG_ERR_INVALID_ARGUMENT, "bad arguments");
    if ((rc = check_gbuf(g))) return rc;
    if ((uint32_t)g->width != u->screen_size[0] || (uint32_t)g->height != u->screen_size[1])
        return pfail(RG_ERR_INVALID_ARGUMENT, "G-buffer size does not match the uniforms");
    const uint32_t np = (uint32_t)g->width * (uint32_t)g->height;
    const int n = (int)(ps->batch < (int)np ? ps->batch : (int)np);
    if ((rc = ensure_train(*ps, n))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const uint32_t stride = np / (uint32_t)n;
    uint64_t h = 0x51ED2701ULL + u->frame;
    const uint32_t offset = (uint32_t)(splitmix(h) % np);
    PR_CUDA(mlp::batch_rows(ps->rows, n, np, offset, stride, st), "batch rows");
    PR_CUDA(cudaMemsetAsync(ps->count, 0, sizeof(int), st), "memset");
    PR_CUDA(mlp::targets(res, ps->rows, n, ps->cluster_of, ps->n_lights, ps->target, ps->count, st), "targets");
    if ((rc = gradients(*ps, make_view(g), u->camera_pos, n, st))) return rc;
    ++ps->step;
    PR_CUDA(mlp::adam(ps->params, ps->grad, ps->adam_m, ps->adam_v, ps->n_params, ps->lr, ps->step, ps->c, st), "Adam");
    PR_CUDA(refresh_images(*ps, st), "refresh");
    ps->has_loss = true;
    return RG_OK;
}

int rg_proposal_last_loss(rg_context *ctx, double *mean_loss, int64_t *rows_with_target) {
    ProposalState *ps = nullptr;
    int rc = get_state(ctx, &ps);
    if (rc) return rc;
    if (!ps->has_loss) return pfail(RG_ERR_INVALID_ARGUMENT, "no training step yet");
    PR_CUDA(cudaDeviceSynchronize(), "sync");
    float l = 0.0f;
    int cnt = 0;
    PR_CUDA(cudaMemcpy(&l, ps->loss, 4, cudaMemcpyDeviceToHost), "loss");
    PR_CUDA(cudaMemcpy(&cnt, ps->count, 4, cudaMemcpyDeviceToHost), "count");
    if (mean_loss) *mean_loss = cnt > 0 ? (double)l / (double)cnt : 0.0;
    if (rows_with_target) *rows_with_target = cnt;
    return RG_OK;
}

}  // extern "C"
