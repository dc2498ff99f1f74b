// kernels.cu -- sm_103a kernels of the ReSTIR direct-lighting passes.
//
// One thread per pixel for the reservoir passes; shadow segments are traced
// with an any-hit walk of the reference's 2-wide AABB tree.  Any-hit is an OR
// over every triangle whose whole box path passes the slab test, so the walk
// may visit nodes in any order and test a leaf as soon as it is reached: the
// visibility bit equals that of the reference's batched stack walk
// (src/shaders/include/softwareRaytracing.glsl:42-85) whenever the latter
// does not overflow its 32-entry stack.
//
// Compiled with -fmad=false and IEEE div/sqrt: see rg_math.cuh.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "mlp.cuh"
#include "rg_internal.h"
#include "rg_math.cuh"
#include "trace_pool.cuh"

using namespace rgm;

__device__ float g_srgb_lut[256];

cudaError_t upload_srgb_lut(const float *lut256) {
    return cudaMemcpyToSymbol(g_srgb_lut, lut256, 256 * sizeof(float));
}

namespace {


struct Texel {
    f3 albedo;
    float albedo_a;
    f3 normal;
    float roughness, metallic;
    f3 wpos;
};

__device__ __forceinline__ f3 load_albedo(const GBufView &g, size_t i, float *alpha) {
    const uint32_t a = __ldg(g.albedo + i);
    if (alpha) *alpha = (float)(a >> 24) / 255.0f;
    return mk(__ldg(&g_srgb_lut[a & 0xffu]), __ldg(&g_srgb_lut[(a >> 8) & 0xffu]), __ldg(&g_srgb_lut[(a >> 16) & 0xffu]));
}
// SNORM16 -> float: max(c / 32767, -1), Vulkan's conversion from normalized
// fixed point (IEEE division).
__device__ __forceinline__ float snorm16(uint16_t c) { return fmaxf((float)(int16_t)c / 32767.0f, -1.0f); }

// The reference's normal attachment candidates (gBufferPass.cpp:81-89);
// nfmt is warp-uniform, so the switch costs a uniform branch.
__device__ __forceinline__ f3 load_normal(const GBufView &g, size_t i) {
    if (g.nfmt == 0) {
        const uint2 n = __ldg(g.normal + i);
        return mk(half_bits_to_float((uint16_t)(n.x & 0xffffu)), half_bits_to_float((uint16_t)(n.x >> 16)),
                  half_bits_to_float((uint16_t)(n.y & 0xffffu)));
    }
    if (g.nfmt == RG_FORMAT_R16G16B16A16_SNORM) {
        const uint2 n = __ldg(g.normal + i);
        return mk(snorm16((uint16_t)(n.x & 0xffffu)), snorm16((uint16_t)(n.x >> 16)), snorm16((uint16_t)(n.y & 0xffffu)));
    }
    if (g.nfmt == RG_FORMAT_R32G32B32_SFLOAT) {
        const float *p = reinterpret_cast<const float *>(g.normal) + 3 * i;
        return mk(__ldg(p), __ldg(p + 1), __ldg(p + 2));
    }
    const unsigned short *p = reinterpret_cast<const unsigned short *>(g.normal) + 3 * i;
    const uint16_t a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
    if (g.nfmt == RG_FORMAT_R16G16B16_SNORM) return mk(snorm16(a), snorm16(b), snorm16(c));
    return mk(half_bits_to_float(a), half_bits_to_float(b), half_bits_to_float(c));  // R16G16B16_SFLOAT
}
// depth: D32F (also the depth plane of D32_SFLOAT_S8_UINT) or the low 24 bits
// of D24_UNORM_S8_UINT's 32-bit words over 2^24 - 1.
__device__ __forceinline__ float load_depth(const GBufView &g, size_t i) {
    if (g.dfmt == 0) return __ldg(g.depth + i);
    const uint32_t w = __ldg(reinterpret_cast<const uint32_t *>(g.depth) + i);
    return (float)(w & 0xffffffu) / 16777215.0f;
}
__device__ __forceinline__ void load_material(const GBufView &g, size_t i, float &rough, float &metal) {
    const uint32_t m = __ldg(g.material + i);
    rough = (float)(m & 0xffffu) / 65535.0f;
    metal = (float)(m >> 16) / 65535.0f;
}
__device__ __forceinline__ f3 load_wpos(const GBufView &g, size_t i) {
    if (g.pfmt == 0) {
        const float4 p = __ldg(g.wpos + i);
        return mk(p.x, p.y, p.z);
    }
    const float *p = reinterpret_cast<const float *>(g.wpos) + 3 * i;  // R32G32B32_SFLOAT
    return mk(__ldg(p), __ldg(p + 1), __ldg(p + 2));
}
__device__ __forceinline__ void load_texel(const GBufView &g, size_t i, Texel &t) {
    t.albedo = load_albedo(g, i, &t.albedo_a);
    t.normal = load_normal(g, i);
    load_material(g, i, t.roughness, t.metallic);
    t.wpos = load_wpos(g, i);
}

template <int R_, bool MIS_>
struct FormatTag {
    static constexpr int R = R_;
    static constexpr bool MIS = MIS_;
};

// ---------------------------------------------------------------- reservoirs
// Reservoir with R samples (RESERVOIR_SIZE) and, with MIS (UNBIASED_MIS), a
// sumPHat per sample (restirStructs.glsl:16-34).  In memory: the std430
// layout, R LightSamples of 48 bytes (64 with MIS) then numStreamSamples,
// padded to 16 bytes; R = 1 without MIS is rg_reservoir (64 bytes).
template <int R, bool MIS>
struct ResV {
    float4 pos_lum[R];
    float4 nrm[R];
    int32_t idx[R];
    float p_hat[R], sum_w[R], w[R];
    float sum_phat[MIS ? R : 1];
    uint32_t m;
};
template <int R, bool MIS>
struct ResLayout {
    static constexpr int kSample4 = MIS ? 4 : 3;          // float4 words per sample
    static constexpr int kWords = R * kSample4 + 1;       // float4 words per reservoir
};

template <int R, bool MIS>
__device__ __forceinline__ ResV<R, MIS> load_resv(const rg_reservoir *base, size_t i) {
    using L = ResLayout<R, MIS>;
    const float4 *p = reinterpret_cast<const float4 *>(base) + i * L::kWords;
    ResV<R, MIS> r;
#pragma unroll
    for (int j = 0; j < R; ++j) {
        r.pos_lum[j] = __ldg(p + j * L::kSample4);
        r.nrm[j] = __ldg(p + j * L::kSample4 + 1);
        const float4 c = __ldg(p + j * L::kSample4 + 2);
        r.idx[j] = __float_as_int(c.x);
        r.p_hat[j] = c.y;
        r.sum_w[j] = c.z;
        r.w[j] = c.w;
        if (MIS) r.sum_phat[j] = __ldg(p + j * L::kSample4 + 3).x;
    }
    r.m = __float_as_uint(__ldg(p + R * L::kSample4).x);
    return r;
}
// load_resv with coherent loads, for a reservoir this thread wrote earlier in
// the same kernel (the read-only path may only read data that no thread of
// the kernel writes).
template <int R, bool MIS>
__device__ __forceinline__ ResV<R, MIS> load_resv_own(const rg_reservoir *base, size_t i) {
    using L = ResLayout<R, MIS>;
    const float4 *p = reinterpret_cast<const float4 *>(base) + i * L::kWords;
    ResV<R, MIS> r;
#pragma unroll
    for (int j = 0; j < R; ++j) {
        r.pos_lum[j] = p[j * L::kSample4];
        r.nrm[j] = p[j * L::kSample4 + 1];
        const float4 c = p[j * L::kSample4 + 2];
        r.idx[j] = __float_as_int(c.x);
        r.p_hat[j] = c.y;
        r.sum_w[j] = c.z;
        r.w[j] = c.w;
        if (MIS) r.sum_phat[j] = p[j * L::kSample4 + 3].x;
    }
    r.m = __float_as_uint(p[R * L::kSample4].x);
    return r;
}
template <int R, bool MIS>
__device__ __forceinline__ void store_resv(rg_reservoir *base, size_t i, const ResV<R, MIS> &r) {
    using L = ResLayout<R, MIS>;
    float4 *p = reinterpret_cast<float4 *>(base) + i * L::kWords;
#pragma unroll
    for (int j = 0; j < R; ++j) {
        p[j * L::kSample4] = r.pos_lum[j];
        p[j * L::kSample4 + 1] = r.nrm[j];
        p[j * L::kSample4 + 2] = make_float4(__int_as_float(r.idx[j]), r.p_hat[j], r.sum_w[j], r.w[j]);
        if (MIS) p[j * L::kSample4 + 3] = make_float4(r.sum_phat[j], 0.0f, 0.0f, 0.0f);
    }
    p[R * L::kSample4] = make_float4(__uint_as_float(r.m), 0.0f, 0.0f, 0.0f);
}

template <int R, bool MIS>
__device__ __forceinline__ ResV<R, MIS> empty_resv() {
    ResV<R, MIS> r;
#pragma unroll
    for (int j = 0; j < R; ++j) {
        r.pos_lum[j] = make_float4(0.f, 0.f, 0.f, 0.f);
        r.nrm[j] = make_float4(0.f, 0.f, 0.f, 0.f);
        r.idx[j] = 0;
        r.p_hat[j] = 0.f;
        r.sum_w[j] = 0.f;
        r.w[j] = 0.f;
        if (MIS) r.sum_phat[j] = 0.f;
    }
    r.m = 0u;
    return r;
}
// reservoir.glsl:6-26
template <int R, bool MIS>
__device__ __forceinline__ void update_at(ResV<R, MIS> &r, int j, float weight, float4 pos_lum, float4 nrm,
                                          int32_t idx, float p_hat, float w, float sum_phat, Pcg &rng) {
    r.sum_w[j] += weight;
    const float replace = weight / r.sum_w[j];
    if (rand_float(rng) < replace) {
        r.pos_lum[j] = pos_lum;
        r.nrm[j] = nrm;
        r.idx[j] = idx;
        r.p_hat[j] = p_hat;
        r.w[j] = w;
        if (MIS) r.sum_phat[j] += sum_phat;
    }
}
// reservoir.glsl:28-42
template <int R, bool MIS>
__device__ __forceinline__ void add_sample(ResV<R, MIS> &r, float4 pos_lum, float4 nrm, int32_t idx, float p_hat,
                                           float sample_p, Pcg &rng) {
    const float weight = p_hat / sample_p;
    r.m += 1u;
#pragma unroll
    for (int j = 0; j < R; ++j) {
        const float w = (r.sum_w[j] + weight) / ((float)r.m * p_hat);
        update_at(r, j, weight, pos_lum, nrm, idx, p_hat, w, p_hat, rng);
    }
}
// add_sample with the reservoir-update uniforms drawn beforehand (u[j] is the
// draw update_at would take for sample j): the same arithmetic.
template <int R, bool MIS>
__device__ __forceinline__ void add_sample_u(ResV<R, MIS> &r, float4 pos_lum, float4 nrm, int32_t idx, float p_hat,
                                             float sample_p, const float (&u)[R]) {
    const float weight = p_hat / sample_p;
    r.m += 1u;
#pragma unroll
    for (int j = 0; j < R; ++j) {
        const float w = (r.sum_w[j] + weight) / ((float)r.m * p_hat);
        r.sum_w[j] += weight;
        const float replace = weight / r.sum_w[j];
        if (u[j] < replace) {
            r.pos_lum[j] = pos_lum;
            r.nrm[j] = nrm;
            r.idx[j] = idx;
            r.p_hat[j] = p_hat;
            r.w[j] = w;
            if (MIS) r.sum_phat[j] += p_hat;
        }
    }
}
// reservoir.glsl:44-64.  With MIS the reference passes other's sumPHat where
// updateReservoirAt takes w and other's w where it takes sumPHat (:55-60);
// RG_FLAG_MIS_SWAP_FIX passes them in the declared order instead.
template <int R, bool MIS>
__device__ __forceinline__ void combine_res(ResV<R, MIS> &self, const ResV<R, MIS> &other, const float (&p_hat)[R],
                                            bool swap_fix, Pcg &rng) {
    self.m += other.m;
#pragma unroll
    for (int j = 0; j < R; ++j) {
        const float weight = p_hat[j] * other.w[j] * (float)other.m;
        if (weight > 0.0f) {
            const float osp = MIS ? other.sum_phat[j] : 0.0f;
            const float wv = (MIS && !swap_fix) ? osp : other.w[j];
            const float sp = (MIS && !swap_fix) ? other.w[j] : osp;
            update_at(self, j, weight, other.pos_lum[j], other.nrm[j], other.idx[j], p_hat[j], wv, sp, rng);
        }
        if (self.w[j] > 0.0f) self.w[j] = self.sum_w[j] / ((float)self.m * self.p_hat[j]);
    }
}

__device__ __forceinline__ f3 xyz(float4 v) { return mk(v.x, v.y, v.z); }

// ---------------------------------------------------------------- shadow rays
// Adds a block's ray count (passed by one thread) and its lanes' traversal
// counters to the context's counters: one atomic per warp and counter.
__device__ __forceinline__ void count_block_rays(const DevScene &s, int rays, const rgpool::TraceStats &ts) {
    constexpr unsigned kFull = 0xffffffffu;
    const unsigned errs = __popc(__ballot_sync(kFull, ts.err));
    const unsigned visits = __reduce_add_sync(kFull, ts.visits);
    const unsigned tris = __reduce_add_sync(kFull, ts.tri_tests);
    const unsigned skipped = __reduce_add_sync(kFull, ts.skipped);
    const int tid = threadIdx.x + threadIdx.y * blockDim.x;
    if ((tid & 31) == 0) {
        // segments the pool skipped are not traced: subtracted from the
        // block's count (modular 64-bit addition; the total stays exact)
        if (skipped) atomicAdd(&s.counters[0], 0ull - (unsigned long long)skipped);
        if (errs) atomicAdd(&s.counters[1], (unsigned long long)errs);
        if (visits) atomicAdd(&s.counters[2], (unsigned long long)visits);
        if (tris) atomicAdd(&s.counters[3], (unsigned long long)tris);
    }
    if (tid == 0 && rays) atomicAdd(&s.counters[0], (unsigned long long)rays);
}

// ---------------------------------------------------------------- RIS + visibility + temporal (restirOmni.glsl:86-212)
// A block of 32x4 threads covers a 32 x (4*PPT) pixel tile, PPT pixels per thread:
//   1. RIS for each pixel; the reservoir goes to `out`, the PCG state stays in
//      registers, the visibility-reuse segment goes to the block's ray pool;
//   2. the block traces its pool (trace_pool);
//   3. per pixel: visibility reuse, then temporal reuse, final store.
// Shared-memory carveout hint (percent of the unified L1/shared storage) for
// the ray-tracing kernels; -1 leaves the driver's choice.
#ifndef RG_SMEM_CARVEOUT
#define RG_SMEM_CARVEOUT -1
#endif

// Pixels per thread of the single-view launch (the batched one is tuned):
// 3 (32 x 12 tiles) measured fastest at 1080p among 2 to 6 (3.33 ms against
// 3.34, 3.48, 3.44 and 4.21 ms for 2, 4, 5 and 6).
#ifndef RG_RIS_PPT
#define RG_RIS_PPT 3
#endif
constexpr int kRisPpt = RG_RIS_PPT;

struct InitialParams {
    DevScene s;
    GBufView cur, prev;
    bool has_prev;
    const rg_reservoir *prev_res;
    rg_reservoir *out;
    rg_restir_uniforms u;
    mlp::LearnedRis learned;  // learned.cand == nullptr: the plain alias-table proposal
    VisCache vc{};            // own-segment answers written for the next ray pass
};

// The cached answer of segment a -> b in entry e (0 unshadowed, 1
// shadowed), or -1 when the entry holds another segment or none.
__device__ __forceinline__ int vcache_find(const VisCache &vc, size_t e, f3 a, f3 b) {
    const float4 s = __ldg(vc.in + 2 * e), t = __ldg(vc.in + 2 * e + 1);
    const uint32_t tag = __float_as_uint(s.w), tt = __float_as_uint(t.w);
    if (tag == 0u || (tt >> 1) != tag) return -1;
    if (__float_as_uint(s.x) != __float_as_uint(a.x) || __float_as_uint(s.y) != __float_as_uint(a.y) ||
        __float_as_uint(s.z) != __float_as_uint(a.z) || __float_as_uint(t.x) != __float_as_uint(b.x) ||
        __float_as_uint(t.y) != __float_as_uint(b.y) || __float_as_uint(t.z) != __float_as_uint(b.z))
        return -1;
    return (int)(tt & 1u);
}
// Entry e := segment a -> b with its answer (ans 0/1), or empty (ans < 0).
__device__ __forceinline__ void vcache_put(const VisCache &vc, size_t e, f3 a, f3 b, int ans) {
    if (ans < 0) {
        vc.out[2 * e] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    vc.out[2 * e] = make_float4(a.x, a.y, a.z, __uint_as_float(vc.tag));
    vc.out[2 * e + 1] = make_float4(b.x, b.y, b.z, __uint_as_float(2u * vc.tag + (uint32_t)ans));
}

// Initial RIS (restirOmni.glsl:86-145).  With the learned proposal, candidate
// c of the pixel comes from its candidate slot: a cluster drawn from q(.|x)
// (the light within it from the cluster's alias table with r1, r2) or a light
// drawn uniformly; either way the source pdf is the mixture density
// mix * q(cluster) * p(light | cluster) + (1 - mix) / N.  The RIS stream keeps
// the shape of the plain path (two uniforms per candidate).
template <int R, bool MIS>
__device__ __forceinline__ ResV<R, MIS> ris(const DevScene &s, const Texel &t, float albedo_lum, f3 cam,
                                            uint32_t count_c, bool zero_normal, int flags, const mlp::LearnedRis &lr,
                                            size_t px, Pcg &rng) {
    ResV<R, MIS> r = empty_resv<R, MIS>();
    if (zero_normal) return r;
    const f3 wo = view_dir(cam, t.wpos);
    const PhatPx pp = phat_px(t.wpos, wo, t.normal, albedo_lum, t.roughness, t.metallic);
    const int count = s.n_alias;
    if (!lr.cand && s.n_point_lights != 0 && count_c > 0) {
        // The plain point-light proposal with a one-candidate lookahead.  A
        // candidate's draws are always r1, r2 and then one reservoir-update
        // uniform per sample, so the next candidate's r1, r2 (and its
        // alias-table column, both lights' positions loaded unconditionally)
        // are taken right after this candidate's update uniforms, and the
        // gather runs under this candidate's p-hat: same draws, same order,
        // same arithmetic as the loop below.
        float r1 = rand_float(rng), r2 = rand_float(rng);
        int col = imin((int)((float)count * r1), count - 1);
        float4 cc = __ldg(&s.alias[col].col), own = __ldg(&s.alias[col].own_pos), ali = __ldg(&s.alias[col].alias_pos);
        const float4 nrm0 = make_float4(0.f, 0.f, 0.f, 0.f);
        for (uint32_t c = 0; c < count_c; ++c) {
            float u[R];
#pragma unroll
            for (int j = 0; j < R; ++j) u[j] = rand_float(rng);
            float r2n = 0.0f;
            int coln = 0;
            float4 ccn = cc, ownn = own, alin = ali;
            if (c + 1 < count_c) {
                const float r1n = rand_float(rng);
                r2n = rand_float(rng);
                coln = imin((int)((float)count * r1n), count - 1);
                ccn = __ldg(&s.alias[coln].col);
                ownn = __ldg(&s.alias[coln].own_pos);
                alin = __ldg(&s.alias[coln].alias_pos);
            }
            const bool keep = cc.x > r2;  // restirOmni.glsl:73-83
            const float4 pos_lum = keep ? own : ali;
            const float prob = keep ? cc.z : cc.w;
            const int32_t lidx = keep ? col : __float_as_int(cc.y);
            const float ph = eval_phat_px(pp, xyz(pos_lum), xyz(nrm0), false, pos_lum.w);
            add_sample_u(r, pos_lum, nrm0, lidx, ph, prob, u);
            r2 = r2n;
            col = coln;
            cc = ccn;
            own = ownn;
            ali = alin;
        }
        if (flags & RG_FLAG_FINAL_RIS_WEIGHT) {
#pragma unroll
            for (int j = 0; j < R; ++j)
                if (r.sum_w[j] > 0.0f) r.w[j] = r.sum_w[j] / ((float)r.m * r.p_hat[j]);
        }
        return r;
    }
    for (uint32_t c = 0; c < count_c; ++c) {
        const float r1 = rand_float(rng), r2 = rand_float(rng);
        const int col = imin((int)((float)count * r1), count - 1);  // restirOmni.glsl:73-83
        float4 pos_lum, nrm;
        float prob;
        int32_t lidx;
        if (lr.cand) {
            const mlp::Candidate cd = lr.cand[px * mlp::kCand + c];
            float pl;
            if (cd.key < 0) {
                const int cl = -1 - cd.key;
                const int b = __ldg(lr.offset + cl), m = __ldg(lr.offset + cl + 1) - b;
                if (m > 0) {
                    const mlp::LearnedCol *lc = lr.lcol + b + imin((int)((float)m * r1), m - 1);
                    const float4 cc = __ldg(&lc->col);
                    if (cc.x > r2) { pos_lum = __ldg(&lc->own_pos); pl = cc.w; lidx = __float_as_int(cc.y); }
                    else { pos_lum = __ldg(&lc->alias_pos); lidx = __float_as_int(cc.z); pl = __ldg(lr.within + lidx); }
                } else {  // an empty cluster (only from non-finite logits): light 0 with weight 0
                    lidx = 0;
                    pos_lum = __ldg(&s.alias[0].own_pos);
                    pl = 0.0f;
                }
            } else {
                lidx = cd.key;
                pos_lum = __ldg(&s.alias[lidx].own_pos);
                pl = __ldg(lr.within + lidx);
            }
            prob = lr.mix * cd.q * pl + lr.uniform_pdf;
            nrm = make_float4(0.f, 0.f, 0.f, 0.f);
        } else if (s.n_point_lights != 0) {
            const AliasLight *al = s.alias + col;
            const float4 cc = __ldg(&al->col);
            if (cc.x > r2) { pos_lum = __ldg(&al->own_pos); prob = cc.z; lidx = col; }
            else { pos_lum = __ldg(&al->alias_pos); prob = cc.w; lidx = __float_as_int(cc.y); }
            nrm = make_float4(0.f, 0.f, 0.f, 0.f);
        } else {
            const rg_alias_table_column cc = s.tri_alias[col];
            int sel;
            if (cc.prob > r2) { sel = col; prob = cc.ori_prob; }
            else { sel = cc.alias; prob = cc.alias_ori_prob; }
            const rg_tri_light &L = s.tri_lights[sel];
            const float ra = rand_float(rng), rb = rand_float(rng);
            const float sa = sqrtf(ra);  // pickPointOnTriangle, restirOmni.glsl:68-71
            const f3 lpos = (scale(1.0f - sa, mk(L.p1[0], L.p1[1], L.p1[2])) +
                             scale(sa * (1.0f - rb), mk(L.p2[0], L.p2[1], L.p2[2]))) +
                            scale(rb * sa, mk(L.p3[0], L.p3[1], L.p3[2]));
            const f3 wi = normalize(t.wpos - lpos);
            const f3 nn = mk(L.normal_area[0], L.normal_area[1], L.normal_area[2]);
            prob /= fabsf(dot(wi, nn)) * L.normal_area[3];
            pos_lum = make_float4(lpos.x, lpos.y, lpos.z, L.emission_luminance[3]);
            nrm = make_float4(nn.x, nn.y, nn.z, 1.0f);
            lidx = -1 - sel;
        }
        const float ph = eval_phat_px(pp, xyz(pos_lum), xyz(nrm), nrm.w > 0.5f, pos_lum.w);
        add_sample(r, pos_lum, nrm, lidx, ph, prob, rng);
    }
    if (flags & RG_FLAG_FINAL_RIS_WEIGHT) {
#pragma unroll
        for (int j = 0; j < R; ++j)
            if (r.sum_w[j] > 0.0f) r.w[j] = r.sum_w[j] / ((float)r.m * r.p_hat[j]);
    }
    return r;
}

#ifndef RG_RIS_MIN_BLOCKS
#define RG_RIS_MIN_BLOCKS 8
#endif
// The pass over one 32 x (4*PPT) pixel tile (tile coordinates bx, by); with
// R samples per reservoir each pixel traces R visibility segments.
template <int PPT, int R, bool MIS>
__device__ __forceinline__ void initial_temporal_tile(const InitialParams &p, int bx, int by) {
    constexpr int kTile = 128 * PPT;
    extern __shared__ __align__(16) unsigned char smem[];
    rgpool::Ray *pool = reinterpret_cast<rgpool::Ray *>(smem);
    float4 *endp = reinterpret_cast<float4 *>(pool + kTile * R);  // sample position per (pixel slot, sample)
    uint8_t *shadow = reinterpret_cast<uint8_t *>(endp + kTile * R);
    int *stack = reinterpret_cast<int *>(shadow + kTile * R);
    __shared__ int s_count, s_next;
    const int tid = threadIdx.x + threadIdx.y * 32;
    if (tid == 0) { s_count = 0; s_next = 0; }
    __syncthreads();
    const DevScene &s = p.s;
    const int W = (int)p.u.screen_size[0], H = (int)p.u.screen_size[1];
    const int x = bx * 32 + threadIdx.x;
    const int y0 = by * (4 * PPT) + threadIdx.y;
    const f3 cam = mk(p.u.camera_pos[0], p.u.camera_pos[1], p.u.camera_pos[2]);
    const bool vis = (p.u.flags & RG_FLAG_VISIBILITY_REUSE) != 0;
    const bool swap_fix = (p.u.flags & RG_FLAG_MIS_SWAP_FIX) != 0;
    uint64_t rng_state[PPT];
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
        const int y = y0 + 4 * j;
        const bool valid = x < W && y < H;
        bool want = false;
        f3 wpos = mk(0.f, 0.f, 0.f);
        float4 lpos[R];
#pragma unroll
        for (int q = 0; q < R; ++q) lpos[q] = make_float4(0.f, 0.f, 0.f, 0.f);
        rng_state[j] = 0;
        if (valid) {
            const size_t i = (size_t)y * (size_t)W + (size_t)x;
            Texel t;
            load_texel(p.cur, i, t);
            const float albedo_lum = luminance(t.albedo.x, t.albedo.y, t.albedo.z);
            Pcg rng = pcg_seed((uint64_t)p.u.frame, (uint64_t)((uint32_t)y * 10007u + (uint32_t)x));
            const bool zero_normal = !(dot(t.normal, t.normal) != 0.0f);
            const ResV<R, MIS> r = ris<R, MIS>(s, t, albedo_lum, cam, p.u.initial_light_sample_count, zero_normal,
                                               p.u.flags, p.learned, i, rng);
            store_resv(p.out, i, r);
            rng_state[j] = rng.state;
            // visibility reuse :147-160; a background pixel's (zero normal) sample is the
            // zero sample, for which zeroing w and sumWeights changes nothing: no ray
            want = vis && !zero_normal;
            wpos = t.wpos;
#pragma unroll
            for (int q = 0; q < R; ++q) lpos[q] = make_float4(r.pos_lum[q].x, r.pos_lum[q].y, r.pos_lum[q].z, 0.0f);
        }
#pragma unroll
        for (int q = 0; q < R; ++q) {
            const int owner = (j * 128 + tid) * R + q;
            shadow[owner] = want ? 0 : 2;  // 2: no segment
            endp[owner] = lpos[q];
            const int slot = rgpool::append_slot(&s_count, want);
            if (want) rgpool::put_ray(pool, slot, wpos, owner);
        }
    }
    __syncthreads();
    rgpool::TraceStats ts;
    rgpool::trace_pool(
        s, pool, s_count, &s_next, stack, s.depth, ts,
        [&](int owner) { const float4 e = endp[owner]; return mk(e.x, e.y, e.z); },
        [&](int owner, bool hit) { shadow[owner] = hit ? 1 : 0; });
    __syncthreads();
#pragma unroll
    for (int j = 0; j < PPT; ++j) {
        const int y = y0 + 4 * j;
        if (x >= W || y >= H) continue;
        const size_t i = (size_t)y * (size_t)W + (size_t)x;
        ResV<R, MIS> r = load_resv_own<R, MIS>(p.out, i);
#pragma unroll
        for (int q = 0; q < R; ++q) {
            const int owner = (j * 128 + tid) * R + q;
            if (shadow[owner] == 1) {
                r.w[q] = 0.0f;
                r.sum_w[q] = 0.0f;
                if (MIS) r.sum_phat[q] = 0.0f;
            }
            if (p.vc.out) {
                const float4 e = endp[owner];
                vcache_put(p.vc, (size_t)q * p.vc.n + i, load_wpos(p.cur, i), mk(e.x, e.y, e.z),
                           shadow[owner] == 2 ? -1 : (int)shadow[owner]);
            }
        }
        if ((p.u.flags & RG_FLAG_TEMPORAL_REUSE) && p.has_prev) {
            Texel t;
            load_texel(p.cur, i, t);
            const float albedo_lum = luminance(t.albedo.x, t.albedo.y, t.albedo.z);
            Pcg rng;
            rng.state = rng_state[j];
            rng.inc = ((uint64_t)((uint32_t)y * 10007u + (uint32_t)x) << 1u) | 1u;
            const float *m = p.u.prev_frame_projection_view;
            float px = ((m[0] * t.wpos.x + m[4] * t.wpos.y) + m[8] * t.wpos.z) + m[12] * 1.0f;
            float py = ((m[1] * t.wpos.x + m[5] * t.wpos.y) + m[9] * t.wpos.z) + m[13] * 1.0f;
            const float pw = ((m[3] * t.wpos.x + m[7] * t.wpos.y) + m[11] * t.wpos.z) + m[15] * 1.0f;
            px /= pw;
            py /= pw;
            px = (px + 1.0f) * 0.5f * (float)p.u.screen_size[0];
            py = (py + 1.0f) * 0.5f * (float)p.u.screen_size[1];
            if (px > 0.0f && py > 0.0f && px < (float)p.u.screen_size[0] && py < (float)p.u.screen_size[1]) {
                const int fx = (int)px, fy = (int)py;
                const size_t pi = (size_t)fy * (size_t)W + (size_t)fx;
                const f3 dp = t.wpos - load_wpos(p.prev, pi);
                if (dot(dp, dp) < 0.01f) {
                    const f3 da = t.albedo - load_albedo(p.prev, pi, nullptr);
                    if (dot(da, da) < 0.01f) {
                        if (dot(t.normal, load_normal(p.prev, pi)) > 0.5f) {
                            ResV<R, MIS> pr = load_resv<R, MIS>(p.prev_res, pi);
                            const uint32_t cap = p.u.temporal_sample_count_multiplier * r.m;
                            pr.m = pr.m < cap ? pr.m : cap;
                            const f3 wo = view_dir(cam, t.wpos);
                            float ph[R];
#pragma unroll
                            for (int q = 0; q < R; ++q)
                                ph[q] = eval_phat_wo(t.wpos, xyz(pr.pos_lum[q]), wo, t.normal, xyz(pr.nrm[q]),
                                                     pr.nrm[q].w > 0.5f, albedo_lum, pr.pos_lum[q].w, t.roughness,
                                                     t.metallic);
                            combine_res(r, pr, ph, swap_fix, rng);
                        }
                    }
                }
            }
        }
        store_resv(p.out, i, r);
    }
    count_block_rays(s, tid == 0 ? s_count : 0, ts);
}

template <int PPT, int R, bool MIS>
__global__ void __launch_bounds__(128, RG_RIS_MIN_BLOCKS) k_initial_temporal(const InitialParams p) {
    initial_temporal_tile<PPT, R, MIS>(p, blockIdx.x, blockIdx.y);
}

// ---------------------------------------------------------------- biased spatial (spatialReuse.comp:30-86)
struct SpatialParams {
    DevScene s;
    GBufView g;
    const rg_reservoir *in;
    rg_reservoir *out;
    rg_restir_uniforms u;
    int iter;           // biased: push-constant iter; unbiased: pass index
    int num_neighbors;  // unbiased: NUM_NEIGHBORS
    float cos_thr;
    VisCache vc{};      // unbiased: own-segment answers of the previous ray pass in, this pass's out
};

// One 32 x 4 pixel tile.
template <int R, bool MIS>
__device__ __forceinline__ void spatial_biased_tile(const SpatialParams &p, int bx, int by) {
    const int x = bx * 32 + threadIdx.x;
    const int y = by * 4 + threadIdx.y;
    const int W = (int)p.u.screen_size[0], H = (int)p.u.screen_size[1];
    if (x >= W || y >= H) return;
    const size_t i = (size_t)y * (size_t)W + (size_t)x;
    Texel t;
    load_texel(p.g, i, t);
    const float depth = load_depth(p.g, i);
    const float albedo_lum = luminance(t.albedo.x, t.albedo.y, t.albedo.z);
    const f3 cam = mk(p.u.camera_pos[0], p.u.camera_pos[1], p.u.camera_pos[2]);
    const PhatPx pp = phat_px(t.wpos, view_dir(cam, t.wpos), t.normal, albedo_lum, t.roughness, t.metallic);
    ResV<R, MIS> r = load_resv<R, MIS>(p.in, i);
    const bool swap_fix = (p.u.flags & RG_FLAG_MIS_SWAP_FIX) != 0;
    Pcg rng = pcg_seed((uint64_t)(p.u.frame * 31u + (uint32_t)p.iter), (uint64_t)((uint32_t)y * 10007u + (uint32_t)x));
    for (uint32_t k = 0; k < p.u.spatial_neighbors; ++k) {
        const float angle = rand_float(rng) * 2.0f * kPi;
        const float radius = sqrtf(rand_float(rng)) * p.u.spatial_radius;
        float sn, cs;
        sincos_cw(angle, sn, cs);
        const int nx = iclamp(x + (int)floorf(cs * radius), 0, W - 1);
        const int ny = iclamp(y + (int)floorf(sn * radius), 0, H - 1);
        const size_t ni = (size_t)ny * (size_t)W + (size_t)nx;
        const float nd = load_depth(p.g, ni);
        const f3 nn = load_normal(p.g, ni);
        if (fabsf(nd - depth) > p.u.spatial_pos_threshold * fabsf(depth) || dot(nn, t.normal) < p.cos_thr) continue;
        const ResV<R, MIS> rr = load_resv<R, MIS>(p.in, ni);
        float ph[R];
#pragma unroll
        for (int q = 0; q < R; ++q)
            ph[q] = eval_phat_px(pp, xyz(rr.pos_lum[q]), xyz(rr.nrm[q]), rr.nrm[q].w > 0.5f, rr.pos_lum[q].w);
        combine_res(r, rr, ph, swap_fix, rng);
    }
    store_resv(p.out, i, r);
}

#ifndef RG_BIASED_MIN_BLOCKS
#define RG_BIASED_MIN_BLOCKS 8
#endif
template <int R, bool MIS>
__global__ void __launch_bounds__(128, RG_BIASED_MIN_BLOCKS) k_spatial_biased(const SpatialParams p) {
    spatial_biased_tile<R, MIS>(p, blockIdx.x, blockIdx.y);
}

// ---------------------------------------------------------------- unbiased spatial (unbiasedReuse.glsl:50-185)
// One pixel per thread, 32x4 threads per block:
//   1. neighbour streaming (:84-124); then, for every neighbour whose
//      hemisphere holds the chosen sample and for the pixel itself, the
//      visibility segment goes to the block's ray pool (:132-166);
//   2. the block traces its pool;
//   3. the normalisation count and the final W (:168-182).
// Shared memory (R samples per reservoir): ray pool [128*(K+1)*R], light
// position per sample and pixel [R][128], neighbour index [K][128], neighbour
// M [K][128] (with MIS: neighbour sumPHat [R][K][128]), not-counted flags
// [R][(K+1)][128], stacks.  The merged reservoir is parked in `out` between
// steps 1 and 3.
constexpr int kMaxNeighbors = 16;

__host__ __device__ inline size_t unbiased_smem_bytes(int K, int depth, int R = 1, bool mis = false, int bt = 128) {
    const size_t slots = (size_t)K + 1, kp = (size_t)(K > 0 ? K : 1);
    size_t b = (size_t)bt * (size_t)R * sizeof(float4);
    b += (size_t)bt * kp * sizeof(uint32_t);
    b += (size_t)bt * kp * (mis ? (size_t)R : 1) * sizeof(uint32_t);
    b += (size_t)bt * slots * (size_t)R * sizeof(int);
    b += ((size_t)bt * slots * (size_t)R + 15) & ~(size_t)15;
    b += (size_t)bt * (size_t)depth * sizeof(int);
    return b;
}

#ifndef RG_UNBIASED_MIN_BLOCKS
#define RG_UNBIASED_MIN_BLOCKS 8
#endif
// One TW x (BT/TW) pixel tile (BT threads); the tile shape and size change
// which pixels share a ray pool, never a result.
template <int TW, int R, bool MIS, int BT = 128>
__device__ __forceinline__ void spatial_unbiased_tile(const SpatialParams &p, int bx, int by) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int K = p.num_neighbors;
    const int slots = K + 1, kp = K > 0 ? K : 1;
    // The ray pool holds owner tags only (a segment's start is re-read from
    // the G-buffer when a lane takes it), which leaves more of the SM's
    // L1/shared storage to the L1 cache that serves the tree.
    float4 *endp = reinterpret_cast<float4 *>(smem);                                // [R][BT]
    uint32_t *nidx = reinterpret_cast<uint32_t *>(endp + BT * R);                  // [K][BT]
    uint32_t *nm = nidx + BT * kp;                                                 // [K][BT]
    float *nsp = reinterpret_cast<float *>(nm);                                     // MIS: [R][K][BT]
    int *pool = reinterpret_cast<int *>(nm + BT * kp * (MIS ? R : 1));             // owners, [R][K+1][BT] slots
    uint8_t *flag = reinterpret_cast<uint8_t *>(pool + BT * slots * R);            // [R][K+1][BT]
    int *stack = reinterpret_cast<int *>(flag + ((BT * slots * R + 15) & ~15));
    __shared__ int s_count, s_next;
    const int tid = threadIdx.x + threadIdx.y * 32;
    if (tid == 0) { s_count = 0; s_next = 0; }
    __syncthreads();
    const DevScene &s = p.s;
    const int W = (int)p.u.screen_size[0], H = (int)p.u.screen_size[1];
    const int x = bx * TW + tid % TW;
    const int y = by * (BT / TW) + tid / TW;
    const bool valid = x < W && y < H;
    const bool vis = (p.u.flags & RG_FLAG_VISIBILITY_REUSE) != 0;
    const size_t i = valid ? (size_t)y * (size_t)W + (size_t)x : 0;
    f3 lpos[R];
#pragma unroll
    for (int q = 0; q < R; ++q) lpos[q] = mk(0.f, 0.f, 0.f);
    uint32_t orig_m = 0;
    f3 own_wpos = mk(0.f, 0.f, 0.f);
    float orig_sp[MIS ? R : 1];
#pragma unroll
    for (int q = 0; q < (MIS ? R : 1); ++q) orig_sp[q] = 0.0f;
    if (valid) {
        Texel t;
        load_texel(p.g, i, t);
        const float albedo_lum = luminance(t.albedo.x, t.albedo.y, t.albedo.z);
        const f3 cam = mk(p.u.camera_pos[0], p.u.camera_pos[1], p.u.camera_pos[2]);
        const f3 wo = view_dir(cam, t.wpos);
        const PhatPx pp = phat_px(t.wpos, wo, t.normal, albedo_lum, t.roughness, t.metallic);
        own_wpos = t.wpos;
        ResV<R, MIS> r = load_resv<R, MIS>(p.in, i);
        orig_m = r.m;
        if (MIS) {
#pragma unroll
            for (int q = 0; q < R; ++q) orig_sp[q] = r.sum_phat[q];
        }
        Pcg rng = pcg_seed((uint64_t)(p.u.frame * 17u + (uint32_t)p.iter),
                           (uint64_t)((uint32_t)y * 10007u + (uint32_t)x));
        for (int k = 0; k < K; ++k) {
            const float angle = rand_float(rng) * 2.0f * kPi;
            const float radius = sqrtf(rand_float(rng)) * p.u.spatial_radius;
            float sn, cs;
            sincos_cw(angle, sn, cs);
            const int nx = iclamp(x + (int)roundf(cs * radius), 0, (int)(p.u.screen_size[0] - 1u));
            const int ny = iclamp(y + (int)roundf(sn * radius), 0, (int)(p.u.screen_size[1] - 1u));
            const size_t ni = (size_t)ny * (size_t)W + (size_t)nx;
            const ResV<R, MIS> rr = load_resv<R, MIS>(p.in, ni);
            nidx[k * BT + tid] = (uint32_t)ni;
            if (MIS) {
#pragma unroll
                for (int q = 0; q < R; ++q) nsp[(q * kp + k) * BT + tid] = rr.sum_phat[q];
            } else {
                nm[k * BT + tid] = rr.m;
            }
            r.m += rr.m;
#pragma unroll
            for (int q = 0; q < R; ++q) {
                const float ph = eval_phat_px(pp, xyz(rr.pos_lum[q]), xyz(rr.nrm[q]), rr.nrm[q].w > 0.5f,
                                              rr.pos_lum[q].w);
                const float weight = ph * rr.w[q] * (float)rr.m;
                if (weight > 0.0f)
                    update_at(r, q, weight, rr.pos_lum[q], rr.nrm[q], rr.idx[q], ph, rr.w[q],
                              MIS ? rr.sum_phat[q] : 0.0f, rng);
            }
        }
#pragma unroll
        for (int q = 0; q < R; ++q) lpos[q] = xyz(r.pos_lum[q]);
        store_resv(p.out, i, r);
    }
    // Each pixel's own segment goes to the front of the pool, so lanes take
    // those first.  When the pixel's own segment is shadowed, its count is
    // reset whatever its neighbours' segments answer (unbiasedReuse.glsl:
    // 168-176), so a lane that takes a neighbour's segment whose pixel's own
    // answer is already known shadowed skips it.  A pixel's neighbour
    // segments (one per neighbour whose hemisphere holds the sample) share the
    // sample's light as their end point: they follow consecutively, so the
    // lanes that take them trace similar paths.
    // Segments whose answer the previous ray pass left in the cache (a pixel
    // that kept its sample meets its own segment again; one that took a
    // neighbour's sample meets that neighbour's own segment) are not traced,
    // and a pixel whose own segment is cached as shadowed traces nothing.
    uint32_t wantm[R];  // bit k: neighbour k's segment
#pragma unroll
    for (int q = 0; q < R; ++q) {
        endp[q * BT + tid] = make_float4(lpos[q].x, lpos[q].y, lpos[q].z, 0.0f);
        wantm[q] = 0u;
        const int own_known =
            valid && vis && p.vc.in ? vcache_find(p.vc, (size_t)q * p.vc.n + i, own_wpos, lpos[q]) : -1;
        for (int k = 0; k < K; ++k) {
            bool excluded = true;
            if (valid) {
                const uint32_t ni = nidx[k * BT + tid];
                const f3 nw = load_wpos(p.g, ni);
                const f3 nn = load_normal(p.g, ni);
                excluded = dot(lpos[q] - nw, nn) < 0.0f;
                if (!excluded && vis && own_known != 1) {
                    const int known = p.vc.in ? vcache_find(p.vc, (size_t)q * p.vc.n + ni, nw, lpos[q]) : -1;
                    if (known < 0) wantm[q] |= 1u << k;
                    else excluded = known == 1;  // a cached shadowed answer counts like an exclusion
                }
            }
            flag[(q * slots + k) * BT + tid] = excluded ? 1 : 0;
        }
        flag[(q * slots + K) * BT + tid] = own_known == 1 ? 1 : 0;
        const bool own = valid && vis && own_known < 0;
        const int slot = rgpool::append_range(&s_count, own ? 1 : 0);
        if (own) pool[slot] = (q * slots + K) * BT + tid;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < R; ++q) {
        int slot = rgpool::append_range(&s_count, __popc(wantm[q]));
        for (uint32_t m = wantm[q]; m != 0u; m &= m - 1u) {
            const int k = __ffs(m) - 1;
            pool[slot++] = (q * slots + k) * BT + tid;
        }
    }
    __syncthreads();
    rgpool::TraceStats ts;
    rgpool::trace_pool_f(
        s,
        [&](int slot, f3 &p1) {  // start: the neighbour's (k < K) or the pixel's own position
            const int owner = pool[slot];
            const int r = owner % (slots * BT);
            const int k = r / BT, t = r % BT;
            if (k < K && reinterpret_cast<volatile const uint8_t *>(flag)[(owner / (slots * BT) * slots + K) * BT + t])
                return -1;  // the pixel's own segment is shadowed: this answer is unobservable
            const size_t pi = k < K ? (size_t)nidx[k * BT + t]
                                    : (size_t)(by * (BT / TW) + t / TW) * (size_t)W + (size_t)(bx * TW + t % TW);
            p1 = load_wpos(p.g, pi);
            return owner;
        },
        s_count, &s_next, stack, s.depth, ts,
        [&](int owner) {
            const float4 e = endp[(owner / (slots * BT)) * BT + (owner % BT)];
            return mk(e.x, e.y, e.z);
        },
        [&](int owner, bool hit) { if (hit) flag[owner] = 1; });
    __syncthreads();
    if (valid) {
        // the merged reservoir went to `out` before the trace; only each
        // sample's (index, p-hat, sumWeights, W) word and, with MIS, its
        // sumPHat word change (coherent loads: this thread wrote them)
        using L = ResLayout<R, MIS>;
        float4 *rw = reinterpret_cast<float4 *>(p.out) + i * L::kWords;
        const f3 wp = p.vc.out ? load_wpos(p.g, i) : mk(0.f, 0.f, 0.f);
#pragma unroll
        for (int q = 0; q < R; ++q) {
            const uint8_t *fq = flag + q * slots * BT;
            if (p.vc.out) {
                const float4 e = endp[q * BT + tid];
                vcache_put(p.vc, (size_t)q * p.vc.n + i, wp, mk(e.x, e.y, e.z), vis ? (int)fq[K * BT + tid] : -1);
            }
            const float4 c = rw[q * L::kSample4 + 2];  // index, p-hat, sumWeights, W
            const float p_hat = c.y;
            float sum_w = c.z, w = c.w;
            if (MIS) {
                float sp = orig_sp[q];
                for (int k = 0; k < K; ++k)
                    if (!fq[k * BT + tid]) sp += nsp[(q * kp + k) * BT + tid];
                if (vis && fq[K * BT + tid]) sp = 0.0f;
                if (sp > 0.0f) {
                    w = sum_w * p_hat / (sp * p_hat);
                } else {
                    w = 0.0f;
                    sum_w = 0.0f;
                    rw[q * L::kSample4 + 3] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);  // sumPHat
                }
            } else {
                uint32_t ns = orig_m;
                for (int k = 0; k < K; ++k)
                    if (!fq[k * BT + tid]) ns += nm[k * BT + tid];
                if (vis && fq[K * BT + tid]) ns = 0;
                if (ns > 0) {
                    w = sum_w / ((float)ns * p_hat);
                } else {
                    w = 0.0f;
                    sum_w = 0.0f;
                }
            }
            rw[q * L::kSample4 + 2] = make_float4(c.x, p_hat, sum_w, w);
        }
    }
    count_block_rays(s, tid == 0 ? s_count : 0, ts);
}

#ifndef RG_UNBIASED_BT
#define RG_UNBIASED_BT 128
#endif
template <int TW, int R, bool MIS, int BT>
__global__ void __launch_bounds__(BT, RG_UNBIASED_MIN_BLOCKS * 128 / BT) k_spatial_unbiased(const SpatialParams p) {
    spatial_unbiased_tile<TW, R, MIS, BT>(p, blockIdx.x, blockIdx.y);
}

// ---------------------------------------------------------------- shading (lighting.frag:43-71,103)
struct ShadeParams {
    DevScene s;
    GBufView g;
    const rg_reservoir *res;
    float4 *out;
    rg_lighting_uniforms u;
};

// One 32 x 4 pixel tile.
template <int R, bool MIS>
__device__ __forceinline__ void shade_pixel(const ShadeParams &p, const Texel &t, const ResV<R, MIS> &r, size_t i) {
    const f3 cam = mk(p.u.camera_pos[0], p.u.camera_pos[1], p.u.camera_pos[2]);
    f3 col = mk(0.0f, 0.0f, 0.0f);
#pragma unroll
    for (int q = 0; q < R; ++q) {
        f3 emission = mk(0.f, 0.f, 0.f);
        if (r.idx[q] < 0) {
            const int k = -1 - r.idx[q];
            if (k < p.s.n_tri_lights) {
                const rg_tri_light &L = p.s.tri_lights[k];
                emission = mk(L.emission_luminance[0], L.emission_luminance[1], L.emission_luminance[2]);
            }
        } else if (r.idx[q] < p.s.n_point_lights) {
            const float4 c = __ldg(p.s.pl_color + r.idx[q]);
            emission = mk(c.x, c.y, c.z);
        }
        const f3 ph = eval_phat_full(t.wpos, xyz(r.pos_lum[q]), cam, t.normal, xyz(r.nrm[q]), r.nrm[q].w > 0.5f,
                                     t.albedo, emission, t.roughness, t.metallic);
        col = mk(col.x + ph.x * r.w[q], col.y + ph.y * r.w[q], col.z + ph.z * r.w[q]);
    }
    col = divs(col, (float)R);  // RESERVOIR_SIZE
    if (t.albedo_a > 0.5f) col = t.albedo;
    if (p.u.gamma != 1.0f) {
        const float ig = 1.0f / p.u.gamma;
        col = mk(powf(col.x, ig), powf(col.y, ig), powf(col.z, ig));
    }
    p.out[i] = make_float4(col.x, col.y, col.z, 1.0f);
}
template <int R, bool MIS>
__device__ __forceinline__ void shade_tile(const ShadeParams &p, int bx, int by) {
    const int x = bx * 32 + threadIdx.x;
    const int y = by * 4 + threadIdx.y;
    const int W = (int)p.u.buffer_size[0], H = (int)p.u.buffer_size[1];
    if (x >= W || y >= H) return;
    const size_t i = (size_t)y * (size_t)W + (size_t)x;
    Texel t;
    load_texel(p.g, i, t);
    shade_pixel<R, MIS>(p, t, load_resv<R, MIS>(p.res, i), i);
}

// RG_SHADE_PPT pixels per thread (rows 4 apart in a 32 x 4*PPT tile): every
// pixel's G-buffer and reservoir loads are issued before the first pixel's
// light gather.  Measured at 1080p: 1, 2, 4 pixels give 0.055, 0.076, 0.116
// ms (more registers, fewer resident warps), hence 1.
#ifndef RG_SHADE_PPT
#define RG_SHADE_PPT 1
#endif
#ifndef RG_SHADE_MIN_BLOCKS
#define RG_SHADE_MIN_BLOCKS 1
#endif
template <int R, bool MIS>
__global__ void __launch_bounds__(128, RG_SHADE_MIN_BLOCKS) k_shade(const ShadeParams p) {
    const int W = (int)p.u.buffer_size[0], H = (int)p.u.buffer_size[1];
    const int x = blockIdx.x * 32 + threadIdx.x;
    Texel t[RG_SHADE_PPT];
    ResV<R, MIS> r[RG_SHADE_PPT];
    size_t idx[RG_SHADE_PPT];
    bool ok[RG_SHADE_PPT];
#pragma unroll
    for (int k = 0; k < RG_SHADE_PPT; ++k) {
        const int y = blockIdx.y * 4 * RG_SHADE_PPT + threadIdx.y + 4 * k;
        ok[k] = x < W && y < H;
        idx[k] = ok[k] ? (size_t)y * (size_t)W + (size_t)x : 0;
        if (ok[k]) {
            load_texel(p.g, idx[k], t[k]);
            r[k] = load_resv<R, MIS>(p.res, idx[k]);
        }
    }
#pragma unroll
    for (int k = 0; k < RG_SHADE_PPT; ++k)
        if (ok[k]) shade_pixel<R, MIS>(p, t[k], r[k], idx[k]);
}

// ---------------------------------------------------------------- visibility batch (testVisibility)
// 128 threads take a chunk of 512 segments into the pool and trace it.
constexpr int kVisChunk = 512;

__global__ void __launch_bounds__(128) k_visibility_batch(const DevScene s, const float4 *p1, const float4 *p2,
                                                          uint8_t *out, int n) {
    extern __shared__ __align__(16) unsigned char smem[];
    rgpool::Ray *pool = reinterpret_cast<rgpool::Ray *>(smem);
    float4 *endp = reinterpret_cast<float4 *>(pool + kVisChunk);
    int *stack = reinterpret_cast<int *>(endp + kVisChunk);
    __shared__ int s_next;
    const int tid = threadIdx.x;
    const int base = blockIdx.x * kVisChunk;
    const int count = min(kVisChunk, n - base);
    if (tid == 0) s_next = 0;
    for (int k = tid; k < count; k += 128) {
        const float4 a = __ldg(p1 + base + k), b = __ldg(p2 + base + k);
        rgpool::put_ray(pool, k, mk(a.x, a.y, a.z), k);
        endp[k] = b;
    }
    __syncthreads();
    rgpool::TraceStats ts;
    rgpool::trace_pool(
        s, pool, count, &s_next, stack, s.depth, ts,
        [&](int owner) { const float4 e = endp[owner]; return mk(e.x, e.y, e.z); },
        [&](int owner, bool hit) { out[base + owner] = hit ? 1 : 0; });
    count_block_rays(s, tid == 0 ? count : 0, ts);
}

// ---------------------------------------------------------------- many views, one launch per pass
// A persistent grid takes tiles from an atomic counter over the tiles of all
// views (view_start: prefix sums of the views' tile counts).  Each tile runs
// the same body as the single-view kernels with that view's parameters (read
// from the parameter array in device memory), so a view's results equal those
// of its own single-view launches.
template <typename P, typename F>
__device__ __forceinline__ void for_each_view_tile(const P *views, const ViewTiles &vt, F body) {
    __shared__ int s_item;
    const int tid = threadIdx.x + threadIdx.y * 32;
    for (;;) {
        __syncthreads();  // the previous tile is done with s_item and shared memory
        if (tid == 0) s_item = (int)atomicAdd(vt.counter, 1u);
        __syncthreads();
        const int item = s_item;
        if (item >= vt.total) break;
        int lo = 0, hi = vt.n_views - 1;  // the last view whose first tile is <= item
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(vt.view_start + mid) <= item) lo = mid;
            else hi = mid - 1;
        }
        const int local = item - __ldg(vt.view_start + lo);
        const int tx = __ldg(vt.tiles_x + lo);
        body(views[lo], local % tx, local / tx);
    }
}

template <int PPT>
__global__ void __launch_bounds__(128, RG_RIS_MIN_BLOCKS) k_initial_temporal_views(const InitialParams *views,
                                                                                     const ViewTiles vt) {
    for_each_view_tile(views, vt,
                       [](const InitialParams &p, int bx, int by) { initial_temporal_tile<PPT, 1, false>(p, bx, by); });
}
template <int TW>
__global__ void __launch_bounds__(128, RG_UNBIASED_MIN_BLOCKS) k_spatial_unbiased_views(const SpatialParams *views,
                                                                                          const ViewTiles vt) {
    for_each_view_tile(views, vt,
                       [](const SpatialParams &p, int bx, int by) { spatial_unbiased_tile<TW, 1, false>(p, bx, by); });
}
__global__ void __launch_bounds__(128) k_spatial_biased_views(const SpatialParams *views, const ViewTiles vt) {
    for_each_view_tile(views, vt,
                       [](const SpatialParams &p, int bx, int by) { spatial_biased_tile<1, false>(p, bx, by); });
}
__global__ void __launch_bounds__(128) k_shade_views(const ShadeParams *views, const ViewTiles vt) {
    for_each_view_tile(views, vt, [](const ShadeParams &p, int bx, int by) { shade_tile<1, false>(p, bx, by); });
}

// ---- candidate-count tuning of a batch (batch.cu): the views' RIS candidate
// count, and the luminance of the views' shaded images (a snapshot, then the
// sum of squared differences to it), over the shading launch's tile map.
__global__ void k_set_candidates(InitialParams *ip, int n_views, uint32_t count) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < n_views) ip[v].u.initial_light_sample_count = count;
}
// The tone value of a pixel: log(1 + luminance), so that a few firefly
// pixels (heavy-tailed near-field lights) do not dominate the variance.
// mode 0: lum[first_px[v] + i] = tone value of pixel i of view v; mode 1: adds
// sum (tone - lum)^2 over finite differences to acc[0] and their count to
// acc[1]
__global__ void __launch_bounds__(128) k_views_luminance(const ShadeParams *views, const ViewTiles vt,
                                                         const long long *first_px, float *lum, int mode,
                                                         double *acc) {
    __shared__ int s_item;
    const int tid = threadIdx.x + threadIdx.y * 32;
    double sq = 0.0, cnt = 0.0;
    for (;;) {
        __syncthreads();
        if (tid == 0) s_item = (int)atomicAdd(vt.counter, 1u);
        __syncthreads();
        const int item = s_item;
        if (item >= vt.total) break;
        int lo = 0, hi = vt.n_views - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(vt.view_start + mid) <= item) lo = mid;
            else hi = mid - 1;
        }
        const int local = item - __ldg(vt.view_start + lo);
        const int tx = __ldg(vt.tiles_x + lo);
        const ShadeParams &p = views[lo];
        const int x = (local % tx) * 32 + threadIdx.x, y = (local / tx) * 4 + threadIdx.y;
        const int W = (int)p.u.buffer_size[0], H = (int)p.u.buffer_size[1];
        if (x < W && y < H) {
            const size_t i = (size_t)y * (size_t)W + (size_t)x;
            const float4 c = p.out[i];
            const float l = log1pf(fmaxf(luminance(c.x, c.y, c.z), 0.0f));
            float *slot = lum + first_px[lo] + (long long)i;
            if (mode == 0) {
                *slot = l;
            } else {
                const double d = (double)l - (double)*slot;
                if (isfinite(d)) {
                    sq += d * d;
                    cnt += 1.0;
                }
            }
        }
    }
    if (mode == 1) {
        for (int o = 16; o > 0; o >>= 1) {
            sq += __shfl_xor_sync(0xffffffffu, sq, o);
            cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        }
        if ((tid & 31) == 0) {
            atomicAdd(acc, sq);
            atomicAdd(acc + 1, cnt);
        }
    }
}

// frame index of every view for the next run: start + (number of runs so far)
__global__ void k_advance_frames(InitialParams *ip, SpatialParams *sp, int n_views, int n_spatial,
                                 const uint32_t *start_frame, uint32_t *runs, uint32_t *frame_out) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t r = *runs;  // the increment is a later launch (k_count_run)
    if (v < n_views) {
        const uint32_t f = start_frame[v] + r;
        ip[v].u.frame = f;
        for (int k = 0; k < n_spatial; ++k) sp[(size_t)k * n_views + v].u.frame = f;
        if (frame_out) frame_out[v] = f;
    }
}
__global__ void k_count_run(uint32_t *runs) { *runs += 1u; }

size_t ris_smem_bytes(int ppt, int depth, int samples = 1) {
    return (size_t)128 * ppt * samples * (sizeof(rgpool::Ray) + sizeof(float4) + 1) +
           128 * (size_t)(RG_STACK_LOCAL ? 0 : depth) * sizeof(int);
}

// Calls f.template operator()<R, MIS>() for the scene's reservoir format.
template <typename F>
cudaError_t with_format(const DevScene &s, F &&f) {
    if (s.res_samples == 2) return s.res_mis ? f(FormatTag<2, true>{}) : f(FormatTag<2, false>{});
    return s.res_mis ? f(FormatTag<1, true>{}) : f(FormatTag<1, false>{});
}

dim3 pixel_grid(int w, int h, dim3 block) {
    return dim3((unsigned)((w + (int)block.x - 1) / (int)block.x), (unsigned)((h + (int)block.y - 1) / (int)block.y));
}

}  // namespace

GBufView make_view(const rg_gbuffer *g) {
    GBufView v;
    v.w = g->width;
    v.h = g->height;
    v.albedo = static_cast<const uint32_t *>(g->albedo);
    v.normal = static_cast<const uint2 *>(g->normal);
    v.material = static_cast<const uint32_t *>(g->material);
    v.wpos = static_cast<const float4 *>(g->world_pos);
    v.depth = static_cast<const float *>(g->depth);
    // the default's explicit VkFormat numbers load like the default
    v.nfmt = g->normal_format == RG_FORMAT_R16G16B16A16_SFLOAT ? 0 : g->normal_format;
    v.pfmt = g->world_pos_format == RG_FORMAT_R32G32B32A32_SFLOAT ? 0 : g->world_pos_format;
    v.dfmt = (g->depth_format == RG_FORMAT_D32_SFLOAT || g->depth_format == RG_FORMAT_D32_SFLOAT_S8_UINT)
                 ? 0 : g->depth_format;
    return v;
}

cudaError_t launch_initial_temporal(const DevScene &s, const GBufView &cur, const GBufView *prev,
                                    const rg_reservoir *prev_res, rg_reservoir *out, const rg_restir_uniforms &u,
                                    const mlp::LearnedRis *learned, cudaStream_t st, const VisCache *vc) {
    InitialParams p;
    if (vc) p.vc = *vc;
    p.learned = learned ? *learned : mlp::LearnedRis{};
    p.s = s;
    p.cur = cur;
    p.has_prev = prev != nullptr && prev_res != nullptr;
    p.prev = prev ? *prev : cur;
    p.prev_res = prev_res;
    p.out = out;
    p.u = u;
    return with_format(s, [&](auto tag) {
        constexpr int R = decltype(tag)::R;
        constexpr bool MIS = decltype(tag)::MIS;
        constexpr int ppt = R == 1 ? kRisPpt : 2;  // pool size per block kept near the single-sample one
        const dim3 block(32, 4);
        const dim3 grid((u.screen_size[0] + 31u) / 32u, (u.screen_size[1] + 4u * ppt - 1u) / (4u * ppt));
        const size_t smem = ris_smem_bytes(ppt, s.depth, R);
        cudaError_t e = cudaFuncSetAttribute(k_initial_temporal<ppt, R, MIS>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k_initial_temporal<ppt, R, MIS><<<grid, block, smem, st>>>(p);
        return cudaGetLastError();
    });
}

cudaError_t launch_spatial_biased(const DevScene &s, const GBufView &g, const rg_reservoir *in, rg_reservoir *out,
                                  const rg_restir_uniforms &u, int iter, cudaStream_t st) {
    SpatialParams p;
    p.s = s;
    p.g = g;
    p.in = in;
    p.out = out;
    p.u = u;
    p.iter = iter;
    p.num_neighbors = 0;
    p.cos_thr = cos_cw(u.spatial_normal_threshold * kDeg2Rad);
    return with_format(s, [&](auto tag) {
        const dim3 block(32, 4);
        k_spatial_biased<decltype(tag)::R, decltype(tag)::MIS>
            <<<pixel_grid((int)u.screen_size[0], (int)u.screen_size[1], block), block, 0, st>>>(p);
        return cudaGetLastError();
    });
}

cudaError_t launch_spatial_unbiased(const DevScene &s, const GBufView &g, const rg_reservoir *in, rg_reservoir *out,
                                    const rg_restir_uniforms &u, int num_neighbors, int pass_index, cudaStream_t st,
                                    const VisCache *vc) {
    if (num_neighbors < 0 || num_neighbors > kMaxNeighbors) return cudaErrorInvalidValue;
    SpatialParams p;
    if (vc) p.vc = *vc;
    p.s = s;
    p.g = g;
    p.in = in;
    p.out = out;
    p.u = u;
    p.iter = pass_index;
    p.num_neighbors = num_neighbors;
    p.cos_thr = 0.0f;
    return with_format(s, [&](auto tag) {
        constexpr int R = decltype(tag)::R;
        constexpr bool MIS = decltype(tag)::MIS;
        constexpr int BT = RG_UNBIASED_BT;  // block threads: the pixels sharing one ray pool
        const dim3 block(32, BT / 32);
        const size_t smem = unbiased_smem_bytes(num_neighbors, RG_STACK_LOCAL ? 0 : s.depth, R, MIS, BT);
        cudaError_t e = cudaFuncSetAttribute(k_spatial_unbiased<32, R, MIS, BT>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        if (RG_SMEM_CARVEOUT >= 0) {
            e = cudaFuncSetAttribute(k_spatial_unbiased<32, R, MIS, BT>,
                                     cudaFuncAttributePreferredSharedMemoryCarveout, RG_SMEM_CARVEOUT);
            if (e != cudaSuccess) return e;
        }
        k_spatial_unbiased<32, R, MIS, BT>
            <<<pixel_grid((int)u.screen_size[0], (int)u.screen_size[1], block), block, smem, st>>>(p);
        return cudaGetLastError();
    });
}

cudaError_t launch_shade(const DevScene &s, const GBufView &g, const rg_reservoir *res, const rg_lighting_uniforms &u,
                         float4 *out, cudaStream_t st) {
    ShadeParams p;
    p.s = s;
    p.g = g;
    p.res = res;
    p.out = out;
    p.u = u;
    return with_format(s, [&](auto tag) {
        const dim3 block(32, 4);
        const dim3 grid((u.buffer_size[0] + 31u) / 32u, (u.buffer_size[1] + 4u * RG_SHADE_PPT - 1u) / (4u * RG_SHADE_PPT));
        k_shade<decltype(tag)::R, decltype(tag)::MIS><<<grid, block, 0, st>>>(p);
        return cudaGetLastError();
    });
}

cudaError_t launch_visibility_batch(const DevScene &s, const float4 *p1, const float4 *p2, uint8_t *out, int n,
                                    cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const size_t smem = kVisChunk * (sizeof(rgpool::Ray) + sizeof(float4)) + 128 * (size_t)(RG_STACK_LOCAL ? 0 : s.depth) * sizeof(int);
    cudaError_t e = cudaFuncSetAttribute(k_visibility_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_visibility_batch<<<(unsigned)((n + kVisChunk - 1) / kVisChunk), 128, smem, st>>>(s, p1, p2, out, n);
    return cudaGetLastError();
}

// ---------------------------------------------------------------- views: parameter records and launches
size_t view_params_size(int kind) {
    return kind == 0 ? sizeof(InitialParams) : kind == 1 ? sizeof(SpatialParams) : sizeof(ShadeParams);
}

void make_initial_params(void *dst, const DevScene &s, const GBufView &cur, const GBufView *prev,
                         const rg_reservoir *prev_res, rg_reservoir *out, const rg_restir_uniforms &u,
                         const mlp::LearnedRis *learned, const VisCache *vc) {
    InitialParams p;
    if (vc) p.vc = *vc;
    p.learned = learned ? *learned : mlp::LearnedRis{};
    p.s = s;
    p.cur = cur;
    p.has_prev = prev != nullptr && prev_res != nullptr;
    p.prev = prev ? *prev : cur;
    p.prev_res = prev_res;
    p.out = out;
    p.u = u;
    memcpy(dst, &p, sizeof(p));
}

void make_spatial_params(void *dst, const DevScene &s, const GBufView &g, const rg_reservoir *in, rg_reservoir *out,
                         const rg_restir_uniforms &u, bool unbiased, int iter_or_pass, int num_neighbors,
                         const VisCache *vc) {
    SpatialParams p;
    if (vc) p.vc = *vc;
    p.s = s;
    p.g = g;
    p.in = in;
    p.out = out;
    p.u = u;
    p.iter = iter_or_pass;
    p.num_neighbors = unbiased ? num_neighbors : 0;
    p.cos_thr = unbiased ? 0.0f : cos_cw(u.spatial_normal_threshold * kDeg2Rad);
    memcpy(dst, &p, sizeof(p));
}

void make_shade_params(void *dst, const DevScene &s, const GBufView &g, const rg_reservoir *res,
                       const rg_lighting_uniforms &u, float4 *out) {
    ShadeParams p;
    p.s = s;
    p.g = g;
    p.res = res;
    p.out = out;
    p.u = u;
    memcpy(dst, &p, sizeof(p));
}

void view_tile_shape(int kind, int variant, int *tw, int *th) {
    if (kind == 0) { *tw = 32; *th = 4 * variant; }       // variant: pixels per thread
    else if (kind == 1) { *tw = variant; *th = 128 / variant; }  // variant: tile width
    else { *tw = 32; *th = 4; }
}

namespace {
template <typename P>
cudaError_t views_grid(void (*kernel)(const P *, const ViewTiles), size_t smem, int total, int ctas_per_sm,
                       int *grid) {
    int dev = 0, sms = 0, occ = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, 128, smem);
    if (e != cudaSuccess) return e;
    if (occ < 1) return cudaErrorInvalidConfiguration;
    const int per_sm = ctas_per_sm > 0 && ctas_per_sm < occ ? ctas_per_sm : occ;
    *grid = sms * per_sm < total ? sms * per_sm : total;
    return cudaSuccess;
}
template <typename P>
cudaError_t views_launch(void (*kernel)(const P *, const ViewTiles), const void *views, const ViewTiles &vt,
                         size_t smem, int grid, cudaStream_t st) {
    if (grid < 1) return cudaSuccess;
    kernel<<<grid, dim3(32, 4), smem, st>>>(static_cast<const P *>(views), vt);
    return cudaGetLastError();
}
// Calls f(kernel, smem) for the kernel of (kind, variant).
template <typename F>
cudaError_t with_views_kernel(int kind, int variant, bool unbiased, int num_neighbors, int depth, F f) {
    if (kind == 0) {
        const size_t smem = ris_smem_bytes(variant, depth);
        switch (variant) {
            case 1: return f(k_initial_temporal_views<1>, smem);
            case 2: return f(k_initial_temporal_views<2>, smem);
            case 4: return f(k_initial_temporal_views<4>, smem);
            default: return cudaErrorInvalidValue;
        }
    }
    if (kind == 1) {
        if (!unbiased) return f(k_spatial_biased_views, (size_t)0);
        if (num_neighbors < 0 || num_neighbors > kMaxNeighbors) return cudaErrorInvalidValue;
        const size_t smem = unbiased_smem_bytes(num_neighbors, RG_STACK_LOCAL ? 0 : depth);
        switch (variant) {
            case 8: return f(k_spatial_unbiased_views<8>, smem);
            case 16: return f(k_spatial_unbiased_views<16>, smem);
            case 32: return f(k_spatial_unbiased_views<32>, smem);
            default: return cudaErrorInvalidValue;
        }
    }
    return f(k_shade_views, (size_t)0);
}
}  // namespace

cudaError_t views_pass_grid(int kind, int variant, bool unbiased, int num_neighbors, int depth, int total,
                            int ctas_per_sm, int *grid) {
    return with_views_kernel(kind, variant, unbiased, num_neighbors, depth, [&](auto kernel, size_t smem) {
        return views_grid(kernel, smem, total, ctas_per_sm, grid);
    });
}

cudaError_t launch_views_pass(int kind, int variant, bool unbiased, int num_neighbors, int depth, const void *params,
                              const ViewTiles &vt, int grid, cudaStream_t st) {
    return with_views_kernel(kind, variant, unbiased, num_neighbors, depth, [&](auto kernel, size_t smem) {
        return views_launch(kernel, params, vt, smem, grid, st);
    });
}

cudaError_t launch_set_candidates(void *initial_params, int n_views, uint32_t count, cudaStream_t st) {
    k_set_candidates<<<(n_views + 127) / 128, 128, 0, st>>>(static_cast<InitialParams *>(initial_params), n_views,
                                                             count);
    return cudaGetLastError();
}

cudaError_t launch_views_luminance(const void *shade_params, const ViewTiles &vt, const long long *first_px, float *lum,
                                   int mode, double *acc, int grid, cudaStream_t st) {
    if (grid < 1) return cudaSuccess;
    k_views_luminance<<<grid, dim3(32, 4), 0, st>>>(static_cast<const ShadeParams *>(shade_params), vt, first_px, lum,
                                                    mode, acc);
    return cudaGetLastError();
}

cudaError_t launch_advance_frames(void *initial_params, void *spatial_params, int n_views, int n_spatial,
                                  const uint32_t *start_frame, uint32_t *runs, uint32_t *frame_out, cudaStream_t st) {
    k_advance_frames<<<(n_views + 127) / 128, 128, 0, st>>>(static_cast<InitialParams *>(initial_params),
                                                             static_cast<SpatialParams *>(spatial_params), n_views,
                                                             n_spatial, start_frame, runs, frame_out);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_count_run<<<1, 1, 0, st>>>(runs);
    return cudaGetLastError();
}
