// mlp.cu -- kernels of the learned light-cluster proposal (network in mlp.cuh).
//
// The forward pass of a 128-pixel tile is one CTA on the tcgen05 tensor cores:
// features -> x tile (shared memory, bf16) -> three 64-wide layers (MMA into
// tensor memory, bias + ReLU + bf16 epilogue back into shared memory) -> the
// cluster logit layer in chunks of 64 clusters, double-buffered in tensor
// memory so that the MMA of chunk c+1 runs under the epilogue of chunk c.
// Weight tiles arrive by cp.async from bf16 images that are already in the MMA
// operand layout.  Logits never leave the SM.  Three epilogues:
//   kLse     log-sum-exp, arg-max and its probability per row;
// Exponentials are 2^x on the MUFU unit with the log2(e) scale folded into
// one FMA per logit.
//   kSample  the learned-branch candidates: each row walks its softmax CDF
//            once with its uniforms drawn as ascending order statistics; a
//            uniform's column inside the 32-column piece that holds it is
//            found by binary search over the piece's running sums, and its
//            probability is the width of its interval.  (The uniform-branch
//            candidates, a light and q of its cluster, are written at the
//            end of kLse.)
//   kGrad    for training: dz = d(loss)/d(logits) = (softmax - onehot) / n
//            per chunk into a bf16 tile, then dh3 += dz W4^T on the tensor
//            cores (accumulated in tensor memory over the chunks), and the
//            cross-entropy loss.  dz never leaves the SM; dW4 and db4 come
//            from k_mlp_dw4, which recomputes the logits chunk by chunk.
// Every wait on the tensor core is bounded; a CTA whose wait runs out records
// an error, waits (bounded) for its last MMA, frees its tensor memory and
// leaves.  At most four CTAs share an SM: each holds 128 tensor-memory
// columns and uses more than a fifth of the shared memory.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "mlp.cuh"
#include "rg_math.cuh"
#include "umma.cuh"

using namespace rgm;

namespace {

constexpr int kRows = 128;                 // rows (pixels) per CTA
constexpr int kChunkN = mlp::kChunkN;      // clusters per logit MMA chunk
constexpr uint32_t kMaxPolls = 1u << 26;   // bounded mbarrier waits
constexpr int kTmemCols = 2 * kChunkN;    // two chunk accumulators; the hidden layers use them first
constexpr int kTmemColsGrad = 4 * kChunkN;  // kGrad: plus the dh3 accumulator (64 columns), rounded up

// shared-memory map (bytes)
constexpr int kOffX = 0;                               // x tile, 128 x 16 bf16
constexpr int kOffH = kOffX + kRows * mlp::kIn * 2;    // h tile, 128 x 64 bf16
constexpr int kOffW1 = kOffH + kRows * mlp::kH * 2;    // W1^T image, 64 x 16
constexpr int kOffW2 = kOffW1 + mlp::kH * mlp::kIn * 2;
constexpr int kOffW3 = kOffW2 + mlp::kH * mlp::kH * 2;
constexpr int kOffB = kOffW3 + mlp::kH * mlp::kH * 2;  // two chunk tiles, 128 x 64
constexpr int kChunkBytes = kChunkN * mlp::kH * 2;
constexpr int kOffBias = kOffB + 2 * kChunkBytes;      // b1 | b2 | b3
constexpr int kSmemUsed = kOffBias + 3 * mlp::kH * 4;
// kGrad: the logit-gradient tile (128 rows x 64 clusters, K-major over
// clusters) and two W4 chunk tiles (64 hidden x 64 clusters) for dh3 += dz W4^T
constexpr int kOffDz = (kSmemUsed + 1023) / 1024 * 1024;
constexpr int kOffWk = kOffDz + kRows * kChunkN * 2;
constexpr int kWkBytes = mlp::kH * kChunkN * 2;
constexpr int kSmemGrad = kOffWk + 2 * kWkBytes;
constexpr int kSmemMin = 52 * 1024;                    // caps residency at four CTAs per SM (TMEM: 4 x 128 columns)
constexpr int kWeightImgBytes = (mlp::kH * mlp::kIn + 2 * mlp::kH * mlp::kH) * 2;

enum { kLse = 0, kSample = 1, kGrad = 2 };

__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

constexpr float kLog2e = 1.44269504088896341f;
// 2^x by the MUFU instruction (results below 2^-126 flush to zero)
__device__ __forceinline__ float ex2(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
// A 32-column piece of one row is held as 16 float2 pairs (columns 2k, 2k+1),
// so that adds and FMAs run as packed FP32x2 operations (each lane of a
// packed op rounds exactly like the scalar op).
__device__ __forceinline__ float col(const float2 (&v)[16], int i) { return (i & 1) ? v[i >> 1].y : v[i >> 1].x; }
// max of three (IEEE maxNum, like fmaxf)
__device__ __forceinline__ float max3f(float a, float b, float c) {
    float y;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(y) : "f"(a), "f"(b), "f"(c));
    return y;
}
__device__ __forceinline__ float max32(const float2 (&v)[16]) {
    float a[11];
#pragma unroll
    for (int k = 0; k < 10; ++k) a[k] = max3f(col(v, 3 * k), col(v, 3 * k + 1), col(v, 3 * k + 2));
    a[10] = fmaxf(col(v, 30), col(v, 31));
    const float b0 = max3f(a[0], a[1], a[2]), b1 = max3f(a[3], a[4], a[5]), b2 = max3f(a[6], a[7], a[8]);
    return fmaxf(max3f(b0, b1, b2), fmaxf(a[9], a[10]));
}
__device__ __forceinline__ float sum32(const float2 (&v)[16]) {
    float2 t[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) t[k] = __fadd2_rn(v[k], v[k + 8]);
#pragma unroll
    for (int k = 0; k < 4; ++k) t[k] = __fadd2_rn(t[k], t[k + 4]);
    t[0] = __fadd2_rn(t[0], t[2]);
    t[1] = __fadd2_rn(t[1], t[3]);
    t[0] = __fadd2_rn(t[0], t[1]);
    return t[0].x + t[0].y;
}
// v[k] = 2^(v[k] * log2(e) + off), both columns of every pair
__device__ __forceinline__ void exp_piece(float2 (&v)[16], float off) {
    const float2 l2 = make_float2(kLog2e, kLog2e), o2 = make_float2(off, off);
#pragma unroll
    for (int k = 0; k < 16; ++k) {
        const float2 t = __ffma2_rn(v[k], l2, o2);
        v[k] = make_float2(ex2(t.x), ex2(t.y));
    }
}
__device__ __forceinline__ float lg2(float x) {
    float y;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcp(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
// Next of n ascending order statistics of U(0,1) given the previous one:
// 1 - (1 - prev) * V^(1/remaining), V uniform; the power as 2^(log2(V) / n)
// on the MUFU unit (V = 0 gives 1: beyond every CDF total).
__device__ __forceinline__ float next_order_stat(Pcg &rng, float prev, int remaining) {
    const float v = rand_float(rng);
    return 1.0f - (1.0f - prev) * ex2(lg2(v) * rcp((float)remaining));
}
// z of cluster cl for the row whose h3 is h: FP32 dot (even and odd terms
// in two packed FMA chains) with the bf16 W4^T image (chunk tiles in the MMA
// operand layout) plus b4.
__device__ __forceinline__ float logit_of(const mlp::ProposalDev &pd, const float (&h)[64], int cl) {
    const unsigned char *tile = reinterpret_cast<const unsigned char *>(pd.w4t) + (size_t)(cl / kChunkN) * kChunkBytes;
    float2 z = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const uint4 w = __ldg(reinterpret_cast<const uint4 *>(tile + umma::kmajor_offset(cl % kChunkN, 8 * j, mlp::kH)));
        const __nv_bfloat162 *b = reinterpret_cast<const __nv_bfloat162 *>(&w);
#pragma unroll
        for (int i = 0; i < 4; ++i)
            z = __ffma2_rn(make_float2(h[8 * j + 2 * i], h[8 * j + 2 * i + 1]), __bfloat1622float2(b[i]), z);
    }
    return (z.x + z.y) + __ldg(pd.b4e + cl);
}

__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gsrc) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(umma::smem_addr(smem_dst)), "l"(gsrc)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_one() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

__device__ __forceinline__ void copy_bytes(unsigned char *dst, const unsigned char *src, int bytes) {
    for (int o = threadIdx.x * 16; o < bytes; o += blockDim.x * 16) cp_async16(dst + o, src + o);
}

struct FusedParams {
    mlp::ProposalDev pd;
    GBufView g;
    float cam[3];
    const int32_t *rows;       // pixel of each row; nullptr: row = pixel
    int n;
    float4 *stat;              // per row: lse, arg-max cluster (int bits), its probability, 0
    // training (kLse with save != 0, kGrad)
    int save;
    __nv_bfloat16 *x, *h1, *h2, *h3;  // [n x 16], [n x 64] x 3
    const int32_t *target;     // cluster per row, -1: no target
    float *dh3;                // [n x 64] FP32: d(loss)/d(h3)
    float inv_n;
    float *loss_sum;
    // sampling
    mlp::Candidate *cand;      // [n x kCand]
    uint32_t frame;
    int n_cand;
    int *err;
    // batched views (kViews): row -> view by binary search over first_row
    const mlp::ViewRows *views;
    int n_views;
    const uint32_t *frames;    // per view
};

// Features of one pixel (mlp.cuh), each rounded to bf16; non-finite values
// (a pixel at the camera position) become 0.
__device__ __forceinline__ void features(const mlp::ProposalDev &pd, const float4 *wpos_plane, const uint2 *normal_plane,
                                         float cx, float cy, float cz, size_t px, float x[mlp::kIn]) {
    const float4 wp = __ldg(wpos_plane + px);
    const uint2 nb = __ldg(normal_plane + px);
    const f3 wpos = mk(wp.x, wp.y, wp.z);
    const f3 n = mk(half_bits_to_float((uint16_t)(nb.x & 0xffffu)), half_bits_to_float((uint16_t)(nb.x >> 16)),
                    half_bits_to_float((uint16_t)(nb.y & 0xffffu)));
    const f3 v = normalize(mk(cx, cy, cz) - wpos);
    x[0] = (wpos.x - pd.box_center.x) * pd.box_inv_half.x;
    x[1] = (wpos.y - pd.box_center.y) * pd.box_inv_half.y;
    x[2] = (wpos.z - pd.box_center.z) * pd.box_inv_half.z;
    x[3] = n.x; x[4] = n.y; x[5] = n.z;
    x[6] = v.x; x[7] = v.y; x[8] = v.z;
#pragma unroll
    for (int i = 0; i < mlp::kIn; ++i) {
        const float t = i < mlp::kInUsed ? x[i] : 0.0f;
        x[i] = isfinite(t) ? bf16r(t) : 0.0f;
    }
}

// Writes 8 consecutive bf16 values (k = k0..k0+7) of row r into a K-major tile.
__device__ __forceinline__ void put8(unsigned char *tile, int r, int k0, int K, const float *v) {
    __align__(16) __nv_bfloat16 b[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) b[i] = __float2bfloat16_rn(v[i]);
    *reinterpret_cast<uint4 *>(tile + umma::kmajor_offset(r, k0, K)) = *reinterpret_cast<const uint4 *>(b);
}
__device__ __forceinline__ void store8(__nv_bfloat16 *dst, const float *v) {
    __align__(16) __nv_bfloat16 b[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) b[i] = __float2bfloat16_rn(v[i]);
    *reinterpret_cast<uint4 *>(dst) = *reinterpret_cast<const uint4 *>(b);
}

// Bounded wait for an MMA commit; warp-uniform result.
__device__ __forceinline__ bool mma_wait(uint64_t *mbar, uint32_t parity) {
    bool w = umma::mbar_wait(mbar, parity, kMaxPolls);
    umma::fence_after_sync();
    return __all_sync(0xffffffffu, w);
}

template <int kMode, bool kViews>
__global__ void __launch_bounds__(128, 4) k_mlp_fused(const FusedParams p) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ uint64_t mbar_layer, mbar_chunk[2], mbar_dh;
    __shared__ uint32_t tmem_base;
    constexpr int kCols = kMode == kGrad ? kTmemColsGrad : kTmemCols;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int row = blockIdx.x * kRows + tid;
    const bool valid = row < p.n;
    size_t px;
    uint32_t frame = p.frame;
    int n_cand = p.n_cand;
    const float4 *wpos_plane = p.g.wpos;
    const uint2 *normal_plane = p.g.normal;
    float cx = p.cam[0], cy = p.cam[1], cz = p.cam[2];
    if constexpr (kViews) {
        // the view holding this row: the last one whose first row is <= row
        const uint32_t r = valid ? (uint32_t)row : 0u;
        int lo = 0, hi = p.n_views - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (__ldg(&p.views[mid].first_row) <= r) lo = mid;
            else hi = mid - 1;
        }
        const mlp::ViewRows &vr = p.views[lo];
        px = (size_t)(r - vr.first_row);
        frame = __ldg(p.frames + lo);
        n_cand = vr.n_cand;
        wpos_plane = vr.g.wpos;
        normal_plane = vr.g.normal;
        cx = vr.cam[0];
        cy = vr.cam[1];
        cz = vr.cam[2];
    } else {
        px = valid ? (p.rows ? (size_t)p.rows[row] : (size_t)row) : 0;
    }
    const int nch = p.pd.c / kChunkN;
    const mlp::Layout L(p.pd.c);
    unsigned char *xtile = smem + kOffX, *htile = smem + kOffH;
    unsigned char *btile[2] = {smem + kOffB, smem + kOffB + kChunkBytes};
    float *bias = reinterpret_cast<float *>(smem + kOffBias);
    const unsigned char *w4img = reinterpret_cast<const unsigned char *>(p.pd.w4t);

    unsigned char *dztile = smem + kOffDz;
    unsigned char *wkslot[2] = {smem + kOffWk, smem + kOffWk + kWkBytes};
    const unsigned char *w4kimg = reinterpret_cast<const unsigned char *>(p.pd.w4k);

    // weights and the first two logit chunks start moving
    copy_bytes(smem + kOffW1, reinterpret_cast<const unsigned char *>(p.pd.w123img), kWeightImgBytes);
    copy_bytes(btile[0], w4img, kChunkBytes);
    if (kMode == kGrad) copy_bytes(wkslot[0], w4kimg, kWkBytes);
    cp_async_commit();
    if (nch > 1) {
        copy_bytes(btile[1], w4img + kChunkBytes, kChunkBytes);
        if (kMode == kGrad) copy_bytes(wkslot[1], w4kimg + kWkBytes, kWkBytes);
    }
    cp_async_commit();
    for (int i = tid; i < 3 * mlp::kH; i += blockDim.x) {
        const size_t b = i < mlp::kH ? L.b1 : i < 2 * mlp::kH ? L.b2 : L.b3;
        bias[i] = p.pd.params[b + (size_t)(i % mlp::kH)];
    }
    if (warp == 0) umma::tmem_alloc(&tmem_base, kCols);
    if (tid == 0) {
        umma::mbar_init(&mbar_layer, 1);
        umma::mbar_init(&mbar_chunk[0], 1);
        umma::mbar_init(&mbar_chunk[1], 1);
        umma::mbar_init(&mbar_dh, 1);
    }
    {
        float x[mlp::kIn];
        if (valid) {
            features(p.pd, wpos_plane, normal_plane, cx, cy, cz, px, x);
        } else {
#pragma unroll
            for (int i = 0; i < mlp::kIn; ++i) x[i] = 0.0f;
        }
        put8(xtile, tid, 0, mlp::kIn, x);
        put8(xtile, tid, 8, mlp::kIn, x + 8);
        if (kMode == kLse && p.save && valid) {
            store8(p.x + (size_t)row * mlp::kIn, x);
            store8(p.x + (size_t)row * mlp::kIn + 8, x + 8);
        }
    }

    // kSample: which candidate slots take the learned branch, and the learned
    // slots' uniforms as ascending order statistics, from the pixel's own PCG
    // stream (two draws per slot: branch, uniform light; then one per
    // learned slot).  The k-th smallest uniform goes to the k-th learned slot.
    uint32_t lmask = 0;  // learned slots not yet assigned
    int n_u = 0, k_u = 0;
    float u_prev = 0.0f;
    Pcg rng{};
    if (kMode == kSample && valid) {
        rng = pcg_seed((uint64_t)frame * mlp::kSeedMul + mlp::kSeedAdd, (uint64_t)px);
        for (int j = 0; j < n_cand; ++j) {
            const float u0 = rand_float(rng);
            rand_float(rng);
            if (u0 < p.pd.mix) lmask |= 1u << j;
        }
        n_u = __popc(lmask);
    }

    cp_async_wait_one();
    umma::fence_proxy_async();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = tmem_base;
    bool ok = true;
    // thread 0's most recent MMA commit (the barrier and the parity of that
    // phase): on a timeout it waits, bounded, for that commit, which covers
    // every MMA issued before it
    uint64_t *last_mbar = nullptr;
    uint32_t last_parity = 0;

    // ---- hidden layers: MMA into columns 64*l, epilogue into the h tile
    const unsigned char *wimg[3] = {smem + kOffW1, smem + kOffW2, smem + kOffW3};
    __nv_bfloat16 *hsave[3] = {p.h1, p.h2, p.h3};
    for (int l = 0; l < 3 && ok; ++l) {
        // layer l accumulates in columns 64*(l&1): layer 3 reuses layer 1's,
        // whose loads completed before the barrier that preceded layer 2
        const uint32_t lcol = tmem + (uint32_t)(64 * (l & 1));
        if (tid == 0) {
            umma::mma_chunk(lcol, l == 0 ? xtile : htile, wimg[l], l == 0 ? mlp::kIn : mlp::kH, kRows, mlp::kH, false);
            umma::mma_commit(&mbar_layer);
            last_mbar = &mbar_layer;
            last_parity = (uint32_t)(l & 1);
        }
        const bool w = mma_wait(&mbar_layer, (uint32_t)(l & 1));
        if (w) {
            float v[64];
            umma::tmem_ld32(lcol, warp, 0, *reinterpret_cast<float(*)[32]>(v));
            umma::tmem_ld32(lcol, warp, 32, *reinterpret_cast<float(*)[32]>(v + 32));
#pragma unroll
            for (int j = 0; j < 64; ++j) v[j] = bf16r(fmaxf(v[j] + bias[64 * l + j], 0.0f));
#pragma unroll
            for (int j = 0; j < 64; j += 8) put8(htile, tid, j, mlp::kH, v + j);
            if (kMode == kLse && p.save && valid) {
#pragma unroll
                for (int j = 0; j < 64; j += 8) store8(hsave[l] + (size_t)row * mlp::kH + j, v + j);
            }
        }
        umma::fence_proxy_async();
        umma::fence_before_sync();
        ok = __syncthreads_and(w) != 0;
        umma::fence_after_sync();
    }

    // ---- logit chunks
    float m = -INFINITY, s = 0.0f;  // kLse: running max and sum
    int amax = 0;
    float lse = 0.0f, cum = 0.0f;   // kSample / kGrad
    float next_u = INFINITY;  // no uniform left (cum never exceeds it, even when it overflows)
    int amax_row = 0;
    float qmax_row = 0.0f;
    int target = -1;
    float zt = 0.0f;
    if (kMode != kLse && valid) {
        const float4 st = p.stat[row];
        lse = st.x;
        amax_row = __float_as_int(st.y);
        qmax_row = st.z;
        if (kMode == kSample) {
            if (n_u > 0) {
                u_prev = next_order_stat(rng, 0.0f, n_u);
                k_u = 1;
                next_u = u_prev;
            }
        } else {
            target = p.target[row];
        }
    }
    const float nl2 = -lse * kLog2e;
    // kSample: the learned slot of the current uniform gets cluster col with q
    auto take = [&](int col, float q) {
        if (!(q > 0.0f)) {  // rounding put the uniform on an empty column: the most probable cluster
            col = amax_row;
            q = qmax_row;
        }
        const int slot = __ffs(lmask) - 1;
        lmask &= lmask - 1;
        p.cand[(size_t)row * mlp::kCand + slot] = mlp::Candidate{-1 - col, q};
        if (k_u < n_u) {
            u_prev = next_order_stat(rng, u_prev, n_u - k_u);
            ++k_u;
            next_u = u_prev;
        } else {
            next_u = INFINITY;
        }
    };
    if (ok && tid == 0) {
        umma::mma_chunk(tmem, htile, btile[0], mlp::kH, kRows, kChunkN, false);
        umma::mma_commit(&mbar_chunk[0]);
        last_mbar = &mbar_chunk[0];
        last_parity = 0;
    }
    // `ok` changes only at block barriers (uniform); `ok_warp` records this
    // warp's waits and joins `ok` at the next barrier, so every warp passes
    // the same sequence of barriers whatever fails.
    bool ok_warp = true;
    for (int c = 0; c < nch; ++c) {
        if (!ok) break;
        if (c + 1 < nch) {
            cp_async_wait_all();
            umma::fence_proxy_async();
            umma::fence_before_sync();
            ok = __syncthreads_and(ok_warp) != 0;
            umma::fence_after_sync();
            if (!ok) break;
            if (tid == 0) {
                umma::mma_chunk(tmem + (uint32_t)(((c + 1) & 1) * kChunkN), htile, btile[(c + 1) & 1], mlp::kH, kRows,
                                kChunkN, false);
                umma::mma_commit(&mbar_chunk[(c + 1) & 1]);
                last_mbar = &mbar_chunk[(c + 1) & 1];
                last_parity = (uint32_t)(((c + 1) >> 1) & 1);
            }
        }
        const bool w = mma_wait(&mbar_chunk[c & 1], (uint32_t)((c >> 1) & 1));
        ok_warp = ok_warp && w;
        if (w) {
        if (c + 2 < nch) {
            copy_bytes(btile[c & 1], w4img + (size_t)(c + 2) * kChunkBytes, kChunkBytes);
            cp_async_commit();
        }
        const uint32_t half = tmem + (uint32_t)((c & 1) * kChunkN);
        uint32_t raw[2][32];
        umma::tmem_ld32_issue(half, warp, 0, raw[0]);
#pragma unroll
        for (int piece = 0; piece < kChunkN / 32; ++piece) {
            umma::tmem_ld32_wait(raw[piece & 1]);
            // the next piece's load runs under this piece's arithmetic
            if (piece + 1 < kChunkN / 32) umma::tmem_ld32_issue(half, warp, (piece + 1) * 32, raw[(piece + 1) & 1]);
            const uint32_t(&rw)[32] = raw[piece & 1];
            const int col0 = c * kChunkN + piece * 32;
            const float4 *be = reinterpret_cast<const float4 *>(p.pd.b4e + col0);
            float2 v[16];  // logits z = MMA result + b4
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const float4 b = __ldg(be + q);
                v[2 * q] = __fadd2_rn(make_float2(__uint_as_float(rw[4 * q]), __uint_as_float(rw[4 * q + 1])),
                                      make_float2(b.x, b.y));
                v[2 * q + 1] = __fadd2_rn(make_float2(__uint_as_float(rw[4 * q + 2]), __uint_as_float(rw[4 * q + 3])),
                                          make_float2(b.z, b.w));
            }
            if (kMode == kLse) {
                const float mp = max32(v);
                if (mp == -INFINITY) continue;
                if (mp > m) {
#pragma unroll
                    for (int i = 31; i >= 0; --i)
                        if (col(v, i) == mp) amax = col0 + i;
                }
                exp_piece(v, -mp * kLog2e);
                const float sp = sum32(v);
                if (mp > m) {
                    s = (m == -INFINITY) ? sp : __fmaf_rn(s, ex2((m - mp) * kLog2e), sp);
                    m = mp;
                } else {
                    s = __fmaf_rn(sp, ex2((mp - m) * kLog2e), s);
                }
            } else if (kMode == kSample) {
                exp_piece(v, nl2);
                const float end = cum + sum32(v);
                // the uniforms below `end` belong to this piece
                if (valid && next_u < end) {
                    // running sums within the piece, left to right
                    float r[32];
                    r[0] = v[0].x;
#pragma unroll
                    for (int i = 1; i < 32; ++i) r[i] = r[i - 1] + col(v, i);
                    do {
                        // the column is the first whose running sum exceeds the
                        // uniform (at most the last), by binary search; its
                        // probability is the width of its interval
                        const float ul = next_u - cum;
                        float a[16];
                        int idx = 0;
                        float lo = 0.0f;
                        {
                            const bool b = r[15] <= ul;
                            lo = b ? r[15] : lo;
                            idx += b ? 16 : 0;
#pragma unroll
                            for (int j = 0; j < 16; ++j) a[j] = b ? r[16 + j] : r[j];
                        }
#pragma unroll
                        for (int h = 8; h >= 1; h >>= 1) {
                            const bool b = a[h - 1] <= ul;
                            lo = b ? a[h - 1] : lo;
                            idx += b ? h : 0;
#pragma unroll
                            for (int j = 0; j < h; ++j) a[j] = b ? a[h + j] : a[j];
                        }
                        take(col0 + idx, a[0] - lo);
                    } while (next_u < end);
                }
                cum = end;
            } else {  // kGrad: the gradient rows go to the dz tile (bf16)
                float d[32];
#pragma unroll
                for (int i = 0; i < 32; ++i) {
                    const float z = col(v, i);
                    const float pr = ex2(__fmaf_rn(z, kLog2e, nl2));
                    const bool hit = (col0 + i) == target;
                    if (hit) zt = z;
                    d[i] = target < 0 ? 0.0f : (pr - (hit ? 1.0f : 0.0f)) * p.inv_n;
                }
#pragma unroll
                for (int q = 0; q < 32; q += 8) put8(dztile, tid, piece * 32 + q, kChunkN, d + q);
            }
        }
        }  // w
        umma::fence_before_sync();
        if (kMode == kGrad) {
            // dh3 += dz_tile . W4[:, chunk]^T once every row's gradient is in the tile
            umma::fence_proxy_async();
            ok = __syncthreads_and(ok && ok_warp) != 0;
            umma::fence_after_sync();
            if (!ok) break;
            if (tid == 0) {
                umma::mma_chunk(tmem + (uint32_t)(2 * kChunkN), dztile, wkslot[c & 1], kChunkN, kRows, mlp::kH, c > 0);
                umma::mma_commit(&mbar_dh);
                last_mbar = &mbar_dh;
                last_parity = (uint32_t)(c & 1);
            }
            const bool w2 = mma_wait(&mbar_dh, (uint32_t)(c & 1));
            ok_warp = ok_warp && w2;
            if (w2 && c + 2 < nch) {  // the slot is free once this product completed
                copy_bytes(wkslot[c & 1], w4kimg + (size_t)(c + 2) * kWkBytes, kWkBytes);
                cp_async_commit();
            }
        }
    }
    ok = __syncthreads_and(ok && ok_warp) != 0;
    if (!ok) {
        if (tid == 0) {
            atomicAdd(p.err, 1);
            if (last_mbar) umma::mbar_wait(last_mbar, last_parity, kMaxPolls);
        }
        cp_async_wait_all();
    } else if (valid) {
        if (kMode == kLse) {
            const float lse_row = m + __logf(s);
            p.stat[row] = make_float4(lse_row, __int_as_float(amax), ex2((m - lse_row) * kLog2e), 0.0f);
            if (p.cand) {
                // uniform-branch candidates: the light and q of its cluster (the
                // same PCG stream as the learned branch's draws in kSample)
                float h[64];
#pragma unroll
                for (int j = 0; j < 64; j += 8) {
                    const uint4 w = *reinterpret_cast<const uint4 *>(htile + umma::kmajor_offset(tid, j, mlp::kH));
                    const __nv_bfloat162 *b = reinterpret_cast<const __nv_bfloat162 *>(&w);
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        const float2 f = __bfloat1622float2(b[i]);
                        h[j + 2 * i] = f.x;
                        h[j + 2 * i + 1] = f.y;
                    }
                }
                Pcg r2 = pcg_seed((uint64_t)frame * mlp::kSeedMul + mlp::kSeedAdd, (uint64_t)px);
                const float nl = -lse_row * kLog2e;
                // first the slots that take the uniform branch (about 1 in 10),
                // then one loop iteration per such slot of this row: the warp
                // runs as many dot products as its busiest row has slots, not
                // one per slot index that any row uses
                uint32_t umask = 0;
                {
                    Pcg r1 = r2;
                    for (int j = 0; j < n_cand; ++j) {
                        const float u0 = rand_float(r1);
                        rand_float(r1);
                        if (!(u0 < p.pd.mix)) umask |= 1u << j;
                    }
                }
                int pos = 0;  // slots of r2's stream consumed
                while (umask) {
                    const int j = __ffs(umask) - 1;
                    umask &= umask - 1;
                    for (; pos < j; ++pos) {
                        rand_float(r2);
                        rand_float(r2);
                    }
                    rand_float(r2);
                    const float u1 = rand_float(r2);
                    ++pos;
                    const int l = imin((int)((float)p.pd.n_lights * u1), p.pd.n_lights - 1);
                    const float z = logit_of(p.pd, h, __ldg(p.pd.cluster_of + l));
                    p.cand[(size_t)row * mlp::kCand + j] = mlp::Candidate{l, ex2(__fmaf_rn(z, kLog2e, nl))};
                }
            }
        } else if (kMode == kSample) {
            // uniforms beyond the rounded CDF total: the most probable cluster
            while (next_u < INFINITY) take(amax_row, qmax_row);
        }
    }
    if (kMode == kGrad && ok) {
        float d[64];
        umma::tmem_ld32(tmem + (uint32_t)(2 * kChunkN), warp, 0, *reinterpret_cast<float(*)[32]>(d));
        umma::tmem_ld32(tmem + (uint32_t)(2 * kChunkN), warp, 32, *reinterpret_cast<float(*)[32]>(d + 32));
        if (valid) {
            float4 *dst = reinterpret_cast<float4 *>(p.dh3 + (size_t)row * mlp::kH);
#pragma unroll
            for (int j = 0; j < 16; ++j) dst[j] = make_float4(d[4 * j], d[4 * j + 1], d[4 * j + 2], d[4 * j + 3]);
        }
    }
    if (kMode == kGrad && ok) {
        float l = (valid && target >= 0) ? lse - zt : 0.0f;
        for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
        if ((tid & 31) == 0 && l != 0.0f) atomicAdd(p.loss_sum, l);
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, kCols);
}

// ---------------------------------------------------------------- dW4, db4
// One CTA per (chunk of 64 clusters, slice of row tiles).  Per 128-row tile:
// the chunk's logits z = h3 . W4[:, chunk] on the tensor cores, the bf16
// gradient dz = (softmax - onehot) / n as in kGrad (same formula, so the same
// values), then dW[0..63] += h3^T dz and dW[64] += 1^T dz (db4) as one MMA
// with M = 128 and K = the tile's 128 rows, accumulated in tensor memory; the
// CTA adds its 65 x 64 result to the gradient with atomics at the end.
//
// No operand is transposed element by element: the h tile (rows x [h3 | 1 |
// 0], K-major over its 128 columns) and the dz tile (rows x clusters, K-major
// over clusters) are read a second time through MN-major descriptors, as
// [h3 | 1 | 0]^T (M = 128 columns, K = rows) and dz^T (N = clusters, K =
// rows): in the canonical no-swizzle layouts a core matrix is 8 rows of 16
// bytes either way, with SBO the step between core matrices along M/N and
// LBO the step along K.  The tiles sit at the start of a 64 KB allocation, so
// every address those descriptors can form stays inside it.
#ifndef RG_DW4_SLICE_CTAS
#define RG_DW4_SLICE_CTAS 4
#endif
struct Dw4Params {
    mlp::ProposalDev pd;
    const __nv_bfloat16 *h3;   // [n x 64]
    const float4 *stat;        // lse per row
    const int32_t *target;
    int n, tiles_per_slice;
    float inv_n;
    float *gw4, *gb4;          // gradient blocks of W4 (64 x C) and b4
    int *err;
};

constexpr int kDwHCols = 128;                                // h tile columns: h3 (64) | 1 | 0 ... 0
constexpr int kDwOffH = 0;                                   // h tile, 128 rows x 128 (K-major, 32 KB)
constexpr int kDwOffDz = kDwOffH + kRows * kDwHCols * 2;     // dz tile, 128 rows x 64 (K-major, 16 KB)
constexpr int kDwOffBz = kDwOffDz + kRows * kChunkN * 2;     // W4^T chunk, 64 x 64 (K-major, 8 KB)
constexpr int kDwSmem = 64 * 1024;

// kind::f16 instruction descriptor with both operands MN-major (bits 15, 16)
__device__ __forceinline__ uint32_t idesc_mn_major(int m, int n) {
    return umma::idesc_bf16_f32(m, n) | (1u << 15) | (1u << 16);
}

__global__ void __launch_bounds__(128, 3) k_mlp_dw4(const Dw4Params p) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __shared__ uint64_t mbar_z, mbar_w;
    __shared__ uint32_t tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int chunk = blockIdx.x;
    const int t0 = blockIdx.y * p.tiles_per_slice;
    const int t1 = min((p.n + kRows - 1) / kRows, t0 + p.tiles_per_slice);
    unsigned char *ht = smem + kDwOffH, *dzt = smem + kDwOffDz, *bz = smem + kDwOffBz;
    copy_bytes(bz, reinterpret_cast<const unsigned char *>(p.pd.w4t) + (size_t)chunk * kChunkBytes, kChunkBytes);
    cp_async_commit();
    {  // this thread's row of the h tile, columns 64..127: 1 (the db4 row of the product), then zeros
        __align__(16) __nv_bfloat16 one[8];
        one[0] = __float2bfloat16_rn(1.0f);
#pragma unroll
        for (int i = 1; i < 8; ++i) one[i] = __float2bfloat16_rn(0.0f);
        *reinterpret_cast<uint4 *>(ht + umma::kmajor_offset(tid, 64, kDwHCols)) = *reinterpret_cast<const uint4 *>(one);
#pragma unroll
        for (int j = 72; j < kDwHCols; j += 8)
            *reinterpret_cast<uint4 *>(ht + umma::kmajor_offset(tid, j, kDwHCols)) = make_uint4(0, 0, 0, 0);
    }
    if (warp == 0) umma::tmem_alloc(&tmem_base, 128);
    if (tid == 0) {
        umma::mbar_init(&mbar_z, 1);
        umma::mbar_init(&mbar_w, 1);
    }
    cp_async_wait_all();
    umma::fence_proxy_async();
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = tmem_base;
    bool ok = t0 < t1, ok_warp = true;
    uint64_t *last_mbar = nullptr;
    uint32_t last_parity = 0;
    const float4 *be = reinterpret_cast<const float4 *>(p.pd.b4e + chunk * kChunkN);
    const uint32_t ht_a = umma::smem_addr(ht), dz_a = umma::smem_addr(dzt), bz_a = umma::smem_addr(bz);
    for (int t = t0; t < t1 && ok; ++t) {
        const int k = t - t0;
        if (k > 0) ok_warp = ok_warp && mma_wait(&mbar_w, (uint32_t)((k - 1) & 1));  // previous tile's operands free
        const int row = t * kRows + tid;
        const bool valid = row < p.n;
        if (valid) {
            const unsigned char *src = reinterpret_cast<const unsigned char *>(p.h3 + (size_t)row * mlp::kH);
#pragma unroll
            for (int j = 0; j < 8; ++j) cp_async16(ht + umma::kmajor_offset(tid, 8 * j, kDwHCols), src + 16 * j);
        } else {
#pragma unroll
            for (int j = 0; j < 8; ++j)
                *reinterpret_cast<uint4 *>(ht + umma::kmajor_offset(tid, 8 * j, kDwHCols)) = make_uint4(0, 0, 0, 0);
        }
        cp_async_commit();
        cp_async_wait_all();
        umma::fence_proxy_async();
        umma::fence_before_sync();
        ok = __syncthreads_and(ok_warp) != 0;
        umma::fence_after_sync();
        if (!ok) break;
        if (tid == 0) {  // z = h3 . W4[:, chunk]: A = h tile (K-major, first 64 columns), B = W4^T chunk
            const uint32_t idesc = umma::idesc_bf16_f32(kRows, kChunkN);
#pragma unroll
            for (int ks = 0; ks < mlp::kH / 16; ++ks)
                umma::mma_bf16(tmem, umma::smem_desc(ht_a + (uint32_t)ks * 256u, 128u, (kDwHCols / 8) * 128u),
                               umma::smem_desc(bz_a + (uint32_t)ks * 256u, 128u, (mlp::kH / 8) * 128u), idesc, ks > 0);
            umma::mma_commit(&mbar_z);
            last_mbar = &mbar_z;
            last_parity = (uint32_t)(k & 1);
        }
        const bool w = mma_wait(&mbar_z, (uint32_t)(k & 1));
        ok_warp = ok_warp && w;
        if (w) {
            float lse = 0.0f;
            int target = -1;
            if (valid) {
                lse = p.stat[row].x;
                target = p.target[row];
            }
            const float nl2 = -lse * kLog2e;
#pragma unroll
            for (int piece = 0; piece < kChunkN / 32; ++piece) {
                float v[32];
                umma::tmem_ld32(tmem, warp, piece * 32, v);
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const float4 b = __ldg(be + piece * 8 + q);
                    v[4 * q] += b.x; v[4 * q + 1] += b.y; v[4 * q + 2] += b.z; v[4 * q + 3] += b.w;
                }
                float d[32];
#pragma unroll
                for (int i = 0; i < 32; ++i) {
                    const int col = chunk * kChunkN + piece * 32 + i;
                    const float pr = ex2(__fmaf_rn(v[i], kLog2e, nl2));
                    d[i] = target < 0 ? 0.0f : (pr - (col == target ? 1.0f : 0.0f)) * p.inv_n;
                }
#pragma unroll
                for (int q = 0; q < 32; q += 8) put8(dzt, tid, piece * 32 + q, kChunkN, d + q);
            }
        }
        umma::fence_proxy_async();
        umma::fence_before_sync();
        ok = __syncthreads_and(ok_warp) != 0;
        umma::fence_after_sync();
        if (!ok) break;
        if (tid == 0) {
            // dW += [h3 | 1 | 0]^T dz: both tiles through MN-major descriptors,
            // K = the tile's rows in steps of 16 (two core matrices along K)
            const uint32_t idesc = idesc_mn_major(128, kChunkN);
            constexpr uint32_t lbo_h = 8 * kDwHCols * 2, lbo_dz = 8 * kChunkN * 2;  // K step: 8 rows of a tile
#pragma unroll
            for (int ks = 0; ks < kRows / 16; ++ks)
                umma::mma_bf16(tmem + 64, umma::smem_desc(ht_a + (uint32_t)ks * 2u * lbo_h, lbo_h, 128u),
                               umma::smem_desc(dz_a + (uint32_t)ks * 2u * lbo_dz, lbo_dz, 128u), idesc,
                               k > 0 || ks > 0);
            umma::mma_commit(&mbar_w);
            last_mbar = &mbar_w;
            last_parity = (uint32_t)(k & 1);
        }
    }
    if (ok && t1 > t0) ok_warp = ok_warp && mma_wait(&mbar_w, (uint32_t)((t1 - t0 - 1) & 1));
    ok = __syncthreads_and(ok && ok_warp) != 0;
    if (!ok && t1 > t0) {
        if (tid == 0) {
            atomicAdd(p.err, 1);
            if (last_mbar) umma::mbar_wait(last_mbar, last_parity, kMaxPolls);
        }
    } else if (ok && warp < 3) {
        // lanes 0..63: dW4 rows (hidden unit), lane 64: db4
        const int m = tid;
#pragma unroll
        for (int piece = 0; piece < kChunkN / 32; ++piece) {
            float v[32];
            umma::tmem_ld32(tmem + 64, warp, piece * 32, v);
            if (m <= 64) {
                float *dst = m < 64 ? p.gw4 + (size_t)m * p.pd.c + chunk * kChunkN + piece * 32
                                    : p.gb4 + chunk * kChunkN + piece * 32;
#pragma unroll
                for (int i = 0; i < 32; ++i) atomicAdd(dst + i, v[i]);
            }
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, 128);
}

// ---------------------------------------------------------------- training helpers
struct BackParams {
    const __nv_bfloat16 *w123;        // bf16 W1 | W2 | W3, row-major (row = input)
    const __nv_bfloat16 *x, *h1, *h2, *h3;
    const float *dh3;
    float *gw1, *gw2, *gw3;           // weight gradients (16 x 64, 64 x 64, 64 x 64), added
    float *gb1, *gb2, *gb3;           // bias gradients, added
    int n;
};

constexpr int kTileStride = 68;  // floats per row of the row tiles (16-byte rows, conflict-free)
// W2^T, W3^T, the da tile and the layer-input tile (128 rows each)
constexpr int kBackSmem = (2 * mlp::kH * mlp::kH + 2 * 128 * kTileStride) * 4;

// One row per thread: dh_{l-1} = W_l da_l for 16 outputs at a time, the
// weights W_l^T in shared memory (row k: W_l[0..63][k]) read as broadcast
// float4s, the products as packed FP32x2 FMAs.
__device__ __forceinline__ void back_matvec(const float *wt, const float (&da)[mlp::kH], int i0, float (&o)[16]) {
    float2 acc[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[j] = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int k = 0; k < mlp::kH; ++k) {
        const float2 d = make_float2(da[k], da[k]);
        const float4 *w = reinterpret_cast<const float4 *>(wt + k * mlp::kH + i0);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float4 w4 = w[j];
            acc[2 * j] = __ffma2_rn(make_float2(w4.x, w4.y), d, acc[2 * j]);
            acc[2 * j + 1] = __ffma2_rn(make_float2(w4.z, w4.w), d, acc[2 * j + 1]);
        }
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        o[2 * j] = acc[j].x;
        o[2 * j + 1] = acc[j].y;
    }
}

template <int W>
__device__ __forceinline__ void load_bf16_row(const __nv_bfloat16 *src, float (&v)[W]) {
    const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
#pragma unroll
    for (int j = 0; j < W / 8; ++j) {
        const uint4 w = s4[j];
        const __nv_bfloat162 *b = reinterpret_cast<const __nv_bfloat162 *>(&w);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const float2 f = __bfloat1622float2(b[i]);
            v[8 * j + 2 * i] = f.x;
            v[8 * j + 2 * i + 1] = f.y;
        }
    }
}

// gW[i][k0 .. k0 + 2*NP) += sum over the tile's rows of in[r][i] * da[r][k]
template <int NP>
__device__ __forceinline__ void tile_outer(const float *in_t, const float *da_t, int i, int k0, float *gw) {
    float2 acc[NP];
#pragma unroll
    for (int j = 0; j < NP; ++j) acc[j] = make_float2(0.0f, 0.0f);
#pragma unroll 4
    for (int r = 0; r < 128; ++r) {
        const float a = in_t[r * kTileStride + i];
        const float2 a2 = make_float2(a, a);
        const float4 *d = reinterpret_cast<const float4 *>(da_t + r * kTileStride + k0);
#pragma unroll
        for (int j = 0; j < NP / 2; ++j) {
            const float4 d4 = d[j];
            acc[2 * j] = __ffma2_rn(a2, make_float2(d4.x, d4.y), acc[2 * j]);
            acc[2 * j + 1] = __ffma2_rn(a2, make_float2(d4.z, d4.w), acc[2 * j + 1]);
        }
    }
#pragma unroll
    for (int j = 0; j < NP; ++j) {
        atomicAdd(gw + i * mlp::kH + k0 + 2 * j, acc[j].x);
        atomicAdd(gw + i * mlp::kH + k0 + 2 * j + 1, acc[j].y);
    }
}

// The hidden layers' backward pass for 128 rows per block, one row per
// thread: da3 = dh3 relu'(h3); for l = 3, 2, 1: db_l += column sums of da_l,
// dW_l += in_l^T da_l (in_3 = h2, in_2 = h1, in_1 = x; from tiles of the
// block's rows in shared memory), and da_{l-1} = (W_l da_l) relu'(h_{l-1}),
// FP32 with the bf16 weights of the forward pass.  The weight and bias
// gradients are added to the output with atomics, once per block.
__global__ void __launch_bounds__(128, 2) k_mlp_backward_rows(const BackParams p) {
    extern __shared__ __align__(16) float bsm[];
    float *wt2 = bsm, *wt3 = bsm + mlp::kH * mlp::kH;
    float *dt = bsm + 2 * mlp::kH * mlp::kH, *it = dt + 128 * kTileStride;  // da tile, layer-input tile
    for (int e = threadIdx.x; e < 2 * mlp::kH * mlp::kH; e += blockDim.x) {
        const int layer = e / (mlp::kH * mlp::kH), f = e % (mlp::kH * mlp::kH);
        const int i = f / mlp::kH, k = f % mlp::kH;  // W[i][k]
        (layer ? wt3 : wt2)[k * mlp::kH + i] = __bfloat162float(p.w123[mlp::kIn * mlp::kH + e]);
    }
    const int t = threadIdx.x;
    const int r = blockIdx.x * blockDim.x + t;
    const bool valid = r < p.n;
    const size_t ro = (size_t)(valid ? r : 0) * mlp::kH;
    float da[mlp::kH];
    if (valid) {
        float h[mlp::kH];
        load_bf16_row(p.h3 + ro, h);
        const float4 *g = reinterpret_cast<const float4 *>(p.dh3 + ro);
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const float4 v = g[j];
            da[4 * j] = h[4 * j] > 0.0f ? v.x : 0.0f;
            da[4 * j + 1] = h[4 * j + 1] > 0.0f ? v.y : 0.0f;
            da[4 * j + 2] = h[4 * j + 2] > 0.0f ? v.z : 0.0f;
            da[4 * j + 3] = h[4 * j + 3] > 0.0f ? v.w : 0.0f;
        }
    } else {
#pragma unroll
        for (int j = 0; j < mlp::kH; ++j) da[j] = 0.0f;
    }
#pragma unroll 1
    for (int layer = 3; layer >= 1; --layer) {
        float hin[mlp::kH];  // this layer's input row (x uses the first 16)
        if (layer > 1) {
            if (valid) load_bf16_row(layer == 3 ? p.h2 + ro : p.h1 + ro, hin);
            else
#pragma unroll
                for (int j = 0; j < mlp::kH; ++j) hin[j] = 0.0f;
        } else {
            float x[mlp::kIn];
            if (valid) load_bf16_row(p.x + (size_t)r * mlp::kIn, x);
            else
#pragma unroll
                for (int j = 0; j < mlp::kIn; ++j) x[j] = 0.0f;
#pragma unroll
            for (int j = 0; j < mlp::kH; ++j) hin[j] = j < mlp::kIn ? x[j] : 0.0f;
        }
        __syncthreads();  // the previous layer's tiles are no longer read (first pass: the weights are in)
        float4 *drow = reinterpret_cast<float4 *>(dt + t * kTileStride);
        float4 *irow = reinterpret_cast<float4 *>(it + t * kTileStride);
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            drow[j] = make_float4(da[4 * j], da[4 * j + 1], da[4 * j + 2], da[4 * j + 3]);
            irow[j] = make_float4(hin[4 * j], hin[4 * j + 1], hin[4 * j + 2], hin[4 * j + 3]);
        }
        __syncthreads();
        {  // db_l: thread t sums half the rows of column t % 64
            const int col = t & 63, half = t >> 6;
            float sum = 0.0f;
#pragma unroll 8
            for (int q = 0; q < 64; ++q) sum += dt[(half * 64 + q) * kTileStride + col];
            atomicAdd((layer == 3 ? p.gb3 : layer == 2 ? p.gb2 : p.gb1) + col, sum);
        }
        if (layer > 1) {
            tile_outer<16>(it, dt, t >> 1, (t & 1) * 32, layer == 3 ? p.gw3 : p.gw2);
            float nx[mlp::kH];
            const float *wt = layer == 3 ? wt3 : wt2;
            const float *own = it + t * kTileStride;  // this row's input: the ReLU mask
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                float o[16];
                back_matvec(wt, da, 16 * c, o);
#pragma unroll
                for (int j = 0; j < 16; ++j) nx[16 * c + j] = own[16 * c + j] > 0.0f ? o[j] : 0.0f;
            }
#pragma unroll
            for (int j = 0; j < mlp::kH; ++j) da[j] = nx[j];
        } else {
            tile_outer<4>(it, dt, t >> 3, (t & 7) * 8, p.gw1);
        }
    }
}

__global__ void k_adam(float *w, const float *g, float *m, float *v, size_t n, float lr, float b1, float b2,
                       float eps, float c1, float c2, size_t w1_pad_begin, size_t w1_pad_end) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || (i >= w1_pad_begin && i < w1_pad_end)) return;  // padded inputs stay zero
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * (gi * gi);
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// bf16 images of the weights: W1^T | W2^T | W3^T in the MMA operand layout
// (w123img), W4^T in chunk tiles (w4t: cluster x hidden, K-major over
// hidden), W4 in chunk tiles (w4k: hidden x cluster, K-major over clusters),
// W1 | W2 | W3 row-major (w123), W4 row-major (w4), and b4 with -inf for
// clusters without lights.
__global__ void k_refresh(const float *params, int c, const uint8_t *valid, __nv_bfloat16 *w123img,
                          __nv_bfloat16 *w4t, __nv_bfloat16 *w4k, __nv_bfloat16 *w123, __nv_bfloat16 *w4,
                          float *b4e) {
    const mlp::Layout L(c);
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t n1 = (size_t)mlp::kIn * mlp::kH, n2 = (size_t)mlp::kH * mlp::kH;
    unsigned char *img = reinterpret_cast<unsigned char *>(w123img);
    if (i < n1) {  // W1[k][n]
        const int k = (int)(i / mlp::kH), nn = (int)(i % mlp::kH);
        const __nv_bfloat16 b = __float2bfloat16_rn(params[L.w1 + i]);
        w123[i] = b;
        *reinterpret_cast<__nv_bfloat16 *>(img + umma::kmajor_offset(nn, k, mlp::kIn)) = b;
    } else if (i < n1 + 2 * n2) {
        const size_t j = i - n1;
        const int layer = (int)(j / n2);
        const size_t e = j % n2;
        const int k = (int)(e / mlp::kH), nn = (int)(e % mlp::kH);
        const __nv_bfloat16 b = __float2bfloat16_rn(params[(layer == 0 ? L.w2 : L.w3) + e]);
        w123[i] = b;
        *reinterpret_cast<__nv_bfloat16 *>(img + n1 * 2 + (size_t)layer * n2 * 2 +
                                           umma::kmajor_offset(nn, k, mlp::kH)) = b;
    } else if (i < n1 + 2 * n2 + (size_t)mlp::kH * c) {
        const size_t e = i - n1 - 2 * n2;  // W4[k][cl]
        const int k = (int)(e / (size_t)c), cl = (int)(e % (size_t)c);
        const __nv_bfloat16 b = __float2bfloat16_rn(params[L.w4 + e]);
        w4[e] = b;
        unsigned char *tile = reinterpret_cast<unsigned char *>(w4t) + (size_t)(cl / kChunkN) * kChunkBytes;
        *reinterpret_cast<__nv_bfloat16 *>(tile + umma::kmajor_offset(cl % kChunkN, k, mlp::kH)) = b;
        unsigned char *ktile = reinterpret_cast<unsigned char *>(w4k) + (size_t)(cl / kChunkN) * kWkBytes;
        *reinterpret_cast<__nv_bfloat16 *>(ktile + umma::kmajor_offset(k, cl % kChunkN, kChunkN)) = b;
    } else if (i < n1 + 2 * n2 + (size_t)(mlp::kH + 1) * c) {
        const size_t cl = i - n1 - 2 * n2 - (size_t)mlp::kH * c;
        b4e[cl] = valid[cl] ? params[L.b4 + cl] : -INFINITY;
    }
}

// Training target of each row: the cluster of its final reservoir's light,
// or -1 (no light kept).
__global__ void k_targets(const rg_reservoir *res, const int32_t *rows, int n, const int32_t *cluster_of,
                          int n_lights, int32_t *target, int *count) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const float4 c = __ldg(reinterpret_cast<const float4 *>(res + rows[r]) + 2);
    const int idx = __float_as_int(c.x);
    int t = -1;
    if (c.w > 0.0f && idx >= 0 && idx < n_lights) t = cluster_of[idx];
    target[r] = t;
    if (t >= 0) atomicAdd(count, 1);
}

// Training rows of one frame: a strided sweep over the pixels.
__global__ void k_batch_rows(int32_t *rows, int n, uint32_t pixels, uint32_t offset, uint32_t stride) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    rows[r] = (int32_t)(((uint64_t)r * stride + offset) % pixels);
}

template <int kMode>
constexpr int fused_smem() {
    return (kMode == kGrad ? kSmemGrad : kSmemUsed) < kSmemMin ? kSmemMin : (kMode == kGrad ? kSmemGrad : kSmemUsed);
}

// set_attr: set the shared-memory attribute first (the batched launches set it
// once, before any stream capture, in prepare_views)
template <int kMode, bool kViews = false>
cudaError_t launch_fused(const FusedParams &p, cudaStream_t st, bool set_attr = true) {
    if (p.pd.c % kChunkN != 0 || p.pd.c < kChunkN) return cudaErrorInvalidValue;
    constexpr int smem = fused_smem<kMode>();
    if (set_attr) {
        cudaError_t e =
            cudaFuncSetAttribute(k_mlp_fused<kMode, kViews>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
    }
    if (p.n > 0) k_mlp_fused<kMode, kViews><<<(p.n + kRows - 1) / kRows, kRows, smem, st>>>(p);
    return cudaGetLastError();
}

}  // namespace

// ---------------------------------------------------------------- launchers (mlp.cuh)
namespace mlp {

size_t weight_image_bytes() { return (size_t)kWeightImgBytes; }

cudaError_t forward_lse(const ProposalDev &pd, const GBufView &g, const float cam[3], const int32_t *rows, int n,
                        float4 *stat, const TrainBuffers *save, uint32_t frame, int n_cand, Candidate *cand, int *err,
                        cudaStream_t st) {
    if (cand && (n_cand < 1 || n_cand > kCand)) return cudaErrorInvalidValue;
    FusedParams p{};
    p.pd = pd; p.g = g; p.cam[0] = cam[0]; p.cam[1] = cam[1]; p.cam[2] = cam[2];
    p.rows = rows; p.n = n; p.stat = stat; p.err = err;
    p.frame = frame; p.n_cand = n_cand; p.cand = cand;
    if (save) { p.save = 1; p.x = save->x; p.h1 = save->h1; p.h2 = save->h2; p.h3 = save->h3; }
    return launch_fused<kLse>(p, st);
}

cudaError_t forward_sample(const ProposalDev &pd, const GBufView &g, const float cam[3], int n, const float4 *stat,
                           uint32_t frame, int n_cand, Candidate *cand, int *err, cudaStream_t st) {
    if (n_cand < 1 || n_cand > kCand) return cudaErrorInvalidValue;
    FusedParams p{};
    p.pd = pd; p.g = g; p.cam[0] = cam[0]; p.cam[1] = cam[1]; p.cam[2] = cam[2];
    p.n = n; p.stat = const_cast<float4 *>(stat); p.frame = frame; p.n_cand = n_cand; p.cand = cand; p.err = err;
    return launch_fused<kSample>(p, st);
}

cudaError_t prepare_views() {
    cudaError_t e = cudaFuncSetAttribute(k_mlp_fused<kLse, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         fused_smem<kLse>());
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_mlp_fused<kSample, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 fused_smem<kSample>());
    return e;
}

cudaError_t forward_lse_views(const ProposalDev &pd, const ViewRows *views, int n_views, const uint32_t *frames,
                              int total, float4 *stat, Candidate *cand, int *err, cudaStream_t st) {
    if (!views || n_views < 1 || !frames || !cand) return cudaErrorInvalidValue;
    FusedParams p{};
    p.pd = pd; p.n = total; p.stat = stat; p.err = err; p.cand = cand;
    p.views = views; p.n_views = n_views; p.frames = frames;
    return launch_fused<kLse, true>(p, st, false);
}

cudaError_t forward_sample_views(const ProposalDev &pd, const ViewRows *views, int n_views, const uint32_t *frames,
                                 int total, const float4 *stat, Candidate *cand, int *err, cudaStream_t st) {
    if (!views || n_views < 1 || !frames || !cand) return cudaErrorInvalidValue;
    FusedParams p{};
    p.pd = pd; p.n = total; p.stat = const_cast<float4 *>(stat); p.err = err; p.cand = cand;
    p.views = views; p.n_views = n_views; p.frames = frames;
    return launch_fused<kSample, true>(p, st, false);
}

cudaError_t forward_grad(const ProposalDev &pd, const GBufView &g, const float cam[3], const int32_t *rows, int n,
                         const float4 *stat, const int32_t *target, float inv_n, float *dh3, float *loss_sum,
                         int *err, cudaStream_t st) {
    FusedParams p{};
    p.pd = pd; p.g = g; p.cam[0] = cam[0]; p.cam[1] = cam[1]; p.cam[2] = cam[2];
    p.rows = rows; p.n = n; p.stat = const_cast<float4 *>(stat); p.target = target; p.inv_n = inv_n; p.dh3 = dh3;
    p.loss_sum = loss_sum; p.err = err;
    return launch_fused<kGrad>(p, st);
}

cudaError_t dw4(const ProposalDev &pd, const __nv_bfloat16 *h3, const float4 *stat, const int32_t *target, int n,
                float inv_n, float *gw4, float *gb4, int *err, cudaStream_t st) {
    if (pd.c % kChunkN != 0 || n <= 0) return cudaErrorInvalidValue;
    Dw4Params p{pd, h3, stat, target, n, 0, inv_n, gw4, gb4, err};
    const int tiles = (n + kRows - 1) / kRows;
    const int chunks = pd.c / kChunkN;
    // about RG_DW4_SLICE_CTAS CTAs per SM in all; each keeps its tiles' sum in tensor memory
    int slices = (RG_DW4_SLICE_CTAS * 152 + chunks - 1) / chunks;
    if (slices > tiles) slices = tiles;
    p.tiles_per_slice = (tiles + slices - 1) / slices;
    slices = (tiles + p.tiles_per_slice - 1) / p.tiles_per_slice;
    cudaError_t e = cudaFuncSetAttribute(k_mlp_dw4, cudaFuncAttributeMaxDynamicSharedMemorySize, kDwSmem);
    if (e != cudaSuccess) return e;
    k_mlp_dw4<<<dim3(chunks, slices), 128, kDwSmem, st>>>(p);
    return cudaGetLastError();
}

cudaError_t backward_rows(const __nv_bfloat16 *w123, const TrainBuffers &t, const float *dh3, float *gw1, float *gw2,
                          float *gw3, float *gb1, float *gb2, float *gb3, int n, cudaStream_t st) {
    BackParams p{w123, t.x, t.h1, t.h2, t.h3, dh3, gw1, gw2, gw3, gb1, gb2, gb3, n};
    cudaError_t e = cudaFuncSetAttribute(k_mlp_backward_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, kBackSmem);
    if (e != cudaSuccess) return e;
    if (n > 0) k_mlp_backward_rows<<<(n + 127) / 128, 128, kBackSmem, st>>>(p);
    return cudaGetLastError();
}

cudaError_t adam(float *w, const float *g, float *m, float *v, size_t n, float lr, int step, int c, cudaStream_t st) {
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
    const Layout L(c);
    k_adam<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(w, g, m, v, n, lr, b1, b2, 1e-8f, c1, c2,
                                                         L.w1 + (size_t)kInUsed * kH, L.w1 + (size_t)kIn * kH);
    return cudaGetLastError();
}

cudaError_t refresh(const float *params, int c, const uint8_t *valid, __nv_bfloat16 *w123img, __nv_bfloat16 *w4t,
                    __nv_bfloat16 *w4k, __nv_bfloat16 *w123, __nv_bfloat16 *w4, float *b4e, cudaStream_t st) {
    const size_t n = (size_t)kIn * kH + 2 * (size_t)kH * kH + (size_t)(kH + 1) * c;
    k_refresh<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(params, c, valid, w123img, w4t, w4k, w123, w4, b4e);
    return cudaGetLastError();
}

cudaError_t targets(const rg_reservoir *res, const int32_t *rows, int n, const int32_t *cluster_of, int n_lights,
                    int32_t *target, int *count, cudaStream_t st) {
    if (n > 0) k_targets<<<(n + 127) / 128, 128, 0, st>>>(res, rows, n, cluster_of, n_lights, target, count);
    return cudaGetLastError();
}

cudaError_t batch_rows(int32_t *rows, int n, uint32_t pixels, uint32_t offset, uint32_t stride, cudaStream_t st) {
    if (n > 0) k_batch_rows<<<(n + 127) / 128, 128, 0, st>>>(rows, n, pixels, offset, stride);
    return cudaGetLastError();
}

}  // namespace mlp
