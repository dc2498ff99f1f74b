// gemm_tc.cu -- D[M x N] (+)= A[M x K] . B[N x K]^T on the tcgen05 tensor
// cores, BF16 operands and FP32 accumulation in tensor memory.
//
// Operands are read from global memory through (row, k) element strides, so
// a transposed source is just another stride pair, and may be BF16 or FP32
// (rounded to BF16 on the way into shared memory).  One 128-thread CTA owns a
// 128 x NT tile of D; K advances in chunks of 64: the threads stage the A and
// B chunk in shared memory in the canonical K-major layout, one thread issues
// the four K=16 MMAs, and completion is signalled through an mbarrier whose
// wait is bounded.  Split-K over gridDim.z with an atomic epilogue.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "rg_internal.h"
#include "umma.cuh"

namespace {

constexpr int kTileM = 128;
constexpr int kChunkK = 64;
constexpr uint32_t kMaxPolls = 1u << 24;  // bounded mbarrier wait

struct Operand {
    const void *ptr;
    int64_t rs, ks;  // element strides of (row, k)
    int rows;
    int fp32;        // 1: float source, 0: bf16 source
};

struct GemmParams {
    Operand a, b;
    int k;
    int k_per_split;
    float *d;
    int64_t ldd;
    int accumulate;  // 1: atomicAdd into d, 0: store
    float alpha;
    int *err;
};

__device__ __forceinline__ __nv_bfloat16 fetch(const Operand &o, int r, int k, int kmax) {
    if (r >= o.rows || k >= kmax) return __float2bfloat16_rn(0.0f);
    const int64_t idx = (int64_t)r * o.rs + (int64_t)k * o.ks;
    if (o.fp32) return __float2bfloat16_rn(static_cast<const float *>(o.ptr)[idx]);
    return static_cast<const __nv_bfloat16 *>(o.ptr)[idx];
}

// Stages rows [row0, row0 + R) x k [kc, kc + 64) of an operand into a
// K-major tile.  Consecutive threads walk k when k is the contiguous index of
// the source, rows otherwise, so that global reads coalesce either way.
__device__ __forceinline__ void stage(const Operand &o, unsigned char *tile, int R, int row0, int kc, int kmax) {
    if (o.rs == 1 && o.ks != 1) {
        for (int e = threadIdx.x; e < R * kChunkK; e += blockDim.x) {
            const int k = e / R, r = e % R;
            *reinterpret_cast<__nv_bfloat16 *>(tile + umma::kmajor_offset(r, k, kChunkK)) =
                fetch(o, row0 + r, kc + k, kmax);
        }
    } else {
        for (int e = threadIdx.x; e < R * kChunkK; e += blockDim.x) {
            const int r = e / kChunkK, k = e % kChunkK;
            *reinterpret_cast<__nv_bfloat16 *>(tile + umma::kmajor_offset(r, k, kChunkK)) =
                fetch(o, row0 + r, kc + k, kmax);
        }
    }
}

template <int NT>
__global__ void __launch_bounds__(128) k_gemm_tc(const GemmParams p) {
    extern __shared__ __align__(1024) unsigned char smem[];
    __nv_bfloat16 *a_tile = reinterpret_cast<__nv_bfloat16 *>(smem);
    __nv_bfloat16 *b_tile = reinterpret_cast<__nv_bfloat16 *>(smem + kTileM * kChunkK * 2);
    __shared__ uint64_t mbar;
    __shared__ uint32_t tmem_base;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * kTileM, n0 = blockIdx.y * NT;
    const int k_begin = blockIdx.z * p.k_per_split;
    const int k_end = min(p.k, k_begin + p.k_per_split);
    if (warp == 0) umma::tmem_alloc(&tmem_base, NT < 32 ? 32 : NT);
    if (tid == 0) umma::mbar_init(&mbar, 1);
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tmem = tmem_base;
    uint32_t phase = 0;
    bool ok = true;
    bool any = false;
    for (int kc = k_begin; kc < k_end; kc += kChunkK) {
        stage(p.a, reinterpret_cast<unsigned char *>(a_tile), kTileM, m0, kc, k_end);
        stage(p.b, reinterpret_cast<unsigned char *>(b_tile), NT, n0, kc, k_end);
        umma::fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            umma::fence_after_sync();
            umma::mma_chunk(tmem, a_tile, b_tile, kChunkK, kTileM, NT, any);
            umma::mma_commit(&mbar);
        }
        any = true;
        const bool w = umma::mbar_wait(&mbar, phase, kMaxPolls);
        umma::fence_after_sync();
        // block-uniform, so that every thread leaves the loop at the same barrier
        ok = __syncthreads_and(w) != 0;
        if (!ok) {
            if (tid == 0) umma::mbar_wait(&mbar, phase, kMaxPolls);  // bounded: the MMA still in flight
            break;
        }
        phase ^= 1u;
    }
    if (!ok && tid == 0) atomicAdd(p.err, 1);
    if (any && ok) {
        const int row = m0 + warp * 32 + lane;
        for (int c = 0; c < NT; c += 32) {
            float v[32];
            umma::tmem_ld32(tmem, warp, c, v);
            if (row < p.a.rows) {
                float *drow = p.d + (int64_t)row * p.ldd;
#pragma unroll
                for (int i = 0; i < 32; ++i) {
                    const int col = n0 + c + i;
                    if (col < p.b.rows) {
                        if (p.accumulate) atomicAdd(drow + col, p.alpha * v[i]);
                        else drow[col] = p.alpha * v[i];
                    }
                }
            }
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, NT < 32 ? 32 : NT);
}

}  // namespace

// D = alpha * A . B^T (accumulate: D += ...).  A: M x K, B: N x K, given by
// element strides; D row-major with leading dimension ldd.
cudaError_t launch_gemm_tc(const void *a, int a_fp32, int64_t a_rs, int64_t a_ks, int m, const void *b, int b_fp32,
                           int64_t b_rs, int64_t b_ks, int n, int k, float *d, int64_t ldd, int accumulate,
                           float alpha, int splits, int *err, cudaStream_t st) {
    GemmParams p;
    p.a = Operand{a, a_rs, a_ks, m, a_fp32};
    p.b = Operand{b, b_rs, b_ks, n, b_fp32};
    p.k = k;
    if (splits < 1) splits = 1;
    const int chunks = (k + kChunkK - 1) / kChunkK;
    const int per = (chunks + splits - 1) / splits;
    p.k_per_split = per * kChunkK;
    splits = (chunks + per - 1) / per;
    if (splits > 1) accumulate = 1;
    p.d = d;
    p.ldd = ldd;
    p.accumulate = accumulate;
    p.alpha = alpha;
    p.err = err;
    if (n <= 64) {
        const size_t smem = (size_t)(kTileM + 64) * kChunkK * 2;
        cudaError_t e = cudaFuncSetAttribute(k_gemm_tc<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k_gemm_tc<64><<<dim3((m + kTileM - 1) / kTileM, (n + 63) / 64, splits), 128, smem, st>>>(p);
    } else {
        const size_t smem = (size_t)(kTileM + 256) * kChunkK * 2;
        cudaError_t e = cudaFuncSetAttribute(k_gemm_tc<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k_gemm_tc<256><<<dim3((m + kTileM - 1) / kTileM, (n + 255) / 256, splits), 128, smem, st>>>(p);
    }
    return cudaGetLastError();
}
