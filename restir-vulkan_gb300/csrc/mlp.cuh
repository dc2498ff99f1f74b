// mlp.cuh -- the learned light-cluster proposal: network definition shared
// by its kernels (mlp.cu) and the context (capi.cu).
//
// Per pixel, features x (16 values, 9 used): the world position mapped to
// [-1, 1]^3 over the scene bounds, the G-buffer normal, and the unit vector
// to the camera, each rounded to bf16.  Network:
//   h1 = bf16(relu(W1^T x  + b1))    W1: 16 x 64 (rows 9..15 stay zero)
//   h2 = bf16(relu(W2^T h1 + b2))    W2: 64 x 64
//   h3 = bf16(relu(W3^T h2 + b3))    W3: 64 x 64
//   z  = W4^T h3 + b4                W4: 64 x C, C = number of light clusters
// with bf16 weights (rounded from FP32 master copies), FP32 accumulation and
// FP32 biases; clusters without lights get z = -inf.  q(c|x) = softmax(z)_c.
//
// Proposal for RIS candidates: with probability `mix` the cluster c ~ q(.|x)
// and a light l ~ p(l|c) (the cluster's lights by luminance), otherwise l is
// uniform over all N lights; every candidate's source pdf is the mixture
// density  p(l) = mix * q(c(l)|x) * p(l|c(l)) + (1 - mix) / N,  so RIS stays
// unbiased wherever the uniform term is positive.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "rg_internal.h"

namespace mlp {

constexpr int kIn = 16;
constexpr int kInUsed = 9;
constexpr int kH = 64;
constexpr int kCand = 32;  // candidate slots per pixel in the learned candidate buffer
constexpr int kChunkN = 64;   // clusters per logit MMA chunk (clusters must be a multiple)
// PCG stream of the proposal's draws for pixel px in frame f:
// pcg_seed(f * kSeedMul + kSeedAdd, px), distinct from the RIS stream.
constexpr uint64_t kSeedMul = 0x9E3779B97F4A7C15ULL;
constexpr uint64_t kSeedAdd = 0x2545F4914F6CDD1DULL;

// Offsets (floats) of the parameters in the packed FP32 vector.
struct Layout {
    int c;  // clusters
    size_t w1, b1, w2, b2, w3, b3, w4, b4, total;
    __host__ __device__ explicit Layout(int clusters) : c(clusters) {
        size_t o = 0;
        w1 = o; o += (size_t)kIn * kH;
        b1 = o; o += kH;
        w2 = o; o += (size_t)kH * kH;
        b2 = o; o += kH;
        w3 = o; o += (size_t)kH * kH;
        b3 = o; o += kH;
        w4 = o; o += (size_t)kH * c;
        b4 = o; o += (size_t)c;
        total = o;
    }
};

// One candidate of the learned proposal for a pixel: key >= 0 is a light
// drawn uniformly, key < 0 is the cluster -1-key drawn from q; q is
// q(cluster|x) of the candidate's cluster.
struct Candidate {
    int32_t key;
    float q;
};

// One column of a cluster's alias table, in grouped-light order, with both
// lights' positions so that a learned-branch candidate is one gather.
struct LearnedCol {
    float4 col;        // prob, own light (int bits), alias light (int bits), p(own | cluster)
    float4 own_pos;    // own light position, luminance
    float4 alias_pos;  // alias light position, luminance
};

struct ProposalDev {
    int c;                          // clusters
    int n_lights;
    float mix;                      // probability of the learned branch
    float3 box_center, box_inv_half;
    const float *params;            // FP32 master (packed, Layout)
    const float *b4e;               // b4, or -inf for clusters without lights
    const __nv_bfloat16 *w123img;   // bf16 W1^T | W2^T | W3^T in the MMA operand layout
    const __nv_bfloat16 *w4t;       // bf16 W4^T in chunk tiles (cluster x hidden), MMA operand layout
    const __nv_bfloat16 *w4k;       // bf16 W4 in chunk tiles (hidden x cluster), MMA operand layout
    const __nv_bfloat16 *w123;      // bf16 W1 | W2 | W3 row-major (row = input)
    const __nv_bfloat16 *w4;        // bf16 W4, 64 x C row-major
    const uint8_t *cluster_valid;   // 1 if the cluster has lights
    const int32_t *cluster_of;      // per light
};

// What the RIS kernel needs to draw and weigh learned candidates.
struct LearnedRis {
    const Candidate *cand;          // [pixels x kCand]; nullptr: plain proposal
    const int32_t *offset;          // C + 1 grouped positions
    const LearnedCol *lcol;         // per grouped position
    const float *within;            // p(light | its cluster), per light
    float mix;
    float uniform_pdf;              // (1 - mix) / N
};

// Activations of the training rows, saved by the forward pass (bf16 values).
struct TrainBuffers {
    __nv_bfloat16 *x, *h1, *h2, *h3;
};

// One view of a batched inference.  The views' pixels are concatenated into
// one row space: view v owns rows first_row .. first_row + w*h - 1 (ascending
// first_row), row first_row + px being its pixel px.
struct ViewRows {
    GBufView g;
    float cam[3];
    uint32_t first_row;
    int32_t n_cand;            // candidates per pixel (1..kCand)
};

size_t weight_image_bytes();
// cand != nullptr (inference): also writes the uniform-branch candidates of frame `frame`
cudaError_t forward_lse(const ProposalDev &pd, const GBufView &g, const float cam[3], const int32_t *rows, int n,
                        float4 *stat, const TrainBuffers *save, uint32_t frame, int n_cand, Candidate *cand, int *err,
                        cudaStream_t st);
cudaError_t forward_sample(const ProposalDev &pd, const GBufView &g, const float cam[3], int n, const float4 *stat,
                           uint32_t frame, int n_cand, Candidate *cand, int *err, cudaStream_t st);
// Both inference passes over all rows of a batch of views in one launch each;
// frames[v] is view v's frame index (device memory, read at run time).  The
// kernels' attributes are set by prepare_views, outside any stream capture.
cudaError_t prepare_views();
cudaError_t forward_lse_views(const ProposalDev &pd, const ViewRows *views, int n_views, const uint32_t *frames,
                              int total, float4 *stat, Candidate *cand, int *err, cudaStream_t st);
cudaError_t forward_sample_views(const ProposalDev &pd, const ViewRows *views, int n_views, const uint32_t *frames,
                                 int total, const float4 *stat, Candidate *cand, int *err, cudaStream_t st);
cudaError_t forward_grad(const ProposalDev &pd, const GBufView &g, const float cam[3], const int32_t *rows, int n,
                         const float4 *stat, const int32_t *target, float inv_n, float *dh3, float *loss_sum,
                         int *err, cudaStream_t st);
// Adds dW4 (64 x C) and db4 of the mean loss to gw4 / gb4.
cudaError_t dw4(const ProposalDev &pd, const __nv_bfloat16 *h3, const float4 *stat, const int32_t *target, int n,
                float inv_n, float *gw4, float *gb4, int *err, cudaStream_t st);
// The hidden layers' weight and bias gradients from dh3, added to gw1..gw3
// (row-major, row = input) and gb1..gb3.
cudaError_t backward_rows(const __nv_bfloat16 *w123, const TrainBuffers &t, const float *dh3, float *gw1, float *gw2,
                          float *gw3, float *gb1, float *gb2, float *gb3, int n, cudaStream_t st);
cudaError_t adam(float *w, const float *g, float *m, float *v, size_t n, float lr, int step, int c, cudaStream_t st);
cudaError_t refresh(const float *params, int c, const uint8_t *valid, __nv_bfloat16 *w123img, __nv_bfloat16 *w4t,
                    __nv_bfloat16 *w4k, __nv_bfloat16 *w123, __nv_bfloat16 *w4, float *b4e, cudaStream_t st);
cudaError_t targets(const rg_reservoir *res, const int32_t *rows, int n, const int32_t *cluster_of, int n_lights,
                    int32_t *target, int *count, cudaStream_t st);
cudaError_t batch_rows(int32_t *rows, int n, uint32_t pixels, uint32_t offset, uint32_t stride, cudaStream_t st);

}  // namespace mlp
