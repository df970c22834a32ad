// aco_mlp.h -- shapes and launchers of the edge-scoring MLP (k_mlp.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "aco_device.cuh"

namespace aco {

constexpr int kFeatures = 12;  // per candidate edge, see k_edge_features
constexpr int kFeatPad = 16;   // K of the first GEMM (a multiple of 16)
constexpr int kHidden = 128;   // width of both hidden layers
// Packed parameter vector: W1[128][12] b1[128] W2[128][128] b2[128] w3[128] b3[1]
constexpr int kParamW1 = 0;
constexpr int kParamB1 = kParamW1 + kHidden * kFeatures;
constexpr int kParamW2 = kParamB1 + kHidden;
constexpr int kParamB2 = kParamW2 + kHidden * kHidden;
constexpr int kParamW3 = kParamB2 + kHidden;
constexpr int kParamB3 = kParamW3 + kHidden;
constexpr int kParamCount = kParamB3 + 1;

enum { kGemmStore = 0, kGemmAccumulate = 1, kGemmAtomic = 2 };

cudaError_t launch_edge_features(const ColonyDev &c, const float *x, const float *y,
                                 float *mean_dk_dev, __nv_bfloat16 *feats, float *labels,
                                 cudaStream_t s);
cudaError_t launch_gemm_tn(const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *B, int ldb,
                           float *C, int ldc, int M, int N, int K, int mode, int splits,
                           cudaStream_t s);
// The same product on the 5th-generation tensor cores (tcgen05 + TMA);
// N must be 128 or 16, A and B 16-byte aligned.  err: device word for
// timeout flags (may be null).
cudaError_t launch_gemm_tn_tc(const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *B, int ldb,
                              float *C, int ldc, int M, int N, int K, int mode, int splits,
                              uint32_t *err, cudaStream_t s);
cudaError_t launch_bias_relu(const float *Z, const float *bias, int E, int Hd,
                             __nv_bfloat16 *Hout, __nv_bfloat16 *Ht, int ldt, cudaStream_t s);
cudaError_t launch_head(const __nv_bfloat16 *H2, const float *w3, const float *b3, int E,
                        const float *labels, float pos_weight, float norm, float *out,
                        float *dlogit, float *gw3, float *gb3, float *loss, cudaStream_t s);
cudaError_t launch_grad_hidden2(const float *dlogit, const float *w3, const __nv_bfloat16 *H2,
                                int E, __nv_bfloat16 *dZ, __nv_bfloat16 *dZt, int ldt, float *gb,
                                cudaStream_t s);
cudaError_t launch_grad_hidden1(const float *dH1, const __nv_bfloat16 *H1, int E,
                                __nv_bfloat16 *dZt, int ldt, float *gb, cudaStream_t s);
cudaError_t launch_transpose_feats(const __nv_bfloat16 *X, int E, __nv_bfloat16 *Xt, int ldt,
                                   cudaStream_t s);
// The whole forward (and, with train, loss and backward) pass over `rows`
// edges in one tcgen05 kernel (k_mlp_fused.cu); grid = mlp_fused_grid().
// Training writes one partial row per CTA into part (ld >= kParamCount + 1,
// a multiple of 4): the gradient in packed order, then the loss.
int mlp_fused_grid(int rows, int sms);
cudaError_t launch_mlp_fused(bool train, const __nv_bfloat16 *X, int rows,
                             const __nv_bfloat16 *w1b, const __nv_bfloat16 *w2b, const float *w,
                             const float *labels, float pos_weight, float norm, float *out,
                             float *part, int part_ld, int grid, uint32_t *err, cudaStream_t s);
// Sums G partial rows in order into gout / loss_out and, with adam, applies
// the Adam step and refreshes the BF16 weight copies.
cudaError_t launch_mlp_reduce(float *part, int G, int ld, bool clear, float *gout, float *loss_out,
                              bool adam, float *w, float *m1, float *m2, float lr, float b1,
                              float b2, float eps, float bc1, float bc2, __nv_bfloat16 *w1b,
                              __nv_bfloat16 *w2b, __nv_bfloat16 *w2tb, cudaStream_t s);
cudaError_t launch_apply_prior(const ColonyDev &c, const float *prob, float floor_,
                               cudaStream_t s);

}  // namespace aco
