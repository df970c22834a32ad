// k_mlp.cu -- the edge-scoring MLP of the learned heuristic prior: feature
// extraction for candidate edges, BF16 tensor-core GEMMs with FP32
// accumulation, and the elementwise pieces of the forward and backward passes.
//
// Network: 12 features (padded to 16) -> 128 -> 128 -> 1, ReLU, logistic
// output.  Every matrix product of the forward and backward pass is written
// as C (+)= A * B^T with both operands K-contiguous ("TN"):
//   forward  Z1 = X W1^T,   Z2 = H1 W2^T
//   backward dH1 = dZ2 W2 (B = W2^T stored), dW2 = dZ2^T H1 (A = dZ2^T,
//            B = H1^T stored E-contiguous), dW1 = dZ1^T X (A = dZ1^T, B = X^T)
// so one GEMM kernel covers them; reductions over the edge dimension split K
// across CTAs and accumulate with atomics.  The last layer (128 -> 1) and the
// bias gradients are dot products and reductions on the CUDA cores.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "aco_kernels.h"
#include "aco_mlp.h"

namespace aco {

// ---------------------------------------------------------------- features
// Feature vector of candidate edge (i -> j = nn[i][r]), see aco_mlp.h.
__global__ void k_edge_features(ColonyDev c, const float *__restrict__ x,
                                const float *__restrict__ y, float mean_dk,
                                __nv_bfloat16 *__restrict__ feats, float *__restrict__ labels) {
  const int64_t total = (int64_t)c.n * c.K;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t / c.K), r = (int)(t % c.K);
    const int32_t *nni = c.nn + (size_t)i * c.ldk;
    const int j = nni[r];
    const int32_t *nnj = c.nn + (size_t)j * c.ldk;
    const float d = (float)c.dist[(size_t)i * c.ld + j];
    const float dki = fmaxf(1.0f, (float)c.dist[(size_t)i * c.ld + nni[c.K - 1]]);
    const float dkj = fmaxf(1.0f, (float)c.dist[(size_t)j * c.ld + nnj[c.K - 1]]);
    const float d1i = (float)c.dist[(size_t)i * c.ld + nni[0]];
    const float d1j = (float)c.dist[(size_t)j * c.ld + nnj[0]];
    int rank_ij = c.K;
    bool top5_ji = false;
    for (int q = 0; q < c.K; q++)
      if (nnj[q] == i) {
        rank_ij = q;
        top5_ji = q < 5;
        break;
      }
    float f[kFeatPad];
    f[0] = d / dki;
    f[1] = d / dkj;
    f[2] = (float)r / (float)c.K;
    f[3] = (float)rank_ij / (float)c.K;
    f[4] = (x[j] - x[i]) / dki;
    f[5] = (y[j] - y[i]) / dki;
    f[6] = d1i / dki;
    f[7] = d1j / dkj;
    f[8] = d / (d1i + d1j + 1.0f);
    f[9] = dki / mean_dk;
    f[10] = dkj / mean_dk;
    f[11] = (r < 5 && top5_ji) ? 1.0f : 0.0f;
#pragma unroll
    for (int q = kFeatures; q < kFeatPad; q++) f[q] = 0.0f;
    __nv_bfloat16 *o = feats + t * kFeatPad;
#pragma unroll
    for (int q = 0; q < kFeatPad; q++) o[q] = __float2bfloat16_rn(f[q]);
    if (labels) {
      // Edge of the best-so-far tour: its successor/predecessor column m.
      const int s = c.succT[(size_t)i * c.ldm + c.m], p = c.predT[(size_t)i * c.ldm + c.m];
      labels[t] = (j == s || j == p) ? 1.0f : 0.0f;
    }
  }
}

// Mean over cities of the distance to the K-th candidate.
__global__ void k_mean_dk(ColonyDev c, float *out) {
  __shared__ float part[32];
  float s = 0.0f;
  for (int i = threadIdx.x; i < c.n; i += blockDim.x)
    s += (float)c.dist[(size_t)i * c.ld + c.nn[(size_t)i * c.ldk + c.K - 1]];
  for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(kFull, s, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.0f;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += part[w];
    *out = fmaxf(1.0f, t / (float)c.n);
  }
}

cudaError_t launch_edge_features(const ColonyDev &c, const float *x, const float *y,
                                 float *mean_dk_dev, __nv_bfloat16 *feats, float *labels,
                                 cudaStream_t s) {
  k_mean_dk<<<1, 1024, 0, s>>>(c, mean_dk_dev);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  float h = 0.0f;
  e = cudaMemcpyAsync(&h, mean_dk_dev, sizeof(float), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return e;
  k_edge_features<<<304, 256, 0, s>>>(c, x, y, h, feats, labels);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- TN GEMM
// C[M x N] (op)= A[M x K] * B[N x K]^T, A and B BF16 row-major (K
// contiguous), C FP32 row-major.  CTA tile 128 x 128 x 32, 8 warps of 64 x 32,
// mma.sync.m16n8k16 BF16 with FP32 accumulation, fragments by ldmatrix.
// split > 1 splits K across gridDim.z and adds into C atomically.
constexpr int kBM = 128, kBN = 128, kBK = 32, kPad = 8;  // smem row = 40 halves

__device__ __forceinline__ void ldmatrix_x4(uint32_t (&r)[4], const void *p) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(smem_u32(p)));
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Loads a kBM x kBK (or kBN x kBK) BF16 tile; rows >= rows_valid and k >=
// k_end read as zero.  ld (elements) must be a multiple of 8.
__device__ __forceinline__ void load_tile(__nv_bfloat16 (*dst)[kBK + kPad],
                                          const __nv_bfloat16 *__restrict__ src, int ld,
                                          int row0, int rows_valid, int k0, int k_end) {
  // 128 rows x 4 chunks of 8 halves = 512 chunks, 2 per thread
  for (int q = threadIdx.x; q < kBM * (kBK / 8); q += blockDim.x) {
    const int rr = q >> 2, cc = (q & 3) * 8;
    const int grow = row0 + rr, gk = k0 + cc;
    uint4 v = make_uint4(0, 0, 0, 0);
    if (grow < rows_valid) {
      if (gk + 8 <= k_end) {
        v = *reinterpret_cast<const uint4 *>(src + (size_t)grow * ld + gk);
      } else if (gk < k_end) {
        __nv_bfloat16 tmp[8];
#pragma unroll
        for (int e = 0; e < 8; e++)
          tmp[e] = gk + e < k_end ? src[(size_t)grow * ld + gk + e] : __float2bfloat16_rn(0.0f);
        v = *reinterpret_cast<const uint4 *>(tmp);
      }
    }
    *reinterpret_cast<uint4 *>(&dst[rr][cc]) = v;
  }
}

__global__ void __launch_bounds__(256) k_gemm_tn(const __nv_bfloat16 *__restrict__ A, int lda,
                                                 const __nv_bfloat16 *__restrict__ B, int ldb,
                                                 float *__restrict__ C, int ldc, int M, int N,
                                                 int K, int k_per_split, int mode) {
  __shared__ __align__(16) __nv_bfloat16 sA[kBM][kBK + kPad];
  __shared__ __align__(16) __nv_bfloat16 sB[kBN][kBK + kPad];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wm = warp >> 2, wn = warp & 3;  // 2 x 4 warps, 64 x 32 each
  const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * kBN;
  const int kb = blockIdx.z * k_per_split, ke = min(K, kb + k_per_split);
  float acc[4][4][4];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int e = 0; e < 4; e++) acc[i][j][e] = 0.0f;

  for (int k0 = kb; k0 < ke; k0 += kBK) {
    load_tile(sA, A, lda, m0, M, k0, ke);
    load_tile(sB, B, ldb, n0, N, k0, ke);
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kBK; kk += 16) {
      uint32_t af[4][4];
#pragma unroll
      for (int i = 0; i < 4; i++) {
        const int row = wm * 64 + i * 16 + (lane & 15);
        ldmatrix_x4(af[i], &sA[row][kk + (lane >> 4) * 8]);
      }
      uint32_t bfr[2][4];
#pragma unroll
      for (int j = 0; j < 2; j++) {
        // two n8 tiles per ldmatrix.x4: lanes 0-7 n0-7@k, 8-15 n0-7@k+8,
        // 16-23 n8-15@k, 24-31 n8-15@k+8
        const int nrow = wn * 32 + j * 16 + (lane & 7) + ((lane >> 4) << 3);
        const int kc = kk + ((lane >> 3) & 1) * 8;
        ldmatrix_x4(bfr[j], &sB[nrow][kc]);
      }
#pragma unroll
      for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) mma_bf16(acc[i][j], af[i], bfr[j >> 1][(j & 1) * 2],
                                              bfr[j >> 1][(j & 1) * 2 + 1]);
    }
    __syncthreads();
  }
  const int g = lane >> 2, tig = lane & 3;
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int e = 0; e < 4; e++) {
        const int row = m0 + wm * 64 + i * 16 + g + (e >> 1) * 8;
        const int col = n0 + wn * 32 + j * 8 + tig * 2 + (e & 1);
        if (row < M && col < N) {
          float *p = C + (size_t)row * ldc + col;
          if (mode == kGemmStore)
            *p = acc[i][j][e];
          else if (mode == kGemmAccumulate)
            *p += acc[i][j][e];
          else
            atomicAdd(p, acc[i][j][e]);
        }
      }
}

cudaError_t launch_gemm_tn(const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *B, int ldb,
                           float *C, int ldc, int M, int N, int K, int mode, int splits,
                           cudaStream_t s) {
  if ((lda & 7) || (ldb & 7) || M <= 0 || N <= 0 || K <= 0) return cudaErrorInvalidValue;
  if (splits < 1) splits = 1;
  int kps = (K + splits - 1) / splits;
  kps = (kps + kBK - 1) / kBK * kBK;
  splits = (K + kps - 1) / kps;
  if (splits > 1) mode = kGemmAtomic;
  dim3 grid((N + kBN - 1) / kBN, (M + kBM - 1) / kBM, splits);
  k_gemm_tn<<<grid, 256, 0, s>>>(A, lda, B, ldb, C, ldc, M, N, K, kps, mode);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- elementwise
// Z (E x H, FP32) + bias -> ReLU -> H (BF16, E x H) and, if Ht, its
// transpose (H x ldt, BF16).
__global__ void k_bias_relu(const float *__restrict__ Z, const float *__restrict__ bias, int E,
                            int Hd, __nv_bfloat16 *__restrict__ Hout,
                            __nv_bfloat16 *__restrict__ Ht, int ldt) {
  const int64_t total = (int64_t)E * Hd;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int e = (int)(t / Hd), h = (int)(t % Hd);
    const float v = fmaxf(0.0f, Z[t] + bias[h]);
    const __nv_bfloat16 b = __float2bfloat16_rn(v);
    Hout[t] = b;
    if (Ht) Ht[(size_t)h * ldt + e] = b;
  }
}

cudaError_t launch_bias_relu(const float *Z, const float *bias, int E, int Hd,
                             __nv_bfloat16 *Hout, __nv_bfloat16 *Ht, int ldt, cudaStream_t s) {
  k_bias_relu<<<1216, 256, 0, s>>>(Z, bias, E, Hd, Hout, Ht, ldt);
  return cudaGetLastError();
}

// Last layer and loss.  logit = H2 . w3 + b3 (FP32 over BF16 H2).  With
// labels: weighted logistic loss, dlogit = w (sigmoid(logit) - y) / norm,
// and the gradients of w3 and b3 accumulated (atomics).  Without labels:
// out = sigmoid(logit).
__global__ void k_head(const __nv_bfloat16 *__restrict__ H2, const float *__restrict__ w3,
                       const float *__restrict__ b3, int E, const float *__restrict__ labels,
                       float pos_weight, float norm, float *__restrict__ out,
                       float *__restrict__ dlogit, float *__restrict__ gw3,
                       float *__restrict__ gb3, float *__restrict__ loss) {
  const int lane = threadIdx.x & 31;
  const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  float gw[kHidden / 32];
#pragma unroll
  for (int q = 0; q < kHidden / 32; q++) gw[q] = 0.0f;
  float gb = 0.0f, ls = 0.0f;
  for (int e = warp_global; e < E; e += warps) {
    const __nv_bfloat16 *h = H2 + (size_t)e * kHidden;
    float hv[kHidden / 32];
    float z = 0.0f;
#pragma unroll
    for (int q = 0; q < kHidden / 32; q++) {
      hv[q] = __bfloat162float(h[q * 32 + lane]);
      z += hv[q] * w3[q * 32 + lane];
    }
    for (int o = 16; o; o >>= 1) z += __shfl_xor_sync(kFull, z, o);
    z += b3[0];
    const float p = 1.0f / (1.0f + __expf(-z));
    if (!labels) {
      if (lane == 0) out[e] = p;
      continue;
    }
    const float yv = labels[e];
    if (yv < 0.0f) {  // padding row of a partial batch: no loss, no gradient
      if (lane == 0) dlogit[e] = 0.0f;
      continue;
    }
    const float wt = yv > 0.5f ? pos_weight : 1.0f;
    const float dz = wt * (p - yv) / norm;
    if (lane == 0) {
      dlogit[e] = dz;
      // log(1 + exp(-|z|)) + max(z, 0) - z y, weighted
      const float l = fmaxf(z, 0.0f) - z * yv + log1pf(__expf(-fabsf(z)));
      ls += wt * l / norm;
      gb += dz;
    }
#pragma unroll
    for (int q = 0; q < kHidden / 32; q++) gw[q] += dz * hv[q];
  }
  if (!labels) return;
#pragma unroll
  for (int q = 0; q < kHidden / 32; q++) atomicAdd(&gw3[q * 32 + lane], gw[q]);
  if (lane == 0) {
    atomicAdd(gb3, gb);
    atomicAdd(loss, ls);
  }
}

cudaError_t launch_head(const __nv_bfloat16 *H2, const float *w3, const float *b3, int E,
                        const float *labels, float pos_weight, float norm, float *out,
                        float *dlogit, float *gw3, float *gb3, float *loss, cudaStream_t s) {
  k_head<<<608, 256, 0, s>>>(H2, w3, b3, E, labels, pos_weight, norm, out, dlogit, gw3, gb3,
                             loss);
  return cudaGetLastError();
}

// dZ2 = dlogit (x) w3, masked by ReLU(Z2 + b2) > 0 (H2 > 0); written as BF16
// row-major (E x H) and transposed (H x ldt); bias gradient accumulated.
__global__ void k_grad_hidden2(const float *__restrict__ dlogit, const float *__restrict__ w3,
                               const __nv_bfloat16 *__restrict__ H2, int E,
                               __nv_bfloat16 *__restrict__ dZ, __nv_bfloat16 *__restrict__ dZt,
                               int ldt, float *__restrict__ gb) {
  const int h = threadIdx.x;  // blockDim.x == kHidden
  float acc = 0.0f;
  for (int e = blockIdx.x; e < E; e += gridDim.x) {
    const size_t t = (size_t)e * kHidden + h;
    const float v = __bfloat162float(H2[t]) > 0.0f ? dlogit[e] * w3[h] : 0.0f;
    const __nv_bfloat16 b = __float2bfloat16_rn(v);
    dZ[t] = b;
    dZt[(size_t)h * ldt + e] = b;
    acc += v;
  }
  atomicAdd(&gb[h], acc);
}

cudaError_t launch_grad_hidden2(const float *dlogit, const float *w3, const __nv_bfloat16 *H2,
                                int E, __nv_bfloat16 *dZ, __nv_bfloat16 *dZt, int ldt, float *gb,
                                cudaStream_t s) {
  k_grad_hidden2<<<1216, kHidden, 0, s>>>(dlogit, w3, H2, E, dZ, dZt, ldt, gb);
  return cudaGetLastError();
}

// dZ1 = dH1 masked by H1 > 0; transposed BF16 (H x ldt); bias gradient.
__global__ void k_grad_hidden1(const float *__restrict__ dH1, const __nv_bfloat16 *__restrict__ H1,
                               int E, __nv_bfloat16 *__restrict__ dZt, int ldt,
                               float *__restrict__ gb) {
  const int h = threadIdx.x;
  float acc = 0.0f;
  for (int e = blockIdx.x; e < E; e += gridDim.x) {
    const size_t t = (size_t)e * kHidden + h;
    const float v = __bfloat162float(H1[t]) > 0.0f ? dH1[t] : 0.0f;
    dZt[(size_t)h * ldt + e] = __float2bfloat16_rn(v);
    acc += v;
  }
  atomicAdd(&gb[h], acc);
}

cudaError_t launch_grad_hidden1(const float *dH1, const __nv_bfloat16 *H1, int E,
                                __nv_bfloat16 *dZt, int ldt, float *gb, cudaStream_t s) {
  k_grad_hidden1<<<1216, kHidden, 0, s>>>(dH1, H1, E, dZt, ldt, gb);
  return cudaGetLastError();
}

// X (E x 16 BF16) -> X^T (16 x ldt BF16).
__global__ void k_transpose_feats(const __nv_bfloat16 *__restrict__ X, int E,
                                  __nv_bfloat16 *__restrict__ Xt, int ldt) {
  const int64_t total = (int64_t)E * kFeatPad;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int e = (int)(t / kFeatPad), f = (int)(t % kFeatPad);
    Xt[(size_t)f * ldt + e] = X[t];
  }
}

cudaError_t launch_transpose_feats(const __nv_bfloat16 *X, int E, __nv_bfloat16 *Xt, int ldt,
                                   cudaStream_t s) {
  k_transpose_feats<<<608, 256, 0, s>>>(X, E, Xt, ldt);
  return cudaGetLastError();
}

// Candidate heuristic with the prior: eta_nn = eta(gathered) * (floor + p).
__global__ void k_apply_prior(ColonyDev c, const float *__restrict__ prob, float floor_) {
  const int64_t total = (int64_t)c.n * c.ldk;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / c.ldk;
    const int r = (int)(t % c.ldk);
    if (r >= c.K) continue;
    const int j = c.nn[t];
    const float e = c.eta[i * c.ld + j];
    const_cast<float *>(c.eta_nn)[t] = __fmul_rn(e, __fadd_rn(floor_, prob[i * c.K + r]));
  }
}

cudaError_t launch_apply_prior(const ColonyDev &c, const float *prob, float floor_,
                               cudaStream_t s) {
  k_apply_prior<<<608, 256, 0, s>>>(c, prob, floor_);
  return cudaGetLastError();
}

}  // namespace aco
