// prior.cu -- host side of the learned heuristic prior (C ABI aco_prior_*).
//
// A small MLP scores each candidate edge (i -> nn[i][r]) of a colony from
// local geometric features; it is trained on the GPU on labels taken from
// the best tours the plain method found (an edge is positive when it lies on
// the colony's best-so-far tour), and its output p multiplies the candidate
// heuristic: eta'_ir = eta_ir * (floor + p).  The plain method is unchanged
// otherwise; its fallback still uses the plain heuristic.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <random>
#include <string>
#include <vector>

#include "aco_mlp.h"
#include "colony_internal.h"

using namespace aco;

struct aco_prior {
  cudaStream_t stream = nullptr;
  // parameters: FP32 masters + Adam moments + gradients, BF16 GEMM copies
  float *w = nullptr, *g = nullptr, *m1 = nullptr, *m2 = nullptr;  // kParamCount each
  __nv_bfloat16 *w1b = nullptr;   // [128][16]
  __nv_bfloat16 *w2b = nullptr;   // [128 out][128 in]
  __nv_bfloat16 *w2tb = nullptr;  // [128 in][128 out]
  // training set
  __nv_bfloat16 *X = nullptr;  // E_cap x 16
  float *Y = nullptr;          // E_cap
  int64_t E = 0, E_cap = 0, positives = 0;
  // per-batch workspace (B rows)
  int B = 0;
  float *Z = nullptr;                                  // B x 128
  __nv_bfloat16 *H1 = nullptr, *H1t = nullptr;         // B x 128, 128 x B
  __nv_bfloat16 *H2 = nullptr;                         // B x 128
  __nv_bfloat16 *dZ2 = nullptr, *dZ2t = nullptr;       // B x 128, 128 x B
  __nv_bfloat16 *dZ1t = nullptr, *Xt = nullptr;        // 128 x B, 16 x B
  float *dlogit = nullptr, *out = nullptr, *loss = nullptr, *scratch = nullptr;
  float *gW1full = nullptr;  // [128][16] gradient of the padded first layer
  // fused engine: one partial-gradient row per CTA (gradient, then loss)
  float *part = nullptr;
  int part_rows = 0;
  float *slots = nullptr;  // per-batch losses of the current epoch
  int64_t slots_cap = 0;
  int sms = 0;
  // features and probabilities of the colony being scored (aco_prior_apply)
  __nv_bfloat16 *ax = nullptr;
  float *aprob = nullptr;
  int64_t a_cap = 0;
  int64_t step = 0;
  int engine = ACO_GEMM_FUSED;  // enum aco_gemm_engine
  std::string err;
};

namespace {

int pfail(aco_prior *p, int status, const std::string &msg) {
  if (p) p->err = msg;
  return status;
}

#define ACO_PCUDA(p, call, what)                                                           \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      return pfail(p, e_ == cudaErrorMemoryAllocation ? ACO_ERR_OUT_OF_MEMORY : ACO_ERR_CUDA, \
                   std::string(what) + ": " + cudaGetErrorString(e_));                    \
  } while (0)

template <class T>
cudaError_t alloc(T **p, size_t count) {
  return cudaMalloc(reinterpret_cast<void **>(p), count * sizeof(T) + 16);
}

// One MLP product on the selected tensor-core engine.
cudaError_t gemm(aco_prior *p, const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *B, int ldb,
                 float *C, int ldc, int M, int N, int K, int mode, int splits) {
  if (p->engine == ACO_GEMM_TCGEN05)
    return launch_gemm_tn_tc(A, lda, B, ldb, C, ldc, M, N, K, mode, splits,
                             reinterpret_cast<uint32_t *>(p->scratch + 2), p->stream);
  return launch_gemm_tn(A, lda, B, ldb, C, ldc, M, N, K, mode, splits, p->stream);
}

// Every transfer of the prior goes through its own stream.  The stream is
// non-blocking, so it is not ordered after the legacy stream that a plain
// cudaMemcpy / cudaMemset uses, and a pageable upload may return before its
// DMA has landed: a kernel launched next could read the old contents.
cudaError_t copy_sync(aco_prior *p, void *dst, const void *src, size_t bytes,
                      cudaMemcpyKind kind) {
  cudaError_t e = cudaMemcpyAsync(dst, src, bytes, kind, p->stream);
  return e == cudaSuccess ? cudaStreamSynchronize(p->stream) : e;
}

cudaError_t zero(aco_prior *p, void *dst, size_t bytes) {
  return cudaMemsetAsync(dst, 0, bytes, p->stream);
}

// Reads (and clears) the device word the tensor-core GEMM sets when one of
// its bounded waits ran out.
int gemm_status(aco_prior *p) {
  uint32_t h = 0;
  uint32_t *w = reinterpret_cast<uint32_t *>(p->scratch + 2);
  if (copy_sync(p, &h, w, 4, cudaMemcpyDeviceToHost) != cudaSuccess)
    return pfail(p, ACO_ERR_CUDA, "read gemm status");
  if (!h) return ACO_OK;
  zero(p, w, 4);
  return pfail(p, ACO_ERR_DEVICE_TIMEOUT, "tensor-core gemm wait timed out");
}

// Refreshes the BF16 copies of W1 (padded to 16 inputs) and W2 from the masters.
int sync_bf16(aco_prior *p) {
  std::vector<float> w(kParamCount);
  ACO_PCUDA(p, copy_sync(p, w.data(), p->w, sizeof(float) * kParamCount, cudaMemcpyDeviceToHost),
            "read weights");
  std::vector<__nv_bfloat16> w1(kHidden * kFeatPad), w2(kHidden * kHidden), w2t(kHidden * kHidden);
  for (int o = 0; o < kHidden; o++)
    for (int f = 0; f < kFeatPad; f++)
      w1[o * kFeatPad + f] =
          __float2bfloat16_rn(f < kFeatures ? w[kParamW1 + o * kFeatures + f] : 0.0f);
  for (int o = 0; o < kHidden; o++)
    for (int i = 0; i < kHidden; i++) {
      w2[o * kHidden + i] = __float2bfloat16_rn(w[kParamW2 + o * kHidden + i]);
      w2t[i * kHidden + o] = w2[o * kHidden + i];
    }
  ACO_PCUDA(p, copy_sync(p, p->w1b, w1.data(), w1.size() * 2, cudaMemcpyHostToDevice), "w1");
  ACO_PCUDA(p, copy_sync(p, p->w2b, w2.data(), w2.size() * 2, cudaMemcpyHostToDevice), "w2");
  ACO_PCUDA(p, copy_sync(p, p->w2tb, w2t.data(), w2t.size() * 2, cudaMemcpyHostToDevice), "w2t");
  return ACO_OK;
}

int ensure_workspace(aco_prior *p, int B) {
  if (B <= p->B) return ACO_OK;
  cudaFree(p->Z); cudaFree(p->H1); cudaFree(p->H1t); cudaFree(p->H2); cudaFree(p->dZ2);
  cudaFree(p->dZ2t); cudaFree(p->dZ1t); cudaFree(p->Xt); cudaFree(p->dlogit); cudaFree(p->out);
  const size_t h = (size_t)B * kHidden;
  ACO_PCUDA(p, alloc(&p->Z, h), "alloc");
  ACO_PCUDA(p, alloc(&p->H1, h), "alloc");
  ACO_PCUDA(p, alloc(&p->H1t, h), "alloc");
  ACO_PCUDA(p, alloc(&p->H2, h), "alloc");
  ACO_PCUDA(p, alloc(&p->dZ2, h), "alloc");
  ACO_PCUDA(p, alloc(&p->dZ2t, h), "alloc");
  ACO_PCUDA(p, alloc(&p->dZ1t, h), "alloc");
  ACO_PCUDA(p, alloc(&p->Xt, (size_t)B * kFeatPad), "alloc");
  ACO_PCUDA(p, alloc(&p->dlogit, (size_t)B), "alloc");
  ACO_PCUDA(p, alloc(&p->out, (size_t)B), "alloc");
  p->B = B;
  return ACO_OK;
}

// Forward pass over rows X[0..B) (B a multiple of 128); with labels also the
// loss and the gradients, accumulated into p->g (W1 part via gW1full).
int forward_backward(aco_prior *p, const __nv_bfloat16 *X, const float *Y, int B, int valid,
                     float pos_weight, bool backward, float *probs_dev, float *loss_dev) {
  cudaStream_t s = p->stream;
  const int splits = std::max(1, std::min(64, B / 1024));
  // Z1 = X W1^T ; H1 = relu(Z1 + b1)
  ACO_PCUDA(p, gemm(p, X, kFeatPad, p->w1b, kFeatPad, p->Z, kHidden, B, kHidden, kFeatPad,
                    kGemmStore, 1), "gemm z1");
  ACO_PCUDA(p, launch_bias_relu(p->Z, p->w + kParamB1, B, kHidden, p->H1,
                                backward ? p->H1t : nullptr, B, s), "h1");
  // Z2 = H1 W2^T ; H2 = relu(Z2 + b2)
  ACO_PCUDA(p, gemm(p, p->H1, kHidden, p->w2b, kHidden, p->Z, kHidden, B, kHidden, kHidden,
                    kGemmStore, 1), "gemm z2");
  ACO_PCUDA(p, launch_bias_relu(p->Z, p->w + kParamB2, B, kHidden, p->H2, nullptr, 0, s), "h2");
  if (!backward) {
    ACO_PCUDA(p, launch_head(p->H2, p->w + kParamW3, p->w + kParamB3, valid, nullptr, 1.0f, 1.0f,
                             probs_dev, nullptr, nullptr, nullptr, nullptr, s), "head");
    return ACO_OK;
  }
  ACO_PCUDA(p, launch_head(p->H2, p->w + kParamW3, p->w + kParamB3, B, Y, pos_weight,
                           (float)std::max(1, valid), nullptr, p->dlogit, p->g + kParamW3,
                           p->g + kParamB3, loss_dev, s), "head");
  // dZ2 = dlogit w3 * [H2 > 0]
  ACO_PCUDA(p, launch_grad_hidden2(p->dlogit, p->w + kParamW3, p->H2, B, p->dZ2, p->dZ2t, B,
                                   p->g + kParamB2, s), "dz2");
  // dW2 += dZ2^T H1
  ACO_PCUDA(p, gemm(p, p->dZ2t, B, p->H1t, B, p->g + kParamW2, kHidden, kHidden, kHidden, B,
                    kGemmAtomic, splits), "gemm dw2");
  // dH1 = dZ2 W2 ; dZ1 = dH1 * [H1 > 0]
  ACO_PCUDA(p, gemm(p, p->dZ2, kHidden, p->w2tb, kHidden, p->Z, kHidden, B, kHidden, kHidden,
                    kGemmStore, 1), "gemm dh1");
  ACO_PCUDA(p, launch_grad_hidden1(p->Z, p->H1, B, p->dZ1t, B, p->g + kParamB1, s), "dz1");
  // dW1 += dZ1^T X
  ACO_PCUDA(p, launch_transpose_feats(X, B, p->Xt, B, s), "xt");
  ACO_PCUDA(p, gemm(p, p->dZ1t, B, p->Xt, B, p->gW1full, kFeatPad, kHidden, kFeatPad, B,
                    kGemmAtomic, splits), "gemm dw1");
  return ACO_OK;
}

// Moves the padded first-layer gradient into the packed gradient vector.
// Each thread owns one padded entry: it reads it, adds it (real features
// only) and clears it, so no entry is cleared by another thread first.
__global__ void k_pack_w1_grad(float *gW1full, float *g) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= kHidden * kFeatPad) return;
  const int o = t / kFeatPad, f = t % kFeatPad;
  if (f < kFeatures) g[kParamW1 + o * kFeatures + f] += gW1full[t];
  gW1full[t] = 0.0f;
}

int pack_grads(aco_prior *p) {
  k_pack_w1_grad<<<(kHidden * kFeatPad + 255) / 256, 256, 0, p->stream>>>(p->gW1full, p->g);
  ACO_PCUDA(p, cudaGetLastError(), "pack grads");
  return ACO_OK;
}

// Row pitch of the fused engine's partial-gradient rows (gradient + loss).
constexpr int kPartLd = (kParamCount + 1 + 3) / 4 * 4;

int ensure_fused(aco_prior *p, int rows) {
  if (!p->sms) {
    int dev = 0;
    ACO_PCUDA(p, cudaGetDevice(&dev), "device");
    ACO_PCUDA(p, cudaDeviceGetAttribute(&p->sms, cudaDevAttrMultiProcessorCount, dev), "SMs");
  }
  const int G = mlp_fused_grid(rows, p->sms);
  if (G > p->part_rows) {
    cudaFree(p->part);
    p->part = nullptr;
    p->part_rows = 0;
    ACO_PCUDA(p, alloc(&p->part, (size_t)G * kPartLd), "alloc partials");
    p->part_rows = G;
  }
  return ACO_OK;
}

int ensure_slots(aco_prior *p, int64_t n) {
  if (n <= p->slots_cap) return ACO_OK;
  cudaFree(p->slots);
  p->slots = nullptr;
  p->slots_cap = 0;
  ACO_PCUDA(p, alloc(&p->slots, (size_t)n), "alloc loss slots");
  p->slots_cap = n;
  return ACO_OK;
}

// One Adam step from the summed gradient rows (the fused engine's
// partials, or the layered engines' accumulated vector, which is cleared),
// with the BF16 weight copies refreshed on the device: no host round trip.
int adam_step(aco_prior *p, float lr, float *part, int G, int ld, bool clear, float *loss_out) {
  p->step++;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float bc1 = 1.0f - powf(b1, (float)p->step), bc2 = 1.0f - powf(b2, (float)p->step);
  ACO_PCUDA(p, launch_mlp_reduce(part, G, ld, clear, nullptr, loss_out, true, p->w, p->m1, p->m2,
                                 lr, b1, b2, eps, bc1, bc2, p->w1b, p->w2b, p->w2tb, p->stream),
            "adam");
  return ACO_OK;
}

// Forward (+ backward) of rows X[0..rows) on the fused engine; with labels
// the summed gradient goes to gout and the loss to loss_out.
int fused_pass(aco_prior *p, const __nv_bfloat16 *X, const float *Y, int rows, float pos_weight,
               float *probs, float *gout, float *loss_out) {
  if (int s = ensure_fused(p, rows)) return s;
  const int G = mlp_fused_grid(rows, p->sms);
  uint32_t *err = reinterpret_cast<uint32_t *>(p->scratch + 2);
  ACO_PCUDA(p, launch_mlp_fused(Y != nullptr, X, rows, p->w1b, p->w2b, p->w, Y,
                                pos_weight, (float)std::max(1, rows), probs, p->part, kPartLd, G,
                                err, p->stream), "fused mlp");
  if (Y)
    ACO_PCUDA(p, launch_mlp_reduce(p->part, G, kPartLd, false, gout, loss_out, false, p->w,
                                   p->m1, p->m2, 0.0f, 0.0f, 0.0f, 0.0f, 1.0f, 1.0f, nullptr,
                                   nullptr, nullptr, p->stream), "reduce");
  return ACO_OK;
}

// Uploads host examples (E x 12 FP32 features) into padded BF16 rows.
int upload_examples(aco_prior *p, const float *feats, const float *labels, int E, int B,
                    __nv_bfloat16 **Xd, float **Yd) {
  std::vector<__nv_bfloat16> x((size_t)B * kFeatPad, __float2bfloat16_rn(0.0f));
  std::vector<float> y((size_t)B, -1.0f);
  for (int e = 0; e < E; e++) {
    for (int f = 0; f < kFeatures; f++)
      x[(size_t)e * kFeatPad + f] = __float2bfloat16_rn(feats[(size_t)e * kFeatures + f]);
    if (labels) y[e] = labels[e];
  }
  ACO_PCUDA(p, alloc(Xd, x.size()), "alloc");
  ACO_PCUDA(p, alloc(Yd, y.size()), "alloc");
  ACO_PCUDA(p, copy_sync(p, *Xd, x.data(), x.size() * 2, cudaMemcpyHostToDevice), "upload x");
  ACO_PCUDA(p, copy_sync(p, *Yd, y.data(), y.size() * 4, cudaMemcpyHostToDevice), "upload y");
  return ACO_OK;
}

int round_rows(int E) { return (E + 127) / 128 * 128; }

}  // namespace

extern "C" {

int aco_prior_create(uint64_t seed, aco_prior **out) {
  if (!out) return ACO_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  aco_prior *p = new (std::nothrow) aco_prior();
  if (!p) return ACO_ERR_OUT_OF_MEMORY;
  if (cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete p;
    return ACO_ERR_CUDA;
  }
  bool ok = alloc(&p->w, kParamCount) == cudaSuccess && alloc(&p->g, kParamCount) == cudaSuccess &&
            alloc(&p->m1, kParamCount) == cudaSuccess &&
            alloc(&p->m2, kParamCount) == cudaSuccess &&
            alloc(&p->w1b, kHidden * kFeatPad) == cudaSuccess &&
            alloc(&p->w2b, kHidden * kHidden) == cudaSuccess &&
            alloc(&p->w2tb, kHidden * kHidden) == cudaSuccess &&
            alloc(&p->loss, 1) == cudaSuccess && alloc(&p->scratch, 4) == cudaSuccess &&
            alloc(&p->gW1full, kHidden * kFeatPad) == cudaSuccess;
  if (!ok) {
    aco_prior_destroy(p);
    return ACO_ERR_OUT_OF_MEMORY;
  }
  // He initialisation (normal, std sqrt(2 / fan_in)), zero biases.
  std::mt19937_64 rng(seed);
  std::normal_distribution<float> nd(0.0f, 1.0f);
  std::vector<float> w(kParamCount, 0.0f);
  for (int t = 0; t < kHidden * kFeatures; t++) w[kParamW1 + t] = nd(rng) * sqrtf(2.0f / kFeatures);
  for (int t = 0; t < kHidden * kHidden; t++) w[kParamW2 + t] = nd(rng) * sqrtf(2.0f / kHidden);
  for (int t = 0; t < kHidden; t++) w[kParamW3 + t] = nd(rng) * sqrtf(1.0f / kHidden);
  zero(p, p->g, sizeof(float) * kParamCount);
  zero(p, p->m1, sizeof(float) * kParamCount);
  zero(p, p->m2, sizeof(float) * kParamCount);
  zero(p, p->gW1full, sizeof(float) * kHidden * kFeatPad);
  zero(p, p->scratch, sizeof(float) * 4);
  if (copy_sync(p, p->w, w.data(), sizeof(float) * kParamCount, cudaMemcpyHostToDevice) !=
          cudaSuccess ||
      sync_bf16(p) != ACO_OK) {
    aco_prior_destroy(p);
    return ACO_ERR_CUDA;
  }
  *out = p;
  return ACO_OK;
}

int aco_prior_get_weights(aco_prior *p, float *out) {
  if (!p || !out) return ACO_ERR_INVALID_ARGUMENT;
  ACO_PCUDA(p, copy_sync(p, out, p->w, sizeof(float) * kParamCount, cudaMemcpyDeviceToHost),
            "read");
  return ACO_OK;
}

int aco_prior_set_weights(aco_prior *p, const float *in) {
  if (!p || !in) return ACO_ERR_INVALID_ARGUMENT;
  ACO_PCUDA(p, copy_sync(p, p->w, in, sizeof(float) * kParamCount, cudaMemcpyHostToDevice),
            "write");
  return sync_bf16(p);
}

int aco_prior_param_count(void) { return kParamCount; }

int aco_prior_add_examples(aco_prior *p, aco_colony *c) {
  if (!p || !c) return ACO_ERR_INVALID_ARGUMENT;
  if (!c->initialized || !c->xy) return pfail(p, ACO_ERR_UNSUPPORTED,
                                              "colony must be initialized and built from coordinates");
  const int64_t add = (int64_t)c->n * c->K;
  if (p->E + add > p->E_cap) {
    const int64_t cap = std::max<int64_t>(p->E_cap * 2, p->E + add + 4096);
    __nv_bfloat16 *X = nullptr;
    float *Y = nullptr;
    ACO_PCUDA(p, alloc(&X, (size_t)cap * kFeatPad), "alloc examples");
    ACO_PCUDA(p, alloc(&Y, (size_t)cap), "alloc labels");
    if (p->E) {
      ACO_PCUDA(p, copy_sync(p, X, p->X, (size_t)p->E * kFeatPad * 2, cudaMemcpyDeviceToDevice),
                "copy");
      ACO_PCUDA(p, copy_sync(p, Y, p->Y, (size_t)p->E * 4, cudaMemcpyDeviceToDevice), "copy");
    }
    cudaFree(p->X);
    cudaFree(p->Y);
    p->X = X;
    p->Y = Y;
    p->E_cap = cap;
  }
  ACO_PCUDA(p, cudaStreamSynchronize(c->stream), "synchronize colony");
  const ColonyDev d = colony_dev(c);
  ACO_PCUDA(p, launch_edge_features(d, c->xy, c->xy + c->n, p->scratch,
                                    p->X + (size_t)p->E * kFeatPad, p->Y + p->E, p->stream),
            "features");
  std::vector<float> y((size_t)add);
  ACO_PCUDA(p, cudaMemcpyAsync(y.data(), p->Y + p->E, (size_t)add * 4, cudaMemcpyDeviceToHost,
                               p->stream), "read labels");
  ACO_PCUDA(p, cudaStreamSynchronize(p->stream), "synchronize");
  for (float v : y) p->positives += v > 0.5f;
  p->E += add;
  return ACO_OK;
}

int aco_prior_num_examples(aco_prior *p, int64_t *E, int64_t *positives) {
  if (!p) return ACO_ERR_INVALID_ARGUMENT;
  if (E) *E = p->E;
  if (positives) *positives = p->positives;
  return ACO_OK;
}

int aco_prior_clear_examples(aco_prior *p) {
  if (!p) return ACO_ERR_INVALID_ARGUMENT;
  p->E = 0;
  p->positives = 0;
  return ACO_OK;
}

int aco_prior_train(aco_prior *p, int32_t epochs, int32_t batch, float lr, uint64_t seed,
                    float *last_loss) {
  if (!p || epochs < 0 || batch < 128) return ACO_ERR_INVALID_ARGUMENT;
  if (p->E == 0) return pfail(p, ACO_ERR_NOT_INITIALIZED, "no training examples");
  const int B = round_rows(batch);
  const bool fused = p->engine == ACO_GEMM_FUSED;
  if (int s = fused ? ensure_fused(p, B) : ensure_workspace(p, B)) return s;
  const float pos_weight =
      p->positives ? (float)(p->E - p->positives) / (float)p->positives : 1.0f;
  const int64_t nb = (p->E + B - 1) / B;
  if (int s = ensure_slots(p, nb)) return s;
  std::vector<int64_t> order((size_t)nb);
  std::mt19937_64 rng(seed);
  __nv_bfloat16 *Xtail = nullptr;
  float *Ytail = nullptr;
  const int64_t tail = p->E - (nb - 1) * B;  // rows of the last batch
  if (tail < B && !fused) {  // the layered engines pad the last batch with label -1 rows
    ACO_PCUDA(p, alloc(&Xtail, (size_t)B * kFeatPad), "alloc");
    ACO_PCUDA(p, alloc(&Ytail, (size_t)B), "alloc");
    ACO_PCUDA(p, zero(p, Xtail, (size_t)B * kFeatPad * 2), "memset");
    std::vector<float> neg((size_t)B, -1.0f);
    ACO_PCUDA(p, copy_sync(p, Ytail, neg.data(), (size_t)B * 4, cudaMemcpyHostToDevice), "init");
    ACO_PCUDA(p, copy_sync(p, Xtail, p->X + (size_t)(nb - 1) * B * kFeatPad,
                           (size_t)tail * kFeatPad * 2, cudaMemcpyDeviceToDevice), "tail");
    ACO_PCUDA(p, copy_sync(p, Ytail, p->Y + (size_t)(nb - 1) * B, (size_t)tail * 4,
                           cudaMemcpyDeviceToDevice), "tail");
  }
  // No host synchronisation inside an epoch: each batch's loss lands in its
  // own device slot, and only the last epoch's slots are read back.
  int s = ACO_OK;
  for (int ep = 0; ep < epochs && !s; ep++) {
    for (int64_t q = 0; q < nb; q++) order[q] = q;
    std::shuffle(order.begin(), order.end(), rng);
    if (!fused && cudaMemsetAsync(p->slots, 0, (size_t)nb * 4, p->stream) != cudaSuccess)
      s = pfail(p, ACO_ERR_CUDA, "memset");
    for (int64_t b = 0; b < nb && !s; b++) {
      const int64_t q = order[(size_t)b];
      const int valid = q == nb - 1 ? (int)tail : B;
      if (fused) {
        const __nv_bfloat16 *X = p->X + (size_t)q * B * kFeatPad;
        const float *Y = p->Y + (size_t)q * B;
        if (!(s = ensure_fused(p, valid))) {
          const int G = mlp_fused_grid(valid, p->sms);
          uint32_t *err = reinterpret_cast<uint32_t *>(p->scratch + 2);
          if (launch_mlp_fused(true, X, valid, p->w1b, p->w2b, p->w, Y, pos_weight,
                               (float)std::max(1, valid), nullptr, p->part, kPartLd, G, err,
                               p->stream) != cudaSuccess)
            s = pfail(p, ACO_ERR_CUDA, "fused mlp");
          if (!s) s = adam_step(p, lr, p->part, G, kPartLd, false, p->slots + b);
        }
      } else {
        const bool last = q == nb - 1 && Xtail;
        const __nv_bfloat16 *X = last ? Xtail : p->X + (size_t)q * B * kFeatPad;
        const float *Y = last ? Ytail : p->Y + (size_t)q * B;
        s = forward_backward(p, X, Y, B, valid, pos_weight, true, nullptr, p->slots + b);
        if (!s) s = pack_grads(p);
        if (!s) s = adam_step(p, lr, p->g, 1, kParamCount, true, nullptr);
      }
    }
  }
  float loss = 0.0f;
  if (!s && epochs > 0) {
    std::vector<float> h((size_t)nb);
    if (cudaMemcpyAsync(h.data(), p->slots, (size_t)nb * 4, cudaMemcpyDeviceToHost, p->stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(p->stream) != cudaSuccess)
      s = pfail(p, ACO_ERR_CUDA, "read losses");
    double ep_loss = 0.0;
    for (float v : h) ep_loss += v;
    loss = (float)(ep_loss / nb);
  } else if (!s) {
    s = cudaStreamSynchronize(p->stream) == cudaSuccess ? ACO_OK : ACO_ERR_CUDA;
  }
  cudaStreamSynchronize(p->stream);
  cudaFree(Xtail);
  cudaFree(Ytail);
  if (s) return s;
  if (last_loss) *last_loss = loss;
  return gemm_status(p);
}

int aco_prior_loss_and_grads(aco_prior *p, const float *feats, const float *labels, int32_t E,
                             float pos_weight, float *loss, float *grads) {
  if (!p || !feats || !labels || E < 1 || !grads) return ACO_ERR_INVALID_ARGUMENT;
  const int B = round_rows(E);
  const bool fused = p->engine == ACO_GEMM_FUSED;
  if (int s = fused ? ensure_fused(p, E) : ensure_workspace(p, B)) return s;
  __nv_bfloat16 *X = nullptr;
  float *Y = nullptr;
  if (int s = upload_examples(p, feats, labels, E, B, &X, &Y)) return s;
  int s = ACO_OK;
  if (fused) {
    s = fused_pass(p, X, Y, E, pos_weight, nullptr, p->g, p->loss);
  } else {
    ACO_PCUDA(p, cudaMemsetAsync(p->g, 0, sizeof(float) * kParamCount, p->stream), "memset");
    ACO_PCUDA(p, cudaMemsetAsync(p->loss, 0, 4, p->stream), "memset");
    s = forward_backward(p, X, Y, B, E, pos_weight, true, nullptr, p->loss);
    if (!s) s = pack_grads(p);
  }
  float h = 0.0f;
  if (!s) {
    cudaMemcpyAsync(&h, p->loss, 4, cudaMemcpyDeviceToHost, p->stream);
    cudaMemcpyAsync(grads, p->g, sizeof(float) * kParamCount, cudaMemcpyDeviceToHost, p->stream);
    if (cudaStreamSynchronize(p->stream) != cudaSuccess) s = ACO_ERR_CUDA;
    cudaMemsetAsync(p->g, 0, sizeof(float) * kParamCount, p->stream);
  }
  cudaStreamSynchronize(p->stream);
  cudaFree(X);
  cudaFree(Y);
  if (loss) *loss = h;
  return s ? s : gemm_status(p);
}

int aco_prior_predict(aco_prior *p, const float *feats, int32_t E, float *probs) {
  if (!p || !feats || E < 1 || !probs) return ACO_ERR_INVALID_ARGUMENT;
  const int B = round_rows(E);
  const bool fused = p->engine == ACO_GEMM_FUSED;
  if (int s = fused ? ensure_fused(p, E) : ensure_workspace(p, B)) return s;
  __nv_bfloat16 *X = nullptr;
  float *Y = nullptr;
  if (int s = upload_examples(p, feats, nullptr, E, B, &X, &Y)) return s;
  float *out = p->out;
  int s = ACO_OK;
  if (fused && alloc(&out, (size_t)B) != cudaSuccess) s = ACO_ERR_OUT_OF_MEMORY;
  if (!s)
    s = fused ? fused_pass(p, X, nullptr, E, 1.0f, out, nullptr, nullptr)
              : forward_backward(p, X, nullptr, B, E, 1.0f, false, out, nullptr);
  if (!s && cudaMemcpyAsync(probs, out, (size_t)E * 4, cudaMemcpyDeviceToHost, p->stream) !=
                cudaSuccess)
    s = ACO_ERR_CUDA;
  if (!s && cudaStreamSynchronize(p->stream) != cudaSuccess) s = ACO_ERR_CUDA;
  cudaStreamSynchronize(p->stream);
  if (fused) cudaFree(out);
  cudaFree(X);
  cudaFree(Y);
  return s ? s : gemm_status(p);
}

int aco_prior_apply(aco_prior *p, aco_colony *c, float floor_) {
  if (!p || !c) return ACO_ERR_INVALID_ARGUMENT;
  if (!c->initialized || !c->xy) return pfail(p, ACO_ERR_UNSUPPORTED,
                                              "colony must be initialized and built from coordinates");
  const int E = c->n * c->K;
  const int B = round_rows(E);
  const bool fused = p->engine == ACO_GEMM_FUSED;
  if (int s = fused ? ensure_fused(p, E) : ensure_workspace(p, B)) return s;
  if (B > p->a_cap) {  // kept across calls: scoring a colony allocates nothing
    cudaFree(p->ax);
    cudaFree(p->aprob);
    p->ax = nullptr;
    p->aprob = nullptr;
    p->a_cap = 0;
    ACO_PCUDA(p, alloc(&p->ax, (size_t)B * kFeatPad), "alloc");
    ACO_PCUDA(p, alloc(&p->aprob, (size_t)B), "alloc");
    p->a_cap = B;
  }
  __nv_bfloat16 *X = p->ax;
  float *prob = p->aprob;
  if (!fused && B > E)  // the layered engines read whole 128-row blocks
    ACO_PCUDA(p, cudaMemsetAsync(X + (size_t)E * kFeatPad, 0, (size_t)(B - E) * kFeatPad * 2,
                                 p->stream), "memset");
  ACO_PCUDA(p, cudaStreamSynchronize(c->stream), "synchronize colony");
  const ColonyDev d = colony_dev(c);
  int s = launch_edge_features(d, c->xy, c->xy + c->n, p->scratch, X, nullptr, p->stream) ==
                  cudaSuccess
              ? ACO_OK
              : ACO_ERR_CUDA;
  if (!s)
    s = fused ? fused_pass(p, X, nullptr, E, 1.0f, prob, nullptr, nullptr)
              : forward_backward(p, X, nullptr, B, E, 1.0f, false, prob, nullptr);
  if (!s && launch_apply_prior(d, prob, floor_, p->stream) != cudaSuccess) s = ACO_ERR_CUDA;
  if (!s && launch_pheromone_rows(d, false, false, false, p->stream) != cudaSuccess)
    s = ACO_ERR_CUDA;
  if (!s && cudaStreamSynchronize(p->stream) != cudaSuccess) s = ACO_ERR_CUDA;
  if (s) return pfail(p, s, "apply failed");
  if (int g = gemm_status(p)) return g;
  // The colony's candidate table changed: a captured iteration graph stays
  // valid (same buffers), the staged copy is reloaded at every launch.
  return ACO_OK;
}

int aco_colony_edge_features(aco_colony *c, float *out) {
  if (!c || !out) return ACO_ERR_INVALID_ARGUMENT;
  if (!c->initialized || !c->xy) return ACO_ERR_UNSUPPORTED;
  const int E = c->n * c->K;
  __nv_bfloat16 *X = nullptr;
  float *scratch = nullptr;
  if (alloc(&X, (size_t)E * kFeatPad) != cudaSuccess || alloc(&scratch, 4) != cudaSuccess)
    return ACO_ERR_OUT_OF_MEMORY;
  int s = ACO_OK;
  if (cudaStreamSynchronize(c->stream) != cudaSuccess ||
      launch_edge_features(colony_dev(c), c->xy, c->xy + c->n, scratch, X, nullptr, c->stream) !=
          cudaSuccess ||
      cudaStreamSynchronize(c->stream) != cudaSuccess)
    s = ACO_ERR_CUDA;
  if (!s) {
    std::vector<__nv_bfloat16> h((size_t)E * kFeatPad);
    if (cudaMemcpyAsync(h.data(), X, h.size() * 2, cudaMemcpyDeviceToHost, c->stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess)
      s = ACO_ERR_CUDA;
    for (int e = 0; e < (s ? 0 : E); e++)
      for (int f = 0; f < kFeatures; f++)
        out[(size_t)e * kFeatures + f] = __bfloat162float(h[(size_t)e * kFeatPad + f]);
  }
  cudaFree(X);
  cudaFree(scratch);
  return s;
}

int aco_prior_set_engine(aco_prior *p, int32_t engine) {
  if (!p || (engine != ACO_GEMM_MMA_SYNC && engine != ACO_GEMM_TCGEN05 &&
             engine != ACO_GEMM_FUSED))
    return ACO_ERR_INVALID_ARGUMENT;
  p->engine = engine;
  return ACO_OK;
}

int aco_gemm_bf16_tn(const uint16_t *A, const uint16_t *B, float *C, int32_t M, int32_t N,
                     int32_t K, int32_t splits, int32_t engine) {
  if (!A || !B || !C || M < 1 || N < 1 || K < 1 || (K & 7)) return ACO_ERR_INVALID_ARGUMENT;
  if (engine == ACO_GEMM_TCGEN05 && N != 128 && N != 16) return ACO_ERR_UNSUPPORTED;
  __nv_bfloat16 *dA = nullptr, *dB = nullptr;
  float *dC = nullptr;
  uint32_t *derr = nullptr;
  int s = ACO_OK;
  if (alloc(&dA, (size_t)M * K) != cudaSuccess || alloc(&dB, (size_t)N * K) != cudaSuccess ||
      alloc(&dC, (size_t)M * N) != cudaSuccess || alloc(&derr, 1) != cudaSuccess)
    s = ACO_ERR_OUT_OF_MEMORY;
  if (!s) {
    cudaMemcpy(dA, A, (size_t)M * K * 2, cudaMemcpyHostToDevice);
    cudaMemcpy(dB, B, (size_t)N * K * 2, cudaMemcpyHostToDevice);
    cudaMemset(dC, 0, (size_t)M * N * 4);
    cudaMemset(derr, 0, 4);
    cudaError_t e = engine == ACO_GEMM_TCGEN05
                        ? launch_gemm_tn_tc(dA, K, dB, K, dC, N, M, N, K, kGemmStore, splits,
                                            derr, 0)
                        : launch_gemm_tn(dA, K, dB, K, dC, N, M, N, K, kGemmStore, splits, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    uint32_t herr = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&herr, derr, 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(C, dC, (size_t)M * N * 4, cudaMemcpyDeviceToHost);
    s = e != cudaSuccess ? ACO_ERR_CUDA : (herr ? ACO_ERR_DEVICE_TIMEOUT : ACO_OK);
  }
  cudaFree(dA);
  cudaFree(dB);
  cudaFree(dC);
  cudaFree(derr);
  return s;
}

const char *aco_prior_last_error(const aco_prior *p) { return p ? p->err.c_str() : ""; }

void aco_prior_destroy(aco_prior *p) {
  if (!p) return;
  if (p->stream) cudaStreamSynchronize(p->stream);
  void *bufs[] = {p->w, p->g, p->m1, p->m2, p->w1b, p->w2b, p->w2tb, p->X, p->Y, p->Z, p->H1,
                  p->H1t, p->H2, p->dZ2, p->dZ2t, p->dZ1t, p->Xt, p->dlogit, p->out, p->loss,
                  p->scratch, p->gW1full, p->part, p->slots, p->ax, p->aprob};
  for (void *b : bufs)
    if (b) cudaFree(b);
  if (p->stream) cudaStreamDestroy(p->stream);
  delete p;
}

}  // extern "C"
