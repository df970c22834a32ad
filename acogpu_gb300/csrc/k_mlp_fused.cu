// k_mlp_fused.cu -- the edge-scoring MLP (12 -> 128 -> 128 -> 1, ReLU,
// weighted logistic loss) as ONE tcgen05 kernel per pass over a set of
// edges: forward, loss and backward of each 128-edge tile stay on the SM.
//
// A CTA (16 warps) owns tiles blockIdx.x, blockIdx.x + gridDim.x, ...; warp w
// reads accumulator lanes 32(w % 4).. (the tile's rows) and columns
// 32(w / 4).. of every 128-column accumulator.  Per tile:
//   Z1  = X W1^T            (TMEM cols [0,128), K = 16)
//   H1  = bf16(relu(Z1 + b1)) -> shared memory
//   Z2  = H1 W2^T           (TMEM cols [0,128), K = 128)
//   H2  = bf16(relu(Z2 + b2)); z = H2 . w3 + b3; p = sigmoid(z)
//   dz  = w (p - y) / norm; dZ2 = bf16(dz w3 [H2 > 0]) -> shared memory
//   dH1 = dZ2 W2            (TMEM cols [0,128))
//   dW2 += dZ2^T H1         (TMEM cols [128,256), accumulated over tiles)
//   dZ1 = bf16(dH1 [H1 > 0]) -> shared memory
//   dW1 += dZ1^T X          (TMEM cols [256,272), accumulated over tiles)
// Every activation is written once, row-major (one row per edge): the
// products that contract over the edges (dW2, dW1) and the one that needs
// W2 rather than W2^T (dH1) read the same tiles as MN-major operands, so no
// transposed copy exists anywhere.
// The w3 and b2 gradients are column sums over the rows too, and go to the
// tensor cores: with H2 and its ReLU mask written row-major, and dz split
// into two BF16 terms (hi = bf16(dz), lo = bf16(dz - hi): 16 significant
// bits) as the two rows of a 16-row B tile, gw3 = H2^T dz and
// sum_e mask dz accumulate in TMEM (cols [320,336) and [352,368)), each
// product exact in FP32; gb2 = w3 * the latter.
// The b1 gradient (over the FP32 dH1) is reduced across each warp's 32 rows
// by a shuffle reduce-scatter and kept per lane.  At the
// end every CTA writes its partial gradient (and loss) to its own row of
// `part`; k_mlp_reduce sums the rows in a fixed order (deterministic, no
// atomics) and applies the Adam step, refreshing the BF16 weight copies.
// The BF16 rounding points are those of the layered kernels in k_mlp.cu.
//
// Operands come from TMA (X tile, W1, W2; 128-byte swizzle) or are
// written by the epilogue threads in the same swizzled K-major layout,
// followed by fence.proxy.async before the MMA that reads them.  Thread 0
// issues every MMA; completion is tracked by tcgen05.commit on an mbarrier.
// Every wait is bounded; a timeout sets the error word, every thread leaves
// the tile loop together (__syncthreads_and), in-flight copies and MMAs are
// drained (bounded) and the tensor memory is released.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <string.h>

#include "aco_mlp.h"
#include "aco_tc.cuh"

namespace aco {

namespace {

using tc::fence_after_sync;
using tc::fence_before_sync;
using tc::idesc_bf16;
using tc::idesc_bf16_major;
using tc::smem_desc_sw128;
using tc::smem_desc_sw128_mn;
using tc::sw128_offset;
using tc::tma_load_2d;
using tc::umma_bf16;
using tc::umma_commit;
using tc::wait_bounded;

constexpr int kThreadsF = 512;
constexpr uint32_t kKT = 128 * 128;  // one 128-row K-tile of BF16 (16 KB)
// Shared-memory map (offsets from a 1024-byte aligned base).
constexpr uint32_t oX = 0;             // X tile [128 e][64] (features 16..63 zero)
constexpr uint32_t oW1 = 16 * 1024;    // W1 [128 o][64] (inputs 16..63 zero)
constexpr uint32_t oW2 = 32 * 1024;    // W2 [128 o][128 i], two K-tiles
constexpr uint32_t oA = 64 * 1024;     // H1 [e][i], two K-tiles
constexpr uint32_t oV = 96 * 1024;     // vectors, partial sums, barriers (10 KB)
constexpr uint32_t oX1 = 106 * 1024;   // second X tile buffer            (training)
constexpr uint32_t oC = 122 * 1024;    // dZ2 [e][o] -> dZ1 [e][o]        (training)
constexpr uint32_t oH2 = 154 * 1024;   // H2 [e][o]                       (training)
constexpr uint32_t oM2 = 186 * 1024;   // [H2 > 0] [e][o] as BF16 0 / 1   (training)
constexpr uint32_t oDZ = 218 * 1024;   // dz hi/lo as rows 0/1 of [16][e] (training)
constexpr uint32_t kEndTrain = 222 * 1024, kEndFwd = 106 * 1024;
constexpr uint32_t kColW3 = 320, kColB2 = 352;  // TMEM columns of the two sums

template <bool TRAIN>
constexpr size_t fused_smem() {
  return (TRAIN ? kEndTrain : kEndFwd) + 1024;
}

__device__ __forceinline__ uint32_t bf2_bits(float lo, float hi) {
  const __nv_bfloat162 b = __floats2bfloat162_rn(lo, hi);
  uint32_t u;
  memcpy(&u, &b, 4);
  return u;
}

// Column sums over the warp's 32 rows: lane l returns the sum of a[l] over
// the lanes (reduce-scatter, 31 shuffles; fixed order).  Destroys a.
__device__ __forceinline__ float colsum32(float (&a)[32], int lane) {
#pragma unroll
  for (int s = 16; s >= 1; s >>= 1) {
    const bool up = (lane & s) != 0;
#pragma unroll
    for (int k = 0; k < s; k++) {
      const float send = up ? a[k] : a[k + s];
      const float keep = up ? a[k + s] : a[k];
      a[k] = keep + __shfl_xor_sync(kFull, send, s);
    }
  }
  return a[0];
}

// 32 BF16 values (packed pairs) as row `r` of a K-major operand, columns
// c0..c0+31 (c0 a multiple of 32): four 16-byte stores.
__device__ __forceinline__ void store_row32(unsigned char *op, int r, int c0,
                                            const uint32_t (&pk)[16]) {
  unsigned char *t = op + (c0 >> 6) * kKT;
#pragma unroll
  for (int u = 0; u < 4; u++)
    *reinterpret_cast<uint4 *>(t + sw128_offset(r, (c0 & 63) + 8 * u)) =
        make_uint4(pk[4 * u], pk[4 * u + 1], pk[4 * u + 2], pk[4 * u + 3]);
}


// MMAs of a 128 x N product with K = 128 (two K-tiles): A K-tiles kKT
// apart, B K-tiles b_step apart.
__device__ __forceinline__ void mma_k128(uint32_t d, const unsigned char *a, const unsigned char *b,
                                         uint32_t b_step, uint32_t idesc, bool accumulate) {
#pragma unroll
  for (int kt = 0; kt < 2; kt++) {
    const uint64_t da = smem_desc_sw128(a + kt * kKT), db = smem_desc_sw128(b + kt * b_step);
#pragma unroll
    for (int j = 0; j < 4; j++)
      umma_bf16(d, da + 2 * j, db + 2 * j, idesc, (accumulate || kt || j) ? 1u : 0u);
  }
}

__device__ __forceinline__ void st16(unsigned char *p, uint32_t v) {
  *reinterpret_cast<unsigned short *>(p) = (unsigned short)v;
}

// Column sums over the tile's rows on the tensor cores: D[o][n] +=
// sum_e A[e][o] B[n][e] with A a row-major activation tile read MN-major and
// B the 16-row K-major dz tile (two 2 KB K-tiles).
__device__ __forceinline__ void mma_sums(uint32_t d, const unsigned char *a,
                                         const unsigned char *bt, bool accumulate) {
  const uint32_t idesc = idesc_bf16_major(16, true, false);
#pragma unroll
  for (int j = 0; j < 8; j++) {
    const uint64_t da = smem_desc_sw128_mn(a + j * 2048, kKT);
    const uint64_t db = smem_desc_sw128(bt + (j >> 2) * 2048) + 2 * (j & 3);
    umma_bf16(d, da, db, idesc, (accumulate || j) ? 1u : 0u);
  }
}

// MMAs of a product with K = 128 running over the rows of row-major tiles:
// A and/or B read MN-major (start advanced 16 rows = 2048 bytes a step,
// M/N atoms the 16 KB K-tiles of the tile set), or A K-major (two K-tiles,
// 32 bytes a step inside a K-tile).
__device__ __forceinline__ void mma_rows(uint32_t d, const unsigned char *a, bool a_mn,
                                         const unsigned char *b, int n, bool accumulate) {
  const uint32_t idesc = idesc_bf16_major(n, a_mn, true);
#pragma unroll
  for (int j = 0; j < 8; j++) {
    const uint64_t da = a_mn ? smem_desc_sw128_mn(a + j * 2048, kKT)
                             : smem_desc_sw128(a + (j >> 2) * kKT) + 2 * (j & 3);
    const uint64_t db = smem_desc_sw128_mn(b + j * 2048, kKT);
    umma_bf16(d, da, db, idesc, (accumulate || j) ? 1u : 0u);
  }
}

}  // namespace

template <bool TRAIN>
__global__ void __launch_bounds__(kThreadsF, 1)
    k_mlp_fused(const __grid_constant__ CUtensorMap tmX, const __grid_constant__ CUtensorMap tmW1,
                const __grid_constant__ CUtensorMap tmW2,
                const float *__restrict__ w, const float *__restrict__ labels, int rows,
                float pos_weight, float norm, float *__restrict__ out, float *__restrict__ part,
                int part_ld, uint32_t *err) {
  extern __shared__ __align__(1024) unsigned char smem_f[];
  unsigned char *base = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(smem_f) + 1023) & ~uintptr_t(1023));
  unsigned char *sX0 = base + oX, *sW1 = base + oW1, *sW2 = base + oW2, *sA = base + oA;
  unsigned char *sX1 = base + oX1, *sC = base + oC;
  unsigned char *sH2 = base + oH2, *sM2 = base + oM2, *sDZ = base + oDZ;
  float *b1s = reinterpret_cast<float *>(base + oV);
  float *b2s = b1s + 128, *w3s = b2s + 128;
  float *zpart = w3s + 128;    // [4 column blocks][128 rows]
  float *colsum = zpart + 512;  // [4 lane quadrants][128 columns] (b1 gradient)
  float *red = colsum + 1536;   // [8]
  uint64_t *bar_x = reinterpret_cast<uint64_t *>(red + 8);
  uint64_t *bar_w = bar_x + 1, *bar_mma = bar_x + 2, *bar_drain = bar_x + 3;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bar_x + 4);

  constexpr uint32_t kCols = TRAIN ? 512 : 128;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int q = warp & 3, cb = warp >> 2;  // lane quadrant, column block
  const int row = q * 32 + lane;           // this thread's row of the tile
  const int c0 = cb * 32;                  // this thread's first column
  const int tiles = (rows + 127) >> 7;

  if (warp == 0) tc::tmem_alloc(tmem_slot, kCols);
  if (threadIdx.x == 0) {
    mbar_init(bar_x, 1);
    mbar_init(bar_w, 1);
    mbar_init(bar_mma, 1);
    mbar_init(bar_drain, 1);
    fence_barrier_init();
  }
  if (TRAIN && threadIdx.x < 256) {  // dz tile: rows 2..15 stay zero
    reinterpret_cast<uint4 *>(sDZ)[threadIdx.x] = make_uint4(0u, 0u, 0u, 0u);
    fence_proxy_async();
  }
  if (threadIdx.x < 128) {
    b1s[threadIdx.x] = w[kParamB1 + threadIdx.x];
    b2s[threadIdx.x] = w[kParamB2 + threadIdx.x];
    w3s[threadIdx.x] = w[kParamW3 + threadIdx.x];
  }
  const float b3 = w[kParamB3];
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = *tmem_slot;
  const uint32_t tl = tmem + ((uint32_t)(q * 32) << 16);  // this warp's lane quadrant

  int tile = blockIdx.x;
  bool x_inflight = false;  // thread 0: a TMA load of X not yet waited for
  if (threadIdx.x == 0 && tile < tiles) {
    mbar_arrive_expect_tx(bar_w, 3u * kKT);
    tma_load_2d(sW1, &tmW1, 0, 0, bar_w);
    tma_load_2d(sW2, &tmW2, 0, 0, bar_w);
    tma_load_2d(sW2 + kKT, &tmW2, 64, 0, bar_w);
    mbar_arrive_expect_tx(bar_x, kKT);
    tma_load_2d(sX0, &tmX, 0, tile * 128, bar_x);
    x_inflight = true;
  }

  uint32_t ph_x = 0, ph_m = 0;
  bool w_ready = false, failed = false;
  float gb1a = 0.0f, lossa = 0.0f, gb3a = 0.0f;
  for (int it = 0; tile < tiles; tile += gridDim.x, it++) {
    // Training double-buffers the X tile: dW1 of this tile reads it after
    // the next tile's copy has been started.
    unsigned char *sX = (TRAIN && (it & 1)) ? sX1 : sX0;
    unsigned char *sXn = (TRAIN && !(it & 1)) ? sX1 : sX0;
    const int grow = tile * 128 + row;
    // The label is first needed after the head; its load is in flight
    // through the first two products.
    const float yv = (TRAIN && grow < rows) ? __ldg(labels + grow) : -1.0f;
    // ---- Z1 = X W1^T (covers the previous tile's dW1 as well)
    bool ok = wait_bounded(bar_x, ph_x, err);
    ph_x ^= 1u;
    if (threadIdx.x == 0) {
      x_inflight = !ok;
      if (ok && !w_ready) ok = w_ready = wait_bounded(bar_w, 0, err);
      if (ok) {
        fence_after_sync();
        umma_bf16(tmem, smem_desc_sw128(sX), smem_desc_sw128(sW1), idesc_bf16(128), 0u);
        umma_commit(bar_mma);
      }
    }
    if (!__syncthreads_and(ok)) {
      failed = true;
      break;
    }
    ok = wait_bounded(bar_mma, ph_m, err);
    ph_m ^= 1u;
    fence_after_sync();
    // ---- H1 = bf16(relu(Z1 + b1)): row-major (A of Z2), transposed (B of dW2)
    uint32_t m1 = 0;  // [H1 > 0] of this thread's 32 columns
    {
      float v[32];
      tc::tmem_load_32(tl + (uint32_t)c0, v);
      uint32_t pk[16];
#pragma unroll
      for (int i = 0; i < 16; i++) {
        const uint32_t u = bf2_bits(fmaxf(v[2 * i] + b1s[c0 + 2 * i], 0.0f),
                                    fmaxf(v[2 * i + 1] + b1s[c0 + 2 * i + 1], 0.0f));
        pk[i] = u;
        m1 |= ((u & 0x7FFFu) ? 1u : 0u) << (2 * i);
        m1 |= ((u & 0x7FFF0000u) ? 1u : 0u) << (2 * i + 1);
      }
      store_row32(sA, row, c0, pk);
    }
    fence_proxy_async();
    fence_before_sync();
    if (!__syncthreads_and(ok)) {
      failed = true;
      break;
    }
    // ---- Z2 = H1 W2^T; then prefetch the next X tile (into the other
    // buffer when training: this one is read again by dW1)
    if (threadIdx.x == 0) {
      fence_after_sync();
      mma_k128(tmem, sA, sW2, kKT, idesc_bf16(128), false);
      umma_commit(bar_mma);
      if (tile + (int)gridDim.x < tiles) {
        fence_proxy_async();
        mbar_arrive_expect_tx(bar_x, kKT);
        tma_load_2d(sXn, &tmX, 0, (tile + gridDim.x) * 128, bar_x);
        x_inflight = true;
      }
    }
    ok = wait_bounded(bar_mma, ph_m, err);
    ph_m ^= 1u;
    fence_after_sync();
    // ---- H2 = bf16(relu(Z2 + b2)); z = H2 . w3 + b3
    float h[32];
    uint32_t m2 = 0;
    {
      float v[32];
      tc::tmem_load_32(tl + (uint32_t)c0, v);
      float zp = 0.0f;
#pragma unroll
      for (int i = 0; i < 32; i++) {
        h[i] = __bfloat162float(__float2bfloat16_rn(fmaxf(v[i] + b2s[c0 + i], 0.0f)));
        m2 |= (h[i] > 0.0f ? 1u : 0u) << i;
        zp = fmaf(h[i], w3s[c0 + i], zp);
      }
      zpart[cb * 128 + row] = zp;
      if (TRAIN) {  // H2 and its mask, row-major (A of the two column sums)
        uint32_t ph[16], pm[16];
#pragma unroll
        for (int i = 0; i < 16; i++) {
          ph[i] = bf2_bits(h[2 * i], h[2 * i + 1]);  // exact: h is BF16 already
          pm[i] = (((m2 >> (2 * i)) & 1u) ? 0x3F80u : 0u) |
                  (((m2 >> (2 * i + 1)) & 1u) ? 0x3F800000u : 0u);
        }
        store_row32(sH2, row, c0, ph);
        store_row32(sM2, row, c0, pm);
      }
    }
    fence_before_sync();
    __syncthreads();
    const float z = (((zpart[row] + zpart[128 + row]) + zpart[256 + row]) + zpart[384 + row]) + b3;
    const float p = 1.0f / (1.0f + __expf(-z));
    if (!TRAIN) {
      if (cb == 0 && grow < rows) out[grow] = p;
      if (!__syncthreads_and(ok)) {
        failed = true;
        break;
      }
      continue;
    }
    // ---- loss, dz; w3 and b3 gradients; dZ2 (A of dH1 K-major, of dW2 MN-major)
    float dz = 0.0f;
    if (yv >= 0.0f) {  // rows past the set and padding rows (label -1) add nothing
      const float wt = yv > 0.5f ? pos_weight : 1.0f;
      dz = wt * (p - yv) / norm;
      if (cb == 0) {
        lossa += wt * (fmaxf(z, 0.0f) - z * yv + log1pf(__expf(-fabsf(z)))) / norm;
        gb3a += dz;
      }
    }
    if (cb == 0) {  // dz ~ hi + lo to 16 significant bits, for the two sums
      const __nv_bfloat16 hi = __float2bfloat16_rn(dz);
      const __nv_bfloat16 lo = __float2bfloat16_rn(dz - __bfloat162float(hi));
      unsigned short hb, lb;
      memcpy(&hb, &hi, 2);
      memcpy(&lb, &lo, 2);
      unsigned char *t = sDZ + (row >> 6) * 2048;
      st16(t + sw128_offset(0, row & 63), hb);
      st16(t + sw128_offset(1, row & 63), lb);
    }
    {
      uint32_t pk[16];
#pragma unroll
      for (int i = 0; i < 16; i++)
        pk[i] = bf2_bits(((m2 >> (2 * i)) & 1u) ? dz * w3s[c0 + 2 * i] : 0.0f,
                         ((m2 >> (2 * i + 1)) & 1u) ? dz * w3s[c0 + 2 * i + 1] : 0.0f);
      store_row32(sC, row, c0, pk);
    }
    fence_proxy_async();
    fence_before_sync();
    if (!__syncthreads_and(ok)) {
      failed = true;
      break;
    }
    // ---- dH1 = dZ2 W2 (W2 read MN-major); dW2 += dZ2^T H1 (both MN-major)
    if (threadIdx.x == 0) {
      fence_after_sync();
      mma_rows(tmem, sC, false, sW2, 128, false);
      mma_rows(tmem + 128, sC, true, sA, 128, it > 0);
      mma_sums(tmem + kColW3, sH2, sDZ, it > 0);
      mma_sums(tmem + kColB2, sM2, sDZ, it > 0);
      umma_commit(bar_mma);
    }
    ok = wait_bounded(bar_mma, ph_m, err);
    ph_m ^= 1u;
    fence_after_sync();
    // ---- dZ1 = dH1 [H1 > 0] -> row-major (MN-major A of dW1); b1 gradient
    {
      float v[32];
      tc::tmem_load_32(tl + (uint32_t)c0, v);
      uint32_t pk[16];
#pragma unroll
      for (int i = 0; i < 32; i++) v[i] = ((m1 >> i) & 1u) ? v[i] : 0.0f;
#pragma unroll
      for (int i = 0; i < 16; i++) pk[i] = bf2_bits(v[2 * i], v[2 * i + 1]);
      store_row32(sC, row, c0, pk);
      gb1a += colsum32(v, lane);
    }
    fence_proxy_async();
    fence_before_sync();
    if (!__syncthreads_and(ok)) {
      failed = true;
      break;
    }
    // ---- dW1 += dZ1^T X (committed with the next tile's Z1, or the drain)
    if (threadIdx.x == 0) {
      fence_after_sync();
      mma_rows(tmem + 256, sC, true, sX, 16, it > 0);
    }
  }

  // Drain: every MMA issued so far, and a prefetch never waited for.
  if (threadIdx.x == 0) {
    umma_commit(bar_drain);
    if (x_inflight) wait_bounded(bar_x, ph_x, err);
  }
  const bool drained = wait_bounded(bar_drain, 0, err);
  fence_after_sync();
  const bool good = __syncthreads_and(drained && !failed);
  if (TRAIN && good && (int)blockIdx.x < tiles) {
    float *pr = part + (size_t)blockIdx.x * part_ld;
    {
      float v[32];  // dW2 rows o = row, columns i = c0..c0+31
      tc::tmem_load_32(tl + 128u + (uint32_t)c0, v);
      float4 *dst = reinterpret_cast<float4 *>(pr + kParamW2 + row * kHidden + c0);
#pragma unroll
      for (int u = 0; u < 8; u++)
        dst[u] = make_float4(v[4 * u], v[4 * u + 1], v[4 * u + 2], v[4 * u + 3]);
    }
    if (cb == 0) {
      float v[32];  // dW1 row o = row, features 0..15 (12 real)
      tc::tmem_load_16(tl + 256u, v);
#pragma unroll
      for (int f = 0; f < kFeatures; f++) pr[kParamW1 + row * kFeatures + f] = v[f];
      tc::tmem_load_16(tl + kColW3, v);  // w3 gradient of hidden unit o = row: hi + lo
      pr[kParamW3 + row] = v[0] + v[1];
      tc::tmem_load_16(tl + kColB2, v);  // sum_e [H2 > 0] dz, times w3
      pr[kParamB2 + row] = w3s[row] * (v[0] + v[1]);
#pragma unroll
      for (int o = 16; o; o >>= 1) {
        lossa += __shfl_xor_sync(kFull, lossa, o);
        gb3a += __shfl_xor_sync(kFull, gb3a, o);
      }
      if (lane == 0) {
        red[q] = lossa;
        red[4 + q] = gb3a;
      }
    }
    colsum[q * 128 + c0 + lane] = gb1a;
    __syncthreads();
    if (threadIdx.x < 128) {
      const int t = threadIdx.x;
      pr[kParamB1 + t] = ((colsum[t] + colsum[128 + t]) + colsum[256 + t]) + colsum[384 + t];
    }
    if (threadIdx.x == 0) {
      pr[kParamB3] = ((red[4] + red[5]) + red[6]) + red[7];
      pr[kParamCount] = ((red[0] + red[1]) + red[2]) + red[3];
    }
  }
  fence_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, kCols);
}

// Sums the per-CTA partial rows (columns 0..kParamCount; the last is the
// loss) in CTA order and, with `adam`, applies the Adam step to the FP32
// masters and refreshes their BF16 copies: W1 into its 16-wide padded rows,
// W2 row-major and transposed.  `clear` zeroes the rows read (one row only).
__global__ void __launch_bounds__(256)
    k_mlp_reduce(float *__restrict__ part, int G, int ld, int clear, float *__restrict__ gout,
                 float *__restrict__ loss_out, int adam, float *__restrict__ w,
                 float *__restrict__ m1, float *__restrict__ m2, float lr, float b1, float b2,
                 float eps, float bc1, float bc2, __nv_bfloat16 *__restrict__ w1b,
                 __nv_bfloat16 *__restrict__ w2b, __nv_bfloat16 *__restrict__ w2tb) {
  __shared__ float sh[8][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int t = blockIdx.x * 32 + tx;
  const bool live = t < kParamCount || (t == kParamCount && loss_out);
  float s = 0.0f;
  if (live)
    for (int c = ty; c < G; c += 8) s += part[(size_t)c * ld + t];
  sh[ty][tx] = s;
  __syncthreads();
  if (ty != 0 || !live) return;
  s = sh[0][tx];
#pragma unroll
  for (int y = 1; y < 8; y++) s += sh[y][tx];
  if (clear) part[t] = 0.0f;
  if (t == kParamCount) {
    *loss_out = s;
    return;
  }
  if (gout) gout[t] = s;
  if (!adam) return;
  const float a = b1 * m1[t] + (1.0f - b1) * s;
  const float b = b2 * m2[t] + (1.0f - b2) * s * s;
  m1[t] = a;
  m2[t] = b;
  const float v = w[t] - lr * (a / bc1) / (sqrtf(b / bc2) + eps);
  w[t] = v;
  const __nv_bfloat16 vb = __float2bfloat16_rn(v);
  if (t < kParamB1) {
    w1b[(t / kFeatures) * kFeatPad + t % kFeatures] = vb;
  } else if (t >= kParamW2 && t < kParamB2) {
    const int o = (t - kParamW2) / kHidden, i = (t - kParamW2) % kHidden;
    w2b[o * kHidden + i] = vb;
    w2tb[i * kHidden + o] = vb;
  }
}

int mlp_fused_grid(int rows, int sms) {
  const int tiles = (rows + 127) / 128;
  return tiles < sms ? tiles : sms;
}

cudaError_t launch_mlp_fused(bool train, const __nv_bfloat16 *X, int rows,
                             const __nv_bfloat16 *w1b, const __nv_bfloat16 *w2b, const float *w,
                             const float *labels, float pos_weight, float norm, float *out,
                             float *part, int part_ld, int grid, uint32_t *err, cudaStream_t s) {
  if (rows < 1 || grid < 1 || grid > (rows + 127) / 128) return cudaErrorInvalidValue;
  if ((reinterpret_cast<uintptr_t>(X) | reinterpret_cast<uintptr_t>(w1b) |
       reinterpret_cast<uintptr_t>(w2b) | reinterpret_cast<uintptr_t>(part)) & 15)
    return cudaErrorInvalidValue;
  if (train && (part_ld & 3)) return cudaErrorInvalidValue;
  CUtensorMap tx, t1, t2;
  if (!tc::make_map_bf16(&tx, X, rows, kFeatPad, kFeatPad, 128) ||
      !tc::make_map_bf16(&t1, w1b, kHidden, kFeatPad, kFeatPad, 128) ||
      !tc::make_map_bf16(&t2, w2b, kHidden, kHidden, kHidden, 128))
    return cudaErrorInvalidValue;
  // Above the 48 KB default; the attribute is set once per device.
  static unsigned long long configured = 0;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev >= 64) return cudaErrorInvalidDevice;
  if (!((configured >> dev) & 1ull)) {
    cudaError_t e = cudaFuncSetAttribute(k_mlp_fused<true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)fused_smem<true>());
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_mlp_fused<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)fused_smem<false>());
    if (e != cudaSuccess) return e;
    configured |= 1ull << dev;
  }
  if (train)
    k_mlp_fused<true><<<grid, kThreadsF, fused_smem<true>(), s>>>(
        tx, t1, t2, w, labels, rows, pos_weight, norm, out, part, part_ld, err);
  else
    k_mlp_fused<false><<<grid, kThreadsF, fused_smem<false>(), s>>>(
        tx, t1, t2, w, labels, rows, pos_weight, norm, out, part, part_ld, err);
  return cudaGetLastError();
}

cudaError_t launch_mlp_reduce(float *part, int G, int ld, bool clear, float *gout, float *loss_out,
                              bool adam, float *w, float *m1, float *m2, float lr, float b1,
                              float b2, float eps, float bc1, float bc2, __nv_bfloat16 *w1b,
                              __nv_bfloat16 *w2b, __nv_bfloat16 *w2tb, cudaStream_t s) {
  if (G < 1 || (clear && G != 1)) return cudaErrorInvalidValue;
  const int blocks = (kParamCount + 1 + 31) / 32;
  k_mlp_reduce<<<blocks, 256, 0, s>>>(part, G, ld, clear ? 1 : 0, gout, loss_out, adam ? 1 : 0,
                                       w, m1, m2, lr, b1, b2, eps, bc1, bc2, w1b, w2b, w2tb);
  return cudaGetLastError();
}

}  // namespace aco
