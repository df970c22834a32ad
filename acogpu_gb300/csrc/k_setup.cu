// k_setup.cu -- one-time kernels of Colony::initialize (reference:
// src/Colony.cu:185-311, src/Setup.cpp:54-70): EUC_2D distances, the
// heuristic, nn-lists, the greedy tour for tau0, and state reset.
#include <cuda_runtime.h>

#include "aco_kernels.h"

namespace aco {

// ---------------------------------------------------------------- distances
// Utils::round_distance (src/Utils.cu:212-218): float differences, double
// root, +0.5, truncation.  The reference defines the metric in double, so
// the one-time O(n^2) build runs in FP64 to reproduce it exactly.
__global__ void k_distances_from_coords(const float *__restrict__ x, const float *__restrict__ y,
                                        int n, int ld, int32_t *__restrict__ dist) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  if (j >= ld) return;
  int32_t d = ACO_MAX_DISTANCE;
  if (j < n && i != j) {
    const double dx = (double)__fsub_rn(x[i], x[j]);
    const double dy = (double)__fsub_rn(y[i], y[j]);
    const double r = __dadd_rn(__dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy))), 0.5);
    d = __double2int_rz(r);
  }
  dist[(size_t)i * ld + j] = d;
}

cudaError_t launch_distances_from_coords(const float *x, const float *y, int n, int ld,
                                         int32_t *dist, cudaStream_t s) {
  dim3 grid((ld + 127) / 128, n);
  k_distances_from_coords<<<grid, 128, 0, s>>>(x, y, n, ld, dist);
  return cudaGetLastError();
}

__global__ void k_fill_padding_int(int32_t *mat, int n, int ld, int32_t value) {
  const int pad = ld - n;
  const int64_t total = (int64_t)n * pad;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / pad, j = n + t % pad;
    mat[i * ld + j] = value;
  }
}

cudaError_t launch_fill_padding_int(int32_t *mat, int n, int ld, int32_t value, cudaStream_t s) {
  if (ld == n) return cudaSuccess;
  k_fill_padding_int<<<304, 256, 0, s>>>(mat, n, ld, value);
  return cudaGetLastError();
}

__global__ void k_max_distance(const int32_t *__restrict__ dist, int n, int ld, int32_t *out) {
  int32_t best = 0;
  const int64_t total = (int64_t)n * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / n, j = t % n;
    if (i != j) best = max(best, dist[i * ld + j]);
  }
  for (int o = 16; o; o >>= 1) best = max(best, __shfl_xor_sync(kFull, best, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, best);
}

cudaError_t launch_max_distance(const int32_t *dist, int n, int ld, int32_t *out, cudaStream_t s) {
  k_max_distance<<<304, 256, 0, s>>>(dist, n, ld, out);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- heuristic
// x^b for integer b >= 1 in double-float arithmetic (exact products by FMA),
// then rounded once: the correctly rounded power except within ~b*2^-46 of a
// rounding midpoint.
__device__ __forceinline__ float pow_int_cr(float x, int b) {
  if (b == 0) return 1.0f;
  if (isinf(x) || x == 0.0f) return isinf(x) ? x : 0.0f;
  float hi = x, lo = 0.0f;
  for (int i = 1; i < b; i++) {
    const float p = __fmul_rn(hi, x);
    float e = __fmaf_rn(hi, x, -p);
    e = __fmaf_rn(lo, x, e);
    const float s = __fadd_rn(p, e);
    lo = __fsub_rn(e, __fsub_rn(s, p));
    hi = s;
  }
  return hi;
}

// HURESTIC(d, beta) (inc/Colony.h:17-21) evaluated on the GPU.
__global__ void k_heuristic_device(const int32_t *__restrict__ dist, int n, int ld, float beta,
                                   float *__restrict__ eta) {
  const int64_t total = (int64_t)n * ld;
  const bool int_beta = beta == floorf(beta) && beta >= 0.0f && beta <= 64.0f;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(t % ld);
    const int32_t d = dist[t];
    float e = 0.0f;
    if (j < n && d != ACO_MAX_DISTANCE) {
      const float x = __frcp_rn(__int2float_rn(d));
      e = int_beta ? pow_int_cr(x, (int)beta) : powf(x, beta);
    }
    eta[t] = e;
  }
}

cudaError_t launch_heuristic_device(const int32_t *dist, int n, int ld, float beta, float *eta,
                                    cudaStream_t s) {
  k_heuristic_device<<<608, 256, 0, s>>>(dist, n, ld, beta, eta);
  return cudaGetLastError();
}

// Expansion of a per-distance table (table[d] = eta of distance d).
__global__ void k_heuristic_table(const int32_t *__restrict__ dist, int n, int ld,
                                  const float *__restrict__ table, int32_t table_len,
                                  float *__restrict__ eta, ColonyState *st) {
  const int64_t total = (int64_t)n * ld;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(t % ld);
    const int32_t d = dist[t];
    float e = 0.0f;
    if (j < n && d != ACO_MAX_DISTANCE) {
      if (d >= 0 && d < table_len) {
        e = table[d];
      } else {
        atomicOr(&st->error, kErrCheck);
      }
    }
    eta[t] = e;
  }
}

cudaError_t launch_heuristic_table(const int32_t *dist, int n, int ld, const float *table,
                                   int32_t table_len, float *eta, ColonyState *st,
                                   cudaStream_t s) {
  k_heuristic_table<<<608, 256, 0, s>>>(dist, n, ld, table, table_len, eta, st);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- nn lists
// Stable nn order: each CTA sorts one row of 64-bit keys (distance << 32 |
// city) with a bitonic network in shared memory.  The row is staged into
// shared memory by a TMA bulk copy.  Equal distances keep city order, which
// is the rank-by-counting order of the reference GPU kernel
// (inc/Colony.cuh:101-123).
constexpr int kSortThreads = 1024;
constexpr int kMaxSortRow = 16384;
constexpr int kSortPerThread = kMaxSortRow / kSortThreads;

__global__ void __launch_bounds__(kSortThreads)
    k_nn_sort_stable(const int32_t *__restrict__ dist, int n, int ld, int K, int ldk,
                     int32_t *__restrict__ nn, int32_t *__restrict__ nn2, int t2, int P,
                     ColonyState *st) {
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t *keys = reinterpret_cast<uint64_t *>(smem);
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem + (size_t)P * 8);
  int *flag = reinterpret_cast<int *>(bar + 1);
  const int row = blockIdx.x, tid = threadIdx.x;
  int32_t *drow = reinterpret_cast<int32_t *>(keys);
  if (tid == 0) {
    mbar_init(bar, 1);
    fence_barrier_init();
  }
  __syncthreads();
  if (tid == 0) {
    const uint32_t bytes = (uint32_t)ld * 4u;
    mbar_arrive_expect_tx(bar, bytes);
    tma_load_1d(drow, dist + (size_t)row * ld, bytes, bar);
    *flag = mbar_wait_bounded(bar, 0, st) ? 1 : 0;
  }
  __syncthreads();
  if (!*flag) return;
  uint64_t v[kSortPerThread];
#pragma unroll
  for (int q = 0; q < kSortPerThread; q++) {
    const int i = tid + q * kSortThreads;
    v[q] = ~0ull;
    if (i < n) v[q] = ((uint64_t)(uint32_t)drow[i] << 32) | (uint32_t)i;
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < kSortPerThread; q++) {
    const int i = tid + q * kSortThreads;
    if (i < P) keys[i] = v[q];
  }
  __syncthreads();
  for (int k = 2; k <= P; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = tid; i < P; i += kSortThreads) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const uint64_t a = keys[i], b = keys[ixj];
          const bool up = (i & k) == 0;
          if ((a > b) == up) {
            keys[i] = b;
            keys[ixj] = a;
          }
        }
      }
      __syncthreads();
    }
  }
  for (int q = tid; q < ldk; q += kSortThreads)
    nn[(size_t)row * ldk + q] = q < K ? (int32_t)(uint32_t)(keys[q] & 0xffffffffu) : -1;
  if (nn2)  // the fallback's second tier: neighbours K .. K + t2 - 1
    for (int q = tid; q < kTier2; q += kSortThreads)
      nn2[(size_t)row * kTier2 + q] =
          q < t2 ? (int32_t)(uint32_t)(keys[K + q] & 0xffffffffu) : -1;
}

cudaError_t launch_nn_sort_stable(const int32_t *dist, int n, int ld, int K, int ldk, int32_t *nn,
                                  ColonyState *st, cudaStream_t s, int32_t *nn2, int t2) {
  if (nn2 && (t2 < 0 || t2 > kTier2 || K + t2 > n - 1)) return cudaErrorInvalidValue;
  if (n > kMaxSortRow) return cudaErrorInvalidValue;
  int P = 1;
  while (P < n) P <<= 1;
  if (P < 32) P = 32;
  const size_t smem = (size_t)P * 8 + 16;
  cudaError_t e = cudaFuncSetAttribute(k_nn_sort_stable,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_nn_sort_stable<<<n, kSortThreads, smem, s>>>(dist, n, ld, K, ldk, nn, nn2, t2, P, st);
  return cudaGetLastError();
}

// Reference CPU order: the permutation Utils::sort2 (src/Utils.cu:136-159)
// produces, ties included.  One thread per row runs the same quicksort
// (middle pivot, pivot kept in the left part) with an explicit stack; the
// smaller part is processed first, so the stack depth stays below 2*log2(n).
// The subranges are disjoint, so the order in which they are processed does
// not change the result.
constexpr int kQsortStack = 96;

__global__ void k_nn_ref_qsort(const int32_t *__restrict__ dist, int n, int ld,
                               int32_t *__restrict__ scratch, int32_t *__restrict__ nn, int ldk,
                               ColonyState *st) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= n) return;
  int32_t *v = scratch + (size_t)row * ld;
  int32_t *v2 = nn + (size_t)row * ldk;
  for (int i = 0; i < n; i++) {
    v[i] = dist[(size_t)row * ld + i];
    v2[i] = i;
  }
  int stack[kQsortStack];
  int sp = 0, left = 0, right = n - 1;
  for (;;) {
    if (left < right) {
      const int mid = (left + right) / 2;
      int t = v[left]; v[left] = v[mid]; v[mid] = t;
      t = v2[left]; v2[left] = v2[mid]; v2[mid] = t;
      int last = left;
      const int pivot = v[left];
      for (int k = left + 1; k <= right; k++) {
        const int vk = v[k];
        if (vk < pivot) {
          ++last;
          t = v[last]; v[last] = vk; v[k] = t;
          t = v2[last]; v2[last] = v2[k]; v2[k] = t;
        }
      }
      t = v[left]; v[left] = v[last]; v[last] = t;
      t = v2[left]; v2[left] = v2[last]; v2[last] = t;
      // parts [left, last] and [last+1, right]
      int al = left, ar = last, bl = last + 1, br = right;
      if (ar - al > br - bl) {
        int tl = al, tr = ar;
        al = bl; ar = br; bl = tl; br = tr;
      }
      // (al, ar) is the smaller part: continue with it, push the larger.
      if (sp + 2 > kQsortStack) {
        atomicOr(&st->error, kErrCheck);
        return;
      }
      stack[sp++] = bl;
      stack[sp++] = br;
      left = al;
      right = ar;
    } else {
      if (sp == 0) break;
      right = stack[--sp];
      left = stack[--sp];
    }
  }
}

cudaError_t launch_nn_ref_qsort(const int32_t *dist, int n, int ld, int32_t *scratch, int32_t *nn,
                                int ldk, ColonyState *st, cudaStream_t s) {
  k_nn_ref_qsort<<<(n + 63) / 64, 64, 0, s>>>(dist, n, ld, scratch, nn, ldk, st);
  return cudaGetLastError();
}

// The same quicksort with the row in shared memory: one warp per row, the
// warp copies the row's distances in (coalesced) and its sorted ids out,
// lane 0 runs the sort (the partition is sequential by definition: its swaps
// fix the order of ties).  Distances and ids sit interleaved, one 8-byte
// pair per entry, so a swap is one 8-byte load and store each way.  A
// shared-memory access costs about a tenth of the scattered L2 accesses of
// the global version (one thread per row, rows ld apart).
__global__ void k_nn_ref_qsort_smem(const int32_t *__restrict__ dist, int n, int ld,
                                    int32_t *__restrict__ nn, int ldk, ColonyState *st) {
  extern __shared__ __align__(16) int2 qs_rows[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int row = blockIdx.x * (blockDim.x >> 5) + warp;
  if (row >= n) return;  // warp-uniform
  int2 *v = qs_rows + (size_t)warp * n;
  for (int i = lane; i < n; i += 32) v[i] = make_int2(dist[(size_t)row * ld + i], i);
  __syncwarp();
  if (lane == 0) {
    int stack[kQsortStack];
    int sp = 0, left = 0, right = n - 1;
    bool ok = true;
    for (;;) {
      if (left < right) {
        const int mid = (left + right) / 2;
        int2 t = v[left];
        v[left] = v[mid];
        v[mid] = t;
        int last = left;
        const int pivot = v[left].x;
        for (int k = left + 1; k <= right; k++) {
          const int2 vk = v[k];
          if (vk.x < pivot) {
            ++last;
            v[k] = v[last];
            v[last] = vk;
          }
        }
        t = v[left];
        v[left] = v[last];
        v[last] = t;
        int al = left, ar = last, bl = last + 1, br = right;
        if (ar - al > br - bl) {
          const int tl = al, tr = ar;
          al = bl;
          ar = br;
          bl = tl;
          br = tr;
        }
        if (sp + 2 > kQsortStack) {
          ok = false;
          break;
        }
        stack[sp++] = bl;
        stack[sp++] = br;
        left = al;
        right = ar;
      } else {
        if (sp == 0) break;
        right = stack[--sp];
        left = stack[--sp];
      }
    }
    if (!ok) atomicOr(&st->error, kErrCheck);
  }
  __syncwarp();
  for (int i = lane; i < n; i += 32) nn[(size_t)row * ldk + i] = v[i].y;
}

int nn_ref_qsort_smem_rows(int n, int max_smem) {
  const int per_row = n * 8;
  int rows = per_row > 0 ? (max_smem - 1024) / per_row : 0;
  return rows > 8 ? 8 : rows;
}

cudaError_t launch_nn_ref_qsort_smem(const int32_t *dist, int n, int ld, int32_t *nn, int ldk,
                                     ColonyState *st, int max_smem, cudaStream_t s) {
  const int rows = nn_ref_qsort_smem_rows(n, max_smem);
  if (rows < 1) return cudaErrorInvalidValue;
  const size_t smem = (size_t)rows * n * 8;
  cudaError_t e = cudaFuncSetAttribute(k_nn_ref_qsort_smem,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k_nn_ref_qsort_smem<<<(n + rows - 1) / rows, rows * 32, smem, s>>>(dist, n, ld, nn, ldk, st);
  return cudaGetLastError();
}

__global__ void k_gather_nn_f32(const float *__restrict__ src, int n, int ld,
                                const int32_t *__restrict__ nn, int K, int ldk,
                                float *__restrict__ dst) {
  const int64_t total = (int64_t)n * ldk;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = t / ldk;
    const int r = (int)(t % ldk);
    dst[t] = r < K ? src[j * ld + nn[t]] : 0.0f;
  }
}

cudaError_t launch_gather_nn_f32(const float *src, int n, int ld, const int32_t *nn, int K, int ldk,
                                 float *dst, cudaStream_t s) {
  k_gather_nn_f32<<<608, 256, 0, s>>>(src, n, ld, nn, K, ldk, dst);
  return cudaGetLastError();
}

// int16 copy of the candidate rows (same pitch; entries past the K
// candidates of a row are -1).  The staged kernel keeps the k <= 32 table in
// shared memory; the long-row kernel copies one row at a time by TMA.
__global__ void k_nn_to_i16(const int32_t *__restrict__ nn, int n, int K, int ldk,
                            int16_t *__restrict__ nn16) {
  const int64_t total = (int64_t)n * ldk;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x)
    nn16[t] = (int)(t % ldk) < K ? (int16_t)nn[t] : (int16_t)-1;
}

cudaError_t launch_nn_to_i16(const int32_t *nn, int n, int K, int ldk, int16_t *nn16,
                             cudaStream_t s) {
  k_nn_to_i16<<<304, 256, 0, s>>>(nn, n, K, ldk, nn16);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- tau0
// Greedy nearest-neighbour tour from city 0 (lowest index on ties); then tau0
// by the requested rule.  The reference's greedyDistance is a stub returning
// 0 (src/Colony.cu:1053-1055) and its tau0 is the constant 1e-6
// (src/AntSystem.cu:200-203).  One CTA of kGreedyThreads: each step reads the
// current row once (coalesced, n / kGreedyThreads cities per thread) and takes
// the block-wide minimum of (distance << 32 | city) over unvisited cities, so
// a step costs one L2 round trip and two barriers.
constexpr int kGreedyThreads = 1024;

__global__ void __launch_bounds__(kGreedyThreads)
    k_greedy_tau0(ColonyDev c, int tau0_mode, float tau0_value) {
  extern __shared__ uint32_t tabu[];
  __shared__ unsigned long long red[kGreedyThreads / 32];
  __shared__ int s_next;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int words = (c.n + 31) >> 5;
  if (tau0_mode != ACO_TAU0_DORIGO) {
    if (tid == 0) {
      c.st->tau0 = tau0_mode == ACO_TAU0_REFERENCE ? (float)0.000001 : tau0_value;
      c.st->greedy_length = 0;
    }
    return;
  }
  for (int w = tid; w < words; w += kGreedyThreads) tabu[w] = w == 0 ? 1u : 0u;
  __syncthreads();
  int cur = 0;
  int64_t len = 0;  // kept by thread 0
  for (int s = 1; s < c.n; s++) {
    const int32_t *row = c.dist + (size_t)cur * c.ld;
    unsigned long long best = ~0ull;
    for (int j = tid; j < c.n; j += kGreedyThreads) {
      if ((tabu[j >> 5] >> (j & 31)) & 1u) continue;
      const unsigned long long key =
          ((unsigned long long)(uint32_t)__ldcg(row + j) << 32) | (uint32_t)j;
      best = key < best ? key : best;
    }
    for (int o = 16; o; o >>= 1) {
      const unsigned long long other = __shfl_xor_sync(kFull, best, o);
      best = other < best ? other : best;
    }
    if (lane == 0) red[warp] = best;
    __syncthreads();
    if (warp == 0) {
      best = red[lane];
      for (int o = 16; o; o >>= 1) {
        const unsigned long long other = __shfl_xor_sync(kFull, best, o);
        best = other < best ? other : best;
      }
      if (lane == 0) {
        const int bj = (int)(uint32_t)best;
        if (best == ~0ull || bj >= c.n) {  // cannot happen with n >= 2; recorded
          atomicOr(&c.st->error, kErrCheck);
          s_next = 0;
        } else {
          tabu[bj >> 5] |= 1u << (bj & 31);
          len += (int64_t)(best >> 32);
          s_next = bj;
        }
      }
    }
    __syncthreads();
    cur = s_next;
  }
  if (tid == 0) {
    len += c.dist[(size_t)cur * c.ld + 0];
    const float cnn = __ll2float_rn(len);
    float t0;
    if (c.variant == ACO_RANK_BASED) {
      const float num = __fmul_rn(__fmul_rn(0.5f, (float)c.rank_w), (float)(c.rank_w - 1));
      t0 = __fdiv_rn(num, __fmul_rn(c.rho, cnn));
    } else {
      t0 = __fdiv_rn((float)c.m, cnn);
    }
    c.st->tau0 = t0;
    c.st->greedy_length = len;
  }
}

cudaError_t launch_greedy_tau0(const ColonyDev &c, int tau0_mode, float tau0_value,
                               cudaStream_t s) {
  const size_t smem = (size_t)((c.n + 31) / 32) * 4;
  k_greedy_tau0<<<1, kGreedyThreads, smem, s>>>(c, tau0_mode, tau0_value);
  return cudaGetLastError();
}

// Colony::initPheromone + initAntAges + initTourLengths and the best-so-far
// reset (src/Colony.cu:216-228, 315-351, 38-39).
__global__ void k_init_colony(ColonyDev c) {
  const float t0 = c.st->tau0;
  const int64_t total = (int64_t)c.n * c.ld;
  const int64_t gtid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t t = gtid; t < total; t += stride) c.tau[t] = t0;
  for (int64_t k = gtid; k < c.m; k += stride) {
    c.age[k] = 0;
    c.perf[k] = 0;
    c.valid[k] = 1;
    c.len[k] = 0;
    c.newlen[k] = 0;
  }
  if (gtid == 0) {
    c.st->iter_best = (int64_t)ACO_MAX_DISTANCE - 1;
    c.st->glob_best = ACO_MAX_DISTANCE;
    c.st->iter_best_ant = -1;
    c.st->iteration = 0;
    c.st->num_valid = c.m;
    c.st->isconverged = 0;
    c.st->globalperformance = 0;
    c.st->dep_count = 0;
    c.st->fallbacks = 0;
    c.st->tours_built = 0;
  }
}

cudaError_t launch_init_colony(const ColonyDev &c, cudaStream_t s) {
  k_init_colony<<<608, 256, 0, s>>>(c);
  return cudaGetLastError();
}

}  // namespace aco
