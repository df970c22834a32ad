// k_construct.cu -- roulette-wheel tour construction, one warp per ant.
//
// Replaces Colony::initTour + constructPath (src/Colony.cu:469-527,
// 689-864) and the reference GPU kernels dev_place_ants /
// dev_compute_probabilities / dev_reduce_probabilities_s / dev_move_ants
// (inc/Colony.cuh:136-162,193-229,290-347; src/Colony.cu:643-685), which the
// reference launches 3(n-1) times per iteration with a device sync after
// each.  Here one launch builds every tour:
//
//  * the tabu list is a bitmask in shared memory (n bits per warp);
//  * step x of ant k reads the candidate row of the current city in
//    candidate order (ids + tau*eta, contiguous), masks visited cities and
//    forms the prefix sums of the weights in candidate order.  The prefix is
//    the sequential float sum of the reference (sum_prob += prob_ptr[i],
//    src/Colony.cu:814; partial_sum += ..., :840): the 32 weights of a chunk
//    are broadcast with __shfl_sync and added in lane order, so every
//    partial sum is bit-identical to the CPU's (adding the zero weight of a
//    visited city changes nothing, as in the reference);
//  * the crossing `first i with partial_sum > u * sum` is a ballot; rows
//    longer than 32 candidates keep the prefix at each chunk end in shared
//    memory and redo only the chunk that holds the crossing;
//  * when the roulette cannot pick (sum <= 0, or no crossing) the fallback is
//    a ballot over the row: the last unvisited city of the full nn row
//    (select_local_best, inc/Colony.cuh:33-43) or the unvisited city with the
//    largest choice value;
//  * ant aging (updateAntAges, src/Colony.cu:353-364; compute_fittness,
//    inc/Colony.cuh:14-31) is fused in; the integer tour length (the
//    reference adds it per move, inc/Colony.cuh:337-340) is summed by the
//    whole warp after the tour is built, so no step waits on a distance load;
//    the successor/predecessor of every city is written transposed for the
//    row-owned deposit.
//
// Staged variant (candidate lists of at most 32 and a table that fits in
// shared memory, e.g. n = 1000, k = 30: 192 KB): each CTA copies the whole
// candidate table -- int16 ids and FP32 choice values, 32 per city -- into
// shared memory with TMA bulk copies once per launch, so a construction step
// touches only shared memory.  One CTA per SM; its warps loop over ants.
#include <cuda_runtime.h>

#include "aco_kernels.h"

namespace aco {

__device__ __forceinline__ bool visited(const uint32_t *tabu, int city) {
  return (tabu[city >> 5] >> (city & 31)) & 1u;
}

// s + w[0] + w[1] + ... + w[31] in lane order (each addition rounded);
// p receives the prefix that includes this lane's weight.
__device__ __forceinline__ float fold32(float s, float w, int lane, float &p) {
  p = s;
#pragma unroll
  for (int b = 0; b < 32; b++) {
    const float v = __shfl_sync(kFull, w, b);
    s = __fadd_rn(s, v);
    p = (lane == b) ? s : p;
  }
  return s;
}

// compute_fittness with the aging blend (inc/Colony.cuh:21-30), every
// operation rounded once.
__device__ __forceinline__ float blend_fitness(float tau, float eta, float meanc, float ratio,
                                               int use_alpha, float alpha) {
  float p = __fadd_rn(__fmul_rn(__fsub_rn(tau, meanc), ratio), meanc);
  if (use_alpha) p = powf(p, alpha);
  return __fmul_rn(p, eta);
}

struct AntCtx {
  bool blend;
  float ratio, meanc;
};

// Candidate r of the row of `cur`: id (or -1) and its weight (0 if visited).
template <bool STAGED>
__device__ __forceinline__ void candidate(const ColonyDev &c, int cur, int r,
                                          const uint32_t *tabu, const int16_t *sids,
                                          const float *scw, const AntCtx &a, int &id, float &w) {
  id = -1;
  w = 0.0f;
  if (r >= c.K) return;
  if (!a.blend) {
    float cw;
    if (STAGED) {
      id = sids[cur * 32 + r];
      cw = scw[cur * 32 + r];
    } else {
      const size_t off = (size_t)cur * c.ldk + r;
      id = __ldg(c.nn + off);
      cw = c.choice_nn[off];
    }
    if (!visited(tabu, id)) w = cw;
  } else {
    const size_t off = (size_t)cur * c.ldk + r;
    id = STAGED ? (int)sids[cur * 32 + r] : __ldg(c.nn + off);
    const float t = c.tau_nn[off];
    const float e = __ldg(c.eta_nn + off);
    if (!visited(tabu, id)) w = blend_fitness(t, e, a.meanc, a.ratio, c.use_alpha, c.alpha);
  }
}

// Fallback choice at city `cur` (warp-uniform result, -1 if none).
__device__ int fallback_city(const ColonyDev &c, int cur, const uint32_t *tabu, const AntCtx &a,
                             int lane) {
  if (c.fallback == ACO_FALLBACK_REFERENCE) {
    // select_local_best: last unvisited city of the full nn row.
    const int32_t *ids = c.nn + (size_t)cur * c.ldk;
    for (int ch = ((c.K + 31) >> 5) - 1; ch >= 0; ch--) {
      const int r = ch * 32 + lane;
      const int id = r < c.K ? __ldg(ids + r) : -1;
      const unsigned m = __ballot_sync(kFull, id >= 0 && !visited(tabu, id));
      if (m) return __shfl_sync(kFull, id, 31 - __clz(m));
    }
    return -1;
  }
  // Largest choice value among unvisited cities, lowest index on ties.
  float bw = -1.0f;
  int bj = -1;
  const float *crow = c.choice + (size_t)cur * c.ld;
  const float *trow = c.tau + (size_t)cur * c.ld;
  const float *erow = c.eta + (size_t)cur * c.ld;
  for (int j = lane; j < c.n; j += 32) {
    if (visited(tabu, j)) continue;
    const float w = a.blend ? blend_fitness(trow[j], erow[j], a.meanc, a.ratio, c.use_alpha,
                                            c.alpha)
                            : crow[j];
    if (w > bw) {
      bw = w;
      bj = j;
    }
  }
  for (int o = 16; o; o >>= 1) {
    const float ow = __shfl_xor_sync(kFull, bw, o);
    const int oj = __shfl_xor_sync(kFull, bj, o);
    if (oj >= 0 && (bj < 0 || ow > bw || (ow == bw && oj < bj))) {
      bw = ow;
      bj = oj;
    }
  }
  return bj;
}

template <bool MULTI, bool AGING, bool STAGED>
__device__ void construct_ant(const ColonyDev &c, int k, uint32_t iter, uint32_t *tabu,
                              float *cend, const int16_t *sids, const float *scw,
                              const float *smean, int nchunks, int lane) {
  const int n = c.n;
  const int words = (n + 31) >> 5;
  int32_t *trow = c.tours + (size_t)k * c.ld;

  AntCtx a;
  a.blend = false;
  a.ratio = 0.0f;
  a.meanc = 0.0f;
  if (AGING) {
    int age = 0;
    if (lane == 0) {
      age = c.age[k] + 1;
      c.age[k] = age;
    }
    age = __shfl_sync(kFull, age, 0);
    if (!c.valid[k]) {  // invalid ants keep a cleared tour (src/Colony.cu:507-510)
      for (int i = lane; i < n; i += 32) trow[i] = 0;
      return;
    }
    a.blend = age < c.min_ret && c.st->isconverged;
    if (a.blend) a.ratio = __fdiv_rn(__int2float_rn(age), __int2float_rn(c.min_ret));
  }
  for (int w = lane; w < words; w += 32) tabu[w] = 0;
  __syncwarp();

  // initTour placement (src/Colony.cu:518-520)
  const float u0 = aco_uniform(c.seed, iter, (uint32_t)k, 0u);
  int start = __float2int_rz(__fmul_rn(u0, __int2float_rn(n)));
  if (start >= n) {  // impossible for u0 < 1; recorded, clamped
    if (lane == 0) atomicOr(&c.st->error, kErrCheck);
    start = n - 1;
  }
  if (lane == 0) {
    tabu[start >> 5] |= 1u << (start & 31);
    trow[0] = start;
  }
  __syncwarp();

  int cur = start;
  int64_t fallbacks = 0;
  for (int x = 1; x < n; x++) {
    const float u = aco_uniform(c.seed, iter, (uint32_t)k, (uint32_t)x);
    if (AGING && a.blend) a.meanc = STAGED ? smean[cur] : c.mean[cur];
    int next = -1;
    if (!MULTI) {
      int id;
      float w;
      candidate<STAGED>(c, cur, lane, tabu, sids, scw, a, id, w);
      float p;
      const float S = fold32(0.0f, w, lane, p);
      if (!(S <= 0.0f)) {
        const float rnd = __fmul_rn(u, S);
        const unsigned hit = __ballot_sync(kFull, lane < c.K && !(p <= rnd));
        if (hit) next = __shfl_sync(kFull, id, __ffs(hit) - 1);
      }
    } else {
      float s = 0.0f;
      for (int ch = 0; ch < nchunks; ch++) {
        int id;
        float w;
        candidate<false>(c, cur, ch * 32 + lane, tabu, sids, scw, a, id, w);
        if (__ballot_sync(kFull, w != 0.0f)) {
          float p;
          s = fold32(s, w, lane, p);
        }
        if (lane == 0) cend[ch] = s;
      }
      __syncwarp();
      const float S = s;
      if (!(S <= 0.0f)) {
        const float rnd = __fmul_rn(u, S);
        int found = -1;
        for (int base = 0; base < nchunks; base += 32) {
          const int q = base + lane;
          const unsigned m = __ballot_sync(kFull, q < nchunks && !(cend[q] <= rnd));
          if (m) {
            found = base + __ffs(m) - 1;
            break;
          }
        }
        if (found >= 0) {
          const float s0 = found > 0 ? cend[found - 1] : 0.0f;
          const int r = found * 32 + lane;
          int id;
          float w;
          candidate<false>(c, cur, r, tabu, sids, scw, a, id, w);
          float p;
          fold32(s0, w, lane, p);
          const unsigned hit = __ballot_sync(kFull, r < c.K && !(p <= rnd));
          if (hit) next = __shfl_sync(kFull, id, __ffs(hit) - 1);
        }
      }
      __syncwarp();
    }
    if (next < 0) {
      next = fallback_city(c, cur, tabu, a, lane);
      fallbacks++;
      if (next < 0 || next >= n) {  // no unvisited city: cannot happen
        if (lane == 0) atomicOr(&c.st->error, kErrCheck);
        break;
      }
    }
    if (lane == 0) {
      tabu[next >> 5] |= 1u << (next & 31);
      trow[x] = next;
      c.succT[(size_t)cur * c.ldm + k] = next;
      c.predT[(size_t)next * c.ldm + k] = cur;
    }
    __syncwarp();
    cur = next;
  }
  if (lane == 0) {
    c.succT[(size_t)cur * c.ldm + k] = start;
    c.predT[(size_t)start * c.ldm + k] = cur;
  }
  __syncwarp();
  // Integer tour length, summed by the whole warp (order-free).
  int64_t len = 0;
  for (int i = lane; i < n; i += 32) {
    const int a0 = trow[i];
    const int b0 = trow[i + 1 == n ? 0 : i + 1];
    len += c.dist[(size_t)a0 * c.ld + b0];
  }
  for (int o = 16; o; o >>= 1) len += __shfl_xor_sync(kFull, len, o);
  if (lane == 0) {
    c.newlen[k] = len;
    if (fallbacks)
      atomicAdd(reinterpret_cast<unsigned long long *>(&c.st->fallbacks),
                (unsigned long long)fallbacks);
  }
}

template <bool MULTI, bool AGING>
__global__ void __launch_bounds__(512) k_construct(ColonyDev c, int nchunks) {
  extern __shared__ __align__(16) uint32_t smem_construct[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int k = blockIdx.x * (blockDim.x >> 5) + warp;
  if (k >= c.m) return;
  const int words = (c.n + 31) >> 5;
  uint32_t *tabu = smem_construct + (size_t)warp * (words + (MULTI ? nchunks : 0));
  float *cend = reinterpret_cast<float *>(tabu + words);
  construct_ant<MULTI, AGING, false>(c, k, c.st->iteration, tabu, cend, nullptr, nullptr,
                                     nullptr, nchunks, lane);
}

// Shared-memory layout of the staged kernel:
//   [choice n*32 f32][ids n*32 int16][mean ld f32, aging][tabu words per warp][mbarrier]
__host__ __device__ inline size_t staged_table_bytes(int n, int ld, bool aging) {
  return (size_t)n * 32 * 4 + (size_t)n * 32 * 2 + (aging ? (size_t)ld * 4 : 0);
}

template <bool AGING>
__global__ void __launch_bounds__(1024) k_construct_staged(ColonyDev c, const int16_t *nn16) {
  extern __shared__ __align__(128) unsigned char smem_staged[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
  const int n = c.n, words = (n + 31) >> 5;
  float *scw = reinterpret_cast<float *>(smem_staged);
  int16_t *sids = reinterpret_cast<int16_t *>(smem_staged + (size_t)n * 128);
  float *smean = reinterpret_cast<float *>(smem_staged + (size_t)n * 192);
  const size_t table = staged_table_bytes(n, c.ld, AGING);
  uint32_t *tabu = reinterpret_cast<uint32_t *>(smem_staged + table) + (size_t)warp * words;
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem_staged + table + (size_t)warps * words * 4 +
                                               ((8 - ((table + (size_t)warps * words * 4) & 7)) & 7));
  __shared__ int flag;

  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    fence_barrier_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t cw_bytes = (uint32_t)n * 128u, id_bytes = (uint32_t)n * 64u;
    const uint32_t mean_bytes = AGING ? (uint32_t)c.ld * 4u : 0u;
    mbar_arrive_expect_tx(bar, cw_bytes + id_bytes + mean_bytes);
    constexpr uint32_t kPiece = 32768;
    const char *g = reinterpret_cast<const char *>(c.choice_nn);
    for (uint32_t o = 0; o < cw_bytes; o += kPiece)
      tma_load_1d(reinterpret_cast<char *>(scw) + o, g + o, min(kPiece, cw_bytes - o), bar);
    g = reinterpret_cast<const char *>(nn16);
    for (uint32_t o = 0; o < id_bytes; o += kPiece)
      tma_load_1d(reinterpret_cast<char *>(sids) + o, g + o, min(kPiece, id_bytes - o), bar);
    if (AGING) tma_load_1d(smean, c.mean, mean_bytes, bar);
    flag = mbar_wait_bounded(bar, 0, c.st) ? 1 : 0;
  }
  __syncthreads();
  if (!flag) return;
  const uint32_t iter = c.st->iteration;
  for (int k = blockIdx.x * warps + warp; k < c.m; k += gridDim.x * warps)
    construct_ant<false, AGING, true>(c, k, iter, tabu, nullptr, sids, scw, smean, 1, lane);
}

size_t construct_smem_bytes(int n, int K, int ants_per_block) {
  const int words = (n + 31) / 32;
  const int nchunks = (K + 31) / 32;
  const int per_warp = words + (K > 32 ? nchunks : 0);
  return (size_t)ants_per_block * per_warp * 4;
}

size_t construct_staged_smem_bytes(int n, int ld, bool aging, int warps) {
  const size_t words = (size_t)(n + 31) / 32;
  return staged_table_bytes(n, ld, aging) + (size_t)warps * words * 4 + 16;
}

cudaError_t configure_construct(size_t smem) {
  const int v = (int)smem;
  cudaError_t e = cudaFuncSetAttribute(k_construct<true, true>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, v);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_construct<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, v);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_construct<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, v);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_construct<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, v);
  return e;
}

cudaError_t configure_construct_staged(size_t smem) {
  const int v = (int)smem;
  cudaError_t e = cudaFuncSetAttribute(k_construct_staged<true>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, v);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_construct_staged<false>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, v);
  return e;
}

template <bool MULTI, bool AGING>
static cudaError_t launch_construct_t(const ColonyDev &c, int apb, cudaStream_t s) {
  const int nchunks = (c.K + 31) / 32;
  const size_t smem = construct_smem_bytes(c.n, c.K, apb);
  const int grid = (c.m + apb - 1) / apb;
  k_construct<MULTI, AGING><<<grid, apb * 32, smem, s>>>(c, nchunks);
  return cudaGetLastError();
}

cudaError_t launch_construct(const ColonyDev &c, int apb, cudaStream_t s) {
  const bool multi = c.K > 32;
  if (multi) return c.aging ? launch_construct_t<true, true>(c, apb, s)
                            : launch_construct_t<true, false>(c, apb, s);
  return c.aging ? launch_construct_t<false, true>(c, apb, s)
                 : launch_construct_t<false, false>(c, apb, s);
}

cudaError_t launch_construct_staged(const ColonyDev &c, const int16_t *nn16, int grid, int warps,
                                    cudaStream_t s) {
  const size_t smem = construct_staged_smem_bytes(c.n, c.ld, c.aging, warps);
  if (c.aging)
    k_construct_staged<true><<<grid, warps * 32, smem, s>>>(c, nn16);
  else
    k_construct_staged<false><<<grid, warps * 32, smem, s>>>(c, nn16);
  return cudaGetLastError();
}

}  // namespace aco
