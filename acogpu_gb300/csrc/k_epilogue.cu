// k_epilogue.cu -- per-iteration bookkeeping in one CTA, so the iteration
// needs no device-to-host copy:
//  * Colony::computeAntDistances (src/Colony.cu:996-1043): the iteration
//    best is the FIRST ant with the smallest length among valid ants, only
//    lengths below MAX_DISTANCE-1 count; the best-so-far tour is copied;
//    aging's per-ant performance counters and globalperformance;
//  * the deposit list of the pheromone update: every valid ant with
//    1/L (AntSystem::updatePheromones, src/AntSystem.cu:296-316), or for the
//    rank-based system the w-1 best ants with weight (w-r)/L and the
//    best-so-far tour with w/L_gb (Bullnheimer, Hartl & Strauss 1999);
//  * Colony::retireAnts / recruiteAnts (src/Colony.cu:379-393, 399-422);
//  * the iteration counter of the random stream.
#include <cuda_runtime.h>

#include "aco_kernels.h"

namespace aco {

constexpr int kEpiThreads = 1024;
constexpr int kMaxRankAnts = 1 << 16;

struct MinKey {
  int64_t v;
  int k;
};

__device__ __forceinline__ bool key_less(const MinKey &a, const MinKey &b) {
  if (b.k < 0) return a.k >= 0;
  if (a.k < 0) return false;
  return a.v < b.v || (a.v == b.v && a.k < b.k);
}

// Block-wide minimum of (v, k), ties to the lower k; k < 0 means "none".
__device__ MinKey block_min(MinKey x, MinKey *scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int o = 16; o; o >>= 1) {
    MinKey y;
    y.v = __shfl_xor_sync(kFull, x.v, o);
    y.k = __shfl_xor_sync(kFull, x.k, o);
    if (key_less(y, x)) x = y;
  }
  if (lane == 0) scratch[warp] = x;
  __syncthreads();
  if (warp == 0) {
    MinKey y = lane < (int)(blockDim.x >> 5) ? scratch[lane] : MinKey{0, -1};
    for (int o = 16; o; o >>= 1) {
      MinKey z;
      z.v = __shfl_xor_sync(kFull, y.v, o);
      z.k = __shfl_xor_sync(kFull, y.k, o);
      if (key_less(z, y)) y = z;
    }
    if (lane == 0) scratch[32] = y;
  }
  __syncthreads();
  MinKey r = scratch[32];
  __syncthreads();
  return r;
}

__device__ void epilogue_body(const ColonyDev &c) {
  __shared__ MinKey scratch[33];
  __shared__ uint32_t taken[kMaxRankAnts / 32];
  __shared__ int s_improved, s_best_ant;
  const int tid = threadIdx.x, m = c.m, n = c.n;
  ColonyState *st = c.st;

  // ---- lengths, aging performance, iteration best
  MinKey best{0, -1};
  for (int k = tid; k < m; k += kEpiThreads) {
    if (c.aging && !c.valid[k]) continue;
    const int64_t L = c.newlen[k];
    if (c.aging) c.perf[k] = (L == c.len[k]) ? c.perf[k] + 1 : 0;
    c.len[k] = L;
    MinKey y{L, k};
    if (key_less(y, best)) best = y;
  }
  best = block_min(best, scratch);
  if (tid == 0) {
    st->tours_built += c.aging ? st->num_valid : m;
    int ant = -1;
    int64_t ib = (int64_t)ACO_MAX_DISTANCE - 1;
    if (best.k >= 0 && best.v < ib) {
      ib = best.v;
      ant = best.k;
    }
    st->iter_best = ib;
    st->iter_best_ant = ant;
    const int improved = (ib < st->glob_best && ant > -1) ? 1 : 0;
    if (improved) {
      st->glob_best = ib;
      st->globalperformance = 0;
    } else {
      st->globalperformance = st->globalperformance + 1;
    }
    s_improved = improved;
    s_best_ant = ant;
  }
  __syncthreads();
  if (s_improved) {
    const int32_t *t = c.tours + (size_t)s_best_ant * c.ld;
    for (int i = tid; i < n; i += kEpiThreads) {
      const int a = t[i], b = t[i + 1 == n ? 0 : i + 1];
      c.gbtour[i] = a;
      c.succT[(size_t)a * c.ldm + m] = b;
      c.predT[(size_t)b * c.ldm + m] = a;
    }
  }

  // ---- deposit list
  if (c.variant == ACO_RANK_BASED) {
    for (int w = tid; w < (m + 31) / 32; w += kEpiThreads) taken[w] = 0;
    __syncthreads();
    int count = 0;
    const int w = c.rank_w;
    for (int r = 0; r < w - 1; r++) {
      MinKey b{0, -1};
      for (int k = tid; k < m; k += kEpiThreads) {
        if ((c.aging && !c.valid[k]) || ((taken[k >> 5] >> (k & 31)) & 1u)) continue;
        MinKey y{c.len[k], k};
        if (key_less(y, b)) b = y;
      }
      b = block_min(b, scratch);
      if (b.k < 0) break;
      if (tid == 0) {
        taken[b.k >> 5] |= 1u << (b.k & 31);
        c.dep_col[count] = b.k;
        c.dep_delta[count] = __fdiv_rn(__int2float_rn(w - 1 - r), __ll2float_rn(b.v));
      }
      count++;
      __syncthreads();
    }
    if (tid == 0) {
      if (st->glob_best < ACO_MAX_DISTANCE) {
        c.dep_col[count] = m;
        c.dep_delta[count] = __fdiv_rn(__int2float_rn(w), __ll2float_rn(st->glob_best));
        count++;
      }
      st->dep_count = count;
    }
  } else {
    for (int k = tid; k < m; k += kEpiThreads) {
      const bool v = !c.aging || c.valid[k];
      c.dep_col[k] = v ? k : -1;
      /* d_tau = 1.0 / (float)L, src/AntSystem.cu:300: 1/x in double then to
       * float equals the float division (double rounding is innocuous for
       * division, 53 >= 2*24+2). */
      c.dep_delta[k] = v ? __fdiv_rn(1.0f, __ll2float_rn(c.len[k])) : 0.0f;
    }
    if (tid == 0) st->dep_count = m;
  }
  __syncthreads();

  // ---- aging: retire one old ant among the first m/2, recruit one
  if (c.aging) {
    MinKey r{0, -1};
    for (int i = tid; i < m / 2; i += kEpiThreads)
      if (c.valid[i] && c.age[i] >= c.max_ret) {
        r = MinKey{0, i};
        break;
      }
    r = block_min(r, scratch);
    if (tid == 0 && r.k >= 0) {
      c.valid[r.k] = 0;
      st->num_valid = st->num_valid - 1;
      st->isconverged = 1;
    }
    __syncthreads();
    const uint32_t va = (uint32_t)st->num_valid;
    if (st->globalperformance >= c.global_perf || va < (uint32_t)c.min_pop) {
      MinKey q{0, -1};
      for (int i = tid; i < m; i += kEpiThreads)
        if (!c.valid[i]) {
          q = MinKey{0, i};
          break;
        }
      q = block_min(q, scratch);
      if (tid == 0 && q.k >= 0) {
        c.valid[q.k] = 1;
        c.age[q.k] = 0;
        st->num_valid = st->num_valid + 1;
      }
    }
  }
  if (tid == 0) st->iteration = st->iteration + 1;
}

__global__ void __launch_bounds__(kEpiThreads) k_epilogue(ColonyDev c) { epilogue_body(c); }

// One CTA per instance of a batch.
__global__ void __launch_bounds__(kEpiThreads) k_batch_epilogue(const ColonyDev *descs) {
  epilogue_body(descs[blockIdx.x]);
}

cudaError_t launch_epilogue(const ColonyDev &c, cudaStream_t s) {
  if (c.m > kMaxRankAnts) return cudaErrorInvalidValue;
  k_epilogue<<<1, kEpiThreads, 0, s>>>(c);
  return cudaGetLastError();
}

cudaError_t launch_batch_epilogue(const ColonyDev *descs, int count, cudaStream_t s) {
  k_batch_epilogue<<<count, kEpiThreads, 0, s>>>(descs);
  return cudaGetLastError();
}

}  // namespace aco
