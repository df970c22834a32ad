// k_construct.cu -- the general, staged and direct construction kernels
// and their launchers (the step loop and the fallbacks they share are in
// k_construct_steps.cuh).
#include "k_construct_steps.cuh"

namespace aco {

template <bool MULTI, bool AGING>
__global__ void __launch_bounds__(512) k_construct(ColonyDev c, int nchunks) {
  extern __shared__ __align__(16) uint32_t smem_construct[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int k = blockIdx.x * (blockDim.x >> 5) + warp;
  if (k >= c.m) return;
  const int words = (c.n + 31) >> 5;
  uint32_t *tabu = smem_construct + (size_t)warp * (words + 32 + (MULTI ? nchunks : 0));
  float *wbuf = reinterpret_cast<float *>(tabu + words);
  float *cend = wbuf + 32;
  construct_ant<MULTI, AGING, false>(c, k, c.st->iteration, tabu, cend, wbuf, nullptr, nullptr,
                                     nullptr, nchunks, lane);
}

// Aging colonies, before the staged construction: updateAntAges
// (src/Colony.cu:353-364) for every ant, then the roles of the iteration's
// ants, each list in index order: the valid ants that blend (age < min_ret
// once the colony has converged, inc/Colony.cuh:21-30), the other valid
// ants, the invalid ants (a cleared tour each).  plan = {B, V, blend[B],
// valid others[V], invalid[m - B - V]}; the valid ones come first so that the
// staged kernel spreads them evenly.  One CTA, block scans over per-thread
// runs of consecutive ants.
__device__ __forceinline__ int2 block_exclusive_scan2(int2 v, int2 *s_warp, int2 *s_total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int2 x = v;  // inclusive within the warp
  for (int o = 1; o < 32; o <<= 1) {
    const int yx = __shfl_up_sync(kFull, x.x, o), yy = __shfl_up_sync(kFull, x.y, o);
    if (lane >= o) {
      x.x += yx;
      x.y += yy;
    }
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int2 w = lane < (int)(blockDim.x >> 5) ? s_warp[lane] : make_int2(0, 0);
    for (int o = 1; o < 32; o <<= 1) {
      const int yx = __shfl_up_sync(kFull, w.x, o), yy = __shfl_up_sync(kFull, w.y, o);
      if (lane >= o) {
        w.x += yx;
        w.y += yy;
      }
    }
    s_warp[lane] = w;
    if (lane == 31) *s_total = w;
  }
  __syncthreads();
  const int2 before = warp ? s_warp[warp - 1] : make_int2(0, 0);
  return make_int2(before.x + x.x - v.x, before.y + x.y - v.y);
}

__device__ __forceinline__ void aging_plan_body(const ColonyDev &c) {
  __shared__ int2 s_warp[32];
  __shared__ int2 s_total;
  const int tid = threadIdx.x, T = blockDim.x;
  const int m = c.m;
  const bool conv = c.st->isconverged != 0;
  const int per = (m + T - 1) / T;
  const int lo = min(m, tid * per), hi = min(m, lo + per);
  int2 cnt = make_int2(0, 0);  // (blend, valid other) in [lo, hi)
  for (int k = lo; k < hi; k++) {
    const int a = c.age[k] + 1;
    c.age[k] = a;
    if (c.valid[k]) {
      if (a < c.min_ret && conv)
        cnt.x++;
      else
        cnt.y++;
    }
  }
  const int2 off = block_exclusive_scan2(cnt, s_warp, &s_total);
  const int B = s_total.x, V = s_total.y;
  int bi = off.x, vi = off.y, ii = lo - off.x - off.y;
  int32_t *list = c.plan + 2;
  for (int k = lo; k < hi; k++) {
    if (!c.valid[k])
      list[B + V + ii++] = k;
    else if (c.age[k] < c.min_ret && conv)
      list[bi++] = k;
    else
      list[B + vi++] = k;
  }
  if (tid == 0) {
    c.plan[0] = B;
    c.plan[1] = V;
  }
}

__global__ void __launch_bounds__(1024) k_aging_plan(ColonyDev c) { aging_plan_body(c); }

// One CTA per instance of a batch.
__global__ void __launch_bounds__(1024) k_batch_aging_plan(const ColonyDev *__restrict__ descs) {
  aging_plan_body(descs[blockIdx.x]);
}

cudaError_t launch_aging_plan(const ColonyDev &c, cudaStream_t s) {
  k_aging_plan<<<1, 1024, 0, s>>>(c);
  return cudaGetLastError();
}

cudaError_t launch_batch_aging_plan(const ColonyDev *descs, int count, cudaStream_t s) {
  k_batch_aging_plan<<<count, 1024, 0, s>>>(descs);
  return cudaGetLastError();
}

// Staged kernel (k <= 32 and a candidate table that fits in shared memory,
// e.g. n = 1000, k = 30: 192 KB): each CTA copies the whole table -- int16
// ids and FP32 choice values at pitch 4G -- into shared memory with TMA bulk
// copies once per launch, so a construction step touches only shared memory.
// One CTA per SM; its warps loop over ants.  Shared-memory layout: the table
// of staged_layout, then per warp 32 f32, then the mbarrier.
//
// Without aging every CTA stages the table and its warps build tours.  With
// aging the ants' roles come from k_aging_plan: CTA b < B takes blend ant b
// (and b + grid, ...) -- it fills its table with that ant's blended weights
// for every candidate of every row (the same blend_fitness as a per-step
// blend, so the same bits) and runs the ant on them at the speed of a plain
// ant; the remaining CTAs stage the plain table and share the other ants.
// TIER: the fallback's second tier is compiled in only where the colony has
// one (its code in the step loop costs the loop a few percent otherwise).
template <bool AGING, int TW, int G, bool TIER>
__global__ void __launch_bounds__(kStagedMaxWarps * 32)
    k_construct_staged(ColonyDev c, const int16_t *nn16) {
  extern __shared__ __align__(128) unsigned char smem_staged[];
  constexpr int SP = 4 * G;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
  const int n = c.n;
  const StagedLayout L = staged_layout(n, c.ld, SP, AGING);
  float *scw = reinterpret_cast<float *>(smem_staged);
  int16_t *sids = reinterpret_cast<int16_t *>(smem_staged + L.ids_off);
  float *smean = reinterpret_cast<float *>(smem_staged + L.mean_off);
  float *wbuf = reinterpret_cast<float *>(smem_staged + L.table) + (size_t)warp * 32;
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem_staged + L.table + (size_t)warps * 128);
  __shared__ int flag;
  const TableRows<SP> rows{sids, scw, smean};

  const int grid = gridDim.x;
  const int B = AGING ? c.plan[0] : 0;
  const int32_t *plan_list = c.plan + 2;
  const int base = B < grid ? B : 0;          // first CTA of the other ants
  const int P = grid - base;                  // CTAs sharing them
  const bool has_blend = AGING && (int)blockIdx.x < B;
  const bool has_other = (int)blockIdx.x >= base;
  const uint32_t cw_bytes = (uint32_t)L.ids_off;

  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    fence_barrier_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const uint32_t id_bytes = (uint32_t)(L.mean_off - L.ids_off);
    const uint32_t mean_bytes = AGING ? (uint32_t)c.ld * 4u : 0u;
    const uint32_t w_bytes = has_blend ? 0u : cw_bytes;  // a blend CTA fills its weights
    mbar_arrive_expect_tx(bar, w_bytes + id_bytes + mean_bytes);
    constexpr uint32_t kPiece = 32768;
    const char *g = reinterpret_cast<const char *>(c.choice_nn);
    for (uint32_t o = 0; o < w_bytes; o += kPiece)
      tma_load_1d(reinterpret_cast<char *>(scw) + o, g + o, min(kPiece, w_bytes - o), bar);
    g = reinterpret_cast<const char *>(nn16);
    for (uint32_t o = 0; o < id_bytes; o += kPiece)
      tma_load_1d(reinterpret_cast<char *>(sids) + o, g + o, min(kPiece, id_bytes - o), bar);
    if (AGING) tma_load_1d(smean, c.mean, mean_bytes, bar);
    flag = mbar_wait_bounded(bar, 0, c.st) ? 1 : 0;
  }
  __syncthreads();
  if (!flag) return;
  const uint32_t iter = c.st->iteration;

  if (AGING && has_blend) {
    for (int b = blockIdx.x; b < B; b += grid) {
      const int k = plan_list[b];
      const float ratio = __fdiv_rn(__int2float_rn(c.age[k]), __int2float_rn(c.min_ret));
      // Rows of the candidate arrays are contiguous at pitch SP (a multiple
      // of 4): four entries of one row per 16-byte load.
      const float4 *tau4 = reinterpret_cast<const float4 *>(c.tau_nn);
      const float4 *eta4 = reinterpret_cast<const float4 *>(c.eta_nn);
      float4 *scw4 = reinterpret_cast<float4 *>(scw);
      // Four entries per thread per round: their eight loads are issued
      // before any is used, so the build waits for ceil(nG / 4T) L2 round
      // trips instead of ceil(nG / T).
      constexpr int kBuildBatch = 4;
      const int stride = blockDim.x;
      for (int t0 = threadIdx.x; t0 < n * G; t0 += kBuildBatch * stride) {
        float4 tv[kBuildBatch], ev[kBuildBatch];
#pragma unroll
        for (int u = 0; u < kBuildBatch; u++) {
          const int t = t0 + u * stride;
          const bool in = t < n * G;
          tv[u] = in ? tau4[t] : make_float4(0.f, 0.f, 0.f, 0.f);
          ev[u] = in ? __ldg(eta4 + t) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < kBuildBatch; u++) {
          const int t = t0 + u * stride;
          if (t >= n * G) break;
          const int j = t / G, r0 = (t - j * G) * 4;
          const float mj = smean[j];
          float4 w;
          w.x = r0 + 0 < c.K ? blend_fitness(tv[u].x, ev[u].x, mj, ratio, c.use_alpha, c.alpha)
                             : 0.0f;
          w.y = r0 + 1 < c.K ? blend_fitness(tv[u].y, ev[u].y, mj, ratio, c.use_alpha, c.alpha)
                             : 0.0f;
          w.z = r0 + 2 < c.K ? blend_fitness(tv[u].z, ev[u].z, mj, ratio, c.use_alpha, c.alpha)
                             : 0.0f;
          w.w = r0 + 3 < c.K ? blend_fitness(tv[u].w, ev[u].w, mj, ratio, c.use_alpha, c.alpha)
                             : 0.0f;
          scw4[t] = w;
        }
      }
      __syncthreads();
      if (warp == 0) {
        AntCtx a;
        a.blend = true;
        a.ratio = ratio;
        a.meanc = 0.0f;
        staged_ant_body<TW, G, false, true, TableRows<SP>, 4, false, TIER>(c, k, iter, wbuf, rows,
                                                                          a, lane);
      }
      __syncthreads();
    }
    if (has_other) {  // more blend ants than CTAs: the plain weights back
      if (threadIdx.x == 0) {
        fence_proxy_async();
        mbar_arrive_expect_tx(bar, cw_bytes);
        constexpr uint32_t kPiece = 32768;
        const char *g = reinterpret_cast<const char *>(c.choice_nn);
        for (uint32_t o = 0; o < cw_bytes; o += kPiece)
          tma_load_1d(reinterpret_cast<char *>(scw) + o, g + o, min(kPiece, cw_bytes - o), bar);
        flag = mbar_wait_bounded(bar, 1, c.st) ? 1 : 0;
      }
      __syncthreads();
      if (!flag) return;
    }
  }
  if (!has_other) return;
  const int others = c.m - B;
  for (int i = ((int)blockIdx.x - base) + P * warp; i < others; i += P * warps) {
    if (!AGING) {
      construct_ant_staged<false, TW, G, TableRows<SP>, 4, false, TIER>(c, i, iter, wbuf, rows,
                                                                         lane);
      continue;
    }
    const int k = plan_list[B + i];
    if (!c.valid[k]) {  // invalid ants keep a cleared tour (src/Colony.cu:507-510)
      int32_t *trow = c.tours + (size_t)k * c.ld;
      for (int q = lane; q < n; q += 32) trow[q] = 0;
      continue;
    }
    AntCtx a;
    a.blend = false;
    a.ratio = 0.0f;
    a.meanc = 0.0f;
    staged_ant_body<TW, G, false, false, TableRows<SP>, 4, false, TIER>(c, k, iter, wbuf, rows, a,
                                                                       lane);
  }
}

// k <= 32 with a candidate table too large for shared memory (e.g. n = 4096,
// k = 32: 768 KB): the staged step loop reading its rows straight from L2
// (the same pitch-`4G` choice values and int16 ids), the tabu list in
// registers (TW words per lane, n <= 1024 * TW).
template <bool AGING, int TW, int G>
__global__ void __launch_bounds__(kStagedMaxWarps * 32) k_construct_direct(ColonyDev c) {
  __shared__ __align__(16) float wb[kStagedMaxWarps * 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
  const uint32_t iter = c.st->iteration;
  for (int k = blockIdx.x * warps + warp; k < c.m; k += gridDim.x * warps)
    construct_ant_staged<AGING, TW, G>(c, k, iter, wb + warp * 32,
                                       TableRows<4 * G>{c.nn16, c.choice_nn, c.mean}, lane);
}

namespace {
template <bool AGING, int G>
cudaError_t direct_launch_tw(const ColonyDev &c, int grid, int warps, cudaStream_t s) {
  if (c.n <= 2048)
    k_construct_direct<AGING, 2, G><<<grid, warps * 32, 0, s>>>(c);
  else if (c.n <= 4096)
    k_construct_direct<AGING, 4, G><<<grid, warps * 32, 0, s>>>(c);
  else
    k_construct_direct<AGING, 8, G><<<grid, warps * 32, 0, s>>>(c);
  return cudaGetLastError();
}
template <int G>
cudaError_t direct_launch(const ColonyDev &c, int grid, int warps, cudaStream_t s) {
  return c.aging ? direct_launch_tw<true, G>(c, grid, warps, s)
                 : direct_launch_tw<false, G>(c, grid, warps, s);
}
}  // namespace

cudaError_t launch_construct_direct(const ColonyDev &c, int grid, int warps, cudaStream_t s) {
  if (c.n > kDirectMaxCities || c.K > 32 || c.ldk != staged_pitch(c.K) || !c.nn16 ||
      warps < 1 || warps > kStagedMaxWarps)
    return cudaErrorInvalidValue;
  switch (c.ldk) {
    case 16: return direct_launch<4>(c, grid, warps, s);
    case 20: return direct_launch<5>(c, grid, warps, s);
    case 24: return direct_launch<6>(c, grid, warps, s);
    default: return direct_launch<8>(c, grid, warps, s);
  }
}

size_t construct_smem_bytes(int n, int K, int ants_per_block) {
  const int words = (n + 31) / 32;
  const int nchunks = (K + 31) / 32;
  const int per_warp = words + 32 + (K > 32 ? nchunks : 0);
  return (size_t)ants_per_block * per_warp * 4;
}

size_t construct_staged_smem_bytes(int n, int ld, int sp, bool aging, int warps) {
  return staged_layout(n, ld, sp, aging).table + (size_t)warps * 128 + 16;
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

namespace {
template <bool AGING, int TW, int G, bool TIER>
cudaError_t staged_attr(int v) {
  return cudaFuncSetAttribute(k_construct_staged<AGING, TW, G, TIER>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, v);
}
template <int G, bool TIER>
cudaError_t staged_attr_tier(int v) {
  cudaError_t e = staged_attr<true, 1, G, TIER>(v);
  if (e == cudaSuccess) e = staged_attr<false, 1, G, TIER>(v);
  if (e == cudaSuccess) e = staged_attr<true, 2, G, TIER>(v);
  if (e == cudaSuccess) e = staged_attr<false, 2, G, TIER>(v);
  return e;
}
template <int G>
cudaError_t staged_attr_all(int v) {
  cudaError_t e = staged_attr_tier<G, false>(v);
  if (e == cudaSuccess) e = staged_attr_tier<G, true>(v);
  return e;
}
template <int G, bool TIER>
cudaError_t staged_launch_t(const ColonyDev &c, const int16_t *nn16, int grid, int warps,
                            size_t smem, cudaStream_t s) {
  const bool two = c.n > 1024;
  if (c.aging) {
    if (two)
      k_construct_staged<true, 2, G, TIER><<<grid, warps * 32, smem, s>>>(c, nn16);
    else
      k_construct_staged<true, 1, G, TIER><<<grid, warps * 32, smem, s>>>(c, nn16);
  } else {
    if (two)
      k_construct_staged<false, 2, G, TIER><<<grid, warps * 32, smem, s>>>(c, nn16);
    else
      k_construct_staged<false, 1, G, TIER><<<grid, warps * 32, smem, s>>>(c, nn16);
  }
  return cudaGetLastError();
}
template <int G>
cudaError_t staged_launch(const ColonyDev &c, const int16_t *nn16, int grid, int warps,
                          size_t smem, cudaStream_t s) {
  return c.t2 > 0 ? staged_launch_t<G, true>(c, nn16, grid, warps, smem, s)
                  : staged_launch_t<G, false>(c, nn16, grid, warps, smem, s);
}
}  // namespace

cudaError_t configure_construct_staged(size_t smem) {
  const int v = (int)smem;
  cudaError_t e = staged_attr_all<4>(v);
  if (e == cudaSuccess) e = staged_attr_all<5>(v);
  if (e == cudaSuccess) e = staged_attr_all<6>(v);
  if (e == cudaSuccess) e = staged_attr_all<8>(v);
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
  if (c.n > 2048 || c.K > 32 || c.ldk != staged_pitch(c.K)) return cudaErrorInvalidValue;
  const size_t smem = construct_staged_smem_bytes(c.n, c.ld, c.ldk, c.aging, warps);
  switch (c.ldk) {
    case 16: return staged_launch<4>(c, nn16, grid, warps, smem, s);
    case 20: return staged_launch<5>(c, nn16, grid, warps, smem, s);
    case 24: return staged_launch<6>(c, nn16, grid, warps, smem, s);
    default: return staged_launch<8>(c, nn16, grid, warps, smem, s);
  }
}

}  // namespace aco
