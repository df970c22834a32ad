// k_pheromone.cu -- pheromone evaporation + deposit, fused with the next
// iteration's choice-info.
//
// Deterministic mode (the default): one CTA owns row j of tau.  It stages
// the tau row and the eta row in shared memory with TMA bulk copies,
// evaporates (AntSystem::evaporatePheromones, src/AntSystem.cu:218-223:
// tau = max((1 - rho) tau, 1e-18)), then applies the deposit list in order.
// The edges that touch row j are already bucketed by row (succT/predT[j][k]
// written by construction), so the row's deposits are a segmented fold: each
// element receives its +delta_k in ascending ant order, exactly the float
// sequence of the reference's sequential update (src/AntSystem.cu:296-316),
// which mirrors tau[j][h] into tau[h][j].  Within a chunk of 32 ants, lanes
// that hit the same element are grouped through a shared-memory mask table
// and the lowest lane folds the group in lane order.
//
// After the update the same CTA writes choice = tau * eta (the noaging
// fitness, inc/Colony.cuh:29-30; the reference's dev_compute_selection,
// inc/Colony.cuh:91-99), choice and tau in candidate order, and for aging the
// row mean of Colony::computePheromoneMean (src/Colony.cu:435-441), a
// sequential float sum.  With a fallback second tier (k <= 32) it also writes
// the choice values of the tier's cities and the largest choice value of the
// row outside the row itself, its candidates and its tier (marked in a
// shared bitmap before the row lands; NaNs ignored, as the fallback never
// picks one).
//
// Atomic mode: a float4 evaporation pass, then one red.global.add.f32 per
// directed edge, then the same row pass without evaporation or deposit.
#include <cuda_runtime.h>

#include "aco_kernels.h"

namespace aco {

constexpr int kRowThreads = 256;
// Deposit entries staged per segment (double-buffered: warps 1.. load the
// next segment's successor, predecessor and delta while warp 0 folds this
// one), so the ordered fold reads shared memory only.
constexpr int kDepSeg = 256;
// Deposit entries a staging thread reads at once (batch rows: 4.53 ms at 1,
// 4.37 at 2, 4.32 at 4; 4 slowed the single-colony row pass by 4 us).
constexpr int kStageBatch = 2;

__device__ __forceinline__ float choice_of(float tau, float eta, int use_alpha, float alpha) {
  const float p = use_alpha ? powf(tau, alpha) : tau;
  return __fmul_rn(p, eta);
}

template <bool EVAP, bool DEPOSIT, bool WRITE_TAU>
__device__ __forceinline__ void pheromone_row_body(const ColonyDev &c, const int j) {
  extern __shared__ __align__(128) unsigned char smem_rows[];
  const int ld = c.ld, n = c.n, tid = threadIdx.x, nthreads = blockDim.x;
  float *row = reinterpret_cast<float *>(smem_rows);
  float *erow = row + ld;
  uint32_t *mt = reinterpret_cast<uint32_t *>(erow + ld);
  int *seg_s = reinterpret_cast<int *>(mt + (DEPOSIT ? ld : 0));  // [2][kDepSeg]
  int *seg_p = seg_s + (DEPOSIT ? 2 * kDepSeg : 0);
  float *seg_d = reinterpret_cast<float *>(seg_p + (DEPOSIT ? 2 * kDepSeg : 0));
  float *dl = seg_d + (DEPOSIT ? 2 * kDepSeg : 0);
  uint64_t *bar = reinterpret_cast<uint64_t *>(dl + 32);
  int *flag = reinterpret_cast<int *>(bar + 1);
  uint32_t *nbm = reinterpret_cast<uint32_t *>(flag + 1);  // [ld / 32]: candidates + tier
  const bool tier = c.t2 > 0;

  if (tid == 0) {
    mbar_init(bar, 1);
    fence_barrier_init();
  }
  if (DEPOSIT)
    for (int h = tid; h < ld; h += nthreads) mt[h] = 0;
  if (tier)
    for (int w = tid; w < ld / 32; w += nthreads) nbm[w] = 0u;
  __syncthreads();
  if (tid == 0) {
    const uint32_t bytes = (uint32_t)ld * 4u;
    mbar_arrive_expect_tx(bar, 2u * bytes);
    tma_load_1d(row, c.tau + (size_t)j * ld, bytes, bar);
    tma_load_1d(erow, c.eta + (size_t)j * ld, bytes, bar);
  }
  if (tier) {  // the row itself, its k candidates and its tier, while the row lands
    const size_t koff = (size_t)j * c.ldk;
    for (int r = tid; r <= c.K + c.t2; r += nthreads) {
      const int id = r < c.K ? c.nn[koff + r]
                             : (r < c.K + c.t2 ? c.nn2[(size_t)j * kTier2 + (r - c.K)] : j);
      if ((unsigned)id < (unsigned)n) atomicOr(&nbm[id >> 5], 1u << (id & 31));
    }
  }
  if (tid == 0) *flag = mbar_wait_bounded(bar, 0, c.st) ? 1 : 0;
  __syncthreads();
  if (!*flag) return;

  if (EVAP) {
    const float keep = __fsub_rn(1.0f, c.rho);
    const float fmin = min_pheromone();
    for (int h = tid; h < n; h += nthreads) {
      const float v = __fmul_rn(keep, row[h]);
      row[h] = v > fmin ? v : fmin;
    }
    __syncthreads();
  }

  if (DEPOSIT) {
    const int cnt = c.st->dep_count;
    const size_t base_row = (size_t)j * c.ldm;
    // Segment `seg` of the deposit list -> buffer `buf`: for each entry the
    // successor and predecessor of city j in that ant's tour and its delta.
    // A staging thread takes kStageBatch entries at a time and issues all
    // their list reads, then all their successor/predecessor reads, so a
    // segment waits for two L2 round trips per batch, not two per entry.
    auto stage = [&](int seg, int buf) {
      const int stride = nthreads - 32;
      for (int q0 = tid - 32; q0 < kDepSeg; q0 += kStageBatch * stride) {
        int col[kStageBatch], sN[kStageBatch], pN[kStageBatch];
        float d[kStageBatch];
#pragma unroll
        for (int u = 0; u < kStageBatch; u++) {
          const int q = q0 + u * stride, e = seg * kDepSeg + q;
          const bool in = q < kDepSeg && e < cnt;
          col[u] = in ? c.dep_col[e] : -1;
          d[u] = in ? c.dep_delta[e] : 0.0f;
        }
#pragma unroll
        for (int u = 0; u < kStageBatch; u++) {
          sN[u] = col[u] >= 0 ? c.succT[base_row + col[u]] : -1;
          pN[u] = col[u] >= 0 ? c.predT[base_row + col[u]] : -1;
        }
#pragma unroll
        for (int u = 0; u < kStageBatch; u++) {
          const int q = q0 + u * stride;
          if (q >= kDepSeg) break;
          if (col[u] >= 0 && ((unsigned)sN[u] >= (unsigned)n || (unsigned)pN[u] >= (unsigned)n)) {
            atomicOr(&c.st->error, kErrCheck);
            sN[u] = pN[u] = -1;
          }
          seg_s[buf * kDepSeg + q] = sN[u];
          seg_p[buf * kDepSeg + q] = pN[u];
          seg_d[buf * kDepSeg + q] = d[u];
        }
      }
    };
    if (tid >= 32) stage(0, 0);
    __syncthreads();
    for (int seg = 0; seg * kDepSeg < cnt; seg++) {
      const int buf = seg & 1;
      if (tid >= 32) {
        if ((seg + 1) * kDepSeg < cnt) stage(seg + 1, buf ^ 1);
      } else {
        const int lane = tid;
        const int end = min(kDepSeg, cnt - seg * kDepSeg);
        for (int base = 0; base < end; base += 32) {
          const int q = buf * kDepSeg + base + lane;
          const bool in = base + lane < end;
          const int sN = in ? seg_s[q] : -1, pN = in ? seg_p[q] : -1;
          dl[lane] = in ? seg_d[q] : 0.0f;
          if (sN >= 0) atomicOr(&mt[sN], 1u << lane);
          if (pN >= 0) atomicOr(&mt[pN], 1u << lane);
          __syncwarp();
          // The lowest lane touching an element leads it and adds the deltas
          // of every lane in its group, in lane (= ant) order: 32 unrolled
          // predicated adds from broadcast registers, the successor and the
          // predecessor element of a lane as two independent chains.
          const unsigned Ms = sN >= 0 ? mt[sN] : 0u, Mp = pN >= 0 ? mt[pN] : 0u;
          const unsigned As = (sN >= 0 && __ffs(Ms) - 1 == lane) ? Ms : 0u;
          const unsigned Ap = (pN >= 0 && __ffs(Mp) - 1 == lane) ? Mp : 0u;
          float vs = As ? row[sN] : 0.0f, vp = Ap ? row[pN] : 0.0f;
          const float4 *dl4 = reinterpret_cast<const float4 *>(dl);
#pragma unroll
          for (int g = 0; g < 8; g++) {
            const float4 q4 = dl4[g];
            const float dq[4] = {q4.x, q4.y, q4.z, q4.w};
#pragma unroll
            for (int e = 0; e < 4; e++) {
              if ((As >> (4 * g + e)) & 1u) vs = __fadd_rn(vs, dq[e]);
              if ((Ap >> (4 * g + e)) & 1u) vp = __fadd_rn(vp, dq[e]);
            }
          }
          if (As) row[sN] = vs;
          if (Ap) row[pN] = vp;
          __syncwarp();
          if (sN >= 0) mt[sN] = 0;
          if (pN >= 0) mt[pN] = 0;
          __syncwarp();
        }
      }
      __syncthreads();
    }
  }

  float *trow = c.tau + (size_t)j * ld;
  float *crow = c.choice + (size_t)j * ld;
  float mx = -1.0f;  // tier: largest choice value outside the marked cities
  for (int h4 = tid; h4 < ld / 4; h4 += nthreads) {
    const float4 t = reinterpret_cast<const float4 *>(row)[h4];
    const float4 e = reinterpret_cast<const float4 *>(erow)[h4];
    if (WRITE_TAU) reinterpret_cast<float4 *>(trow)[h4] = t;
    float4 cv;
    cv.x = choice_of(t.x, e.x, c.use_alpha, c.alpha);
    cv.y = choice_of(t.y, e.y, c.use_alpha, c.alpha);
    cv.z = choice_of(t.z, e.z, c.use_alpha, c.alpha);
    cv.w = choice_of(t.w, e.w, c.use_alpha, c.alpha);
    reinterpret_cast<float4 *>(crow)[h4] = cv;
    if (tier) {
      const int h = 4 * h4;  // four cities of one bitmap word
      const uint32_t marked = nbm[h >> 5] >> (h & 31);
      if (h + 0 < n && !(marked & 1u)) mx = fmaxf(mx, cv.x);
      if (h + 1 < n && !(marked & 2u)) mx = fmaxf(mx, cv.y);
      if (h + 2 < n && !(marked & 4u)) mx = fmaxf(mx, cv.z);
      if (h + 3 < n && !(marked & 8u)) mx = fmaxf(mx, cv.w);
    }
  }
  if (tier) {
    for (int e = tid; e < c.t2; e += nthreads) {
      const int id = c.nn2[(size_t)j * kTier2 + e];
      c.t2v[(size_t)j * kTier2 + e] =
          (unsigned)id < (unsigned)n ? choice_of(row[id], erow[id], c.use_alpha, c.alpha) : -1.0f;
    }
    for (int o = 16; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(kFull, mx, o));
    __syncthreads();  // dl is free again (the deposit fold used it)
    if ((tid & 31) == 0) dl[tid >> 5] = mx;
    __syncthreads();
    if (tid < 32) {
      float v = tid < (nthreads >> 5) ? dl[tid] : -1.0f;
      for (int o = 16; o; o >>= 1) v = fmaxf(v, __shfl_xor_sync(kFull, v, o));
      if (tid == 0) c.mout[j] = v;
    }
  }
  const size_t koff = (size_t)j * c.ldk;
  for (int r = tid; r < c.ldk; r += nthreads) {
    float cv = 0.0f, tv = 0.0f;
    if (r < c.K) {
      const int id = c.nn[koff + r];
      tv = row[id];
      // eta_nn is eta gathered in candidate order (times the learned prior,
      // when one is installed), so without a prior this is tau * eta.
      cv = choice_of(tv, c.eta_nn[koff + r], c.use_alpha, c.alpha);
    }
    c.choice_nn[koff + r] = cv;
    if (c.aging) c.tau_nn[koff + r] = tv;
  }
  if (c.aging && tid == 0) {
    float s = 0.0f;
    for (int h = 0; h < n; h++) s = __fadd_rn(s, row[h]);
    c.mean[j] = __fdiv_rn(s, __int2float_rn(n));
  }
}

template <bool EVAP, bool DEPOSIT, bool WRITE_TAU>
__global__ void __launch_bounds__(512) k_pheromone_rows(ColonyDev c) {
  pheromone_row_body<EVAP, DEPOSIT, WRITE_TAU>(c, blockIdx.x);
}

// Batch form: global row g is row rowmap[g].y of instance rowmap[g].x.
template <bool EVAP, bool DEPOSIT, bool WRITE_TAU>
__global__ void __launch_bounds__(512) k_batch_pheromone_rows(const ColonyDev *descs,
                                                            const int2 *rowmap) {
  const int2 r = rowmap[blockIdx.x];
  pheromone_row_body<EVAP, DEPOSIT, WRITE_TAU>(descs[r.x], r.y);
}

static size_t rows_smem(int ld, bool deposit) {
  return (size_t)ld * 4 * (deposit ? 3 : 2) + (deposit ? 2 * kDepSeg * 12 : 0) + 32 * 4 + 16 +
         (size_t)(ld / 32) * 4;
}

// At least two warps: warp 0 folds the deposits, the others stage them.
static int row_threads(int threads) { return threads >= 64 ? threads : kRowThreads; }

template <bool EVAP, bool DEPOSIT, bool WRITE_TAU>
static cudaError_t launch_rows_t(const ColonyDev &c, int threads, cudaStream_t s) {
  const size_t smem = rows_smem(c.ld, DEPOSIT);
  k_pheromone_rows<EVAP, DEPOSIT, WRITE_TAU><<<c.n, row_threads(threads), smem, s>>>(c);
  return cudaGetLastError();
}

template <bool EVAP, bool DEPOSIT, bool WRITE_TAU>
static cudaError_t configure_t(int ld) {
  const int v = (int)rows_smem(ld, DEPOSIT);
  cudaError_t e = cudaFuncSetAttribute(k_pheromone_rows<EVAP, DEPOSIT, WRITE_TAU>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, v);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_batch_pheromone_rows<EVAP, DEPOSIT, WRITE_TAU>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, v);
  return e;
}

cudaError_t configure_pheromone_rows(int ld) {
  cudaError_t e = configure_t<true, true, true>(ld);
  if (e == cudaSuccess) e = configure_t<false, true, true>(ld);
  if (e == cudaSuccess) e = configure_t<true, false, true>(ld);
  if (e == cudaSuccess) e = configure_t<false, false, true>(ld);
  if (e == cudaSuccess) e = configure_t<false, false, false>(ld);
  return e;
}

cudaError_t launch_pheromone_rows(const ColonyDev &c, bool evaporate, bool deposit,
                                  bool write_tau, cudaStream_t s, int threads) {
  if (evaporate && deposit) return launch_rows_t<true, true, true>(c, threads, s);
  if (evaporate) return launch_rows_t<true, false, true>(c, threads, s);
  if (deposit) return launch_rows_t<false, true, true>(c, threads, s);
  return write_tau ? launch_rows_t<false, false, true>(c, threads, s)
                   : launch_rows_t<false, false, false>(c, threads, s);
}

cudaError_t launch_batch_pheromone_rows(const ColonyDev *descs, const int2 *rowmap, int rows,
                                        int max_ld, bool deposit_and_evaporate, cudaStream_t s,
                                        int threads) {
  const int t = row_threads(threads);
  if (deposit_and_evaporate) {
    k_batch_pheromone_rows<true, true, true><<<rows, t, rows_smem(max_ld, true), s>>>(descs, rowmap);
  } else {
    k_batch_pheromone_rows<false, false, false><<<rows, t, rows_smem(max_ld, false), s>>>(descs,
                                                                                          rowmap);
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------- atomic mode
__global__ void k_evaporate(float *__restrict__ tau, int64_t total4, float rho) {
  const float keep = __fsub_rn(1.0f, rho);
  const float fmin = min_pheromone();
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total4;
       t += (int64_t)gridDim.x * blockDim.x) {
    float4 v = reinterpret_cast<float4 *>(tau)[t];
    v.x = __fmul_rn(keep, v.x);
    v.y = __fmul_rn(keep, v.y);
    v.z = __fmul_rn(keep, v.z);
    v.w = __fmul_rn(keep, v.w);
    v.x = v.x > fmin ? v.x : fmin;
    v.y = v.y > fmin ? v.y : fmin;
    v.z = v.z > fmin ? v.z : fmin;
    v.w = v.w > fmin ? v.w : fmin;
    reinterpret_cast<float4 *>(tau)[t] = v;
  }
}

cudaError_t launch_evaporate(const ColonyDev &c, cudaStream_t s) {
  k_evaporate<<<4 * 152, 256, 0, s>>>(c.tau, (int64_t)c.n * c.ld / 4, c.rho);
  return cudaGetLastError();
}

// One thread per (deposit entry, tour position): both directions of the
// edge receive +delta (the reference's GPU kernel updated one direction
// only, src/AntSystem.cu:105-128; its CPU path is symmetric).
__global__ void k_deposit_atomic(ColonyDev c) {
  const int n = c.n;
  const int cnt = c.st->dep_count;
  const int64_t total = (int64_t)cnt * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int q = (int)(t / n), i = (int)(t % n);
    const int col = c.dep_col[q];
    if (col < 0) continue;
    const int32_t *tour = col < c.m ? c.tours + (size_t)col * c.ld : c.gbtour;
    const int a = tour[i], b = tour[i + 1 == n ? 0 : i + 1];
    const float d = c.dep_delta[q];
    atomicAdd(c.tau + (size_t)a * c.ld + b, d);
    atomicAdd(c.tau + (size_t)b * c.ld + a, d);
  }
}

cudaError_t launch_deposit_atomic(const ColonyDev &c, cudaStream_t s) {
  k_deposit_atomic<<<8 * 152, 256, 0, s>>>(c);
  return cudaGetLastError();
}

}  // namespace aco
