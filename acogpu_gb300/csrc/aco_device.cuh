// aco_device.cuh -- device-side layout and helpers shared by the kernels of
// the GB300 ACO engine.
//
// HBM layout of one colony (all matrices row-major, rows padded to a stride
// that is a multiple of 32 elements = 128 bytes, so every row starts on a
// TMA-legal 16-byte boundary and warp loads are full 128-byte lines):
//   dist     n x ld   int32   EUC_2D distances, MAX on the diagonal
//   eta      n x ld   f32     heuristic (1/d)^beta
//   tau      n x ld   f32     pheromone
//   choice   n x ld   f32     tau * eta (natural city order; fallback scans)
//   nn       n x ldk  int32   candidate list of each city (first K of the
//                             sorted row; K = n for the full row)
//   eta_nn   n x ldk  f32     eta in candidate order
//   choice_nn n x ldk f32     tau * eta in candidate order (the roulette row)
//   tau_nn   n x ldk  f32     tau in candidate order (aging blend only)
//   tours    m x ld   int32   one tour per ant
//   succT    n x ldm  int32   successor of city j in the tour of ant k, at
//   predT    n x ldm  int32   [j][k]; column m holds the best-so-far tour.
//                             Bucketing edges by row j is what lets the
//                             deposit run row-owned and in ant order.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "acogpu.h"
#include "acogpu_rng.h"

namespace aco {

constexpr unsigned kFull = 0xffffffffu;

// Device error bits (ColonyState::error).
enum : uint32_t { kErrTimeout = 1u, kErrCheck = 2u };

// Per-colony scalars that live on the device so that a captured iteration
// needs no host round trip.
struct ColonyState {
  int64_t iter_best;       // Colony::iterBestDist
  int64_t glob_best;       // Colony::globBestDist
  int32_t iter_best_ant;
  uint32_t iteration;      // counter of the injected random stream
  int32_t num_valid;       // numValidAnts (aging)
  int32_t isconverged;     // isconverged (aging)
  int32_t globalperformance;
  int32_t dep_count;       // entries in the deposit list
  uint32_t error;
  int32_t error_info;
  float tau0;
  int32_t greedy_pad;
  int64_t greedy_length;   // C_nn
  int64_t fallbacks;       // steps resolved by the fallback rule
  int64_t tours_built;     // valid ants that built a tour, summed over iterations
};

struct ColonyDev {
  int n, m, K, ld, ldk, ldm;
  const int32_t *dist;
  const float *eta;
  float *tau;
  float *choice;
  const int32_t *nn;
  const int16_t *nn16;  // n x 32 candidate ids (-1 padded) when k <= 32, else null
  const float *eta_nn;
  float *tau_nn;
  float *choice_nn;
  int32_t *tours;
  int64_t *newlen;
  int64_t *len;
  int32_t *succT;
  int32_t *predT;
  int32_t *gbtour;
  int32_t *age;
  int32_t *perf;
  uint8_t *valid;
  float *mean;
  int32_t *dep_col;
  float *dep_delta;
  int32_t *plan;  // aging, staged: {B, V, blend[B], valid others[V], invalid} (m + 2)
  // Second tier of the fallback (k <= 32): the t2 nearest neighbours after
  // the k candidates (row pitch kTier2, -1 padded), their choice values and
  // the largest choice value of the row outside candidates and tier, both
  // rewritten by the row pass every iteration; t2 = 0 without a tier.
  const int32_t *nn2;
  float *t2v;
  float *mout;
  int t2;
  ColonyState *st;
  float rho, alpha;
  int use_alpha;
  int aging, min_ret, max_ret, global_perf, min_pop;
  int variant, rank_w, fallback;
  uint64_t seed;
};

__host__ __device__ inline int round_up(int x, int a) { return (x + a - 1) / a * a; }

constexpr int kTier2 = 128;  // row pitch (and most entries) of the fallback's second tier

// (float)1e-18: MIN_PHEROMONE of the reference (inc/default.h:16) as a float.
__host__ __device__ inline float min_pheromone() { return (float)0.000000000000000001; }

// ---- shared-memory addresses, mbarriers and TMA bulk copies ----------------

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

// 1-D TMA bulk copy global -> shared, completion counted on `bar`.  Both
// addresses must be 16-byte aligned and `bytes` a multiple of 16.
__device__ __forceinline__ void tma_load_1d(void *smem_dst, const void *gsrc, uint32_t bytes,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(smem_dst)),
      "l"(gsrc), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: gives up after a fixed number of polls (each poll may
// suspend the thread for a hardware-chosen interval), records the timeout in
// the colony state and returns false.  No trap, no endless spin.
constexpr uint32_t kMaxPolls = 1u << 22;
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity,
                                                  ColonyState *st, uint32_t polls = kMaxPolls) {
  for (uint32_t i = 0; i < polls; i++)
    if (mbar_try_wait(bar, parity)) return true;
  atomicOr(&st->error, kErrTimeout);
  return false;
}

}  // namespace aco
