// k_construct_steps.cuh -- roulette-wheel tour construction, one warp per
// ant: the device code shared by the construction kernels (k_construct.cu:
// general, staged and direct; k_construct_cluster.cu; k_construct_batch.cu).
//
// Replaces Colony::initTour + constructPath (src/Colony.cu:469-527,
// 689-864) and the reference GPU kernels dev_place_ants /
// dev_compute_probabilities / dev_reduce_probabilities_s / dev_move_ants
// (inc/Colony.cuh:136-162,193-229,290-347; src/Colony.cu:643-685), which the
// reference launches 3(n-1) times per iteration with a device sync after
// each.  Here one launch builds every tour.  Two step loops:
//
//  * construct_ant (any k, full rows included): the tabu list is a bitmask
//    in shared memory; the non-zero weights of each 32-candidate chunk are
//    compacted by ballot and folded in lane order, so every partial sum is
//    the reference's sequential float sum (sum_prob += prob_ptr[i],
//    src/Colony.cu:814; partial_sum += ..., :840); rows longer than 32 keep
//    the prefix at each chunk end and redo only the chunk of the crossing;
//  * staged_steps (k <= 32; the staged, cluster, direct and batch kernels):
//    the tabu list in registers, lane r holding candidate r of the current
//    row, every lane's prefix formed by masked FMAs (see staged_steps), the
//    rows read through a policy (TableRows: shared or global memory;
//    ClusterRows: distributed shared memory of a thread-block cluster).
//
// In both, the crossing `first i with partial_sum > u * sum` is a ballot;
// when the roulette cannot pick (sum <= 0, or no crossing) the fallback is
// the last unvisited city of the full nn row (select_local_best,
// inc/Colony.cuh:33-43) or the unvisited city with the largest choice value
// (through the second tier where the colony keeps one, see fallback_tier2).
// Ant aging (updateAntAges, src/Colony.cu:353-364; compute_fittness,
// inc/Colony.cuh:14-31) is fused in; the integer tour length (the reference
// adds it per move, inc/Colony.cuh:337-340) is summed by the whole warp after
// the tour is built, so no step waits on a distance load; the
// successor/predecessor of every city is written transposed for the
// row-owned deposit.
#pragma once
#include <cuda_runtime.h>

#include "aco_kernels.h"

namespace aco {

__device__ __forceinline__ bool visited(const uint32_t *tabu, int city) {
  return (tabu[city >> 5] >> (city & 31)) & 1u;
}

// Ordered fold of one chunk of 32 candidates.  The reference adds every
// weight of the row in order, zeros included (src/Colony.cu:801-816); adding
// +0 leaves a non-negative float sum unchanged, so only the non-zero weights
// need to be added, still in lane order.  They are compacted through a
// 32-float shared buffer (ballot + popc rank), then folded with broadcast
// reads; `mine` receives the prefix that ends at this lane's weight (only
// meaningful for lanes with a non-zero weight).
__device__ __forceinline__ float fold_nonzero(float s, float w, int lane, float *wbuf,
                                              float &mine) {
  const unsigned nz = __ballot_sync(kFull, w != 0.0f);
  const int cnt = __popc(nz);
  const int rank = __popc(nz & ((1u << lane) - 1u));
  if (w != 0.0f) wbuf[rank] = w;
  __syncwarp();
  mine = s;
  int i = 0;
#pragma unroll 1
  for (; i + 4 <= cnt; i += 4) {
    const float a0 = wbuf[i], a1 = wbuf[i + 1], a2 = wbuf[i + 2], a3 = wbuf[i + 3];
    s = __fadd_rn(s, a0);
    mine = (rank == i) ? s : mine;
    s = __fadd_rn(s, a1);
    mine = (rank == i + 1) ? s : mine;
    s = __fadd_rn(s, a2);
    mine = (rank == i + 2) ? s : mine;
    s = __fadd_rn(s, a3);
    mine = (rank == i + 3) ? s : mine;
  }
  for (; i < cnt; i++) {
    s = __fadd_rn(s, wbuf[i]);
    mine = (rank == i) ? s : mine;
  }
  __syncwarp();
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
static __device__ int fallback_city(const ColonyDev &c, int cur, const uint32_t *tabu,
                                    const AntCtx &a, int lane) {
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
  // Largest choice value among unvisited cities, lowest index on ties.  Each
  // lane scans groups of 4 consecutive cities with float4 loads (rows are
  // 128-byte aligned); the loads of a lane are independent of each other.
  float bw = -1.0f;
  int bj = -1;
  const float *crow = c.choice + (size_t)cur * c.ld;
  const float *trow = c.tau + (size_t)cur * c.ld;
  const float *erow = c.eta + (size_t)cur * c.ld;
#pragma unroll 2
  for (int j4 = lane * 4; j4 < c.n; j4 += 128) {
    const uint32_t bits = (tabu[j4 >> 5] >> (j4 & 31)) & 0xfu;
    if (bits == 0xfu) continue;
    float v[4];
    if (!a.blend) {
      const float4 q = *reinterpret_cast<const float4 *>(crow + j4);
      v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
    } else {
      const float4 t = *reinterpret_cast<const float4 *>(trow + j4);
      const float4 e = *reinterpret_cast<const float4 *>(erow + j4);
      v[0] = blend_fitness(t.x, e.x, a.meanc, a.ratio, c.use_alpha, c.alpha);
      v[1] = blend_fitness(t.y, e.y, a.meanc, a.ratio, c.use_alpha, c.alpha);
      v[2] = blend_fitness(t.z, e.z, a.meanc, a.ratio, c.use_alpha, c.alpha);
      v[3] = blend_fitness(t.w, e.w, a.meanc, a.ratio, c.use_alpha, c.alpha);
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
      if (!((bits >> q) & 1u) && j4 + q < c.n && v[q] > bw) {
        bw = v[q];
        bj = j4 + q;
      }
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
                              float *cend, float *wbuf, const int16_t *sids, const float *scw,
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
  const uint32_t akey = aco_ant_key(c.seed, iter, (uint32_t)k);
  const float u0 = aco_uniform_key(akey, 0u);
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
    const float u = aco_uniform_key(akey, (uint32_t)x);
    if (AGING && a.blend) a.meanc = STAGED ? smean[cur] : c.mean[cur];
    int next = -1;
    if (!MULTI) {
      int id;
      float w;
      candidate<STAGED>(c, cur, lane, tabu, sids, scw, a, id, w);
      float p;
      const float S = fold_nonzero(0.0f, w, lane, wbuf, p);
      if (!(S <= 0.0f)) {
        const float rnd = __fmul_rn(u, S);
        const unsigned hit = __ballot_sync(kFull, w != 0.0f && !(p <= rnd));
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
          s = fold_nonzero(s, w, lane, wbuf, p);
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
          fold_nonzero(s0, w, lane, wbuf, p);
          const unsigned hit = __ballot_sync(kFull, w != 0.0f && !(p <= rnd));
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
    if ((unsigned)a0 < (unsigned)n && (unsigned)b0 < (unsigned)n)
      len += c.dist[(size_t)a0 * c.ld + b0];
    else
      atomicOr(&c.st->error, kErrCheck);
  }
  for (int o = 16; o; o >>= 1) len += __shfl_xor_sync(kFull, len, o);
  if (lane == 0) {
    c.newlen[k] = len;
    if (fallbacks)
      atomicAdd(reinterpret_cast<unsigned long long *>(&c.st->fallbacks),
                (unsigned long long)fallbacks);
  }
}

// ---------------------------------------------------------------------------
// Staged construction step, specialised for the short critical path of one
// ant: candidate rows in shared memory, the tabu bitmask in registers (lane
// l owns the 32-city words l, l+32, ...; a lookup is one __shfl_sync and the
// owner lane sets the bit), the non-zero weights compacted into a
// zero-padded 32-float buffer and folded in lane order from broadcast
// 16-byte reads.
// TW words per lane cover 1024*TW cities: word w of the tabu list is held
// by lane w % 32 as its register w / 32.  A city past the list (a padding id)
// reads as unvisited.
template <int TW>
__device__ __forceinline__ bool reg_visited(const uint32_t (&tw)[TW], int city) {
  const int word = city >> 5;
  uint32_t v = __shfl_sync(kFull, tw[0], word & 31);
#pragma unroll
  for (int t = 1; t < TW; t++) {
    const uint32_t x = __shfl_sync(kFull, tw[t], word & 31);
    v = (word >> 5) == t ? x : v;
  }
  if (TW > 1 && (word >> 5) >= TW) v = 0u;
  return (v >> (city & 31)) & 1u;
}

// Every register is updated (with the bit or with 0), so the compiler never
// turns the update into a store at a computed index.
template <int TW>
__device__ __forceinline__ void reg_mark(uint32_t (&tw)[TW], int city, int lane) {
  const int word = city >> 5;
  const uint32_t bit = lane == (word & 31) ? 1u << (city & 31) : 0u;
  if constexpr (TW == 1) {  // every city is below 1024
    tw[0] |= bit;
  } else {
#pragma unroll
    for (int t = 0; t < TW; t++) tw[t] |= (word >> 5) == t ? bit : 0u;
  }
}

// Register t of the tabu words, t uniform across the warp (a select chain,
// so the array never needs a dynamic index).
template <int TW>
__device__ __forceinline__ uint32_t tw_pick(const uint32_t (&tw)[TW], int t) {
  uint32_t v = tw[0];
#pragma unroll
  for (int i = 1; i < TW; i++) v = t == i ? tw[i] : v;
  return v;
}

// Largest choice value among unvisited cities (register tabu version).  The
// plain rule issues the row loads FB 128-city chunks at a time, so a scan of
// n cities waits for ceil(n / (128 FB)) L2 round trips, not one per chunk
// (FB = 16 holds 64 registers of loads: kernels launched for at most
// kWideFallbackWarps warps).  Inlined: the tabu words must stay in registers
// (a call would take the array's address and move it to local memory).
// WIDE: the blend scan also issues its loads two chunks at a time (more
// registers; used where the kernel has them to spare).
template <int TW, bool WIDE, int FB = 4>
__device__ __forceinline__ int fallback_best_reg(const ColonyDev &c, int cur,
                                                 const uint32_t (&tw)[TW], const AntCtx &a,
                                                 int lane) {
  float bw = -1.0f;
  int bj = -1;
  const float *crow = c.choice + (size_t)cur * c.ld;
  const float *trow = c.tau + (size_t)cur * c.ld;
  const float *erow = c.eta + (size_t)cur * c.ld;
  if (!a.blend) {
    // Four independent running maxima, one per float4 component (each sees
    // its cities in increasing order, so a strict > keeps the lowest index
    // of a tie), merged below; visited and out-of-range cities enter as -1,
    // below every weight, so the scan has no branch.
    float cw[4] = {-1.0f, -1.0f, -1.0f, -1.0f};
    int cj[4] = {-1, -1, -1, -1};
#pragma unroll
    for (int t0 = 0; t0 < 8 * TW; t0 += FB) {  // n <= 1024 * TW
      if (t0 * 128 >= c.n) continue;  // (not break: the loop stays fully unrolled)
      float4 q[FB];
#pragma unroll
      for (int t = 0; t < FB; t++) {
        const int j4 = (t0 + t) * 128 + lane * 4;  // j4 < n implies j4 + 3 < ld (ld % 32 == 0)
        q[t] = j4 < c.n ? __ldcg(reinterpret_cast<const float4 *>(crow + j4))
                        : make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int t = 0; t < FB; t++) {
        const int j4 = (t0 + t) * 128 + lane * 4;
        const uint32_t v =
            __shfl_sync(kFull, tw_pick(tw, (t0 + t) >> 3), ((t0 + t) * 4 + (lane >> 3)) & 31);
        const int left = c.n - j4;  // cities of this float4 inside the instance
        const uint32_t in = left >= 4 ? 0xfu : (left > 0 ? (1u << left) - 1u : 0u);
        const uint32_t open = ~(v >> (j4 & 31)) & in;
        const float qq[4] = {q[t].x, q[t].y, q[t].z, q[t].w};
#pragma unroll
        for (int r = 0; r < 4; r++) {
          const float x = (open >> r) & 1u ? qq[r] : -1.0f;
          const bool up = x > cw[r];
          cw[r] = up ? x : cw[r];
          cj[r] = up ? j4 + r : cj[r];
        }
      }
    }
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const bool take = cj[r] >= 0 && (bj < 0 || cw[r] > bw || (cw[r] == bw && cj[r] < bj));
      bw = take ? cw[r] : bw;
      bj = take ? cj[r] : bj;
    }
  } else if (WIDE) {  // aging blend (young ants after convergence): tau and
                      // eta rows, four 128-city chunks at a time, the same
                      // four branch-free running maxima
    float cw[4] = {-1.0f, -1.0f, -1.0f, -1.0f};
    int cj[4] = {-1, -1, -1, -1};
#pragma unroll
    for (int t0 = 0; t0 < 8 * TW; t0 += 4) {  // n <= 1024 * TW
      if (t0 * 128 >= c.n) continue;
      float4 tq[4], eq[4];
#pragma unroll
      for (int t = 0; t < 4; t++) {
        const int j4 = (t0 + t) * 128 + lane * 4;
        const bool in = j4 < c.n;
        tq[t] = in ? __ldcg(reinterpret_cast<const float4 *>(trow + j4))
                   : make_float4(0.f, 0.f, 0.f, 0.f);
        eq[t] = in ? __ldg(reinterpret_cast<const float4 *>(erow + j4))
                   : make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int t = 0; t < 4; t++) {
        const int j4 = (t0 + t) * 128 + lane * 4;
        const uint32_t v =
            __shfl_sync(kFull, tw_pick(tw, (t0 + t) >> 3), ((t0 + t) * 4 + (lane >> 3)) & 31);
        const int left = c.n - j4;
        const uint32_t in = left >= 4 ? 0xfu : (left > 0 ? (1u << left) - 1u : 0u);
        const uint32_t open = ~(v >> (j4 & 31)) & in;
        const float ta[4] = {tq[t].x, tq[t].y, tq[t].z, tq[t].w};
        const float ea[4] = {eq[t].x, eq[t].y, eq[t].z, eq[t].w};
#pragma unroll
        for (int r = 0; r < 4; r++) {
          const float q = blend_fitness(ta[r], ea[r], a.meanc, a.ratio, c.use_alpha, c.alpha);
          const float x = (open >> r) & 1u ? q : -1.0f;
          const bool up = x > cw[r];
          cw[r] = up ? x : cw[r];
          cj[r] = up ? j4 + r : cj[r];
        }
      }
    }
#pragma unroll
    for (int r = 0; r < 4; r++) {
      const bool take = cj[r] >= 0 && (bj < 0 || cw[r] > bw || (cw[r] == bw && cj[r] < bj));
      bw = take ? cw[r] : bw;
      bj = take ? cj[r] : bj;
    }
  } else {  // aging blend, one 128-city chunk per round trip
    for (int base = 0; base < c.n; base += 128) {
      const int j4 = base + lane * 4;
      const int word = j4 >> 5;  // register word >> 5 (uniform), lane word & 31
      const uint32_t v = __shfl_sync(kFull, tw_pick(tw, word >> 5), word & 31);
      if (j4 >= c.n) continue;
      const uint32_t bits = (v >> (j4 & 31)) & 0xfu;
      if (bits == 0xfu) continue;
      const float4 t = *reinterpret_cast<const float4 *>(trow + j4);
      const float4 e = *reinterpret_cast<const float4 *>(erow + j4);
      const float q[4] = {blend_fitness(t.x, e.x, a.meanc, a.ratio, c.use_alpha, c.alpha),
                          blend_fitness(t.y, e.y, a.meanc, a.ratio, c.use_alpha, c.alpha),
                          blend_fitness(t.z, e.z, a.meanc, a.ratio, c.use_alpha, c.alpha),
                          blend_fitness(t.w, e.w, a.meanc, a.ratio, c.use_alpha, c.alpha)};
#pragma unroll
      for (int r = 0; r < 4; r++) {
        if (!((bits >> r) & 1u) && j4 + r < c.n && q[r] > bw) {
          bw = q[r];
          bj = j4 + r;
        }
      }
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

// The fallback's second tier: the largest plain choice value among the
// unvisited cities of the row's k candidates (this lane's) and of its tier
// (the next t2 nearest neighbours, up to four a lane), lowest index on ties.
// Every other city of the row has a choice value of at most mout[cur] (the
// row pass's maximum outside them; NaNs, which the fallback never picks,
// left out), so when the tier's best is larger it is the full scan's answer;
// otherwise -1 sends the step to the full scan.  One L2 round trip instead
// of a pass over the row.  The candidates count too because the fallback also
// runs when u*S rounds up to S with unvisited candidates left; their value
// is read from the choice matrix, as the full scan does, not from the
// candidate table (which may carry a learned prior).
template <int TW>
__device__ __forceinline__ int fallback_tier2(const ColonyDev &c, int cur,
                                              const uint32_t (&tw)[TW], int id, bool vis,
                                              int lane) {
  constexpr int Q = kTier2 / 32;
  const size_t base = (size_t)cur * kTier2;
  const bool own = lane < c.K && (unsigned)id < (unsigned)c.n && !vis;
  const float v1 = own ? __ldcg(c.choice + (size_t)cur * c.ld + id) : -1.0f;
  int id2[Q];
  float v2[Q];
#pragma unroll
  for (int q = 0; q < Q; q++) {
    const int e = lane + 32 * q;
    const bool in = e < c.t2;
    id2[q] = in ? __ldg(c.nn2 + base + e) : -1;
    v2[q] = in ? __ldcg(c.t2v + base + e) : -1.0f;
  }
  const float mo = __ldcg(c.mout + cur);
  float bw = -1.0f;
  int bj = -1;
  if (own && v1 > bw) {
    bw = v1;
    bj = id;
  }
#pragma unroll
  for (int q = 0; q < Q; q++) {
    const int city = (unsigned)id2[q] < (unsigned)c.n ? id2[q] : -1;
    const bool seen = reg_visited(tw, city < 0 ? 0 : city);  // every lane takes part
    if (city >= 0 && !seen && (v2[q] > bw || (v2[q] == bw && city < bj))) {
      bw = v2[q];
      bj = city;
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
  return bj >= 0 && bw > mo ? bj : -1;
}

// The whole fallback as a called function (the tabu words by value, so they
// stay in registers): the step loop that calls it is smaller and needs fewer
// registers.  Used where that measured faster (the cluster kernel at n =
// 4096: 1.56 -> 1.52 ms), not in the staged kernel (0.334 -> 0.343 ms).
template <int TW>
struct TwPack {
  uint32_t w[TW];
};
template <int TW, bool WIDE, int FB>
__device__ __noinline__ int fallback_outline(const ColonyDev &c, int cur, TwPack<TW> p, AntCtx a,
                                             int lane, int id, bool vis, bool tier_ok) {
  uint32_t tw[TW];
#pragma unroll
  for (int t = 0; t < TW; t++) tw[t] = p.w[t];
  int next = -1;
  if (tier_ok && c.t2 > 0) next = fallback_tier2<TW>(c, cur, tw, id, vis, lane);
  if (next < 0) next = fallback_best_reg<TW, WIDE, FB>(c, cur, tw, a, lane);
  return next;
}

// Where the step loop reads the candidate rows (pitch SP): a whole table in
// shared or global memory, or -- in a thread-block cluster -- the slice of
// the CTA that owns the row (rows r*1024 .. r*1024+1023 in cluster rank r,
// at the same shared-memory offsets in every CTA), through DSMEM.
template <int SP>
struct TableRows {
  static constexpr bool kOutlineFallback = false;
  const int16_t *ids;
  const float *w;
  const float *mean;
  __device__ __forceinline__ int id(int cur, int lr) const { return ids[cur * SP + lr]; }
  __device__ __forceinline__ float weight(int cur, int lr) const { return w[cur * SP + lr]; }
  __device__ __forceinline__ float row_mean(int cur) const { return mean[cur]; }
};

constexpr int kClusterRows = 1024;  // rows in each CTA's slice

template <int SP>
struct ClusterRows {
  static constexpr bool kOutlineFallback = true;
  uint32_t ids, w, mean;  // shared::cta addresses of the slice arrays
  __device__ __forceinline__ static uint32_t owner_addr(uint32_t local, int cur) {
    uint32_t r;
    asm("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local), "r"(cur >> 10));
    return r;
  }
  __device__ __forceinline__ int id(int cur, int lr) const {
    short v;
    asm("ld.shared::cluster.s16 %0, [%1];"
        : "=h"(v)
        : "r"(owner_addr(ids + (uint32_t)((cur & (kClusterRows - 1)) * SP + lr) * 2u, cur)));
    return v;
  }
  __device__ __forceinline__ float weight(int cur, int lr) const {
    float v;
    asm("ld.shared::cluster.f32 %0, [%1];"
        : "=f"(v)
        : "r"(owner_addr(w + (uint32_t)((cur & (kClusterRows - 1)) * SP + lr) * 4u, cur)));
    return v;
  }
  __device__ __forceinline__ float row_mean(int cur) const {
    float v;
    asm("ld.shared::cluster.f32 %0, [%1];"
        : "=f"(v)
        : "r"(owner_addr(mean + (uint32_t)(cur & (kClusterRows - 1)) * 4u, cur)));
    return v;
  }
};

// The step loop of one ant; BLEND (the aging fitness blend, fixed for the
// ant's whole tour) is a template parameter so the loop carries no per-step
// test of it.  Rows of the staged table are padded to 32 entries with id -1
// and weight 0, so every lane loads unconditionally.
//
// One step, with no data-dependent branch on the common path:
//  * lane r holds candidate r: its id and its weight, zeroed when the city is
//    visited (one __shfl_sync of the owner's tabu word);
//  * the 32 weights go through a per-warp shared buffer and every lane reads
//    all of them back with broadcast 16-byte loads;
//  * lane l forms the reference's sequential prefix s_l = (..(w_0 + w_1) +
//    ..) + w_l as acc = fma(w_e, incl_e, acc) over e = 0..31 with incl_e = 1
//    for e <= l and 0 after: w*1 + acc rounds exactly like the reference's
//    float add, and w*0 + acc = acc, so every lane runs the same 32 FMAs
//    (zero weights change no non-negative float sum, as in the reference,
//    which adds them too); each lane also adds all 32 for the full sum S;
//  * the pick is the first candidate with !(s <= u*S) (src/Colony.cu:833-846):
//    prefixes never decrease, so the crossing lanes form a suffix of the warp
//    and the first of them is a ballot + ffs; the crossing candidate always
//    has a non-zero weight.  No crossing (S = 0, or u*S rounding up to S)
//    takes the fallback, as the reference does.  An infinite weight (two
//    cities at distance 0) turns the masked product inf*0 into a NaN prefix
//    in the lanes before it, where the reference has a finite one, so the
//    test is written acc > rnd || rnd is NaN: the same as !(s <= rnd) for
//    every prefix the reference forms (its prefixes are NaN only when a
//    weight is, and then S and rnd are NaN too), false for the masks' NaNs.
//    With S = +inf this gives the reference's walk: past the row into the
//    fallback for rnd = +inf, candidate 0 for rnd = NaN (u = 0).
// The next row is loaded before the (rare) fallback test resolves.  The
// uniforms of 32 consecutive steps are computed one per lane and broadcast;
// the tour positions of the current 32-step block stay in one register per
// lane and are stored together.
template <int TW, bool BLEND, int G, bool WIDE, class ROWS, int FB = 4, bool LEAN = false,
          bool TIER = true>
__device__ __forceinline__ int staged_steps(const ColonyDev &c, int k, uint32_t akey, int start,
                                            uint32_t (&tw)[TW], float *wbuf, const ROWS &rows,
                                            AntCtx a, int lane, int64_t &fallbacks) {
  constexpr int SP = 4 * G;  // row pitch of the staged table
  const int n = c.n;
  int32_t *trow = c.tours + (size_t)k * c.ld;
  const float4 *wbuf4 = reinterpret_cast<const float4 *>(wbuf);
  float incl[SP];
#pragma unroll
  for (int e = 0; e < SP; e++) incl[e] = e <= lane ? 1.0f : 0.0f;
  // Lanes past the pitch repeat the last entry: their prefix equals the full
  // sum, so they are never the first crossing.
  const int lr = lane < SP ? lane : SP - 1;
  int cur = start;
  int id = rows.id(cur, lr);
  float wraw = BLEND ? 0.0f : rows.weight(cur, lr);
  bool ok = true;
  for (int xb = 0; xb < n && ok; xb += 32) {
    const float ublk = aco_uniform_key(akey, (uint32_t)(xb + lane));
    int tpos = (xb == 0 && lane == 0) ? start : 0;  // tour position xb + lane
    const int xe = min(n, xb + 32);
#pragma unroll 1
    for (int x = xb == 0 ? 1 : xb; x < xe; x++) {
      const float u = __shfl_sync(kFull, ublk, x & 31);
      float w = wraw;
      if (BLEND) {
        a.meanc = rows.row_mean(cur);  // every lane: the fallback scan uses it too
        const size_t off = (size_t)cur * c.ldk + lane;
        w = lane < c.K ? blend_fitness(c.tau_nn[off], __ldg(c.eta_nn + off), a.meanc, a.ratio,
                                       c.use_alpha, c.alpha)
                       : 0.0f;
      }
      // Padding entries (id -1) carry weight 0, so their tabu lookup result
      // is irrelevant; every lane must take part in the shuffle.
      const bool vis = reg_visited(tw, id & 0xffff);
      if (vis) w = 0.0f;
      wbuf[lane] = w;
      __syncwarp();
      // Two independent chains: this lane's prefix and the full sum S (the
      // second fills the first's latency gaps and saves a broadcast).  LEAN
      // (launches with many warps a scheduler, bound by issue rather than by
      // one ant's latency): S is lane 31's prefix -- the same adds in the
      // same order -- broadcast, for 4G fewer instructions a step.
      float acc = 0.0f, sum = 0.0f;
#pragma unroll
      for (int g = 0; g < G; g++) {
        const float4 p = wbuf4[g];
        acc = __fmaf_rn(p.x, incl[4 * g + 0], acc);
        if constexpr (!LEAN) sum = __fadd_rn(sum, p.x);
        acc = __fmaf_rn(p.y, incl[4 * g + 1], acc);
        if constexpr (!LEAN) sum = __fadd_rn(sum, p.y);
        acc = __fmaf_rn(p.z, incl[4 * g + 2], acc);
        if constexpr (!LEAN) sum = __fadd_rn(sum, p.z);
        acc = __fmaf_rn(p.w, incl[4 * g + 3], acc);
        if constexpr (!LEAN) sum = __fadd_rn(sum, p.w);
      }
      if constexpr (LEAN) sum = __shfl_sync(kFull, acc, 31);
      const float rnd = __fmul_rn(u, sum);
      // The reference's !(s <= rnd), with the mask's NaNs (inf*0) left out.
      const unsigned hit = __ballot_sync(kFull, acc > rnd || rnd != rnd);
      int next = __shfl_sync(kFull, id, (__ffs(hit) - 1) & 31);
      // The next row, loaded before the fallback test resolves (an in-range
      // stand-in keeps the loads inside the table) and reloaded if the
      // fallback picks the city.
      const int nx = (unsigned)next < (unsigned)n ? next : 0;
      int id_next = rows.id(nx, lr);
      float w_next = BLEND ? 0.0f : rows.weight(nx, lr);
      if (hit == 0u || (unsigned)next >= (unsigned)n) {
        if (hit != 0u) {  // a candidate id outside the instance: recorded, not used
          ok = false;
        } else if (c.fallback == ACO_FALLBACK_BEST) {
          if (!BLEND && a.blend) a.meanc = rows.row_mean(cur);  // pre-blended table
          next = -1;
          if constexpr (ROWS::kOutlineFallback) {
            TwPack<TW> pk;
#pragma unroll
            for (int t = 0; t < TW; t++) pk.w[t] = tw[t];
            next = fallback_outline<TW, WIDE, FB>(c, cur, pk, a, lane, id, vis,
                                                  TIER && !BLEND && !a.blend);
          } else {
            if (TIER && !BLEND && !a.blend && c.t2 > 0)
              next = fallback_tier2<TW>(c, cur, tw, id, vis, lane);
            if (next < 0) next = fallback_best_reg<TW, WIDE, FB>(c, cur, tw, a, lane);
          }
        } else {  // select_local_best on a full row of at most 32 cities (k == n)
          const unsigned um = __ballot_sync(kFull, lane < c.K && id >= 0 && !vis);
          next = um ? __shfl_sync(kFull, id, 31 - __clz(um)) : -1;
        }
        fallbacks += hit == 0u;
        if (next < 0 || next >= n) ok = false;  // no unvisited city, or a bad id
        if (!ok) {
          if (lane == 0) atomicOr(&c.st->error, kErrCheck);
          break;
        }
        id_next = rows.id(next, lr);
        w_next = BLEND ? 0.0f : rows.weight(next, lr);
      }
      reg_mark(tw, next, lane);
      tpos = lane == (x & 31) ? next : tpos;
      cur = next;
      id = id_next;
      wraw = w_next;
    }
    if (xb + lane < xe) trow[xb + lane] = tpos;
  }
  return cur;
}

// The tour of one valid ant once its blend context is known: placement,
// the step loop (BLEND: the aging fitness blend of every candidate per step;
// otherwise the weights come blended, or plain, from the table), then the
// integer length and the transposed successor/predecessor lists.
template <int TW, int G, bool BLEND, bool WIDE, class ROWS, int FB = 4, bool LEAN = false,
          bool TIER = true>
__device__ void staged_ant_body(const ColonyDev &c, int k, uint32_t iter, float *wbuf,
                                const ROWS &rows, AntCtx a, int lane) {
  const int n = c.n;
  int32_t *trow = c.tours + (size_t)k * c.ld;
  uint32_t tw[TW];
#pragma unroll
  for (int t = 0; t < TW; t++) tw[t] = 0u;

  // initTour placement (src/Colony.cu:518-520)
  const uint32_t akey = aco_ant_key(c.seed, iter, (uint32_t)k);
  int start = __float2int_rz(__fmul_rn(aco_uniform_key(akey, 0u), __int2float_rn(n)));
  if (start >= n) {  // impossible for u < 1; recorded, clamped
    if (lane == 0) atomicOr(&c.st->error, kErrCheck);
    start = n - 1;
  }
  reg_mark(tw, start, lane);

  int64_t fallbacks = 0;
  staged_steps<TW, BLEND, G, WIDE, ROWS, FB, LEAN, TIER>(c, k, akey, start, tw, wbuf, rows, a, lane,
                                             fallbacks);
  __syncwarp();
  // Tour length (order-free integer sum) and the transposed successor /
  // predecessor of every city for the row-owned deposit, one edge per lane;
  // unrolled so a lane's distance reads (scattered, from HBM when the L2 is
  // cold) are in flight together.
  int64_t len = 0;
#pragma unroll 8
  for (int i = lane; i < n; i += 32) {
    const int a0 = trow[i];
    const int b0 = trow[i + 1 == n ? 0 : i + 1];
    if ((unsigned)a0 < (unsigned)n && (unsigned)b0 < (unsigned)n) {
      len += c.dist[(size_t)a0 * c.ld + b0];
      c.succT[(size_t)a0 * c.ldm + k] = b0;
      c.predT[(size_t)b0 * c.ldm + k] = a0;
    } else {
      atomicOr(&c.st->error, kErrCheck);
    }
  }
  for (int o = 16; o; o >>= 1) len += __shfl_xor_sync(kFull, len, o);
  if (lane == 0) {
    c.newlen[k] = len;
    if (fallbacks)
      atomicAdd(reinterpret_cast<unsigned long long *>(&c.st->fallbacks),
                (unsigned long long)fallbacks);
  }
}

// One ant with its aging step: updateAntAges (src/Colony.cu:353-364), the
// cleared tour of an invalid ant (src/Colony.cu:507-510) and the blend
// decision of compute_fittness (inc/Colony.cuh:21-30).
template <bool AGING, int TW, int G, class ROWS, int FB = 4, bool LEAN = false, bool TIER = true>
__device__ void construct_ant_staged(const ColonyDev &c, int k, uint32_t iter, float *wbuf,
                                     const ROWS &rows, int lane) {
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
    if (!c.valid[k]) {
      int32_t *trow = c.tours + (size_t)k * c.ld;
      for (int i = lane; i < c.n; i += 32) trow[i] = 0;
      return;
    }
    a.blend = age < c.min_ret && c.st->isconverged;
    if (a.blend) a.ratio = __fdiv_rn(__int2float_rn(age), __int2float_rn(c.min_ret));
  }
  if (AGING && a.blend)
    staged_ant_body<TW, G, true, false, ROWS, FB, LEAN, TIER>(c, k, iter, wbuf, rows, a, lane);
  else
    staged_ant_body<TW, G, false, false, ROWS, FB, LEAN, TIER>(c, k, iter, wbuf, rows, a, lane);
}

}  // namespace aco
