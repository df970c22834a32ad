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
//    src/Colony.cu:814; partial_sum += ..., :840): the non-zero weights of a
//    chunk are compacted by ballot and added in lane order, so every partial
//    sum is bit-identical to the CPU's (the zero weight of a visited city
//    changes no sum);
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

// Where the step loop reads the candidate rows (pitch SP): a whole table in
// shared or global memory, or -- in a thread-block cluster -- the slice of
// the CTA that owns the row (rows r*1024 .. r*1024+1023 in cluster rank r,
// at the same shared-memory offsets in every CTA), through DSMEM.
template <int SP>
struct TableRows {
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
template <int TW, bool BLEND, int G, bool WIDE, class ROWS, int FB = 4, bool LEAN = false>
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
          next = fallback_best_reg<TW, WIDE, FB>(c, cur, tw, a, lane);
        } else {  // select_local_best on a full row of at most 32 cities (k == n)
          const unsigned um = __ballot_sync(kFull, id >= 0 && !vis);
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
template <int TW, int G, bool BLEND, bool WIDE, class ROWS, int FB = 4, bool LEAN = false>
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
  staged_steps<TW, BLEND, G, WIDE, ROWS, FB, LEAN>(c, k, akey, start, tw, wbuf, rows, a, lane,
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
template <bool AGING, int TW, int G, class ROWS, int FB = 4, bool LEAN = false>
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
    staged_ant_body<TW, G, true, false, ROWS, FB, LEAN>(c, k, iter, wbuf, rows, a, lane);
  else
    staged_ant_body<TW, G, false, false, ROWS, FB, LEAN>(c, k, iter, wbuf, rows, a, lane);
}

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

__global__ void __launch_bounds__(1024) k_aging_plan(ColonyDev c) {
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

cudaError_t launch_aging_plan(const ColonyDev &c, cudaStream_t s) {
  k_aging_plan<<<1, 1024, 0, s>>>(c);
  return cudaGetLastError();
}

// Shared-memory layout of the staged kernel: the table of staged_layout,
// then per warp 32 f32, then the mbarrier.  G = pitch / 4.
//
// Without aging every CTA stages the table and its warps build tours.  With
// aging the ants' roles come from k_aging_plan: CTA b < B takes blend ant b
// (and b + grid, ...) -- it fills its table with that ant's blended weights
// for every candidate of every row (the same blend_fitness as a per-step
// blend, so the same bits) and runs the ant on them at the speed of a plain
// ant; the remaining CTAs stage the plain table and share the other ants.
template <bool AGING, int TW, int G>
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
        staged_ant_body<TW, G, false, true>(c, k, iter, wbuf, rows, a, lane);
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
      construct_ant_staged<false, TW, G>(c, i, iter, wbuf, rows, lane);
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
    staged_ant_body<TW, G, false, false>(c, k, iter, wbuf, rows, a, lane);
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

// ---------------------------------------------------------------------------
// Candidate table split over a thread-block cluster (k <= 32, n <= 8192, a
// table too large for one CTA): cluster rank r holds rows r*1024 .. r*1024 +
// 1023 (choice values, int16 ids, aging row means) at the same offsets as
// every other rank.  Each CTA stages its slice with TMA bulk copies; after a
// cluster barrier the ants read every row from its owner's shared memory
// (mapa + ld.shared::cluster) with the staged step loop; a second barrier
// keeps each slice alive until the whole cluster is done.  Every thread
// reaches both barriers on every path (a copy that timed out only records
// the error).  All CTAs share all ants.
__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

__device__ __forceinline__ uint32_t cluster_size() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
  return r;
}

__device__ __forceinline__ void cluster_barrier() {
  asm volatile(
      "barrier.cluster.arrive.release.aligned;\n\t"
      "barrier.cluster.wait.acquire.aligned;" ::
          : "memory");
}

template <bool AGING, int TW, int G, int FB>
__global__ void __launch_bounds__((FB > 4 ? kWideFallbackWarps : kStagedMaxWarps) * 32)
    k_construct_cluster(ColonyDev c) {
  extern __shared__ __align__(128) unsigned char smem_cl[];
  constexpr int SP = 4 * G;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
  const StagedLayout L = staged_layout(kClusterRows, kClusterRows, SP, AGING);
  float *scw = reinterpret_cast<float *>(smem_cl);
  int16_t *sids = reinterpret_cast<int16_t *>(smem_cl + L.ids_off);
  float *smean = reinterpret_cast<float *>(smem_cl + L.mean_off);
  float *wbuf = reinterpret_cast<float *>(smem_cl + L.table) + (size_t)warp * 32;
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem_cl + L.table + (size_t)warps * 128);
  __shared__ int flag, all_ok;

  const int r0 = (int)cluster_rank() * kClusterRows;
  const int rows_here = max(0, min(kClusterRows, c.n - r0));
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    fence_barrier_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    // sizes rounded up to 16 bytes (the buffers carry 16 bytes of slack)
    const uint32_t cw_bytes = (uint32_t)rows_here * SP * 4u;
    const uint32_t id_bytes = ((uint32_t)rows_here * SP * 2u + 15u) & ~15u;
    const uint32_t mean_bytes = AGING ? (((uint32_t)rows_here * 4u + 15u) & ~15u) : 0u;
    const uint32_t total = cw_bytes + id_bytes + mean_bytes;
    int ok = 1;
    if (total) {
      mbar_arrive_expect_tx(bar, total);
      constexpr uint32_t kPiece = 32768;
      const char *g = reinterpret_cast<const char *>(c.choice_nn + (size_t)r0 * SP);
      for (uint32_t o = 0; o < cw_bytes; o += kPiece)
        tma_load_1d(reinterpret_cast<char *>(scw) + o, g + o, min(kPiece, cw_bytes - o), bar);
      g = reinterpret_cast<const char *>(c.nn16 + (size_t)r0 * SP);
      for (uint32_t o = 0; o < id_bytes; o += kPiece)
        tma_load_1d(reinterpret_cast<char *>(sids) + o, g + o, min(kPiece, id_bytes - o), bar);
      if (AGING) tma_load_1d(smean, c.mean + r0, mean_bytes, bar);
      ok = mbar_wait_bounded(bar, 0, c.st) ? 1 : 0;
    }
    flag = ok;
  }
  __syncthreads();
  cluster_barrier();  // every slice of the cluster is in place
  if (threadIdx.x == 0) {
    // ants read every slice: run them only when every CTA staged its own
    int all = 1;
    for (uint32_t r = 0; r < cluster_size(); r++) {
      uint32_t a;
      int v;
      asm("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(a) : "r"(smem_u32(&flag)), "r"(r));
      asm volatile("ld.shared::cluster.s32 %0, [%1];" : "=r"(v) : "r"(a));
      all &= v;
    }
    all_ok = all;
  }
  __syncthreads();
  if (all_ok) {
    const ClusterRows<SP> rows{smem_u32(sids), smem_u32(scw), smem_u32(smean)};
    const uint32_t iter = c.st->iteration;
    for (int k = blockIdx.x * warps + warp; k < c.m; k += gridDim.x * warps)
      construct_ant_staged<AGING, TW, G, ClusterRows<SP>, FB>(c, k, iter, wbuf, rows, lane);
  }
  __syncthreads();
  cluster_barrier();  // no slice is released while another CTA may read it
}

size_t construct_cluster_smem_bytes(int sp, bool aging, int warps) {
  return staged_layout(kClusterRows, kClusterRows, sp, aging).table + (size_t)warps * 128 + 16;
}

namespace {
template <bool AGING, int TW, int G, int FB>
cudaError_t cluster_launch_t(const ColonyDev &c, int grid, int warps, int cs, cudaStream_t s,
                             int *max_clusters) {
  const size_t smem = construct_cluster_smem_bytes(4 * G, AGING, warps);
  if (max_clusters) {
    // the query, at planning time, opens the kernel to any warp count, so a
    // launch (possibly under stream capture) sets no attribute
    const size_t most = construct_cluster_smem_bytes(4 * G, AGING, kStagedMaxWarps);
    cudaError_t e = cudaFuncSetAttribute(k_construct_cluster<AGING, TW, G, FB>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)most);
    if (e != cudaSuccess) return e;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(warps * 32);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = cs;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  if (max_clusters)
    return cudaOccupancyMaxActiveClusters(max_clusters, k_construct_cluster<AGING, TW, G, FB>, &cfg);
  return cudaLaunchKernelEx(&cfg, k_construct_cluster<AGING, TW, G, FB>, c);
}
template <bool AGING, int G>
cudaError_t cluster_launch_tw(const ColonyDev &c, int grid, int warps, int cs, cudaStream_t s,
                              int *max_clusters) {
  // n > 2048 with few ants per CTA: the fallback scan with 16 chunks in flight
  const bool wide = warps <= kWideFallbackWarps;
  if (c.n <= 2048) return cluster_launch_t<AGING, 2, G, 4>(c, grid, warps, cs, s, max_clusters);
  if (c.n <= 4096)
    return wide ? cluster_launch_t<AGING, 4, G, 16>(c, grid, warps, cs, s, max_clusters)
                : cluster_launch_t<AGING, 4, G, 4>(c, grid, warps, cs, s, max_clusters);
  return wide ? cluster_launch_t<AGING, 8, G, 16>(c, grid, warps, cs, s, max_clusters)
              : cluster_launch_t<AGING, 8, G, 4>(c, grid, warps, cs, s, max_clusters);
}
template <int G>
cudaError_t cluster_launch_g(const ColonyDev &c, int grid, int warps, int cs, cudaStream_t s,
                             int *max_clusters) {
  return c.aging ? cluster_launch_tw<true, G>(c, grid, warps, cs, s, max_clusters)
                 : cluster_launch_tw<false, G>(c, grid, warps, cs, s, max_clusters);
}
cudaError_t cluster_dispatch(const ColonyDev &c, int grid, int warps, int cs, cudaStream_t s,
                             int *max_clusters) {
  if (c.n > kDirectMaxCities || c.K > 32 || c.ldk != staged_pitch(c.K) || !c.nn16 ||
      warps < 1 || warps > kStagedMaxWarps || cs < 1 || cs > 8 ||
      cs * kClusterRows < c.n || (max_clusters == nullptr && grid % cs))
    return cudaErrorInvalidValue;
  switch (c.ldk) {
    case 16: return cluster_launch_g<4>(c, grid, warps, cs, s, max_clusters);
    case 20: return cluster_launch_g<5>(c, grid, warps, cs, s, max_clusters);
    case 24: return cluster_launch_g<6>(c, grid, warps, cs, s, max_clusters);
    default: return cluster_launch_g<8>(c, grid, warps, cs, s, max_clusters);
  }
}
}  // namespace

cudaError_t query_construct_cluster(const ColonyDev &c, int warps, int cs, int *max_clusters) {
  *max_clusters = 0;
  // Both fallback widths (the query also opens each kernel's shared memory):
  // the launch picks one by its final warp count.
  int wide = 0, narrow = 0;
  cudaError_t e = cluster_dispatch(c, cs, kWideFallbackWarps, cs, nullptr, &wide);
  if (e == cudaSuccess) e = cluster_dispatch(c, cs, kStagedMaxWarps, cs, nullptr, &narrow);
  if (e == cudaSuccess) *max_clusters = warps <= kWideFallbackWarps ? wide : narrow;
  return e;
}

cudaError_t launch_construct_cluster(const ColonyDev &c, int grid, int warps, int cs,
                                     cudaStream_t s) {
  return cluster_dispatch(c, grid, warps, cs, s, nullptr);
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
template <bool AGING, int TW, int G>
cudaError_t staged_attr(int v) {
  return cudaFuncSetAttribute(k_construct_staged<AGING, TW, G>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, v);
}
template <int G>
cudaError_t staged_attr_all(int v) {
  cudaError_t e = staged_attr<true, 1, G>(v);
  if (e == cudaSuccess) e = staged_attr<false, 1, G>(v);
  if (e == cudaSuccess) e = staged_attr<true, 2, G>(v);
  if (e == cudaSuccess) e = staged_attr<false, 2, G>(v);
  return e;
}
template <int G>
cudaError_t staged_launch(const ColonyDev &c, const int16_t *nn16, int grid, int warps,
                          size_t smem, cudaStream_t s) {
  const bool two = c.n > 1024;
  if (c.aging) {
    if (two)
      k_construct_staged<true, 2, G><<<grid, warps * 32, smem, s>>>(c, nn16);
    else
      k_construct_staged<true, 1, G><<<grid, warps * 32, smem, s>>>(c, nn16);
  } else {
    if (two)
      k_construct_staged<false, 2, G><<<grid, warps * 32, smem, s>>>(c, nn16);
    else
      k_construct_staged<false, 1, G><<<grid, warps * 32, smem, s>>>(c, nn16);
  }
  return cudaGetLastError();
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

namespace aco {

// ---------------------------------------------------------------------------
// Batches of instances of uneven size in one persistent launch.  Each CTA
// takes work items -- (instance, first ant, ant count, staged) -- from a
// global queue with atomicAdd until the queue is empty; no CTA ever waits for
// another.  Items are ordered by decreasing instance size on the host
// (longest job first), so the tail of the launch is made of small items.  The
// instance's descriptor is copied into shared memory once per item.
//
// A staged item (k <= 32 and a candidate table that fits the CTA's table
// region) first copies its instance's table -- FP32 choice values, int16
// ids, and the aging row means -- into shared memory with TMA bulk copies on
// one mbarrier, then its warps build tours with the staged step loop of the
// single-colony kernel.  Other items with the same pitch (n <= 2048) run that
// step loop on rows read from L2; the rest use the general kernel with the
// tabu list in the region.  Shared layout:
//   [region: table, or per-warp tabu lists][per warp: 32 f32][mbarrier]
template <bool MULTI, bool AGING, int G>
__global__ void __launch_bounds__(512) k_batch_construct(const ColonyDev *__restrict__ descs,
                                                         const int4 *__restrict__ items,
                                                         int num_items, int *queue_head,
                                                         int words, int max_chunks,
                                                         uint32_t region_bytes) {
  extern __shared__ __align__(128) unsigned char smem_bc[];
  __shared__ ColonyDev s_desc;
  __shared__ int s_item, s_ok;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, warps = blockDim.x >> 5;
  uint32_t *tabu = reinterpret_cast<uint32_t *>(smem_bc) +
                   (size_t)warp * (words + 32 + (MULTI ? max_chunks : 0));
  float *wbuf = reinterpret_cast<float *>(tabu + words);
  float *cend = wbuf + 32;
  float *swbuf = reinterpret_cast<float *>(smem_bc + region_bytes) + (size_t)warp * 32;
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem_bc + region_bytes + (size_t)warps * 128);
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    fence_barrier_init();
  }
  __syncthreads();
  uint32_t phase = 0;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(queue_head, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= num_items) break;
    const int4 w = items[it];
    if (threadIdx.x == 0) s_desc = descs[w.x];
    __syncthreads();
    const ColonyDev &c = s_desc;
    if (!MULTI && w.w) {
      const int n = c.n;
      const StagedLayout L = staged_layout(n, c.ld, 4 * G, AGING);
      float *scw = reinterpret_cast<float *>(smem_bc);
      int16_t *sids = reinterpret_cast<int16_t *>(smem_bc + L.ids_off);
      float *smean = reinterpret_cast<float *>(smem_bc + L.mean_off);
      if (threadIdx.x == 0) {
        // The previous item's reads of the region (generic proxy) come
        // before the copies' writes (async proxy).
        fence_proxy_async();
        const uint32_t cw_bytes = (uint32_t)L.ids_off;
        const uint32_t id_bytes = (uint32_t)(L.mean_off - L.ids_off);
        const uint32_t mean_bytes = AGING ? (uint32_t)c.ld * 4u : 0u;
        mbar_arrive_expect_tx(bar, cw_bytes + id_bytes + mean_bytes);
        constexpr uint32_t kPiece = 32768;
        const char *g = reinterpret_cast<const char *>(c.choice_nn);
        for (uint32_t o = 0; o < cw_bytes; o += kPiece)
          tma_load_1d(reinterpret_cast<char *>(scw) + o, g + o, min(kPiece, cw_bytes - o), bar);
        g = reinterpret_cast<const char *>(c.nn16);
        for (uint32_t o = 0; o < id_bytes; o += kPiece)
          tma_load_1d(reinterpret_cast<char *>(sids) + o, g + o, min(kPiece, id_bytes - o), bar);
        if (AGING) tma_load_1d(smean, c.mean, mean_bytes, bar);
        bool ok = mbar_wait_bounded(bar, phase, c.st);
        // After a timeout, wait (bounded again) for the copies still in
        // flight before the CTA stops taking items.
        if (!ok) mbar_wait_bounded(bar, phase, c.st);
        s_ok = ok ? 1 : 0;
      }
      phase ^= 1u;
      __syncthreads();
      if (!s_ok) break;
      if (warp < w.z) {
        if (n <= 1024)
          construct_ant_staged<AGING, 1, G, TableRows<4 * G>, 4, true>(
              c, w.y + warp, c.st->iteration, swbuf, TableRows<4 * G>{sids, scw, smean}, lane);
        else
          construct_ant_staged<AGING, 2, G, TableRows<4 * G>, 4, true>(
              c, w.y + warp, c.st->iteration, swbuf, TableRows<4 * G>{sids, scw, smean}, lane);
      }
    } else if (!MULTI && c.nn16 && c.ldk == 4 * G && c.n <= 2048) {
      // Too large to stage: the same step loop on rows read from L2.
      if (warp < w.z)
        construct_ant_staged<AGING, 2, G, TableRows<4 * G>, 4, true>(
            c, w.y + warp, c.st->iteration, swbuf,
            TableRows<4 * G>{c.nn16, c.choice_nn, c.mean}, lane);
    } else if (warp < w.z) {
      construct_ant<MULTI, AGING, false>(c, w.y + warp, c.st->iteration, tabu, cend, wbuf,
                                         nullptr, nullptr, nullptr, (c.K + 31) >> 5, lane);
    }
    __syncthreads();  // s_item, s_desc and the region are rewritten by the next item
  }
}

// Bytes of the shared region: the largest staged table of the batch, or the
// per-warp tabu lists of L2-row items, whichever is larger (128-byte
// multiple).
size_t batch_region_bytes(int max_n, int max_k, int warps, size_t max_table) {
  const int words = (max_n + 31) / 32;
  const int chunks = (max_k + 31) / 32;
  const size_t tabu = (size_t)warps * (words + 32 + (max_k > 32 ? chunks : 0)) * 4;
  return ((tabu > max_table ? tabu : max_table) + 127) / 128 * 128;
}

size_t batch_construct_smem_bytes(size_t region_bytes, int warps) {
  return region_bytes + (size_t)warps * 128 + 16;
}

size_t batch_staged_table_bytes(int n, int ld, int sp, bool aging) {
  return staged_layout(n, ld, sp, aging).table;
}

namespace {
template <bool MULTI, bool AGING, int G>
cudaError_t batch_attr(int v) {
  return cudaFuncSetAttribute(k_batch_construct<MULTI, AGING, G>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, v);
}
template <bool MULTI, bool AGING, int G>
cudaError_t batch_launch(const ColonyDev *descs, const int4 *items, int num_items, int *queue_head,
                         int grid, int warps, size_t smem, int words, int chunks, uint32_t rb,
                         cudaStream_t s) {
  k_batch_construct<MULTI, AGING, G><<<grid, warps * 32, smem, s>>>(descs, items, num_items,
                                                                   queue_head, words, chunks, rb);
  return cudaGetLastError();
}
template <bool AGING, int G>
const void *batch_fn(bool multi) {
  return multi ? (const void *)k_batch_construct<true, AGING, 8>
               : (const void *)k_batch_construct<false, AGING, G>;
}
const void *batch_fn_for(bool multi, int sp, bool aging) {
  switch (sp) {
    case 16: return aging ? batch_fn<true, 4>(multi) : batch_fn<false, 4>(multi);
    case 20: return aging ? batch_fn<true, 5>(multi) : batch_fn<false, 5>(multi);
    case 24: return aging ? batch_fn<true, 6>(multi) : batch_fn<false, 6>(multi);
    default: return aging ? batch_fn<true, 8>(multi) : batch_fn<false, 8>(multi);
  }
}
}  // namespace

cudaError_t configure_batch_construct(size_t smem) {
  const int v = (int)smem;
  cudaError_t e = batch_attr<true, true, 8>(v);
  if (e == cudaSuccess) e = batch_attr<true, false, 8>(v);
  if (e == cudaSuccess) e = batch_attr<false, true, 4>(v);
  if (e == cudaSuccess) e = batch_attr<false, false, 4>(v);
  if (e == cudaSuccess) e = batch_attr<false, true, 5>(v);
  if (e == cudaSuccess) e = batch_attr<false, false, 5>(v);
  if (e == cudaSuccess) e = batch_attr<false, true, 6>(v);
  if (e == cudaSuccess) e = batch_attr<false, false, 6>(v);
  if (e == cudaSuccess) e = batch_attr<false, true, 8>(v);
  if (e == cudaSuccess) e = batch_attr<false, false, 8>(v);
  return e;
}

int batch_construct_blocks_per_sm(int warps, size_t smem, bool multi, int sp, bool aging) {
  int blocks = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, batch_fn_for(multi, sp, aging),
                                                    warps * 32, smem) != cudaSuccess)
    return 1;
  return blocks > 0 ? blocks : 1;
}

cudaError_t launch_batch_construct(const ColonyDev *descs, const int4 *items, int num_items,
                                   int *queue_head, int grid, int warps, int max_n, int max_k,
                                   size_t region_bytes, int sp, bool aging, cudaStream_t s) {
  const int words = (max_n + 31) / 32;
  const int chunks = (max_k + 31) / 32;
  const size_t smem = batch_construct_smem_bytes(region_bytes, warps);
  const uint32_t rb = (uint32_t)region_bytes;
  if (max_k > 32)
    return aging ? batch_launch<true, true, 8>(descs, items, num_items, queue_head, grid, warps,
                                               smem, words, chunks, rb, s)
                 : batch_launch<true, false, 8>(descs, items, num_items, queue_head, grid, warps,
                                                smem, words, chunks, rb, s);
#define ACO_BATCH_CASE(PITCH, GG)                                                            \
  case PITCH:                                                                                \
    return aging ? batch_launch<false, true, GG>(descs, items, num_items, queue_head, grid,   \
                                                 warps, smem, words, chunks, rb, s)           \
                 : batch_launch<false, false, GG>(descs, items, num_items, queue_head, grid,  \
                                                  warps, smem, words, chunks, rb, s);
  switch (sp) {
    ACO_BATCH_CASE(16, 4)
    ACO_BATCH_CASE(20, 5)
    ACO_BATCH_CASE(24, 6)
    default:
    ACO_BATCH_CASE(32, 8)
  }
#undef ACO_BATCH_CASE
}

}  // namespace aco
