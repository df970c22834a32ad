// k_construct_rows.cu -- tour construction over long candidate rows (k > 32,
// the reference's full-row roulette included).
//
// Replaces the reference CPU step calculateProbabilityOfSelection +
// selectCities / chooseBestNext (src/Colony.cu:795-864) and the GPU kernels
// dev_compute_probabilities / dev_reduce_probabilities_s / dev_move_ants
// (inc/Colony.cuh:193-229,290-347; src/Colony.cu:643-685).  The reference
// walks all n entries of the current city's nn row for every ant and step:
// it adds the weight of every unvisited entry, in row order, into sum_prob,
// then walks the same entries again until the running sum exceeds
// u * sum_prob.  Visited entries carry weight 0, and adding +0 leaves a
// non-negative float sum unchanged, so the same bits come out of a walk over
// the non-zero weights alone, in row order.
//
// The sequential float sum is the step's critical path: one dependent add
// per unvisited city of the row, about n^2/2 adds per tour, which no
// reordering may shorten without changing the rounding.  The kernel is built
// around it.  A CTA holds A ants (A <= kRowsMaxAnts) of one instance, all at
// the same step, and A + 1 warps:
//
//  * scan warp a (one per ant): reads the row it needs straight from L2
//    (choice values, or tau and eta for an ant that blends its fitness, and
//    the int16 city ids; 16-byte loads, eight 128-entry chunks in flight a
//    lane), zeroes the weights of visited cities (a byte per city in shared
//    memory) and compacts the non-zero weights, in row order, into one of the
//    ant's two buffers (a lane's offset is the count of the lanes before it,
//    from three ballots of the count bits).  Rows of up to 1024 entries keep
//    no city ids there: the guess (below) keeps its index instead;
//  * the chain warp: lane a adds ant a's compacted weights in order,
//    s = fl(s + w) (sum_prob += prob_ptr[i], partial_sum += prob_ptr[i],
//    src/Colony.cu:814,840), records the sum at the end of every 32 entries
//    and the total S, then finds ant a's exact pick (below), forming the
//    running sums of the one block it needs again from that block's start.  The A chains and picks share one
//    instruction stream.
//
// One step: the scan warps hand their buffers, with the step's uniform u,
// to the chain warp (named barrier R).  While the chain runs, each scan warp
// compacts the row of its guessed pick into its other buffer, and from that
// row's weights, still in registers, guesses the pick after it (an
// approximate prefix: chunk sums, a scan over chunks and lanes, the same
// crossing rule); it then issues the loads of that guessed row into the
// registers the scan just freed, so they are in flight while it waits for
// the chain and passes the barriers.  After its chain, lane a of the chain
// warp finds ant a's exact pick: rnd = fl(u * S) (src/Colony.cu:826-828);
// the first 32-entry block whose recorded end sum exceeds rnd, then in that
// block the first running sum with !(sum <= rnd) -- written sum > rnd || rnd
// is NaN, as in the k <= 32 step loop -- is the pick (sums never decrease,
// so both are binary searches), and hands it back with named barrier C, a
// bar.red that also tells every scan warp whether every pick of the CTA was
// its guess (the common case reads nothing back).  No crossing (S <= 0,
// u * S rounding to S, or S = +inf from an infinite weight) takes the
// fallback, as the reference does (chooseBestNext / select_local_best).
// A right guess (nearly always: the approximate and the exact prefix differ
// by a few ulps) leaves the next row compacted before the chain ends, so row
// loads and scans stay off the critical path; a wrong one is undone, the
// pick's city found again from its index (rows without ids: the row's
// unvisited entries counted again) and its row scanned.  (The rows once went
// through shared memory by TMA bulk copies, one row ahead; reading them from
// L2 in the scan, with eight loads in flight a lane, measured faster and
// needs no mbarriers.)
//
// Every warp of a CTA passes the two named barriers once per step, n - 1
// steps per item, with no early exit: an inconsistency is recorded in the
// colony's error word and the step continues on a stand-in city.  The
// kernel has no other wait.
#include "k_construct_steps.cuh"

namespace aco {

// ---- shared-memory layout -------------------------------------------------

// Per-ant region (rows_ant_bytes, a multiple of 128 plus 16 so the regions of
// consecutive ants start four banks apart and the chain warp's 16-byte reads
// of A buffers at once spread over the banks; offsets in rows_layout).
// S = rows_slots(K), P = ldk:
//   w[2]:  2 x S f32        compacted weights (two buffers)
//   id[2]: 2 x S int16      their city ids (rows longer than 1024 entries)
//   bend:  S/32 f32         running sum at the end of every 32 entries
//   tw:    tabu bits        visited cities, 32 a word (words padded to 4),
//                           rebuilt from the bytes by the fallback, which
//                           scans them
//   tb:    tabu bytes       visited cities, 0xff or 0 (the scan's lookups: a
//                           sign-extended byte is the AND mask itself)
// Buffer b is addressed arithmetically (no array of pointers, which a
// run-time index would move to local memory).
//
// Entry i of a compacted buffer (weights, sums and ids alike) sits in slot
// i / 4 at component (i % 4) ^ ((i / 32) % 4) (rows_swz).  A chunk's stores
// put lane l's entries near entry 4l, so lanes l, l + 8, l + 16, l + 24 would
// hit one bank; the key, which differs between them, spreads them over four.
// Within a block of 32 entries the key is constant, so a reader of whole
// blocks undoes it with a fixed permutation.
struct RowsAnt {
  float *w0;
  int16_t *id0;
  float *bend;
  uint32_t *tw;
  uint8_t *tb;
  int S;
  __device__ __forceinline__ float *w(int b) const { return w0 + b * S; }
  __device__ __forceinline__ int16_t *id(int b) const { return id0 + b * S; }
};

__device__ __forceinline__ RowsAnt rows_ant_at(unsigned char *base, int n, int K) {
  const RowsLayout L = rows_layout(n, K);
  RowsAnt r;
  r.S = L.S;
  r.w0 = reinterpret_cast<float *>(base);
  r.id0 = reinterpret_cast<int16_t *>(base + L.id_off);
  r.bend = reinterpret_cast<float *>(base + L.bend_off);
  r.tw = reinterpret_cast<uint32_t *>(base + L.tw_off);
  r.tb = base + L.tb_off;
  return r;
}

__device__ __forceinline__ int rows_swz(int i) { return i ^ ((i >> 5) & 3); }

// Chain length of step x: the entries a compacted buffer can hold at that
// step (at most min(K, n - x) non-zero weights), rounded up to whole blocks
// of 32; every buffer is zero-padded to it.
__device__ __forceinline__ int rows_chain_len(int K, int n, int x) {
  const int c = K < n - x ? K : n - x;
  return (c + 31) & ~31;
}

__device__ __forceinline__ void named_bar_sync(int id, int threads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(threads) : "memory");
}
__device__ __forceinline__ void named_bar_arrive(int id, int threads) {
  asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(threads) : "memory");
}
constexpr int kBarRowsReady = 1, kBarChainDone = 2;

// ---- scan warp: compaction -------------------------------------------------

// Visited masking of one chunk (four consecutive row positions p0 .. p0+3 of
// this lane): bit t of the result is set where entry t is an unvisited city
// (inside the first K positions); the weights (bits) of the others become 0.
// Every unvisited entry is kept, a zero weight too: adding +0 changes no
// running sum, and an entry whose sum does not rise is never the pick.  Ids
// past K (-1 in the table) are replaced by city 0 so the lookup stays in the
// list.
template <bool PARTIAL>
__device__ __forceinline__ unsigned rows_mask4(uint4 &wbits, uint2 &ip, int p0, int K,
                                               const uint8_t *tb) {
  uint32_t id[4] = {ip.x & 0xffffu, ip.x >> 16, ip.y & 0xffffu, ip.y >> 16};
  uint32_t wb[4] = {wbits.x, wbits.y, wbits.z, wbits.w};
  unsigned keep = 0u;
#pragma unroll
  for (int t = 0; t < 4; t++) {
    if (PARTIAL && p0 + t >= K) id[t] = 0u;
    uint32_t m = (uint32_t)(int32_t)(int8_t)tb[id[t]];  // 0, or all ones if visited
    if (PARTIAL && p0 + t >= K) m = ~0u;
    wb[t] &= ~m;
    keep |= ~m & (1u << t);
  }
  wbits = make_uint4(wb[0], wb[1], wb[2], wb[3]);
  if (PARTIAL) ip = make_uint2(id[0] | (id[1] << 16), id[2] | (id[3] << 16));
  return keep;
}

// Approximate pick of a row still in registers (one round of JB = 8 chunks
// of 128 entries): the chunk sums (a transposing butterfly: each of three
// levels hands half of a lane's chunk sums to its partner, so lane l ends
// with a partial sum of chunk l >> 2, then two plain levels), gathered into
// every lane and scanned there, the first chunk where the running total
// passes u * S', then within it the lanes' inclusive scan and the entry of
// the first lane that passes.
// Any summation order will do: the guess only decides which row is scanned
// early.  Returns the city, or -1, and its position in the round (128 js +
// 4 lane + t) in pos.
template <int JB>
__device__ __forceinline__ int rows_guess_regs(const uint4 (&q)[JB], const uint2 (&ip)[JB],
                                               float u, int lane, int &pos) {
  static_assert(JB == 8, "the transposing butterfly assumes eight chunks");
  float ls[JB];
#pragma unroll
  for (int j = 0; j < JB; j++)
    ls[j] = (__uint_as_float(q[j].x) + __uint_as_float(q[j].y)) +
            (__uint_as_float(q[j].z) + __uint_as_float(q[j].w));
  const bool h4 = (lane >> 4) & 1, h3 = (lane >> 3) & 1, h2 = (lane >> 2) & 1;
  float t4[4];
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const float keep = h4 ? ls[i + 4] : ls[i], give = h4 ? ls[i] : ls[i + 4];
    t4[i] = keep + __shfl_xor_sync(kFull, give, 16);
  }
  float t2[2];
#pragma unroll
  for (int i = 0; i < 2; i++) {
    const float keep = h3 ? t4[i + 2] : t4[i], give = h3 ? t4[i] : t4[i + 2];
    t2[i] = keep + __shfl_xor_sync(kFull, give, 8);
  }
  float t1;
  {
    const float keep = h2 ? t2[1] : t2[0], give = h2 ? t2[0] : t2[1];
    t1 = keep + __shfl_xor_sync(kFull, give, 4);
  }
  t1 += __shfl_xor_sync(kFull, t1, 2);
  t1 += __shfl_xor_sync(kFull, t1, 1);  // lane l: the sum of chunk l >> 2
  // Every lane gathers the eight chunk sums (lane 4c holds chunk c's) and
  // scans them itself: the same values in every lane, so js is uniform.
  float ct[JB];
#pragma unroll
  for (int cc = 0; cc < JB; cc++) ct[cc] = __shfl_sync(kFull, t1, 4 * cc);
  const float S = ((ct[0] + ct[1]) + (ct[2] + ct[3])) + ((ct[4] + ct[5]) + (ct[6] + ct[7]));
  const bool s_ok = S > 0.0f && S < INFINITY;
  const float rnd = u * S;
  int js = -1;
  float base = 0.0f, acc0 = 0.0f;
#pragma unroll
  for (int cc = 0; cc < JB; cc++) {
    const float nx = acc0 + ct[cc];
    if (js < 0 && nx > rnd) {
      js = cc;
      base = acc0;
    }
    acc0 = nx;
  }
  const bool hc = js >= 0;
  if (js < 0) js = 0;
  // Chunk js's registers, by a (warp-uniform) branch rather than a chain of
  // selects over all eight chunks.
  float x;
  uint4 qq;
  uint2 ii;
  switch (js) {
#define ACO_GUESS_CHUNK(J) \
  case J:                  \
    x = ls[J];             \
    qq = q[J];             \
    ii = ip[J];            \
    break;
    ACO_GUESS_CHUNK(0)
    ACO_GUESS_CHUNK(1)
    ACO_GUESS_CHUNK(2)
    ACO_GUESS_CHUNK(3)
    ACO_GUESS_CHUNK(4)
    ACO_GUESS_CHUNK(5)
    ACO_GUESS_CHUNK(6)
    default:
      x = ls[7];
      qq = q[7];
      ii = ip[7];
      break;
#undef ACO_GUESS_CHUNK
  }
  float incl = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const float y = __shfl_up_sync(kFull, incl, o);
    if (lane >= o) incl += y;
  }
  incl += base;
  const unsigned hit = __ballot_sync(kFull, incl > rnd);
  const int l = hit ? __ffs(hit) - 1 : 0;
  const float w[4] = {__uint_as_float(qq.x), __uint_as_float(qq.y), __uint_as_float(qq.z),
                      __uint_as_float(qq.w)};
  const int id[4] = {(int)(ii.x & 0xffffu), (int)(ii.x >> 16), (int)(ii.y & 0xffffu),
                     (int)(ii.y >> 16)};
  float acc = incl - x;
  int city = -1, tc = 0;
#pragma unroll
  for (int t = 0; t < 4; t++) {
    acc += w[t];
    const bool take = city < 0 && w[t] != 0.0f && acc > rnd;
    city = take ? id[t] : city;
    tc = take ? t : tc;
  }
  city = __shfl_sync(kFull, city, l);
  pos = js * 128 + l * 4 + __shfl_sync(kFull, tc, l);
  return (s_ok && hc && hit) ? city : -1;
}

// Approximate pick of a compacted buffer (rows of more than 128 JB entries):
// block sums of 32 entries (each lane one block, its eight 16-byte reads in
// a lane-rotated order so the lanes spread over the banks), their inclusive
// warp scan, the first block past u * S', then within it the lanes'
// masked-FMA prefixes from the block's approximate start.  NR rounds of 32
// blocks (cnt <= 1024 NR).  Returns the city, or -1.
template <int NR>
__device__ __forceinline__ int rows_guess_smem(const float *w, const int16_t *id, int cnt, float u,
                                               int lane) {
  if (cnt <= 0 || cnt > 1024 * NR) return -1;
  const float4 *w4 = reinterpret_cast<const float4 *>(w);
  float bs[NR];
#pragma unroll
  for (int r = 0; r < NR; r++) {
    const int b = r * 32 + lane;
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
    if (b * 32 < cnt) {
#pragma unroll
      for (int g = 0; g < 8; g++) {
        const float4 v = w4[b * 8 + ((g + lane) & 7)];  // zero-padded past cnt
        s0 += v.x;
        s1 += v.y;
        s2 += v.z;
        s3 += v.w;
      }
    }
    bs[r] = (s0 + s1) + (s2 + s3);
  }
  float carry = 0.0f, incl[NR];
#pragma unroll
  for (int r = 0; r < NR; r++) {
    float x = bs[r];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const float y = __shfl_up_sync(kFull, x, o);
      if (lane >= o) x += y;
    }
    incl[r] = carry + x;
    carry += __shfl_sync(kFull, x, 31);
  }
  const float S = carry;
  if (!(S > 0.0f) || !(S < INFINITY)) return -1;
  const float rnd = u * S;
  int blk = -1;
  float start = 0.0f;
#pragma unroll
  for (int r = 0; r < NR; r++) {
    const unsigned hit = __ballot_sync(kFull, (r * 32 + lane) * 32 < cnt && incl[r] > rnd);
    if (hit && blk < 0) {
      const int l = __ffs(hit) - 1;
      blk = r * 32 + l;
      start = __shfl_sync(kFull, incl[r] - bs[r], l);
    }
  }
  if (blk < 0) return -1;
  float acc = start;
  const float *b1 = w + blk * 32;
  const int key = blk & 3;
#pragma unroll
  for (int e = 0; e < 32; e++) acc = __fmaf_rn(b1[e ^ key], e <= lane ? 1.0f : 0.0f, acc);
  const unsigned hit = __ballot_sync(kFull, blk * 32 + lane < cnt && acc > rnd);
  if (!hit) return -1;
  return id[rows_swz(blk * 32 + __ffs(hit) - 1)];
}

struct RowsScan {
  int cnt;    // non-zero weights written
  int guess;  // approximate pick (u >= 0), or -1
  int gidx;   // its index in the compacted buffer (rows of one round)
};

// Loads round j0 of a city's row from L2 into registers: lane l takes row
// positions j0 + 128j + 4l .. +3 of chunk j (16-byte weight loads, 8-byte id
// loads, all JB chunks before any use).  For an ant that blends its fitness
// the weights are formed from tau and eta as they arrive.  Round 0 of the
// next step's row is loaded ahead this way, across the barriers (its
// registers stay live through the whole step): loading only half of it
// ahead measured slower, and so did freeing registers for more ants a CTA
// (13 to 15 ants spill at their lower register cap).
template <int JB>
__device__ __forceinline__ void rows_load(const ColonyDev &c, int city, int j0, bool blend,
                                          float meanc, float ratio, int lane, uint4 (&q)[JB],
                                          uint2 (&ip)[JB]) {
  const int K = c.K;
  const float *erow = c.eta_nn + (size_t)city * c.ldk;
  const float *grow = (blend ? c.tau_nn : c.choice_nn) + (size_t)city * c.ldk;
  const int16_t *irow = c.nn16 + (size_t)city * c.ldk;
#pragma unroll
  for (int j = 0; j < JB; j++) {
    const int p0 = j0 + j * 128 + lane * 4;
    const bool in = p0 < K;  // p0 < K <= ldk, ldk % 4 == 0: the four entries are in the row
    ip[j] = in ? __ldg(reinterpret_cast<const uint2 *>(irow + p0)) : make_uint2(0u, 0u);
    if (!blend) {
      q[j] = in ? __ldg(reinterpret_cast<const uint4 *>(grow + p0)) : make_uint4(0, 0, 0, 0);
    } else {
      const float4 t = in ? __ldg(reinterpret_cast<const float4 *>(grow + p0))
                          : make_float4(0.f, 0.f, 0.f, 0.f);
      const float4 e = in ? __ldg(reinterpret_cast<const float4 *>(erow + p0))
                          : make_float4(0.f, 0.f, 0.f, 0.f);
      q[j].x = __float_as_uint(blend_fitness(t.x, e.x, meanc, ratio, c.use_alpha, c.alpha));
      q[j].y = __float_as_uint(blend_fitness(t.y, e.y, meanc, ratio, c.use_alpha, c.alpha));
      q[j].z = __float_as_uint(blend_fitness(t.z, e.z, meanc, ratio, c.use_alpha, c.alpha));
      q[j].w = __float_as_uint(blend_fitness(t.w, e.w, meanc, ratio, c.use_alpha, c.alpha));
    }
  }
}

// Steps of the header for the row of `city`: into wo (and the city ids
// into io when IDS), zero-padded to L; with u >= 0 also the approximate pick
// of that row.  Rows of one round (K <= 128 JB) keep no ids: the guess's
// index in the compacted buffer stands for it.  JB chunks of 128
// entries per round, in q/ip: all of a round's loads first (round 0's already
// issued by the caller when `loaded`), then every chunk's visited lookups,
// then the ballots of every chunk, then the compacting stores.
template <int JB, bool IDS>
__device__ __forceinline__ RowsScan rows_scan(const ColonyDev &c, const RowsAnt &ra, int city,
                                              bool blend, float meanc, float ratio, float *wo,
                                              int16_t *io, int L, float u, int lane,
                                              uint4 (&q)[JB], uint2 (&ip)[JB], bool loaded) {
  const int K = c.K;
  RowsScan r;
  r.cnt = 0;
  r.guess = -1;
  r.gidx = -1;
#pragma unroll 1
  for (int j0 = 0; j0 < K; j0 += JB * 128) {
    unsigned nz = 0u;  // keep bits, four a chunk: chunk j at bits 4j .. 4j+3
    if (!(loaded && j0 == 0))  // round 0 may be in q/ip already
      rows_load<JB>(c, city, j0, blend, meanc, ratio, lane, q, ip);
#pragma unroll
    for (int j = 0; j < JB; j++) {
      const int c0 = j0 + j * 128;
      if (c0 < K) {  // warp-uniform
        if (c0 + 128 <= K)
          nz |= rows_mask4<false>(q[j], ip[j], c0 + lane * 4, K, ra.tb) << (4 * j);
        else
          nz |= rows_mask4<true>(q[j], ip[j], c0 + lane * 4, K, ra.tb) << (4 * j);
      } else {
        q[j] = make_uint4(0, 0, 0, 0);
      }
    }
    int gpos = -1;
    if (u >= 0.0f && K <= JB * 128) r.guess = rows_guess_regs<JB>(q, ip, u, lane, gpos);
    const int gj = r.guess >= 0 ? gpos >> 7 : -1, gt = gpos & 3;
    int gi = -1;  // the guess's compacted index, in the lane that holds it
    // Chunk by chunk: a lane's offset is the count of the lanes before it,
    // from three ballots of the count bits; every entry is stored (no
    // branch): a kept one at its place, a dropped one at this lane's sink
    // slot past any chain length.
    const unsigned lt = (1u << lane) - 1u;
    const int sink = ra.S - 32 + lane;
#pragma unroll
    for (int j = 0; j < JB; j++) {
      const unsigned kp = (nz >> (4 * j)) & 0xfu;
      const int cl = __popc(kp);
      const unsigned b0 = __ballot_sync(kFull, cl & 1), b1 = __ballot_sync(kFull, cl & 2),
                     b2 = __ballot_sync(kFull, cl & 4);
      const int o = r.cnt + __popc(b0 & lt) + 2 * __popc(b1 & lt) + 4 * __popc(b2 & lt);
      const int rk[4] = {0, (int)(kp & 1u), (int)(kp & 1u) + (int)((kp >> 1) & 1u),
                         __popc(kp & 7u)};
      const uint32_t wb[4] = {q[j].x, q[j].y, q[j].z, q[j].w};
      const int16_t id[4] = {(int16_t)(ip[j].x & 0xffffu), (int16_t)(ip[j].x >> 16),
                             (int16_t)(ip[j].y & 0xffffu), (int16_t)(ip[j].y >> 16)};
#pragma unroll
      for (int t = 0; t < 4; t++) {
        const int e = rows_swz(((kp >> t) & 1u) ? o + rk[t] : sink);
        wo[e] = __uint_as_float(wb[t]);
        if (IDS) io[e] = id[t];
      }
      if (!IDS && j == gj) gi = o + __popc(kp & ((1u << gt) - 1u));
      r.cnt += __popc(b0) + 2 * __popc(b1) + 4 * __popc(b2);
    }
    if (!IDS && gj >= 0) r.gidx = __shfl_sync(kFull, gi, (gpos >> 2) & 31);
  }
  for (int i = r.cnt + lane; i < L; i += 32) wo[rows_swz(i)] = 0.0f;
  if (u >= 0.0f && K > JB * 128) {
    __syncwarp();
    r.guess = rows_guess_smem<2>(wo, io, r.cnt, u, lane);
  }
  return r;
}

// Exact pick (see the header) of one ant by one lane: rnd = fl(u * S), the
// first block of 32 whose recorded end sum passes rnd (the sums never
// decrease, so a binary search, a fixed number of steps in every lane), then
// in that block the first entry whose running sum has !(sum <= rnd): the
// block's running sums formed again from the sum at the end of the block
// before, by the chain's own adds in the chain's own order, so the same bits.
// Entries past cnt (the padding adds zeros) are not candidates; a NaN rnd
// (u = 0 with S = +inf, or a NaN sum) passes at the first entry.  Index, or
// -1.
__device__ __forceinline__ int rows_exact_lane(const float *w, const float *bend, int cnt, int L,
                                               float S, float u) {
  if (S <= 0.0f) return -1;  // chooseBestNext (src/Colony.cu:776-778)
  const float rnd = __fmul_rn(u, S);
  const int nb = L >> 5;
  if (rnd != rnd) return (nb > 0 && cnt > 0) ? 0 : -1;
  int blk = 0;  // blocks whose end sum is <= rnd
  int step = 1;
  while (step * 2 <= nb) step *= 2;
  for (; step > 0; step >>= 1)
    if (blk + step <= nb && bend[blk + step - 1] <= rnd) blk += step;
  if (blk >= nb) return -1;
  // The block's last running sum is bend[blk] > rnd, so one entry passes.
  const float *wb = w + blk * 32;
  const int key = blk & 3;
  float s = blk > 0 ? bend[blk - 1] : 0.0f;
  int e = 31;
#pragma unroll 1
  for (int t = 0; t < 32; t++) {
    s = __fadd_rn(s, wb[t ^ key]);
    if (s > rnd) {
      e = t;
      break;
    }
  }
  const int i = blk * 32 + e;
  return i < cnt ? i : -1;
}

// Marks (or unmarks) a city visited.  The step path keeps the tabu bytes
// only (a plain store, no read-modify-write of a bit word).
__device__ __forceinline__ void tb_set(uint8_t *tb, int city, bool on, int lane) {
  __syncwarp();
  if (lane == 0) tb[city] = on ? 0xffu : 0u;
  __syncwarp();
}

// The fallback (rare): out of line, so its code stays out of the step loop's
// instruction stream.  It first rebuilds the tabu bits it scans from the
// tabu bytes (bits of cities >= n stay 0).
__device__ __noinline__ int rows_fallback(const ColonyDev &c, int cur, uint32_t *tw,
                                          const uint8_t *tb, AntCtx a, int lane) {
  const int n = c.n;
  __syncwarp();
  for (int w = lane; w < (n + 31) / 32; w += 32) {
    uint32_t bits = 0u;
    for (int i = 0; i < 32 && w * 32 + i < n; i++)
      if (tb[w * 32 + i]) bits |= 1u << i;
    tw[w] = bits;
  }
  __syncwarp();
  return fallback_city(c, cur, tw, a, lane);
}

// The city of entry idx of the compacted buffer of `city`'s row, for rows of
// one round that keep no ids (a pick that was not the guess: rare).  The
// kept entries are the positions below K whose city is unvisited, in row
// order, and the tabu bytes are as they were when the row was compacted
// (the guess's mark is undone first), so counting them again finds it.
__device__ __noinline__ int rows_city_at(const ColonyDev &c, const uint8_t *tb, int city, int idx,
                                         int lane) {
  const int K = c.K;
  const int16_t *irow = c.nn16 + (size_t)city * c.ldk;
  __syncwarp();
  int base = 0;
  for (int c0 = 0; c0 < K; c0 += 128) {
    int id[4];
    unsigned kp = 0u;
#pragma unroll
    for (int t = 0; t < 4; t++) {
      const int p = c0 + lane * 4 + t;
      id[t] = p < K ? (int)irow[p] : 0;
      if (p < K && tb[id[t]] == 0u) kp |= 1u << t;
    }
    const int cl = __popc(kp);
    int inc = cl;  // inclusive scan of the counts over the lanes
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(kFull, inc, o);
      if (lane >= o) inc += y;
    }
    const int tot = __shfl_sync(kFull, inc, 31);
    if (idx < base + tot) {
      int r = idx - base - (inc - cl);  // rank among this lane's kept entries
      int found = -1;
      if (r >= 0 && r < cl) {
#pragma unroll
        for (int t = 0; t < 4; t++) {
          if ((kp >> t) & 1u) {
            if (r == 0 && found < 0) found = id[t];
            r--;
          }
        }
      }
      const unsigned m = __ballot_sync(kFull, found >= 0);
      return m ? __shfl_sync(kFull, found, __ffs(m) - 1) : -1;
    }
    base += tot;
  }
  return -1;
}

// Barrier `id` over `threads` threads that also returns the AND of every
// participant's predicate (bar.red.and); it orders shared memory as
// bar.sync does.
__device__ __forceinline__ bool named_bar_red_and(int id, int threads, bool pred) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\t"
      "bar.red.and.pred q, %2, %3, p;\n\tselp.u32 %0, 1, 0, q;\n\t}"
      : "=r"(r)
      : "r"((uint32_t)pred), "r"(id), "r"(threads)
      : "memory");
  return r != 0u;
}

// ---- chain warp --------------------------------------------------------------

// Adds one block of 32 entries (slot g, logical component t at physical
// component t ^ KEY), in order.
template <int KEY>
__device__ __forceinline__ void rows_chain_add32(const float4 (&a)[8], float &s) {
#pragma unroll
  for (int g = 0; g < 8; g++) {
    const float in[4] = {a[g].x, a[g].y, a[g].z, a[g].w};
#pragma unroll
    for (int t = 0; t < 4; t++) s = __fadd_rn(s, in[t ^ KEY]);
  }
}

// Lane a < A: the sequential sum of ant a's buffer w over L entries (a
// multiple of 32, zero-padded past its count), with the running sum at the
// end of every 32 entries in bend; returns the total S.  The running sums
// inside the blocks are not kept: the exact pick forms those of its one
// block again.  Four blocks of 32 per trip (their swizzle keys 0..3), each
// block's weights read while the previous block is added.
__device__ __forceinline__ float rows_chain(float *w, float *bend, int L) {
  float4 *w4 = reinterpret_cast<float4 *>(w);
  const int nb = L >> 5;
  float s = 0.0f;
  float4 a[8], v[8];
  if (nb > 0) {
#pragma unroll
    for (int g = 0; g < 8; g++) a[g] = w4[g];
  }
#define ACO_CHAIN_BLOCK(KEY, CUR, NXT)                                     \
  {                                                                        \
    const int bb = b + KEY;                                                \
    if (bb >= nb) break;                                                   \
    const int nx = bb + 1 < nb ? bb + 1 : bb;                              \
    _Pragma("unroll") for (int g = 0; g < 8; g++) NXT[g] = w4[nx * 8 + g]; \
    rows_chain_add32<KEY>(CUR, s);                                         \
    bend[bb] = s;                                                          \
  }
#pragma unroll 1
  for (int b = 0; b < nb; b += 4) {
    ACO_CHAIN_BLOCK(0, a, v)
    ACO_CHAIN_BLOCK(1, v, a)
    ACO_CHAIN_BLOCK(2, a, v)
    ACO_CHAIN_BLOCK(3, v, a)
  }
#undef ACO_CHAIN_BLOCK
  return s;
}

// ---- the kernel ----------------------------------------------------------------

// Per-CTA control block in static shared memory: which scan warps hold a
// valid ant, and per step what scan warp a hands the chain warp with its
// buffer (the step's uniform u, the buffer's count, its guess) and gets back
// (the pick).
struct RowsCtl {
  float u[kRowsMaxAnts];
  int cnt[kRowsMaxAnts];
  int key[kRowsMaxAnts];   // the guess: its city with ids, else its compacted index (-1: none)
  int next[kRowsMaxAnts];  // the pick, in the same terms
  int active[kRowsMaxAnts];
};

// One item: ants `first` .. `first + count - 1` of the colony (positions in
// the aging plan's list when PLAN: the valid ants come first), all warps of
// the CTA.  `region` holds the A per-ant regions.
template <bool AGING, bool PLAN, bool IDS>
__device__ __forceinline__ void rows_item(const ColonyDev &c, int first, int count, unsigned char *region,
                          size_t ant_bytes, RowsCtl &ctl) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int A = (blockDim.x >> 5) - 1;  // scan warps; warp A is the chain warp
  const int threads = blockDim.x;
  const int n = c.n, K = c.K;
  const uint32_t iter = c.st->iteration;

  if (warp < A) {
    // ---- scan warp: ant of this warp (if any), its aging state
    int k = -1;
    bool valid = false;
    AntCtx a;
    a.blend = false;
    a.ratio = 0.0f;
    a.meanc = 0.0f;
    if (warp < count) {
      const int pos = first + warp;
      if (PLAN) {
        k = c.plan[2 + pos];
        valid = pos < c.plan[0] + c.plan[1];
      } else {
        k = pos;
        valid = true;
      }
      if (AGING && !PLAN) {  // updateAntAges (src/Colony.cu:353-364)
        int age = 0;
        if (lane == 0) {
          age = c.age[k] + 1;
          c.age[k] = age;
        }
        age = __shfl_sync(kFull, age, 0);
        valid = c.valid[k] != 0;
      }
      if (AGING && valid) {
        const int age = c.age[k];
        a.blend = age < c.min_ret && c.st->isconverged;
        if (a.blend) a.ratio = __fdiv_rn(__int2float_rn(age), __int2float_rn(c.min_ret));
      }
      if (!valid) {  // an invalid ant keeps a cleared tour (src/Colony.cu:507-510)
        int32_t *trow = c.tours + (size_t)k * c.ld;
        for (int i = lane; i < n; i += 32) trow[i] = 0;
      }
    }
    if (lane == 0) ctl.active[warp] = valid ? 1 : 0;
    const RowsAnt ra =
        rows_ant_at(region + (size_t)warp * ant_bytes, n, K);
    int32_t *trow = valid ? c.tours + (size_t)k * c.ld : nullptr;
    uint32_t akey = 0;
    float ux = 0.0f;  // the uniform of the current step (drawn once)
    int cur = 0, start = 0, cnt = 0;
    int guess = -1;  // predicted pick of the current step (its row is scanned early)
    int gidx = -1;   // its index in the current buffer (rows without ids)
    // Round 0 of the row of city `pre`, loaded ahead (-1: none): issued once a
    // step's scan has stored its entries, in flight across the barriers.
    uint4 rq[8];
    uint2 rip[8];
    int pre = -1;
    int64_t fallbacks = 0;
    bool ok = true;
    if (valid) {
      for (int i = lane; i < (n + 31) / 32; i += 32) ra.tw[i] = 0u;
      for (int i = lane; i < (n + 15) / 16 * 4; i += 32) reinterpret_cast<uint32_t *>(ra.tb)[i] = 0u;
      akey = aco_ant_key(c.seed, iter, (uint32_t)k);
      start = __float2int_rz(__fmul_rn(aco_uniform_key(akey, 0u), __int2float_rn(n)));
      if (start >= n) {  // impossible for u < 1; recorded, clamped
        ok = false;
        start = n - 1;
      }
      cur = start;
      ux = aco_uniform_key(akey, 1u);
      tb_set(ra.tb, start, true, lane);
      if (lane == 0) trow[0] = start;
      if (AGING && a.blend) a.meanc = c.mean[start];
      const RowsScan r0 = rows_scan<8, IDS>(c, ra, start, a.blend, a.meanc, a.ratio, ra.w(0), ra.id(0),
                                       rows_chain_len(K, n, 1), n > 2 ? ux : -1.0f, lane, rq,
                                       rip, false);
      cnt = r0.cnt;
      if (r0.guess >= 0 && n > 2) {
        guess = r0.guess;
        gidx = r0.gidx;
      }
      if (guess >= 0 && !a.blend) {
        rows_load<8>(c, guess, 0, false, 0.0f, 0.0f, lane, rq, rip);
        pre = guess;
      }
    }
    int b = 0;
#pragma unroll 1
    for (int x = 1; x < n; x++) {
      if (lane == 0) {
        if (valid) {
          ctl.u[warp] = ux;
          ctl.cnt[warp] = cnt;
        }
        ctl.key[warp] = valid && guess >= 0 ? (IDS ? guess : gidx) : -1;
      }
      __syncwarp();
      named_bar_arrive(kBarRowsReady, threads);
      const float un = valid && x + 1 < n ? aco_uniform_key(akey, (uint32_t)(x + 1)) : 0.0f;
      // Pass 0 scans the guessed pick's row (while the chain warp runs the
      // chain and finds the exact pick); pass 1 scans the real pick's row
      // after a wrong or missing guess.  One call site of the scan serves both.
      RowsScan g;
      g.cnt = 0;
      g.guess = -1;
      g.gidx = -1;
      int todo = -1;  // city whose row goes into buffer b ^ 1 in this pass
      bool ahead = false, hit = false;
      int next = cur;
      if (valid) {
        if (guess >= 0) {  // its row is scanned while the chain runs (x + 1 < n)
          tb_set(ra.tb, guess, true, lane);
          todo = guess;
          ahead = true;
        }
      }
#pragma unroll 1
      for (int pass = 0; pass < 2; pass++) {
        if (todo >= 0) {
          const float m = (AGING && a.blend) ? c.mean[todo] : 0.0f;
          g = rows_scan<8, IDS>(c, ra, todo, a.blend, m, a.ratio, ra.w(b ^ 1), ra.id(b ^ 1),
                           rows_chain_len(K, n, x + 1), x + 2 < n ? un : -1.0f, lane, rq, rip,
                           todo == pre);
          if (!(x + 2 < n)) g.guess = -1;
          todo = -1;
          pre = -1;
          if (g.guess >= 0 && !a.blend) {  // the next step's row, loaded across the barriers
            rows_load<8>(c, g.guess, 0, false, 0.0f, 0.0f, lane, rq, rip);
            pre = g.guess;
          }
        }
        if (pass == 1) break;
        __syncwarp();
        // Once per step, in pass 0: every ant's pick equal to its guess (the
        // common case) needs no read of the pick.
        const bool all_hit = named_bar_red_and(kBarChainDone, threads, true);
        if (!valid) break;
        const int key = IDS ? guess : gidx;
        const int got = all_hit ? key : ctl.next[warp];
        hit = ahead && got >= 0 && got == key;
        next = hit ? guess : got;
        if (ahead && !hit) tb_set(ra.tb, guess, false, lane);  // undo the guess
        if (!IDS && !hit && got >= 0) next = rows_city_at(c, ra.tb, cur, got, lane);
        if (next < 0) {
          next = rows_fallback(c, cur, ra.tw, ra.tb, a, lane);
          fallbacks++;
        }
        if ((unsigned)next >= (unsigned)n || (!hit && ra.tb[next])) {
          ok = false;  // no unvisited city, or a bad id: cannot happen
          next = cur;
        }
        if (!hit) tb_set(ra.tb, next, true, lane);
        if (lane == 0) trow[x] = next;
        if (AGING && a.blend) a.meanc = c.mean[next];
        if (!hit && x + 1 < n) todo = next;
      }
      if (valid) {
        cnt = g.cnt;
        guess = g.guess;
        gidx = g.gidx;
        cur = next;
        ux = un;
      }
      b ^= 1;
    }
    if (valid) {
      __syncwarp();
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
          ok = false;
        }
      }
      for (int o = 16; o; o >>= 1) len += __shfl_xor_sync(kFull, len, o);
      if (!__all_sync(kFull, ok) && lane == 0) atomicOr(&c.st->error, kErrCheck);
      if (lane == 0) {
        c.newlen[k] = len;
        if (fallbacks)
          atomicAdd(reinterpret_cast<unsigned long long *>(&c.st->fallbacks),
                    (unsigned long long)fallbacks);
      }
    }
  } else {
    // ---- chain warp: lane a runs ant a's chain, then finds its exact pick
    int b = 0;
#pragma unroll 1
    for (int x = 1; x < n; x++) {
      named_bar_sync(kBarRowsReady, threads);
      bool hit = true;  // lanes without an ant vote yes
      if (lane < A && ctl.active[lane]) {
        const RowsAnt ra =
            rows_ant_at(region + (size_t)lane * ant_bytes, n, K);
        const int L = rows_chain_len(K, n, x);
        const float S = rows_chain(ra.w(b), ra.bend, L);
        const int i = rows_exact_lane(ra.w(b), ra.bend, ctl.cnt[lane], L, S, ctl.u[lane]);
        const int nx = IDS ? (i >= 0 ? ra.id(b)[rows_swz(i)] : -1) : i;
        ctl.next[lane] = nx;
        hit = nx >= 0 && nx == ctl.key[lane];
      }
      __syncwarp();
      named_bar_red_and(kBarChainDone, threads, hit);
      b ^= 1;
    }
  }
}

// Rows longer than one round of the scan (K > 1024) keep the city ids in
// the compacted buffers (their guess is taken from the buffer); shorter ones
// keep none.
constexpr int kRowsIdsAbove = 8 * 128;

// Single colony: CTA g takes ant groups g, g + grid, ... of A ants (A + 1
// warps a CTA).  With aging the ants come from the plan's list (k_aging_plan
// updated the ages), valid ones first.
template <bool AGING, bool IDS>
__global__ void __launch_bounds__((kRowsMaxAnts + 1) * 32) k_construct_rows(ColonyDev c) {
  extern __shared__ __align__(16) unsigned char smem_rows[];
  __shared__ RowsCtl ctl;
  const int A = (blockDim.x >> 5) - 1;
  const size_t ant_bytes = rows_ant_bytes(c.n, c.K);
  for (int first = blockIdx.x * A; first < c.m; first += gridDim.x * A) {
    rows_item<AGING, AGING, IDS>(c, first, min(A, c.m - first), smem_rows, ant_bytes, ctl);
    __syncthreads();
  }
}

template <typename F>
static cudaError_t set_smem_all(F f0, F f1, F f2, F f3, size_t smem) {
  const F fs[4] = {f0, f1, f2, f3};
  for (F f : fs) {
    const cudaError_t e =
        cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t configure_construct_rows(size_t smem) {
  return set_smem_all(k_construct_rows<false, false>, k_construct_rows<false, true>,
                      k_construct_rows<true, false>, k_construct_rows<true, true>, smem);
}

cudaError_t launch_construct_rows(const ColonyDev &c, int grid, int ants, cudaStream_t s) {
  const size_t smem = (size_t)ants * rows_ant_bytes(c.n, c.K);
  const bool ids = c.K > kRowsIdsAbove;
  if (c.aging) {
    cudaError_t e = launch_aging_plan(c, s);
    if (e != cudaSuccess) return e;
    if (ids)
      k_construct_rows<true, true><<<grid, (ants + 1) * 32, smem, s>>>(c);
    else
      k_construct_rows<true, false><<<grid, (ants + 1) * 32, smem, s>>>(c);
  } else {
    if (ids)
      k_construct_rows<false, true><<<grid, (ants + 1) * 32, smem, s>>>(c);
    else
      k_construct_rows<false, false><<<grid, (ants + 1) * 32, smem, s>>>(c);
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Batches: CTAs take (instance, first plan position, ant count, -) items from
// the work queue (largest instances first) until it is empty.  The per-ant
// regions are sized for the batch's largest instance and candidate row; the
// ids are kept when the longest candidate row needs them.
template <bool AGING, bool IDS>
__global__ void __launch_bounds__((kRowsMaxAnts + 1) * 32)
    k_batch_construct_rows(const ColonyDev *__restrict__ descs, const int4 *__restrict__ items,
                           int num_items, int *queue_head, int max_n, int max_ldk) {
  extern __shared__ __align__(16) unsigned char smem_brows[];
  __shared__ ColonyDev s_desc;
  __shared__ RowsCtl ctl;
  __shared__ int s_item;
  const size_t ant_bytes = rows_ant_bytes(max_n, max_ldk);
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(queue_head, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= num_items) break;
    const int4 w = items[it];
    if (threadIdx.x == 0) s_desc = descs[w.x];
    __syncthreads();
    rows_item<AGING, AGING, IDS>(s_desc, w.y, w.z, smem_brows, ant_bytes, ctl);
    __syncthreads();  // s_item, s_desc and the regions are rewritten by the next item
  }
}

size_t batch_rows_smem_bytes(int max_n, int max_ldk, int ants) {
  return (size_t)ants * rows_ant_bytes(max_n, max_ldk);
}

cudaError_t configure_batch_construct_rows(size_t smem) {
  return set_smem_all(k_batch_construct_rows<false, false>, k_batch_construct_rows<false, true>,
                      k_batch_construct_rows<true, false>, k_batch_construct_rows<true, true>,
                      smem);
}

int batch_rows_blocks_per_sm(int ants, size_t smem, bool aging) {
  // The smaller of the two variants' occupancies (the launch picks one by
  // the batch's longest row).
  const void *fns[2] = {
      aging ? (const void *)k_batch_construct_rows<true, false>
            : (const void *)k_batch_construct_rows<false, false>,
      aging ? (const void *)k_batch_construct_rows<true, true>
            : (const void *)k_batch_construct_rows<false, true>};
  int best = 0;
  for (const void *fn : fns) {
    int blocks = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, (ants + 1) * 32, smem) !=
        cudaSuccess)
      return 1;
    best = best == 0 ? blocks : std::min(best, blocks);
  }
  return best > 0 ? best : 1;
}

cudaError_t launch_batch_construct_rows(const ColonyDev *descs, const int4 *items, int num_items,
                                        int *queue_head, int grid, int ants, int max_n,
                                        int max_ldk, bool aging, cudaStream_t s) {
  const size_t smem = batch_rows_smem_bytes(max_n, max_ldk, ants);
  const bool ids = max_ldk > kRowsIdsAbove;
#define ACO_BATCH_ROWS(AG, ID)                                                            \
  k_batch_construct_rows<AG, ID><<<grid, (ants + 1) * 32, smem, s>>>(descs, items, num_items, \
                                                                     queue_head, max_n, max_ldk)
  if (aging) {
    if (ids)
      ACO_BATCH_ROWS(true, true);
    else
      ACO_BATCH_ROWS(true, false);
  } else {
    if (ids)
      ACO_BATCH_ROWS(false, true);
    else
      ACO_BATCH_ROWS(false, false);
  }
#undef ACO_BATCH_ROWS
  return cudaGetLastError();
}

}  // namespace aco
