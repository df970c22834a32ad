// k_construct_batch.cu -- the persistent batch construction kernel (the
// step loop and the general per-ant construction are in
// k_construct_steps.cuh).
#include "k_construct_steps.cuh"

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
__global__ void __launch_bounds__(kBatchMaxWarps * 32) k_batch_construct(const ColonyDev *__restrict__ descs,
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
