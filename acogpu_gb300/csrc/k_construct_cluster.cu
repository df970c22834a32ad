// k_construct_cluster.cu -- the thread-block-cluster construction kernel
// (the step loop is in k_construct_steps.cuh).
#include "k_construct_steps.cuh"

namespace aco {

// ---------------------------------------------------------------------------
// Candidate table split over a thread-block cluster (k <= 32, n <= 8192, a
// table too large for one CTA): cluster rank r holds rows r*1024 .. r*1024 +
// 1023 (choice values, int16 ids, aging row means) at the same offsets as
// every other rank.  Each CTA stages its slice with TMA bulk copies; after a
// cluster barrier the ants read every row from its owner's shared memory
// (mapa + ld.shared::cluster) with the staged step loop; a second barrier
// keeps each slice alive until the whole cluster is done.  Every thread
// reaches both barriers on every path (a copy that timed out only records
// the error, and the ants run only when every rank staged its slice).  All
// CTAs share all ants.  Launches of at most kWideFallbackWarps warps use the
// FB = 16 instantiation (255 registers a thread: the fallback's full-row scan
// keeps 16 row chunks in flight); the fallback is a called function here
// (ClusterRows::kOutlineFallback), which keeps the step loop small.
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

}  // namespace aco
