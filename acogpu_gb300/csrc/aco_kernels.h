// aco_kernels.h -- host-side launchers of the engine's kernels.  Each
// returns the cudaError_t of its launch; all work is enqueued on `s`.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "aco_device.cuh"

namespace aco {

// ---- setup (k_setup.cu) ----
cudaError_t launch_distances_from_coords(const float *x, const float *y, int n, int ld,
                                         int32_t *dist, cudaStream_t s);
cudaError_t launch_fill_padding_int(int32_t *mat, int n, int ld, int32_t value, cudaStream_t s);
cudaError_t launch_max_distance(const int32_t *dist, int n, int ld, int32_t *out, cudaStream_t s);
cudaError_t launch_heuristic_device(const int32_t *dist, int n, int ld, float beta, float *eta,
                                    cudaStream_t s);
cudaError_t launch_heuristic_table(const int32_t *dist, int n, int ld, const float *table,
                                   int32_t table_len, float *eta, ColonyState *st, cudaStream_t s);
// Stable (distance, city) sort of each row, first K entries kept.
// nn2 (optional, pitch kTier2): neighbours K .. K + t2 - 1 of every row.
cudaError_t launch_nn_sort_stable(const int32_t *dist, int n, int ld, int K, int ldk, int32_t *nn,
                                  ColonyState *st, cudaStream_t s, int32_t *nn2 = nullptr,
                                  int t2 = 0);
// The reference CPU quicksort permutation (full rows only): one thread per
// row on a global scratch of n rows of ld int32, or (the _smem version) one
// warp per row in shared memory; nn_ref_qsort_smem_rows gives the rows a CTA
// holds within max_smem bytes (0: the row does not fit).
cudaError_t launch_nn_ref_qsort(const int32_t *dist, int n, int ld, int32_t *scratch, int32_t *nn,
                                int ldk, ColonyState *st, cudaStream_t s);
int nn_ref_qsort_smem_rows(int n, int max_smem);
cudaError_t launch_nn_ref_qsort_smem(const int32_t *dist, int n, int ld, int32_t *nn, int ldk,
                                     ColonyState *st, int max_smem, cudaStream_t s);
cudaError_t launch_gather_nn_f32(const float *src, int n, int ld, const int32_t *nn, int K,
                                 int ldk, float *dst, cudaStream_t s);
cudaError_t launch_greedy_tau0(const ColonyDev &c, int tau0_mode, float tau0_value,
                               cudaStream_t s);
cudaError_t launch_init_colony(const ColonyDev &c, cudaStream_t s);

// ---- iteration ----
size_t construct_smem_bytes(int n, int K, int ants_per_block);
// Raise the dynamic shared-memory limits once, outside any stream capture.
cudaError_t configure_construct(size_t smem);
cudaError_t configure_pheromone_rows(int ld);
cudaError_t launch_construct(const ColonyDev &c, int ants_per_block, cudaStream_t s);
// Candidate table staged in shared memory (k <= 32, n <= 2048); at most
// kStagedMaxWarps warps (ants in flight) per CTA.
constexpr int kStagedMaxWarps = 16;
// Warps (ants) per CTA of the batch kernel: 20 fit the register file
// without spilling (launch bound 640 threads, at most 102 registers).
constexpr int kBatchMaxWarps = 20;
// Launches of at most this many warps per CTA may hold 255 registers a thread.
constexpr int kWideFallbackWarps = 8;
// Pitch of the candidate rows (nn, eta_nn, tau_nn, choice_nn, nn16) for
// k <= 32: the staged step folds pitch/4 groups of four weights, and the
// pitch takes one of four values so the fold length is a template constant.
__host__ __device__ constexpr int staged_pitch(int K) {
  return K <= 16 ? 16 : K <= 20 ? 20 : K <= 24 ? 24 : 32;
}
// Shared-memory layout of a staged table of n rows with pitch sp:
//   [choice n*sp f32][ids n*sp int16, padded to 16 B][row means ld f32, aging]
struct StagedLayout {
  size_t ids_off, mean_off, table;
};
__host__ __device__ inline StagedLayout staged_layout(int n, int ld, int sp, bool aging) {
  StagedLayout L;
  L.ids_off = (size_t)n * sp * 4;
  L.mean_off = L.ids_off + ((size_t)n * sp * 2 + 15) / 16 * 16;
  L.table = L.mean_off + (aging ? (size_t)ld * 4 : 0);
  return L;
}
size_t construct_staged_smem_bytes(int n, int ld, int sp, bool aging, int warps);
cudaError_t configure_construct_staged(size_t smem);
cudaError_t launch_construct_staged(const ColonyDev &c, const int16_t *nn16, int grid, int warps,
                                    cudaStream_t s);
// Aging colonies: the age update and the ants' roles that the staged kernel
// reads (launched right before it).
cudaError_t launch_aging_plan(const ColonyDev &c, cudaStream_t s);
cudaError_t launch_batch_aging_plan(const ColonyDev *descs, int count, cudaStream_t s);
// k <= 32, rows read from L2 by the staged step loop (n <= kDirectMaxCities).
constexpr int kDirectMaxCities = 8192;
cudaError_t launch_construct_direct(const ColonyDev &c, int grid, int warps, cudaStream_t s);
// k <= 32, the table split over a cluster of cs = ceil(n / 1024) CTAs (cs <= 8)
// read through DSMEM.  The query gives how many such clusters fit at once.
cudaError_t query_construct_cluster(const ColonyDev &c, int warps, int cs, int *max_clusters);
cudaError_t launch_construct_cluster(const ColonyDev &c, int grid, int warps, int cs,
                                     cudaStream_t s);
// Long candidate rows (k > 32, full rows included; n <= kRowsMaxCities): a
// CTA holds A <= kRowsMaxAnts ants of one instance, one scan warp per ant and
// one chain warp (k_construct_rows.cu).  Each ant has a region of
// rows_ant_bytes in shared memory (rows_layout): two buffers of compacted
// weights and int16 ids (S = rows_slots(K) entries each), the running sums at
// every 32nd entry, the tabu bits and a visited byte per city.  The scan
// warps read the rows themselves from L2.
// The last 32 slots of each buffer are per-lane sinks for the stores of
// dropped entries (past any chain length).  With aging,
// launch_construct_rows runs the aging plan first (two launches).
constexpr int kRowsMaxCities = 8192;
constexpr int kRowsMaxAnts = 11;
__host__ __device__ inline int rows_slots(int K) { return (K + 31) / 32 * 32 + 32; }
struct RowsLayout {
  int S;
  size_t id_off, bend_off, tw_off, tb_off, bytes;
};
__host__ __device__ inline RowsLayout rows_layout(int n, int K) {
  RowsLayout L;
  L.S = rows_slots(K);
  L.id_off = (size_t)L.S * 8;
  L.bend_off = (size_t)L.S * 12;
  L.tw_off = L.bend_off + ((size_t)L.S / 32 * 4 + 15) / 16 * 16;
  L.tb_off = L.tw_off + (size_t)(((n + 31) / 32 + 3) / 4) * 16;
  L.bytes = L.tb_off + (size_t)(n + 15) / 16 * 16;
  return L;
}
__host__ __device__ inline size_t rows_ant_bytes(int n, int K) {
  const size_t b = rows_layout(n, K).bytes;
  return (b + 127) / 128 * 128 + 16;  // consecutive regions start four banks apart
}
cudaError_t configure_construct_rows(size_t smem);
cudaError_t launch_construct_rows(const ColonyDev &c, int grid, int ants, cudaStream_t s);
// max_ldk: the largest candidate-row pitch of the batch (every instance's
// layout fits in rows_ant_bytes(max_n, max_ldk), as K <= ldk).
size_t batch_rows_smem_bytes(int max_n, int max_ldk, int ants);
cudaError_t configure_batch_construct_rows(size_t smem);
int batch_rows_blocks_per_sm(int ants, size_t smem, bool aging);
cudaError_t launch_batch_construct_rows(const ColonyDev *descs, const int4 *items, int num_items,
                                        int *queue_head, int grid, int ants, int max_n,
                                        int max_ldk, bool aging, cudaStream_t s);
cudaError_t launch_nn_to_i16(const int32_t *nn, int n, int K, int ldk, int16_t *nn16,
                             cudaStream_t s);
cudaError_t launch_epilogue(const ColonyDev &c, cudaStream_t s);

// ---- batches of instances (descs: one ColonyDev per instance, in device memory) ----
cudaError_t launch_batch_epilogue(const ColonyDev *descs, int count, cudaStream_t s);
cudaError_t launch_batch_pheromone_rows(const ColonyDev *descs, const int2 *rowmap, int rows,
                                        int max_ld, bool deposit_and_evaporate, cudaStream_t s,
                                        int threads = 0);
// Persistent construction over a queue of work items (instance, first ant,
// ants, staged).  The shared region holds a staged item's candidate table or
// the per-warp tabu lists of an L2-row item.
size_t batch_staged_table_bytes(int n, int ld, int sp, bool aging);
size_t batch_region_bytes(int max_n, int max_k, int warps, size_t max_table);
size_t batch_construct_smem_bytes(size_t region_bytes, int warps);
cudaError_t configure_batch_construct(size_t smem);
int batch_construct_blocks_per_sm(int warps, size_t smem, bool multi, int sp, bool aging);
// sp: the pitch of the staged items (every staged item's ldk equals it).
cudaError_t launch_batch_construct(const ColonyDev *descs, const int4 *items, int num_items,
                                   int *queue_head, int grid, int warps, int max_n, int max_k,
                                   size_t region_bytes, int sp, bool aging, cudaStream_t s);
// Row-owned pheromone pass: optional evaporation, optional ordered deposit
// of the deposit list, then choice / choice_nn / tau_nn / row means.
cudaError_t launch_pheromone_rows(const ColonyDev &c, bool evaporate, bool deposit,
                                  bool write_tau, cudaStream_t s, int threads = 0);
// Atomic-mode pieces.
cudaError_t launch_evaporate(const ColonyDev &c, cudaStream_t s);
cudaError_t launch_deposit_atomic(const ColonyDev &c, cudaStream_t s);

}  // namespace aco
