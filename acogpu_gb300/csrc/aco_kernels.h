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
cudaError_t launch_nn_sort_stable(const int32_t *dist, int n, int ld, int K, int ldk, int32_t *nn,
                                  ColonyState *st, cudaStream_t s);
// The reference CPU quicksort permutation (full rows only).
cudaError_t launch_nn_ref_qsort(const int32_t *dist, int n, int ld, int32_t *scratch, int32_t *nn,
                                int ldk, ColonyState *st, cudaStream_t s);
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
size_t construct_staged_smem_bytes(int n, int ld, bool aging, int warps);
cudaError_t configure_construct_staged(size_t smem);
cudaError_t launch_construct_staged(const ColonyDev &c, const int16_t *nn16, int grid, int warps,
                                    cudaStream_t s);
cudaError_t launch_nn_to_i16(const int32_t *nn, int n, int ldk, int16_t *nn16, cudaStream_t s);
cudaError_t launch_epilogue(const ColonyDev &c, cudaStream_t s);

// ---- batches of instances (descs: one ColonyDev per instance, in device memory) ----
cudaError_t launch_batch_epilogue(const ColonyDev *descs, int count, cudaStream_t s);
cudaError_t launch_batch_pheromone_rows(const ColonyDev *descs, const int2 *rowmap, int rows,
                                        int max_ld, bool deposit_and_evaporate, cudaStream_t s,
                                        int threads = 0);
// Persistent construction over a queue of work items (instance, first ant, ants).
size_t batch_construct_smem_bytes(int max_n, int max_k, int warps);
cudaError_t configure_batch_construct(size_t smem);
int batch_construct_blocks_per_sm(int warps, size_t smem, bool multi, bool aging);
cudaError_t launch_batch_construct(const ColonyDev *descs, const int4 *items, int num_items,
                                   int *queue_head, int grid, int warps, int max_n, int max_k,
                                   bool aging, cudaStream_t s);
// Row-owned pheromone pass: optional evaporation, optional ordered deposit
// of the deposit list, then choice / choice_nn / tau_nn / row means.
cudaError_t launch_pheromone_rows(const ColonyDev &c, bool evaporate, bool deposit,
                                  bool write_tau, cudaStream_t s, int threads = 0);
// Atomic-mode pieces.
cudaError_t launch_evaporate(const ColonyDev &c, cudaStream_t s);
cudaError_t launch_deposit_atomic(const ColonyDev &c, cudaStream_t s);

}  // namespace aco
