/*
 * acogpu.h -- C ABI of the GB300 Ant Colony Optimization engine for the
 * symmetric Euclidean TSP.
 *
 * This is the drop-in boundary for the reference's `Colony` / `AntSystem` /
 * `RankBasedAntSystem` C++ surface (reference: inc/Colony.h:24-155,
 * inc/AntSystem.h:7-23, inc/RankBasedAntSystem.h:12-28).  Every entry point
 * takes plain pointers and sizes, returns an int status (ACO_OK == 0) and
 * never throws or exits; aco_colony_last_error() gives the message.  The
 * reference instead prints and calls exit(EXIT_FAILURE) on any CUDA error
 * (inc/helper_cuda.h:316-325); the C++ classes in acogpu_colony.hpp keep that
 * behaviour on top of this ABI.
 *
 * One colony lives on one GPU (the current device when it is created) and
 * runs its kernels on one CUDA stream.  Calls on one colony are not
 * thread-safe; different colonies are independent.
 *
 * Thread safety, ownership: the library copies the distance matrix (or
 * builds it from coordinates) into its own device layout; the caller keeps
 * ownership of every pointer it passes.
 */
#ifndef ACOGPU_H
#define ACOGPU_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define ACO_API __attribute__((visibility("default")))
#else
#define ACO_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define ACOGPU_VERSION_MAJOR 1
#define ACOGPU_VERSION_MINOR 0

/* MAX_DISTANCE of the reference (inc/def.h:69): the diagonal of the
 * distance matrix. */
#define ACO_MAX_DISTANCE 0x7fffffff

/* ---- status codes ------------------------------------------------------ */
enum aco_status {
  ACO_OK = 0,
  ACO_ERR_INVALID_ARGUMENT = 1,
  ACO_ERR_OUT_OF_MEMORY = 2,
  ACO_ERR_CUDA = 3,
  ACO_ERR_NOT_INITIALIZED = 4,
  ACO_ERR_UNSUPPORTED = 5,
  ACO_ERR_DEVICE_TIMEOUT = 6, /* a bounded device-side wait gave up */
  ACO_ERR_DEVICE_CHECK = 7,   /* a device-side consistency check failed */
  ACO_ERR_IO = 8,             /* a file could not be opened or read */
  ACO_ERR_FORMAT = 9          /* a file is not in a supported format */
};

/* ---- parameter enums ----------------------------------------------------- */
enum aco_variant {
  ACO_ANT_SYSTEM = 0,  /* AntSystem: all ants deposit 1/L (src/AntSystem.cu:235-318) */
  ACO_RANK_BASED = 1   /* RankBasedAntSystem: w-1 ranked ants + best-so-far
                          (Bullnheimer, Hartl & Strauss 1999); the reference's
                          update is an empty stub (src/RankBasedAntSystem.cu:48-56) */
};

enum aco_nn_order {
  ACO_NN_STABLE = 0,          /* rows sorted by (distance, city): the order of the
                                 reference GPU kernel (inc/Colony.cuh:101-123) */
  ACO_NN_REFERENCE_QSORT = 1  /* the permutation of the reference CPU quicksort
                                 Utils::sort2 (src/Utils.cu:136-159), ties included */
};

enum aco_heuristic_mode {
  ACO_HEURISTIC_DEVICE = 0, /* eta = (1/d)^beta on the GPU, correctly rounded for
                               integer beta in [0, 64] */
  ACO_HEURISTIC_LIBM = 1    /* eta = powf((float)(1.0/(double)(float)d), beta)
                               through the host C library, as the reference CPU path
                               (inc/Colony.h:20); evaluated once per distinct
                               distance into a table that the GPU expands */
};

enum aco_fallback {
  ACO_FALLBACK_REFERENCE = 0, /* select_local_best: the LAST unvisited city of the
                                 full nn row (inc/Colony.cuh:33-43); needs a full row */
  ACO_FALLBACK_BEST = 1       /* the unvisited city with the largest choice value,
                                 lowest index on ties (choose_best_next of ACOTSP) */
};

/* Second tier of the best-choice fallback (k <= 32): the next 128 nearest
 * neighbours' choice values and the row's largest value outside them, written
 * by the pheromone pass, settle most fallbacks without a scan of the row (same
 * results either way).  It pays while the pheromone is spread over many
 * edges (the Ant System) and not when a few reinforced edges hold it (the
 * rank-based system after convergence). */
enum aco_fallback_tier {
  ACO_FALLBACK_TIER_AUTO = 0, /* on for ACO_ANT_SYSTEM, off for ACO_RANK_BASED */
  ACO_FALLBACK_TIER_ON = 1,
  ACO_FALLBACK_TIER_OFF = 2
};

enum aco_deposit_mode {
  ACO_DEPOSIT_DETERMINISTIC = 0, /* row-owned ordered fold: bit-exact with the
                                    reference's sequential CPU update */
  ACO_DEPOSIT_ATOMIC = 1         /* red.global.add.f32; order-free, fastest */
};

enum aco_tau0_mode {
  ACO_TAU0_REFERENCE = 0, /* 1e-6 (src/AntSystem.cu:200-203, inc/default.h:15) */
  ACO_TAU0_DORIGO = 1,    /* AS: m / C_nn, RBAS: 0.5 w (w-1) / (rho C_nn), with
                             C_nn the greedy nearest-neighbour tour from city 0 */
  ACO_TAU0_VALUE = 2      /* aco_params.tau0 */
};

enum aco_construct_mode {
  ACO_CONSTRUCT_AUTO = 0,    /* k <= 32: staged when the candidate table fits in one CTA's
                                shared memory, else split over a thread-block cluster
                                (n <= 8192), else the step loop on rows read from L2;
                                k > 32 (full rows included): the long-row kernel
                                (n <= 8192), otherwise the general kernel */
  ACO_CONSTRUCT_GLOBAL = 1,  /* the general kernel: candidate rows read from global memory */
  ACO_CONSTRUCT_STAGED = 2,  /* whole candidate table in shared memory; k <= 32, n <= 2048 */
  ACO_CONSTRUCT_DIRECT = 3,  /* the staged step loop on rows read from L2; k <= 32, n <= 8192 */
  ACO_CONSTRUCT_CLUSTER = 4, /* the table split over a cluster of ceil(n/1024) CTAs, rows
                                read through distributed shared memory; k <= 32, n <= 8192 */
  ACO_CONSTRUCT_ROWS = 5     /* the long-row kernel: rows read from L2 and compacted by a
                                warp per ant, the roulette's sequential prefix over the
                                non-zero weights by a chain warp; k > 32, n <= 8192 */
};

/* Stage timers filled by aco_colony_construct_solution, indexed like the
 * reference's StatsTimer enum (inc/Statistics.h:7-15). */
enum aco_timer {
  ACO_TIME_INIT_TOUR = 0,
  ACO_TIME_TOUR = 1,
  ACO_TIME_COMPUTE_ANT_DISTANCE = 2,
  ACO_TIME_EVAPORATE_PHEROMONE = 3,
  ACO_TIME_UPDATE_PHEROMONE = 4,
  ACO_TIME_COMPUTE_PROBABILITIES = 5,
  ACO_TOTAL_TIMERS = 6
};

typedef struct aco_params {
  int32_t variant;   /* enum aco_variant */
  int32_t num_ants;  /* m */
  float alpha;       /* stored; the reference ignores it (inc/Colony.cuh:29-30)
                        unless use_alpha is set */
  float beta;
  float rho;
  int32_t use_alpha; /* 0: choice = tau * eta^beta exactly as the reference */
  int32_t cand_k;    /* candidate-list length; <= 0 or >= n means the full row */
  int32_t nn_order;  /* enum aco_nn_order */
  int32_t heuristic; /* enum aco_heuristic_mode */
  int32_t fallback;  /* enum aco_fallback */
  int32_t deposit;   /* enum aco_deposit_mode */
  int32_t tau0_mode; /* enum aco_tau0_mode */
  float tau0;        /* used when tau0_mode == ACO_TAU0_VALUE */
  int32_t rank_w;    /* RBAS w (reference default 5, inc/default.h:19) */
  int32_t aging;     /* 0: noaging variant, 1: aging variant */
  /* aging parameters (reference: inc/Colony.h:118-124, defaults inc/default.h:34-39) */
  int32_t min_retirement_age;
  int32_t max_retirement_age;
  int32_t local_performance;
  int32_t global_performance;
  int32_t min_population_limit;
  int32_t max_population_limit;
  int32_t broker;    /* accepted for the broker/nobroker variant; the reference's
                        broker build defines a flag and nothing else
                        (inc/broker/parallel.h:3, inc/Colony.h:142-149) */
  uint64_t seed;     /* seed of the injected uniform stream (acogpu_rng.h) */
  int32_t ants_per_block; /* construction warps per CTA; 0 = tuned default */
  int32_t construct_mode; /* enum aco_construct_mode */
  int32_t fallback_tier;  /* enum aco_fallback_tier */
  int32_t reserved[5];
} aco_params;

/* Reference defaults (inc/default.h, src/Colony.cu:31-36): AS, m = 10,
 * alpha 1, beta 5, rho 0.1, full-row candidates, reference quicksort order,
 * libm heuristic, reference fallback, deterministic deposit, tau0 = 1e-6,
 * w = 5, noaging, aging parameters 30/50/10/10/40/100, seed 12345678. */
ACO_API void aco_params_default(aco_params *p);

typedef struct aco_colony aco_colony;

/* Create a colony on the current device.
 *   dist: n*n int32 row-major EUC_2D distances with ACO_MAX_DISTANCE on the
 *         diagonal (the reference's distance vector, src/Setup.cpp:54-70).
 *   dist_on_device: 0 if dist is host memory, 1 if it is device memory on the
 *         current device (the reference GPU build passes a device pointer,
 *         src/Setup.cpp:60-66), -1 to let the library find out.
 * Replaces the constructors AntSystem::AntSystem (src/AntSystem.cu:160-182),
 * RankBasedAntSystem::RankBasedAntSystem (src/RankBasedAntSystem.cu:14-18)
 * and Colony::Colony (src/Colony.cu:25-137). */
ACO_API int aco_colony_create(const aco_params *params, const int32_t *dist, int32_t n,
                      int32_t dist_on_device, aco_colony **out);

/* Create a colony from float coordinates; the EUC_2D distance matrix
 * (reference: Utils::compute_distance, src/Utils.cu:162-182,212-218) is built
 * on the GPU. */
ACO_API int aco_colony_create_coords(const aco_params *params, const float *x,
                             const float *y, int32_t n, aco_colony **out);

/* Colony::initialize (src/Colony.cu:185-214): initial pheromone, heuristic,
 * nn-list, aging state, best-so-far reset. */
ACO_API int aco_colony_initialize(aco_colony *c);

/* Colony::constructSolution (src/Colony.cu:537-594): one iteration.  timers
 * (may be NULL) receives per-stage device times in ms, indexed by
 * enum aco_timer; passing timers makes the call synchronous. */
ACO_API int aco_colony_construct_solution(aco_colony *c, float *timers_ms);

/* Run `iterations` iterations back to back from a captured CUDA graph, with
 * no host synchronisation in between.  Returns once they are enqueued. */
ACO_API int aco_colony_run(aco_colony *c, int32_t iterations);

/* Wait for all enqueued work; reports device-side errors. */
ACO_API int aco_colony_synchronize(aco_colony *c);

/* Getters of the reference surface (inc/Colony.h:38-48,152). */
ACO_API int aco_colony_get_iter_best(aco_colony *c, int64_t *out);  /* getIterBestDist */
ACO_API int aco_colony_get_glob_best(aco_colony *c, int64_t *out);  /* getGlobBestDist */
ACO_API int aco_colony_get_num_valid_ants(aco_colony *c, int32_t *out); /* getNumValidAnts */
ACO_API int aco_colony_get_best_tour(aco_colony *c, int32_t *out_n);   /* getTour, 0-based */
ACO_API int aco_colony_get_iteration(aco_colony *c, int32_t *out);
ACO_API int aco_colony_get_reps(aco_colony *c, int32_t *out);        /* getReps (always 0) */
ACO_API int aco_colony_get_size(aco_colony *c, int32_t *n, int32_t *m, int32_t *k);
ACO_API int aco_colony_get_params(aco_colony *c, aco_params *out);
/* Setters of the reference surface: setAlpha/setBeta/setRho/setOptimum
 * (inc/Colony.h:35-37,49), RankBasedAntSystem::setW, and the aging setters
 * (inc/Colony.h:128-139).  beta, w and tau0-relevant values take effect at
 * the next aco_colony_initialize. */
ACO_API int aco_colony_set_alpha(aco_colony *c, float v);
ACO_API int aco_colony_set_beta(aco_colony *c, float v);
ACO_API int aco_colony_set_rho(aco_colony *c, float v);
ACO_API int aco_colony_set_optimum(aco_colony *c, int64_t v);
ACO_API int aco_colony_set_rank_w(aco_colony *c, int32_t w);
ACO_API int aco_colony_set_aging_params(aco_colony *c, const int32_t six[6]);
/* antSystemName(): "Ant System" or "Rank-based Ant System". */
ACO_API const char *aco_colony_name(const aco_colony *c);

/* Checkpoint / resume (the reference has none).  aco_colony_save writes the
 * state a colony's next iterations depend on -- pheromone, the device state
 * block (bests, iteration counter of the random stream, aging flags), the
 * best-so-far tour and its successor/predecessor lists, the aging arrays,
 * the last tours and lengths and the candidate heuristic -- with the
 * parameters and a hash of the distances.  aco_colony_load restores it into
 * an initialized colony of the same instance and parameters (otherwise
 * ACO_ERR_INVALID_ARGUMENT; a damaged file ACO_ERR_FORMAT; file errors
 * ACO_ERR_IO); the loaded colony then continues bit for bit as the saved one
 * would have. */
ACO_API int aco_colony_save(aco_colony *c, const char *path);
ACO_API int aco_colony_load(aco_colony *c, const char *path);

/* State export/import (host buffers), for checking and checkpointing. */
ACO_API int aco_colony_read_pheromone(aco_colony *c, float *out_nn);      /* n*n */
ACO_API int aco_colony_write_pheromone(aco_colony *c, const float *in_nn);
ACO_API int aco_colony_read_heuristic(aco_colony *c, float *out_nn);      /* n*n */
ACO_API int aco_colony_read_choice_info(aco_colony *c, float *out_nn);    /* n*n */
ACO_API int aco_colony_read_nn_list(aco_colony *c, int32_t *out_nk);      /* n*k */
ACO_API int aco_colony_read_distances(aco_colony *c, int32_t *out_nn);    /* n*n */
ACO_API int aco_colony_read_tours(aco_colony *c, int32_t *out_mn);        /* m*n */
ACO_API int aco_colony_read_tour_lengths(aco_colony *c, int64_t *out_m);
/* age[m], performance[m], valid[m], pheromone row means[n],
 * misc[2] = {isconverged, globalperformance} */
ACO_API int aco_colony_read_aging(aco_colony *c, int32_t *age, int32_t *perf,
                          uint8_t *valid, float *mean, int32_t *misc);

/* Counters kept on the device. */
typedef struct aco_stats {
  int64_t iteration;     /* iterations run since aco_colony_initialize */
  int64_t tours_built;   /* tours constructed (valid ants) since initialize */
  int64_t fallbacks;     /* construction steps resolved by the fallback rule */
  int64_t greedy_length; /* C_nn of the tau0 rule (0 unless ACO_TAU0_DORIGO) */
  int64_t iter_best;
  int64_t glob_best;
  int32_t num_valid;
  float tau0;
  int64_t reserved[4];
} aco_stats;
ACO_API int aco_colony_get_stats(aco_colony *c, aco_stats *out);

/* Bind the colony to a CUDA stream (cudaStream_t passed as void*). */
ACO_API int aco_colony_set_stream(aco_colony *c, void *stream);
/* Number of kernel launches this colony has issued (graph nodes count once
 * per replay). */
ACO_API int aco_colony_get_launch_count(aco_colony *c, int64_t *out);

/* ---- batches of instances ------------------------------------------------
 * Many TSP instances of uneven size advanced together on one GPU: one
 * iteration of the whole batch is a persistent construction launch fed by a
 * per-instance work queue, one epilogue CTA per instance and one pheromone
 * CTA per row, captured once into a CUDA graph.  The reference runs one
 * instance per process (src/Setup.cpp:73-129); this has no counterpart there
 * and exists for throughput on many instances.  Instance i gets
 * m_i = min(params->num_ants, n_i) ants and seed params->seed + i*0x9E3779B97F4A7C15,
 * and evolves exactly like a colony created with those parameters.
 * coords: for each instance in turn, its n_i x values then its n_i y values.
 * Only ACO_DEPOSIT_DETERMINISTIC is supported. */
typedef struct aco_batch aco_batch;

typedef struct aco_tuning {
  int32_t ants_per_block; /* warps (ants) per CTA of the construction launch */
  int32_t row_threads;    /* threads per CTA of the pheromone row pass */
  float construct_ms;     /* best timed construction launch */
  float rows_ms;          /* best timed row pass */
  int32_t staged_instances; /* instances whose candidate table is staged in shared memory */
  int32_t construct_mode;   /* aco_colony_autotune: the construction kernel kept (enum
                               aco_construct_mode) */
  int32_t reserved[2];
} aco_tuning;

ACO_API int aco_batch_create(const aco_params *params, int32_t count, const int32_t *sizes,
                             const float *coords, aco_batch **out);
ACO_API int aco_batch_initialize(aco_batch *b);
/* `iterations` graph-replayed iterations of every instance, asynchronous. */
ACO_API int aco_batch_run(aco_batch *b, int32_t iterations);
ACO_API int aco_batch_synchronize(aco_batch *b);
/* Times the construction launch for 1..20 ants per CTA (2..11 on the
 * long-row batch kernel) and the row pass for
 * 128..512 threads, keeps the fastest, then returns every instance to its
 * initialised state.  Call after aco_batch_initialize, before running.
 * Construction: instances with k <= 32 whose candidate table fits in shared
 * memory (about n <= 1150) are staged there, per work item, unless the batch
 * parameters ask for ACO_CONSTRUCT_GLOBAL; the others read rows from L2. */
ACO_API int aco_batch_autotune(aco_batch *b, aco_tuning *out);
/* One colony: times its construction launch on every kernel and launch shape
 * that builds the same tours -- k <= 32: the staged, cluster and direct
 * kernels, with 1..16 ants (warps) per CTA on the staged kernel without aging
 * and on the direct kernel; k > 32: the long-row kernel with 1..11 ants per
 * CTA; any k: the general kernel -- keeps the fastest (as if construct_mode
 * had named it), returns the colony to its initialised state and drops the
 * captured iteration graph.  Call after aco_colony_initialize, before
 * running.  Not tuned, by design: the candidate-list length k (it changes
 * which tours the method builds, so it is a parameter of the method, not of
 * the launch) and the fallback's second tier (its benefit depends on how
 * concentrated the pheromone is, which a freshly initialised colony cannot
 * show; its rule is fixed by variant, see aco_fallback_tier). */
ACO_API int aco_colony_autotune(aco_colony *c, aco_tuning *out);
/* ants_per_block 1..20 (1..11 for long rows); row_threads 0 (keep) or 64..512 in steps of 32 (warp
 * 0 folds the deposits in order, the other warps stage them). */
ACO_API int aco_batch_set_tuning(aco_batch *b, int32_t ants_per_block, int32_t row_threads);
ACO_API int aco_batch_get_size(aco_batch *b, int32_t *count);
/* Borrowed handle of instance i (read its state with the colony getters;
 * do not destroy or run it). */
ACO_API int aco_batch_get_colony(aco_batch *b, int32_t i, aco_colony **out);
ACO_API int aco_batch_get_glob_best(aco_batch *b, int64_t *out_count);
ACO_API int aco_batch_get_tours_built(aco_batch *b, int64_t *out);
ACO_API int aco_batch_get_launch_count(aco_batch *b, int64_t *out);
ACO_API const char *aco_batch_last_error(const aco_batch *b);
ACO_API void aco_batch_destroy(aco_batch *b);

/* ---- learned heuristic prior ------------------------------------------------
 * An edge-scoring MLP (12 features per candidate edge -> 128 -> 128 -> 1,
 * ReLU, logistic output; BF16 tensor-core GEMMs with FP32 accumulation) that
 * predicts whether a candidate edge lies on the best tour the plain method
 * finds.  Its output p multiplies the candidate heuristic of a colony:
 * eta'_ir = eta_ir * (floor + p).  No counterpart in the reference.
 * Features of edge i -> j = nn[i][r] (distances d, K = candidate count):
 *   d/dK_i, d/dK_j, r/K, rank of i in j's list / K (1 if absent),
 *   (x_j-x_i)/dK_i, (y_j-y_i)/dK_i, d1_i/dK_i, d1_j/dK_j, d/(d1_i+d1_j+1),
 *   dK_i/mean dK, dK_j/mean dK, mutual top-5 flag
 * (dK = distance to the K-th candidate, d1 = to the nearest).
 * Parameters are packed as W1[128][12] b1[128] W2[128][128] b2[128] w3[128] b3. */
typedef struct aco_prior aco_prior;
/* Engine of the MLP's forward and backward passes.  The first two run
 * layer by layer (one GEMM launch per product, elementwise kernels between
 * them); ACO_GEMM_FUSED (the default) runs the whole pass over each
 * 128-edge tile in one tcgen05 kernel, activations kept in shared and
 * tensor memory, gradients summed per CTA and reduced in a fixed order. */
enum aco_gemm_engine {
  ACO_GEMM_MMA_SYNC = 0, /* layered, warp-level mma.sync.m16n8k16 */
  ACO_GEMM_TCGEN05 = 1,  /* layered, tcgen05.mma with TMA-staged operands, TMEM accumulator */
  ACO_GEMM_FUSED = 2     /* one fused tcgen05 kernel per pass (default) */
};
ACO_API int aco_prior_create(uint64_t seed, aco_prior **out);
ACO_API int aco_prior_set_engine(aco_prior *p, int32_t engine);
/* The MLP's GEMM on host data, for checking: C (M x N, FP32) = A (M x K) *
 * B (N x K)^T with A and B raw BF16 bit patterns; K a multiple of 8;
 * engine ACO_GEMM_MMA_SYNC or ACO_GEMM_TCGEN05 (N = 128 or 16). */
ACO_API int aco_gemm_bf16_tn(const uint16_t *A, const uint16_t *B, float *C, int32_t M, int32_t N,
                             int32_t K, int32_t splits, int32_t engine);
ACO_API int aco_prior_param_count(void);
ACO_API int aco_prior_get_weights(aco_prior *p, float *out);
ACO_API int aco_prior_set_weights(aco_prior *p, const float *in);
/* Appends the candidate edges of an initialized colony built from
 * coordinates, labelled by its best-so-far tour. */
ACO_API int aco_prior_add_examples(aco_prior *p, aco_colony *c);
ACO_API int aco_prior_num_examples(aco_prior *p, int64_t *examples, int64_t *positives);
ACO_API int aco_prior_clear_examples(aco_prior *p);
/* Adam on the weighted logistic loss (positives weighted by #neg/#pos). */
ACO_API int aco_prior_train(aco_prior *p, int32_t epochs, int32_t batch, float lr, uint64_t seed,
                            float *last_loss);
/* Loss and packed gradient of a batch given on the host (E x 12 features). */
ACO_API int aco_prior_loss_and_grads(aco_prior *p, const float *feats, const float *labels,
                                     int32_t E, float pos_weight, float *loss, float *grads);
ACO_API int aco_prior_predict(aco_prior *p, const float *feats, int32_t E, float *probs);
/* Scores the colony's candidate edges and installs the prior. */
ACO_API int aco_prior_apply(aco_prior *p, aco_colony *c, float floor);
ACO_API const char *aco_prior_last_error(const aco_prior *p);
ACO_API void aco_prior_destroy(aco_prior *p);
/* Features of every candidate edge of a colony built from coordinates
 * (n*k rows of 12, row i*k + r), and its candidate heuristic (n*k). */
ACO_API int aco_colony_edge_features(aco_colony *c, float *out);
ACO_API int aco_colony_read_candidate_heuristic(aco_colony *c, float *out_nk);

/* Largest city count accepted by aco_nn_list_reference_order_noalloc. */
#define ACO_NOALLOC_MAX_CITIES 1024

/* nn-list build that allocates no device memory.  This entry point has no
 * counterpart in the reference.  It exists for callers that cannot call
 * cudaMalloc or cudaFree: code that must not trigger the device-wide
 * synchronisation of cudaFree while other streams run, code whose device
 * memory belongs to a framework allocator or a fixed budget, code that must
 * not meet an out-of-memory error midway.
 *
 *   dist_dev: n*n int32 distances in device memory (row-major, MAX on the
 *             diagonal); nn_dev: n*n int32 output in device memory, each row
 *             the cities sorted by distance, ties in the order of the
 *             ACO_NN_REFERENCE_QSORT rule -- the same rows as a colony built
 *             with ACO_NN_REFERENCE_QSORT and full-row candidates.
 *   n: 1 <= n <= ACO_NOALLOC_MAX_CITIES, otherwise ACO_ERR_UNSUPPORTED.
 *   stream: cudaStream_t (NULL for the default stream).  The call is
 *           synchronous: it waits for its own work on the stream, reads the
 *           kernel's error flags back, and returns the status.
 *
 * The sort's scratch is a fixed 4 MiB __device__ array inside the library,
 * held by every GPU that loads the library until the process exits.  Its
 * device address is looked up once per CUDA context, with the device
 * current: the first call on a device does this set-up (make that first
 * call before any stream capture), and so does the first call after the
 * device's context was replaced, e.g. by cudaDeviceReset.  All calls share
 * the one array and the kernel's error flags: calls that overlap on the GPU
 * (from several host threads or streams at once) race and must not be
 * issued. */
ACO_API int aco_nn_list_reference_order_noalloc(const int32_t *dist_dev, int32_t n,
                                                int32_t *nn_dev, void *stream);

ACO_API const char *aco_colony_last_error(const aco_colony *c);
ACO_API const char *aco_status_string(int status);
ACO_API void aco_colony_destroy(aco_colony *c);

/* ---- run loop ------------------------------------------------------------
 * aco_execute replaces TSP::execute (src/TSP.cpp:23-79), without its file
 * output: setOptimum, initialize (timed on the host: t_inittime, ms), then
 * aco_colony_construct_solution with the stage timers while not
 *   t_totaltime >= max_time || iter >= max_iter || reps >= max_reps ||
 *   (float)iteration best <= (float)optimum
 * (TSP::terminationCondition, src/TSP.cpp:166-170; t_totaltime is the sum of
 * the stage timers in ms; reps is always 0, as in the reference).  stats, if
 * not null, receives the Statistics of the first stats_cap iterations
 * (TSP::computeStatistics, src/TSP.cpp:124-149); summary the
 * SummaryStatistics (src/TSP.cpp:81-122), with d_error =
 * (d_calulated - d_optimal) / d_optimal * 100 in float (inc/def.h:76). */
typedef struct aco_iteration_stats { /* Statistics, inc/Statistics.h:17-30 */
  int32_t ants;
  int32_t iter;
  int64_t iterbest;
  int64_t globalbest;
  float t_inittour;
  float t_computeprob;
  float t_tour;
  float t_antdist;
  float t_evapphoremone;
  float t_updatephoremone;
  float t_itertime;
  float t_globaltime;
} aco_iteration_stats;

typedef struct aco_run_summary { /* SummaryStatistics, inc/Statistics.h:32-53,
                                    without the platform and file-name strings */
  int32_t numcities;
  int32_t numants;
  int32_t numiter;
  float t_inittime;
  float t_inittour;
  float t_computeprob;
  float t_tour;
  float t_antdist;
  float t_distcalc;
  float t_updatephoremone;
  float t_evappheromnes;
  float t_totaltime;
  float d_optimal;
  float d_calulated;
  float d_error;
  float p_alpha;
  float p_beta;
  float p_rho;
} aco_run_summary;

ACO_API int aco_execute(aco_colony *c, int32_t max_time, int32_t max_iter, int32_t max_reps,
                        int32_t optimum, float calcdisttime, aco_iteration_stats *stats,
                        int32_t stats_cap, aco_run_summary *summary);

/* ---- TSPLIB instances --------------------------------------------------------
 * aco_tsplib_read replaces TSPReader::read (src/TSPReader.cu:25-95): TYPE TSP
 * or STSP, EDGE_WEIGHT_TYPE EUC_2D, DIMENSION, then NODE_COORD_SECTION lines
 * "id x y" read as "%ld %f %f" (float coordinates).  Files the reference would
 * read past (no DIMENSION before the coordinates, a short or unreadable
 * coordinate section) give ACO_ERR_FORMAT; an unopenable file ACO_ERR_IO.  The
 * getters replace TSPReader::getNumNodes / getName / getXcoords / getYcoords
 * (src/TSPReader.cu:97-118); the arrays live until aco_tsplib_destroy.  Feed
 * them to aco_colony_create_coords (the distances of src/Setup.cpp:54-70). */
typedef struct aco_tsplib aco_tsplib;
ACO_API int aco_tsplib_read(const char *path, aco_tsplib **out);
ACO_API int32_t aco_tsplib_num_nodes(const aco_tsplib *t);
ACO_API const char *aco_tsplib_name(const aco_tsplib *t);
ACO_API const float *aco_tsplib_xcoords(const aco_tsplib *t);
ACO_API const float *aco_tsplib_ycoords(const aco_tsplib *t);
/* Message of the calling thread's last failed aco_tsplib_read. */
ACO_API const char *aco_tsplib_last_error(void);
ACO_API void aco_tsplib_destroy(aco_tsplib *t);

/* ---- failure path self-tests ---------------------------------------------
 * The reference exits on every CUDA error (inc/helper_cuda.h:316-325); here
 * every entry point returns a status and every device-side wait is bounded.
 * These two calls exercise those paths without faulting or hanging a GPU.
 *
 * aco_selftest_bounded_wait: one kernel waits on an mbarrier that nothing
 * arrives on, gives up after `polls` polls (1 .. 2^22), records the timeout
 * as the engine's kernels do, and exits normally.  Returns
 * ACO_ERR_DEVICE_TIMEOUT -- the expected outcome -- once the kernel has
 * finished and the flag has been read back; ACO_ERR_CUDA if the launch or
 * the copy failed.  The CUDA context stays usable.
 *
 * aco_debug_fail_allocation: the after-th next device array requested by a
 * colony (0 = the next one; a colony's arrays share one allocation, made
 * once every request has passed) reports ACO_ERR_OUT_OF_MEMORY without
 * allocating; a negative value switches the injection off.  Process-wide. */
ACO_API int aco_selftest_bounded_wait(uint32_t polls);
ACO_API void aco_debug_fail_allocation(int32_t after);

#ifdef __cplusplus
}
#endif

#endif /* ACOGPU_H */
