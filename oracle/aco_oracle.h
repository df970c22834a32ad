/*
 * aco_oracle.h -- TEST INFRASTRUCTURE: the CPU oracle of the GB300 ACO
 * engine.  Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline
 * may load it; the product never links it.
 *
 * It restates the reference's CPU path (src/Colony.cu, src/AntSystem.cu,
 * src/Utils.cu, inc/Colony.cuh) operation by operation, with the random
 * stream of include/acogpu_rng.h, and extends it with the engine's new
 * options (candidate lists, best-choice fallback, rank-based update, tau0
 * rules, stable nn order, device heuristic) so every mode of the GPU path
 * has a bit-exact CPU counterpart.  Parameters use aco_params from the
 * public header.
 */
#ifndef ACO_ORACLE_H
#define ACO_ORACLE_H

#include <stdint.h>

#include "acogpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oc_colony oc_colony;

/* EUC_2D rounded distances, diagonal MAX (src/Utils.cu:162-182,212-218). */
void oc_distances(const float *x, const float *y, int32_t n, int32_t *out);

/* Full sorted nn rows (n*n), ACO_NN_STABLE or ACO_NN_REFERENCE_QSORT. */
void oc_nn_rows(const int32_t *dist, int32_t n, int32_t order, int32_t *out);

/* eta for one distance, ACO_HEURISTIC_DEVICE or ACO_HEURISTIC_LIBM. */
float oc_heuristic(int32_t d, float beta, int32_t mode);

/* Greedy nearest-neighbour tour length from city 0 (lowest index on ties). */
int64_t oc_greedy_length(const int32_t *dist, int32_t n);

int oc_create(const aco_params *p, const int32_t *dist, int32_t n, oc_colony **out);
void oc_set_threads(oc_colony *c, int32_t threads);
void oc_initialize(oc_colony *c);
void oc_iterate(oc_colony *c);
void oc_destroy(oc_colony *c);

int64_t oc_iter_best(const oc_colony *c);
int64_t oc_glob_best(const oc_colony *c);
int32_t oc_num_valid(const oc_colony *c);
int32_t oc_cand_k(const oc_colony *c);
float oc_tau0(const oc_colony *c);
void oc_get_pheromone(const oc_colony *c, float *out);
void oc_set_pheromone(oc_colony *c, const float *in);
void oc_get_heuristic(const oc_colony *c, float *out);
void oc_get_choice(const oc_colony *c, float *out);
void oc_get_nn(const oc_colony *c, int32_t *out); /* n*k */
void oc_get_tours(const oc_colony *c, int32_t *out);
void oc_get_lengths(const oc_colony *c, int64_t *out);
void oc_get_best_tour(const oc_colony *c, int32_t *out);
void oc_get_aging(const oc_colony *c, int32_t *age, int32_t *perf, uint8_t *valid,
                  float *mean, int32_t *misc);
/* Installs a candidate heuristic (n*k, candidate order), as the GPU does
 * when a learned prior is applied; the fallback keeps the plain one. */
void oc_set_candidate_heuristic(oc_colony *c, const float *eta_nk);
/* Fallback decisions taken in the last iteration (steps where the candidate
 * roulette could not pick a city). */
int64_t oc_fallback_count(const oc_colony *c);

/* FP64 restatement of one pheromone update (evaporation + deposits of the
 * given tours with the given lengths and weights), for the 1e-5 tolerance
 * check of the FP32 paths.  tau is n*n doubles, updated in place.
 * weights[q] multiplies 1/len[q]; tours are q*n cities. */
void oc_pheromone_update_f64(double *tau, int32_t n, double rho, int32_t count,
                             const int32_t *tours, const int64_t *lens,
                             const double *weights);

#ifdef __cplusplus
}
#endif

#endif
