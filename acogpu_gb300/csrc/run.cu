// run.cu -- the run loop of the C ABI (aco_execute), host code.
//
// Restates TSP::execute (src/TSP.cpp:23-79) on the public colony calls, minus
// its file output (the stats writer is the caller's): setOptimum, a timed
// initialize, then constructSolution with the six stage timers until
// TSP::terminationCondition (src/TSP.cpp:166-170) holds, the per-iteration
// Statistics of TSP::computeStatistics (src/TSP.cpp:124-149) and the
// SummaryStatistics of TSP::writeSummaryStatistics / initStatistics
// (src/TSP.cpp:81-122).
#include <chrono>

#include "acogpu.h"

extern "C" {

int aco_execute(aco_colony *c, int32_t max_time, int32_t max_iter, int32_t max_reps,
                int32_t optimum, float calcdisttime, aco_iteration_stats *stats,
                int32_t stats_cap, aco_run_summary *summary) {
  if (!c || stats_cap < 0 || (stats_cap > 0 && !stats)) return ACO_ERR_INVALID_ARGUMENT;
  aco_params p;
  int s = aco_colony_get_params(c, &p);
  if (s) return s;
  aco_run_summary sum = {};
  sum.p_alpha = p.alpha;
  sum.p_beta = p.beta;
  sum.p_rho = p.rho;

  const auto t0 = std::chrono::steady_clock::now();
  if ((s = aco_colony_set_optimum(c, optimum))) return s;
  if ((s = aco_colony_initialize(c))) return s;
  if ((s = aco_colony_synchronize(c))) return s;
  const float inittime =
      std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();

  int32_t i = 0;
  for (;; i++) {
    int64_t iterbest = 0;
    int32_t reps = 0;
    if ((s = aco_colony_get_iter_best(c, &iterbest))) return s;
    if ((s = aco_colony_get_reps(c, &reps))) return s;
    // terminationCondition(elapsed, iter, reps, (float)tourlen) with int limits
    if (sum.t_totaltime >= (float)max_time || i >= max_iter || reps >= max_reps ||
        (float)iterbest <= (float)optimum)
      break;
    float t[ACO_TOTAL_TIMERS];
    if ((s = aco_colony_construct_solution(c, t))) return s;
    int64_t ib = 0, gb = 0;
    int32_t ants = 0;
    if ((s = aco_colony_get_num_valid_ants(c, &ants))) return s;
    if ((s = aco_colony_get_iter_best(c, &ib))) return s;
    if ((s = aco_colony_get_glob_best(c, &gb))) return s;
    float itertime = 0.0f;
    for (int k = 0; k < ACO_TOTAL_TIMERS; k++) itertime += t[k];
    sum.t_totaltime += itertime;
    sum.t_inittour += t[ACO_TIME_INIT_TOUR];
    sum.t_computeprob += t[ACO_TIME_COMPUTE_PROBABILITIES];
    sum.t_tour += t[ACO_TIME_TOUR];
    sum.t_antdist += t[ACO_TIME_COMPUTE_ANT_DISTANCE];
    sum.t_evappheromnes += t[ACO_TIME_EVAPORATE_PHEROMONE];
    sum.t_updatephoremone += t[ACO_TIME_UPDATE_PHEROMONE];
    if (i < stats_cap) {
      aco_iteration_stats &st = stats[i];
      st.iter = i;
      st.ants = ants;
      st.iterbest = ib;
      st.globalbest = gb;
      st.t_inittour = t[ACO_TIME_INIT_TOUR];
      st.t_tour = t[ACO_TIME_TOUR];
      st.t_antdist = t[ACO_TIME_COMPUTE_ANT_DISTANCE];
      st.t_evapphoremone = t[ACO_TIME_EVAPORATE_PHEROMONE];
      st.t_updatephoremone = t[ACO_TIME_UPDATE_PHEROMONE];
      st.t_computeprob = t[ACO_TIME_COMPUTE_PROBABILITIES];
      st.t_itertime = itertime;
      st.t_globaltime = sum.t_totaltime;
    }
  }

  int32_t n = 0, m = 0, k = 0;
  int64_t gb = 0;
  if ((s = aco_colony_get_size(c, &n, &m, &k))) return s;
  if ((s = aco_colony_get_glob_best(c, &gb))) return s;
  sum.numants = m;
  sum.numcities = n;
  sum.numiter = i;
  sum.t_inittime = inittime;
  sum.t_distcalc = calcdisttime;
  sum.d_optimal = (float)optimum;
  sum.d_calulated = (float)gb;
  // CALCULATE_DISTANCE_ERROR(c, o) = ((c - o) / o) * 100 (inc/def.h:76), in float
  sum.d_error = ((sum.d_calulated - sum.d_optimal) / sum.d_optimal) * 100;
  if (summary) *summary = sum;
  return ACO_OK;
}

}  // extern "C"
