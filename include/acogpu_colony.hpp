// acogpu_colony.hpp -- the reference's Colony / AntSystem / RankBasedAntSystem
// C++ surface (reference: inc/Colony.h:24-155, inc/AntSystem.h:7-23,
// inc/RankBasedAntSystem.h:12-28) on top of the C ABI of acogpu.h.
//
// Same public signatures, same behaviour on failure: a failing call prints
// the error and exits (the reference's checkCudaErrors,
// inc/helper_cuda.h:316-325).  Header-only; link libacogpu.so.
#ifndef ACOGPU_COLONY_HPP
#define ACOGPU_COLONY_HPP

#include <stdio.h>
#include <stdlib.h>

#include <string>
#include <vector>

#include "acogpu.h"

namespace acogpu_detail {
inline void check(int status, const aco_colony *c, const char *what) {
  if (status != ACO_OK) {
    fprintf(stderr, "acogpu: %s failed: %s%s%s\n", what, aco_status_string(status),
            c ? ": " : "", c ? aco_colony_last_error(c) : "");
    exit(EXIT_FAILURE);
  }
}
}  // namespace acogpu_detail

class Colony {
 public:
  virtual ~Colony() { aco_colony_destroy(h_); }

  void initialize() { acogpu_detail::check(aco_colony_initialize(h_), h_, "initialize"); }
  // timers[6] receives the stage times in ms (inc/Statistics.h:7-15).
  void constructSolution(float timers[]) {
    acogpu_detail::check(aco_colony_construct_solution(h_, timers), h_, "constructSolution");
  }
  void setAlpha(float v) { acogpu_detail::check(aco_colony_set_alpha(h_, v), h_, "setAlpha"); }
  void setRho(float v) { acogpu_detail::check(aco_colony_set_rho(h_, v), h_, "setRho"); }
  void setBeta(float v) { acogpu_detail::check(aco_colony_set_beta(h_, v), h_, "setBeta"); }
  float getAlpha() { return params().alpha; }
  float getRho() { return params().rho; }
  float getBeta() { return params().beta; }
  int getNumAnts() { return params().num_ants; }
  int getNumCities() {
    int32_t n = 0;
    aco_colony_get_size(h_, &n, nullptr, nullptr);
    return n;
  }
  long getIterBestDist() {
    int64_t v = 0;
    acogpu_detail::check(aco_colony_get_iter_best(h_, &v), h_, "getIterBestDist");
    return (long)v;
  }
  long getGlobBestDist() {
    int64_t v = 0;
    acogpu_detail::check(aco_colony_get_glob_best(h_, &v), h_, "getGlobBestDist");
    return (long)v;
  }
  int getReps() {
    int32_t v = 0;
    aco_colony_get_reps(h_, &v);
    return v;
  }
  unsigned int getNumValidAnts() {
    int32_t v = 0;
    acogpu_detail::check(aco_colony_get_num_valid_ants(h_, &v), h_, "getNumValidAnts");
    return (unsigned int)v;
  }
  // computeParameters runs inside initialize (tau0, w = min(w, n)).
  virtual void computeParameters() {}
  virtual const char *antSystemName() { return aco_colony_name(h_); }
  // 1-based, comma after each city (src/Colony.cu:1173-1180).
  std::string getTour() {
    std::vector<int32_t> t(getNumCities());
    acogpu_detail::check(aco_colony_get_best_tour(h_, t.data()), h_, "getTour");
    std::string r;
    for (int32_t c : t) r += std::to_string(c + 1) + ",";
    return r;
  }
  void setOptimum(const int optimum) { aco_colony_set_optimum(h_, optimum); }

  // aging surface (inc/Colony.h:128-139)
  int getMinRetirementAge() { return params().min_retirement_age; }
  void setMinRetirementAge(int v) { set_aging(0, v); }
  int getMaxRetirementAge() { return params().max_retirement_age; }
  void setMaxRetirementAge(int v) { set_aging(1, v); }
  int getLocalPeformance() { return params().local_performance; }
  void setLocalPeformance(int v) { set_aging(2, v); }
  int getGlobalPerformance() { return params().global_performance; }
  void setGlobalPerformance(int v) { set_aging(3, v); }
  int getMinPopulationLimit() { return params().min_population_limit; }
  void setMinPopulationLimit(int v) { set_aging(4, v); }
  int getMaxPopulationLimit() { return params().max_population_limit; }
  void setMaxPopulationLimit(int v) { set_aging(5, v); }

  aco_colony *handle() { return h_; }

 protected:
  // distances: host or device pointer, n*n int32 (located automatically).
  Colony(int *distances, int cities, const aco_params &p) : h_(nullptr) {
    acogpu_detail::check(aco_colony_create(&p, distances, cities, -1, &h_), nullptr,
                         "Colony construction");
  }
  aco_params params() {
    aco_params p;
    aco_colony_get_params(h_, &p);
    return p;
  }
  void set_aging(int which, int v) {
    aco_params p = params();
    int32_t six[6] = {p.min_retirement_age, p.max_retirement_age, p.local_performance,
                      p.global_performance, p.min_population_limit, p.max_population_limit};
    six[which] = v;
    acogpu_detail::check(aco_colony_set_aging_params(h_, six), h_, "aging setter");
  }
  static aco_params base(int ants, int variant) {
    aco_params p;
    aco_params_default(&p);
    p.num_ants = ants;
    p.variant = variant;
    return p;
  }
  aco_colony *h_;
};

class AntSystem : public Colony {
 public:
  AntSystem(int *distances, int cities, int ants, float alpha, float beta, float rho)
      : Colony(distances, cities, with(base(ants, ACO_ANT_SYSTEM), alpha, beta, rho)) {}
  AntSystem(int *distances, int cities, int ants, float alpha, float beta, float rho,
            int minRetirementAge, int maxRetirementAge, int localPeformance,
            int globalPerformance, int minPopulationLimit, int maxPopulationLimit)
      : Colony(distances, cities,
               aging(with(base(ants, ACO_ANT_SYSTEM), alpha, beta, rho), minRetirementAge,
                     maxRetirementAge, localPeformance, globalPerformance, minPopulationLimit,
                     maxPopulationLimit)) {}
  const char *antSystemName() override { return "Ant System"; }

 private:
  static aco_params with(aco_params p, float a, float b, float r) {
    p.alpha = a;
    p.beta = b;
    p.rho = r;
    return p;
  }
  static aco_params aging(aco_params p, int a, int b, int c, int d, int e, int f) {
    p.aging = 1;
    p.min_retirement_age = a;
    p.max_retirement_age = b;
    p.local_performance = c;
    p.global_performance = d;
    p.min_population_limit = e;
    p.max_population_limit = f;
    return p;
  }
};

class RankBasedAntSystem : public Colony {
 public:
  RankBasedAntSystem(int *distances, int cities, int ants)
      : Colony(distances, cities, base(ants, ACO_RANK_BASED)) {}
  void setW(int w) { acogpu_detail::check(aco_colony_set_rank_w(h_, w), h_, "setW"); }
  int getW() { return params().rank_w; }
  const char *antSystemName() override { return "Rank-based Ant System"; }
};

#endif  // ACOGPU_COLONY_HPP
