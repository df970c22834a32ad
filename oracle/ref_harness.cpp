/*
 * ref_harness.cpp -- TEST INFRASTRUCTURE.  Drives the reference's own CPU
 * AntSystem (compiled in place from the reference's sources by
 * oracle/Makefile) through a small C interface, so tests can compare the
 * GPU library with the reference on identical inputs.
 *
 * What the harness changes, and nothing else:
 *  - the random stream: the reference's Utils::random (src/Utils.cu:112-114)
 *    is replaced at link time (ld --wrap) by the counter-based stream of
 *    include/acogpu_rng.h.  The wrapper works out which (iteration, ant,
 *    step) is drawing from the colony's own state, because the two draw
 *    sites (src/Colony.cu:518 in initTour, src/Colony.cu:826 in
 *    selectCities) do not pass the ant index;
 *  - optionally the nn-list tie order: Utils::sort2 (src/Utils.cu:136-159,
 *    called at src/Colony.cu:301) can be replaced by a stable sort on
 *    (distance, city), the order the reference's GPU kernel produces
 *    (inc/Colony.cuh:101-123).  Off by default: the reference's own
 *    quicksort runs.
 *
 * State is read through a subclass of AntSystem (the members are protected,
 * inc/Colony.h:71-98).
 */
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "AntSystem.h"
#include "acogpu_rng.h"

#if ANTS_AGING
extern unsigned int numValidAnts; /* inc/Colony.cuh:10 */
extern int isconverged;           /* inc/Colony.cuh:11 */
#endif

namespace {

class OracleAS : public AntSystem {
 public:
  OracleAS(int *d, int n, int m, float a, float b, float r)
      : AntSystem(d, n, m, a, b, r) {}
#if ANTS_AGING
  OracleAS(int *d, int n, int m, float a, float b, float r, int minRet,
           int maxRet, int localPerf, int globalPerf, int minPop, int maxPop)
      : AntSystem(d, n, m, a, b, r, minRet, maxRet, localPerf, globalPerf,
                  minPop, maxPop) {}
#endif
  int cities() const { return numCities; }
  int ants() const { return numAnts; }
  const long *tours() const { return tour; }
  const unsigned char *visits() const { return visited; }
  const float *pher() const { return pheromones; }
  const float *heur() const { return hurestics; }
  const int *nn() const { return nnlist; }
  const long *lengths() const { return tourlength; }
  const long *best_tour() const { return gbtour; }
  bool valid(int k) const {
#if ANTS_AGING
    return validants[k] != 0;
#else
    (void)k;
    return true;
#endif
  }
#if ANTS_AGING
  const int *ages() const { return antage; }
  const int *perfs() const { return antperformance; }
  const unsigned char *valids() const { return validants; }
  const float *means() const { return pheromone_mean; }
  int global_perf() const { return globalperformance; }
#endif
};

struct DrawCursor {
  int phase; /* 0: initTour placements, 1: construction */
  int step;
  int ant;
};

OracleAS *g_cur = 0;
uint64_t g_seed = 0;
uint32_t g_iter = 0;
DrawCursor g_cursor = {0, 1, 0};
long g_draws = 0;
int g_stable_nn = 0;

/* Has ant k already taken its step-x city?  The tour row is cleared to 0 at
 * initTour (src/Colony.cu:507-510), so a non-zero entry is a move; a zero
 * entry is a move to city 0 only if city 0 is visited and not earlier in the
 * tour. */
bool moved(const OracleAS *c, int k, int x) {
  const int n = c->cities();
  const long *t = c->tours() + (long)k * n;
  if (t[x] != 0) return true;
  if (!c->visits()[(long)k * n + 0]) return false;
  for (int i = 0; i < x; i++)
    if (t[i] == 0) return false;
  return true;
}

bool placed(const OracleAS *c, int k) {
  const int n = c->cities();
  const long s = c->tours()[(long)k * n];
  return c->visits()[(long)k * n + s] != 0;
}

float draw_for_current_caller() {
  OracleAS *c = g_cur;
  const int n = c->cities(), m = c->ants();
  if (g_cursor.phase == 0) {
    for (int k = g_cursor.ant; k < m; k++) {
      if (!c->valid(k) || placed(c, k)) continue;
      g_cursor.ant = k + 1;
      return aco_uniform(g_seed, g_iter, (uint32_t)k, 0u);
    }
    g_cursor.phase = 1;
    g_cursor.step = 1;
    g_cursor.ant = 0;
  }
  for (int x = g_cursor.step; x < n; x++) {
    for (int k = (x == g_cursor.step ? g_cursor.ant : 0); k < m; k++) {
      if (!c->valid(k) || moved(c, k, x)) continue;
      g_cursor.step = x;
      g_cursor.ant = k + 1;
      return aco_uniform(g_seed, g_iter, (uint32_t)k, (uint32_t)x);
    }
  }
  fprintf(stderr, "acoref: draw outside any known site\n");
  abort();
}

}  // namespace

extern "C" {

/* ld --wrap targets: Utils::random(long*) and Utils::sort2(int*, int*, int, int). */
float __real__ZN5Utils6randomEPl(long *idum);
float __wrap__ZN5Utils6randomEPl(long *idum) {
  (void)idum;
  g_draws++;
  return draw_for_current_caller();
}

void __real__ZN5Utils5sort2EPiS0_ii(int v[], int v2[], int left, int right);
void __wrap__ZN5Utils5sort2EPiS0_ii(int v[], int v2[], int left, int right) {
  if (!g_stable_nn) {
    __real__ZN5Utils5sort2EPiS0_ii(v, v2, left, right);
    return;
  }
  std::vector<std::pair<int, int> > p;
  for (int i = left; i <= right; i++) p.push_back(std::make_pair(v[i], v2[i]));
  std::stable_sort(p.begin(), p.end(),
                   [](const std::pair<int, int> &a, const std::pair<int, int> &b) {
                     return a.first < b.first;
                   });
  for (int i = left; i <= right; i++) {
    v[i] = p[i - left].first;
    v2[i] = p[i - left].second;
  }
}

int acoref_is_aging(void) { return ANTS_AGING ? 1 : 0; }

void acoref_set_stable_nn(int stable) { g_stable_nn = stable; }

void *acoref_create(int *dist, int n, int m, float alpha, float beta, float rho,
                    const int *aging6) {
  OracleAS *c;
#if ANTS_AGING
  if (!aging6) return 0;
  c = new OracleAS(dist, n, m, alpha, beta, rho, aging6[0], aging6[1], aging6[2],
                   aging6[3], aging6[4], aging6[5]);
#else
  (void)aging6;
  c = new OracleAS(dist, n, m, alpha, beta, rho);
#endif
  g_cur = c;
  g_iter = 0;
  return c;
}

void acoref_set_rng(void *h, uint64_t seed) {
  g_cur = (OracleAS *)h;
  g_seed = seed;
  g_iter = 0;
}

void acoref_initialize(void *h) {
  g_cur = (OracleAS *)h;
  g_cur->initialize();
}

void acoref_iterate(void *h, float *timers6) {
  float t[6] = {0, 0, 0, 0, 0, 0};
  g_cur = (OracleAS *)h;
  g_cursor.phase = 0;
  g_cursor.step = 1;
  g_cursor.ant = 0;
  g_cur->constructSolution(t);
  g_iter++;
  if (timers6) memcpy(timers6, t, sizeof(t));
}

long acoref_draw_count(void) { return g_draws; }

void acoref_get_pheromone(void *h, float *out) {
  OracleAS *c = (OracleAS *)h;
  memcpy(out, c->pher(), sizeof(float) * c->cities() * c->cities());
}

void acoref_get_heuristic(void *h, float *out) {
  OracleAS *c = (OracleAS *)h;
  memcpy(out, c->heur(), sizeof(float) * c->cities() * c->cities());
}

void acoref_get_nnlist(void *h, int32_t *out) {
  OracleAS *c = (OracleAS *)h;
  const long nn2 = (long)c->cities() * c->cities();
  for (long i = 0; i < nn2; i++) out[i] = c->nn()[i];
}

void acoref_get_tours(void *h, int32_t *out) {
  OracleAS *c = (OracleAS *)h;
  const long mn = (long)c->ants() * c->cities();
  for (long i = 0; i < mn; i++) out[i] = (int32_t)c->tours()[i];
}

void acoref_get_lengths(void *h, int64_t *out) {
  OracleAS *c = (OracleAS *)h;
  for (int k = 0; k < c->ants(); k++) out[k] = c->lengths()[k];
}

void acoref_get_best_tour(void *h, int32_t *out) {
  OracleAS *c = (OracleAS *)h;
  for (int i = 0; i < c->cities(); i++) out[i] = (int32_t)c->best_tour()[i];
}

long acoref_iter_best(void *h) { return ((OracleAS *)h)->getIterBestDist(); }
long acoref_glob_best(void *h) { return ((OracleAS *)h)->getGlobBestDist(); }
unsigned acoref_num_valid(void *h) { return ((OracleAS *)h)->getNumValidAnts(); }

/* Aging state: age[m], performance[m], valid[m], pheromone row means[n],
 * misc[2] = {isconverged, globalperformance}.  No-op on the noaging build. */
void acoref_get_aging(void *h, int32_t *age, int32_t *perf, uint8_t *valid,
                      float *mean, int32_t *misc) {
#if ANTS_AGING
  OracleAS *c = (OracleAS *)h;
  for (int k = 0; k < c->ants(); k++) {
    age[k] = c->ages()[k];
    perf[k] = c->perfs()[k];
    valid[k] = c->valids()[k];
  }
  for (int i = 0; i < c->cities(); i++) mean[i] = c->means()[i];
  misc[0] = isconverged;
  misc[1] = c->global_perf();
#else
  (void)h; (void)age; (void)perf; (void)valid; (void)mean; (void)misc;
#endif
}

void acoref_destroy(void *h) {
  OracleAS *c = (OracleAS *)h;
  if (g_cur == c) g_cur = 0;
  delete c;
}

}  /* extern "C" */
