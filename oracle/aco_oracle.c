/*
 * aco_oracle.c -- TEST INFRASTRUCTURE: CPU oracle of the GB300 ACO engine
 * (see aco_oracle.h).  Compiled with -ffp-contract=off so every float
 * operation rounds once, as in the reference's CPU build and in the GPU
 * kernels (which spell out __fmul_rn/__fadd_rn).
 *
 * Construction runs ant-major and can use several threads: with the
 * counter-based random stream each ant's tour depends only on its own
 * counters and the shared read-only state, so the result is identical to
 * the reference's step-major order (src/Colony.cu:766-787).
 */
#define _GNU_SOURCE
#include "aco_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "acogpu_rng.h"

/* ---------------------------------------------------------------- helpers */

/* Utils::round_distance, src/Utils.cu:212-218: the coordinate differences
 * are taken in float, the root in double. */
static int32_t round_distance(float xi, float xj, float yi, float yj) {
  double xd = xi - xj;
  double yd = yi - yj;
  double r = sqrt(xd * xd + yd * yd) + 0.5;
  return (int32_t)r;
}

void oc_distances(const float *x, const float *y, int32_t n, int32_t *out) {
  for (int32_t i = 0; i < n; i++) {
    out[(int64_t)i * n + i] = ACO_MAX_DISTANCE;
    for (int32_t j = i + 1; j < n; j++) {
      int32_t d = round_distance(x[i], x[j], y[i], y[j]);
      out[(int64_t)i * n + j] = d;
      out[(int64_t)j * n + i] = d;
    }
  }
}

/* Utils::sort2 (src/Utils.cu:136-159): quicksort with the middle element as
 * pivot, the pivot kept in the left part.  Restated with an explicit stack;
 * the subranges are disjoint, so the processing order does not change the
 * final permutation. */
static void ref_quicksort(int32_t *v, int32_t *v2, int32_t left0, int32_t right0,
                          int32_t *stack) {
  int32_t sp = 0;
  stack[sp++] = left0;
  stack[sp++] = right0;
  while (sp > 0) {
    int32_t right = stack[--sp];
    int32_t left = stack[--sp];
    if (left >= right) continue;
    int32_t mid = (left + right) / 2, t;
    t = v[left]; v[left] = v[mid]; v[mid] = t;
    t = v2[left]; v2[left] = v2[mid]; v2[mid] = t;
    int32_t last = left;
    for (int32_t k = left + 1; k <= right; k++) {
      if (v[k] < v[left]) {
        ++last;
        t = v[last]; v[last] = v[k]; v[k] = t;
        t = v2[last]; v2[last] = v2[k]; v2[k] = t;
      }
    }
    t = v[left]; v[left] = v[last]; v[last] = t;
    t = v2[left]; v2[left] = v2[last]; v2[last] = t;
    stack[sp++] = left;
    stack[sp++] = last;
    stack[sp++] = last + 1;
    stack[sp++] = right;
  }
}

typedef struct { int32_t d, i; } dkey;
static int dkey_cmp(const void *a, const void *b) {
  const dkey *x = (const dkey *)a, *y = (const dkey *)b;
  if (x->d != y->d) return x->d < y->d ? -1 : 1;
  return x->i < y->i ? -1 : (x->i > y->i);
}

void oc_nn_rows(const int32_t *dist, int32_t n, int32_t order, int32_t *out) {
  if (order == ACO_NN_REFERENCE_QSORT) {
    int32_t *v = (int32_t *)malloc(sizeof(int32_t) * n);
    int32_t *stack = (int32_t *)malloc(sizeof(int32_t) * (4 * (size_t)n + 8));
    for (int32_t r = 0; r < n; r++) {
      int32_t *v2 = out + (int64_t)r * n;
      for (int32_t i = 0; i < n; i++) {
        v[i] = dist[(int64_t)r * n + i];
        v2[i] = i;
      }
      ref_quicksort(v, v2, 0, n - 1, stack);
    }
    free(stack);
    free(v);
  } else {
    dkey *k = (dkey *)malloc(sizeof(dkey) * n);
    for (int32_t r = 0; r < n; r++) {
      for (int32_t i = 0; i < n; i++) {
        k[i].d = dist[(int64_t)r * n + i];
        k[i].i = i;
      }
      qsort(k, (size_t)n, sizeof(dkey), dkey_cmp);
      for (int32_t i = 0; i < n; i++) out[(int64_t)r * n + i] = k[i].i;
    }
    free(k);
  }
}

/* x^b for integer b >= 1, correctly rounded except within ~b*2^-46 of a
 * rounding midpoint: double-float accumulation with exact products (fmaf). */
static float pow_int_cr(float x, int b) {
  if (b == 0) return 1.0f;
  if (isinf(x) || x == 0.0f) return b > 0 ? (isinf(x) ? x : 0.0f) : 1.0f;
  float hi = x, lo = 0.0f;
  for (int i = 1; i < b; i++) {
    float p = hi * x;
    float e = fmaf(hi, x, -p);
    e = fmaf(lo, x, e);
    float s = p + e;
    lo = e - (s - p);
    hi = s;
  }
  return hi;
}

float oc_heuristic(int32_t d, float beta, int32_t mode) {
  if (d == ACO_MAX_DISTANCE) return 0.0f;
  if (mode == ACO_HEURISTIC_LIBM) {
    /* HURESTIC(d,b), inc/Colony.h:20 */
    return powf((float)(1.0 / ((float)d)), beta);
  }
  float x = 1.0f / (float)d;
  if (beta == floorf(beta) && beta >= 0.0f && beta <= 64.0f) return pow_int_cr(x, (int)beta);
  return powf(x, beta);
}

int64_t oc_greedy_length(const int32_t *dist, int32_t n) {
  uint8_t *vis = (uint8_t *)calloc((size_t)n, 1);
  int32_t cur = 0;
  int64_t len = 0;
  vis[0] = 1;
  for (int32_t s = 1; s < n; s++) {
    int32_t best = -1, bd = 0;
    for (int32_t j = 0; j < n; j++) {
      if (vis[j]) continue;
      int32_t d = dist[(int64_t)cur * n + j];
      if (best < 0 || d < bd) { best = j; bd = d; }
    }
    len += bd;
    vis[best] = 1;
    cur = best;
  }
  len += dist[(int64_t)cur * n + 0];
  free(vis);
  return len;
}

/* ---------------------------------------------------------------- colony */

struct oc_colony {
  aco_params p;
  int32_t n, m, k; /* k = candidates per row */
  int32_t threads;
  int32_t *dist;   /* n*n */
  int32_t *nn;     /* n*n full sorted rows */
  float *eta;      /* n*n */
  float *tau;      /* n*n */
  float *choice;   /* n*n, tau*eta */
  float tau0;
  int32_t *tour;   /* m*n */
  int64_t *newlen; /* m: lengths of this iteration */
  int64_t *len;    /* m: the reference's tourlength[] */
  int32_t *gbtour; /* n */
  int64_t iter_best, glob_best;
  uint32_t iteration;
  int64_t fallbacks;
  /* aging (inc/Colony.h:100-125) */
  int32_t *age, *perf;
  uint8_t *valid;
  float *mean;
  int32_t num_valid, isconverged, globalperformance;
  /* candidate heuristic (n*k, candidate order) when a learned prior is
   * installed; NULL: the plain heuristic */
  float *eta_nn;
  /* deposit list of the current iteration */
  int32_t *dep_src; /* ant index, or -1 for the best-so-far tour */
  float *dep_delta;
  int32_t dep_count;
};

int oc_create(const aco_params *p, const int32_t *dist, int32_t n, oc_colony **out) {
  if (!p || !dist || !out || n < 3 || p->num_ants < 1) return ACO_ERR_INVALID_ARGUMENT;
  oc_colony *c = (oc_colony *)calloc(1, sizeof(oc_colony));
  c->p = *p;
  c->n = n;
  c->m = p->num_ants;
  c->k = (p->cand_k <= 0 || p->cand_k >= n) ? n : p->cand_k;
  if (c->k < n && p->fallback == ACO_FALLBACK_REFERENCE) {
    free(c);
    return ACO_ERR_UNSUPPORTED;
  }
  c->threads = 1;
  size_t nn2 = (size_t)n * n, mn = (size_t)c->m * n;
  c->dist = (int32_t *)malloc(sizeof(int32_t) * nn2);
  memcpy(c->dist, dist, sizeof(int32_t) * nn2);
  c->nn = (int32_t *)malloc(sizeof(int32_t) * nn2);
  c->eta = (float *)malloc(sizeof(float) * nn2);
  c->tau = (float *)malloc(sizeof(float) * nn2);
  c->choice = (float *)malloc(sizeof(float) * nn2);
  c->tour = (int32_t *)calloc(mn, sizeof(int32_t));
  c->newlen = (int64_t *)calloc((size_t)c->m, sizeof(int64_t));
  c->len = (int64_t *)calloc((size_t)c->m, sizeof(int64_t));
  c->gbtour = (int32_t *)calloc((size_t)n, sizeof(int32_t));
  c->age = (int32_t *)calloc((size_t)c->m, sizeof(int32_t));
  c->perf = (int32_t *)calloc((size_t)c->m, sizeof(int32_t));
  c->valid = (uint8_t *)calloc((size_t)c->m, 1);
  c->mean = (float *)calloc((size_t)n, sizeof(float));
  c->dep_src = (int32_t *)malloc(sizeof(int32_t) * ((size_t)c->m + 1));
  c->dep_delta = (float *)malloc(sizeof(float) * ((size_t)c->m + 1));
  *out = c;
  return ACO_OK;
}

void oc_set_threads(oc_colony *c, int32_t threads) { c->threads = threads < 1 ? 1 : threads; }

void oc_destroy(oc_colony *c) {
  if (!c) return;
  free(c->dist); free(c->nn); free(c->eta); free(c->tau); free(c->choice);
  free(c->tour); free(c->newlen); free(c->len); free(c->gbtour);
  free(c->age); free(c->perf); free(c->valid); free(c->mean);
  free(c->dep_src); free(c->dep_delta); free(c->eta_nn);
  free(c);
}

/* adj_pheromone (src/AntSystem.cu:9-11) with MIN_PHEROMONE 1e-18
 * (inc/default.h:16): the double comparison equals a float max against
 * (float)1e-18. */
static float adj_pheromone(float x) {
  const float fmin = (float)0.000000000000000001;
  return x > fmin ? x : fmin;
}

/* Derived per-row state after tau changes: choice = tau*eta (the noaging
 * fitness, inc/Colony.cuh:29-30) and, for aging, the row means of
 * Colony::computePheromoneMean (src/Colony.cu:435-441). */
static void refresh_rows(oc_colony *c) {
  const int32_t n = c->n;
  for (int32_t i = 0; i < n; i++) {
    const float *t = c->tau + (int64_t)i * n;
    const float *e = c->eta + (int64_t)i * n;
    float *ch = c->choice + (int64_t)i * n;
    for (int32_t j = 0; j < n; j++) {
      float tj = t[j];
      if (c->p.use_alpha) tj = powf(tj, c->p.alpha);
      ch[j] = tj * e[j];
    }
    if (c->p.aging) {
      float sum = 0;
      for (int32_t j = 0; j < n; j++) sum += t[j];
      c->mean[i] = sum / (float)n;
    }
  }
}

void oc_initialize(oc_colony *c) {
  const int32_t n = c->n, m = c->m;
  const size_t nn2 = (size_t)n * n;
  /* computeParameters -> computeInitialPheromone */
  if (c->p.variant == ACO_RANK_BASED && c->p.rank_w > n) c->p.rank_w = n; /* src/RankBasedAntSystem.cu:31-36 */
  if (c->p.tau0_mode == ACO_TAU0_REFERENCE) {
    c->tau0 = (float)0.000001; /* DEFAULT_PHEROMONE, inc/default.h:15 */
  } else if (c->p.tau0_mode == ACO_TAU0_VALUE) {
    c->tau0 = c->p.tau0;
  } else {
    int64_t cnn = oc_greedy_length(c->dist, n);
    if (c->p.variant == ACO_RANK_BASED) {
      float w = (float)c->p.rank_w;
      float num = (0.5f * w) * (float)(c->p.rank_w - 1);
      c->tau0 = num / (c->p.rho * (float)cnn);
    } else {
      c->tau0 = (float)m / (float)cnn;
    }
  }
  for (size_t i = 0; i < nn2; i++) c->tau[i] = c->tau0;
  for (size_t i = 0; i < nn2; i++) c->eta[i] = oc_heuristic(c->dist[i], c->p.beta, c->p.heuristic);
  oc_nn_rows(c->dist, n, c->p.nn_order, c->nn);
  /* initAntAges (src/Colony.cu:339-349): initial population = m */
  for (int32_t k = 0; k < m; k++) {
    c->age[k] = 0;
    c->perf[k] = 0;
    c->valid[k] = 1;
    c->len[k] = 0;
  }
  c->num_valid = m;
  c->isconverged = 0;
  c->globalperformance = 0;
  c->iter_best = (int64_t)ACO_MAX_DISTANCE - 1;
  c->glob_best = ACO_MAX_DISTANCE;
  c->iteration = 0;
  refresh_rows(c);
}

/* compute_fittness, inc/Colony.cuh:14-31 (alpha ignored unless use_alpha) */
static float fitness(const oc_colony *c, int32_t cur, int32_t city, int32_t ant) {
  const int64_t xy = (int64_t)cur * c->n + city;
  if (!c->p.aging) return c->choice[xy];
  float p = c->tau[xy];
  if (c->age[ant] < c->p.min_retirement_age && c->isconverged) {
    float ratio = (float)c->age[ant] / (float)c->p.min_retirement_age;
    p = ((p - c->mean[cur]) * ratio) + c->mean[cur];
  }
  if (c->p.use_alpha) p = powf(p, c->p.alpha);
  return p * c->eta[xy];
}

/* Weight of candidate r (city `city`) of row `cur`: the fitness with the
 * candidate heuristic in place of eta when a prior is installed. */
static float cand_fitness(const oc_colony *c, int32_t cur, int32_t r, int32_t city, int32_t ant) {
  if (!c->eta_nn) return fitness(c, cur, city, ant);
  const int64_t xy = (int64_t)cur * c->n + city;
  float p = c->tau[xy];
  if (c->p.aging && c->age[ant] < c->p.min_retirement_age && c->isconverged) {
    float ratio = (float)c->age[ant] / (float)c->p.min_retirement_age;
    p = ((p - c->mean[cur]) * ratio) + c->mean[cur];
  }
  if (c->p.use_alpha) p = powf(p, c->p.alpha);
  return p * c->eta_nn[(int64_t)cur * c->k + r];
}

void oc_set_candidate_heuristic(oc_colony *c, const float *eta_nk) {
  if (!c->eta_nn) c->eta_nn = (float *)malloc(sizeof(float) * (size_t)c->n * c->k);
  memcpy(c->eta_nn, eta_nk, sizeof(float) * (size_t)c->n * c->k);
}

/* select_local_best, inc/Colony.cuh:33-43: index of the last unvisited city
 * of the full nn row. */
static int32_t last_unvisited(const oc_colony *c, const int32_t *nnrow, const uint8_t *vis) {
  for (int32_t i = c->n - 1; i >= 0; i--)
    if (!vis[nnrow[i]]) return i;
  return -1;
}

static int32_t fallback_city(const oc_colony *c, int32_t cur, const uint8_t *vis, int32_t ant) {
  if (c->p.fallback == ACO_FALLBACK_REFERENCE) {
    const int32_t *row = c->nn + (int64_t)cur * c->n;
    return row[last_unvisited(c, row, vis)];
  }
  int32_t best = -1;
  float vbest = -1.0f;
  for (int32_t j = 0; j < c->n; j++) {
    if (vis[j]) continue;
    float w = fitness(c, cur, j, ant);
    if (w > vbest) { vbest = w; best = j; }
  }
  return best;
}

typedef struct {
  oc_colony *c;
  int32_t first, last;
  int64_t fallbacks;
} worker_arg;

static void construct_ant(oc_colony *c, int32_t k, float *w, uint8_t *vis, int64_t *fb) {
  const int32_t n = c->n, K = c->k;
  int32_t *t = c->tour + (int64_t)k * n;
  memset(vis, 0, (size_t)n);
  /* initTour placement, src/Colony.cu:514-524 */
  float u0 = aco_uniform(c->p.seed, c->iteration, (uint32_t)k, 0u);
  int32_t start = (int32_t)(u0 * (float)n);
  t[0] = start;
  vis[start] = 1;
  int64_t len = 0;
  for (int32_t x = 1; x < n; x++) {
    const int32_t cur = t[x - 1];
    const int32_t *row = c->nn + (int64_t)cur * n;
    /* calculateProbabilityOfSelection, src/Colony.cu:795-818 (first K of the row) */
    float sum = 0;
    for (int32_t i = 0; i < K; i++) {
      int32_t city = row[i];
      w[i] = vis[city] ? 0.0f : cand_fitness(c, cur, i, city, k);
      sum += w[i];
    }
    int32_t next;
    if (sum <= 0.0f) { /* chooseBestNext, src/Colony.cu:776-778,853-864 */
      next = fallback_city(c, cur, vis, k);
      (*fb)++;
    } else { /* selectCities, src/Colony.cu:821-851 */
      float rnd = aco_uniform(c->p.seed, c->iteration, (uint32_t)k, (uint32_t)x);
      rnd *= sum;
      int32_t i = 0;
      float partial = w[0];
      while (partial <= rnd) {
        i++;
        if (i >= K) { i = -1; break; }
        partial += w[i];
      }
      if (i >= 0) {
        next = row[i];
      } else {
        next = fallback_city(c, cur, vis, k);
        (*fb)++;
      }
    }
    t[x] = next;
    vis[next] = 1;
    len += c->dist[(int64_t)cur * n + next];
  }
  len += c->dist[(int64_t)t[n - 1] * n + t[0]];
  c->newlen[k] = len;
}

static void *construct_worker(void *argp) {
  worker_arg *a = (worker_arg *)argp;
  oc_colony *c = a->c;
  float *w = (float *)malloc(sizeof(float) * c->n);
  uint8_t *vis = (uint8_t *)malloc((size_t)c->n);
  for (int32_t k = a->first; k < a->last; k++) {
    if (c->valid[k])
      construct_ant(c, k, w, vis, &a->fallbacks);
    else /* initTour clears every tour row (src/Colony.cu:507-510) */
      memset(c->tour + (int64_t)k * c->n, 0, sizeof(int32_t) * c->n);
  }
  free(w);
  free(vis);
  return 0;
}

static void construct_all(oc_colony *c) {
  int32_t T = c->threads > c->m ? c->m : c->threads;
  worker_arg *args = (worker_arg *)calloc((size_t)T, sizeof(worker_arg));
  pthread_t *th = (pthread_t *)calloc((size_t)T, sizeof(pthread_t));
  for (int32_t i = 0; i < T; i++) {
    args[i].c = c;
    args[i].first = (int32_t)((int64_t)c->m * i / T);
    args[i].last = (int32_t)((int64_t)c->m * (i + 1) / T);
  }
  for (int32_t i = 1; i < T; i++) pthread_create(&th[i], 0, construct_worker, &args[i]);
  construct_worker(&args[0]);
  c->fallbacks = args[0].fallbacks;
  for (int32_t i = 1; i < T; i++) {
    pthread_join(th[i], 0);
    c->fallbacks += args[i].fallbacks;
  }
  free(th);
  free(args);
}

static void add_edge(float *tau, int32_t n, int32_t j, int32_t h, float d) {
  tau[(int64_t)j * n + h] += d;
  tau[(int64_t)h * n + j] = tau[(int64_t)j * n + h];
}

void oc_iterate(oc_colony *c) {
  const int32_t n = c->n, m = c->m;
  /* updateAntAges (src/Colony.cu:361-362): every ant, valid or not; the
   * placement draws do not read the ages, so the order is immaterial. */
  if (c->p.aging)
    for (int32_t k = 0; k < m; k++) c->age[k] = c->age[k] + 1;
  construct_all(c);

  /* computeAntDistances, src/Colony.cu:996-1043 */
  int32_t best_ant = -1;
  c->iter_best = (int64_t)ACO_MAX_DISTANCE - 1;
  for (int32_t k = 0; k < m; k++) {
    if (!c->valid[k]) continue;
    int64_t L = c->newlen[k];
    if (c->p.aging) c->perf[k] = (L == c->len[k]) ? c->perf[k] + 1 : 0;
    c->len[k] = L;
    if (L < c->iter_best) {
      best_ant = k;
      c->iter_best = L;
    }
  }
  if (c->iter_best < c->glob_best && best_ant > -1) {
    c->glob_best = c->iter_best;
    memcpy(c->gbtour, c->tour + (int64_t)best_ant * n, sizeof(int32_t) * n);
    c->globalperformance = 0;
  } else {
    c->globalperformance++;
  }

  /* deposit list */
  c->dep_count = 0;
  if (c->p.variant == ACO_RANK_BASED) {
    int32_t w = c->p.rank_w;
    uint8_t *taken = (uint8_t *)calloc((size_t)m, 1);
    for (int32_t r = 0; r < w - 1; r++) {
      int32_t b = -1;
      for (int32_t k = 0; k < m; k++) {
        if (!c->valid[k] || taken[k]) continue;
        if (b < 0 || c->len[k] < c->len[b]) b = k;
      }
      if (b < 0) break;
      taken[b] = 1;
      c->dep_src[c->dep_count] = b;
      c->dep_delta[c->dep_count] = (float)(w - 1 - r) / (float)c->len[b];
      c->dep_count++;
    }
    free(taken);
    if (c->glob_best < ACO_MAX_DISTANCE) {
      c->dep_src[c->dep_count] = -1;
      c->dep_delta[c->dep_count] = (float)w / (float)c->glob_best;
      c->dep_count++;
    }
  } else {
    for (int32_t k = 0; k < m; k++) {
      if (!c->valid[k]) continue;
      c->dep_src[c->dep_count] = k;
      c->dep_delta[c->dep_count] = (float)(1.0 / (float)c->len[k]); /* src/AntSystem.cu:300 */
      c->dep_count++;
    }
  }

  /* evaporatePheromones, src/AntSystem.cu:218-223 (tau stays symmetric, so
   * the elementwise form is the same) */
  const float keep = 1 - c->p.rho;
  for (size_t i = 0; i < (size_t)n * n; i++) c->tau[i] = adj_pheromone(keep * c->tau[i]);

  /* updatePheromones, src/AntSystem.cu:296-316 */
  for (int32_t q = 0; q < c->dep_count; q++) {
    const int32_t *t = c->dep_src[q] < 0 ? c->gbtour : c->tour + (int64_t)c->dep_src[q] * n;
    float d = c->dep_delta[q];
    for (int32_t i = 0; i < n - 1; i++) add_edge(c->tau, n, t[i], t[i + 1], d);
    add_edge(c->tau, n, t[n - 1], t[0], d);
  }

  /* retireAnts / recruiteAnts, src/Colony.cu:379-393, 399-422 */
  if (c->p.aging) {
    for (int32_t i = 0; i < m / 2; i++) {
      if (c->valid[i] && c->age[i] >= c->p.max_retirement_age) {
        c->valid[i] = 0;
        c->num_valid--;
        c->isconverged = 1;
        break;
      }
    }
    uint32_t va = (uint32_t)c->num_valid;
    if (c->globalperformance >= c->p.global_performance ||
        va < (uint32_t)c->p.min_population_limit) {
      for (int32_t i = 0; i < m; i++) {
        if (!c->valid[i]) {
          c->valid[i] = 1;
          c->age[i] = 0;
          c->num_valid++;
          break;
        }
      }
    }
  }
  refresh_rows(c);
  c->iteration++;
}

int64_t oc_iter_best(const oc_colony *c) { return c->iter_best; }
int64_t oc_glob_best(const oc_colony *c) { return c->glob_best; }
int32_t oc_num_valid(const oc_colony *c) { return c->p.aging ? c->num_valid : c->m; }
int32_t oc_cand_k(const oc_colony *c) { return c->k; }
float oc_tau0(const oc_colony *c) { return c->tau0; }
int64_t oc_fallback_count(const oc_colony *c) { return c->fallbacks; }

void oc_get_pheromone(const oc_colony *c, float *out) {
  memcpy(out, c->tau, sizeof(float) * (size_t)c->n * c->n);
}
void oc_set_pheromone(oc_colony *c, const float *in) {
  memcpy(c->tau, in, sizeof(float) * (size_t)c->n * c->n);
  refresh_rows(c);
}
void oc_get_heuristic(const oc_colony *c, float *out) {
  memcpy(out, c->eta, sizeof(float) * (size_t)c->n * c->n);
}
void oc_get_choice(const oc_colony *c, float *out) {
  memcpy(out, c->choice, sizeof(float) * (size_t)c->n * c->n);
}
void oc_get_nn(const oc_colony *c, int32_t *out) {
  for (int32_t i = 0; i < c->n; i++)
    memcpy(out + (int64_t)i * c->k, c->nn + (int64_t)i * c->n, sizeof(int32_t) * c->k);
}
void oc_get_tours(const oc_colony *c, int32_t *out) {
  memcpy(out, c->tour, sizeof(int32_t) * (size_t)c->m * c->n);
}
void oc_get_lengths(const oc_colony *c, int64_t *out) {
  memcpy(out, c->len, sizeof(int64_t) * (size_t)c->m);
}
void oc_get_best_tour(const oc_colony *c, int32_t *out) {
  memcpy(out, c->gbtour, sizeof(int32_t) * (size_t)c->n);
}
void oc_get_aging(const oc_colony *c, int32_t *age, int32_t *perf, uint8_t *valid,
                  float *mean, int32_t *misc) {
  memcpy(age, c->age, sizeof(int32_t) * c->m);
  memcpy(perf, c->perf, sizeof(int32_t) * c->m);
  memcpy(valid, c->valid, (size_t)c->m);
  memcpy(mean, c->mean, sizeof(float) * c->n);
  misc[0] = c->isconverged;
  misc[1] = c->globalperformance;
}

void oc_pheromone_update_f64(double *tau, int32_t n, double rho, int32_t count,
                             const int32_t *tours, const int64_t *lens,
                             const double *weights) {
  for (size_t i = 0; i < (size_t)n * n; i++) {
    double v = (1.0 - rho) * tau[i];
    tau[i] = v > 1e-18 ? v : 1e-18;
  }
  for (int32_t q = 0; q < count; q++) {
    const int32_t *t = tours + (int64_t)q * n;
    double d = weights[q] / (double)lens[q];
    for (int32_t i = 0; i < n; i++) {
      int32_t a = t[i], b = t[(i + 1) % n];
      tau[(int64_t)a * n + b] += d;
      tau[(int64_t)b * n + a] = tau[(int64_t)a * n + b];
    }
  }
}
