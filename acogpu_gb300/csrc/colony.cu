// colony.cu -- host implementation of the C ABI in include/acogpu.h.
//
// One colony = one set of device buffers (layout in aco_device.cuh) + one
// stream.  An iteration is three kernels (construct, epilogue, pheromone
// rows), or five in atomic-deposit mode, with no host synchronisation; the
// iteration is captured once into a CUDA graph and replayed by
// aco_colony_run.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <atomic>
#include <new>
#include <string>
#include <vector>

#include "acogpu.h"
#include "aco_kernels.h"

using namespace aco;

#include "colony_internal.h"

namespace {

const char *kNameAS = "Ant System";             // src/AntSystem.cu:7
const char *kNameRBAS = "Rank-based Ant System";  // src/RankBasedAntSystem.cu:10

// NVTX range over an API call: named in a profiler's timeline (nsys), a
// no-op without one attached.
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
};

int fail(aco_colony *c, int status, const std::string &msg) {
  if (c) c->err = msg;
  return status;
}

int cuda_fail(aco_colony *c, cudaError_t e, const char *what) {
  std::string msg = std::string(what) + ": " + cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) return fail(c, ACO_ERR_OUT_OF_MEMORY, msg);
  return fail(c, ACO_ERR_CUDA, msg);
}

#define ACO_CUDA(c, call, what)                          \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return cuda_fail(c, e_, what); \
  } while (0)

// Fault injection on the host: the `g_fail_alloc`-th next device allocation
// of a colony reports out-of-memory without allocating (-1: off).
std::atomic<int> g_fail_alloc{-1};

// Counts one allocation against the injected failure; true if it fails.
bool injected_failure() {
  int k = g_fail_alloc.load();
  while (k >= 0 && !g_fail_alloc.compare_exchange_weak(k, k - 1)) {
  }
  return k == 0;
}

template <class T>
int dalloc(aco_colony *c, T **ptr, size_t count) {
  if (injected_failure())
    return fail(c, ACO_ERR_OUT_OF_MEMORY, "cudaMalloc: injected allocation failure");
  void *p = nullptr;
  cudaError_t e = cudaMalloc(&p, count * sizeof(T) + 16);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaMalloc");
  c->allocations.push_back(p);
  *ptr = static_cast<T *>(p);
  return ACO_OK;
}

// A colony's arrays from one device allocation (a cudaMalloc costs tens of
// microseconds, and a batch creates a few hundred arrays): the requests are
// listed first, then each counts against the injected failure in turn, then
// one block is allocated and carved at 256-byte boundaries (16 bytes of
// slack past each array, as dalloc leaves).
struct Carve {
  std::vector<std::pair<void **, size_t>> req;
  template <class T>
  void add(T **ptr, size_t count) {
    req.emplace_back(reinterpret_cast<void **>(ptr), count * sizeof(T) + 16);
  }
  int commit(aco_colony *c) {
    size_t total = 0;
    for (const auto &r : req) {
      if (injected_failure())
        return fail(c, ACO_ERR_OUT_OF_MEMORY, "cudaMalloc: injected allocation failure");
      total += (r.second + 255) / 256 * 256;
    }
    void *base = nullptr;
    const cudaError_t e = cudaMalloc(&base, total);
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaMalloc");
    c->allocations.push_back(base);
    char *p = static_cast<char *>(base);
    for (const auto &r : req) {
      *r.first = p;
      p += (r.second + 255) / 256 * 256;
    }
    return ACO_OK;
  }
};

ColonyDev make_dev(const aco_colony *c) {
  ColonyDev d;
  d.n = c->n; d.m = c->m; d.K = c->K; d.ld = c->ld; d.ldk = c->ldk; d.ldm = c->ldm;
  d.dist = c->dist; d.eta = c->eta; d.tau = c->tau; d.choice = c->choice;
  d.nn = c->nn; d.nn16 = c->nn16;
  d.eta_nn = c->eta_nn; d.tau_nn = c->tau_nn; d.choice_nn = c->choice_nn;
  d.tours = c->tours; d.newlen = c->newlen; d.len = c->len;
  d.succT = c->succT; d.predT = c->predT; d.gbtour = c->gbtour;
  d.age = c->age; d.perf = c->perf; d.valid = c->valid; d.mean = c->mean;
  d.dep_col = c->dep_col; d.dep_delta = c->dep_delta; d.plan = c->plan; d.st = c->st;
  d.nn2 = c->nn2; d.t2v = c->t2v; d.mout = c->mout; d.t2 = c->t2;
  d.rho = c->p.rho; d.alpha = c->p.alpha; d.use_alpha = c->p.use_alpha;
  d.aging = c->p.aging; d.min_ret = c->p.min_retirement_age;
  d.max_ret = c->p.max_retirement_age; d.global_perf = c->p.global_performance;
  d.min_pop = c->p.min_population_limit;
  d.variant = c->p.variant; d.rank_w = c->p.rank_w; d.fallback = c->p.fallback;
  d.seed = c->p.seed;
  return d;
}

void drop_graph(aco_colony *c) {
  if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
  if (c->graph) cudaGraphDestroy(c->graph);
  c->graph_exec = nullptr;
  c->graph = nullptr;
}

int check_params(const aco_params *p, int n) {
  if (!p || n < 3) return ACO_ERR_INVALID_ARGUMENT;
  if (p->num_ants < 1 || p->num_ants > 65536) return ACO_ERR_INVALID_ARGUMENT;
  if (n >= (1 << 21)) return ACO_ERR_UNSUPPORTED;
  if (p->variant != ACO_ANT_SYSTEM && p->variant != ACO_RANK_BASED) return ACO_ERR_INVALID_ARGUMENT;
  if (p->nn_order != ACO_NN_STABLE && p->nn_order != ACO_NN_REFERENCE_QSORT)
    return ACO_ERR_INVALID_ARGUMENT;
  if (p->heuristic != ACO_HEURISTIC_DEVICE && p->heuristic != ACO_HEURISTIC_LIBM)
    return ACO_ERR_INVALID_ARGUMENT;
  if (p->fallback != ACO_FALLBACK_REFERENCE && p->fallback != ACO_FALLBACK_BEST)
    return ACO_ERR_INVALID_ARGUMENT;
  if (p->deposit != ACO_DEPOSIT_DETERMINISTIC && p->deposit != ACO_DEPOSIT_ATOMIC)
    return ACO_ERR_INVALID_ARGUMENT;
  if (p->tau0_mode < ACO_TAU0_REFERENCE || p->tau0_mode > ACO_TAU0_VALUE)
    return ACO_ERR_INVALID_ARGUMENT;
  const int K = (p->cand_k <= 0 || p->cand_k >= n) ? n : p->cand_k;
  if (K < n && p->fallback == ACO_FALLBACK_REFERENCE) return ACO_ERR_UNSUPPORTED;
  if (p->nn_order == ACO_NN_STABLE && n > 16384) return ACO_ERR_UNSUPPORTED;
  if (p->variant == ACO_RANK_BASED && p->rank_w < 1) return ACO_ERR_INVALID_ARGUMENT;
  if (p->ants_per_block < 0 || p->ants_per_block > 16) return ACO_ERR_INVALID_ARGUMENT;
  if (p->construct_mode < ACO_CONSTRUCT_AUTO || p->construct_mode > ACO_CONSTRUCT_ROWS)
    return ACO_ERR_INVALID_ARGUMENT;
  if (p->fallback_tier < ACO_FALLBACK_TIER_AUTO || p->fallback_tier > ACO_FALLBACK_TIER_OFF)
    return ACO_ERR_INVALID_ARGUMENT;
  if (p->construct_mode == ACO_CONSTRUCT_STAGED && (K > 32 || n > 2048))
    return ACO_ERR_UNSUPPORTED;
  if ((p->construct_mode == ACO_CONSTRUCT_DIRECT || p->construct_mode == ACO_CONSTRUCT_CLUSTER) &&
      (K > 32 || n > kDirectMaxCities))
    return ACO_ERR_UNSUPPORTED;
  if (p->construct_mode == ACO_CONSTRUCT_ROWS && (K <= 32 || n > kRowsMaxCities))
    return ACO_ERR_UNSUPPORTED;
  return ACO_OK;
}

int allocate(aco_colony *c) {
  const size_t n = c->n, m = c->m, ld = c->ld, ldk = c->ldk, ldm = c->ldm;
  int s;
  Carve a;
  a.add(&c->dist, n * ld);
  a.add(&c->eta, n * ld);
  a.add(&c->tau, n * ld);
  a.add(&c->choice, n * ld);
  a.add(&c->nn, n * ldk);
  a.add(&c->eta_nn, n * ldk);
  a.add(&c->choice_nn, n * ldk);
  a.add(&c->tau_nn, c->p.aging ? n * ldk : 32);
  a.add(&c->tours, m * ld);
  a.add(&c->newlen, m);
  a.add(&c->len, m);
  a.add(&c->succT, n * ldm);
  a.add(&c->predT, n * ldm);
  a.add(&c->gbtour, n);
  a.add(&c->age, m);
  a.add(&c->perf, m);
  a.add(&c->valid, m);
  a.add(&c->mean, ld);
  // Candidate ids as int16, for the k <= 32 kernels and the long-row kernel
  // (16 bytes of slack: the cluster kernel stages slices in 16-byte units).
  if (c->K <= 32 ? c->n < 32768 : c->n <= kRowsMaxCities) a.add(&c->nn16, n * ldk + 8);
  // The fallback's second tier, for the k <= 32 step loop.
  const bool tier = c->p.fallback_tier == ACO_FALLBACK_TIER_ON ||
                    (c->p.fallback_tier == ACO_FALLBACK_TIER_AUTO &&
                     c->p.variant == ACO_ANT_SYSTEM);
  c->t2 = (tier && c->K <= 32 && c->n < 32768) ? std::min(kTier2, c->n - 1 - c->K) : 0;
  if (c->t2 < 0) c->t2 = 0;
  if (c->t2 > 0) {
    a.add(&c->nn2, n * kTier2);
    a.add(&c->t2v, n * kTier2);
    a.add(&c->mout, n);
  }
  a.add(&c->plan, m + 2);
  a.add(&c->dep_col, m + 1);
  a.add(&c->dep_delta, m + 1);
  a.add(&c->st, 1);
  if ((s = a.commit(c))) return s;
  ACO_CUDA(c, cudaMemsetAsync(c->tours, 0, m * ld * 4, c->stream), "memset tours");
  ACO_CUDA(c, cudaMemsetAsync(c->st, 0, sizeof(ColonyState), c->stream), "memset state");
  ACO_CUDA(c, cudaMemsetAsync(c->gbtour, 0, n * 4, c->stream), "memset gbtour");
  return ACO_OK;
}

int create_common(const aco_params *params, int32_t n, aco_colony **out, aco_colony **cp) {
  if (!out) return ACO_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int s = check_params(params, n);
  if (s) return s;
  aco_colony *c = new (std::nothrow) aco_colony();
  if (!c) return ACO_ERR_OUT_OF_MEMORY;
  c->p = *params;
  c->n = n;
  c->m = params->num_ants;
  c->K = (params->cand_k <= 0 || params->cand_k >= n) ? n : params->cand_k;
  c->ld = round_up(n, 32);
  c->ldk = c->K <= 32 ? staged_pitch(c->K) : round_up(c->K, 32);
  c->ldm = round_up(c->m + 1, 32);
  c->apb = params->ants_per_block > 0 ? params->ants_per_block : 4;
  cudaGetDevice(&c->device);
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device);
  cudaDeviceGetAttribute(&c->max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device);
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    return ACO_ERR_CUDA;
  }
  c->own_stream = true;
  for (int i = 0; i < 4; i++) cudaEventCreate(&c->ev[i]);
  *cp = c;
  if ((s = allocate(c))) {
    aco_colony_destroy(c);
    *cp = nullptr;
    return s;
  }
  return ACO_OK;
}

}  // namespace

ColonyDev aco::colony_dev(const aco_colony *c) { return make_dev(c); }
int aco::colony_fail(aco_colony *c, int status, const std::string &msg) {
  return fail(c, status, msg);
}

namespace {

int device_error(aco_colony *c) {
  ColonyState h;
  ACO_CUDA(c, cudaMemcpyAsync(&h, c->st, sizeof(h), cudaMemcpyDeviceToHost, c->stream),
           "read state");
  ACO_CUDA(c, cudaStreamSynchronize(c->stream), "synchronize");
  if (h.error & kErrTimeout) return fail(c, ACO_ERR_DEVICE_TIMEOUT, "a bounded device wait expired");
  if (h.error & kErrCheck) return fail(c, ACO_ERR_DEVICE_CHECK, "a device-side check failed");
  return ACO_OK;
}

int read_state(aco_colony *c, ColonyState *h) {
  if (!c->initialized) return fail(c, ACO_ERR_NOT_INITIALIZED, "colony not initialized");
  if (!c->state_fresh) {
    if (!c->h_state && cudaMallocHost(&c->h_state, sizeof(ColonyState)) != cudaSuccess) {
      c->h_state = nullptr;
      return fail(c, ACO_ERR_OUT_OF_MEMORY, "cudaMallocHost");
    }
    ACO_CUDA(c, cudaMemcpyAsync(c->h_state, c->st, sizeof(*h), cudaMemcpyDeviceToHost, c->stream),
             "read state");
    ACO_CUDA(c, cudaStreamSynchronize(c->stream), "synchronize");
    c->h_cache = *c->h_state;
    c->state_fresh = true;
  }
  *h = c->h_cache;
  return ACO_OK;
}

// Launches of one construction: the staged kernel of an aging colony is
// preceded by the plan of the ants' roles.
int construction_launches(const aco_colony *c) {
  return (c->staged || c->rows) && c->p.aging ? 2 : 1;
}

cudaError_t launch_construction(aco_colony *c, const ColonyDev &d) {
  if (c->staged) {
    if (c->p.aging) {
      cudaError_t e = launch_aging_plan(d, c->stream);
      if (e != cudaSuccess) return e;
    }
    return launch_construct_staged(d, c->nn16, c->staged_grid, c->staged_warps, c->stream);
  }
  if (c->rows) return launch_construct_rows(d, c->staged_grid, c->staged_warps, c->stream);
  if (c->cluster)
    return launch_construct_cluster(d, c->staged_grid, c->staged_warps, c->cluster, c->stream);
  if (c->direct) return launch_construct_direct(d, c->staged_grid, c->staged_warps, c->stream);
  return launch_construct(d, c->apb, c->stream);
}

// Chooses the construction kernel, for k <= 32: the staged kernel (whole
// candidate table in shared memory, one CTA per SM) when the table fits, else
// the cluster kernel (the table split over ceil(n/1024) CTAs, n <= 8192),
// else the direct kernel (the same step loop on rows read from L2); otherwise,
// and in ACO_CONSTRUCT_GLOBAL mode, the general global-memory kernel.  The
// k <= 32 kernels put one ant per warp.  For k > 32 (mode AUTO or ROWS) the
// long-row kernel: A ants a CTA (a scan warp each, plus the chain warp), one
// CTA per SM, the ants spread evenly over the SMs (each ant's steps are a
// latency-bound chain of float adds).
int plan_construction(aco_colony *c) {
  c->staged = false;
  c->direct = false;
  c->cluster = 0;
  c->rows = false;
  const int mode = c->p.construct_mode;
  const int sms = c->num_sms > 0 ? c->num_sms : 1;
  if (c->nn16 && c->n <= kRowsMaxCities && c->K > 32 &&
      (mode == ACO_CONSTRUCT_ROWS || mode == ACO_CONSTRUCT_AUTO)) {
    const size_t per_ant = rows_ant_bytes(c->n, c->K);
    const size_t avail = (size_t)c->max_smem_optin - 1024;  // static shared memory
    int ants = c->tune_warps > 0 ? c->tune_warps : (c->m + sms - 1) / sms;
    ants = std::max(1, std::min(ants, kRowsMaxAnts));
    ants = std::min<int>(ants, (int)(avail / per_ant));
    if (ants < 1) return fail(c, ACO_ERR_UNSUPPORTED, "a long row does not fit in shared memory");
    ACO_CUDA(c, configure_construct_rows((size_t)ants * per_ant), "configure row construct");
    c->rows = true;
    c->staged_warps = ants;
    c->staged_grid = std::min(sms, (c->m + ants - 1) / ants);
    return ACO_OK;
  }
  if (c->K > 32 || !c->nn16 || mode == ACO_CONSTRUCT_GLOBAL) return ACO_OK;
  int warps = c->tune_warps > 0 ? c->tune_warps : (c->m + sms - 1) / sms;
  warps = warps < 1 ? 1 : (warps > kStagedMaxWarps ? kStagedMaxWarps : warps);
  int grid = (c->m + warps - 1) / warps;
  if (grid > sms) grid = sms;
  c->staged_warps = warps;
  c->staged_grid = grid;
  if (c->p.aging && c->n <= 2048) {
    // All SMs; up to min(m, min_ret) of them may run blend ants (one ant
    // recruited per iteration blends for min_ret iterations), and the
    // others' ants must fit in the remaining CTAs' warps.
    const int young = std::min(c->m, std::max(0, c->p.min_retirement_age));
    const int rest = std::max(1, sms - young);
    warps = (c->m + rest - 1) / rest;
    c->staged_warps = warps < 1 ? 1 : (warps > kStagedMaxWarps ? kStagedMaxWarps : warps);
    c->staged_grid = sms;
  }
  if (c->n <= 2048 && (mode == ACO_CONSTRUCT_AUTO || mode == ACO_CONSTRUCT_STAGED)) {
    const size_t smem =
        construct_staged_smem_bytes(c->n, c->ld, c->ldk, c->p.aging != 0, c->staged_warps);
    if (smem <= (size_t)c->max_smem_optin) {
      ACO_CUDA(c, configure_construct_staged(smem), "configure staged construct");
      c->staged = true;
      return ACO_OK;
    }
    if (mode == ACO_CONSTRUCT_STAGED)
      return fail(c, ACO_ERR_UNSUPPORTED, "candidate table does not fit in shared memory");
  }
  if (c->n > kDirectMaxCities) return ACO_OK;
  if (mode == ACO_CONSTRUCT_AUTO || mode == ACO_CONSTRUCT_CLUSTER) {
    const int cs = (c->n + 1023) / 1024;
    int clusters = 0;
    const ColonyDev d = make_dev(c);
    // A table of at most 1024 rows fits one CTA (the staged kernel); a
    // cluster of one is taken only when asked for.
    if (cs >= (mode == ACO_CONSTRUCT_CLUSTER ? 1 : 2) && cs <= 8) {
      // warps per CTA for the ants over the CTAs that fit, one pass
      int w = (c->m + sms - 1) / sms;
      w = w < 1 ? 1 : (w > kStagedMaxWarps ? kStagedMaxWarps : w);
      if (query_construct_cluster(d, w, cs, &clusters) == cudaSuccess && clusters > 0) {
        int ctas = clusters * cs;
        w = (c->m + ctas - 1) / ctas;
        w = w < 1 ? 1 : (w > kStagedMaxWarps ? kStagedMaxWarps : w);
        const int need = (c->m + w - 1) / w;  // CTAs that get ants
        ctas = std::min(ctas, (need + cs - 1) / cs * cs);
        c->cluster = cs;
        c->staged_warps = w;
        c->staged_grid = ctas;
        return ACO_OK;
      }
    }
    cudaGetLastError();  // a refused query leaves no error behind
    if (mode == ACO_CONSTRUCT_CLUSTER)
      return fail(c, ACO_ERR_UNSUPPORTED, "no cluster of the needed size fits");
  }
  c->direct = true;
  return ACO_OK;
}

int enqueue_iteration(aco_colony *c) {
  const ColonyDev d = make_dev(c);
  ACO_CUDA(c, launch_construction(c, d), "construct");
  ACO_CUDA(c, launch_epilogue(d, c->stream), "epilogue");
  if (c->p.deposit == ACO_DEPOSIT_ATOMIC) {
    ACO_CUDA(c, launch_evaporate(d, c->stream), "evaporate");
    ACO_CUDA(c, launch_deposit_atomic(d, c->stream), "deposit");
    ACO_CUDA(c, launch_pheromone_rows(d, false, false, false, c->stream), "choice rows");
    c->launches += 4 + construction_launches(c);
  } else {
    ACO_CUDA(c, launch_pheromone_rows(d, true, true, true, c->stream), "pheromone rows");
    c->launches += 2 + construction_launches(c);
  }
  return ACO_OK;
}

int read_matrix_f32(aco_colony *c, const float *src, int cols, int ldsrc, float *out) {
  if (!out) return fail(c, ACO_ERR_INVALID_ARGUMENT, "null output");
  if (!c->initialized) return fail(c, ACO_ERR_NOT_INITIALIZED, "colony not initialized");
  ACO_CUDA(c, cudaMemcpy2DAsync(out, (size_t)cols * 4, src, (size_t)ldsrc * 4, (size_t)cols * 4,
                                c->n, cudaMemcpyDeviceToHost, c->stream),
           "read matrix");
  ACO_CUDA(c, cudaStreamSynchronize(c->stream), "synchronize");
  return ACO_OK;
}

}  // namespace

extern "C" {

void aco_debug_fail_allocation(int32_t after) { g_fail_alloc.store(after < 0 ? -1 : after); }

void aco_params_default(aco_params *p) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->variant = ACO_ANT_SYSTEM;
  p->num_ants = 10;      // DEFAULT_NUM_ANTS
  p->alpha = 1.0f;       // DEFAULT_ALPHA
  p->beta = 5.0f;        // DEFAULT_BETA
  p->rho = 0.1f;         // DEFAULT_RHO
  p->use_alpha = 0;
  p->cand_k = 0;
  p->nn_order = ACO_NN_REFERENCE_QSORT;
  p->heuristic = ACO_HEURISTIC_LIBM;
  p->fallback = ACO_FALLBACK_REFERENCE;
  p->deposit = ACO_DEPOSIT_DETERMINISTIC;
  p->tau0_mode = ACO_TAU0_REFERENCE;
  p->tau0 = 1e-6f;
  p->rank_w = 5;         // DEFAULT_NUM_RANK_ANTS
  p->aging = 0;
  p->min_retirement_age = 30;
  p->max_retirement_age = 50;
  p->local_performance = 10;
  p->global_performance = 10;
  p->min_population_limit = 40;
  p->max_population_limit = 100;
  p->seed = 12345678;    // RANDOM_SEED, inc/Colony.h:15
}

int aco_colony_create(const aco_params *params, const int32_t *dist, int32_t n,
                      int32_t dist_on_device, aco_colony **out) {
  if (!dist) return ACO_ERR_INVALID_ARGUMENT;
  aco_colony *c = nullptr;
  int s = create_common(params, n, out, &c);
  if (s) return s;
  if (dist_on_device < 0) {  // locate the pointer (the reference passes either kind)
    cudaPointerAttributes attr;
    dist_on_device = (cudaPointerGetAttributes(&attr, dist) == cudaSuccess &&
                      (attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged))
                         ? 1
                         : 0;
    cudaGetLastError();  // clear a possible "invalid value" from a plain host pointer
  }
  const cudaMemcpyKind kind = dist_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  // A device matrix may still be in flight on the caller's stream, which the
  // colony's non-blocking stream is not ordered after: wait for it once.
  cudaError_t e = dist_on_device ? cudaDeviceSynchronize() : cudaSuccess;
  if (e == cudaSuccess)
    e = cudaMemcpy2DAsync(c->dist, (size_t)c->ld * 4, dist, (size_t)n * 4, (size_t)n * 4, n, kind,
                          c->stream);
  if (e == cudaSuccess) e = launch_fill_padding_int(c->dist, n, c->ld, ACO_MAX_DISTANCE, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    aco_colony_destroy(c);
    return ACO_ERR_CUDA;
  }
  *out = c;
  return ACO_OK;
}

int aco_colony_create_coords(const aco_params *params, const float *x, const float *y, int32_t n,
                             aco_colony **out) {
  if (!x || !y) return ACO_ERR_INVALID_ARGUMENT;
  aco_colony *c = nullptr;
  int s = create_common(params, n, out, &c);
  if (s) return s;
  // The coordinates stay on the device: the learned prior's features use them.
  if ((s = dalloc(c, &c->xy, (size_t)2 * n))) {
    aco_colony_destroy(c);
    return s;
  }
  float *dxy = c->xy;
  cudaError_t e = cudaMemcpyAsync(dxy, x, (size_t)n * 4, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dxy + n, y, (size_t)n * 4, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = launch_distances_from_coords(dxy, dxy + n, n, c->ld, c->dist, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    aco_colony_destroy(c);
    return ACO_ERR_CUDA;
  }
  *out = c;
  return ACO_OK;
}

namespace {

// The device work of aco_colony_initialize, enqueued on the colony's stream
// (the libm heuristic table, read back to the host, is the one wait); the
// caller checks the device state before the colony counts as initialised.
// The setup of an initialised colony, in three parts so that a batch can
// run every instance's first part before any host wait: init_begin resets
// the state and starts the heuristic (the whole of it on the device; in the
// libm mode the largest distance, into *dmax, which the host reads back),
// init_heuristic_table finishes the libm mode from that distance, init_rest
// does the rest (nn-lists, tau0, the ants).
int init_begin(aco_colony *c, int32_t *dmax) {
  state_changed(c);
  drop_graph(c);
  c->initialized = false;
  const int n = c->n;
  // RankBasedAntSystem::computeParameters (src/RankBasedAntSystem.cu:31-36)
  if (c->p.variant == ACO_RANK_BASED && c->p.rank_w > n) c->p.rank_w = n;
  ACO_CUDA(c, cudaMemsetAsync(c->st, 0, sizeof(ColonyState), c->stream), "reset state");
  // heuristic (Colony::computeHurestics, src/Colony.cu:232-246)
  if (c->p.heuristic == ACO_HEURISTIC_DEVICE) {
    ACO_CUDA(c, launch_heuristic_device(c->dist, n, c->ld, c->p.beta, c->eta, c->stream),
             "heuristic");
  } else {
    ACO_CUDA(c, cudaMemsetAsync(dmax, 0, 4, c->stream), "memset");
    ACO_CUDA(c, launch_max_distance(c->dist, n, c->ld, dmax, c->stream), "max distance");
  }
  return ACO_OK;
}

// The libm mode's table, HURESTIC(d, beta) of the reference CPU build
// (inc/Colony.h:20), one entry per distinct distance value d = 0 .. hmax,
// on the host.  It depends on beta and hmax alone, so a batch builds one up
// to its largest distance and every instance reads its own prefix.
bool libm_table(int32_t hmax, float beta, std::vector<float> &table) {
  if (hmax < 0 || hmax >= (1 << 26)) return false;
  table.resize((size_t)hmax + 1);
  for (int32_t d = 0; d <= hmax; d++) table[d] = powf((float)(1.0 / ((float)d)), beta);
  return true;
}
const char *const kTooFar = "distances too large for the libm heuristic table";

// eta from a table already on the device (entries > the colony's largest
// distance).
int init_heuristic_table(aco_colony *c, const float *dtab, int32_t entries) {
  ACO_CUDA(c, launch_heuristic_table(c->dist, c->n, c->ld, dtab, entries, c->eta, c->st,
                                     c->stream),
           "heuristic table");
  return ACO_OK;
}

int init_rest(aco_colony *c) {
  const int n = c->n;
  // nn-list (Colony::computeNNlist, src/Colony.cu:276-311)
  if (c->p.nn_order == ACO_NN_STABLE) {
    ACO_CUDA(c, launch_nn_sort_stable(c->dist, n, c->ld, c->K, c->ldk, c->nn, c->st, c->stream,
                                      c->nn2, c->t2),
             "nn sort");
  } else {
    // The sort runs in shared memory when a row fits (one warp per row),
    // else on a global scratch (one thread per row); same permutation.
    const bool smem_sort = nn_ref_qsort_smem_rows(n, c->max_smem_optin) >= 1;
    int32_t *scratch = nullptr, *full = nullptr;
    if (!smem_sort)
      ACO_CUDA(c, cudaMallocAsync(&scratch, (size_t)n * c->ld * 4, c->stream), "alloc scratch");
    if (c->K == n) {
      full = c->nn;  // the sort writes n ids a row; the pitch's padding is -1
      ACO_CUDA(c, cudaMemsetAsync(c->nn, 0xff, (size_t)n * c->ldk * 4, c->stream), "memset nn");
    } else {
      ACO_CUDA(c, cudaMallocAsync(&full, (size_t)n * c->ld * 4, c->stream), "alloc scratch");
    }
    if (smem_sort)
      ACO_CUDA(c, launch_nn_ref_qsort_smem(c->dist, n, c->ld, full, c->K == n ? c->ldk : c->ld,
                                           c->st, c->max_smem_optin, c->stream),
               "nn quicksort");
    else
      ACO_CUDA(c, launch_nn_ref_qsort(c->dist, n, c->ld, scratch, full,
                                      c->K == n ? c->ldk : c->ld, c->st, c->stream),
               "nn quicksort");
    if (full != c->nn) {
      ACO_CUDA(c, cudaMemsetAsync(c->nn, 0xff, (size_t)n * c->ldk * 4, c->stream), "memset nn");
      ACO_CUDA(c, cudaMemcpy2DAsync(c->nn, (size_t)c->ldk * 4, full, (size_t)c->ld * 4,
                                    (size_t)c->K * 4, n, cudaMemcpyDeviceToDevice, c->stream),
               "copy nn");
      if (c->t2 > 0) {  // the fallback's second tier: neighbours K .. K + t2 - 1
        ACO_CUDA(c, cudaMemsetAsync(c->nn2, 0xff, (size_t)n * kTier2 * 4, c->stream),
                 "memset nn2");
        ACO_CUDA(c, cudaMemcpy2DAsync(c->nn2, (size_t)kTier2 * 4, full + c->K,
                                      (size_t)c->ld * 4, (size_t)c->t2 * 4, n,
                                      cudaMemcpyDeviceToDevice, c->stream),
                 "copy nn2");
      }
      ACO_CUDA(c, cudaFreeAsync(full, c->stream), "free");
    }
    if (scratch) ACO_CUDA(c, cudaFreeAsync(scratch, c->stream), "free");
  }
  ACO_CUDA(c, launch_gather_nn_f32(c->eta, n, c->ld, c->nn, c->K, c->ldk, c->eta_nn, c->stream),
           "eta_nn");
  if (c->nn16) ACO_CUDA(c, launch_nn_to_i16(c->nn, n, c->K, c->ldk, c->nn16, c->stream), "nn16");

  const ColonyDev d = make_dev(c);
  ACO_CUDA(c, launch_greedy_tau0(d, c->p.tau0_mode, c->p.tau0, c->stream), "tau0");
  ACO_CUDA(c, launch_init_colony(d, c->stream), "init");
  ACO_CUDA(c, configure_construct(construct_smem_bytes(n, c->K, c->apb)), "configure construct");
  ACO_CUDA(c, configure_pheromone_rows(c->ld), "configure rows");
  if (int s0 = plan_construction(c)) return s0;
  ACO_CUDA(c, launch_pheromone_rows(d, false, false, false, c->stream), "choice rows");
  return ACO_OK;
}

// One colony's whole setup, with the libm mode's one read-back in the middle.
int initialize_enqueue(aco_colony *c) {
  const bool libm = c->p.heuristic != ACO_HEURISTIC_DEVICE;
  int32_t *dmax = nullptr;
  if (libm) ACO_CUDA(c, cudaMallocAsync(&dmax, 4, c->stream), "alloc");
  if (int s = init_begin(c, dmax)) return s;
  if (libm) {
    int32_t hmax = 0;
    ACO_CUDA(c, cudaMemcpyAsync(&hmax, dmax, 4, cudaMemcpyDeviceToHost, c->stream), "read max");
    ACO_CUDA(c, cudaFreeAsync(dmax, c->stream), "free");
    ACO_CUDA(c, cudaStreamSynchronize(c->stream), "synchronize");
    std::vector<float> table;
    if (!libm_table(hmax, c->p.beta, table)) return fail(c, ACO_ERR_UNSUPPORTED, kTooFar);
    float *dtab = nullptr;
    ACO_CUDA(c, cudaMallocAsync(&dtab, table.size() * 4, c->stream), "alloc table");
    ACO_CUDA(c, cudaMemcpyAsync(dtab, table.data(), table.size() * 4, cudaMemcpyHostToDevice,
                                c->stream),
             "upload table");
    if (int s = init_heuristic_table(c, dtab, hmax + 1)) return s;
    ACO_CUDA(c, cudaFreeAsync(dtab, c->stream), "free table");
    ACO_CUDA(c, cudaStreamSynchronize(c->stream), "synchronize");
  }
  return init_rest(c);
}

}  // namespace

int aco_colony_initialize(aco_colony *c) {
  NvtxRange range("aco_colony_initialize");
  if (!c) return ACO_ERR_INVALID_ARGUMENT;
  if (int s = initialize_enqueue(c)) return s;
  if (int s = device_error(c)) return s;
  c->initialized = true;
  return ACO_OK;
}

int aco_colony_construct_solution(aco_colony *c, float *timers_ms) {
  NvtxRange range("aco_colony_construct_solution");
  if (!c) return ACO_ERR_INVALID_ARGUMENT;
  if (!c->initialized) return fail(c, ACO_ERR_NOT_INITIALIZED, "colony not initialized");
  state_changed(c);
  // Without timers one iteration is one replay of the captured graph (the
  // legacy default stream cannot be captured: direct launches there).
  if (!timers_ms) {
    const bool capturable = c->stream != nullptr && c->stream != cudaStreamLegacy &&
                            c->stream != cudaStreamPerThread;
    return capturable ? aco_colony_run(c, 1) : enqueue_iteration(c);
  }
  const ColonyDev d = make_dev(c);
  ACO_CUDA(c, cudaEventRecord(c->ev[0], c->stream), "event");
  ACO_CUDA(c, launch_construction(c, d), "construct");
  ACO_CUDA(c, cudaEventRecord(c->ev[1], c->stream), "event");
  ACO_CUDA(c, launch_epilogue(d, c->stream), "epilogue");
  ACO_CUDA(c, cudaEventRecord(c->ev[2], c->stream), "event");
  if (c->p.deposit == ACO_DEPOSIT_ATOMIC) {
    ACO_CUDA(c, launch_evaporate(d, c->stream), "evaporate");
    ACO_CUDA(c, launch_deposit_atomic(d, c->stream), "deposit");
    ACO_CUDA(c, launch_pheromone_rows(d, false, false, false, c->stream), "choice rows");
    c->launches += 4 + construction_launches(c);
  } else {
    ACO_CUDA(c, launch_pheromone_rows(d, true, true, true, c->stream), "pheromone rows");
    c->launches += 2 + construction_launches(c);
  }
  ACO_CUDA(c, cudaEventRecord(c->ev[3], c->stream), "event");
  ACO_CUDA(c, cudaEventSynchronize(c->ev[3]), "synchronize");
  float t[3];
  for (int i = 0; i < 3; i++) cudaEventElapsedTime(&t[i], c->ev[i], c->ev[i + 1]);
  for (int i = 0; i < ACO_TOTAL_TIMERS; i++) timers_ms[i] = 0.0f;
  // initTour and the choice-info are fused into construction and into the
  // pheromone pass; their slots stay 0.
  timers_ms[ACO_TIME_TOUR] = t[0];
  timers_ms[ACO_TIME_COMPUTE_ANT_DISTANCE] = t[1];
  timers_ms[ACO_TIME_UPDATE_PHEROMONE] = t[2];
  return device_error(c);
}

int aco_colony_run(aco_colony *c, int32_t iterations) {
  NvtxRange range("aco_colony_run");
  if (!c || iterations < 0) return ACO_ERR_INVALID_ARGUMENT;
  state_changed(c);
  if (!c->initialized) return fail(c, ACO_ERR_NOT_INITIALIZED, "colony not initialized");
  if (iterations == 0) return ACO_OK;
  if (!c->graph_exec) {
    const int64_t before = c->launches;
    ACO_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "capture");
    int s = enqueue_iteration(c);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (s) {
      if (g) cudaGraphDestroy(g);
      return s;
    }
    if (e != cudaSuccess) return cuda_fail(c, e, "end capture");
    c->graph = g;
    ACO_CUDA(c, cudaGraphInstantiate(&c->graph_exec, g, 0), "instantiate");
    c->launches = before;  // capture itself launches nothing
  }
  const int per_iter = (c->p.deposit == ACO_DEPOSIT_ATOMIC ? 4 : 2) + construction_launches(c);
  for (int32_t i = 0; i < iterations; i++)
    ACO_CUDA(c, cudaGraphLaunch(c->graph_exec, c->stream), "graph launch");
  c->launches += (int64_t)per_iter * iterations;
  return ACO_OK;
}

int aco_colony_synchronize(aco_colony *c) {
  if (!c) return ACO_ERR_INVALID_ARGUMENT;
  return device_error(c);
}

int aco_colony_get_iter_best(aco_colony *c, int64_t *out) {
  if (!c || !out) return ACO_ERR_INVALID_ARGUMENT;
  ColonyState h;
  int s = read_state(c, &h);
  if (!s) *out = h.iter_best;
  return s;
}

int aco_colony_get_glob_best(aco_colony *c, int64_t *out) {
  if (!c || !out) return ACO_ERR_INVALID_ARGUMENT;
  ColonyState h;
  int s = read_state(c, &h);
  if (!s) *out = h.glob_best;
  return s;
}

int aco_colony_get_num_valid_ants(aco_colony *c, int32_t *out) {
  if (!c || !out) return ACO_ERR_INVALID_ARGUMENT;
  if (!c->p.aging) {  // Colony::getNumValidAnts, src/Colony.cu:464-466
    *out = c->m;
    return ACO_OK;
  }
  ColonyState h;
  int s = read_state(c, &h);
  if (!s) *out = h.num_valid;
  return s;
}

int aco_colony_get_iteration(aco_colony *c, int32_t *out) {
  if (!c || !out) return ACO_ERR_INVALID_ARGUMENT;
  ColonyState h;
  int s = read_state(c, &h);
  if (!s) *out = (int32_t)h.iteration;
  return s;
}

int aco_colony_get_reps(aco_colony *c, int32_t *out) {
  if (!c || !out) return ACO_ERR_INVALID_ARGUMENT;
  *out = 0;  // reps is never incremented by the reference (src/Colony.cu:35)
  return ACO_OK;
}

int aco_colony_get_size(aco_colony *c, int32_t *n, int32_t *m, int32_t *k) {
  if (!c) return ACO_ERR_INVALID_ARGUMENT;
  if (n) *n = c->n;
  if (m) *m = c->m;
  if (k) *k = c->K;
  return ACO_OK;
}

int aco_colony_get_params(aco_colony *c, aco_params *out) {
  if (!c || !out) return ACO_ERR_INVALID_ARGUMENT;
  *out = c->p;
  return ACO_OK;
}

int aco_colony_set_alpha(aco_colony *c, float v) {
  if (!c) return ACO_ERR_INVALID_ARGUMENT;
  c->p.alpha = v;
  drop_graph(c);
  return ACO_OK;
}

int aco_colony_set_beta(aco_colony *c, float v) {
  if (!c) return ACO_ERR_INVALID_ARGUMENT;
  c->p.beta = v;
  return ACO_OK;
}

int aco_colony_set_rho(aco_colony *c, float v) {
  if (!c) return ACO_ERR_INVALID_ARGUMENT;
  c->p.rho = v;
  drop_graph(c);
  return ACO_OK;
}

int aco_colony_set_optimum(aco_colony *c, int64_t v) {
  if (!c) return ACO_ERR_INVALID_ARGUMENT;
  c->optimum = v;
  return ACO_OK;
}

int aco_colony_set_rank_w(aco_colony *c, int32_t w) {
  if (!c || w < 1) return ACO_ERR_INVALID_ARGUMENT;
  c->p.rank_w = w;
  drop_graph(c);
  return ACO_OK;
}

int aco_colony_set_aging_params(aco_colony *c, const int32_t six[6]) {
  if (!c || !six) return ACO_ERR_INVALID_ARGUMENT;
  c->p.min_retirement_age = six[0];
  c->p.max_retirement_age = six[1];
  c->p.local_performance = six[2];
  c->p.global_performance = six[3];
  c->p.min_population_limit = six[4];
  c->p.max_population_limit = six[5];
  drop_graph(c);
  return ACO_OK;
}

const char *aco_colony_name(const aco_colony *c) {
  if (!c) return "";
  return c->p.variant == ACO_RANK_BASED ? kNameRBAS : kNameAS;
}

int aco_colony_get_best_tour(aco_colony *c, int32_t *out) {
  if (!c || !out) return ACO_ERR_INVALID_ARGUMENT;
  if (!c->initialized) return fail(c, ACO_ERR_NOT_INITIALIZED, "colony not initialized");
  ACO_CUDA(c, cudaMemcpyAsync(out, c->gbtour, (size_t)c->n * 4, cudaMemcpyDeviceToHost, c->stream),
           "read best tour");
  ACO_CUDA(c, cudaStreamSynchronize(c->stream), "synchronize");
  return ACO_OK;
}

int aco_colony_read_pheromone(aco_colony *c, float *out) {
  if (!c) return ACO_ERR_INVALID_ARGUMENT;
  return read_matrix_f32(c, c->tau, c->n, c->ld, out);
}

int aco_colony_write_pheromone(aco_colony *c, const float *in) {
  if (c) state_changed(c);
  if (!c || !in) return ACO_ERR_INVALID_ARGUMENT;
  if (!c->initialized) return fail(c, ACO_ERR_NOT_INITIALIZED, "colony not initialized");
  ACO_CUDA(c, cudaMemcpy2DAsync(c->tau, (size_t)c->ld * 4, in, (size_t)c->n * 4, (size_t)c->n * 4,
                                c->n, cudaMemcpyHostToDevice, c->stream),
           "write pheromone");
  ACO_CUDA(c, launch_pheromone_rows(make_dev(c), false, false, false, c->stream), "choice rows");
  return device_error(c);
}

int aco_colony_read_heuristic(aco_colony *c, float *out) {
  if (!c) return ACO_ERR_INVALID_ARGUMENT;
  return read_matrix_f32(c, c->eta, c->n, c->ld, out);
}

int aco_colony_read_choice_info(aco_colony *c, float *out) {
  if (!c) return ACO_ERR_INVALID_ARGUMENT;
  return read_matrix_f32(c, c->choice, c->n, c->ld, out);
}

int aco_colony_read_nn_list(aco_colony *c, int32_t *out) {
  if (!c) return ACO_ERR_INVALID_ARGUMENT;
  return read_matrix_f32(c, reinterpret_cast<const float *>(c->nn), c->K, c->ldk,
                         reinterpret_cast<float *>(out));
}

int aco_colony_read_candidate_heuristic(aco_colony *c, float *out) {
  if (!c) return ACO_ERR_INVALID_ARGUMENT;
  return read_matrix_f32(c, c->eta_nn, c->K, c->ldk, out);
}

int aco_colony_read_distances(aco_colony *c, int32_t *out) {
  if (!c || !out) return ACO_ERR_INVALID_ARGUMENT;
  ACO_CUDA(c, cudaMemcpy2DAsync(out, (size_t)c->n * 4, c->dist, (size_t)c->ld * 4,
                                (size_t)c->n * 4, c->n, cudaMemcpyDeviceToHost, c->stream),
           "read distances");
  ACO_CUDA(c, cudaStreamSynchronize(c->stream), "synchronize");
  return ACO_OK;
}

int aco_colony_read_tours(aco_colony *c, int32_t *out) {
  if (!c || !out) return ACO_ERR_INVALID_ARGUMENT;
  if (!c->initialized) return fail(c, ACO_ERR_NOT_INITIALIZED, "colony not initialized");
  ACO_CUDA(c, cudaMemcpy2DAsync(out, (size_t)c->n * 4, c->tours, (size_t)c->ld * 4,
                                (size_t)c->n * 4, c->m, cudaMemcpyDeviceToHost, c->stream),
           "read tours");
  ACO_CUDA(c, cudaStreamSynchronize(c->stream), "synchronize");
  return ACO_OK;
}

int aco_colony_read_tour_lengths(aco_colony *c, int64_t *out) {
  if (!c || !out) return ACO_ERR_INVALID_ARGUMENT;
  if (!c->initialized) return fail(c, ACO_ERR_NOT_INITIALIZED, "colony not initialized");
  ACO_CUDA(c, cudaMemcpyAsync(out, c->len, (size_t)c->m * 8, cudaMemcpyDeviceToHost, c->stream),
           "read lengths");
  ACO_CUDA(c, cudaStreamSynchronize(c->stream), "synchronize");
  return ACO_OK;
}

int aco_colony_read_aging(aco_colony *c, int32_t *age, int32_t *perf, uint8_t *valid, float *mean,
                          int32_t *misc) {
  if (!c) return ACO_ERR_INVALID_ARGUMENT;
  ColonyState h;
  int s = read_state(c, &h);
  if (s) return s;
  if (age) ACO_CUDA(c, cudaMemcpy(age, c->age, (size_t)c->m * 4, cudaMemcpyDeviceToHost), "read");
  if (perf) ACO_CUDA(c, cudaMemcpy(perf, c->perf, (size_t)c->m * 4, cudaMemcpyDeviceToHost), "read");
  if (valid) ACO_CUDA(c, cudaMemcpy(valid, c->valid, (size_t)c->m, cudaMemcpyDeviceToHost), "read");
  if (mean) ACO_CUDA(c, cudaMemcpy(mean, c->mean, (size_t)c->n * 4, cudaMemcpyDeviceToHost), "read");
  if (misc) {
    misc[0] = h.isconverged;
    misc[1] = h.globalperformance;
  }
  return ACO_OK;
}

int aco_colony_get_stats(aco_colony *c, aco_stats *out) {
  if (!c || !out) return ACO_ERR_INVALID_ARGUMENT;
  ColonyState h;
  int s = read_state(c, &h);
  if (s) return s;
  memset(out, 0, sizeof(*out));
  out->iteration = h.iteration;
  out->tours_built = h.tours_built;
  out->fallbacks = h.fallbacks;
  out->greedy_length = h.greedy_length;
  out->iter_best = h.iter_best;
  out->glob_best = h.glob_best;
  out->num_valid = c->p.aging ? h.num_valid : c->m;
  out->tau0 = h.tau0;
  return ACO_OK;
}

int aco_colony_set_stream(aco_colony *c, void *stream) {
  if (!c) return ACO_ERR_INVALID_ARGUMENT;
  ACO_CUDA(c, cudaStreamSynchronize(c->stream), "synchronize");
  if (c->own_stream) cudaStreamDestroy(c->stream);
  c->stream = static_cast<cudaStream_t>(stream);
  c->own_stream = false;
  drop_graph(c);
  return ACO_OK;
}

int aco_colony_get_launch_count(aco_colony *c, int64_t *out) {
  if (!c || !out) return ACO_ERR_INVALID_ARGUMENT;
  *out = c->launches;
  return ACO_OK;
}

const char *aco_colony_last_error(const aco_colony *c) { return c ? c->err.c_str() : ""; }

const char *aco_status_string(int status) {
  switch (status) {
    case ACO_OK: return "ok";
    case ACO_ERR_INVALID_ARGUMENT: return "invalid argument";
    case ACO_ERR_OUT_OF_MEMORY: return "out of device memory";
    case ACO_ERR_CUDA: return "CUDA error";
    case ACO_ERR_NOT_INITIALIZED: return "not initialized";
    case ACO_ERR_UNSUPPORTED: return "unsupported configuration";
    case ACO_ERR_DEVICE_TIMEOUT: return "device wait timed out";
    case ACO_ERR_DEVICE_CHECK: return "device check failed";
    default: return "unknown status";
  }
}

void aco_colony_destroy(aco_colony *c) {
  if (!c) return;
  if (c->stream) cudaStreamSynchronize(c->stream);
  drop_graph(c);
  for (void *p : c->allocations) cudaFree(p);
  for (int i = 0; i < 4; i++)
    if (c->ev[i]) cudaEventDestroy(c->ev[i]);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  if (c->h_state) cudaFreeHost(c->h_state);
  delete c;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batches: many instances of uneven size advanced together.  Each instance
// is a colony (same buffers, same initialisation); an iteration of the whole
// batch is three launches over all instances -- a persistent construction
// kernel fed by a work queue, one epilogue CTA per instance, one pheromone
// CTA per row of every instance -- captured once into a CUDA graph.
struct aco_batch {
  aco_params p;
  std::vector<aco_colony *> cols;
  cudaStream_t stream = nullptr;
  ColonyDev *d_descs = nullptr;
  int2 *d_rowmap = nullptr;
  int4 *d_items = nullptr;
  int *d_queue = nullptr;
  int total_rows = 0, num_items = 0;
  int max_n = 0, max_k = 0, max_ld = 0, num_sms = 1, max_smem_optin = 0;
  int sp = 0;  // row pitch of the staged items: the largest among instances with k <= 32
  int apb = 8, row_threads = 256, grid = 0;
  size_t region_bytes = 0;  // shared region of the construction launch
  int staged_count = 0;     // instances built from a staged table
  bool rows = false;        // construction by the long-row batch kernel (every k > 32)
  int min_k = 1 << 30, max_ldk_rows = 0;
  bool initialized = false;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  int64_t launches = 0;
  ColonyState *h_states = nullptr;  // pinned, one a instance (the first batch read allocates it)
  std::string err;
};

namespace {

int bfail(aco_batch *b, int status, const std::string &msg) {
  if (b) b->err = msg;
  return status;
}

#define ACO_BCUDA(b, call, what)                                                         \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return bfail(b, e_ == cudaErrorMemoryAllocation ? ACO_ERR_OUT_OF_MEMORY : ACO_ERR_CUDA, \
                   std::string(what) + ": " + cudaGetErrorString(e_));                   \
  } while (0)

void batch_drop_graph(aco_batch *b) {
  if (b->graph_exec) cudaGraphExecDestroy(b->graph_exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->graph_exec = nullptr;
  b->graph = nullptr;
}

// Host -> device upload on the batch's own stream.  The stream is
// non-blocking, so a plain cudaMemcpy (legacy stream; a pageable upload may
// return before its DMA lands) would not be ordered before the next launch.
cudaError_t upload_sync(aco_batch *b, void *dst, const void *src, size_t bytes) {
  cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, b->stream);
  return e == cudaSuccess ? cudaStreamSynchronize(b->stream) : e;
}

// Shared memory of the construction launch with `apb` warps per CTA: the
// largest staged table that fits next to the per-warp buffers, and which
// instances are staged.
size_t batch_plan_region(const aco_batch *b, int apb, std::vector<char> *staged, int *count) {
  const bool aging = b->p.aging != 0;
  // static shared memory of the kernel (descriptor, item, flags) plus slack
  const size_t fixed = sizeof(ColonyDev) + 256;
  const size_t avail = (size_t)b->max_smem_optin - batch_construct_smem_bytes(0, apb) - fixed;
  size_t max_table = 0;
  int cnt = 0;
  if (staged) staged->assign(b->cols.size(), 0);
  for (size_t i = 0; i < b->cols.size(); i++) {
    const aco_colony *c = b->cols[i];
    if (b->p.construct_mode == ACO_CONSTRUCT_GLOBAL || c->K > 32 || !c->nn16 || c->n > 2048 ||
        c->ldk != b->sp)
      continue;
    const size_t t = batch_staged_table_bytes(c->n, c->ld, b->sp, aging);
    if (t > avail) continue;
    max_table = std::max(max_table, t);
    cnt++;
    if (staged) (*staged)[i] = 1;
  }
  if (count) *count = cnt;
  return batch_region_bytes(b->max_n, b->max_k, apb, max_table);
}

// Work items (instance, first ant, ants, staged), largest instances first.
int batch_build_items(aco_batch *b) {
  std::vector<int> order(b->cols.size());
  for (size_t i = 0; i < order.size(); i++) order[i] = (int)i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int c) { return b->cols[a]->n > b->cols[c]->n; });
  std::vector<char> staged;
  if (b->rows) {
    staged.assign(b->cols.size(), 0);
    b->region_bytes = 0;
    b->staged_count = 0;
  } else {
    b->region_bytes = batch_plan_region(b, b->apb, &staged, &b->staged_count);
  }
  // The launch shape first: the grid decides how many items make whole waves.
  if (b->rows) {
    const size_t smem = batch_rows_smem_bytes(b->max_n, b->max_ldk_rows, b->apb);
    if (b->apb > kRowsMaxAnts || smem + 1024 > (size_t)b->max_smem_optin)
      return bfail(b, ACO_ERR_UNSUPPORTED, "too many ants per CTA for the long rows' buffers");
    ACO_BCUDA(b, configure_batch_construct_rows(smem), "configure batch row construct");
    b->grid = b->num_sms * batch_rows_blocks_per_sm(b->apb, smem, b->p.aging != 0);
  } else {
    const size_t smem = batch_construct_smem_bytes(b->region_bytes, b->apb);
    ACO_BCUDA(b, configure_batch_construct(smem), "configure batch construct");
    b->grid = b->num_sms * batch_construct_blocks_per_sm(b->apb, smem, b->max_k > 32, b->sp,
                                                         b->p.aging != 0);
  }
  // ceil(m / apb) items of nearly equal size per instance (no item far below
  // apb ants, which would leave most of its CTA's warps idle for a whole
  // tour).  When every instance has the same n and m the items take equally
  // long, and their count is raised to whole waves of the grid (at most apb
  // and at least one ant an item): the last wave then runs as many items as
  // the others, each a little lighter, instead of leaving CTAs idle.
  const size_t ni = b->cols.size();
  std::vector<int> parts(ni);
  bool uniform = true;
  long total = 0;
  for (size_t i = 0; i < ni; i++) {
    const aco_colony *c = b->cols[i];
    parts[i] = (c->m + b->apb - 1) / b->apb;
    total += parts[i];
    uniform = uniform && c->n == b->cols[0]->n && c->m == b->cols[0]->m;
  }
  if (uniform && b->grid > 0 && total % b->grid != 0) {
    const long target = (total + b->grid - 1) / b->grid * b->grid;
    for (size_t i = 0; i < ni; i++) {
      const long want = target / (long)ni + ((long)i < target % (long)ni ? 1 : 0);
      parts[i] = (int)std::max<long>(parts[i], std::min<long>(want, b->cols[i]->m));
    }
  }
  std::vector<int4> items;
  for (int i : order) {
    const int m = b->cols[i]->m;
    for (int q = 0, a0 = 0; q < parts[i]; q++) {
      const int cnt = m / parts[i] + (q < m % parts[i] ? 1 : 0);
      items.push_back(make_int4(i, a0, cnt, staged[i]));
      a0 += cnt;
    }
  }
  if (b->d_items) cudaFree(b->d_items);
  b->d_items = nullptr;
  ACO_BCUDA(b, cudaMalloc(&b->d_items, items.size() * sizeof(int4)), "alloc items");
  ACO_BCUDA(b, upload_sync(b, b->d_items, items.data(), items.size() * sizeof(int4)),
            "upload items");
  b->num_items = (int)items.size();
  batch_drop_graph(b);
  return ACO_OK;
}

int batch_enqueue(aco_batch *b, bool construct, bool epilogue, bool rows, bool update) {
  for (aco_colony *c : b->cols) state_changed(c);
  if (construct) {
    ACO_BCUDA(b, cudaMemsetAsync(b->d_queue, 0, sizeof(int), b->stream), "reset queue");
    if (b->rows && b->p.aging) {
      ACO_BCUDA(b, launch_batch_aging_plan(b->d_descs, (int)b->cols.size(), b->stream),
                "batch aging plan");
      b->launches++;
    }
    if (b->rows)
      ACO_BCUDA(b, launch_batch_construct_rows(b->d_descs, b->d_items, b->num_items, b->d_queue,
                                               b->grid, b->apb, b->max_n, b->max_ldk_rows,
                                               b->p.aging != 0, b->stream),
                "batch row construct");
    else
      ACO_BCUDA(b, launch_batch_construct(b->d_descs, b->d_items, b->num_items, b->d_queue,
                                          b->grid, b->apb, b->max_n, b->max_k, b->region_bytes,
                                          b->sp, b->p.aging != 0, b->stream),
                "batch construct");
    b->launches++;
  }
  if (epilogue) {
    ACO_BCUDA(b, launch_batch_epilogue(b->d_descs, (int)b->cols.size(), b->stream),
              "batch epilogue");
    b->launches++;
  }
  if (rows) {
    ACO_BCUDA(b, launch_batch_pheromone_rows(b->d_descs, b->d_rowmap, b->total_rows, b->max_ld,
                                             update, b->stream, b->row_threads),
              "batch pheromone rows");
    b->launches++;
  }
  return ACO_OK;
}

// The state words of every instance whose copy on the host is stale: their
// read-backs queued on the batch stream (the instances' own stream between
// calls), then one wait -- rather than a wait per instance.  The getters
// want initialised instances; the error check does not.
int batch_read_states(aco_batch *b, bool need_init) {
  if (!b->h_states &&
      cudaMallocHost(&b->h_states, b->cols.size() * sizeof(ColonyState)) != cudaSuccess) {
    b->h_states = nullptr;
    return bfail(b, ACO_ERR_OUT_OF_MEMORY, "cudaMallocHost");
  }
  for (size_t i = 0; i < b->cols.size(); i++) {
    aco_colony *c = b->cols[i];
    if (need_init && !c->initialized)
      return bfail(b, ACO_ERR_NOT_INITIALIZED, "colony not initialized");
    if (c->state_fresh) continue;
    ACO_BCUDA(b, cudaMemcpyAsync(&b->h_states[i], c->st, sizeof(ColonyState),
                                 cudaMemcpyDeviceToHost, b->stream),
              "read state");
  }
  ACO_BCUDA(b, cudaStreamSynchronize(b->stream), "synchronize");
  for (size_t i = 0; i < b->cols.size(); i++) {
    aco_colony *c = b->cols[i];
    if (c->state_fresh) continue;
    c->h_cache = b->h_states[i];
    c->state_fresh = c->initialized;  // the getters' copy, once there is one to keep
  }
  return ACO_OK;
}

// The device error words of every instance, after the batch stream has run.
int batch_state_check(aco_batch *b) {
  if (int s = batch_read_states(b, false)) return s;
  for (size_t i = 0; i < b->cols.size(); i++) {
    aco_colony *c = b->cols[i];
    const uint32_t err = c->state_fresh ? c->h_cache.error : b->h_states[i].error;
    if (err & kErrTimeout) return bfail(b, ACO_ERR_DEVICE_TIMEOUT, "a bounded device wait expired");
    if (err & kErrCheck) return bfail(b, ACO_ERR_DEVICE_CHECK, "a device-side check failed");
  }
  return ACO_OK;
}

}  // namespace

extern "C" {

int aco_batch_create(const aco_params *params, int32_t count, const int32_t *sizes,
                     const float *coords, aco_batch **out) {
  if (!out || !params || !sizes || !coords || count < 1) return ACO_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  if (params->deposit != ACO_DEPOSIT_DETERMINISTIC) return ACO_ERR_UNSUPPORTED;
  aco_batch *b = new (std::nothrow) aco_batch();
  if (!b) return ACO_ERR_OUT_OF_MEMORY;
  b->p = *params;
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete b;
    return ACO_ERR_CUDA;
  }
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&b->max_smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  size_t off = 0;
  for (int32_t i = 0; i < count; i++) {
    const int n = sizes[i];
    aco_params pi = *params;
    pi.num_ants = std::min(params->num_ants, n);
    pi.seed = params->seed + (uint64_t)i * 0x9E3779B97F4A7C15ULL;
    pi.construct_mode = ACO_CONSTRUCT_GLOBAL;
    aco_colony *c = nullptr;
    int s = aco_colony_create_coords(&pi, coords + off, coords + off + n, n, &c);
    if (s) {
      aco_batch_destroy(b);
      return s;
    }
    aco_colony_set_stream(c, b->stream);
    b->cols.push_back(c);
    off += 2 * (size_t)n;
    b->max_n = std::max(b->max_n, c->n);
    b->max_k = std::max(b->max_k, c->K);
    b->min_k = std::min(b->min_k, c->K);
    b->max_ldk_rows = std::max(b->max_ldk_rows, c->ldk);
    if (c->K <= 32) b->sp = std::max(b->sp, c->ldk);
    b->max_ld = std::max(b->max_ld, c->ld);
    b->total_rows += n;
  }
  if (b->sp == 0) b->sp = 32;
  // Candidate rows longer than 32 in every instance (full rows included):
  // the long-row batch kernel, when every instance has int16 ids and one
  // ant's buffers fit.
  b->rows = b->min_k > 32 && params->construct_mode != ACO_CONSTRUCT_GLOBAL &&
            batch_rows_smem_bytes(b->max_n, b->max_ldk_rows, 1) + 1024 <=
                (size_t)b->max_smem_optin;
  for (aco_colony *c : b->cols)
    if (!c->nn16) b->rows = false;
  if (b->rows) b->apb = kRowsMaxAnts;  // as many ants a CTA as the registers allow
  while (b->rows && b->apb > 1 &&
         batch_rows_smem_bytes(b->max_n, b->max_ldk_rows, b->apb) + 1024 >
             (size_t)b->max_smem_optin)
    b->apb--;
  *out = b;
  return ACO_OK;
}

int aco_batch_initialize(aco_batch *b) {
  NvtxRange range("aco_batch_initialize");
  if (!b) return ACO_ERR_INVALID_ARGUMENT;
  b->initialized = false;
  batch_drop_graph(b);
  std::vector<ColonyDev> descs;
  std::vector<int2> rowmap;
  // The instances' setup kernels are small (the greedy tour is one CTA):
  // they run on a pool of streams, ordered after the batch stream, so that
  // they overlap, with one wait at the end instead of one per instance.
  constexpr int kInitStreams = 16;
  const int npool = (int)std::min<size_t>(kInitStreams, b->cols.size());
  std::vector<cudaStream_t> pool(npool, nullptr);
  cudaEvent_t ready = nullptr;
  int s = ACO_OK;
  if (cudaEventCreateWithFlags(&ready, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventRecord(ready, b->stream) != cudaSuccess)
    s = bfail(b, ACO_ERR_CUDA, "initialize: event");
  for (int q = 0; q < npool && !s; q++)
    if (cudaStreamCreateWithFlags(&pool[q], cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamWaitEvent(pool[q], ready, 0) != cudaSuccess)
      s = bfail(b, ACO_ERR_CUDA, "initialize: streams");
  // In the libm heuristic mode every instance's largest distance is read
  // back once, for all of them after their first part, rather than with a
  // wait per instance; one table up to the largest serves every instance.
  const size_t ni = b->cols.size();
  const bool libm = b->p.heuristic != ACO_HEURISTIC_DEVICE;
  int32_t *d_hmax = nullptr;
  float *d_table = nullptr;
  int32_t entries = 0;
  std::vector<int32_t> hmax(ni, 0);
  if (!s && libm && cudaMalloc(&d_hmax, ni * sizeof(int32_t)) != cudaSuccess)
    s = bfail(b, ACO_ERR_OUT_OF_MEMORY, "initialize: alloc");
  for (size_t i = 0; i < ni && !s; i++) {
    aco_colony *c = b->cols[i];
    c->stream = pool[i % npool];
    if (int e = init_begin(c, libm ? d_hmax + i : nullptr)) s = bfail(b, e, c->err);
  }
  if (libm) {
    for (int q = 0; q < npool; q++)
      if (pool[q] && cudaStreamSynchronize(pool[q]) != cudaSuccess && !s)
        s = bfail(b, ACO_ERR_CUDA, "initialize: synchronize");
    if (!s && cudaMemcpy(hmax.data(), d_hmax, ni * sizeof(int32_t), cudaMemcpyDeviceToHost) !=
                  cudaSuccess)
      s = bfail(b, ACO_ERR_CUDA, "initialize: read max");
    std::vector<float> table;
    const int32_t hm = s ? 0 : *std::max_element(hmax.begin(), hmax.end());
    if (!s && !libm_table(hm, b->p.beta, table)) s = bfail(b, ACO_ERR_UNSUPPORTED, kTooFar);
    entries = (int32_t)table.size();
    if (!s && (cudaMalloc(&d_table, table.size() * 4) != cudaSuccess ||
               cudaMemcpy(d_table, table.data(), table.size() * 4, cudaMemcpyHostToDevice) !=
                   cudaSuccess))
      s = bfail(b, ACO_ERR_CUDA, "initialize: upload table");
  }
  for (size_t i = 0; i < ni && !s; i++) {
    aco_colony *c = b->cols[i];
    if (libm)
      if (int e = init_heuristic_table(c, d_table, entries)) s = bfail(b, e, c->err);
    if (!s)
      if (int e = init_rest(c)) s = bfail(b, e, c->err);
  }
  for (int q = 0; q < npool; q++)
    if (pool[q] && cudaStreamSynchronize(pool[q]) != cudaSuccess && !s)
      s = bfail(b, ACO_ERR_CUDA, "initialize: synchronize");
  if (d_hmax) cudaFree(d_hmax);
  if (d_table) cudaFree(d_table);
  for (aco_colony *c : b->cols) c->stream = b->stream;
  for (int q = 0; q < npool; q++)
    if (pool[q]) cudaStreamDestroy(pool[q]);
  if (ready) cudaEventDestroy(ready);
  if (s) return s;
  for (size_t i = 0; i < b->cols.size(); i++) {
    aco_colony *c = b->cols[i];
    if (int e = device_error(c)) return bfail(b, e, c->err);
    c->initialized = true;
    descs.push_back(make_dev(c));
    for (int j = 0; j < c->n; j++) rowmap.push_back(make_int2((int)i, j));
  }
  if (!b->d_descs) {
    ACO_BCUDA(b, cudaMalloc(&b->d_descs, descs.size() * sizeof(ColonyDev)), "alloc descs");
    ACO_BCUDA(b, cudaMalloc(&b->d_rowmap, rowmap.size() * sizeof(int2)), "alloc rowmap");
    ACO_BCUDA(b, cudaMalloc(&b->d_queue, sizeof(int)), "alloc queue");
  }
  ACO_BCUDA(b, upload_sync(b, b->d_descs, descs.data(), descs.size() * sizeof(ColonyDev)),
            "upload descs");
  ACO_BCUDA(b, upload_sync(b, b->d_rowmap, rowmap.data(), rowmap.size() * sizeof(int2)),
            "upload rowmap");
  ACO_BCUDA(b, configure_pheromone_rows(b->max_ld), "configure rows");
  if (int s = batch_build_items(b)) return s;
  b->initialized = true;
  return ACO_OK;
}

int aco_batch_run(aco_batch *b, int32_t iterations) {
  NvtxRange range("aco_batch_run");
  if (!b || iterations < 0) return ACO_ERR_INVALID_ARGUMENT;
  if (!b->initialized) return bfail(b, ACO_ERR_NOT_INITIALIZED, "batch not initialized");
  for (aco_colony *c : b->cols) state_changed(c);  // the replays rewrite every state block
  if (!b->graph_exec) {
    const int64_t before = b->launches;
    ACO_BCUDA(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "capture");
    int s = batch_enqueue(b, true, true, true, true);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (s) {
      if (g) cudaGraphDestroy(g);
      return s;
    }
    ACO_BCUDA(b, e, "end capture");
    b->graph = g;
    ACO_BCUDA(b, cudaGraphInstantiate(&b->graph_exec, g, 0), "instantiate");
    b->launches = before;
  }
  for (int32_t i = 0; i < iterations; i++)
    ACO_BCUDA(b, cudaGraphLaunch(b->graph_exec, b->stream), "graph launch");
  b->launches += (3 + (b->rows && b->p.aging ? 1 : 0)) * (int64_t)iterations;
  return ACO_OK;
}

int aco_batch_synchronize(aco_batch *b) {
  if (!b) return ACO_ERR_INVALID_ARGUMENT;
  return batch_state_check(b);
}

int aco_colony_autotune(aco_colony *c, aco_tuning *out) {
  if (!c) return ACO_ERR_INVALID_ARGUMENT;
  if (!c->initialized) return fail(c, ACO_ERR_NOT_INITIALIZED, "colony not initialized");
  // Candidates: the kernels and launch shapes that build the same tours.
  // k <= 32: staged, cluster and direct kernels; the ants (warps) per CTA
  // of the staged kernel without aging and of the direct kernel (the
  // cluster kernel and the aging staged kernel keep their plan: their ants
  // per CTA follow from the cluster size and the blend ants).  k > 32: the
  // long-row kernel with 1..11 ants per CTA.  Always: the general kernel.
  struct Cand {
    int mode, warps;
  };
  std::vector<Cand> cands;
  const int warps_try[6] = {0, 1, 2, 4, 8, 16};
  if (c->K > 32) {
    const int ants_try[7] = {0, 1, 2, 4, 6, 8, 11};
    for (int a : ants_try) cands.push_back({ACO_CONSTRUCT_ROWS, a});
  } else if (c->nn16) {
    for (int w : warps_try) {
      if (w == 0 || !c->p.aging) cands.push_back({ACO_CONSTRUCT_STAGED, w});
    }
    cands.push_back({ACO_CONSTRUCT_CLUSTER, 0});
    for (int w : warps_try) cands.push_back({ACO_CONSTRUCT_DIRECT, w});
  }
  cands.push_back({ACO_CONSTRUCT_GLOBAL, 0});
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  ACO_CUDA(c, cudaEventCreate(&e0), "event");
  ACO_CUDA(c, cudaEventCreate(&e1), "event");
  const int user_mode = c->p.construct_mode, user_warps = c->tune_warps;
  float best_ms = 1e30f;
  Cand best{user_mode, user_warps};
  int status = ACO_OK;
  for (const Cand &k : cands) {
    c->p.construct_mode = k.mode;
    c->tune_warps = k.warps;
    if (plan_construction(c) != ACO_OK) continue;  // not available at this size
    const bool match = (k.mode == ACO_CONSTRUCT_STAGED && c->staged) ||
                       (k.mode == ACO_CONSTRUCT_CLUSTER && c->cluster > 0) ||
                       (k.mode == ACO_CONSTRUCT_DIRECT && c->direct) ||
                       (k.mode == ACO_CONSTRUCT_ROWS && c->rows) ||
                       (k.mode == ACO_CONSTRUCT_GLOBAL && !c->staged && !c->cluster &&
                        !c->direct && !c->rows);
    if (!match) continue;
    // A forced shape the plan had to change (clamped to what fits) is not a
    // new candidate.
    if (k.warps > 0 && k.warps != c->staged_warps) continue;
    float ms = 1e30f;
    const ColonyDev d = make_dev(c);
    for (int rep = 0; rep < 2 && status == ACO_OK; rep++) {
      if (cudaEventRecord(e0, c->stream) != cudaSuccess || launch_construction(c, d) != cudaSuccess ||
          cudaEventRecord(e1, c->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) {
        status = fail(c, ACO_ERR_CUDA, "tune construct");
        break;
      }
      float t = 0.0f;
      cudaEventElapsedTime(&t, e0, e1);
      ms = std::min(ms, t);
    }
    if (status != ACO_OK) break;
    if (int e = device_error(c)) {
      status = e;
      break;
    }
    if (ms < best_ms) {
      best_ms = ms;
      best = k;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  c->p.construct_mode = best.mode;
  c->tune_warps = best.warps;
  if (status != ACO_OK) {
    c->p.construct_mode = user_mode;
    c->tune_warps = user_warps;
  }
  if (int s = plan_construction(c)) return s;
  if (status != ACO_OK) return status;
  // The timing launches advanced the ages: back to the initialised state
  // (the pheromone was never touched), and the captured graph is rebuilt.
  state_changed(c);
  const ColonyDev d = make_dev(c);
  ACO_CUDA(c, launch_init_colony(d, c->stream), "reset");
  ACO_CUDA(c, launch_pheromone_rows(d, false, false, false, c->stream), "reset rows");
  ACO_CUDA(c, cudaStreamSynchronize(c->stream), "synchronize");
  if (int e = device_error(c)) return e;
  drop_graph(c);  // captured with the previous construction launch
  if (out) {
    memset(out, 0, sizeof(*out));
    out->ants_per_block = c->rows || c->staged || c->direct || c->cluster ? c->staged_warps : c->apb;
    out->construct_ms = best_ms;
    out->staged_instances = c->staged ? 1 : 0;
    out->construct_mode = c->p.construct_mode;
  }
  return ACO_OK;
}

int aco_batch_autotune(aco_batch *b, aco_tuning *out) {
  if (!b) return ACO_ERR_INVALID_ARGUMENT;
  if (!b->initialized) return bfail(b, ACO_ERR_NOT_INITIALIZED, "batch not initialized");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  // Ants per CTA: warps of the k <= 32 kernels (launch-bounded to 512
  // threads); ants (scan warps, plus the chain warp) of the long-row kernel.
  const int apbs_short[6] = {1, 2, 4, 8, 16, kBatchMaxWarps};
  const int apbs_rows[6] = {2, 4, 6, 8, 11, 11};
  const int *apbs = b->rows ? apbs_rows : apbs_short;
  float best_ms = 1e30f;
  int best_apb = b->apb;
  for (int ai = 0; ai < 6; ai++) {
    const int apb = apbs[ai];
    const size_t need = b->rows ? batch_rows_smem_bytes(b->max_n, b->max_ldk_rows, apb) + 1024
                                : batch_construct_smem_bytes(
                                      batch_plan_region(b, apb, nullptr, nullptr), apb);
    if (need > (size_t)b->max_smem_optin || (b->rows && apb > kRowsMaxAnts)) continue;
    b->apb = apb;
    if (int s = batch_build_items(b)) return s;
    float ms = 1e30f;
    for (int rep = 0; rep < 2; rep++) {
      cudaEventRecord(e0, b->stream);
      if (int s = batch_enqueue(b, true, false, false, false)) return s;
      cudaEventRecord(e1, b->stream);
      ACO_BCUDA(b, cudaEventSynchronize(e1), "tune construct");
      float t = 0;
      cudaEventElapsedTime(&t, e0, e1);
      ms = std::min(ms, t);
    }
    if (ms < best_ms) {
      best_ms = ms;
      best_apb = apb;
    }
  }
  // The row pass is timed as it runs in an iteration (evaporation and the
  // deposit list of one epilogue); the instances are reset afterwards.
  if (int s = batch_enqueue(b, false, true, false, false)) return s;
  const int threads[3] = {128, 256, 512};
  float best_rows = 1e30f;
  int best_threads = b->row_threads;
  for (int t : threads) {
    b->row_threads = t;
    float ms = 1e30f;
    for (int rep = 0; rep < 2; rep++) {
      cudaEventRecord(e0, b->stream);
      if (int s = batch_enqueue(b, false, false, true, true)) return s;
      cudaEventRecord(e1, b->stream);
      ACO_BCUDA(b, cudaEventSynchronize(e1), "tune rows");
      float v = 0;
      cudaEventElapsedTime(&v, e0, e1);
      ms = std::min(ms, v);
    }
    if (ms < best_rows) {
      best_rows = ms;
      best_threads = t;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  b->apb = best_apb;
  b->row_threads = best_threads;
  if (int s = batch_build_items(b)) return s;
  // The timing runs advanced ages and counters: back to the initialised state.
  for (aco_colony *c : b->cols) {
    state_changed(c);
    const ColonyDev d = make_dev(c);
    ACO_BCUDA(b, launch_init_colony(d, b->stream), "reset");
    ACO_BCUDA(b, launch_pheromone_rows(d, false, false, false, b->stream), "reset rows");
  }
  if (int s = batch_state_check(b)) return s;
  if (out) {
    memset(out, 0, sizeof(*out));
    out->ants_per_block = best_apb;
    out->row_threads = best_threads;
    out->construct_ms = best_ms;
    out->rows_ms = best_rows;
    out->staged_instances = b->staged_count;
  }
  return ACO_OK;
}

int aco_batch_set_tuning(aco_batch *b, int32_t ants_per_block, int32_t row_threads) {
  if (!b || ants_per_block < 1 || ants_per_block > kBatchMaxWarps ||
      (row_threads != 0 && (row_threads < 64 || row_threads > 512 || row_threads % 32)))
    return ACO_ERR_INVALID_ARGUMENT;
  b->apb = ants_per_block;
  if (row_threads) b->row_threads = row_threads;
  if (!b->initialized) return ACO_OK;
  return batch_build_items(b);
}

int aco_batch_get_size(aco_batch *b, int32_t *count) {
  if (!b || !count) return ACO_ERR_INVALID_ARGUMENT;
  *count = (int32_t)b->cols.size();
  return ACO_OK;
}

int aco_batch_get_colony(aco_batch *b, int32_t i, aco_colony **out) {
  if (!b || !out || i < 0 || i >= (int32_t)b->cols.size()) return ACO_ERR_INVALID_ARGUMENT;
  *out = b->cols[i];
  return ACO_OK;
}

int aco_batch_get_glob_best(aco_batch *b, int64_t *out) {
  if (!b || !out) return ACO_ERR_INVALID_ARGUMENT;
  if (int s = batch_read_states(b, true)) return s;
  for (size_t i = 0; i < b->cols.size(); i++) {
    int s = aco_colony_get_glob_best(b->cols[i], &out[i]);
    if (s) return bfail(b, s, b->cols[i]->err);
  }
  return ACO_OK;
}

int aco_batch_get_tours_built(aco_batch *b, int64_t *out) {
  if (!b || !out) return ACO_ERR_INVALID_ARGUMENT;
  if (int s = batch_read_states(b, true)) return s;
  int64_t total = 0;
  for (aco_colony *c : b->cols) {
    aco_stats st;
    int s = aco_colony_get_stats(c, &st);
    if (s) return bfail(b, s, c->err);
    total += st.tours_built;
  }
  *out = total;
  return ACO_OK;
}

int aco_batch_get_launch_count(aco_batch *b, int64_t *out) {
  if (!b || !out) return ACO_ERR_INVALID_ARGUMENT;
  *out = b->launches;
  return ACO_OK;
}

const char *aco_batch_last_error(const aco_batch *b) { return b ? b->err.c_str() : ""; }

void aco_batch_destroy(aco_batch *b) {
  if (!b) return;
  if (b->stream) cudaStreamSynchronize(b->stream);
  batch_drop_graph(b);
  for (aco_colony *c : b->cols) aco_colony_destroy(c);
  if (b->d_descs) cudaFree(b->d_descs);
  if (b->d_rowmap) cudaFree(b->d_rowmap);
  if (b->d_items) cudaFree(b->d_items);
  if (b->d_queue) cudaFree(b->d_queue);
  if (b->h_states) cudaFreeHost(b->h_states);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

}  // extern "C"
