// checkpoint.cu -- saving and resuming a colony (aco_colony_save / _load).
//
// The reference has no checkpoint.  A colony's evolution depends on the
// pheromone matrix, the device state block (bests, the iteration counter that
// keys the injected random stream, aging flags), the best-so-far tour with
// its successor/predecessor column, the aging arrays, the previous tour
// lengths and the candidate heuristic (a learned prior rewrites it).  Those
// are written; choice, choice_nn, tau_nn and the row means are recomputed
// from them on load by the row pass, so a loaded colony continues bit for bit
// as the saved one would have.  The file also records the parameters and a
// hash of the distance matrix, and a load into a colony of another instance
// or configuration is refused.
//
// Layout (little-endian host structs):
//   header | ColonyState | tau n*n f32 | eta_nn n*K f32 | best tour n i32 |
//   best succ n i32 | best pred n i32 | age m i32 | perf m i32 | valid m u8 |
//   len m i64 | tours m*n i32 | newlen m i64
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "colony_internal.h"

using namespace aco;

namespace {

constexpr char kMagic[8] = {'A', 'C', 'O', 'C', 'K', 'P', 'T', '1'};

struct CheckpointHeader {
  char magic[8];
  uint32_t version, header_bytes;
  aco_params params;
  int32_t n, m, K, state_bytes;
  int64_t optimum;
  uint64_t dist_hash;  // FNV-1a over the n x n distances
};

uint64_t fnv1a(const void *data, size_t bytes, uint64_t h = 1469598103934665603ull) {
  const unsigned char *p = static_cast<const unsigned char *>(data);
  for (size_t i = 0; i < bytes; i++) {
    h ^= p[i];
    h *= 1099511628211ull;
  }
  return h;
}

struct File {
  FILE *f = nullptr;
  ~File() {
    if (f) fclose(f);
  }
};

// Host copy of an r x cols block with device pitch `ld` (elements).
template <class T>
cudaError_t d2h(aco_colony *c, std::vector<T> &out, const T *src, size_t rows, size_t cols,
                size_t ld) {
  out.resize(rows * cols);
  return cudaMemcpy2DAsync(out.data(), cols * sizeof(T), src, ld * sizeof(T), cols * sizeof(T),
                           rows, cudaMemcpyDeviceToHost, c->stream);
}

template <class T>
cudaError_t h2d(aco_colony *c, T *dst, const std::vector<T> &in, size_t rows, size_t cols,
                size_t ld) {
  return cudaMemcpy2DAsync(dst, ld * sizeof(T), in.data(), cols * sizeof(T), cols * sizeof(T),
                           rows, cudaMemcpyHostToDevice, c->stream);
}

template <class T>
bool put(FILE *f, const std::vector<T> &v) {
  return fwrite(v.data(), sizeof(T), v.size(), f) == v.size();
}

template <class T>
bool get(FILE *f, std::vector<T> &v, size_t count) {
  v.resize(count);
  return fread(v.data(), sizeof(T), count, f) == count;
}

int cuda_status(aco_colony *c, cudaError_t e, const char *what) {
  return colony_fail(c, e == cudaErrorMemoryAllocation ? ACO_ERR_OUT_OF_MEMORY : ACO_ERR_CUDA,
                     std::string(what) + ": " + cudaGetErrorString(e));
}

uint64_t distance_hash(aco_colony *c, cudaError_t *e) {
  std::vector<int32_t> d;
  *e = d2h(c, d, c->dist, c->n, c->n, c->ld);
  if (*e == cudaSuccess) *e = cudaStreamSynchronize(c->stream);
  return *e == cudaSuccess ? fnv1a(d.data(), d.size() * 4) : 0;
}

}  // namespace

extern "C" {

int aco_colony_save(aco_colony *c, const char *path) {
  if (!c || !path) return ACO_ERR_INVALID_ARGUMENT;
  if (!c->initialized) return colony_fail(c, ACO_ERR_NOT_INITIALIZED, "colony not initialized");
  const size_t n = c->n, m = c->m, K = c->K;
  CheckpointHeader h;
  memset(&h, 0, sizeof(h));
  memcpy(h.magic, kMagic, 8);
  h.version = 1;
  h.header_bytes = sizeof(h);
  h.params = c->p;
  h.n = c->n;
  h.m = c->m;
  h.K = c->K;
  h.state_bytes = sizeof(ColonyState);
  h.optimum = c->optimum;
  cudaError_t e;
  h.dist_hash = distance_hash(c, &e);
  if (e != cudaSuccess) return cuda_status(c, e, "read distances");

  std::vector<unsigned char> st(sizeof(ColonyState));
  std::vector<float> tau, eta_nn;
  std::vector<int32_t> best, bsucc, bpred, age, perf, tours;
  std::vector<uint8_t> valid;
  std::vector<int64_t> len, newlen;
  e = cudaMemcpyAsync(st.data(), c->st, st.size(), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = d2h(c, tau, c->tau, n, n, c->ld);
  if (e == cudaSuccess) e = d2h(c, eta_nn, c->eta_nn, n, K, c->ldk);
  if (e == cudaSuccess) e = d2h(c, best, c->gbtour, 1, n, n);
  if (e == cudaSuccess) e = d2h(c, bsucc, (const int32_t *)c->succT + m, n, 1, c->ldm);
  if (e == cudaSuccess) e = d2h(c, bpred, (const int32_t *)c->predT + m, n, 1, c->ldm);
  if (e == cudaSuccess) e = d2h(c, age, c->age, 1, m, m);
  if (e == cudaSuccess) e = d2h(c, perf, c->perf, 1, m, m);
  if (e == cudaSuccess) e = d2h(c, valid, c->valid, 1, m, m);
  if (e == cudaSuccess) e = d2h(c, len, c->len, 1, m, m);
  if (e == cudaSuccess) e = d2h(c, tours, c->tours, m, n, c->ld);
  if (e == cudaSuccess) e = d2h(c, newlen, c->newlen, 1, m, m);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_status(c, e, "read colony state");

  File f;
  f.f = fopen(path, "wb");
  if (!f.f) return colony_fail(c, ACO_ERR_IO, std::string("cannot write ") + path);
  const bool ok = fwrite(&h, sizeof(h), 1, f.f) == 1 && put(f.f, st) && put(f.f, tau) &&
                  put(f.f, eta_nn) && put(f.f, best) && put(f.f, bsucc) && put(f.f, bpred) &&
                  put(f.f, age) && put(f.f, perf) && put(f.f, valid) && put(f.f, len) &&
                  put(f.f, tours) && put(f.f, newlen);
  if (!ok || fflush(f.f) != 0) return colony_fail(c, ACO_ERR_IO, std::string("write failed: ") + path);
  return ACO_OK;
}

int aco_colony_load(aco_colony *c, const char *path) {
  if (!c || !path) return ACO_ERR_INVALID_ARGUMENT;
  state_changed(c);
  if (!c->initialized) return colony_fail(c, ACO_ERR_NOT_INITIALIZED, "colony not initialized");
  File f;
  f.f = fopen(path, "rb");
  if (!f.f) return colony_fail(c, ACO_ERR_IO, std::string("cannot open ") + path);
  CheckpointHeader h;
  if (fread(&h, sizeof(h), 1, f.f) != 1 || memcmp(h.magic, kMagic, 8) != 0 || h.version != 1 ||
      h.header_bytes != sizeof(h) || h.state_bytes != (int32_t)sizeof(ColonyState))
    return colony_fail(c, ACO_ERR_FORMAT, std::string("not a colony checkpoint: ") + path);
  if (h.n != c->n || h.m != c->m || h.K != c->K || memcmp(&h.params, &c->p, sizeof(aco_params)))
    return colony_fail(c, ACO_ERR_INVALID_ARGUMENT,
                       "checkpoint of another configuration (sizes or parameters differ)");
  cudaError_t e;
  if (distance_hash(c, &e) != h.dist_hash || e != cudaSuccess)
    return e != cudaSuccess ? cuda_status(c, e, "read distances")
                            : colony_fail(c, ACO_ERR_INVALID_ARGUMENT,
                                          "checkpoint of another instance (distances differ)");
  const size_t n = c->n, m = c->m, K = c->K;
  std::vector<unsigned char> st;
  std::vector<float> tau, eta_nn;
  std::vector<int32_t> best, bsucc, bpred, age, perf, tours;
  std::vector<uint8_t> valid;
  std::vector<int64_t> len, newlen;
  const bool ok = get(f.f, st, sizeof(ColonyState)) && get(f.f, tau, n * n) &&
                  get(f.f, eta_nn, n * K) && get(f.f, best, n) && get(f.f, bsucc, n) &&
                  get(f.f, bpred, n) && get(f.f, age, m) && get(f.f, perf, m) &&
                  get(f.f, valid, m) && get(f.f, len, m) && get(f.f, tours, m * n) &&
                  get(f.f, newlen, m);
  if (!ok) return colony_fail(c, ACO_ERR_FORMAT, std::string("truncated checkpoint: ") + path);
  for (size_t i = 0; i < n; i++)
    if ((uint32_t)best[i] >= (uint32_t)n || (uint32_t)bsucc[i] >= (uint32_t)n ||
        (uint32_t)bpred[i] >= (uint32_t)n)
      return colony_fail(c, ACO_ERR_FORMAT, "checkpoint holds a city outside the instance");

  e = cudaMemcpyAsync(c->st, st.data(), st.size(), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = h2d(c, c->tau, tau, n, n, c->ld);
  if (e == cudaSuccess) e = h2d(c, c->eta_nn, eta_nn, n, K, c->ldk);
  if (e == cudaSuccess) e = h2d(c, c->gbtour, best, 1, n, n);
  if (e == cudaSuccess) e = h2d(c, c->succT + m, bsucc, n, 1, c->ldm);
  if (e == cudaSuccess) e = h2d(c, c->predT + m, bpred, n, 1, c->ldm);
  if (e == cudaSuccess) e = h2d(c, c->age, age, 1, m, m);
  if (e == cudaSuccess) e = h2d(c, c->perf, perf, 1, m, m);
  if (e == cudaSuccess) e = h2d(c, c->valid, valid, 1, m, m);
  if (e == cudaSuccess) e = h2d(c, c->len, len, 1, m, m);
  if (e == cudaSuccess) e = h2d(c, c->tours, tours, m, n, c->ld);
  if (e == cudaSuccess) e = h2d(c, c->newlen, newlen, 1, m, m);
  // choice, choice_nn, tau_nn and the row means from the restored tau/eta_nn
  if (e == cudaSuccess)
    e = launch_pheromone_rows(colony_dev(c), false, false, false, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_status(c, e, "restore colony state");
  c->optimum = h.optimum;
  return ACO_OK;
}

}  // extern "C"
