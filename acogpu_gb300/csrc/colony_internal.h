// colony_internal.h -- the colony object behind the opaque aco_colony
// handle, shared by the translation units of the library (not installed).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "acogpu.h"
#include "aco_kernels.h"

struct aco_colony {
  aco_params p;
  int n = 0, m = 0, K = 0, ld = 0, ldk = 0, ldm = 0;
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int32_t *dist = nullptr;
  float *eta = nullptr, *tau = nullptr, *choice = nullptr;
  int32_t *nn = nullptr;
  float *eta_nn = nullptr, *tau_nn = nullptr, *choice_nn = nullptr;
  int32_t *tours = nullptr;
  int64_t *newlen = nullptr, *len = nullptr;
  int32_t *succT = nullptr, *predT = nullptr, *gbtour = nullptr;
  int32_t *age = nullptr, *perf = nullptr;
  uint8_t *valid = nullptr;
  float *mean = nullptr;
  int32_t *dep_col = nullptr;
  float *dep_delta = nullptr;
  int32_t *plan = nullptr;  // aging colonies: the ants' roles of an iteration
  aco::ColonyState *st = nullptr;
  int16_t *nn16 = nullptr;  // candidate ids as int16, pitch ldk (k <= 32 kernels)
  float *xy = nullptr;      // coordinates (x then y) when created from coordinates
  bool staged = false;      // construction by the staged kernel
  bool direct = false;      // construction by the direct (L2-row) kernel
  int cluster = 0;          // construction by the cluster kernel: CTAs per cluster
  bool rows = false;        // construction by the long-row kernel (k > 32)
  int32_t *nn2 = nullptr;   // fallback second tier (see ColonyDev)
  float *t2v = nullptr;
  float *mout = nullptr;
  int t2 = 0;
  int staged_grid = 0, staged_warps = 0;
  int tune_warps = 0;  // ants per CTA forced by the autotuner (0: the plan's choice)
  int num_sms = 0, max_smem_optin = 0;
  std::vector<void *> allocations;
  bool initialized = false;
  int64_t optimum = -1;
  int apb = 4;
  int64_t launches = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  // Host copy of the device state block, valid until the next call that
  // enqueues work on the colony: the getters of one iteration share one
  // device-to-host read.  A colony read on its own stages it through a
  // pinned word allocated at its first read; a batch reads all its
  // instances through one pinned array of its own.
  aco::ColonyState h_cache{};
  aco::ColonyState *h_state = nullptr;
  bool state_fresh = false;
  std::string err;
};

// Every call that enqueues work on a colony (or rewrites its state) marks the
// cached state block stale.
inline void state_changed(aco_colony *c) { c->state_fresh = false; }

namespace aco {
// Device view of a colony (pointers and parameters passed to the kernels).
ColonyDev colony_dev(const aco_colony *c);
// Records `msg` as the colony's last error and returns `status`.
int colony_fail(aco_colony *c, int status, const std::string &msg);
}  // namespace aco
