// noalloc.cu -- nn-list build in the reference's quicksort order without any
// device allocation.
//
// The colony path (aco_colony_initialize with ACO_NN_REFERENCE_QSORT) gets
// the per-row key scratch of the quicksort kernel from cudaMallocAsync.  Some
// callers cannot allocate: code that runs between other streams' work and
// cannot afford the device-wide synchronisation of cudaFree, callers whose
// memory is owned by a framework's caching allocator or a fixed budget, and
// callers that must not fail with an out-of-memory error halfway through a
// pipeline.  For them this entry point keeps the scratch in a file-scope
// __device__ array of fixed size, which the CUDA runtime creates when the
// library's module is loaded on a device and keeps until the process exits.
//
// In host code the array's name only stands for the symbol; its device
// address comes from cudaGetSymbolAddress, taken with the device current.
// That set-up runs once per CUDA context: the first call on a device does
// it, and so does the first call after the device's context was replaced
// (cudaDeviceReset, or the primary context released and created again),
// because the module -- and with it the array -- may then sit at another
// address.  The context is identified by its driver-assigned unique id; if
// the driver entry points that give it cannot be resolved, every call looks
// the address up again (a host-side table lookup, no device work).
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <mutex>

#include "acogpu.h"
#include "aco_kernels.h"

namespace {

constexpr int kNoAllocMaxCities = ACO_NOALLOC_MAX_CITIES;
constexpr int kMaxDevices = 64;

// Per-row distance keys of the quicksort: n rows of n int32.
static __device__ __align__(256) int32_t g_nn_scratch[kNoAllocMaxCities * kNoAllocMaxCities];
// Error flags written by the kernel's own checks (shared by every call, like
// the scratch).
static __device__ __align__(256) aco::ColonyState g_nn_state;

struct DeviceSymbols {
  bool ready;
  unsigned long long ctx_id;
  int32_t *scratch;
  aco::ColonyState *state;
};

DeviceSymbols g_symbols[kMaxDevices];
std::mutex g_symbols_mutex;

using CtxGetCurrentFn = CUresult (*)(CUcontext *);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long *);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;
bool g_entry_points_tried = false;

// Unique id of the calling thread's current context; false if unknown.
bool current_context_id(unsigned long long *id) {
  if (!g_entry_points_tried) {
    g_entry_points_tried = true;
    void *f1 = nullptr, *f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) ==
            cudaSuccess &&
        q1 == cudaDriverEntryPointSuccess &&
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) ==
            cudaSuccess &&
        q2 == cudaDriverEntryPointSuccess) {
      g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
      g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(f2);
    }
  }
  if (!g_ctx_get_current || !g_ctx_get_id) return false;
  CUcontext ctx = nullptr;
  if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx) return false;
  return g_ctx_get_id(ctx, id) == CUDA_SUCCESS;
}

// Device addresses of the static arrays for the current device (which the
// caller has made current, and whose context the runtime has created).
int resolve_symbols(int device, DeviceSymbols *out) {
  std::lock_guard<std::mutex> lock(g_symbols_mutex);
  DeviceSymbols &s = g_symbols[device];
  unsigned long long id = 0;
  const bool known = current_context_id(&id);
  if (!known || !s.ready || s.ctx_id != id) {
    void *scratch = nullptr, *state = nullptr;
    s.ready = false;
    if (cudaGetSymbolAddress(&scratch, g_nn_scratch) != cudaSuccess) return ACO_ERR_CUDA;
    if (cudaGetSymbolAddress(&state, g_nn_state) != cudaSuccess) return ACO_ERR_CUDA;
    s.scratch = static_cast<int32_t *>(scratch);
    s.state = static_cast<aco::ColonyState *>(state);
    s.ctx_id = id;
    s.ready = known;
  }
  *out = s;
  return ACO_OK;
}

}  // namespace

extern "C" int aco_nn_list_reference_order_noalloc(const int32_t *dist_dev, int32_t n,
                                                   int32_t *nn_dev, void *stream) {
  if (!dist_dev || !nn_dev) return ACO_ERR_INVALID_ARGUMENT;
  if (n < 1 || n > kNoAllocMaxCities) return ACO_ERR_UNSUPPORTED;
  int device = 0;
  if (cudaGetDevice(&device) != cudaSuccess || device < 0 || device >= kMaxDevices)
    return ACO_ERR_CUDA;
  // cudaSetDevice creates the device's primary context if it does not exist
  // yet (and keeps the device current), so its id can be read.
  if (cudaSetDevice(device) != cudaSuccess) return ACO_ERR_CUDA;
  DeviceSymbols sym;
  int status = resolve_symbols(device, &sym);
  if (status != ACO_OK) return status;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // The error flags must start at zero; the scratch is written before it is read.
  if (cudaMemsetAsync(sym.state, 0, sizeof(aco::ColonyState), s) != cudaSuccess)
    return ACO_ERR_CUDA;
  if (aco::launch_nn_ref_qsort(dist_dev, n, n, sym.scratch, nn_dev, n, sym.state, s) !=
      cudaSuccess)
    return ACO_ERR_CUDA;
  uint32_t err = 0;
  if (cudaMemcpyAsync(&err, &sym.state->error, sizeof(err), cudaMemcpyDeviceToHost, s) !=
      cudaSuccess)
    return ACO_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return ACO_ERR_CUDA;
  return err ? ACO_ERR_DEVICE_CHECK : ACO_OK;
}
