// selftest.cu -- self-test of the device failure path.
//
// Every wait in the engine's kernels is bounded: mbar_wait_bounded gives up
// after a number of polls, records kErrTimeout in the colony state and
// returns, and the host turns the flag into ACO_ERR_DEVICE_TIMEOUT.  This
// kernel exercises that path on purpose without faulting anything: it waits
// on an mbarrier that nothing ever arrives on (no copy is issued), with a
// short poll limit, and exits normally.  The context stays usable.
#include <cuda_runtime.h>

#include "aco_kernels.h"

namespace aco {
namespace {

__global__ void k_selftest_wait(ColonyState *st, uint32_t polls) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);  // one arrival expected, none will come
    fence_barrier_init();
  }
  __syncthreads();
  if (threadIdx.x == 0 && mbar_wait_bounded(&bar, 0, st, polls))
    atomicOr(&st->error, kErrCheck);  // a completed phase here would be a defect
}

}  // namespace
}  // namespace aco

extern "C" int aco_selftest_bounded_wait(uint32_t polls) {
  using namespace aco;
  if (polls == 0 || polls > kMaxPolls) return ACO_ERR_INVALID_ARGUMENT;
  ColonyState *st = nullptr;
  if (cudaMalloc(&st, sizeof(ColonyState)) != cudaSuccess) return ACO_ERR_OUT_OF_MEMORY;
  ColonyState h;
  cudaError_t e = cudaMemset(st, 0, sizeof(ColonyState));
  if (e == cudaSuccess) {
    k_selftest_wait<<<1, 32>>>(st, polls);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(&h, st, sizeof(ColonyState), cudaMemcpyDeviceToHost);
  cudaFree(st);
  if (e != cudaSuccess) return ACO_ERR_CUDA;
  if (h.error & kErrCheck) return ACO_ERR_DEVICE_CHECK;
  return (h.error & kErrTimeout) ? ACO_ERR_DEVICE_TIMEOUT : ACO_OK;
}
