// k_gemm_tc.cu -- BF16 "TN" GEMM on the 5th-generation tensor cores:
// C[M x N] (op)= A[M x K] * B[N x K]^T, A and B K-contiguous, FP32 C.
//
// One CTA (4 warps) computes a 128 x BN tile:
//  * thread 0 stages each 64-wide K block of A (128 x 64) and B (BN x 64)
//    into shared memory with 2-D TMA loads (cp.async.bulk.tensor, 128-byte
//    swizzle; rows and columns outside the tensors read as zero) on an
//    mbarrier;
//  * it issues four tcgen05.mma.kind::f16 (M=128, N=BN, K=16 each) with
//    the accumulator in tensor memory, then tcgen05.commit to a second
//    mbarrier, which also frees the staging buffers for the next block;
//  * warp w reads accumulator lanes 32w..32w+31 with tcgen05.ld and writes
//    (or atomically adds, for split K) its rows of C.
// Tensor memory is allocated by warp 0 and released on every path; every
// wait is bounded and reports a timeout through the error word.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include "aco_kernels.h"
#include "aco_mlp.h"
#include "aco_tc.cuh"

namespace aco {

namespace {

using tc::fence_after_sync;
using tc::fence_before_sync;
using tc::idesc_bf16;
using tc::smem_desc_sw128;
using tc::tma_load_2d;
using tc::tmem_load_16;
using tc::tmem_load_32;
using tc::umma_bf16;
using tc::umma_commit;
using tc::wait_bounded;
constexpr int kTcBM = tc::kBM, kTcBK = tc::kBK;

}  // namespace

template <int BN>
__global__ void __launch_bounds__(128) k_gemm_tn_tc(const __grid_constant__ CUtensorMap tmA,
                                                    const __grid_constant__ CUtensorMap tmB,
                                                    float *__restrict__ C, int ldc, int M, int N,
                                                    int K, int k_per_split, int mode,
                                                    uint32_t *err) {
  constexpr int kCols = BN < 32 ? 32 : BN;  // tensor-memory columns (power of two >= 32)
  extern __shared__ __align__(1024) unsigned char smem_tc[];
  unsigned char *base = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(smem_tc) + 1023) & ~uintptr_t(1023));
  unsigned char *sA = base;                  // 128 x 64 BF16 = 16 KB
  unsigned char *sB = base + kTcBM * 128;    // BN x 64 BF16
  uint64_t *bar_load = reinterpret_cast<uint64_t *>(sB + BN * 128);
  uint64_t *bar_mma = bar_load + 1;
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bar_mma + 1);
  int *flag = reinterpret_cast<int *>(tmem_slot + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(kCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (threadIdx.x == 0) {
    mbar_init(bar_load, 1);
    mbar_init(bar_mma, 1);
    fence_barrier_init();
    *flag = 1;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  const int m0 = blockIdx.y * kTcBM, n0 = blockIdx.x * BN;
  const int kb = blockIdx.z * k_per_split, ke = min(K, kb + k_per_split);
  const uint32_t idesc = idesc_bf16(BN);
  uint32_t phase = 0;
  bool pending = false;  // an MMA commit not yet waited for (thread 0)
  for (int k0 = kb; k0 < ke; k0 += kTcBK) {
    if (threadIdx.x == 0) {
      mbar_arrive_expect_tx(bar_load, (uint32_t)(kTcBM * 128 + BN * 128));
      tma_load_2d(sA, &tmA, k0, m0, bar_load);
      tma_load_2d(sB, &tmB, k0, n0, bar_load);
      bool ok = wait_bounded(bar_load, phase, err);
      if (ok) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint64_t da = smem_desc_sw128(sA), db = smem_desc_sw128(sB);
#pragma unroll
        for (int j = 0; j < kTcBK / 16; j++)  // K = 16 per instruction: +32 bytes
          umma_bf16(tmem, da + 2 * j, db + 2 * j, idesc, (k0 > kb || j > 0) ? 1u : 0u);
        umma_commit(bar_mma);
        pending = true;
        // The commit completes when the MMAs have read the staging buffers
        // and written the accumulator.
        ok = wait_bounded(bar_mma, phase, err);
        pending = !ok;
      }
      if (!ok) *flag = 0;
    }
    phase ^= 1u;
    __syncthreads();
    if (!*flag) break;
  }
  if (threadIdx.x == 0 && pending) wait_bounded(bar_mma, phase ^ 1u, err);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

  if (*flag && kb < ke) {
    const int row = m0 + warp * 32 + lane;
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
#pragma unroll
    for (int c0 = 0; c0 < BN; c0 += 32) {
      float v[32];
      if (BN >= 32)
        tmem_load_32(lane_base + (uint32_t)c0, v);
      else
        tmem_load_16(lane_base + (uint32_t)c0, v);
      if (row < M) {
        float *crow = C + (size_t)row * ldc;
#pragma unroll
        for (int i = 0; i < (BN >= 32 ? 32 : BN); i++) {
          const int col = n0 + c0 + i;
          if (col < N) {
            if (mode == kGemmStore)
              crow[col] = v[i];
            else if (mode == kGemmAccumulate)
              crow[col] += v[i];
            else
              atomicAdd(crow + col, v[i]);
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCols)
                 : "memory");
}

// ---------------------------------------------------------------- host side
namespace {

// Dynamic shared memory per CTA.  For BN = 128 it is padded to 56 KB so at
// most 4 CTAs share an SM: 4 x 128 tensor-memory columns = the SM's 512, so
// no tcgen05.alloc has to wait for another CTA to free its columns.
template <int BN>
constexpr size_t tc_smem() {
  return BN >= 128 ? (size_t)56 * 1024 : 1024 + (size_t)kTcBM * 128 + (size_t)BN * 128 + 64;
}

}  // namespace

cudaError_t launch_gemm_tn_tc(const __nv_bfloat16 *A, int lda, const __nv_bfloat16 *B, int ldb,
                              float *C, int ldc, int M, int N, int K, int mode, int splits,
                              uint32_t *err, cudaStream_t s) {
  if ((lda & 7) || (ldb & 7) || M <= 0 || K <= 0 || (N != 128 && N != 16))
    return cudaErrorInvalidValue;
  if ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(B)) & 15)
    return cudaErrorInvalidValue;
  if (splits < 1) splits = 1;
  int kps = (K + splits - 1) / splits;
  kps = (kps + kTcBK - 1) / kTcBK * kTcBK;
  splits = (K + kps - 1) / kps;
  if (splits > 1) mode = kGemmAtomic;
  CUtensorMap ta, tb;
  if (!tc::make_map_bf16(&ta, A, M, K, lda, kTcBM) || !tc::make_map_bf16(&tb, B, N, K, ldb, N))
    return cudaErrorInvalidValue;
  dim3 grid(1, (M + kTcBM - 1) / kTcBM, splits);
  if (N == 128) {
    // 56 KB is above the 48 KB default limit; the attribute is set per device.
    static unsigned long long configured = 0;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev >= 64) return cudaErrorInvalidDevice;
    if (!((configured >> dev) & 1ull)) {
      cudaError_t e = cudaFuncSetAttribute(k_gemm_tn_tc<128>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)tc_smem<128>());
      if (e != cudaSuccess) return e;
      configured |= 1ull << dev;
    }
    k_gemm_tn_tc<128><<<grid, 128, tc_smem<128>(), s>>>(ta, tb, C, ldc, M, N, K, kps, mode, err);
  } else {
    k_gemm_tn_tc<16><<<grid, 128, tc_smem<16>(), s>>>(ta, tb, C, ldc, M, N, K, kps, mode, err);
  }
  return cudaGetLastError();
}

namespace tc {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

bool make_map_bf16(CUtensorMap *map, const __nv_bfloat16 *ptr, int rows, int cols, int ld,
                   int box_rows) {
  auto fn = encode_fn();
  if (!fn) return false;
  cuuint64_t gdim[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  cuuint64_t gstride[1] = {(cuuint64_t)ld * 2};
  cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_rows};
  cuuint32_t estride[2] = {1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16 *>(ptr), gdim,
            gstride, box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace tc
}  // namespace aco
