// aco_tc.cuh -- building blocks of the tcgen05 kernels (k_gemm_tc.cu,
// k_mlp_fused.cu): K-major BF16 operand tiles with 128-byte swizzle, 2-D TMA
// loads, tcgen05.mma / commit / ld, and the host-side tensor-map encoder.
//
// Operand layout in shared memory: a K-major operand of R rows is a series
// of 64-wide K-tiles of R x 128 bytes; inside a K-tile, row r starts at
// r * 128 and its 16-byte chunk c (elements 8c..8c+7) is stored at chunk
// c ^ (r & 7).  A 2-D TMA load with CU_TENSOR_MAP_SWIZZLE_128B into a
// 1024-byte aligned buffer writes exactly this layout, and the descriptor
// below reads it (8-row groups 1024 bytes apart).
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include "aco_device.cuh"

namespace aco {
namespace tc {

constexpr int kBM = 128;  // M of every MMA here (one accumulator lane per row)
constexpr int kBK = 64;   // K-tile width in elements (128 bytes of BF16)

// Byte offset of element (r, k) inside one K-tile (k < 64).
__device__ __forceinline__ uint32_t sw128_offset(int r, int k) {
  return (uint32_t)(r * 128 + ((((k >> 3) ^ (r & 7)) & 7) << 4) + ((k & 7) << 1));
}

// Bounded mbarrier wait reporting into `err` (no trap, no endless spin).
__device__ __forceinline__ bool wait_bounded(uint64_t *bar, uint32_t parity, uint32_t *err) {
  for (uint32_t i = 0; i < kMaxPolls; i++)
    if (mbar_try_wait(bar, parity)) return true;
  if (err) atomicOr(err, kErrTimeout);
  return false;
}

// Shared-memory descriptor of a K-major operand K-tile with 128-byte
// swizzle: start address, stride between 8-row groups (1024 bytes),
// descriptor version 1, layout type SWIZZLE_128B.  Advancing K by 16
// elements inside the K-tile adds 32 bytes (2 in the encoded address).
__device__ __forceinline__ uint64_t smem_desc_sw128(const void *tile) {
  const uint64_t addr = smem_u32(tile);
  uint64_t d = (addr >> 4) & 0x3FFFull;
  d |= 1ull << 16;                   // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;  // stride byte offset
  d |= 1ull << 46;                   // version
  d |= 2ull << 61;                   // SWIZZLE_128B
  return d;
}

// Shared-memory descriptor of an MN-major operand with 128-byte swizzle.
// An MN-major atom is 8 K-rows of 64 contiguous M (or N) elements, 128 bytes
// a row, chunks swizzled by the row like the K-major layout -- so a
// K-major tile set [rows][64-wide K-tiles] written for one product is, read
// this way, the MN-major operand of a product whose K runs over those rows:
// M/N atoms `atom_stride` bytes apart (the K-tiles), 8-row groups 1024
// bytes apart.  Advancing K by 16 rows adds 2048 bytes to the start.
__device__ __forceinline__ uint64_t smem_desc_sw128_mn(const void *start, uint32_t atom_stride) {
  const uint64_t addr = smem_u32(start);
  uint64_t d = (addr >> 4) & 0x3FFFull;
  d |= (uint64_t)((atom_stride >> 4) & 0x3FFFu) << 16;  // leading byte offset: M/N atoms
  d |= (uint64_t)(1024 >> 4) << 32;                     // stride byte offset: 8-row K groups
  d |= 1ull << 46;                                      // version
  d |= 2ull << 61;                                      // SWIZZLE_128B
  return d;
}

// Instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, M = 128, N = n.
__host__ __device__ constexpr uint32_t idesc_bf16(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(kBM >> 4) << 24);
}

// The same with A and/or B MN-major (bits 15 and 16 of the descriptor).
__host__ __device__ constexpr uint32_t idesc_bf16_major(int n, bool a_mn, bool b_mn) {
  return idesc_bf16(n) | (a_mn ? 1u << 15 : 0u) | (b_mn ? 1u << 16 : 0u);
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y,
                                            uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, "
      "{%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(da), "l"(db), "r"(idesc), "r"(accumulate));
}

// Arrives on `bar` once every tcgen05 operation issued before it by this
// thread has completed (MMAs included: their shared-memory reads and
// accumulator writes).
__device__ __forceinline__ void umma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// 32 consecutive accumulator columns of this thread's lane.
__device__ __forceinline__ void tmem_load_32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
      "%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// 16 consecutive accumulator columns (the first 16 entries of v).
__device__ __forceinline__ void tmem_load_16(uint32_t taddr, float (&v)[32]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t cols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(slot)),
               "r"(cols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t tmem, uint32_t cols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(cols)
               : "memory");
}

// 2-D map of a row-major BF16 matrix (rows x cols, leading dimension ld in
// elements), boxes of box_rows x 64 with 128-byte swizzle; entries outside
// the matrix read as zero.  Host only.
bool make_map_bf16(CUtensorMap *map, const __nv_bfloat16 *ptr, int rows, int cols, int ld,
                   int box_rows);

}  // namespace tc
}  // namespace aco
