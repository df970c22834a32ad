/*
 * ref_shim.h -- force-included (g++ -include) when the reference's CPU
 * variant is compiled in place from its own sources.  TEST INFRASTRUCTURE:
 * only the checker build under oracle/ uses it.
 *
 * The reference's CPU variant (`acouav_cpu`, PLATFORM=cpu) does not compile
 * as shipped, for two reasons, and this header supplies what is missing
 * without touching a line of the reference:
 *
 *  1. src/Colony.cu:596-685 (verifySUM, dev_reduce_probabilities_xs/_s) sit
 *     outside any `#if _GPU_` and name CUDA-only identifiers.  They are never
 *     called on the CPU path; the stubs below only let them compile.
 *  2. src/Colony.cu:85 assigns `new float[...]` to the `int* probabilities`
 *     member (inc/Colony.h:80).  When ACO_REF_COLONY_TU is defined (the
 *     Colony.cu translation unit only), every `new` expression that follows
 *     the system headers is wrapped so its result converts to any pointer
 *     type.  The array is never read on the CPU path (src/Colony.cu:809 reads
 *     the pheromone and heuristic arrays instead).
 *
 *  src/Utils.cu uses sqrt/cos/... without including <math.h> on the CPU
 *  variant (def.h only pulls CUDA headers on the GPU variant); <math.h> is
 *  included here.
 */
#ifndef ACO_REF_SHIM_H
#define ACO_REF_SHIM_H

#include <assert.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <sys/time.h>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <limits>
#include <new>
#include <sstream>
#include <string>

/* CUDA spellings used by dead code in the CPU variant. */
#define __global__
struct aco_ref_dim3 { unsigned int x, y, z; };
static const aco_ref_dim3 blockIdx = {0u, 0u, 0u};
static const aco_ref_dim3 threadIdx = {0u, 0u, 0u};
static const aco_ref_dim3 blockDim = {1u, 1u, 1u};
static inline void __syncthreads(void) {}
template <class T> struct SharedMemory {
  operator T *() { return (T *)0; }
};
enum { cudaMemcpyDeviceToHost = 2 };
static inline int cudaMemcpy(void *, const void *, size_t, int) { return 0; }
#define checkCudaErrors(x) ((void)(x))

#ifdef ACO_REF_COLONY_TU
struct aco_ref_any_ptr {
  void *p;
  template <class T> operator T *() const { return static_cast<T *>(p); }
};
struct aco_ref_new_tag {};
template <class T> static inline aco_ref_any_ptr operator*(aco_ref_new_tag, T *p) {
  aco_ref_any_ptr r = {static_cast<void *>(p)};
  return r;
}
#define new aco_ref_new_tag() * new
#endif

#endif /* ACO_REF_SHIM_H */
