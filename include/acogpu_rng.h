/*
 * acogpu_rng.h -- the injected uniform stream shared by the GPU kernels, the
 * CPU oracle and the compiled-reference checker.
 *
 * The reference draws its random numbers from a stateful ran2 generator
 * seeded from time(NULL) (reference: src/Utils.cu:19-125, draw sites
 * src/Colony.cu:518 and src/Colony.cu:826) or from per-ant cuRAND XORWOW
 * states (inc/Colony.cuh:58-72).  Neither is reproducible across
 * implementations, so every implementation here draws from one
 * counter-based stream instead:
 *
 *     u(seed, iteration, ant, step)
 *
 * step 0 is the start-city draw of initTour, step x (1 <= x < n) is the
 * roulette draw that picks the x-th city.  A draw that is never used (an ant
 * that takes the fallback branch) shifts nothing, because each draw is a pure
 * function of its counters.
 *
 * The mixer is the 32-bit "lowbias32" integer hash (C. Wellons, "Prospecting
 * for hash functions", 2018): x ^= x>>16; x *= 0x7feb352d; x ^= x>>15;
 * x *= 0x846ca68b; x ^= x>>16.  A per-ant key folds (seed, iteration, ant)
 * once; each step then costs one hash.  The result is a float in
 * {2^-25} U {j * 2^-24 : 1 <= j < 2^24}: never 0 and never 1, so
 * (long)(u * (float)n) < n and u * sum < sum for every float sum.
 */
#ifndef ACOGPU_RNG_H
#define ACOGPU_RNG_H

#include <stdint.h>

#if defined(__CUDACC__)
#define ACO_RNG_FN __host__ __device__ __forceinline__
#else
#define ACO_RNG_FN static inline
#endif

ACO_RNG_FN uint32_t aco_hash32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}

/* Key of one ant in one iteration. */
ACO_RNG_FN uint32_t aco_ant_key(uint64_t seed, uint32_t iteration, uint32_t ant) {
  uint32_t h = aco_hash32((uint32_t)seed ^ aco_hash32((uint32_t)(seed >> 32) + 0x9E3779B9U));
  h = aco_hash32(h ^ (iteration * 0x9E3779B9U + 0x632BE5ABU));
  return aco_hash32(h ^ (ant * 0x85EBCA6BU + 0xC2B2AE35U));
}

/* Draw `step` of the ant whose key is `key`. */
ACO_RNG_FN float aco_uniform_key(uint32_t key, uint32_t step) {
  uint32_t top = aco_hash32(key + step * 0x9E3779B9U) >> 8; /* 24 bits */
  /* top * 2^-24 is exact in float; 0 maps to 2^-25. */
  return top ? (float)top * 5.9604644775390625e-08f : 2.98023223876953125e-08f;
}

ACO_RNG_FN float aco_uniform(uint64_t seed, uint32_t iteration, uint32_t ant, uint32_t step) {
  return aco_uniform_key(aco_ant_key(seed, iteration, ant), step);
}

#endif /* ACOGPU_RNG_H */
