/*
 * acogpu_rng.h -- the injected uniform stream shared by the GPU kernels, the
 * CPU oracle and the compiled-reference checker.
 *
 * The reference draws its two random numbers per ant from a stateful ran2
 * generator seeded from time(NULL) (reference: src/Utils.cu:19-125, draw
 * sites src/Colony.cu:518 and src/Colony.cu:826) or from per-ant cuRAND
 * XORWOW states (inc/Colony.cuh:58-72).  Neither is reproducible across
 * implementations, so every implementation here draws from one counter-based
 * stream instead:
 *
 *     u(seed, iteration, ant, step)
 *
 * step 0 is the start-city draw of initTour, step x (1 <= x < n) is the
 * roulette draw that picks the x-th city.  A draw that is never used (an ant
 * that takes the fallback branch) shifts nothing, because each draw is a pure
 * function of its counters.
 *
 * The mixer is the SplitMix64 finaliser (Steele, Lea & Flood, "Fast
 * splittable pseudorandom number generators", OOPSLA 2014), applied twice.
 * The result is a float in {2^-25} U {j * 2^-24 : 1 <= j < 2^24}: never 0 and
 * never 1, so (long)(u * (float)n) < n and u * sum < sum for every float sum.
 */
#ifndef ACOGPU_RNG_H
#define ACOGPU_RNG_H

#include <stdint.h>

#if defined(__CUDACC__)
#define ACO_RNG_FN __host__ __device__ __forceinline__
#else
#define ACO_RNG_FN static inline
#endif

ACO_RNG_FN uint64_t aco_mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

/* Field widths of the counter key: iteration 22 bits, ant 21 bits, step 21
 * bits (so up to 2^21 ants and cities; iterations wrap after 2^22). */
ACO_RNG_FN uint64_t aco_rng_key(uint32_t iteration, uint32_t ant, uint32_t step) {
  return ((uint64_t)(iteration & 0x3FFFFFu) << 42) |
         ((uint64_t)(ant & 0x1FFFFFu) << 21) | (uint64_t)(step & 0x1FFFFFu);
}

ACO_RNG_FN float aco_uniform(uint64_t seed, uint32_t iteration, uint32_t ant,
                             uint32_t step) {
  uint64_t h = aco_mix64(aco_mix64(seed) ^ aco_rng_key(iteration, ant, step));
  uint32_t top = (uint32_t)(h >> 40); /* 24 bits */
  /* top * 2^-24 is exact in float; 0 maps to 2^-25. */
  return top ? (float)top * 5.9604644775390625e-08f : 2.98023223876953125e-08f;
}

#endif /* ACOGPU_RNG_H */
