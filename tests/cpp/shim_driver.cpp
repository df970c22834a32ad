// Drives the engine through the reference-shaped C++ classes of
// acogpu_colony.hpp, the way TSP::execute drives a Colony
// (reference: src/TSP.cpp:43-71).  Reads an n*n int32 distance matrix from a
// file, prints the best-so-far length and tour after `iters` iterations.
//   shim_driver <dist.bin> <n> <ants> <iters> <aging 0|1>
#include <stdio.h>
#include <stdlib.h>

#include <vector>

#include "acogpu_colony.hpp"

int main(int argc, char **argv) {
  if (argc != 6) return 2;
  const int n = atoi(argv[2]), m = atoi(argv[3]), iters = atoi(argv[4]), aging = atoi(argv[5]);
  std::vector<int> dist((size_t)n * n);
  FILE *f = fopen(argv[1], "rb");
  if (!f || fread(dist.data(), sizeof(int), dist.size(), f) != dist.size()) return 3;
  fclose(f);
  Colony *colony = aging ? static_cast<Colony *>(new AntSystem(dist.data(), n, m, 1.0f, 2.0f,
                                                               0.5f, 3, 5, 10, 2, m / 2, 100))
                         : static_cast<Colony *>(new AntSystem(dist.data(), n, m, 1.0f, 2.0f,
                                                               0.5f));
  colony->initialize();
  float timers[6];
  for (int i = 0; i < iters; i++) {
    colony->constructSolution(timers);
    printf("iter %d ants %u iterbest %ld globalbest %ld\n", i, colony->getNumValidAnts(),
           colony->getIterBestDist(), colony->getGlobBestDist());
  }
  printf("name %s\n", colony->antSystemName());
  printf("best %ld\n", colony->getGlobBestDist());
  printf("tour %s\n", colony->getTour().c_str());
  delete colony;
  return 0;
}
