// Colony.h -- include-path shim: the reference's driver (src/TSP.cpp,
// src/Setup.cpp) includes "Colony.h"; with this directory first on the
// include path it gets the GB300 engine's classes instead of
// inc/Colony.h.
#ifndef COLONY_H
#define COLONY_H
#include "def.h"
#include "acogpu_colony.hpp"
#endif
