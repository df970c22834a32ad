// AntSystem.h -- include-path shim for the reference's driver (see Colony.h
// in this directory).
#ifndef ANTSYSTEM_H
#define ANTSYSTEM_H
#include "Colony.h"
#endif
