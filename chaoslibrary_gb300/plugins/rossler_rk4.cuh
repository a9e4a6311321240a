// Rossler (a, b, c) with one classic RK4 step per call, written as a ChaosLibrary
// plug-in: it defines calcDiscreteModel, SIZE_X, SIZE_A and
// CALC_DISCRETE_MODEL(X, a, h) exactly as the reference's systems/systems.cuh
// does (systems/systems.cuh:12-38), so it can replace that header in a
// reference build or be compiled into this engine as its user plug-in.
// The arithmetic is the engine's own RK4 step (csrc/systems.h), so a
// reference build that includes this header integrates bit-identically.
#ifndef ROSSLER_RK4_CUH
#define ROSSLER_RK4_CUH
#include "../csrc/systems.h"

__device__ inline void calcDiscreteModel(double* X, const double* a, double h) {
    chaos::rk4_step<chaos::Rossler>(X, a, chaos::RK4H<double>(h));
}
#define SIZE_X 3
#define SIZE_A 3
#define CALC_DISCRETE_MODEL(X, a, h) calcDiscreteModel(X, a, h)
#endif
