// Host shim used ONLY to compile the reference's per-thread CUDA functions as
// plain host functions for the checker (see oracle/build_ref.py). It maps the
// CUDA qualifiers to nothing, a launch index to three thread-local globals the
// harness sets before each "thread", and the few device intrinsics the extracted code
// uses to their host equivalents (same IEEE rounding for the _rn forms; the
// fast __logf becomes the accurate logf).
#pragma once
#include <math.h>
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <stdexcept>

#define __global__
#define __device__
#define __host__
#define __constant__
#define __shared__
#define __forceinline__ inline

struct dim3 {
    unsigned x, y, z;
};
extern thread_local dim3 threadIdx, blockIdx, blockDim;  // per host thread (OpenMP replays)
typedef int cudaError_t;

inline double __fma_rn(double a, double b, double c) { return std::fma(a, b, c); }
inline float __fmaf_rn(float a, float b, float c) { return std::fmaf(a, b, c); }
inline float __logf(float x) { return logf(x); }
inline double atomicAdd(double* p, double v) { double o = *p; *p = o + v; return o; }
inline int atomicAdd(int* p, int v) { int o = *p; *p = o + v; return o; }
using std::isinf;
using std::isnan;
