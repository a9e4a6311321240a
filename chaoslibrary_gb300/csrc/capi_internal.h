// Internal helpers of the C-ABI layer shared by its translation units.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "../../include/chaos_gb300.h"
#include "launch.h"

namespace chaos {

int set_error(int code, const char* fmt, ...);
int cuda_error(cudaError_t e, const char* what);

// One C-ABI call: resolves the device and stream, hands out stream-ordered
// device buffers from the library's pool (freed when the call finishes),
// stages host inputs and outputs, and synchronises host-memory calls.
struct Call {
    chaos_exec ex{};
    int device = 0, prevDevice = 0;
    cudaStream_t stream = nullptr;
    cudaMemPool_t pool = nullptr;
    std::vector<void*> owned;
    bool failed = false;

    int begin(const chaos_exec* e);
    void* alloc(size_t bytes);  // device scratch, freed at finish()
    const void* input(const void* user, size_t bytes);  // device view of a caller input
    void* output(void* user, size_t bytes);             // device buffer for a caller output
    int to_host(void* host, const void* dev, size_t bytes);  // copy back (host-memory calls)
    int finish(int rc);
};

// The device's auxiliary streams (8, created on first use) for concurrent branches.
int aux_streams(int device, std::vector<cudaStream_t>& out);

// Argument checks + parameter blocks shared by the entry points (capi.cu).
// gridMode: CHAOS_GRID_* bits; kGridStepAxis lets indicesOfMutVars[0] be
// CHAOS_MUT_STEP (the step-size sweep of chaos_bifurcation_sweep).
constexpr int kGridStepAxis = 1 << 16;
int fill_sweep(SweepParams& P, int system, int dim, double tMax, int nPts, double h, int nIC, const double* ic,
               const double* ranges, const int* mut, int wv, double maxValue, double transientTime,
               const double* values, int nValues, int preScaller, bool basins, int gridMode = 0);
int fill_lle(LleParams& L, int system, double tMax, double NT, int nPts, double h, double eps,
             const double* initialConditions, int amountOfInitialConditions, const double* ranges,
             const int* indicesOfMutVars, double transientTime, const double* values, int amountOfValues,
             int dim = 2, int gridMode = 0);
// Host values of a log-scale axis (the legacy getValueByIdxLog, then 10^x).
void log_axis_values(double r0, double r1, int nPts, bool f32, std::vector<double>& out);

}  // namespace chaos
