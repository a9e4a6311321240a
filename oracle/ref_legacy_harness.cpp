// Host harness around functions of the reference's legacy library
// (debri/cudaLibrary.cu), for pinning the engine's restatements of its
// analyses. TEST INFRASTRUCTURE ONLY (never shipped, never called by the
// engine). oracle/build_ref.py extracts, unchanged, these __device__ __host__
// functions into oracle/_ref/ref_legacy.inc and compiles them with this file
// into oracle/_ref/libref_legacy.so:
//   getValueByIdx, getValueByIdxLog (debri/cudaLibrary.cu:1182-1196),
//   peakFinder (:1205-1263), projectionOperator, gramSchmidtProcess (:2141-2187).
// leg_ls_replay re-sequences the block loop of LSKernelCUDA (:2293-2327) on
// the host around the verbatim Gram-Schmidt: the legacy kernel integrates a
// system hard-wired into the legacy sources and starts its twins from sinf of
// the chunk-relative thread index, so the replay takes the orbit step, the
// twin start and the block count from its caller.
#include "cuda_runtime.h"

#include <cmath>

#include "../chaoslibrary_gb300/csrc/systems.h"

namespace legacy_src {
#include "ref_legacy.inc"
}

extern "C" {

double leg_value(int idx, int nPts, double start, double finish, int valueNumber) {
    return legacy_src::legacy::getValueByIdx(idx, nPts, start, finish, valueNumber);
}

double leg_value_log(int idx, int nPts, double start, double finish, int valueNumber) {
    return legacy_src::legacy::getValueByIdxLog(idx, nPts, start, finish, valueNumber);
}

int leg_peak_finder(double* data, int len, double* outPeaks, double* timeOfPeaks, double h) {
    return legacy_src::legacy::peakFinder(data, 0, len, outPeaks, timeOfPeaks, h);
}

void leg_gram_schmidt(double* a, double* b, int n, double* denominators) {
    legacy_src::legacy::gramSchmidtProcess(a, b, n, denominators);
}

// The legacy spectrum's block loop for one point: `trans` steps of the orbit,
// twins y_j = x + eps * dir_j (dir: n x n rows), then nBlocks blocks of ntp
// steps of the orbit and every twin, differences to the orbit through the
// verbatim gramSchmidtProcess, exponent k += log(denominator_k / eps), twin k
// restarts at x + z_k * eps; out[k] = sum_k / tMax.
void leg_ls_replay(int system, const double* x0, const double* a, double h, int trans, int ntp, int nBlocks,
                   double eps, double tMax, const double* dir, double* out) {
    const int n = chaos::system_nx(system);
    const chaos::StepCtx<double> c(h);
    double x[12], y[144], z[144], den[12], result[12];
    double pa[32];
    for (int i = 0; i < chaos::system_na(system); ++i) pa[i] = a[i];
    for (int i = 0; i < n; ++i) {
        x[i] = x0[i];
        result[i] = 0;
    }
    for (int s = 0; s < trans; ++s) chaos::step_dyn(system, x, pa, c);
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) y[j * n + i] = x[i] + dir[j * n + i] * eps;
    for (int b = 0; b < nBlocks; ++b) {
        for (int s = 0; s < ntp; ++s) chaos::step_dyn(system, x, pa, c);
        for (int j = 0; j < n; ++j)
            for (int s = 0; s < ntp; ++s) chaos::step_dyn(system, y + j * n, pa, c);
        for (int k = 0; k < n; ++k)
            for (int l = 0; l < n; ++l) y[k * n + l] = y[k * n + l] - x[l];
        legacy_src::legacy::gramSchmidtProcess(y, z, n, den);
        for (int k = 0; k < n; ++k) {
            result[k] += log(den[k] / eps);
            for (int j = 0; j < n; ++j) y[k * n + j] = (double)(x[j] + z[k * n + j] * eps);
        }
    }
    for (int i = 0; i < n; ++i) out[i] = result[i] / tMax;
}

}  // extern "C"
