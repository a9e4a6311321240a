// Host harness around functions of the reference's legacy library
// (debri/cudaLibrary.cu), for pinning the engine's restatements of its
// analyses. TEST INFRASTRUCTURE ONLY (never shipped, never called by the
// engine). oracle/build_ref.py extracts, unchanged, these functions into
// oracle/_ref/ref_legacy.inc and compiles them with this file into
// oracle/_ref/libref_legacy.so:
//   getValueByIdx, getValueByIdxLog (debri/cudaLibrary.cu:1182-1196),
//   peakFinder (:1205-1263), projectionOperator, gramSchmidtProcess (:2141-2187),
//   the hard-wired system calculateDiscreteModel (:415-464), the loops
//   loopCalculateDiscreteModel (:472-527) and loopCalculateDiscreteModel_int
//   (:604-680), distance and dbscan (:1577-1666), and the kernels
//   calculateDiscreteModelICCUDA (:1022-1116), calculateDiscreteModelCUDA_H
//   (:955-1016), peakFinderCUDA (:1345-1367), peakFinderCUDA_H (:1396-1412),
//   avgPeakFinderCUDA (:2334-2380), dbscanCUDA (:1835-1863), LLEKernelCUDA
//   (:1897-2031), LLEKernelICCUDA (:2034-2139) and LSKernelCUDA (:2189-2330).
// leg_ls_replay re-sequences the block loop of LSKernelCUDA (:2293-2327) on
// the host around the verbatim Gram-Schmidt: the legacy kernel integrates a
// system hard-wired into the legacy sources and starts its twins from sinf of
// the chunk-relative thread index, so the replay takes the orbit step, the
// twin start and the block count from its caller. leg_ic_bifurcation,
// leg_basins_v1, leg_step_sweep, leg_lle and leg_ls run the legacy kernels
// themselves, one host "thread" per point (block size 1, one chunk of all
// points), in the order the legacy host functions launch them. LLEKernelCUDA
// draws its twin direction from cuRAND: here curand_init keeps the seed and
// curand_uniform returns the caller's uniform for that seed.
#include "cuda_runtime.h"

#include <cmath>
#include <vector>

#include "../chaoslibrary_gb300/csrc/systems.h"

thread_local dim3 threadIdx, blockIdx, blockDim;

// the two cuRAND device calls of LLEKernelCUDA, fed from the caller's uniforms
struct curandState_t {
    unsigned long long seed;
};
thread_local const float* g_uniforms = nullptr;
inline void curand_init(unsigned long long seed, unsigned long long, unsigned long long, curandState_t* s) {
    s->seed = seed;
}
inline float curand_uniform(curandState_t* s) { return g_uniforms[s->seed]; }

namespace legacy_src {
namespace legacy {
// the two loops' default arguments, declared as debri/cudaLibrary.cuh declares them
bool loopCalculateDiscreteModel(double* x, const double* values, const double h, const int amountOfIterations,
                                const int amountOfX, const int preScaller = 0, const int writableVar = 0,
                                const double maxValue = 0, double* data = nullptr, const int startDataIndex = 0,
                                const int writeStep = 1);
int loopCalculateDiscreteModel_int(double* x, const double* values, const double h, const int amountOfIterations,
                                   const int amountOfX, const int preScaller = 0, const int writableVar = 0,
                                   const double maxValue = 0, double* data = nullptr, const int startDataIndex = 0,
                                   const int writeStep = 1);
}  // namespace legacy
#include "ref_legacy.inc"
}

namespace {
// one host "thread" of a 1-D launch with block size 1: global index k
void as_thread(long long k) {
    threadIdx = dim3{0, 0, 0};
    blockDim = dim3{1, 1, 1};
    blockIdx = dim3{(unsigned)k, 0, 0};
}
}  // namespace

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

// The legacy bifurcation1DIC (dim 1, debri/hostLibrary.cu:1243-1486) or
// bifurcation2DIC (dim 2, :2819-3107) kernels over all n = nPts^dim points:
// calculateDiscreteModelICCUDA, then peakFinderCUDA (dim 1: peaks into their
// own array, no times; dim 2: peaks in place, intervals in units h *
// preScaller) and for dim 2 dbscanCUDA. counts[n]: the kept peaks, or the -1
// / 0 the peak kernel leaves; peaks[n][B] and intervals[n][B] (dim 2) with B =
// (int)(tMax / h / preScaller); labels[n] (dim 2). The caller's arrays are not
// written by the kernels (they take non-const pointers).
int leg_ic_bifurcation(int dim, int nPts, double tMax, double h, double transientTime, int preScaller,
                       const double* ic, int nIC, const double* values, int nValues, const double* ranges,
                       const int* mut, int wv, double maxValue, double eps, int* counts, double* peaks,
                       double* intervals, int* labels) {
    const int B = tMax / h / preScaller;
    const int S = transientTime / h;
    const long long n = dim == 1 ? (long long)nPts : (long long)nPts * nPts;
    if (B < 1 || nIC + nValues > 4096 || n > 0x7fffffffLL) return 1;
    std::vector<double> data((size_t)n * B), out((size_t)n * B), iv((size_t)n * B), help((size_t)n * B);
    std::vector<double> rng(ranges, ranges + 2 * dim), x0(ic, ic + nIC), a(values, values + nValues);
    std::vector<int> mv(mut, mut + dim);
    for (long long k = 0; k < n; ++k) {
        as_thread(k);
        legacy_src::legacy::calculateDiscreteModelICCUDA(nPts, (int)n, B, 0, S, dim, rng.data(), h, mv.data(),
                                                         x0.data(), nIC, a.data(), nValues, B, preScaller, wv,
                                                         maxValue, data.data(), counts);
    }
    for (long long k = 0; k < n; ++k) {
        as_thread(k);
        if (dim == 1)
            legacy_src::legacy::peakFinderCUDA(data.data(), B, (int)n, counts, out.data(), nullptr, 0);
        else
            legacy_src::legacy::peakFinderCUDA(data.data(), B, (int)n, counts, data.data(), iv.data(),
                                               h * preScaller);
    }
    // the peaks as the peak kernel left them (dbscanCUDA then works in data)
    const std::vector<double>& pk = dim == 1 ? out : data;
    for (size_t i = 0; i < (size_t)n * B; ++i) {
        peaks[i] = pk[i];
        intervals[i] = iv[i];
    }
    if (dim == 2)
        for (long long k = 0; k < n; ++k) {
            as_thread(k);
            legacy_src::legacy::dbscanCUDA(data.data(), B, (int)n, counts, iv.data(), help.data(), eps, labels);
        }
    return 0;
}

// The legacy basinsOfAttraction (debri/hostLibrary.cu:4115-4556) kernels over
// the nPts x nPts map: calculateDiscreteModelICCUDA (dim 2), then
// avgPeakFinderCUDA with intervals in units h * preScaller. flags[n] (its
// systemCheker), avgPeaks[n], avgIntervals[n].
int leg_basins_v1(int nPts, double tMax, double h, double transientTime, int preScaller, const double* ic, int nIC,
                  const double* values, int nValues, const double* ranges, const int* mut, int wv, double maxValue,
                  int* flags, double* avgPeaks, double* avgIntervals) {
    const int B = tMax / h / preScaller;
    const int S = transientTime / h;
    const long long n = (long long)nPts * nPts;
    if (B < 1 || nIC + nValues > 4096 || n > 0x7fffffffLL) return 1;
    std::vector<double> data((size_t)n * B), iv((size_t)n * B);
    std::vector<double> rng(ranges, ranges + 4), x0(ic, ic + nIC), a(values, values + nValues);
    std::vector<int> mv(mut, mut + 2);
    for (long long k = 0; k < n; ++k) {
        as_thread(k);
        legacy_src::legacy::calculateDiscreteModelICCUDA(nPts, (int)n, B, 0, S, 2, rng.data(), h, mv.data(),
                                                         x0.data(), nIC, a.data(), nValues, B, preScaller, wv,
                                                         maxValue, data.data(), flags);
    }
    for (long long k = 0; k < n; ++k) {
        as_thread(k);
        legacy_src::legacy::avgPeakFinderCUDA(data.data(), B, (int)n, avgPeaks, avgIntervals, data.data(), iv.data(),
                                              flags, h * preScaller);
    }
    return 0;
}

// The legacy bifurcation1DForH (debri/hostLibrary.cu:1005-1240) kernels over
// nPts steps on the log scale of ranges[0..1]: calculateDiscreteModelCUDA_H,
// then peakFinderCUDA_H (peaks into their own array). The block of a point
// is (int)(tMax / min(ranges) / preScaller) samples, as the legacy host sizes
// it; a step whose sample count exceeds it (a powf-rounded step below the
// smaller end) would write into the next block there, and is refused here
// (return 2). counts[n] (kept peaks, or 0), peaks[n][block]; *block receives
// the block size.
int leg_step_sweep(int nPts, double tMax, double transientTime, int preScaller, const double* ic, int nIC,
                   const double* values, int nValues, const double* ranges, int wv, double maxValue, int* counts,
                   double* peaks, int peakRows, int* block) {
    const int blk = tMax / (ranges[0] < ranges[1] ? ranges[0] : ranges[1]) / preScaller;
    *block = blk;
    if (blk < 1 || nIC + nValues > 4096 || blk > peakRows) return 1;
    std::vector<double> rng(ranges, ranges + 2), x0(ic, ic + nIC), a(values, values + nValues);
    for (int k = 0; k < nPts; ++k) {
        const double hk = (double)powf(10, legacy_src::legacy::getValueByIdxLog(k, nPts, rng[0], rng[1], 0));
        const int Bk = tMax / hk / preScaller;
        if (Bk > blk) return 2;
    }
    std::vector<double> data((size_t)nPts * blk), out((size_t)nPts * blk);
    for (int k = 0; k < nPts; ++k) {
        as_thread(k);
        legacy_src::legacy::calculateDiscreteModelCUDA_H(nPts, nPts, blk, 0, transientTime, 1, rng.data(), x0.data(),
                                                         nIC, a.data(), nValues, tMax, preScaller, wv, maxValue,
                                                         data.data(), counts);
    }
    for (int k = 0; k < nPts; ++k) {
        as_thread(k);
        legacy_src::legacy::peakFinderCUDA_H(data.data(), blk, nPts, counts, out.data(), nullptr, 0);
    }
    for (size_t i = 0; i < (size_t)nPts * blk; ++i) peaks[i] = out[i];
    return 0;
}

// The legacy LLE1D (kind 0: LLEKernelCUDA, debri/hostLibrary.cu:3111-3325) or
// LLE1DIC / LLE2DIC (kind 1: LLEKernelICCUDA, :3328-3542, 3692-3825) kernel
// over all n = nPts^dim points: (int)(tMax / NT) blocks, the transient of
// (int)(transientTime / h) steps. uniforms[seed] (kind 0): the cuRAND uniform
// of each seed the kernel draws (seeds 0 .. n + nIC - 2). out[n].
int leg_lle(int kind, int dim, int nPts, double tMax, double NT, double h, double eps, double transientTime,
            const double* ic, int nIC, const double* values, int nValues, const double* ranges, const int* mut,
            double maxValue, const float* uniforms, double* out) {
    const int blocks = tMax / NT;
    const int S = transientTime / h;
    const long long n = dim == 1 ? (long long)nPts : (long long)nPts * nPts;
    if (3 * nIC + nValues > 4096 || n > 0x7fffffffLL || (kind == 0 && !uniforms)) return 1;
    std::vector<double> rng(ranges, ranges + 2 * dim), x0(ic, ic + nIC), a(values, values + nValues);
    std::vector<int> mv(mut, mut + dim);
    g_uniforms = uniforms;
    for (long long k = 0; k < n; ++k) {
        as_thread(k);
        if (kind == 0)
            legacy_src::legacy::LLEKernelCUDA(nPts, (int)n, NT, tMax, blocks, 0, S, dim, rng.data(), h, eps, mv.data(),
                                              x0.data(), nIC, a.data(), nValues, tMax / NT, 1, 0, maxValue, out);
        else
            legacy_src::legacy::LLEKernelICCUDA(nPts, (int)n, NT, tMax, blocks, 0, S, dim, rng.data(), h, eps,
                                                mv.data(), x0.data(), nIC, a.data(), nValues, tMax / NT, 1, 0,
                                                maxValue, out);
    }
    g_uniforms = nullptr;
    return 0;
}

// The legacy LS1D / LS2D kernel (LSKernelCUDA, debri/hostLibrary.cu:3829-4111)
// over all n = nPts^dim points of a parameter grid: (int)(tMax / NT) blocks,
// the transient of (int)(transientTime / h) steps. out[n][nIC].
int leg_ls(int dim, int nPts, double tMax, double NT, double h, double eps, double transientTime, const double* ic,
           int nIC, const double* values, int nValues, const double* ranges, const int* mut, double maxValue,
           double* out) {
    const int blocks = tMax / NT;
    const int S = transientTime / h;
    const long long n = dim == 1 ? (long long)nPts : (long long)nPts * nPts;
    if (3 * nIC + 2 * nIC * nIC + nValues > 4096 || n > 0x7fffffffLL) return 1;
    std::vector<double> rng(ranges, ranges + 2 * dim), x0(ic, ic + nIC), a(values, values + nValues);
    std::vector<int> mv(mut, mut + dim);
    for (long long k = 0; k < n; ++k) {
        as_thread(k);
        legacy_src::legacy::LSKernelCUDA(nPts, (int)n, NT, tMax, blocks, 0, S, dim, rng.data(), h, eps, mv.data(),
                                         x0.data(), nIC, a.data(), nValues, tMax / NT, 1, 0, maxValue, out);
    }
    return 0;
}

}  // extern "C"
