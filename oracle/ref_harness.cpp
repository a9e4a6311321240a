// Host harness around the reference's own per-thread CUDA code.
//
// TEST INFRASTRUCTURE ONLY (never shipped, never called by the engine).
// oracle/build_ref.py extracts, unchanged, the reference functions listed
// below from the reference sources into oracle/_ref/*.inc and compiles them
// together with this file and a chosen systems.cuh plug-in into
// oracle/_ref/libref_<system>.so. Each "kernel launch" of the reference is
// replayed here as a loop over thread indices, one thread after another.
//   Bifurcation/src/bifurcationCUDA.cu: calculateTransTimeCUDA, calculateDiscreteModelCUDA,
//     peakFinderCUDA, dbscanCUDA, getValueByIdx, loopCalculateDiscreteModel_int,
//     peakFinder, dbscan, distance
//   Basins/src/basinsCUDA.cu: getValueByIdx, calculateDiscreteModel, calculateTransTimeCUDA,
//     calculateDiscreteModelCUDA, loopCalculateDiscreteModel_int, peakFinder,
//     avgPeakFinderCUDA, CUDA_dbscan_search_clear_points_kernel,
//     CUDA_dbscan_search_fixed_points_kernel, CUDA_dbscan_kernel
//   LLE/src/LLECUDA.cu: loopCalculateDiscreteModel, calculateDiscreteModel, calculateSystem, linspace
// The host drivers (bifurcation1D/2D, LLE2D, basinsOfAttraction_2, CUDA_dbscan)
// allocate device memory and launch kernels, so they are re-sequenced here
// for a single chunk. The LLE twin starts at x + eps*e_x instead of the
// reference's cuRAND draw (calculateTransTime, which needs cuRAND, is not built).
#include "cuda_runtime.h"

#include <bifurcationCUDA.cuh>
#include <basinsCUDA.cuh>
#include <LLECUDA.cuh>
#include <systems.cuh>

#include <omp.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <vector>

thread_local dim3 threadIdx, blockIdx, blockDim;

#include "ref_bif.inc"
#include "ref_basins.inc"
#include "ref_lle.inc"

static void as_thread(long long idx) {
    threadIdx = dim3{0, 0, 0};
    blockDim = dim3{1, 1, 1};
    blockIdx = dim3{(unsigned)idx, 0, 0};
}

extern "C" {

int refh_size_x() { return SIZE_X; }
int refh_size_a() { return SIZE_A; }

void refh_steps(double* x, const double* a, double h, int n) {
    for (int i = 0; i < n; ++i) CALC_DISCRETE_MODEL(x, a, h);
}

// Bifurcation_constants::peakFinder on one series (in place, as the reference).
int refh_peak_finder(double* data, int len, double* outPeaks, double* timeOfPeaks, double h) {
    return Bifurcation_constants::peakFinder(data, 0, len, outPeaks, timeOfPeaks, h);
}

// Bifurcation_constants::dbscan on one point: data holds the peaks (zeroed by
// the call), intervals the intervals, helpful is scratch of sizeOfBlock doubles.
int refh_point_dbscan(double* data, double* intervals, double* helpful, int amountOfPeaks, int sizeOfBlock,
                      double eps) {
    return Bifurcation_constants::dbscan(data, intervals, helpful, 0, amountOfPeaks, sizeOfBlock, 0, eps, nullptr);
}

// bifurcation1D (dim 1) / bifurcation2D (dim 2) for one chunk of all points:
// fills amountOfPeaks (N), data and intervals (N*B, after peakFinderCUDA) and,
// for dim 2, dbscanOut (N) using helpful (N*B) as the reference's scratch.
int refh_bifurcation(int dim, double tMax, int nPts, double h, int nIC, const double* ic, const double* ranges,
                     const int* mut, int wv, double maxValue, double transientTime, const double* values,
                     int nValues, int preScaller, double eps, int* amountOfPeaks, double* data, double* intervals,
                     int* dbscanOut, double* helpful) {
    using namespace Bifurcation_constants;
    int B = tMax / h / preScaller;
    int S = transientTime / h;
    long long N = dim == 1 ? (long long)nPts : (long long)nPts * nPts;
    d_tMax = tMax; d_nPts = nPts; d_h = h; d_amountOfInitialConditions = nIC; d_writableVar = wv;
    d_maxValue = maxValue; d_transientTime = transientTime; d_amountOfValues = nValues;
    d_preScaller = preScaller; d_eps = eps; d_amountOfPointsInBlock = B; d_originalNPtsLimiter = (int)N;
    d_amountOfPointsForSkip = S; d_dimension = dim; d_nPtsLimiter = (int)N; d_amountOfCalculatedPoints = 0;
    std::vector<double> semi((size_t)N * (nIC + nValues));
    for (long long i = 0; i < N; ++i) {
        as_thread(i);
        calculateTransTimeCUDA((double*)ranges, (int*)mut, (double*)ic, values, semi.data(), amountOfPeaks);
    }
    for (long long i = 0; i < N; ++i) {
        as_thread(i);
        calculateDiscreteModelCUDA((double*)ranges, (int*)mut, (double*)ic, values, data, semi.data(), amountOfPeaks);
    }
    for (long long i = 0; i < N; ++i) {
        as_thread(i);
        peakFinderCUDA(data, amountOfPeaks, data, intervals, h * (double)preScaller);
    }
    if (dim == 2 && dbscanOut) {
        std::vector<double> d2(data, data + (size_t)N * B);
        for (long long i = 0; i < N; ++i) {
            as_thread(i);
            dbscanCUDA(d2.data(), B, (int)N, amountOfPeaks, intervals, helpful, eps, dbscanOut);
        }
    }
    return B;
}

// basinsOfAttraction_2 up to (not including) CUDA_dbscan, one chunk:
// helpful = flags, avgPeaks / avgIntervals = features, data = N*B scratch.
int refh_basins(double tMax, int nPts, double h, int nIC, const double* ic, const double* ranges, const int* mut,
                int wv, double maxValue, double transientTime, const double* values, int nValues, int preScaller,
                int* helpful, double* avgPeaks, double* avgIntervals, double* data) {
    using namespace basinsGPU;
    int B = tMax / h / preScaller;
    int S = transientTime / h;
    long long N = (long long)nPts * nPts;
    d_h = h; d_tMax = tMax; d_nPts = nPts; d_amountOfIterations = 1; d_amountOfInitialConditions = nIC;
    d_amountOfValues = nValues; d_amountOfPointsInBlock = B; d_amountOfPointsForSkip = S; d_writableVar = wv;
    d_maxValue = maxValue; d_preScaller = preScaller; d_dimension = 2; d_nPtsLimiter = (int)N;
    d_amountOfCalculatedPoints = 0;
    std::vector<double> semi((size_t)N * (nIC + nValues));
    std::vector<double> intervals((size_t)N * B);
    for (long long i = 0; i < N; ++i) {
        as_thread(i);
        calculateTransTimeCUDA((double*)ranges, (int*)mut, (double*)ic, values, semi.data(), helpful);
    }
    for (long long i = 0; i < N; ++i) {
        as_thread(i);
        calculateDiscreteModelCUDA((double*)ranges, (int*)mut, (double*)ic, values, data, semi.data(), helpful);
    }
    for (long long i = 0; i < N; ++i) {
        as_thread(i);
        avgPeakFinderCUDA(data, B, (int)N, avgPeaks, avgIntervals, data, intervals.data(), helpful, h * preScaller);
    }
    return B;
}

// CUDA_dbscan's host loop (Basins/src/basinsCUDA.cu:35-179) with every launch
// replayed thread by thread. labels must start at 0.
void refh_basins_dbscan(double* avgPeaks, double* avgIntervals, int* labels, int* helpful, int n, double eps) {
    using namespace basinsGPU;
    int pos = 0, neg = 0, result = 0;
    int amountOfNeighbors = 0;
    std::vector<int> neighbors(n > 0 ? n : 1, 0);
    for (int it = 0; it < n; ++it) {
        int clearIdx = -1;
        for (int i = 0; i < n; ++i) {
            as_thread(i);
            CUDA_dbscan_search_fixed_points_kernel(avgPeaks, avgIntervals, helpful, labels, n, &clearIdx);
        }
        if (clearIdx == -1) {
            for (int i = 0; i < n; ++i) {
                as_thread(i);
                CUDA_dbscan_search_clear_points_kernel(avgPeaks, avgIntervals, helpful, labels, n, &clearIdx);
            }
            ++pos;
            result = pos;
            if (clearIdx == -1) break;
        } else {
            --neg;
            result = neg;
        }
        amountOfNeighbors = 0;
        std::fill(neighbors.begin(), neighbors.end(), 0);
        for (int i = 0; i < n; ++i) {
            as_thread(i);
            CUDA_dbscan_kernel(avgPeaks, avgIntervals, labels, n, eps, result, &amountOfNeighbors, neighbors.data(),
                               clearIdx, helpful);
        }
        for (int k = 0; k < amountOfNeighbors; ++k) {
            int cur = neighbors[k];
            for (int i = 0; i < n; ++i) {
                as_thread(i);
                CUDA_dbscan_kernel(avgPeaks, avgIntervals, labels, n, eps, result, &amountOfNeighbors,
                                   neighbors.data(), cur, helpful);
            }
        }
    }
}

// LLE2D for one segment: the transient by the reference's
// loopCalculateDiscreteModel, the twin at x + eps*e_x, then calculateSystem
// for every (a, b); out[b*nPts + a] (the CSV's transposed layout).
void refh_lle(double tMax, double NT, int nPts, double h, double eps, int nIC, const double* ic,
              const double* ranges, const int* mut, double transientTime, const double* values, int nValues,
              double* out) {
    using namespace LLE_constants;
    int ntp = static_cast<int>(NT / h);
    int trans = static_cast<int>(transientTime / h);
    int all = static_cast<int>(tMax / h);
    int calcBlocks = static_cast<int>(all / ntp) + 1;
    double* linA = linspace(ranges[0], ranges[1], nPts);
    double* linB = linspace(ranges[2], ranges[3], nPts);
    d_idxParamA = mut[0]; d_idxParamB = mut[1]; d_size_linspace_A = nPts; d_size_linspace_B = nPts;
    d_h = h; d_transTime = transientTime; d_tMax = tMax; d_Nt_steps = ntp; d_paramsSize = nValues;
    d_XSize = nIC; d_amountOfNTPoints = ntp; d_amountOfTransPoints = trans; d_amountOfAllpoints = all;
    d_amountOfCalcBlocks = calcBlocks; d_eps = eps;
    const int per = 2 * nIC + nValues;
    std::vector<double> semi((size_t)nPts * nPts * per);
    std::vector<double*> rows(nPts);
    std::vector<double> store((size_t)nPts * nPts, 0.0);
    for (int a = 0; a < nPts; ++a) rows[a] = store.data() + (size_t)a * nPts;
    for (int a = 0; a < nPts; ++a)
        for (int b = 0; b < nPts; ++b) {
            double* r = semi.data() + ((size_t)a * nPts + b) * per;
            for (int i = 0; i < nIC; ++i) r[i] = ic[i];
            for (int i = 0; i < nValues; ++i) r[nIC + i] = values[i];
            r[nIC + mut[0]] = linA[a];
            r[nIC + mut[1]] = linB[b];
            loopCalculateDiscreteModel(r, r + nIC, trans);
            for (int i = 0; i < nIC; ++i) r[nIC + nValues + i] = r[i];
            r[nIC + nValues] = r[0] + eps;
        }
    for (int a = 0; a < nPts; ++a)
        for (int b = 0; b < nPts; ++b) {
            threadIdx = dim3{0, 0, 0};
            blockDim = dim3{1, 1, 1};
            blockIdx = dim3{(unsigned)a, (unsigned)b, 0};
            calculateSystem(nullptr, nullptr, linA, linB, semi.data(), rows.data());
        }
    for (int a = 0; a < nPts; ++a)
        for (int b = 0; b < nPts; ++b) out[(size_t)b * nPts + a] = rows[a][b];
    delete[] linA;
    delete[] linB;
}

// bifurcation1D / bifurcation2D points [pBegin, pEnd) through the reference's
// own chunking (d_amountOfCalculatedPoints, d_nPtsLimiter), chunks of up to
// 4096 points, the replayed threads of a chunk spread over nthreads host
// threads (OpenMP; launch indices and shared memory are thread-local): the
// transient, recorded and peak-finder kernels of each point in turn.
// counts[p - pBegin] = the point's amountOfPeaks after peakFinderCUDA.
void refh_bifurcation_range(int dim, double tMax, int nPts, double h, int nIC, const double* ic,
                            const double* ranges, const int* mut, int wv, double maxValue, double transientTime,
                            const double* values, int nValues, int preScaller, long long pBegin, long long pEnd,
                            int* counts, int nthreads) {
    using namespace Bifurcation_constants;
    const int B = tMax / h / preScaller;
    const int S = transientTime / h;
    const long long N = dim == 1 ? (long long)nPts : (long long)nPts * nPts;
    const long long chunk = 4096;
    d_tMax = tMax; d_nPts = nPts; d_h = h; d_amountOfInitialConditions = nIC; d_writableVar = wv;
    d_maxValue = maxValue; d_transientTime = transientTime; d_amountOfValues = nValues;
    d_preScaller = preScaller; d_amountOfPointsInBlock = B; d_originalNPtsLimiter = (int)std::min(chunk, N);
    d_amountOfPointsForSkip = S; d_dimension = dim;
    std::unique_ptr<double[]> data(new double[(size_t)chunk * B]), intervals(new double[(size_t)chunk * B]);
    std::unique_ptr<double[]> semi(new double[(size_t)chunk * (nIC + nValues)]);
    std::unique_ptr<int[]> amount(new int[chunk]);
    if (nthreads > 0) omp_set_num_threads(nthreads);
    for (long long c0 = pBegin; c0 < pEnd; c0 += chunk) {
        const long long cnt = std::min(chunk, pEnd - c0);
        d_nPtsLimiter = (int)cnt;
        d_amountOfCalculatedPoints = (int)c0;
#pragma omp parallel for schedule(dynamic, 4)
        for (long long i = 0; i < cnt; ++i) {
            as_thread(i);
            calculateTransTimeCUDA((double*)ranges, (int*)mut, (double*)ic, values, semi.get(), amount.get());
            calculateDiscreteModelCUDA((double*)ranges, (int*)mut, (double*)ic, values, data.get(), semi.get(),
                                       amount.get());
            peakFinderCUDA(data.get(), amount.get(), data.get(), intervals.get(), h * (double)preScaller);
            counts[c0 - pBegin + i] = amount[i];
        }
    }
}

// basinsOfAttraction_2's per-point kernels for points [pBegin, pEnd) of the
// nPts^2 grid, chunked and replayed as refh_bifurcation_range: flags and
// features into helpful / avgPeaks / avgIntervals[p - pBegin].
void refh_basins_range(double tMax, int nPts, double h, int nIC, const double* ic, const double* ranges,
                       const int* mut, int wv, double maxValue, double transientTime, const double* values,
                       int nValues, int preScaller, long long pBegin, long long pEnd, int* helpful,
                       double* avgPeaks, double* avgIntervals, int nthreads) {
    using namespace basinsGPU;
    const int B = tMax / h / preScaller;
    const int S = transientTime / h;
    const long long chunk = 4096;
    d_h = h; d_tMax = tMax; d_nPts = nPts; d_amountOfIterations = 1; d_amountOfInitialConditions = nIC;
    d_amountOfValues = nValues; d_amountOfPointsInBlock = B; d_amountOfPointsForSkip = S; d_writableVar = wv;
    d_maxValue = maxValue; d_preScaller = preScaller; d_dimension = 2;
    std::unique_ptr<double[]> data(new double[(size_t)chunk * B]), intervals(new double[(size_t)chunk * B]);
    std::unique_ptr<double[]> semi(new double[(size_t)chunk * (nIC + nValues)]);
    if (nthreads > 0) omp_set_num_threads(nthreads);
    for (long long c0 = pBegin; c0 < pEnd; c0 += chunk) {
        const long long cnt = std::min(chunk, pEnd - c0);
        d_nPtsLimiter = (int)cnt;
        d_amountOfCalculatedPoints = (int)c0;
        int* hf = helpful + (c0 - pBegin);
#pragma omp parallel for schedule(dynamic, 4)
        for (long long i = 0; i < cnt; ++i) {
            as_thread(i);
            calculateTransTimeCUDA((double*)ranges, (int*)mut, (double*)ic, values, semi.get(), hf);
            calculateDiscreteModelCUDA((double*)ranges, (int*)mut, (double*)ic, values, data.get(), semi.get(), hf);
            avgPeakFinderCUDA(data.get(), B, (int)cnt, avgPeaks + (c0 - pBegin), avgIntervals + (c0 - pBegin),
                              data.get(), intervals.get(), hf, h * preScaller);
        }
    }
}

// The same LLE2D points [pBegin, pEnd) (p = b*nPts + a, the CSV layout) with
// the replayed threads spread over nthreads host threads (OpenMP; the launch
// indices and the shared-memory array are thread-local): the reference's own
// per-thread code as a CPU baseline. out[p - pBegin].
void refh_lle_range(double tMax, double NT, int nPts, double h, double eps, int nIC, const double* ic,
                    const double* ranges, const int* mut, double transientTime, const double* values, int nValues,
                    long long pBegin, long long pEnd, double* out, int nthreads) {
    using namespace LLE_constants;
    int ntp = static_cast<int>(NT / h);
    int trans = static_cast<int>(transientTime / h);
    int all = static_cast<int>(tMax / h);
    int calcBlocks = static_cast<int>(all / ntp) + 1;
    double* linA = linspace(ranges[0], ranges[1], nPts);
    double* linB = linspace(ranges[2], ranges[3], nPts);
    d_idxParamA = mut[0]; d_idxParamB = mut[1]; d_size_linspace_A = nPts; d_size_linspace_B = nPts;
    d_h = h; d_transTime = transientTime; d_tMax = tMax; d_Nt_steps = ntp; d_paramsSize = nValues;
    d_XSize = nIC; d_amountOfNTPoints = ntp; d_amountOfTransPoints = trans; d_amountOfAllpoints = all;
    d_amountOfCalcBlocks = calcBlocks; d_eps = eps;
    const int per = 2 * nIC + nValues;
    // whole-map index space, touched only at the sampled points (no zero fill)
    std::unique_ptr<double[]> semi(new double[(size_t)nPts * nPts * per]);
    std::unique_ptr<double[]> store(new double[(size_t)nPts * nPts]);
    std::vector<double*> rows(nPts);
    for (int a = 0; a < nPts; ++a) rows[a] = store.get() + (size_t)a * nPts;
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 4)
    for (long long p = pBegin; p < pEnd; ++p) {
        const int a = (int)(p % nPts), b = (int)(p / nPts);
        rows[a][b] = 0.0;
        double* r = semi.get() + ((size_t)a * nPts + b) * per;
        for (int i = 0; i < nIC; ++i) r[i] = ic[i];
        for (int i = 0; i < nValues; ++i) r[nIC + i] = values[i];
        r[nIC + mut[0]] = linA[a];
        r[nIC + mut[1]] = linB[b];
        loopCalculateDiscreteModel(r, r + nIC, trans);
        for (int i = 0; i < nIC; ++i) r[nIC + nValues + i] = r[i];
        r[nIC + nValues] = r[0] + eps;
        threadIdx = dim3{0, 0, 0};
        blockDim = dim3{1, 1, 1};
        blockIdx = dim3{(unsigned)a, (unsigned)b, 0};
        calculateSystem(nullptr, nullptr, linA, linB, semi.get(), rows.data());
        out[p - pBegin] = rows[a][b];
    }
    delete[] linA;
    delete[] linB;
}

}  // extern "C"
