// Timing harness around the reference's own GPU path: its unchanged sources
// (staged and compiled by oracle/build_ref_gpu.py) called through its host
// entry points, exactly as the reference's src/main.cu calls them.
// MEASUREMENT INFRASTRUCTURE ONLY: never shipped, never called by the engine.
//
//   ref_gpu_bif1d <out.csv> [nPts] [tMax]   Bifurcation::bifurcation1D, Lorenz RK4
//                                           (h 0.01, rho in [20, 200], transient 100)
//   ref_gpu_bif2d <out.csv> [nPts] [tMax]   Bifurcation::bifurcation2D, the reference's own
//                                           Chameleon model and its timing sweep's settings
//                                           (src/main.cu:447-505: transient 2000, eps 0.001)
//   ref_gpu_lle2d <out.csv> [nPts] [tMax]   LLE::LLE2D, Rossler RK4 (h 0.01, NT 0.1,
//                                           a in [0.1, 0.4], c in [2, 10], transient 50)
//   ref_gpu_basins <out> [nPts] [tMax]      Basins::basinsOfAttraction_2, Lorenz RK4 rho 24
//                                           (h 0.01, x, y in [-30, 30], z 27, transient 200,
//                                           eps 0.05): its integration and its host-driven
//                                           clustering, one kernel launch per reached point
//
// One small warm-up call (module loading), then the timed call; prints one
// JSON line with the wall time of the timed call. The reference's call
// includes its own host work: device allocation, the per-element zeroing
// copies of the LLE result rows, the copy back and the CSV writing.
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <string>

#if defined(REF_BIF1D) || defined(REF_BIF2D)
#include "bifurcationHOST.h"
#elif defined(REF_BASINS)
#include "basinsHOST.h"
#else
#include "LLEHost.h"
#endif

// The reference's basins loop allocates its previous-state array with device
// new in every thread (Basins/src/basinsCUDA.cu:331) and ends with
// cudaDeviceReset (:811). Each call therefore starts on a fresh context whose
// device heap is raised well above what its threads hold at once (24 B each).
static void prepare_context() {
    cudaFree(nullptr);
#if defined(REF_BASINS)
    cudaDeviceSetLimit(cudaLimitMallocHeapSize, (size_t)256 << 20);
#endif
}

static double run(const std::string& out, int nPts, double tMax) {
    prepare_context();
    const auto t0 = std::chrono::steady_clock::now();
#if defined(REF_BIF1D)
    const double ic[3] = {0.1, 0.1, 0.1}, ranges[2] = {20.0, 200.0}, values[3] = {10.0, 28.0, 8.0 / 3.0};
    const int mut[1] = {1};
    Bifurcation::bifurcation1D(tMax, nPts, 0.01, 3, ic, ranges, mut, 0, 1e4, 100.0, values, 3, 1, out);
#elif defined(REF_BIF2D)
    const double ic[3] = {3.0, 3.0, 0.0}, ranges[4] = {0.0, 5.0, 0.0, 20.0}, values[7] = {0.5, 3, 0, 2, 1, 18, 1};
    const int mut[2] = {3, 5};
    Bifurcation::bifurcation2D(tMax, nPts, 0.01, 3, ic, ranges, mut, 0, 1e4, 2000.0, values, 7, 1, 0.001, out);
#elif defined(REF_BASINS)
    const double ic[3] = {0.0, 0.0, 27.0}, ranges[4] = {-30.0, 30.0, -30.0, 30.0}, values[3] = {10.0, 24.0, 8.0 / 3.0};
    const int mut[2] = {0, 1};
    Basins::basinsOfAttraction_2(tMax, nPts, 0.01, 3, ic, ranges, mut, 0, 1e8, 200.0, values, 3, 1, 0.05, out);
#else
    const double ic[3] = {1.0, 1.0, 1.0}, ranges[4] = {0.1, 0.4, 2.0, 10.0}, values[3] = {0.2, 0.2, 5.7};
    const int mut[2] = {0, 2};
    LLE::LLE2D(tMax, 0.1, nPts, 0.01, 1e-8, ic, 3, ranges, mut, 0, 0.0, 50.0, values, 3, out);
#endif
    cudaDeviceSynchronize();
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

int main(int argc, char** argv) {
    const std::string out = argc > 1 ? argv[1] : "ref_out.csv";
#if defined(REF_BIF1D)
    const int nPts = argc > 2 ? atoi(argv[2]) : 1000;
    const double tMax = argc > 3 ? atof(argv[3]) : 100.0;
#elif defined(REF_BIF2D)
    const int nPts = argc > 2 ? atoi(argv[2]) : 200;
    const double tMax = argc > 3 ? atof(argv[3]) : 400.0;
    // The reference indexes its trajectory buffer with int (idx * amountOfPointsInBlock,
    // bifurcationCUDA.cu:338, 369), and on this GPU's memory one chunk holds every point: a
    // product past 2^31 would write outside the buffer. Refuse such sizes.
    if ((double)nPts * nPts * (tMax / 0.01) >= 2147483647.0) {
        fprintf(stderr, "nPts^2 * tMax/h >= 2^31: the reference's int indexing would overflow\n");
        return 2;
    }
#elif defined(REF_BASINS)
    const int nPts = argc > 2 ? atoi(argv[2]) : 200;
    const double tMax = argc > 3 ? atof(argv[3]) : 50.0;
    // The same int indexing of the trajectory buffer (idx * amountOfPointsInBlock,
    // Basins/src/basinsCUDA.cu:306, 342): refuse sizes whose product passes 2^31.
    if ((double)nPts * nPts * (tMax / 0.01) >= 2147483647.0) {
        fprintf(stderr, "nPts^2 * tMax/h >= 2^31: the reference's int indexing would overflow\n");
        return 2;
    }
#else
    const int nPts = argc > 2 ? atoi(argv[2]) : 1024;
    const double tMax = argc > 3 ? atof(argv[3]) : 500.0;
#endif
    cudaFree(nullptr);     // context
#if defined(REF_BIF2D)
    run(out, 4, 1.0);      // warm-up: module load
#else
    run(out, 16, 1.0);     // warm-up: module load
#endif
    const double s = run(out, nPts, tMax);
    printf("{\"nPts\": %d, \"tMax\": %g, \"seconds\": %.6f}\n", nPts, tMax, s);
    return 0;
}
