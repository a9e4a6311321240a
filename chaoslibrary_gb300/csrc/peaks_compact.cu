// Dense peak lists of a 1-D bifurcation sweep (chaos_compact_peaks, declared
// in include/chaos_gb300.h). The sweep keeps up to peakCapacity peaks per
// point in fixed rows; most rows are mostly empty (a Lorenz sweep keeps ~180
// of B/2 = 5,000 rows). This pass turns the rows into one dense run per point:
// the kept counts clamped to the rows (fixed points and diverged points keep
// none), their exclusive prefix sum (block scans with warp shuffles), then a
// warp per point copying its run with coalesced loads and stores. The output
// is the reference CSV's row order (point by point, peaks in time order).
#include <cuda_runtime.h>

#include <algorithm>

#include "../../include/chaos_gb300.h"
#include "capi_internal.h"
#include "dbscan.h"
#include "launch.h"

namespace chaos {
namespace {

constexpr int kTPB = 256;

inline unsigned blocks_of(long long n, int tpb = kTPB) { return (unsigned)((n + tpb - 1) / tpb); }

// kept[k] = clamp(counts[k], 0, cap), with kept[n] = 0 so that the scan of
// n + 1 entries leaves the total in offsets[n]
__global__ void kept_kernel(const int* counts, long long n, int cap, long long* kept) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) kept[k] = (long long)min(max(counts[k], 0), cap);
    else if (k == n) kept[k] = 0;
}

// warp per point: lane j of the warp moves peaks j, j + 32, ... of the run
__global__ void compact_kernel(const long long* offsets, long long n, int cap, const double* peaks,
                               const double* intervals, long long first, long long count, double* densePeaks,
                               double* denseIntervals, int* densePoint) {
    const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= n) return;
    const long long off = offsets[w], m = offsets[w + 1] - off;
    for (long long j = lane; j < m; j += 32) {
        const long long d = off + j - first;  // position in this slice of the dense list
        if (d < 0 || d >= count) continue;
        const long long src = w * (long long)cap + j;
        if (densePeaks) densePeaks[d] = peaks[src];
        if (denseIntervals) denseIntervals[d] = intervals[src];
        if (densePoint) densePoint[d] = (int)w;
    }
}

}  // namespace
}  // namespace chaos

using namespace chaos;

extern "C" int chaos_compact_peaks(const chaos_exec* ex, const int* counts, const double* peaks,
                                   const double* intervals, long long n, int peakCapacity, long long* offsets,
                                   double* densePeaks, double* denseIntervals, int* densePoint,
                                   long long denseCapacity, long long* total) {
    if (!counts || !total) return set_error(CHAOS_E_ARGS, "counts and total are required");
    if (n < 0 || peakCapacity < 1) return set_error(CHAOS_E_ARGS, "need n >= 0 and peakCapacity >= 1");
    const bool dense = densePeaks || denseIntervals || densePoint;
    if ((densePeaks && !peaks) || (denseIntervals && !intervals))
        return set_error(CHAOS_E_ARGS, "dense peaks / intervals need the peak / interval rows");
    if (dense && denseCapacity < 0) return set_error(CHAOS_E_ARGS, "denseCapacity must be >= 0");
    if (n > 0 && (double)n * peakCapacity > 9.0e18) return set_error(CHAOS_E_ARGS, "n * peakCapacity too large");
    Call c;
    int rc = c.begin(ex);
    if (rc) return rc;
    const size_t rowBytes = (size_t)n * peakCapacity * sizeof(double);
    const int* dCounts = (const int*)c.input(counts, (size_t)n * sizeof(int));
    long long* dOff = offsets ? (long long*)c.output(offsets, (size_t)(n + 1) * sizeof(long long))
                              : (long long*)c.alloc((size_t)(n + 1) * sizeof(long long));
    if (c.failed) return c.finish(CHAOS_E_NOMEM);
    kept_kernel<<<blocks_of(n + 1), kTPB, 0, c.stream>>>(dCounts, n, peakCapacity, dOff);
    note_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return c.finish(cuda_error(e, "kept counts"));
    long long tot = 0;
    if ((rc = exclusive_scan64(c, dOff, dOff, n + 1, &tot))) return c.finish(rc);
    *total = tot;
    if (dense) {
        const long long count = std::min(tot, denseCapacity);
        const double* dPeaks = densePeaks ? (const double*)c.input(peaks, rowBytes) : nullptr;
        const double* dIntervals = denseIntervals ? (const double*)c.input(intervals, rowBytes) : nullptr;
        double* dP = densePeaks ? (double*)c.output(densePeaks, (size_t)count * sizeof(double)) : nullptr;
        double* dI = denseIntervals ? (double*)c.output(denseIntervals, (size_t)count * sizeof(double)) : nullptr;
        int* dW = densePoint ? (int*)c.output(densePoint, (size_t)count * sizeof(int)) : nullptr;
        if (c.failed) return c.finish(CHAOS_E_NOMEM);
        if (n > 0 && count > 0) {
            compact_kernel<<<blocks_of(n * 32), kTPB, 0, c.stream>>>(dOff, n, peakCapacity, dPeaks, dIntervals, 0,
                                                                      count, dP, dI, dW);
            note_launch();
            if ((e = cudaGetLastError()) != cudaSuccess) return c.finish(cuda_error(e, "peak compaction"));
        }
        if (!rc) rc = c.to_host(densePeaks, dP, (size_t)count * sizeof(double));
        if (!rc) rc = c.to_host(denseIntervals, dI, (size_t)count * sizeof(double));
        if (!rc) rc = c.to_host(densePoint, dW, (size_t)count * sizeof(int));
    }
    if (!rc) rc = c.to_host(offsets, dOff, (size_t)(n + 1) * sizeof(long long));
    if (!rc && dense && tot > denseCapacity)
        rc = set_error(CHAOS_E_ARGS, "denseCapacity %lld < %lld kept peaks (the first denseCapacity are written)",
                       denseCapacity, tot);
    return c.finish(rc);
}
