// Normalised feature matrix of the basins map for the textbook DBSCAN mode:
// per point (amplitude, kept peak count, mean interval) -- amplitude is the
// mean peak value, or the last recorded sample for a point without peaks --
// min-max scaled to [0, 1] per feature over the points with flag != 0.
// Two passes over n points: the min / max keys, then the scaled features.
#include <cuda_runtime.h>

#include <cfloat>

#include "launch.h"

namespace chaos {
namespace {

constexpr int kTPB = 256;

__device__ __forceinline__ void raw_features(const BasinsOut& O, long long i, double* f) {
    const int c = O.counts[i];
    f[0] = c > 0 ? O.avgPeaks[i] : O.last[i];
    f[1] = (double)c;
    f[2] = c > 0 ? O.avgIntervals[i] : 0.0;
}

// order-preserving map of a double to an unsigned 64-bit key (for atomicMin/Max)
__device__ __forceinline__ unsigned long long okey(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double ounkey(unsigned long long k) {
    const unsigned long long b = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
    return __longlong_as_double((long long)b);
}

__global__ void minmax_init_kernel(unsigned long long* mm) {
    if (threadIdx.x < 3) mm[threadIdx.x] = ~0ull;        // min keys
    else if (threadIdx.x < 6) mm[threadIdx.x] = 0ull;    // max keys
}

// min and max keys per feature over the points with flag != 0: reduced across
// the warp with shuffles, then one shared-memory atomic per warp and feature
// and one global atomic per block and feature.
__global__ void minmax_kernel(BasinsOut O, long long n, unsigned long long* mm, int* mask) {
    __shared__ unsigned long long smin[3], smax[3];
    if (threadIdx.x < 3) { smin[threadIdx.x] = ~0ull; smax[threadIdx.x] = 0ull; }
    __syncthreads();
    unsigned long long lo[3] = {~0ull, ~0ull, ~0ull}, hi[3] = {0ull, 0ull, 0ull};
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int in = O.flags[i] != 0;
        mask[i] = in;
        if (!in) continue;
        double f[3];
        raw_features(O, i, f);
        for (int d = 0; d < 3; ++d) {
            const unsigned long long k = okey(f[d]);
            lo[d] = lo[d] < k ? lo[d] : k;
            hi[d] = hi[d] > k ? hi[d] : k;
        }
    }
    for (int d = 0; d < 3; ++d) {
        for (int o = 16; o > 0; o >>= 1) {
            const unsigned long long a = __shfl_xor_sync(0xffffffffu, lo[d], o);
            const unsigned long long b = __shfl_xor_sync(0xffffffffu, hi[d], o);
            lo[d] = lo[d] < a ? lo[d] : a;
            hi[d] = hi[d] > b ? hi[d] : b;
        }
        if ((threadIdx.x & 31) == 0) {
            atomicMin(&smin[d], lo[d]);
            atomicMax(&smax[d], hi[d]);
        }
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        atomicMin(&mm[threadIdx.x], smin[threadIdx.x]);
        atomicMax(&mm[3 + threadIdx.x], smax[threadIdx.x]);
    }
}

// v = (f - lo) * (1 / (hi - lo)) per feature: the three reciprocals once per
// block (a divide per point and feature would keep the FP64 pipe busy for
// most of the kernel). Written as the row-major n x 3 matrix F and / or as
// three columns (the clustering's layout) -- whichever pointers are set.
__global__ void normalise_kernel(BasinsOut O, long long n, const unsigned long long* mm, double* F, double* c0,
                                 double* c1, double* c2) {
    __shared__ double slo[3], sinv[3];
    __shared__ int sok[3];
    if (threadIdx.x < 3) {
        const int d = threadIdx.x;
        const bool any = mm[d] != ~0ull;
        const double lo = any ? ounkey(mm[d]) : 0.0, hi = any ? ounkey(mm[3 + d]) : 0.0;
        slo[d] = lo;
        sok[d] = any && hi > lo;
        sinv[d] = sok[d] ? 1.0 / (hi - lo) : 0.0;
    }
    __syncthreads();
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double f[3];
    raw_features(O, i, f);
    const bool in = O.flags[i] != 0;
    double v[3];
    for (int d = 0; d < 3; ++d) v[d] = in && sok[d] ? (f[d] - slo[d]) * sinv[d] : 0.0;
    if (F)
        for (int d = 0; d < 3; ++d) F[i * 3 + d] = v[d];
    if (c0) {
        c0[i] = v[0];
        c1[i] = v[1];
        c2[i] = v[2];
    }
}

}  // namespace

cudaError_t launch_basin_feature_matrix(const BasinsOut& O, long long n, double* minmax, double* features,
                                        double* const* columns, int* mask, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    unsigned long long* mm = reinterpret_cast<unsigned long long*>(minmax);
    minmax_init_kernel<<<1, 32, 0, st>>>(mm);
    note_launch();
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long need = (n + kTPB - 1) / kTPB;
    const unsigned grid = (unsigned)(need < (long long)sms * 8 ? need : (long long)sms * 8);
    minmax_kernel<<<grid, kTPB, 0, st>>>(O, n, mm, mask);
    note_launch();
    normalise_kernel<<<(unsigned)need, kTPB, 0, st>>>(O, n, mm, features, columns ? columns[0] : nullptr,
                                                      columns ? columns[1] : nullptr, columns ? columns[2] : nullptr);
    note_launch();
    return cudaGetLastError();
}

}  // namespace chaos
