// Order keys of doubles and their warp reductions, shared by the basins
// kernels (the clustering features' minima and maxima) and the clustering.
#pragma once

#include <cuda_runtime.h>

namespace chaos {

// Order-preserving map of a double to an unsigned 64-bit key, for atomicMin /
// atomicMax, and back.
__device__ __forceinline__ unsigned long long okey(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double unkey(unsigned long long k) {
    const unsigned long long b = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
    return __longlong_as_double((long long)b);
}

// 64-bit minimum / maximum over the lanes of grp (each of them calls it), as
// two 32-bit warp reductions: the high words, then the low words of the
// lanes that hold the extreme high word.
__device__ __forceinline__ unsigned long long group_min64(unsigned grp, unsigned long long v) {
    const unsigned hi = (unsigned)(v >> 32);
    const unsigned mh = __reduce_min_sync(grp, hi);
    const unsigned ml = __reduce_min_sync(grp, hi == mh ? (unsigned)v : 0xffffffffu);
    return ((unsigned long long)mh << 32) | ml;
}
__device__ __forceinline__ unsigned long long group_max64(unsigned grp, unsigned long long v) {
    const unsigned hi = (unsigned)(v >> 32);
    const unsigned mh = __reduce_max_sync(grp, hi);
    const unsigned ml = __reduce_max_sync(grp, hi == mh ? (unsigned)v : 0u);
    return ((unsigned long long)mh << 32) | ml;
}

// Replicas of the six feature keys (minima of the three features, then their
// maxima), each written by the blocks with blockIdx.x % kKeyReplicas equal to
// its index: mm[k * kKeyReplicas + r].
constexpr int kKeyReplicas = 64;

// The clustering features of the basin points with flag != 0 -- amplitude
// (mean peak value, or the last recorded sample for a point without peaks),
// kept peak count, mean interval (0 without peaks) -- folded into running
// minimum / maximum order keys, then across the active lanes of the warp and
// into the block's replica with one atomic per key, so that the clustering
// reads the normalisation bounds instead of making a pass over the map.
struct FeatureKeys {
    unsigned long long lo[3], hi[3];
    __device__ __forceinline__ FeatureKeys() {
        for (int d = 0; d < 3; ++d) {
            lo[d] = ~0ull;
            hi[d] = 0ull;
        }
    }
    __device__ __forceinline__ void add(int flag, int count, double avgPeak, double avgInterval, double last) {
        if (flag == 0) return;
        const double f[3] = {count > 0 ? avgPeak : last, (double)count, count > 0 ? avgInterval : 0.0};
        for (int d = 0; d < 3; ++d) {
            const unsigned long long k = okey(f[d]);
            lo[d] = k < lo[d] ? k : lo[d];
            hi[d] = k > hi[d] ? k : hi[d];
        }
    }
    // called by every active lane
    __device__ __forceinline__ void flush(unsigned long long* mm) const {
        const unsigned m = __activemask();
        const int lane = threadIdx.x & 31;
        const int r = (int)(blockIdx.x % kKeyReplicas);
        for (int d = 0; d < 3; ++d) {
            const unsigned long long l = group_min64(m, lo[d]);
            const unsigned long long h = group_max64(m, hi[d]);
            if (lane == __ffs(m) - 1) {
                if (l != ~0ull) atomicMin(&mm[d * kKeyReplicas + r], l);
                if (h != 0ull) atomicMax(&mm[(3 + d) * kKeyReplicas + r], h);
            }
        }
    }
};

}  // namespace chaos
