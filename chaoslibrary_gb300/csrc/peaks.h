// The streaming peak detector of the sweeps (the reference's peakFinder,
// bifurcationCUDA.cu:469-514, one sample at a time) and its sample tests.
// Host and device: the kernels include it through engine.cuh, and the CPU
// tests compile it with g++ against the golden peak lists and the oracle.
#pragma once

#include <stdint.h>
#include <string.h>

#include "systems.h"

namespace chaos {

// The bits of a double as a signed integer.
CHAOS_HD long long bits_of(double v) {
#if defined(__CUDA_ARCH__)
    return __double_as_longlong(v);
#else
    long long b;
    memcpy(&b, &v, sizeof b);
    return b;
#endif
}

// Comparisons of a new sample v with the previous one p1 through the one
// difference d = RN(v - p1): RN(p1 - v) = -d exactly, so "p1 < v" is d > 0,
// "p1 - v > 1e-13" is d < -1e-13 and "v - p1 > 1e-13" is d > 1e-13, all false
// for NaN as the direct comparisons are; "p1 >= v" is d <= 0, or v == p1 for
// equal infinities (where d is NaN). For double they run on the integer pipe:
// the bits of a double order like signed integers on either side of zero.
struct DiffTest {
    bool up, ge, above, below;  // p1 < v, p1 >= v, v - p1 > 1e-13, p1 - v > 1e-13
};
CHAOS_HD DiffTest diff_test(double v, double p1) {
    const long long b = bits_of(v - p1);
    const unsigned long long a = (unsigned long long)b & 0x7fffffffffffffffull;
    constexpr unsigned long long kEps = 0x3d3c25c268497682ull;  // bits of 1e-13
    constexpr unsigned long long kInf = 0x7ff0000000000000ull;
    if (a <= kInf) return {b > 0, b <= 0, b > (long long)kEps, b < 0 && a > kEps};
    const long long vb = bits_of(v);
    const bool eqInf = vb == bits_of(p1) && ((unsigned long long)vb & 0x7fffffffffffffffull) == kInf;
    return {false, eqInf, false, false};
}
CHAOS_HD DiffTest diff_test(float v, float p1) {
    const float d = v - p1;
    return {d > 0.f, p1 >= v, d > 1e-13f, d < -1e-13f};
}

// Streaming form of the reference peakFinder (bifurcationCUDA.cu:469-514).
// Samples arrive one at a time; a candidate i is judged when d[i+1] arrives
// and a plateau walk advances one sample per arrival, with exactly the
// reference's rules: rise > 1e-13 and d[i] >= d[i+1] opens a plateau; a
// sample above ends it without a peak; a drop > 1e-13 ends it with a peak of
// value d[j] at time trunc((i+j)/2); after either end the scan resumes at
// j+2. The first detected peak is dropped and every later one is reported
// with the interval to its predecessor, (t_k - t_{k-1}) * h.
//
// One subtraction per sample (diff_test): the next sample's rise test
// "d[k] - d[k-1] > 1e-13" is taken when d[k] arrives and kept as a flag.
template <class T, bool Sel = false> struct PeakStream {
    T p1;          // d[k-1]
    bool rise;     // d[k-1] - d[k-2] > 1e-13
    bool plateau;  // a plateau is open: it started at candidate i0 and runs to j = k-1
    int k;         // index of the next sample
    int nc;        // candidate k-1 is judged when k > nc (outside a plateau)
    int i0;        // plateau: index of the candidate that opened it
    int n;         // peaks detected so far (the dropped first one included)
    int tprev;     // time index of the previous detected peak

    CHAOS_HD void init() {
        k = 0; nc = 1; plateau = false; i0 = 0; n = 0; tprev = 0; p1 = T(0); rise = false;
    }

    // Pushes d[k] = v; returns true and sets (val, t) when a peak was detected.
    // Outside a plateau, candidate k-1 (d[k-2], d[k-1] and d[k] known) is
    // judged when k > nc; the first judged candidate is 1 (nc = 1), and after
    // a plateau ends at j = k-1 the scan resumes at candidate j+2 = k+1
    // (nc = k+1). A judged candidate that is no peak leaves nc as it is, so the
    // common sample costs one compare of k with nc besides the sample tests.
    //
    // Sel: the same transitions as selects, without branches (a candidate
    // that opens a plateau and a running plateau are one state; "up" and
    // "below" exclude each other, "ge" excludes "up"). A warp whose threads
    // each run one latency-bound trajectory (small sweeps) then overlaps the
    // detector with the next step's arithmetic instead of waiting on its
    // branches: 1000 Lorenz points 2.50 -> 1.87 ms, 20,000 points 2.87 ->
    // 2.28 ms, equal at 100,000. Sweeps that fill the GPU (the paired kernels)
    // keep the branches, which issue fewer instructions.
    CHAOS_HD bool push(T v, T& val, int& t) {
        const DiffTest c = diff_test(v, p1);
        if constexpr (Sel) {
            const bool open = !plateau && k > nc && rise && c.ge;
            const bool pl = plateau || open;
            const bool end = pl && (c.up || c.below);
            i0 = open ? k - 1 : i0;
            const bool hit = pl && c.below;
            val = p1;
            t = (i0 + k - 1) >> 1;
            nc = end ? k + 1 : nc;
            plateau = pl && !end;
            rise = c.above;
            p1 = v;
            ++k;
            return hit;
        }
        bool hit = false;
        if (plateau) {  // j = k-1
            if (c.up) {
                plateau = false;
                nc = k + 1;
            } else if (c.below) {
                hit = true; val = p1; t = (i0 + k - 1) >> 1;
                plateau = false;
                nc = k + 1;
            }
        } else if (k > nc && rise && c.ge) {
            i0 = k - 1;
            if (c.below) {
                hit = true; val = p1; t = k - 1;
                nc = k + 1;
            } else {
                plateau = true;
            }
        }
        rise = c.above;
        p1 = v;
        ++k;
        return hit;
    }
};


}  // namespace chaos
