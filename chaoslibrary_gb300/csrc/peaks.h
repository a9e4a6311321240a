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
    // Gate (float, branching form): the common sample -- no plateau open and
    // no candidate to judge -- costs one subtraction, one compare against a
    // threshold and one select. The threshold holds the state the branches
    // read: -inf (not rising), 0 (rising: a sample with d <= 0 is a candidate)
    // or +inf (a plateau is open: every sample is judged). "d > thr" fails for
    // every sample the branches would act on (and for NaN), so those take the
    // full transitions below with rise and plateau read back from thr.
    static constexpr bool Gate = !Sel && sizeof(T) == sizeof(float);
    T p1;          // d[k-1]
    bool rise;     // d[k-1] - d[k-2] > 1e-13
    bool plateau;  // a plateau is open: it started at candidate i0 and runs to j = k-1
    int k;         // index of the next sample
    int nc;        // candidate k-1 is judged when k > nc (outside a plateau)
    int i0;        // plateau: index of the candidate that opened it
    int n;         // peaks detected so far (the dropped first one included)
    int tprev;     // time index of the previous detected peak
    T thr;         // Gate: -inf, 0 or +inf as above

    CHAOS_HD void init() {
        k = 0; nc = 1; plateau = false; i0 = 0; n = 0; tprev = 0; p1 = T(0); rise = false; thr = -kInfT();
    }
    static CHAOS_HD T kInfT() { return T(__builtin_huge_valf()); }

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
    // 2.28 ms against the branching form. Larger sweeps run the branching
    // form behind its gate in blocks of samples (push_block), which issues
    // fewer instructions.
    CHAOS_HD bool push(T v, T& val, int& t) {
        if constexpr (Gate) {
            const T d = v - p1;
            if (__builtin_expect(d > thr, 1)) {
                thr = d > T(1e-13f) ? T(0) : -kInfT();
                p1 = v;
                ++k;
                return false;
            }
            rise = thr == T(0);
            plateau = thr > T(0);
        }
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
        if constexpr (Gate) thr = plateau ? kInfT() : (rise ? T(0) : -kInfT());
        return hit;
    }

    // Pushes the K samples s[0..K-1] (Gate form); on_peak(val, t) for every
    // peak detected, in order. The gate runs over the whole block first: when
    // no sample of it would leave the common path (the threshold of each
    // sample follows from the previous one's difference), the block costs
    // four operations a sample and one branch; otherwise every sample goes
    // through push, exactly as one at a time.
    template <int K, class OnPeak> CHAOS_HD void push_block(const T* s, OnPeak&& on_peak) {
        static_assert(Gate, "push_block is the float detector's block form");
        T th = thr, p = p1;
        bool slow = false;
#pragma unroll
        for (int j = 0; j < K; ++j) {
            const T d = s[j] - p;
            slow |= !(d > th);
            th = d > T(1e-13f) ? T(0) : -kInfT();
            p = s[j];
        }
        if (__builtin_expect(!slow, 1)) {
            thr = th;
            p1 = p;
            k += K;
            return;
        }
#pragma unroll
        for (int j = 0; j < K; ++j) {
            T val;
            int t;
            if (push(s[j], val, t)) on_peak(val, t);
        }
    }
};


}  // namespace chaos
