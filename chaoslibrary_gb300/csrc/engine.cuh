// Device-side building blocks of the sweep engine: per-launch parameter
// blocks, the streaming peak detector, the divergence / fixed-point tests and
// the per-point work functions of the three analyses. Included by the FP64
// and the FP32 kernel translation units, which instantiate the templates for
// their arithmetic type.
//
// Layout rule for every kernel here: one CUDA thread owns one trajectory; its
// full state, its parameters and its peak detector live in registers; the
// trajectory itself never reaches HBM. What a point writes to HBM is its
// result row (a few scalars, plus its peak list for the bifurcation sweeps).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "launch.h"
#include "order_keys.h"
#include "peaks.h"
#include "systems.h"
#include "ff.h"

namespace chaos {

template <int S> struct Traits {
    static constexpr int NX = (S == SYS_SIN2) ? 2 : 3;
    static constexpr int NA = (S == SYS_CHAMELEON) ? 7 : (S == SYS_ROSSLER_CD) ? 4 : (S == SYS_SIN3) ? 5
                            : (S == SYS_SIN2 || S == SYS_MEMRISTOR) ? 2 : 3;
};
#if defined(CHAOS_USER_SYSTEM)
template <> struct Traits<SYS_USER> {
    static constexpr int NX = CHAOS_USER_NX;
    static constexpr int NA = CHAOS_USER_NA;
};
#endif

// Swept value of grid dimension d for linear point index p (the reference's
// getValueByIdx, bifurcationCUDA.cu:400-419 / basinsCUDA.cu:185-189):
// start + n*scale with n = (p / nPts^d) % nPts, multiply and add rounded apart
// (the source as written), or as one FMA when g.fused (the reference's own
// GPU build: nvcc contracts the expression by default).
__device__ __forceinline__ double grid_value(const GridSpec& g, long long p, int d) {
    long long q = p;
    if (d == 1) q /= g.nPts;
    const long long n = q % g.nPts;
    if (g.table[d]) return g.table[d][n];
    return g.fused ? __fma_rn((double)n, g.scale[d], g.start[d]) : __dadd_rn(g.start[d], __dmul_rn((double)n, g.scale[d]));
}

// The maxValue test of both loops, (double)fabsf((float)v) > maxValue, for a
// double v on the integer pipe (this GPU's FP64 pipe is its bottleneck in the
// FP64 sweeps): with b the bits of |v| (not NaN), it holds exactly when
// b > maxBits, or b == maxBits and maxTie (the host derives maxBits from the
// rounding boundary of float(v) at maxValue, see fill_sweep).
__device__ __forceinline__ bool max_exceeded(unsigned long long b, const SweepParams& P) {
    return b > P.maxBits || (b == P.maxBits && P.maxTie);
}

// Divergence test of the bifurcation loop (bifurcationCUDA.cu:445-453):
// v != v || v == v + 1.0  <=>  !(|v| < 2^53); then |(float)v| > maxValue.
template <class T> __device__ __forceinline__ bool bif_diverged(T v, const SweepParams& P);
template <> __device__ __forceinline__ bool bif_diverged<double>(double v, const SweepParams& P) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
    if (b >= 0x4340000000000000ull) return true;  // |v| >= 2^53, infinite or NaN
    return P.checkMax && max_exceeded(b, P);
}
// The same test for a float v, as one compare against a limit that does not
// change in the loop: !(|v| < 2^53) || (checkMax && |v| > maxValueF) holds
// exactly when !(|v| <= lim), lim = min(maxValueF, 2^53 - 2^29) with checkMax,
// else 2^53 - 2^29 (the largest float below 2^53); NaN fails every compare.
template <> __device__ __forceinline__ bool bif_diverged<float>(float v, const SweepParams& P) {
    constexpr float kBelow2p53 = 9007198717870080.0f;
    const float lim = P.checkMax ? fminf(P.maxValueF, kBelow2p53) : kBelow2p53;
    return !(fabsf(v) <= lim);
}
// Divergence test of the basins loop (basinsCUDA.cu:350-361): isnan || isinf, then maxValue.
template <class T> __device__ __forceinline__ bool basins_diverged(T v, const SweepParams& P);
template <> __device__ __forceinline__ bool basins_diverged<double>(double v, const SweepParams& P) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
    if (b > 0x7fefffffffffffffull) return true;  // NaN or +-inf
    return P.checkMax && max_exceeded(b, P);
}
template <> __device__ __forceinline__ bool basins_diverged<float>(float v, const SweepParams& P) {
    const float av = fabsf(v);
    return !(av <= 3.4028234663852886e38f) || (P.checkMax && av > P.maxValueF);
}

// The sample tests and the streaming peak detector (PeakStream) live in
// peaks.h, which the host compiles too.

// x[wv] for a run-time wv without indexing the register array (which would
// move the whole state to local memory).
template <int NX, class T> __device__ __forceinline__ T pick(const T* x, int wv) {
    T v = x[0];
#pragma unroll
    for (int j = 1; j < NX; ++j)
        if (j == wv) v = x[j];
    return v;
}

// Loads state and parameters of point p of a sweep (mutated parameters or
// mutated initial-condition components, per P.mutateState).
template <int S, class T> __device__ __forceinline__ void load_point(const SweepParams& P, long long p, T* x, T* a) {
    constexpr int NX = Traits<S>::NX, NA = Traits<S>::NA;
    double v0 = 0.0, v1 = 0.0;
    v0 = grid_value(P.grid, p, 0);
    if (P.dim > 1) v1 = grid_value(P.grid, p, 1);
#pragma unroll
    for (int i = 0; i < NX; ++i) {
        double v = P.ic[i];
        if (P.mutateState) {  // dimension 1 is written last, as in the reference loop
            if (i == P.mut[0]) v = v0;
            if (P.dim > 1 && i == P.mut[1]) v = v1;
        }
        x[i] = (T)v;
    }
#pragma unroll
    for (int i = 0; i < NA; ++i) {
        double v = P.values[i];
        if (!P.mutateState) {
            if (i == P.mut[0]) v = v0;
            if (P.dim > 1 && i == P.mut[1]) v = v1;
        }
        a[i] = (T)v;
    }
}

// Fixed-point test of the bifurcation loop: sqrtf(fabsf(sum)) < 1e-9 in float.
template <int NX, class T> __device__ __forceinline__ bool bif_fixed(const T* x, const T* xp) {
    T s = T(0);
#pragma unroll
    for (int j = 0; j < NX; ++j) s = s + (x[j] - xp[j]) * (x[j] - xp[j]);
    return (double)sqrtf(fabsf((float)s)) < 1e-9;
}
// Fixed-point test of the basins loop: sqrt(abs(sum)) < 1e-9 in FP64.
template <int NX, class T> __device__ __forceinline__ bool basins_fixed(const T* x, const T* xp) {
    T s = T(0);
#pragma unroll
    for (int j = 0; j < NX; ++j) s = s + (x[j] - xp[j]) * (x[j] - xp[j]);
    return sqrt(fabs((double)s)) < 1e-9;
}

// Samples per block of the recorded loops' block form: the steps of a block
// run back to back, then the gate judges its samples together.
constexpr int kRecordBlock = 4;
// Steps per block of the bifurcation transients' block form.
constexpr int kTransientBlock = 8;

// The block form runs for the float detector (the branching form behind its
// gate) on the built-in systems; a user system keeps the one-step loop (its
// equations are not stepped past a divergence).
template <int S, class T, bool Sel> struct RecordBlocks {
    static constexpr bool value = PeakStream<T, Sel>::Gate && S != SYS_USER;
};

// The recorded part of a bifurcation point, from its state x after a
// transient that ended bounded and not fixed: nB samples through the
// streaming peak detector (intervals in units hI), divergence and fixed-point
// tests; writes flags/counts/first and the first `cap` kept peaks/intervals
// of row o.
//
// Block form: kRecordBlock steps without a branch, their divergence tests
// or-ed together, then the samples through PeakStream::push_block. A block in
// which the orbit diverged pushes its samples up to the divergent one, as the
// one-step loop does, and ends the loop (the steps after the divergent one
// change nothing that is reported). The last step, whose starting state the
// fixed-point test keeps, always runs in the one-step loop.
template <int S, class T, bool Sel = false>
__device__ __forceinline__ void bif_record(const SweepParams& P, const BifOut& O, T* x, const T* a,
                                           const StepCtx<T>& c, int nB, double hI, long long o) {
    constexpr int NX = Traits<S>::NX;
    T xp[NX];
    const int wv = P.wv;
    int flag = 1;
    PeakStream<T, Sel> ps;
    ps.init();
    const double first = (double)pick<NX>(x, wv);
    double* pk = O.peaks ? O.peaks + o * (long long)O.cap : nullptr;
    double* iv = O.intervals ? O.intervals + o * (long long)O.cap : nullptr;
    auto on_peak = [&](T val, int t) {
        if (ps.n >= 1) {
            const int q = ps.n - 1;
            if (q < O.cap) {
                if (pk) pk[q] = (double)val;
                if (iv) iv[q] = __dmul_rn((double)(t - ps.tprev), hI);
            }
        }
        ps.tprev = t;
        ++ps.n;
    };
    T v = pick<NX>(x, wv);  // the recorded sample, carried from one step to the next
#pragma unroll
    for (int j = 0; j < NX; ++j) xp[j] = x[j];
    int i = 0;
    if constexpr (RecordBlocks<S, T, Sel>::value) {
        constexpr int K = kRecordBlock;
        for (; i + K < nB; i += K) {
            T s[K + 1];
            s[0] = v;
            bool dv = false;
#pragma unroll
            for (int j = 1; j <= K; ++j) {
                step<S>(x, a, c);
                s[j] = pick<NX>(x, wv);
                dv |= bif_diverged(s[j], P);
            }
            if (__builtin_expect(!dv, 1)) {
                ps.template push_block<K>(s, on_peak);
                v = s[K];
                continue;
            }
#pragma unroll
            for (int j = 0; j < K; ++j) {
                T val;
                int t;
                if (ps.push(s[j], val, t)) on_peak(val, t);
                if (bif_diverged(s[j + 1], P)) break;
            }
            flag = 0;
            break;
        }
    }
    if (flag == 1)
        for (; i < nB; ++i) {
#pragma unroll
            for (int j = 0; j < NX; ++j) xp[j] = x[j];
            T val;
            int t;
            if (ps.push(v, val, t)) on_peak(val, t);
            step<S>(x, a, c);
            v = pick<NX>(x, wv);
            if (bif_diverged(v, P)) { flag = 0; break; }
        }
    if (flag == 1 && nB > 0 && bif_fixed<NX>(x, xp)) flag = -1;
    const int kept = ps.n > 1 ? ps.n - 1 : 0;
    O.flags[o] = flag;
    O.counts[o] = flag == 1 ? kept : (flag == -1 ? -1 : 0);
    if (O.first) O.first[o] = first;
}

// ---------------------------------------------------------------------------
// Bifurcation point (reference kernels calculateTransTimeCUDA +
// calculateDiscreteModelCUDA + peakFinderCUDA, bifurcationCUDA.cu:258-371),
// fused. Writes flags/counts/first and the first `cap` kept peaks/intervals.
template <int S, class T, bool Sel = false>
__device__ __forceinline__ void bif_point(const SweepParams& P, const BifOut& O, long long p, long long o) {
    constexpr int NX = Traits<S>::NX, NA = Traits<S>::NA;
    T x[NX], a[NA], xp[NX];
    load_point<S, T>(P, p, x, a);
    double hp = P.h, hI = P.hInterval;
    int nS = P.S, nB = P.B;
    if (P.sweepStep) {  // this point's own step and step counts, as the host derives them from h
        hp = grid_value(P.grid, p, 0);
        nS = (int)__ddiv_rn(P.transientTime, hp);
        nB = (int)__ddiv_rn(__ddiv_rn(P.tMax, hp), (double)P.bPre);
        hI = __dmul_rn(hp, (double)P.bPre);
    }
    const StepCtx<T> c((T)hp);
    const int wv = P.wv;
    int flag = 1;
    if (nS > 0) {
        // the state before the last step is kept for the fixed-point test:
        // the last step is peeled off the loop, so the others copy nothing
        int s = 0;
        if constexpr (S != SYS_USER && !Sel) {
            // blocks of kTransientBlock steps, one divergence branch a block:
            // a point's flags do not depend on the step at which it diverged
            // (the steps after it on an unbounded state report nothing). The
            // select form (small sweeps, one latency-bound orbit a warp)
            // keeps the one-step loop and its registers.
            constexpr int K = kTransientBlock;
            for (; s + K <= nS - 1; s += K) {
                bool dv = false;
#pragma unroll
                for (int j = 0; j < K; ++j) {
                    step<S>(x, a, c);
                    dv |= bif_diverged(pick<NX>(x, wv), P);
                }
                if (dv) { flag = 0; break; }
            }
        }
        if (flag == 1)
            for (; s < nS - 1; ++s) {
                step<S>(x, a, c);
                if (bif_diverged(pick<NX>(x, wv), P)) { flag = 0; break; }
            }
        if (flag == 1) {
#pragma unroll
            for (int j = 0; j < NX; ++j) xp[j] = x[j];
            step<S>(x, a, c);
            if (bif_diverged(pick<NX>(x, wv), P)) flag = 0;
            else if (bif_fixed<NX>(x, xp)) flag = -1;
        }
    }
    if (flag == 1) {
        bif_record<S, T, Sel>(P, O, x, a, c, nB, hI, o);
    } else {  // a transient that ended diverged or fixed is reported as diverged
        O.flags[o] = 0;
        O.counts[o] = 0;
        if (O.first) O.first[o] = 0.0;
    }
}

// Bifurcation point of the legacy library's analyses (P.legacyLoop, FP64),
// with the legacy per-point loop in place of the current library's.
// P.legacyLoop 1, the grids over initial conditions or parameters
// (calculateDiscreteModelICCUDA, debri/cudaLibrary.cu:1022-1116, over
// loopCalculateDiscreteModel_int, :604-680, then peakFinderCUDA, :1345-1367):
//  - the transient (one step a sample, no bound) ends the point with flag 0
//    when state component 0 becomes NaN or infinite;
//  - its fixed-point verdict does not stop the recorded part.
// P.legacyLoop 2, the step-size sweep (calculateDiscreteModelCUDA_H,
// :955-1000, over loopCalculateDiscreteModel, :472-527, then
// peakFinderCUDA_H, :1396-1412):
//  - the transient stops early at a NaN or infinite component 0, and its
//    verdict is ignored.
// Both recorded parts take sample x[wv] and then preScaller steps, and test
// the sample for NaN, infinity and |(float)x[wv]| > maxValue (flag 0). The
// change of state over the last sample, s = sum of squared differences,
// marks a fixed point (flag -1, count -1):
//  - loop 1: when sqrt(|s|) < 1e-9;
//  - loop 2: when s == 0 or sqrt(s) < 1e-12 (the legacy keeps no peaks).
// Peaks and intervals (units h * preScaller) are written as in bif_record.
template <int S>
__device__ __forceinline__ void bif_point_legacy(const SweepParams& P, const BifOut& O, long long p, long long o) {
    constexpr int NX = Traits<S>::NX, NA = Traits<S>::NA;
    double x[NX], a[NA], xp[NX];
    load_point<S, double>(P, p, x, a);
    double hp = P.h, hI = P.hInterval;
    int nS = P.S, nB = P.B;
    if (P.sweepStep) {
        hp = grid_value(P.grid, p, 0);
        nS = (int)__ddiv_rn(P.transientTime, hp);
        nB = (int)__ddiv_rn(__ddiv_rn(P.tMax, hp), (double)P.bPre);
        hI = __dmul_rn(hp, (double)P.bPre);
    }
    const StepCtx<double> c(hp);
    const int wv = P.wv, pre = P.bPre;
    auto nan_or_inf = [](double v) {
        return ((unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull) > 0x7fefffffffffffffull;
    };
    int flag = 1;
    for (int s = 0; s < nS; ++s) {
        step<S>(x, a, c);
        if (nan_or_inf(x[0])) {
            if (P.legacyLoop == 1) flag = 0;
            break;
        }
    }
    PeakStream<double> ps;
    ps.init();
    double* pk = O.peaks ? O.peaks + o * (long long)O.cap : nullptr;
    double* iv = O.intervals ? O.intervals + o * (long long)O.cap : nullptr;
    auto on_peak = [&](double val, int t) {
        if (ps.n >= 1) {
            const int q = ps.n - 1;
            if (q < O.cap) {
                if (pk) pk[q] = val;
                if (iv) iv[q] = __dmul_rn((double)(t - ps.tprev), hI);
            }
        }
        ps.tprev = t;
        ++ps.n;
    };
    double first = 0.0;
    if (flag == 1) {
        double v = pick<NX>(x, wv);
        first = v;
        for (int i = 0; i < nB; ++i) {
#pragma unroll
            for (int j = 0; j < NX; ++j) xp[j] = x[j];
            double val;
            int t;
            if (ps.push(v, val, t)) on_peak(val, t);
            for (int r = 0; r < pre; ++r) step<S>(x, a, c);
            v = pick<NX>(x, wv);
            if (basins_diverged(v, P)) { flag = 0; break; }
        }
        if (flag == 1 && nB > 0) {
            double s = 0.0;
#pragma unroll
            for (int j = 0; j < NX; ++j) {
                const double d = __dsub_rn(x[j], xp[j]);
                s = __dadd_rn(s, __dmul_rn(d, d));
            }
            const bool fixed = P.legacyLoop == 1 ? __dsqrt_rn(fabs(s)) < 1e-9 : (s == 0.0 || __dsqrt_rn(s) < 1e-12);
            if (fixed) flag = -1;
        }
    }
    const int kept = ps.n > 1 ? ps.n - 1 : 0;
    O.flags[o] = flag;
    O.counts[o] = flag == 1 ? kept : (flag == -1 ? -1 : 0);
    if (O.first) O.first[o] = flag == -1 ? first : 0.0;
}

// Sums over the kept peaks of a basins point: peak values and intervals.
// FP64 path: the reference's per-peak FP64 sums (avgPeakFinderCUDA,
// basinsCUDA.cu:818-864). FP32 path: no FP64 instruction per peak (the FP64
// pipe of this GPU is a small fraction of the FP32 rate): the values are
// summed as an unevaluated float pair with the error-free TwoSum (about 48
// significant bits), the intervals as the integer time span they telescope
// to, and both are widened to FP64 once at the end.
template <class T> struct PeakSums;
template <> struct PeakSums<double> {
    double sp = 0.0, si = 0.0;
    __device__ __forceinline__ void add(double val, int dt, double hI) {
        sp = sp + val;
        si = si + __dmul_rn((double)dt, hI);
    }
    __device__ __forceinline__ double peaks() const { return sp; }
    __device__ __forceinline__ double intervals(double) const { return si; }
};
template <> struct PeakSums<float> {
    float hi = 0.f, lo = 0.f;
    int span = 0;
    __device__ __forceinline__ void add(float val, int dt, double) {
        const float s = hi + val;  // TwoSum(hi, val) = s + err exactly
        const float bv = s - hi;
        const float err = (hi - (s - bv)) + (val - bv);
        hi = s;
        lo = lo + err;
        span += dt;
    }
    __device__ __forceinline__ double peaks() const { return (double)hi + (double)lo; }
    __device__ __forceinline__ double intervals(double hI) const { return __dmul_rn((double)span, hI); }
};

// ---------------------------------------------------------------------------
// Basins point (reference calculateTransTimeCUDA + calculateDiscreteModelCUDA
// + avgPeakFinderCUDA, basinsCUDA.cu:233-314 and 818-864), fused. PRE1: the
// sweep has preScaller == 1 (one step per sample, no inner loop).
// The recorded part of a basins point, from its state x after the transient:
// peak detector, divergence and fixed-point tests, features into row o.
template <int S, class T, bool PRE1, bool Sel = false>
__device__ __forceinline__ void basins_record(const SweepParams& P, const BasinsOut& O, T* x, const T* a,
                                              const StepCtx<T>& c, long long o) {
    constexpr int NX = Traits<S>::NX;
    T xp[NX];
    const int wv = P.wv;
#pragma unroll
    for (int j = 0; j < NX; ++j) xp[j] = x[j];
    PeakStream<T, Sel> ps;
    ps.init();
    int flag = 1;
    PeakSums<T> sums;
    T lastT = T(0);  // widened once after the loop (a per-step FP64 convert costs FP64-pipe time)
    auto on_peak = [&](T val, int t) {
        if (ps.n >= 1) sums.add(val, t - ps.tprev, P.hInterval);
        ps.tprev = t;
        ++ps.n;
    };
    T v = pick<NX>(x, wv);  // the recorded sample, carried from one step to the next
    int i = 0;
    if constexpr (RecordBlocks<S, T, Sel>::value) {  // the block form of bif_record
        constexpr int K = kRecordBlock;
        for (; i + K < P.B; i += K) {
            T s[K + 1];
            s[0] = v;
            bool dv = false;
#pragma unroll
            for (int j = 1; j <= K; ++j) {
                if (PRE1) step<S>(x, a, c);
                else
                    for (int r = 0; r < P.preScaller; ++r) step<S>(x, a, c);
                s[j] = pick<NX>(x, wv);
                dv |= basins_diverged(s[j], P);
            }
            if (__builtin_expect(!dv, 1)) {
                ps.template push_block<K>(s, on_peak);
                lastT = s[K - 1];
                v = s[K];
                continue;
            }
#pragma unroll
            for (int j = 0; j < K; ++j) {
                lastT = s[j];
                T val;
                int t;
                if (ps.push(s[j], val, t)) on_peak(val, t);
                if (basins_diverged(s[j + 1], P)) break;
            }
            flag = 0;
            break;
        }
    }
    if (flag == 1)
        for (; i < P.B; ++i) {
#pragma unroll
            for (int j = 0; j < NX; ++j) xp[j] = x[j];
            lastT = v;
            T val;
            int t;
            if (ps.push(v, val, t)) on_peak(val, t);
            if (PRE1) step<S>(x, a, c);
            else
                for (int r = 0; r < P.preScaller; ++r) step<S>(x, a, c);
            v = pick<NX>(x, wv);
            if (basins_diverged(v, P)) { flag = 0; break; }
        }
    if (flag == 1 && P.B > 0 && basins_fixed<NX>(x, xp)) flag = -1;
    const double last = (double)lastT;
    const int kept = ps.n > 1 ? ps.n - 1 : 0;
    double ap, ai;
    if (flag == 0) { ap = 999.0; ai = 999.0; }
    else if (flag == -1) { ap = last; ai = -1.0; }
    else if (kept <= 0) { ap = 1000.0; ai = 1000.0; }
    else { ap = sums.peaks() / (double)kept; ai = sums.intervals(P.hInterval) / (double)kept; }
    O.flags[o] = flag;
    O.avgPeaks[o] = ap;
    O.avgIntervals[o] = ai;
    if (O.counts) O.counts[o] = flag == 1 ? kept : 0;
    if (O.last) O.last[o] = last;
    if (O.mm) {  // the clustering's normalisation bounds
        FeatureKeys fk;
        fk.add(flag, flag == 1 ? kept : 0, ap, ai, last);
        fk.flush(O.mm);
    }
}

template <int S, class T, bool PRE1 = false, bool Sel = false>
__device__ __forceinline__ void basins_point(const SweepParams& P, const BasinsOut& O, long long p, long long o) {
    constexpr int NX = Traits<S>::NX, NA = Traits<S>::NA;
    T x[NX], a[NA];
    load_point<S, T>(P, p, x, a);
    const StepCtx<T> c((T)P.h);
    for (int s = 0; s < P.S; ++s) step<S>(x, a, c);
    basins_record<S, T, PRE1, Sel>(P, O, x, a, c, o);
}

// ---------------------------------------------------------------------------
// LLE point, the reference's Benettin scheme (LLECUDA.cu:114-166) in full
// precision T for both trajectories: calcBlocks+1 blocks of NT steps of x and
// of its twin q; d = |x-q|/eps; sum += log(d); q = x - (x-q)/d; sum / tMax.
// The twin starts at x + eps along state component 0.
// State and parameters of point p of an LLE-type sweep: a 1-D grid (p = i)
// or the 2-D map (p = j*nPts + i), over parameters values[mut] or initial
// conditions ic[mut] (L.mutateState); the second dimension is written last.
// Swept values are linspace start + n*step, multiply and add rounded apart.
template <int NX, int NA, class T>
__device__ __forceinline__ void lle_load(const LleParams& L, long long p, T* x, T* a) {
    const long long i = L.dim == 1 ? p : p % L.nPts, j = L.dim == 1 ? 0 : p / L.nPts;
    const double va = L.table[0]    ? L.table[0][i]
                      : L.nPts == 1 ? L.rangeA[0]
                                    : __dadd_rn(L.rangeA[0], __dmul_rn((double)i, L.stepA));
    const double vb = L.table[1]                      ? L.table[1][j]
                      : (L.nPts == 1 || L.dim == 1) ? L.rangeB[0]
                                                    : __dadd_rn(L.rangeB[0], __dmul_rn((double)j, L.stepB));
#pragma unroll
    for (int k = 0; k < NX; ++k) {
        double v = L.ic[k];
        if (L.mutateState) {
            if (k == L.mut[0]) v = va;
            if (k == L.mut[1]) v = vb;
        }
        x[k] = (T)v;
    }
#pragma unroll
    for (int k = 0; k < NA; ++k) {
        double v = L.values[k];
        if (!L.mutateState) {
            if (k == L.mut[0]) v = va;
            if (k == L.mut[1]) v = vb;
        }
        a[k] = (T)v;
    }
}

// The Benettin blocks of the reference's calculateSystem (LLE/src/LLECUDA.cu:
// 146-162) from an orbit x and a full twin trajectory q: calcBlocks + 1
// blocks of ntp steps of each, dist = sqrt(sum (x - q)^2) / eps, sum +=
// log(dist), q = x - (x - q) / dist; the sum over tMax.
template <int S, class T>
__device__ __forceinline__ double lle_benettin_full(const LleParams& L, T* x, T* q, const T* a) {
    constexpr int NX = Traits<S>::NX;
    const StepCtx<T> c((T)L.h);
    double sum = 0.0;
    for (int b = 0; b <= L.calcBlocks; ++b) {
        for (int s = 0; s < L.ntp; ++s) step<S>(x, a, c);
        for (int s = 0; s < L.ntp; ++s) step<S>(q, a, c);
        double dist = 0.0;
#pragma unroll
        for (int k = 0; k < NX; ++k) {
            const double df = (double)x[k] - (double)q[k];
            dist = dist + df * df;
        }
        dist = sqrt(dist) / L.eps;
        sum = sum + log(dist);
#pragma unroll
        for (int k = 0; k < NX; ++k) q[k] = (T)((double)x[k] - (((double)x[k] - (double)q[k]) / dist));
    }
    return sum / L.tMax;
}

template <int S, class T>
__device__ __forceinline__ double lle_point_full(const LleParams& L, long long p) {
    constexpr int NX = Traits<S>::NX, NA = Traits<S>::NA;
    T x[NX], q[NX], a[NA];
    lle_load<NX, NA>(L, p, x, a);
    const StepCtx<T> c((T)L.h);
    for (int s = 0; s < L.trans; ++s) step<S>(x, a, c);
#pragma unroll
    for (int k = 0; k < NX; ++k) q[k] = x[k];
    if (L.twin == 1) {
        // the reference's twin start (LLECUDA.cu:97-101): a float FMA of a unit
        // direction times eps onto the float-rounded state, here with the
        // direction e_x instead of its cuRAND draw
#pragma unroll
        for (int k = 0; k < NX; ++k) q[k] = (T)__fmaf_rn(k == 0 ? 1.0f : 0.0f, (float)L.eps, (float)x[k]);
    } else {
        q[0] = x[0] + (T)L.eps;
    }
    return lle_benettin_full<S>(L, x, q, a);
}

// LLE point with the twin carried as the exact difference e = q - x (only for
// the quadratic RK4 systems): x and e in FP32 registers. Same block count and
// division by tMax as above. How the stretch of every block is measured and
// the twin renormalised is the Stretch mode:
//   kRenormPow2 (default): e is scaled by a power of two 2^-k that brings |e|
//     back to within a factor sqrt(2) of eps -- exact in FP32 -- and k is
//     summed as an integer, so the sum of the blocks' log-stretches telescopes
//     exactly to k ln 2 + log(|e_final| / eps), taken once in FP64 from the
//     FP64 norm of the final e (ff.h);
//   kRenormF32Log: log2(|e|^2 / eps^2) per block on the SFU (__log2f), e
//     rescaled to length eps with rsqrtf, the logs summed in FP32 over groups
//     of kLleGroup blocks and the group sums in FP64;
//   kRenormF64: the reference's arithmetic (LLE/src/LLECUDA.cu:146-162):
//     dist = sqrt(sum (x - p)^2) / eps in FP64, sum += log(dist), e /= dist.
enum LleRenorm { kRenormPow2 = 0, kRenormF32Log = 1, kRenormF64 = 2 };
constexpr int kLleGroup = 16;

__device__ __forceinline__ double nan_if_not_finite(double v) {
    return isfinite(v) ? v : __longlong_as_double(0x7ff8000000000000LL);
}

template <int RN> struct Stretch;
template <> struct Stretch<kRenormPow2> {
    double eps;  // the stretch of every block is measured against eps, as the reference measures it
    int eps2Exp, k = 0;
    double v = 0.0;
    __device__ __forceinline__ explicit Stretch(double eps_) : eps(eps_) {
        const float e0 = (float)eps_;
        eps2Exp = (int)((__float_as_uint(e0 * e0) >> 23) & 0xff) - 126;
    }
    __device__ __forceinline__ float renorm(float e0_, float e1, float e2) {
        const int j = pow2_rescale_exponent(fmaf(e0_, e0_, fmaf(e1, e1, e2 * e2)), eps2Exp);
        k += j;
        return pow2_scale(j);
    }
    __device__ __forceinline__ void last(float e0_, float e1, float e2) {
        const double n2 = (double)e0_ * e0_ + (double)e1 * e1 + (double)e2 * e2;
        v = pow2_log_stretch(k, n2, eps);
    }
    __device__ __forceinline__ double result(double tMax) const { return nan_if_not_finite(v / tMax); }
};
template <> struct Stretch<kRenormF32Log> {
    float eps, inv_eps2, part = 0.f;
    int cnt = 0;
    double sum = 0.0;  // sum of log2(d^2)
    __device__ __forceinline__ Stretch(float eps_, double epsd) : eps(eps_), inv_eps2((float)(1.0 / (epsd * epsd))) {}
    __device__ __forceinline__ float add(float n2) {
        part += __log2f(n2 * inv_eps2);
        if (++cnt == kLleGroup) {
            sum += (double)part;
            part = 0.f;
            cnt = 0;
        }
        return n2;
    }
    __device__ __forceinline__ float renorm(float e0, float e1, float e2) {
        const float n2 = add(fmaf(e0, e0, fmaf(e1, e1, e2 * e2)));
        return eps * rsqrtf(n2);
    }
    __device__ __forceinline__ void last(float e0, float e1, float e2) { add(fmaf(e0, e0, fmaf(e1, e1, e2 * e2))); }
    __device__ __forceinline__ double result(double tMax) const {
        return (sum + (double)part) * (0.5 * 0.69314718055994530942) / tMax;  // log2(d^2) -> ln(d)
    }
};
template <> struct Stretch<kRenormF64> {
    double eps, sum = 0.0;
    __device__ __forceinline__ explicit Stretch(double eps_) : eps(eps_) {}
    __device__ __forceinline__ double dist(float e0, float e1, float e2) const {
        return sqrt((double)e0 * e0 + (double)e1 * e1 + (double)e2 * e2) / eps;
    }
    __device__ __forceinline__ float renorm(float e0, float e1, float e2) {
        const double d = dist(e0, e1, e2);
        sum += log(d);
        return (float)(1.0 / d);
    }
    __device__ __forceinline__ void last(float e0, float e1, float e2) { sum += log(dist(e0, e1, e2)); }
    __device__ __forceinline__ double result(double tMax) const { return sum / tMax; }
};
template <int RN> __device__ __forceinline__ Stretch<RN> make_stretch(const LleParams& L);
template <> __device__ __forceinline__ Stretch<kRenormPow2> make_stretch<kRenormPow2>(const LleParams& L) {
    return Stretch<kRenormPow2>(L.eps);
}
template <> __device__ __forceinline__ Stretch<kRenormF32Log> make_stretch<kRenormF32Log>(const LleParams& L) {
    return Stretch<kRenormF32Log>((float)L.eps, L.eps);
}
template <> __device__ __forceinline__ Stretch<kRenormF64> make_stretch<kRenormF64>(const LleParams& L) {
    return Stretch<kRenormF64>(L.eps);
}

template <class F, class T>
__device__ __forceinline__ void twin_steps(T* x, T* e, const T* a, const RK4H<T>& c, int n) {  // n steps, 2 per trip
    int s = 0;
    for (; s + 2 <= n; s += 2) {
        rk4_step_twin<F>(x, e, a, c);
        rk4_step_twin<F>(x, e, a, c);
    }
    if (s < n) rk4_step_twin<F>(x, e, a, c);
}

// The Benettin blocks of an FP32 twin carried as a difference e (three state
// components): steps(e, n) advances the orbit and e by n steps.
template <int RN = kRenormPow2, class Steps>
__device__ __forceinline__ double lle_twin_blocks(const LleParams& L, Steps&& steps) {
    Stretch<RN> st = make_stretch<RN>(L);
    float e[3] = {(float)L.eps, 0.f, 0.f};
    const int nb = L.calcBlocks + 1;
    for (int b = 0; b < nb; ++b) {
        steps(e, L.ntp);
        if (b + 1 < nb) {
            const float r = st.renorm(e[0], e[1], e[2]);
            e[0] *= r;
            e[1] *= r;
            e[2] *= r;
        } else {
            st.last(e[0], e[1], e[2]);
        }
    }
    return st.result(L.tMax);
}

template <class F>
__device__ __forceinline__ double lle_point_twin(const LleParams& L, long long p) {
    float x[3], a[3];
    lle_load<3, 3>(L, p, x, a);
    const RK4H<float> c((float)L.h);
    for (int s = 0; s < L.trans; ++s) rk4_step<F>(x, a, c);
    return lle_twin_blocks(L, [&](float* e, int n) { twin_steps<F>(x, e, a, c, n); });
}

// The FP32 LLE point of Chameleon (the reference's default system): the twin
// as the difference of chameleon_step_twin.
__device__ __forceinline__ double lle_point_twin_chameleon(const LleParams& L, long long p) {
    float x[3], a[7];
    lle_load<3, 7>(L, p, x, a);
    const float h = (float)L.h;
    for (int s = 0; s < L.trans; ++s) chameleon_step<float>(x, a, h);
    return lle_twin_blocks(L, [&](float* e, int n) {
        for (int s = 0; s < n; ++s) chameleon_step_twin<float>(x, e, a, h);
    });
}

// ---------------------------------------------------------------------------
// Lyapunov spectrum of one point: one twin per state dimension, started along
// the unit vectors (x + eps e_j), integrated NT at a time beside the base
// trajectory; after every block the differences y_j - x are orthogonalised by
// classical Gram-Schmidt (b_j = d_j - sum_{m<j} (d_j.b_m / b_m.b_m) b_m), each
// norm |b_j| adds log(|b_j| / eps) to exponent j and the twins restart at
// x + eps b_j/|b_j| -- the scheme of the legacy library's spectrum kernel
// (debri/cudaLibrary.cu:2141-2330). Blocks and the division by tMax are the
// LLE map's (calcBlocks + 1 blocks), so exponent 0 estimates the same
// quantity as lle_point_full. out[p*NX + j] = exponent j.
template <int S>
__device__ __forceinline__ void spectrum_point_full(const LleParams& L, long long p, double* out) {
    constexpr int N = Traits<S>::NX, NA = Traits<S>::NA;
    double x[N], y[N][N], a[NA], sum[N];
    lle_load<N, NA>(L, p, x, a);
    const StepCtx<double> c(L.h);
    for (int s = 0; s < L.trans; ++s) step<S>(x, a, c);
#pragma unroll
    for (int j = 0; j < N; ++j) {
        sum[j] = 0.0;
#pragma unroll
        for (int i = 0; i < N; ++i) y[j][i] = i == j ? x[i] + L.eps : x[i];
    }
    for (int b = 0; b <= L.calcBlocks; ++b) {
        for (int s = 0; s < L.ntp; ++s) step<S>(x, a, c);
#pragma unroll
        for (int j = 0; j < N; ++j)
            for (int s = 0; s < L.ntp; ++s) step<S>(y[j], a, c);
        double d[N][N], g[N][N];
#pragma unroll
        for (int j = 0; j < N; ++j) {
#pragma unroll
            for (int i = 0; i < N; ++i) {
                d[j][i] = y[j][i] - x[i];
                g[j][i] = d[j][i];
            }
#pragma unroll
            for (int m = 0; m < j; ++m) {
                double num = 0.0, den = 0.0;
#pragma unroll
                for (int i = 0; i < N; ++i) {
                    num = num + d[j][i] * g[m][i];
                    den = den + g[m][i] * g[m][i];
                }
                const double frac = den == 0.0 ? 0.0 : num / den;
#pragma unroll
                for (int i = 0; i < N; ++i) g[j][i] = g[j][i] - frac * g[m][i];
            }
        }
#pragma unroll
        for (int j = 0; j < N; ++j) {
            double n2 = 0.0;
#pragma unroll
            for (int i = 0; i < N; ++i) n2 = n2 + g[j][i] * g[j][i];
            const double nrm = sqrt(n2);
            sum[j] = sum[j] + log(nrm / L.eps);
#pragma unroll
            for (int i = 0; i < N; ++i) y[j][i] = x[i] + (nrm == 0.0 ? 0.0 : g[j][i] / nrm) * L.eps;
        }
    }
#pragma unroll
    for (int j = 0; j < N; ++j) out[p * N + j] = sum[j] / L.tMax;
}

// The spectrum in FP32 for the quadratic RK4 systems and Chameleon: the twins
// carried as exact differences e_j, Gram-Schmidt in FP32, per block
// log2(|b_j|^2/eps^2) on the SFU summed in FP32 groups of kLleGroup blocks and
// added into FP64, as the FP32 LLE map does. steps(e, n) advances the orbit
// and the three differences by n steps.
template <class Steps>
__device__ __forceinline__ void spectrum_twin_blocks(const LleParams& L, long long p, double* out, Steps&& steps) {
    float e[3][3];
    const float eps = (float)L.eps;
    const float inv_eps2 = (float)(1.0 / (L.eps * L.eps));
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int i = 0; i < 3; ++i) e[j][i] = i == j ? eps : 0.f;
    double sum[3] = {0.0, 0.0, 0.0};
    const int nb = L.calcBlocks + 1;
    for (int b0 = 0; b0 < nb; b0 += kLleGroup) {
        const int bn = min(kLleGroup, nb - b0);
        float part[3] = {0.f, 0.f, 0.f};
        for (int b = 0; b < bn; ++b) {
            steps(e, L.ntp);
            float g[3][3];
#pragma unroll
            for (int j = 0; j < 3; ++j) {
#pragma unroll
                for (int i = 0; i < 3; ++i) g[j][i] = e[j][i];
#pragma unroll
                for (int m = 0; m < j; ++m) {
                    const float num = fmaf(e[j][0], g[m][0], fmaf(e[j][1], g[m][1], e[j][2] * g[m][2]));
                    const float den = fmaf(g[m][0], g[m][0], fmaf(g[m][1], g[m][1], g[m][2] * g[m][2]));
                    const float frac = den == 0.f ? 0.f : num / den;
#pragma unroll
                    for (int i = 0; i < 3; ++i) g[j][i] = fmaf(-frac, g[m][i], g[j][i]);
                }
            }
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const float n2 = fmaf(g[j][0], g[j][0], fmaf(g[j][1], g[j][1], g[j][2] * g[j][2]));
                part[j] += __log2f(n2 * inv_eps2);
                const float r = n2 > 0.f ? eps * rsqrtf(n2) : 0.f;
#pragma unroll
                for (int i = 0; i < 3; ++i) e[j][i] = g[j][i] * r;
            }
        }
#pragma unroll
        for (int j = 0; j < 3; ++j) sum[j] += (double)part[j];
    }
#pragma unroll
    for (int j = 0; j < 3; ++j) out[p * 3 + j] = sum[j] * (0.5 * 0.69314718055994530942) / L.tMax;
}

template <class F>
__device__ __forceinline__ void spectrum_point_twin(const LleParams& L, long long p, double* out) {
    float x[3], a[3];
    lle_load<3, 3>(L, p, x, a);
    const RK4H<float> c((float)L.h);
    for (int s = 0; s < L.trans; ++s) rk4_step<F>(x, a, c);
    spectrum_twin_blocks(L, p, out, [&](float (*e)[3], int n) {
        for (int s = 0; s < n; ++s) rk4_step_multi<F, 3>(x, e, a, c);
    });
}

__device__ __forceinline__ void spectrum_point_twin_chameleon(const LleParams& L, long long p, double* out) {
    float x[3], a[7];
    lle_load<3, 7>(L, p, x, a);
    const float h = (float)L.h;
    for (int s = 0; s < L.trans; ++s) chameleon_step<float>(x, a, h);
    spectrum_twin_blocks(L, p, out, [&](float (*e)[3], int n) {
        for (int s = 0; s < n; ++s) chameleon_step_multi<float, 3>(x, e, a, h);
    });
}

// ---------------------------------------------------------------------------
// Packed pair of FP32 values: two trajectories advanced by one instruction
// stream with Blackwell's paired FP32 instructions (fma.rn.f32x2,
// add.rn.f32x2, mul.rn.f32x2). Each lane of the pair is rounded exactly as
// the scalar FP32 operation would be; the pair halves the instructions the
// schedulers issue for the same flops.
struct P2 {
    float2 v;
    __device__ __forceinline__ P2() {}
    __device__ __forceinline__ explicit P2(double s) : v(make_float2((float)s, (float)s)) {}
    __device__ __forceinline__ P2(float a, float b) : v(make_float2(a, b)) {}
};
__device__ __forceinline__ P2 mk(float2 f) { P2 r; r.v = f; return r; }
__device__ __forceinline__ P2 operator+(P2 a, P2 b) { return mk(__fadd2_rn(a.v, b.v)); }
__device__ __forceinline__ P2 operator-(P2 a) { return mk(make_float2(-a.v.x, -a.v.y)); }
__device__ __forceinline__ P2 operator-(P2 a, P2 b) { return mk(__fadd2_rn(a.v, make_float2(-b.v.x, -b.v.y))); }
__device__ __forceinline__ P2 operator*(P2 a, P2 b) { return mk(__fmul2_rn(a.v, b.v)); }
__device__ __forceinline__ P2& operator*=(P2& a, P2 b) { a = a * b; return a; }
__device__ __forceinline__ P2 fmaT(P2 a, P2 b, P2 c) { return mk(__ffma2_rn(a.v, b.v, c.v)); }
__device__ __forceinline__ P2 addR(P2 a, P2 b) { return a + b; }
// Word operations of float-float pairs of packed lanes (ff.h): each one
// paired instruction, rounded per lane exactly as the scalar operation;
// a - b as fma(b, -1, a), which is RN(a - b) in one instruction.
__device__ __forceinline__ P2 w_add(P2 a, P2 b) { return mk(__fadd2_rn(a.v, b.v)); }
__device__ __forceinline__ P2 w_sub(P2 a, P2 b) { return mk(__ffma2_rn(b.v, make_float2(-1.f, -1.f), a.v)); }
__device__ __forceinline__ P2 w_mul(P2 a, P2 b) { return mk(__fmul2_rn(a.v, b.v)); }
__device__ __forceinline__ P2 w_fma(P2 a, P2 b, P2 c) { return mk(__ffma2_rn(a.v, b.v, c.v)); }
__device__ __forceinline__ P2 w_neg(P2 a) { return mk(make_float2(-a.v.x, -a.v.y)); }

// Step constants of a packed pair: rounded exactly as RK4H<float> rounds them.
template <> struct RK4H<P2> {
    P2 h, hh, h6;
    __device__ __forceinline__ explicit RK4H(float h_)
        : h((double)h_), hh((double)(h_ * 0.5f)), h6((double)(h_ / 6.0f)) {}
};

// Two LLE points per thread (indices p and q), lanes of P2. Same arithmetic
// per lane as lle_point_twin with T = float; the per-block stretch and
// renormalisation (Stretch mode RN) run per lane.
template <class F, int RN = kRenormPow2>
__device__ __forceinline__ void lle_pair_twin(const LleParams& L, long long p, long long q, double* outp,
                                              double* outq) {
    P2 x[3], e[3], a[3];
    float xs[2][3], as[2][3];
    lle_load<3, 3>(L, p, xs[0], as[0]);
    lle_load<3, 3>(L, q, xs[1], as[1]);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        a[k] = P2(as[0][k], as[1][k]);
        x[k] = P2(xs[0][k], xs[1][k]);
    }
    const RK4H<P2> c((float)L.h);
    for (int s = 0; s < L.trans; ++s) rk4_step<F>(x, a, c);
    const float eps = (float)L.eps;
    e[0] = P2((double)eps);
    e[1] = P2(0.0);
    e[2] = P2(0.0);
    Stretch<RN> s0 = make_stretch<RN>(L), s1 = make_stretch<RN>(L);
    const int nb = L.calcBlocks + 1;
    for (int b = 0; b < nb; ++b) {
        twin_steps<F>(x, e, a, c, L.ntp);
        if (b + 1 < nb) {
            const P2 r(s0.renorm(e[0].v.x, e[1].v.x, e[2].v.x), s1.renorm(e[0].v.y, e[1].v.y, e[2].v.y));
            e[0] *= r;
            e[1] *= r;
            e[2] *= r;
        } else {
            s0.last(e[0].v.x, e[1].v.x, e[2].v.x);
            s1.last(e[0].v.y, e[1].v.y, e[2].v.y);
        }
    }
    *outp = s0.result(L.tMax);
    if (outq) *outq = s1.result(L.tMax);
}

// ---------------------------------------------------------------------------
// Two bifurcation / basins points per thread in packed FP32x2 lanes (RK4
// systems). Each lane keeps its own flag, peak detector and outputs and
// follows exactly the scalar FP32 path: a lane that diverges stops recording
// while the pair keeps stepping (its state is then ignored), and the loop
// ends when neither lane is recording.
__device__ __forceinline__ float lane(const P2& v, int l) { return l ? v.v.y : v.v.x; }

template <int NX> __device__ __forceinline__ P2 pick2(const P2* x, int wv) {
    P2 v = x[0];
#pragma unroll
    for (int j = 1; j < NX; ++j)
        if (j == wv) v = x[j];
    return v;
}

// sqrtf(fabsf(sum (x - xp)^2)) < 1e-9 per lane, as bif_fixed<NX, float>
template <int NX> __device__ __forceinline__ bool bif_fixed_lane(const P2* x, const P2* xp, int l) {
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < NX; ++j) {
        const float d = lane(x[j], l) - lane(xp[j], l);
        s = s + d * d;
    }
    return (double)sqrtf(fabsf(s)) < 1e-9;
}
template <int NX> __device__ __forceinline__ bool basins_fixed_lane(const P2* x, const P2* xp, int l) {
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < NX; ++j) {
        const float d = lane(x[j], l) - lane(xp[j], l);
        s = s + d * d;
    }
    return sqrt(fabs((double)s)) < 1e-9;
}

template <class F>
__device__ __forceinline__ void load_pair(const SweepParams& P, long long p0, long long p1, P2* x, P2* a) {
    float xs[2][3], as[2][3];
    load_point<SYS_LORENZ_RK4, float>(P, p0, xs[0], as[0]);  // any 3-state, 3-parameter system loads alike
    load_point<SYS_LORENZ_RK4, float>(P, p1, xs[1], as[1]);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        x[k] = P2(xs[0][k], xs[1][k]);
        a[k] = P2(as[0][k], as[1][k]);
    }
}

// The transient of two bifurcation points in packed FP32x2 lanes, the last
// step peeled off for the fixed-point test; flag[l] (1 on entry for a lane in
// use, 0 otherwise) ends 1, 0 (diverged) or -1 (fixed), as bif_point's.
// Blocks of kTransientBlock steps with one test a block, as in bif_point.
template <class F>
__device__ __forceinline__ void bif_pair_transient(const SweepParams& P, P2* x, const P2* a, int* flag) {
    P2 xp[3];
    const int wv = P.wv;
    if (P.S > 0) {
        const RK4H<P2> c((float)P.h);
        int s = 0;
        {  // blocks of kTransientBlock steps with one test a block, as in bif_point
            constexpr int K = kTransientBlock;
            for (; s + K <= P.S - 1; s += K) {
                bool d0 = false, d1 = false;
#pragma unroll
                for (int j = 0; j < K; ++j) {
                    rk4_step<F>(x, a, c);
                    const P2 v = pick2<3>(x, wv);
                    d0 |= bif_diverged(v.v.x, P);
                    d1 |= bif_diverged(v.v.y, P);
                }
                if (d0) flag[0] = 0;
                if (d1) flag[1] = 0;
                if (flag[0] != 1 && flag[1] != 1) break;
            }
        }
        if (flag[0] == 1 || flag[1] == 1)
            for (; s < P.S - 1; ++s) {  // the last step peeled off, as in bif_point
                rk4_step<F>(x, a, c);
                const P2 v = pick2<3>(x, wv);
                if (flag[0] == 1 && bif_diverged(v.v.x, P)) flag[0] = 0;
                if (flag[1] == 1 && bif_diverged(v.v.y, P)) flag[1] = 0;
                if (flag[0] != 1 && flag[1] != 1) break;
            }
        if (flag[0] == 1 || flag[1] == 1) {
#pragma unroll
            for (int j = 0; j < 3; ++j) xp[j] = x[j];
            rk4_step<F>(x, a, c);
            const P2 v = pick2<3>(x, wv);
            if (flag[0] == 1 && bif_diverged(v.v.x, P)) flag[0] = 0;
            if (flag[1] == 1 && bif_diverged(v.v.y, P)) flag[1] = 0;
#pragma unroll
            for (int l = 0; l < 2; ++l)
                if (flag[l] == 1 && bif_fixed_lane<3>(x, xp, l)) flag[l] = -1;
        }
    }
}

template <class F>
__device__ __forceinline__ void bif_pair_point(const SweepParams& P, const BifOut& O, long long p0, long long p1,
                                               long long o0, long long o1, bool two) {
    P2 x[3], a[3], xp[3];
    load_pair<F>(P, p0, p1, x, a);
    const RK4H<P2> c((float)P.h);
    const int wv = P.wv;
    int flag[2] = {1, two ? 1 : 0};
    bif_pair_transient<F>(P, x, a, flag);
    bool rec[2];
    double first[2] = {0.0, 0.0};  // stays 0 for a lane that does not record (as the scalar path)
    PeakStream<float> ps[2];
#pragma unroll
    for (int l = 0; l < 2; ++l) {
        rec[l] = flag[l] == 1;
        if (!rec[l]) flag[l] = 0;
        ps[l].init();
    }
    const long long oo[2] = {o0, o1};
    if (rec[0] || rec[1]) {
        {
            const P2 v = pick2<3>(x, wv);
            if (rec[0]) first[0] = (double)v.v.x;
            if (rec[1]) first[1] = (double)v.v.y;
        }
        P2 v = pick2<3>(x, wv);  // carried from one step to the next
        auto on_peak = [&](int l, float val, int t) {
            if (ps[l].n >= 1) {
                const int q = ps[l].n - 1;
                if (q < O.cap) {
                    if (O.peaks) O.peaks[oo[l] * O.cap + q] = (double)val;
                    if (O.intervals)
                        O.intervals[oo[l] * O.cap + q] = __dmul_rn((double)(t - ps[l].tprev), P.hInterval);
                }
            }
            ps[l].tprev = t;
            ++ps[l].n;
        };
        int i = 0;
        {  // the block form of bif_record, per lane (a lane that stopped skips its detector)
            constexpr int K = kRecordBlock;
            for (; i + K < P.B; i += K) {
                float s[2][K + 1];
                s[0][0] = v.v.x;
                s[1][0] = v.v.y;
                bool dv[2] = {false, false};
#pragma unroll
                for (int j = 1; j <= K; ++j) {
                    rk4_step<F>(x, a, c);
                    const P2 w = pick2<3>(x, wv);
                    s[0][j] = w.v.x;
                    s[1][j] = w.v.y;
                    dv[0] |= bif_diverged(w.v.x, P);
                    dv[1] |= bif_diverged(w.v.y, P);
                }
#pragma unroll
                for (int l = 0; l < 2; ++l) {
                    if (!rec[l]) continue;
                    if (__builtin_expect(!dv[l], 1)) {
                        ps[l].template push_block<K>(s[l], [&](float val, int t) { on_peak(l, val, t); });
                        continue;
                    }
#pragma unroll
                    for (int j = 0; j < K; ++j) {
                        float val;
                        int t;
                        if (ps[l].push(s[l][j], val, t)) on_peak(l, val, t);
                        if (bif_diverged(s[l][j + 1], P)) break;
                    }
                    rec[l] = false;
                    flag[l] = 0;
                }
                v = P2(s[0][K], s[1][K]);
                if (!rec[0] && !rec[1]) break;
            }
        }
        for (; i < P.B && (rec[0] || rec[1]); ++i) {
#pragma unroll
            for (int j = 0; j < 3; ++j) xp[j] = x[j];
#pragma unroll
            for (int l = 0; l < 2; ++l) {
                float val;
                int t;
                const bool hit = ps[l].push(lane(v, l), val, t);  // a lane that stopped keeps stepping its detector
                if (rec[l] && hit) on_peak(l, val, t);
            }
            rk4_step<F>(x, a, c);
            v = pick2<3>(x, wv);
            if (rec[0] && bif_diverged(v.v.x, P)) { rec[0] = false; flag[0] = 0; }
            if (rec[1] && bif_diverged(v.v.y, P)) { rec[1] = false; flag[1] = 0; }
            if (!rec[0] && !rec[1]) break;
        }
#pragma unroll
        for (int l = 0; l < 2; ++l)
            if (rec[l] && P.B > 0 && bif_fixed_lane<3>(x, xp, l)) flag[l] = -1;
    }
#pragma unroll
    for (int l = 0; l < (two ? 2 : 1); ++l) {
        const int kept = ps[l].n > 1 ? ps[l].n - 1 : 0;
        O.flags[oo[l]] = flag[l];
        O.counts[oo[l]] = flag[l] == 1 ? kept : (flag[l] == -1 ? -1 : 0);
        if (O.first) O.first[oo[l]] = first[l];
    }
}

template <class F, bool PRE1 = false>
__device__ __forceinline__ void basins_pair_point(const SweepParams& P, const BasinsOut& O, long long p0,
                                                  long long p1, long long o0, long long o1, bool two) {
    P2 x[3], a[3], xp[3];
    load_pair<F>(P, p0, p1, x, a);
    const RK4H<P2> c((float)P.h);
    const int wv = P.wv;
    for (int s = 0; s < P.S; ++s) rk4_step<F>(x, a, c);
#pragma unroll
    for (int j = 0; j < 3; ++j) xp[j] = x[j];
    PeakStream<float> ps[2];
    int flag[2] = {1, two ? 1 : 0};
    bool rec[2] = {true, two};
    PeakSums<float> sums[2];
    float lastF[2] = {0.f, 0.f};  // widened after the loop
    ps[0].init();
    ps[1].init();
    P2 v = pick2<3>(x, wv);  // carried from one step to the next
    auto on_peak = [&](int l, float val, int t) {
        if (ps[l].n >= 1) sums[l].add(val, t - ps[l].tprev, P.hInterval);
        ps[l].tprev = t;
        ++ps[l].n;
    };
    int i = 0;
    {  // the block form of basins_record, per lane
        constexpr int K = kRecordBlock;
        for (; i + K < P.B; i += K) {
            float s[2][K + 1];
            s[0][0] = v.v.x;
            s[1][0] = v.v.y;
            bool dv[2] = {false, false};
#pragma unroll
            for (int j = 1; j <= K; ++j) {
                if (PRE1) rk4_step<F>(x, a, c);
                else
                    for (int r = 0; r < P.preScaller; ++r) rk4_step<F>(x, a, c);
                const P2 w = pick2<3>(x, wv);
                s[0][j] = w.v.x;
                s[1][j] = w.v.y;
                dv[0] |= basins_diverged(w.v.x, P);
                dv[1] |= basins_diverged(w.v.y, P);
            }
#pragma unroll
            for (int l = 0; l < 2; ++l) {
                if (!rec[l]) continue;
                if (__builtin_expect(!dv[l], 1)) {
                    ps[l].template push_block<K>(s[l], [&](float val, int t) { on_peak(l, val, t); });
                    lastF[l] = s[l][K - 1];
                    continue;
                }
#pragma unroll
                for (int j = 0; j < K; ++j) {
                    lastF[l] = s[l][j];
                    float val;
                    int t;
                    if (ps[l].push(s[l][j], val, t)) on_peak(l, val, t);
                    if (basins_diverged(s[l][j + 1], P)) break;
                }
                rec[l] = false;
                flag[l] = 0;
            }
            v = P2(s[0][K], s[1][K]);
            if (!rec[0] && !rec[1]) break;
        }
    }
    for (; i < P.B && (rec[0] || rec[1]); ++i) {
#pragma unroll
        for (int j = 0; j < 3; ++j) xp[j] = x[j];
#pragma unroll
        for (int l = 0; l < 2; ++l) {
            if (!rec[l]) continue;
            lastF[l] = lane(v, l);
            float val;
            int t;
            if (ps[l].push(lane(v, l), val, t)) on_peak(l, val, t);
        }
        if (PRE1) rk4_step<F>(x, a, c);
        else
            for (int r = 0; r < P.preScaller; ++r) rk4_step<F>(x, a, c);
        v = pick2<3>(x, wv);
        if (rec[0] && basins_diverged(v.v.x, P)) { rec[0] = false; flag[0] = 0; }
        if (rec[1] && basins_diverged(v.v.y, P)) { rec[1] = false; flag[1] = 0; }
        if (!rec[0] && !rec[1]) break;
    }
    const long long oo[2] = {o0, o1};
    FeatureKeys fk;
#pragma unroll
    for (int l = 0; l < (two ? 2 : 1); ++l) {
        if (rec[l] && P.B > 0 && basins_fixed_lane<3>(x, xp, l)) flag[l] = -1;
        const double last = (double)lastF[l];
        const int kept = ps[l].n > 1 ? ps[l].n - 1 : 0;
        double ap, ai;
        if (flag[l] == 0) { ap = 999.0; ai = 999.0; }
        else if (flag[l] == -1) { ap = last; ai = -1.0; }
        else if (kept <= 0) { ap = 1000.0; ai = 1000.0; }
        else { ap = sums[l].peaks() / (double)kept; ai = sums[l].intervals(P.hInterval) / (double)kept; }
        O.flags[oo[l]] = flag[l];
        O.avgPeaks[oo[l]] = ap;
        O.avgIntervals[oo[l]] = ai;
        if (O.counts) O.counts[oo[l]] = flag[l] == 1 ? kept : 0;
        if (O.last) O.last[oo[l]] = last;
        fk.add(flag[l], flag[l] == 1 ? kept : 0, ap, ai, last);
    }
    if (O.mm) fk.flush(O.mm);
}

// Two basins points per thread, hybrid: the transient (no tests, 80 % of the
// steps of a typical map) runs packed, two trajectories per FP32x2
// instruction; the recorded part then runs lane by lane with the scalar loop,
// whose per-sample peak detector and divergence test a packed loop would have
// to run for both lanes anyway. Bit-identical to basins_point.
template <class F> struct SysOf;
template <> struct SysOf<Lorenz> { static constexpr int S = SYS_LORENZ_RK4; };
template <> struct SysOf<Rossler> { static constexpr int S = SYS_ROSSLER_RK4; };
template <> struct SysOf<Chen> { static constexpr int S = SYS_CHEN_RK4; };

template <class F, bool PRE1 = false>
__device__ __forceinline__ void basins_hybrid_point(const SweepParams& P, const BasinsOut& O, long long p0,
                                                    long long p1, long long o0, long long o1, bool two) {
    P2 x[3], a[3];
    load_pair<F>(P, p0, p1, x, a);
    {
        const RK4H<P2> c((float)P.h);
        for (int s = 0; s < P.S; ++s) rk4_step<F>(x, a, c);
    }
    const StepCtx<float> cs((float)P.h);
#pragma unroll 1
    for (int l = 0; l < (two ? 2 : 1); ++l) {
        float xs[3], as[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            xs[k] = lane(x[k], l);
            as[k] = lane(a[k], l);
        }
        basins_record<SysOf<F>::S, float, PRE1>(P, O, xs, as, cs, l ? o1 : o0);
    }
}

// Two bifurcation points per thread, hybrid: the transient packed (per-lane
// divergence and fixed-point tests, as bif_pair_point), the recorded part lane
// by lane with the scalar loop (bif_record). Bit-identical to bif_point.
template <class F>
__device__ __forceinline__ void bif_hybrid_point(const SweepParams& P, const BifOut& O, long long p0, long long p1,
                                                 long long o0, long long o1, bool two) {
    P2 x[3], a[3];
    load_pair<F>(P, p0, p1, x, a);
    int flag[2] = {1, two ? 1 : 0};
    bif_pair_transient<F>(P, x, a, flag);
    const StepCtx<float> cs((float)P.h);
#pragma unroll 1
    for (int l = 0; l < (two ? 2 : 1); ++l) {
        const long long o = l ? o1 : o0;
        if (flag[l] != 1) {  // diverged or fixed in the transient: reported as diverged
            O.flags[o] = 0;
            O.counts[o] = 0;
            if (O.first) O.first[o] = 0.0;
            continue;
        }
        float xs[3], as[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            xs[k] = lane(x[k], l);
            as[k] = lane(a[k], l);
        }
        bif_record<SysOf<F>::S, float>(P, O, xs, as, cs, P.B, P.hInterval, o);
    }
}

// ---------------------------------------------------------------------------
// Trajectory recorder: nSteps steps of one trajectory per thread, writing the
// state before the first step and after every step.
template <int S, class T>
__device__ __forceinline__ void trajectory_point(const double* x0, const double* a0, double h, int nSteps,
                                                 double* out, long long t) {
    constexpr int NX = Traits<S>::NX, NA = Traits<S>::NA;
    T x[NX], a[NA];
#pragma unroll
    for (int j = 0; j < NX; ++j) x[j] = (T)x0[t * NX + j];
#pragma unroll
    for (int j = 0; j < NA; ++j) a[j] = (T)a0[t * NA + j];
    const StepCtx<T> c((T)h);
    double* o = out + t * (long long)(nSteps + 1) * NX;
#pragma unroll
    for (int j = 0; j < NX; ++j) o[j] = (double)x[j];
    for (int s = 1; s <= nSteps; ++s) {
        step<S>(x, a, c);
#pragma unroll
        for (int j = 0; j < NX; ++j) o[(long long)s * NX + j] = (double)x[j];
    }
}

}  // namespace chaos
