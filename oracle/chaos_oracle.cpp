// CPU oracle for the bifurcation / LLE / basins path.
//
// TEST INFRASTRUCTURE ONLY. This file is the oracle the parity tests, the
// smoke check and the CPU-baseline leg of the benchmark compare the CUDA
// engine against; the engine never calls it and never falls back to it.
//
// It restates the reference's per-point algorithms in plain C++ (FP64,
// compiled with -ffp-contract=off so each rounding is the one written):
//   * loopCalculateDiscreteModel_int, bifurcation flavour
//       Bifurcation/src/bifurcationCUDA.cu:421-467
//   * peakFinder           Bifurcation/src/bifurcationCUDA.cu:469-514
//                          (identical copy: Basins/src/basinsCUDA.cu:382-440)
//   * per-point dbscan + distance  Bifurcation/src/bifurcationCUDA.cu:516-583
//   * getValueByIdx        Bifurcation/src/bifurcationCUDA.cu:400-419,
//                          Basins/src/basinsCUDA.cu:185-189
//   * the bifurcation kernels' control flow
//                          Bifurcation/src/bifurcationCUDA.cu:258-371
//   * LLE transient + Benettin loop   LLE/src/LLECUDA.cu:56-166 (offset: see lle)
//   * linspace             LLE/src/LLECUDA.cu:172-203
//   * basins loop (preScaller, isnan/isinf, sqrt(abs))  Basins/src/basinsCUDA.cu:318-380
//   * avgPeakFinderCUDA    Basins/src/basinsCUDA.cu:818-864
//   * CUDA_dbscan + kernels Basins/src/basinsCUDA.cu:35-179, 866-923
//   * the legacy library's bifurcation loops (grid mode kModeLegacy):
//       calculateDiscreteModelICCUDA  debri/cudaLibrary.cu:1022-1116 (its loop,
//       :604-680, is the basins loop above, token for token), and
//       calculateDiscreteModelCUDA_H :955-1000 over loopCalculateDiscreteModel :472-527
//   * the legacy library's LLE kernels: LLEKernelCUDA debri/cudaLibrary.cu:1897-2031,
//       LLEKernelICCUDA :2034-2139 (orc_lle_sweep_legacy), and its spectrum
//       kernel LSKernelCUDA :2189-2330 (orc_lyapunov_spectrum_legacy)
// Unlike the engine (which streams samples through a peak state machine and
// never stores a trajectory), the oracle records every trajectory into an
// array and scans it exactly as the reference does.
//
// The step maps come from the engine's plug-in header (systems.h): the
// plug-in defines the system being integrated, the same role the reference's
// systems.cuh plays for both its kernels and any host code.
#include "../chaoslibrary_gb300/csrc/systems.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

using chaos::StepCtx;

namespace {

constexpr int kMaxX = 12;  // MAX_REG_SIZE of the reference loop

inline void set_threads(int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
}

// getValueByIdx of the bifurcation/basins kernels: start + n*scale with the
// multiply and the add rounded separately, as written (and as the
// reference's own host code prints the swept value).
inline double grid_value(long long idx, int nPts, double start, double finish, int dim) {
    long long div = 1;
    for (int d = 0; d < dim; ++d) div *= nPts;
    long long n = (idx / div) % nPts;
    double scale = (finish - start) / (double)(nPts - 1);
    return start + (double)n * scale;
}

// Log-scale axis value (the legacy getValueByIdxLog, debri/cudaLibrary.cu:1191-1196:
// log10(start) + n*((log10(finish) - log10(start)) / (nPts - 1))), raised to
// 10^x in FP64, or through powf as the legacy step-size sweep does
// (debri/cudaLibrary.cu:1001: (double)powf(10, x)).
inline double log_value(long long n, int nPts, double start, double finish, bool f32) {
    const double l0 = std::log10(start);
    const double x = l0 + (double)n * ((std::log10(finish) - l0) / (double)(nPts - 1));
    return f32 ? (double)powf(10.0f, (float)x) : std::pow(10.0, x);
}

// Grid modes (the engine's CHAOS_GRID_* bits): initial conditions instead of
// parameters, log-scale dimension 0 / 1, FP32 rounding of log values, the
// legacy library's per-point loop (bifurcation sweeps).
constexpr int kModeState = 1, kModeLog0 = 2, kModeLog1 = 4, kModeLogF32 = 8, kModeLegacy = 16;

// Value of dimension d at grid point idx of a bifurcation-type sweep.
inline double sweep_value(long long idx, int nPts, const double* ranges, int d, int mode) {
    if (!(mode & (d ? kModeLog1 : kModeLog0))) return grid_value(idx, nPts, ranges[2 * d], ranges[2 * d + 1], d);
    long long div = 1;
    for (int k = 0; k < d; ++k) div *= nPts;
    return log_value((idx / div) % nPts, nPts, ranges[2 * d], ranges[2 * d + 1], (mode & kModeLogF32) != 0);
}

// linspace of LLE/src/LLECUDA.cu:172-203 (host code, no contraction).
inline double linspace_value(int i, int num, double start, double end) {
    if (num == 1) return start;
    double step = (end - start) / (num - 1);
    return start + i * step;
}

// loopCalculateDiscreteModel_int, bifurcation flavour. Records x[wv] before
// every step into data (when given). Returns 1 / 0 (diverged) / -1 (fixed point).
int loop_bif(int sys, double* x, const double* a, const StepCtx<double>& c, int iters, int nx, int wv,
             double maxValue, double* data) {
    double xPrev[kMaxX];
    for (int j = 0; j < nx; ++j) xPrev[j] = x[j];
    if (iters <= 0) return 1;  // the reference reads an uninitialised xPrev here
    for (int i = 0; i < iters; ++i) {
        for (int j = 0; j < nx; ++j) xPrev[j] = x[j];
        if (data) data[i] = x[wv];
        chaos::step_dyn(sys, x, a, c);
        double val = x[wv];
        if (val != val || val == val + 1.0) return 0;
        if (maxValue != 0)
            if ((double)fabsf((float)x[wv]) > maxValue) return 0;
    }
    double t = 0;
    for (int j = 0; j < nx; ++j) t += (x[j] - xPrev[j]) * (x[j] - xPrev[j]);
    if ((double)sqrtf(fabsf((float)t)) < 1e-9) return -1;
    return 1;
}

// loopCalculateDiscreteModel_int, basins flavour: preScaller sub-steps per
// recorded sample, isnan/isinf test, FP64 sqrt(abs()) fixed-point test.
int loop_basins(int sys, double* x, const double* a, const StepCtx<double>& c, int iters, int nx,
                int preScaller, int wv, double maxValue, double* data) {
    double xPrev[kMaxX];
    for (int j = 0; j < nx; ++j) xPrev[j] = x[j];
    if (iters <= 0) return 1;
    for (int i = 0; i < iters; ++i) {
        for (int j = 0; j < nx; ++j) xPrev[j] = x[j];
        if (data) data[i] = x[wv];
        for (int j = 0; j < preScaller - 1; ++j) chaos::step_dyn(sys, x, a, c);
        chaos::step_dyn(sys, x, a, c);
        if (std::isnan(x[wv]) || std::isinf(x[wv])) return 0;
        if (maxValue != 0)
            if ((double)fabsf((float)x[wv]) > maxValue) return 0;
    }
    double t = 0;
    for (int j = 0; j < nx; ++j) t += (x[j] - xPrev[j]) * (x[j] - xPrev[j]);
    if (std::sqrt(std::fabs(t)) < 1e-9) return -1;
    return 1;
}

// loopCalculateDiscreteModel of the legacy library (debri/cudaLibrary.cu:472-527),
// the loop of its step-size sweep: x[wv] recorded before preScaller steps,
// isnan/isinf and maxValue tests; a last state change of exactly 0, or of
// norm below 1e-12, ends it as a fixed point. Returns 1 / 0 (diverged) / -1
// (fixed point; the legacy returns false for both).
int loop_legacy_bool(int sys, double* x, const double* a, const StepCtx<double>& c, int iters, int nx,
                     int preScaller, int wv, double maxValue, double* data) {
    double xPrev[kMaxX];
    for (int j = 0; j < nx; ++j) xPrev[j] = x[j];
    if (iters <= 0) return 1;  // the legacy reads an uninitialised xPrev here
    for (int i = 0; i < iters; ++i) {
        for (int j = 0; j < nx; ++j) xPrev[j] = x[j];
        if (data) data[i] = x[wv];
        for (int j = 0; j < preScaller; ++j) chaos::step_dyn(sys, x, a, c);
        if (std::isnan(x[wv]) || std::isinf(x[wv])) return 0;
        if (maxValue != 0)
            if ((double)fabsf((float)x[wv]) > maxValue) return 0;
    }
    double t = 0;
    for (int j = 0; j < nx; ++j) t += (x[j] - xPrev[j]) * (x[j] - xPrev[j]);
    if (t == 0) return -1;
    if (std::sqrt(t) < 1e-12) return -1;
    return 1;
}

// peakFinder over one recorded series d[0..n). Writes the kept peaks (the
// first detected peak is dropped) and the intervals between consecutive
// detected peaks, (t[k+1]-t[k])*h, into peaks/intervals (capacity n each).
// Returns the number kept (0 when fewer than two peaks were detected).
int peak_finder(const double* d, int n, double h, double* peaks, double* times) {
    int cnt = 0;
    for (int i = 1; i < n - 1; ++i) {
        if (d[i] - d[i - 1] > 1e-13 && d[i] >= d[i + 1]) {
            for (int j = i; j < n - 1; ++j) {
                if (d[j] < d[j + 1]) { i = j + 1; break; }
                if (d[j] - d[j + 1] > 1e-13) {
                    peaks[cnt] = d[j];
                    times[cnt] = std::trunc(((double)j + (double)i) / 2.0);
                    ++cnt;
                    i = j + 1;
                    break;
                }
            }
        }
    }
    if (cnt > 1) {
        for (int k = 0; k < cnt - 1; ++k) {
            peaks[k] = peaks[k + 1];
            times[k] = (times[k + 1] - times[k]) * h;
        }
        return cnt - 1;
    }
    return 0;
}

// Per-point dbscan of the 2-D bifurcation (bifurcationCUDA.cu:516-583). The
// amplitudes are zeroed first, so only the intervals matter; the last peak is
// never a neighbour; distance is hypotf(0, dy) = |(float)dy| and the test is
// strict (< eps). The neighbour "stack" writes slot k but pops slot NN-1,
// exactly as the reference does. Returns cluster - 1.
int point_dbscan(const double* iv, int P, double eps, std::vector<int>& lab, std::vector<int>& slot) {
    if (P <= 0) return 0;
    if (P == 1) return 1;
    lab.assign(P, 0);
    slot.assign(P, 0);
    int cluster = 0, nn = 0;
    auto dist = [&](int i, int k) -> double {
        if (iv[i] == iv[k]) return 0.0;
        return (double)fabsf((float)(iv[k] - iv[i]));
    };
    auto expand = [&](int i) {
        for (int k = 0; k < P - 1; ++k)
            if (i != k && lab[k] == 0 && dist(i, k) < eps) { lab[k] = cluster; slot[k] = k; ++nn; }
    };
    for (int i = 0; i < P; ++i) {
        if (nn >= 1) {
            i = slot[nn - 1];
            slot[nn - 1] = 0;
            --nn;
            expand(i);
        } else if (lab[i] == 0) {
            nn = 0;
            ++cluster;
            lab[i] = cluster;
            expand(i);
        }
    }
    return cluster - 1;
}

struct UF {
    std::vector<int> p;
    explicit UF(int n) : p(n) { for (int i = 0; i < n; ++i) p[i] = i; }
    int find(int x) { while (p[x] != x) { p[x] = p[p[x]]; x = p[x]; } return x; }
    void unite(int a, int b) { a = find(a); b = find(b); if (a == b) return; if (a < b) p[b] = a; else p[a] = b; }
};

// Exact (collision-free) integer cell coordinates used as hash-map keys.
struct Cell {
    long long x, y, z;
    bool operator==(const Cell& o) const { return x == o.x && y == o.y && z == o.z; }
};
struct CellHash {
    size_t operator()(const Cell& c) const {
        uint64_t h = (uint64_t)c.x * 0x9E3779B97F4A7C15ull;
        h ^= (uint64_t)c.y + 0x7F4A7C159E3779B9ull + (h << 6) + (h >> 2);
        h ^= (uint64_t)c.z + 0x94D049BB133111EBull + (h << 6) + (h >> 2);
        return (size_t)h;
    }
};
inline Cell cell_key(long long cx, long long cy, long long cz) { return Cell{cx, cy, cz}; }

}  // namespace

extern "C" {

int orc_version() { return 1; }

// nsteps steps of system sys from x (in place), FP64.
void orc_steps(int sys, double* x, const double* a, double h, int nsteps) {
    StepCtx<double> c(h);
    for (int i = 0; i < nsteps; ++i) chaos::step_dyn(sys, x, a, c);
}

// Records nsteps samples of every state component (before each step), FP64.
void orc_trajectory(int sys, const double* x0, const double* a, double h, int nsteps, double* out) {
    StepCtx<double> c(h);
    int nx = chaos::system_nx(sys);
    double x[kMaxX];
    for (int j = 0; j < nx; ++j) x[j] = x0[j];
    for (int i = 0; i < nsteps; ++i) {
        for (int j = 0; j < nx; ++j) out[(size_t)i * nx + j] = x[j];
        chaos::step_dyn(sys, x, a, c);
    }
}

// peakFinder on nSeries independent series of length len (row-major).
// counts[s] = kept peaks; peaks/intervals rows have capacity cap.
void orc_peak_finder(const double* data, int nSeries, int len, double h, int cap, int* counts,
                     double* peaks, double* intervals) {
    std::vector<double> pk(len > 0 ? len : 1), tm(len > 0 ? len : 1);
    for (int s = 0; s < nSeries; ++s) {
        int c = peak_finder(data + (size_t)s * len, len, h, pk.data(), tm.data());
        counts[s] = c;
        for (int k = 0; k < c && k < cap; ++k) {
            peaks[(size_t)s * cap + k] = pk[k];
            intervals[(size_t)s * cap + k] = tm[k];
        }
    }
}

// Per-point dbscan (2-D bifurcation) over given interval series.
void orc_point_dbscan(const double* intervals, const int* counts, int nSeries, int stride, double eps,
                      int* out) {
    std::vector<int> lab, slot;
    for (int s = 0; s < nSeries; ++s) {
        int P = counts[s];
        if (P == -1) { out[s] = -1; continue; }
        if (P == 0) { out[s] = 0; continue; }
        out[s] = point_dbscan(intervals + (size_t)s * stride, P, eps, lab, slot);
    }
}

// Bifurcation sweep over nPts^dim parameter points (dim = 1 or 2), FP64.
// Per point: counts (-1 fixed point, 0 diverged / no peaks, else kept peaks),
// flags (1/0/-1 as the reference's maxValueCheckerArray), first (x[wv] at the
// first recorded sample), the first `cap` peaks and intervals, and for dim 2
// the per-point dbscan result (labels, may be null).
// [pBegin, pEnd) restricts the work to a sub-range of points.
// gridMode: kMode* bits; mut[0] == -1 makes dimension 0 the integration step
// (dim 1): point k runs with its own h_k, (int)(transientTime / h_k)
// transient steps, (int)(tMax / h_k / preScaller) samples, intervals in units
// h_k * preScaller (the legacy step-size sweep, debri/hostLibrary.cu:1005-1240).
// kModeLegacy: the legacy library's per-point loop instead of the current one.
int orc_bifurcation_sweep(int sys, int dim, int gridMode, double tMax, int nPts, double h, const double* ic,
                          const double* ranges, const int* mut, int wv, double maxValue, double transientTime,
                          const double* values, int preScaller, double eps, int cap, long long pBegin,
                          long long pEnd, int* counts, int* flags, double* first, double* peaks, double* intervals,
                          int* labels, int nthreads) {
    const bool stepAxis = mut[0] == -1;
    if (stepAxis && (dim != 1 || !(ranges[0] > 0) || !(ranges[1] > 0))) return 1;
    const double hMin = stepAxis ? std::min(ranges[0], ranges[1]) * (1.0 - 1e-9) : h;
    const int Bmax = (int)(tMax / hMin / preScaller);
    const int nx = chaos::system_nx(sys), na = chaos::system_na(sys);
    long long total = 1;
    for (int d = 0; d < dim; ++d) total *= nPts;
    if (pEnd < 0 || pEnd > total) pEnd = total;
    if (Bmax < 1 || nx > kMaxX) return 1;
    set_threads(nthreads);
#pragma omp parallel
    {
        std::vector<double> data(Bmax + 1), pk(Bmax + 1), tm(Bmax + 1);
        std::vector<int> lab, slot;
#pragma omp for schedule(dynamic, 4)
        for (long long p = pBegin; p < pEnd; ++p) {
            const long long o = p - pBegin;
            double x[kMaxX], a[32];
            for (int j = 0; j < nx; ++j) x[j] = ic[j];
            for (int j = 0; j < na; ++j) a[j] = values[j];
            double hp = h;
            for (int d = 0; d < dim; ++d) {
                const double v = sweep_value(p, nPts, ranges, d, gridMode);
                if (d == 0 && stepAxis) hp = v;
                else if (gridMode & kModeState) x[mut[d]] = v;
                else a[mut[d]] = v;
            }
            const int B = (int)(tMax / hp / preScaller);
            const int S = (int)(transientTime / hp);
            const StepCtx<double> c(hp);
            const double hh = hp * (double)preScaller;
            int flag;
            if (gridMode & kModeLegacy) {
                // the legacy kernels: calculateDiscreteModelICCUDA (debri/cudaLibrary.cu:1022-1116) runs
                // its transient with preScaller 1, writableVar 0 and no bound and stops the point only
                // when it diverged; calculateDiscreteModelCUDA_H (:955-1000) ignores the transient's verdict
                flag = 1;
                if (stepAxis) loop_legacy_bool(sys, x, a, c, S, nx, 1, 0, 0.0, nullptr);
                else if (loop_basins(sys, x, a, c, S, nx, 1, 0, 0.0, nullptr) == 0) flag = 0;
                if (flag == 1 && B >= 1)
                    flag = stepAxis ? loop_legacy_bool(sys, x, a, c, B, nx, preScaller, wv, maxValue, data.data())
                                    : loop_basins(sys, x, a, c, B, nx, preScaller, wv, maxValue, data.data());
            } else {
                flag = loop_bif(sys, x, a, c, S, nx, wv, maxValue, nullptr);
                if (B < 1) flag = flag == 1 ? 1 : 0;
                else if (flag == 1) flag = loop_bif(sys, x, a, c, B, nx, wv, maxValue, data.data());
                else flag = 0;
            }
            if (B < 1) {  // no recorded sample: the transient decides alone
                flags[o] = flag;
                first[o] = 0.0;
                counts[o] = 0;
                if (labels) labels[o] = 0;
                continue;
            }
            flags[o] = flag;
            first[o] = (flag == -1) ? data[0] : 0.0;
            int cnt;
            if (flag == -1) cnt = -1;
            else if (flag == 0) cnt = 0;
            else cnt = peak_finder(data.data(), B, hh, pk.data(), tm.data());
            counts[o] = cnt;
            for (int k = 0; k < cnt && k < cap; ++k) {
                peaks[o * cap + k] = pk[k];
                intervals[o * cap + k] = tm[k];
            }
            if (labels) {
                if (cnt == -1) labels[o] = -1;
                else if (cnt == 0) labels[o] = 0;
                else labels[o] = point_dbscan(tm.data(), cnt, eps, lab, slot);
            }
        }
    }
    return 0;
}

// Bifurcation sweep over nPts^dim parameter points: orc_bifurcation_sweep with gridMode 0.
int orc_bifurcation(int sys, int dim, double tMax, int nPts, double h, const double* ic, const double* ranges,
                    const int* mut, int wv, double maxValue, double transientTime, const double* values,
                    int preScaller, double eps, int cap, long long pBegin, long long pEnd, int* counts, int* flags,
                    double* first, double* peaks, double* intervals, int* labels, int nthreads) {
    if ((int)(tMax / h / preScaller) < 1) return 1;
    return orc_bifurcation_sweep(sys, dim, 0, tMax, nPts, h, ic, ranges, mut, wv, maxValue, transientTime, values,
                                 preScaller, eps, cap, pBegin, pEnd, counts, flags, first, peaks, intervals, labels,
                                 nthreads);
}

// LLE map, FP64, the reference's Benettin scheme (LLECUDA.cu:114-166):
// calcBlocks+1 blocks of NT steps of x and of its twin p, d = |x-p|/eps,
// sum += log(d), p = x - (x-p)/d, result sum / tMax. The twin starts at
// x + eps * e_x (the reference draws a random unit offset with cuRAND).
// out[j*nPts + i] is the point (A = linspace A[i], B = linspace B[j]), the
// CSV's transposed layout (row = B index).
int orc_lle2d(int sys, double tMax, double NT, int nPts, double h, double eps, const double* ic,
              const double* ranges, const int* mut, double transientTime, const double* values,
              long long pBegin, long long pEnd, double* out, int nthreads) {
    const int ntp = (int)(NT / h);
    const int trans = (int)(transientTime / h);
    const int all = (int)(tMax / h);
    if (ntp <= 0) return 1;
    const int calcBlocks = all / ntp + 1;
    const int nx = chaos::system_nx(sys), na = chaos::system_na(sys);
    const long long total = (long long)nPts * nPts;
    if (pEnd < 0 || pEnd > total) pEnd = total;
    set_threads(nthreads);
    const StepCtx<double> c(h);
#pragma omp parallel for schedule(dynamic, 4)
    for (long long p = pBegin; p < pEnd; ++p) {
        const int i = (int)(p % nPts), j = (int)(p / nPts);
        double x[kMaxX], q[kMaxX], a[32];
        for (int k = 0; k < nx; ++k) x[k] = ic[k];
        for (int k = 0; k < na; ++k) a[k] = values[k];
        a[mut[0]] = linspace_value(i, nPts, ranges[0], ranges[1]);
        a[mut[1]] = linspace_value(j, nPts, ranges[2], ranges[3]);
        for (int s = 0; s < trans; ++s) chaos::step_dyn(sys, x, a, c);
        for (int k = 0; k < nx; ++k) q[k] = x[k];
        q[0] = x[0] + eps;
        double sum = 0.0;
        for (int b = 0; b <= calcBlocks; ++b) {
            for (int s = 0; s < ntp; ++s) chaos::step_dyn(sys, x, a, c);
            for (int s = 0; s < ntp; ++s) chaos::step_dyn(sys, q, a, c);
            double dist = 0.0;
            for (int k = 0; k < nx; ++k) { double df = x[k] - q[k]; dist += df * df; }
            dist = std::sqrt(dist) / eps;
            sum += std::log(dist);
            for (int k = 0; k < nx; ++k) q[k] = x[k] - ((x[k] - q[k]) / dist);
        }
        out[p - pBegin] = sum / tMax;
    }
    return 0;
}

// Grid point p of an LLE-type sweep (1-D: p = i; 2-D: p = j*nPts + i) over
// parameters or initial conditions (kModeState), linspace or log-scale axes;
// dimension 1 last.
static void lle_grid_point(int dim, int gridMode, long long p, int nPts, const double* ranges, const int* mut,
                           double* x, double* a) {
    const int i = dim == 1 ? (int)p : (int)(p % nPts), j = dim == 1 ? 0 : (int)(p / nPts);
    double* tgt = (gridMode & kModeState) ? x : a;
    const bool f32 = (gridMode & kModeLogF32) != 0;
    tgt[mut[0]] = (gridMode & kModeLog0) ? log_value(i, nPts, ranges[0], ranges[1], f32)
                                         : linspace_value(i, nPts, ranges[0], ranges[1]);
    if (dim == 2)
        tgt[mut[1]] = (gridMode & kModeLog1) ? log_value(j, nPts, ranges[2], ranges[3], f32)
                                             : linspace_value(j, nPts, ranges[2], ranges[3]);
}

// LLE over 1-D / 2-D grids of parameters or initial conditions: the scheme
// of orc_lle2d (which is dim 2, gridMode 0) at every grid point.
int orc_lle_sweep(int sys, int dim, int gridMode, double tMax, double NT, int nPts, double h, double eps,
                  const double* ic, const double* ranges, const int* mut, double transientTime,
                  const double* values, long long pBegin, long long pEnd, double* out, int nthreads) {
    const int ntp = (int)(NT / h);
    const int trans = (int)(transientTime / h);
    const int all = (int)(tMax / h);
    if (ntp <= 0 || (dim != 1 && dim != 2)) return 1;
    const int calcBlocks = all / ntp + 1;
    const int nx = chaos::system_nx(sys), na = chaos::system_na(sys);
    const long long total = dim == 2 ? (long long)nPts * nPts : nPts;
    if (pEnd < 0 || pEnd > total) pEnd = total;
    set_threads(nthreads);
    const StepCtx<double> c(h);
#pragma omp parallel for schedule(dynamic, 4)
    for (long long p = pBegin; p < pEnd; ++p) {
        double x[kMaxX], q[kMaxX], a[32];
        for (int k = 0; k < nx; ++k) x[k] = ic[k];
        for (int k = 0; k < na; ++k) a[k] = values[k];
        lle_grid_point(dim, gridMode, p, nPts, ranges, mut, x, a);
        for (int s = 0; s < trans; ++s) chaos::step_dyn(sys, x, a, c);
        for (int k = 0; k < nx; ++k) q[k] = x[k];
        q[0] = x[0] + eps;
        double sum = 0.0;
        for (int b = 0; b <= calcBlocks; ++b) {
            for (int s = 0; s < ntp; ++s) chaos::step_dyn(sys, x, a, c);
            for (int s = 0; s < ntp; ++s) chaos::step_dyn(sys, q, a, c);
            double dist = 0.0;
            for (int k = 0; k < nx; ++k) { double df = x[k] - q[k]; dist += df * df; }
            dist = std::sqrt(dist) / eps;
            sum += std::log(dist);
            for (int k = 0; k < nx; ++k) q[k] = x[k] - ((x[k] - q[k]) / dist);
        }
        out[p - pBegin] = sum / tMax;
    }
    return 0;
}

// loopCalculateDiscreteModel (debri/cudaLibrary.cu:472-527) as the legacy
// LLE kernels call it: n steps, preScaller 1, writableVar 0, no samples; it
// stops early when x[0] is NaN or infinite or |(float)x[0]| > maxValue
// (maxValue != 0), and its verdict is not used.
static void legacy_lle_run(int sys, double* x, const double* a, const StepCtx<double>& c, int n, double maxValue) {
    for (int s = 0; s < n; ++s) {
        chaos::step_dyn(sys, x, a, c);
        if (std::isnan(x[0]) || std::isinf(x[0])) return;
        if (maxValue != 0)
            if ((double)fabsf((float)x[0]) > maxValue) return;
    }
}

// The legacy library's LLE analyses with its own kernels' scheme:
// LLEKernelCUDA (debri/cudaLibrary.cu:1897-2031; parameter grids, LLE1D) and
// LLEKernelICCUDA (:2034-2139; grids of initial conditions, kModeState, LLE1DIC
// / LLE2DIC). draws[p*nx + k]: the raw twin draws of point p before
// normalisation; null is allowed for the initial-condition grids, whose draw
// is restated from the kernel: 0.5 * sinf(p * (k*p + 1) + 1) in 32-bit
// wrap-around arithmetic, through the C library's sinf. The parameter grids'
// draws come from cuRAND in the legacy kernel and must be given.
// (int)(tMax / NT) blocks of (int)(NT / h) steps; out[p - pBegin].
int orc_lle_sweep_legacy(int sys, int dim, int gridMode, double tMax, double NT, int nPts, double h, double eps,
                         const double* ic, const double* ranges, const int* mut, double maxValue,
                         double transientTime, const double* values, const double* draws, long long pBegin,
                         long long pEnd, double* out, int nthreads) {
    const int ntp = (int)(NT / h);
    const int trans = (int)(transientTime / h);
    const int blocks = (int)(tMax / NT);
    const bool state = (gridMode & kModeState) != 0;
    if (ntp < 0 || (dim != 1 && dim != 2) || (!state && !draws)) return 1;
    const int nx = chaos::system_nx(sys), na = chaos::system_na(sys);
    const long long total = dim == 2 ? (long long)nPts * nPts : nPts;
    if (pEnd < 0 || pEnd > total) pEnd = total;
    set_threads(nthreads);
    const StepCtx<double> c(h);
#pragma omp parallel for schedule(dynamic, 4)
    for (long long p = pBegin; p < pEnd; ++p) {
        double x[kMaxX], y[kMaxX], z[kMaxX], a[32];
        for (int k = 0; k < nx; ++k) x[k] = ic[k];
        for (int k = 0; k < na; ++k) a[k] = values[k];
        lle_grid_point(dim, gridMode, p, nPts, ranges, mut, x, a);
        double zp = 0;
        for (int k = 0; k < nx; ++k) {
            if (draws) {
                z[k] = draws[p * nx + k];
            } else {
                const uint32_t i = (uint32_t)p;
                const int32_t arg = (int32_t)(i * ((uint32_t)k * i + 1u) + 1u);
                z[k] = 0.5 * (double)sinf((float)arg);
            }
            zp += z[k] * z[k];
        }
        zp = std::sqrt(zp);
        for (int k = 0; k < nx; ++k) z[k] = z[k] / zp;
        legacy_lle_run(sys, x, a, c, trans, maxValue);
        for (int k = 0; k < nx; ++k) y[k] = x[k] + z[k] * eps;
        double result = 0;
        for (int b = 0; b < blocks; ++b) {
            legacy_lle_run(sys, x, a, c, ntp, maxValue);
            legacy_lle_run(sys, y, a, c, ntp, maxValue);
            double d = 0;
            if (!state) {  // LLEKernelCUDA
                for (int k = 0; k < nx; ++k) {
                    double t2 = 1 / eps;
                    t2 = t2 * (x[k] - y[k]);
                    d += t2 * t2;
                }
                d = std::sqrt(d);
                result += std::log(d);
                for (int k = 0; k < nx; ++k) y[k] = x[k] - ((x[k] - y[k]) / d);
            } else {  // LLEKernelICCUDA
                for (int k = 0; k < nx; ++k) d += (x[k] - y[k]) * (x[k] - y[k]);
                d = std::sqrt(d) / eps;
                result += std::log(d);
                if (d != 0) d = 1 / d;
                for (int k = 0; k < nx; ++k) y[k] = x[k] - ((x[k] - y[k]) * d);
            }
        }
        out[p - pBegin] = result / tMax;
    }
    return 0;
}

// Lyapunov spectrum (the legacy library's LSKernelCUDA scheme,
// debri/cudaLibrary.cu:2141-2330, with the LLE map's block count): one twin
// per dimension from x + eps e_j; after every block of NT steps the twin
// differences go through classical Gram-Schmidt, exponent j adds
// log(|b_j| / eps) and twin j restarts at x + eps b_j/|b_j|.
// out[(p - pBegin)*nx + j].
int orc_lyapunov_spectrum(int sys, int dim, int gridMode, double tMax, double NT, int nPts, double h,
                          double eps, const double* ic, const double* ranges, const int* mut, double transientTime,
                          const double* values, long long pBegin, long long pEnd, double* out, int nthreads) {
    const int ntp = (int)(NT / h);
    const int trans = (int)(transientTime / h);
    const int all = (int)(tMax / h);
    if (ntp <= 0 || (dim != 1 && dim != 2)) return 1;
    const int calcBlocks = all / ntp + 1;
    const int nx = chaos::system_nx(sys), na = chaos::system_na(sys);
    const long long total = dim == 2 ? (long long)nPts * nPts : nPts;
    if (pEnd < 0 || pEnd > total) pEnd = total;
    set_threads(nthreads);
    const StepCtx<double> c(h);
#pragma omp parallel for schedule(dynamic, 4)
    for (long long p = pBegin; p < pEnd; ++p) {
        double x[kMaxX], y[kMaxX][kMaxX], a[32], sum[kMaxX];
        for (int k = 0; k < nx; ++k) x[k] = ic[k];
        for (int k = 0; k < na; ++k) a[k] = values[k];
        lle_grid_point(dim, gridMode, p, nPts, ranges, mut, x, a);
        for (int s = 0; s < trans; ++s) chaos::step_dyn(sys, x, a, c);
        for (int j = 0; j < nx; ++j) {
            sum[j] = 0.0;
            for (int i = 0; i < nx; ++i) y[j][i] = i == j ? x[i] + eps : x[i];
        }
        for (int b = 0; b <= calcBlocks; ++b) {
            for (int s = 0; s < ntp; ++s) chaos::step_dyn(sys, x, a, c);
            for (int j = 0; j < nx; ++j)
                for (int s = 0; s < ntp; ++s) chaos::step_dyn(sys, y[j], a, c);
            double d[kMaxX][kMaxX], g[kMaxX][kMaxX];
            for (int j = 0; j < nx; ++j) {
                for (int i = 0; i < nx; ++i) {
                    d[j][i] = y[j][i] - x[i];
                    g[j][i] = d[j][i];
                }
                for (int m = 0; m < j; ++m) {
                    double num = 0.0, den = 0.0;
                    for (int i = 0; i < nx; ++i) {
                        num += d[j][i] * g[m][i];
                        den += g[m][i] * g[m][i];
                    }
                    const double frac = den == 0.0 ? 0.0 : num / den;
                    for (int i = 0; i < nx; ++i) g[j][i] -= frac * g[m][i];
                }
            }
            for (int j = 0; j < nx; ++j) {
                double n2 = 0.0;
                for (int i = 0; i < nx; ++i) n2 += g[j][i] * g[j][i];
                const double nrm = std::sqrt(n2);
                sum[j] += std::log(nrm / eps);
                for (int i = 0; i < nx; ++i) y[j][i] = x[i] + (nrm == 0.0 ? 0.0 : g[j][i] / nrm) * eps;
            }
        }
        for (int j = 0; j < nx; ++j) out[(p - pBegin) * nx + j] = sum[j] / tMax;
    }
    return 0;
}

// Classical Gram-Schmidt of the rows of v (n x n), as gramSchmidtProcess
// (debri/cudaLibrary.cu:2141-2187): w_j = v_j minus its projections
// <v_j, w_m>/<w_m, w_m> w_m on the earlier w_m, u_j = w_j/|w_j| (0 for a zero
// w_j), nrm[j] = |w_j|.
static void gram_schmidt(const double (*v)[kMaxX], double (*u)[kMaxX], double* nrm, int n) {
    double w[kMaxX][kMaxX];
    for (int j = 0; j < n; ++j) {
        for (int i = 0; i < n; ++i) w[j][i] = v[j][i];
        for (int m = 0; m < j; ++m) {
            double num = 0.0, den = 0.0;
            for (int i = 0; i < n; ++i) {
                num += v[j][i] * w[m][i];
                den += w[m][i] * w[m][i];
            }
            const double frac = den == 0.0 ? 0.0 : num / den;
            for (int i = 0; i < n; ++i) w[j][i] -= frac * w[m][i];
        }
    }
    for (int j = 0; j < n; ++j) {
        double n2 = 0.0;
        for (int i = 0; i < n; ++i) n2 += w[j][i] * w[j][i];
        nrm[j] = std::sqrt(n2);
        for (int i = 0; i < n; ++i) u[j][i] = nrm[j] == 0.0 ? 0.0 : w[j][i] / nrm[j];
    }
}

// The legacy library's LS1D / LS2D with its own kernel's scheme
// (LSKernelCUDA, debri/cudaLibrary.cu:2189-2330): twin j along row j of the
// raw draws (draws[(p*nx + j)*nx + i]; null: restated from the kernel, 0.5 *
// sinf((float)(0.2171828 (i+1)(j+1) + p + (0.2171828 + i j p))) through the
// C library's sinf), each row normalised; after the transient the rows
// orthonormalised and twin j started at x + eps u_j; (int)(tMax / NT) blocks
// of (int)(NT / h) steps (runs stopping early as legacy_lle_run), the
// differences through Gram-Schmidt, exponent j adding log(|w_j| / eps) and
// twin j restarting at x + eps u_j; sums / tMax. out[(p - pBegin)*nx + j].
int orc_lyapunov_spectrum_legacy(int sys, int dim, int gridMode, double tMax, double NT, int nPts, double h,
                                 double eps, const double* ic, const double* ranges, const int* mut, double maxValue,
                                 double transientTime, const double* values, const double* draws, long long pBegin,
                                 long long pEnd, double* out, int nthreads) {
    const int ntp = (int)(NT / h);
    const int trans = (int)(transientTime / h);
    const int blocks = (int)(tMax / NT);
    if (ntp < 0 || (dim != 1 && dim != 2)) return 1;
    const int nx = chaos::system_nx(sys), na = chaos::system_na(sys);
    const long long total = dim == 2 ? (long long)nPts * nPts : nPts;
    if (pEnd < 0 || pEnd > total) pEnd = total;
    set_threads(nthreads);
    const StepCtx<double> c(h);
#pragma omp parallel for schedule(dynamic, 4)
    for (long long p = pBegin; p < pEnd; ++p) {
        double x[kMaxX], y[kMaxX][kMaxX], z[kMaxX][kMaxX], a[32], sum[kMaxX], nrm[kMaxX];
        for (int k = 0; k < nx; ++k) x[k] = ic[k];
        for (int k = 0; k < na; ++k) a[k] = values[k];
        lle_grid_point(dim, gridMode, p, nPts, ranges, mut, x, a);
        const int idx = (int)p;
        for (int j = 0; j < nx; ++j) {
            double zp = 0;
            for (int i = 0; i < nx; ++i) {
                if (draws) {
                    z[j][i] = draws[(p * nx + j) * nx + i];
                } else {
                    const double arg = 0.2171828 * (i + 1) * (j + 1) + idx + (0.2171828 + i * j * idx);
                    z[j][i] = (double)sinf((float)arg) * 0.5;
                }
                zp += z[j][i] * z[j][i];
            }
            zp = std::sqrt(zp);
            for (int i = 0; i < nx; ++i) z[j][i] = z[j][i] / zp;
        }
        legacy_lle_run(sys, x, a, c, trans, maxValue);
        gram_schmidt(z, y, nrm, nx);
        for (int j = 0; j < nx; ++j) {
            sum[j] = 0.0;
            for (int i = 0; i < nx; ++i) y[j][i] = y[j][i] * eps + x[i];
        }
        for (int b = 0; b < blocks; ++b) {
            legacy_lle_run(sys, x, a, c, ntp, maxValue);
            for (int j = 0; j < nx; ++j) legacy_lle_run(sys, y[j], a, c, ntp, maxValue);
            for (int j = 0; j < nx; ++j)
                for (int i = 0; i < nx; ++i) y[j][i] = y[j][i] - x[i];
            gram_schmidt(y, z, nrm, nx);
            for (int j = 0; j < nx; ++j) {
                sum[j] += std::log(nrm[j] / eps);
                for (int i = 0; i < nx; ++i) y[j][i] = x[i] + z[j][i] * eps;
            }
        }
        for (int j = 0; j < nx; ++j) out[(p - pBegin) * nx + j] = sum[j] / tMax;
    }
    return 0;
}

// Basins features over the nPts^2 grid of initial conditions
// (Basins/src/basinsCUDA.cu:233-314 + 818-864): flags, avgPeaks, avgIntervals
// (the reference's sentinels: flag 0 -> 999/999, flag -1 -> last sample/-1,
// no peaks -> 1000/1000), the kept peak count (counts, may be null) and the
// last recorded sample (last, may be null; meaningful for flag != 0).
int orc_basins_features(int sys, double tMax, int nPts, double h, const double* ic, const double* ranges,
                        const int* mut, int wv, double maxValue, double transientTime, const double* values,
                        int preScaller, long long pBegin, long long pEnd, int* flags, double* avgPeaks,
                        double* avgIntervals, int* counts, double* last, int nthreads) {
    const int B = (int)(tMax / h / preScaller);
    const int S = (int)(transientTime / h);
    const int nx = chaos::system_nx(sys), na = chaos::system_na(sys);
    const long long total = (long long)nPts * nPts;
    if (pEnd < 0 || pEnd > total) pEnd = total;
    if (B < 1) return 1;
    set_threads(nthreads);
    const StepCtx<double> c(h);
    const double hh = h * (double)preScaller;
#pragma omp parallel
    {
        std::vector<double> data(B), pk(B), tm(B);
#pragma omp for schedule(dynamic, 4)
        for (long long p = pBegin; p < pEnd; ++p) {
            const long long o = p - pBegin;
            double x[kMaxX], a[32];
            for (int k = 0; k < nx; ++k) x[k] = ic[k];
            for (int k = 0; k < na; ++k) a[k] = values[k];
            for (int d = 0; d < 2; ++d) x[mut[d]] = grid_value(p, nPts, ranges[2 * d], ranges[2 * d + 1], d);
            for (int s = 0; s < S; ++s) chaos::step_dyn(sys, x, a, c);
            int flag = loop_basins(sys, x, a, c, B, nx, preScaller, wv, maxValue, data.data());
            flags[o] = flag;
            int cnt = 0;
            if (flag == 0) { avgPeaks[o] = 999; avgIntervals[o] = 999; }
            else if (flag == -1) { avgPeaks[o] = data[B - 1]; avgIntervals[o] = -1.0; }
            else {
                cnt = peak_finder(data.data(), B, hh, pk.data(), tm.data());
                if (cnt <= 0) { avgPeaks[o] = 1000; avgIntervals[o] = 1000; }
                else {
                    double sp = 0, si = 0;
                    for (int k = 0; k < cnt; ++k) { sp += pk[k]; si += tm[k]; }
                    avgPeaks[o] = sp / cnt;
                    avgIntervals[o] = si / cnt;
                }
            }
            if (counts) counts[o] = cnt;
            if (last) last[o] = data[flag == 0 ? 0 : B - 1];
        }
    }
    return 0;
}

// The reference's global DBSCAN (CUDA_dbscan, basinsCUDA.cu:35-179), run as
// written: repeatedly take an unlabelled fixed-point seed (flag -1) and give
// its component the next negative id, else an unlabelled flag-1 seed and the
// next positive id, else stop; expand breadth-first over points within
// sqrt(dp^2 + di^2) <= eps; a reached flag-0 point is reset to 0 and not
// expanded. The reference picks a racy seed; here it is the smallest index.
// O(n^2): for small inputs.
void orc_dbscan_compat_bfs(const double* ap, const double* ai, const int* flags, int n, double eps, int* labels) {
    for (int i = 0; i < n; ++i) labels[i] = 0;
    int pos = 0, neg = 0;
    std::vector<int> queue;
    while (true) {
        int seed = -1, id = 0;
        for (int i = 0; i < n; ++i) if (flags[i] == -1 && labels[i] == 0) { seed = i; break; }
        if (seed >= 0) id = --neg;
        else {
            for (int i = 0; i < n; ++i) if (labels[i] == 0 && flags[i] == 1) { seed = i; break; }
            if (seed < 0) break;
            id = ++pos;
        }
        queue.clear();
        queue.push_back(seed);
        labels[seed] = id;
        for (size_t q = 0; q < queue.size(); ++q) {
            int cur = queue[q];
            labels[cur] = id;
            if (flags[cur] == 0) { labels[cur] = 0; continue; }
            for (int k = 0; k < n; ++k) {
                if (labels[k] != 0 || k == cur) continue;
                double dp = ap[cur] - ap[k], di = ai[cur] - ai[k];
                if (std::sqrt(dp * dp + di * di) <= eps) { labels[k] = id; queue.push_back(k); }
            }
        }
    }
}

// Same partition and numbering as orc_dbscan_compat_bfs, grid-accelerated so
// that millions of points finish: cells of side eps/1.5 (any two points of a
// cell are within eps), union-find over cells, exact point-pair tests between
// cells at most 2 cells apart. Negative ids are numbered by the smallest
// fixed-point member index, positive ids by the smallest member index.
void orc_dbscan_compat_grid(const double* ap, const double* ai, const int* flags, int n, double eps, int* labels) {
    const double side = eps / 1.5;
    std::vector<Cell> key(n);
    std::vector<int> order;
    order.reserve(n);
    for (int i = 0; i < n; ++i) {
        labels[i] = 0;
        if (flags[i] == 0) continue;
        long long cx = (long long)std::floor(ap[i] / side), cy = (long long)std::floor(ai[i] / side);
        key[i] = cell_key(cx, cy, 0);
        order.push_back(i);
    }
    std::sort(order.begin(), order.end(), [&](int a, int b) {
        if (key[a].x != key[b].x) return key[a].x < key[b].x;
        if (key[a].y != key[b].y) return key[a].y < key[b].y;
        return a < b;
    });
    std::vector<int> cstart;
    std::unordered_map<Cell, int, CellHash> cid;
    for (size_t t = 0; t < order.size(); ++t)
        if (t == 0 || !(key[order[t]] == key[order[t - 1]])) { cid[key[order[t]]] = (int)cstart.size(); cstart.push_back((int)t); }
    const int nc = (int)cstart.size();
    cstart.push_back((int)order.size());
    UF uf(nc);
    for (int c = 0; c < nc; ++c) {
        int p0 = order[cstart[c]];
        long long cx = (long long)std::floor(ap[p0] / side), cy = (long long)std::floor(ai[p0] / side);
        for (int dx = -2; dx <= 2; ++dx)
            for (int dy = -2; dy <= 2; ++dy) {
                auto it = cid.find(cell_key(cx + dx, cy + dy, 0));
                if (it == cid.end()) continue;
                int c2 = it->second;
                if (c2 <= c || uf.find(c) == uf.find(c2)) continue;
                bool hit = false;
                for (int s = cstart[c]; s < cstart[c + 1] && !hit; ++s)
                    for (int t = cstart[c2]; t < cstart[c2 + 1]; ++t) {
                        int i = order[s], k = order[t];
                        double dp = ap[i] - ap[k], di = ai[i] - ai[k];
                        if (std::sqrt(dp * dp + di * di) <= eps) { hit = true; break; }
                    }
                if (hit) uf.unite(c, c2);
            }
    }
    // per component: smallest member, smallest fixed-point member
    std::vector<int> minAll(nc, n), minFix(nc, n);
    std::vector<int> comp(n, -1);
    for (int c = 0; c < nc; ++c) {
        int r = uf.find(c);
        for (int s = cstart[c]; s < cstart[c + 1]; ++s) {
            int i = order[s];
            comp[i] = r;
            minAll[r] = std::min(minAll[r], i);
            if (flags[i] == -1) minFix[r] = std::min(minFix[r], i);
        }
    }
    std::vector<std::pair<int, int>> negs, poss;
    for (int c = 0; c < nc; ++c) {
        if (uf.find(c) != c) continue;
        if (minFix[c] < n) negs.push_back({minFix[c], c});
        else poss.push_back({minAll[c], c});
    }
    std::sort(negs.begin(), negs.end());
    std::sort(poss.begin(), poss.end());
    std::vector<int> id(nc, 0);
    for (size_t t = 0; t < negs.size(); ++t) id[negs[t].second] = -(int)(t + 1);
    for (size_t t = 0; t < poss.size(); ++t) id[poss[t].second] = (int)(t + 1);
    for (int i = 0; i < n; ++i) if (comp[i] >= 0) labels[i] = id[comp[i]];
}

// Textbook DBSCAN with scikit-learn's semantics on an n x d feature matrix
// (row-major), d <= 3: a point is core when at least minPts points (itself
// included) lie within distance <= eps; clusters are the eps-connected
// components of core points, numbered 0,1,... in order of their smallest core
// index; a non-core point within eps of core points joins the cluster with
// the smallest number among them; the rest are noise (-1). Points with
// mask[i] == 0 take part in nothing and get label -2 (mask may be null).
// Grid-accelerated (cells of side just above eps).
void orc_dbscan(const double* f, int n, int d, double eps, int minPts, const int* mask, int* labels) {
    auto dist_ok = [&](int i, int k) {
        double s = 0;
        for (int t = 0; t < d; ++t) { double df = f[(size_t)i * d + t] - f[(size_t)k * d + t]; s += df * df; }
        return std::sqrt(s) <= eps;
    };
    const double side = eps * 1.000001;  // |a-b| <= eps  =>  cell coordinates differ by at most 1
    std::vector<long long> cc(3 * (size_t)n, 0);
    std::unordered_map<Cell, std::vector<int>, CellHash> cells;
    for (int i = 0; i < n; ++i) {
        if (mask && !mask[i]) continue;
        long long c3[3] = {0, 0, 0};
        for (int t = 0; t < d; ++t) c3[t] = (long long)std::floor(f[(size_t)i * d + t] / side);
        for (int t = 0; t < 3; ++t) cc[3 * (size_t)i + t] = c3[t];
        cells[cell_key(c3[0], c3[1], c3[2])].push_back(i);
    }
    const int r1 = 1, rz = d >= 3 ? 1 : 0, ry = d >= 2 ? 1 : 0;
    auto for_nbrs = [&](int i, auto&& fn) {
        for (int dx = -r1; dx <= r1; ++dx)
            for (int dy = -ry; dy <= ry; ++dy)
                for (int dz = -rz; dz <= rz; ++dz) {
                    auto it = cells.find(cell_key(cc[3 * (size_t)i] + dx, cc[3 * (size_t)i + 1] + dy, cc[3 * (size_t)i + 2] + dz));
                    if (it == cells.end()) continue;
                    for (int k : it->second) if (dist_ok(i, k)) fn(k);
                }
    };
    std::vector<char> core(n, 0);
    for (int i = 0; i < n; ++i) {
        if (mask && !mask[i]) continue;
        int cnt = 0;
        for_nbrs(i, [&](int) { ++cnt; });
        core[i] = cnt >= minPts;
    }
    UF uf(n);
    for (int i = 0; i < n; ++i)
        if (core[i]) for_nbrs(i, [&](int k) { if (core[k]) uf.unite(i, k); });
    // cluster number = rank of the component's smallest core index (= its UF root)
    std::vector<int> num(n, -1);
    int next = 0;
    for (int i = 0; i < n; ++i) if (core[i] && uf.find(i) == i) num[i] = next++;
    for (int i = 0; i < n; ++i) {
        if (mask && !mask[i]) { labels[i] = -2; continue; }
        if (core[i]) { labels[i] = num[uf.find(i)]; continue; }
        int best = -1;
        for_nbrs(i, [&](int k) {
            if (core[k]) { int v = num[uf.find(k)]; if (best < 0 || v < best) best = v; }
        });
        labels[i] = best;
    }
}

}  // extern "C"
