// The reference's host entry points (Bifurcation::bifurcation1D/2D,
// LLE::LLE2D, Basins::basinsOfAttraction_2) on top of the C ABI, writing the
// reference's CSV files byte for byte: same headers, same stream precisions
// (default for headers and LLE values, 12 for bifurcation rows, 15 for every
// basins file), same ", " separators with the reference's line-break rule
// (a row break is written as ", " then "\n"), NaN LLE values printed as 0.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/chaos_compat.hpp"
#include "../../include/chaos_gb300.h"
#include "capi_internal.h"

namespace {

int g_system = -1;
int g_precision = -1;

int parse_system(const char* s) {
    static const char* names[] = {"lorenz", "rossler", "chen", "chameleon", "rossler_cd", "sin3", "sin2", "memristor"};
    for (int i = 0; i < 8; ++i)
        if (strcmp(s, names[i]) == 0) return i;
    if (strcmp(s, "user") == 0) return CHAOS_SYS_USER;
    char* end = nullptr;
    long v = strtol(s, &end, 10);
    // an unknown name is an error, never a silent choice of another system:
    // -1 makes every entry point return CHAOS_E_ARGS ("unknown system -1")
    return (*s && end && *end == 0) ? (int)v : -1;
}

int active_system() {
    if (g_system >= 0) return g_system;
    const char* s = getenv("CHAOS_SYSTEM");
    return s ? parse_system(s) : CHAOS_SYS_CHAMELEON;
}

// The arithmetic chosen by chaos_compat_set_precision or CHAOS_PRECISION
// (fp64 / fp32 / ff32).
chaos_exec chosen_exec() {
    int prec = g_precision;
    if (prec < 0) {
        const char* s = getenv("CHAOS_PRECISION");
        prec = (s && (strcmp(s, "fp32") == 0 || strcmp(s, "1") == 0))   ? CHAOS_FP32
               : (s && (strcmp(s, "ff32") == 0 || strcmp(s, "2") == 0)) ? CHAOS_FF32
                                                                       : CHAOS_FP64;
    }
    return chaos_exec{prec, CHAOS_MEM_HOST, nullptr, -1};
}

// The bifurcation and basins wrappers: float-float is an LLE arithmetic, so
// CHAOS_FF32 runs these sweeps in FP64.
chaos_exec active_exec() {
    chaos_exec ex = chosen_exec();
    if (ex.precision == CHAOS_FF32) ex.precision = CHAOS_FP64;
    return ex;
}

// The LLE wrappers: FP32 where the engine has it (the RK4 systems and
// Chameleon), float-float for the RK4 systems; FP64 otherwise.
chaos_exec lle_exec() {
    chaos_exec ex = chosen_exec();
    const int sys = active_system();
    if (ex.precision == CHAOS_FP32 && sys > CHAOS_SYS_CHAMELEON) ex.precision = CHAOS_FP64;
    if (ex.precision == CHAOS_FF32 && sys > CHAOS_SYS_CHEN_RK4) ex.precision = CHAOS_FP64;
    return ex;
}

// getValueByIdx as the reference's host code evaluates it for the CSV
// (Bifurcation/src/bifurcationCUDA.cu:400-419): start + n*scale.
double host_grid_value(long long idx, int nPts, double start, double finish) {
    const long long n = idx % nPts;
    const double scale = (finish - start) / (nPts - 1);
    return start + n * scale;
}

// Writes n values with the reference's matrix rule: ", " before every value
// but the first, "\n" (after the ", ") whenever nPts values are on the line.
template <class T, class F> void write_matrix(std::ofstream& o, const T* v, long long n, int nPts, F fmt) {
    int counter = 0;
    for (long long i = 0; i < n; ++i) {
        if (counter != 0) o << ", ";
        if (counter == nPts) {
            o << "\n";
            counter = 0;
        }
        fmt(o, v[i]);
        ++counter;
    }
}

// Runs a C-ABI body and turns a failed host allocation (or any other C++
// exception) into a status: nothing thrown here crosses the C boundary.
template <class F> int guarded(F&& f) {
    try {
        return f();
    } catch (const std::bad_alloc&) {
        return chaos::set_error(CHAOS_E_NOMEM, "host allocation failed");
    } catch (const std::exception& e) {
        return chaos::set_error(CHAOS_E_IO, "%s", e.what());
    }
}

// Every kept peak of a 1-D sweep: a first pass with at most 1024 rows per
// point, then, only when some point kept more, a second pass with rows for the
// largest count. Host memory follows the peaks that exist, not B/2 rows per
// point (B can be 1e7 for a long sweep at a small step).
struct Bif1dRows {
    std::vector<int> counts, flags;
    std::vector<double> first, peaks, intervals;
    int cap = 1;
};

int bif1d_rows(int gridMode, double tMax, int nPts, double h, int amountOfInitialConditions,
               const double* initialConditions, const double* ranges, const int* indicesOfMutVars, int writableVar,
               double maxValue, double transientTime, const double* values, int amountOfValues, int preScaller,
               int capFull, Bif1dRows& r) {
    chaos_exec ex = active_exec();
    int cap = std::max(1, std::min(capFull, 1024));
    for (int pass = 0; pass < 2; ++pass) {
        r.counts.assign(nPts, 0);
        r.flags.assign(nPts, 0);
        r.first.assign(nPts, 0.0);
        r.peaks.assign((size_t)nPts * cap, 0.0);
        r.intervals.assign((size_t)nPts * cap, 0.0);
        int rc = chaos_bifurcation_sweep(&ex, active_system(), 1, gridMode, tMax, nPts, h, amountOfInitialConditions,
                                         initialConditions, ranges, indicesOfMutVars, writableVar, maxValue,
                                         transientTime, values, amountOfValues, preScaller, 0.0, cap,
                                         r.counts.data(), r.flags.data(), r.first.data(), r.peaks.data(),
                                         r.intervals.data(), nullptr);
        if (rc) return rc;
        const int mx = *std::max_element(r.counts.begin(), r.counts.end());
        r.cap = cap;
        if (mx <= cap) return CHAOS_OK;
        cap = mx;
    }
    return CHAOS_OK;
}

}  // namespace

extern "C" {

int chaos_compat_set_system(int system) {
    if ((system < 0 || system > CHAOS_SYS_MEMRISTOR) && system != CHAOS_SYS_USER)
        return chaos::set_error(CHAOS_E_ARGS, "unknown system %d", system);
    g_system = system;
    return CHAOS_OK;
}

int chaos_compat_set_precision(int precision) {
    if (precision != CHAOS_FP64 && precision != CHAOS_FP32 && precision != CHAOS_FF32)
        return chaos::set_error(CHAOS_E_ARGS, "bad precision");
    g_precision = precision;
    return CHAOS_OK;
}

int chaos_compat_get_system(void) { return active_system(); }

int chaos_compat_bifurcation1D(double tMax, int nPts, double h, int amountOfInitialConditions,
                               const double* initialConditions, const double* ranges, const int* indicesOfMutVars,
                               int writableVar, double maxValue, double transientTime, const double* values,
                               int amountOfValues, int preScaller, const char* OUT_FILE_PATH) {
    return guarded([&]() -> int {
        if (nPts < 2 || !(h > 0) || preScaller < 1) return chaos::set_error(CHAOS_E_ARGS, "bad sweep arguments");
        const int B = (int)(tMax / h / preScaller);
        Bif1dRows r;
        int rc = bif1d_rows(0, tMax, nPts, h, amountOfInitialConditions, initialConditions, ranges,
                            indicesOfMutVars, writableVar, maxValue, transientTime, values, amountOfValues,
                            preScaller, B / 2 > 0 ? B / 2 : 1, r);
        if (rc) return rc;
        std::ofstream o(OUT_FILE_PATH);
        if (!o.is_open()) return chaos::set_error(CHAOS_E_IO, "cannot open %s", OUT_FILE_PATH);
        o << ranges[0] << " " << ranges[1] << "\n";
        o << std::setprecision(12);
        for (int k = 0; k < nPts; ++k) {
            const double p = host_grid_value(k, nPts, ranges[0], ranges[1]);
            if (r.counts[k] == -1) {
                o << p << ", " << r.first[k] << ", " << 0 << '\n';
            } else {
                for (int j = 0; j < r.counts[k]; ++j)
                    o << p << ", " << r.peaks[(size_t)k * r.cap + j] << ", " << r.intervals[(size_t)k * r.cap + j]
                      << '\n';
            }
        }
        return o.good() ? CHAOS_OK : chaos::set_error(CHAOS_E_IO, "write failed: %s", OUT_FILE_PATH);
    });
}

int chaos_compat_bifurcation2D(double tMax, int nPts, double h, int amountOfInitialConditions,
                               const double* initialConditions, const double* ranges, const int* indicesOfMutVars,
                               int writableVar, double maxValue, double transientTime, const double* values,
                               int amountOfValues, int preScaller, double eps, const char* OUT_FILE_PATH) {
    return guarded([&]() -> int {
        if (nPts < 2) return chaos::set_error(CHAOS_E_ARGS, "nPts must be >= 2");
        const long long n = (long long)nPts * nPts;
        std::vector<int> labels(n);
        chaos_exec ex = active_exec();
        int rc = chaos_bifurcation2d(&ex, active_system(), tMax, nPts, h, amountOfInitialConditions, initialConditions,
                                     ranges, indicesOfMutVars, writableVar, maxValue, transientTime, values,
                                     amountOfValues, preScaller, eps, labels.data(), nullptr);
        if (rc) return rc;
        std::ofstream o(OUT_FILE_PATH);
        if (!o.is_open()) return chaos::set_error(CHAOS_E_IO, "cannot open %s", OUT_FILE_PATH);
        o << ranges[0] << " " << ranges[1] << "\n";
        o << ranges[2] << " " << ranges[3] << "\n";
        o << std::setprecision(12);
        write_matrix(o, labels.data(), n, nPts, [](std::ofstream& s, int v) { s << v; });
        return o.good() ? CHAOS_OK : chaos::set_error(CHAOS_E_IO, "write failed: %s", OUT_FILE_PATH);
    });
}

int chaos_compat_LLE2D(double tMax, double NT, int nPts, double h, double eps, const double* initialConditions,
                       int amountOfInitialConditions, const double* ranges, const int* indicesOfMutVars,
                       int writableVar, double maxValue, double transientTime, const double* values,
                       int amountOfValues, const char* OUT_FILE_PATH) {
    return guarded([&]() -> int {
        if (nPts < 1) return chaos::set_error(CHAOS_E_ARGS, "nPts must be >= 1");
        const long long n = (long long)nPts * nPts;
        std::vector<double> lle(n);
        chaos_exec ex = lle_exec();
        std::ofstream o(OUT_FILE_PATH);
        if (!o.is_open()) return chaos::set_error(CHAOS_E_IO, "cannot open %s", OUT_FILE_PATH);
        o << ranges[0] << " " << ranges[1] << "\n";
        o << ranges[2] << " " << ranges[3] << "\n";
        int rc = chaos_lle2d(&ex, active_system(), tMax, NT, nPts, h, eps, initialConditions, amountOfInitialConditions,
                             ranges, indicesOfMutVars, writableVar, maxValue, transientTime, values, amountOfValues,
                             lle.data());
        if (rc) return rc;
        write_matrix(o, lle.data(), n, nPts, [](std::ofstream& s, double v) { s << (std::isnan(v) ? 0 : v); });
        return o.good() ? CHAOS_OK : chaos::set_error(CHAOS_E_IO, "write failed: %s", OUT_FILE_PATH);
    });
}

int chaos_compat_basinsOfAttraction_2(double tMax, int nPts, double h, int amountOfInitialConditions,
                                      const double* initialConditions, const double* ranges,
                                      const int* indicesOfMutVars, int writableVar, double maxValue,
                                      double transientTime, const double* values, int amountOfValues,
                                      int preScaller, double eps, const char* OUT_FILE_PATH) {
    return guarded([&]() -> int {
        if (nPts < 2) return chaos::set_error(CHAOS_E_ARGS, "nPts must be >= 2");
        const long long n = (long long)nPts * nPts;
        std::vector<int> labels(n), flags(n);
        std::vector<double> ap(n), ai(n);
        chaos_exec ex = active_exec();
        int rc = chaos_basins(&ex, active_system(), tMax, nPts, h, amountOfInitialConditions, initialConditions, ranges,
                              indicesOfMutVars, writableVar, maxValue, transientTime, values, amountOfValues, preScaller,
                              eps, labels.data(), ap.data(), ai.data(), flags.data());
        if (rc) return rc;
        const std::string base(OUT_FILE_PATH);
        const std::string paths[4] = {base, base + "_1.csv", base + "_2.csv", base + "_3.csv"};
        for (int f = 0; f < 4; ++f) {
            std::ofstream o(paths[f]);
            if (!o.is_open()) return chaos::set_error(CHAOS_E_IO, "cannot open %s", paths[f].c_str());
            o << std::setprecision(15);
            o << ranges[0] << " " << ranges[1] << "\n";
            o << ranges[2] << " " << ranges[3] << "\n";
            if (f == 0) write_matrix(o, labels.data(), n, nPts, [](std::ofstream& s, int v) { s << v; });
            if (f == 1) write_matrix(o, ap.data(), n, nPts, [](std::ofstream& s, double v) { s << v; });
            if (f == 2) write_matrix(o, ai.data(), n, nPts, [](std::ofstream& s, double v) { s << v; });
            if (f == 3) write_matrix(o, flags.data(), n, nPts, [](std::ofstream& s, int v) { s << v; });
            if (!o.good()) return chaos::set_error(CHAOS_E_IO, "write failed: %s", paths[f].c_str());
        }
        return CHAOS_OK;
    });
}

// ---- the legacy library's analyses (namespace old_library, debri/hostLibrary.cuh) ----
// Each runs the engine's sweep with the matching grid mode and writes the
// legacy function's file format. The bifurcation analyses run the legacy
// per-point loop (CHAOS_GRID_LEGACY_LOOP, FP64).

// Rows "value, peak" per kept peak, precision 12, no header: bifurcation1DIC
// and bifurcation1DForH (debri/hostLibrary.cu:1447-1460, 1197-1210). The
// step-size sweep labels its rows with the linear getValueByIdx of the range,
// not the step it used, as the legacy writer does.
static int legacy_bif1d(int gridMode, double tMax, int nPts, double h, int amountOfInitialConditions,
                        const double* initialConditions, const double* ranges, const int* indicesOfMutVars,
                        int writableVar, double maxValue, double transientTime, const double* values,
                        int amountOfValues, int preScaller, const char* OUT_FILE_PATH) {
    if (nPts < 2 || preScaller < 1) return chaos::set_error(CHAOS_E_ARGS, "bad sweep arguments");
    const bool stepAxis = indicesOfMutVars && indicesOfMutVars[0] == CHAOS_MUT_STEP;
    const double hMin = stepAxis ? std::min(ranges[0], ranges[1]) * (1.0 - 1e-9) : h;
    if (!(hMin > 0)) return chaos::set_error(CHAOS_E_ARGS, "need a positive step");
    const int B = (int)(tMax / hMin / preScaller);
    Bif1dRows r;
    int rc = bif1d_rows(gridMode, tMax, nPts, h, amountOfInitialConditions, initialConditions, ranges,
                        indicesOfMutVars, writableVar, maxValue, transientTime, values, amountOfValues, preScaller,
                        B / 2 > 0 ? B / 2 : 1, r);
    if (rc) return rc;
    std::ofstream o(OUT_FILE_PATH);
    if (!o.is_open()) return chaos::set_error(CHAOS_E_IO, "cannot open %s", OUT_FILE_PATH);
    o << std::setprecision(12);
    for (int k = 0; k < nPts; ++k) {
        const double p = host_grid_value(k, nPts, ranges[0], ranges[1]);
        for (int j = 0; j < r.counts[k]; ++j) o << p << ", " << r.peaks[(size_t)k * r.cap + j] << '\n';
    }
    return o.good() ? CHAOS_OK : chaos::set_error(CHAOS_E_IO, "write failed: %s", OUT_FILE_PATH);
}


// LLE1D / LLE1DIC: rows "value, lle" at precision 12, no header
// (debri/hostLibrary.cu:3291-3300, 3508-3517); LLE2DIC: the matrix rule at the
// default precision, no header (debri/hostLibrary.cu:3793-3805).
// The legacy LLE kernels' scheme (chaos_lle_sweep_legacy, FP64). Their
// writableVar argument reaches no loop (they run their loops on component 0).
static int legacy_lle(int dim, int gridMode, double tMax, double NT, int nPts, double h, double eps,
                      const double* initialConditions, int amountOfInitialConditions, const double* ranges,
                      const int* indicesOfMutVars, double maxValue, double transientTime, const double* values,
                      int amountOfValues, const char* OUT_FILE_PATH) {
    if (nPts < 1) return chaos::set_error(CHAOS_E_ARGS, "nPts must be >= 1");
    const long long n = dim == 2 ? (long long)nPts * nPts : nPts;
    std::vector<double> lle(n);
    chaos_exec ex = lle_exec();
    int rc = chaos_lle_sweep_legacy(&ex, active_system(), dim, gridMode, tMax, NT, nPts, h, eps, initialConditions,
                                    amountOfInitialConditions, ranges, indicesOfMutVars, maxValue, transientTime,
                                    values, amountOfValues, nullptr, lle.data());
    if (rc) return rc;
    std::ofstream o(OUT_FILE_PATH);
    if (!o.is_open()) return chaos::set_error(CHAOS_E_IO, "cannot open %s", OUT_FILE_PATH);
    if (dim == 1) {
        o << std::setprecision(12);
        for (int k = 0; k < nPts; ++k) o << host_grid_value(k, nPts, ranges[0], ranges[1]) << ", " << lle[k] << '\n';
    } else {
        write_matrix(o, lle.data(), n, nPts, [](std::ofstream& s, double v) { s << v; });
    }
    return o.good() ? CHAOS_OK : chaos::set_error(CHAOS_E_IO, "write failed: %s", OUT_FILE_PATH);
}

// LS1D: rows "value, l_0, ..., l_{n-1}" at the default precision, no header
// (debri/hostLibrary.cu:3927-3936). LS2D: one file per exponent,
// OUT_FILE_PATH + "<k+1>.csv", the range header then the matrix rule
// (debri/hostLibrary.cu:4030-4040, 4078-4094).
// The legacy spectrum kernel's scheme (chaos_lyapunov_spectrum_legacy, FP64).
static int legacy_ls(int dim, double tMax, double NT, int nPts, double h, double eps,
                     const double* initialConditions, int amountOfInitialConditions, const double* ranges,
                     const int* indicesOfMutVars, double maxValue, double transientTime, const double* values,
                     int amountOfValues, const char* OUT_FILE_PATH) {
    if (nPts < 1 || amountOfInitialConditions < 1) return chaos::set_error(CHAOS_E_ARGS, "bad sweep arguments");
    const long long n = dim == 2 ? (long long)nPts * nPts : nPts;
    const int nx = amountOfInitialConditions;
    std::vector<double> sp((size_t)n * nx);
    chaos_exec ex = lle_exec();
    int rc = chaos_lyapunov_spectrum_legacy(&ex, active_system(), dim, 0, tMax, NT, nPts, h, eps, initialConditions,
                                            amountOfInitialConditions, ranges, indicesOfMutVars, maxValue,
                                            transientTime, values, amountOfValues, nullptr, sp.data());
    if (rc) return rc;
    if (dim == 1) {
        std::ofstream o(OUT_FILE_PATH);
        if (!o.is_open()) return chaos::set_error(CHAOS_E_IO, "cannot open %s", OUT_FILE_PATH);
        for (int k = 0; k < nPts; ++k) {
            o << host_grid_value(k, nPts, ranges[0], ranges[1]);
            for (int j = 0; j < nx; ++j) o << ", " << sp[(size_t)k * nx + j];
            o << '\n';
        }
        return o.good() ? CHAOS_OK : chaos::set_error(CHAOS_E_IO, "write failed: %s", OUT_FILE_PATH);
    }
    std::vector<double> col(n);
    for (int j = 0; j < nx; ++j) {
        const std::string path = std::string(OUT_FILE_PATH) + std::to_string(j + 1) + ".csv";
        std::ofstream o(path);
        if (!o.is_open()) return chaos::set_error(CHAOS_E_IO, "cannot open %s", path.c_str());
        o << ranges[0] << " " << ranges[1] << "\n";
        o << ranges[2] << " " << ranges[3] << "\n";
        for (long long p = 0; p < n; ++p) col[p] = sp[(size_t)p * nx + j];
        write_matrix(o, col.data(), n, nPts, [](std::ofstream& s, double v) { s << v; });
        if (!o.good()) return chaos::set_error(CHAOS_E_IO, "write failed: %s", path.c_str());
    }
    return CHAOS_OK;
}

int chaos_compat_bifurcation1DIC(double tMax, int nPts, double h, int amountOfInitialConditions,
                                 const double* initialConditions, const double* ranges, const int* indicesOfMutVars,
                                 int writableVar, double maxValue, double transientTime, const double* values,
                                 int amountOfValues, int preScaller, const char* OUT_FILE_PATH) {
    return guarded([&]() -> int {
        return legacy_bif1d(CHAOS_GRID_STATE | CHAOS_GRID_LEGACY_LOOP, tMax, nPts, h, amountOfInitialConditions,
                            initialConditions, ranges, indicesOfMutVars, writableVar, maxValue, transientTime, values,
                            amountOfValues, preScaller, OUT_FILE_PATH);
    });
}

int chaos_compat_bifurcation1DForH(double tMax, int nPts, int amountOfInitialConditions,
                                   const double* initialConditions, const double* ranges, int writableVar,
                                   double maxValue, double transientTime, const double* values, int amountOfValues,
                                   int preScaller, const char* OUT_FILE_PATH) {
    return guarded([&]() -> int {
        const int mut[1] = {CHAOS_MUT_STEP};
        return legacy_bif1d(CHAOS_GRID_LOG0 | CHAOS_GRID_LOG_F32 | CHAOS_GRID_LEGACY_LOOP, tMax, nPts, 0.0,
                            amountOfInitialConditions, initialConditions, ranges, mut, writableVar, maxValue,
                            transientTime, values, amountOfValues, preScaller, OUT_FILE_PATH);
    });
}

// bifurcation2DIC writes bifurcation2D's file (debri/hostLibrary.cu:2932-2936, 3058-3076).
int chaos_compat_bifurcation2DIC(double tMax, int nPts, double h, int amountOfInitialConditions,
                                 const double* initialConditions, const double* ranges, const int* indicesOfMutVars,
                                 int writableVar, double maxValue, double transientTime, const double* values,
                                 int amountOfValues, int preScaller, double eps, const char* OUT_FILE_PATH) {
    return guarded([&]() -> int {
        if (nPts < 2) return chaos::set_error(CHAOS_E_ARGS, "nPts must be >= 2");
        const long long n = (long long)nPts * nPts;
        std::vector<int> labels(n);
        chaos_exec ex = active_exec();
        int rc = chaos_bifurcation_sweep(&ex, active_system(), 2, CHAOS_GRID_STATE | CHAOS_GRID_LEGACY_LOOP, tMax,
                                         nPts, h, amountOfInitialConditions, initialConditions, ranges,
                                         indicesOfMutVars, writableVar, maxValue, transientTime, values,
                                         amountOfValues, preScaller, eps, 0, nullptr, nullptr, nullptr, nullptr,
                                         nullptr, labels.data());
        if (rc) return rc;
        std::ofstream o(OUT_FILE_PATH);
        if (!o.is_open()) return chaos::set_error(CHAOS_E_IO, "cannot open %s", OUT_FILE_PATH);
        o << ranges[0] << " " << ranges[1] << "\n";
        o << ranges[2] << " " << ranges[3] << "\n";
        o << std::setprecision(12);
        write_matrix(o, labels.data(), n, nPts, [](std::ofstream& s, int v) { s << v; });
        return o.good() ? CHAOS_OK : chaos::set_error(CHAOS_E_IO, "write failed: %s", OUT_FILE_PATH);
    });
}

int chaos_compat_LLE1D(double tMax, double NT, int nPts, double h, double eps, const double* initialConditions,
                       int amountOfInitialConditions, const double* ranges, const int* indicesOfMutVars,
                       int writableVar, double maxValue, double transientTime, const double* values,
                       int amountOfValues, const char* OUT_FILE_PATH) {
    return guarded([&]() -> int {
        (void)writableVar;
        return legacy_lle(1, 0, tMax, NT, nPts, h, eps, initialConditions, amountOfInitialConditions, ranges,
                          indicesOfMutVars, maxValue, transientTime, values, amountOfValues, OUT_FILE_PATH);
    });
}

int chaos_compat_LLE1DIC(double tMax, double NT, int nPts, double h, double eps, const double* initialConditions,
                         int amountOfInitialConditions, const double* ranges, const int* indicesOfMutVars,
                         int writableVar, double maxValue, double transientTime, const double* values,
                         int amountOfValues, const char* OUT_FILE_PATH) {
    return guarded([&]() -> int {
        (void)writableVar;
        return legacy_lle(1, CHAOS_GRID_STATE, tMax, NT, nPts, h, eps, initialConditions, amountOfInitialConditions,
                          ranges, indicesOfMutVars, maxValue, transientTime, values, amountOfValues, OUT_FILE_PATH);
    });
}

int chaos_compat_LLE2DIC(double tMax, double NT, int nPts, double h, double eps, const double* initialConditions,
                         int amountOfInitialConditions, const double* ranges, const int* indicesOfMutVars,
                         int writableVar, double maxValue, double transientTime, const double* values,
                         int amountOfValues, const char* OUT_FILE_PATH) {
    return guarded([&]() -> int {
        (void)writableVar;
        return legacy_lle(2, CHAOS_GRID_STATE, tMax, NT, nPts, h, eps, initialConditions, amountOfInitialConditions,
                          ranges, indicesOfMutVars, maxValue, transientTime, values, amountOfValues, OUT_FILE_PATH);
    });
}

int chaos_compat_LS1D(double tMax, double NT, int nPts, double h, double eps, const double* initialConditions,
                      int amountOfInitialConditions, const double* ranges, const int* indicesOfMutVars,
                      int writableVar, double maxValue, double transientTime, const double* values,
                      int amountOfValues, const char* OUT_FILE_PATH) {
    return guarded([&]() -> int {
        (void)writableVar;
        return legacy_ls(1, tMax, NT, nPts, h, eps, initialConditions, amountOfInitialConditions, ranges,
                         indicesOfMutVars, maxValue, transientTime, values, amountOfValues, OUT_FILE_PATH);
    });
}

int chaos_compat_LS2D(double tMax, double NT, int nPts, double h, double eps, const double* initialConditions,
                      int amountOfInitialConditions, const double* ranges, const int* indicesOfMutVars,
                      int writableVar, double maxValue, double transientTime, const double* values,
                      int amountOfValues, const char* OUT_FILE_PATH) {
    return guarded([&]() -> int {
        (void)writableVar;
        return legacy_ls(2, tMax, NT, nPts, h, eps, initialConditions, amountOfInitialConditions, ranges,
                         indicesOfMutVars, maxValue, transientTime, values, amountOfValues, OUT_FILE_PATH);
    });
}

// The legacy basins map (debri/hostLibrary.cu:4115-4556) writes the four files
// of basinsOfAttraction_2; its main file holds an array it never fills
// (the clustering kernel is not launched), here the basin labels.
int chaos_compat_basinsOfAttraction(double tMax, int nPts, double h, int amountOfInitialConditions,
                                    const double* initialConditions, const double* ranges,
                                    const int* indicesOfMutVars, int writableVar, double maxValue,
                                    double transientTime, const double* values, int amountOfValues, int preScaller,
                                    double eps, const char* OUT_FILE_PATH) {
    return guarded([&]() -> int {
        return chaos_compat_basinsOfAttraction_2(tMax, nPts, h, amountOfInitialConditions, initialConditions, ranges,
                                                 indicesOfMutVars, writableVar, maxValue, transientTime, values,
                                                 amountOfValues, preScaller, eps, OUT_FILE_PATH);
    });
}

}  // extern "C"

namespace Bifurcation {
int bifurcation1D(const double tMax, const int nPts, const double h, const int amountOfInitialConditions,
                  const double* initialConditions, const double* ranges, const int* indicesOfMutVars,
                  const int writableVar, const double maxValue, const double transientTime, const double* values,
                  const int amountOfValues, const int preScaller, std::string OUT_FILE_PATH) {
    return chaos_compat_bifurcation1D(tMax, nPts, h, amountOfInitialConditions, initialConditions, ranges,
                                      indicesOfMutVars, writableVar, maxValue, transientTime, values, amountOfValues,
                                      preScaller, OUT_FILE_PATH.c_str());
}
int bifurcation2D(const double tMax, const int nPts, const double h, const int amountOfInitialConditions,
                  const double* initialConditions, const double* ranges, const int* indicesOfMutVars,
                  const int writableVar, const double maxValue, const double transientTime, const double* values,
                  const int amountOfValues, const int preScaller, const double eps, std::string OUT_FILE_PATH) {
    return chaos_compat_bifurcation2D(tMax, nPts, h, amountOfInitialConditions, initialConditions, ranges,
                                      indicesOfMutVars, writableVar, maxValue, transientTime, values, amountOfValues,
                                      preScaller, eps, OUT_FILE_PATH.c_str());
}
}  // namespace Bifurcation

namespace LLE {
int LLE2D(const double tMax, const double NT, const int nPts, const double h, const double eps,
          const double* initialConditions, const int amountOfInitialConditions, const double* ranges,
          const int* indicesOfMutVars, const int writableVar, const double maxValue, const double transientTime,
          const double* values, const int amountOfValues, std::string OUT_FILE_PATH) {
    return chaos_compat_LLE2D(tMax, NT, nPts, h, eps, initialConditions, amountOfInitialConditions, ranges,
                              indicesOfMutVars, writableVar, maxValue, transientTime, values, amountOfValues,
                              OUT_FILE_PATH.c_str());
}
}  // namespace LLE

namespace Basins {
int basinsOfAttraction_2(const double tMax, const int nPts, const double h, const int amountOfInitialConditions,
                         const double* initialConditions, const double* ranges, const int* indicesOfMutVars,
                         const int writableVar, const double maxValue, const double transientTime,
                         const double* values, const int amountOfValues, const int preScaller, const double eps,
                         std::string OUT_FILE_PATH) {
    return chaos_compat_basinsOfAttraction_2(tMax, nPts, h, amountOfInitialConditions, initialConditions, ranges,
                                             indicesOfMutVars, writableVar, maxValue, transientTime, values,
                                             amountOfValues, preScaller, eps, OUT_FILE_PATH.c_str());
}
}  // namespace Basins

namespace old_library {
#define CHAOS_LEGACY_BIF_ARGS                                                                                   \
    const double tMax, const int nPts, const double h, const int amountOfInitialConditions,                     \
        const double *initialConditions, const double *ranges, const int *indicesOfMutVars,                     \
        const int writableVar, const double maxValue, const double transientTime, const double *values,         \
        const int amountOfValues, const int preScaller
#define CHAOS_LEGACY_LLE_ARGS                                                                                   \
    const double tMax, const double NT, const int nPts, const double h, const double eps,                       \
        const double *initialConditions, const int amountOfInitialConditions, const double *ranges,             \
        const int *indicesOfMutVars, const int writableVar, const double maxValue, const double transientTime,  \
        const double *values, const int amountOfValues
#define CHAOS_LEGACY_BIF_PASS                                                                                   \
    tMax, nPts, h, amountOfInitialConditions, initialConditions, ranges, indicesOfMutVars, writableVar, maxValue, \
        transientTime, values, amountOfValues, preScaller
#define CHAOS_LEGACY_LLE_PASS                                                                                   \
    tMax, NT, nPts, h, eps, initialConditions, amountOfInitialConditions, ranges, indicesOfMutVars, writableVar, \
        maxValue, transientTime, values, amountOfValues

int bifurcation1DIC(CHAOS_LEGACY_BIF_ARGS, std::string OUT_FILE_PATH) {
    return chaos_compat_bifurcation1DIC(CHAOS_LEGACY_BIF_PASS, OUT_FILE_PATH.c_str());
}
int bifurcation2DIC(CHAOS_LEGACY_BIF_ARGS, const double eps, std::string OUT_FILE_PATH) {
    return chaos_compat_bifurcation2DIC(CHAOS_LEGACY_BIF_PASS, eps, OUT_FILE_PATH.c_str());
}
int bifurcation1DForH(const double tMax, const int nPts, const int amountOfInitialConditions,
                      const double* initialConditions, const double* ranges, const int writableVar,
                      const double maxValue, const double transientTime, const double* values,
                      const int amountOfValues, const int preScaller, std::string OUT_FILE_PATH) {
    return chaos_compat_bifurcation1DForH(tMax, nPts, amountOfInitialConditions, initialConditions, ranges,
                                          writableVar, maxValue, transientTime, values, amountOfValues, preScaller,
                                          OUT_FILE_PATH.c_str());
}
int LLE1D(CHAOS_LEGACY_LLE_ARGS, std::string OUT_FILE_PATH) {
    return chaos_compat_LLE1D(CHAOS_LEGACY_LLE_PASS, OUT_FILE_PATH.c_str());
}
int LLE1DIC(CHAOS_LEGACY_LLE_ARGS, std::string OUT_FILE_PATH) {
    return chaos_compat_LLE1DIC(CHAOS_LEGACY_LLE_PASS, OUT_FILE_PATH.c_str());
}
int LLE2DIC(CHAOS_LEGACY_LLE_ARGS, std::string OUT_FILE_PATH) {
    return chaos_compat_LLE2DIC(CHAOS_LEGACY_LLE_PASS, OUT_FILE_PATH.c_str());
}
int LS1D(CHAOS_LEGACY_LLE_ARGS, std::string OUT_FILE_PATH) {
    return chaos_compat_LS1D(CHAOS_LEGACY_LLE_PASS, OUT_FILE_PATH.c_str());
}
int LS2D(CHAOS_LEGACY_LLE_ARGS, std::string OUT_FILE_PATH) {
    return chaos_compat_LS2D(CHAOS_LEGACY_LLE_PASS, OUT_FILE_PATH.c_str());
}
int basinsOfAttraction(CHAOS_LEGACY_BIF_ARGS, const double eps, std::string OUT_FILE_PATH) {
    return chaos_compat_basinsOfAttraction(CHAOS_LEGACY_BIF_PASS, eps, OUT_FILE_PATH.c_str());
}
}  // namespace old_library
