// chaos_perf: the reference benchmark driver's performance sweeps
// (src/main.cu:26-624, runBifurcationPerformanceTests / runLLEPerformanceTests
// / runBasinsPerformanceTests) as a Linux command-line program over the
// reference-signature entry points (chaos_compat.hpp). Each sweep times one
// entry-point call per resolution and per modelling time with a wall clock in
// whole milliseconds, writes the diagram files under --out, and appends one
// row per call to the reference's result tables, in the reference's row
// formats:
//   bifurcation_performance_results.csv  "Resolution,<n>,Bifurcation,<ms>,2D"
//   lle_performance_results.csv          "Resolution,<n>,LLE,<ms>"
//   basins_performance_results.csv       "Resolution,<n>,Basins,<ms>"
// (and "ModelingTime,<TT>,..." for the modelling-time sweeps; "ERROR" in place
// of the time when a call fails). The reference compares each call with its
// legacy library, which has no counterpart here: only the library's own rows
// are written.
//
// Usage: chaos_perf [--suite all|bifurcation|lle|basins] [--precision fp64|fp32]
//                   [--out DIR] [--resolutions 100,200,...] [--times 1000,...]
//                   [--fixed-resolution 300] [--basins-system sin3]
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/chaos_compat.hpp"
#include "../../include/chaos_gb300.h"

namespace {

struct Options {
    std::string suite = "all";
    std::string out = ".";
    int precision = CHAOS_FP64;
    std::vector<int> resolutions{100, 200, 300, 400, 500, 600};  // src/main.cu:460
    std::vector<int> times{1000, 2000, 3000, 4000, 5000, 6000};   // src/main.cu:461
    int fixedResolution = 300;                                    // src/main.cu:483
    int basinsSystem = CHAOS_SYS_SIN3;
};

std::vector<int> parse_list(const char* s) {
    std::vector<int> v;
    std::stringstream ss(s);
    std::string item;
    while (std::getline(ss, item, ','))
        if (!item.empty()) v.push_back(std::atoi(item.c_str()));
    return v;
}

int parse_system(const char* s) {
    static const char* names[] = {"lorenz", "rossler", "chen", "chameleon", "rossler_cd", "sin3", "sin2", "memristor"};
    for (int i = 0; i < 8; ++i)
        if (std::strcmp(s, names[i]) == 0) return i;
    char* end = nullptr;
    const long v = std::strtol(s, &end, 10);
    return (*s && end && *end == 0) ? (int)v : -1;  // -1: unknown (rejected by the caller)
}

void usage() {
    std::cout << "usage: chaos_perf [--suite all|bifurcation|lle|basins] [--precision fp64|fp32] [--out DIR]\n"
                 "                  [--resolutions 100,200,...] [--times 1000,2000,...] [--fixed-resolution N]\n"
                 "                  [--basins-system NAME]\n";
}

// Times one call in whole milliseconds (std::chrono, as the reference does).
long long time_call(const std::function<int()>& f, int* rc) {
    const auto t0 = std::chrono::high_resolution_clock::now();
    *rc = f();
    const auto t1 = std::chrono::high_resolution_clock::now();
    return std::chrono::duration_cast<std::chrono::milliseconds>(t1 - t0).count();
}

void row(std::ofstream& f, const char* test, int value, const char* library, int rc, long long ms,
         const char* suffix) {
    f << test << "," << value << "," << library << ",";
    if (rc == CHAOS_OK) f << ms;
    else f << "ERROR";
    f << suffix << std::endl;
    std::cout << "  " << test << " " << value << ": ";
    if (rc == CHAOS_OK) std::cout << ms << " ms" << std::endl;
    else std::cout << "error " << rc << ": " << chaos_last_error() << std::endl;
}

// The Chameleon model of the bifurcation and LLE sweeps (src/main.cu:464-472, 233-241).
const double kChameleonA[7] = {0.5, 3, 0, 2, 1, 18, 1};
const double kChameleonX[3] = {3, 3, 0};
const double kChameleonRanges[4] = {0, 5, 0, 20};
const int kChameleonMut[2] = {3, 5};

// runBifurcationPerformanceTests (src/main.cu:449-624): bifurcation2D, CT 400,
// h 0.01, preScaller 1, eps 0.001, TT 2000 over the resolutions, then TT over
// the modelling times at the fixed resolution.
int run_bifurcation(const Options& o) {
    std::ofstream f(o.out + "/bifurcation_performance_results.csv");
    if (!f) return 1;
    f << "Test,Parameter,Value,Library,ExecutionTime_ms,Dimension" << std::endl;
    chaos_compat_set_system(CHAOS_SYS_CHAMELEON);
    const double h = 0.01, CT = 400, TT = 2000, maxValue = 10000, eps = 0.001;
    std::cout << "bifurcation 2D: resolution" << std::endl;
    for (int r : o.resolutions) {
        const std::string path = o.out + "/bif2d_res_test_" + std::to_string(r) + ".csv";
        int rc = 0;
        const long long ms = time_call([&] {
            return Bifurcation::bifurcation2D(CT, r, h, 3, kChameleonX, kChameleonRanges, kChameleonMut, 0, maxValue,
                                              TT, kChameleonA, 7, 1, eps, path);
        }, &rc);
        row(f, "Resolution", r, "Bifurcation", rc, ms, ",2D");
    }
    std::cout << "bifurcation 2D: modelling time" << std::endl;
    for (int t : o.times) {
        const std::string path = o.out + "/bif2d_tt_test_" + std::to_string(t) + ".csv";
        int rc = 0;
        const long long ms = time_call([&] {
            return Bifurcation::bifurcation2D(CT, o.fixedResolution, h, 3, kChameleonX, kChameleonRanges,
                                              kChameleonMut, 0, maxValue, t, kChameleonA, 7, 1, eps, path);
        }, &rc);
        row(f, "ModelingTime", t, "Bifurcation", rc, ms, ",2D");
    }
    return 0;
}

// runLLEPerformanceTests (src/main.cu:219-447): LLE2D, CT 400, NT 0.5,
// h 0.01, eps 1e-6, TT 2000 over the resolutions, then TT over the modelling
// times at the fixed resolution.
int run_lle(const Options& o) {
    std::ofstream f(o.out + "/lle_performance_results.csv");
    if (!f) return 1;
    f << "Test,Parameter,Value,Library,ExecutionTime_ms" << std::endl;
    chaos_compat_set_system(CHAOS_SYS_CHAMELEON);
    const double h = 0.01, eps = 1e-6, NT = 0.5, CT = 400, TT = 2000, maxValue = 10000;
    std::cout << "LLE 2D: resolution" << std::endl;
    for (int r : o.resolutions) {
        const std::string path = o.out + "/lle_res_test_" + std::to_string(r) + ".csv";
        int rc = 0;
        const long long ms = time_call([&] {
            return LLE::LLE2D(CT, NT, r, h, eps, kChameleonX, 3, kChameleonRanges, kChameleonMut, 0, maxValue, TT,
                              kChameleonA, 7, path);
        }, &rc);
        row(f, "Resolution", r, "LLE", rc, ms, "");
    }
    std::cout << "LLE 2D: modelling time" << std::endl;
    for (int t : o.times) {
        const std::string path = o.out + "/lle_tt_test_" + std::to_string(t) + ".csv";
        int rc = 0;
        const long long ms = time_call([&] {
            return LLE::LLE2D(CT, NT, o.fixedResolution, h, eps, kChameleonX, 3, kChameleonRanges, kChameleonMut, 0,
                              maxValue, t, kChameleonA, 7, path);
        }, &rc);
        row(f, "ModelingTime", t, "LLE", rc, ms, "");
    }
    return 0;
}

// runBasinsPerformanceTests (src/main.cu:26-217): basinsOfAttraction_2, tMax
// 500, h 0.01, writable variable 1, maxValue 1e8, preScaller 1, eps 0.05 on
// the five-parameter system the parameters belong to (the reference runs them
// on whatever system it was compiled with), TT 4000 over the resolutions,
// then TT over the modelling times at the fixed resolution.
int run_basins(const Options& o) {
    std::ofstream f(o.out + "/basins_performance_results.csv");
    if (!f) return 1;
    f << "Test,Parameter,Value,Library,ExecutionTime_ms" << std::endl;
    chaos_compat_set_system(o.basinsSystem);
    const double params[5] = {0.5, 0.1, 1.4, 15.552, 2};
    const double init[3] = {0, 0, 0};
    const double ranges[4] = {-6, 6, -6, 6};
    const int mut[2] = {0, 1};
    const double tMax = 500, h = 0.01, maxValue = 100000000, eps = 0.05;
    std::cout << "basins: resolution" << std::endl;
    for (int r : o.resolutions) {
        const std::string path = o.out + "/basins_res_test_" + std::to_string(r) + ".csv";
        int rc = 0;
        const long long ms = time_call([&] {
            return Basins::basinsOfAttraction_2(tMax, r, h, 3, init, ranges, mut, 1, maxValue, 4000, params, 5, 1,
                                                eps, path);
        }, &rc);
        row(f, "Resolution", r, "Basins", rc, ms, "");
    }
    std::cout << "basins: modelling time" << std::endl;
    for (int t : o.times) {
        const std::string path = o.out + "/basins_time_test_" + std::to_string(t) + ".csv";
        int rc = 0;
        const long long ms = time_call([&] {
            return Basins::basinsOfAttraction_2(tMax, o.fixedResolution, h, 3, init, ranges, mut, 1, maxValue, t,
                                                params, 5, 1, eps, path);
        }, &rc);
        row(f, "ModelingTime", t, "Basins", rc, ms, "");
    }
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    Options o;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        const char* v = i + 1 < argc ? argv[i + 1] : nullptr;
        if (a == "--help" || a == "-h") {
            usage();
            return 0;
        } else if (a == "--suite" && v) {
            o.suite = v;
            ++i;
        } else if (a == "--precision" && v) {
            o.precision = std::strcmp(v, "fp32") == 0 ? CHAOS_FP32 : CHAOS_FP64;
            ++i;
        } else if (a == "--out" && v) {
            o.out = v;
            ++i;
        } else if (a == "--resolutions" && v) {
            o.resolutions = parse_list(v);
            ++i;
        } else if (a == "--times" && v) {
            o.times = parse_list(v);
            ++i;
        } else if (a == "--fixed-resolution" && v) {
            o.fixedResolution = std::atoi(v);
            ++i;
        } else if (a == "--basins-system" && v) {
            o.basinsSystem = parse_system(v);
            if (o.basinsSystem < 0) {
                std::cerr << "chaos_perf: unknown system '" << v << "'\n";
                return 2;
            }
            ++i;
        } else {
            usage();
            return 2;
        }
    }
    if (o.suite != "all" && o.suite != "bifurcation" && o.suite != "lle" && o.suite != "basins") {
        usage();
        return 2;
    }
    if (chaos_compat_set_precision(o.precision) != CHAOS_OK) return 2;
    int rc = 0;
    if (o.suite == "all" || o.suite == "bifurcation") rc |= run_bifurcation(o);
    if (o.suite == "all" || o.suite == "lle") rc |= run_lle(o);
    if (o.suite == "all" || o.suite == "basins") rc |= run_basins(o);
    if (rc) std::cerr << "cannot write the result tables under " << o.out << std::endl;
    return rc;
}
