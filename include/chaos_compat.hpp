// Drop-in replacements for ChaosLibrary's host entry points, with the
// reference's exact C++ signatures. Each one runs the GB300 engine through
// the C ABI (chaos_gb300.h) and writes the same CSV files, in the same byte
// format, as the reference function it replaces. Unlike the reference they
// return a status (CHAOS_OK or a CHAOS_E_* code) instead of calling exit().
//
// The reference compiles one system in (systems/systems.cuh:9). Here the
// system is chosen at run time: chaos_compat_set_system(), or the environment
// variable CHAOS_SYSTEM (a CHAOS_SYS_* number or a name: lorenz, rossler,
// chen, chameleon, rossler_cd, sin3, sin2, memristor); the default is
// Chameleon, the reference's default. The arithmetic is FP64 unless
// chaos_compat_set_precision(CHAOS_FP32) or CHAOS_PRECISION=fp32; with
// CHAOS_FF32 (CHAOS_PRECISION=ff32) the LLE wrappers of the RK4 systems run
// float-float and every other wrapper FP64.
#ifndef CHAOS_COMPAT_HPP
#define CHAOS_COMPAT_HPP

#include <string>

#include "chaos_gb300.h"

namespace Bifurcation {
// Bifurcation/include/bifurcationHOST.h:16-30
int bifurcation1D(const double tMax, const int nPts, const double h, const int amountOfInitialConditions,
                  const double* initialConditions, const double* ranges, const int* indicesOfMutVars,
                  const int writableVar, const double maxValue, const double transientTime, const double* values,
                  const int amountOfValues, const int preScaller, std::string OUT_FILE_PATH);
// Bifurcation/include/bifurcationHOST.h:35-50
int bifurcation2D(const double tMax, const int nPts, const double h, const int amountOfInitialConditions,
                  const double* initialConditions, const double* ranges, const int* indicesOfMutVars,
                  const int writableVar, const double maxValue, const double transientTime, const double* values,
                  const int amountOfValues, const int preScaller, const double eps, std::string OUT_FILE_PATH);
}  // namespace Bifurcation

namespace LLE {
// LLE/include/LLEHost.h:25-41
int LLE2D(const double tMax, const double NT, const int nPts, const double h, const double eps,
          const double* initialConditions, const int amountOfInitialConditions, const double* ranges,
          const int* indicesOfMutVars, const int writableVar, const double maxValue, const double transientTime,
          const double* values, const int amountOfValues, std::string OUT_FILE_PATH);
}  // namespace LLE

namespace Basins {
// Basins/include/basinsHOST.h:15-30
int basinsOfAttraction_2(const double tMax, const int nPts, const double h, const int amountOfInitialConditions,
                         const double* initialConditions, const double* ranges, const int* indicesOfMutVars,
                         const int writableVar, const double maxValue, const double transientTime,
                         const double* values, const int amountOfValues, const int preScaller, const double eps,
                         std::string OUT_FILE_PATH);
}  // namespace Basins

// The legacy library's analyses (debri/hostLibrary.cuh:30-400, namespace
// old_library) with their signatures and file formats, on the engine's sweeps:
// the *IC variants sweep initial conditions (CHAOS_GRID_STATE), the step-size
// sweep runs the step on the legacy log scale, the LLE and LS analyses run the
// legacy kernels' schemes in FP64 (chaos_lle_sweep_legacy,
// chaos_lyapunov_spectrum_legacy). The bifurcation analyses run the legacy
// per-point loop in FP64 (CHAOS_GRID_LEGACY_LOOP);
// the peak rule and the per-point clustering are the same in both libraries;
// basinsOfAttraction is the current library's basins map (its loop is the
// legacy one). The legacy kernels integrate a system hard-wired into the
// legacy sources; here the system is the one selected.
namespace old_library {
// debri/hostLibrary.cu:1243-1486
int bifurcation1DIC(const double tMax, const int nPts, const double h, const int amountOfInitialConditions,
                    const double* initialConditions, const double* ranges, const int* indicesOfMutVars,
                    const int writableVar, const double maxValue, const double transientTime, const double* values,
                    const int amountOfValues, const int preScaller, std::string OUT_FILE_PATH);
// debri/hostLibrary.cu:2819-3107
int bifurcation2DIC(const double tMax, const int nPts, const double h, const int amountOfInitialConditions,
                    const double* initialConditions, const double* ranges, const int* indicesOfMutVars,
                    const int writableVar, const double maxValue, const double transientTime, const double* values,
                    const int amountOfValues, const int preScaller, const double eps, std::string OUT_FILE_PATH);
// debri/hostLibrary.cu:1005-1240: ranges[0..1] is the range of the step h (log scale)
int bifurcation1DForH(const double tMax, const int nPts, const int amountOfInitialConditions,
                      const double* initialConditions, const double* ranges, const int writableVar,
                      const double maxValue, const double transientTime, const double* values,
                      const int amountOfValues, const int preScaller, std::string OUT_FILE_PATH);
// debri/hostLibrary.cu:3111-3325, 3328-3542, 3692-3825, 3829-3958, 3961-4111
int LLE1D(const double tMax, const double NT, const int nPts, const double h, const double eps,
          const double* initialConditions, const int amountOfInitialConditions, const double* ranges,
          const int* indicesOfMutVars, const int writableVar, const double maxValue, const double transientTime,
          const double* values, const int amountOfValues, std::string OUT_FILE_PATH);
int LLE1DIC(const double tMax, const double NT, const int nPts, const double h, const double eps,
            const double* initialConditions, const int amountOfInitialConditions, const double* ranges,
            const int* indicesOfMutVars, const int writableVar, const double maxValue, const double transientTime,
            const double* values, const int amountOfValues, std::string OUT_FILE_PATH);
int LLE2DIC(const double tMax, const double NT, const int nPts, const double h, const double eps,
            const double* initialConditions, const int amountOfInitialConditions, const double* ranges,
            const int* indicesOfMutVars, const int writableVar, const double maxValue, const double transientTime,
            const double* values, const int amountOfValues, std::string OUT_FILE_PATH);
int LS1D(const double tMax, const double NT, const int nPts, const double h, const double eps,
         const double* initialConditions, const int amountOfInitialConditions, const double* ranges,
         const int* indicesOfMutVars, const int writableVar, const double maxValue, const double transientTime,
         const double* values, const int amountOfValues, std::string OUT_FILE_PATH);
int LS2D(const double tMax, const double NT, const int nPts, const double h, const double eps,
         const double* initialConditions, const int amountOfInitialConditions, const double* ranges,
         const int* indicesOfMutVars, const int writableVar, const double maxValue, const double transientTime,
         const double* values, const int amountOfValues, std::string OUT_FILE_PATH);
// debri/hostLibrary.cu:4115-4556
int basinsOfAttraction(const double tMax, const int nPts, const double h, const int amountOfInitialConditions,
                       const double* initialConditions, const double* ranges, const int* indicesOfMutVars,
                       const int writableVar, const double maxValue, const double transientTime,
                       const double* values, const int amountOfValues, const int preScaller, const double eps,
                       std::string OUT_FILE_PATH);
}  // namespace old_library

extern "C" {
// Run-time selection of the system and arithmetic the wrappers above use.
int chaos_compat_set_system(int system);
int chaos_compat_set_precision(int precision);
int chaos_compat_get_system(void);

// The same four wrappers with a C string path, for C and FFI callers.
int chaos_compat_bifurcation1D(double tMax, int nPts, double h, int amountOfInitialConditions,
                               const double* initialConditions, const double* ranges, const int* indicesOfMutVars,
                               int writableVar, double maxValue, double transientTime, const double* values,
                               int amountOfValues, int preScaller, const char* OUT_FILE_PATH);
int chaos_compat_bifurcation2D(double tMax, int nPts, double h, int amountOfInitialConditions,
                               const double* initialConditions, const double* ranges, const int* indicesOfMutVars,
                               int writableVar, double maxValue, double transientTime, const double* values,
                               int amountOfValues, int preScaller, double eps, const char* OUT_FILE_PATH);
int chaos_compat_LLE2D(double tMax, double NT, int nPts, double h, double eps, const double* initialConditions,
                       int amountOfInitialConditions, const double* ranges, const int* indicesOfMutVars,
                       int writableVar, double maxValue, double transientTime, const double* values,
                       int amountOfValues, const char* OUT_FILE_PATH);
int chaos_compat_basinsOfAttraction_2(double tMax, int nPts, double h, int amountOfInitialConditions,
                                      const double* initialConditions, const double* ranges,
                                      const int* indicesOfMutVars, int writableVar, double maxValue,
                                      double transientTime, const double* values, int amountOfValues,
                                      int preScaller, double eps, const char* OUT_FILE_PATH);

// The legacy analyses with a C string path.
int chaos_compat_bifurcation1DIC(double tMax, int nPts, double h, int amountOfInitialConditions,
                                 const double* initialConditions, const double* ranges, const int* indicesOfMutVars,
                                 int writableVar, double maxValue, double transientTime, const double* values,
                                 int amountOfValues, int preScaller, const char* OUT_FILE_PATH);
int chaos_compat_bifurcation2DIC(double tMax, int nPts, double h, int amountOfInitialConditions,
                                 const double* initialConditions, const double* ranges, const int* indicesOfMutVars,
                                 int writableVar, double maxValue, double transientTime, const double* values,
                                 int amountOfValues, int preScaller, double eps, const char* OUT_FILE_PATH);
int chaos_compat_bifurcation1DForH(double tMax, int nPts, int amountOfInitialConditions,
                                   const double* initialConditions, const double* ranges, int writableVar,
                                   double maxValue, double transientTime, const double* values, int amountOfValues,
                                   int preScaller, const char* OUT_FILE_PATH);
int chaos_compat_LLE1D(double tMax, double NT, int nPts, double h, double eps, const double* initialConditions,
                       int amountOfInitialConditions, const double* ranges, const int* indicesOfMutVars,
                       int writableVar, double maxValue, double transientTime, const double* values,
                       int amountOfValues, const char* OUT_FILE_PATH);
int chaos_compat_LLE1DIC(double tMax, double NT, int nPts, double h, double eps, const double* initialConditions,
                         int amountOfInitialConditions, const double* ranges, const int* indicesOfMutVars,
                         int writableVar, double maxValue, double transientTime, const double* values,
                         int amountOfValues, const char* OUT_FILE_PATH);
int chaos_compat_LLE2DIC(double tMax, double NT, int nPts, double h, double eps, const double* initialConditions,
                         int amountOfInitialConditions, const double* ranges, const int* indicesOfMutVars,
                         int writableVar, double maxValue, double transientTime, const double* values,
                         int amountOfValues, const char* OUT_FILE_PATH);
int chaos_compat_LS1D(double tMax, double NT, int nPts, double h, double eps, const double* initialConditions,
                      int amountOfInitialConditions, const double* ranges, const int* indicesOfMutVars,
                      int writableVar, double maxValue, double transientTime, const double* values,
                      int amountOfValues, const char* OUT_FILE_PATH);
int chaos_compat_LS2D(double tMax, double NT, int nPts, double h, double eps, const double* initialConditions,
                      int amountOfInitialConditions, const double* ranges, const int* indicesOfMutVars,
                      int writableVar, double maxValue, double transientTime, const double* values,
                      int amountOfValues, const char* OUT_FILE_PATH);
int chaos_compat_basinsOfAttraction(double tMax, int nPts, double h, int amountOfInitialConditions,
                                    const double* initialConditions, const double* ranges,
                                    const int* indicesOfMutVars, int writableVar, double maxValue,
                                    double transientTime, const double* values, int amountOfValues, int preScaller,
                                    double eps, const char* OUT_FILE_PATH);
}

#endif  // CHAOS_COMPAT_HPP
