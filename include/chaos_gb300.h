/*
 * C ABI of the GB300 (sm_103a) engine for ChaosLibrary's bifurcation / LLE /
 * basins hot path.
 *
 * Every entry point takes plain pointers and sizes, returns an int status
 * (CHAOS_OK or a negative CHAOS_E_* code; never exits the process) and keeps
 * the reference's argument names and meaning. The reference's entry points
 * write CSV files only; these return the same results in caller-owned arrays
 * (host or device memory, chosen by chaos_exec.memory). The C++ wrappers with
 * the reference's exact signatures, which write the reference's CSV files,
 * are declared in chaos_compat.hpp.
 *
 * Per-point flags keep the reference's values: 1 = bounded, 0 = diverged
 * (NaN, |x| >= 2^53 or |x| > maxValue), -1 = fixed point.
 *
 * Threading: calls are reentrant (no global device state); calls on one
 * stream run in order, calls on different streams may overlap.
 */
#ifndef CHAOS_GB300_H
#define CHAOS_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

#define CHAOS_ABI_VERSION 1

/* status codes */
#define CHAOS_OK 0
#define CHAOS_E_ARGS (-1)        /* invalid argument (message in chaos_last_error) */
#define CHAOS_E_NOMEM (-2)       /* device or host allocation failed */
#define CHAOS_E_CUDA (-3)        /* CUDA runtime error */
#define CHAOS_E_IO (-4)          /* file could not be written (compat wrappers) */
#define CHAOS_E_TIMEOUT (-5)     /* a bounded wait ran out */
#define CHAOS_E_UNSUPPORTED (-6) /* combination not implemented (e.g. FP32 LLE of a non-polynomial system) */
#define CHAOS_E_BUSY (-7)        /* admission refused: no slot or HBM budget left */
#define CHAOS_E_NODEV (-8)       /* no CUDA device */

/* arithmetic of the trajectories */
#define CHAOS_FP64 0 /* the reference's FP64 arithmetic; bit-identical to the CPU oracle */
#define CHAOS_FP32 1 /* FP32 state, FP64 accumulation (peak times, means, log-stretch sums) */
/* Float-float state: the base trajectory as the unevaluated sum of two FP32
   words (about 48 significant bits, every operation on the FP32 pipe), the LLE
   twin as an exact FP32 difference, the log-stretch exact (power-of-two
   renormalisation) with one FP64 log. The LLE maps (chaos_lle2d,
   chaos_lle_sweep) and chaos_trajectory of the RK4 systems 0-2; other calls
   return CHAOS_E_UNSUPPORTED. */
#define CHAOS_FF32 2

/* where the caller's arrays live */
#define CHAOS_MEM_HOST 0   /* results are copied back and the call returns when they are there */
#define CHAOS_MEM_DEVICE 1 /* device pointers; the call is asynchronous on `stream` */

/* built-in systems (the reference selects one at compile time in systems/systems.cuh:9) */
#define CHAOS_SYS_LORENZ_RK4 0  /* x'=s(y-x), y'=x(r-z)-y, z'=xy-bz; a={sigma,rho,beta}; classic RK4 */
#define CHAOS_SYS_ROSSLER_RK4 1 /* x'=-y-z, y'=x+ay, z'=b+z(x-c); a={a,b,c}; classic RK4 */
#define CHAOS_SYS_CHEN_RK4 2    /* x'=a(y-x), y'=(c-a)x-xz+cy, z'=xy-bz; a={a,b,c}; classic RK4 */
#define CHAOS_SYS_CHAMELEON 3   /* reference systems/systems.cuh:11-39 */
#define CHAOS_SYS_ROSSLER_CD 4  /* reference systems/systems.cuh:41-63 */
#define CHAOS_SYS_SIN3 5        /* reference systems/systems.cuh:67-83 (USE_SYSTEM_FOR_BASINS) */
#define CHAOS_SYS_SIN2 6        /* reference systems/systems.cuh:85-101 (USE_SYSTEM_FOR_BASINS_2) */
#define CHAOS_SYS_MEMRISTOR 7   /* reference systems/systems.cuh:103-178 (USE_DAMIR_SYSTEM) */
/* A reference-format plug-in header (SIZE_X, SIZE_A, CALC_DISCRETE_MODEL; systems/systems.cuh:12-38)
   compiled in at build time (CHAOS_USER_SYSTEMS=<header>); FP64 single sweeps only. */
#define CHAOS_SYS_USER 15

/* Grid modes of the sweep calls that take one (chaos_bifurcation_sweep,
   chaos_lle_sweep, chaos_lyapunov_spectrum), OR-ed together. */
#define CHAOS_GRID_STATE 1 /* indicesOfMutVars address initial conditions, not parameters (the *IC analyses) */
#define CHAOS_GRID_LOG0 2  /* dimension 0 on a log scale: value n = 10^(log10(r0) + n*((log10(r1) - log10(r0)) /
                              (nPts - 1))), the legacy getValueByIdxLog (debri/cudaLibrary.cu:1191-1196) */
#define CHAOS_GRID_LOG1 4  /* dimension 1 on a log scale (ranges[2..3]) */
#define CHAOS_GRID_LOG_F32 8 /* log-scale values rounded as the legacy step-size sweep does,
                                (double)powf(10, (float)x) (debri/cudaLibrary.cu:1001); else pow in FP64 */
#define CHAOS_GRID_LEGACY_LOOP 16 /* chaos_bifurcation_sweep only: the legacy library's per-point loop
                                     instead of the current library's, in FP64 whatever the precision (see
                                     chaos_bifurcation_sweep) */
/* indicesOfMutVars[0] == CHAOS_MUT_STEP: dimension 0 sweeps the integration step h itself
   (chaos_bifurcation_sweep, dim 1; the legacy bifurcation1DForH, debri/hostLibrary.cu:1005-1240). */
#define CHAOS_MUT_STEP (-1)

typedef struct chaos_exec {
    int precision; /* CHAOS_FP64 or CHAOS_FP32 */
    int memory;    /* CHAOS_MEM_HOST or CHAOS_MEM_DEVICE */
    void* stream;  /* cudaStream_t; NULL = the library's stream for the device (pass
                      cudaStreamLegacy, not 0, to run on the legacy default stream) */
    int device;    /* CUDA device ordinal; -1 = the current device */
} chaos_exec;

/* Library version (CHAOS_ABI_VERSION) and last error message of this thread. */
int chaos_abi_version(void);
const char* chaos_last_error(void);

/* Number of kernels this library has launched in the process so far (all
 * devices and threads; a plan replay adds the kernels of its graph). No
 * reference counterpart: lets a caller count the launches of a region. */
int chaos_launch_count(long long* count);

/* SIZE_X / SIZE_A of a built-in system (reference systems/systems.cuh SIZE_X, SIZE_A). */
int chaos_system_info(int system, int* sizeX, int* sizeA);

/* Waits for the work of `ex` (its stream) to finish. */
int chaos_synchronize(const chaos_exec* ex);

/*
 * 1-D bifurcation sweep. Replaces Bifurcation::bifurcation1D
 * (Bifurcation/include/bifurcationHOST.h:16-30, Bifurcation/src/bifurcationCUDA.cu:587-783).
 * Point k sweeps values[indicesOfMutVars[0]] over ranges[0..1] (nPts points).
 * Outputs per point k (arrays of nPts, rows of peakCapacity):
 *   counts[k]  kept peaks (the reference's amountOfPeaks), -1 fixed point, 0 diverged / none;
 *              the true count even when it exceeds peakCapacity
 *   flags[k]   1 / 0 / -1
 *   firstSample[k]  x[writableVar] at the first recorded sample (the reference's row for -1)
 *   peaks[k*cap + j], intervals[k*cap + j]  for j < min(counts[k], peakCapacity)
 *              (entries past that are left unspecified, as in the reference)
 * firstSample, peaks and intervals may be NULL.
 */
int chaos_bifurcation1d(const chaos_exec* ex, int system, double tMax, int nPts, double h,
                        int amountOfInitialConditions, const double* initialConditions, const double* ranges,
                        const int* indicesOfMutVars, int writableVar, double maxValue, double transientTime,
                        const double* values, int amountOfValues, int preScaller, int peakCapacity, int* counts,
                        int* flags, double* firstSample, double* peaks, double* intervals);

/*
 * 2-D bifurcation sweep with the per-point interval clustering. Replaces
 * Bifurcation::bifurcation2D (Bifurcation/include/bifurcationHOST.h:35-50,
 * Bifurcation/src/bifurcationCUDA.cu:43-256). labels[nPts*nPts] receives the
 * reference's dbscanCUDA result per point (point k: first swept value index
 * k % nPts, second k / nPts). counts (may be NULL) as in chaos_bifurcation1d.
 */
int chaos_bifurcation2d(const chaos_exec* ex, int system, double tMax, int nPts, double h,
                        int amountOfInitialConditions, const double* initialConditions, const double* ranges,
                        const int* indicesOfMutVars, int writableVar, double maxValue, double transientTime,
                        const double* values, int amountOfValues, int preScaller, double eps, int* labels,
                        int* counts);

/*
 * Bifurcation sweep over a 1-D or 2-D grid with a grid mode (CHAOS_GRID_*):
 * parameters or initial conditions, linear or log-scale axes, or the step
 * size. The legacy library's bifurcation1DIC / bifurcation2DIC
 * (debri/hostLibrary.cu:1243-1486, 2819-3107) are gridMode CHAOS_GRID_STATE |
 * CHAOS_GRID_LEGACY_LOOP; its step-size sweep bifurcation1DForH
 * (debri/hostLibrary.cu:1005-1240) is dim 1, indicesOfMutVars[0] =
 * CHAOS_MUT_STEP, gridMode CHAOS_GRID_LOG0 | CHAOS_GRID_LOG_F32 |
 * CHAOS_GRID_LEGACY_LOOP (h is then ignored: point k integrates with its own step
 * h_k, (int)(transientTime / h_k) transient steps, (int)(tMax / h_k /
 * preScaller) samples, intervals in units h_k * preScaller). Loop, peak rule
 * and clustering are chaos_bifurcation1d's / chaos_bifurcation2d's, which are
 * this call with gridMode 0.
 * CHAOS_GRID_LEGACY_LOOP runs the legacy library's per-point loop, as its
 * analyses do, in FP64. Grids over initial conditions or parameters follow
 * calculateDiscreteModelICCUDA (debri/cudaLibrary.cu:1022-1116, the loop
 * :604-680):
 *   - the transient tests only state component 0, and only for NaN or
 *     infinity (flag 0);
 *   - a transient that ends at a fixed point still runs the recorded part;
 *   - every recorded sample is followed by preScaller steps;
 *   - the fixed-point test is sqrt(|sum|) < 1e-9 in FP64 (flag -1, count -1).
 * The step-size sweep follows calculateDiscreteModelCUDA_H (:955-1000, the
 * loop :472-527):
 *   - the transient's verdict is ignored (it only stops early at a NaN or
 *     infinite component 0);
 *   - a point whose last state change is exactly 0, or has a norm below
 *     1e-12, keeps no peaks (flag -1).
 * The peak rule and the per-point clustering are the same in both libraries.
 * dim 1: outputs as chaos_bifurcation1d (labels must be NULL).
 * dim 2: labels[nPts*nPts] and counts (may be NULL) as chaos_bifurcation2d;
 *        flags, firstSample, peaks and intervals must be NULL, peakCapacity 0.
 */
int chaos_bifurcation_sweep(const chaos_exec* ex, int system, int dim, int gridMode, double tMax, int nPts,
                            double h, int amountOfInitialConditions, const double* initialConditions,
                            const double* ranges, const int* indicesOfMutVars, int writableVar, double maxValue,
                            double transientTime, const double* values, int amountOfValues, int preScaller,
                            double eps, int peakCapacity, int* counts, int* flags, double* firstSample,
                            double* peaks, double* intervals, int* labels);

/*
 * Dense peak list of a 1-D sweep's rows (chaos_bifurcation1d /
 * chaos_bifurcation_sweep outputs): the kept peaks of point k, min(max(counts[k],
 * 0), peakCapacity) of them, move from row k to positions offsets[k] ..
 * offsets[k+1]-1 of densePeaks / denseIntervals (densePoint receives k there):
 * the reference CSV's row order without the empty rows. Prefix sums of the
 * counts on the device, then a warp per point. offsets (n + 1 entries) and the
 * dense arrays may be NULL; *total (host memory) always receives the number of
 * kept peaks, so a first call with NULL dense arrays sizes them. When
 * denseCapacity < *total the first denseCapacity entries are written and the
 * call returns CHAOS_E_ARGS.
 */
int chaos_compact_peaks(const chaos_exec* ex, const int* counts, const double* peaks, const double* intervals,
                        long long n, int peakCapacity, long long* offsets, double* densePeaks,
                        double* denseIntervals, int* densePoint, long long denseCapacity, long long* total);

/*
 * Largest-Lyapunov-exponent map. Replaces LLE::LLE2D (LLE/include/LLEHost.h:25-41,
 * LLE/src/LLECUDA.cu:205-428). lle[j*nPts + i] is the value at
 * values[indicesOfMutVars[0]] = linspace(ranges[0], ranges[1])[i] and
 * values[indicesOfMutVars[1]] = linspace(ranges[2], ranges[3])[j]: the
 * reference CSV's transposed layout (row = second parameter). The twin
 * trajectory starts at x + eps along state component 0 (the reference draws a
 * random unit direction with cuRAND). writableVar and maxValue are accepted
 * and unused, as in the reference. CHAOS_FP32 is supported for the three RK4
 * systems and Chameleon (the twin carried as an exact difference, FP64 log
 * sum).
 */
int chaos_lle2d(const chaos_exec* ex, int system, double tMax, double NT, int nPts, double h, double eps,
                const double* initialConditions, int amountOfInitialConditions, const double* ranges,
                const int* indicesOfMutVars, int writableVar, double maxValue, double transientTime,
                const double* values, int amountOfValues, double* lle);

/*
 * The Benettin stage of the LLE map on caller-supplied starting states:
 * replaces the reference's calculateSystem kernel (LLE/src/LLECUDA.cu:114-166),
 * which reads the semi_result rows its transient kernel wrote
 * (LLECUDA.cu:56-112). states holds n rows of 2*SIZE_X + SIZE_A values:
 * the orbit after the transient, the point's parameters, the twin's start
 * (the reference's row layout). lle[k] = sum over calcBlocks + 1 blocks of
 * NT/h steps of log(|x - p| / eps), over tMax, with the reference's
 * renormalisation (CHAOS_FP64), or with the orbit in float-float and the twin
 * as the FP32 difference p - x (CHAOS_FF32, RK4 systems). No transient is
 * run: a caller can hand over the reference's own randomised twin starts
 * (its cuRAND draw, LLECUDA.cu:88-101) and compare on identical inputs.
 */
int chaos_lle_from_states(const chaos_exec* ex, int system, long long n, const double* states, double tMax,
                          double NT, double h, double eps, double* lle);

/*
 * LLE over a 1-D or 2-D grid of parameters (gridMode 0) or of initial
 * conditions (gridMode CHAOS_GRID_STATE), linear or log-scale axes
 * (CHAOS_GRID_LOG0 / LOG1 / LOG_F32): the grids of the legacy library's
 * LLE1D, LLE1DIC, LLE2D and LLE2DIC analyses (debri/hostLibrary.cu:3111-3828;
 * their own kernels' scheme is chaos_lle_sweep_legacy) with the
 * Benettin scheme of chaos_lle2d (twin at x + eps*e_x, calcBlocks + 1 blocks,
 * sum / tMax). dim 1: ranges[0..1] and indicesOfMutVars[0], lle[i] for
 * i < nPts; dim 2: ranges[0..3], indicesOfMutVars[0..1], lle[j*nPts + i] as
 * chaos_lle2d (which is this call with dim 2, gridMode 0). CHAOS_FP32 for the
 * RK4 systems and Chameleon.
 */
int chaos_lle_sweep(const chaos_exec* ex, int system, int dim, int gridMode, double tMax, double NT, int nPts,
                    double h, double eps, const double* initialConditions, int amountOfInitialConditions,
                    const double* ranges, const int* indicesOfMutVars, double transientTime, const double* values,
                    int amountOfValues, double* lle);

/*
 * The legacy library's LLE analyses with its own kernels' scheme, in FP64
 * whatever the precision: LLEKernelCUDA (debri/cudaLibrary.cu:1897-2031;
 * LLE1D, gridMode without CHAOS_GRID_STATE) and LLEKernelICCUDA (:2034-2139;
 * LLE1DIC / LLE2DIC, gridMode CHAOS_GRID_STATE). Grids and outputs as
 * chaos_lle_sweep. Per point:
 *   - the twin direction is the normalised raw draw z (see
 *     chaos_legacy_lle_draws), or draws[p*SIZE_X + k] when draws is not NULL;
 *   - transientTime / h steps of the orbit, then the twin y = x + eps*z;
 *   - (int)(tMax / NT) blocks of NT / h steps of the orbit and of the twin;
 *     every run of steps stops early where state component 0 becomes NaN or
 *     infinite or |(float)x[0]| > maxValue (maxValue 0: no bound);
 *   - each block adds log(d) with d = |x - y| / eps, computed and applied as
 *     the kernel of the grid kind computes it;
 *   - the sum is divided by tMax.
 */
int chaos_lle_sweep_legacy(const chaos_exec* ex, int system, int dim, int gridMode, double tMax, double NT,
                           int nPts, double h, double eps, const double* initialConditions,
                           int amountOfInitialConditions, const double* ranges, const int* indicesOfMutVars,
                           double maxValue, double transientTime, const double* values, int amountOfValues,
                           const double* draws, double* lle);

/*
 * The legacy library's LS1D / LS2D with its own kernel's scheme, in FP64
 * (LSKernelCUDA, debri/cudaLibrary.cu:2189-2330; built-in systems). Grids and
 * spectrum[p*SIZE_X + j] as chaos_lyapunov_spectrum. Per point:
 *   - twin j starts along row j of the raw draws (chaos_legacy_lle_draws kind
 *     2, or draws[(p*SIZE_X + j)*SIZE_X + i]), each row normalised, after the
 *     transient the rows orthonormalised by classical Gram-Schmidt, twin j at
 *     x + eps*u_j;
 *   - (int)(tMax / NT) blocks of NT / h steps of the orbit and of every twin,
 *     each run stopping early as in chaos_lle_sweep_legacy;
 *   - the differences through Gram-Schmidt, exponent j adding
 *     log(|w_j| / eps), twin j restarting at x + eps*w_j/|w_j|;
 *   - the sums divided by tMax.
 */
int chaos_lyapunov_spectrum_legacy(const chaos_exec* ex, int system, int dim, int gridMode, double tMax, double NT,
                                   int nPts, double h, double eps, const double* initialConditions,
                                   int amountOfInitialConditions, const double* ranges, const int* indicesOfMutVars,
                                   double maxValue, double transientTime, const double* values, int amountOfValues,
                                   const double* draws, double* spectrum);

/*
 * The raw twin-direction draws of the legacy LLE kernels for points [0, n)
 * of a one-chunk grid (the legacy thread index is the point index), nx
 * components each: draws[p*nx + k].
 *   kind 0 (parameter grids, LLEKernelCUDA): the uniform of cuRAND's default
 *     generator seeded p + k (curand_init(p + k, 0, 0)), minus 0.5;
 *   kind 1 (initial-condition grids, LLEKernelICCUDA): 0.5 * sinf(p * (k * p
 *     + 1) + 1), the integer expression in 32-bit wrap-around arithmetic;
 *   kind 2 (the spectrum, LSKernelCUDA): nx rows of nx, draws[(p*nx + j)*nx +
 *     i] = 0.5 * sinf(0.2171828 (i+1)(j+1) + p + (0.2171828 + i j p)), the
 *     argument in FP64 rounded to float.
 */
int chaos_legacy_lle_draws(const chaos_exec* ex, int kind, long long n, int nx, double* draws);

/*
 * Lyapunov spectrum over the same grids (the legacy library's LS1D / LS2D,
 * debri/hostLibrary.cu:3829-4111, kernel debri/cudaLibrary.cu:2141-2330; its
 * own kernel's twin start and block count are chaos_lyapunov_spectrum_legacy):
 * one twin per state dimension started along the unit vectors, classical
 * Gram-Schmidt of the twin differences after every block of NT, exponent j =
 * sum of log(|b_j| / eps) / tMax over calcBlocks + 1 blocks (the LLE map's
 * count; exponent 0 estimates what chaos_lle_sweep estimates).
 * spectrum[p*SIZE_X + j], p and gridMode as in chaos_lle_sweep. Built-in systems; FP32
 * for the RK4 systems and Chameleon (exact-difference twins).
 */
int chaos_lyapunov_spectrum(const chaos_exec* ex, int system, int dim, int gridMode, double tMax, double NT,
                            int nPts, double h, double eps, const double* initialConditions,
                            int amountOfInitialConditions, const double* ranges, const int* indicesOfMutVars,
                            double transientTime, const double* values, int amountOfValues, double* spectrum);

/*
 * LLE map in FP32 with an FP64 sign re-check (no reference counterpart: the
 * reference computes in FP64 only). Arguments as chaos_lle2d (RK4 systems
 * 0-2 and Chameleon; ex->precision is ignored). The map is computed as chaos_lle2d with
 * CHAOS_FP32; every point whose FP32 value v has |v| <= band or is not finite
 * is integrated again in FP64 over a short horizon of checkTMax time units
 * (same transient, NT and eps). Where the check's class (positive,
 * non-positive, not finite) differs from v's, the point's value is replaced by
 * its FP64 value over the full horizon, bit-identical to chaos_lle2d with
 * CHAOS_FP64 there. checkTMax >= tMax makes the check itself that full run.
 * nChecked / nReplaced (may be NULL) receive the numbers of points checked and
 * replaced. The call waits for the selection and the check (two host syncs).
 */
int chaos_lle2d_checked(const chaos_exec* ex, int system, double tMax, double NT, int nPts, double h, double eps,
                        const double* initialConditions, int amountOfInitialConditions, const double* ranges,
                        const int* indicesOfMutVars, double transientTime, const double* values, int amountOfValues,
                        double band, double checkTMax, double* lle, long long* nChecked, long long* nReplaced);

/*
 * Per-point basin features over the nPts x nPts grid of initial conditions
 * (initialConditions[indicesOfMutVars[0]] over ranges[0..1] fastest,
 * initialConditions[indicesOfMutVars[1]] over ranges[2..3]). The first stage
 * of Basins::basinsOfAttraction_2 (Basins/src/basinsCUDA.cu:602-692, kernels
 * :233-314 and avgPeakFinderCUDA :818-864): flags, avgPeaks, avgIntervals
 * with the reference's sentinels (flag 0: 999/999; flag -1: last sample/-1;
 * no peaks: 1000/1000) and counts = kept peaks (may be NULL).
 */
int chaos_basins_features(const chaos_exec* ex, int system, double tMax, int nPts, double h,
                          int amountOfInitialConditions, const double* initialConditions, const double* ranges,
                          const int* indicesOfMutVars, int writableVar, double maxValue, double transientTime,
                          const double* values, int amountOfValues, int preScaller, int* flags, double* avgPeaks,
                          double* avgIntervals, int* counts);

/*
 * Basins of attraction. Replaces Basins::basinsOfAttraction_2
 * (Basins/include/basinsHOST.h:15-30, Basins/src/basinsCUDA.cu:442-813):
 * features as chaos_basins_features, then the reference's global clustering
 * (CUDA_dbscan, basinsCUDA.cu:35-179) as chaos_dbscan_compat. Any output
 * pointer but labels may be NULL.
 */
int chaos_basins(const chaos_exec* ex, int system, double tMax, int nPts, double h, int amountOfInitialConditions,
                 const double* initialConditions, const double* ranges, const int* indicesOfMutVars,
                 int writableVar, double maxValue, double transientTime, const double* values, int amountOfValues,
                 int preScaller, double eps, int* labels, double* avgPeaks, double* avgIntervals, int* flags);

/*
 * Basins of attraction with the features and clustering of the benchmark's
 * basins workload (no reference counterpart; the reference clusters with the
 * rule of chaos_dbscan_compat): per grid point the features (mean peak
 * amplitude, kept peak count, mean peak interval) of the reference's peak
 * rules, with a point without peaks taking (last sample, 0, 0); each feature
 * min-max scaled to [0, 1] over the points with flag != 0; then chaos_dbscan
 * (eps, minPts) on that n x 3 matrix. labels: clusters 0.., noise -1,
 * diverged points (flag 0) -2. features (n x 3, normalised) and flags may be NULL.
 */
int chaos_basins_dbscan(const chaos_exec* ex, int system, double tMax, int nPts, double h,
                        int amountOfInitialConditions, const double* initialConditions, const double* ranges,
                        const int* indicesOfMutVars, int writableVar, double maxValue, double transientTime,
                        const double* values, int amountOfValues, int preScaller, double eps, int minPts,
                        int* labels, double* features, int* flags);

/*
 * The reference's basin clustering on given feature arrays
 * (CUDA_dbscan + CUDA_dbscan_kernel, Basins/src/basinsCUDA.cu:35-179, 894-923):
 * eps-connected components (sqrt(dp^2 + di^2) <= eps, FP64) over the points
 * with flag != 0. Components that hold a fixed point (flag -1) are numbered
 * -1, -2, ... in order of their smallest fixed-point index, the others 1, 2,
 * ... in order of their smallest index; flag-0 points get 0. (The reference
 * numbers components in a racy seed order; the partition is the same.)
 */
int chaos_dbscan_compat(const chaos_exec* ex, const double* avgPeaks, const double* avgIntervals, const int* flags,
                        long long n, double eps, int* labels);

/*
 * DBSCAN with scikit-learn semantics on an n x dims feature matrix (row-major,
 * dims 1..3): core points have >= minPts points (themselves included) within
 * distance <= eps; clusters are numbered 0, 1, ... by their smallest core
 * index; a border point joins the lowest-numbered adjacent cluster; noise is
 * -1; points with mask[i] == 0 (mask may be NULL) are left out and get -2.
 * No reference counterpart (the reference clusters with chaos_dbscan_compat's rule).
 */
int chaos_dbscan(const chaos_exec* ex, const double* features, long long n, int dims, double eps, int minPts,
                 const int* mask, int* labels);

/*
 * The reference's peakFinder on caller series (Bifurcation/src/bifurcationCUDA.cu:469-514):
 * data is nSeries x len (row-major); counts, peaks and intervals as in
 * chaos_bifurcation1d, with intervals in units of h.
 */
int chaos_peak_finder(const chaos_exec* ex, const double* data, long long nSeries, int len, double h,
                      int peakCapacity, int* counts, double* peaks, double* intervals);

/*
 * The reference's per-point clustering of the 2-D bifurcation on caller
 * interval rows (dbscanCUDA + dbscan, Bifurcation/src/bifurcationCUDA.cu:373-398, 516-572):
 * intervals is n x stride, counts[k] the number of intervals of row k (-1 and
 * 0 pass through as in the reference). labels[k] = clusters - 1; a row whose
 * count exceeds stride gets INT_MIN.
 */
int chaos_point_dbscan(const chaos_exec* ex, const double* intervals, const int* counts, long long n, int stride,
                       double eps, int* labels);

/*
 * Batched sweeps (no reference counterpart: the reference compiles one system
 * in and runs one sweep per call). Many independent jobs of different kinds,
 * systems, sizes and transients run in ONE persistent launch that pulls
 * chunks of points from a device work queue. FP32 trajectories with FP64
 * accumulation, or float-float for CHAOS_JOB_LLE2D_FF32 jobs (ex->precision
 * is ignored); a point's result is bit-identical to the single-job call's in
 * that arithmetic. Arguments mean what they mean in the
 * single-job entry points; outputs are host or device arrays per ex->memory.
 */
#define CHAOS_JOB_BIF1D 1  /* chaos_bifurcation1d: counts, flags, first?, peaks?, intervals? */
#define CHAOS_JOB_LLE2D 2  /* chaos_lle2d (RK4 systems and Chameleon): lle */
#define CHAOS_JOB_BASINS 3 /* chaos_basins_features: flags, avgPeaks, avgIntervals, counts? */
#define CHAOS_JOB_LLE2D_FF32 4 /* chaos_lle2d with CHAOS_FF32 (RK4 systems 0-2): lle; bit-identical to
                                  the single-sweep CHAOS_FF32 call */

typedef struct chaos_job {
    int kind;
    int system;
    double tMax;
    int nPts;
    double h;
    const double* initialConditions; /* SIZE_X host values */
    const double* ranges;            /* 2 (bifurcation) or 4 values */
    const int* indicesOfMutVars;     /* 1 or 2 indices */
    int writableVar;
    double maxValue;
    double transientTime;
    const double* values;            /* SIZE_A host values */
    int preScaller;
    double NT;                       /* LLE */
    double eps;                      /* LLE */
    int peakCapacity;                /* bifurcation */
    int* counts;
    int* flags;
    double* first;
    double* peaks;
    double* intervals;
    double* lle;
    double* avgPeaks;
    double* avgIntervals;
    int* labels; /* basins in a server: with eps > 0, the reference clustering at completion */
} chaos_job;

/* Runs the jobs in one persistent launch (chunks ordered longest work first). */
int chaos_run_batch(const chaos_exec* ex, const chaos_job* jobs, int nJobs);

/*
 * A prepared batch: descriptors uploaded and the launch captured in a CUDA
 * graph once, replayed by chaos_batch_run (outputs rewritten every run).
 * Runs are ordered after the earlier work of ex->stream and before its later
 * work (the graph itself runs on a stream the plan owns). Outputs must stay
 * valid while the plan exists.
 */
typedef struct chaos_batch chaos_batch;
int chaos_batch_create(const chaos_exec* ex, const chaos_job* jobs, int nJobs, chaos_batch** plan);
int chaos_batch_run(chaos_batch* plan);
int chaos_batch_destroy(chaos_batch* plan);

/*
 * Serving (no reference counterpart): a request loop on one GPU. Requests
 * (chaos_job, any kind) are admitted first-come-first-served while their
 * device memory fits the HBM budget and fewer than maxActive are resident;
 * their parameters and partial results stay on the device until they are
 * complete. A scheduler thread runs iterations: each takes block-sized
 * chunks from the resident requests up to a work budget (iterationSteps
 * trajectory-steps), first an equal share for every request with work left,
 * then the rest oldest-first, so requests that arrive while others run join
 * the next iteration (continuous batching) and small requests are not held
 * behind large ones; two iterations are in flight at a time on two streams. A completion thread copies results back
 * (host-memory servers), runs the basins clustering for jobs that ask for it,
 * and records latency (submit -> results ready). A result is bit-identical to
 * the same job run alone (the same device function computes every point).
 */
typedef struct chaos_server chaos_server;
#define CHAOS_REQ_PENDING 0 /* waiting for admission */
#define CHAOS_REQ_RUNNING 1
#define CHAOS_REQ_DONE 2
#define CHAOS_REQ_FAILED 3
int chaos_server_create(const chaos_exec* ex, size_t hbmBudgetBytes, int maxActive, double iterationSteps,
                        chaos_server** server);
/* Copies the job's parameters; its output arrays must stay valid until the request is done. */
int chaos_server_submit(chaos_server* server, const chaos_job* job, long long* requestId);
int chaos_server_poll(chaos_server* server, long long requestId, int* state);
/* Waits at most timeoutSeconds; CHAOS_E_TIMEOUT when the request is not done by then. */
int chaos_server_wait(chaos_server* server, long long requestId, double timeoutSeconds, int* state);
/*
 * stats[0..11] = completed, failed, pending, running, p50 latency (s), p99 latency (s),
 * mean latency (s), trajectory-steps completed, seconds since the first submission,
 * iterations launched, peak HBM bytes in use, max latency (s).
 */
int chaos_server_stats(chaos_server* server, double* stats, int n);
/* Latency (s) of a completed request, -1 otherwise. */
double chaos_server_latency(chaos_server* server, long long requestId);
/* Stops admitting, finishes the resident requests, fails the pending ones, frees everything. */
int chaos_server_destroy(chaos_server* server);

/*
 * chaos_point_dbscan without any allocation. No counterpart in the reference:
 * for callers that cannot call cudaMalloc during the call (hosts that reserve
 * all device memory through their own allocator and budget, latency-critical
 * loops where cudaMalloc / cudaFree would synchronise the device). Every array
 * is a device pointer (ex->memory must be CHAOS_MEM_DEVICE); ex->stream NULL
 * means the legacy default stream; the call is asynchronous. The scratch rows
 * live in one fixed array compiled into the library (8 MiB per GPU that loads
 * it, kept until exit), so n * stride is limited to 1,048,576 (larger sizes
 * return CHAOS_E_ARGS). All calls share that array: calls whose kernels
 * overlap on the GPU race and must be serialised by the caller. Every call
 * looks up the array's device address in the current context (a lookup, no
 * allocation); the first call on a device also loads the library's device
 * code there, so make it before any stream capture.
 */
int chaos_point_dbscan_noalloc(const chaos_exec* ex, const double* intervals, const int* counts, long long n,
                               int stride, double eps, int* labels);

/*
 * Trajectories of a built-in system (no reference counterpart; the
 * reference's phase portraits come from a separate Python script): nTraj
 * independent trajectories, x0 (nTraj x SIZE_X) and a (nTraj x SIZE_A)
 * row-major, nSteps steps of CALC_DISCRETE_MODEL each. out holds
 * nTraj x (nSteps + 1) x SIZE_X states: the start and the state after every step.
 */
int chaos_trajectory(const chaos_exec* ex, int system, long long nTraj, const double* x0, const double* a, double h,
                     int nSteps, double* out);

/*
 * Kernel-shape knobs (no reference counterpart). CHAOS_TUNE_LLE_F32_VARIANT:
 * 2 = two grid points per thread in packed FP32x2 instructions, 12 / 16 = one
 * point per thread with registers shaped for 12 / 16 resident blocks per SM,
 * 0 = the library default. Process-wide; results do not depend on it.
 */
#define CHAOS_TUNE_LLE_F32_VARIANT 1
/* CHAOS_TUNE_SWEEP_PAIRS: FP32 bifurcation / basins sweeps of the RK4 systems
   run two points per thread in packed FP32x2 lanes: 1 (default) for sweeps
   of at least 4 x SMs x 1024 points -- 1-D bifurcations as hybrid pairs
   (packed transient, recorded part lane by lane), basins maps fully packed --
   2 always fully packed, 0 never (one point per thread), 3 always hybrid.
   Results are identical in every mode. */
#define CHAOS_TUNE_SWEEP_PAIRS 2
/* CHAOS_TUNE_GRID_FMA: 0 (default) swept values start + n*scale with the
   multiply and the add rounded apart, as the reference's getValueByIdx is
   written (bifurcationCUDA.cu:400-419); 1 as one fused multiply-add, which is
   what the reference's own GPU build computes (nvcc contracts the expression
   by default): with 1, FP64 bifurcation and basins sweeps reproduce that
   build's output bit for bit (for plug-ins free of contractible products).
   With 1 the LLE map (chaos_lle2d) also takes its swept values as one FMA,
   as the reference's host linspace (LLECUDA.cu:195-200) computes them where
   its host compiler contracts the expression (aarch64 by default).
   Initial value from the environment: CHAOS_GRID_FMA=1. */
#define CHAOS_TUNE_GRID_FMA 3
/* CHAOS_TUNE_LLE_TWIN: 0 (default) the twin trajectory starts at x + eps*e_x;
   1 the reference's start (LLECUDA.cu:97-101) along e_x: every state
   component rounded to float and eps added by a float FMA; 2 the reference's
   start itself (LLECUDA.cu:87-101): the direction drawn by cuRAND's device
   API seeded with the point index, normalised and applied in FP32 as there.
   FP64 only. Initial value: CHAOS_LLE_TWIN=1 or 2. */
#define CHAOS_TUNE_LLE_TWIN 4
/* CHAOS_TUNE_BIF2D_CAP: peak rows per point of the 2-D bifurcation's
   clustering scratch. 0 (default): B/2 (the most a point can keep) when the
   grid fits the scratch budget with it, else what lets the grid run as one
   chunk (at least 512), else measured from the kept-peak counts of up to
   4096 evenly spread points (+25 % + 16); > 0 that many; -1 always B/2.
   Points with more peaks than the capacity are run again with B/2 rows:
   results never depend on it. */
#define CHAOS_TUNE_BIF2D_CAP 5
/* CHAOS_TUNE_SHAPES: 0 forgets the launch shapes chaos_autotune installed
   (the built-in rules apply again). */
#define CHAOS_TUNE_SHAPES 6
/* CHAOS_TUNE_LLE_RENORM: how the FP32 LLE maps of the RK4 systems
   (chaos_lle2d, chaos_lle_sweep) measure each Benettin block's stretch.
   0 (default): the twin is rescaled by an exact power of two and the
   stretch summed exactly (an integer count of octaves plus one FP64 log of
   the final FP64 norm); 1: log2 of the FP32 norm per block on the SFU,
   summed in FP32 groups of 16 blocks added in FP64; 2: the reference's
   arithmetic, FP64 norm and FP64 log per block (LLE/src/LLECUDA.cu:146-162).
   Modes 1 and 2 run the two-points-per-thread kernel; process-wide. */
#define CHAOS_TUNE_LLE_RENORM 7
/* CHAOS_TUNE_FF_PAIRS: CHAOS_FF32 LLE maps run two points per thread in
   packed FP32x2 words (1, default) or one (0); results are identical. */
#define CHAOS_TUNE_FF_PAIRS 8
int chaos_set_tuning(int knob, int value);
int chaos_get_tuning(int knob);

/*
 * Self-timing tuner (no reference counterpart). Times the launch shapes of the
 * FP32 sweeps of the three RK4 systems -- one or two trajectories per thread,
 * the LLE map's register shapes, blocks of 64 / 128 / 256 threads -- on probe
 * sweeps that fill the GPU of ex (about 2-3 s in all), and installs the
 * fastest per (kind, system) for every later call in the process; a shape
 * replaces the built-in rule only when at least 1 % faster. Results do not
 * depend on shapes. An explicit CHAOS_TUNE_SWEEP_PAIRS (0 / 2 / 3) or
 * CHAOS_TUNE_LLE_F32_VARIANT still wins. table (may be NULL) receives nTable
 * rows (9 fill all) of 6 doubles: kind (0 1-D bifurcation, 1 basins, 2 LLE
 * map), system, form (0 rule; 1 / 2 trajectories per thread; 3 basins hybrid
 * pairs; 12 / 16 LLE register shapes), block, best ms, the built-in rule's ms.
 */
int chaos_autotune(const chaos_exec* ex, double* table, int nTable);

/*
 * FP32 FMA-pipe probe (no reference counterpart): times `iters` rounds of 8
 * independent fmaf chains in 2048 threads per SM and returns the elapsed
 * seconds and the flops executed, the measured denominator of the
 * integration kernels' roofline.
 */
int chaos_fma_probe(const chaos_exec* ex, long long iters, double* seconds, double* flops);

/*
 * Architecture of the device code the library loaded on `device` (-1 = the
 * current one): cudaFuncAttributes.binaryVersion and .ptxVersion of one of
 * its kernels (103 for an sm_103a build). No reference counterpart.
 */
int chaos_device_code_version(int device, int* binaryVersion, int* ptxVersion);

#ifdef __cplusplus
}
#endif
#endif /* CHAOS_GB300_H */
