// Parameter blocks passed by value to the sweep kernels, and the launchers
// the C-ABI layer calls. Every per-call scalar travels in a kernel argument
// (no __constant__ globals), so calls on different streams never interfere.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace chaos {

// Kernels launched by this library (all devices and threads): every launch
// site adds one; a captured CUDA graph adds its kernel nodes at each replay.
void note_launch(long long n = 1);
long long launch_count();

constexpr int kMaxState = 12;
constexpr int kMaxParams = 16;

// Parameter or initial-condition grid of a sweep: point p has coordinate
// n_d = (p / nPts^d) % nPts in dimension d and value start[d] + n_d*scale[d].
// A dimension with a table (log-scale axes) takes its value from table[d][n_d]
// instead: nPts values the host computed.
struct GridSpec {
    long long nPts;
    double start[2];
    double scale[2];
    int fused;  // 1: start + n*scale as one FMA (what nvcc's default contraction makes of the reference's getValueByIdx)
    const double* table[2];  // device arrays of nPts values, or null (linear axis)
};

struct SweepParams {
    int system;
    int dim;          // 1 or 2 swept dimensions
    int S;            // transient steps
    int B;            // recorded samples
    int preScaller;   // steps per recorded sample (basins); 1 for bifurcation
    int wv;           // recorded state component
    int checkMax;     // maxValue != 0
    int mutateState;  // 1: the grid sets initial conditions (basins); 0: parameters
    double h;
    double hInterval;  // h * preScaller, the time unit of peak intervals
    double maxValue;
    float maxValueF;   // the largest float <= maxValue: for a float v, |v| > maxValue <=> |v| > maxValueF
    unsigned long long maxBits;  // for a double v: (double)fabsf((float)v) > maxValue <=> bits(|v|) > maxBits,
    int maxTie;                  //   or == maxBits with maxTie (the rounding boundary of float(v))
    double ic[kMaxState];
    double values[kMaxParams];
    int mut[2];
    GridSpec grid;
    long long pBegin;   // first point of this launch
    long long nPoints;  // points in this launch
    // Step-size sweep (bifurcation): dimension 0 sets the integration step h of
    // each point, which then runs (int)(transientTime / h) transient steps and
    // (int)(tMax / h / bPre) recorded samples with intervals in units h * bPre.
    int sweepStep;
    int bPre;  // the caller's preScaller
    double tMax, transientTime;
    // The legacy library's per-point loop (FP64 kernels only): 0 off, 1 the
    // initial-condition / parameter grids, 2 the step-size sweep.
    int legacyLoop;
};

// Per-point results of a bifurcation sweep (point-major rows of `cap`).
struct BifOut {
    int* counts;        // kept peaks, or -1 fixed point, 0 diverged / none
    int* flags;         // 1 / 0 / -1
    double* first;      // first recorded sample (the reference's row for fixed points)
    double* peaks;      // [n][cap] (may be null)
    double* intervals;  // [n][cap] (may be null)
    int cap;
};

struct BasinsOut {
    int* flags;
    double* avgPeaks;
    double* avgIntervals;
    int* counts;   // kept peaks (may be null)
    double* last;  // x[writableVar] at the last recorded sample (may be null)
    // order-key minima / maxima of the clustering features of the points with
    // flag != 0, kKeyReplicas replicas per key (order_keys.h); null: not kept
    unsigned long long* mm = nullptr;
};

struct LleParams {
    int system;
    int nPts;
    int trans, ntp, calcBlocks;
    double h, eps, tMax;
    double ic[kMaxState];
    double values[kMaxParams];
    int mut[2];
    double rangeA[2], rangeB[2];
    double stepA, stepB;  // linspace steps (end - start) / (nPts - 1)
    long long pBegin, nPoints;
    int twin;  // twin start: 0 x + eps e_x; 1 the reference's, every component rounded to float (FP64 only)
    int dim;          // 1: point p = index i of rangeA; 2: p = j*nPts + i (the LLE2D map)
    int mutateState;  // 0: the grid sets values[mut]; 1: it sets initial conditions ic[mut]
    const double* table[2];  // log-scale axes: device arrays of nPts values (null: linspace)
    // The legacy library's LLE kernels' scheme (legacy_lle.cuh, FP64): legacyLoop
    // 1, legacyBlocks = (int)(tMax / NT) blocks, the bound maxValue (0: none)
    // and the raw twin draws of every point (null: the legacy's own).
    int legacyLoop, legacyBlocks;
    double maxValue;
    const double* draws;
};

// precision-specific launchers (kern_f64.cu / kern_f32.cu)
cudaError_t launch_bif_f64(const SweepParams& P, const BifOut& O, cudaStream_t st);
cudaError_t launch_bif_f32(const SweepParams& P, const BifOut& O, cudaStream_t st);
cudaError_t launch_basins_f64(const SweepParams& P, const BasinsOut& O, cudaStream_t st);
cudaError_t launch_basins_f32(const SweepParams& P, const BasinsOut& O, cudaStream_t st);
cudaError_t launch_lle_f64(const LleParams& L, double* out, cudaStream_t st);
// the legacy LLE kernels' raw twin draws of points [0, n) (kern_f64.cu): kind 0
// parameter grids (cuRAND), 1 initial-condition grids (sinf), out[p*nx + k];
// kind 2 the spectrum's, out[(p*nx + j)*nx + i] for component i of twin j
cudaError_t launch_legacy_draws(int kind, long long n, int nx, double* out, cudaStream_t st);
cudaError_t launch_lle_f32(const LleParams& L, double* out, cudaStream_t st);
// float-float base trajectory, FP32 twin difference (kern_ff.cu; RK4 systems)
cudaError_t launch_lle_ff(const LleParams& L, double* out, cudaStream_t st);
// Benettin blocks from caller-supplied states, rows of 2*SIZE_X + SIZE_A (orbit, parameters,
// twin; kern_f64.cu / kern_ff.cu)
cudaError_t launch_lle_states_f64(const LleParams& L, const double* states, double* out, cudaStream_t st);
cudaError_t launch_lle_states_ff(const LleParams& L, const double* states, double* out, cudaStream_t st);
int set_ff_pairs(int v);  // 1: two points per thread (default), 0: one
int get_ff_pairs();
// Lyapunov spectrum, out[p*SIZE_X + j] (FP64: every built-in system; FP32: the RK4 systems)
cudaError_t launch_spectrum_f64(const LleParams& L, double* out, cudaStream_t st);
cudaError_t launch_spectrum_f32(const LleParams& L, double* out, cudaStream_t st);
// bifurcation points of a list (row k for list[k]); points whose kept-peak
// count exceeds cap (kern_f64.cu / kern_f32.cu)
cudaError_t launch_bif_list_f64(const SweepParams& P, const BifOut& O, const int* list, int count, cudaStream_t st);
cudaError_t launch_bif_list_f32(const SweepParams& P, const BifOut& O, const int* list, int count, cudaStream_t st);
cudaError_t launch_overflow_select(const int* counts, long long n, int cap, int* list, int* count, cudaStream_t st);
// FP64 sign re-check of an FP32 LLE map (kern_f64.cu): select the points with
// |v| <= band or v not finite, FP64 LLE of a point list, compare classes
cudaError_t launch_lle_select(const double* v, long long n, double band, int* list, int* count, cudaStream_t st);
cudaError_t launch_lle_list_f64(const LleParams& L, const int* list, const int* count, long long maxCount,
                                double* out, bool scatter, cudaStream_t st);
cudaError_t launch_lle_flip(const double* v32, const int* list, const int* count, long long maxCount,
                            const double* check, bool final_, double* out, int* list2, int* count2, cudaStream_t st);
// reference-semantics kernels on caller arrays (kern_f64.cu)
cudaError_t launch_peak_finder(const double* data, long long nSeries, int len, double h, int cap, int* counts,
                               double* peaks, double* intervals, cudaStream_t st);
cudaError_t launch_point_dbscan(const double* intervals, const int* counts, long long n, int stride, double eps,
                                int* labScratch, int* slotScratch, int* out, cudaStream_t st,
                                const int* outIdx = nullptr);  // outIdx: label of row w goes to out[outIdx[w]]

cudaError_t launch_trajectory_f64(int system, const double* x0, const double* a0, double h, int nSteps,
                                  double* out, long long n, cudaStream_t st);
cudaError_t launch_trajectory_f32(int system, const double* x0, const double* a0, double h, int nSteps,
                                  double* out, long long n, cudaStream_t st);
cudaError_t launch_trajectory_ff(int system, const double* x0, const double* a0, double h, int nSteps,
                                 double* out, long long n, cudaStream_t st);

// FP32 LLE kernel variant (kern_f32.cu): 0 = default, 2 = two points per
// thread (packed FP32x2), 12 / 16 = one point per thread at that occupancy.
int set_lle_variant(int v);
int get_lle_variant();
int set_lle_renorm(int v);  // LleRenorm mode of the FP32 LLE maps of the RK4 systems
int get_lle_renorm();
// Paired FP32 bifurcation / basins kernels for the RK4 systems (kern_f32.cu).
int sweep_pairs();
// launch shapes found by the tuner (kern_f32.cu): kind 0 bifurcation, 1 basins,
// 2 LLE map; code 0 = built-in rule, else form * 1024 + block
int set_launch_shape(int kind, int system, int code);
int get_launch_shape(int kind, int system);  // 0 never, 1 large sweeps, 2 always
int set_sweep_pairs(int v);

// The build-time user plug-in (kern_user.cu, or user_stub.cu when the build
// has none): FP64 kernels of system SYS_USER.
bool user_system_available();
void user_system_sizes(int* nx, int* na);
cudaError_t launch_bif_user(const SweepParams& P, const BifOut& O, cudaStream_t st);
cudaError_t launch_basins_user(const SweepParams& P, const BasinsOut& O, cudaStream_t st);
cudaError_t launch_lle_user(const LleParams& L, double* out, cudaStream_t st);
cudaError_t launch_trajectory_user(const double* x0, const double* a0, double h, int nSteps, double* out,
                                   long long n, cudaStream_t st);

bool system_supported(int system);
int launch_block_size();  // threads per block of the sweep kernels

}  // namespace chaos
