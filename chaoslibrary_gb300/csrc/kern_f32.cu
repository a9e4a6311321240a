// FP32 kernels: trajectories in FP32 registers (contraction allowed), peak
// times, intervals and means in FP64. The LLE kernel carries the twin as the
// exact difference e = q - x (quadratic RK4 systems only) and accumulates the
// log-stretch sum in FP64.
#include <algorithm>
#include <atomic>
#include <cstdlib>

#include "engine.cuh"

namespace chaos {

namespace {
constexpr int kBlock = 128;     // default block
constexpr int kMaxBlock = 256;  // largest block a tuned launch may use

// Sel: the peak detector as selects (sweeps of at most 8 warps per SM, where
// each warp waits on its own trajectory) or in the block form.
template <int S, bool Sel>
__global__ void __launch_bounds__(kMaxBlock) bif_kernel_f32(SweepParams P, BifOut O) {
    const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= P.nPoints) return;
    bif_point<S, float, Sel>(P, O, P.pBegin + o, o);
}

template <int S>
__global__ void __launch_bounds__(kBlock) bif_list_kernel_f32(SweepParams P, BifOut O, const int* list, int count) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    bif_point<S, float, true>(P, O, list[k], k);
}

template <int S, bool PRE1, bool Sel>
__global__ void __launch_bounds__(kMaxBlock) basins_kernel_f32(SweepParams P, BasinsOut O) {
    const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= P.nPoints) return;
    basins_point<S, float, PRE1, Sel>(P, O, P.pBegin + o, o);
}

// MINB = resident blocks per SM the register allocation is shaped for:
// 12 (40 registers, 48 warps/SM) or 16 (32 registers, 64 warps/SM, a few
// bytes of spill outside the step loop). Picked per system by the tuner.
template <class F, int MINB>
__global__ void __launch_bounds__(kBlock, MINB) lle_twin_kernel_f32(LleParams L, double* out) {
    const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= L.nPoints) return;
    out[o] = lle_point_twin<F>(L, L.pBegin + o);
}

__global__ void __launch_bounds__(kBlock) spectrum_chameleon_kernel_f32(LleParams L, double* out) {
    const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= L.nPoints) return;
    spectrum_point_twin_chameleon(L, L.pBegin + o, out);
}

__global__ void __launch_bounds__(kBlock) lle_chameleon_kernel_f32(LleParams L, double* out) {
    const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= L.nPoints) return;
    out[o] = lle_point_twin_chameleon(L, L.pBegin + o);
}

template <int S>
__global__ void __launch_bounds__(kBlock) trajectory_kernel_f32(const double* x0, const double* a0, double h, int nSteps,
                                                       double* out, long long n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    trajectory_point<S, float>(x0, a0, h, nSteps, out, t);
}

template <class F>
__global__ void __launch_bounds__(kBlock) spectrum_kernel_f32(LleParams L, double* out) {
    const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= L.nPoints) return;
    spectrum_point_twin<F>(L, L.pBegin + o, out);
}

// Bifurcation / basins, two points per thread in packed FP32x2 lanes (RK4 systems).
template <class F>
__global__ void __launch_bounds__(kMaxBlock) bif_pair_kernel_f32(SweepParams P, BifOut O) {
    const long long o = 2 * ((long long)blockIdx.x * blockDim.x + threadIdx.x);
    if (o >= P.nPoints) return;
    const bool two = o + 1 < P.nPoints;
    bif_pair_point<F>(P, O, P.pBegin + o, P.pBegin + (two ? o + 1 : o), o, two ? o + 1 : o, two);
}

template <class F, bool PRE1>
__global__ void __launch_bounds__(kMaxBlock) basins_pair_kernel_f32(SweepParams P, BasinsOut O) {
    const long long o = 2 * ((long long)blockIdx.x * blockDim.x + threadIdx.x);
    if (o >= P.nPoints) return;
    const bool two = o + 1 < P.nPoints;
    basins_pair_point<F, PRE1>(P, O, P.pBegin + o, P.pBegin + (two ? o + 1 : o), o, two ? o + 1 : o, two);
}

template <class F>
__global__ void __launch_bounds__(kMaxBlock) bif_hybrid_kernel_f32(SweepParams P, BifOut O) {
    const long long o = 2 * ((long long)blockIdx.x * blockDim.x + threadIdx.x);
    if (o >= P.nPoints) return;
    const bool two = o + 1 < P.nPoints;
    bif_hybrid_point<F>(P, O, P.pBegin + o, P.pBegin + (two ? o + 1 : o), o, two ? o + 1 : o, two);
}

template <class F, bool PRE1>
__global__ void __launch_bounds__(kMaxBlock) basins_hybrid_kernel_f32(SweepParams P, BasinsOut O) {
    const long long o = 2 * ((long long)blockIdx.x * blockDim.x + threadIdx.x);
    if (o >= P.nPoints) return;
    const bool two = o + 1 < P.nPoints;
    basins_hybrid_point<F, PRE1>(P, O, P.pBegin + o, P.pBegin + (two ? o + 1 : o), o, two ? o + 1 : o, two);
}

inline unsigned grid_for(long long n) { return (unsigned)((n + kBlock - 1) / kBlock); }
}  // namespace
namespace {

// Variant of the FP32 LLE kernel: 12 / 16 = one point per thread shaped for
// 12 or 16 resident blocks per SM; 2 = two points per thread in packed
// FP32x2 lanes. CHAOS_LLE_MINB forces one, otherwise the measured default.
std::atomic<int> g_lle_variant{0};

int lle_env_variant() {
    static int forced = [] {
        const char* s = getenv("CHAOS_LLE_MINB");
        return s ? atoi(s) : 0;
    }();
    return forced;
}

int lle_occupancy_variant(int system) {
    (void)system;
    const int set = g_lle_variant.load(std::memory_order_relaxed);
    if (set) return set;
    return lle_env_variant() ? lle_env_variant() : 2;
}

bool lle_variant_forced() { return g_lle_variant.load(std::memory_order_relaxed) != 0 || lle_env_variant() != 0; }

#define CHAOS_SYSTEM_SWITCH(sys, CALL) \
    switch (sys) {                     \
        case SYS_LORENZ_RK4: CALL(SYS_LORENZ_RK4); break; \
        case SYS_ROSSLER_RK4: CALL(SYS_ROSSLER_RK4); break; \
        case SYS_CHEN_RK4: CALL(SYS_CHEN_RK4); break; \
        case SYS_CHAMELEON: CALL(SYS_CHAMELEON); break; \
        case SYS_ROSSLER_CD: CALL(SYS_ROSSLER_CD); break; \
        case SYS_SIN3: CALL(SYS_SIN3); break; \
        case SYS_SIN2: CALL(SYS_SIN2); break; \
        case SYS_MEMRISTOR: CALL(SYS_MEMRISTOR); break; \
        default: return cudaErrorInvalidValue; \
    }
}  // namespace

std::atomic<int> g_sweep_pairs{-1};

// Paired (two points per thread) FP32 sweeps for the RK4 systems. Mode 1
// (default): sweeps of at least 4 x SMs x 1024 points run as pairs -- 1-D
// bifurcations as hybrid pairs (packed transient, recorded part lane by lane),
// basins maps fully packed -- and smaller ones one point per thread (pairs
// halve the threads of a latency-bound sweep). Measured on GB300 with the
// recorded loops' block form: a 1.6 M-point Lorenz 1-D bifurcation 53.4 ms
// hybrid, 57.5 ms fully packed (Rossler 45.5 / 45.3 ms); the 2048^2 Lorenz
// basins map 145.9 ms fully packed, 147.7 ms hybrid, and at 1024^2 the
// packed form ahead by 1.3 / 1.7 / 2.0 % on Lorenz / Rossler / Chen.
// 2: always fully packed; 0: never; 3: always hybrid. Set with
// chaos_set_tuning or CHAOS_SWEEP_PAIRS.
int sweep_pairs() {
    const int v = g_sweep_pairs.load(std::memory_order_relaxed);
    if (v >= 0) return v;
    static int env = [] {
        const char* s = getenv("CHAOS_SWEEP_PAIRS");
        const int m = s ? atoi(s) : 1;
        return m < 0 || m > 3 ? 1 : m;
    }();
    return env;
}
int set_sweep_pairs(int v) {
    if (v < 0 || v > 3) return -1;
    g_sweep_pairs.store(v);
    return 0;
}

inline unsigned grid_of(long long threads, int block) { return (unsigned)((threads + block - 1) / block); }

// Launch shapes the self-timing tuner (tune.cu) found, per kind (0 1-D
// bifurcation, 1 basins, 2 LLE map) and RK4 system: 0 = none (the built-in
// rules below), else form * 1024 + block with form 1 (one point per thread)
// or 2 (two points per thread in packed FP32x2 lanes); for basins also form 3
// (two points per thread, packed transient, recorded part lane by lane); for
// the LLE map also form 12 / 16 (one point per thread, registers shaped for
// 12 / 16 resident blocks per SM, block 128).
std::atomic<int> g_shape[3][3];

int shape_of(int kind, int system) {
    return system >= 0 && system <= SYS_CHEN_RK4 ? g_shape[kind][system].load(std::memory_order_relaxed) : 0;
}

long long pair_threshold() {
    static long long threshold = [] {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        return 4LL * std::max(sms, 1) * 1024;
    }();
    return threshold;
}

// Sweeps of at most 8 warps per SM (SMs x 256 points) run the peak detector
// as selects: there every warp waits on its own dependent chain, and the
// selects overlap the detector with the next step; larger sweeps run the
// block form. Measured on GB300 (1-D Lorenz, 20,000 steps): 1,000 points
// 1.84 ms selects / 2.02 ms blocks, 5,000 1.94 / 2.00, 20,000 2.26 / 2.43,
// 50,000 2.87 / 2.80; the reference's 300^2 Chameleon sweep 50.6 / 46.5 ms.
long long select_form_threads() {
    static long long threads = [] {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        return (long long)std::max(sms, 1) * 256;
    }();
    return threads;
}

struct Launch {
    int form;  // 1 one point per thread, 2 packed pairs, 3 hybrid pairs
    int block;
};

// Pairs halve the threads: worth it when the sweep fills the GPU several
// times over, not for small (latency-bound) sweeps. An explicit sweep-pairs
// mode (0 / 2 / 3) wins; then a tuned shape; then the measured rule.
Launch sweep_launch(const SweepParams& P, bool basins) {
    if (P.system > SYS_CHEN_RK4 || P.sweepStep) return {1, kBlock};  // a pair shares one step size
    const int mode = sweep_pairs();
    const int shape = shape_of(basins ? 1 : 0, P.system);
    const int block = shape ? shape % 1024 : kBlock;
    const bool big = P.nPoints >= pair_threshold();
    if (mode == 0) return {1, block};
    if (mode == 2) return {2, block};
    if (mode == 3) return {3, block};
    if (shape) {
        const int form = shape / 1024;
        return {form >= 2 && !big ? 1 : form, block};
    }
    return {big ? (basins ? 2 : 3) : 1, kBlock};
}

template <class F> void launch_bif_pairs(const SweepParams& P, const BifOut& O, int block, cudaStream_t st) {
    bif_pair_kernel_f32<F><<<grid_of((P.nPoints + 1) / 2, block), block, 0, st>>>(P, O);
    note_launch();
}

template <class F> void launch_basins_pairs(const SweepParams& P, const BasinsOut& O, int block, cudaStream_t st) {
    const unsigned g = grid_of((P.nPoints + 1) / 2, block);
    if (P.preScaller == 1) basins_pair_kernel_f32<F, true><<<g, block, 0, st>>>(P, O);
    else basins_pair_kernel_f32<F, false><<<g, block, 0, st>>>(P, O);
    note_launch();
}

template <class F> void launch_bif_hybrid(const SweepParams& P, const BifOut& O, int block, cudaStream_t st) {
    bif_hybrid_kernel_f32<F><<<grid_of((P.nPoints + 1) / 2, block), block, 0, st>>>(P, O);
    note_launch();
}

template <class F> void launch_basins_hybrid(const SweepParams& P, const BasinsOut& O, int block, cudaStream_t st) {
    const unsigned g = grid_of((P.nPoints + 1) / 2, block);
    if (P.preScaller == 1) basins_hybrid_kernel_f32<F, true><<<g, block, 0, st>>>(P, O);
    else basins_hybrid_kernel_f32<F, false><<<g, block, 0, st>>>(P, O);
    note_launch();
}

cudaError_t launch_bif_f32(const SweepParams& P, const BifOut& O, cudaStream_t st) {
    if (P.nPoints <= 0) return cudaSuccess;
    const Launch l = sweep_launch(P, false);
    if (l.form == 2) {
        if (P.system == SYS_LORENZ_RK4) launch_bif_pairs<Lorenz>(P, O, l.block, st);
        else if (P.system == SYS_ROSSLER_RK4) launch_bif_pairs<Rossler>(P, O, l.block, st);
        else launch_bif_pairs<Chen>(P, O, l.block, st);
        return cudaGetLastError();
    }
    if (l.form == 3) {
        if (P.system == SYS_LORENZ_RK4) launch_bif_hybrid<Lorenz>(P, O, l.block, st);
        else if (P.system == SYS_ROSSLER_RK4) launch_bif_hybrid<Rossler>(P, O, l.block, st);
        else launch_bif_hybrid<Chen>(P, O, l.block, st);
        return cudaGetLastError();
    }
    const bool sel = P.nPoints <= select_form_threads();
#define CALL(S)                                                                           \
    (sel ? bif_kernel_f32<S, true><<<grid_of(P.nPoints, l.block), l.block, 0, st>>>(P, O) \
         : bif_kernel_f32<S, false><<<grid_of(P.nPoints, l.block), l.block, 0, st>>>(P, O), \
     note_launch())
    CHAOS_SYSTEM_SWITCH(P.system, CALL)
#undef CALL
    return cudaGetLastError();
}

cudaError_t launch_bif_list_f32(const SweepParams& P, const BifOut& O, const int* list, int count, cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
#define CALL(S) (bif_list_kernel_f32<S><<<grid_for(count), kBlock, 0, st>>>(P, O, list, count), note_launch())
    CHAOS_SYSTEM_SWITCH(P.system, CALL)
#undef CALL
    return cudaGetLastError();
}

cudaError_t launch_basins_f32(const SweepParams& P, const BasinsOut& O, cudaStream_t st) {
    if (P.nPoints <= 0) return cudaSuccess;
    const Launch l = sweep_launch(P, true);
    if (l.form == 2) {
        if (P.system == SYS_LORENZ_RK4) launch_basins_pairs<Lorenz>(P, O, l.block, st);
        else if (P.system == SYS_ROSSLER_RK4) launch_basins_pairs<Rossler>(P, O, l.block, st);
        else launch_basins_pairs<Chen>(P, O, l.block, st);
        return cudaGetLastError();
    }
    if (l.form == 3) {
        if (P.system == SYS_LORENZ_RK4) launch_basins_hybrid<Lorenz>(P, O, l.block, st);
        else if (P.system == SYS_ROSSLER_RK4) launch_basins_hybrid<Rossler>(P, O, l.block, st);
        else launch_basins_hybrid<Chen>(P, O, l.block, st);
        return cudaGetLastError();
    }
    const unsigned g = grid_of(P.nPoints, l.block);
    const bool sel = P.nPoints <= select_form_threads();  // the detector as selects, as in the 1-D sweeps
#define CALL(S)                                                                               \
    (P.preScaller == 1 ? (sel ? basins_kernel_f32<S, true, true><<<g, l.block, 0, st>>>(P, O)    \
                              : basins_kernel_f32<S, true, false><<<g, l.block, 0, st>>>(P, O))  \
                       : (sel ? basins_kernel_f32<S, false, true><<<g, l.block, 0, st>>>(P, O)   \
                              : basins_kernel_f32<S, false, false><<<g, l.block, 0, st>>>(P, O)), \
     note_launch())
    CHAOS_SYSTEM_SWITCH(P.system, CALL)
#undef CALL
    return cudaGetLastError();
}

// Two points per thread in packed FP32x2 lanes. Registers capped at 56 (three
// resident blocks of 384 threads): nine blocks of 128 per SM instead of eight
// at the 62 the kernel takes unbounded. The cap costs a few bytes of spills
// outside the step loop; the 1024^2 Rössler map went from 133.7 to 128.6 ms
// (from 3.37 waves of resident blocks to 2.99) and the Lorenz map from 39.1
// to 36.2 ms, results unchanged. Blocks of 64, 128 and 256 (the tuner's
// choices) all launch under the bound.
template <class F, int RN = kRenormPow2>
__global__ void __launch_bounds__(384, 3) lle_pair_kernel_f32(LleParams L, double* out) {
    const long long o = 2 * ((long long)blockIdx.x * blockDim.x + threadIdx.x);
    if (o >= L.nPoints) return;
    const bool two = o + 1 < L.nPoints;
    lle_pair_twin<F, RN>(L, L.pBegin + o, L.pBegin + (two ? o + 1 : o), out + o, two ? out + o + 1 : nullptr);
}

// Stretch mode of the FP32 LLE maps of the RK4 systems (LleRenorm): 0 the
// exact power-of-two renormalisation (default); 1 and 2 run the pair kernel
// with the per-block FP32 log or the per-block FP64 norm and log instead.
std::atomic<int> g_lle_renorm{0};

template <class F>
static void launch_twin(const LleParams& L, double* out, cudaStream_t st, int minb, int block) {
    const int rn = g_lle_renorm.load(std::memory_order_relaxed);
    const unsigned gp = grid_of((L.nPoints + 1) / 2, minb == 2 ? block : kBlock);
    const int bp = minb == 2 ? block : kBlock;
    if (rn == kRenormF32Log) lle_pair_kernel_f32<F, kRenormF32Log><<<gp, bp, 0, st>>>(L, out);
    else if (rn == kRenormF64) lle_pair_kernel_f32<F, kRenormF64><<<gp, bp, 0, st>>>(L, out);
    else if (minb == 2) lle_pair_kernel_f32<F><<<gp, bp, 0, st>>>(L, out);
    else if (minb >= 16) lle_twin_kernel_f32<F, 16><<<grid_for(L.nPoints), kBlock, 0, st>>>(L, out);
    else lle_twin_kernel_f32<F, 12><<<grid_for(L.nPoints), kBlock, 0, st>>>(L, out);
    note_launch();
}

int set_launch_shape(int kind, int system, int code) {
    if (kind < 0 || kind > 2 || system < 0 || system > SYS_CHEN_RK4 || code < 0) return -1;
    g_shape[kind][system].store(code);
    return 0;
}
int get_launch_shape(int kind, int system) {
    return kind >= 0 && kind <= 2 ? shape_of(kind, system) : 0;
}

int set_lle_variant(int v) {
    if (v != 0 && v != 2 && v != 12 && v != 16) return -1;
    g_lle_variant.store(v);
    return 0;
}
int get_lle_variant() { return lle_occupancy_variant(0); }

int set_lle_renorm(int v) {
    if (v < kRenormPow2 || v > kRenormF64) return -1;
    g_lle_renorm.store(v);
    return 0;
}
int get_lle_renorm() { return g_lle_renorm.load(); }

cudaError_t launch_lle_f32(const LleParams& L, double* out, cudaStream_t st) {
    if (L.nPoints <= 0) return cudaSuccess;
    // an explicit variant (chaos_set_tuning / CHAOS_LLE_MINB) wins, then a tuned shape
    int minb = lle_occupancy_variant(L.system), block = kBlock;
    const int shape = shape_of(2, L.system);
    if (shape && !lle_variant_forced()) {
        minb = shape / 1024;
        block = minb == 2 ? shape % 1024 : kBlock;
    }
    switch (L.system) {
        case SYS_LORENZ_RK4: launch_twin<Lorenz>(L, out, st, minb, block); break;
        case SYS_ROSSLER_RK4: launch_twin<Rossler>(L, out, st, minb, block); break;
        case SYS_CHEN_RK4: launch_twin<Chen>(L, out, st, minb, block); break;
        case SYS_CHAMELEON:
            lle_chameleon_kernel_f32<<<grid_for(L.nPoints), kBlock, 0, st>>>(L, out);
            note_launch();
            break;
        default: return cudaErrorNotSupported;
    }
    return cudaGetLastError();
}

cudaError_t launch_spectrum_f32(const LleParams& L, double* out, cudaStream_t st) {
    if (L.nPoints <= 0) return cudaSuccess;
    const unsigned g = grid_for(L.nPoints);
    switch (L.system) {
        case SYS_LORENZ_RK4: spectrum_kernel_f32<Lorenz><<<g, kBlock, 0, st>>>(L, out); break;
        case SYS_ROSSLER_RK4: spectrum_kernel_f32<Rossler><<<g, kBlock, 0, st>>>(L, out); break;
        case SYS_CHEN_RK4: spectrum_kernel_f32<Chen><<<g, kBlock, 0, st>>>(L, out); break;
        case SYS_CHAMELEON: spectrum_chameleon_kernel_f32<<<g, kBlock, 0, st>>>(L, out); break;
        default: return cudaErrorNotSupported;
    }
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_trajectory_f32(int system, const double* x0, const double* a0, double h, int nSteps,
                                  double* out, long long n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
#define CALL(S) \
    (trajectory_kernel_f32<S><<<grid_for(n), kBlock, 0, st>>>(x0, a0, h, nSteps, out, n), note_launch())
    CHAOS_SYSTEM_SWITCH(system, CALL)
#undef CALL
    return cudaGetLastError();
}

}  // namespace chaos
