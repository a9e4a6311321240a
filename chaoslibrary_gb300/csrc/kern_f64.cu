// FP64 kernels: the reference's arithmetic, one rounding per written
// operation. This translation unit is compiled with --fmad=false, so a*b+c
// stays two roundings unless the source calls fma(); together with IEEE
// division and square root the FP64 sweeps reproduce the CPU oracle bit for
// bit. Also holds the reference-semantics kernels that run on caller arrays
// (peak finder, per-point dbscan of the 2-D bifurcation).
#include <climits>

#include "engine.cuh"
#include "legacy_lle.cuh"

namespace chaos {

namespace {
constexpr int kBlock = 128;

// Legacy: the legacy library's per-point loop (P.legacyLoop != 0).
template <int S, bool Legacy>
__global__ void __launch_bounds__(kBlock) bif_kernel(SweepParams P, BifOut O) {
    const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= P.nPoints) return;
    if constexpr (Legacy) bif_point_legacy<S>(P, O, P.pBegin + o, o);
    else bif_point<S, double>(P, O, P.pBegin + o, o);
}

// Bifurcation points list[0, count), result row k for list[k].
template <int S, bool Legacy>
__global__ void __launch_bounds__(kBlock) bif_list_kernel(SweepParams P, BifOut O, const int* list, int count) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    if constexpr (Legacy) bif_point_legacy<S>(P, O, list[k], k);
    else bif_point<S, double>(P, O, list[k], k);
}

template <int S>
__global__ void __launch_bounds__(kBlock) basins_kernel(SweepParams P, BasinsOut O) {
    const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= P.nPoints) return;
    basins_point<S, double>(P, O, P.pBegin + o, o);
}

template <int S>
__global__ void __launch_bounds__(kBlock) lle_kernel(LleParams L, double* out) {
    const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= L.nPoints) return;
    out[o] = lle_point_full<S, double>(L, L.pBegin + o);
}

// The legacy library's LLE kernels' scheme (L.legacyLoop).
template <int S>
__global__ void __launch_bounds__(kBlock) lle_legacy_kernel(LleParams L, double* out) {
    const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= L.nPoints) return;
    out[o] = lle_point_legacy<S>(L, L.pBegin + o);
}

// The LLE map with the reference's cuRAND twin start (L.twin == 2).
template <int S>
__global__ void __launch_bounds__(kBlock) lle_reftwin_kernel(LleParams L, double* out) {
    const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= L.nPoints) return;
    out[o] = lle_point_reftwin<S>(L, L.pBegin + o);
}

// kind 0 / 1: out[p*nx + k] = legacy_twin_draw; kind 2: out[(p*nx + j)*nx + i] = legacy_spectrum_draw
__global__ void legacy_draws_kernel(int kind, long long n, int nx, double* out) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long per = kind == 2 ? (long long)nx * nx : nx;
    if (t >= n * per) return;
    const long long p = t / per;
    const int r = (int)(t % per);
    out[t] = kind == 2 ? legacy_spectrum_draw(p, r % nx, r / nx) : legacy_twin_draw(kind, p, r);
}

// Benettin blocks from caller-supplied starting states (the reference's
// semi_result layout, LLE/src/LLECUDA.cu:102-111): point k's row of 2*NX + NA
// values holds the orbit after the transient, the parameters and the twin.
template <int S>
__global__ void __launch_bounds__(kBlock) lle_states_kernel(LleParams L, const double* states, double* out) {
    constexpr int NX = Traits<S>::NX, NA = Traits<S>::NA, W = 2 * NX + NA;
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= L.nPoints) return;
    const double* r = states + k * W;
    double x[NX], q[NX], a[NA];
#pragma unroll
    for (int i = 0; i < NX; ++i) {
        x[i] = r[i];
        q[i] = r[NX + NA + i];
    }
#pragma unroll
    for (int i = 0; i < NA; ++i) a[i] = r[NX + i];
    out[k] = lle_benettin_full<S>(L, x, q, a);
}

// Lyapunov spectrum, out[p*SIZE_X + j]
template <int S>
__global__ void __launch_bounds__(kBlock) spectrum_kernel(LleParams L, double* out) {
    const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= L.nPoints) return;
    spectrum_point_full<S>(L, L.pBegin + o, out);
}

// The legacy library's spectrum kernel's scheme (L.legacyLoop).
template <int S>
__global__ void __launch_bounds__(kBlock) spectrum_legacy_kernel(LleParams L, double* out) {
    const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= L.nPoints) return;
    spectrum_point_legacy<S>(L, L.pBegin + o, out);
}

// FP64 LLE of the points list[0, *count): out[k] (scatter = 0) or out[list[k]]
// (scatter = 1). The same device function as lle_kernel, so a point's value
// is the FP64 map's value bit for bit.
template <int S>
__global__ void __launch_bounds__(kBlock) lle_list_kernel(LleParams L, const int* list, const int* count,
                                                          double* out, int scatter) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= *count) return;
    const int p = list[k];
    const double v = lle_point_full<S, double>(L, p);
    out[scatter ? p : k] = v;
}

// class of an LLE value for the sign re-check: 1 positive, 0 non-positive,
// -1 not finite
__device__ __forceinline__ int lle_class(double v) { return !(fabs(v) <= 1.7976931348623157e308) ? -1 : v > 0.0; }

// warp-aggregated append of p to list (one atomic per warp; list may be null
// to count only)
__device__ __forceinline__ void append(bool take, int p, int* list, int* count) {
    const unsigned m = __ballot_sync(0xffffffffu, take);
    if (!m) return;
    const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(count, __popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (take && list) list[base + __popc(m & ((1u << lane) - 1))] = p;
}

// points whose value is within band of zero or not finite
__global__ void lle_select_kernel(const double* v, long long n, double band, int* list, int* count) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool take = i < n && !(fabs(v[i]) > band);
    append(take, (int)i, list, count);
}

// checked points whose FP64 check disagrees in class with the FP32 value are
// counted in count2 and appended to list2 (when not null); with final = 1
// (the check ran the full horizon) their check value is stored into out.
// Every thread of the grid reaches the warp vote.
__global__ void lle_flip_kernel(const double* v32, const int* list, const int* count, const double* check,
                                int final_, double* out, int* list2, int* count2) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    bool take = false;
    int p = 0;
    if (k < *count) {
        p = list[k];
        take = lle_class(v32[p]) != lle_class(check[k]);
    }
    append(take, p, list2, count2);
    if (take && final_) out[p] = check[k];
}

template <int S>
__global__ void __launch_bounds__(kBlock) trajectory_kernel(const double* x0, const double* a0, double h, int nSteps,
                                                       double* out, long long n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    trajectory_point<S, double>(x0, a0, h, nSteps, out, t);
}

inline unsigned grid_for(long long n) { return (unsigned)((n + kBlock - 1) / kBlock); }

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

// Peak finder over caller series (the reference's peakFinderCUDA semantics on
// identical input arrays): one thread streams one series.
__global__ void peak_array_kernel(const double* __restrict__ data, long long nSeries, int len, double h, int cap,
                                  int* counts, double* peaks, double* intervals) {
    const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nSeries) return;
    const double* d = data + s * (long long)len;
    PeakStream<double> ps;
    ps.init();
    for (int k = 0; k < len; ++k) {
        double val;
        int t;
        if (ps.push(d[k], val, t)) {
            if (ps.n >= 1) {
                const int q = ps.n - 1;
                if (q < cap) {
                    peaks[s * (long long)cap + q] = val;
                    intervals[s * (long long)cap + q] = __dmul_rn((double)(t - ps.tprev), h);
                }
            }
            ps.tprev = t;
            ++ps.n;
        }
    }
    counts[s] = ps.n > 1 ? ps.n - 1 : 0;
}

// Per-point dbscan of the 2-D bifurcation (bifurcationCUDA.cu:516-583), one
// warp per point. The sequential control (new cluster / pop of slot NN-1) is
// uniform across the warp; each expansion pass over k < P-1 is split across
// the lanes, which is exact because pass k only reads and writes entry k.
__global__ void point_dbscan_kernel(const double* __restrict__ intervals, const int* __restrict__ counts, long long n,
                                    int stride, double eps, int* labScratch, int* slotScratch, int* outBase,
                                    const int* outIdx) {
    const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= n) return;
    const long long oi = outIdx ? (long long)outIdx[w] : w;  // where this point's label goes
    const int P = counts[w];
    if (P > stride) {  // more intervals than the row holds: reported, not read
        if (lane == 0) outBase[oi] = INT_MIN;
        return;
    }
    if (P <= 1) {  // dbscanCUDA: -1 passes through; dbscan returns 0 for P <= 0 and 1 for P == 1
        if (lane == 0) outBase[oi] = P == -1 ? -1 : (P == 1 ? 1 : 0);
        return;
    }
    const double* iv = intervals + w * (long long)stride;
    int* lab = labScratch + w * (long long)stride;
    int* slot = slotScratch + w * (long long)stride;
    for (int k = lane; k < P; k += 32) { lab[k] = 0; slot[k] = 0; }
    __syncwarp();
    int cluster = 0, nn = 0;
    for (int i = 0; i < P; ++i) {
        bool expand = false;
        if (nn >= 1) {
            i = slot[nn - 1];
            __syncwarp();
            if (lane == 0) slot[nn - 1] = 0;
            --nn;
            expand = true;
        } else if (lab[i] == 0) {
            nn = 0;
            ++cluster;
            __syncwarp();
            if (lane == 0) lab[i] = cluster;
            expand = true;
        }
        if (expand) {
            __syncwarp();
            const double ivi = iv[i];
            for (int k0 = 0; k0 < P - 1; k0 += 32) {
                const int k = k0 + lane;
                bool hit = false;
                if (k < P - 1 && k != i && lab[k] == 0) {
                    const double ivk = iv[k];
                    const double dist = (ivi == ivk) ? 0.0 : (double)fabsf((float)(ivk - ivi));
                    if (dist < eps) {
                        lab[k] = cluster;
                        slot[k] = k;
                        hit = true;
                    }
                }
                nn += __popc(__ballot_sync(0xffffffffu, hit));
            }
            __syncwarp();
        }
    }
    if (lane == 0) outBase[oi] = cluster - 1;
}

}  // namespace

bool system_supported(int system) {
    return (system >= 0 && system < SYS_COUNT) || (system == SYS_USER && user_system_available());
}
int launch_block_size() { return kBlock; }

cudaError_t launch_bif_f64(const SweepParams& P, const BifOut& O, cudaStream_t st) {
    if (P.nPoints <= 0) return cudaSuccess;
#define CALL(S)                                                             \
    {                                                                       \
        if (P.legacyLoop) bif_kernel<S, true><<<grid_for(P.nPoints), kBlock, 0, st>>>(P, O); \
        else bif_kernel<S, false><<<grid_for(P.nPoints), kBlock, 0, st>>>(P, O); \
        note_launch();                                                      \
    }
    CHAOS_SYSTEM_SWITCH(P.system, CALL)
#undef CALL
    return cudaGetLastError();
}

cudaError_t launch_basins_f64(const SweepParams& P, const BasinsOut& O, cudaStream_t st) {
    if (P.nPoints <= 0) return cudaSuccess;
#define CALL(S) (basins_kernel<S><<<grid_for(P.nPoints), kBlock, 0, st>>>(P, O), note_launch())
    CHAOS_SYSTEM_SWITCH(P.system, CALL)
#undef CALL
    return cudaGetLastError();
}

cudaError_t launch_lle_f64(const LleParams& L, double* out, cudaStream_t st) {
    if (L.nPoints <= 0) return cudaSuccess;
#define CALL(S)                                                               \
    {                                                                         \
        if (L.legacyLoop) lle_legacy_kernel<S><<<grid_for(L.nPoints), kBlock, 0, st>>>(L, out); \
        else if (L.twin == 2) lle_reftwin_kernel<S><<<grid_for(L.nPoints), kBlock, 0, st>>>(L, out); \
        else lle_kernel<S><<<grid_for(L.nPoints), kBlock, 0, st>>>(L, out); \
        note_launch();                                                        \
    }
    CHAOS_SYSTEM_SWITCH(L.system, CALL)
#undef CALL
    return cudaGetLastError();
}

cudaError_t launch_legacy_draws(int kind, long long n, int nx, double* out, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    legacy_draws_kernel<<<grid_for(n * (kind == 2 ? (long long)nx * nx : nx)), kBlock, 0, st>>>(kind, n, nx, out);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_lle_states_f64(const LleParams& L, const double* states, double* out, cudaStream_t st) {
    if (L.nPoints <= 0) return cudaSuccess;
#define CALL(S) (lle_states_kernel<S><<<grid_for(L.nPoints), kBlock, 0, st>>>(L, states, out), note_launch())
    CHAOS_SYSTEM_SWITCH(L.system, CALL)
#undef CALL
    return cudaGetLastError();
}

cudaError_t launch_spectrum_f64(const LleParams& L, double* out, cudaStream_t st) {
    if (L.nPoints <= 0) return cudaSuccess;
#define CALL(S)                                                                    \
    {                                                                              \
        if (L.legacyLoop) spectrum_legacy_kernel<S><<<grid_for(L.nPoints), kBlock, 0, st>>>(L, out); \
        else spectrum_kernel<S><<<grid_for(L.nPoints), kBlock, 0, st>>>(L, out); \
        note_launch();                                                             \
    }
    CHAOS_SYSTEM_SWITCH(L.system, CALL)
#undef CALL
    return cudaGetLastError();
}

cudaError_t launch_bif_list_f64(const SweepParams& P, const BifOut& O, const int* list, int count, cudaStream_t st) {
    if (count <= 0) return cudaSuccess;
#define CALL(S)                                                                       \
    {                                                                                 \
        if (P.legacyLoop) bif_list_kernel<S, true><<<grid_for(count), kBlock, 0, st>>>(P, O, list, count); \
        else bif_list_kernel<S, false><<<grid_for(count), kBlock, 0, st>>>(P, O, list, count); \
        note_launch();                                                                \
    }
    CHAOS_SYSTEM_SWITCH(P.system, CALL)
#undef CALL
    return cudaGetLastError();
}

// indices of the points whose kept-peak count exceeds cap
__global__ void overflow_select_kernel(const int* counts, long long n, int cap, int* list, int* count) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    append(i < n && counts[i] > cap, (int)i, list, count);
}

cudaError_t launch_overflow_select(const int* counts, long long n, int cap, int* list, int* count, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    overflow_select_kernel<<<grid_for(n), kBlock, 0, st>>>(counts, n, cap, list, count);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_lle_select(const double* v, long long n, double band, int* list, int* count, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    lle_select_kernel<<<grid_for(n), kBlock, 0, st>>>(v, n, band, list, count);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_lle_list_f64(const LleParams& L, const int* list, const int* count, long long maxCount,
                                double* out, bool scatter, cudaStream_t st) {
    if (maxCount <= 0) return cudaSuccess;
#define CALL(S) \
    (lle_list_kernel<S><<<grid_for(maxCount), kBlock, 0, st>>>(L, list, count, out, scatter ? 1 : 0), note_launch())
    CHAOS_SYSTEM_SWITCH(L.system, CALL)
#undef CALL
    return cudaGetLastError();
}

cudaError_t launch_lle_flip(const double* v32, const int* list, const int* count, long long maxCount,
                            const double* check, bool final_, double* out, int* list2, int* count2, cudaStream_t st) {
    if (maxCount <= 0) return cudaSuccess;
    lle_flip_kernel<<<grid_for(maxCount), kBlock, 0, st>>>(v32, list, count, check, final_ ? 1 : 0, out, list2,
                                                            count2);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_peak_finder(const double* data, long long nSeries, int len, double h, int cap, int* counts,
                               double* peaks, double* intervals, cudaStream_t st) {
    if (nSeries <= 0) return cudaSuccess;
    peak_array_kernel<<<grid_for(nSeries), kBlock, 0, st>>>(data, nSeries, len, h, cap, counts, peaks, intervals);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_point_dbscan(const double* intervals, const int* counts, long long n, int stride, double eps,
                                int* labScratch, int* slotScratch, int* out, cudaStream_t st, const int* outIdx) {
    if (n <= 0) return cudaSuccess;
    const long long threads = n * 32;
    point_dbscan_kernel<<<(unsigned)((threads + kBlock - 1) / kBlock), kBlock, 0, st>>>(
        intervals, counts, n, stride, eps, labScratch, slotScratch, out, outIdx);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_trajectory_f64(int system, const double* x0, const double* a0, double h, int nSteps,
                                  double* out, long long n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
#define CALL(S) \
    (trajectory_kernel<S><<<grid_for(n), kBlock, 0, st>>>(x0, a0, h, nSteps, out, n), note_launch())
    CHAOS_SYSTEM_SWITCH(system, CALL)
#undef CALL
    return cudaGetLastError();
}

}  // namespace chaos
