// Float-float LLE kernels (precision CHAOS_FF32): the base trajectory in FF
// arithmetic (ff.h, about 48 significant bits, every operation on the FP32
// pipe), the twin as the exact FP32 difference e = p - x advanced beside it,
// renormalised by exact powers of two, the stretch summed as an integer count
// of octaves plus one FP64 logarithm of the final FP64 norm.
//
// Why: a finite-time LLE of a chaotic orbit depends on every rounding of the
// orbit. Plain FP32 state rounds each step at 2^-24 and its orbit leaves the
// FP64 orbit after ~100 time units of the 550; the FF orbit rounds at ~2^-48
// and stays with the FP64 orbit about as long as an FP64 orbit started 1e-13
// away does, so its LLE map differs from the FP64 map no more than the FP64
// map differs from itself under that perturbation. This GPU's FP64 pipe runs
// at 1/64 of its FP32 rate: the FF step costs ~6x an FP32 step, an FP64 step
// ~64x.
//
// Compiled with --fmad=false and written with explicit round-to-nearest
// intrinsics: a product contracted into a following sum would break the
// error-free transformations.
#include <atomic>

#include "batch.h"
#include "engine.cuh"

namespace chaos {

namespace {
constexpr int kBlock = 128;

// frexp exponent of a positive normal float (0 for +0 gives -126).
__device__ __forceinline__ int exp_of(float v) { return (int)((__float_as_uint(v) >> 23) & 0xff) - 126; }

__device__ __forceinline__ double finite_or_nan(double v) { return isfinite(v) ? v : __longlong_as_double(0x7ff8000000000000LL); }

// The Benettin blocks of an FF orbit x with the FP32 twin difference e
// (started where the caller put it), renormalised by powers of two; the
// stretch of the blocks relative to eps, as the reference measures it.
template <class F>
__device__ __forceinline__ double ff_benettin(const LleParams& L, FF<float>* x, float* e, const FF<float>* a,
                                              const float* af, const FFH<float>& c, const RK4H<float>& cf) {
    const int eps2Exp = exp_of((float)L.eps * (float)L.eps);
    int ktot = 0;
    const int nb = L.calcBlocks + 1;
    for (int b = 0; b < nb; ++b) {
        for (int s = 0; s < L.ntp; ++s) ff_rk4_step<F, true>(x, e, a, af, c, cf);
        if (b + 1 < nb) {
            const float n2 = fmaf(e[0], e[0], fmaf(e[1], e[1], e[2] * e[2]));
            const int k = pow2_rescale_exponent(n2, eps2Exp);
            const float sc = pow2_scale(k);
            e[0] *= sc;
            e[1] *= sc;
            e[2] *= sc;
            ktot += k;
        }
    }
    const double n2 = (double)e[0] * e[0] + (double)e[1] * e[1] + (double)e[2] * e[2];
    return finite_or_nan(pow2_log_stretch(ktot, n2, L.eps) / L.tMax);
}

__device__ __forceinline__ FFH<float> ff_consts(double h) {
    FFH<float> c;
    c.hh = ff_from_double(h * 0.5);
    c.h = ff_from_double(h);
    c.h6 = ff_from_double(h / 6.0);
    return c;
}

template <class F>
__device__ __forceinline__ double lle_point_ff(const LleParams& L, long long p) {
    double xd[3], ad[3];
    lle_load<3, 3>(L, p, xd, ad);
    FF<float> x[3], a[3];
    float af[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        x[k] = ff_from_double(xd[k]);
        a[k] = ff_from_double(ad[k]);
        af[k] = (float)ad[k];
    }
    const FFH<float> c = ff_consts(L.h);
    const RK4H<float> cf((float)L.h);
    for (int s = 0; s < L.trans; ++s) ff_rk4_step<F, false>(x, (float*)nullptr, a, af, c, cf);
    float e[3] = {(float)L.eps, 0.f, 0.f};
    return ff_benettin<F>(L, x, e, a, af, c, cf);
}

// From caller-supplied starting states (the reference's semi_result layout:
// orbit, parameters, twin): the twin difference is q - x, exact in FP64 for
// a twin this close to its orbit, then rounded to FP32.
template <class F>
__global__ void __launch_bounds__(kBlock) lle_ff_states_kernel(LleParams L, const double* states, double* out) {
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= L.nPoints) return;
    const double* r = states + k * 9;
    FF<float> x[3], a[3];
    float af[3], e[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        x[i] = ff_from_double(r[i]);
        a[i] = ff_from_double(r[3 + i]);
        af[i] = (float)r[3 + i];
        e[i] = (float)(r[6 + i] - r[i]);
    }
    out[k] = ff_benettin<F>(L, x, e, a, af, ff_consts(L.h), RK4H<float>((float)L.h));
}

// Two points per thread: FF words are packed pairs (one paired FP32
// instruction per word operation for both points).
template <class F>
__device__ __forceinline__ void lle_pair_ff(const LleParams& L, long long p, long long q, double* outp, double* outq) {
    double xd[2][3], ad[2][3];
    lle_load<3, 3>(L, p, xd[0], ad[0]);
    lle_load<3, 3>(L, q, xd[1], ad[1]);
    FF<P2> x[3], a[3];
    P2 af[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const FF<float> x0 = ff_from_double(xd[0][k]), x1 = ff_from_double(xd[1][k]);
        const FF<float> a0 = ff_from_double(ad[0][k]), a1 = ff_from_double(ad[1][k]);
        x[k] = ff_make(P2(x0.hi, x1.hi), P2(x0.lo, x1.lo));
        a[k] = ff_make(P2(a0.hi, a1.hi), P2(a0.lo, a1.lo));
        af[k] = P2((float)ad[0][k], (float)ad[1][k]);
    }
    FFH<P2> c;
    {
        const FF<float> hh = ff_from_double(L.h * 0.5), h = ff_from_double(L.h), h6 = ff_from_double(L.h / 6.0);
        c.hh = ff_make(P2(hh.hi, hh.hi), P2(hh.lo, hh.lo));
        c.h = ff_make(P2(h.hi, h.hi), P2(h.lo, h.lo));
        c.h6 = ff_make(P2(h6.hi, h6.hi), P2(h6.lo, h6.lo));
    }
    const RK4H<P2> cf((float)L.h);
    for (int s = 0; s < L.trans; ++s) ff_rk4_step<F, false>(x, (P2*)nullptr, a, af, c, cf);
    const float e0 = (float)L.eps;
    const int eps2Exp = exp_of(e0 * e0);
    P2 e[3] = {P2(e0, e0), P2(0.f, 0.f), P2(0.f, 0.f)};
    int k0 = 0, k1 = 0;
    const int nb = L.calcBlocks + 1;
    for (int b = 0; b < nb; ++b) {
        for (int s = 0; s < L.ntp; ++s) ff_rk4_step<F, true>(x, e, a, af, c, cf);
        if (b + 1 < nb) {
            const P2 n2 = fmaT(e[0], e[0], fmaT(e[1], e[1], e[2] * e[2]));
            const int j0 = pow2_rescale_exponent(n2.v.x, eps2Exp), j1 = pow2_rescale_exponent(n2.v.y, eps2Exp);
            const P2 sc(pow2_scale(j0), pow2_scale(j1));
            e[0] *= sc;
            e[1] *= sc;
            e[2] *= sc;
            k0 += j0;
            k1 += j1;
        }
    }
    const double n0 = (double)e[0].v.x * e[0].v.x + (double)e[1].v.x * e[1].v.x + (double)e[2].v.x * e[2].v.x;
    const double n1 = (double)e[0].v.y * e[0].v.y + (double)e[1].v.y * e[1].v.y + (double)e[2].v.y * e[2].v.y;
    *outp = finite_or_nan(pow2_log_stretch(k0, n0, L.eps) / L.tMax);
    if (outq) *outq = finite_or_nan(pow2_log_stretch(k1, n1, L.eps) / L.tMax);
}

template <class F>
__global__ void __launch_bounds__(kBlock) lle_ff_kernel(LleParams L, double* out) {
    const long long o = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= L.nPoints) return;
    out[o] = lle_point_ff<F>(L, L.pBegin + o);
}

template <class F>
__global__ void __launch_bounds__(kBlock) lle_ff_pair_kernel(LleParams L, double* out) {
    const long long o = 2 * ((long long)blockIdx.x * blockDim.x + threadIdx.x);
    if (o >= L.nPoints) return;
    const bool two = o + 1 < L.nPoints;
    lle_pair_ff<F>(L, L.pBegin + o, L.pBegin + (two ? o + 1 : o), out + o, two ? out + o + 1 : nullptr);
}

// FF trajectory of an RK4 system: out[t][s][k] = hi + lo of component k after
// s steps, rounded to double.
template <class F>
__global__ void __launch_bounds__(kBlock) trajectory_kernel_ff(const double* x0, const double* a0, double h,
                                                               int nSteps, double* out, long long n) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    FF<float> x[3], a[3];
    float af[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        x[k] = ff_from_double(x0[t * 3 + k]);
        a[k] = ff_from_double(a0[t * 3 + k]);
        af[k] = (float)a0[t * 3 + k];
    }
    FFH<float> c;
    c.hh = ff_from_double(h * 0.5);
    c.h = ff_from_double(h);
    c.h6 = ff_from_double(h / 6.0);
    const RK4H<float> cf((float)h);
    double* o = out + t * (long long)(nSteps + 1) * 3;
    for (int s = 0;; ++s) {
#pragma unroll
        for (int k = 0; k < 3; ++k) o[(long long)s * 3 + k] = ff_to_double(x[k]);
        if (s == nSteps) break;
        ff_rk4_step<F, false>(x, (float*)nullptr, a, af, c, cf);
    }
}

// Persistent kernel of a batch's float-float LLE jobs of one system
// (CHAOS_JOB_LLE2D_FF32): pulls chunks of two blocks' worth of points from
// its counter; every point runs lle_pair_ff, the single-sweep kernel's device
// function, with the job's parameters staged in shared memory.
template <class F>
__global__ void __launch_bounds__(kBlock) group_ff_kernel(const JobDesc* __restrict__ jobs,
                                                          const Chunk* __restrict__ chunks, int count, int* counter) {
    __shared__ int slot;
    __shared__ LleParams sL;
    for (;;) {
        if (threadIdx.x == 0) slot = atomicAdd(counter, 1);
        __syncthreads();
        const int c = slot;
        __syncthreads();
        if (c >= count) return;
        const Chunk ch = chunks[c];
        const JobDesc& J = jobs[ch.job];
        if (threadIdx.x == 0) sL = J.lp;
        __syncthreads();
#pragma unroll 1
        for (int t = 2 * threadIdx.x; t < ch.count; t += 2 * blockDim.x) {
            const long long p = ch.begin + t;
            const bool two = t + 1 < ch.count;
            lle_pair_ff<F>(sL, p, two ? p + 1 : p, J.lle + p, two ? J.lle + p + 1 : nullptr);
        }
    }
}

using GroupFF = void (*)(const JobDesc*, const Chunk*, int, int*);
GroupFF group_ff_for(int system) {
    switch (system) {
        case SYS_LORENZ_RK4: return group_ff_kernel<Lorenz>;
        case SYS_ROSSLER_RK4: return group_ff_kernel<Rossler>;
        case SYS_CHEN_RK4: return group_ff_kernel<Chen>;
        default: return nullptr;
    }
}

unsigned blocks_for(long long threads) { return (unsigned)((threads + kBlock - 1) / kBlock); }

// 1 (default): two points per thread in packed words; 0: one point per thread.
// Results are identical either way (every paired operation rounds each lane as
// the scalar operation does).
std::atomic<int> g_ff_pairs{1};

template <class F> void launch_ff(const LleParams& L, double* out, cudaStream_t st) {
    if (g_ff_pairs.load(std::memory_order_relaxed)) lle_ff_pair_kernel<F><<<blocks_for((L.nPoints + 1) / 2), kBlock, 0, st>>>(L, out);
    else lle_ff_kernel<F><<<blocks_for(L.nPoints), kBlock, 0, st>>>(L, out);
    note_launch();
}
}  // namespace

int set_ff_pairs(int v) {
    if (v != 0 && v != 1) return -1;
    g_ff_pairs.store(v);
    return 0;
}
int get_ff_pairs() { return g_ff_pairs.load(); }

cudaError_t launch_lle_ff(const LleParams& L, double* out, cudaStream_t st) {
    if (L.nPoints <= 0) return cudaSuccess;
    switch (L.system) {
        case SYS_LORENZ_RK4: launch_ff<Lorenz>(L, out, st); break;
        case SYS_ROSSLER_RK4: launch_ff<Rossler>(L, out, st); break;
        case SYS_CHEN_RK4: launch_ff<Chen>(L, out, st); break;
        default: return cudaErrorNotSupported;
    }
    return cudaGetLastError();
}

int group_ff_resident_blocks(int system, int device) {
    GroupFF k = group_ff_for(system);
    if (!k) return 0;
    int perSm = 0, sms = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, k, kBlock, 0);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    return (perSm > 1 ? perSm : 1) * (sms > 1 ? sms : 1);
}

cudaError_t launch_group_ff(int system, const JobDesc* jobs, const Chunk* chunks, int count, int* counter,
                            int gridBlocks, cudaStream_t st) {
    GroupFF k = group_ff_for(system);
    if (!k) return cudaErrorInvalidValue;
    if (count <= 0) return cudaSuccess;
    k<<<gridBlocks, kBlock, 0, st>>>(jobs, chunks, count, counter);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_lle_states_ff(const LleParams& L, const double* states, double* out, cudaStream_t st) {
    if (L.nPoints <= 0) return cudaSuccess;
    const unsigned g = blocks_for(L.nPoints);
    switch (L.system) {
        case SYS_LORENZ_RK4: lle_ff_states_kernel<Lorenz><<<g, kBlock, 0, st>>>(L, states, out); break;
        case SYS_ROSSLER_RK4: lle_ff_states_kernel<Rossler><<<g, kBlock, 0, st>>>(L, states, out); break;
        case SYS_CHEN_RK4: lle_ff_states_kernel<Chen><<<g, kBlock, 0, st>>>(L, states, out); break;
        default: return cudaErrorNotSupported;
    }
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_trajectory_ff(int system, const double* x0, const double* a0, double h, int nSteps, double* out,
                                 long long n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    const unsigned g = blocks_for(n);
    switch (system) {
        case SYS_LORENZ_RK4: trajectory_kernel_ff<Lorenz><<<g, kBlock, 0, st>>>(x0, a0, h, nSteps, out, n); break;
        case SYS_ROSSLER_RK4: trajectory_kernel_ff<Rossler><<<g, kBlock, 0, st>>>(x0, a0, h, nSteps, out, n); break;
        case SYS_CHEN_RK4: trajectory_kernel_ff<Chen><<<g, kBlock, 0, st>>>(x0, a0, h, nSteps, out, n); break;
        default: return cudaErrorNotSupported;
    }
    note_launch();
    return cudaGetLastError();
}

}  // namespace chaos
