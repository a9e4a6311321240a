// LLE and Lyapunov spectrum of the legacy library's analyses (FP64): the
// scheme of its kernels LLEKernelCUDA (debri/cudaLibrary.cu:1897-2031, LLE1D:
// a grid of parameters), LLEKernelICCUDA (:2034-2139, LLE1DIC / LLE2DIC: a
// grid of initial conditions) and LSKernelCUDA (:2189-2330, LS1D / LS2D),
// which differs from the LLE map's (LLE/src/LLECUDA.cu) in its block count,
// its twin start and its renormalisation arithmetic; and the LLE map's own
// cuRAND twin start. Included by the FP64 translation units (built-in and
// user systems).
#pragma once

#include <curand_kernel.h>

#include "engine.cuh"

namespace chaos {

// The raw twin-direction component k of point p (before normalisation), as
// the legacy kernels draw it for a grid of one chunk (their thread index is
// the point index):
//  - parameter grids: the uniform of cuRAND's default generator seeded p + k
//    (curand_init(p + k, 0, 0)), minus 0.5;
//  - initial-condition grids: 0.5 * sinf(p * (k * p + 1) + 1), the integer
//    expression in 32-bit wrap-around arithmetic.
__device__ __forceinline__ double legacy_twin_draw(int stateGrid, long long p, int k) {
    if (!stateGrid) {
        curandState_t st;
        curand_init((unsigned long long)p + (unsigned long long)k, 0ull, 0ull, &st);
        return (double)curand_uniform(&st) - 0.5;
    }
    const unsigned i = (unsigned)p;
    const int arg = (int)(i * ((unsigned)k * i + 1u) + 1u);
    return 0.5 * (double)sinf((float)arg);
}

// loopCalculateDiscreteModel (:472-527) as the legacy LLE kernels call it:
// n steps, preScaller 1, writableVar 0, no samples. It stops early when
// x[0] becomes NaN or infinite, or |(float)x[0]| > maxValue (maxValue != 0);
// its verdict is not used.
template <int S>
__device__ __forceinline__ void legacy_lle_run(double* x, const double* a, const StepCtx<double>& c, int n,
                                               double maxValue) {
    for (int s = 0; s < n; ++s) {
        step<S>(x, a, c);
        const double v = x[0];
        if (((unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull) > 0x7fefffffffffffffull) return;
        if (maxValue != 0.0 && (double)fabsf((float)v) > maxValue) return;
    }
}

// LLE of point p (L.legacyLoop): the twin direction z (draws[p*NX + k], or
// legacy_twin_draw) normalised in FP64; the transient of L.trans steps; the
// twin y = x + eps z; then L.legacyBlocks = (int)(tMax / NT) blocks of
// L.ntp steps of the orbit and of the twin, each adding log(d) for
//  - parameter grids: d = sqrt(sum ((1/eps) (x - y))^2), y = x - (x - y) / d;
//  - initial-condition grids: d = sqrt(sum (x - y)^2) / eps,
//    y = x - (x - y) * (1/d) (1/d only when d != 0);
// the sum divided by tMax.
template <int S>
__device__ __forceinline__ double lle_point_legacy(const LleParams& L, long long p) {
    constexpr int NX = Traits<S>::NX, NA = Traits<S>::NA;
    double x[NX], y[NX], z[NX], a[NA];
    lle_load<NX, NA>(L, p, x, a);
    double zp = 0.0;
#pragma unroll
    for (int k = 0; k < NX; ++k) {
        z[k] = L.draws ? L.draws[p * NX + k] : legacy_twin_draw(L.mutateState, p, k);
        zp = zp + z[k] * z[k];
    }
    zp = sqrt(zp);
#pragma unroll
    for (int k = 0; k < NX; ++k) z[k] = z[k] / zp;
    const StepCtx<double> c(L.h);
    legacy_lle_run<S>(x, a, c, L.trans, L.maxValue);
#pragma unroll
    for (int k = 0; k < NX; ++k) y[k] = x[k] + z[k] * L.eps;
    double result = 0.0;
    for (int b = 0; b < L.legacyBlocks; ++b) {
        legacy_lle_run<S>(x, a, c, L.ntp, L.maxValue);
        legacy_lle_run<S>(y, a, c, L.ntp, L.maxValue);
        double d = 0.0;
        if (!L.mutateState) {
#pragma unroll
            for (int k = 0; k < NX; ++k) {
                const double t = (1.0 / L.eps) * (x[k] - y[k]);
                d = d + t * t;
            }
            d = sqrt(d);
            result = result + log(d);
#pragma unroll
            for (int k = 0; k < NX; ++k) y[k] = x[k] - ((x[k] - y[k]) / d);
        } else {
#pragma unroll
            for (int k = 0; k < NX; ++k) d = d + (x[k] - y[k]) * (x[k] - y[k]);
            d = sqrt(d) / L.eps;
            result = result + log(d);
            if (d != 0.0) d = 1.0 / d;
#pragma unroll
            for (int k = 0; k < NX; ++k) y[k] = x[k] - ((x[k] - y[k]) * d);
        }
    }
    return result / L.tMax;
}

// The raw draw of component i of twin j of point p of the legacy spectrum
// (LSKernelCUDA, :2250): sinf of 0.2171828 (i+1)(j+1) + p + (0.2171828 +
// i j p), the argument in FP64 rounded to float, times 0.5.
__device__ __forceinline__ double legacy_spectrum_draw(long long p, int i, int j) {
    const int idx = (int)p;
    const double arg = 0.2171828 * (i + 1) * (j + 1) + idx + (0.2171828 + i * j * idx);
    return (double)sinf((float)arg) * 0.5;
}

// Classical Gram-Schmidt of the rows of v as gramSchmidtProcess
// (:2141-2187) computes it: w_j = v_j minus, for m < j, <v_j, w_m> / <w_m,
// w_m> w_m (0 for a zero w_m); then u_j = w_j / |w_j| (0 where |w_j| = 0)
// and nrm[j] = |w_j|.
template <int N>
__device__ __forceinline__ void legacy_gram_schmidt(const double (&v)[N][N], double (&u)[N][N], double (&nrm)[N]) {
    double w[N][N];
#pragma unroll
    for (int j = 0; j < N; ++j) {
#pragma unroll
        for (int i = 0; i < N; ++i) w[j][i] = v[j][i];
#pragma unroll
        for (int m = 0; m < j; ++m) {
            double num = 0.0, den = 0.0;
#pragma unroll
            for (int i = 0; i < N; ++i) {
                num = num + v[j][i] * w[m][i];
                den = den + w[m][i] * w[m][i];
            }
            const double frac = den == 0.0 ? 0.0 : num / den;
#pragma unroll
            for (int i = 0; i < N; ++i) w[j][i] = w[j][i] - frac * w[m][i];
        }
    }
#pragma unroll
    for (int j = 0; j < N; ++j) {
        double n2 = 0.0;
#pragma unroll
        for (int i = 0; i < N; ++i) n2 = n2 + w[j][i] * w[j][i];
        nrm[j] = sqrt(n2);
#pragma unroll
        for (int i = 0; i < N; ++i) u[j][i] = nrm[j] == 0.0 ? 0.0 : w[j][i] / nrm[j];
    }
}

// Lyapunov spectrum of point p (L.legacyLoop), LSKernelCUDA's scheme: twin
// directions from the normalised raw draws (draws[(p*N + j)*N + i], or
// legacy_spectrum_draw), the transient, the directions orthonormalised and
// the twins started at x + eps u_j; then L.legacyBlocks blocks of L.ntp steps
// of the orbit and of every twin (each run stopping early as
// legacy_lle_run), the differences y_j - x through Gram-Schmidt, exponent j
// adding log(|w_j| / eps) and twin j restarting at x + eps u_j; the sums
// divided by tMax. out[p*N + j].
template <int S>
__device__ __forceinline__ void spectrum_point_legacy(const LleParams& L, long long p, double* out) {
    constexpr int N = Traits<S>::NX, NA = Traits<S>::NA;
    double x[N], y[N][N], z[N][N], a[NA], sum[N], nrm[N];
    lle_load<N, NA>(L, p, x, a);
#pragma unroll
    for (int j = 0; j < N; ++j) {
        double zp = 0.0;
#pragma unroll
        for (int i = 0; i < N; ++i) {
            z[j][i] = L.draws ? L.draws[(p * N + j) * N + i] : legacy_spectrum_draw(p, i, j);
            zp = zp + z[j][i] * z[j][i];
        }
        zp = sqrt(zp);
#pragma unroll
        for (int i = 0; i < N; ++i) z[j][i] = z[j][i] / zp;
    }
    const StepCtx<double> c(L.h);
    legacy_lle_run<S>(x, a, c, L.trans, L.maxValue);
    legacy_gram_schmidt<N>(z, y, nrm);
#pragma unroll
    for (int j = 0; j < N; ++j) {
        sum[j] = 0.0;
#pragma unroll
        for (int i = 0; i < N; ++i) y[j][i] = y[j][i] * L.eps + x[i];
    }
    for (int b = 0; b < L.legacyBlocks; ++b) {
        legacy_lle_run<S>(x, a, c, L.ntp, L.maxValue);
#pragma unroll
        for (int j = 0; j < N; ++j) legacy_lle_run<S>(y[j], a, c, L.ntp, L.maxValue);
#pragma unroll
        for (int j = 0; j < N; ++j)
#pragma unroll
            for (int i = 0; i < N; ++i) y[j][i] = y[j][i] - x[i];
        legacy_gram_schmidt<N>(y, z, nrm);
#pragma unroll
        for (int j = 0; j < N; ++j) {
            sum[j] = sum[j] + log(nrm[j] / L.eps);
#pragma unroll
            for (int i = 0; i < N; ++i) y[j][i] = x[i] + z[j][i] * L.eps;
        }
    }
#pragma unroll
    for (int j = 0; j < N; ++j) out[p * N + j] = sum[j] / L.tMax;
}

// The LLE map's twin start as the reference draws it (LLE/src/LLECUDA.cu:87-101):
// cuRAND's default generator seeded with the point index (the first swept
// parameter fastest), 2*NX uniforms in turn. The first NX give the norm
// factor n = sum of (u - 0.5)^2 by float FMAs, then n * rsqrtf(n) in float;
// the next NX the direction z_k = (u - 0.5) / n (float division) and the twin
// q_k = fmaf(z_k, (float)eps, (float)x_k), every step in FP32 as there.
template <int NX>
__device__ __forceinline__ void reference_twin_start(long long p, double eps, const double* x, double* q) {
    curandState_t st;
    curand_init((unsigned long long)p, 0ull, 0ull, &st);
    float nf = 0.0f;
#pragma unroll
    for (int k = 0; k < NX; ++k) {
        const float z = curand_uniform(&st) - 0.5f;
        nf = __fmaf_rn(z, z, nf);
    }
    nf = __fmul_rn(rsqrtf(nf), nf);
#pragma unroll
    for (int k = 0; k < NX; ++k) {
        const float z = __fdiv_rn(curand_uniform(&st) - 0.5f, nf);
        q[k] = (double)__fmaf_rn(z, (float)eps, (float)x[k]);
    }
}

// LLE point of the LLE map with that twin start (L.twin == 2): the
// transient, reference_twin_start, then the Benettin blocks of
// lle_point_full.
template <int S>
__device__ __forceinline__ double lle_point_reftwin(const LleParams& L, long long p) {
    constexpr int NX = Traits<S>::NX, NA = Traits<S>::NA;
    double x[NX], q[NX], a[NA];
    lle_load<NX, NA>(L, p, x, a);
    const StepCtx<double> c(L.h);
    for (int s = 0; s < L.trans; ++s) step<S>(x, a, c);
    reference_twin_start<NX>(p, L.eps, x, q);
    return lle_benettin_full<S, double>(L, x, q, a);
}

}  // namespace chaos
