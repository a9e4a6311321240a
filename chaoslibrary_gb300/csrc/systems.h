// Step maps of the dynamical systems the engine integrates.
//
// Every system is one in-place step of a discrete map, X <- step(X, a, h), the
// contract of ChaosLibrary's plug-in `CALC_DISCRETE_MODEL(X, a, h)` with
// `SIZE_X` / `SIZE_A` (systems/systems.cuh:12-38 in the reference). Here the
// step is a template over the arithmetic type T so that one definition serves
//   * the FP64 kernels (T = double; the translation unit is compiled with
//     contraction off, so every rounding is the one written below),
//   * the FP32 kernels (T = float; the compiler may contract), and
//   * the host-side checker (g++ with -ffp-contract=off).
// Only IEEE-exact operations (+, -, *, /, fma, sqrt) appear in the polynomial
// systems, so the FP64 results are bit-identical on the GPU and on any host.
//
// Systems 0-2 are the classic-RK4 Lorenz, Rossler and Chen flows the benchmark
// workloads name (the reference ships none of them); systems 3-7 restate the
// reference's own plug-ins formula by formula (same operation order, same
// float-typed temporaries where the reference has them), because a plug-in is
// an interface whose arithmetic must stay the same to be the same system.
#pragma once

#if defined(__CUDACC__)
#define CHAOS_HD __host__ __device__ __forceinline__
#else
#define CHAOS_HD inline
#endif
#if defined(__CUDA_ARCH__)
#define CHAOS_UNROLL _Pragma("unroll")
#else
#define CHAOS_UNROLL
#endif

#include <math.h>

#include <type_traits>

namespace chaos {

enum SystemId {
    SYS_LORENZ_RK4 = 0,   // x'=s(y-x), y'=x(r-z)-y, z'=xy-bz; a = {sigma, rho, beta}
    SYS_ROSSLER_RK4 = 1,  // x'=-y-z, y'=x+ay, z'=b+z(x-c);    a = {a, b, c}
    SYS_CHEN_RK4 = 2,     // x'=a(y-x), y'=(c-a)x-xz+cy, z'=xy-bz; a = {a, b, c}
    SYS_CHAMELEON = 3,    // reference systems/systems.cuh:11-39 (7 params)
    SYS_ROSSLER_CD = 4,   // reference systems/systems.cuh:41-63 (4 params)
    SYS_SIN3 = 5,         // reference systems/systems.cuh:67-83 (5 params)
    SYS_SIN2 = 6,         // reference systems/systems.cuh:85-101 (2-D, 2 params)
    SYS_MEMRISTOR = 7,    // reference systems/systems.cuh:103-178 (Euler, 2 params)
    SYS_COUNT = 8,
    SYS_USER = 15         // a reference-format plug-in header compiled in at build time
};

// State / parameter sizes per system (SIZE_X / SIZE_A of the reference plug-ins).
CHAOS_HD int system_nx(int s) { return s == SYS_SIN2 ? 2 : 3; }
CHAOS_HD int system_na(int s) {
    switch (s) {
        case SYS_LORENZ_RK4: case SYS_ROSSLER_RK4: case SYS_CHEN_RK4: return 3;
        case SYS_CHAMELEON: return 7;
        case SYS_ROSSLER_CD: return 4;
        case SYS_SIN3: return 5;
        case SYS_SIN2: return 2;
        case SYS_MEMRISTOR: return 2;
        default: return 0;
    }
}
// Systems whose vector field is polynomial (quadratic): they have an exact
// difference form f(X+e)-f(X), used by the FP32 twin-trajectory LLE.
CHAOS_HD bool system_has_difference_form(int s) { return s <= SYS_CHEN_RK4; }
// Systems whose FP32 LLE map carries the twin as an exact difference: the
// quadratic RK4 systems and Chameleon (chameleon_step_twin).
CHAOS_HD bool system_has_fp32_lle(int s) { return s <= SYS_CHEN_RK4 || s == SYS_CHAMELEON; }

// ---- math shims: one name per operation for both precisions ---------------
CHAOS_HD double fmaT(double a, double b, double c) { return fma(a, b, c); }
CHAOS_HD float fmaT(float a, float b, float c) { return fmaf(a, b, c); }
CHAOS_HD double cosT(double a) { return cos(a); }
CHAOS_HD float cosT(float a) { return cosf(a); }
CHAOS_HD double sinT(double a) { return sin(a); }
CHAOS_HD float sinT(float a) { return sinf(a); }
CHAOS_HD double expT(double a) { return exp(a); }
CHAOS_HD float expT(float a) { return expf(a); }
CHAOS_HD double atanT(double a) { return atan(a); }
CHAOS_HD float atanT(float a) { return atanf(a); }

// x / d for a divisor d that stays the same step after step, given r = 1/d
// (computed once, outside the step loop): the product q = RN(x r) corrected
// once with the residual of an FMA, q + (q d - x)(-r) (Markstein, IBM J. Res.
// Dev. 34(1), 1990). Three FMA-pipe instructions in place of a division. For
// divisors in [1, 1.03) (the implicit stages of Chameleon and sin3 at their
// sweeps' step sizes) it equals the correctly rounded quotient: every mantissa
// of x against x / d for the sweeps' divisors and 10,000 random ones on the
// CPU (a sample of it in tests/test_div_by_cpu.py); for any divisor it is
// within one ulp in the normal range. With the residual taken as q d - x a
// signed zero keeps its sign. FP64 divides as written.
CHAOS_HD float div_by(float x, float d, float r) {
    const float q = x * r;
    return fmaf(fmaf(q, d, -x), -r, q);
}
CHAOS_HD double div_by(double x, double d, double) { return x / d; }

// A sum that no compiler may merge with a neighbouring product. In FP64
// device code it is an explicit round-to-nearest add: the plug-in headers
// put this RK4 step into reference builds, which contract a*b + c into one
// FMA by default, and the step must round the same way there as here.
CHAOS_HD double addR(double a, double b) {
#if defined(__CUDA_ARCH__)
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}
CHAOS_HD float addR(float a, float b) { return a + b; }

// a*b + c as each arithmetic's kernels round it: FP64 as written, a product
// and a sum (the FP64 translation units and the host checker compile without
// contraction); FP32 one fused multiply-add, written out so that every FP32
// kernel -- single sweep, batch, server -- rounds it the same way instead of
// leaving the choice of which product to fuse to the compiler.
CHAOS_HD double madd(double a, double b, double c) { return a * b + c; }
CHAOS_HD float madd(float a, float b, float c) { return fmaf(a, b, c); }
// a + b that no compiler may merge with a neighbouring product (FP32).
CHAOS_HD double add_rn(double a, double b) { return a + b; }
CHAOS_HD float add_rn(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}

// ---- vector fields of the RK4 systems ---------------------------------------
struct Lorenz {
    template <class T> static CHAOS_HD void f(const T* x, const T* a, T* k) {
        k[0] = a[0] * (x[1] - x[0]);
        k[1] = fmaT(x[0], a[1] - x[2], -x[1]);
        k[2] = fmaT(x[0], x[1], -(a[2] * x[2]));
    }
    // Exact difference f(x+e) - f(x) of the quadratic field (no cancellation).
    template <class T> static CHAOS_HD void df(const T* x, const T* e, const T* a, T* d) {
        d[0] = a[0] * (e[1] - e[0]);
        d[1] = fmaT(e[0], (a[1] - x[2]) - e[2], -fmaT(x[0], e[2], e[1]));
        d[2] = fmaT(x[0], e[1], fmaT(e[0], x[1] + e[1], -(a[2] * e[2])));
    }
};

struct Rossler {
    template <class T> static CHAOS_HD void f(const T* x, const T* a, T* k) {
        k[0] = -(x[1] + x[2]);
        k[1] = fmaT(a[0], x[1], x[0]);
        k[2] = fmaT(x[2], x[0] - a[2], a[1]);
    }
    template <class T> static CHAOS_HD void df(const T* x, const T* e, const T* a, T* d) {
        d[0] = -(e[1] + e[2]);
        d[1] = fmaT(a[0], e[1], e[0]);
        d[2] = fmaT(x[2], e[0], e[2] * ((x[0] - a[2]) + e[0]));
    }
};

struct Chen {
    template <class T> static CHAOS_HD void f(const T* x, const T* a, T* k) {
        k[0] = a[0] * (x[1] - x[0]);
        k[1] = fmaT(x[0], (a[2] - a[0]) - x[2], a[2] * x[1]);
        k[2] = fmaT(x[0], x[1], -(a[1] * x[2]));
    }
    template <class T> static CHAOS_HD void df(const T* x, const T* e, const T* a, T* d) {
        d[0] = a[0] * (e[1] - e[0]);
        d[1] = fmaT(e[0], (a[2] - a[0]) - x[2], fmaT(a[2], e[1], -((x[0] + e[0]) * e[2])));
        d[2] = fmaT(x[0], e[1], fmaT(e[0], x[1] + e[1], -(a[1] * e[2])));
    }
};

// Step-size constants of one classic RK4 step, computed once per launch.
template <class T> struct RK4H {
    T h, hh, h6;
    CHAOS_HD RK4H() {}
    CHAOS_HD explicit RK4H(T h_) : h(h_), hh(h_ * T(0.5)), h6(h_ / T(6)) {}
};

// Classic fourth-order Runge-Kutta step of a 3-D autonomous field:
// x += h/6 (k1 + 2 k2 + 2 k3 + k4), the sum accumulated as the stages are
// produced (acc = k1; acc += 2 k2; acc += 2 k3; acc += k4), which keeps only
// one stage vector alive at a time.
template <class F, class T> CHAOS_HD void rk4_step(T* x, const T* a, const RK4H<T>& c);

// The Lorenz RK4 step of the FP32 paths (float and packed pairs): the stages
// carry w = rho - z instead of z, so dy = x w - y is one FMA and
// dz = x y - beta z = x y + (beta w - beta rho) two, and each stage's z update
// becomes the w update w_s = w - hh k_z: 42 FMA-pipe instructions a step
// instead of 45 (the FP32 integrations of this GPU are bound by that pipe).
// Rounded differently from the FP64 step, which keeps the reference's
// formula; every FP32 path (one point or two per thread, batches, the
// server) runs this same arithmetic.
template <class T> CHAOS_HD void lorenz_rk4_step_w(T* x, const T* a, const RK4H<T>& c) {
    const T br = a[2] * a[1];
    const T w = a[1] - x[2];
    T k[3], y[3], acc[3], wy;
    k[0] = a[0] * (x[1] - x[0]);
    k[1] = fmaT(x[0], w, -x[1]);
    k[2] = fmaT(x[0], x[1], -(a[2] * x[2]));
CHAOS_UNROLL
    for (int i = 0; i < 3; ++i) acc[i] = k[i];
    y[0] = fmaT(c.hh, k[0], x[0]);
    y[1] = fmaT(c.hh, k[1], x[1]);
    wy = fmaT(-c.hh, k[2], w);
CHAOS_UNROLL
    for (int s = 0; s < 3; ++s) {
        k[0] = a[0] * (y[1] - y[0]);
        k[1] = fmaT(y[0], wy, -y[1]);
        k[2] = fmaT(y[0], y[1], fmaT(a[2], wy, -br));
        if (s < 2) {
            const T hs = s == 0 ? c.hh : c.h;
CHAOS_UNROLL
            for (int i = 0; i < 3; ++i) acc[i] = fmaT(T(2), k[i], acc[i]);
            y[0] = fmaT(hs, k[0], x[0]);
            y[1] = fmaT(hs, k[1], x[1]);
            wy = fmaT(-hs, k[2], w);
        }
    }
CHAOS_UNROLL
    for (int i = 0; i < 3; ++i) x[i] = fmaT(c.h6, addR(acc[i], k[i]), x[i]);
}

template <class F, class T> CHAOS_HD void rk4_step(T* x, const T* a, const RK4H<T>& c) {
    if constexpr (std::is_same<F, Lorenz>::value && !std::is_same<T, double>::value) {
        lorenz_rk4_step_w(x, a, c);
        return;
    }
    T k[3], y[3], acc[3];
    F::f(x, a, k);
CHAOS_UNROLL
    for (int i = 0; i < 3; ++i) { acc[i] = k[i]; y[i] = fmaT(c.hh, k[i], x[i]); }
    F::f(y, a, k);
CHAOS_UNROLL
    for (int i = 0; i < 3; ++i) { acc[i] = fmaT(T(2), k[i], acc[i]); y[i] = fmaT(c.hh, k[i], x[i]); }
    F::f(y, a, k);
CHAOS_UNROLL
    for (int i = 0; i < 3; ++i) { acc[i] = fmaT(T(2), k[i], acc[i]); y[i] = fmaT(c.h, k[i], x[i]); }
    F::f(y, a, k);
CHAOS_UNROLL
    for (int i = 0; i < 3; ++i) x[i] = fmaT(c.h6, addR(acc[i], k[i]), x[i]);
}

// One RK4 step of the base trajectory x together with the exact difference
// e = p - x of a twin trajectory p. The twin's stages are carried as
// differences from the base stages, so e keeps full relative precision even
// when |e| is far below the resolution of x (FP32 with e ~ 1e-8).
template <class F, class T> CHAOS_HD void rk4_step_twin(T* x, T* e, const T* a, const RK4H<T>& c) {
    T k[3], y[3], acc[3], d[3], g[3], dacc[3];
    F::f(x, a, k);
    F::df(x, e, a, d);
CHAOS_UNROLL
    for (int i = 0; i < 3; ++i) {
        acc[i] = k[i];
        dacc[i] = d[i];
        y[i] = fmaT(c.hh, k[i], x[i]);
        g[i] = fmaT(c.hh, d[i], e[i]);
    }
    F::f(y, a, k);
    F::df(y, g, a, d);
CHAOS_UNROLL
    for (int i = 0; i < 3; ++i) {
        acc[i] = fmaT(T(2), k[i], acc[i]);
        dacc[i] = fmaT(T(2), d[i], dacc[i]);
        y[i] = fmaT(c.hh, k[i], x[i]);
        g[i] = fmaT(c.hh, d[i], e[i]);
    }
    F::f(y, a, k);
    F::df(y, g, a, d);
CHAOS_UNROLL
    for (int i = 0; i < 3; ++i) {
        acc[i] = fmaT(T(2), k[i], acc[i]);
        dacc[i] = fmaT(T(2), d[i], dacc[i]);
        y[i] = fmaT(c.h, k[i], x[i]);
        g[i] = fmaT(c.h, d[i], e[i]);
    }
    F::f(y, a, k);
    F::df(y, g, a, d);
CHAOS_UNROLL
    for (int i = 0; i < 3; ++i) {
        x[i] = fmaT(c.h6, acc[i] + k[i], x[i]);
        e[i] = fmaT(c.h6, dacc[i] + d[i], e[i]);
    }
}

// The same step for NE twins at once, p_q = x + e[q]: the base stages are
// evaluated once and each twin adds only its difference stages (the
// Lyapunov spectrum carries one twin per state dimension).
template <class F, int NE, class T>
CHAOS_HD void rk4_step_multi(T* x, T (*e)[3], const T* a, const RK4H<T>& c) {
    T k[3], y[3], acc[3], d[NE][3], g[NE][3], dacc[NE][3];
    F::f(x, a, k);
CHAOS_UNROLL
    for (int q = 0; q < NE; ++q) F::df(x, e[q], a, d[q]);
CHAOS_UNROLL
    for (int i = 0; i < 3; ++i) {
        acc[i] = k[i];
        y[i] = fmaT(c.hh, k[i], x[i]);
CHAOS_UNROLL
        for (int q = 0; q < NE; ++q) {
            dacc[q][i] = d[q][i];
            g[q][i] = fmaT(c.hh, d[q][i], e[q][i]);
        }
    }
    F::f(y, a, k);
CHAOS_UNROLL
    for (int q = 0; q < NE; ++q) F::df(y, g[q], a, d[q]);
CHAOS_UNROLL
    for (int i = 0; i < 3; ++i) {
        acc[i] = fmaT(T(2), k[i], acc[i]);
        y[i] = fmaT(c.hh, k[i], x[i]);
CHAOS_UNROLL
        for (int q = 0; q < NE; ++q) {
            dacc[q][i] = fmaT(T(2), d[q][i], dacc[q][i]);
            g[q][i] = fmaT(c.hh, d[q][i], e[q][i]);
        }
    }
    F::f(y, a, k);
CHAOS_UNROLL
    for (int q = 0; q < NE; ++q) F::df(y, g[q], a, d[q]);
CHAOS_UNROLL
    for (int i = 0; i < 3; ++i) {
        acc[i] = fmaT(T(2), k[i], acc[i]);
        y[i] = fmaT(c.h, k[i], x[i]);
CHAOS_UNROLL
        for (int q = 0; q < NE; ++q) {
            dacc[q][i] = fmaT(T(2), d[q][i], dacc[q][i]);
            g[q][i] = fmaT(c.h, d[q][i], e[q][i]);
        }
    }
    F::f(y, a, k);
CHAOS_UNROLL
    for (int q = 0; q < NE; ++q) F::df(y, g[q], a, d[q]);
CHAOS_UNROLL
    for (int i = 0; i < 3; ++i) {
        x[i] = fmaT(c.h6, acc[i] + k[i], x[i]);
CHAOS_UNROLL
        for (int q = 0; q < NE; ++q) e[q][i] = fmaT(c.h6, dacc[q][i] + d[q][i], e[q][i]);
    }
}

// ---- the reference's own plug-in systems, restated --------------------------
// Chameleon, semi-implicit two-stage composition (systems/systems.cuh:11-39).
// The sums of products are written with madd: in FP64 they round exactly as
// the reference's expressions (a6*X0 + a1*X2, a2 - a3*X2 + a4*cos, 1 + a3*h2,
// a2 + a4*cos); in FP32 each is a fixed fused form.
template <class T> CHAOS_HD void chameleon_step(T* X, const T* a, T h) {
    T h1 = a[0] * h;
    T h2 = (T(1) - a[0]) * h;
    X[0] = fmaT(h1, -a[6] * X[1], X[0]);
    X[1] = fmaT(h1, madd(a[6], X[0], a[1] * X[2]), X[1]);
    T cos_term = cosT(a[5] * X[1]);
    X[2] = fmaT(h1, madd(a[4], cos_term, madd(-a[3], X[2], a[2])), X[2]);
    const T den = madd(a[3], h2, T(1));
    X[2] = div_by(fmaT(h2, madd(a[4], cos_term, a[2]), X[2]), den, T(1) / den);
    X[1] = fmaT(h2, madd(a[6], X[0], a[1] * X[2]), X[1]);
    X[0] = fmaT(h2, -a[6] * X[1], X[0]);
}

// The Chameleon step of NE twins carried as differences E[q] = Q_q - X from
// the orbit X (FP32 LLE map and spectrum). Every update of the composition is
// linear in the state except the cos term, whose difference is taken in
// product form, cos(u + d) - cos(u) = -2 sin(u + d/2) sin(d/2) with
// u = a5*X1, d = a5*E1: each E keeps its full relative precision while |E| is
// far below the resolution of X. X advances exactly as chameleon_step does.
template <class T, int NE> CHAOS_HD void chameleon_step_multi(T* X, T (*E)[3], const T* a, T h) {
    const T h1 = a[0] * h;
    const T h2 = (T(1) - a[0]) * h;
    X[0] = fmaT(h1, -a[6] * X[1], X[0]);
CHAOS_UNROLL
    for (int q = 0; q < NE; ++q) E[q][0] = fmaT(h1, -a[6] * E[q][1], E[q][0]);
    X[1] = fmaT(h1, madd(a[6], X[0], a[1] * X[2]), X[1]);
CHAOS_UNROLL
    for (int q = 0; q < NE; ++q) E[q][1] = fmaT(h1, madd(a[6], E[q][0], a[1] * E[q][2]), E[q][1]);
    const T u = a[5] * X[1];
    const T cos_term = cosT(u);
    T dcos[NE];
CHAOS_UNROLL
    for (int q = 0; q < NE; ++q) {
        const T half = T(0.5) * (a[5] * E[q][1]);
        dcos[q] = T(-2) * sinT(add_rn(u, half)) * sinT(half);
    }
    X[2] = fmaT(h1, madd(a[4], cos_term, madd(-a[3], X[2], a[2])), X[2]);
CHAOS_UNROLL
    for (int q = 0; q < NE; ++q) E[q][2] = fmaT(h1, madd(a[4], dcos[q], -(a[3] * E[q][2])), E[q][2]);
    const T den = madd(a[3], h2, T(1));
    const T rden = T(1) / den;
    X[2] = div_by(fmaT(h2, madd(a[4], cos_term, a[2]), X[2]), den, rden);
CHAOS_UNROLL
    for (int q = 0; q < NE; ++q) E[q][2] = div_by(fmaT(h2, a[4] * dcos[q], E[q][2]), den, rden);
    X[1] = fmaT(h2, madd(a[6], X[0], a[1] * X[2]), X[1]);
CHAOS_UNROLL
    for (int q = 0; q < NE; ++q) E[q][1] = fmaT(h2, madd(a[6], E[q][0], a[1] * E[q][2]), E[q][1]);
    X[0] = fmaT(h2, -a[6] * X[1], X[0]);
CHAOS_UNROLL
    for (int q = 0; q < NE; ++q) E[q][0] = fmaT(h2, -a[6] * E[q][1], E[q][0]);
}

// One twin (the LLE map).
template <class T> CHAOS_HD void chameleon_step_twin(T* X, T* E, const T* a, T h) {
    T Em[1][3] = {{E[0], E[1], E[2]}};
    chameleon_step_multi<T, 1>(X, Em, a, h);
    E[0] = Em[0][0];
    E[1] = Em[0][1];
    E[2] = Em[0][2];
}

// Rossler, "CD" composition (systems/systems.cuh:41-63).
template <class T> CHAOS_HD void rossler_cd_step(T* x, const T* a, T h) {
    T h1 = T(0.5) * h + a[0];
    T h2 = T(0.5) * h - a[0];
    x[0] = fmaT(h1, -x[1] - x[2], x[0]);
    x[1] = fmaT(h1, x[0] + a[1] * x[1], x[1]);
    x[2] = fmaT(h1, a[2] + x[2] * (x[0] - a[3]), x[2]);
    T temp = fmaT(-h2, x[0] - a[3], T(1));
    x[2] = fmaT(h2, a[2], x[2]) / temp;
    temp = fmaT(-h2, a[1], T(1));
    x[1] = fmaT(h2, x[0], x[1]) / temp;
    x[0] = fmaT(h2, -x[1] - x[2], x[0]);
}

// Three sin-coupled oscillators for basins (systems/systems.cuh:67-83). The
// reference keeps h2 in a float, so it is rounded to float here as well.
template <class T> CHAOS_HD void sin3_step(T* X, const T* a, T h) {
    const T h2 = (T)(float)(h * (T(1) - a[0]));
    X[0] = X[0] + h * (sinT(X[1]) - a[1] * X[0]);
    X[1] = X[1] + h * (sinT(X[2]) - a[1] * X[1]);
    X[2] = X[2] + h * (sinT(X[0]) - a[1] * X[2]);
    const T den = T(1) + h2 * a[1];
    const T rden = T(1) / den;
    X[2] = div_by(X[2] + h2 * sinT(X[0]), den, rden);
    X[1] = div_by(X[1] + h2 * sinT(X[2]), den, rden);
    X[0] = div_by(X[0] + h2 * sinT(X[1]), den, rden);
}

// 2-D sin system for basins (systems/systems.cuh:85-101); h1, h2 and the
// intermediate z are floats in the reference.
template <class T> CHAOS_HD void sin2_step(T* X, const T* a, T h) {
    const T h1 = (T)(float)(h * a[0]);
    const T h2 = (T)(float)(h * (T(1) - a[0]));
    X[0] = X[0] + h1 * (-X[1]);
    X[1] = X[1] + h1 * (a[1] * X[0] + sinT(X[1]));
    const T z = (T)(float)X[1];
    X[1] = z + h2 * (a[1] * X[0] + sinT(X[1]));
    X[0] = X[0] + h2 * (-X[1]);
}

// Memristor circuit with a tunnel diode, explicit Euler (systems/systems.cuh:103-178).
template <class T> CHAOS_HD void memristor_step(T* X, const T* a, T h) {
    const T Vc = X[0], XSV = X[1], t = X[2];
    const T U1 = T(0.0), U2 = T(-0.04), C1 = T(22e-9);
    const T Is = T(1.15E-7), Vt = T(1.0) / T(15.0), Vp = T(0.09), Ip = T(2.1e-5), Iv = T(-3e-6);
    const T D = T(26.0), E = T(0.14);
    const T Vd = Vc + U2;
    const T Vm = Vc + U1;
    const T idiode = Is * (expT(Vd / Vt) - expT(-Vd / Vt));
    const T itunnel = Ip / Vp * Vd * expT(-(Vd - Vp) / Vp);
    const T iex = Iv * (atanT(D * (Vd - E)) + atanT(D * (Vd + E)));
    const T Id = idiode + itunnel + iex;
    const T Ron = T(1434.0), Roff = T(1e6), Von1 = T(0.28), Voff1 = T(0.14), Von2 = T(-0.12), Voff2 = T(-0.006);
    const T TAU = T(1e-7), TT = T(2.0), boltz = T(1.380649e-23), echarge = T(1.602176634e-19);
    const T g = XSV / Ron + (T(1.0) - XSV) / Roff;
    const T arg1 = -T(1.0) / (TT * boltz / echarge) * (Vm - Von1) * (Vm - Von2);
    const T arg2 = -T(1.0) / (TT * boltz / echarge) * (Vm - Voff2) * (Vm - Voff1);
    const T exp1 = expT(arg1), exp2 = expT(arg2);
    const T f1 = T(1.0) / (T(1.0) + exp1);
    const T f2 = T(1.0) / (T(1.0) + exp2);
    const T Ix = (T(1.0) / TAU) * (f1 * (T(1.0) - XSV) - (T(1.0) - f2) * XSV);
    const T Imem = Vm * g;
    const T Iin = a[0] * sinT(a[1] * t);
    const T dVc = (Iin - Imem - Id) / C1;
    const T dXSV = Ix;
    X[0] = Vc + h * dVc;
    X[1] = XSV + h * dXSV;
    X[2] = t + h;
}

#if defined(CHAOS_USER_SYSTEM)
// The step of a reference-format plug-in header compiled into the library
// (kern_user.cu): CALC_DISCRETE_MODEL(X, a, h) on doubles.
template <class T> __device__ void user_step(T* x, const T* a, T h);
#endif

// Per-launch step constants: the RK4 fractions of h for systems 0-2, plain h otherwise.
template <class T> struct StepCtx {
    RK4H<T> rk;
    CHAOS_HD StepCtx() {}
    CHAOS_HD explicit StepCtx(T h) : rk(h) {}
};

// One step of system S (compile-time id).
template <int S, class T> CHAOS_HD void step(T* x, const T* a, const StepCtx<T>& c) {
    if (S == SYS_LORENZ_RK4) rk4_step<Lorenz>(x, a, c.rk);
    else if (S == SYS_ROSSLER_RK4) rk4_step<Rossler>(x, a, c.rk);
    else if (S == SYS_CHEN_RK4) rk4_step<Chen>(x, a, c.rk);
    else if (S == SYS_CHAMELEON) chameleon_step(x, a, c.rk.h);
    else if (S == SYS_ROSSLER_CD) rossler_cd_step(x, a, c.rk.h);
    else if (S == SYS_SIN3) sin3_step(x, a, c.rk.h);
    else if (S == SYS_SIN2) sin2_step(x, a, c.rk.h);
    else if (S == SYS_MEMRISTOR) memristor_step(x, a, c.rk.h);
#if defined(CHAOS_USER_SYSTEM)
    else if (S == SYS_USER) user_step(x, a, c.rk.h);
#endif
}

// Runtime-dispatched step (host checker, tests).
template <class T> inline void step_dyn(int s, T* x, const T* a, const StepCtx<T>& c) {
    switch (s) {
        case SYS_LORENZ_RK4: step<SYS_LORENZ_RK4>(x, a, c); break;
        case SYS_ROSSLER_RK4: step<SYS_ROSSLER_RK4>(x, a, c); break;
        case SYS_CHEN_RK4: step<SYS_CHEN_RK4>(x, a, c); break;
        case SYS_CHAMELEON: step<SYS_CHAMELEON>(x, a, c); break;
        case SYS_ROSSLER_CD: step<SYS_ROSSLER_CD>(x, a, c); break;
        case SYS_SIN3: step<SYS_SIN3>(x, a, c); break;
        case SYS_SIN2: step<SYS_SIN2>(x, a, c); break;
        case SYS_MEMRISTOR: step<SYS_MEMRISTOR>(x, a, c); break;
        default: break;
    }
}

}  // namespace chaos
