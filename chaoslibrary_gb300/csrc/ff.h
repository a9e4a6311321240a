// Float-float ("FF") arithmetic: a value is the unevaluated sum hi + lo of two
// FP32 words W (a float, or a packed pair P2 of two independent values), with
// |lo| at most a few units in the last place of hi. Every operation runs on
// the FP32 pipe, which on this GPU is 64x faster than its FP64 pipe, and
// keeps about 46-48 significant bits: the error-free transformations of
// Knuth (TwoSum: s = RN(a + b), e = a + b - s exactly) and of the fused
// multiply-add (TwoProd: p = RN(a b), e = fma(a, b, -p) exactly), combined as
// in Dekker (Numer. Math. 18, 1971) and the "sloppy" double-word sum of
// Hida, Li and Bailey's QD library (2001).
//
// Results of add / mul are left unnormalised (lo may exceed half an ulp of
// hi by a small factor); normalise() restores |lo| <= ulp(hi)/2 and is applied
// to state that is carried across steps, so lo cannot grow. Every word
// operation is an explicit round-to-nearest intrinsic: a contraction of a
// product into a following sum would break the error-free transformations.
#pragma once

#include "systems.h"

namespace chaos {

// ---- word operations (explicitly rounded, never contracted) ----------------
CHAOS_HD float w_add(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
CHAOS_HD float w_sub(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
CHAOS_HD float w_mul(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
CHAOS_HD float w_fma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return fmaf(a, b, c);
#endif
}
CHAOS_HD float w_neg(float a) { return -a; }

template <class W> struct FF {
    W hi, lo;
};

template <class W> CHAOS_HD FF<W> ff_make(W hi, W lo) {
    FF<W> r;
    r.hi = hi;
    r.lo = lo;
    return r;
}
// The FF nearest a double (hi = RN(d), lo = RN(d - hi)): within 2^-48 |d|.
CHAOS_HD FF<float> ff_from_double(double d) {
    const float h = (float)d;
    return ff_make(h, (float)(d - (double)h));
}
CHAOS_HD double ff_to_double(const FF<float>& a) { return (double)a.hi + (double)a.lo; }

// Knuth's TwoSum: s + e == a + b exactly, s = RN(a + b) (six operations).
template <class W> CHAOS_HD FF<W> two_sum(W a, W b) {
    const W s = w_add(a, b);
    const W bb = w_sub(s, a);
    const W e = w_add(w_sub(a, w_sub(s, bb)), w_sub(b, bb));
    return ff_make(s, e);
}

// a + b: TwoSum of the high words, the low words added into its error
// (eight operations, unnormalised).
template <class W> CHAOS_HD FF<W> operator+(const FF<W>& a, const FF<W>& b) {
    FF<W> s = two_sum(a.hi, b.hi);
    s.lo = w_add(s.lo, w_add(a.lo, b.lo));
    return s;
}
template <class W> CHAOS_HD FF<W> operator-(const FF<W>& a) { return ff_make(w_neg(a.hi), w_neg(a.lo)); }
template <class W> CHAOS_HD FF<W> operator-(const FF<W>& a, const FF<W>& b) {
    FF<W> s = two_sum(a.hi, w_neg(b.hi));
    s.lo = w_add(s.lo, w_sub(a.lo, b.lo));
    return s;
}
// a * b: TwoProd of the high words plus the two cross terms (four
// operations, unnormalised; the lo*lo term is below the format's precision).
template <class W> CHAOS_HD FF<W> operator*(const FF<W>& a, const FF<W>& b) {
    const W p = w_mul(a.hi, b.hi);
    W e = w_fma(a.hi, b.hi, w_neg(p));
    e = w_fma(a.hi, b.lo, e);
    e = w_fma(a.lo, b.hi, e);
    return ff_make(p, e);
}
// The names the step templates of systems.h use.
template <class W> CHAOS_HD FF<W> fmaT(const FF<W>& a, const FF<W>& b, const FF<W>& c) { return a * b + c; }
template <class W> CHAOS_HD FF<W> addR(const FF<W>& a, const FF<W>& b) { return a + b; }
// 2 a + c: doubling is exact, so it folds into the sum at no cost.
template <class W> CHAOS_HD FF<W> twice_plus(const FF<W>& a, const FF<W>& c) {
    const W two = W(2.0);
    const W s = w_fma(two, a.hi, c.hi);  // RN(2 a.hi + c.hi)
    const W bb = w_sub(s, c.hi);
    const W e = w_add(w_sub(c.hi, w_sub(s, bb)), w_fma(two, a.hi, w_neg(bb)));
    return ff_make(s, w_add(e, w_fma(two, a.lo, c.lo)));
}
// Fast TwoSum of hi and lo (|lo| <= |hi| or hi == 0): |lo'| <= ulp(hi')/2.
template <class W> CHAOS_HD FF<W> normalise(const FF<W>& a) {
    const W h = w_add(a.hi, a.lo);
    return ff_make(h, w_sub(a.lo, w_sub(h, a.hi)));
}

// Step constants of a classic RK4 step in FF: h/2, h and h/6 of the FP64
// step (rounded as RK4H<double> rounds them), each to 2^-48.
template <class W> struct FFH {
    FF<W> hh, h, h6;
};

// One classic RK4 step of the base trajectory x in FF (rk4_step's stage
// order and sums), and with TWIN the exact FP32 difference e = p - x of the
// twin advanced beside it as rk4_step_twin advances it: its stages take the
// high words of the FF stage states. x is normalised at the end of the step.
template <class F, bool TWIN, class W>
CHAOS_HD void ff_rk4_step(FF<W>* x, W* e, const FF<W>* a, const W* af, const FFH<W>& c, const RK4H<W>& cf) {
    FF<W> k[3], y[3], acc[3];
    W yw[3], d[3], g[3], dacc[3];
    F::f(x, a, k);
    if (TWIN) {
CHAOS_UNROLL
        for (int i = 0; i < 3; ++i) yw[i] = x[i].hi;
        F::df(yw, e, af, d);
    }
CHAOS_UNROLL
    for (int i = 0; i < 3; ++i) {
        acc[i] = k[i];
        y[i] = fmaT(c.hh, k[i], x[i]);
        if (TWIN) {
            dacc[i] = d[i];
            g[i] = fmaT(cf.hh, d[i], e[i]);
        }
    }
CHAOS_UNROLL
    for (int s = 0; s < 3; ++s) {
        F::f(y, a, k);
        if (TWIN) {
CHAOS_UNROLL
            for (int i = 0; i < 3; ++i) yw[i] = y[i].hi;
            F::df(yw, g, af, d);
        }
        if (s < 2) {
CHAOS_UNROLL
            for (int i = 0; i < 3; ++i) {
                acc[i] = twice_plus(k[i], acc[i]);
                y[i] = fmaT(s == 0 ? c.hh : c.h, k[i], x[i]);
                if (TWIN) {
                    dacc[i] = fmaT(W(2.0), d[i], dacc[i]);
                    g[i] = fmaT(s == 0 ? cf.hh : cf.h, d[i], e[i]);
                }
            }
        }
    }
CHAOS_UNROLL
    for (int i = 0; i < 3; ++i) {
        x[i] = normalise(fmaT(c.h6, acc[i] + k[i], x[i]));
        if (TWIN) e[i] = fmaT(cf.h6, dacc[i] + d[i], e[i]);
    }
}

// Benettin renormalisation by a power of two: e is scaled by 2^-k, with k
// chosen from the exponent of |e|^2 so that |e| returns to within a factor
// sqrt(2) of eps. The scaling is exact in FP32, so the stretch of every block
// is kept exactly: the sum over blocks of log(|e_end| / |e_start|) telescopes
// to k_total ln 2 + log(|e_final| / eps), taken once in FP64 at the end.
// eps2Exp is the binary exponent of RN(eps^2) (frexp convention).
CHAOS_HD int pow2_rescale_exponent(float n2, int eps2Exp) {
    int E;
#if defined(__CUDA_ARCH__)
    E = (int)((__float_as_uint(n2) >> 23) & 0xff) - 126;  // frexp exponent of a normal n2
#else
    frexpf(n2, &E);
#endif
    int k = (E - eps2Exp) >> 1;
    return k < -120 ? -120 : (k > 120 ? 120 : k);
}
CHAOS_HD float pow2_scale(int k) {  // 2^-k for |k| <= 120
#if defined(__CUDA_ARCH__)
    return __uint_as_float((unsigned)(127 - k) << 23);
#else
    return ldexpf(1.0f, -k);
#endif
}
// log of the whole stretch over the blocks, in FP64: ln 2 * kTotal + log(|e| / eps).
CHAOS_HD double pow2_log_stretch(long long kTotal, double n2, double eps) {
    return (double)kTotal * 0.69314718055994530942 + 0.5 * log(n2) - log(eps);
}

}  // namespace chaos
