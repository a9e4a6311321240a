"""Float-float arithmetic (chaoslibrary_gb300/csrc/ff.h) on the host: the
same header the CHAOS_FF32 kernels include, compiled with g++ and no
contraction. Checks the error-free transformations (TwoSum exact), the
accuracy of the unnormalised sum and product against FP64, the FF RK4 step of
the three RK4 systems against the FP64 step (the oracle's arithmetic), and
the exactness of the power-of-two renormalisation of the Benettin twin."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

CHECKER = r"""
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <random>
#include "ff.h"
using namespace chaos;

static double rel(double a, double b) { return std::fabs(a - b) / std::fmax(std::fabs(b), 1e-300); }

template <class F> double step_err(std::mt19937_64& g, const double* a0, double scale, int steps) {
    std::uniform_real_distribution<double> U(-scale, scale);
    double worst = 0;
    for (int t = 0; t < 200; ++t) {
        double x[3] = {U(g), U(g), U(g)};
        FF<float> xf[3], af[3];
        float aw[3];
        for (int k = 0; k < 3; ++k) { xf[k] = ff_from_double(x[k]); af[k] = ff_from_double(a0[k]); aw[k] = (float)a0[k]; }
        // the FP64 orbit starts from the FF start's exact value, so only the steps are compared
        for (int k = 0; k < 3; ++k) x[k] = ff_to_double(xf[k]);
        double ad[3];
        for (int k = 0; k < 3; ++k) ad[k] = ff_to_double(af[k]);
        const RK4H<double> cd(0.01);
        FFH<float> c;
        c.hh = ff_from_double(0.01 * 0.5); c.h = ff_from_double(0.01); c.h6 = ff_from_double(0.01 / 6.0);
        const RK4H<float> cw(0.01f);
        for (int s = 0; s < steps; ++s) {
            rk4_step<F>(x, ad, cd);
            ff_rk4_step<F, false>(xf, (float*)nullptr, af, aw, c, cw);
        }
        const double n = std::sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
        for (int k = 0; k < 3; ++k) worst = std::fmax(worst, std::fabs(ff_to_double(xf[k]) - x[k]) / n);
    }
    return worst;
}

int main() {
    std::mt19937_64 g(11);
    std::uniform_real_distribution<double> U(-1.0, 1.0);
    std::uniform_int_distribution<int> E(-20, 20);
    // TwoSum: s + e == a + b exactly (exponents within 20: the sum is exact in double)
    long long twosum_bad = 0;
    for (int t = 0; t < 200000; ++t) {
        const float a = (float)std::ldexp(U(g), E(g)), b = (float)std::ldexp(U(g), E(g));
        const FF<float> r = two_sum(a, b);
        if ((double)r.hi + (double)r.lo != (double)a + (double)b || r.hi != a + b) ++twosum_bad;
    }
    // sum and product of FF values against FP64 (same signs for the sum: no cancellation)
    double add_err = 0, mul_err = 0, sub_err = 0;
    for (int t = 0; t < 200000; ++t) {
        const double x = std::ldexp(0.5 + 0.5 * std::fabs(U(g)), E(g)), y = std::ldexp(0.5 + 0.5 * std::fabs(U(g)), E(g));
        const FF<float> fx = ff_from_double(x), fy = ff_from_double(y);
        const double dx = ff_to_double(fx), dy = ff_to_double(fy);
        add_err = std::fmax(add_err, rel(ff_to_double(normalise(fx + fy)), dx + dy));
        mul_err = std::fmax(mul_err, rel(ff_to_double(normalise(fx * fy)), dx * dy));
        const FF<float> d = fx - fy;  // cancellation: absolute error against the operands' size
        sub_err = std::fmax(sub_err, std::fabs(ff_to_double(d) - (dx - dy)) / std::fmax(dx, dy));
    }
    // the FF value of a double: within 2^-48
    double conv_err = 0;
    for (int t = 0; t < 100000; ++t) {
        const double x = std::ldexp(U(g), E(g));
        conv_err = std::fmax(conv_err, rel(ff_to_double(ff_from_double(x)), x));
    }
    // RK4 steps against FP64 (non-chaotic horizons: 1 and 100 steps)
    const double lor[3] = {10.0, 28.0, 8.0 / 3.0}, ros[3] = {0.2, 0.2, 5.7}, chen[3] = {35.0, 3.0, 28.0};
    double s1 = 0, s100 = 0;
    s1 = std::fmax(s1, step_err<Lorenz>(g, lor, 15.0, 1));
    s1 = std::fmax(s1, step_err<Rossler>(g, ros, 8.0, 1));
    s1 = std::fmax(s1, step_err<Chen>(g, chen, 15.0, 1));
    s100 = std::fmax(s100, step_err<Lorenz>(g, lor, 15.0, 100));
    s100 = std::fmax(s100, step_err<Rossler>(g, ros, 8.0, 100));
    s100 = std::fmax(s100, step_err<Chen>(g, chen, 15.0, 100));
    // power-of-two renormalisation: exact scaling, |e| back within [eps/sqrt2, eps*sqrt2*sqrt2)
    const float eps = 1e-8f;
    int e2;
    std::frexp(eps * eps, &e2);
    long long renorm_bad = 0;
    for (int t = 0; t < 100000; ++t) {
        float e[3] = {(float)(eps * std::ldexp(U(g), E(g) / 2)), (float)(eps * U(g)), (float)(eps * U(g))};
        const float n2 = e[0] * e[0] + e[1] * e[1] + e[2] * e[2];
        if (!(n2 > 0)) continue;
        const int k = pow2_rescale_exponent(n2, e2);
        const float sc = pow2_scale(k);
        double before = 0, after = 0;
        for (int i = 0; i < 3; ++i) {
            const float r = e[i] * sc;
            if ((double)r != (double)e[i] * std::ldexp(1.0, -k)) ++renorm_bad;  // exact
            before += (double)e[i] * e[i];
            after += (double)r * r;
        }
        const double ratio = std::sqrt(after) / eps;
        if (ratio < 0.5 || ratio > 2.0) ++renorm_bad;
        // the stretch is kept: log(|e_after|) + k ln 2 == log(|e_before|)
        if (std::fabs(0.5 * std::log(after) + k * std::log(2.0) - 0.5 * std::log(before)) > 1e-12) ++renorm_bad;
    }
    std::printf("%lld %.3e %.3e %.3e %.3e %.3e %.3e %lld\n", twosum_bad, add_err, mul_err, sub_err, conv_err, s1,
                s100, renorm_bad);
    return 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_float_float_arithmetic(tmp_path):
    src = tmp_path / "ff_check.cpp"
    src.write_text(CHECKER)
    exe = tmp_path / "ff_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", f"-I{ROOT / 'chaoslibrary_gb300' / 'csrc'}",
                    str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    twosum_bad, renorm_bad = int(out[0]), int(out[7])
    add_err, mul_err, sub_err, conv_err, s1, s100 = map(float, out[1:7])
    assert twosum_bad == 0
    assert add_err < 2 ** -46, add_err   # FP32 alone: 2^-24
    assert mul_err < 2 ** -45, mul_err
    assert sub_err < 2 ** -46, sub_err
    assert conv_err <= 2 ** -48, conv_err
    assert s1 < 1e-13, s1                 # one RK4 step of each system, relative to the state's norm
    assert s100 < 2e-11, s100             # 100 steps from random states (Rossler's z(x - c) term grows
                                          # errors ~10x over 1 time unit); FP32 would be ~1e-6
    assert renorm_bad == 0
