"""The FP32 implicit stages divide by a per-point constant through div_by
(chaoslibrary_gb300/csrc/systems.h): one reciprocal, then a product corrected
once with an FMA residual. This checks the helper itself on the host (g++, the
same header the kernels include): equal to the IEEE quotient for the divisors
of the Chameleon and sin3 sweeps and for divisors in [1, 1.03), within one ulp
in the normal range for any divisor, and signed zeros kept."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

CHECKER = r"""
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <cfloat>
#include <initializer_list>
#include "systems.h"
using chaos::div_by;
static float bits(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }
static uint32_t ubits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
static long long exact_for(float d, int stride) {  // mismatches over one binade of x (every stride-th mantissa)
    const float r = 1.0f / d;
    long long bad = 0;
    for (uint32_t m = 0; m < (1u << 23); m += stride) {
        const float x = bits(0x3f800000u | m);
        if (ubits(div_by(x, d, r)) != ubits(x / d)) ++bad;
        if (ubits(div_by(-x, d, r)) != ubits(-x / d)) ++bad;
    }
    return bad;
}
int main() {
    long long bad = 0, divisors = 0;
    // the implicit-stage divisors of the Chameleon sweeps (a3 in [0, 5], h 0.01, a0 0.5) and of sin3 (h 0.01)
    for (int n : {300, 600})
        for (int i = 0; i < n; ++i) {
            const float a3 = (float)(i * (5.0 / (n - 1))), h2 = (1.0f - 0.5f) * 0.01f;
            bad += exact_for(1.0f + a3 * h2, 64); ++divisors;
        }
    bad += exact_for(1.0f + (float)(0.01 * (1.0 - 0.5)) * 0.1f, 1); ++divisors;
    // divisors spread over [1, 1.03)
    const uint32_t lo = ubits(1.0f), hi = ubits(1.03f);
    uint32_t s = 12345u;
    for (int k = 0; k < 400; ++k) {
        s = s * 1664525u + 1013904223u;
        bad += exact_for(bits(lo + (s >> 8) % (hi - lo)), 64); ++divisors;
    }
    // any divisor, normal range: within one ulp
    long long far = 0, checked = 0;
    for (int k = 0; k < 2000; ++k) {
        s = s * 1664525u + 1013904223u;
        const float d = bits(0x3f800000u | (s & 0x7fffff)) * (float)(1 + (k % 7));
        const float r = 1.0f / d;
        for (int t = 0; t < 4096; ++t) {
            s = s * 1664525u + 1013904223u;
            const float x = bits(((100u + (s >> 27)) << 23) | (s & 0x7fffff));
            const long long diff = (long long)ubits(div_by(x, d, r)) - (long long)ubits(x / d);
            if (diff > 1 || diff < -1) ++far;
            ++checked;
        }
    }
    int zeros = ubits(div_by(0.0f, 1.01f, 1.0f / 1.01f)) == ubits(0.0f) &&
                ubits(div_by(-0.0f, 1.01f, 1.0f / 1.01f)) == ubits(-0.0f);
    std::printf("%lld %lld %lld %lld %d\n", divisors, bad, checked, far, zeros);
    return 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_div_by_matches_the_quotient(tmp_path):
    src = tmp_path / "div_by_check.cpp"
    src.write_text(CHECKER)
    exe = tmp_path / "div_by_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", f"-I{ROOT / 'chaoslibrary_gb300' / 'csrc'}",
                    str(src), "-o", str(exe)], check=True)
    divisors, bad, checked, far, zeros = map(int, subprocess.run([str(exe)], check=True, capture_output=True,
                                                                  text=True).stdout.split())
    assert divisors == 1301 and checked == 2000 * 4096
    assert bad == 0, f"{bad} quotients differ from x / d"
    assert far == 0, f"{far} quotients more than one ulp from x / d"
    assert zeros == 1
