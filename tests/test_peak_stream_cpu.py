"""The streaming peak detector of the sweeps (PeakStream, chaoslibrary_gb300/
csrc/peaks.h) on the host: both of its forms (branches, and the select form
the one-wave sweeps use), in double and in float, give the golden peak lists
of the reference's peakFinder and the oracle's peaks on plateau-heavy random
series (ties, runs of equal samples, rises and drops at the 1e-13 threshold,
NaN and infinities in the double series)."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"

CHECKER = r"""
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "peaks.h"
using chaos::PeakStream;
// series (n x len doubles) in argv[1]; writes counts, peaks and intervals of the
// four detector variants to argv[2] as doubles, variant-major
template <class T, bool Sel>
static void run(const std::vector<double>& d, int n, int len, int cap, double h, std::vector<double>& out) {
    for (int s = 0; s < n; ++s) {
        PeakStream<T, Sel> ps;
        ps.init();
        std::vector<double> pk(cap, 0.0), iv(cap, 0.0);
        for (int k = 0; k < len; ++k) {
            T val;
            int t;
            if (ps.push((T)d[(size_t)s * len + k], val, t)) {
                if (ps.n >= 1 && ps.n - 1 < cap) {
                    pk[ps.n - 1] = (double)val;
                    iv[ps.n - 1] = (double)(t - ps.tprev) * h;
                }
                ps.tprev = t;
                ++ps.n;
            }
        }
        out.push_back(ps.n > 1 ? ps.n - 1 : 0);
        out.insert(out.end(), pk.begin(), pk.end());
        out.insert(out.end(), iv.begin(), iv.end());
    }
}
int main(int argc, char** argv) {
    const int n = atoi(argv[3]), len = atoi(argv[4]), cap = atoi(argv[5]);
    const double h = atof(argv[6]);
    std::vector<double> d((size_t)n * len), out;
    FILE* f = fopen(argv[1], "rb");
    if (!f || fread(d.data(), sizeof(double), d.size(), f) != d.size()) return 1;
    fclose(f);
    run<double, false>(d, n, len, cap, h, out);
    run<double, true>(d, n, len, cap, h, out);
    run<float, false>(d, n, len, cap, h, out);
    run<float, true>(d, n, len, cap, h, out);
    f = fopen(argv[2], "wb");
    if (!f) return 1;
    fwrite(out.data(), sizeof(double), out.size(), f);
    fclose(f);
    return 0;
}
"""


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("needs g++")
    d = tmp_path_factory.mktemp("peaks")
    src = d / "peak_stream_check.cpp"
    src.write_text(CHECKER)
    exe = d / "peak_stream_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", f"-I{ROOT / 'chaoslibrary_gb300' / 'csrc'}",
                    str(src), "-o", str(exe)], check=True)

    def run(data, h, cap):
        data = np.ascontiguousarray(np.atleast_2d(data), dtype=np.float64)
        n, ln = data.shape
        fin, fout = d / "in.bin", d / "out.bin"
        data.tofile(fin)
        subprocess.run([str(exe), str(fin), str(fout), str(n), str(ln), str(cap), repr(h)], check=True)
        out = np.fromfile(fout, dtype=np.float64).reshape(4, n, 1 + 2 * cap)
        return [(o[:, 0].astype(np.int64), o[:, 1:1 + cap], o[:, 1 + cap:]) for o in out]

    return run


def _same(a, b, counts):
    for s, c in enumerate(counts):
        c = int(c)
        if not np.array_equal(a[s, :c], b[s, :c], equal_nan=True):
            return False
    return True


@pytest.mark.parametrize("name", ["peaks_crafted", "peaks_random"])
def test_double_forms_match_golden(checker, name):
    g = np.load(GOLDEN / f"{name}.npz")
    h, cap = float(g["h"]), g["data"].shape[1]
    for counts, pk, iv in checker(g["data"], h, cap)[:2]:
        assert np.array_equal(counts, g["counts"])
        assert _same(pk, g["peaks"], counts)
        assert _same(iv, g["intervals"], counts)


def _plateau_series(rng, n, ln, with_specials):
    d = rng.integers(0, 5, size=(n, ln)).astype(np.float64) * 0.25
    d[: n // 4] = np.repeat(d[: n // 4, ::4], 4, axis=1)[:, :ln]  # long runs of equal samples
    tiny = rng.random((n, ln)) < 0.05
    d[tiny] += rng.choice([1e-14, -1e-14, 2e-13, -2e-13], size=int(tiny.sum()))
    if with_specials:
        sp = rng.random((n, ln)) < 0.01
        d[sp] = rng.choice([np.nan, np.inf, -np.inf], size=int(sp.sum()))
    return d


def test_double_forms_match_oracle(checker, oracle):
    rng = np.random.default_rng(5)
    d = _plateau_series(rng, 300, 120, with_specials=True)
    oc, opk, oiv = oracle.peak_finder(d, 0.01, cap=120)
    assert oc.sum() > 1000  # the series are full of peaks and plateaus
    for counts, pk, iv in checker(d, 0.01, 120)[:2]:
        assert np.array_equal(counts, oc)
        assert _same(pk, opk, counts)
        assert _same(iv, oiv, counts)


def test_float_forms_match_oracle(checker, oracle):
    """Float series whose differences are exact in float (multiples of 1/4,
    no 1e-13 offsets): the float detector finds the oracle's peaks."""
    rng = np.random.default_rng(6)
    d = rng.integers(0, 5, size=(300, 120)).astype(np.float64) * 0.25
    d[:75] = np.repeat(d[:75, ::4], 4, axis=1)[:, :120]
    oc, opk, oiv = oracle.peak_finder(d, 0.01, cap=120)
    assert oc.sum() > 1000
    for counts, pk, iv in checker(d, 0.01, 120)[2:]:
        assert np.array_equal(counts, oc)
        assert _same(pk, opk, counts)
        assert _same(iv, oiv, counts)


def test_float_forms_agree_on_hard_series(checker):
    """The float detector's two forms -- branches behind the one-compare gate,
    and selects -- on series built to exercise the gate's slow path: long
    runs of equal samples, rises and drops just above and below the 1e-13
    threshold (values near 1e-12, where such steps are representable in
    float), NaN and infinities."""
    rng = np.random.default_rng(7)
    d = _plateau_series(rng, 400, 160, with_specials=True) * 4e-12
    small = rng.random(d.shape) < 0.3
    d[small] = rng.choice([0.0, 1e-12, 1.1e-12, 1.2e-12], size=int(small.sum()))
    gated, sel = checker(d, 0.01, 160)[2:]
    assert gated[0].sum() > 1000
    assert np.array_equal(gated[0], sel[0])
    assert _same(gated[1], sel[1], gated[0])
    assert _same(gated[2], sel[2], gated[0])
