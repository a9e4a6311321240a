"""The oracle's restatements of the legacy library's analyses (the engine's
old_library::* and grid modes, chaos_lyapunov_spectrum) against the legacy
library's own functions, extracted unchanged from debri/cudaLibrary.cu and
compiled for the host by oracle/build_ref.py. Runs where that build exists.

Pinned bit for bit: the log-scale axis (getValueByIdxLog, raised to 10^x as
the engine's CHAOS_GRID_LOG* tables are), the linear axis (getValueByIdx), the
legacy peakFinder against the current library's (the engine follows the
latter), and the spectrum's per-block classical Gram-Schmidt and
renormalisation (projectionOperator, gramSchmidtProcess, the block loop of
LSKernelCUDA replayed around them) against orc_lyapunov_spectrum with the same
twin start and block count. Not pinned, by design: the legacy kernels'
twin directions (cuRAND in LLEKernelCUDA; sinf of the chunk-relative thread
index in LSKernelCUDA) and their hard-wired system."""
import math

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.skipif(not O.legacy_available(), reason="host build of the legacy library not present")


@pytest.fixture(scope="module")
def leg():
    return O.LegacyLib()


@pytest.mark.parametrize("r0, r1, n", [(1e-3, 1e-1, 300), (0.01, 0.02, 1000), (2.0, 2000.0, 37), (0.5, 0.25, 64)])
def test_log_axis_matches_legacy(leg, r0, r1, n):
    """The exponent of every log-scale grid value: log10(r0) + n * ((log10(r1)
    - log10(r0)) / (nPts - 1)) with the C library's log10, as the engine's host
    table computes it (the table then raises 10 to it with the C library)."""
    l0 = math.log10(r0)
    step = (math.log10(r1) - l0) / (n - 1)
    ours = [l0 + k * step for k in range(n)]
    assert ours == [leg.value_log(k, n, r0, r1, 0) for k in range(n)]
    # the second dimension of a 2-D grid indexes with idx / nPts
    assert ours == [leg.value_log(k * n + 3, n, r0, r1, 1) for k in range(n)]


def test_linear_axis_matches_legacy(leg):
    for r0, r1, n in [(20.0, 200.0, 1000), (0.1, 0.4, 1024), (-30.0, 30.0, 2048)]:
        for k in range(0, n, 7):
            ours = r0 + k * ((r1 - r0) / (n - 1))
            assert ours == leg.value(k, n, r0, r1, 0)
            assert ours == leg.value(k * n + 5, n, r0, r1, 1)


def test_legacy_peak_finder_matches_current(leg, oracle):
    rng = np.random.default_rng(17)
    for trial in range(200):
        n = int(rng.integers(3, 400))
        vals = np.round(rng.normal(size=n).cumsum(), int(rng.integers(0, 3)))  # plateaus from rounding
        data = np.repeat(vals, rng.integers(1, 4, size=n))[:n] if trial % 2 else vals  # and from repeats
        c, pk, tm = leg.peak_finder(data, 0.01)
        counts, peaks, intervals = oracle.peak_finder(data[None, :], 0.01)
        assert c == int(counts[0])
        assert np.array_equal(pk, peaks[0, :c])
        assert np.array_equal(tm, intervals[0, :c])


@pytest.mark.parametrize("system, values, ic, nx", [(0, [10.0, 28.0, 8 / 3], [1.0, 1.0, 1.0], 3),
                                                    (1, [0.2, 0.2, 5.7], [1.0, 1.0, 1.0], 3),
                                                    (2, [35.0, 3.0, 28.0], [-10.0, 0.0, 37.0], 3)])
def test_spectrum_block_loop_matches_legacy_gram_schmidt(leg, oracle, system, values, ic, nx):
    tMax, NT, h, eps, trans_t = 20.0, 0.1, 0.01, 1e-8, 5.0
    ranges, mut = [values[0], values[0]], [0]  # a 1-D grid of one point: the given parameters
    ours = oracle.lyapunov_spectrum(system, 1, 0, tMax, NT, 1, h, eps, ic, ranges, mut, trans_t, values)
    ntp, trans = int(NT / h), int(trans_t / h)
    blocks = int(tMax / h) // ntp + 2  # the LLE map's calcBlocks + 1
    legacy = leg.ls_replay(system, ic, values, h, trans, ntp, blocks, eps, tMax, np.eye(nx))
    assert np.array_equal(np.asarray(ours).ravel(), legacy)
