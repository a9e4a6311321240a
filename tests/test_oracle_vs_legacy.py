"""The oracle's restatements of the legacy library's analyses (the engine's
old_library::* and grid modes, chaos_lyapunov_spectrum) against the legacy
library's own functions, extracted unchanged from debri/cudaLibrary.cu and
compiled for the host by oracle/build_ref.py. Runs where that build exists.

Pinned bit for bit: the log-scale axis (getValueByIdxLog, raised to 10^x as
the engine's CHAOS_GRID_LOG* tables are), the linear axis (getValueByIdx), the
legacy peakFinder against the current library's (the engine follows the
latter), the spectrum's per-block classical Gram-Schmidt and renormalisation
(projectionOperator, gramSchmidtProcess, the block loop of LSKernelCUDA
replayed around them) against orc_lyapunov_spectrum with the same twin start
and block count, and the legacy bifurcation1DIC / bifurcation2DIC,
basinsOfAttraction and bifurcation1DForH kernels themselves (run one host
thread per point; their hard-wired system is the sin3 plug-in's arithmetic)
against the oracle's sweeps with the legacy loop (GRID_LEGACY_LOOP) and its
basins features, and the legacy LLE kernels (LLEKernelCUDA with its cuRAND
uniforms supplied, LLEKernelICCUDA with its sinf twin) against
orc_lle_sweep_legacy, and the legacy spectrum kernel LSKernelCUDA against
orc_lyapunov_spectrum_legacy."""
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


SIN3 = [0.5, 0.1, 1.4, 15.552, 2.0]  # the hard-wired legacy system's parameters; a[1] is the damping b


def _sin3(b):
    return [SIN3[0], b] + SIN3[2:]


# b = 0.1 chaotic (maxValue 4 leaves most orbits unbounded), 0.5 every orbit ends at a fixed point,
# 1.1 fixed points beside decaying orbits
@pytest.mark.parametrize("b", [0.1, 0.5, 1.1])
@pytest.mark.parametrize("pre", [1, 3])
@pytest.mark.parametrize("dim", [1, 2])
def test_ic_bifurcation_matches_legacy_kernels(leg, oracle, b, pre, dim):
    """bifurcation1DIC / bifurcation2DIC: calculateDiscreteModelICCUDA,
    peakFinderCUDA and dbscanCUDA against the oracle's sweep over initial
    conditions with the legacy loop, on sin3: counts (with the legacy's -1 /
    0), every kept peak, the intervals and the labels."""
    n, rng, mut = (40, [-6.0, 6.0], [0]) if dim == 1 else (14, [-6.0, 6.0, -6.0, 6.0], [0, 1])
    args = (30.0, n, 0.01)
    L = leg.ic_bifurcation(dim, n, 30.0, 0.01, 50.0, pre, [0.0, 0.0, 0.0], _sin3(b), rng, mut, 0, 4.0, eps=0.05)
    o = oracle.bifurcation_sweep(5, dim, oracle.GRID_STATE | oracle.GRID_LEGACY_LOOP, *args, [0.0, 0.0, 0.0], rng,
                                 mut, 0, 4.0, 50.0, _sin3(b), preScaller=pre, eps=0.05)
    assert np.array_equal(L["counts"], o["counts"])
    for k, c in enumerate(L["counts"]):
        assert np.array_equal(L["peaks"][k, :max(c, 0)], o["peaks"][k, :max(c, 0)]), k
        if dim == 2:
            assert np.array_equal(L["intervals"][k, :max(c, 0)], o["intervals"][k, :max(c, 0)]), k
    if dim == 2:
        assert np.array_equal(L["labels"], o["labels"])


def test_legacy_loop_differs_from_current_loop(leg, oracle):
    """Why the legacy analyses need their own loop: where every orbit ends at
    a fixed point, the legacy kernels report it (-1) after the recorded part,
    the current library's loop stops at the transient and reports 0; with
    preScaller 3 the legacy samples every third step, the current loop every
    step."""
    rng, mut = [-6.0, 6.0, -6.0, 6.0], [0, 1]
    L = leg.ic_bifurcation(2, 10, 30.0, 0.01, 50.0, 1, [0.0, 0.0, 0.0], _sin3(0.5), rng, mut, 0, 4.0, eps=0.05)
    cur = oracle.bifurcation_sweep(5, 2, oracle.GRID_STATE, 30.0, 10, 0.01, [0.0, 0.0, 0.0], rng, mut, 0, 4.0, 50.0,
                                   _sin3(0.5), eps=0.05)
    assert (L["labels"] == -1).all() and (cur["labels"] == 0).all()
    L = leg.ic_bifurcation(1, 40, 30.0, 0.01, 50.0, 3, [0.0, 0.0, 0.0], _sin3(0.2), [-6.0, 6.0], [0], 0, 1e8)
    cur = oracle.bifurcation_sweep(5, 1, oracle.GRID_STATE, 30.0, 40, 0.01, [0.0, 0.0, 0.0], [-6.0, 6.0], [0], 0,
                                   1e8, 50.0, _sin3(0.2), preScaller=3)
    assert not np.array_equal(L["counts"], cur["counts"])


@pytest.mark.parametrize("b", [0.1, 0.2, 0.5, 1.1])
@pytest.mark.parametrize("pre", [1, 3])
@pytest.mark.parametrize("maxValue", [1e8, 4.0])
def test_basins_v1_matches_legacy_kernels(leg, oracle, b, pre, maxValue):
    """basinsOfAttraction (the legacy basins map): calculateDiscreteModelICCUDA
    and avgPeakFinderCUDA against the oracle's basins features (the current
    library's basins loop, which the engine's basins map runs): flags, mean
    peaks and mean intervals bit for bit."""
    rng, mut = [-6.0, 6.0, -6.0, 6.0], [0, 1]
    L = leg.basins_v1(14, 30.0, 0.01, 50.0, pre, [0.0, 0.0, 0.0], _sin3(b), rng, mut, 0, maxValue)
    o = oracle.basins_features(5, 30.0, 14, 0.01, [0.0, 0.0, 0.0], rng, mut, 0, maxValue, 50.0, _sin3(b),
                               preScaller=pre)
    assert np.array_equal(L["flags"], o["flags"])
    assert np.array_equal(L["avgPeaks"], o["avg_peaks"])
    assert np.array_equal(L["avgIntervals"], o["avg_intervals"])


@pytest.mark.parametrize("pre", [1, 2, 3])
@pytest.mark.parametrize("rng", [[0.005, 0.02], [0.01, 0.05], [0.02, 0.004]])
def test_step_sweep_matches_legacy_kernels(leg, oracle, pre, rng):
    """bifurcation1DForH: calculateDiscreteModelCUDA_H and peakFinderCUDA_H
    (the step on the powf-rounded log scale) against the oracle's step-size
    sweep with the legacy loop: kept-peak counts and every kept peak."""
    V = _sin3(0.2)
    L = leg.step_sweep(24, 30.0, 20.0, pre, [0.3, 0.1, 0.0], V, rng, 0, 1e8)
    o = oracle.bifurcation_sweep(5, 1, oracle.GRID_LOG0 | oracle.GRID_LOG_F32 | oracle.GRID_LEGACY_LOOP, 30.0, 24,
                                 0.0, [0.3, 0.1, 0.0], rng, [oracle.MUT_STEP], 0, 1e8, 20.0, V, preScaller=pre)
    assert np.array_equal(L["counts"], np.maximum(o["counts"], 0))
    for k, c in enumerate(L["counts"]):
        assert np.array_equal(L["peaks"][k, :c], o["peaks"][k, :c]), k


@pytest.mark.parametrize("maxValue", [0.0, 3.0])
def test_lle1d_matches_legacy_kernel(leg, oracle, maxValue):
    """LLE1D: LLEKernelCUDA, its cuRAND uniforms supplied (seed p + k for
    component k of point p, so neighbouring points share draws), against
    orc_lle_sweep_legacy given the same raw draws u[p + k] - 0.5, over the sin3
    damping b; maxValue 3 stops runs of steps early."""
    n = 30
    u = np.random.default_rng(5).random(n + 2).astype(np.float32)
    V = _sin3(0.2)
    L = leg.lle(0, 1, n, 50.0, 0.5, 0.01, 1e-6, 20.0, [0.3, 0.1, 0.0], V, [0.1, 0.4], [1], maxValue, uniforms=u)
    draws = np.array([[float(u[p + k]) - 0.5 for k in range(3)] for p in range(n)])
    o = oracle.lle_sweep_legacy(5, 1, 0, 50.0, 0.5, n, 0.01, 1e-6, [0.3, 0.1, 0.0], [0.1, 0.4], [1], maxValue, 20.0,
                                V, draws=draws)
    assert np.array_equal(L, o)


@pytest.mark.parametrize("dim", [1, 2])
@pytest.mark.parametrize("maxValue", [0.0, 3.0])
def test_lle_ic_matches_legacy_kernel(leg, oracle, dim, maxValue):
    """LLE1DIC / LLE2DIC: LLEKernelICCUDA (twin 0.5 sinf(p (k p + 1) + 1),
    normalised) against orc_lle_sweep_legacy over initial conditions."""
    n, rng, mut = (30, [-3.0, 3.0], [0]) if dim == 1 else (8, [-3.0, 3.0, -3.0, 3.0], [0, 2])
    V = _sin3(0.2)
    L = leg.lle(1, dim, n, 50.0, 0.5, 0.01, 1e-6, 20.0, [0.3, 0.1, 0.0], V, rng, mut, maxValue)
    o = oracle.lle_sweep_legacy(5, dim, oracle.GRID_STATE, 50.0, 0.5, n, 0.01, 1e-6, [0.3, 0.1, 0.0], rng, mut,
                                maxValue, 20.0, V)
    assert np.array_equal(L, o)


@pytest.mark.parametrize("dim", [1, 2])
@pytest.mark.parametrize("maxValue", [0.0, 3.0])
def test_ls_matches_legacy_kernel(leg, oracle, dim, maxValue):
    """LS1D / LS2D: LSKernelCUDA (twins from its sinf draws, orthonormalised
    after the transient, classical Gram-Schmidt every block) against
    orc_lyapunov_spectrum_legacy, every exponent bit for bit."""
    n, rng, mut = (20, [0.1, 0.4], [1]) if dim == 1 else (6, [0.1, 0.4, 0.3, 0.7], [1, 0])
    V = _sin3(0.2)
    L = leg.ls(dim, n, 50.0, 0.5, 0.01, 1e-6, 20.0, [0.3, 0.1, 0.0], V, rng, mut, maxValue)
    o = oracle.lyapunov_spectrum_legacy(5, dim, 0, 50.0, 0.5, n, 0.01, 1e-6, [0.3, 0.1, 0.0], rng, mut, maxValue,
                                        20.0, V)
    assert np.array_equal(L, o)


@pytest.mark.parametrize("seed", range(8))
def test_legacy_kernels_random_configurations(leg, oracle, seed):
    """Random configurations of the legacy system (damping, preScaller 1-4,
    bound, recorded component, ranges, horizons): every legacy kernel above
    against its oracle restatement, bit for bit."""
    rng = np.random.default_rng(100 + seed)
    b = float(rng.uniform(0.05, 1.2))
    V = _sin3(b)
    pre = int(rng.integers(1, 5))
    mx = float(rng.choice([0.0, 2.5, 4.0, 1e8]))
    wv = int(rng.integers(0, 3))
    lo = float(rng.uniform(-6.0, -1.0))
    hi = float(rng.uniform(1.0, 6.0))
    tmax, trans = float(rng.choice([10.0, 20.0, 30.0])), float(rng.choice([5.0, 20.0, 50.0]))
    ic = [float(v) for v in rng.uniform(-1.0, 1.0, 3)]
    # bifurcation over initial conditions, 1-D and 2-D
    for dim in (1, 2):
        n, rg, mut = (24, [lo, hi], [int(rng.integers(0, 3))]) if dim == 1 else (8, [lo, hi, lo, hi], [0, 2])
        L = leg.ic_bifurcation(dim, n, tmax, 0.01, trans, pre, ic, V, rg, mut, wv, mx, eps=0.05)
        o = oracle.bifurcation_sweep(5, dim, oracle.GRID_STATE | oracle.GRID_LEGACY_LOOP, tmax, n, 0.01, ic, rg, mut,
                                     wv, mx, trans, V, preScaller=pre, eps=0.05)
        assert np.array_equal(L["counts"], o["counts"])
        for k, c in enumerate(L["counts"]):
            assert np.array_equal(L["peaks"][k, :max(c, 0)], o["peaks"][k, :max(c, 0)])
        if dim == 2:
            assert np.array_equal(L["labels"], o["labels"])
    # the basins map
    L = leg.basins_v1(8, tmax, 0.01, trans, pre, ic, V, [lo, hi, lo, hi], [0, 1], wv, mx)
    o = oracle.basins_features(5, tmax, 8, 0.01, ic, [lo, hi, lo, hi], [0, 1], wv, mx, trans, V, preScaller=pre)
    assert np.array_equal(L["flags"], o["flags"])
    assert np.array_equal(L["avgPeaks"], o["avg_peaks"]) and np.array_equal(L["avgIntervals"], o["avg_intervals"])
    # the step-size sweep (a range whose rounded steps stay within the legacy's blocks)
    hr = [0.008, 0.02] if seed % 2 else [0.02, 0.008]
    L = leg.step_sweep(16, tmax, trans, pre, ic, V, hr, wv, mx)
    o = oracle.bifurcation_sweep(5, 1, oracle.GRID_LOG0 | oracle.GRID_LOG_F32 | oracle.GRID_LEGACY_LOOP, tmax, 16,
                                 0.0, ic, hr, [oracle.MUT_STEP], wv, mx, trans, V, preScaller=pre)
    assert np.array_equal(L["counts"], np.maximum(o["counts"], 0))
    for k, c in enumerate(L["counts"]):
        assert np.array_equal(L["peaks"][k, :c], o["peaks"][k, :c])
    # the LLE kernels and the spectrum (NT 0.2, the bound on component 0)
    mxl = float(rng.choice([0.0, 3.0]))
    u = rng.random(30).astype(np.float32)
    L = leg.lle(0, 1, 12, tmax, 0.2, 0.01, 1e-6, trans, ic, V, [0.1, 0.6], [1], mxl, uniforms=u)
    draws = np.array([[float(u[p + k]) - 0.5 for k in range(3)] for p in range(12)])
    o = oracle.lle_sweep_legacy(5, 1, 0, tmax, 0.2, 12, 0.01, 1e-6, ic, [0.1, 0.6], [1], mxl, trans, V, draws=draws)
    assert np.array_equal(L, o)
    L = leg.lle(1, 2, 5, tmax, 0.2, 0.01, 1e-6, trans, ic, V, [lo, hi, lo, hi], [0, 1], mxl)
    o = oracle.lle_sweep_legacy(5, 2, oracle.GRID_STATE, tmax, 0.2, 5, 0.01, 1e-6, ic, [lo, hi, lo, hi], [0, 1], mxl,
                                trans, V)
    assert np.array_equal(L, o)
    L = leg.ls(1, 6, tmax, 0.2, 0.01, 1e-6, trans, ic, V, [0.1, 0.6], [1], mxl)
    o = oracle.lyapunov_spectrum_legacy(5, 1, 0, tmax, 0.2, 6, 0.01, 1e-6, ic, [0.1, 0.6], [1], mxl, trans, V)
    assert np.array_equal(L, o)
