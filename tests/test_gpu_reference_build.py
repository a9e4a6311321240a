"""GPU parity against the reference's own GPU build: its unchanged sources
compiled for sm_103a by oracle/build_ref_gpu.py (with the engine's Lorenz /
Rossler RK4 plug-ins as systems.cuh), run through its own host entry points
by oracle/ref_gpu_main.cu. The build exists only where the reference sources
were staged; without it these tests skip.

Findings they pin: the reference's stock build contracts start + n*scale in
getValueByIdx into one FMA (nvcc's default), so the engine reproduces its
1-D bifurcation CSV byte for byte with CHAOS_TUNE_GRID_FMA = 1, and with the
default (the source as written, as the host build of the reference computes)
differs exactly on the grid points where that contraction changes the value.
The reference's LLE starts its twin from the float-rounded state;
CHAOS_TUNE_LLE_TWIN = 1 reproduces that start up to its cuRAND direction, and
CHAOS_TUNE_LLE_TWIN = 2 draws that direction as the reference does."""
import subprocess
from fractions import Fraction
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent
REF_BIF = ROOT / "oracle" / "_ref" / "ref_gpu_bif1d"
REF_LLE = ROOT / "oracle" / "_ref" / "ref_gpu_lle2d"
BIF = dict(ic=[0.1, 0.1, 0.1], ranges=[20.0, 200.0], values=[10.0, 28.0, 8 / 3])  # as in ref_gpu_main.cu


def _need(p: Path):
    if not p.exists():
        pytest.skip("the reference's GPU build is not present here (its sources were not staged)")


def _rows(path):
    d = {}
    for ln in Path(path).read_text().splitlines()[1:]:
        d.setdefault(ln.split(", ")[0], []).append(ln)
    return d


def _engine_bif_csv(engine, path, nPts, tMax, fused):
    engine.set_system("lorenz")
    engine.set_precision("fp64")
    engine.set_tuning(engine.TUNE_GRID_FMA, fused)
    try:
        engine.bifurcation1D(tMax, nPts, 0.01, 3, BIF["ic"], BIF["ranges"], [1], 0, 1e4, 100.0, BIF["values"], 3, 1,
                             str(path))
    finally:
        engine.set_tuning(engine.TUNE_GRID_FMA, 0)


def test_bif1d_byte_identical_to_reference_gpu_build(engine, tmp_path):
    _need(REF_BIF)
    ref, eng = tmp_path / "ref.csv", tmp_path / "eng.csv"
    subprocess.run([str(REF_BIF), str(ref), "1000", "100"], check=True, capture_output=True, timeout=600)
    _engine_bif_csv(engine, eng, 1000, 100.0, 1)
    assert ref.read_bytes() == eng.read_bytes()


def test_bif1d_as_written_differs_only_at_contracted_grid_values(engine, tmp_path):
    _need(REF_BIF)
    n = 1000
    ref, eng = tmp_path / "ref.csv", tmp_path / "eng.csv"
    subprocess.run([str(REF_BIF), str(ref), str(n), "100"], check=True, capture_output=True, timeout=600)
    _engine_bif_csv(engine, eng, n, 100.0, 0)
    lo, hi = BIF["ranges"]
    scale = (hi - lo) / (n - 1)
    fused = {k for k in range(n) if lo + k * scale != float(Fraction(lo) + Fraction(k) * Fraction(scale))}
    r, e = _rows(ref), _rows(eng)
    keys = list(r)
    assert len(keys) == n and list(e) == keys  # the printed parameter is the host's, unfused, in both
    differing = {k for k, key in enumerate(keys) if r[key] != e[key]}
    assert differing <= fused
    assert len(fused) > 0


def test_lle_reference_twin_start_agrees_with_reference_gpu_build(engine, tmp_path):
    _need(REF_LLE)
    n, tmax = 128, 500.0
    ref_csv, eng_csv = tmp_path / "ref.csv", tmp_path / "eng.csv"
    subprocess.run([str(REF_LLE), str(ref_csv), str(n), str(tmax)], check=True, capture_output=True, timeout=600)

    def values(path):
        t = Path(path).read_text().splitlines()
        return np.array([float(v) for v in ", ".join(t[2:]).split(", ") if v.strip()])

    ref = values(ref_csv)
    engine.set_system("rossler")
    engine.set_precision("fp64")
    within = {}
    for twin in (0, 1, 2):
        engine.set_tuning(engine.TUNE_LLE_TWIN, twin)
        try:
            engine.LLE2D(tmax, 0.1, n, 0.01, 1e-8, [1.0, 1.0, 1.0], 3, [0.1, 0.4, 2.0, 10.0], [0, 2], 0, 0.0, 50.0,
                         [0.2, 0.2, 5.7], 3, str(eng_csv))
        finally:
            engine.set_tuning(engine.TUNE_LLE_TWIN, 0)
        d = np.abs(values(eng_csv) - ref)
        regular = ref < 0.01
        within[twin] = (np.mean(d <= 1e-3), np.mean(d[regular] <= 1e-3))
    # measured on GB300: twin 1 -> 82.6 % of all points and 97.4 % of the regular ones within 1e-3
    assert within[1][0] >= 0.80 and within[1][1] >= 0.95
    assert within[1][0] > within[0][0]
    # twin 2 draws the reference's own cuRAND start (bit for bit: the states test below). The points it
    # still misses are those where the reference's host linspace, contracted into an FMA by the host
    # compiler on this aarch64 machine, gives parameters an ulp off the engine's start + i*step.
    # Measured on GB300: 84.8 % of all points and 99.87 % of the regular ones within 1e-3.
    assert within[2][0] > within[1][0] and within[2][1] >= 0.995, within


def test_lle_twin_start_and_fused_linspace_reproduce_reference_gpu_build(engine, tmp_path):
    """With the reference's own twin start (CHAOS_TUNE_LLE_TWIN 2) and its
    host linspace as this machine's host compiler builds it (contracted into
    an FMA on aarch64: CHAOS_TUNE_GRID_FMA 1), the engine's FP64 map agrees
    with the reference's own GPU build within 1e-3 on >= 99.9 % of the points
    (only the per-block log differs: FP32 __logf there), and its map equals
    the map from the reference's dumped starting states bit for bit."""
    import platform

    _need(REF_LLE)
    _need(REF_STATES)
    if platform.machine() not in ("aarch64", "arm64"):
        pytest.skip("the reference's host linspace is contracted by the aarch64 host compiler only")
    n, tmax = 128, 500.0
    ref_csv, eng_csv = tmp_path / "ref.csv", tmp_path / "eng.csv"
    subprocess.run([str(REF_LLE), str(ref_csv), str(n), str(tmax)], check=True, capture_output=True, timeout=600)
    semi, ref_states = _ref_states(tmp_path, n, tmax)
    engine.set_system("rossler")
    engine.set_precision("fp64")
    engine.set_tuning(engine.TUNE_LLE_TWIN, 2)
    engine.set_tuning(engine.TUNE_GRID_FMA, 1)
    try:
        engine.LLE2D(tmax, 0.1, n, 0.01, 1e-8, [1.0, 1.0, 1.0], 3, [0.1, 0.4, 2.0, 10.0], [0, 2], 0, 0.0, 50.0,
                     [0.2, 0.2, 5.7], 3, str(eng_csv))
        own = engine.lle2d("rossler", tmax, 0.1, n, 0.01, 1e-8, [1.0, 1.0, 1.0], [0.1, 0.4, 2.0, 10.0], [0, 2],
                           50.0, [0.2, 0.2, 5.7])
    finally:
        engine.set_tuning(engine.TUNE_LLE_TWIN, 0)
        engine.set_tuning(engine.TUNE_GRID_FMA, 0)

    def values(path):
        rows = Path(path).read_text().splitlines()
        return np.array([float(v) for v in ", ".join(rows[2:]).split(", ") if v.strip()])

    d = np.abs(values(eng_csv) - values(ref_csv))
    assert np.mean(d <= 1e-3) >= 0.999, np.mean(d <= 1e-3)
    l64 = engine.lle_from_states("rossler", semi, tmax, 0.1, 0.01, 1e-8, precision=engine.FP64)
    assert np.array_equal(own.reshape(n, n).T.ravel(), l64, equal_nan=True)


REF_STATES = ROOT / "oracle" / "_ref" / "ref_gpu_lle_states"


def _ref_states(tmp_path, n, tmax):
    """The reference's semi_result rows (orbit after its transient, parameters,
    its cuRAND twin start) and its map from them, indexed ia * n + ib."""
    out = tmp_path / "states.bin"
    subprocess.run([str(REF_STATES), str(out), str(n), str(tmax)], check=True, capture_output=True, timeout=600)
    raw = out.read_bytes()
    nP, W = (int(v) for v in np.frombuffer(raw[:8], np.int32))
    body = np.frombuffer(raw[8:], np.float64)
    return body[: nP * nP * W].reshape(nP * nP, W), body[nP * nP * W:]


def test_lle_on_reference_twin_starts_matches_reference_gpu_build(engine, tmp_path):
    """Parity on identical inputs. The reference starts each point's twin from
    a cuRAND draw rounded through FP32 (LLE/src/LLECUDA.cu:88-101); handed
    those starting states (its own semi_result rows), the engine's FP64
    Benettin stage reproduces the reference's map within 1e-3 on >= 99.9 %
    of a 128^2 map of the benchmark's Rossler ranges (only the per-block log
    differs: the reference takes it in FP32, __logf). The float-float stage
    on the same states keeps every regular point within 1e-3. The engine's
    own FP64 transient from the reference's parameters lands on the
    reference's post-transient orbit bit for bit."""
    _need(REF_STATES)
    n, tmax = 128, 500.0
    semi, ref = _ref_states(tmp_path, n, tmax)
    assert semi.shape == (n * n, 9)
    fin = np.isfinite(ref)
    l64 = engine.lle_from_states("rossler", semi, tmax, 0.1, 0.01, 1e-8, precision=engine.FP64)
    d64 = np.abs(l64 - ref)[fin & np.isfinite(l64)]
    assert np.mean(d64 <= 1e-3) >= 0.999, np.mean(d64 <= 1e-3)
    assert np.median(d64) < 1e-5
    lff = engine.lle_from_states("rossler", semi, tmax, 0.1, 0.01, 1e-8, precision=engine.FF32)
    ok = fin & np.isfinite(lff)
    reg = ok & (ref < 0.005)
    assert np.mean(np.abs(lff - ref)[reg] <= 1e-3) >= 0.999
    # CHAOS_TUNE_LLE_TWIN 2 draws the reference's own cuRAND start: where the engine's swept parameters
    # equal the reference's (its host linspace may be contracted into an FMA), the engine's map from its
    # own start equals its map from the reference's starting states, point for point
    ia, ib = np.divmod(np.arange(n * n), n)  # reference row ia * n + ib
    pa = 0.1 + ia * ((0.4 - 0.1) / (n - 1))
    pc = 2.0 + ib * ((10.0 - 2.0) / (n - 1))
    same = (semi[:, 3] == pa) & (semi[:, 5] == pc)
    assert same.mean() > 0.5
    engine.set_tuning(engine.TUNE_LLE_TWIN, 2)
    try:
        own = engine.lle2d("rossler", tmax, 0.1, n, 0.01, 1e-8, [1.0, 1.0, 1.0], [0.1, 0.4, 2.0, 10.0], [0, 2],
                           50.0, [0.2, 0.2, 5.7])
    finally:
        engine.set_tuning(engine.TUNE_LLE_TWIN, 0)
    own_rows = own.reshape(n, n).T.ravel()  # the engine's point (ia, ib) sits at ib * n + ia
    assert np.array_equal(own_rows[same], l64[same], equal_nan=True)
    # the transient: 5,000 FP64 steps from (1, 1, 1) with the reference's parameters
    rows = np.random.default_rng(5).choice(n * n, 256, replace=False)
    t = engine.trajectory("rossler", np.tile([1.0, 1.0, 1.0], (256, 1)), semi[rows, 3:6], 0.01, 5000,
                          precision=engine.FP64)
    assert np.array_equal(t[:, -1, :], semi[rows, 0:3])


REF_BASINS = ROOT / "oracle" / "_ref" / "ref_gpu_basins"


def _matrix_cells(path):
    body = Path(path).read_text().split("\n", 2)[2]
    return [c for c in body.replace("\n", "").split(", ") if c != ""]


def _matched_agreement(a, b, fixed=(0,)):
    """Share of points whose labels agree after the best one-to-one matching of
    cluster ids (the reference numbers its clusters in a racy order)."""
    from scipy.optimize import linear_sum_assignment

    a, b = np.asarray(a), np.asarray(b)
    same_fixed = sum(int(np.sum((a == f) & (b == f))) for f in fixed)
    m = ~np.isin(a, fixed) & ~np.isin(b, fixed)
    ua, ia = np.unique(a[m], return_inverse=True)
    ub, ib = np.unique(b[m], return_inverse=True)
    M = np.zeros((ua.size, ub.size), np.int64)
    np.add.at(M, (ia, ib), 1)
    r, c = linear_sum_assignment(-M)
    return (same_fixed + int(M[r, c].sum())) / a.size


def test_basins_agree_with_reference_gpu_build(engine, tmp_path):
    """The basins map (Lorenz rho 24, the basins workload's ranges, 64^2)
    through the engine's Basins::basinsOfAttraction_2 against the reference's
    own GPU build: with CHAOS_TUNE_GRID_FMA = 1 (the contraction the stock
    build applies to the grid values) the flag file is identical, the feature
    files agree on at least 99.9 % of the cells and the basin labels on at
    least 99.9 % of the points after matching cluster ids."""
    pytest.importorskip("scipy")
    _need(REF_BASINS)
    n = 64
    ref = tmp_path / "ref"
    subprocess.run([str(REF_BASINS), str(ref), str(n)], check=True, capture_output=True, timeout=600)
    engine.set_system("lorenz")
    engine.set_precision("fp64")
    engine.set_tuning(engine.TUNE_GRID_FMA, 1)
    try:
        engine.Basins.basinsOfAttraction_2(50.0, n, 0.01, 3, [0.0, 0.0, 27.0], [-30.0, 30.0, -30.0, 30.0], [0, 1], 0,
                                           1e8, 200.0, [10.0, 24.0, 8 / 3], 3, 1, 0.05, str(tmp_path / "eng"))
    finally:
        engine.set_tuning(engine.TUNE_GRID_FMA, 0)
    assert (tmp_path / "ref_3.csv").read_text() == (tmp_path / "eng_3.csv").read_text()
    for k in (1, 2):
        r, e = _matrix_cells(tmp_path / f"ref_{k}.csv"), _matrix_cells(tmp_path / f"eng_{k}.csv")
        assert len(r) == len(e) == n * n
        assert np.mean([x == y for x, y in zip(r, e)]) >= 0.999
    lr = [int(c) for c in _matrix_cells(ref)]
    le = [int(c) for c in _matrix_cells(tmp_path / "eng")]
    assert _matched_agreement(le, lr) >= 0.999
