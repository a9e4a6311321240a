"""GPU parity of the grid modes (CHAOS_GRID_*): bifurcation and LLE sweeps
over initial conditions (the legacy *IC analyses), log-scale axes (the legacy
getValueByIdxLog, debri/cudaLibrary.cu:1191-1196), the step-size sweep (the
legacy bifurcation1DForH, debri/hostLibrary.cu:1005-1240), and the legacy
analyses' file formats, against the CPU oracle. FP64 results are compared bit
for bit."""
import numpy as np
import pytest

from test_gpu_parity import _csv_matrix, _g

pytestmark = pytest.mark.gpu

LORENZ = [10.0, 28.0, 8 / 3]
IC = [0.1, 0.1, 0.1]


def _assert_bif_equal(g, o, cap):
    assert np.array_equal(g["counts"], o["counts"])
    assert np.array_equal(g["flags"], o["flags"])
    for k, c in enumerate(g["counts"]):
        m = min(max(int(c), 0), cap)
        assert np.array_equal(g["peaks"][k, :m], o["peaks"][k, :m]), k
        assert np.array_equal(g["intervals"][k, :m], o["intervals"][k, :m]), k
        if c == -1:
            assert g["first"][k] == o["first"][k]


@pytest.mark.parametrize("mode, rng, mut", [
    ("state", [-8.0, 8.0], [2]),
    ("log", [20.0, 200.0], [1]),
    ("log_f32", [20.0, 200.0], [1]),
    ("state_log", [0.5, 30.0], [2]),
])
def test_bifurcation_1d_modes_fp64_vs_oracle(engine, oracle, mode, rng, mut):
    gm = {"state": engine.GRID_STATE, "log": engine.GRID_LOG0, "log_f32": engine.GRID_LOG0 | engine.GRID_LOG_F32,
          "state_log": engine.GRID_STATE | engine.GRID_LOG0}[mode]
    n, cap = 64, 400
    kw = dict(tMax=10.0, nPts=n, h=0.01, initialConditions=IC, ranges=rng, indicesOfMutVars=mut, writableVar=0,
              maxValue=1e4, transientTime=5.0, values=LORENZ)
    g = engine.bifurcation_sweep("lorenz", 1, gm, peakCapacity=cap, **kw)
    o = oracle.bifurcation_sweep(0, 1, gm, 10.0, n, 0.01, IC, rng, mut, 0, 1e4, 5.0, LORENZ, cap=cap)
    _assert_bif_equal(g, o, cap)


@pytest.mark.parametrize("mode", ["state", "log1"])
def test_bifurcation_2d_modes_fp64_vs_oracle(engine, oracle, mode):
    """2-D sweeps with the per-point clustering: initial conditions (the
    legacy bifurcation2DIC) and a log-scale second axis."""
    if mode == "state":
        gm, rng, mut = engine.GRID_STATE, [-10.0, 10.0, -10.0, 10.0], [0, 1]
    else:
        gm, rng, mut = engine.GRID_LOG1, [20.0, 200.0, 1.0, 30.0], [1, 0]
    n = 24
    g = engine.bifurcation_sweep("lorenz", 2, gm, tMax=6.0, nPts=n, h=0.01, initialConditions=IC, ranges=rng,
                                 indicesOfMutVars=mut, writableVar=0, maxValue=1e4, transientTime=4.0, values=LORENZ,
                                 eps=0.05)
    o = oracle.bifurcation_sweep(0, 2, gm, 6.0, n, 0.01, IC, rng, mut, 0, 1e4, 4.0, LORENZ, eps=0.05)
    assert np.array_equal(g["counts"], o["counts"])
    assert np.array_equal(g["labels"], o["labels"])


@pytest.mark.parametrize("mode", ["log_f32", "linear"])
def test_step_sweep_fp64_vs_oracle(engine, oracle, mode):
    """Every point integrates with its own step h_k, (int)(transientTime/h_k)
    transient steps and (int)(tMax/h_k) samples; intervals in units h_k."""
    gm = engine.GRID_LOG0 | engine.GRID_LOG_F32 if mode == "log_f32" else 0
    n, cap, rng = 40, 1200, [0.001, 0.03]
    kw = dict(tMax=20.0, nPts=n, h=0.0, initialConditions=[1.0, 1.0, 1.0], ranges=rng,
              indicesOfMutVars=[engine.MUT_STEP], writableVar=0, maxValue=1e4, transientTime=10.0,
              values=[0.2, 0.2, 5.7])
    g = engine.bifurcation_sweep("rossler", 1, gm, peakCapacity=cap, **kw)
    o = oracle.bifurcation_sweep(1, 1, gm, 20.0, n, 0.0, [1.0, 1.0, 1.0], rng, [-1], 0, 1e4, 10.0,
                                 [0.2, 0.2, 5.7], cap=cap)
    _assert_bif_equal(g, o, cap)
    assert np.all(g["counts"] > 0)


def test_step_sweep_fp32_runs_single_point_kernels(engine):
    """The FP32 step sweep (one point per thread: a pair would share one step)
    keeps the FP64 sweep's flags and nearly its peak counts."""
    kw = dict(tMax=40.0, nPts=2048, h=0.0, initialConditions=[1.0, 1.0, 1.0], ranges=[0.002, 0.02],
              indicesOfMutVars=[engine.MUT_STEP], writableVar=0, maxValue=1e4, transientTime=10.0,
              values=[0.2, 0.2, 5.7], peakCapacity=64)
    old = engine.get_tuning(engine.TUNE_SWEEP_PAIRS)
    try:
        engine.set_tuning(engine.TUNE_SWEEP_PAIRS, 2)  # pairs forced on: the step sweep must still run singly
        g32 = engine.bifurcation_sweep("rossler", 1, engine.GRID_LOG0, precision=engine.FP32, **kw)
    finally:
        engine.set_tuning(engine.TUNE_SWEEP_PAIRS, old)
    g64 = engine.bifurcation_sweep("rossler", 1, engine.GRID_LOG0, **kw)
    assert np.array_equal(g32["flags"], g64["flags"])
    assert np.mean(np.abs(g32["counts"] - g64["counts"]) <= 1) > 0.99


def test_log_axis_values_are_the_oracles(engine, oracle):
    """Point k of the engine's log-scale sweep equals the engine's linear
    sweep over [v_k, v_k] with v_k from the oracle's formula: the device uses
    exactly these values."""
    n = 16
    for f32 in (False, True):
        gm = engine.GRID_LOG0 | (engine.GRID_LOG_F32 if f32 else 0)
        vk = oracle.log_axis(20.0, 200.0, n, f32=f32)
        kw = dict(tMax=8.0, h=0.01, initialConditions=IC, indicesOfMutVars=[1], writableVar=0, maxValue=1e4,
                  transientTime=4.0, values=LORENZ, peakCapacity=200)
        g = engine.bifurcation_sweep("lorenz", 1, gm, nPts=n, ranges=[20.0, 200.0], **kw)
        for k in (0, 7, n - 1):
            s = engine.bifurcation1d("lorenz", nPts=2, ranges=[vk[k], vk[k]], **kw)
            assert g["counts"][k] == s["counts"][0]
            c = max(int(s["counts"][0]), 0)
            assert np.array_equal(g["peaks"][k, :c], s["peaks"][0, :c])


def test_step_sweep_constant_range_is_bifurcation1d(engine):
    kw = dict(tMax=10.0, initialConditions=IC, writableVar=0, maxValue=1e4, transientTime=5.0, values=LORENZ,
              peakCapacity=300)
    g = engine.bifurcation_sweep("lorenz", 1, 0, nPts=3, h=0.0, ranges=[0.01, 0.01],
                                 indicesOfMutVars=[engine.MUT_STEP], **kw)
    s = engine.bifurcation1d("lorenz", nPts=3, h=0.01, ranges=[28.0, 28.0], indicesOfMutVars=[1], **kw)
    for k in ("counts", "flags", "peaks", "intervals"):
        assert np.array_equal(g[k], s[k]), k


@pytest.mark.parametrize("dim, mode", [(1, "log"), (2, "log_state")])
def test_lle_sweep_log_axes_fp64_vs_oracle(engine, oracle, dim, mode):
    if mode == "log":
        gm, rng, mut = engine.GRID_LOG0, [10.0, 100.0], [1]
    else:
        gm, rng, mut = engine.GRID_LOG0 | engine.GRID_LOG1 | engine.GRID_STATE, [0.5, 10.0, 0.5, 10.0], [0, 1]
    n = 24 if dim == 1 else 8
    kw = dict(tMax=15.0, NT=0.1, nPts=n, h=0.01, eps=1e-8, initialConditions=[1.0, 1.0, 1.0], ranges=rng,
              indicesOfMutVars=mut, transientTime=5.0, values=LORENZ)
    g = engine.lle_sweep("lorenz", dim, gridMode=gm, **kw)
    o = oracle.lle_sweep(0, dim, gm, 15.0, 0.1, n, 0.01, 1e-8, [1.0, 1.0, 1.0], rng, mut, 5.0, LORENZ)
    assert np.max(np.abs(g - o)) < 1e-12
    g32 = engine.lle_sweep("lorenz", dim, gridMode=gm, precision=engine.FP32, **kw)
    assert np.all(np.isfinite(g32))


@pytest.mark.parametrize("rho, pre, maxValue", [(0.5, 1, 1e4), (0.5, 3, 1e4), (28.0, 3, 17.0), (28.0, 2, 1e4)])
@pytest.mark.parametrize("dim", [1, 2])
def test_bifurcation_legacy_loop_fp64_vs_oracle(engine, oracle, rho, pre, maxValue, dim):
    """The legacy per-point loop (GRID_STATE | GRID_LEGACY_LOOP: the loop of
    the legacy bifurcation1DIC / bifurcation2DIC, whose oracle restatement
    the CPU tests pin to the legacy kernels) bit for bit against the oracle:
    fixed points reported after the recorded part (rho 0.5), preScaller
    sub-steps, the bound tested in the recorded part only (maxValue 17 at rho
    28). Requested in FP32, the legacy loop still runs in FP64."""
    vals = [10.0, rho, 8 / 3]
    n, rng, mut = (48, [-20.0, 20.0], [2]) if dim == 1 else (16, [-20.0, 20.0, -20.0, 20.0], [0, 2])
    gm = engine.GRID_STATE | engine.GRID_LEGACY_LOOP
    kw = dict(tMax=10.0, nPts=n, h=0.01, initialConditions=IC, ranges=rng, indicesOfMutVars=mut, writableVar=0,
              maxValue=maxValue, transientTime=40.0, values=vals, preScaller=pre)
    o = oracle.bifurcation_sweep(0, dim, gm, 10.0, n, 0.01, IC, rng, mut, 0, maxValue, 40.0, vals, preScaller=pre,
                                 eps=0.05, cap=400)
    for prec in (engine.FP64, engine.FP32):
        if dim == 1:
            g = engine.bifurcation_sweep("lorenz", 1, gm, peakCapacity=400, precision=prec, **kw)
            _assert_bif_equal(g, o, 400)
        else:
            g = engine.bifurcation_sweep("lorenz", 2, gm, eps=0.05, precision=prec, **kw)
            assert np.array_equal(g["counts"], o["counts"])
            assert np.array_equal(g["labels"], o["labels"])
    if rho == 0.5:  # every orbit ends at the origin: reported as fixed points
        assert (o["counts"] == -1).all()


def test_step_sweep_legacy_loop_fp64_vs_oracle(engine, oracle):
    """The legacy step-size sweep's loop (bifurcation1DForH) with preScaller
    3, bit for bit against the oracle."""
    gm = engine.GRID_LOG0 | engine.GRID_LOG_F32 | engine.GRID_LEGACY_LOOP
    kw = dict(tMax=10.0, nPts=40, h=0.0, initialConditions=IC, ranges=[0.004, 0.02],
              indicesOfMutVars=[engine.MUT_STEP], writableVar=0, maxValue=1e4, transientTime=5.0, values=LORENZ,
              preScaller=3)
    g = engine.bifurcation_sweep("lorenz", 1, gm, peakCapacity=500, **kw)
    o = oracle.bifurcation_sweep(0, 1, gm, 10.0, 40, 0.0, IC, [0.004, 0.02], [-1], 0, 1e4, 5.0, LORENZ, preScaller=3,
                                 cap=500)
    _assert_bif_equal(g, o, 500)


@pytest.mark.parametrize("state, dim, maxValue", [(False, 1, 0.0), (False, 2, 18.0), (True, 1, 0.0), (True, 2, 18.0)])
def test_lle_legacy_scheme_fp64_vs_oracle(engine, oracle, state, dim, maxValue):
    """The legacy LLE kernels' scheme (chaos_lle_sweep_legacy: LLEKernelCUDA
    on parameter grids, LLEKernelICCUDA on initial conditions; the oracle's
    restatement is pinned to those kernels on the CPU) against the oracle fed
    the twin draws the engine made: within 1e-12 (CUDA's log and glibc's may
    differ in the last bit). The same draws passed in give the same map."""
    n = 40 if dim == 1 else 9
    if state:
        rng, mut = ([-8.0, 8.0], [2]) if dim == 1 else ([-8.0, 8.0, -8.0, 8.0], [0, 2])
    else:
        rng, mut = ([20.0, 60.0], [1]) if dim == 1 else ([20.0, 60.0, 5.0, 15.0], [1, 0])
    kw = dict(tMax=20.0, NT=0.2, nPts=n, h=0.01, eps=1e-7, initialConditions=[1.0, 1.0, 1.0], ranges=rng,
              indicesOfMutVars=mut, transientTime=5.0, values=LORENZ, maxValue=maxValue, mutateState=state)
    g = engine.lle_sweep_legacy("lorenz", dim, **kw)
    draws = engine.legacy_lle_draws(int(state), n ** dim, 3)
    o = oracle.lle_sweep_legacy(0, dim, oracle.GRID_STATE if state else 0, 20.0, 0.2, n, 0.01, 1e-7,
                                [1.0, 1.0, 1.0], rng, mut, maxValue, 5.0, LORENZ, draws=draws)
    assert np.allclose(g, o, rtol=1e-12, atol=1e-12), np.max(np.abs(g - o))
    assert np.array_equal(engine.lle_sweep_legacy("lorenz", dim, draws=draws, **kw), g)


@pytest.mark.parametrize("dim, maxValue", [(1, 0.0), (2, 18.0)])
def test_spectrum_legacy_scheme_fp64_vs_oracle(engine, oracle, dim, maxValue):
    """The legacy spectrum kernel's scheme (chaos_lyapunov_spectrum_legacy;
    the oracle's restatement is pinned to LSKernelCUDA on the CPU) against the
    oracle fed the engine's twin draws: every exponent within 1e-12."""
    n, rng, mut = (24, [20.0, 60.0], [1]) if dim == 1 else (6, [20.0, 60.0, 5.0, 15.0], [1, 0])
    kw = dict(tMax=20.0, NT=0.2, nPts=n, h=0.01, eps=1e-7, initialConditions=[1.0, 1.0, 1.0], ranges=rng,
              indicesOfMutVars=mut, transientTime=5.0, values=LORENZ, maxValue=maxValue)
    g = engine.lyapunov_spectrum_legacy("lorenz", dim, **kw)
    draws = engine.legacy_lle_draws(2, n ** dim, 3)
    o = oracle.lyapunov_spectrum_legacy(0, dim, 0, 20.0, 0.2, n, 0.01, 1e-7, [1.0, 1.0, 1.0], rng, mut, maxValue,
                                        5.0, LORENZ, draws=draws)
    assert np.allclose(g, o, rtol=1e-12, atol=1e-12), np.max(np.abs(g - o))
    assert np.array_equal(engine.lyapunov_spectrum_legacy("lorenz", dim, draws=draws, **kw), g)


def test_legacy_lle_draws(engine):
    """The legacy kernels' twin draws: cuRAND seeded p + k (so neighbouring
    points share draws, each a uniform in (0, 1] minus 0.5), and 0.5 sinf(p (k
    p + 1) + 1) within CUDA's sinf error bound of the exact sine."""
    d0 = engine.legacy_lle_draws(0, 200, 3)
    assert np.array_equal(d0[1:, :2], d0[:-1, 1:])
    assert (d0 > -0.5).all() and (d0 <= 0.5).all() and np.unique(d0).size == 202
    d1 = engine.legacy_lle_draws(1, 200, 3)
    p = np.arange(200, dtype=np.uint32)[:, None]
    k = np.arange(3, dtype=np.uint32)[None, :]
    arg = (p * (k * p + np.uint32(1)) + np.uint32(1)).astype(np.int32).astype(np.float32)
    ref = 0.5 * np.sin(arg.astype(np.float64))
    ulp = np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)  # of the halved value, in float
    assert np.all(np.abs(d1 - ref) <= 3 * ulp)  # sinf's 2-ulp bound, plus the rounding of the float result
    d2 = engine.legacy_lle_draws(2, 50, 3)  # the spectrum's rows: [p, twin j, component i]
    p = np.arange(50)[:, None, None]
    j = np.arange(3)[None, :, None]
    i = np.arange(3)[None, None, :]
    arg = ((0.2171828 * (i + 1) * (j + 1) + p) + (0.2171828 + i * j * p)).astype(np.float32)
    ref = np.sin(arg.astype(np.float64)) * 0.5
    ulp = np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)
    assert np.all(np.abs(d2 - ref) <= 3 * ulp)


def test_spectrum_log_axis_fp64_vs_oracle(engine, oracle):
    kw = dict(tMax=10.0, NT=0.1, nPts=12, h=0.01, eps=1e-8, initialConditions=[1.0, 1.0, 1.0], ranges=[10.0, 100.0],
              indicesOfMutVars=[1], transientTime=2.0, values=LORENZ)
    g = engine.lyapunov_spectrum("lorenz", 1, gridMode=engine.GRID_LOG0, **kw)
    o = oracle.lyapunov_spectrum(0, 1, engine.GRID_LOG0, 10.0, 0.1, 12, 0.01, 1e-8, [1.0, 1.0, 1.0],
                                 [10.0, 100.0], [1], 2.0, LORENZ)
    assert np.max(np.abs(g - o)) < 1e-12


def test_legacy_csv_bytes(engine, oracle, tmp_path):
    """old_library's analyses write the legacy files: bifurcation1DIC /
    bifurcation1DForH rows 'value, peak' (precision 12, the step sweep
    labelled with the linear range), bifurcation2DIC's labels matrix,
    LLE1D / LLE1DIC rows (precision 12), LLE2DIC's matrix and LS1D / LS2D."""
    L, old = engine, engine.old_library
    L.set_system("lorenz")
    L.set_precision(L.FP64)
    n = 20
    lin = [-8.0 + k * (16.0 / (n - 1)) for k in range(n)]
    LEG = oracle.GRID_LEGACY_LOOP  # the legacy analyses run the legacy per-point loop
    # bifurcation1DIC (preScaller 2: a sample every second step)
    p = tmp_path / "bic.csv"
    old.bifurcation1DIC(8.0, n, 0.01, 3, IC, [-8.0, 8.0], [2], 0, 1e4, 4.0, LORENZ, 3, 2, p)
    o = oracle.bifurcation_sweep(0, 1, oracle.GRID_STATE | LEG, 8.0, n, 0.01, IC, [-8.0, 8.0], [2], 0, 1e4, 4.0,
                                 LORENZ, preScaller=2)
    expect = "".join("%.12g, %.12g\n" % (lin[k], o["peaks"][k, j]) for k in range(n)
                     for j in range(max(int(o["counts"][k]), 0)))
    assert p.read_text() == expect
    # bifurcation1DForH (log-scale step, FP32-rounded; rows labelled with the linear range)
    p = tmp_path / "bh.csv"
    old.bifurcation1DForH(8.0, n, 3, IC, [0.005, 0.02], 0, 1e4, 4.0, LORENZ, 3, 2, p)
    o = oracle.bifurcation_sweep(0, 1, oracle.GRID_LOG0 | oracle.GRID_LOG_F32 | LEG, 8.0, n, 0.0, IC, [0.005, 0.02],
                                 [-1], 0, 1e4, 4.0, LORENZ, preScaller=2)
    hl = [0.005 + k * ((0.02 - 0.005) / (n - 1)) for k in range(n)]
    expect = "".join("%.12g, %.12g\n" % (hl[k], o["peaks"][k, j]) for k in range(n)
                     for j in range(max(int(o["counts"][k]), 0)))
    assert p.read_text() == expect
    # bifurcation2DIC
    p = tmp_path / "b2.csv"
    old.bifurcation2DIC(5.0, 9, 0.01, 3, IC, [-10.0, 10.0, -10.0, 10.0], [0, 1], 0, 1e4, 4.0, LORENZ, 3, 2, 0.05, p)
    o = oracle.bifurcation_sweep(0, 2, oracle.GRID_STATE | LEG, 5.0, 9, 0.01, IC, [-10.0, 10.0, -10.0, 10.0], [0, 1],
                                 0, 1e4, 4.0, LORENZ, preScaller=2, eps=0.05)
    assert p.read_text() == "-10 10\n-10 10\n" + _csv_matrix(o["labels"], 9, str)
    # LLE1D / LLE1DIC / LLE2DIC
    kw = (10.0, 0.1)
    for name, dim, gm, rng, mut in (("LLE1D", 1, 0, [20.0, 60.0], [1]), ("LLE1DIC", 1, 1, [-8.0, 8.0], [2]),
                                    ("LLE2DIC", 2, 1, [-8.0, 8.0, -8.0, 8.0], [0, 2])):
        m = 12 if dim == 1 else 5
        p = tmp_path / f"{name}.csv"
        getattr(old, name)(*kw, m, 0.01, 1e-8, [1.0, 1.0, 1.0], 3, rng, mut, 0, 0.0, 5.0, LORENZ, 3, p)
        # the legacy LLE kernels' scheme, with the twin draws the engine made
        draws = engine.legacy_lle_draws(gm, m ** dim, 3)
        o = oracle.lle_sweep_legacy(0, dim, gm, 10.0, 0.1, m, 0.01, 1e-8, [1.0, 1.0, 1.0], rng, mut, 0.0, 5.0,
                                    LORENZ, draws=draws)
        got = p.read_text()
        if dim == 1:
            par = [rng[0] + k * ((rng[1] - rng[0]) / (m - 1)) for k in range(m)]
            expect = "".join("%.12g, %.12g\n" % (par[k], o[k]) for k in range(m))
            # the last digit of a printed LLE may differ where the last bit of log does
            assert [ln.split(", ")[0] for ln in got.splitlines()] == [ln.split(", ")[0] for ln in expect.splitlines()]
            assert np.allclose([float(ln.split(", ")[1]) for ln in got.splitlines()], o, rtol=1e-10, atol=1e-12)
        else:
            cells = [float(c) for c in got.replace("\n", "").split(", ")]
            assert np.allclose(cells, o, rtol=1e-5, atol=1e-6) and got.count("\n") == m - 1
    # LS1D / LS2D (the legacy spectrum kernel's scheme, with the engine's twin draws)
    rng = [20.0, 60.0]
    p = tmp_path / "ls1.csv"
    old.LS1D(10.0, 0.1, 6, 0.01, 1e-8, [1.0, 1.0, 1.0], 3, rng, [1], 0, 0.0, 5.0, LORENZ, 3, p)
    o = oracle.lyapunov_spectrum_legacy(0, 1, 0, 10.0, 0.1, 6, 0.01, 1e-8, [1.0, 1.0, 1.0], rng, [1], 0.0, 5.0,
                                        LORENZ, draws=engine.legacy_lle_draws(2, 6, 3))
    rows = [ln.split(", ") for ln in p.read_text().splitlines()]
    assert [r[0] for r in rows] == [_g(6)(20.0 + k * 8.0) for k in range(6)]
    assert np.allclose(np.array([[float(x) for x in r[1:]] for r in rows]), o, rtol=1e-5, atol=1e-6)
    base = tmp_path / "ls2_"
    old.LS2D(10.0, 0.1, 4, 0.01, 1e-8, [1.0, 1.0, 1.0], 3, [20.0, 60.0, 5.0, 15.0], [1, 0], 0, 0.0, 5.0, LORENZ, 3,
             base)
    o = oracle.lyapunov_spectrum_legacy(0, 2, 0, 10.0, 0.1, 4, 0.01, 1e-8, [1.0, 1.0, 1.0],
                                        [20.0, 60.0, 5.0, 15.0], [1, 0], 0.0, 5.0, LORENZ,
                                        draws=engine.legacy_lle_draws(2, 16, 3))
    for j in range(3):
        t = (tmp_path / f"ls2_{j + 1}.csv").read_text()
        assert t.startswith("20 60\n5 15\n")
        cells = [float(c) for c in t.split("\n", 2)[2].replace("\n", "").split(", ")]
        assert np.allclose(cells, o[:, j], rtol=1e-5, atol=1e-6)


def test_perf_cli_tables(engine, tmp_path):
    """chaos_perf runs the reference's three performance sweeps (here at
    small resolutions and modelling times) and writes the reference's result
    tables row for row, with the diagram files beside them."""
    import re
    import subprocess

    cli = engine.lib_path().parent / "chaos_perf"
    r = subprocess.run([str(cli), "--suite", "all", "--resolutions", "16,24", "--times", "100,200",
                        "--fixed-resolution", "16", "--out", str(tmp_path)], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    bif = (tmp_path / "bifurcation_performance_results.csv").read_text().splitlines()
    assert bif[0] == "Test,Parameter,Value,Library,ExecutionTime_ms,Dimension"
    assert [ln.rsplit(",", 2)[0] for ln in bif[1:]] == ["Resolution,16,Bifurcation", "Resolution,24,Bifurcation",
                                                       "ModelingTime,100,Bifurcation", "ModelingTime,200,Bifurcation"]
    assert all(re.fullmatch(r"\w+,\d+,Bifurcation,\d+,2D", ln) for ln in bif[1:])
    for name, lib in (("lle", "LLE"), ("basins", "Basins")):
        t = (tmp_path / f"{name}_performance_results.csv").read_text().splitlines()
        assert t[0] == "Test,Parameter,Value,Library,ExecutionTime_ms"
        assert len(t) == 5 and all(re.fullmatch(rf"(Resolution|ModelingTime),\d+,{lib},\d+", ln) for ln in t[1:])
    assert (tmp_path / "bif2d_res_test_24.csv").read_text().startswith("0 5\n0 20\n")
    assert (tmp_path / "lle_tt_test_200.csv").exists() and (tmp_path / "basins_res_test_16.csv_3.csv").exists()


def test_compact_peaks_dense_list(engine):
    """chaos_compact_peaks: the kept peaks of every row, in row order, clamped
    to the rows (a point keeping more peaks than its row holds contributes the
    row), none for fixed or diverged points; a too-small capacity is refused
    with the total reported."""
    kw = dict(tMax=15.0, nPts=301, h=0.01, initialConditions=[0.1, 0.1, 0.1], ranges=[20.0, 200.0],
              indicesOfMutVars=[1], writableVar=0, maxValue=40.0, transientTime=5.0, values=LORENZ)
    cap = 20  # the rows keep 16-24 peaks: some rows overflow, some do not
    r = engine.bifurcation1d("lorenz", precision=engine.FP32, peakCapacity=cap, **kw)
    assert (r["counts"] > cap).any() and (r["counts"] <= 0).any() and ((r["counts"] > 0) & (r["counts"] <= cap)).any()
    d = engine.compact_peaks(r["counts"], r["peaks"], r["intervals"])
    kept = np.clip(r["counts"], 0, cap)
    assert np.array_equal(d["offsets"], np.concatenate([[0], np.cumsum(kept)]))
    exp_p = np.concatenate([r["peaks"][k, :kept[k]] for k in range(len(kept))])
    exp_i = np.concatenate([r["intervals"][k, :kept[k]] for k in range(len(kept))])
    exp_w = np.concatenate([np.full(kept[k], k) for k in range(len(kept))])
    assert np.array_equal(d["peaks"], exp_p) and np.array_equal(d["intervals"], exp_i)
    assert np.array_equal(d["point"], exp_w)
    import ctypes as C

    L = engine.lib()
    ex = engine._native._exec(engine.FP64, {}, None)
    total = C.c_longlong(0)
    small = np.zeros(5)
    cnt = np.ascontiguousarray(r["counts"], np.int32)
    pk = np.ascontiguousarray(r["peaks"])
    rc = L.chaos_compact_peaks(C.byref(ex), cnt.ctypes.data, pk.ctypes.data, None, len(cnt), cap, None,
                               small.ctypes.data, None, None, 5, C.byref(total))
    assert rc == -1 and total.value == int(kept.sum())
    assert np.array_equal(small, exp_p[:5])
