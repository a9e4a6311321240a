"""GPU parity: the CUDA engine (through the C ABI) against the golden
fixtures made by the reference's own code and against the CPU oracle.

FP64 polynomial systems are compared bit for bit (peak counts, peak values,
intervals, flags, features, labels). Systems whose step calls cos/sin/exp are
compared within tolerances, because CUDA's libm and the host's may differ in
the last bit and chaos amplifies that."""
import numpy as np
import pytest

from conftest import golden, sweep_kwargs

pytestmark = pytest.mark.gpu

SYS = {"lorenz": 0, "rossler": 1, "chen": 2, "chameleon": 3, "sin3": 5}


def eng_kw(kw):
    return dict(tMax=kw["tMax"], nPts=kw["nPts"], h=kw["h"], initialConditions=kw["ic"], ranges=kw["ranges"],
                indicesOfMutVars=kw["mut"], writableVar=kw["wv"], maxValue=kw["maxValue"],
                transientTime=kw["transientTime"], values=kw["values"])


def test_device_code_is_sm_103a(engine):
    """The kernels that run were built for sm_103a (cudaFuncGetAttributes)."""
    binary, ptx = engine.device_code_version(0)
    assert binary == 103, (binary, ptx)


@pytest.mark.parametrize("name", ["peaks_crafted", "peaks_random"])
def test_peak_finder_golden(engine, name):
    g = golden(name)
    r = engine.peak_finder(g["data"], float(g["h"]), peakCapacity=g["data"].shape[1])
    assert np.array_equal(r["counts"], g["counts"])
    for s, c in enumerate(r["counts"]):
        assert np.array_equal(r["peaks"][s, :c], g["peaks"][s, :c])
        assert np.array_equal(r["intervals"][s, :c], g["intervals"][s, :c])


def test_point_dbscan_golden(engine):
    g = golden("point_dbscan")
    out = engine.point_dbscan(g["intervals"], g["counts"], float(g["eps"]))
    assert np.array_equal(out, g["labels"])


@pytest.mark.parametrize("name", ["bif1d_lorenz", "bif2d_lorenz"])
def test_bifurcation_golden_exact(engine, name):
    g = golden(name)
    kw = eng_kw(sweep_kwargs(g))
    if int(g["dim"]) == 1:
        r = engine.bifurcation1d("lorenz", **kw)
        assert np.array_equal(r["counts"], g["counts"])
        for k, c in enumerate(r["counts"]):
            if c > 0:
                assert np.array_equal(r["peaks"][k, :c], g["peaks"][k, :c])
                assert np.array_equal(r["intervals"][k, :c], g["intervals"][k, :c])
            if c == -1:
                assert r["first"][k] == g["first"][k]
    else:
        r = engine.bifurcation2d("lorenz", eps=float(g["eps"]), **kw)
        assert np.array_equal(r["counts"], g["counts"])
        assert np.array_equal(r["labels"], g["labels"])


@pytest.mark.parametrize("name", ["bif1d_chameleon", "bif2d_chameleon"])
def test_bifurcation_golden_transcendental(engine, name):
    """Chameleon calls cos(): counts agree on almost every point, peaks closely."""
    g = golden(name)
    kw = eng_kw(sweep_kwargs(g))
    if int(g["dim"]) == 1:
        r = engine.bifurcation1d("chameleon", **kw)
        same = r["counts"] == g["counts"]
        assert same.mean() >= 0.9
        for k in np.where(same & (r["counts"] > 0))[0]:
            c = r["counts"][k]
            np.testing.assert_allclose(r["peaks"][k, :c], g["peaks"][k, :c], rtol=1e-3, atol=1e-6)
    else:
        r = engine.bifurcation2d("chameleon", eps=float(g["eps"]), **kw)
        assert (r["labels"] == g["labels"]).mean() >= 0.9


@pytest.mark.parametrize("system, values, ic, mi, rng", [
    ("lorenz", [10.0, 28.0, 8 / 3], [0.1, 0.1, 0.1], 1, [20.0, 200.0]),
    ("rossler", [0.2, 0.2, 5.7], [1.0, 1.0, 1.0], 2, [2.0, 10.0]),
    ("chen", [35.0, 3.0, 28.0], [-10.0, 0.0, 37.0], 2, [20.0, 30.0]),
])
def test_bifurcation_vs_oracle_fp64(engine, oracle, system, values, ic, mi, rng):
    kw = dict(tMax=40.0, nPts=96, h=0.01, initialConditions=ic, ranges=rng, indicesOfMutVars=[mi], writableVar=0,
              maxValue=1e4, transientTime=20.0, values=values)
    r = engine.bifurcation1d(system, **kw)
    o = oracle.bifurcation(SYS[system], 1, kw["tMax"], kw["nPts"], kw["h"], ic, rng, [mi], 0, kw["maxValue"],
                           kw["transientTime"], values, cap=r["peaks"].shape[1])
    assert np.array_equal(r["flags"], o["flags"])
    assert np.array_equal(r["counts"], o["counts"])
    for k, c in enumerate(r["counts"]):
        if c > 0:
            assert np.array_equal(r["peaks"][k, :c], o["peaks"][k, :c])
            assert np.array_equal(r["intervals"][k, :c], o["intervals"][k, :c])
        if c == -1:
            assert r["first"][k] == o["first"][k]


def test_bifurcation_small_capacity_reports_true_count(engine, oracle):
    g = golden("bif1d_lorenz")
    kw = eng_kw(sweep_kwargs(g))
    r = engine.bifurcation1d("lorenz", peakCapacity=3, **kw)
    assert np.array_equal(r["counts"], g["counts"])
    for k, c in enumerate(r["counts"]):
        m = min(c, 3)
        if m > 0:
            assert np.array_equal(r["peaks"][k, :m], g["peaks"][k, :m])


@pytest.mark.parametrize("name", ["basins_lorenz"])
def test_basins_golden_exact(engine, oracle, name):
    g = golden(name)
    kw = eng_kw(sweep_kwargs(g))
    f = engine.basins_features("lorenz", **kw)
    assert np.array_equal(f["flags"], g["flags"])
    assert np.array_equal(f["avg_peaks"], g["avg_peaks"])
    assert np.array_equal(f["avg_intervals"], g["avg_intervals"])
    b = engine.basins("lorenz", eps=float(g["eps"]), **kw)
    assert np.array_equal(oracle.canonical_labels(b["labels"]), oracle.canonical_labels(g["labels"]))
    o = oracle.dbscan_compat(g["avg_peaks"], g["avg_intervals"], g["flags"], float(g["eps"]))
    assert np.array_equal(b["labels"], o)  # same canonical numbering as the oracle


def test_basins_golden_transcendental(engine, oracle):
    g = golden("basins_sin3")
    kw = eng_kw(sweep_kwargs(g))
    f = engine.basins_features("sin3", **kw)
    assert (f["flags"] == g["flags"]).mean() >= 0.95
    close = np.isclose(f["avg_peaks"], g["avg_peaks"], rtol=1e-6, atol=1e-9)
    assert close.mean() >= 0.9


def test_dbscan_compat_golden(engine, oracle):
    g = golden("dbscan_compat")
    lab = engine.dbscan_compat(g["avg_peaks"], g["avg_intervals"], g["flags"], float(g["eps"]))
    assert np.array_equal(oracle.canonical_labels(lab), oracle.canonical_labels(g["labels"]))
    assert np.array_equal(lab, oracle.dbscan_compat(g["avg_peaks"], g["avg_intervals"], g["flags"], float(g["eps"])))


def test_dbscan_sklearn_golden(engine):
    g = golden("dbscan_sklearn")
    lab = engine.dbscan(g["X"], float(g["eps"]), int(g["min_pts"]))
    assert np.array_equal(lab, g["labels"])


@pytest.mark.parametrize("n, d, eps, min_pts, seed", [(20000, 2, 0.01, 4, 1), (50000, 3, 0.03, 8, 2),
                                                      (5000, 1, 0.001, 3, 3), (30000, 3, 0.05, 1, 4)])
def test_dbscan_random_vs_oracle(engine, oracle, n, d, eps, min_pts, seed):
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0, 1, size=(20, d))
    X = centres[rng.integers(0, 20, n)] + rng.normal(scale=0.02, size=(n, d))
    X[: n // 10] = rng.uniform(0, 1, size=(n // 10, d))
    mask = (rng.random(n) > 0.02).astype(np.int32)
    lab = engine.dbscan(X, eps, min_pts, mask=mask)
    ref = oracle.dbscan(X, eps, min_pts, mask=mask)
    assert np.array_equal(lab, ref)


@pytest.mark.parametrize("d, min_pts, seed", [(3, 8, 11), (2, 5, 12)])
def test_dbscan_concentrated_vs_oracle(engine, oracle, d, min_pts, seed):
    """Thousands of points on one spot (attractors that are fixed points give
    identical features), tight blobs, points on shells at eps +- 1e-12 around
    a spot, and sparse noise: the cell bounding-box shortcuts of the device
    clustering change no label."""
    rng = np.random.default_rng(seed)
    eps = 0.05
    spot = np.full(d, 0.2)
    parts = [np.tile(spot, (6000, 1)),
             np.full(d, 0.7) + rng.normal(scale=1e-7, size=(6000, d)),
             np.full(d, 0.5) + rng.uniform(-0.02, 0.02, size=(3000, d))]
    u = rng.normal(size=(400, d))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    parts.append(spot + u * (eps + rng.choice([-1e-12, 1e-12], size=(400, 1))))
    parts.append(rng.uniform(0, 1, size=(3000 if d == 3 else 300, d)))
    X = np.concatenate(parts)
    X = X[rng.permutation(len(X))]
    lab = engine.dbscan(X, eps, min_pts)
    ref = oracle.dbscan(X, eps, min_pts)
    assert np.array_equal(lab, ref)


def test_dbscan_unsafe_cells_vs_oracle(engine, oracle):
    """Groups of points far out (features ~1e5 against eps 0.05: their cell
    coordinates clamp at 2^19), NaN features and a mask: the clamped and NaN
    cells lose the one-cell shortcuts and are resolved by exact pair tests
    (a node per core point in the union-find); labels identical to the
    oracle's, which keeps 64-bit cell coordinates and no clamp."""
    rng = np.random.default_rng(21)
    d, eps = 3, 0.05
    parts = [rng.normal(scale=0.03, size=(3000, d)) + 0.5,
             np.full((1, d), 1e5) + rng.normal(scale=0.02, size=(400, d)),
             np.full((1, d), -2e5) + rng.normal(scale=0.02, size=(300, d)),
             np.array([[1e5, -1e5, 3e5]]) + rng.normal(scale=0.2, size=(200, d)),
             rng.uniform(0, 1, size=(500, d))]
    X = np.concatenate(parts)
    X[rng.choice(len(X), 40, replace=False), rng.integers(0, d, 40)] = np.nan
    X = X[rng.permutation(len(X))]
    mask = (rng.random(len(X)) > 0.03).astype(np.int32)
    for min_pts in (1, 5):
        lab = engine.dbscan(X, eps, min_pts, mask=mask)
        ref = oracle.dbscan(X, eps, min_pts, mask=mask)
        assert np.array_equal(lab, ref), min_pts
        assert (lab[np.isnan(X).any(axis=1) & (mask != 0)] == -1).all()


def test_dbscan_compat_eps0_and_far_vs_oracle(engine, oracle):
    """The reference clustering at eps = 0 (every cell unsafe: only equal
    features connect) on data full of exact duplicates, and at eps = 0.05
    with points far out (clamped cell coordinates), against the oracle's
    brute-force breadth-first search."""
    rng = np.random.default_rng(22)
    n = 3000
    ap = rng.integers(0, 40, n) * 0.1
    ai = rng.integers(0, 40, n) * 0.1
    flags = rng.choice([-1, 0, 1], size=n, p=[0.1, 0.1, 0.8]).astype(np.int32)
    lab = engine.dbscan_compat(ap, ai, flags, 0.0)
    assert np.array_equal(lab, oracle.dbscan_compat(ap, ai, flags, 0.0, method="bfs"))
    ap2 = ap + rng.normal(scale=0.01, size=n)
    ap2[:300] += 1e6
    ai2 = ai + rng.normal(scale=0.01, size=n)
    lab = engine.dbscan_compat(ap2, ai2, flags, 0.05)
    assert np.array_equal(lab, oracle.dbscan_compat(ap2, ai2, flags, 0.05, method="bfs"))


@pytest.mark.parametrize("n, spread, eps, seed", [(100000, 1.0, 0.005, 5), (400000, 3.0, 0.01, 6)])
def test_dbscan_compat_random_vs_oracle(engine, oracle, n, spread, eps, seed):
    rng = np.random.default_rng(seed)
    ap = rng.uniform(0, spread, n)
    ai = rng.uniform(0, spread, n)
    ap[:1000] = 7.83  # one dense cell of identical features
    ai[:1000] = -1.0
    flags = rng.choice([-1, 0, 1], size=n, p=[0.05, 0.05, 0.9]).astype(np.int32)
    lab = engine.dbscan_compat(ap, ai, flags, eps)
    ref = oracle.dbscan_compat(ap, ai, flags, eps)
    assert np.array_equal(lab, ref)


def test_lle_fp64_golden_and_oracle(engine, oracle):
    g = golden("lle_rossler")
    kw = dict(tMax=float(g["tMax"]), NT=float(g["NT"]), nPts=int(g["nPts"]), h=float(g["h"]), eps=float(g["eps"]),
              initialConditions=g["ic"], ranges=g["ranges"], indicesOfMutVars=g["mut"],
              transientTime=float(g["transientTime"]), values=g["values"])
    r = engine.lle2d("rossler", precision=engine.FP64, **kw)
    fin = np.isfinite(g["lle"])
    assert np.array_equal(np.isfinite(r), fin)
    assert np.max(np.abs(r[fin] - g["lle"][fin])) < 1e-6
    o = oracle.lle2d(1, kw["tMax"], kw["NT"], kw["nPts"], kw["h"], kw["eps"], g["ic"], g["ranges"], g["mut"],
                     kw["transientTime"], g["values"])
    assert np.max(np.abs(r[fin] - o[fin])) < 1e-12  # same trajectories, libm log may differ in the last bit


@pytest.mark.parametrize("system, values, ranges, mut", [
    ("rossler", [0.2, 0.2, 5.7], [0.1, 0.4, 2.0, 10.0], [0, 2]),
    ("lorenz", [10.0, 28.0, 8 / 3], [20.0, 60.0, 5.0, 15.0], [1, 0]),
    ("chen", [35.0, 3.0, 28.0], [30.0, 40.0, 20.0, 30.0], [0, 2]),
])
def test_lle_fp32_vs_fp64_oracle(engine, oracle, system, values, ranges, mut):
    """FP32 twin-difference LLE against the FP64 oracle. Chaotic orbits in FP32
    and FP64 decorrelate after a few hundred time units and multistable points
    can land on different attractors, so the comparison is statistical: most
    regular points (FP64 LLE < 0.005) agree within 1e-3, nearly all points
    agree on chaotic vs not (0.01) and on finiteness."""
    ic = [1.0, 1.0, 1.0] if system != "chen" else [-10.0, 0.0, 37.0]
    kw = dict(tMax=100.0, NT=0.1, nPts=16, h=0.01, eps=1e-8, initialConditions=ic, ranges=ranges,
              indicesOfMutVars=mut, transientTime=20.0, values=values)
    r = engine.lle2d(system, precision=engine.FP32, **kw)
    o = oracle.lle2d(SYS[system], kw["tMax"], kw["NT"], kw["nPts"], kw["h"], kw["eps"], ic, ranges, mut,
                     kw["transientTime"], values)
    assert (np.isfinite(o) == np.isfinite(r)).mean() >= 0.98
    fin = np.isfinite(o) & np.isfinite(r)
    reg = fin & (o < 0.005)
    if reg.sum() >= 10:
        assert (np.abs(r[reg] - o[reg]) <= 1e-3).mean() >= 0.9
    chaotic_o, chaotic_r = o[fin] > 0.01, r[fin] > 0.01
    assert (chaotic_o == chaotic_r).mean() >= 0.95


TRAJ = {  # system: (x0, a, h)
    "lorenz": ([0.1, 0.1, 0.1], [10.0, 28.0, 8 / 3], 0.01),
    "rossler": ([1.0, 1.0, 1.0], [0.2, 0.2, 5.7], 0.01),
    "chen": ([-10.0, 0.0, 37.0], [35.0, 3.0, 28.0], 0.01),
    "chameleon": ([3.0, 3.0, 0.0], [0.5, 3.0, 0.0, 2.0, 1.0, 18.0, 1.0], 0.01),
    "rossler_cd": ([1.0, 1.0, 1.0], [0.2, 0.2, 0.2, 5.7], 0.01),
    "sin3": ([0.3, -0.2, 0.1], [0.5, 0.1, 1.4, 15.552, 2.0], 0.01),
    "sin2": ([0.5, 0.5], [0.5, 1.0], 0.01),
    "memristor": ([0.1, 0.5, 0.0], [1e-5, 1e6], 1e-9),
}


@pytest.mark.parametrize("name", list(TRAJ))
def test_fp64_trajectory_1e3_steps(engine, oracle, name):
    """FP64 trajectories agree with the oracle to 1e-12 relative over 1e3
    steps; the polynomial RK4 systems bit for bit."""
    x0, a, h = TRAJ[name]
    rng = np.random.default_rng(0)
    X0 = np.array(x0) * (1 + 0.01 * rng.standard_normal((64, len(x0))))
    g = engine.trajectory(name, X0, a, h, 1000)
    for t in range(0, 64, 9):
        o = oracle.trajectory(SYS_ALL[name], X0[t], a, h, 1001)
        if name in ("lorenz", "rossler", "chen"):
            assert np.array_equal(g[t], o)
        else:  # relative to the state's magnitude at each step
            err = np.max(np.abs(g[t] - o), axis=1) / np.maximum(np.max(np.abs(o), axis=1), 1e-300)
            assert err.max() < 1e-12, (err.max(), int(np.argmax(err > 1e-12)))


SYS_ALL = {"lorenz": 0, "rossler": 1, "chen": 2, "chameleon": 3, "rossler_cd": 4, "sin3": 5, "sin2": 6,
           "memristor": 7}


@pytest.mark.parametrize("system, values, ranges, mut", [
    ("rossler", [0.2, 0.2, 5.7], [0.1, 0.4, 2.0, 10.0], [0, 2]),
    ("lorenz", [10.0, 28.0, 8 / 3], [20.0, 60.0, 5.0, 15.0], [1, 0]),
])
def test_lle_fp32_variants_identical(engine, system, values, ranges, mut):
    """The packed two-points-per-thread kernel and the one-point kernels give
    bit-identical maps (each FP32x2 lane rounds as the scalar instruction)."""
    kw = dict(tMax=30.0, NT=0.1, nPts=15, h=0.01, eps=1e-8, initialConditions=[1.0, 1.0, 1.0], ranges=ranges,
              indicesOfMutVars=mut, transientTime=5.0, values=values)
    knob = engine.TUNE_LLE_F32_VARIANT
    old = engine.get_tuning(knob)
    try:
        maps = {}
        for v in (12, 16, 2):
            engine.set_tuning(knob, v)
            maps[v] = engine.lle2d(system, precision=engine.FP32, **kw)
    finally:
        engine.set_tuning(knob, 0)
    for v in (16, 2):
        assert np.array_equal(maps[v], maps[12], equal_nan=True), (v, np.nanmax(np.abs(maps[v] - maps[12])))


@pytest.mark.parametrize("precision", ["fp64"])
def test_basins_dbscan_vs_oracle(engine, oracle, precision):
    """Basins with normalised features and DBSCAN (eps, minPts) bit for bit
    against the oracle's features and DBSCAN on a small Lorenz rho=24 grid."""
    kw = dict(tMax=10.0, nPts=40, h=0.01, initialConditions=[0.0, 0.0, 27.0], ranges=[-30.0, 30.0, -30.0, 30.0],
              indicesOfMutVars=[0, 1], writableVar=0, maxValue=1e8, transientTime=20.0, values=[10.0, 24.0, 8 / 3])
    g = engine.basins_dbscan("lorenz", eps=0.05, minPts=8, **kw)
    lab, F, feat = oracle.basins_dbscan(0, kw["tMax"], kw["nPts"], kw["h"], kw["initialConditions"], kw["ranges"],
                                        kw["indicesOfMutVars"], kw["writableVar"], kw["maxValue"],
                                        kw["transientTime"], kw["values"], eps=0.05, min_pts=8)
    assert np.array_equal(g["flags"], feat["flags"])
    assert np.array_equal(g["features"], F)
    assert np.array_equal(g["labels"], lab)


def _batch_jobs():
    """A small mixed batch: every kind, four systems, uneven sizes."""
    return [
        ("bif", "lorenz", dict(tMax=20.0, nPts=300, h=0.01, initialConditions=[0.1, 0.1, 0.1], ranges=[20.0, 200.0],
                               indicesOfMutVars=[1], writableVar=0, maxValue=1e4, transientTime=5.0,
                               values=[10.0, 28.0, 8 / 3])),
        ("lle", "rossler", dict(tMax=20.0, NT=0.1, nPts=23, h=0.01, eps=1e-8, initialConditions=[1.0, 1.0, 1.0],
                                ranges=[0.1, 0.4, 2.0, 10.0], indicesOfMutVars=[0, 2], transientTime=10.0,
                                values=[0.2, 0.2, 5.7])),
        ("bif", "chen", dict(tMax=10.0, nPts=129, h=0.01, initialConditions=[-10.0, 0.0, 37.0], ranges=[20.0, 30.0],
                             indicesOfMutVars=[2], writableVar=0, maxValue=1e4, transientTime=20.0,
                             values=[35.0, 3.0, 28.0])),
        ("lle", "lorenz", dict(tMax=10.0, NT=0.2, nPts=16, h=0.01, eps=1e-8, initialConditions=[0.1, 0.1, 0.1],
                               ranges=[20.0, 60.0, 5.0, 15.0], indicesOfMutVars=[1, 0], transientTime=3.0,
                               values=[10.0, 28.0, 8 / 3])),
        ("basins", "lorenz", dict(tMax=4.0, nPts=20, h=0.01, initialConditions=[0.0, 0.0, 27.0],
                                  ranges=[-30.0, 30.0, -30.0, 30.0], indicesOfMutVars=[0, 1], writableVar=0,
                                  maxValue=1e8, transientTime=10.0, values=[10.0, 24.0, 8 / 3])),
        ("bif", "chameleon", dict(tMax=10.0, nPts=77, h=0.01, initialConditions=[3.0, 3.0, 0.0], ranges=[0.0, 5.0],
                                  indicesOfMutVars=[3], writableVar=0, maxValue=1e4, transientTime=5.0,
                                  values=[0.5, 3, 0, 2, 1, 18, 1])),
        ("lle", "chameleon", dict(tMax=10.0, NT=0.5, nPts=19, h=0.01, eps=1e-6, initialConditions=[3.0, 3.0, 0.0],
                                  ranges=[0.0, 5.0, 0.0, 20.0], indicesOfMutVars=[3, 5], transientTime=5.0,
                                  values=[0.5, 3, 0, 2, 1, 18, 1])),
        ("lleff", "rossler", dict(tMax=20.0, NT=0.1, nPts=21, h=0.01, eps=1e-8, initialConditions=[1.0, 1.0, 1.0],
                                  ranges=[0.1, 0.4, 2.0, 10.0], indicesOfMutVars=[0, 2], transientTime=10.0,
                                  values=[0.2, 0.2, 5.7])),
        ("lleff", "chen", dict(tMax=5.0, NT=0.1, nPts=12, h=0.01, eps=1e-8, initialConditions=[-10.0, 0.0, 37.0],
                               ranges=[20.0, 30.0, 30.0, 40.0], indicesOfMutVars=[2, 0], transientTime=2.0,
                               values=[35.0, 3.0, 28.0])),
    ]


@pytest.mark.parametrize("mode", ["run", "graph", "device", "device_graph"])
def test_batch_equals_single_jobs(engine, mode):
    """Every job of a mixed batch (one submission, persistent group kernels)
    is bit-identical to the same job run alone through its FP32 entry point;
    a captured plan gives the same results when replayed twice."""
    b = engine.Batch(device=mode.startswith("device"))
    outs = []
    for kind, system, kw in _batch_jobs():
        if kind == "bif":
            outs.append(b.add_bifurcation1d(system, peakCapacity=32, **kw))
        elif kind == "lle":
            outs.append(b.add_lle2d(system, **kw))
        elif kind == "lleff":
            outs.append(b.add_lle2d(system, precision=engine.FF32, **kw))
        else:
            outs.append(b.add_basins(system, **kw))
    runs = 2 if mode.endswith("graph") else 1
    for _ in range(runs):
        if mode.endswith("graph"):
            b.replay()
        else:
            b.run()
        if mode.startswith("device"):
            import torch
            torch.cuda.synchronize()
        for (kind, system, kw), o in zip(_batch_jobs(), outs):
            got = {k: (v.cpu().numpy() if hasattr(v, "cpu") else v) for k, v in o.items()}
            if kind == "bif":
                ref = engine.bifurcation1d(system, precision=engine.FP32, peakCapacity=32, **kw)
                assert np.array_equal(got["counts"], ref["counts"]), system
                assert np.array_equal(got["flags"], ref["flags"])
                for r, c in enumerate(ref["counts"]):  # entries past the count are unspecified
                    m = min(int(c), 32)
                    assert np.array_equal(got["peaks"][r, :m], ref["peaks"][r, :m])
                    assert np.array_equal(got["intervals"][r, :m], ref["intervals"][r, :m])
            elif kind in ("lle", "lleff"):
                p = engine.FF32 if kind == "lleff" else engine.FP32
                ref = engine.lle2d(system, precision=p, **kw)
                assert np.array_equal(got["lle"], ref, equal_nan=True), (kind, system)
            else:
                ref = engine.basins_features(system, precision=engine.FP32, **kw)
                for k in ("flags", "avg_peaks", "avg_intervals", "counts"):
                    assert np.array_equal(got[k], ref[k]), k
    b.close()


SYSID = {"lorenz": 0, "rossler": 1, "chen": 2, "chameleon": 3}


def test_batch_jobs_match_fp64_oracle(engine, oracle):
    """Every job of the mixed batch against the CPU oracle (FP64, the
    reference's algorithm, pinned to its own code), at the stated tolerances
    of each arithmetic over these short horizons. Chaotic orbits in FP32
    leave the FP64 orbit within a few time units, so for them the bars are on
    distributions, per point only where the arithmetic holds the orbit:
    * bifurcation (FP32): flags equal on >= 99 % of points; the peak-count
      distribution's deciles within 1 and its mean within 2 %;
    * basins features (FP32): flags equal on >= 99 %, kept-peak counts on
      >= 95 %, median relative deviation of the mean peak amplitude <= 1e-3;
    * LLE in FP32: Rossler within 2e-4 everywhere, Chameleon median within
      1e-3, Lorenz (10 time units of a chaotic orbit) median within 3e-2;
    * LLE in float-float: Rossler within 2e-5, Chen within 5e-4 everywhere
      (the FP64 twin's own cancellation noise is of that order)."""
    b = engine.Batch()
    jobs = _batch_jobs()
    outs = []
    for kind, system, kw in jobs:
        if kind == "bif":
            outs.append(b.add_bifurcation1d(system, peakCapacity=32, **kw))
        elif kind in ("lle", "lleff"):
            outs.append(b.add_lle2d(system, precision=engine.FF32 if kind == "lleff" else engine.FP32, **kw))
        else:
            outs.append(b.add_basins(system, **kw))
    b.run()
    lle_max = {("lle", "rossler"): 2e-4, ("lleff", "rossler"): 2e-5, ("lleff", "chen"): 5e-4}
    lle_median = {("lle", "chameleon"): 1e-3, ("lle", "lorenz"): 3e-2}
    for (kind, system, kw), got in zip(jobs, outs):
        s = SYSID[system]
        if kind == "bif":
            o = oracle.bifurcation(s, 1, kw["tMax"], kw["nPts"], kw["h"], kw["initialConditions"], kw["ranges"],
                                   kw["indicesOfMutVars"], kw["writableVar"], kw["maxValue"], kw["transientTime"],
                                   kw["values"], cap=32)
            assert np.mean(got["flags"] == o["flags"]) >= 0.99, system
            dec = [abs(np.percentile(got["counts"], q) - np.percentile(o["counts"], q)) for q in range(10, 100, 10)]
            assert max(dec) <= 1, (system, dec)
            assert abs(got["counts"].mean() - o["counts"].mean()) <= 0.02 * o["counts"].mean(), system
        elif kind in ("lle", "lleff"):
            o = oracle.lle2d(s, kw["tMax"], kw["NT"], kw["nPts"], kw["h"], kw["eps"], kw["initialConditions"],
                             kw["ranges"], kw["indicesOfMutVars"], kw["transientTime"], kw["values"])
            fin = np.isfinite(o) & np.isfinite(got["lle"])
            assert fin.mean() > 0.95
            d = np.abs(got["lle"] - o)[fin]
            if (kind, system) in lle_max:
                assert d.max() < lle_max[(kind, system)], (kind, system, d.max())
            else:
                assert np.median(d) < lle_median[(kind, system)], (kind, system, np.median(d))
        else:
            o = oracle.basins_features(s, kw["tMax"], kw["nPts"], kw["h"], kw["initialConditions"], kw["ranges"],
                                       kw["indicesOfMutVars"], kw["writableVar"], kw["maxValue"],
                                       kw["transientTime"], kw["values"])
            assert np.mean(got["flags"] == o["flags"]) >= 0.99
            assert np.mean(got["counts"] == o["counts"]) >= 0.95
            ap, oa = got["avg_peaks"], o["avg_peaks"]
            assert np.median(np.abs(ap - oa) / np.maximum(1.0, np.abs(oa))) <= 1e-3
    b.close()


def test_server_results_equal_alone(engine):
    """Requests served concurrently (continuous batching, staggered arrivals,
    several iterations in flight) give exactly the results of the same jobs
    run alone, including the basins clustering."""
    import time

    srv = engine.Server(hbm_budget_bytes=1 << 30, max_active=8, iteration_steps=2e8)
    reqs = []
    for i, (kind, system, kw) in enumerate(_batch_jobs() * 2):
        if kind == "bif":
            rid, out = srv.submit_bifurcation1d(system, peakCapacity=32, **kw)
        elif kind in ("lle", "lleff"):
            rid, out = srv.submit_lle2d(system, precision=engine.FF32 if kind == "lleff" else engine.FP32, **kw)
        else:
            rid, out = srv.submit_basins(system, eps=0.05, **kw)
        reqs.append((rid, kind, system, kw, out))
        if i % 3 == 0:
            time.sleep(0.002)
    for rid, *_ in reqs:
        assert srv.wait(rid, timeout=120) == engine._native.REQ_DONE
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["p99_s"] >= st["p50_s"] > 0
    for rid, kind, system, kw, got in reqs:
        if kind == "bif":
            ref = engine.bifurcation1d(system, precision=engine.FP32, peakCapacity=32, **kw)
            assert np.array_equal(got["counts"], ref["counts"])
            for r, c in enumerate(ref["counts"]):
                m = min(int(c), 32)
                assert np.array_equal(got["peaks"][r, :m], ref["peaks"][r, :m])
        elif kind in ("lle", "lleff"):
            ref = engine.lle2d(system, precision=engine.FF32 if kind == "lleff" else engine.FP32, **kw)
            assert np.array_equal(got["lle"], ref, equal_nan=True)
        else:
            ref = engine.basins(system, precision=engine.FP32, eps=0.05, **kw)
            assert np.array_equal(got["avg_peaks"], ref["avg_peaks"])
            assert np.array_equal(got["labels"], ref["labels"])
    srv.close()


def test_server_bounded_wait_times_out(engine):
    """A wait shorter than the request's run returns CHAOS_E_TIMEOUT (the host
    gives up, the GPU keeps working) and a later wait sees it done."""
    srv = engine.Server(max_active=2, iteration_steps=1e8)
    rid, out = srv.submit_lle2d("lorenz", tMax=200.0, NT=0.1, nPts=256, h=0.01, eps=1e-8,
                                initialConditions=[0.1, 0.1, 0.1], ranges=[20.0, 60.0, 5.0, 15.0],
                                indicesOfMutVars=[1, 0], transientTime=10.0, values=[10.0, 28.0, 8 / 3])
    with pytest.raises(engine.ChaosError) as e:
        srv.wait(rid, timeout=1e-4)
    assert e.value.code == -5
    assert srv.wait(rid, timeout=300) == engine._native.REQ_DONE
    assert np.isfinite(out["lle"]).mean() > 0.99
    srv.close()


def test_server_budget_admission(engine):
    """With an HBM budget smaller than the sum of the requests, admission
    queues them and the peak device footprint stays within the budget."""
    budget = 4 << 20
    srv = engine.Server(hbm_budget_bytes=budget, max_active=64, iteration_steps=5e7)
    rids = []
    for k in range(12):
        rid, _ = srv.submit_lle2d("rossler", tMax=5.0, NT=0.1, nPts=300, h=0.01, eps=1e-8,
                                  initialConditions=[1.0, 1.0, 1.0], ranges=[0.1, 0.4, 2.0, 10.0],
                                  indicesOfMutVars=[0, 2], transientTime=1.0, values=[0.2, 0.2, 5.7])
        rids.append(rid)
    for rid in rids:
        assert srv.wait(rid, timeout=120) == engine._native.REQ_DONE
    st = srv.stats()
    assert st["peak_hbm_bytes"] <= budget
    srv.close()


def _csv_matrix(values, nPts, fmt):
    """The reference's matrix rule: ', ' before every value but the first and
    '\\n' (after the ', ') whenever nPts values are on the line."""
    out, counter = [], 0
    for v in values:
        if counter != 0:
            out.append(", ")
        if counter == nPts:
            out.append("\n")
            counter = 0
        out.append(fmt(v))
        counter += 1
    return "".join(out)


def _g(p):
    return lambda v: ("%." + str(p) + "g") % v


def test_compat_csv_bytes(engine, oracle, tmp_path):
    """The reference-signature wrappers write the reference's CSV bytes:
    bifurcation1D rows at precision 12 after a precision-6 header,
    bifurcation2D / LLE2D matrices, basins' four files at precision 15."""
    L = engine
    L.set_system("lorenz")
    vals = np.array([10.0, 28.0, 8 / 3])
    # 1-D bifurcation
    p = tmp_path / "bif1d.csv"
    L.Bifurcation.bifurcation1D(20.0, 40, 0.01, 3, [0.1, 0.1, 0.1], [20.0, 200.0], [1], 0, 1e4, 10.0, vals, 3, 1, p)
    o = oracle.bifurcation(0, 1, 20.0, 40, 0.01, [0.1, 0.1, 0.1], [20.0, 200.0], [1], 0, 1e4, 10.0, vals)
    lines = ["%g %g\n" % (20.0, 200.0)]
    for k in range(40):
        par = 20.0 + k * ((200.0 - 20.0) / 39)
        if o["counts"][k] == -1:
            lines.append("%.12g, %.12g, 0\n" % (par, o["first"][k]))
        for j in range(max(o["counts"][k], 0)):
            lines.append("%.12g, %.12g, %.12g\n" % (par, o["peaks"][k, j], o["intervals"][k, j]))
    assert p.read_text() == "".join(lines)
    # 2-D bifurcation
    p = tmp_path / "bif2d.csv"
    L.Bifurcation.bifurcation2D(5.0, 9, 0.01, 3, [0.1, 0.1, 0.1], [20.0, 200.0, 5.0, 15.0], [1, 0], 0, 1e4, 5.0,
                                vals, 3, 1, 0.05, p)
    o = oracle.bifurcation(0, 2, 5.0, 9, 0.01, [0.1, 0.1, 0.1], [20.0, 200.0, 5.0, 15.0], [1, 0], 0, 1e4, 5.0, vals,
                           eps=0.05)
    expect = "20 200\n5 15\n" + _csv_matrix(o["labels"], 9, str)
    assert p.read_text() == expect
    # LLE (values at the default precision 6, NaN printed as 0)
    L.set_system("rossler")
    p = tmp_path / "lle.csv"
    L.LLE.LLE2D(20.0, 0.1, 7, 0.01, 1e-8, [1.0, 1.0, 1.0], 3, [0.1, 0.4, 2.0, 10.0], [0, 2], 0, 0.0, 5.0,
                [0.2, 0.2, 5.7], 3, p)
    o = oracle.lle2d(1, 20.0, 0.1, 7, 0.01, 1e-8, [1.0, 1.0, 1.0], [0.1, 0.4, 2.0, 10.0], [0, 2], 5.0,
                     [0.2, 0.2, 5.7])
    expect = "0.1 0.4\n2 10\n" + _csv_matrix(np.nan_to_num(o, nan=0.0), 7, _g(6))
    got = p.read_text()
    # values agree to the printed digits except where the last FP64 bit of log differs
    assert got.count("\n") == expect.count("\n") and got.split("\n")[:2] == expect.split("\n")[:2]
    g_cells = [c.strip() for c in got.split("\n", 2)[2].replace("\n", "").split(",")]
    e_cells = [c.strip() for c in expect.split("\n", 2)[2].replace("\n", "").split(",")]
    assert len(g_cells) == len(e_cells) == 49
    assert sum(a != b for a, b in zip(g_cells, e_cells)) <= 1
    # basins: four files, precision 15
    L.set_system("lorenz")
    base = tmp_path / "bas"
    kw = (4.0, 12, 0.01, 3, [0.0, 0.0, 27.0], [-30.0, 30.0, -30.0, 30.0], [0, 1], 0, 1e8, 10.0,
          [10.0, 24.0, 8 / 3], 3, 1, 0.05)
    L.Basins.basinsOfAttraction_2(*kw, base)
    f = oracle.basins_features(0, 4.0, 12, 0.01, [0.0, 0.0, 27.0], [-30.0, 30.0, -30.0, 30.0], [0, 1], 0, 1e8, 10.0,
                               [10.0, 24.0, 8 / 3])
    lab = oracle.dbscan_compat(f["avg_peaks"], f["avg_intervals"], f["flags"], 0.05)
    head = "-30 30\n-30 30\n"
    assert (tmp_path / "bas").read_text() == head + _csv_matrix(lab, 12, str)
    assert (tmp_path / "bas_1.csv").read_text() == head + _csv_matrix(f["avg_peaks"], 12, _g(15))
    assert (tmp_path / "bas_2.csv").read_text() == head + _csv_matrix(f["avg_intervals"], 12, _g(15))
    assert (tmp_path / "bas_3.csv").read_text() == head + _csv_matrix(f["flags"], 12, str)


@pytest.mark.parametrize("system, values, ic, mi, rng, maxv", [
    ("lorenz", [10.0, 28.0, 8 / 3], [0.1, 0.1, 0.1], 1, [20.0, 200.0], 40.0),   # many points diverge (|x| > 40)
    ("rossler", [0.2, 0.2, 5.7], [1.0, 1.0, 1.0], 2, [2.0, 10.0], 1e4),
    ("chen", [35.0, 3.0, 28.0], [-10.0, 0.0, 37.0], 2, [20.0, 30.0], 1e4),
])
def test_paired_sweeps_identical(engine, system, values, ic, mi, rng, maxv):
    """FP32 bifurcation and basins sweeps give bit-identical results with two
    points per thread (packed FP32x2 lanes) and with one, including lanes that
    diverge while their partner keeps recording and an odd point count."""
    knob = engine.TUNE_SWEEP_PAIRS
    kw = dict(tMax=15.0, nPts=101, h=0.01, initialConditions=ic, ranges=rng, indicesOfMutVars=[mi], writableVar=0,
              maxValue=maxv, transientTime=5.0, values=values)
    bk = dict(tMax=6.0, nPts=23, h=0.01, initialConditions=ic, ranges=[-20.0, 20.0, -20.0, 20.0],
              indicesOfMutVars=[0, 1], writableVar=0, maxValue=maxv * 2, transientTime=3.0, values=values)
    res = {}
    try:
        for v in (0, 2, 3):  # one point per thread, fully packed, hybrid (packed transient)
            engine.set_tuning(knob, v)
            res[v] = (engine.bifurcation1d(system, precision=engine.FP32, peakCapacity=40, **kw),
                      engine.basins_features(system, precision=engine.FP32, preScaller=2, **bk),
                      engine.basins_features(system, precision=engine.FP32, preScaller=1, **bk))
    finally:
        engine.set_tuning(knob, 1)
    for k in ("flags", "avg_peaks", "avg_intervals", "counts"):
        assert np.array_equal(res[0][1][k], res[3][1][k]), k
        assert np.array_equal(res[0][2][k], res[3][2][k]), k
        assert np.array_equal(res[0][2][k], res[2][2][k]), k
    b3 = res[3][0]
    for k in ("flags", "counts", "first"):
        assert np.array_equal(res[0][0][k], b3[k]), k
    for r, c in enumerate(res[0][0]["counts"]):
        m = min(int(c), 40)
        if m > 0:
            assert np.array_equal(res[0][0]["peaks"][r, :m], b3["peaks"][r, :m])
            assert np.array_equal(res[0][0]["intervals"][r, :m], b3["intervals"][r, :m])
    (b0, f0, _), (b1, f1, _) = res[0], res[2]
    assert np.array_equal(b0["flags"], b1["flags"]) and np.array_equal(b0["counts"], b1["counts"])
    assert np.array_equal(b0["first"], b1["first"])
    for r, c in enumerate(b0["counts"]):
        m = min(int(c), 40)
        if m > 0:
            assert np.array_equal(b0["peaks"][r, :m], b1["peaks"][r, :m])
            assert np.array_equal(b0["intervals"][r, :m], b1["intervals"][r, :m])
    for k in ("flags", "avg_peaks", "avg_intervals", "counts"):
        assert np.array_equal(f0[k], f1[k]), k
    if system == "lorenz":
        assert (b0["flags"] == 0).any() and (b0["flags"] == 1).any()


def test_launch_count(engine):
    """chaos_launch_count grows by one for a single-kernel sweep and by the
    graph's kernels (counter reset + one per (kind, system) group) for each
    replay of a prepared batch, not at capture."""
    lle = dict(tMax=1.0, NT=0.1, nPts=8, h=0.01, eps=1e-8, initialConditions=[1.0, 1.0, 1.0],
               ranges=[0.1, 0.4, 2.0, 10.0], indicesOfMutVars=[0, 2], transientTime=0.5, values=[0.2, 0.2, 5.7])
    n0 = engine.launch_count()
    engine.lle2d("rossler", precision=engine.FP32, **lle)
    assert engine.launch_count() - n0 == 1
    b = engine.Batch(device=False)
    b.add_lle2d("rossler", **lle)
    b.add_bifurcation1d("lorenz", tMax=1.0, nPts=50, h=0.01, initialConditions=[0.1, 0.1, 0.1], ranges=[20.0, 30.0],
                        indicesOfMutVars=[1], writableVar=0, maxValue=1e4, transientTime=0.5,
                        values=[10.0, 28.0, 8 / 3], peakCapacity=8)
    n1 = engine.launch_count()
    b.prepare()
    assert engine.launch_count() == n1
    b.replay()
    b.replay()
    assert engine.launch_count() - n1 == 2 * 3
    b.close()


CHAM_LLE = dict(NT=0.5, h=0.01, eps=1e-6, initialConditions=[3.0, 3.0, 0.0], ranges=[0.0, 5.0, 0.0, 20.0],
                indicesOfMutVars=[3, 5], values=[0.5, 3, 0, 2, 1, 18, 1])


@pytest.mark.parametrize("system", ["rossler", "chameleon"])
def test_lle_sign_recheck(engine, system):
    """FP32 LLE map with the FP64 sign re-check: points outside the band keep
    their FP32 value; exactly the checked points whose short FP64 check
    disagrees in class (positive / non-positive / not finite) are replaced,
    by the FP64 map's value bit for bit; with a full-horizon check the
    replaced points are those whose FP32 and FP64 classes differ."""
    if system == "rossler":
        kw = dict(tMax=60.0, NT=0.1, nPts=40, h=0.01, eps=1e-8, initialConditions=[1.0, 1.0, 1.0],
                  ranges=[0.1, 0.4, 2.0, 10.0], indicesOfMutVars=[0, 2], transientTime=10.0,
                  values=[0.2, 0.2, 5.7])
    else:
        kw = dict(tMax=60.0, NT=0.5, nPts=32, h=0.01, eps=1e-6, **{k: v for k, v in CHAM_LLE.items()
                                                                   if k not in ("NT", "h", "eps")},
                  transientTime=20.0)
    band, ct = 0.02, 15.0
    v32 = engine.lle2d(system, precision=engine.FP32, **kw)
    v64 = engine.lle2d(system, precision=engine.FP64, **kw)
    vs = engine.lle2d(system, precision=engine.FP64, **dict(kw, tMax=ct))

    def cls(v):
        return np.where(~np.isfinite(v), -1, (v > 0).astype(int))

    checked = ~(np.abs(v32) > band)
    got, nc, nr = engine.lle2d_checked(system, band=band, checkTMax=ct, **kw)
    flip = checked & (cls(v32) != cls(vs))
    assert nc == int(checked.sum()) and nr == int(flip.sum())
    assert np.array_equal(got[~flip], v32[~flip], equal_nan=True)
    assert np.array_equal(got[flip], v64[flip], equal_nan=True)
    got2, nc2, nr2 = engine.lle2d_checked(system, band=band, checkTMax=kw["tMax"], **kw)
    flip2 = checked & (cls(v32) != cls(v64))
    assert nc2 == nc and nr2 == int(flip2.sum())
    assert np.array_equal(got2[flip2], v64[flip2], equal_nan=True)
    assert np.array_equal(got2[~flip2], v32[~flip2], equal_nan=True)
    assert np.all(cls(got2)[checked] == cls(v64)[checked])


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_bif2d_capacity_never_changes_results(engine, precision, monkeypatch):
    """The 2-D bifurcation's peak-buffer capacity (B/2, fitted to the scratch
    budget, measured by a probe under a 1 MB budget, or fixed) changes memory
    and speed only: points with more kept peaks than the capacity are run
    again with B/2 rows, so labels and counts are the same in every mode."""
    kw = dict(tMax=40.0, nPts=24, h=0.01, initialConditions=[3.0, 3.0, 0.0], ranges=[0.0, 5.0, 0.0, 20.0],
              indicesOfMutVars=[3, 5], writableVar=0, maxValue=1e4, transientTime=20.0,
              values=[0.5, 3, 0, 2, 1, 18, 1], eps=0.001)
    knob = engine.TUNE_BIF2D_CAP
    res = {}
    try:
        for name, mode, budget_mb in (("full", -1, None), ("default", 0, None), ("fixed3", 3, None),
                                      ("probe", 0, "1")):
            if budget_mb:
                monkeypatch.setenv("CHAOS_SCRATCH_BUDGET_MB", budget_mb)
            engine.set_tuning(knob, mode)
            res[name] = engine.bifurcation2d("chameleon", precision=precision, **kw)
    finally:
        engine.set_tuning(knob, 0)
    assert (res["full"]["counts"] > 3).any()  # the fixed capacity 3 really overflows
    for name in ("default", "fixed3", "probe"):
        assert np.array_equal(res[name]["labels"], res["full"]["labels"]), name
        assert np.array_equal(res[name]["counts"], res["full"]["counts"]), name


def test_autotune_changes_no_result(engine):
    """chaos_autotune times the FP32 sweeps' launch shapes on this GPU and
    installs the fastest; bifurcation, basins and LLE results are the same
    before and after it, and CHAOS_TUNE_SHAPES 0 restores the rules."""
    bif = dict(tMax=10.0, nPts=3000, h=0.01, initialConditions=[0.1, 0.1, 0.1], ranges=[20.0, 200.0],
               indicesOfMutVars=[1], writableVar=0, maxValue=1e4, transientTime=5.0, values=[10.0, 28.0, 8 / 3])
    bas = dict(tMax=5.0, nPts=60, h=0.01, initialConditions=[0.0, 0.0, 27.0], ranges=[-30.0, 30.0, -30.0, 30.0],
               indicesOfMutVars=[0, 1], writableVar=0, maxValue=1e8, transientTime=5.0, values=[10.0, 24.0, 8 / 3])
    lle = dict(tMax=5.0, NT=0.1, nPts=60, h=0.01, eps=1e-8, initialConditions=[1.0, 1.0, 1.0],
               ranges=[0.1, 0.4, 2.0, 10.0], indicesOfMutVars=[0, 2], transientTime=2.0, values=[0.2, 0.2, 5.7])

    def run():
        return (engine.bifurcation1d("lorenz", precision=engine.FP32, peakCapacity=16, **bif),
                engine.basins_features("lorenz", precision=engine.FP32, **bas),
                engine.lle2d("rossler", precision=engine.FP32, **lle))

    before = run()
    try:
        table = engine.autotune()
        assert len(table) == 9 and all(r["best_ms"] > 0 and r["rule_ms"] > 0 for r in table)
        assert all(r["best_ms"] <= r["rule_ms"] for r in table)
        after = run()
    finally:
        engine.set_tuning(engine.TUNE_SHAPES, 0)
    (b0, f0, l0), (b1, f1, l1) = before, after
    for k in ("counts", "flags"):
        assert np.array_equal(b0[k], b1[k]), k
    for r, c in enumerate(b0["counts"]):
        m = min(int(c), 16)
        assert np.array_equal(b0["peaks"][r, :m], b1["peaks"][r, :m])
    for k in ("flags", "avg_peaks", "avg_intervals"):
        assert np.array_equal(f0[k], f1[k]), k
    assert np.array_equal(l0, l1, equal_nan=True)


LORENZ28 = dict(values=[10.0, 28.0, 8 / 3], initialConditions=[1.0, 1.0, 1.0])


@pytest.mark.parametrize("dim, state", [(1, False), (1, True), (2, True)])
def test_lle_sweep_fp64_vs_oracle(engine, oracle, dim, state):
    """LLE over 1-D parameter grids and 1-D / 2-D grids of initial conditions
    (the legacy LLE1D / LLE1DIC / LLE2DIC analyses) against the oracle."""
    if state:
        rng, mut = ([-10.0, 10.0, -10.0, 10.0][: 2 * dim], [0, 1][:dim])
    else:
        rng, mut = [20.0, 60.0], [1]
    n = 9 if dim == 2 else 40
    kw = dict(tMax=20.0, NT=0.1, nPts=n, h=0.01, eps=1e-8, ranges=rng, indicesOfMutVars=mut, transientTime=5.0,
              **LORENZ28)
    g = engine.lle_sweep("lorenz", dim, mutateState=state, **kw)
    o = oracle.lle_sweep(0, dim, int(state), kw["tMax"], kw["NT"], n, kw["h"], kw["eps"], kw["initialConditions"],
                         rng, mut, kw["transientTime"], kw["values"])
    assert np.max(np.abs(g - o)) < 1e-12


def test_lle_sweep_2d_params_is_lle2d(engine):
    kw = dict(tMax=10.0, NT=0.1, nPts=12, h=0.01, eps=1e-8, initialConditions=[1.0, 1.0, 1.0],
              ranges=[0.1, 0.4, 2.0, 10.0], indicesOfMutVars=[0, 2], transientTime=2.0, values=[0.2, 0.2, 5.7])
    for p in (engine.FP64, engine.FP32):
        assert np.array_equal(engine.lle_sweep("rossler", 2, precision=p, **kw),
                              engine.lle2d("rossler", precision=p, **kw), equal_nan=True)


@pytest.mark.parametrize("system, sid, vals, ic", [("lorenz", 0, [10.0, 28.0, 8 / 3], [1.0, 1.0, 1.0]),
                                                    ("rossler", 1, [0.2, 0.2, 5.7], [1.0, 1.0, 1.0]),
                                                    ("chameleon", 3, [0.5, 3, 0, 2, 1, 18, 1], [3.0, 3.0, 0.0])])
def test_spectrum_fp64_vs_oracle(engine, oracle, system, sid, vals, ic):
    """Lyapunov spectrum (one twin per dimension, classical Gram-Schmidt per
    block) against the oracle's restatement."""
    k = 3 if sid == 3 else 0
    rng, mut = [vals[k] * 0.9, vals[k] * 1.1], [k]
    kw = dict(tMax=10.0, NT=0.1, nPts=16, h=0.01, eps=1e-8, ranges=rng, indicesOfMutVars=mut, transientTime=2.0)
    g = engine.lyapunov_spectrum(system, 1, initialConditions=ic, values=vals, **kw)
    o = oracle.lyapunov_spectrum(sid, 1, 0, kw["tMax"], kw["NT"], 16, kw["h"], kw["eps"], ic, rng, mut,
                                 kw["transientTime"], vals)
    fin = np.isfinite(o)
    assert np.array_equal(fin, np.isfinite(g))
    # cos: CUDA's libm and glibc may differ in the last bit, which the chaotic
    # Chameleon flow amplifies over the 1,200 steps (measured 4e-7)
    tol = 1e-12 if sid <= 2 else 1e-5
    assert np.max(np.abs(g[fin] - o[fin])) < tol


def test_spectrum_lorenz_physics_fp32_and_fp64(engine):
    """Lorenz at rho = 28: exponents near (0.906, 0, -14.57) and their sum
    near -(sigma + 1 + beta) times the blocks' span over tMax, in FP64 and in
    the FP32 exact-difference path."""
    kw = dict(tMax=200.0, NT=0.1, nPts=4, h=0.01, eps=1e-8, ranges=[28.0, 28.0], indicesOfMutVars=[1],
              transientTime=20.0, **LORENZ28)
    span = (int(round(kw["tMax"] / kw["h"])) // 10 + 2) * kw["NT"] / kw["tMax"]
    for p in (engine.FP64, engine.FP32):
        s = engine.lyapunov_spectrum("lorenz", 1, precision=p, **kw)
        assert np.all(np.abs(s[:, 0] - 0.906) < 0.1), s
        assert np.all(np.abs(s[:, 1]) < 0.05), s
        assert np.all(np.abs(s[:, 2] + 14.57) < 0.15), s
        assert np.all(np.abs(s.sum(axis=1) + (10 + 1 + 8 / 3) * span) < 0.02), s



def test_chameleon_fp32_lle_short_horizon(engine):
    """The FP32 Chameleon LLE (twin as the difference of chameleon_step_twin,
    the cos term in product form) against FP64 over a horizon too short for
    chaos to amplify rounding: the difference form loses no precision."""
    kw = dict(tMax=2.0, nPts=16, transientTime=1.0, **CHAM_LLE)
    l32 = engine.lle2d("chameleon", precision=engine.FP32, **kw)
    l64 = engine.lle2d("chameleon", precision=engine.FP64, **kw)
    assert np.all(np.isfinite(l32)) and np.all(np.isfinite(l64))
    assert np.max(np.abs(l32 - l64)) < 2e-4


def test_chameleon_fp32_lle_within_the_maps_conditioning(engine):
    """Over the reference's LLE timing sweep horizon the FP32 map differs from
    the FP64 map no more than the FP64 map differs from itself started 1e-13
    away (the conditioning of a finite-time LLE; measured on 300^2: p50 2.6e-3
    vs 1.5e-3, p99 0.33 vs 0.33, sign classes 91.7 % vs 93.0 %)."""
    kw = dict(tMax=400.0, nPts=32, transientTime=2000.0, **CHAM_LLE)
    l32 = engine.lle2d("chameleon", precision=engine.FP32, **kw)
    l64 = engine.lle2d("chameleon", precision=engine.FP64, **kw)
    l64b = engine.lle2d("chameleon", precision=engine.FP64, **dict(kw, initialConditions=[3.0 + 1e-13, 3.0, 0.0]))
    assert np.array_equal(np.isfinite(l32), np.isfinite(l64))
    d32, dself = np.abs(l32 - l64), np.abs(l64b - l64)
    assert np.percentile(d32, 50) <= max(3 * np.percentile(dself, 50), 5e-3)
    assert np.percentile(d32, 90) <= 2 * np.percentile(dself, 90) + 0.02
    cls = lambda v: (v > 0.01).astype(int)  # noqa: E731
    assert np.mean(cls(l32) == cls(l64)) >= np.mean(cls(l64b) == cls(l64)) - 0.05


def test_chameleon_spectrum_sum_is_the_jacobian_volume(engine):
    """Chameleon's step is volume-contracting by the constant factor
    (1 - h1*a3) / (1 + a3*h2) (the only non-shear updates of its composition),
    so the exponents of the spectrum sum to blocks * NT/h * log(factor) / tMax
    at every grid point: checked in FP64 and in the FP32 difference-form twins.
    (The twins span a parallelepiped of side eps = 1e-6, not an infinitesimal
    one: with cos(18 x) in the field its volume follows the Jacobian's to
    about 4e-4 of the sum.)"""
    kw = dict(tMax=50.0, NT=0.5, nPts=8, h=0.01, eps=1e-6, initialConditions=[3.0, 3.0, 0.0], ranges=[0.5, 4.0],
              indicesOfMutVars=[3], transientTime=100.0, values=[0.5, 3, 0, 2, 1, 18, 1])
    a3 = np.array([0.5 + k * (3.5 / 7) for k in range(8)])
    h = kw["h"]
    h1, h2 = 0.5 * h, (1 - 0.5) * h
    ntp = int(round(kw["NT"] / h))
    blocks = int(round(kw["tMax"] / h)) // ntp + 2
    expect = blocks * ntp * np.log((1 - h1 * a3) / (1 + a3 * h2)) / kw["tMax"]
    for p, tol in ((engine.FP64, 1e-3), (engine.FP32, 2e-3)):
        s = engine.lyapunov_spectrum("chameleon", 1, precision=p, **kw)
        assert np.all(np.isfinite(s))
        assert np.max(np.abs(s.sum(axis=1) - expect)) < tol, (p, s.sum(axis=1), expect)


def test_chameleon_fp32_spectrum_short_horizon(engine):
    kw = dict(tMax=2.0, NT=0.5, nPts=12, h=0.01, eps=1e-6, initialConditions=[3.0, 3.0, 0.0], ranges=[0.0, 5.0],
              indicesOfMutVars=[3], transientTime=1.0, values=[0.5, 3, 0, 2, 1, 18, 1])
    s32 = engine.lyapunov_spectrum("chameleon", 1, precision=engine.FP32, **kw)
    s64 = engine.lyapunov_spectrum("chameleon", 1, precision=engine.FP64, **kw)
    assert np.max(np.abs(s32 - s64)) < 2e-3
