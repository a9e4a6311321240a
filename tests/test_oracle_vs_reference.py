"""The oracle against the host build of the reference's own functions on fresh
random inputs, for every plug-in system. Runs only where the reference
sources were available to oracle/build_ref.py (this container)."""
import numpy as np
import pytest

from oracle import build_ref

pytestmark = pytest.mark.skipif(not build_ref.available(), reason="reference sources not present")

SYSTEMS = {  # name: (id, values, ic, param range index, range, basins ic range)
    "lorenz": (0, [10.0, 28.0, 8.0 / 3.0], [0.1, 0.1, 0.1], 1, [20.0, 200.0]),
    "rossler": (1, [0.2, 0.2, 5.7], [1.0, 1.0, 1.0], 2, [2.0, 10.0]),
    "chen": (2, [35.0, 3.0, 28.0], [-10.0, 0.0, 37.0], 2, [20.0, 30.0]),
    "chameleon": (3, [0.5, 3.0, 0.0, 2.0, 1.0, 18.0, 1.0], [3.0, 3.0, 0.0], 3, [0.0, 5.0]),
    "rossler_cd": (4, [0.2, 0.2, 0.2, 5.7], [1.0, 1.0, 1.0], 3, [2.0, 8.0]),
    "sin3": (5, [0.5, 0.1, 1.4, 15.552, 2.0], [0.0, 0.0, 0.0], 1, [0.05, 0.3]),
    "sin2": (6, [0.5, 1.0], [0.5, 0.5], 1, [0.5, 1.5]),
    "memristor": (7, [1e-5, 1e6], [0.1, 0.5, 0.0], 0, [1e-6, 2e-5]),
}


@pytest.fixture(scope="module")
def refs():
    build_ref.build()
    from oracle import oracle as O

    return {n: O.RefLib(n) for n in SYSTEMS}


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_step_map(oracle, refs, name):
    sysid, values, ic, _, _ = SYSTEMS[name]
    h = 1e-9 if name == "memristor" else 0.01
    assert np.array_equal(oracle.steps(sysid, ic, values, h, 500), refs[name].steps(ic, values, h, 500))


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_bifurcation_1d(oracle, refs, name):
    sysid, values, ic, mi, rng = SYSTEMS[name]
    h = 1e-9 if name == "memristor" else 0.01
    kw = dict(tMax=400 * h, nPts=24, h=h, ic=ic, ranges=rng, mut=[mi], wv=0, maxValue=1e4,
              transientTime=300 * h, values=values)
    r = refs[name].bifurcation(1, **kw)
    o = oracle.bifurcation(sysid, 1, **kw)
    assert np.array_equal(o["counts"], r["counts"])
    for k, c in enumerate(o["counts"]):
        if c > 0:
            assert np.array_equal(o["peaks"][k, :c], r["data"][k, :c])
            assert np.array_equal(o["intervals"][k, :c], r["intervals"][k, :c])
        if c == -1:
            assert o["first"][k] == r["data"][k, 0]


@pytest.mark.parametrize("name", ["lorenz", "chameleon", "rossler_cd", "sin3"])
def test_bifurcation_2d(oracle, refs, name):
    sysid, values, ic, mi, rng = SYSTEMS[name]
    other = 0 if mi != 0 else 1
    kw = dict(tMax=3.0, nPts=9, h=0.01, ic=ic, ranges=rng + [values[other] * 0.5, values[other] * 1.5 + 0.1],
              mut=[mi, other], wv=0, maxValue=1e4, transientTime=2.0, values=values)
    for eps in (0.001, 0.05):
        r = refs[name].bifurcation(2, eps=eps, **kw)
        o = oracle.bifurcation(sysid, 2, eps=eps, **kw)
        assert np.array_equal(o["labels"], r["labels"])


@pytest.mark.parametrize("name", ["lorenz", "sin3", "sin2", "chameleon"])
def test_basins_features_and_clustering(oracle, refs, name):
    sysid, values, ic, _, _ = SYSTEMS[name]
    nx = len(ic)
    kw = dict(tMax=4.0, nPts=12, h=0.01, ic=ic, ranges=[-5.0, 5.0, -5.0, 5.0], mut=[0, nx - 1], wv=0,
              maxValue=1e6, transientTime=6.0, values=values)
    for ps in (1, 3):
        r = refs[name].basins(preScaller=ps, **kw)
        o = oracle.basins_features(sysid, preScaller=ps, **kw)
        for k in ("flags", "avg_peaks", "avg_intervals"):
            assert np.array_equal(o[k], r[k]), k
        lr = refs[name].basins_dbscan(r["avg_peaks"], r["avg_intervals"], r["flags"], 0.05)
        lo = oracle.dbscan_compat(o["avg_peaks"], o["avg_intervals"], o["flags"], 0.05)
        assert np.array_equal(oracle.canonical_labels(lo), oracle.canonical_labels(lr))


def test_peak_finder_random_ties(oracle, refs):
    rng = np.random.default_rng(7)
    for _ in range(200):
        n = int(rng.integers(3, 120))
        d = np.round(rng.normal(size=n).cumsum(), int(rng.integers(0, 3)))
        if rng.random() < 0.3:
            d = d + rng.choice([0.0, 1e-13, 2e-13, -1e-13], size=n)
        c, p, t = refs["lorenz"].peak_finder(d, 0.01)
        oc, op, ot = oracle.peak_finder(d, 0.01)
        assert oc[0] == c
        assert np.array_equal(op[0, :c], p) and np.array_equal(ot[0, :c], t)


def test_point_dbscan_random(oracle, refs):
    rng = np.random.default_rng(3)
    for _ in range(100):
        P = int(rng.integers(1, 60))
        iv = np.round(rng.uniform(0, 1, size=P), int(rng.integers(1, 4)))
        eps = float(rng.choice([1e-3, 0.01, 0.05, 0.2]))
        r = refs["lorenz"].point_dbscan(np.zeros(P), iv, P, 2 * P + 2, eps)
        o = oracle.point_dbscan(iv[None, :], np.array([P]), eps)[0]
        assert o == r


def test_lle(oracle, refs):
    kw = dict(tMax=30.0, NT=0.2, nPts=6, h=0.01, eps=1e-7, ic=[0.1, 0.1, 0.1], ranges=[10.0, 30.0, 1.0, 4.0],
              mut=[1, 2], transientTime=5.0, values=[10.0, 28.0, 8.0 / 3.0])
    r = refs["lorenz"].lle(**kw)
    o = oracle.lle2d(0, **kw)
    assert np.max(np.abs(r - o)) < 1e-6


def test_dbscan_compat_grid_equals_bfs(oracle):
    rng = np.random.default_rng(11)
    for n, spread in [(300, 0.3), (2000, 1.0), (800, 0.05)]:
        ap = rng.uniform(0, spread, n)
        ai = rng.uniform(0, spread, n)
        flags = rng.choice([-1, 0, 1], size=n, p=[0.1, 0.1, 0.8]).astype(np.int32)
        a = oracle.dbscan_compat(ap, ai, flags, 0.02, "grid")
        b = oracle.dbscan_compat(ap, ai, flags, 0.02, "bfs")
        assert np.array_equal(a, b)


def test_threaded_range_replays_equal_the_full_replays(refs):
    """The chunked, multi-threaded replays of the reference's kernels (the CPU
    baselines of bench.py) give the sequential full replay's results."""
    R = refs["lorenz"]
    kw = (10.0, 50, 0.01, [0.1, 0.1, 0.1], [20.0, 200.0], [1], 0, 1e4, 5.0, [10.0, 28.0, 8.0 / 3.0])
    assert np.array_equal(R.bifurcation(1, *kw)["counts"][7:43], R.bifurcation_range(1, *kw, 7, 43, nthreads=4))
    kb = (4.0, 24, 0.01, [0.0, 0.0, 27.0], [-30.0, 30.0, -30.0, 30.0], [0, 1], 0, 1e8, 5.0, [10.0, 24.0, 8.0 / 3.0])
    full, part = R.basins(*kb), R.basins_range(*kb, 100, 576, nthreads=4)
    for k in ("flags", "avg_peaks", "avg_intervals"):
        assert np.array_equal(np.asarray(full[k])[100:576], part[k]), k
    kl = (20.0, 0.1, 12, 0.01, 1e-8, [1.0, 1.0, 1.0], [0.1, 0.4, 2.0, 10.0], [0, 2], 5.0, [0.2, 0.2, 5.7])
    Rr = refs["rossler"]
    assert np.array_equal(Rr.lle(*kl)[5:130], Rr.lle_range(*kl, 5, 130, nthreads=4))
