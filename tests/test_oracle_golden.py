"""The CPU oracle against the golden fixtures made by the reference's own code
(tests/golden/make_golden.py). Pins the oracle before anything is compared
with it."""
import numpy as np
import pytest

from conftest import golden, sweep_kwargs

SYS = {"lorenz": 0, "chameleon": 3, "sin3": 5}


@pytest.mark.parametrize("name", ["peaks_crafted", "peaks_random"])
def test_peak_finder_golden(oracle, name):
    g = golden(name)
    counts, pk, iv = oracle.peak_finder(g["data"], float(g["h"]), cap=g["data"].shape[1])
    assert np.array_equal(counts, g["counts"])
    for s, c in enumerate(counts):
        assert np.array_equal(pk[s, :c], g["peaks"][s, :c])
        assert np.array_equal(iv[s, :c], g["intervals"][s, :c])


def test_point_dbscan_golden(oracle):
    g = golden("point_dbscan")
    out = oracle.point_dbscan(g["intervals"], g["counts"], float(g["eps"]))
    assert np.array_equal(out, g["labels"])


@pytest.mark.parametrize("name", ["bif1d_lorenz", "bif1d_chameleon", "bif2d_lorenz", "bif2d_chameleon"])
def test_bifurcation_golden(oracle, name):
    g = golden(name)
    kw = sweep_kwargs(g)
    sysid = SYS[name.split("_")[1]]
    dim = int(g["dim"])
    o = oracle.bifurcation(sysid, dim, kw["tMax"], kw["nPts"], kw["h"], kw["ic"], kw["ranges"], kw["mut"], kw["wv"],
                           kw["maxValue"], kw["transientTime"], kw["values"], eps=float(g["eps"]))
    assert np.array_equal(o["counts"], g["counts"])
    for k, c in enumerate(o["counts"]):
        if c > 0:
            assert np.array_equal(o["peaks"][k, :c], g["peaks"][k, :c])
            assert np.array_equal(o["intervals"][k, :c], g["intervals"][k, :c])
        if c == -1:
            assert o["first"][k] == g["first"][k]
    if dim == 2:
        assert np.array_equal(o["labels"], g["labels"])


@pytest.mark.parametrize("name", ["basins_lorenz", "basins_sin3"])
def test_basins_golden(oracle, name):
    g = golden(name)
    kw = sweep_kwargs(g)
    o = oracle.basins_features(SYS[name.split("_")[1]], kw["tMax"], kw["nPts"], kw["h"], kw["ic"], kw["ranges"],
                               kw["mut"], kw["wv"], kw["maxValue"], kw["transientTime"], kw["values"])
    assert np.array_equal(o["flags"], g["flags"])
    assert np.array_equal(o["avg_peaks"], g["avg_peaks"])
    assert np.array_equal(o["avg_intervals"], g["avg_intervals"])
    for method in ("grid", "bfs"):
        lab = oracle.dbscan_compat(o["avg_peaks"], o["avg_intervals"], o["flags"], float(g["eps"]), method)
        assert np.array_equal(oracle.canonical_labels(lab), oracle.canonical_labels(g["labels"]))


def test_dbscan_compat_golden(oracle):
    g = golden("dbscan_compat")
    for method in ("grid", "bfs"):
        lab = oracle.dbscan_compat(g["avg_peaks"], g["avg_intervals"], g["flags"], float(g["eps"]), method)
        assert np.array_equal(oracle.canonical_labels(lab), oracle.canonical_labels(g["labels"]))
        assert np.array_equal(lab == 0, g["labels"] == 0)
        assert np.array_equal(lab < 0, g["labels"] < 0)


def test_dbscan_sklearn_golden(oracle):
    g = golden("dbscan_sklearn")
    lab = oracle.dbscan(g["X"], float(g["eps"]), int(g["min_pts"]))
    assert np.array_equal(lab, g["labels"])


def test_lle_golden(oracle):
    g = golden("lle_rossler")
    o = oracle.lle2d(1, float(g["tMax"]), float(g["NT"]), int(g["nPts"]), float(g["h"]), float(g["eps"]), g["ic"],
                     g["ranges"], g["mut"], float(g["transientTime"]), g["values"])
    fin = np.isfinite(g["lle"])
    assert np.array_equal(fin, np.isfinite(o))
    # the reference sums float logs (__logf); the oracle sums FP64 logs
    assert np.max(np.abs(o[fin] - g["lle"][fin])) < 1e-6


def test_basin_features_dbscan_matches_sklearn(oracle):
    """The oracle's DBSCAN on real basin features (Lorenz rho=24) equals
    scikit-learn's labels."""
    sk = pytest.importorskip("sklearn.cluster")
    lab, F, feat = oracle.basins_dbscan(0, 6.0, 30, 0.01, [0.0, 0.0, 27.0], [-30.0, 30.0, -30.0, 30.0], [0, 1], 0,
                                        1e8, 10.0, [10.0, 24.0, 8 / 3], eps=0.05, min_pts=8)
    m = feat["flags"] != 0
    ref = sk.DBSCAN(eps=0.05, min_samples=8).fit(F[m]).labels_
    assert np.array_equal(lab[m], ref)
    assert np.all(lab[~m] == -2)


# the legacy library's kernels (tests/golden/make_golden.py legacy_fixtures); its hard-wired system is sin3's arithmetic
@pytest.mark.parametrize("regime", ["fixed", "bound"])
@pytest.mark.parametrize("dim", [1, 2])
def test_legacy_ic_bifurcation_golden(oracle, regime, dim):
    g = golden(f"legacy_ic_bif{dim}d_{regime}")
    o = oracle.bifurcation_sweep(5, dim, oracle.GRID_STATE | oracle.GRID_LEGACY_LOOP, float(g["tMax"]),
                                 int(g["nPts"]), float(g["h"]), g["ic"], g["ranges"], g["mut"], int(g["wv"]),
                                 float(g["maxValue"]), float(g["transientTime"]), g["values"],
                                 preScaller=int(g["preScaller"]), eps=float(g["eps"]))
    assert np.array_equal(o["counts"], g["counts"])
    for k, c in enumerate(g["counts"]):
        assert np.array_equal(o["peaks"][k, :max(c, 0)], g["peaks"][k, :max(c, 0)])
        if dim == 2:
            assert np.array_equal(o["intervals"][k, :max(c, 0)], g["intervals"][k, :max(c, 0)])
    if dim == 2:
        assert np.array_equal(o["labels"], g["labels"])


@pytest.mark.parametrize("regime", ["fixed", "bound"])
def test_legacy_basins_golden(oracle, regime):
    g = golden(f"legacy_basins_{regime}")
    o = oracle.basins_features(5, float(g["tMax"]), int(g["nPts"]), float(g["h"]), g["ic"], g["ranges"], g["mut"],
                               int(g["wv"]), float(g["maxValue"]), float(g["transientTime"]), g["values"],
                               preScaller=int(g["preScaller"]))
    assert np.array_equal(o["flags"], g["flags"])
    assert np.array_equal(o["avg_peaks"], g["avg_peaks"]) and np.array_equal(o["avg_intervals"], g["avg_intervals"])


@pytest.mark.parametrize("regime", ["fixed", "bound"])
def test_legacy_step_sweep_golden(oracle, regime):
    g = golden(f"legacy_step_sweep_{regime}")
    o = oracle.bifurcation_sweep(5, 1, oracle.GRID_LOG0 | oracle.GRID_LOG_F32 | oracle.GRID_LEGACY_LOOP,
                                 float(g["tMax"]), int(g["nPts"]), 0.0, g["ic"], g["ranges"], [oracle.MUT_STEP],
                                 int(g["wv"]), float(g["maxValue"]), float(g["transientTime"]), g["values"],
                                 preScaller=int(g["preScaller"]))
    assert np.array_equal(np.maximum(o["counts"], 0), g["counts"])
    for k, c in enumerate(g["counts"]):
        assert np.array_equal(o["peaks"][k, :c], g["peaks"][k, :c])


def test_legacy_lle_golden(oracle):
    g = golden("legacy_lle")
    a = (float(g["tMax"]), float(g["NT"]))
    rest = (float(g["h"]), float(g["eps"]), g["ic"])
    u = g["uniforms"]
    draws = np.array([[float(u[p + k]) - 0.5 for k in range(3)] for p in range(32)])
    assert np.array_equal(oracle.lle_sweep_legacy(5, 1, 0, *a, 32, *rest, [0.1, 0.6], [1], 0.0,
                                                  float(g["transientTime"]), g["values"], draws=draws), g["lle1d"])
    assert np.array_equal(oracle.lle_sweep_legacy(5, 1, oracle.GRID_STATE, *a, 32, *rest, [-3.0, 3.0], [0], 3.0,
                                                  float(g["transientTime"]), g["values"]), g["lle1dic"])
    assert np.array_equal(oracle.lyapunov_spectrum_legacy(5, 1, 0, *a, 12, *rest, [0.1, 0.6], [1], 0.0,
                                                          float(g["transientTime"]), g["values"]), g["ls1d"])
