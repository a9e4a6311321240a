"""CHAOS_FF32 (float-float orbit, exact FP32 twin difference, exact
power-of-two renormalisation) against the FP64 engine, which the parity tests
pin to the oracle and the reference's own code bit for bit.

Tolerances, stated:
* trajectories: FF within 1e-12 of the state's norm of FP64 over 100 steps
  (1 time unit) of Lorenz, Rossler and Chen; FP32 is ~1e-6 there;
* LLE over a 2-time-unit horizon (no chaotic amplification): FF within 5e-6
  of FP64 (FP32: 2e-4). The bound is set by FP64, not FF: the FP64 twin is a
  full second trajectory 1e-8 away, so its difference x - p loses
  ulp(x) / eps ~ 1e-7 of its value to cancellation every step, while the FF
  path carries the difference exactly;
* LLE over the benchmark's full horizon on a 128 x 128 map of the
  benchmark's Rossler ranges: the FF map's median and 90th-percentile error
  against FP64 at most 1.25x the FP64 map's own spread (FP64 started 1e-13
  away in x: the finite-time LLE's sensitivity), and >= 99.9 % of the regular
  points (FP64 LLE < 0.005) within 1e-3;
* FF results do not depend on the launch shape (one or two points per
  thread: bit-identical), and chaos_lle_sweep equals chaos_lle2d bit for bit;
* the FP32 map's three stretch measurements (CHAOS_TUNE_LLE_RENORM) agree to
  1e-3 everywhere and 1e-6 at the median: the FP32 error is the FP32 orbit's."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROSS = dict(tMax=500.0, NT=0.1, h=0.01, eps=1e-8, initialConditions=[1.0, 1.0, 1.0],
            ranges=[0.1, 0.4, 2.0, 10.0], indicesOfMutVars=[0, 2], transientTime=50.0, values=[0.2, 0.2, 5.7])


@pytest.mark.parametrize("system, a, scale", [("lorenz", [10.0, 28.0, 8 / 3], 15.0),
                                              ("rossler", [0.2, 0.2, 5.7], 5.0),
                                              ("chen", [35.0, 3.0, 28.0], 15.0)])
def test_ff_trajectory_tracks_fp64(engine, system, a, scale):
    rng = np.random.default_rng(3)
    x0 = rng.uniform(-scale, scale, size=(256, 3))
    t64 = engine.trajectory(system, x0, np.array([a]), 0.01, 100, precision=engine.FP64)
    tff = engine.trajectory(system, x0, np.array([a]), 0.01, 100, precision=engine.FF32)
    t32 = engine.trajectory(system, x0, np.array([a]), 0.01, 100, precision=engine.FP32)
    nrm = np.linalg.norm(t64, axis=2)
    err_ff = np.max(np.linalg.norm(tff - t64, axis=2) / nrm)
    err_32 = np.max(np.linalg.norm(t32 - t64, axis=2) / nrm)
    assert err_ff < 1e-12, err_ff
    assert err_32 > 1e3 * err_ff  # the FF orbit is a different class of accuracy


def test_ff_lle_short_horizon_matches_fp64(engine):
    kw = dict(ROSS, tMax=2.0, transientTime=1.0, nPts=32)
    l64 = engine.lle2d("rossler", precision=engine.FP64, **kw)
    lff = engine.lle2d("rossler", precision=engine.FF32, **kw)
    fin = np.isfinite(l64)
    assert fin.all() and np.isfinite(lff).all()
    assert np.max(np.abs(lff - l64)) < 5e-6


def test_ff_lle_map_within_fp64_self_spread(engine):
    kw = dict(ROSS, nPts=128)
    a = engine.lle2d("rossler", precision=engine.FP64, **kw)
    p13 = engine.lle2d("rossler", precision=engine.FP64, **dict(kw, initialConditions=[1.0 + 1e-13, 1.0, 1.0]))
    ff = engine.lle2d("rossler", precision=engine.FF32, **kw)
    fin = np.isfinite(a) & np.isfinite(p13) & np.isfinite(ff)
    assert fin.mean() > 0.9
    d_self, d_ff = np.abs(p13 - a)[fin], np.abs(ff - a)[fin]
    assert np.median(d_ff) <= 1.25 * np.median(d_self), (np.median(d_ff), np.median(d_self))
    assert np.percentile(d_ff, 90) <= 1.25 * np.percentile(d_self, 90)
    reg = a[fin] < 0.005
    assert reg.sum() > 1000
    assert np.mean(d_ff[reg] <= 1e-3) >= 0.999


def test_ff_shape_and_sweep_do_not_change_results(engine):
    kw = dict(ROSS, tMax=20.0, transientTime=5.0, nPts=33)  # odd count: the last pair has one point
    old = engine.get_tuning(engine.TUNE_FF_PAIRS)
    try:
        engine.set_tuning(engine.TUNE_FF_PAIRS, 1)
        pairs = engine.lle2d("rossler", precision=engine.FF32, **kw)
        engine.set_tuning(engine.TUNE_FF_PAIRS, 0)
        single = engine.lle2d("rossler", precision=engine.FF32, **kw)
    finally:
        engine.set_tuning(engine.TUNE_FF_PAIRS, old)
    assert np.array_equal(pairs, single, equal_nan=True)
    sweep = engine.lle_sweep("rossler", 2, kw["tMax"], kw["NT"], kw["nPts"], kw["h"], kw["eps"],
                             kw["initialConditions"], kw["ranges"], kw["indicesOfMutVars"], kw["transientTime"],
                             kw["values"], precision=engine.FF32)
    assert np.array_equal(sweep, pairs, equal_nan=True)


@pytest.mark.parametrize("system, values, ranges, mut, tol", [
    ("lorenz", [10.0, 28.0, 8 / 3], [20.0, 60.0, 5.0, 15.0], [1, 0], 3e-4),
    ("chen", [35.0, 3.0, 28.0], [20.0, 30.0, 30.0, 40.0], [2, 0], 1e-3)])
def test_ff_lle_other_systems_short_horizon(engine, system, values, ranges, mut, tol):
    """One time unit of Lorenz and Chen, whose short-time stretch rates reach
    4-6: the FP64 map's own twin cancellation (|x| up to ~60 against eps
    1e-8) is ~1e-4 here, so the bound is looser than Rossler's."""
    kw = dict(tMax=1.0, NT=0.1, h=0.01, eps=1e-8, initialConditions=[1.0, 1.0, 1.0], ranges=ranges,
              indicesOfMutVars=mut, transientTime=0.5, values=values, nPts=16)
    l64 = engine.lle2d(system, precision=engine.FP64, **kw)
    lff = engine.lle2d(system, precision=engine.FF32, **kw)
    assert np.all(np.isfinite(lff))
    assert np.max(np.abs(lff - l64)) < tol


def test_fp32_stretch_modes_agree(engine):
    kw = dict(ROSS, nPts=64)
    old = engine.get_tuning(engine.TUNE_LLE_RENORM)
    maps = []
    try:
        for mode in (0, 1, 2):
            engine.set_tuning(engine.TUNE_LLE_RENORM, mode)
            maps.append(engine.lle2d("rossler", precision=engine.FP32, **kw))
    finally:
        engine.set_tuning(engine.TUNE_LLE_RENORM, old)
    fin = np.isfinite(maps[0]) & np.isfinite(maps[1]) & np.isfinite(maps[2])
    for m in maps[1:]:
        d = np.abs(m - maps[0])[fin]
        assert d.max() < 1e-3 and np.median(d) < 1e-6
