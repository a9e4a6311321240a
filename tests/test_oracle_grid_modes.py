"""The oracle's grid modes on the CPU: sweeps over initial conditions,
log-scale axes and the step size reduce to the plain parameter sweep at each
grid point (size-independent properties), and the log-scale values follow the
legacy getValueByIdxLog formula (debri/cudaLibrary.cu:1191-1196)."""
import numpy as np

LORENZ = dict(values=[10.0, 28.0, 8 / 3])


def _point(o, r, k):
    c = int(r["counts"][k])
    return c, int(r["flags"][k]), r["peaks"][k, :max(c, 0)], r["intervals"][k, :max(c, 0)]


def _same(a, b):
    return a[0] == b[0] and a[1] == b[1] and np.array_equal(a[2], b[2]) and np.array_equal(a[3], b[3])


def test_log_axis_formula(oracle):
    v = oracle.log_axis(0.01, 100.0, 9)
    assert np.allclose(v, np.logspace(-2, 2, 9), rtol=1e-14, atol=0)
    f = oracle.log_axis(0.01, 100.0, 9, f32=True)
    assert np.all(f == f.astype(np.float32).astype(np.float64))
    assert np.allclose(f, v, rtol=1e-6)


def test_log_sweep_is_pointwise_linear_sweep(oracle):
    """Point k of a log-scale sweep equals a sweep whose range is [v_k, v_k]."""
    n = 12
    kw = dict(tMax=8.0, h=0.01, ic=[0.1, 0.1, 0.1], wv=0, maxValue=1e4, transientTime=4.0, **LORENZ)
    for mode in (oracle.GRID_LOG0, oracle.GRID_LOG0 | oracle.GRID_LOG_F32):
        vk = oracle.log_axis(20.0, 200.0, n, f32=bool(mode & oracle.GRID_LOG_F32))
        r = oracle.bifurcation_sweep(0, 1, mode, kw["tMax"], n, kw["h"], kw["ic"], [20.0, 200.0], [1], kw["wv"],
                                     kw["maxValue"], kw["transientTime"], kw["values"])
        for k in (0, 5, n - 1):
            s = oracle.bifurcation_sweep(0, 1, 0, kw["tMax"], 2, kw["h"], kw["ic"], [vk[k], vk[k]], [1], kw["wv"],
                                         kw["maxValue"], kw["transientTime"], kw["values"], cap=r["peaks"].shape[1])
            assert _same(_point(oracle, r, k), _point(oracle, s, 0)), (mode, k)


def test_state_sweep_is_pointwise_initial_condition(oracle):
    """Point k of a sweep over initial conditions equals the parameter sweep
    started from that initial condition."""
    n = 10
    r = oracle.bifurcation_sweep(0, 1, oracle.GRID_STATE, 8.0, n, 0.01, [0.1, 0.1, 0.1], [-5.0, 5.0], [2], 0, 1e4,
                                 4.0, LORENZ["values"])
    for k in (0, 3, n - 1):
        z = -5.0 + k * (10.0 / (n - 1))
        s = oracle.bifurcation_sweep(0, 1, 0, 8.0, 2, 0.01, [0.1, 0.1, z], [28.0, 28.0], [1], 0, 1e4, 4.0,
                                     LORENZ["values"], cap=r["peaks"].shape[1])
        assert _same(_point(oracle, r, k), _point(oracle, s, 0)), k


def test_step_sweep_constant_range_is_fixed_step(oracle):
    r = oracle.bifurcation_sweep(0, 1, 0, 8.0, 3, 0.0, [0.1, 0.1, 0.1], [0.01, 0.01], [oracle.MUT_STEP], 0, 1e4,
                                 4.0, LORENZ["values"])
    s = oracle.bifurcation(0, 1, 8.0, 3, 0.01, [0.1, 0.1, 0.1], [28.0, 28.0], [1], 0, 1e4, 4.0, LORENZ["values"],
                           cap=r["peaks"].shape[1])
    for k in range(3):
        assert _same(_point(oracle, r, k), _point(oracle, s, k))


def test_step_sweep_counts_follow_the_step(oracle):
    """A coarser step records fewer samples over the same tMax: intervals are
    in units of the point's own step, so periods agree across steps."""
    r = oracle.bifurcation_sweep(1, 1, oracle.GRID_LOG0, 200.0, 5, 0.0, [1.0, 1.0, 1.0], [0.002, 0.02],
                                 [oracle.MUT_STEP], 0, 1e4, 100.0, [0.2, 0.2, 2.5])
    periods = [np.median(r["intervals"][k, :r["counts"][k]]) for k in range(5) if r["counts"][k] > 2]
    assert len(periods) >= 4 and np.ptp(periods) < 0.2 * np.median(periods)


def test_lle_log_axis_is_pointwise(oracle):
    n = 6
    kw = dict(tMax=10.0, NT=0.5, h=0.01, eps=1e-6, ic=[0.1, 0.1, 0.1], transientTime=5.0, **LORENZ)
    r = oracle.lle_sweep(0, 1, oracle.GRID_LOG0, kw["tMax"], kw["NT"], n, kw["h"], kw["eps"], kw["ic"],
                         [10.0, 100.0], [1], kw["transientTime"], kw["values"])
    vk = oracle.log_axis(10.0, 100.0, n)
    for k in (0, 2, n - 1):
        s = oracle.lle_sweep(0, 1, 0, kw["tMax"], kw["NT"], 1, kw["h"], kw["eps"], kw["ic"], [vk[k], vk[k]], [1],
                             kw["transientTime"], kw["values"])
        assert r[k] == s[0]
