"""The drop-in plug-in slot: a header in the reference's systems.cuh format
(SIZE_X, SIZE_A, CALC_DISCRETE_MODEL) compiled into the engine at build time
as CHAOS_SYS_USER runs through the same kernels as the built-in systems."""
import ctypes as C

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

# A plug-in written the way the reference's systems.cuh writes one (plain
# FP64 arithmetic, one explicit Euler step of the Lorenz flow).
EULER_LORENZ = r"""
#pragma once
#include "cuda_runtime.h"
__device__ inline void calcDiscreteModel(double* X, const double* a, double h) {
    double dx = a[0] * (X[1] - X[0]);
    double dy = X[0] * (a[1] - X[2]) - X[1];
    double dz = X[0] * X[1] - a[2] * X[2];
    X[0] = X[0] + h * dx;
    X[1] = X[1] + h * dy;
    X[2] = X[2] + h * dz;
}
#define SIZE_X 3
#define SIZE_A 3
#define CALC_DISCRETE_MODEL(X, a, h) calcDiscreteModel(X, a, h)
"""


def _load(path):
    from chaoslibrary_gb300 import _native as N

    L = C.CDLL(str(path))
    for name, (args, res) in N._SIGS.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    return L


@pytest.fixture(scope="module")
def user_libs(tmp_path_factory):
    from chaoslibrary_gb300 import build as B

    d = tmp_path_factory.mktemp("user")
    (d / "euler_lorenz.cuh").write_text(EULER_LORENZ)
    rk4 = B.build(user_systems=str(ROOT / "chaoslibrary_gb300/plugins/lorenz_rk4.cuh"), lib=d / "rk4/lib.so",
                  build_dir=d / "rk4/b")
    euler = B.build(user_systems=str(d / "euler_lorenz.cuh"), lib=d / "euler/lib.so", build_dir=d / "euler/b")
    return _load(rk4), _load(euler)


def _bif(L, system, n=48):
    from chaoslibrary_gb300 import _native as N

    ex = N.Exec(N.FP64, N.MEM_HOST, None, -1)
    counts = np.zeros(n, np.int32)
    flags = np.zeros(n, np.int32)
    first = np.zeros(n)
    cap = 500
    pk = np.zeros((n, cap))
    iv = np.zeros((n, cap))
    d = lambda a: np.ascontiguousarray(a, np.float64).ctypes.data
    keep = [np.array([0.1, 0.1, 0.1]), np.array([20.0, 200.0]), np.array([1], np.int32), np.array([10.0, 28.0, 8 / 3])]
    rc = L.chaos_bifurcation1d(C.byref(ex), system, 20.0, n, 0.01, 3, keep[0].ctypes.data, keep[1].ctypes.data,
                               keep[2].ctypes.data, 0, 1e4, 10.0, keep[3].ctypes.data, 3, 1, cap, counts.ctypes.data,
                               flags.ctypes.data, first.ctypes.data, pk.ctypes.data, iv.ctypes.data)
    assert rc == 0, L.chaos_last_error()
    return counts, flags, pk, iv


def test_user_plugin_equals_builtin(engine, user_libs):
    """plugins/lorenz_rk4.cuh compiled in as CHAOS_SYS_USER reproduces the
    built-in Lorenz RK4 bit for bit (same arithmetic, other kernel)."""
    rk4, _ = user_libs
    nx, na = C.c_int(), C.c_int()
    assert rk4.chaos_system_info(15, C.byref(nx), C.byref(na)) == 0 and (nx.value, na.value) == (3, 3)
    u = _bif(rk4, 15)
    b = _bif(rk4, 0)
    for x, y in zip(u, b):
        assert np.array_equal(x, y)
    # the main library has no user plug-in
    assert engine.lib().chaos_system_info(15, C.byref(nx), C.byref(na)) == -6


def test_reference_style_plugin_trajectory(user_libs):
    """A plug-in in the reference's plain style integrates exactly as the
    same FP64 operations evaluated in numpy (no contraction on the device)."""
    from chaoslibrary_gb300 import _native as N

    _, euler = user_libs
    x0 = np.array([[0.1, 0.2, 0.3], [1.0, -1.0, 20.0]])
    a = np.array([[10.0, 28.0, 8 / 3], [10.0, 28.0, 8 / 3]])
    steps = 500
    out = np.zeros((2, steps + 1, 3))
    ex = N.Exec(N.FP64, N.MEM_HOST, None, -1)
    rc = euler.chaos_trajectory(C.byref(ex), 15, 2, x0.ctypes.data, a.ctypes.data, 0.01, steps, out.ctypes.data)
    assert rc == 0, euler.chaos_last_error()
    for t in range(2):
        X = x0[t].copy()
        s, r, b = a[t]
        h = 0.01
        for k in range(steps + 1):
            assert np.array_equal(out[t, k], X), k
            dx = s * (X[1] - X[0])
            dy = X[0] * (r - X[2]) - X[1]
            dz = X[0] * X[1] - b * X[2]
            X = np.array([X[0] + h * dx, X[1] + h * dy, X[2] + h * dz])
