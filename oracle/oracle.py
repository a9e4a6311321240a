"""ctypes front end of the CPU oracle (and of the host build of the reference).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` as the reference result. The engine package never
imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
SRC = HERE / "chaos_oracle.cpp"
REF_DIR = HERE / "_ref"

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")

SYSTEMS = {"lorenz": 0, "rossler": 1, "chen": 2, "chameleon": 3, "rossler_cd": 4, "sin3": 5, "sin2": 6,
           "memristor": 7}


def build(force: bool = False) -> Path:
    deps = [SRC, HERE.parent / "chaoslibrary_gb300" / "csrc" / "systems.h"]
    if not force and LIB.exists() and all(LIB.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return LIB
    tmp = LIB.with_suffix(f".{os.getpid()}.tmp")
    subprocess.run(["g++", "-O3", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
                    str(SRC), "-o", str(tmp)], check=True)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        _lib = C.CDLL(str(build()))
        L = _lib
        L.orc_steps.argtypes = [C.c_int, _dp, _dp, C.c_double, C.c_int]
        L.orc_trajectory.argtypes = [C.c_int, _dp, _dp, C.c_double, C.c_int, _dp]
        L.orc_peak_finder.argtypes = [_dp, C.c_int, C.c_int, C.c_double, C.c_int, _ip, _dp, _dp]
        L.orc_point_dbscan.argtypes = [_dp, _ip, C.c_int, C.c_int, C.c_double, _ip]
        L.orc_bifurcation.argtypes = [C.c_int, C.c_int, C.c_double, C.c_int, C.c_double, _dp, _dp, _ip, C.c_int,
                                      C.c_double, C.c_double, _dp, C.c_int, C.c_double, C.c_int, C.c_longlong,
                                      C.c_longlong, _ip, _ip, _dp, _dp, _dp, C.c_void_p, C.c_int]
        L.orc_bifurcation_sweep.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_double, _dp, _dp,
                                            _ip, C.c_int, C.c_double, C.c_double, _dp, C.c_int, C.c_double, C.c_int,
                                            C.c_longlong, C.c_longlong, _ip, _ip, _dp, _dp, _dp, C.c_void_p,
                                            C.c_int]
        L.orc_lle2d.argtypes = [C.c_int, C.c_double, C.c_double, C.c_int, C.c_double, C.c_double, _dp, _dp, _ip,
                                C.c_double, _dp, C.c_longlong, C.c_longlong, _dp, C.c_int]
        for name in ("orc_lle_sweep", "orc_lyapunov_spectrum"):
            getattr(L, name).argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.c_double,
                                         C.c_double, _dp, _dp, _ip, C.c_double, _dp, C.c_longlong, C.c_longlong,
                                         _dp, C.c_int]
        L.orc_lle_sweep_legacy.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.c_double,
                                           C.c_double, _dp, _dp, _ip, C.c_double, C.c_double, _dp, C.c_void_p,
                                           C.c_longlong, C.c_longlong, _dp, C.c_int]
        L.orc_lyapunov_spectrum_legacy.argtypes = L.orc_lle_sweep_legacy.argtypes
        L.orc_basins_features.argtypes = [C.c_int, C.c_double, C.c_int, C.c_double, _dp, _dp, _ip, C.c_int,
                                          C.c_double, C.c_double, _dp, C.c_int, C.c_longlong, C.c_longlong, _ip,
                                          _dp, _dp, C.c_void_p, C.c_void_p, C.c_int]
        L.orc_dbscan_compat_bfs.argtypes = [_dp, _dp, _ip, C.c_int, C.c_double, _ip]
        L.orc_dbscan_compat_grid.argtypes = [_dp, _dp, _ip, C.c_int, C.c_double, _ip]
        L.orc_dbscan.argtypes = [_dp, C.c_int, C.c_int, C.c_double, C.c_int, C.c_void_p, _ip]
    return _lib


def _d(x):
    return np.ascontiguousarray(x, dtype=np.float64)


def _i(x):
    return np.ascontiguousarray(x, dtype=np.int32)


def steps(system: int, x0, a, h: float, n: int) -> np.ndarray:
    x = _d(x0).copy()
    lib().orc_steps(system, x, _d(a), h, n)
    return x


def trajectory(system: int, x0, a, h: float, n: int) -> np.ndarray:
    x0 = _d(x0)
    out = np.zeros((n, x0.size), np.float64)
    lib().orc_trajectory(system, x0, _d(a), h, n, out)
    return out


def peak_finder(data, h: float, cap: int | None = None):
    data = _d(np.atleast_2d(data))
    n, ln = data.shape
    cap = cap or max(ln, 1)
    counts = np.zeros(n, np.int32)
    pk = np.zeros((n, cap), np.float64)
    iv = np.zeros((n, cap), np.float64)
    lib().orc_peak_finder(data, n, ln, h, cap, counts, pk, iv)
    return counts, pk, iv


def point_dbscan(intervals, counts, eps: float) -> np.ndarray:
    intervals = _d(np.atleast_2d(intervals))
    counts = _i(counts)
    out = np.zeros(counts.size, np.int32)
    lib().orc_point_dbscan(intervals, counts, counts.size, intervals.shape[1], eps, out)
    return out


def bifurcation(system: int, dim: int, tMax, nPts, h, ic, ranges, mut, wv, maxValue, transientTime, values,
                preScaller=1, eps=0.0, cap=None, p_begin=0, p_end=-1, nthreads=0):
    """Per point: counts, flags, first, peaks[cap], intervals[cap], labels (dim 2)."""
    B = int(tMax / h / preScaller)
    total = nPts ** dim
    p_end = total if p_end < 0 else p_end
    n = p_end - p_begin
    cap = cap or max(B // 2 + 1, 1)
    counts = np.zeros(n, np.int32)
    flags = np.zeros(n, np.int32)
    first = np.zeros(n, np.float64)
    pk = np.zeros((n, cap), np.float64)
    iv = np.zeros((n, cap), np.float64)
    labels = np.zeros(n, np.int32)
    rc = lib().orc_bifurcation(system, dim, tMax, nPts, h, _d(ic), _d(ranges), _i(mut), wv, maxValue,
                               transientTime, _d(values), preScaller, eps, cap, p_begin, p_end, counts, flags,
                               first, pk, iv, labels.ctypes.data if dim == 2 else None, nthreads)
    if rc:
        raise ValueError("bad bifurcation arguments")
    return dict(counts=counts, flags=flags, first=first, peaks=pk, intervals=iv,
                labels=labels if dim == 2 else None)


# grid modes (the engine's CHAOS_GRID_* bits) and the step-size axis marker
GRID_STATE, GRID_LOG0, GRID_LOG1, GRID_LOG_F32, GRID_LEGACY_LOOP = 1, 2, 4, 8, 16
MUT_STEP = -1


def bifurcation_sweep(system: int, dim: int, grid_mode: int, tMax, nPts, h, ic, ranges, mut, wv, maxValue,
                      transientTime, values, preScaller=1, eps=0.0, cap=None, p_begin=0, p_end=-1, nthreads=0):
    """bifurcation() over initial conditions, log-scale axes or the step size
    (mut[0] == MUT_STEP, dim 1). cap defaults to the largest B/2 + 1 on the grid."""
    if mut[0] == MUT_STEP:
        h_min = min(ranges[0], ranges[1]) * (1.0 - 1e-9)
        B = int(tMax / h_min / preScaller)
    else:
        B = int(tMax / h / preScaller)
    total = nPts ** dim
    p_end = total if p_end < 0 else p_end
    n = p_end - p_begin
    cap = cap or max(B // 2 + 1, 1)
    counts = np.zeros(n, np.int32)
    flags = np.zeros(n, np.int32)
    first = np.zeros(n, np.float64)
    pk = np.zeros((n, cap), np.float64)
    iv = np.zeros((n, cap), np.float64)
    labels = np.zeros(n, np.int32)
    rc = lib().orc_bifurcation_sweep(system, dim, grid_mode, tMax, nPts, h, _d(ic), _d(ranges), _i(mut), wv,
                                     maxValue, transientTime, _d(values), preScaller, eps, cap, p_begin, p_end,
                                     counts, flags, first, pk, iv, labels.ctypes.data if dim == 2 else None,
                                     nthreads)
    if rc:
        raise ValueError("bad bifurcation arguments")
    return dict(counts=counts, flags=flags, first=first, peaks=pk, intervals=iv,
                labels=labels if dim == 2 else None)


def log_axis(r0: float, r1: float, nPts: int, f32: bool = False) -> np.ndarray:
    """Values of a log-scale axis, computed as the oracle's C code does."""
    l0 = np.log10(r0)
    x = l0 + np.arange(nPts, dtype=np.float64) * ((np.log10(r1) - l0) / (nPts - 1))
    return np.power(np.float32(10.0), x.astype(np.float32)).astype(np.float64) if f32 else np.power(10.0, x)


def lle2d(system: int, tMax, NT, nPts, h, eps, ic, ranges, mut, transientTime, values, p_begin=0, p_end=-1,
          nthreads=0) -> np.ndarray:
    total = nPts * nPts
    p_end = total if p_end < 0 else p_end
    out = np.zeros(p_end - p_begin, np.float64)
    rc = lib().orc_lle2d(system, tMax, NT, nPts, h, eps, _d(ic), _d(ranges), _i(mut), transientTime, _d(values),
                         p_begin, p_end, out, nthreads)
    if rc:
        raise ValueError("bad LLE arguments")
    return out


def lle_sweep(system: int, dim, grid_mode, tMax, NT, nPts, h, eps, ic, ranges, mut, transientTime, values,
              p_begin=0, p_end=-1, nthreads=0) -> np.ndarray:
    total = nPts * nPts if dim == 2 else nPts
    p_end = total if p_end < 0 else p_end
    out = np.zeros(p_end - p_begin, np.float64)
    rc = lib().orc_lle_sweep(system, dim, grid_mode, tMax, NT, nPts, h, eps, _d(ic), _d(ranges), _i(mut),
                             transientTime, _d(values), p_begin, p_end, out, nthreads)
    if rc:
        raise ValueError("bad LLE arguments")
    return out


def lle_sweep_legacy(system: int, dim, grid_mode, tMax, NT, nPts, h, eps, ic, ranges, mut, maxValue, transientTime,
                     values, draws=None, p_begin=0, p_end=-1, nthreads=0) -> np.ndarray:
    """The legacy LLE kernels' scheme (orc_lle_sweep_legacy); draws: raw twin
    draws [points, SIZE_X] (required for parameter grids)."""
    total = nPts * nPts if dim == 2 else nPts
    p_end = total if p_end < 0 else p_end
    out = np.zeros(p_end - p_begin, np.float64)
    dr = None if draws is None else _d(draws).ravel()
    rc = lib().orc_lle_sweep_legacy(system, dim, grid_mode, tMax, NT, nPts, h, eps, _d(ic), _d(ranges), _i(mut),
                                    maxValue, transientTime, _d(values), None if dr is None else dr.ctypes.data,
                                    p_begin, p_end, out, nthreads)
    if rc:
        raise ValueError("bad legacy LLE arguments")
    return out


def lyapunov_spectrum_legacy(system: int, dim, grid_mode, tMax, NT, nPts, h, eps, ic, ranges, mut, maxValue,
                             transientTime, values, draws=None, p_begin=0, p_end=-1, nthreads=0) -> np.ndarray:
    """The legacy spectrum kernel's scheme (orc_lyapunov_spectrum_legacy):
    [points, SIZE_X]; draws: raw twin draws [points, SIZE_X, SIZE_X]."""
    total = nPts * nPts if dim == 2 else nPts
    p_end = total if p_end < 0 else p_end
    nx = len(ic)
    out = np.zeros((p_end - p_begin) * nx, np.float64)
    dr = None if draws is None else _d(draws).ravel()
    rc = lib().orc_lyapunov_spectrum_legacy(system, dim, grid_mode, tMax, NT, nPts, h, eps, _d(ic), _d(ranges),
                                            _i(mut), maxValue, transientTime, _d(values),
                                            None if dr is None else dr.ctypes.data, p_begin, p_end, out, nthreads)
    if rc:
        raise ValueError("bad legacy spectrum arguments")
    return out.reshape(p_end - p_begin, nx)


def lyapunov_spectrum(system: int, dim, grid_mode, tMax, NT, nPts, h, eps, ic, ranges, mut, transientTime,
                      values, p_begin=0, p_end=-1, nthreads=0) -> np.ndarray:
    """[points, SIZE_X] exponents."""
    total = nPts * nPts if dim == 2 else nPts
    p_end = total if p_end < 0 else p_end
    nx = len(ic)
    out = np.zeros((p_end - p_begin) * nx, np.float64)
    rc = lib().orc_lyapunov_spectrum(system, dim, grid_mode, tMax, NT, nPts, h, eps, _d(ic), _d(ranges), _i(mut),
                                     transientTime, _d(values), p_begin, p_end, out, nthreads)
    if rc:
        raise ValueError("bad spectrum arguments")
    return out.reshape(-1, nx)


def basins_features(system: int, tMax, nPts, h, ic, ranges, mut, wv, maxValue, transientTime, values,
                    preScaller=1, p_begin=0, p_end=-1, nthreads=0):
    total = nPts * nPts
    p_end = total if p_end < 0 else p_end
    n = p_end - p_begin
    flags = np.zeros(n, np.int32)
    ap = np.zeros(n, np.float64)
    ai = np.zeros(n, np.float64)
    counts = np.zeros(n, np.int32)
    last = np.zeros(n, np.float64)
    rc = lib().orc_basins_features(system, tMax, nPts, h, _d(ic), _d(ranges), _i(mut), wv, maxValue,
                                   transientTime, _d(values), preScaller, p_begin, p_end, flags, ap, ai,
                                   counts.ctypes.data, last.ctypes.data, nthreads)
    if rc:
        raise ValueError("bad basins arguments")
    return dict(flags=flags, avg_peaks=ap, avg_intervals=ai, counts=counts, last=last)


def basin_feature_matrix(feat: dict):
    """(amplitude, kept peak count, mean interval) per point -- the mean peak,
    or the last sample without peaks -- min-max scaled over flag != 0 points,
    (f - lo) * (1 / (hi - lo)); returns (features n x 3, mask)."""
    c = feat["counts"]
    f = np.stack([np.where(c > 0, feat["avg_peaks"], feat["last"]), c.astype(np.float64),
                  np.where(c > 0, feat["avg_intervals"], 0.0)], axis=1)
    mask = (feat["flags"] != 0).astype(np.int32)
    out = np.zeros_like(f)
    if mask.any():
        lo = f[mask == 1].min(axis=0)
        hi = f[mask == 1].max(axis=0)
        for d in range(3):
            if hi[d] > lo[d]:
                out[:, d] = np.where(mask == 1, (f[:, d] - lo[d]) * (1.0 / (hi[d] - lo[d])), 0.0)
    return out, mask


def basins_dbscan(system: int, tMax, nPts, h, ic, ranges, mut, wv, maxValue, transientTime, values, preScaller=1,
                  eps=0.05, min_pts=8, nthreads=0):
    feat = basins_features(system, tMax, nPts, h, ic, ranges, mut, wv, maxValue, transientTime, values,
                           preScaller=preScaller, nthreads=nthreads)
    F, mask = basin_feature_matrix(feat)
    return dbscan(F, eps, min_pts, mask=mask), F, feat


def dbscan_compat(avg_peaks, avg_intervals, flags, eps: float, method: str = "grid") -> np.ndarray:
    ap, ai, fl = _d(avg_peaks), _d(avg_intervals), _i(flags)
    out = np.zeros(ap.size, np.int32)
    fn = lib().orc_dbscan_compat_grid if method == "grid" else lib().orc_dbscan_compat_bfs
    fn(ap, ai, fl, ap.size, eps, out)
    return out


def dbscan(features, eps: float, min_pts: int, mask=None) -> np.ndarray:
    f = _d(np.atleast_2d(features))
    n, d = f.shape
    out = np.zeros(n, np.int32)
    m = None if mask is None else _i(mask)
    lib().orc_dbscan(f, n, d, eps, min_pts, None if m is None else m.ctypes.data, out)
    return out


# ---------------------------------------------------------------------------
# the reference's own code compiled for the host (only where the sources are)

class RefLib:
    """Host build of the reference per-thread code for one plug-in system."""

    def __init__(self, name: str):
        path = REF_DIR / f"libref_{name}.so"
        if not path.exists():
            raise FileNotFoundError(path)
        L = self.L = C.CDLL(str(path))
        L.refh_steps.argtypes = [_dp, _dp, C.c_double, C.c_int]
        L.refh_peak_finder.argtypes = [_dp, C.c_int, _dp, _dp, C.c_double]
        L.refh_point_dbscan.argtypes = [_dp, _dp, _dp, C.c_int, C.c_int, C.c_double]
        L.refh_bifurcation.argtypes = [C.c_int, C.c_double, C.c_int, C.c_double, C.c_int, _dp, _dp, _ip, C.c_int,
                                       C.c_double, C.c_double, _dp, C.c_int, C.c_int, C.c_double, _ip, _dp, _dp,
                                       C.c_void_p, C.c_void_p]
        L.refh_basins.argtypes = [C.c_double, C.c_int, C.c_double, C.c_int, _dp, _dp, _ip, C.c_int, C.c_double,
                                  C.c_double, _dp, C.c_int, C.c_int, _ip, _dp, _dp, _dp]
        L.refh_basins_dbscan.argtypes = [_dp, _dp, _ip, _ip, C.c_int, C.c_double]
        L.refh_lle.argtypes = [C.c_double, C.c_double, C.c_int, C.c_double, C.c_double, C.c_int, _dp, _dp, _ip,
                               C.c_double, _dp, C.c_int, _dp]
        L.refh_bifurcation_range.argtypes = [C.c_int, C.c_double, C.c_int, C.c_double, C.c_int, _dp, _dp, _ip,
                                             C.c_int, C.c_double, C.c_double, _dp, C.c_int, C.c_int, C.c_longlong,
                                             C.c_longlong, _ip, C.c_int]
        L.refh_basins_range.argtypes = [C.c_double, C.c_int, C.c_double, C.c_int, _dp, _dp, _ip, C.c_int,
                                        C.c_double, C.c_double, _dp, C.c_int, C.c_int, C.c_longlong, C.c_longlong,
                                        _ip, _dp, _dp, C.c_int]
        L.refh_lle_range.argtypes = [C.c_double, C.c_double, C.c_int, C.c_double, C.c_double, C.c_int, _dp, _dp,
                                     _ip, C.c_double, _dp, C.c_int, C.c_longlong, C.c_longlong, _dp, C.c_int]

    def steps(self, x0, a, h, n):
        x = _d(x0).copy()
        self.L.refh_steps(x, _d(a), h, n)
        return x

    def peak_finder(self, series, h):
        d = _d(series).copy()
        pk = np.zeros(max(d.size, 1))
        tm = np.zeros(max(d.size, 1))
        c = self.L.refh_peak_finder(d, d.size, pk, tm, h)
        return c, pk[:max(c, 0)], tm[:max(c, 0)]

    def point_dbscan(self, peaks, intervals, count, size_of_block, eps):
        data = np.zeros(size_of_block)
        iv = np.zeros(size_of_block)
        data[:count] = peaks[:count]
        iv[:count] = intervals[:count]
        helpful = np.zeros(size_of_block)
        return self.L.refh_point_dbscan(data, iv, helpful, count, size_of_block, eps)

    def bifurcation(self, dim, tMax, nPts, h, ic, ranges, mut, wv, maxValue, transientTime, values,
                    preScaller=1, eps=0.0):
        B = int(tMax / h / preScaller)
        N = nPts ** dim
        ic, values = _d(ic), _d(values)
        amount = np.zeros(N, np.int32)
        data = np.zeros(N * B)
        iv = np.zeros(N * B)
        db = np.zeros(N, np.int32)
        helpful = np.zeros(N * B)
        self.L.refh_bifurcation(dim, tMax, nPts, h, ic.size, ic, _d(ranges), _i(mut), wv, maxValue, transientTime,
                                values, values.size, preScaller, eps, amount, data, iv,
                                db.ctypes.data if dim == 2 else None, helpful.ctypes.data)
        return dict(counts=amount, data=data.reshape(N, B), intervals=iv.reshape(N, B),
                    labels=db if dim == 2 else None)

    def basins(self, tMax, nPts, h, ic, ranges, mut, wv, maxValue, transientTime, values, preScaller=1):
        B = int(tMax / h / preScaller)
        N = nPts * nPts
        ic, values = _d(ic), _d(values)
        helpful = np.zeros(N, np.int32)
        ap = np.zeros(N)
        ai = np.zeros(N)
        data = np.zeros(N * B)
        self.L.refh_basins(tMax, nPts, h, ic.size, ic, _d(ranges), _i(mut), wv, maxValue, transientTime, values,
                           values.size, preScaller, helpful, ap, ai, data)
        return dict(flags=helpful, avg_peaks=ap, avg_intervals=ai)

    def basins_dbscan(self, avg_peaks, avg_intervals, flags, eps):
        ap, ai, fl = _d(avg_peaks).copy(), _d(avg_intervals).copy(), _i(flags).copy()
        labels = np.zeros(ap.size, np.int32)
        self.L.refh_basins_dbscan(ap, ai, labels, fl, ap.size, eps)
        return labels

    def bifurcation_range(self, dim, tMax, nPts, h, ic, ranges, mut, wv, maxValue, transientTime, values,
                          p_begin, p_end, preScaller=1, nthreads=0):
        """Kept-peak counts of points [p_begin, p_end) by the reference's own
        per-thread code (its chunking), spread over nthreads host threads."""
        ic, values = _d(ic), _d(values)
        counts = np.zeros(p_end - p_begin, np.int32)
        self.L.refh_bifurcation_range(dim, tMax, nPts, h, ic.size, ic, _d(ranges), _i(mut), wv, maxValue,
                                      transientTime, values, values.size, preScaller, p_begin, p_end, counts,
                                      nthreads)
        return counts

    def basins_range(self, tMax, nPts, h, ic, ranges, mut, wv, maxValue, transientTime, values, p_begin, p_end,
                     preScaller=1, nthreads=0):
        """Flags and features of points [p_begin, p_end) by the reference's own
        per-thread code (its chunking), spread over nthreads host threads."""
        ic, values = _d(ic), _d(values)
        n = p_end - p_begin
        flags, ap, ai = np.zeros(n, np.int32), np.zeros(n), np.zeros(n)
        self.L.refh_basins_range(tMax, nPts, h, ic.size, ic, _d(ranges), _i(mut), wv, maxValue, transientTime,
                                 values, values.size, preScaller, p_begin, p_end, flags, ap, ai, nthreads)
        return dict(flags=flags, avg_peaks=ap, avg_intervals=ai)

    def lle_range(self, tMax, NT, nPts, h, eps, ic, ranges, mut, transientTime, values, p_begin, p_end,
                  nthreads=0):
        """LLE2D points [p_begin, p_end) (p = b*nPts + a) by the reference's own
        per-thread code, spread over nthreads host threads."""
        ic, values = _d(ic), _d(values)
        out = np.zeros(p_end - p_begin)
        self.L.refh_lle_range(tMax, NT, nPts, h, eps, ic.size, ic, _d(ranges), _i(mut), transientTime, values,
                              values.size, p_begin, p_end, out, nthreads)
        return out

    def lle(self, tMax, NT, nPts, h, eps, ic, ranges, mut, transientTime, values):
        ic, values = _d(ic), _d(values)
        out = np.zeros(nPts * nPts)
        self.L.refh_lle(tMax, NT, nPts, h, eps, ic.size, ic, _d(ranges), _i(mut), transientTime, values,
                        values.size, out)
        return out


class LegacyLib:
    """Host build of the reference's legacy library functions
    (debri/cudaLibrary.cu, extracted unchanged: the helpers, the hard-wired
    system and its loops, the bifurcation / basins / step-sweep kernels) with
    host replays around them (oracle/ref_legacy_harness.cpp): the spectrum's
    block loop, and the legacy kernels of bifurcation1DIC / bifurcation2DIC,
    basinsOfAttraction and bifurcation1DForH run one host thread per point."""

    def __init__(self):
        path = REF_DIR / "libref_legacy.so"
        if not path.exists():
            raise FileNotFoundError(path)
        L = self.L = C.CDLL(str(path))
        L.leg_value.argtypes = L.leg_value_log.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_int]
        L.leg_value.restype = L.leg_value_log.restype = C.c_double
        L.leg_peak_finder.argtypes = [_dp, C.c_int, _dp, _dp, C.c_double]
        L.leg_peak_finder.restype = C.c_int
        L.leg_gram_schmidt.argtypes = [_dp, _dp, C.c_int, _dp]
        L.leg_ls_replay.argtypes = [C.c_int, _dp, _dp, C.c_double, C.c_int, C.c_int, C.c_int, C.c_double,
                                    C.c_double, _dp, _dp]
        L.leg_ic_bifurcation.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, _dp,
                                         C.c_int, _dp, C.c_int, _dp, _ip, C.c_int, C.c_double, C.c_double, _ip, _dp,
                                         _dp, _ip]
        L.leg_basins_v1.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, _dp, C.c_int, _dp,
                                    C.c_int, _dp, _ip, C.c_int, C.c_double, _ip, _dp, _dp]
        L.leg_step_sweep.argtypes = [C.c_int, C.c_double, C.c_double, C.c_int, _dp, C.c_int, _dp, C.c_int, _dp,
                                     C.c_int, C.c_double, _ip, _dp, C.c_int, C.POINTER(C.c_int)]
        L.leg_lle.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                              _dp, C.c_int, _dp, C.c_int, _dp, _ip, C.c_double, C.c_void_p, _dp]
        L.leg_ls.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, _dp,
                             C.c_int, _dp, C.c_int, _dp, _ip, C.c_double, _dp]
        for f in (L.leg_ic_bifurcation, L.leg_basins_v1, L.leg_step_sweep, L.leg_lle, L.leg_ls):
            f.restype = C.c_int

    def value_log(self, idx, nPts, start, finish, dim=0):
        return self.L.leg_value_log(idx, nPts, start, finish, dim)

    def value(self, idx, nPts, start, finish, dim=0):
        return self.L.leg_value(idx, nPts, start, finish, dim)

    def peak_finder(self, data, h):
        d = _d(data).copy()
        pk, tm = np.zeros(d.size), np.zeros(d.size)
        c = self.L.leg_peak_finder(d, d.size, pk, tm, h)
        return c, pk[:max(c, 0)], tm[:max(c, 0)]

    def ic_bifurcation(self, dim, nPts, tMax, h, transientTime, preScaller, ic, values, ranges, mut, wv,
                       maxValue, eps=0.0):
        """The legacy bifurcation1DIC (dim 1) / bifurcation2DIC (dim 2) kernels:
        counts, peaks [n][B], intervals [n][B] (dim 2), labels (dim 2)."""
        B = int(tMax / h / preScaller)
        n = nPts ** dim
        counts, labels = np.zeros(n, np.int32), np.zeros(n, np.int32)
        pk, iv = np.zeros(n * B), np.zeros(n * B)
        ic, vals = _d(ic), _d(values)
        rc = self.L.leg_ic_bifurcation(dim, nPts, tMax, h, transientTime, preScaller, ic, ic.size, vals, vals.size,
                                       _d(ranges), _i(mut), wv, maxValue, eps, counts, pk, iv, labels)
        if rc:
            raise ValueError("bad legacy bifurcation arguments")
        return dict(counts=counts, peaks=pk.reshape(n, B), intervals=iv.reshape(n, B),
                    labels=labels if dim == 2 else None)

    def basins_v1(self, nPts, tMax, h, transientTime, preScaller, ic, values, ranges, mut, wv, maxValue):
        """The legacy basinsOfAttraction kernels: flags, avgPeaks, avgIntervals."""
        n = nPts * nPts
        flags, ap, ai = np.zeros(n, np.int32), np.zeros(n), np.zeros(n)
        ic, vals = _d(ic), _d(values)
        rc = self.L.leg_basins_v1(nPts, tMax, h, transientTime, preScaller, ic, ic.size, vals, vals.size,
                                  _d(ranges), _i(mut), wv, maxValue, flags, ap, ai)
        if rc:
            raise ValueError("bad legacy basins arguments")
        return dict(flags=flags, avgPeaks=ap, avgIntervals=ai)

    def step_sweep(self, nPts, tMax, transientTime, preScaller, ic, values, ranges, wv, maxValue):
        """The legacy bifurcation1DForH kernels: counts, peaks [n][block]."""
        rows = int(tMax / min(ranges[0], ranges[1]) / preScaller) + 1
        counts, pk = np.zeros(nPts, np.int32), np.zeros(nPts * rows)
        ic, vals = _d(ic), _d(values)
        blk = C.c_int(0)
        rc = self.L.leg_step_sweep(nPts, tMax, transientTime, preScaller, ic, ic.size, vals, vals.size, _d(ranges),
                                   wv, maxValue, counts, pk, rows, C.byref(blk))
        if rc:
            raise ValueError(f"legacy step sweep refused ({rc})")
        return dict(counts=counts, peaks=pk[:nPts * blk.value].reshape(nPts, blk.value))

    def lle(self, kind, dim, nPts, tMax, NT, h, eps, transientTime, ic, values, ranges, mut, maxValue,
            uniforms=None):
        """The legacy LLE1D (kind 0, LLEKernelCUDA; uniforms[seed]: its cuRAND
        draws) or LLE1DIC / LLE2DIC (kind 1, LLEKernelICCUDA) kernel."""
        n = nPts ** dim
        out = np.zeros(n)
        ic, vals = _d(ic), _d(values)
        u = None if uniforms is None else np.ascontiguousarray(uniforms, np.float32)
        rc = self.L.leg_lle(kind, dim, nPts, tMax, NT, h, eps, transientTime, ic, ic.size, vals, vals.size,
                            _d(ranges), _i(mut), maxValue, None if u is None else u.ctypes.data, out)
        if rc:
            raise ValueError("bad legacy LLE arguments")
        return out

    def ls(self, dim, nPts, tMax, NT, h, eps, transientTime, ic, values, ranges, mut, maxValue):
        """The legacy LS1D / LS2D kernel LSKernelCUDA: [points, SIZE_X]."""
        n = nPts ** dim
        ic, vals = _d(ic), _d(values)
        out = np.zeros(n * ic.size)
        rc = self.L.leg_ls(dim, nPts, tMax, NT, h, eps, transientTime, ic, ic.size, vals, vals.size, _d(ranges),
                           _i(mut), maxValue, out)
        if rc:
            raise ValueError("bad legacy spectrum arguments")
        return out.reshape(n, ic.size)

    def ls_replay(self, system, x0, a, h, trans, ntp, nblocks, eps, tmax, directions):
        n = len(x0)
        out = np.zeros(n)
        self.L.leg_ls_replay(system, _d(x0), _d(a), h, trans, ntp, nblocks, eps, tmax,
                             _d(np.asarray(directions, np.float64).ravel()), out)
        return out


def legacy_available() -> bool:
    return (REF_DIR / "libref_legacy.so").exists()


def ref_available(name: str = "lorenz") -> bool:
    return (REF_DIR / f"libref_{name}.so").exists()


def canonical_labels(labels) -> np.ndarray:
    """Relabel a compat basin labelling: negative ids numbered -1, -2, ... by
    their smallest member index, positive ids 1, 2, ... likewise, 0 kept."""
    labels = np.asarray(labels)
    out = np.zeros_like(labels)
    for sign in (-1, 1):
        ids = np.unique(labels[labels * sign > 0])
        firsts = sorted((int(np.argmax(labels == v)), v) for v in ids)
        for rank, (_, v) in enumerate(firsts, start=1):
            out[labels == v] = sign * rank
    return out
