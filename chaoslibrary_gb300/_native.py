"""ctypes bindings of libchaos_gb300.so (see include/chaos_gb300.h)."""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path
from types import SimpleNamespace

import numpy as np

_PKG = Path(__file__).resolve().parent
FP64, FP32, FF32 = 0, 1, 2  # CHAOS_FP64, CHAOS_FP32, CHAOS_FF32
CUDA_STREAM_LEGACY = 1  # cudaStreamLegacy
MEM_HOST, MEM_DEVICE = 0, 1
SYSTEMS = {"lorenz": 0, "rossler": 1, "chen": 2, "chameleon": 3, "rossler_cd": 4, "sin3": 5, "sin2": 6,
           "memristor": 7, "user": 15}
STATUS = {0: "CHAOS_OK", -1: "CHAOS_E_ARGS", -2: "CHAOS_E_NOMEM", -3: "CHAOS_E_CUDA", -4: "CHAOS_E_IO",
          -5: "CHAOS_E_TIMEOUT", -6: "CHAOS_E_UNSUPPORTED", -7: "CHAOS_E_BUSY", -8: "CHAOS_E_NODEV"}


class ChaosError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class Exec(C.Structure):
    _fields_ = [("precision", C.c_int), ("memory", C.c_int), ("stream", C.c_void_p), ("device", C.c_int)]


JOB_BIF1D, JOB_LLE2D, JOB_BASINS, JOB_LLE2D_FF32 = 1, 2, 3, 4


class Job(C.Structure):
    """chaos_job of include/chaos_gb300.h."""
    _fields_ = [("kind", C.c_int), ("system", C.c_int), ("tMax", C.c_double), ("nPts", C.c_int),
                ("h", C.c_double), ("initialConditions", C.c_void_p), ("ranges", C.c_void_p),
                ("indicesOfMutVars", C.c_void_p), ("writableVar", C.c_int), ("maxValue", C.c_double),
                ("transientTime", C.c_double), ("values", C.c_void_p), ("preScaller", C.c_int),
                ("NT", C.c_double), ("eps", C.c_double), ("peakCapacity", C.c_int), ("counts", C.c_void_p),
                ("flags", C.c_void_p), ("first", C.c_void_p), ("peaks", C.c_void_p), ("intervals", C.c_void_p),
                ("lle", C.c_void_p), ("avgPeaks", C.c_void_p), ("avgIntervals", C.c_void_p),
                ("labels", C.c_void_p)]


def lib_path() -> Path:
    return Path(os.environ.get("CHAOS_GB300_LIB", _PKG / "lib" / "libchaos_gb300.so"))


_lib = None
_P = C.c_void_p
_D = C.c_double
_I = C.c_int
_L = C.c_longlong

_SIGS = {
    "chaos_abi_version": ([], _I),
    "chaos_last_error": ([], C.c_char_p),
    "chaos_system_info": ([_I, _P, _P], _I),
    "chaos_synchronize": ([_P], _I),
    "chaos_bifurcation1d": ([_P, _I, _D, _I, _D, _I, _P, _P, _P, _I, _D, _D, _P, _I, _I, _I, _P, _P, _P, _P, _P], _I),
    "chaos_bifurcation2d": ([_P, _I, _D, _I, _D, _I, _P, _P, _P, _I, _D, _D, _P, _I, _I, _D, _P, _P], _I),
    "chaos_lle2d": ([_P, _I, _D, _D, _I, _D, _D, _P, _I, _P, _P, _I, _D, _D, _P, _I, _P], _I),
    "chaos_bifurcation_sweep": ([_P, _I, _I, _I, _D, _I, _D, _I, _P, _P, _P, _I, _D, _D, _P, _I, _I, _D, _I, _P, _P, _P,
                                 _P, _P, _P], _I),
    "chaos_compact_peaks": ([_P, _P, _P, _P, C.c_longlong, _I, _P, _P, _P, _P, C.c_longlong, _P], _I),
    "chaos_lle_from_states": ([_P, _I, C.c_longlong, _P, _D, _D, _D, _D, _P], _I),
    "chaos_lle_sweep": ([_P, _I, _I, _I, _D, _D, _I, _D, _D, _P, _I, _P, _P, _D, _P, _I, _P], _I),
    "chaos_lle_sweep_legacy": ([_P, _I, _I, _I, _D, _D, _I, _D, _D, _P, _I, _P, _P, _D, _D, _P, _I, _P, _P], _I),
    "chaos_legacy_lle_draws": ([_P, _I, C.c_longlong, _I, _P], _I),
    "chaos_lyapunov_spectrum_legacy": ([_P, _I, _I, _I, _D, _D, _I, _D, _D, _P, _I, _P, _P, _D, _D, _P, _I, _P, _P],
                                       _I),
    "chaos_lyapunov_spectrum": ([_P, _I, _I, _I, _D, _D, _I, _D, _D, _P, _I, _P, _P, _D, _P, _I, _P], _I),
    "chaos_lle2d_checked": ([_P, _I, _D, _D, _I, _D, _D, _P, _I, _P, _P, _D, _P, _I, _D, _D, _P, _P, _P], _I),
    "chaos_basins_features": ([_P, _I, _D, _I, _D, _I, _P, _P, _P, _I, _D, _D, _P, _I, _I, _P, _P, _P, _P], _I),
    "chaos_basins": ([_P, _I, _D, _I, _D, _I, _P, _P, _P, _I, _D, _D, _P, _I, _I, _D, _P, _P, _P, _P], _I),
    "chaos_dbscan_compat": ([_P, _P, _P, _P, _L, _D, _P], _I),
    "chaos_basins_dbscan": ([_P, _I, _D, _I, _D, _I, _P, _P, _P, _I, _D, _D, _P, _I, _I, _D, _I, _P, _P, _P], _I),
    "chaos_dbscan": ([_P, _P, _L, _I, _D, _I, _P, _P], _I),
    "chaos_peak_finder": ([_P, _P, _L, _I, _D, _I, _P, _P, _P], _I),
    "chaos_point_dbscan": ([_P, _P, _P, _L, _I, _D, _P], _I),
    "chaos_fma_probe": ([_P, _L, _P, _P], _I),
    "chaos_device_code_version": ([_I, _P, _P], _I),
    "chaos_launch_count": ([_P], _I),
    "chaos_autotune": ([_P, _P, _I], _I),
    "chaos_trajectory": ([_P, _I, _L, _P, _P, _D, _I, _P], _I),
    "chaos_set_tuning": ([_I, _I], _I),
    "chaos_run_batch": ([_P, _P, _I], _I),
    "chaos_batch_create": ([_P, _P, _I, _P], _I),
    "chaos_batch_run": ([_P], _I),
    "chaos_batch_destroy": ([_P], _I),
    "chaos_server_create": ([_P, C.c_size_t, _I, _D, _P], _I),
    "chaos_server_submit": ([_P, _P, _P], _I),
    "chaos_server_poll": ([_P, C.c_longlong, _P], _I),
    "chaos_server_wait": ([_P, C.c_longlong, _D, _P], _I),
    "chaos_server_stats": ([_P, _P, _I], _I),
    "chaos_server_latency": ([_P, C.c_longlong], _D),
    "chaos_server_destroy": ([_P], _I),
    "chaos_get_tuning": ([_I], _I),
    "chaos_compat_set_system": ([_I], _I),
    "chaos_compat_set_precision": ([_I], _I),
    "chaos_compat_get_system": ([], _I),
    "chaos_compat_bifurcation1D": ([_D, _I, _D, _I, _P, _P, _P, _I, _D, _D, _P, _I, _I, C.c_char_p], _I),
    "chaos_compat_bifurcation2D": ([_D, _I, _D, _I, _P, _P, _P, _I, _D, _D, _P, _I, _I, _D, C.c_char_p], _I),
    "chaos_compat_LLE2D": ([_D, _D, _I, _D, _D, _P, _I, _P, _P, _I, _D, _D, _P, _I, C.c_char_p], _I),
    "chaos_compat_basinsOfAttraction_2": ([_D, _I, _D, _I, _P, _P, _P, _I, _D, _D, _P, _I, _I, _D, C.c_char_p], _I),
    "chaos_compat_bifurcation1DIC": ([_D, _I, _D, _I, _P, _P, _P, _I, _D, _D, _P, _I, _I, C.c_char_p], _I),
    "chaos_compat_bifurcation2DIC": ([_D, _I, _D, _I, _P, _P, _P, _I, _D, _D, _P, _I, _I, _D, C.c_char_p], _I),
    "chaos_compat_bifurcation1DForH": ([_D, _I, _I, _P, _P, _I, _D, _D, _P, _I, _I, C.c_char_p], _I),
    "chaos_compat_LLE1D": ([_D, _D, _I, _D, _D, _P, _I, _P, _P, _I, _D, _D, _P, _I, C.c_char_p], _I),
    "chaos_compat_LLE1DIC": ([_D, _D, _I, _D, _D, _P, _I, _P, _P, _I, _D, _D, _P, _I, C.c_char_p], _I),
    "chaos_compat_LLE2DIC": ([_D, _D, _I, _D, _D, _P, _I, _P, _P, _I, _D, _D, _P, _I, C.c_char_p], _I),
    "chaos_compat_LS1D": ([_D, _D, _I, _D, _D, _P, _I, _P, _P, _I, _D, _D, _P, _I, C.c_char_p], _I),
    "chaos_compat_LS2D": ([_D, _D, _I, _D, _D, _P, _I, _P, _P, _I, _D, _D, _P, _I, C.c_char_p], _I),
    "chaos_compat_basinsOfAttraction": ([_D, _I, _D, _I, _P, _P, _P, _I, _D, _D, _P, _I, _I, _D, C.c_char_p], _I),
}


def lib() -> C.CDLL:
    """The loaded engine library; raises if it has not been built."""
    global _lib
    if _lib is None:
        path = lib_path()
        if not path.exists():
            raise ChaosError(-8, f"{path} is missing: build it with chaoslibrary_gb300.build.build() "
                                 "(the engine has no CPU fallback)")
        L = C.CDLL(str(path))
        for name, (args, res) in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def _check(rc: int) -> None:
    if rc != 0:
        raise ChaosError(rc, lib().chaos_last_error().decode(errors="replace"))


def _sys(system) -> int:
    return SYSTEMS[system] if isinstance(system, str) else int(system)


_PREC_NAMES = {"fp64": FP64, "f64": FP64, "float64": FP64, "fp32": FP32, "f32": FP32, "float32": FP32,
               "ff32": FF32, "float-float": FF32}


def _prec(precision) -> int:
    if isinstance(precision, str):
        if precision.lower() not in _PREC_NAMES:
            raise ChaosError(-1, f"unknown precision {precision!r} (fp64, fp32 or ff32)")
        return _PREC_NAMES[precision.lower()]
    return int(precision)


def system_info(system) -> tuple[int, int]:
    nx, na = C.c_int(), C.c_int()
    _check(lib().chaos_system_info(_sys(system), C.byref(nx), C.byref(na)))
    return nx.value, na.value


class _Args:
    """Keeps the ctypes views of numpy inputs alive for one call."""

    def __init__(self):
        self.keep = []

    def d(self, x):
        a = np.ascontiguousarray(x, dtype=np.float64)
        self.keep.append(a)
        return a.ctypes.data

    def i(self, x):
        a = np.ascontiguousarray(x, dtype=np.int32)
        self.keep.append(a)
        return a.ctypes.data


def _out_ptr(arr):
    if arr is None:
        return None
    if hasattr(arr, "data_ptr"):
        return arr.data_ptr()
    return arr.ctypes.data


def _exec(precision, outs: dict, stream=None, device=None) -> Exec:
    """Host-memory call unless the outputs are CUDA tensors (device call on
    torch's current stream of that device, asynchronous)."""
    tensors = [v for v in outs.values() if v is not None and hasattr(v, "data_ptr")]
    if tensors:
        import torch

        dev = tensors[0].device
        st = stream if stream is not None else torch.cuda.current_stream(dev).cuda_stream
        if not st:
            st = CUDA_STREAM_LEGACY  # torch's default stream; NULL would select the library's own stream
        return Exec(_prec(precision), MEM_DEVICE, C.c_void_p(st), dev.index if dev.index is not None else -1)
    return Exec(_prec(precision), MEM_HOST, None, -1 if device is None else int(device))


def fma_probe(iters: int = 200000, device=None) -> float:
    """Measured FP32 FMA throughput of the device, in flop/s."""
    ex = Exec(FP64, MEM_HOST, None, -1 if device is None else int(device))
    sec, fl = C.c_double(), C.c_double()
    _check(lib().chaos_fma_probe(C.byref(ex), iters, C.byref(sec), C.byref(fl)))
    return fl.value / sec.value


def device_code_version(device: int = -1) -> tuple[int, int]:
    """(binaryVersion, ptxVersion) of the library's device code on `device`
    (cudaFuncGetAttributes of one of its kernels): (103, 103) for sm_103a."""
    b, p = C.c_int(), C.c_int()
    _check(lib().chaos_device_code_version(int(device), C.byref(b), C.byref(p)))
    return b.value, p.value


def autotune(device=None) -> list[dict]:
    """Times the FP32 sweeps' launch shapes on this GPU and installs the
    fastest (chaos_autotune); returns one row per (kind, system)."""
    ex = Exec(FP32, MEM_HOST, None, -1 if device is None else int(device))
    t = np.zeros((9, 6))
    _check(lib().chaos_autotune(C.byref(ex), t.ctypes.data, 9))
    kinds = ("bif1d", "basins", "lle")
    return [dict(kind=kinds[int(r[0])], system=int(r[1]), form=int(r[2]), block=int(r[3]), best_ms=float(r[4]),
                 rule_ms=float(r[5])) for r in t]


def launch_count() -> int:
    """Kernels the library has launched in this process so far."""
    n = C.c_longlong()
    _check(lib().chaos_launch_count(C.byref(n)))
    return n.value


def trajectory(system, x0, a, h, n_steps, precision=FP64):
    """States of trajectories [nTraj, n_steps + 1, SIZE_X] (x0: [nTraj, SIZE_X], a: [nTraj, SIZE_A])."""
    A = _Args()
    x0 = np.ascontiguousarray(np.atleast_2d(x0), np.float64)
    a = np.ascontiguousarray(np.atleast_2d(a), np.float64)
    n, nx = x0.shape
    if a.shape[0] == 1 and n > 1:
        a = np.repeat(a, n, axis=0)
    out = np.zeros((n, n_steps + 1, nx))
    ex = _exec(precision, {})
    _check(lib().chaos_trajectory(C.byref(ex), _sys(system), n, A.d(x0), A.d(a), h, n_steps, _out_ptr(out)))
    return out


# grid modes (CHAOS_GRID_*) and the step-size axis marker (CHAOS_MUT_STEP)
GRID_STATE, GRID_LOG0, GRID_LOG1, GRID_LOG_F32, GRID_LEGACY_LOOP = 1, 2, 4, 8, 16
MUT_STEP = -1

TUNE_LLE_F32_VARIANT = 1
TUNE_SWEEP_PAIRS = 2
TUNE_GRID_FMA = 3
TUNE_LLE_TWIN = 4
TUNE_BIF2D_CAP = 5
TUNE_SHAPES = 6
TUNE_LLE_RENORM = 7
TUNE_FF_PAIRS = 8


def set_tuning(knob: int, value: int) -> None:
    _check(lib().chaos_set_tuning(knob, value))


def get_tuning(knob: int) -> int:
    return lib().chaos_get_tuning(knob)


class Batch:
    """Many sweeps run by one submission (chaos_run_batch / chaos_batch_*).

    add_bifurcation1d / add_lle2d / add_basins take the same arguments as the
    array functions and return the dict of output arrays (numpy, or CUDA
    tensors when device=True) that the batch fills."""

    def __init__(self, device: bool = False):
        self.device = device
        self.jobs = []
        self.keep = _Args()
        self.outputs = []
        self._plan = None

    def _alloc(self, shape, dtype):
        if self.device:
            import torch

            tdt = {np.float64: torch.float64, np.int32: torch.int32}[dtype]
            return torch.zeros(shape, dtype=tdt, device="cuda")
        return np.zeros(shape, dtype)

    def _common(self, kind, system, tMax, nPts, h, ic, ranges, mut, wv, maxValue, transientTime, values,
                preScaller):
        j = Job()
        j.kind, j.system, j.tMax, j.nPts, j.h = kind, _sys(system), tMax, nPts, h
        j.initialConditions = self.keep.d(ic)
        j.ranges = self.keep.d(ranges)
        j.indicesOfMutVars = self.keep.i(mut)
        j.writableVar, j.maxValue, j.transientTime = wv, maxValue, transientTime
        j.values = self.keep.d(values)
        j.preScaller = preScaller
        return j

    def add_bifurcation1d(self, system, tMax, nPts, h, initialConditions, ranges, indicesOfMutVars, writableVar,
                          maxValue, transientTime, values, preScaller=1, peakCapacity=64):
        j = self._common(JOB_BIF1D, system, tMax, nPts, h, initialConditions, ranges, indicesOfMutVars,
                         writableVar, maxValue, transientTime, values, preScaller)
        out = dict(counts=self._alloc(nPts, np.int32), flags=self._alloc(nPts, np.int32),
                   first=self._alloc(nPts, np.float64), peaks=self._alloc((nPts, peakCapacity), np.float64),
                   intervals=self._alloc((nPts, peakCapacity), np.float64))
        j.peakCapacity = peakCapacity
        j.counts, j.flags, j.first = _out_ptr(out["counts"]), _out_ptr(out["flags"]), _out_ptr(out["first"])
        j.peaks, j.intervals = _out_ptr(out["peaks"]), _out_ptr(out["intervals"])
        self.jobs.append(j)
        self.outputs.append(out)
        return out

    def add_lle2d(self, system, tMax, NT, nPts, h, eps, initialConditions, ranges, indicesOfMutVars, transientTime,
                  values, precision=FP32):
        """An LLE map job: FP32 (CHAOS_JOB_LLE2D) or float-float (precision
        FF32: CHAOS_JOB_LLE2D_FF32, RK4 systems)."""
        kind = JOB_LLE2D_FF32 if _prec(precision) == FF32 else JOB_LLE2D
        j = self._common(kind, system, tMax, nPts, h, initialConditions, ranges, indicesOfMutVars, 0, 0.0,
                         transientTime, values, 1)
        j.NT, j.eps = NT, eps
        out = dict(lle=self._alloc(nPts * nPts, np.float64))
        j.lle = _out_ptr(out["lle"])
        self.jobs.append(j)
        self.outputs.append(out)
        return out

    def add_basins(self, system, tMax, nPts, h, initialConditions, ranges, indicesOfMutVars, writableVar, maxValue,
                   transientTime, values, preScaller=1):
        j = self._common(JOB_BASINS, system, tMax, nPts, h, initialConditions, ranges, indicesOfMutVars,
                         writableVar, maxValue, transientTime, values, preScaller)
        n = nPts * nPts
        out = dict(flags=self._alloc(n, np.int32), avg_peaks=self._alloc(n, np.float64),
                   avg_intervals=self._alloc(n, np.float64), counts=self._alloc(n, np.int32))
        j.flags, j.avgPeaks = _out_ptr(out["flags"]), _out_ptr(out["avg_peaks"])
        j.avgIntervals, j.counts = _out_ptr(out["avg_intervals"]), _out_ptr(out["counts"])
        self.jobs.append(j)
        self.outputs.append(out)
        return out

    def _exec(self):
        if self.device:
            import torch

            st = torch.cuda.current_stream().cuda_stream or CUDA_STREAM_LEGACY
            return Exec(FP32, MEM_DEVICE, C.c_void_p(st), torch.cuda.current_device())
        return Exec(FP32, MEM_HOST, None, -1)

    def run(self):
        """One-shot submission (chaos_run_batch)."""
        arr = (Job * len(self.jobs))(*self.jobs)
        ex = self._exec()
        _check(lib().chaos_run_batch(C.byref(ex), arr, len(self.jobs)))
        return self.outputs

    def prepare(self):
        """Uploads descriptors and captures the launch in a CUDA graph (chaos_batch_create)."""
        if self._plan is None:
            arr = (Job * len(self.jobs))(*self.jobs)
            ex = self._exec()
            plan = C.c_void_p()
            _check(lib().chaos_batch_create(C.byref(ex), arr, len(self.jobs), C.byref(plan)))
            self._plan = plan
        return self

    def replay(self):
        """Runs the prepared graph (chaos_batch_run)."""
        self.prepare()
        _check(lib().chaos_batch_run(self._plan))
        return self.outputs

    def close(self):
        if self._plan is not None:
            lib().chaos_batch_destroy(self._plan)
            self._plan = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


REQ_PENDING, REQ_RUNNING, REQ_DONE, REQ_FAILED = 0, 1, 2, 3
STATS = ["completed", "failed", "pending", "running", "p50_s", "p99_s", "mean_s", "steps", "elapsed_s",
         "iterations", "peak_hbm_bytes", "max_s"]


class Server:
    """The request loop (chaos_server_*): submit jobs at any time, wait for
    them, read latency statistics. Outputs are host numpy arrays filled when a
    request completes."""

    def __init__(self, hbm_budget_bytes=64 << 30, max_active=1024, iteration_steps=2e10, device=None):
        ex = Exec(FP32, MEM_HOST, None, -1 if device is None else int(device))
        self._s = C.c_void_p()
        _check(lib().chaos_server_create(C.byref(ex), int(hbm_budget_bytes), int(max_active),
                                         float(iteration_steps), C.byref(self._s)))
        self._keep = {}

    def _submit(self, job, keep, out):
        rid = C.c_longlong()
        _check(lib().chaos_server_submit(self._s, C.byref(job), C.byref(rid)))
        self._keep[rid.value] = (keep, out)
        return rid.value

    def submit_bifurcation1d(self, system, tMax, nPts, h, initialConditions, ranges, indicesOfMutVars, writableVar,
                             maxValue, transientTime, values, preScaller=1, peakCapacity=16):
        b = Batch()
        out = b.add_bifurcation1d(system, tMax, nPts, h, initialConditions, ranges, indicesOfMutVars, writableVar,
                                  maxValue, transientTime, values, preScaller, peakCapacity)
        return self._submit(b.jobs[0], b, out), out

    def submit_lle2d(self, system, tMax, NT, nPts, h, eps, initialConditions, ranges, indicesOfMutVars,
                     transientTime, values, precision=FP32):
        b = Batch()
        out = b.add_lle2d(system, tMax, NT, nPts, h, eps, initialConditions, ranges, indicesOfMutVars,
                          transientTime, values, precision)
        return self._submit(b.jobs[0], b, out), out

    def submit_basins(self, system, tMax, nPts, h, initialConditions, ranges, indicesOfMutVars, writableVar,
                      maxValue, transientTime, values, preScaller=1, eps=0.05):
        b = Batch()
        out = b.add_basins(system, tMax, nPts, h, initialConditions, ranges, indicesOfMutVars, writableVar,
                           maxValue, transientTime, values, preScaller)
        j = b.jobs[0]
        if eps and eps > 0:
            out["labels"] = np.zeros(nPts * nPts, np.int32)
            j.labels = out["labels"].ctypes.data
            j.eps = eps
        return self._submit(j, b, out), out

    def wait(self, rid, timeout=600.0):
        st = C.c_int()
        _check(lib().chaos_server_wait(self._s, rid, float(timeout), C.byref(st)))
        return st.value

    def poll(self, rid):
        st = C.c_int()
        _check(lib().chaos_server_poll(self._s, rid, C.byref(st)))
        return st.value

    def latency(self, rid):
        return lib().chaos_server_latency(self._s, rid)

    def stats(self):
        arr = (C.c_double * len(STATS))()
        _check(lib().chaos_server_stats(self._s, arr, len(STATS)))
        return dict(zip(STATS, list(arr)))

    def close(self):
        if self._s:
            lib().chaos_server_destroy(self._s)
            self._s = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def set_system(system) -> None:
    """System used by the reference-signature wrappers (bifurcation1D, ...)."""
    _check(lib().chaos_compat_set_system(_sys(system)))


def set_precision(precision) -> None:
    _check(lib().chaos_compat_set_precision(_prec(precision)))


# ---- array API ---------------------------------------------------------------

def bifurcation1d(system, tMax, nPts, h, initialConditions, ranges, indicesOfMutVars, writableVar, maxValue,
                  transientTime, values, preScaller=1, peakCapacity=None, precision=FP64, out=None, stream=None):
    """1-D sweep; returns counts, flags, first, peaks[nPts, cap], intervals[nPts, cap]."""
    A = _Args()
    B = int(tMax / h / preScaller) if h > 0 and preScaller > 0 else 1
    cap = int(peakCapacity or max(B // 2, 1))
    if out is None:
        out = dict(counts=np.zeros(nPts, np.int32), flags=np.zeros(nPts, np.int32), first=np.zeros(nPts),
                   peaks=np.zeros((nPts, cap)), intervals=np.zeros((nPts, cap)))
    ex = _exec(precision, out, stream)
    ic = np.asarray(initialConditions, np.float64)
    vals = np.asarray(values, np.float64)
    _check(lib().chaos_bifurcation1d(C.byref(ex), _sys(system), tMax, nPts, h, ic.size, A.d(ic), A.d(ranges),
                                     A.i(indicesOfMutVars), writableVar, maxValue, transientTime, A.d(vals),
                                     vals.size, preScaller, cap, _out_ptr(out["counts"]), _out_ptr(out["flags"]),
                                     _out_ptr(out.get("first")), _out_ptr(out.get("peaks")),
                                     _out_ptr(out.get("intervals"))))
    return out


def bifurcation2d(system, tMax, nPts, h, initialConditions, ranges, indicesOfMutVars, writableVar, maxValue,
                  transientTime, values, preScaller=1, eps=0.001, precision=FP64, out=None, stream=None):
    A = _Args()
    n = nPts * nPts
    if out is None:
        out = dict(labels=np.zeros(n, np.int32), counts=np.zeros(n, np.int32))
    ex = _exec(precision, out, stream)
    ic = np.asarray(initialConditions, np.float64)
    vals = np.asarray(values, np.float64)
    _check(lib().chaos_bifurcation2d(C.byref(ex), _sys(system), tMax, nPts, h, ic.size, A.d(ic), A.d(ranges),
                                     A.i(indicesOfMutVars), writableVar, maxValue, transientTime, A.d(vals),
                                     vals.size, preScaller, eps, _out_ptr(out["labels"]),
                                     _out_ptr(out.get("counts"))))
    return out


def bifurcation_sweep(system, dim, gridMode, tMax, nPts, h, initialConditions, ranges, indicesOfMutVars,
                      writableVar, maxValue, transientTime, values, preScaller=1, eps=0.001, peakCapacity=None,
                      precision=FP64, out=None, stream=None):
    """Bifurcation over parameters or initial conditions (GRID_STATE), linear
    or log-scale axes, or the step size (indicesOfMutVars[0] = MUT_STEP, dim 1)
    (chaos_bifurcation_sweep); GRID_LEGACY_LOOP runs the legacy library's
    per-point loop in FP64. dim 1: counts, flags, first, peaks, intervals;
    dim 2: labels, counts."""
    A = _Args()
    ic = np.asarray(initialConditions, np.float64)
    vals = np.asarray(values, np.float64)
    n = nPts ** dim
    if dim == 1:
        h_min = min(ranges[0], ranges[1]) * (1.0 - 1e-9) if indicesOfMutVars[0] == MUT_STEP else h
        B = int(tMax / h_min / preScaller) if h_min > 0 and preScaller > 0 else 1
        cap = int(peakCapacity or max(B // 2, 1))
        if out is None:
            out = dict(counts=np.zeros(n, np.int32), flags=np.zeros(n, np.int32), first=np.zeros(n),
                       peaks=np.zeros((n, cap)), intervals=np.zeros((n, cap)))
        ex = _exec(precision, out, stream)
        _check(lib().chaos_bifurcation_sweep(
            C.byref(ex), _sys(system), 1, gridMode, tMax, nPts, h, ic.size, A.d(ic), A.d(ranges),
            A.i(indicesOfMutVars), writableVar, maxValue, transientTime, A.d(vals), vals.size, preScaller, eps, cap,
            _out_ptr(out["counts"]), _out_ptr(out["flags"]), _out_ptr(out.get("first")),
            _out_ptr(out.get("peaks")), _out_ptr(out.get("intervals")), None))
        return out
    if out is None:
        out = dict(labels=np.zeros(n, np.int32), counts=np.zeros(n, np.int32))
    ex = _exec(precision, out, stream)
    _check(lib().chaos_bifurcation_sweep(
        C.byref(ex), _sys(system), 2, gridMode, tMax, nPts, h, ic.size, A.d(ic), A.d(ranges), A.i(indicesOfMutVars),
        writableVar, maxValue, transientTime, A.d(vals), vals.size, preScaller, eps, 0, _out_ptr(out.get("counts")),
        None, None, None, None, _out_ptr(out["labels"])))
    return out


def compact_peaks(counts, peaks, intervals):
    """Dense peak list of a 1-D sweep's rows (chaos_compact_peaks): returns
    offsets[n + 1], peaks, intervals and the point of every kept peak."""
    A = _Args()
    cnt = np.ascontiguousarray(counts, np.int32)
    pk = np.ascontiguousarray(peaks, np.float64)
    iv = np.ascontiguousarray(intervals, np.float64)
    n, cap = pk.shape
    ex = _exec(FP64, {}, None)
    total = C.c_longlong(0)
    offsets = np.zeros(n + 1, np.int64)
    _check(lib().chaos_compact_peaks(C.byref(ex), A.i(cnt), None, None, n, cap, offsets.ctypes.data, None, None,
                                     None, 0, C.byref(total)))
    m = int(total.value)
    dp, di, dw = np.zeros(m), np.zeros(m), np.zeros(m, np.int32)
    _check(lib().chaos_compact_peaks(C.byref(ex), A.i(cnt), A.d(pk), A.d(iv), n, cap, offsets.ctypes.data,
                                     _out_ptr(dp), _out_ptr(di), _out_ptr(dw), m, C.byref(total)))
    return dict(offsets=offsets, peaks=dp, intervals=di, point=dw)


def lle2d(system, tMax, NT, nPts, h, eps, initialConditions, ranges, indicesOfMutVars, transientTime, values,
          writableVar=0, maxValue=0.0, precision=FP64, out=None, stream=None):
    """LLE map; result[j*nPts + i] (row = second parameter), as the reference CSV."""
    A = _Args()
    if out is None:
        out = np.zeros(nPts * nPts)
    ex = _exec(precision, {"lle": out}, stream)
    ic = np.asarray(initialConditions, np.float64)
    vals = np.asarray(values, np.float64)
    _check(lib().chaos_lle2d(C.byref(ex), _sys(system), tMax, NT, nPts, h, eps, A.d(ic), ic.size, A.d(ranges),
                             A.i(indicesOfMutVars), writableVar, maxValue, transientTime, A.d(vals), vals.size,
                             _out_ptr(out)))
    return out


def lle_from_states(system, states, tMax, NT, h, eps, precision=FP64, out=None, stream=None):
    """Benettin stage of the LLE map from starting states (chaos_lle_from_states):
    states[n, 2*SIZE_X + SIZE_A] = (orbit after the transient, parameters,
    twin start) per point, the reference's semi_result rows."""
    A = _Args()
    st = np.ascontiguousarray(np.atleast_2d(states), np.float64)
    n = st.shape[0]
    if out is None:
        out = np.zeros(n)
    ex = _exec(precision, {"lle": out}, stream)
    _check(lib().chaos_lle_from_states(C.byref(ex), _sys(system), n, A.d(st), tMax, NT, h, eps, _out_ptr(out)))
    return out


def lle_sweep(system, dim, tMax, NT, nPts, h, eps, initialConditions, ranges, indicesOfMutVars, transientTime,
              values, mutateState=False, precision=FP64, out=None, stream=None, gridMode=0):
    """LLE over a 1-D (lle[i]) or 2-D (lle[j*nPts + i]) grid of parameters or,
    with mutateState, of initial conditions; gridMode adds log-scale axes
    (GRID_LOG0 / LOG1 / LOG_F32) (chaos_lle_sweep)."""
    A = _Args()
    n = nPts ** dim
    if out is None:
        out = np.zeros(n)
    ex = _exec(precision, {"lle": out}, stream)
    ic = np.asarray(initialConditions, np.float64)
    vals = np.asarray(values, np.float64)
    mode = gridMode | (GRID_STATE if mutateState else 0)
    _check(lib().chaos_lle_sweep(C.byref(ex), _sys(system), dim, mode, tMax, NT, nPts, h, eps,
                                 A.d(ic), ic.size, A.d(ranges), A.i(indicesOfMutVars), transientTime, A.d(vals),
                                 vals.size, _out_ptr(out)))
    return out


def lle_sweep_legacy(system, dim, tMax, NT, nPts, h, eps, initialConditions, ranges, indicesOfMutVars,
                     transientTime, values, maxValue=0.0, mutateState=False, draws=None, out=None, stream=None,
                     gridMode=0):
    """The legacy library's LLE analyses with its own kernels' scheme, FP64
    (chaos_lle_sweep_legacy): LLE1D (a grid of parameters) or, with
    mutateState, LLE1DIC / LLE2DIC. draws: raw twin draws [points, SIZE_X]
    (None: the legacy's own, legacy_lle_draws)."""
    A = _Args()
    n = nPts ** dim
    if out is None:
        out = np.zeros(n)
    ex = _exec(FP64, {"lle": out}, stream)
    ic = np.asarray(initialConditions, np.float64)
    vals = np.asarray(values, np.float64)
    mode = gridMode | (GRID_STATE if mutateState else 0)
    dr = None if draws is None else np.ascontiguousarray(draws, np.float64)
    _check(lib().chaos_lle_sweep_legacy(C.byref(ex), _sys(system), dim, mode, tMax, NT, nPts, h, eps,
                                        A.d(ic), ic.size, A.d(ranges), A.i(indicesOfMutVars), maxValue,
                                        transientTime, A.d(vals), vals.size, None if dr is None else A.d(dr),
                                        _out_ptr(out)))
    return out


def lyapunov_spectrum_legacy(system, dim, tMax, NT, nPts, h, eps, initialConditions, ranges, indicesOfMutVars,
                             transientTime, values, maxValue=0.0, mutateState=False, draws=None, out=None,
                             stream=None, gridMode=0):
    """The legacy library's LS1D / LS2D with its own kernel's scheme, FP64
    (chaos_lyapunov_spectrum_legacy): [points, SIZE_X]. draws: raw twin
    draws [points, SIZE_X, SIZE_X] (None: the legacy's own)."""
    A = _Args()
    ic = np.asarray(initialConditions, np.float64)
    n = nPts ** dim
    if out is None:
        out = np.zeros((n, ic.size))
    ex = _exec(FP64, {"spectrum": out}, stream)
    vals = np.asarray(values, np.float64)
    mode = gridMode | (GRID_STATE if mutateState else 0)
    dr = None if draws is None else np.ascontiguousarray(draws, np.float64)
    _check(lib().chaos_lyapunov_spectrum_legacy(C.byref(ex), _sys(system), dim, mode, tMax, NT, nPts, h, eps,
                                                A.d(ic), ic.size, A.d(ranges), A.i(indicesOfMutVars), maxValue,
                                                transientTime, A.d(vals), vals.size,
                                                None if dr is None else A.d(dr), _out_ptr(out)))
    return out


def legacy_lle_draws(kind, n, nx, stream=None):
    """The legacy kernels' raw twin draws drawn on the device
    (chaos_legacy_lle_draws): kind 0 parameter-grid LLE (cuRAND) and 1
    initial-condition LLE (sinf), [n, nx]; kind 2 the spectrum, [n, nx, nx]."""
    out = np.zeros((n, nx, nx) if kind == 2 else (n, nx))
    ex = _exec(FP64, {"draws": out}, stream)
    _check(lib().chaos_legacy_lle_draws(C.byref(ex), kind, n, nx, _out_ptr(out)))
    return out


def lyapunov_spectrum(system, dim, tMax, NT, nPts, h, eps, initialConditions, ranges, indicesOfMutVars,
                      transientTime, values, mutateState=False, precision=FP64, out=None, stream=None, gridMode=0):
    """Lyapunov spectrum [points, SIZE_X] over the grids of lle_sweep
    (chaos_lyapunov_spectrum)."""
    A = _Args()
    ic = np.asarray(initialConditions, np.float64)
    n = nPts ** dim
    if out is None:
        out = np.zeros((n, ic.size))
    ex = _exec(precision, {"spectrum": out}, stream)
    vals = np.asarray(values, np.float64)
    mode = gridMode | (GRID_STATE if mutateState else 0)
    _check(lib().chaos_lyapunov_spectrum(C.byref(ex), _sys(system), dim, mode, tMax, NT, nPts, h,
                                         eps, A.d(ic), ic.size, A.d(ranges), A.i(indicesOfMutVars), transientTime,
                                         A.d(vals), vals.size, _out_ptr(out)))
    return out


def lle2d_checked(system, tMax, NT, nPts, h, eps, initialConditions, ranges, indicesOfMutVars, transientTime,
                  values, band=0.01, checkTMax=None, out=None, stream=None):
    """FP32 LLE map whose points with |value| <= band (or not finite) get an
    FP64 re-check over checkTMax (default tMax / 10) time units; points whose
    sign class the check contradicts carry their full FP64 value. Returns
    (lle, n_checked, n_replaced)."""
    A = _Args()
    if out is None:
        out = np.zeros(nPts * nPts)
    ex = _exec(FP32, {"lle": out}, stream)
    ic = np.asarray(initialConditions, np.float64)
    vals = np.asarray(values, np.float64)
    nc, nr = C.c_longlong(), C.c_longlong()
    _check(lib().chaos_lle2d_checked(C.byref(ex), _sys(system), tMax, NT, nPts, h, eps, A.d(ic), ic.size,
                                     A.d(ranges), A.i(indicesOfMutVars), transientTime, A.d(vals), vals.size, band,
                                     tMax / 10 if checkTMax is None else checkTMax, _out_ptr(out), C.byref(nc),
                                     C.byref(nr)))
    return out, nc.value, nr.value


def basins_features(system, tMax, nPts, h, initialConditions, ranges, indicesOfMutVars, writableVar, maxValue,
                    transientTime, values, preScaller=1, precision=FP64, out=None, stream=None):
    A = _Args()
    n = nPts * nPts
    if out is None:
        out = dict(flags=np.zeros(n, np.int32), avg_peaks=np.zeros(n), avg_intervals=np.zeros(n),
                   counts=np.zeros(n, np.int32))
    ex = _exec(precision, out, stream)
    ic = np.asarray(initialConditions, np.float64)
    vals = np.asarray(values, np.float64)
    _check(lib().chaos_basins_features(C.byref(ex), _sys(system), tMax, nPts, h, ic.size, A.d(ic), A.d(ranges),
                                       A.i(indicesOfMutVars), writableVar, maxValue, transientTime, A.d(vals),
                                       vals.size, preScaller, _out_ptr(out["flags"]), _out_ptr(out["avg_peaks"]),
                                       _out_ptr(out["avg_intervals"]), _out_ptr(out.get("counts"))))
    return out


def basins(system, tMax, nPts, h, initialConditions, ranges, indicesOfMutVars, writableVar, maxValue,
           transientTime, values, preScaller=1, eps=0.05, precision=FP64, out=None, stream=None):
    A = _Args()
    n = nPts * nPts
    if out is None:
        out = dict(labels=np.zeros(n, np.int32), avg_peaks=np.zeros(n), avg_intervals=np.zeros(n),
                   flags=np.zeros(n, np.int32))
    ex = _exec(precision, out, stream)
    ic = np.asarray(initialConditions, np.float64)
    vals = np.asarray(values, np.float64)
    _check(lib().chaos_basins(C.byref(ex), _sys(system), tMax, nPts, h, ic.size, A.d(ic), A.d(ranges),
                              A.i(indicesOfMutVars), writableVar, maxValue, transientTime, A.d(vals), vals.size,
                              preScaller, eps, _out_ptr(out["labels"]), _out_ptr(out.get("avg_peaks")),
                              _out_ptr(out.get("avg_intervals")), _out_ptr(out.get("flags"))))
    return out


def basins_dbscan(system, tMax, nPts, h, initialConditions, ranges, indicesOfMutVars, writableVar, maxValue,
                  transientTime, values, preScaller=1, eps=0.05, minPts=8, precision=FP64, out=None, stream=None,
                  with_features=True):
    """Basins with normalised (amplitude, peak count, interval) features and
    textbook DBSCAN; labels 0.. clusters, -1 noise, -2 diverged. The n x 3
    feature matrix is returned when with_features (or when out holds it)."""
    A = _Args()
    n = nPts * nPts
    if out is None:
        out = dict(labels=np.zeros(n, np.int32), flags=np.zeros(n, np.int32))
        if with_features:
            out["features"] = np.zeros((n, 3))
    ex = _exec(precision, out, stream)
    ic = np.asarray(initialConditions, np.float64)
    vals = np.asarray(values, np.float64)
    _check(lib().chaos_basins_dbscan(C.byref(ex), _sys(system), tMax, nPts, h, ic.size, A.d(ic), A.d(ranges),
                                     A.i(indicesOfMutVars), writableVar, maxValue, transientTime, A.d(vals),
                                     vals.size, preScaller, eps, minPts, _out_ptr(out["labels"]),
                                     _out_ptr(out.get("features")), _out_ptr(out.get("flags"))))
    return out


def dbscan_compat(avg_peaks, avg_intervals, flags, eps, out=None, stream=None):
    A = _Args()
    n = len(avg_peaks)
    if out is None:
        out = np.zeros(n, np.int32)
    if hasattr(out, "data_ptr"):
        ex = _exec(FP64, {"labels": out}, stream)
        ptrs = (avg_peaks.data_ptr(), avg_intervals.data_ptr(), flags.data_ptr())
    else:
        ex = _exec(FP64, {}, stream)
        ptrs = (A.d(avg_peaks), A.d(avg_intervals), A.i(flags))
    _check(lib().chaos_dbscan_compat(C.byref(ex), *ptrs, n, eps, _out_ptr(out)))
    return out


def dbscan(features, eps, min_pts, mask=None, out=None, stream=None):
    A = _Args()
    if hasattr(features, "data_ptr"):
        n, d = features.shape
        if out is None:
            import torch

            out = torch.empty(n, dtype=torch.int32, device=features.device)
        ex = _exec(FP64, {"labels": out}, stream)
        _check(lib().chaos_dbscan(C.byref(ex), features.data_ptr(), n, d, eps, min_pts,
                                  None if mask is None else mask.data_ptr(), out.data_ptr()))
        return out
    f = np.ascontiguousarray(np.atleast_2d(features), np.float64)
    n, d = f.shape
    if out is None:
        out = np.zeros(n, np.int32)
    ex = _exec(FP64, {}, stream)
    _check(lib().chaos_dbscan(C.byref(ex), A.d(f), n, d, eps, min_pts, None if mask is None else A.i(mask),
                              _out_ptr(out)))
    return out


def peak_finder(data, h, peakCapacity=None, stream=None):
    A = _Args()
    d = np.ascontiguousarray(np.atleast_2d(data), np.float64)
    n, ln = d.shape
    cap = int(peakCapacity or max(ln // 2, 1))
    out = dict(counts=np.zeros(n, np.int32), peaks=np.zeros((n, cap)), intervals=np.zeros((n, cap)))
    ex = _exec(FP64, {}, stream)
    _check(lib().chaos_peak_finder(C.byref(ex), A.d(d), n, ln, h, cap, _out_ptr(out["counts"]),
                                   _out_ptr(out["peaks"]), _out_ptr(out["intervals"])))
    return out


def point_dbscan(intervals, counts, eps, stream=None):
    A = _Args()
    iv = np.ascontiguousarray(np.atleast_2d(intervals), np.float64)
    n, stride = iv.shape
    out = np.zeros(n, np.int32)
    ex = _exec(FP64, {}, stream)
    _check(lib().chaos_point_dbscan(C.byref(ex), A.d(iv), A.i(counts), n, stride, eps, _out_ptr(out)))
    return out


# ---- the reference's entry points (CSV files) -----------------------------------

def bifurcation1D(tMax, nPts, h, amountOfInitialConditions, initialConditions, ranges, indicesOfMutVars,
                  writableVar, maxValue, transientTime, values, amountOfValues, preScaller, OUT_FILE_PATH):
    A = _Args()
    _check(lib().chaos_compat_bifurcation1D(tMax, nPts, h, amountOfInitialConditions, A.d(initialConditions),
                                            A.d(ranges), A.i(indicesOfMutVars), writableVar, maxValue,
                                            transientTime, A.d(values), amountOfValues, preScaller,
                                            str(OUT_FILE_PATH).encode()))


def bifurcation2D(tMax, nPts, h, amountOfInitialConditions, initialConditions, ranges, indicesOfMutVars,
                  writableVar, maxValue, transientTime, values, amountOfValues, preScaller, eps, OUT_FILE_PATH):
    A = _Args()
    _check(lib().chaos_compat_bifurcation2D(tMax, nPts, h, amountOfInitialConditions, A.d(initialConditions),
                                            A.d(ranges), A.i(indicesOfMutVars), writableVar, maxValue,
                                            transientTime, A.d(values), amountOfValues, preScaller, eps,
                                            str(OUT_FILE_PATH).encode()))


def LLE2D(tMax, NT, nPts, h, eps, initialConditions, amountOfInitialConditions, ranges, indicesOfMutVars,
          writableVar, maxValue, transientTime, values, amountOfValues, OUT_FILE_PATH):
    A = _Args()
    _check(lib().chaos_compat_LLE2D(tMax, NT, nPts, h, eps, A.d(initialConditions), amountOfInitialConditions,
                                    A.d(ranges), A.i(indicesOfMutVars), writableVar, maxValue, transientTime,
                                    A.d(values), amountOfValues, str(OUT_FILE_PATH).encode()))


def basinsOfAttraction_2(tMax, nPts, h, amountOfInitialConditions, initialConditions, ranges, indicesOfMutVars,
                         writableVar, maxValue, transientTime, values, amountOfValues, preScaller, eps,
                         OUT_FILE_PATH):
    A = _Args()
    _check(lib().chaos_compat_basinsOfAttraction_2(tMax, nPts, h, amountOfInitialConditions, A.d(initialConditions),
                                                   A.d(ranges), A.i(indicesOfMutVars), writableVar, maxValue,
                                                   transientTime, A.d(values), amountOfValues, preScaller, eps,
                                                   str(OUT_FILE_PATH).encode()))


# namespaces as in the reference (Bifurcation::bifurcation1D, LLE::LLE2D, Basins::basinsOfAttraction_2)
Bifurcation = SimpleNamespace(bifurcation1D=bifurcation1D, bifurcation2D=bifurcation2D)
LLE = SimpleNamespace(LLE2D=LLE2D)
Basins = SimpleNamespace(basinsOfAttraction_2=basinsOfAttraction_2)


# ---- the legacy library's analyses (old_library::..., CSV files) -----------------

def _legacy_bif(name, with_eps):
    def call(tMax, nPts, h, amountOfInitialConditions, initialConditions, ranges, indicesOfMutVars, writableVar,
             maxValue, transientTime, values, amountOfValues, preScaller, *rest):
        A = _Args()
        tail = (rest[0], str(rest[1]).encode()) if with_eps else (str(rest[0]).encode(),)
        _check(getattr(lib(), name)(tMax, nPts, h, amountOfInitialConditions, A.d(initialConditions), A.d(ranges),
                                    A.i(indicesOfMutVars), writableVar, maxValue, transientTime, A.d(values),
                                    amountOfValues, preScaller, *tail))
    call.__name__ = name.replace("chaos_compat_", "")
    return call


def _legacy_lle(name):
    def call(tMax, NT, nPts, h, eps, initialConditions, amountOfInitialConditions, ranges, indicesOfMutVars,
             writableVar, maxValue, transientTime, values, amountOfValues, OUT_FILE_PATH):
        A = _Args()
        _check(getattr(lib(), name)(tMax, NT, nPts, h, eps, A.d(initialConditions), amountOfInitialConditions,
                                    A.d(ranges), A.i(indicesOfMutVars), writableVar, maxValue, transientTime,
                                    A.d(values), amountOfValues, str(OUT_FILE_PATH).encode()))
    call.__name__ = name.replace("chaos_compat_", "")
    return call


def bifurcation1DForH(tMax, nPts, amountOfInitialConditions, initialConditions, ranges, writableVar, maxValue,
                      transientTime, values, amountOfValues, preScaller, OUT_FILE_PATH):
    A = _Args()
    _check(lib().chaos_compat_bifurcation1DForH(tMax, nPts, amountOfInitialConditions, A.d(initialConditions),
                                                A.d(ranges), writableVar, maxValue, transientTime, A.d(values),
                                                amountOfValues, preScaller, str(OUT_FILE_PATH).encode()))


old_library = SimpleNamespace(
    bifurcation1DIC=_legacy_bif("chaos_compat_bifurcation1DIC", False),
    bifurcation2DIC=_legacy_bif("chaos_compat_bifurcation2DIC", True),
    bifurcation1DForH=bifurcation1DForH,
    basinsOfAttraction=_legacy_bif("chaos_compat_basinsOfAttraction", True),
    LLE1D=_legacy_lle("chaos_compat_LLE1D"),
    LLE1DIC=_legacy_lle("chaos_compat_LLE1DIC"),
    LLE2DIC=_legacy_lle("chaos_compat_LLE2DIC"),
    LS1D=_legacy_lle("chaos_compat_LS1D"),
    LS2D=_legacy_lle("chaos_compat_LS2D"),
)
