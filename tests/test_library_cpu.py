"""The engine library without a GPU: it builds for sm_103a, loads, exports
every entry point the public headers declare, and rejects bad arguments on
the host (CHAOS_E_ARGS) before touching a device."""
import ctypes as C
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def native():
    from chaoslibrary_gb300 import build as B

    B.build()
    from chaoslibrary_gb300 import _native as N

    N.lib()
    return N


def declared_c_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h*"):
        text = h.read_text()
        names.update(re.findall(r"^\s*(?:const\s+)?\w+\**\s+\**(chaos_\w+)\s*\(", text, re.M))
    return sorted(names)


def test_headers_declare_entry_points():
    names = declared_c_functions()
    for must in ("chaos_bifurcation1d", "chaos_bifurcation2d", "chaos_lle2d", "chaos_basins", "chaos_dbscan",
                 "chaos_dbscan_compat", "chaos_peak_finder", "chaos_point_dbscan", "chaos_compat_LLE2D"):
        assert must in names


def test_every_declared_symbol_is_exported(native):
    L = native.lib()
    missing = [n for n in declared_c_functions() if not hasattr(L, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-DC", str(native.lib_path())], capture_output=True, text=True).stdout
    for cxx in ("Bifurcation::bifurcation1D(", "Bifurcation::bifurcation2D(", "LLE::LLE2D(",
                "Basins::basinsOfAttraction_2(", "old_library::bifurcation1DIC(", "old_library::bifurcation2DIC(",
                "old_library::bifurcation1DForH(", "old_library::LLE1D(", "old_library::LLE1DIC(",
                "old_library::LLE2DIC(", "old_library::LS1D(", "old_library::LS2D(",
                "old_library::basinsOfAttraction("):
        assert cxx in out, cxx


def test_build_targets_sm_103a_only():
    from chaoslibrary_gb300 import build as B

    assert B.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_abi_version_and_system_info(native):
    assert native.lib().chaos_abi_version() == 1
    assert native.system_info("lorenz") == (3, 3)
    assert native.system_info("chameleon") == (3, 7)
    assert native.system_info("sin2") == (2, 2)
    with pytest.raises(native.ChaosError) as e:
        native.system_info(42)
    assert e.value.code == -1


BIF = dict(tMax=1.0, nPts=8, h=0.01, initialConditions=[0.1, 0.1, 0.1], ranges=[20.0, 200.0],
           indicesOfMutVars=[1], writableVar=0, maxValue=1e4, transientTime=1.0, values=[10.0, 28.0, 8 / 3])


@pytest.mark.parametrize("bad, frag", [
    (dict(system=99), "unknown system"),
    (dict(values=[10.0, 28.0]), "amountOfValues"),
    (dict(initialConditions=[0.1, 0.1]), "amountOfInitialConditions"),
    (dict(nPts=1), "nPts"),
    (dict(h=0.0), "h > 0"),
    (dict(indicesOfMutVars=[5]), "indicesOfMutVars"),
    (dict(writableVar=3), "writableVar"),
    (dict(preScaller=0), "preScaller"),
])
def test_bifurcation_argument_errors(native, bad, frag):
    kw = dict(BIF)
    system = bad.pop("system", "lorenz")
    kw.update(bad)
    with pytest.raises(native.ChaosError) as e:
        native.bifurcation1d(system, **kw)
    assert e.value.code == -1 and frag in str(e.value)


def test_lle_argument_errors(native):
    kw = dict(tMax=10.0, NT=0.1, nPts=4, h=0.01, eps=1e-8, initialConditions=[1.0, 1.0, 1.0],
              ranges=[0.1, 0.4, 2.0, 10.0], indicesOfMutVars=[0, 2], transientTime=5.0, values=[0.2, 0.2, 5.7])
    with pytest.raises(native.ChaosError, match="NT / h"):
        native.lle2d("rossler", **{**kw, "NT": 0.001})
    with pytest.raises(native.ChaosError) as e:
        native.lle2d("rossler_cd", **{**kw, "values": [0.2, 0.2, 5.7, 0.0]}, precision=native.FP32)
    assert e.value.code == -6  # FP32 LLE needs a quadratic RK4 system or Chameleon


def test_ff32_refused_where_not_implemented(native):
    """CHAOS_FF32 runs the LLE maps and trajectories of the RK4 systems; every
    other call refuses it (CHAOS_E_UNSUPPORTED) before touching a device,
    instead of running another precision."""
    with pytest.raises(native.ChaosError) as e:
        native.lle2d("chameleon", precision=native.FF32, tMax=1.0, NT=0.1, nPts=4, h=0.01, eps=1e-6,
                     initialConditions=[3.0, 3.0, 0.0], ranges=[0.0, 5.0, 0.0, 20.0], indicesOfMutVars=[3, 5],
                     transientTime=1.0, values=[0.5, 3, 0, 2, 1, 18, 1])
    assert e.value.code == -6
    with pytest.raises(native.ChaosError) as e:
        native.bifurcation1d("lorenz", precision=native.FF32, **BIF)
    assert e.value.code == -6 and "CHAOS_FF32" in str(e.value)
    with pytest.raises(native.ChaosError) as e:
        native.trajectory("sin3", [[0.1, 0.1, 0.1]], [[1, 1, 1, 1, 1]], 0.01, 3, precision=native.FF32)
    assert e.value.code == -6
    with pytest.raises(native.ChaosError, match="unknown precision"):
        native.lle2d("rossler", precision="fp16", tMax=1.0, NT=0.1, nPts=4, h=0.01, eps=1e-8,
                     initialConditions=[1.0, 1.0, 1.0], ranges=[0.1, 0.4, 2.0, 10.0], indicesOfMutVars=[0, 2],
                     transientTime=1.0, values=[0.2, 0.2, 5.7])


def test_lle_from_states_argument_errors(native):
    st = np.zeros((4, 9))
    with pytest.raises(native.ChaosError) as e:
        native.lle_from_states("rossler", st, 10.0, 0.1, 0.01, 1e-8, precision=native.FP32)
    assert e.value.code == -6
    with pytest.raises(native.ChaosError) as e:
        native.lle_from_states("chameleon", np.zeros((4, 13)), 10.0, 0.1, 0.01, 1e-8, precision=native.FF32)
    assert e.value.code == -6
    with pytest.raises(native.ChaosError, match="NT / h"):
        native.lle_from_states("rossler", st, 10.0, 0.001, 0.01, 1e-8)


def test_dbscan_argument_errors(native):
    with pytest.raises(native.ChaosError, match="dims"):
        native.dbscan(np.zeros((4, 5)), 0.1, 2)
    with pytest.raises(native.ChaosError, match="minPts"):
        native.dbscan(np.zeros((4, 2)), 0.1, 0)


def test_grid_mode_argument_errors(native):
    kw = dict(tMax=5.0, nPts=8, h=0.01, initialConditions=[0.1, 0.1, 0.1], writableVar=0, maxValue=1e4,
              transientTime=1.0, values=[10.0, 28.0, 8 / 3])
    with pytest.raises(native.ChaosError, match="positive"):
        native.bifurcation_sweep("lorenz", 1, native.GRID_LOG0, ranges=[-1.0, 10.0], indicesOfMutVars=[1], **kw)
    with pytest.raises(native.ChaosError, match="1-D"):
        native.bifurcation_sweep("lorenz", 2, 0, ranges=[0.01, 0.02, 1.0, 2.0],
                                 indicesOfMutVars=[native.MUT_STEP, 0], **kw)
    with pytest.raises(native.ChaosError, match="grid mode"):
        native.bifurcation_sweep("lorenz", 1, 64, ranges=[1.0, 10.0], indicesOfMutVars=[1], **kw)
    with pytest.raises(native.ChaosError, match="dim 2"):
        native.lle_sweep("lorenz", 1, 5.0, 0.1, 8, 0.01, 1e-8, [0.1, 0.1, 0.1], [1.0, 10.0], [1], 1.0,
                         [10.0, 28.0, 8 / 3], gridMode=native.GRID_LOG1)
    # the legacy per-point loop belongs to the bifurcation sweep; the LLE sweeps have their own legacy scheme
    with pytest.raises(native.ChaosError, match="bifurcation sweep"):
        native.lle_sweep("lorenz", 1, 5.0, 0.1, 8, 0.01, 1e-8, [0.1, 0.1, 0.1], [1.0, 10.0], [1], 1.0,
                         [10.0, 28.0, 8 / 3], gridMode=native.GRID_LEGACY_LOOP)
    with pytest.raises(native.ChaosError, match="bifurcation sweep"):
        native.lle_sweep_legacy("lorenz", 1, 5.0, 0.1, 8, 0.01, 1e-8, [0.1, 0.1, 0.1], [1.0, 10.0], [1], 1.0,
                                [10.0, 28.0, 8 / 3], gridMode=native.GRID_LEGACY_LOOP)


def test_legacy_scheme_argument_errors(native):
    """The legacy LLE / spectrum schemes and their twin draws validate on the
    host; the twin-start knob takes 0, 1 or 2."""
    with pytest.raises(native.ChaosError, match="twin-draw"):
        native.legacy_lle_draws(3, 10, 3)
    with pytest.raises(native.ChaosError, match="twin-draw"):
        native.legacy_lle_draws(0, 10, 13)
    with pytest.raises(native.ChaosError, match="built-in systems"):  # 15: CHAOS_SYS_USER
        native.lyapunov_spectrum_legacy(15, 1, 5.0, 0.1, 8, 0.01, 1e-8, [0.1, 0.1, 0.1], [1.0, 10.0], [1], 1.0,
                                        [10.0, 28.0, 8 / 3])
    with pytest.raises(native.ChaosError, match="NT / h"):
        native.lle_sweep_legacy("lorenz", 1, 5.0, 0.001, 8, 0.01, 1e-8, [0.1, 0.1, 0.1], [1.0, 10.0], [1], 1.0,
                                [10.0, 28.0, 8 / 3])
    knob = native.TUNE_LLE_TWIN
    try:
        native.set_tuning(knob, 2)
        assert native.get_tuning(knob) == 2
        with pytest.raises(native.ChaosError, match="0 to 2"):
            native.set_tuning(knob, 3)
        with pytest.raises(native.ChaosError, match="0 to 1"):
            native.set_tuning(native.TUNE_GRID_FMA, 2)
    finally:
        native.set_tuning(knob, 0)


def test_compact_peaks_argument_errors(native):
    import ctypes as C

    L = native.lib()
    total = C.c_longlong(0)
    cnt = np.zeros(4, np.int32)
    assert L.chaos_compact_peaks(None, cnt.ctypes.data, None, None, 4, 0, None, None, None, None, 0,
                                 C.byref(total)) == -1
    assert L.chaos_compact_peaks(None, None, None, None, 4, 8, None, None, None, None, 0, C.byref(total)) == -1
    out = np.zeros(4)
    assert L.chaos_compact_peaks(None, cnt.ctypes.data, None, None, 4, 8, None, out.ctypes.data, None, None, 4,
                                 C.byref(total)) == -1  # dense peaks without the peak rows


def test_compat_system_selection(native):
    L = native.lib()
    assert L.chaos_compat_set_system(99) == -1
    assert L.chaos_compat_set_system(0) == 0
    assert L.chaos_compat_get_system() == 0
    assert L.chaos_compat_set_system(3) == 0


def test_compat_unknown_system_name_is_an_error(native, tmp_path):
    """CHAOS_SYSTEM with a name the library does not know makes the
    reference-signature wrappers fail with CHAOS_E_ARGS instead of running
    another system (fresh process: the selection is read once)."""
    code = (
        "import ctypes as C\n"
        f"L = C.CDLL({str(native.lib_path())!r})\n"
        "L.chaos_last_error.restype = C.c_char_p\n"
        "assert L.chaos_compat_get_system() == -1\n"
        "D = C.c_double * 3\n"
        "f = L.chaos_compat_bifurcation1D\n"
        "f.argtypes = [C.c_double, C.c_int, C.c_double, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,\n"
        "              C.c_double, C.c_double, C.c_void_p, C.c_int, C.c_int, C.c_char_p]\n"
        "ic, rg, v = D(0.1, 0.1, 0.1), D(20.0, 200.0, 0.0), D(10.0, 28.0, 8.0 / 3.0)\n"
        "mv = (C.c_int * 1)(1)\n"
        f"rc = f(1.0, 8, 0.01, 3, ic, rg, mv, 0, 1e4, 1.0, v, 3, 1, {str(tmp_path / 'out.csv')!r}.encode())\n"
        "assert rc == -1, rc\n"
        "assert b'unknown system' in L.chaos_last_error(), L.chaos_last_error()\n"
    )
    import os
    import sys

    env = {**os.environ, "CHAOS_SYSTEM": "lorenzz"}
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env)
    assert out.returncode == 0, out.stderr
    assert not (tmp_path / "out.csv").exists()


def test_no_cpu_fallback(monkeypatch, tmp_path):
    """Without the built library the package raises instead of computing."""
    from chaoslibrary_gb300 import _native as N

    monkeypatch.setattr(N, "_lib", None)
    monkeypatch.setenv("CHAOS_GB300_LIB", str(tmp_path / "missing.so"))
    with pytest.raises(N.ChaosError, match="no CPU fallback"):
        N.bifurcation1d("lorenz", **BIF)


def test_perf_cli_builds_and_parses(native, tmp_path):
    """chaos_perf (the reference's performance sweeps as a Linux CLI) links
    against the library and rejects unknown options without touching a GPU."""
    cli = native.lib_path().parent / "chaos_perf"
    assert cli.exists()
    out = subprocess.run([str(cli), "--help"], capture_output=True, text=True)
    assert out.returncode == 0 and "--suite" in out.stdout
    bad = subprocess.run([str(cli), "--suite", "nothing"], capture_output=True, text=True)
    assert bad.returncode == 2
    bad = subprocess.run([str(cli), "--basins-system", "sin33"], capture_output=True, text=True)
    assert bad.returncode == 2 and "unknown system" in bad.stderr
