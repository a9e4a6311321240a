"""GB300 (sm_103a) engine for ChaosLibrary's bifurcation / LLE / basins hot path.

Python front end over the C ABI in include/chaos_gb300.h (libchaos_gb300.so,
built by ``chaoslibrary_gb300.build``). Two layers:

* the reference's four entry points with their exact argument lists
  (``bifurcation1D``, ``bifurcation2D``, ``LLE2D``, ``basinsOfAttraction_2``),
  which write the reference's CSV files;
* array functions (``bifurcation1d``, ``lle2d``, ``basins``, ``dbscan`` ...)
  that return numpy arrays, or write into CUDA tensors when given ``out=``.

There is no CPU implementation here: without the built library every call
raises.
"""
from __future__ import annotations

from ._native import (  # noqa: F401
    Batch,
    FF32,
    FP32,
    FP64,
    SYSTEMS,
    ChaosError,
    LLE2D,
    Server,
    Basins,
    Bifurcation,
    LLE,
    basins,
    basins_dbscan,
    basins_features,
    basinsOfAttraction_2,
    bifurcation1D,
    bifurcation1d,
    bifurcation2D,
    bifurcation2d,
    bifurcation_sweep,
    compact_peaks,
    GRID_STATE,
    GRID_LOG0,
    GRID_LOG1,
    GRID_LOG_F32,
    GRID_LEGACY_LOOP,
    MUT_STEP,
    dbscan,
    dbscan_compat,
    device_code_version,
    fma_probe,
    autotune,
    launch_count,
    lle2d_checked,
    lle_from_states,
    lle_sweep,
    lle_sweep_legacy,
    legacy_lle_draws,
    lyapunov_spectrum_legacy,
    lyapunov_spectrum,
    get_tuning,
    set_tuning,
    TUNE_LLE_F32_VARIANT,
    TUNE_SWEEP_PAIRS,
    TUNE_GRID_FMA,
    TUNE_LLE_TWIN,
    TUNE_BIF2D_CAP,
    TUNE_SHAPES,
    TUNE_LLE_RENORM,
    TUNE_FF_PAIRS,
    lib,
    lib_path,
    lle2d,
    old_library,
    peak_finder,
    point_dbscan,
    set_precision,
    set_system,
    system_info,
    trajectory,
)

__all__ = [
    "Server", "Batch", "FF32", "FP32", "FP64", "SYSTEMS", "ChaosError", "bifurcation1D", "bifurcation2D", "LLE2D", "basinsOfAttraction_2",
    "Bifurcation", "LLE", "Basins", "bifurcation1d", "bifurcation2d", "bifurcation_sweep", "compact_peaks", "GRID_STATE",
    "GRID_LOG0", "GRID_LOG1", "GRID_LOG_F32", "GRID_LEGACY_LOOP", "MUT_STEP", "lle2d", "old_library", "basins", "basins_dbscan", "basins_features",
    "dbscan", "dbscan_compat", "device_code_version", "fma_probe", "autotune", "launch_count", "lle2d_checked", "lle_from_states", "lle_sweep", "lle_sweep_legacy", "legacy_lle_draws", "lyapunov_spectrum", "lyapunov_spectrum_legacy", "trajectory", "get_tuning", "set_tuning", "TUNE_LLE_F32_VARIANT", "TUNE_SWEEP_PAIRS", "TUNE_GRID_FMA", "TUNE_LLE_TWIN", "TUNE_BIF2D_CAP", "TUNE_SHAPES", "TUNE_LLE_RENORM", "TUNE_FF_PAIRS", "peak_finder", "point_dbscan", "lib", "lib_path", "set_system", "set_precision", "system_info",
]
