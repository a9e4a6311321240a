"""Build the reference's own GPU path for timing on the GB300 (measurement only).

Recipe: copy the reference sources the 1-D bifurcation and LLE paths need,
unchanged, from the reference checkout into ``oracle/_ref/gpu_src/``
(git-ignored; the benchmark machine has no reference checkout), then compile
them with nvcc for sm_103a together with ``oracle/ref_gpu_main.cu`` and the
Lorenz / Rossler RK4 plug-ins (``chaoslibrary_gb300/plugins/``) standing in
for ``systems/systems.cuh``:

  oracle/_ref/ref_gpu_bif1d   Bifurcation::bifurcation1D with the Lorenz RK4 plug-in
  oracle/_ref/ref_gpu_bif2d   Bifurcation::bifurcation2D with the reference's own systems.cuh (Chameleon)
  oracle/_ref/ref_gpu_lle2d   LLE::LLE2D with the Rossler RK4 plug-in
  oracle/_ref/ref_gpu_basins  Basins::basinsOfAttraction_2 with the Lorenz RK4 plug-in

Nothing here is shipped or called by the engine; ``bench.py`` runs these
binaries, when present, to time the reference beside the engine.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
OUT = HERE / "_ref"
STAGE = OUT / "gpu_src"
# The reference checkout: CHAOS_REFERENCE_DIR, else a directory named
# "reference" beside this repository.
REF = Path(os.environ.get("CHAOS_REFERENCE_DIR") or (REPO.parent / "reference"))
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")

FILES = ["Bifurcation/src/bifurcationCUDA.cu", "Bifurcation/src/bifurcationHOST.cpp",
         "Bifurcation/include/bifurcationCUDA.cuh", "Bifurcation/include/bifurcationHOST.h",
         "LLE/src/LLECUDA.cu", "LLE/src/LLEHost.cpp", "LLE/include/LLECUDA.cuh", "LLE/include/LLEHost.h",
         "Basins/src/basinsCUDA.cu", "Basins/src/basinsHOST.cpp", "Basins/include/basinsCUDA.cuh",
         "Basins/include/basinsHOST.h", "debri/cudaMacros.cu", "debri/cudaMacros.cuh", "systems/systems.cuh"]
TARGETS = {
    "bif1d": ("lorenz", "REF_BIF1D", ["Bifurcation/src/bifurcationCUDA.cu", "Bifurcation/src/bifurcationHOST.cpp"]),
    # the reference's own systems.cuh as shipped (its default plug-in, the Chameleon model)
    "bif2d": (None, "REF_BIF2D", ["Bifurcation/src/bifurcationCUDA.cu", "Bifurcation/src/bifurcationHOST.cpp"]),
    "lle2d": ("rossler", "REF_LLE2D", ["LLE/src/LLECUDA.cu", "LLE/src/LLEHost.cpp"]),
    "basins": ("lorenz", "REF_BASINS", ["Basins/src/basinsCUDA.cu", "Basins/src/basinsHOST.cpp"]),
    # the reference's LLE kernels on their own, dumping their starting states (ref_gpu_lle_states.cu
    # includes LLE/src/LLECUDA.cu itself)
    "lle_states": ("rossler", "REF_LLE_STATES", []),
}
MAINS = {"lle_states": "ref_gpu_lle_states.cu"}


def binary(name: str) -> Path:
    return OUT / f"ref_gpu_{name}"


def staged() -> bool:
    return all((STAGE / f).is_file() for f in FILES)


def stage() -> None:
    """Copies the listed reference sources (when the checkout is present)."""
    if not (REF / FILES[0]).is_file():
        return
    for f in FILES:
        dst = STAGE / f
        dst.parent.mkdir(parents=True, exist_ok=True)
        shutil.copy2(REF / f, dst)


def _build_one(name: str, verbose: bool) -> Path:
    system, macro, srcs = TARGETS[name]
    if system is None:
        sysdir = STAGE / "systems"
    else:
        sysdir = OUT / f"gsys_{system}"
        sysdir.mkdir(parents=True, exist_ok=True)
        (sysdir / "systems.cuh").write_text(f'#include "{REPO}/chaoslibrary_gb300/plugins/{system}_rk4.cuh"\n')
    exe = binary(name)
    cmd = [NVCC, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-w", f"-D{macro}",
           f"-I{sysdir}", f"-I{STAGE / 'Bifurcation/include'}", f"-I{STAGE / 'LLE/include'}",
           f"-I{STAGE / 'Basins/include'}",
           f"-I{STAGE / 'debri'}", f"-I{STAGE / 'LLE/src'}", "-x", "cu"] + [str(STAGE / s) for s in srcs] + \
          [str(STAGE / "debri/cudaMacros.cu"), str(HERE / MAINS.get(name, "ref_gpu_main.cu")), "-o", str(exe)]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True, capture_output=not verbose)
    return exe


def build(verbose: bool = False) -> list[Path]:
    stage()
    if not staged():
        raise FileNotFoundError("reference GPU sources are not staged (no reference checkout here)")
    OUT.mkdir(exist_ok=True)
    with ThreadPoolExecutor(len(TARGETS)) as ex:
        return list(ex.map(lambda n: _build_one(n, verbose), TARGETS))


if __name__ == "__main__":
    for p in build(verbose=True):
        print("built", p)
