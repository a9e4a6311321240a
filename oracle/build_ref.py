"""Build the reference's own per-thread code for the host (checker only).

Recipe: read the reference sources where they lie, copy the bodies of the
functions named below verbatim into ``oracle/_ref/*.inc`` (git-ignored), and
compile them with ``oracle/ref_harness.cpp`` and the CUDA host shim in
``oracle/ref_shim/`` into one shared library per plug-in system,
``oracle/_ref/libref_<system>.so``. Nothing here is shipped or called by the
engine; the tests use these libraries to pin the oracle to the reference, and
``bench.py``'s CPU baseline times the reference's own LLE code through them.
Where the reference checkout is absent (the benchmark machine), the recipe
compiles the extracted files and headers already under ``oracle/_ref``.

The reference's host drivers (which allocate device memory and launch
kernels) and its cuRAND-seeded LLE transient are not built.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent
OUT = HERE / "_ref"
# The reference checkout: CHAOS_REFERENCE_DIR, else a directory named
# "reference" beside this repository.
REF = Path(os.environ.get("CHAOS_REFERENCE_DIR") or (REPO.parent / "reference"))

BIF_FUNCS = ["calculateTransTimeCUDA", "calculateDiscreteModelCUDA", "peakFinderCUDA", "dbscanCUDA",
             "getValueByIdx", "loopCalculateDiscreteModel_int", "peakFinder", "dbscan", "distance"]
BASINS_FUNCS = ["getValueByIdx", "calculateDiscreteModel", "calculateTransTimeCUDA", "calculateDiscreteModelCUDA",
                "loopCalculateDiscreteModel_int", "peakFinder", "avgPeakFinderCUDA",
                "CUDA_dbscan_search_clear_points_kernel", "CUDA_dbscan_search_fixed_points_kernel",
                "CUDA_dbscan_kernel"]
LLE_FUNCS = ["loopCalculateDiscreteModel", "calculateDiscreteModel", "calculateSystem", "linspace"]
# the legacy library's functions behind the engine's legacy analyses (debri/cudaLibrary.cu): the
# helpers, its hard-wired system and loops, and the per-thread kernels of its bifurcation and
# basins analyses (in dependency order)
LEGACY_FUNCS = ["getValueByIdx", "getValueByIdxLog", "peakFinder", "projectionOperator", "gramSchmidtProcess",
                "calculateDiscreteModel", "loopCalculateDiscreteModel", "loopCalculateDiscreteModel_int",
                "distance", "dbscan", "calculateDiscreteModelICCUDA", "calculateDiscreteModelCUDA_H",
                "peakFinderCUDA", "peakFinderCUDA_H", "avgPeakFinderCUDA", "dbscanCUDA", "LLEKernelCUDA",
                "LLEKernelICCUDA", "LSKernelCUDA"]

# plug-in systems: name -> (header text of a systems.cuh stand-in)
PLUGINS = {
    "lorenz": f'#include "{REPO}/chaoslibrary_gb300/plugins/lorenz_rk4.cuh"\n',
    "rossler": f'#include "{REPO}/chaoslibrary_gb300/plugins/rossler_rk4.cuh"\n',
    "chen": f'#include "{REPO}/chaoslibrary_gb300/plugins/chen_rk4.cuh"\n',
}
# the reference's own plug-ins, one #ifdef block of systems/systems.cuh each
REF_SYSTEMS = {"chameleon": "USE_CHAMELEON_MODEL", "rossler_cd": "USE_ROSSLER_MODEL",
               "sin3": "USE_SYSTEM_FOR_BASINS", "sin2": "USE_SYSTEM_FOR_BASINS_2",
               "memristor": "USE_DAMIR_SYSTEM"}


def _strip_comment_mask(text: str) -> list[bool]:
    """True for every character that sits inside a // or /* */ comment."""
    mask = [False] * len(text)
    i, n = 0, len(text)
    while i < n:
        if text.startswith("//", i):
            j = text.find("\n", i)
            j = n if j < 0 else j
            for k in range(i, j):
                mask[k] = True
            i = j
        elif text.startswith("/*", i):
            j = text.find("*/", i + 2)
            j = n if j < 0 else j + 2
            for k in range(i, j):
                mask[k] = True
            i = j
        else:
            i += 1
    return mask


def extract_function(text: str, name: str) -> str:
    """Verbatim text of the (non-commented) definition of ``name``."""
    mask = _strip_comment_mask(text)
    pat = re.compile(r"(__global__|__device__|__host__)[\w\s\*&:<>]*?\b" + re.escape(name) + r"\s*\(")
    for m in pat.finditer(text):
        if mask[m.start()]:
            continue
        # find the ')' closing the parameter list, then the body
        depth, i = 0, m.end() - 1
        while i < len(text):
            c = text[i]
            if not mask[i]:
                if c == "(":
                    depth += 1
                elif c == ")":
                    depth -= 1
                    if depth == 0:
                        break
            i += 1
        j = i + 1
        while j < len(text) and (mask[j] or text[j].isspace()):
            j += 1
        if j >= len(text) or text[j] != "{":
            continue  # a declaration
        depth, k = 0, j
        while k < len(text):
            c = text[k]
            if not mask[k]:
                if c == "{":
                    depth += 1
                elif c == "}":
                    depth -= 1
                    if depth == 0:
                        return text[m.start():k + 1]
            k += 1
    raise RuntimeError(f"definition of {name} not found")


def extract_constants(text: str) -> str:
    return "\n".join(line for line in text.splitlines() if re.match(r"\s*__constant__\s", line))


def write_inc(src: Path, namespace: str, funcs: list[str], shared: str | None, dst: Path) -> None:
    text = src.read_text(encoding="utf-8", errors="replace")
    parts = [f"// extracted verbatim from {src} by oracle/build_ref.py", f"namespace {namespace} {{",
             extract_constants(text)]
    if shared:  # the kernel's shared memory: one array per replaying host thread
        parts.append(f"thread_local double {shared}[4096];")
    for f in funcs:
        parts.append(extract_function(text, f))
    parts.append("}")
    dst.write_text("\n\n".join(parts) + "\n")


def system_header(name: str) -> str:
    if name in PLUGINS:
        return PLUGINS[name]
    text = (REF / "systems" / "systems.cuh").read_text(encoding="utf-8", errors="replace")
    macro = REF_SYSTEMS[name]
    m = re.search(r"#ifdef\s+" + macro + r"\s*\n(.*?)\n#endif", text, re.S)
    if not m:
        raise RuntimeError(f"{macro} block not found")
    return ("#pragma once\n#include \"cuda_runtime.h\"\n#include <math.h>\n"
            f"// the {macro} block of {REF / 'systems' / 'systems.cuh'}\n" + m.group(1) + "\n")


STAGED = OUT / "gpu_src"  # the reference's headers, staged by oracle/build_ref_gpu.py


def _checkout() -> bool:
    return (REF / "Bifurcation" / "src" / "bifurcationCUDA.cu").is_file()


def _staged() -> bool:
    """The extracted functions, the system headers and the reference's headers
    are already under oracle/_ref (they travel with the tree to a machine
    without the reference checkout, where this recipe then compiles them)."""
    return all((OUT / f).is_file() for f in ("ref_bif.inc", "ref_basins.inc", "ref_lle.inc")) and \
        (STAGED / "Bifurcation/include").is_dir()


def available() -> bool:
    return _checkout() or _staged()


def build(systems: list[str] | None = None, verbose: bool = False) -> list[Path]:
    if not available():
        raise FileNotFoundError(f"reference sources not found under {REF}")
    OUT.mkdir(exist_ok=True)
    fresh = _checkout()
    inc_root = REF if fresh else STAGED
    if fresh:
        write_inc(REF / "Bifurcation/src/bifurcationCUDA.cu", "Bifurcation_constants", BIF_FUNCS, "s",
                  OUT / "ref_bif.inc")
        write_inc(REF / "Basins/src/basinsCUDA.cu", "basinsGPU", BASINS_FUNCS, None, OUT / "ref_basins.inc")
        write_inc(REF / "LLE/src/LLECUDA.cu", "LLE_constants", LLE_FUNCS, "sh_mem", OUT / "ref_lle.inc")
        write_inc(REF / "debri/cudaLibrary.cu", "legacy", LEGACY_FUNCS, "s", OUT / "ref_legacy.inc")
    built = []
    if (OUT / "ref_legacy.inc").is_file():
        lib = OUT / "libref_legacy.so"
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-w", f"-I{HERE / 'ref_shim'}",
               f"-I{OUT}", str(HERE / "ref_legacy_harness.cpp"), "-o", str(lib)]
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)
        built.append(lib)
    for name in systems or list(PLUGINS) + list(REF_SYSTEMS):
        sysdir = OUT / f"sys_{name}"
        sysdir.mkdir(exist_ok=True)
        if fresh or name in PLUGINS:
            (sysdir / "systems.cuh").write_text(system_header(name))
        elif not (sysdir / "systems.cuh").is_file():
            continue
        lib = OUT / f"libref_{name}.so"
        cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-w",
               f"-I{HERE / 'ref_shim'}", f"-I{sysdir}", f"-I{OUT}",
               f"-I{inc_root / 'Bifurcation/include'}", f"-I{inc_root / 'Basins/include'}",
               f"-I{inc_root / 'LLE/include'}", f"-I{inc_root / 'debri'}", str(HERE / "ref_harness.cpp"),
               "-o", str(lib)]
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)
        built.append(lib)
    return built


if __name__ == "__main__":
    for p in build(sys.argv[1:] or None, verbose=True):
        print("built", p)
