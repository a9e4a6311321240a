"""Builds libchaos_gb300.so (all CUDA kernels + the C ABI + the compat wrappers)
for sm_103a with nvcc, in-tree, translation units compiled in parallel."""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIBDIR = PKG / "lib"
LIB = LIBDIR / "libchaos_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code keeps every rounding it writes too (gcc contracts a*b + c into an
# FMA on aarch64 by default): grid values and CSV coordinates match the oracle.
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
          "-Xcompiler", "-ffp-contract=off"]

# (source, extra flags). The FP64 and clustering units keep every rounding
# the source writes (no multiply-add contraction).
SOURCES = [
    ("kern_f64.cu", ["--fmad=false"]),
    ("tune.cu", []),
    ("kern_f32.cu", []),
    ("kern_ff.cu", ["--fmad=false"]),
    ("dbscan.cu", ["--fmad=false", "--extended-lambda"]),
    ("capi.cu", []),
    ("batch.cu", []),
    ("batch_host.cu", []),
    ("server.cu", []),
    ("probe.cu", []),
    ("noalloc.cu", []),
    ("peaks_compact.cu", []),
    ("compat.cpp", []),
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise FileNotFoundError("nvcc not found")


def _deps() -> list[Path]:
    return sorted(CSRC.glob("*")) + sorted((PKG.parent / "include").glob("*.h*")) + [Path(__file__)]


def up_to_date() -> bool:
    if not LIB.exists() or not (LIBDIR / "chaos_perf").exists():
        return False
    t = LIB.stat().st_mtime
    return all(d.stat().st_mtime <= t for d in _deps())


def build(force: bool = False, verbose: bool = False, user_systems: str | None = None, lib: Path | None = None,
          build_dir: Path | None = None) -> Path:
    """Builds the library. user_systems (or the environment variable
    CHAOS_USER_SYSTEMS) names a reference-format systems.cuh plug-in header to
    compile in as system CHAOS_SYS_USER; lib / build_dir redirect the output."""
    user_systems = user_systems or os.environ.get("CHAOS_USER_SYSTEMS")
    out = Path(lib).resolve() if lib else LIB
    bdir = Path(build_dir) if build_dir else BUILD
    if not force and out == LIB and not user_systems and up_to_date():
        return LIB
    bdir.mkdir(parents=True, exist_ok=True)
    out.parent.mkdir(parents=True, exist_ok=True)
    cc = nvcc()
    procs = []
    objs = []
    sources = list(SOURCES)
    if user_systems:
        hdr = Path(user_systems).resolve()
        sources.append(("kern_user.cu", ["--fmad=false", f'-DCHAOS_USER_SYSTEM_HEADER="{hdr}"', f"-I{hdr.parent}"]))
    else:
        sources.append(("user_stub.cu", []))
    for src, extra in sources:
        obj = bdir / (src + ".o")
        objs.append(obj)
        cmd = [cc, *ARCH, *COMMON, *extra, "-c", str(CSRC / src), "-o", str(obj)]
        if src.endswith(".cpp"):
            cmd = [cc, *COMMON, "-x", "c++", "-c", str(CSRC / src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    failed = []
    for src, p in procs:
        log, _ = p.communicate()
        if p.returncode != 0:
            failed.append(f"--- {src}\n{log}")
        elif verbose and log.strip():
            print(log)
    if failed:
        raise RuntimeError("nvcc failed:\n" + "\n".join(failed))
    tmp = out.with_suffix(f".{os.getpid()}.tmp")
    link = [cc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
    if verbose:
        print(" ".join(link), flush=True)
    subprocess.run(link, check=True)
    os.replace(tmp, out)
    if out == LIB:
        build_cli(verbose)
    return out


CLI = LIBDIR / "chaos_perf"


def build_cli(verbose: bool = False) -> Path:
    """Builds chaos_perf, the command-line driver of the reference's
    performance sweeps, linked against the library beside it."""
    tmp = CLI.with_suffix(f".{os.getpid()}.tmp")
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", str(CSRC / "perf_main.cpp"), "-o", str(tmp), f"-L{LIBDIR}",
           "-lchaos_gb300", "-Wl,-rpath,$ORIGIN"]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.run(cmd, check=True)
    os.replace(tmp, CLI)
    return CLI


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
