#!/usr/bin/env python
"""Benchmark of the bifurcation / LLE / basins engine on one GB300 (or N
replicas, one per GPU, under torchrun).

Default workload: the 2-D LLE map of the Rossler flow (classic RK4, h=0.01),
a in [0.1, 0.4] x c in [2, 10] on a 1024 x 1024 grid, b = 0.2, x0 = (1,1,1),
5,000 transient steps, then 5,002 Benettin blocks of 10 steps of the orbit
and of its twin (offset 1e-8 along x): 105,040 trajectory-steps per grid
point, 1.101e11 per map. One bench step = one full map. The engine arm runs
the float-float kernel (CHAOS_FF32: the orbit in two FP32 words, ~48 bits,
on the FP32 pipe; the twin as an exact FP32 difference; exact log-stretch
sum), whose map agrees with the plain FP64 map as closely as the FP64 map
agrees with itself started 1e-13 away. The line also carries, on the same
1024^2 map, the plain FP64 kernel's rate, the FP32 kernel's rate and
roofline, and every map's error against FP64.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference]
                  [--workload lle|bif1d|bif2d|basins|spectrum|batch|serve]
                  [--precision auto|ff32|fp32|fp64]

--impl reference times the reference's own per-thread code for the path,
compiled for the host (FP64, OpenMP over all host cores), on a bounded sample
of the same workload (the reference has no CPU implementation of its own; its
GPU build is timed separately as reference_gpu).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "steps/s on 1 GB300, batched FP32 vs plain FP64 at stated LLE error; p99 latency"
UNIT = "trajectory-steps/s"
REGULAR = 0.005  # a point is "regular" (periodic orbit or fixed point) when its FP64 LLE is below this

# ---- workloads -----------------------------------------------------------------
LLE = dict(system="rossler", sysid=1, flops=63, tMax=500.0, NT=0.1, nPts=1024, h=0.01, eps=1e-8,
           initialConditions=[1.0, 1.0, 1.0], ranges=[0.1, 0.4, 2.0, 10.0], indicesOfMutVars=[0, 2],
           transientTime=50.0, values=[0.2, 0.2, 5.7])
BIF1D = dict(system="lorenz", sysid=0, flops=71, tMax=100.0, nPts=1000, h=0.01, initialConditions=[0.1, 0.1, 0.1],
             ranges=[20.0, 200.0], indicesOfMutVars=[1], writableVar=0, maxValue=1e4, transientTime=100.0,
             values=[10.0, 28.0, 8.0 / 3.0])
# the reference's own 2-D bifurcation timing sweep (src/main.cu:447-505): Chameleon,
# CT 400 (40,000 recorded steps), TT 2000 (200,000 transient steps), eps 0.001, at 300^2
BIF2D = dict(system="chameleon", sysid=3, flops=None, tMax=400.0, nPts=300, h=0.01,
             initialConditions=[3.0, 3.0, 0.0], ranges=[0.0, 5.0, 0.0, 20.0], indicesOfMutVars=[3, 5], writableVar=0,
             maxValue=1e4, transientTime=2000.0, values=[0.5, 3, 0, 2, 1, 18, 1], eps=0.001)
BASINS = dict(system="lorenz", sysid=0, flops=71, tMax=50.0, nPts=2048, h=0.01, initialConditions=[0.0, 0.0, 27.0],
              ranges=[-30.0, 30.0, -30.0, 30.0], indicesOfMutVars=[0, 1], writableVar=0, maxValue=1e8,
              transientTime=200.0, values=[10.0, 24.0, 8.0 / 3.0], eps=0.05, minPts=8)

# Lyapunov spectrum (the legacy LS2D analysis): Lorenz, (rho, sigma) in [20,200] x [5,15],
# 1024^2, tMax 100 (1,002 blocks of NT 0.1), 2,000 transient steps; the orbit and one
# twin per state dimension
SPECTRUM = dict(system="lorenz", sysid=0, flops=71, tMax=100.0, NT=0.1, nPts=1024, h=0.01, eps=1e-8,
                initialConditions=[1.0, 1.0, 1.0], ranges=[20.0, 200.0, 5.0, 15.0], indicesOfMutVars=[1, 0],
                transientTime=20.0, values=[10.0, 28.0, 8.0 / 3.0])


SYS_FLOPS = {"lorenz": 71, "rossler": 63, "chen": 79}
SYS_ID = {"lorenz": 0, "rossler": 1, "chen": 2}


def pinned(shape, dtype):
    """A page-locked host buffer as a numpy array: the end-to-end legs write
    each step's results into buffers a caller would reuse, so the timed copies
    are the library's, not first-touch page faults of fresh arrays."""
    import torch

    return torch.empty(shape, dtype=dtype, pin_memory=True).numpy()


def batch_jobs(seed: int = 2024, n_jobs: int = 256):
    """The heterogeneous batch: n_jobs jobs, point counts log-uniform in
    [1e3, 1e6], system uniform over Lorenz / Rossler / Chen (a=35, b=3, c swept
    20..30), transients uniform in [2000, 20000] steps, alternately a 1-D
    bifurcation (tMax 100: 10,000 recorded steps, 64 peaks kept per point) and
    a 2-D LLE map (sqrt(N) x sqrt(N) points, tMax 100, NT 0.1, eps 1e-8)."""
    rng = np.random.default_rng(seed)
    jobs = []
    for k in range(n_jobs):
        n = int(round(10 ** rng.uniform(3, 6)))
        system = ["lorenz", "rossler", "chen"][int(rng.integers(0, 3))]
        trans = int(rng.integers(2000, 20001)) * 0.01
        if system == "lorenz":
            vals, ic, bif_mut, bif_rng, lle_mut, lle_rng = [10.0, 28.0, 8 / 3], [0.1, 0.1, 0.1], [1], [20.0, 200.0], \
                [1, 0], [20.0, 200.0, 5.0, 15.0]
        elif system == "rossler":
            vals, ic, bif_mut, bif_rng, lle_mut, lle_rng = [0.2, 0.2, 5.7], [1.0, 1.0, 1.0], [2], [2.0, 10.0], \
                [0, 2], [0.1, 0.4, 2.0, 10.0]
        else:
            vals, ic, bif_mut, bif_rng, lle_mut, lle_rng = [35.0, 3.0, 28.0], [-10.0, 0.0, 37.0], [2], [20.0, 30.0], \
                [2, 0], [20.0, 30.0, 30.0, 40.0]
        if k % 2 == 0:
            jobs.append(("bif", system, dict(tMax=100.0, nPts=n, h=0.01, initialConditions=ic, ranges=bif_rng,
                                             indicesOfMutVars=bif_mut, writableVar=0, maxValue=1e4,
                                             transientTime=trans, values=vals)))
        else:
            m = max(int(round(n ** 0.5)), 2)
            jobs.append(("lle", system, dict(tMax=100.0, NT=0.1, nPts=m, h=0.01, eps=1e-8, initialConditions=ic,
                                             ranges=lle_rng, indicesOfMutVars=lle_mut, transientTime=trans,
                                             values=vals)))
    return jobs


def serve_requests(seed: int = 7, n: int = 10000):
    """The served stream: n requests, 40 % 1-D bifurcation, 40 % LLE maps,
    20 % basins maps (features + the reference clustering), systems uniform
    over Lorenz / Rossler / Chen, grid sizes log-uniform in [1e3, 4e6] points,
    with the horizons of the single-workload configurations: bifurcation
    10,000 transient + 10,000 recorded steps, LLE 5,000 transient + 5,002
    blocks of 10 steps of orbit and twin, basins 20,000 transient + 5,000
    recorded steps (h = 0.01)."""
    rng = np.random.default_rng(seed)
    reqs = []
    for _ in range(n):
        u = rng.random()
        kind = "bif" if u < 0.4 else ("lle" if u < 0.8 else "basins")
        system = ["lorenz", "rossler", "chen"][int(rng.integers(0, 3))]
        N = int(round(10 ** rng.uniform(3, np.log10(4e6))))
        m = max(int(round(N ** 0.5)), 2)
        vals = {"lorenz": [10.0, 28.0, 8 / 3], "rossler": [0.2, 0.2, 5.7], "chen": [35.0, 3.0, 28.0]}[system]
        ic = {"lorenz": [0.1, 0.1, 0.1], "rossler": [1.0, 1.0, 1.0], "chen": [-10.0, 0.0, 37.0]}[system]
        if kind == "bif":
            mut, rg = {"lorenz": ([1], [20.0, 200.0]), "rossler": ([2], [2.0, 10.0]), "chen": ([2], [20.0, 30.0])}[system]
            reqs.append((kind, system, dict(tMax=100.0, nPts=N, h=0.01, initialConditions=ic, ranges=rg,
                                            indicesOfMutVars=mut, writableVar=0, maxValue=1e4, transientTime=100.0,
                                            values=vals)))
        elif kind == "lle":
            mut, rg = {"lorenz": ([1, 0], [20.0, 200.0, 5.0, 15.0]), "rossler": ([0, 2], [0.1, 0.4, 2.0, 10.0]),
                       "chen": ([2, 0], [20.0, 30.0, 30.0, 40.0])}[system]
            reqs.append((kind, system, dict(tMax=500.0, NT=0.1, nPts=m, h=0.01, eps=1e-8, initialConditions=ic,
                                            ranges=rg, indicesOfMutVars=mut, transientTime=50.0, values=vals)))
        else:
            icb = {"lorenz": [0.0, 0.0, 27.0], "rossler": [0.0, 0.0, 0.5], "chen": [0.0, 0.0, 20.0]}[system]
            vb = {"lorenz": [10.0, 24.0, 8 / 3], "rossler": [0.2, 0.2, 5.7], "chen": [35.0, 3.0, 28.0]}[system]
            reqs.append((kind, system, dict(tMax=50.0, nPts=m, h=0.01, initialConditions=icb,
                                            ranges=[-30.0, 30.0, -30.0, 30.0], indicesOfMutVars=[0, 1],
                                            writableVar=0, maxValue=1e8, transientTime=200.0, values=vb)))
    return reqs


def job_points_steps(kind, kw):
    if kind == "basins":
        return kw["nPts"] ** 2, int(kw["transientTime"] / kw["h"]) + int(kw["tMax"] / kw["h"])
    if kind == "bif":
        return kw["nPts"], int(kw["transientTime"] / kw["h"]) + int(kw["tMax"] / kw["h"])
    ntp = int(kw["NT"] / kw["h"])
    calc = int(kw["tMax"] / kw["h"]) // ntp + 1
    return kw["nPts"] ** 2, int(kw["transientTime"] / kw["h"]) + 2 * ntp * (calc + 1)


def lle_steps_per_point(w) -> int:
    ntp = int(w["NT"] / w["h"])
    calc = int(w["tMax"] / w["h"]) // ntp + 1
    return int(w["transientTime"] / w["h"]) + 2 * ntp * (calc + 1)


def spectrum_steps_per_point(w, nx=3) -> int:
    ntp = int(w["NT"] / w["h"])
    calc = int(w["tMax"] / w["h"]) // ntp + 1
    return int(w["transientTime"] / w["h"]) + (1 + nx) * ntp * (calc + 1)


def sweep_steps_per_point(w) -> int:
    return int(w["transientTime"] / w["h"]) + int(w["tMax"] / w["h"])


def kw_of(w, drop=("system", "sysid", "flops")):
    return {k: v for k, v in w.items() if k not in drop}


# ---- distributed / clocks -----------------------------------------------------------
def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(ws, x: float) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpus):
        self.gpus = gpus
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "100"], stdout=self.f, stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.p = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.p:
            time.sleep(0.2)
            self.p.terminate()
            self.p.wait()

    def summary(self):
        self.f.flush()
        rows = [r.split(", ") for r in Path(self.f.name).read_text().splitlines() if r.strip()]
        rows = [r for r in rows if len(r) >= 9 and r[0].strip().isdigit() and int(r[0]) in self.gpus]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no nvidia-smi samples"]}
        sm = [float(r[1]) for r in rows]
        smax = max(float(r[2]) for r in rows)
        load = [s for s, r in zip(sm, rows) if float(r[3]) > 200.0] or sm
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[j] for r in rows for j in range(4) if r[5 + j].strip().lower() == "active"})
        return {"sm_mhz": statistics.median(load), "sm_max_mhz": smax, "reasons": reasons,
                "samples": len(rows), "power_w_max": max(float(r[3]) for r in rows)}


# ---- CPU leg (the oracle restatement of the reference algorithm) --------------------------
def cpu_sample_lle(w, target_s=10.0):
    """The LLE map on the host cores over a bounded sample of its points: the
    reference's own per-thread code (its calculateSystem and step loop,
    compiled for the host by oracle/build_ref.py, OpenMP over points) where
    that build exists, else the oracle's C++ restatement."""
    from oracle import oracle as O

    nthreads = os.cpu_count() or 1
    n_all = w["nPts"] * w["nPts"]
    kind = "port"
    try:
        ref = O.RefLib(w["system"])
        args = (w["tMax"], w["NT"], w["nPts"], w["h"], w["eps"], w["initialConditions"], w["ranges"],
                w["indicesOfMutVars"], w["transientTime"], w["values"])

        def run(b, e):
            ref.lle_range(*args, b, e, nthreads=nthreads)
        kind = "reference"
    except (OSError, AttributeError):
        args = (w["sysid"], w["tMax"], w["NT"], w["nPts"], w["h"], w["eps"], w["initialConditions"], w["ranges"],
                w["indicesOfMutVars"], w["transientTime"], w["values"])

        def run(b, e):
            O.lle2d(*args, p_begin=b, p_end=e, nthreads=nthreads)
    probe = 2 * nthreads
    t = time.perf_counter()
    run(n_all // 2, n_all // 2 + probe)
    dt = time.perf_counter() - t
    n = int(min(n_all, max(probe, probe * target_s / max(dt, 1e-3))))
    begin = n_all // 2 - n // 2
    t = time.perf_counter()
    run(begin, begin + n)
    dt = time.perf_counter() - t
    steps = n * lle_steps_per_point(w)
    what = ("the reference's own calculateSystem and step loop (LLE/src/LLECUDA.cu) compiled for the host, "
            "its transient by its loopCalculateDiscreteModel, twin at x + eps*e_x" if kind == "reference"
            else "the oracle's C++ restatement")
    return {"value": steps / dt, "unit": UNIT, "cores": nthreads, "kind": kind,
            "sample": f"{n} contiguous grid points from the middle of the 1024x1024 map, full 105,040 steps each, "
                      f"FP64, {dt:.1f} s; {what}"}


def cpu_sample_spectrum(w, target_s=10.0):
    from oracle import oracle as O

    nthreads = os.cpu_count() or 1
    n_all = w["nPts"] * w["nPts"]
    args = (w["sysid"], 2, 0, w["tMax"], w["NT"], w["nPts"], w["h"], w["eps"], w["initialConditions"], w["ranges"],
            w["indicesOfMutVars"], w["transientTime"], w["values"])
    probe = 2 * nthreads
    t = time.perf_counter()
    O.lyapunov_spectrum(*args, p_begin=n_all // 2, p_end=n_all // 2 + probe, nthreads=nthreads)
    dt = time.perf_counter() - t
    n = int(min(n_all, max(probe, probe * target_s / max(dt, 1e-3))))
    begin = n_all // 2 - n // 2
    t = time.perf_counter()
    O.lyapunov_spectrum(*args, p_begin=begin, p_end=begin + n, nthreads=nthreads)
    dt = time.perf_counter() - t
    return {"value": n * spectrum_steps_per_point(w) / dt, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": f"{n} contiguous grid points from the middle of the map, full horizon, FP64, {dt:.1f} s"}


def cpu_sample_sweep(w, kind, target_s=10.0):
    """A sweep on the host cores over a bounded sample of its points: the
    reference's own per-thread kernels (transient, recorded loop, peak finder
    or peak averages; compiled for the host by oracle/build_ref.py, replayed
    through its own chunking, OpenMP over points) where that build exists,
    else the oracle's C++ restatement."""
    from oracle import oracle as O

    nthreads = os.cpu_count() or 1
    dim = 1 if kind == "bif1d" else 2
    n_all = w["nPts"] ** dim
    probe = 2 * nthreads
    args = (w["tMax"], w["nPts"], w["h"], w["initialConditions"], w["ranges"], w["indicesOfMutVars"],
            w["writableVar"], w["maxValue"], w["transientTime"], w["values"])
    impl = "port"
    try:
        ref = O.RefLib(w["system"])
        impl = "reference"
    except (OSError, AttributeError):
        ref = None

    def run(b, e):
        if ref is not None and kind in ("bif1d", "bif2d"):
            ref.bifurcation_range(dim, *args, b, e, nthreads=nthreads)
        elif ref is not None:
            ref.basins_range(*args, b, e, nthreads=nthreads)
        elif kind in ("bif1d", "bif2d"):
            O.bifurcation(w["sysid"], dim, *args, cap=64, p_begin=b, p_end=e, nthreads=nthreads)
        else:
            O.basins_features(w["sysid"], *args, p_begin=b, p_end=e, nthreads=nthreads)
    t = time.perf_counter()
    run(0, probe)
    dt = time.perf_counter() - t
    n = int(min(n_all, max(probe, probe * target_s / max(dt, 1e-3))))
    b = n_all // 2 - n // 2 if n < n_all else 0
    t = time.perf_counter()
    run(b, b + n)
    dt = time.perf_counter() - t
    what = ("the reference's own per-thread kernels compiled for the host" if impl == "reference"
            else "the oracle's C++ restatement")
    return {"value": n * sweep_steps_per_point(w) / dt, "unit": UNIT, "cores": nthreads, "kind": impl,
            "sample": f"{n} of {n_all} grid points, full horizon, FP64, {dt:.1f} s; {what}"
                      + ("; per-point integration and features (the clustering needs the whole map and is not "
                         "in the sample)" if kind == "basins" else "")
                      + ("; per-point integration and peaks (the per-point clustering is not in the sample)"
                         if kind == "bif2d" else "")}


def reference_arm(args, ws, rank):
    if rank != 0:
        return
    w = {"lle": LLE, "bif1d": BIF1D, "basins": BASINS, "batch": LLE, "serve": LLE, "bif2d": BIF2D,
         "spectrum": SPECTRUM}[args.workload]
    if args.workload in ("lle", "batch", "serve"):
        fn = lambda: cpu_sample_lle(w, args.cpu_seconds)  # noqa: E731
    elif args.workload == "spectrum":
        fn = lambda: cpu_sample_spectrum(w, args.cpu_seconds)  # noqa: E731
    else:
        fn = lambda: cpu_sample_sweep(w, args.workload, args.cpu_seconds)  # noqa: E731
    vals, last = [], None
    for _ in range(args.steps):
        last = fn()
        vals.append(last["value"])
    v = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {**config_of(args), "precision": "fp64"}, "cpu_baseline": {**last, "value": v},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def config_of(args):
    if args.npts or args.tmax:
        return {"workload": f"{args.workload} profiling case (nPts={args.npts}, tMax={args.tmax})"}
    if args.workload == "lle":
        return {"workload": "LLE map, Rossler RK4 h=0.01, a in [0.1,0.4] x c in [2,10], 1024x1024, b=0.2, "
                            "x0=(1,1,1), 5000 transient + 5002 blocks x 10 steps x 2 trajectories",
                "grid_points": 1048576, "steps_per_point": lle_steps_per_point(LLE), "eps": 1e-8,
                "precision": args.precision,
                "arithmetic": {"ff32": "float-float orbit (two FP32 words, ~48 bits, FP32 pipe), twin as an "
                                       "exact FP32 difference, exact power-of-two renormalisation, FP64 log",
                               "fp32": "FP32 orbit, twin as an exact FP32 difference, exact power-of-two "
                                       "renormalisation, FP64 log",
                               "fp64": "FP64 orbit and twin, the reference's per-block FP64 norm and log"
                               }.get(args.precision),
                "l2": "256 MB buffer written between timed steps; the map's state "
                      "lives in registers (inputs: 88 B of parameters)"}
    if args.workload == "spectrum":
        return {"workload": "Lyapunov spectrum (Gram-Schmidt per block), Lorenz RK4 h=0.01, rho in [20,200] x "
                            "sigma in [5,15], 1024x1024, beta=8/3, x0=(1,1,1), 2000 transient steps + 1002 blocks "
                            "x 10 steps x (orbit + 3 twins)", "grid_points": 1048576,
                "steps_per_point": spectrum_steps_per_point(SPECTRUM), "eps": 1e-8, "precision": args.precision,
                "l2": "256 MB buffer written between timed steps; state in registers, 24 B written per point"}
    if args.workload == "bif2d":
        return {"workload": "2-D bifurcation (the reference's own timing sweep), Chameleon, 300x300 over "
                            "(values[3], values[5]) in [0,5] x [0,20], 200000 transient + 40000 recorded steps, "
                            "per-point interval clustering eps=0.001", "grid_points": 90000,
                "steps_per_point": sweep_steps_per_point(BIF2D), "precision": args.precision,
                "l2": "256 MB buffer written between timed steps"}
    if args.workload == "bif1d":
        return {"workload": "1-D bifurcation, Lorenz RK4 h=0.01, rho in [20,200] x 1000, 10000 transient + "
                            "10000 recorded steps, peaks of x", "grid_points": 1000,
                "steps_per_point": sweep_steps_per_point(BIF1D), "precision": args.precision,
                "l2": "256 MB buffer written between timed steps"}
    return {"workload": "basins, Lorenz rho=24 RK4 h=0.01, 2048x2048 ICs x,y in [-30,30], z=27, 20000 transient + "
                        "5000 recorded steps, features (mean peak of x, peak count, mean interval) min-max "
                        "normalised, DBSCAN eps=0.05 minPts=8",
            "grid_points": 2048 * 2048, "steps_per_point": sweep_steps_per_point(BASINS),
            "precision": args.precision, "l2": "256 MB buffer written between timed steps"}


def traffic_from_profiles(kernel_tag: str):
    """dram bytes per launch recorded in profiles/<kernel_tag>.md (a line
    'dram_bytes_per_launch: N'), or None."""
    p = ROOT / "profiles" / f"{kernel_tag}.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.strip().startswith("dram_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def pipe_busy_from_profiles(kernel_tag: str):
    """FMA-pipe busy fraction recorded in profiles/<kernel_tag>.md (a line
    'fp32_pipe_busy: F'), or None."""
    p = ROOT / "profiles" / f"{kernel_tag}.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.strip().startswith("fp32_pipe_busy:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


# ---- engine arm ----------------------------------------------------------------------------
def batch_arm(args, ws, rank, local):
    """The heterogeneous batch as one prepared submission (CUDA graph of the
    grouped persistent kernels), against the same jobs run one by one. The
    LLE jobs run float-float (--precision ff32, the default: the arithmetic
    whose maps match FP64 to the FP64 map's own spread) or FP32; the line
    carries the other batch's rate too, and the sampled jobs' FP64 rate and
    LLE error."""
    import torch

    import chaoslibrary_gb300 as C

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    lle_prec = C.FP32 if args.precision == "fp32" else C.FF32
    jobs = batch_jobs()
    total_steps = sum(np.prod(job_points_steps(k, kw)) for k, _, kw in jobs)
    flops = sum(SYS_FLOPS[s_] * float(np.prod(job_points_steps(k, kw))) for k, s_, kw in jobs)

    def make(prec, device=True):
        b = C.Batch(device=device)
        outs = []
        for kind, system, kw in jobs:
            if kind == "bif":
                outs.append(b.add_bifurcation1d(system, peakCapacity=64, **kw))
            else:
                outs.append(b.add_lle2d(system, precision=prec, **kw))
        return b, outs

    def timed(b, steps, flush, stream):
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for k in range(steps):
            flush.fill_(k & 0xff)
            ev[k][0].record(stream)
            b.replay()
            ev[k][1].record(stream)
        torch.cuda.synchronize()
        return [a.elapsed_time(c) for a, c in ev]

    b, outs = make(lle_prec)
    b.prepare()
    for _ in range(args.warmup):
        b.replay()
    torch.cuda.synchronize()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    with Clocks([local] if ws == 1 else list(range(ws))) as clk:
        barrier(ws)
        torch.cuda.synchronize()
        l0 = C.launch_count()
        ms = timed(b, args.steps, flush, stream)
        launches = C.launch_count() - l0
        barrier(ws)
    t_total = max_over_ranks(ws, sum(ms) / 1e3)
    value = ws * total_steps * args.steps / t_total
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (bifurcation) / ff32 (LLE)" if lle_prec == C.FF32 else "f32",
            "data": "synthetic (seeded job list)",
            "config": {"workload": "256 heterogeneous jobs (seed 2024): N log-uniform 1e3..1e6, systems "
                                   "Lorenz/Rossler/Chen, transients 2000..20000 steps, half 1-D bifurcation "
                                   "(10000 recorded steps), half LLE maps (tMax 100, NT 0.1)",
                       "lle_precision": "ff32" if lle_prec == C.FF32 else "fp32",
                       "total_steps": float(total_steps), "jobs": len(jobs),
                       "l2": "256 MB buffer written between timed steps"},
            "clocks": clk.summary(), "gpu_launches": launches}
    if rank == 0:
        mean_s = statistics.mean(ms) / 1e3
        peak = C.fma_probe() / 1e12
        line["roofline"] = {"bound": "fp32_fma", "achieved": flops / mean_s / 1e12, "peak": peak,
                            "unit": "TFLOP/s", "frac": flops / mean_s / 1e12 / peak, "traffic": None,
                            "algorithmic": "71/63/79 flops per Lorenz/Rossler/Chen RK4 step",
                            "peak_source": "measured in this run: chaos_fma_probe"}
        if lle_prec == C.FF32:
            line["roofline"]["note"] = (
                "the LLE half runs float-float (~7 FP32 operations per algorithmic flop), so the algorithmic "
                "fraction is low by construction; other_lle_precision.roofline is the same batch with FP32 LLE jobs")
    # e2e: one-shot host-memory submission (descriptor upload, launch, results copied back)
    bh, _ = make(lle_prec, device=False)
    bh.run()
    t0 = time.perf_counter()
    bh.run()
    e2e_s = max_over_ranks(ws, time.perf_counter() - t0)
    d2h = sum(sum(v.nbytes for v in o.values()) for o in bh.outputs)
    bh.close()
    line["e2e"] = {"value": ws * total_steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": d2h}
    if rank == 0 and not args.no_extras:
        # the other LLE arithmetic, same jobs, same timing
        other = C.FP32 if lle_prec == C.FF32 else C.FF32
        b2, _ = make(other)
        b2.prepare()
        b2.replay()
        torch.cuda.synchronize()
        ms2 = timed(b2, max(2, min(args.steps, 5)), flush, stream)
        b2.close()
        s2 = statistics.mean(ms2) / 1e3
        line["other_lle_precision"] = {"lle_precision": "fp32" if other == C.FP32 else "ff32",
                                       "value": total_steps / s2, "unit": UNIT, "ms_per_step": s2 * 1e3,
                                       "roofline": {"bound": "fp32_fma", "achieved": flops / s2 / 1e12,
                                                    "peak": peak, "unit": "TFLOP/s",
                                                    "frac": flops / s2 / 1e12 / peak}}
        # the same jobs one at a time through the single-sweep entry points (device outputs)
        single = []
        for kind, system, kw in jobs:
            n, _ = job_points_steps(kind, kw)
            if kind == "bif":
                single.append(dict(counts=torch.empty(n, dtype=torch.int32, device=dev),
                                   flags=torch.empty(n, dtype=torch.int32, device=dev),
                                   first=torch.empty(n, dtype=torch.float64, device=dev),
                                   peaks=torch.empty(n * 64, dtype=torch.float64, device=dev),
                                   intervals=torch.empty(n * 64, dtype=torch.float64, device=dev)))
            else:
                single.append(torch.empty(n, dtype=torch.float64, device=dev))
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for (kind, system, kw), o in zip(jobs, single):
            if kind == "bif":
                C.bifurcation1d(system, precision=C.FP32, peakCapacity=64, out=o, **kw)
            else:
                C.lle2d(system, precision=lle_prec, out=o, **kw)
        e1.record()
        torch.cuda.synchronize()
        t_seq = e0.elapsed_time(e1) / 1e3
        # plain FP64 single-sweep kernel on every 15th job (both kinds), and the
        # batch's LLE maps of those jobs against their FP64 maps
        sample = list(range(0, len(jobs), 15))
        s_steps = sum(np.prod(job_points_steps(*jobs[k][::2])) for k in sample)
        errs = []
        t64 = 0.0
        for k in sample:
            kind, system, kw = jobs[k]
            e0.record()
            if kind == "bif":
                C.bifurcation1d(system, precision=C.FP64, peakCapacity=64, **kw)
            else:
                a = C.lle2d(system, precision=C.FP64, **kw)
            e1.record()
            torch.cuda.synchronize()
            t64 += e0.elapsed_time(e1) / 1e3
            if kind != "bif":
                v = outs[k]["lle"].cpu().numpy()
                ic = list(kw["initialConditions"])
                a13 = C.lle2d(system, precision=C.FP64, **dict(kw, initialConditions=[ic[0] + 1e-13] + ic[1:]))
                fin = np.isfinite(a) & np.isfinite(v) & np.isfinite(a13)
                errs.append((np.abs(v - a)[fin], np.abs(a13 - a)[fin], (a < REGULAR)[fin]))
        d = np.concatenate([e for e, _, _ in errs]) if errs else np.zeros(1)
        d13 = np.concatenate([e for _, e, _ in errs]) if errs else np.zeros(1)
        reg = np.concatenate([r for _, _, r in errs]) if errs else np.zeros(1, bool)
        line["one_by_one"] = {"value": total_steps / t_seq, "unit": UNIT,
                              "batched_speedup": t_seq / (statistics.mean(ms) / 1e3)}
        line["fp64_plain"] = {"value": s_steps / t64, "unit": UNIT, "sample": "every 15th job, one by one",
                              "batched_speedup": value / (s_steps / t64)}
        def st(x):
            return {"p50": float(np.median(x)), "p90": float(np.percentile(x, 90)), "max": float(x.max()),
                    "frac_le_1e-3": float(np.mean(x <= 1e-3)),
                    "regular_frac_le_1e-3": float(np.mean(x[reg] <= 1e-3)) if reg.any() else None}
        line["lle_error_vs_fp64"] = {"jobs": len(errs), "points": int(d.size), "regular_points": int(reg.sum()),
                                     "batched": st(d), "fp64_started_1e-13_away": st(d13)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    b.close()


def serve_stream(C, args, seed, lle_prec, local):
    """One served stream: Poisson arrivals of serve_requests(seed) into the
    request loop. Returns its line fields and the outputs of the small LLE
    requests kept for the precision check."""
    import threading

    reqs = serve_requests(seed=seed, n=args.requests)
    rng = np.random.default_rng(seed + 1000)
    gaps = rng.exponential(1.0 / args.rate, size=len(reqs))
    keep = {k for k, (kind, _, kw) in enumerate(reqs) if kind == "lle" and kw["nPts"] ** 2 <= 16384}
    keep = set(sorted(keep)[:12])
    srv = C.Server(hbm_budget_bytes=args.hbm_budget_gb << 30, max_active=256, iteration_steps=args.iteration_steps)
    ids, kept, done_lat = [], {}, []
    lock = threading.Lock()

    def waiter():
        k = 0
        while True:
            with lock:
                if k >= len(ids):
                    if len(ids) == len(reqs):
                        return
                    rid = None
                else:
                    rid = ids[k][0]
            if rid is None:
                time.sleep(0.001)
                continue
            srv.wait(rid, timeout=3600)
            done_lat.append(srv.latency(rid))
            with lock:
                if k in keep:
                    kept[k] = ids[k][1]["lle"].copy()
                ids[k] = (rid, None)  # drop the output arrays
            k += 1

    th = threading.Thread(target=waiter)
    th.start()
    with Clocks([local]) as clk:
        l0 = C.launch_count()
        t0 = time.perf_counter()
        t_next = t0
        for (kind, system, kw), gap in zip(reqs, gaps):
            t_next += gap
            d = t_next - time.perf_counter()
            if d > 0:
                time.sleep(d)
            if kind == "bif":
                rid, out = srv.submit_bifurcation1d(system, peakCapacity=4, **kw)
            elif kind == "lle":
                rid, out = srv.submit_lle2d(system, precision=lle_prec, **kw)
            else:
                rid, out = srv.submit_basins(system, eps=0.05, **kw)
            with lock:
                ids.append((rid, out))
        th.join()
        wall = time.perf_counter() - t0
        launches = C.launch_count() - l0
    st = srv.stats()
    srv.close()
    total_steps = sum(np.prod(job_points_steps(k, kw)) for k, _, kw in reqs)
    lat = np.array(done_lat)
    return {"seed": seed, "value": total_steps / wall, "wall_s": wall, "total_steps": float(total_steps),
            "latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                          "mean": float(lat.mean()), "max": float(lat.max())},
            "server": st, "clocks": clk.summary(), "gpu_launches": launches}, reqs, kept


def serve_arm(args, ws, rank, local):
    """Poisson arrivals of the served stream into the request loop, repeated
    over --repeats seeds; reports p50/p99 latency per stream and their
    spread, aggregate throughput, and the served LLE maps' error against the
    plain FP64 maps of the same requests (the small ones, <= 128^2 points)."""
    import chaoslibrary_gb300 as C

    lle_prec = C.FF32 if args.precision == "ff32" else C.FP32
    srv = C.Server(hbm_budget_bytes=args.hbm_budget_gb << 30, max_active=256, iteration_steps=args.iteration_steps)
    # warm-up: a small request of each kind and system (kernel loading), not counted
    w = []
    for kind, system, kw in serve_requests(n=60):
        kw = dict(kw, nPts=min(kw["nPts"], 1000 if kind == "bif" else 32), tMax=min(kw["tMax"], 5.0))
        if kind == "bif":
            w.append(srv.submit_bifurcation1d(system, peakCapacity=4, **kw))
        elif kind == "lle":
            w.append(srv.submit_lle2d(system, precision=lle_prec, **kw))
        else:
            w.append(srv.submit_basins(system, eps=0.05, **kw))
    for rid, _ in w:
        srv.wait(rid)
    srv.close()
    runs, errs = [], []
    for r in range(args.repeats):
        run, reqs, kept = serve_stream(C, args, 7 + r, lle_prec, local)
        runs.append(run)
        for k, v in kept.items():
            _, system, kw = reqs[k]
            a = C.lle2d(system, precision=C.FP64, **kw)
            ic = list(kw["initialConditions"])
            a13 = C.lle2d(system, precision=C.FP64, **dict(kw, initialConditions=[ic[0] + 1e-13] + ic[1:]))
            fin = np.isfinite(a) & np.isfinite(v) & np.isfinite(a13)
            errs.append((np.abs(v - a)[fin], np.abs(a13 - a)[fin], (a < REGULAR)[fin]))
    first = runs[0]
    d = np.concatenate([e for e, _, _ in errs]) if errs else np.zeros(0)
    d13 = np.concatenate([e for _, e, _ in errs]) if errs else np.zeros(0)
    reg = np.concatenate([g for _, _, g in errs]) if errs else np.zeros(0, bool)

    def st(x):
        return {"p50": float(np.median(x)), "p90": float(np.percentile(x, 90)), "max": float(x.max()),
                "frac_le_1e-3": float(np.mean(x <= 1e-3)),
                "regular_frac_le_1e-3": float(np.mean(x[reg] <= 1e-3)) if reg.any() else None}
    p50s, p99s = [x["latency_s"]["p50"] for x in runs], [x["latency_s"]["p99"] for x in runs]
    line = {"metric": METRIC, "value": first["value"], "unit": UNIT, "n_gpus": 1, "steps": args.requests,
            "warmup": 1, "ms_per_step": 1e3 * first["wall_s"] / args.requests, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "ff32 (LLE requests) / f32" if lle_prec == C.FF32
            else "f32", "data": "synthetic (seeded request streams)",
            "config": {"workload": f"served stream: {args.requests} Poisson requests at {args.rate}/s, 40% 1-D "
                                   "bifurcation (10,000 + 10,000 steps), 40% LLE maps (5,000 + 5,002 x 10 x 2 "
                                   "steps), 20% basins (20,000 + 5,000 steps, + the reference clustering), "
                                   "Lorenz/Rossler/Chen, 1e3..4e6 points",
                       "lle_precision": "ff32" if lle_prec == C.FF32 else "fp32", "rate_per_s": args.rate,
                       "requests": args.requests, "repeats": args.repeats, "hbm_budget_gb": args.hbm_budget_gb,
                       "iteration_steps": args.iteration_steps},
            "latency_s": first["latency_s"], "server": first["server"], "clocks": first["clocks"],
            "total_steps": first["total_steps"], "wall_s": first["wall_s"], "gpu_launches": first["gpu_launches"],
            "repeats": [{k: x[k] for k in ("seed", "value", "wall_s", "latency_s")} for x in runs],
            "latency_spread_s": {"p50_min": min(p50s), "p50_max": max(p50s), "p99_min": min(p99s),
                                 "p99_max": max(p99s)},
            "lle_error_vs_fp64": None if d.size == 0 else {
                "requests": len(errs), "points": int(d.size), "regular_points": int(reg.sum()),
                "served": st(d), "fp64_started_1e-13_away": st(d13)},
            "e2e": {"value": first["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": None}}
    print(json.dumps(line), flush=True)


def engine_arm(args, ws, rank, local):
    import torch

    import chaoslibrary_gb300 as C

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    if args.lle_variant:
        C.set_tuning(C.TUNE_LLE_F32_VARIANT, args.lle_variant)
    prec = {"fp32": C.FP32, "fp64": C.FP64, "ff32": C.FF32}[args.precision]
    w = {"lle": LLE, "bif1d": BIF1D, "bif2d": BIF2D, "basins": BASINS, "spectrum": SPECTRUM}[args.workload]
    n_points = w["nPts"] ** (1 if args.workload == "bif1d" else 2)
    if args.workload == "spectrum":
        steps_pp = spectrum_steps_per_point(w)
        out = torch.empty((n_points, 3), dtype=torch.float64, device=dev)
        kw = kw_of(w)

        def step(o=None):
            return C.lyapunov_spectrum(w["system"], 2, precision=prec, out=out, **kw)

        hout = pinned((n_points, 3), torch.float64)

        def step_host():
            return C.lyapunov_spectrum(w["system"], 2, precision=prec, out=hout, **kw)
        d2h = n_points * 24
        tag = f"spectrum_{args.precision}_lorenz_1024"
    elif args.workload == "lle":
        steps_pp = lle_steps_per_point(w)
        out = torch.empty(n_points, dtype=torch.float64, device=dev)
        kw = kw_of(w)

        def step(o=None):
            return C.lle2d(w["system"], precision=prec, out=out if o is None else o, **kw)

        hout = pinned(n_points, torch.float64)

        def step_host():
            return C.lle2d(w["system"], precision=prec, out=hout, **kw)
        d2h = n_points * 8
        tag = f"lle_{args.precision}_rossler_1024"
        line_extra = {"lle_variant": C.get_tuning(C.TUNE_LLE_F32_VARIANT)} if prec == C.FP32 else {}
    elif args.workload == "bif1d":
        steps_pp = sweep_steps_per_point(w)
        cap = 64
        outs = dict(counts=torch.empty(n_points, dtype=torch.int32, device=dev),
                    flags=torch.empty(n_points, dtype=torch.int32, device=dev),
                    first=torch.empty(n_points, dtype=torch.float64, device=dev),
                    peaks=torch.empty(n_points * cap, dtype=torch.float64, device=dev),
                    intervals=torch.empty(n_points * cap, dtype=torch.float64, device=dev))
        kw = kw_of(w)

        def step(o=None):
            return C.bifurcation1d(w["system"], precision=prec, peakCapacity=cap, out=outs, **kw)

        houts = dict(counts=pinned(n_points, torch.int32), flags=pinned(n_points, torch.int32),
                     first=pinned(n_points, torch.float64), peaks=pinned((n_points, cap), torch.float64),
                     intervals=pinned((n_points, cap), torch.float64))

        def step_host():
            return C.bifurcation1d(w["system"], precision=prec, peakCapacity=cap, out=houts, **kw)
        d2h = n_points * (4 + 4 + 8 + 16 * cap)
        tag = f"bif1d_{args.precision}_lorenz_1000"
    elif args.workload == "bif2d":
        steps_pp = sweep_steps_per_point(w)
        outs = dict(labels=torch.empty(n_points, dtype=torch.int32, device=dev),
                    counts=torch.empty(n_points, dtype=torch.int32, device=dev))
        kw = kw_of(w)

        def step(o=None):
            return C.bifurcation2d(w["system"], precision=prec, out=outs, **kw)

        houts = dict(labels=pinned(n_points, torch.int32), counts=pinned(n_points, torch.int32))

        def step_host():
            return C.bifurcation2d(w["system"], precision=prec, out=houts, **kw)
        d2h = n_points * 8
        tag = None
    else:
        # the basins map as specified: (amplitude, peak count, interval) features
        # min-max normalised, textbook DBSCAN eps=0.05, minPts=8
        steps_pp = sweep_steps_per_point(w)
        outs = dict(labels=torch.empty(n_points, dtype=torch.int32, device=dev),
                    flags=torch.empty(n_points, dtype=torch.int32, device=dev))
        kw = kw_of(w)

        def step(o=None):
            return C.basins_dbscan(w["system"], precision=prec, out=outs, **kw)

        houts = dict(labels=pinned(n_points, torch.int32), flags=pinned(n_points, torch.int32))

        def step_host():
            return C.basins_dbscan(w["system"], precision=prec, out=houts, **kw)
        d2h = n_points * (4 + 4)
        tag = "basins_lorenz_2048" if args.precision == "fp32" else None
    steps_per_call = n_points * steps_pp
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    stream = torch.cuda.current_stream(dev)
    with Clocks([local] if ws == 1 else list(range(ws))) as clk:
        barrier(ws)
        torch.cuda.synchronize()
        wall0 = time.perf_counter()
        l0 = C.launch_count()
        for k in range(args.steps):
            flush.fill_(k & 0xff)
            ev[k][0].record(stream)
            step()
            ev[k][1].record(stream)
        torch.cuda.synchronize()
        launches = C.launch_count() - l0
        barrier(ws)
        wall = time.perf_counter() - wall0
    ms = [a.elapsed_time(b) for a, b in ev]
    t_total = max_over_ranks(ws, sum(ms) / 1e3)
    value = ws * steps_per_call * args.steps / t_total
    clocks = clk.summary()

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": {C.FP32: "f32", C.FP64: "f64", C.FF32: "ff32"}[prec],
            "data": "synthetic (deterministic parameter / initial-condition grids)",
            "config": config_of(args), "clocks": clocks, "wall_s_timed_region": wall, "gpu_launches": launches}
    if args.workload == "lle":
        line["config"].update(line_extra)

    # roofline: FP32 (or FP64) FMA pipe, algorithmic flops of the integration
    if rank == 0 and w["flops"] is None:
        line["roofline"] = {"bound": "latency / SFU (the Chameleon step calls sin, cos and exp)", "achieved": None,
                            "peak": None, "unit": None, "frac": None, "traffic": None}
    elif rank == 0:
        mean_s = statistics.mean(ms) / 1e3
        algo = w["flops"] * steps_per_call
        achieved = algo / mean_s / 1e12
        peak = C.fma_probe() / 1e12 if prec in (C.FP32, C.FF32) else None
        line["roofline"] = {"bound": "fp64_fma" if prec == C.FP64 else "fp32_fma", "achieved": achieved,
                            "peak": peak, "unit": "TFLOP/s", "frac": (achieved / peak) if peak else None,
                            "traffic": traffic_from_profiles(tag) if tag else None,
                            "algorithmic": f"{w['flops']} flops per RK4 step x {steps_per_call:.4g} steps per launch",
                            "peak_source": "measured in this run: FP32 fmaf-chain probe (chaos_fma_probe), "
                                           "2048 threads/SM; MEASURED_PEAKS.json has only HBM and bf16 tensor peaks"}
        if prec == C.FF32:
            line["roofline"]["note"] = (
                "float-float arithmetic issues ~7 FP32 operations per algorithmic flop, so the algorithmic "
                "fraction is low by construction; fp32_pipe_busy is the FMA pipe's busy fraction in the ncu "
                "capture of this kernel")
            line["roofline"]["fp32_pipe_busy"] = pipe_busy_from_profiles(tag)

    # e2e through the public API with host buffers (pinned, reused; the copies inside the timed region)
    t_e2e = []
    for _ in range(max(1, min(args.steps, 5))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        step_host()
        t_e2e.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(ws, statistics.median(t_e2e))
    line["e2e"] = {"value": ws * steps_per_call / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 88,
                   "d2h_bytes_per_step": d2h}

    if rank == 0 and ws == 1 and args.workload in ("lle", "bif1d", "bif2d") and not args.no_extras \
            and not args.npts and not args.tmax:
        ref = reference_gpu_run(args.workload, steps_per_call)
        if ref:
            line["reference_gpu"] = ref
    if rank == 0 and ws == 1 and args.workload == "basins" and not args.no_extras and not args.npts \
            and not args.tmax:
        ref = basins_reference_gpu(C)
        if ref:
            line["reference_gpu"] = ref
    if rank == 0 and ws == 1 and args.workload == "bif2d" and not args.no_extras:
        line.update(bif2d_extras(C, prec, w))
    if rank == 0 and ws == 1 and args.workload == "lle" and not args.no_extras and not args.npts \
            and not args.tmax:
        line.update(lle_precision_report(C, prec, dev, w, out.cpu().numpy(), statistics.mean(ms) / 1e3,
                                         line.get("roofline", {}).get("peak")))
    if rank == 0 and ws == 1 and args.workload == "basins" and not args.no_extras:
        line.update(basins_extras(C, prec, dev, w))
    if rank == 0 and ws == 1 and not args.no_extras:
        try:
            if args.workload == "lle":
                line["cpu_baseline"] = cpu_sample_lle(w, args.cpu_seconds)
            elif args.workload == "spectrum":
                line["cpu_baseline"] = cpu_sample_spectrum(w, args.cpu_seconds)
            else:
                line["cpu_baseline"] = cpu_sample_sweep(w, args.workload, args.cpu_seconds)
        except Exception as e:  # the oracle is optional at run time
            line["cpu_baseline"] = {"value": None, "error": str(e)}
    if rank == 0:
        print(json.dumps(line), flush=True)


def reference_gpu_run(workload, steps):
    """The reference's own GPU path on this GPU (its unchanged sources built by
    oracle/build_ref_gpu.py, when that build is present): wall time of one call
    of its host entry point on the same configuration, including its own host
    work (allocation, per-element zeroing copies, copy back, CSV writing). The
    2-D bifurcation runs at 200^2: at 300^2 the reference's int indexing of its
    trajectory buffer would overflow."""
    exe = ROOT / "oracle" / "_ref" / f"ref_gpu_{ {'lle': 'lle2d', 'bif1d': 'bif1d', 'bif2d': 'bif2d'}[workload]}"
    if not exe.exists():
        return None
    extra = []
    if workload == "bif2d":
        extra = ["200"]
        steps = 200 * 200 * sweep_steps_per_point(BIF2D)
    with tempfile.TemporaryDirectory() as d:
        try:
            p = subprocess.run([str(exe), str(Path(d) / "out.csv")] + extra, capture_output=True, text=True,
                               timeout=300)
        except subprocess.TimeoutExpired:
            return {"value": None, "error": "timed out after 300 s"}
    if p.returncode != 0:
        return {"value": None, "error": f"exit {p.returncode}"}
    s = json.loads(p.stdout.strip().splitlines()[-1])["seconds"]
    return {"value": steps / s, "unit": UNIT, "seconds": s, "steps": float(steps),
            "what": "the reference's unchanged sources (its host entry point, FP64, nvcc defaults) built for "
                    "sm_103a with the same plug-in, timed around one call incl. its host work"}


def _csv_matrix_cells(path, skip=2):
    """Cells of a reference-format matrix file (header lines, then ', '
    separators with a line break after every row)."""
    body = Path(path).read_text().split("\n", skip)[skip]
    return [c for c in body.replace("\n", "").split(", ") if c != ""]


def basins_reference_gpu(C, n=200):
    """The reference's own basins path (its unchanged sources built by
    oracle/build_ref_gpu.py) on the basins workload's ranges at n^2 -- its
    host-driven clustering launches one kernel per reached point, so the
    2048^2 map is out of its reach -- beside the engine's reference-signature
    entry point (same CSV files) in FP64 and FP32, with the basin-label
    agreement of each against the reference (after the best one-to-one
    matching of cluster ids: the reference numbers clusters in a racy order)."""
    exe = ROOT / "oracle" / "_ref" / "ref_gpu_basins"
    if not exe.exists():
        return None
    w = BASINS
    steps = n * n * sweep_steps_per_point(w)
    args = (w["tMax"], n, w["h"], 3, w["initialConditions"], w["ranges"], w["indicesOfMutVars"], w["writableVar"],
            w["maxValue"], w["transientTime"], w["values"], 3, 1, w["eps"])
    with tempfile.TemporaryDirectory() as d:
        try:
            p = subprocess.run([str(exe), str(Path(d) / "ref"), str(n)], capture_output=True, text=True,
                               timeout=600)
        except subprocess.TimeoutExpired:
            return {"value": None, "error": "timed out after 600 s"}
        if p.returncode != 0:
            return {"value": None, "error": f"exit {p.returncode}"}
        s = json.loads(p.stdout.strip().splitlines()[-1])["seconds"]
        ref_labels = np.array([int(float(c)) for c in _csv_matrix_cells(Path(d) / "ref")])
        out = {"value": steps / s, "unit": UNIT, "seconds": s, "steps": float(steps), "grid": f"{n}x{n}",
               "what": "the reference's unchanged basins sources (FP64, nvcc defaults) built for sm_103a with the "
                       "Lorenz RK4 plug-in, timed around one call of Basins::basinsOfAttraction_2 incl. its "
                       "host work and its host-driven clustering"}
        C.set_system("lorenz")
        # engine_fp64_grid_fma: the grid values rounded as the reference's stock build computes them
        # (CHAOS_TUNE_GRID_FMA = 1); the default keeps the source's separate multiply and add
        for prec, name, fma in ((C.FP64, "engine_fp64", 0), (C.FP64, "engine_fp64_grid_fma", 1),
                                (C.FP32, "engine_fp32", 0)):
            C.set_precision(prec)
            C.set_tuning(C.TUNE_GRID_FMA, fma)
            try:
                C.Basins.basinsOfAttraction_2(*args[:1], 16, *args[2:], Path(d) / "warm")
                t0 = time.perf_counter()
                C.Basins.basinsOfAttraction_2(*args, Path(d) / "eng")
                dt = time.perf_counter() - t0
            finally:
                C.set_tuning(C.TUNE_GRID_FMA, 0)
            eng = np.array([int(float(c)) for c in _csv_matrix_cells(Path(d) / "eng")])
            out[name] = {"value": steps / dt, "unit": UNIT, "seconds": dt, "speedup_vs_reference": s / dt,
                         "label_agreement_vs_reference": label_agreement(eng, ref_labels, fixed=(0,))}
        C.set_precision(C.FP64)
    return out


def bif2d_extras(C, prec, w):
    """The same 300^2 map in plain FP64 (time and labels), and how many FP32
    labels equal the FP64 ones."""
    import time as _t

    kw = kw_of(w)
    other = C.FP64 if prec == C.FP32 else C.FP32
    C.bifurcation2d(w["system"], precision=other, **dict(kw, nPts=8))
    t0 = _t.perf_counter()
    r_other = C.bifurcation2d(w["system"], precision=other, **kw)
    dt = _t.perf_counter() - t0
    r_this = C.bifurcation2d(w["system"], precision=prec, **kw)
    steps = w["nPts"] ** 2 * sweep_steps_per_point(w)
    name = "fp64_plain" if other == C.FP64 else "fp32"
    return {name: {"value": steps / dt, "unit": UNIT, "seconds": dt},
            "labels_fp32_equal_fp64": float(np.mean(r_other["labels"] == r_this["labels"])),
            "labels_note": "per-point clustering of peak intervals at eps 0.001 (steps of 0.01): one-step shifts "
                           "of FP32 peak times change the cluster count"}


def label_agreement(a, b, fixed=()):
    """Fraction of points with the same label in a and b after the best
    one-to-one matching of cluster ids; labels listed in `fixed` (noise,
    diverged) match only themselves."""
    from scipy.optimize import linear_sum_assignment

    a = np.asarray(a).ravel()
    b = np.asarray(b).ravel()
    same_fixed = sum(int(np.sum((a == f) & (b == f))) for f in fixed)
    m = ~np.isin(a, fixed) & ~np.isin(b, fixed)
    if not m.any():
        return same_fixed / a.size
    ua, ia = np.unique(a[m], return_inverse=True)
    ub, ib = np.unique(b[m], return_inverse=True)
    M = np.zeros((ua.size, ub.size), np.int64)
    np.add.at(M, (ia, ib), 1)
    r, c = linear_sum_assignment(-M)
    return (same_fixed + int(M[r, c].sum())) / a.size


def basins_extras(C, prec, dev, w):
    """The reference's own clustering (2 raw features, eps-components) on the
    same 2048^2 map, and the label agreement of the FP32 map with the FP64
    map (same engine, same inputs) on a 512^2 grid over the same ranges."""
    import torch

    out = {}
    kw = {k: v for k, v in kw_of(w).items() if k != "minPts"}
    n = w["nPts"] ** 2
    o = dict(labels=torch.empty(n, dtype=torch.int32, device=dev),
             avg_peaks=torch.empty(n, dtype=torch.float64, device=dev),
             avg_intervals=torch.empty(n, dtype=torch.float64, device=dev),
             flags=torch.empty(n, dtype=torch.int32, device=dev))
    C.basins(w["system"], precision=prec, out=o, **kw)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    C.basins(w["system"], precision=prec, out=o, **kw)
    e1.record()
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3
    out["reference_clustering_mode"] = {"value": n * sweep_steps_per_point(w) / t, "unit": UNIT,
                                        "ms_per_map": 1e3 * t,
                                        "clusters": "2 raw features (mean peak, mean interval), eps-connected "
                                                    "components, fixed-point components negative"}
    small = dict(kw_of(w), nPts=512)
    res = {}
    t_small = {}
    for p in (C.FP64, C.FP32):
        C.basins_dbscan(w["system"], precision=p, **dict(small, nPts=16))
        t0 = time.perf_counter()
        r1 = C.basins_dbscan(w["system"], precision=p, **small)
        t_small[p] = time.perf_counter() - t0
        r2 = C.basins(w["system"], precision=p, **{k: v for k, v in small.items() if k != "minPts"})
        res[p] = (r1, r2)
    (b64, c64), (b32, c32) = res[C.FP64], res[C.FP32]
    steps_small = 512 * 512 * sweep_steps_per_point(w)
    out["basins_fp32_vs_fp64"] = {
        "map": "512x512 (same ranges)", "points": 512 * 512,
        "label_agreement": label_agreement(b32["labels"], b64["labels"], fixed=(-1, -2)),
        "reference_clustering_label_agreement": label_agreement(c32["labels"], c64["labels"], fixed=(0,)),
        "flag_agreement": float(np.mean(b32["flags"] == b64["flags"])),
        "clusters_fp64": int(len(set(b64["labels"].tolist()) - {-1, -2})),
        "clusters_fp32": int(len(set(b32["labels"].tolist()) - {-1, -2})),
        "fp64_plain": {"value": steps_small / t_small[C.FP64], "unit": UNIT},
        "fp32": {"value": steps_small / t_small[C.FP32], "unit": UNIT}}
    return out


def lle_error_stats(v, a):
    """|v - a| over the points finite in both maps (a = the plain FP64 map):
    quantiles, the fraction within 1e-3, the same over the regular points,
    agreement of the chaotic class (LLE > 0.01) and the points finite in one
    map and not the other."""
    fin = np.isfinite(a) & np.isfinite(v)
    d = np.abs(v[fin] - a[fin])
    reg = a[fin] < REGULAR
    return {"points": int(fin.sum()), "p50": float(np.median(d)), "p90": float(np.percentile(d, 90)),
            "p99": float(np.percentile(d, 99)), "max": float(d.max()), "frac_le_1e-3": float(np.mean(d <= 1e-3)),
            "regular_points": int(reg.sum()), "regular_frac_le_1e-3": float(np.mean(d[reg] <= 1e-3)),
            "regular_max": float(d[reg].max()) if reg.any() else None,
            "chaotic_class_agreement": float(np.mean((a[fin] > 0.01) == (v[fin] > 0.01))),
            "nonfinite_mismatch": int(np.sum(np.isfinite(a) != np.isfinite(v)))}


def lle_precision_report(C, prec, dev, w, head_map, head_s, fma_peak):
    """Everything on the benchmark's own 1024x1024 map: the plain FP64
    kernel's rate (one timed launch) and map; the FP64 map started 1e-13
    away in x (the finite-time LLE's own sensitivity: the self-spread every
    other arithmetic is measured against); the float-float map of the timed
    region; the FP32 kernel's rate and roofline under its three stretch
    measurements (CHAOS_TUNE_LLE_RENORM 0/1/2: exact power-of-two, per-block
    FP32 log, per-block FP64 norm and log); each map's error against FP64;
    and the FP32 map with the FP64 sign re-check."""
    import torch

    kw = kw_of(w)
    n = w["nPts"] ** 2
    steps = n * lle_steps_per_point(w)
    buf = torch.empty(n, dtype=torch.float64, device=dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def run(p, **over):
        e0.record()
        C.lle2d(w["system"], precision=p, out=buf, **dict(kw, **over))
        e1.record()
        torch.cuda.synchronize()
        return buf.cpu().numpy().copy(), e0.elapsed_time(e1) / 1e3

    run(C.FP64, nPts=64)  # warm-up launch
    a, t64 = run(C.FP64)
    ic = list(w["initialConditions"])
    p13, _ = run(C.FP64, initialConditions=[ic[0] + 1e-13] + ic[1:])
    self_spread = lle_error_stats(p13, a)
    out = {"fp64_plain": {"value": steps / t64, "unit": UNIT, "seconds": t64,
                          "map": f"{w['nPts']}x{w['nPts']} (the benchmark's map), one launch"}}
    errs = {"fp64_started_1e-13_away": self_spread}

    def vs_self(st):
        return {**st, "p50_vs_self_spread": st["p50"] / self_spread["p50"],
                "p90_vs_self_spread": st["p90"] / self_spread["p90"]}
    if prec == C.FF32:
        errs["ff32"] = vs_self(lle_error_stats(head_map, a))
        out["speedup_vs_fp64_plain"] = {"ff32": t64 / head_s}
    fp32 = {}
    old = C.get_tuning(C.TUNE_LLE_RENORM)
    for mode, name in ((0, "pow2_exact"), (1, "fp32_log_per_block"), (2, "fp64_norm_log_per_block")):
        C.set_tuning(C.TUNE_LLE_RENORM, mode)
        run(C.FP32, nPts=64)
        v, t32 = run(C.FP32)
        fp32[name] = {"value": steps / t32, "unit": UNIT, "seconds": t32,
                      "error_vs_fp64": vs_self(lle_error_stats(v, a))}
        if mode == 0:
            achieved = w["flops"] * steps / t32 / 1e12
            fp32[name]["roofline"] = {"bound": "fp32_fma", "achieved": achieved, "peak": fma_peak,
                                      "unit": "TFLOP/s", "frac": achieved / fma_peak if fma_peak else None}
            errs["fp32"] = fp32[name]["error_vs_fp64"]
            out.setdefault("speedup_vs_fp64_plain", {})["fp32"] = t64 / t32
    C.set_tuning(C.TUNE_LLE_RENORM, old)
    out["fp32"] = {"renorm_ablation": fp32,
                   "note": "the FP32 map's error does not depend on how the stretch is measured: it comes from "
                           "the FP32 orbit (rounded at 2^-24 every step), which the float-float orbit removes"}
    out["lle_error_vs_fp64"] = {**errs, "regular": f"FP64 LLE < {REGULAR}"}
    # FP32 map with the FP64 sign re-check of the points within 0.01 of zero
    C.lle2d_checked(w["system"], **dict(kw, nPts=64))
    e0.record()
    oc, n_checked, n_replaced = C.lle2d_checked(w["system"], band=0.01, checkTMax=w["tMax"] / 10, **kw)
    e1.record()
    torch.cuda.synchronize()
    tc = e0.elapsed_time(e1) / 1e3

    def cls(v):
        return np.where(~np.isfinite(v), -1, (v > 0).astype(int))
    out["fp64_sign_recheck"] = {
        "band": 0.01, "check_tmax": w["tMax"] / 10, "points_checked": n_checked, "points_replaced": n_replaced,
        "value": steps / tc, "unit": UNIT,
        "sign_class_agreement_with_fp64": {"fp32_rechecked": float(np.mean(cls(oc) == cls(a))),
                                           "ff32": float(np.mean(cls(head_map) == cls(a)))
                                           if prec == C.FF32 else None}}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--workload", default="lle",
                    choices=["lle", "bif1d", "bif2d", "basins", "spectrum", "batch", "serve"])
    ap.add_argument("--requests", type=int, default=10000, help="served stream length")
    ap.add_argument("--rate", type=float, default=16.0, help="served stream arrival rate (requests/s)")
    ap.add_argument("--repeats", type=int, default=1, help="served streams (seeds 7, 8, ...)")
    ap.add_argument("--hbm-budget-gb", type=int, default=64)
    ap.add_argument("--iteration-steps", type=float, default=2e10)
    ap.add_argument("--precision", default="auto", choices=["auto", "ff32", "fp32", "fp64"],
                    help="auto: ff32 for the LLE map (the arithmetic that meets the FP64 map's own spread), "
                         "fp32 for the other workloads")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-extras", action="store_true", help="skip the FP64 comparison and the CPU baseline")
    ap.add_argument("--lle-variant", type=int, default=0, help="FP32 LLE kernel variant (0 default, 2, 12, 16)")
    ap.add_argument("--npts", type=int, default=None, help="grid resolution override (profiling runs only)")
    ap.add_argument("--tmax", type=float, default=None, help="tMax override (profiling runs only)")
    args = ap.parse_args()
    if args.precision == "auto":  # the LLE arithmetic that matches FP64 to the FP64 map's own spread
        if args.impl == "reference":
            args.precision = "fp64"  # the reference's own code computes in FP64
        else:
            args.precision = "ff32" if args.workload in ("lle", "batch") else "fp32"
    for w in (LLE, BIF1D, BIF2D, BASINS, SPECTRUM):
        if args.npts:
            w["nPts"] = args.npts
        if args.tmax:
            w["tMax"] = args.tmax
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        reference_arm(args, ws, rank)
    elif args.workload == "batch":
        batch_arm(args, ws, rank, local)
    elif args.workload == "serve":
        if rank == 0:
            serve_arm(args, ws, rank, local)
    else:
        engine_arm(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
