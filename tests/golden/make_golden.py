"""Generates the golden fixtures in this folder from the reference's own code.

Run here, where the reference sources are present:
    python oracle/build_ref.py && python tests/golden/make_golden.py [legacy]
Every fixture is produced by the host build of the reference's functions
(oracle/_ref/libref_<system>.so, see oracle/build_ref.py), except
dbscan_sklearn.npz, which records scikit-learn's DBSCAN labels. The legacy_*
fixtures come from the legacy library's own kernels run on the host
(oracle/_ref/libref_legacy.so); "legacy" writes only those. The fixtures
are small .npz files; the tests compare both the oracle and the GPU engine
against them.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))
from oracle import oracle as O  # noqa: E402

LORENZ = dict(values=[10.0, 28.0, 8.0 / 3.0], ic=[0.1, 0.1, 0.1])
CHAMELEON = dict(values=[0.5, 3.0, 0.0, 2.0, 1.0, 18.0, 1.0], ic=[3.0, 3.0, 0.0])


def crafted_series(rng) -> np.ndarray:
    """Series exercising the peak rules: plateaus, equal neighbours, rises and
    drops at and around 1e-13, first/last-sample peaks, flat series."""
    L = 64
    rows = []
    base = np.sin(np.arange(L) * 0.4)
    rows.append(base)
    rows.append(np.round(base * 4) / 4)  # long plateaus at maxima
    r = base.copy(); r[10:14] = r[10]; rows.append(r)  # plateau on a rise
    r = np.zeros(L); r[5] = 1e-13; r[20] = 2e-13; r[21] = 2e-13; r[40] = 1.0; rows.append(r)
    r = np.zeros(L); r[::2] = 1.0; rows.append(r)  # zig-zag
    r = np.zeros(L); r[1::3] = 1.0; r[2::3] = 1.0; rows.append(r)  # two-sample plateaus
    rows.append(np.ones(L))
    r = np.arange(L, dtype=float); rows.append(r)  # monotone
    r = -np.arange(L, dtype=float); r[0] = 100; rows.append(r)  # peak at sample 0
    r = np.arange(L, dtype=float); r[-1] = -1; rows.append(r)  # peak at the last-but-one
    r = np.zeros(L); r[7:12] = [1, 1, 1 + 5e-14, 1, 0]; rows.append(r)
    r = np.zeros(L); r[7:12] = [1, 1 + 2e-13, 1 + 2e-13, 1 + 1e-13, 0]; rows.append(r)
    for _ in range(20):
        rows.append(np.round(rng.normal(size=L).cumsum(), 1))
    return np.array(rows)


def main(out: Path = HERE) -> None:
    rng = np.random.default_rng(12345)
    lor = O.RefLib("lorenz")
    cham = O.RefLib("chameleon")

    # peak finder on crafted and random series (Bifurcation_constants::peakFinder)
    for name, data in [("peaks_crafted", crafted_series(rng)),
                       ("peaks_random", np.round(rng.normal(size=(64, 400)).cumsum(axis=1), 2))]:
        counts, pk, iv = [], np.zeros((len(data), data.shape[1])), np.zeros((len(data), data.shape[1]))
        for s, row in enumerate(data):
            c, p, t = lor.peak_finder(row, 0.01)
            counts.append(c)
            pk[s, :c], iv[s, :c] = p, t
        np.savez_compressed(out / f"{name}.npz", data=data, h=0.01, counts=np.array(counts, np.int32),
                            peaks=pk, intervals=iv)

    # per-point dbscan of the 2-D bifurcation (Bifurcation_constants::dbscan)
    P = 48
    iv = np.round(rng.uniform(0.5, 1.5, size=(60, P)), 3)
    iv[::7] = np.round(iv[::7], 1)
    counts = rng.integers(-1, P + 1, size=60).astype(np.int32)
    counts[:4] = [-1, 0, 1, 2]
    labels = []
    for k in range(60):
        c = int(counts[k])
        if c <= 0:
            labels.append(-1 if c == -1 else 0)
        else:
            labels.append(lor.point_dbscan(np.zeros(P), iv[k], c, 2 * P + 2, 0.05))
    np.savez_compressed(out / "point_dbscan.npz", intervals=iv, counts=counts, eps=0.05,
                        labels=np.array(labels, np.int32))

    # 1-D / 2-D bifurcation sweeps through the reference kernels
    sweeps = {
        "bif1d_lorenz": (lor, 1, dict(tMax=20.0, nPts=64, h=0.01, ic=LORENZ["ic"], ranges=[20.0, 200.0], mut=[1],
                                      wv=0, maxValue=1e4, transientTime=20.0, values=LORENZ["values"]), 0.0),
        "bif1d_chameleon": (cham, 1, dict(tMax=40.0, nPts=48, h=0.01, ic=CHAMELEON["ic"], ranges=[0.0, 5.0],
                                          mut=[3], wv=0, maxValue=1e4, transientTime=20.0,
                                          values=CHAMELEON["values"]), 0.0),
        "bif2d_lorenz": (lor, 2, dict(tMax=10.0, nPts=14, h=0.01, ic=LORENZ["ic"], ranges=[20.0, 200.0, 5.0, 15.0],
                                      mut=[1, 0], wv=0, maxValue=1e4, transientTime=10.0,
                                      values=LORENZ["values"]), 0.05),
        "bif2d_chameleon": (cham, 2, dict(tMax=20.0, nPts=12, h=0.01, ic=CHAMELEON["ic"],
                                          ranges=[0.0, 5.0, 0.0, 20.0], mut=[3, 5], wv=0, maxValue=1e4,
                                          transientTime=10.0, values=CHAMELEON["values"]), 0.001),
    }
    for name, (R, dim, kw, eps) in sweeps.items():
        r = R.bifurcation(dim, eps=eps, **kw)
        c = r["counts"]
        cap = max(int(c.max()), 1)
        pk = np.zeros((c.size, cap))
        iv = np.zeros((c.size, cap))
        first = np.zeros(c.size)
        for k in range(c.size):
            if c[k] > 0:
                pk[k, :c[k]] = r["data"][k, :c[k]]
                iv[k, :c[k]] = r["intervals"][k, :c[k]]
            if c[k] == -1:
                first[k] = r["data"][k, 0]
        extra = dict(labels=r["labels"]) if dim == 2 else {}
        np.savez_compressed(out / f"{name}.npz", dim=dim, eps=eps, counts=c, peaks=pk, intervals=iv, first=first,
                            **{k: np.asarray(v) for k, v in kw.items()}, **extra)

    # basins: features and the reference's global clustering
    bas = {
        "basins_lorenz": (lor, dict(tMax=5.0, nPts=24, h=0.01, ic=[0.0, 0.0, 27.0], ranges=[-30.0, 30.0, -30.0, 30.0],
                                    mut=[0, 1], wv=0, maxValue=1e8, transientTime=20.0,
                                    values=[10.0, 24.0, 8.0 / 3.0]), 0.05),
        "basins_sin3": (O.RefLib("sin3"), dict(tMax=30.0, nPts=16, h=0.01, ic=[0.0, 0.0, 0.0],
                                               ranges=[-6.0, 6.0, -6.0, 6.0], mut=[0, 1], wv=1, maxValue=1e8,
                                               transientTime=50.0, values=[0.5, 0.1, 1.4, 15.552, 2.0]), 0.05),
    }
    for name, (R, kw, eps) in bas.items():
        r = R.basins(**kw)
        labels = R.basins_dbscan(r["avg_peaks"], r["avg_intervals"], r["flags"], eps)
        np.savez_compressed(out / f"{name}.npz", eps=eps, flags=r["flags"], avg_peaks=r["avg_peaks"],
                            avg_intervals=r["avg_intervals"], labels=labels,
                            **{k: np.asarray(v) for k, v in kw.items()})

    # the reference clustering on synthetic feature arrays with all three flags
    n = 1500
    centres = rng.uniform(0, 2, size=(12, 2))
    lab = rng.integers(0, 12, size=n)
    ap = centres[lab, 0] + rng.normal(scale=0.02, size=n)
    ai = centres[lab, 1] + rng.normal(scale=0.02, size=n)
    flags = np.ones(n, np.int32)
    flags[rng.random(n) < 0.1] = -1
    zero = rng.random(n) < 0.05
    flags[zero] = 0
    ap[zero], ai[zero] = 999.0, 999.0
    ap[:20] = np.round(ap[:20], 1)  # exact duplicates
    labels = lor.basins_dbscan(ap, ai, flags, 0.05)
    np.savez_compressed(out / "dbscan_compat.npz", avg_peaks=ap, avg_intervals=ai, flags=flags, eps=0.05,
                        labels=labels)

    # LLE through the reference's calculateSystem (deterministic twin offset)
    rl = O.RefLib("rossler")
    kw = dict(tMax=50.0, NT=0.1, nPts=8, h=0.01, eps=1e-8, ic=[1.0, 1.0, 1.0], ranges=[0.1, 0.4, 2.0, 10.0],
              mut=[0, 2], transientTime=10.0, values=[0.2, 0.2, 5.7])
    lle = rl.lle(**kw)
    np.savez_compressed(out / "lle_rossler.npz", lle=lle, **{k: np.asarray(v) for k, v in kw.items()})

    # textbook DBSCAN labels from scikit-learn
    from sklearn.cluster import DBSCAN
    import sklearn

    X = np.concatenate([rng.normal(loc=c, scale=0.02, size=(150, 3)) for c in rng.uniform(0, 1, size=(6, 3))])
    X = np.concatenate([X, rng.uniform(0, 1, size=(200, 3))])
    X = np.round(X, 4)
    sk = DBSCAN(eps=0.05, min_samples=8).fit(X).labels_.astype(np.int32)
    np.savez_compressed(out / "dbscan_sklearn.npz", X=X, eps=0.05, min_pts=8, labels=sk,
                        sklearn_version=sklearn.__version__)
    print("fixtures written to", out)


# the legacy library's hard-wired system (the sin3 plug-in's arithmetic) in two regimes: damping 0.4
# under a bound of 2.5 (fixed points beside oscillations), damping 0.15 under 4 (mostly unbounded)
LEGACY_IC = [0.2, -0.1, 0.0]
LEGACY_REGIMES = {"fixed": (0.4, 2.5), "bound": (0.15, 4.0)}


def legacy_values(b: float) -> list:
    return [0.5, b, 1.4, 15.552, 2.0]


def legacy_fixtures(out: Path = HERE) -> None:
    """The legacy kernels of bifurcation1DIC / bifurcation2DIC, basinsOfAttraction
    and bifurcation1DForH in both regimes, and of LLE1D (with recorded cuRAND
    uniforms), LLE1DIC and LS1D."""
    leg = O.LegacyLib()
    ic = LEGACY_IC
    for regime, (b, mx) in LEGACY_REGIMES.items():
        V = legacy_values(b)
        for dim, n, rng, mut in ((1, 48, [-6.0, 6.0], [0]), (2, 12, [-6.0, 6.0, -6.0, 6.0], [0, 1])):
            kw = dict(tMax=40.0, nPts=n, h=0.01, transientTime=30.0, preScaller=2, ic=ic, values=V, ranges=rng,
                      mut=mut, wv=0, maxValue=mx, eps=0.05)
            r = leg.ic_bifurcation(dim, n, 40.0, 0.01, 30.0, 2, ic, V, rng, mut, 0, mx, eps=0.05)
            c = r["counts"]
            m = max(int(c.max()), 1)
            np.savez_compressed(out / f"legacy_ic_bif{dim}d_{regime}.npz", counts=c, peaks=r["peaks"][:, :m],
                                intervals=r["intervals"][:, :m],
                                labels=r["labels"] if dim == 2 else np.zeros(0, np.int32), dim=dim,
                                **{k: np.asarray(v) for k, v in kw.items()})
        kw = dict(tMax=40.0, nPts=12, h=0.01, transientTime=30.0, preScaller=3, ic=ic, values=V,
                  ranges=[-6.0, 6.0, -6.0, 6.0], mut=[0, 1], wv=1, maxValue=mx)
        r = leg.basins_v1(12, 40.0, 0.01, 30.0, 3, ic, V, kw["ranges"], [0, 1], 1, mx)
        np.savez_compressed(out / f"legacy_basins_{regime}.npz", flags=r["flags"], avg_peaks=r["avgPeaks"],
                            avg_intervals=r["avgIntervals"], **{k: np.asarray(v) for k, v in kw.items()})
        kw = dict(tMax=40.0, nPts=24, transientTime=10.0, preScaller=2, ic=ic, values=V, ranges=[0.005, 0.02],
                  wv=0, maxValue=mx)
        r = leg.step_sweep(24, 40.0, 10.0, 2, ic, V, [0.005, 0.02], 0, mx)
        m = max(int(r["counts"].max()), 1)
        np.savez_compressed(out / f"legacy_step_sweep_{regime}.npz", counts=r["counts"], peaks=r["peaks"][:, :m],
                            **{k: np.asarray(v) for k, v in kw.items()})
    V = legacy_values(0.2)
    u = np.random.default_rng(321).random(40).astype(np.float32)
    lle1d = leg.lle(0, 1, 32, 30.0, 0.5, 0.01, 1e-6, 10.0, ic, V, [0.1, 0.6], [1], 0.0, uniforms=u)
    lle1dic = leg.lle(1, 1, 32, 30.0, 0.5, 0.01, 1e-6, 10.0, ic, V, [-3.0, 3.0], [0], 3.0)
    ls1d = leg.ls(1, 12, 30.0, 0.5, 0.01, 1e-6, 10.0, ic, V, [0.1, 0.6], [1], 0.0)
    np.savez_compressed(out / "legacy_lle.npz", uniforms=u, lle1d=lle1d, lle1dic=lle1dic, ls1d=ls1d,
                        tMax=30.0, NT=0.5, h=0.01, eps=1e-6, transientTime=10.0, ic=np.asarray(ic),
                        values=np.asarray(V))
    print("legacy fixtures written to", out)


if __name__ == "__main__":
    if sys.argv[1:] == ["legacy"]:
        legacy_fixtures()
    else:
        main()
        legacy_fixtures()
