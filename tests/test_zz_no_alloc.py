"""chaos_point_dbscan_noalloc: the per-point interval clustering of the 2-D
bifurcation for callers that cannot call cudaMalloc during the call (hosts
that own all device memory through their own allocator and budget,
latency-critical loops where an allocation would synchronise the device).
Its scratch is a fixed array inside the library, so the test calls it twice
in a row through the C ABI and checks each result against the allocating
entry point, chaos_point_dbscan, exactly (integer labels). Counts below -1
(accepted from callers) must give 0, as the reference's dbscan does for any
count <= 0. Collected last on purpose: it runs alone or after the rest."""
import ctypes as C

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def _noalloc(engine):
    fn = engine.lib().chaos_point_dbscan_noalloc
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_longlong, C.c_int, C.c_double, C.c_void_p]
    fn.restype = C.c_int
    return fn


def _cases():
    g = golden("point_dbscan")
    yield g["intervals"], g["counts"], float(g["eps"])
    rng = np.random.default_rng(99)
    iv = np.round(rng.uniform(0.3, 1.7, size=(500, 96)), 2)
    counts = rng.integers(-1, 97, size=500).astype(np.int32)
    counts[:4] = [-2, -7, -1, 0]  # below -1: 0, as dbscan (bifurcationCUDA.cu:520-521) returns for P <= 0
    yield iv, counts, 0.02


def test_point_dbscan_noalloc_matches_allocating_entry(engine):
    import torch

    from chaoslibrary_gb300 import _native as N

    fn = _noalloc(engine)
    dev = torch.device("cuda", 0)
    ex = N.Exec(N.FP64, N.MEM_DEVICE, C.c_void_p(N.CUDA_STREAM_LEGACY), 0)
    for iv, counts, eps in _cases():
        expected = engine.point_dbscan(iv, counts, eps)
        n, stride = iv.shape
        d_iv = torch.tensor(iv, dtype=torch.float64, device=dev)
        d_counts = torch.tensor(counts, dtype=torch.int32, device=dev)
        for call in range(2):  # the second call starts from the first call's scratch contents
            out = torch.full((n,), -777, dtype=torch.int32, device=dev)
            rc = fn(C.byref(ex), d_iv.data_ptr(), d_counts.data_ptr(), n, stride, eps, out.data_ptr())
            assert rc == 0, engine.lib().chaos_last_error()
            torch.cuda.synchronize()
            assert np.array_equal(out.cpu().numpy(), expected), f"call {call}"
        if counts[0] == -2:
            assert list(expected[:4]) == [0, 0, -1, 0]


def test_point_dbscan_noalloc_rejects_oversize(engine):
    from chaoslibrary_gb300 import _native as N

    fn = _noalloc(engine)
    ex = N.Exec(N.FP64, N.MEM_DEVICE, C.c_void_p(N.CUDA_STREAM_LEGACY), 0)
    rc = fn(C.byref(ex), 1 << 20, 1 << 20, 1 << 11, 1 << 10, 0.01, 1 << 20)  # 2^21 entries: refused before use
    assert rc == -1
    assert b"exceeds the fixed scratch" in engine.lib().chaos_last_error()
