import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built engine library")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    O.build()
    return O


@pytest.fixture(scope="session")
def engine():
    """The engine package with its CUDA library built and loaded (GPU tests only)."""
    from chaoslibrary_gb300 import build as B

    B.build()
    import chaoslibrary_gb300 as C

    C.lib()
    return C


def golden(name: str) -> dict:
    with np.load(GOLDEN / f"{name}.npz") as z:
        return {k: z[k] for k in z.files}


def sweep_kwargs(g: dict) -> dict:
    """Reference-style keyword arguments stored in a sweep fixture."""
    return dict(tMax=float(g["tMax"]), nPts=int(g["nPts"]), h=float(g["h"]), ic=g["ic"], ranges=g["ranges"],
                mut=g["mut"], wv=int(g["wv"]), maxValue=float(g["maxValue"]),
                transientTime=float(g["transientTime"]), values=g["values"])
