"""The committed fixtures are what tests/golden/make_golden.py makes from the
reference's own code: regenerated into a temporary folder where the host build
of the reference exists (oracle/build_ref.py), every array of every fixture is
bit-identical to the committed one."""
import importlib.util
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O

GOLDEN = Path(__file__).resolve().parent / "golden"

pytestmark = pytest.mark.skipif(
    not (all(O.ref_available(s) for s in ("lorenz", "chameleon", "sin3", "rossler")) and O.legacy_available()),
    reason="host build of the reference not present")


def test_fixtures_regenerate_bit_identical(tmp_path):
    pytest.importorskip("sklearn")
    spec = importlib.util.spec_from_file_location("make_golden", GOLDEN / "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    mg.main(tmp_path)
    mg.legacy_fixtures(tmp_path)
    committed = sorted(GOLDEN.glob("*.npz"))
    assert {f.name for f in committed} == {f.name for f in tmp_path.glob("*.npz")}
    for f in committed:
        with np.load(f) as a, np.load(tmp_path / f.name) as b:
            assert set(a.files) == set(b.files), f.name
            for k in a.files:
                x, y = a[k], b[k]
                assert np.array_equal(x, y, equal_nan=x.dtype.kind == "f"), (f.name, k)
