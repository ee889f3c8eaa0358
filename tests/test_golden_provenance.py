"""The committed golden vectors are the reference's own output.

Every fixture under tests/golden/ is regenerated by make_golden.py from the
reference's kernels, host builders and snapshot code (compiled for the CPU
from the reference tree by oracle/ref_build.py) into a scratch directory and
compared with the committed file, array by array and bit for bit. Skipped
where the reference tree is absent; the fixtures themselves never need it."""
from __future__ import annotations

import importlib.util
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


def _bits(a):
    return a.view(np.uint8) if a.dtype.kind in "fc" else a


def test_committed_fixtures_regenerate_bit_for_bit(tmp_path):
    from oracle import ref_build
    if not ref_build.available():
        pytest.skip("reference tree not present")
    spec = importlib.util.spec_from_file_location("make_golden_regen", GOLDEN / "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    mg.OUT = tmp_path
    mg.main([])
    committed = sorted(GOLDEN.glob("*.npz"))
    assert committed and {f.name for f in committed} == {f.name for f in tmp_path.glob("*.npz")}
    diff = []
    for f in committed:
        a, b = np.load(f), np.load(tmp_path / f.name)
        if set(a.files) != set(b.files):
            diff.append(f"{f.name}: arrays {sorted(set(a.files) ^ set(b.files))}")
            continue
        for k in a.files:
            x, y = a[k], b[k]
            if x.dtype != y.dtype or x.shape != y.shape or not np.array_equal(_bits(x), _bits(y)):
                diff.append(f"{f.name}:{k}")
    assert not diff, diff
