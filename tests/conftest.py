"""Shared fixtures of the solver-step tests. `gpu` marks tests that need a
CUDA device (the parity tests proper); everything else runs on the CPU."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (parity tests through the C ABI)")


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return dict(np.load(GOLDEN / f"{name}.npz"))
    return load


@pytest.fixture(scope="session")
def mg():
    """The golden-vector generator's case definitions (geometries, layouts);
    importing it needs no reference tree."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", GOLDEN / "make_golden.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def built_lib():
    from foil_cfd_gb300 import build_lib
    return build_lib.build()


def written_mask(flags):
    """Cells a stream-collide step writes (fluid, inlet, outlets)."""
    f = np.asarray(flags)
    return (f == 0) | (f == 2) | (f == 3) | (f == 9)


def rel_err(a, b, mask=None):
    """max |a - b| / max |b| over the masked cells (ρ or a velocity field)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    if mask is not None:
        a, b = a[..., mask], b[..., mask]
    den = np.abs(b).max()
    return float(np.abs(a - b).max() / (den if den > 0 else 1.0))
