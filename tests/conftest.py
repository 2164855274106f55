"""Shared test setup: the `gpu` marker, import paths and case helpers."""
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
for p in (ROOT, ROOT / "oracle"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


def rel_err(got, exp):
    """max |got-exp| / (|exp| + tiny), the per-cell relative error."""
    got = np.asarray(got, dtype=np.float64)
    exp = np.asarray(exp, dtype=np.float64)
    return float(np.max(np.abs(got - exp) / (np.abs(exp) + 1e-300))) if exp.size else 0.0
