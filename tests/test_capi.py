"""CPU checks of the C ABI: the library loads and exports every entry point
that include/fast_gb300.h declares (no compute call, no GPU needed)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _declared():
    h = (ROOT / "include" / "fast_gb300.h").read_text()
    return sorted(set(re.findall(r"\b(fgb_[a-z0-9_]+)\s*\(", h)))


@pytest.fixture(scope="module")
def lib():
    from fast_gb300 import build as fb
    path = fb.LIB
    if not path.exists():
        pytest.skip("library not built (run __graft_entry__.build())")
    return ctypes.CDLL(str(path))


def test_every_declared_symbol_is_exported(lib):
    names = _declared()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n


def test_binding_covers_header():
    from fast_gb300 import _native
    assert set(_declared()) == set(_native.SIGNATURES)


def test_last_error_is_empty_string(lib):
    lib.fgb_last_error.restype = ctypes.c_char_p
    assert isinstance(lib.fgb_last_error(), bytes)


def test_null_arguments_are_rejected_without_gpu(lib):
    lib.fgb_create.argtypes = [ctypes.c_int, ctypes.c_void_p]
    assert lib.fgb_create(0, None) == 1          # FGB_ERR_ARG, no device touched
    lib.fgb_compute.argtypes = [ctypes.c_void_p] + [ctypes.c_int] * 5
    assert lib.fgb_compute(None, 1, 1, 3, 1, 1) == 1
