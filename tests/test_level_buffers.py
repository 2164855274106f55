"""Time-level arrays (fastc._level_buffers): the levels of a zone of at
least one transparent huge page each share one huge-page-advised anonymous
mapping, aligned to the huge page; smaller ones are plain numpy arrays.  Either is a writable,
C-contiguous (rows, n) float64 array, and a level can be saved, swapped and
reloaded like any other tree array."""
import numpy as np
import pytest

from fast_gb300 import cases, fastc, fasts
from fast_gb300 import pytree as I


def test_small_level_is_a_plain_array():
    for a in fastc._level_buffers(3, 5, 1000):
        assert a.shape == (5, 1000) and a.dtype == np.float64
        assert a.flags.c_contiguous and a.flags.writeable


def test_large_level_is_aligned_and_usable():
    hp = fastc._huge_page_bytes()
    if hp <= 0:
        pytest.skip("no transparent huge pages on this host")
    n = hp // 8 // 5 + 1000          # a level just over one huge page
    levels = fastc._level_buffers(3, 5, n)
    assert levels[0].ctypes.data % hp == 0
    for q, a in enumerate(levels):
        assert a.shape == (5, n) and a.flags.c_contiguous and a.flags.writeable
        a[:] = 3.0 + q
        a[4, -1] = 7.0
    for q, a in enumerate(levels):   # disjoint
        assert float(a.sum()) == (3.0 + q) * (5 * n - 1) + 7.0


def test_tree_levels_behave_like_numpy_arrays():
    t = cases.taylor_green(n=8, ss_iteration=2)
    fasts.prepare(t)
    z = I.getZones(t)[0]
    before = [np.array(fastc.compactArray(z, s)) for s in ("", "_M1", "_P1")]
    fastc.switchPointers__([z])
    after = [fastc.compactArray(z, s) for s in ("", "_M1", "_P1")]
    assert np.array_equal(after[0], before[2])
    assert np.array_equal(after[1], before[0])
    assert np.array_equal(after[2], before[1])
