"""Restart files and convergence files: the neighbours of the solve step on
disk (FastC/FastC/PyTree.py:3514-3560 save / load; conv2pytree.for
residuals.bin / residuals.dat).

save / load keep the CGNS/Python tree node for node in a numpy .npz
container (Cassiopee's HDF5 writer and h5py are not available), without the
_P1 level and the solver's own data as FastC.saveTree does; a reloaded tree
restarts with its _M1 level (first_iter = 1: BDF2 at once), so a run cut
in two by a restart gives the bits of the uninterrupted run."""
import os

import numpy as np
import pytest

from fast_gb300 import cases, fastc, fasts
from fast_gb300 import pytree as I


def _sol(t, n=0):
    return I.getNodeFromName1(I.getZones(t)[n], I.__FlowSolutionCenters__)


def test_save_load_round_trip(tmp_path):
    t = cases.bc_box(n=(8, 6, 4), outflow="BCOutpres", model="NSTurbulent")
    fasts.prepare(t)
    I.createUniqueChild(t, "Iteration", "DataArray_t", 12)
    I.createUniqueChild(t, "Time", "DataArray_t", 0.375)
    f = str(tmp_path / "restart.npz")
    fastc.save(t, f)
    t2, tc, ts, graph = fastc.load(f)
    assert tc is None and ts is None and graph is None
    assert I.getValue(I.getNodeFromName1(t2, "Iteration")) == 12
    assert I.getValue(I.getNodeFromName1(t2, "Time")) == 0.375
    s1, s2 = _sol(t), _sol(t2)
    names2 = [c[0] for c in s2[2]]
    assert not any(n.endswith("_P1") for n in names2)
    for c in s1[2]:
        if c[0].endswith("_P1"):
            continue
        b = I.getNodeFromName1(s2, c[0])[1]
        assert b.shape == c[1].shape and np.array_equal(b, c[1])
    z2 = I.getZones(t2)[0]
    assert I.getNodeFromName1(z2, ".Solver#ownData") is None
    assert I.getNodeFromName1(z2, ".Solver#define") is not None
    bc = [b for b in I.getNodesFromType(t2, "BC_t") if I.getValue(b) == "BCOutpres"][0]
    p = I.getNodeFromName(bc, "Pressure")
    assert p is not None and p[1].size == 6 * 4
    # a reloaded tree is prepared as a restart
    fasts.prepare(t2)
    assert fasts.PREPARED_FIRST_IT == 1
    t3 = cases.bc_box(n=(8, 6, 4))
    fasts.prepare(t3)
    assert fasts.PREPARED_FIRST_IT == 0


@pytest.mark.gpu
def test_restart_continues_bit_for_bit(tmp_path):
    """2 steps, save, load, warmup, 2 steps == 4 uninterrupted steps."""
    mk = lambda: cases.taylor_green(n=(12, 10, 8), ss_iteration=3)
    t = mk()
    t, tc, m = fasts.warmup(t, None)
    for it in range(1, 5):
        fasts._compute(t, m, it)
    ref = fastc.compactArray(I.getZones(t)[0], "").copy()
    ref_m1 = fastc.compactArray(I.getZones(t)[0], "_M1").copy()
    fasts.HOOK["solver"].close()
    t = mk()
    t, tc, m = fasts.warmup(t, None)
    for it in range(1, 3):
        fasts._compute(t, m, it)
    f = str(tmp_path / "restart.npz")
    fastc.save(t, f)
    fasts.HOOK["solver"].close()
    t2, _, _, _ = fastc.load(f)
    t2, tc, m2 = fasts.warmup(t2, None)
    assert fasts.HOOK["FIRST_IT"] == 1
    for it in range(3, 5):
        fasts._compute(t2, m2, it)
    z = I.getZones(t2)[0]
    assert np.array_equal(fastc.compactArray(z, ""), ref)
    assert np.array_equal(fastc.compactArray(z, "_M1"), ref_m1)
    fasts.HOOK["solver"].close()
    fasts.HOOK = None


@pytest.mark.gpu
def test_convergence_files(tmp_path, monkeypatch):
    """display_temporal_criteria 'store' records, then 'ascii' writes them to
    residuals.dat and 'flush' appends them to residuals.bin as one Fortran
    unformatted record per zone and releases them."""
    monkeypatch.chdir(tmp_path)
    t = cases.taylor_green(n=(10, 8, 6), ss_iteration=2)
    t, tc, m = fasts.warmup(t, None)
    fasts._createConvergenceHistory(t, 10)
    for it in range(1, 4):
        fasts._compute(t, m, it)
        fasts.display_temporal_criteria(t, m, it, format="store")
    z = I.getZones(t)[0]
    ch = I.getNodeFromName1(z, "ZoneConvergenceHistory")
    assert int(I.getValue(ch)) == 3
    l2 = I.getNodeFromName1(ch, "RSD_L2")[1][:15].reshape(3, 5).copy()
    fasts.display_temporal_criteria(t, m, 3, format="ascii")
    assert os.path.exists("residuals.dat")
    lines = open("residuals.dat").read().splitlines()
    assert lines[0].startswith("VARIABLES") and lines[1].startswith("ZONE") and len(lines) == 5
    assert int(I.getValue(ch)) == 3
    fasts.display_temporal_criteria(t, m, 3, format="flush")
    assert int(I.getValue(ch)) == 0
    recs = fasts.read_residuals_bin("residuals.bin")
    assert len(recs) == 1
    name, its, rl2, roo = recs[0]
    assert name == z[0] and list(its) == [1, 2, 3]
    assert np.array_equal(rl2, l2)
    raw = open("residuals.bin", "rb").read()
    n = int(np.frombuffer(raw, "<i4", 1, 0)[0])
    assert len(raw) == n + 8 and int(np.frombuffer(raw, "<i4", 1, n + 4)[0]) == n
    fasts.HOOK["solver"].close()
    fasts.HOOK = None
