"""temporal_scheme = 'explicit_local' at the drop-in boundary.

FastS packs an explicit_local tree (FastC/FastC/PyTree.py:1080-1110,
1163-1166, 1841-1843: the time level of each zone from centers:niveaux_temps
in its middle cell, nssiter = 4 x the largest level, RK3, EXPLOC = 1,
explicit ITYPCP) and its warmup succeeds, but FastS._compute refuses the
C layer for it (FastS/FastS/PyTree.py:73-76: ValueError "compute:
'explicit_local' & 'c layer' is not implemented."); only the Python layer,
through Cassiopee's Connector transfers, runs it.  The drop-in replaces the C
layer, so it packs the same parameters and raises the same error.  No GPU is
needed: warmup builds no solver for such a tree.
"""
import numpy as np
import pytest

from fast_gb300 import cases, fastc, fasts
from fast_gb300 import pytree as I


def _local_tree(levels):
    zs = []
    for m, lv in enumerate(levels):
        t = cases.taylor_green(n=8, ss_iteration=4, name="tgv%d" % m,
                               numb={"temporal_scheme": "explicit_local", "modulo_verif": 10})
        z = I.getZones(t)[0]
        sol = I.getNodeFromName1(z, I.__FlowSolutionCenters__)
        ro = I.getNodeFromName1(sol, "Density")[1]
        field = np.full(ro.shape, float(lv), order="F")
        field.flat[0] = 7.0   # a corner value: only the middle cell counts
        I.createUniqueChild(sol, "niveaux_temps", "DataArray_t", field)
        zs.append((t, z))
    t = zs[0][0]
    base = I.getBases(t)[0]
    for _, z in zs[1:]:
        base[2].append(z)
    return t


def test_explicit_local_parameters_follow_fastc():
    t = _local_tree([1, 2])
    fastc._buildOwnData(t)
    dtloc = I.getNodeFromName1(I.getNodeFromName1(t, ".Solver#ownData"), ".Solver#dtloc")[1]
    assert int(dtloc[0]) == 8          # nssiter = 4 x maxlevel
    assert int(dtloc[9]) == 2          # maxlevel
    for z, lv in zip(I.getZones(t), (1, 2)):
        pi = I.getNodeFromName2(z, "Parameter_int")[1]
        assert int(pi[fastc.LEVEL]) == lv
        assert int(pi[fastc.EXPLOC]) == 1
        assert int(pi[fastc.RK]) == 3
        assert int(pi[fastc.ITYPCP]) == 2
        assert int(pi[fastc.NSSITER]) == 8


def test_explicit_local_compute_refused_like_fasts_c_layer():
    t = _local_tree([1, 2])
    t, tc, metrics = fasts.warmup(t, None)
    assert fasts.HOOK["solver"] is None
    with pytest.raises(ValueError, match="'explicit_local' & 'c layer' is not implemented"):
        fasts._compute(t, metrics, 1)
    fasts.HOOK = None


def test_explicit_local_needs_levels():
    t = cases.taylor_green(n=8, numb={"temporal_scheme": "explicit_local"})
    with pytest.raises(ValueError, match="niveaux_temps"):
        fastc._buildOwnData(t)
