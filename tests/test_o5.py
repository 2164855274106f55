"""The fifth-order slopes o5 and o5sc (islope 5 and 7, FastC/FastC/PyTree.py:
1699-1706) with AUSM+(P): Slope/o5_slope_var.for (qm = c50 q_l + c51 q_nm +
c52 q_np + c53 q_nm2 + c54 q_np2, qp its mirror with q_nm3; constants of
template_FluxAndBalance.for:149-154) and o5sc_slope_var.for (the o5 states
blended with the first-order ones by the shock-sensor weight, as o3sc).
The six-point stencil needs three ghost layers, which the reference
requires of these slopes (FastS/FastS/Metric/allocate_metric.cpp:101-117).

CPU: the ghost-layer rule and known answers of the oracle.  GPU: the sm_103a
solve step against the oracle (1e-12 relative per cell)."""
import numpy as np
import pytest

from conftest import rel_err
from fast_gb300 import cases, fasts
from fast_gb300 import pytree as I


@pytest.mark.parametrize("slope", ["o5", "o5sc"])
def test_three_ghost_layers(slope):
    t = cases.taylor_green(n=(10, 8, 6), slope=slope)
    zd = fasts.zone_data(t, fasts.prepare(t))
    pi = zd[0]["pi"]
    assert [int(pi[3]), int(pi[4])] == [3, 3]
    assert int(pi[41]) == 16 * 14 * 12
    assert int(pi[64]) == {"o5": 5, "o5sc": 7}[slope]


def test_o5_without_three_ghost_layers_is_refused():
    t = cases.taylor_green(n=(10, 8, 6), slope="o3")
    for z in I.getZones(t):
        I.getNodeFromName1(z, ".Solver#define")
    from fast_gb300 import fastc
    fastc._setNum2Zones(t, {"slope": "o5"})
    with pytest.raises(ValueError, match="o\\(5\\)"):
        fasts.prepare(t)


@pytest.mark.parametrize("slope", ["o5", "o5sc"])
def test_o5_free_stream_preservation(oracle_mod, slope):
    t = cases.bc_box(n=(12, 10, 6), perturb=0.0, wall="BCWallInviscid", model="Euler",
                     slope=slope)
    zd = fasts.zone_data(t, fasts.prepare(t))
    c = oracle_mod.Case(zd)
    c.apply_bc(0)
    c.apply_bc(1)
    q0 = c.z[0]["lv"][0].copy()
    for it in range(1, 4):
        c.compute(it, 1, 3, 1, modulo_verif=1000)
    assert np.max(np.abs(c.z[0]["lv"][0] - q0)) < 1e-13


def test_o5_differs_from_o3(oracle_mod):
    """The o5 flux is not the o3 one (the stencil is read) and both advance
    the vortex alike to the order of the scheme difference."""
    out = []
    for sl in ("o3", "o5"):
        t = cases.taylor_green(n=(16, 16, 8), slope=sl, ss_iteration=2,
                               numb={"temporal_scheme": "explicit", "ss_iteration": 1,
                                     "modulo_verif": 1000}, dt=0.02)
        zd = fasts.zone_data(t, fasts.prepare(t))
        c = oracle_mod.Case(zd)
        c.apply_bc(0)
        c.apply_bc(1)
        for it in range(1, 3):
            c.compute(it, 1, 3, 1, modulo_verif=1000)
        ng = int(zd[0]["pi"][3])
        q = c.z[0]["lv"][0].reshape(5, 8 + 2 * ng, 16 + 2 * ng, 16 + 2 * ng)
        out.append(q[:, ng:-ng, ng:-ng, ng:-ng])
    d = np.max(np.abs(out[0] - out[1]))
    assert 1e-9 < d < 1e-3


CASES = [
    ("tgv", dict(slope="o5"), "implicit"),
    ("tgv", dict(slope="o5sc"), "implicit"),
    ("tgv", dict(slope="o5", wavy=0.3), "explicit"),
    ("tgv", dict(slope="o5sc", model="NSTurbulent"), "implicit"),
    ("box", dict(slope="o5", model="NSLaminar", wavy=0.3), "explicit"),
    ("box", dict(slope="o5sc", model="Euler", wall="BCWallInviscid"), "implicit"),
    ("box", dict(slope="o5", model="NSTurbulent"), "explicit"),
    ("box2d", dict(slope="o5", model="NSLaminar", wavy=0.3), "explicit"),
    ("box2d", dict(slope="o5sc", model="Euler", wall="BCWallInviscid"), "implicit"),
]


@pytest.mark.gpu
@pytest.mark.parametrize("kind,kw,temporal", CASES)
def test_o5_gpu_parity(oracle_mod, kind, kw, temporal):
    from test_gpu_parity import _check_levels, _pair
    kw = dict(kw)
    if kind == "tgv":
        numb = {"temporal_scheme": temporal, "ss_iteration": 3, "modulo_verif": 1}
        t = cases.taylor_green(n=(14, 12, 10), numb=numb, dt=0.05 if temporal == "implicit" else 0.02,
                               ss_iteration=3, **kw)
    else:
        two_d = kind == "box2d"
        t = cases.bc_box(n=(14, 10, 1) if two_d else (14, 10, 6), two_d=two_d, temporal=temporal,
                         ss_iteration=3, time_step=0.05 if temporal == "implicit" else 0.02, **kw)
    zd, ref, s = _pair(t, oracle_mod, 1)
    nfin = 4 if temporal == "implicit" else 3
    for it in range(1, 3):
        ref.compute(it, 1, nfin, 1, modulo_verif=1)
        s.compute(it, 1, nfin, 1, 1)
    _check_levels(ref, s)
    s.close()


@pytest.mark.gpu
def test_o5_senseur_is_refused():
    from fast_gb300._native import FastGB300Error, Solver
    t = cases.bc_box(n=(8, 8, 6), scheme="senseur", slope="o5")
    zd = fasts.zone_data(t, fasts.prepare(t))
    s = Solver(0)
    with pytest.raises(FastGB300Error, match="o5"):
        s.add_zone(zd[0]["pi"], zd[0]["pr"], zd[0]["ti"], zd[0]["tj"], zd[0]["tk"], zd[0]["vol"])
    s.close()
