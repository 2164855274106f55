"""Laminar Navier-Stokes and Spalart-Allmaras on 2-d zones
(fluvisq_2d_{i,j}.for, SA/fluvisq_SA_2d_*, SA/sourceSA_grad_2d.for,
lu_{i,j}_2d_SA.for, mjr_newton_2d_SA.for).

CPU: the 2-d restatements against the 3-d cartesian ones (fluvisq_3dcart_*,
sourceSA_grad_3dcart.for) on the same flow extruded in k -- written from
different reference routines, so agreement to rounding checks both.
GPU: the sm_103a path against the oracle on curvilinear 2-d zones with a
no-slip wall, inflow, outflow and farfield (explicit and implicit, Roe with
its wall-face correction and AUSM+(P)).
"""
import numpy as np
import pytest

from conftest import rel_err
from fast_gb300 import cases, fasts


def _first_stage_residual(oracle_mod, t):
    zd = fasts.zone_data(t, fasts.prepare(t))
    c = oracle_mod.Case(zd)
    c.apply_bc(0)
    c.apply_bc(1)
    c.compute(1, 1, 1, 1, modulo_verif=1000)    # the first RK3 stage only
    return zd[0]["pi"], c.z[0]["drodm"]


@pytest.mark.parametrize("scheme,slope,wall,model", [
    ("ausmpred", "o3", "BCWallViscous", "NSLaminar"), ("roe", "o3", "BCWallViscous", "NSLaminar"),
    ("ausmpred", "o3", "BCWallInviscid", "NSLaminar"),
    ("ausmpred", "o3", "BCWallViscous", "NSTurbulent"), ("roe", "o3", "BCWallViscous", "NSTurbulent")])
def test_2d_laminar_equals_extruded_3d(oracle_mod, scheme, slope, wall, model):
    """The first-stage residual of a 2-d laminar case equals that of the same
    case extruded over 6 cells in k (periodic), on the k layers whose
    stencils stay clear of the k ghost layers (their edges with the j / i
    ghost rows are corner averages, so the extruded case is k-invariant only
    away from them)."""
    kw = dict(wall=wall, model=model, reynolds=200.0, scheme=scheme, slope=slope,
              temporal="explicit", time_step=0.01)
    pi2, r2 = _first_stage_residual(oracle_mod, cases.bc_box(n=(16, 12, 1), two_d=True, **kw))
    pi3, r3 = _first_stage_residual(oracle_mod, cases.bc_box(n=(16, 12, 6), extrude=True, **kw))
    assert int(pi2[25]) == 3 and int(pi3[25]) == 2
    ni, nj = 16, 12
    nv = 6 if model == "NSTurbulent" else 5
    a = r2.reshape(nv, 1, nj + 4, ni + 4)[:, 0, 2:-2, 2:-2]
    b = r3.reshape(nv, 10, nj + 4, ni + 4)[:, 2:-2, 2:-2, 2:-2]
    for k in (2, 3):                       # k = 3, 4 (1-based) of 6
        for v in (0, 1, 2, 4) + ((5,) if nv == 6 else ()):
            scale = np.max(np.abs(a[v]))
            assert np.max(np.abs(b[v, k] - a[v])) <= 1e-12 * scale, (k, v)
        assert np.max(np.abs(b[3, k])) <= 1e-12 * np.max(np.abs(a[1]))
    # the viscous terms act: the Euler residual of the same state differs
    _, re = _first_stage_residual(oracle_mod, cases.bc_box(n=(16, 12, 1), two_d=True,
                                                           **dict(kw, model="Euler")))
    e = re.reshape(5, 1, nj + 4, ni + 4)[:, 0, 2:-2, 2:-2]
    if nv == 6:
        return
    assert np.max(np.abs(e[1] - a[1])) > 1e-3 * np.max(np.abs(a[1]))


@pytest.mark.gpu
@pytest.mark.parametrize("scheme,slope,temporal,wavy", [
    ("ausmpred", "o3", "explicit", 0.3), ("roe", "o3", "explicit", 0.3),
    ("roe_min", "minmod", "implicit", 0.3), ("ausmpred", "o3", "implicit", 0.0),
    ("roe", "o1", "implicit", 0.3), ("senseur", "o3", "explicit", 0.3)])
def test_2d_laminar_gpu_parity(oracle_mod, scheme, slope, temporal, wavy):
    from test_gpu_parity import _check_levels, _pair
    t = cases.bc_box(n=(16, 12, 1), two_d=True, wall="BCWallViscous", model="NSLaminar",
                     reynolds=500.0, scheme=scheme, slope=slope, wavy=wavy, temporal=temporal,
                     ss_iteration=3, time_step=0.01 if temporal == "explicit" else 0.05)
    mv = 1000 if temporal == "explicit" else 1
    zd, ref, s = _pair(t, oracle_mod, mv)
    assert int(zd[0]["pi"][25]) == 3 and int(zd[0]["pi"][27]) == 2
    nfin = 3 if temporal == "explicit" else 4
    for it in range(1, 4):
        ref.compute(it, 1, nfin, 1, modulo_verif=mv)
        s.compute(it, 1, nfin, 1, 1)
    _check_levels(ref, s)
    if temporal == "implicit":
        nss = int(zd[0]["pi"][58])
        assert rel_err(s.residuals(0), ref.residual_norms(0, nss)) <= 1e-12
    s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("scheme,slope,temporal,wavy", [
    ("ausmpred", "o3", "explicit", 0.3), ("roe", "o3", "explicit", 0.0),
    ("ausmpred", "o3", "implicit", 0.3), ("roe_min", "minmod", "implicit", 0.3),
    ("senseur", "o3", "implicit", 0.3)])
def test_2d_spalart_allmaras_gpu_parity(oracle_mod, scheme, slope, temporal, wavy):
    from test_gpu_parity import _check_levels, _pair
    t = cases.bc_box(n=(16, 12, 1), two_d=True, wall="BCWallViscous", model="NSTurbulent",
                     reynolds=500.0, scheme=scheme, slope=slope, wavy=wavy, temporal=temporal,
                     ss_iteration=3, time_step=0.01 if temporal == "explicit" else 0.05)
    mv = 1000 if temporal == "explicit" else 1
    zd, ref, s = _pair(t, oracle_mod, mv)
    assert int(zd[0]["pi"][25]) == 3 and int(zd[0]["pi"][36]) == 6
    nfin = 3 if temporal == "explicit" else 4
    for it in range(1, 4):
        ref.compute(it, 1, nfin, 1, modulo_verif=mv)
        s.compute(it, 1, nfin, 1, 1)
    _check_levels(ref, s)
    s.close()
