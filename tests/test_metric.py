"""Curvilinear (3-d general) zones on the CPU: the host metric restatement
against the oracle's, and the oracle's known answers on a periodic
curvilinear mesh (free-stream preservation, discrete conservation)."""
import numpy as np
import pytest

from fast_gb300 import cases, fasts, pytree as I


def _coords(t):
    z = I.getZones(t)[0]
    gc = I.getNodeFromName1(z, "GridCoordinates")
    return [I.getNodeFromName1(gc, n)[1] for n in ("CoordinateX", "CoordinateY", "CoordinateZ")]


@pytest.mark.parametrize("wavy", [0.0, 0.3])
def test_metric_equals_oracle(oracle_mod, wavy):
    t = cases.isentropic_vortex(n=(10, 8, 6), wavy=wavy)
    zd = fasts.zone_data(t, fasts.prepare(t))[0]
    pi = zd["pi"]
    assert int(pi[25]) == (0 if wavy else 2)
    o = oracle_mod.metric(pi, *_coords(t))
    for a, b in zip(o, (zd["ti"], zd["tj"], zd["tk"], zd["vol"])):
        assert np.array_equal(a, b)


def test_metric_closes_cells(oracle_mod):
    """Sum of the outward face vectors of every cell vanishes (to round-off)
    and the volumes add up to the box."""
    t = cases.isentropic_vortex(n=(10, 8, 6), wavy=0.3)
    zd = fasts.zone_data(t, fasts.prepare(t))[0]
    pi = zd["pi"]
    nvi, nvj, nvk = int(pi[10]), int(pi[11]), int(pi[12])
    ti, tj, tk = (zd[k].reshape(3, nvk, nvj, nvi) for k in ("ti", "tj", "tk"))
    clo = (ti[:, :-1, :-1, 1:] - ti[:, :-1, :-1, :-1] + tj[:, :-1, 1:, :-1] - tj[:, :-1, :-1, :-1]
           + tk[:, 1:, :-1, :-1] - tk[:, :-1, :-1, :-1])
    assert np.max(np.abs(clo)) < 1e-12
    vol = zd["vol"].reshape(nvk, nvj, nvi)[2:-3, 2:-3, 2:-3]   # interior cells
    box = 20.0 * 20.0 * (20.0 / 10 * 6)
    assert abs(vol.sum() - box) < 1e-9 * box


@pytest.mark.parametrize("scheme,slope", [("roe", "o1"), ("roe_min", "minmod"), ("roe", "o3"),
                                          ("ausmpred", "o3")])
def test_free_stream_preservation_curvilinear(oracle_mod, scheme, slope):
    t = cases.isentropic_vortex(n=(12, 10, 6), beta=0.0, wavy=0.3,
                                numz={"scheme": scheme, "slope": slope, "time_step": 0.05})
    zd = fasts.zone_data(t, fasts.prepare(t))
    c = oracle_mod.Case(zd)
    c.apply_bc(0)
    c.apply_bc(1)
    q0 = c.z[0]["lv"][0].copy()
    for it in range(1, 4):
        c.compute(it, 1, 3, 1, modulo_verif=1000)
    assert np.max(np.abs(c.z[0]["lv"][0] - q0)) < 1e-13


def test_conservation_curvilinear(oracle_mod):
    """sum over the periodic box of vol x (W^{n+1} - W^n) (conservative)
    vanishes on a curvilinear mesh too."""
    t = cases.isentropic_vortex(n=(16, 16, 4), wavy=0.3,
                                numz={"scheme": "roe", "slope": "o3", "time_step": 0.05})
    zd = fasts.zone_data(t, fasts.prepare(t))
    c = oracle_mod.Case(zd)
    c.apply_bc(0)
    c.apply_bc(1)
    pi, pr = zd[0]["pi"], zd[0]["pr"]
    nd, cv = int(pi[41]), pr[2]
    ni, nj, nk = int(pi[0]), int(pi[1]), int(pi[2])
    nvi, nvj = int(pi[10]), int(pi[11])
    vol = zd[0]["vol"].reshape(-1, nvj, nvi)[2:nk - 2, 2:nj - 2, 2:ni - 2]

    def total(q):
        ro, u, v, w, T = q.reshape(5, nk, nj, ni)[:, 2:nk - 2, 2:nj - 2, 2:ni - 2]
        e = ro * (cv * T + 0.5 * (u * u + v * v + w * w))
        cons = np.stack([ro, ro * u, ro * v, ro * w, e])
        return (cons * vol).sum(axis=(1, 2, 3)), (np.abs(cons) * vol).sum(axis=(1, 2, 3))

    w0, _ = total(c.z[0]["lv"][0])
    c.compute(1, 1, 3, 1, modulo_verif=1000)
    w1, scale = total(c.z[0]["lv"][0])
    assert np.all(np.abs(w1 - w0) <= 1e-13 * scale)


def test_free_stream_preservation_curvilinear_viscous(oracle_mod):
    """Navier-Stokes on the curvilinear mesh: the Green-Gauss cells of
    fluvisq_3dfull_*.for are closed, so a uniform field has no gradient."""
    t = cases.taylor_green(n=(10, 8, 6), wavy=0.3, mach=0.2, ss_iteration=2, dt=0.05,
                           numb={"temporal_scheme": "explicit", "ss_iteration": 1,
                                 "modulo_verif": 1000})
    zd = fasts.zone_data(t, fasts.prepare(t))
    # uniform state (moving): ro = 1, u = (0.2, -0.1, 0.05), T = 1/(gamma cv)
    nd = int(zd[0]["pi"][41])
    for key in ("ro", "ro_m1", "ro_p1"):
        q = zd[0][key].reshape(5, nd)
        q[0], q[1], q[2], q[3] = 1.0, 0.2, -0.1, 0.05
        q[4] = q[4].mean()
    c = oracle_mod.Case(zd)
    c.apply_bc(0)
    c.apply_bc(1)
    q0 = c.z[0]["lv"][0].copy()
    for it in range(1, 3):
        c.compute(it, 1, 3, 1, modulo_verif=1000)
    assert np.max(np.abs(c.z[0]["lv"][0] - q0)) < 1e-13


@pytest.mark.parametrize("wavy", [0.0, 0.3])
def test_metric_2d_equals_oracle_and_free_stream(oracle_mod, wavy):
    """2-d zones (one cell in k, no k ghosts): cp_tijk / cp_vol 2-d branches
    against the oracle, and a free stream that stays a free stream."""
    t = cases.isentropic_vortex(n=(12, 10, 1), two_d=True, wavy=wavy, beta=0.0,
                                numz={"scheme": "roe", "slope": "o3", "time_step": 0.05})
    zd = fasts.zone_data(t, fasts.prepare(t))
    pi = zd[0]["pi"]
    assert int(pi[25]) == 3 and int(pi[4]) == 0
    o = oracle_mod.metric(pi, *_coords(t))
    for a, b in zip(o, (zd[0]["ti"], zd[0]["tj"], zd[0]["tk"], zd[0]["vol"])):
        assert np.array_equal(a, b)
    c = oracle_mod.Case(zd)
    c.apply_bc(0)
    c.apply_bc(1)
    q0 = c.z[0]["lv"][0].copy()
    for it in range(1, 4):
        c.compute(it, 1, 3, 1, modulo_verif=1000)
    assert np.max(np.abs(c.z[0]["lv"][0] - q0)) < 1e-14
