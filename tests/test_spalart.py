"""Spalart-Allmaras (IFLOW 3, six equations) in the oracle: known answers
and internal consistency on the CPU.

* a uniform flow with uniform nutilde and no wall nearby stays uniform on a
  curvilinear periodic mesh, with the AUSM+(P) and the Roe SA fluxes (the SA
  fluxes and the source gradients of sourceSA_grad_3d.for are closed,
  production / destruction vanish);
* nutilde stays in [0, ratiom nu_lam] (core3ark3.for / mjr_newton_SA.for
  clip it there);
* the curvilinear restatements (fluvisq_SA_3dfull, sourceSA_grad_3d) agree
  with the cartesian ones (fluvisq_SA_3dcart, sourceSA_grad_3dcart) on a
  mesh displaced by 1e-5 of a step, to O(1e-5);
* the implicit SA diagonal: coe6 = coe5 - min(dS/d(ro nutilde), 0) coe1
  >= coe5, and the Newton residual of every equation contracts.
"""
import numpy as np
import pytest

from fast_gb300 import cases, fasts


def _case(oracle_mod, t):
    zd = fasts.zone_data(t, fasts.prepare(t))
    c = oracle_mod.Case(zd)
    c.apply_bc(0)
    c.apply_bc(1)
    return zd, c


def _interior(pi, q, nv=6):
    ni, nj, nk = int(pi[0]), int(pi[1]), int(pi[2])
    return q.reshape(nv, nk, nj, ni)[:, 2:nk - 2, 2:nj - 2, 2:ni - 2]


@pytest.mark.parametrize("temporal,scheme", [("explicit", "ausmpred"), ("implicit", "ausmpred"),
                                             ("explicit", "roe"), ("implicit", "roe"),
                                             ("explicit", "senseur")])
def test_sa_free_stream_curvilinear(oracle_mod, temporal, scheme):
    numb = ({"temporal_scheme": "explicit", "ss_iteration": 1, "modulo_verif": 1000}
            if temporal == "explicit" else None)
    t = cases.taylor_green(n=(10, 8, 6), wavy=0.3, mach=0.2, model="NSTurbulent", dt=0.05,
                           ss_iteration=2, numb=numb, scheme=scheme)
    zd = fasts.zone_data(t, fasts.prepare(t))
    pi = zd[0]["pi"]
    assert int(pi[36]) == 6 and int(pi[25]) == 0
    nd = int(pi[41])
    for key in ("ro", "ro_m1", "ro_p1"):
        q = zd[0][key].reshape(6, nd)
        q[0], q[1], q[2], q[3] = 1.0, 0.2, -0.1, 0.05
        q[4] = q[4].mean()
        q[5] = q[5].mean()
    c = oracle_mod.Case(zd)
    c.apply_bc(0)
    c.apply_bc(1)
    q0 = c.z[0]["lv"][0].copy()
    for it in range(1, 3):
        c.compute(it, 1, 3, 1, modulo_verif=1000)
    q = c.z[0]["lv"][0]
    scale = np.abs(q0.reshape(6, nd)).max(axis=1, keepdims=True)
    assert np.max(np.abs(q - q0).reshape(6, nd) / scale) < 1e-13


@pytest.mark.parametrize("temporal,wavy,scheme", [("explicit", 0.0, "ausmpred"),
                                                ("implicit", 0.3, "ausmpred"),
                                                ("explicit", 0.3, "roe"), ("implicit", 0.0, "roe")])
def test_sa_nutilde_bounds(oracle_mod, temporal, wavy, scheme):
    t = cases.bc_box(n=(12, 10, 6), model="NSTurbulent", temporal=temporal, ss_iteration=3,
                     wavy=wavy, reynolds=500.0, time_step=0.02, scheme=scheme)
    zd, c = _case(oracle_mod, t)
    pi, pr = zd[0]["pi"], zd[0]["pr"]
    for it in range(1, 5):
        c.compute(it, 1, 3, 1, modulo_verif=1)
    q = _interior(pi, c.z[0]["lv"][0])
    assert np.isfinite(q).all()
    ro, T, nu = q[0], q[4], q[5]
    cmus1, temp01 = pr[13], 1.0 / pr[12]
    mulam = pr[11] * (1.0 + cmus1 * temp01) * np.sqrt(T * temp01) / (1.0 + cmus1 / T)
    assert nu.min() >= 0.0
    assert np.all(nu <= pr[18] * mulam / ro * (1 + 1e-12))
    # the model is active: nutilde moved away from its initial field
    q0 = _interior(pi, zd[0]["ro"])
    assert np.max(np.abs(nu - q0[5])) > 1e-3 * np.max(np.abs(q0[5]))


def test_sa_curvilinear_matches_cartesian(oracle_mod):
    """One RK3 step of the SA box on a cartesian mesh (3dcart routines) and on
    the same mesh displaced by 1e-5 of a step (3dfull routines)."""
    out = []
    for wavy in (0.0, 1e-5):
        t = cases.bc_box(n=(12, 10, 6), model="NSTurbulent", temporal="explicit", wavy=wavy,
                         reynolds=500.0, time_step=0.02)
        zd, c = _case(oracle_mod, t)
        assert int(zd[0]["pi"][25]) == (2 if wavy == 0.0 else 0)
        c.compute(1, 1, 3, 1, modulo_verif=1000)
        out.append(_interior(zd[0]["pi"], c.z[0]["lv"][0]))
    a, b = out
    scale = np.max(np.abs(a), axis=(1, 2, 3), keepdims=True)
    scale[3] = np.max(np.abs(a[1]))   # w is small: measure it on the velocity scale
    err = np.max(np.abs(a - b) / scale)
    assert err < 1e-3, err
    # the equation-6 update itself must differ by O(1e-5), not O(1)
    d0 = a[5] - _interior(zd[0]["pi"], zd[0]["ro"])[5]
    assert np.max(np.abs((b[5] - a[5]))) < 1e-3 * np.max(np.abs(d0))


@pytest.mark.parametrize("wavy", [0.0, 0.3])
def test_sa_implicit_diagonal_and_contraction(oracle_mod, wavy):
    t = cases.bc_box(n=(12, 10, 6), model="NSTurbulent", temporal="implicit", ss_iteration=6,
                     wavy=wavy, reynolds=500.0, time_step=0.05)
    zd, c = _case(oracle_mod, t)
    pi = zd[0]["pi"]
    nd = int(pi[41])
    c.compute(1, 1, 6, 1, modulo_verif=1)
    coe = c.z[0]["coe"].reshape(6, nd)
    ni, nj, nk = int(pi[0]), int(pi[1]), int(pi[2])
    m = np.zeros((nk, nj, ni), dtype=bool)
    m[2:nk - 2, 2:nj - 2, 2:ni - 2] = True
    m = m.reshape(-1)
    assert np.all(coe[5, m] >= coe[4, m])
    assert np.any(coe[5, m] > coe[4, m])   # destruction-dominated cells exist near the wall
    r = c.residual_norms(0, 6)
    assert np.all(r[:6, -1] < r[:6, 0])
