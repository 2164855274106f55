"""CPU tests of the oracle: known-answer and invariant checks that pin the
restatement where the reference ships no expected values (no GPU needed)."""
import numpy as np
import pytest

from conftest import rel_err
from fast_gb300 import cases, fasts


def _case(t, oracle_mod):
    m = fasts.prepare(t)
    zd = fasts.zone_data(t, m)
    c = oracle_mod.Case(zd)
    c.apply_bc(0)
    c.apply_bc(1)
    return zd, c


def _cons(pi, pr, q):
    nd = int(pi[41])
    q = q.reshape(5, nd)
    ro, u, v, w, T = q
    cv = pr[2]
    return np.stack([ro, ro * u, ro * v, ro * w, ro * (cv * T + 0.5 * (u * u + v * v + w * w))])


def _interior(pi, a):
    ni, nj, nk = (int(pi[0]), int(pi[1]), int(pi[2]))
    ng, ngk = int(pi[3]), int(pi[4])
    a = a.reshape(-1, nk, nj, ni)
    return a[:, ngk:nk - ngk, ng:nj - ng, ng:ni - ng]


@pytest.mark.parametrize("scheme,slope", [("roe", "o1"), ("roe_min", "minmod"), ("roe", "o3"),
                                          ("senseur", "o3")])
def test_free_stream_preservation_explicit(oracle_mod, scheme, slope):
    t = cases.isentropic_vortex(n=(12, 10, 6), beta=0.0,
                                numz={"scheme": scheme, "slope": slope, "time_step": 0.05})
    zd, c = _case(t, oracle_mod)
    q0 = c.z[0]["lv"][0].copy()
    for it in range(1, 4):
        c.compute(it, 1, 3, 1, modulo_verif=1000)
    assert np.max(np.abs(c.z[0]["lv"][0] - q0)) < 1e-14


@pytest.mark.parametrize("scheme,slope", [("ausmpred", "o3"), ("roe_min", "minmod")])
def test_free_stream_preservation_implicit(oracle_mod, scheme, slope):
    t = cases.isentropic_vortex(n=(8, 8, 8), beta=0.0,
                                numb={"temporal_scheme": "implicit", "ss_iteration": 3,
                                      "modulo_verif": 1},
                                numz={"scheme": scheme, "slope": slope, "time_step": 0.05})
    zd, c = _case(t, oracle_mod)
    q0 = c.z[0]["lv"][0].copy()
    c.compute(1, 1, 4, 1, modulo_verif=1)
    # zero velocity components may pick up round-off: compare on the scale 1
    assert np.max(np.abs(c.z[0]["lv"][0] - q0)) < 1e-13


@pytest.mark.parametrize("scheme,slope", [("roe_min", "minmod"), ("ausmpred", "o3"),
                                          ("senseur", "o3")])
def test_conservation_periodic(oracle_mod, scheme, slope):
    """Sum over a periodic box of V*(W^{n+1}-W^n) in conservative variables
    vanishes: every face flux enters two cells with opposite signs."""
    t = cases.isentropic_vortex(n=(16, 16, 4), numz={"scheme": scheme, "slope": slope,
                                                      "time_step": 0.05})
    zd, c = _case(t, oracle_mod)
    pi, pr = zd[0]["pi"], zd[0]["pr"]
    w0 = _interior(pi, _cons(pi, pr, c.z[0]["lv"][0])).sum(axis=(1, 2, 3))
    c.compute(1, 1, 3, 1, modulo_verif=1000)
    w1 = _interior(pi, _cons(pi, pr, c.z[0]["lv"][0])).sum(axis=(1, 2, 3))
    scale = np.abs(_interior(pi, _cons(pi, pr, c.z[0]["lv"][0]))).sum(axis=(1, 2, 3))
    assert np.all(np.abs(w1 - w0) <= 1e-13 * scale)


def test_vortex_advects(oracle_mod):
    """The isentropic vortex translates with the free stream: after 20 steps
    the density minimum has moved by about U dt n."""
    t = cases.isentropic_vortex(n=(40, 40, 4), numz={"scheme": "roe_min", "slope": "minmod",
                                                      "time_step": 0.05})
    zd, c = _case(t, oracle_mod)
    pi = zd[0]["pi"]
    ro0 = _interior(pi, c.z[0]["lv"][0])[0, 2]
    for it in range(1, 21):
        c.compute(it, 1, 3, 1, modulo_verif=1000)
    ro1 = _interior(pi, c.z[0]["lv"][0])[0, 2]
    i0 = np.unravel_index(np.argmin(ro0), ro0.shape)[1]
    i1 = np.unravel_index(np.argmin(ro1), ro1.shape)[1]
    dx = 20.0 / 40
    assert abs((i1 - i0) * dx - 0.5 * 0.05 * 20) <= dx


def test_threads_do_not_change_bits(oracle_mod):
    t1 = cases.taylor_green(n=(12, 10, 8), ss_iteration=2)
    t2 = cases.taylor_green(n=(12, 10, 8), ss_iteration=2)
    _, c1 = _case(t1, oracle_mod)
    _, c2 = _case(t2, oracle_mod)
    oracle_mod.set_threads(1)
    c1.compute(1, 1, 3, 1, modulo_verif=1)
    oracle_mod.set_threads(4)
    c2.compute(1, 1, 3, 1, modulo_verif=1)
    oracle_mod.set_threads(1)
    for a, b in zip(c1.z[0]["lv"], c2.z[0]["lv"]):
        assert np.array_equal(a, b)


def test_implicit_newton_residual_decreases(oracle_mod):
    """Dual-time sub-iterations contract the Newton residual (L2 of the last
    sub-iteration below the first)."""
    t = cases.taylor_green(n=(16, 16, 16), ss_iteration=6)
    zd, c = _case(t, oracle_mod)
    c.compute(1, 1, 7, 1, modulo_verif=1)
    r = c.residual_norms(0, 7)
    assert np.all(r[:5, -1] < r[:5, 0])


def test_periodic_ghosts_and_corners(oracle_mod):
    t = cases.taylor_green(n=(8, 6, 5), ss_iteration=2)
    zd, c = _case(t, oracle_mod)
    pi = zd[0]["pi"]
    ni, nj, nk = (int(pi[0]), int(pi[1]), int(pi[2]))
    q = c.z[0]["lv"][0].reshape(5, nk, nj, ni)
    # i-ghosts are periodic copies
    assert np.array_equal(q[:, 2:-2, 2:-2, 0:2], q[:, 2:-2, 2:-2, ni - 4:ni - 2])
    assert np.array_equal(q[:, 2:-2, 2:-2, ni - 2:], q[:, 2:-2, 2:-2, 2:4])
    # edge (i ghost, j ghost) = mean of the adjacent face ghosts (correct_coins.for)
    e = q[:, 3, 1, 1]
    a = q[:, 3, 2, 0]   # i0 + i1*is with i=1 -> i1=2: i index 2-2 = 0
    b = q[:, 3, 0, 2]
    assert np.array_equal(e, (a + b) * 0.5)


def test_free_stream_with_characteristic_bcs(oracle_mod):
    """The free stream is a solution with inflow, outflow, farfield and a
    slip wall aligned with it: the characteristic BCs (non_reflection.for)
    rebuild the free stream in the ghost cells."""
    t = cases.bc_box(n=(12, 10, 6), perturb=0.0, wall="BCWallInviscid", model="Euler")
    zd, c = _case(t, oracle_mod)
    q0 = c.z[0]["lv"][0].copy()
    for it in range(1, 4):
        c.compute(it, 1, 3, 1, modulo_verif=1000)
    assert np.max(np.abs(c.z[0]["lv"][0] - q0)) < 1e-14


def test_wall_ghosts(oracle_mod):
    """Slip wall: mirror state with the normal velocity reversed; no-slip
    adiabatic wall: mirror state with the velocity reversed."""
    for wall, model, flip in (("BCWallInviscid", "Euler", (1, -1, 1)),
                              ("BCWallViscous", "NSLaminar", (-1, -1, -1))):
        t = cases.bc_box(n=(8, 6, 4), wall=wall, model=model)
        zd, c = _case(t, oracle_mod)
        pi = zd[0]["pi"]
        ni, nj, nk = (int(pi[0]), int(pi[1]), int(pi[2]))
        q = c.z[0]["lv"][0].reshape(5, nk, nj, ni)
        for g, m in ((1, 2), (0, 3)):          # ghost j index -> mirror j index
            for v, sgn in zip((1, 2, 3), flip):
                a = q[v, 2:nk - 2, g, 2:ni - 2]
                b = q[v, 2:nk - 2, m, 2:ni - 2]
                assert np.array_equal(a, sgn * b)
            for v in (0, 4):
                assert np.array_equal(q[v, 2:nk - 2, g, 2:ni - 2], q[v, 2:nk - 2, m, 2:ni - 2])


def test_roe_slip_wall_keeps_parallel_free_stream(oracle_mod):
    """With the Roe wall-face correction (correct_flux.for) a free stream
    parallel to a slip wall stays the free stream."""
    t = cases.bc_box(n=(12, 10, 6), perturb=0.0, wall="BCWallInviscid", model="Euler",
                     scheme="roe", slope="o3")
    zd, c = _case(t, oracle_mod)
    q0 = c.z[0]["lv"][0].copy()
    for it in range(1, 4):
        c.compute(it, 1, 3, 1, modulo_verif=1000)
    assert np.max(np.abs(c.z[0]["lv"][0] - q0)) < 1e-14


@pytest.mark.parametrize("model", ["Euler", "NSLaminar"])
def test_cfl_statistics_uniform_flow(oracle_mod, model):
    """cpcfl3.for on a uniform flow in a cartesian box: every cell has the
    same CFL dt (|u| + c) / (2 vol surf) (Euler) or dt / min(vis, conv), so
    max = min = mean = the closed form."""
    import math
    from fast_gb300 import cases, fasts
    t = cases.bc_box(n=(12, 10, 6), model=model, wall="BCWallInviscid" if model == "Euler" else "BCWallViscous",
                     perturb=0.0, temporal="explicit", reynolds=50.0, time_step=0.01)
    zd = fasts.zone_data(t, fasts.prepare(t))
    c = oracle_mod.Case(zd)
    c.apply_bc(0)
    c.apply_bc(1)
    c.compute(1, 1, 3, 1, modulo_verif=1)
    cmax, cmin, cmean = c.cfl(0)
    pr = zd[0]["pr"]
    gam, cv, dt = pr[1], pr[2], pr[0]
    hx, hy, hz = 1 / 12, 1 / 10, 1 / 12
    vol = hx * hy * hz
    surf = 1.0 / (2 * max(hy * hz, hx * hz, hx * hy))
    q = zd[0]["ro"].reshape(5, -1)[:, 0]
    snd = math.sqrt(gam * cv * (gam - 1) * q[4])
    conv = 2 * vol * surf / (math.sqrt(q[1] ** 2 + q[2] ** 2 + q[3] ** 2) + snd)
    comp = conv
    if model != "Euler":
        nip, njp = 12 + 4, 10 + 4
        mu = c.z[0]["xmut"][2 + 2 * nip + 2 * nip * njp]     # first interior cell
        assert mu > 0
        vis = 2 * q[0] * vol * vol * surf * surf * (gam / pr[10]) / mu
        comp = min(vis, conv)
    exp = dt / comp
    assert abs(cmax - exp) <= 1e-13 * exp and abs(cmin - exp) <= 1e-13 * exp
    assert abs(cmean - exp) <= 1e-12 * exp
