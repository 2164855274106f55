"""Shock capturing against the exact Riemann solution (oracle, CPU): Sod's
shock tube (density 1 / 0.125, pressure 1 / 0.1, at rest, diaphragm at
x = 0.5) on nx x 4 x 4 cells, extrapolation BCs at the x ends
(bvbs_extrapolate.for) and periodic in y and z, explicit RK3 at CFL 0.4 to
t = 0.2.  The density matches the exact solution (the exact Riemann solver
of Toro, Riemann Solvers and Numerical Methods for Fluid Dynamics, ch. 4,
restated below) with an L1 error that falls with the grid at the rate
discontinuities allow (about 0.85 with the minmod slope, 0.65 first order,
0.9 for AUSM+(P) with the unlimited o3 slope or with o3sc's shock sensor),
the Roe (with Harten's fix) and AUSM+(P) fluxes alike, and the solution is
exactly uniform across y and z.  Slip wall (bvbs_wall_inviscid.for): a
uniform flow at u = 0.5 into a wall at x = 1 reflects as a shock, the
symmetric Riemann problem (u, -u) with the wall as the contact; near the
wall the density matches it within 1.5 % (the usual start-up deficit of a
reflecting wall) and in L1 within 0.006 on 400 cells."""
import math

import numpy as np
import pytest

from fast_gb300 import cases, fasts


def exact_sod(x, t, x0=0.5, g=1.4, rl=1.0, ul=0.0, pl=1.0, rr=0.125, ur=0.0, pr=0.1):
    """Density of the exact solution of the Riemann problem at positions x,
    time t: the star pressure from Newton iterations on the pressure
    function, then the wave pattern sampled at x / t."""
    cl, cr = math.sqrt(g * pl / rl), math.sqrt(g * pr / rr)
    gm, gp = (g - 1) / (g + 1), (g + 1) / (2 * g)

    def side(p, rk, pk, ck):   # pressure function of one side and its derivative
        if p > pk:   # shock
            a, b = 2 / ((g + 1) * rk), gm * pk
            return (p - pk) * math.sqrt(a / (p + b)), math.sqrt(a / (b + p)) * (1 - (p - pk) / (2 * (b + p)))
        e = (g - 1) / (2 * g)   # rarefaction
        return 2 * ck / (g - 1) * ((p / pk) ** e - 1), (p / pk) ** (-gp) / (rk * ck)

    p = 0.5 * (pl + pr)
    for _ in range(50):
        fl, dl = side(p, rl, pl, cl)
        fr, dr = side(p, rr, pr, cr)
        dp = (fl + fr + ur - ul) / (dl + dr)
        p = max(p - dp, 1e-8)
        if abs(dp) < 1e-14:
            break
    fl, _ = side(p, rl, pl, cl)
    fr, _ = side(p, rr, pr, cr)
    u = 0.5 * (ul + ur) + 0.5 * (fr - fl)
    e = (g - 1) / (2 * g)
    out = np.empty_like(x)
    for i, xi in enumerate(x):
        s = (xi - x0) / t
        if s <= u:   # left of the contact
            if p > pl:
                sl = ul - cl * math.sqrt(gp * p / pl + e)
                out[i] = rl if s < sl else rl * (p / pl + gm) / (gm * p / pl + 1)
            elif s < ul - cl:
                out[i] = rl
            elif s > u - cl * (p / pl) ** e:
                out[i] = rl * (p / pl) ** (1 / g)
            else:
                out[i] = rl * (2 / (g + 1) + (g - 1) / ((g + 1) * cl) * (ul - s)) ** (2 / (g - 1))
        else:
            if p > pr:
                sr = ur + cr * math.sqrt(gp * p / pr + e)
                out[i] = rr if s > sr else rr * (p / pr + gm) / (gm * p / pr + 1)
            elif s > ur + cr:
                out[i] = rr
            elif s < u + cr * (p / pr) ** e:
                out[i] = rr * (p / pr) ** (1 / g)
            else:
                out[i] = rr * (2 / (g + 1) - (g - 1) / ((g + 1) * cr) * (ur - s)) ** (2 / (g - 1))
    return out


def sod_tree(nx, scheme, slope, t_end=0.2, two_d=False):
    """Sod's tube on nx x 4 x 4 cells (two_d: nx x 4 cells, a 2-d zone) and
    the number of RK3 steps to t_end."""
    g = 1.4
    h = 1.0 / nx
    z = cases.cart_zone("sod", (0.0, 0.0, 0.0), (h, h, h), (nx, 4, 1 if two_d else 4),
                        ngk=0 if two_d else None)
    xc, _, _ = cases.cell_centers(z)
    left = xc < 0.5
    ro = np.where(left, 1.0, 0.125)
    p = np.where(left, 1.0, 0.1)
    zero = np.zeros_like(ro)
    cases.set_conservative(z, ro, zero, zero, zero, p, g)
    cases.add_bc(z, "ex_imin", "BCExtrapolate", "imin")
    cases.add_bc(z, "ex_imax", "BCExtrapolate", "imax")
    for f in ("jmin", "jmax") + (() if two_d else ("kmin", "kmax")):
        cases.add_bc(z, "per_" + f, "BCautoperiod", f)
    nsteps = int(math.ceil(t_end / (0.4 * h / (math.sqrt(g) + 1.0))))
    t = cases._tree([z], "Euler", {"temporal_scheme": "explicit", "rk": 3, "modulo_verif": 10 ** 6},
                    {"scheme": scheme, "slope": slope, "time_step": t_end / nsteps}, 0.5, 0.0, gamma=g)
    return t, nsteps


def _sod_density(oracle_mod, nx, scheme, slope, t_end=0.2, two_d=False):
    t, nsteps = sod_tree(nx, scheme, slope, t_end, two_d)
    zd = fasts.zone_data(t, fasts.prepare(t))
    assert int(zd[0]["pi"][25]) == (3 if two_d else 2)   # 2-d / 3-d cartesian zone
    c = oracle_mod.Case(zd, ())
    c.apply_bc(0)
    c.apply_bc(1)
    for it in range(1, nsteps + 1):
        c.compute(it, 1, 3, 1, modulo_verif=10 ** 6)
    pi = zd[0]["pi"]
    nip, njp, nd, ngk = int(pi[0]), int(pi[1]), int(pi[41]), int(pi[4])
    q = np.array(c.z[0]["lv"][0][:nd]).reshape(-1, njp, nip)
    return q[ngk:q.shape[0] - ngk, 2:-2, 2:-2]


def _sod_l1(oracle_mod, nx, scheme, slope, t_end=0.2):
    h = 1.0 / nx
    t, nsteps = sod_tree(nx, scheme, slope, t_end)
    zd = fasts.zone_data(t, fasts.prepare(t))
    c = oracle_mod.Case(zd, ())
    c.apply_bc(0)
    c.apply_bc(1)
    for it in range(1, nsteps + 1):
        c.compute(it, 1, 3, 1, modulo_verif=10 ** 6)
    pi = zd[0]["pi"]
    nip, njp, nd = int(pi[0]), int(pi[1]), int(pi[41])
    q = np.array(c.z[0]["lv"][0][:nd]).reshape(-1, njp, nip)[2:-2, 2:-2, 2:-2]
    assert np.array_equal(q, np.broadcast_to(q[0:1, 0:1, :], q.shape))   # uniform in y, z
    x = (np.arange(nx) + 0.5) * h
    return float(np.mean(np.abs(q[0, 0, :] - exact_sod(x, t_end))))


def test_sod_in_a_2d_zone(oracle_mod):
    """The same tube as a 2-d zone (ITYPZONE 3: one cell in k, no k ghosts;
    the *_2d_*.for fluxes) gives the 3-d cartesian zone's solution to
    round-off (3.7e-15 measured) and so the same match with the exact one."""
    q2 = _sod_density(oracle_mod, 200, "roe", "minmod", two_d=True)
    q3 = _sod_density(oracle_mod, 200, "roe", "minmod")
    assert np.max(np.abs(q2[0, 0, :] - q3[0, 0, :])) < 1e-13
    x = (np.arange(200) + 0.5) / 200
    assert float(np.mean(np.abs(q2[0, 0, :] - exact_sod(x, 0.2)))) < 0.0055


@pytest.mark.parametrize("scheme,slope,bound,rate", [("roe", "minmod", 0.0055, 0.7),
                                                     ("ausmpred", "minmod", 0.0045, 0.7),
                                                     ("ausmpred", "o3", 0.0035, 0.8),
                                                     ("ausmpred", "o3sc", 0.0037, 0.8),
                                                     ("roe", "o1", 0.015, 0.5)])
def test_sod_shock_tube(oracle_mod, scheme, slope, bound, rate):
    e200 = _sod_l1(oracle_mod, 200, scheme, slope)
    e400 = _sod_l1(oracle_mod, 400, scheme, slope)
    assert e200 < bound, e200
    assert math.log2(e200 / e400) > rate, (e200, e400)


def _wall_reflection(oracle_mod, nx, scheme, t_end=0.3, u0=0.5):
    g = 1.4
    h = 1.0 / nx
    z = cases.cart_zone("wall", (0.0, 0.0, 0.0), (h, h, h), (nx, 4, 4))
    xc, _, _ = cases.cell_centers(z)
    zero = np.zeros_like(xc)
    cases.set_conservative(z, np.ones_like(xc), np.full_like(xc, u0), zero, zero,
                           np.full_like(xc, 1.0 / g), g)
    cases.add_bc(z, "ex_imin", "BCExtrapolate", "imin")
    cases.add_bc(z, "wall_imax", "BCWallInviscid", "imax")
    for f in ("jmin", "jmax", "kmin", "kmax"):
        cases.add_bc(z, "per_" + f, "BCautoperiod", f)
    nsteps = int(math.ceil(t_end / (0.4 * h / 2.0)))
    t = cases._tree([z], "Euler", {"temporal_scheme": "explicit", "rk": 3, "modulo_verif": 10 ** 6},
                    {"scheme": scheme, "slope": "minmod", "time_step": t_end / nsteps}, 0.5, 0.0, gamma=g)
    zd = fasts.zone_data(t, fasts.prepare(t))
    c = oracle_mod.Case(zd, ())
    c.apply_bc(0)
    c.apply_bc(1)
    for it in range(1, nsteps + 1):
        c.compute(it, 1, 3, 1, modulo_verif=10 ** 6)
    pi = zd[0]["pi"]
    nip, njp, nd = int(pi[0]), int(pi[1]), int(pi[41])
    ro = np.array(c.z[0]["lv"][0][:nd]).reshape(-1, njp, nip)[2:-2, 2:-2, 2:-2][0, 0, :]
    x = (np.arange(nx) + 0.5) * h
    ex = exact_sod(x, t_end, x0=1.0, rl=1.0, ul=u0, pl=1.0 / g, rr=1.0, ur=-u0, pr=1.0 / g)
    near = x > 0.7   # away from the left boundary's disturbance
    return float(np.mean(np.abs(ro[near] - ex[near]))), float(ro[-1] / ex[-1])


@pytest.mark.parametrize("scheme", ["roe", "ausmpred"])
def test_slip_wall_shock_reflection(oracle_mod, scheme):
    l1, wall = _wall_reflection(oracle_mod, 400, scheme)
    assert l1 < 0.006, l1
    assert abs(wall - 1.0) < 0.015, wall
