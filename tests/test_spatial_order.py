"""Spatial accuracy of the reconstructions (oracle, CPU): an entropy wave
(density 1 + 0.1 sin(2 pi x), uniform velocity and pressure) advected on
periodic boxes of nx = 16, 32, 64 cells in x (4 in y and z) with explicit RK3
at a small, fixed CFL (halving it changes no digit shown: the time error is
negligible), against the translated exact wave.  FastS stores and
reconstructs point values of the primitive variables, so the update is of
second order in the limit: the o1 slope gives first order
(Slope/o1_slope_var.for), the o3 slope (o3_slope_var.for, with the Roe and
AUSM+(P) fluxes) third order on the coarse pair of grids, tending to two,
and the o5 slope (o5_slope_var.for, AUSM+(P)) second order with a coarse-
grid error five times below o3's."""
import math

import numpy as np
import pytest

from fast_gb300 import cases, fasts


def _wave_error(oracle_mod, nx, scheme, slope, cfl=0.02, t_end=0.25):
    gamma, mach = 1.4, 0.5
    L = 1.0
    ng = 3 if slope in ("o5", "o5sc") else 2
    h = L / nx
    z = cases.cart_zone("wave", (0.0, 0.0, 0.0), (h, h, h), (nx, 4, 4), ng=ng)
    xc, _, _ = cases.cell_centers(z)
    ro = 1.0 + 0.1 * np.sin(2 * math.pi * xc / L)
    u = np.full_like(ro, mach)
    p = np.full_like(ro, 1.0 / gamma)
    cases.set_conservative(z, ro, u, np.zeros_like(ro), np.zeros_like(ro), p, gamma)
    for f in ("imin", "imax", "jmin", "jmax", "kmin", "kmax"):
        cases.add_bc(z, "per_" + f, "BCautoperiod", f, ng=ng)
    c_max = mach + math.sqrt(gamma * (1.0 / gamma) / 0.9)   # |u| + c, lowest density
    nsteps = int(math.ceil(t_end / (cfl * h / c_max)))
    dt = t_end / nsteps
    numb = {"temporal_scheme": "explicit", "rk": 3, "modulo_verif": 1000000}
    numz = {"scheme": scheme, "slope": slope, "time_step": dt}
    t = cases._tree([z], "Euler", numb, numz, mach, 0.0, gamma=gamma)
    zd = fasts.zone_data(t, fasts.prepare(t))
    c = oracle_mod.Case(zd, ())
    c.apply_bc(0)
    c.apply_bc(1)
    for it in range(1, nsteps + 1):
        c.compute(it, 1, 3, 1, modulo_verif=1000000)
    pi = zd[0]["pi"]
    nip, njp = int(pi[0]), int(pi[1])
    q = np.array(c.z[0]["lv"][0][:int(pi[41])]).reshape(-1, njp, nip)[ng:-ng, ng:-ng, ng:-ng]
    xi = (np.arange(nx) + 0.5) * h
    exact = 1.0 + 0.1 * np.sin(2 * math.pi * (xi - mach * t_end) / L)
    return float(np.max(np.abs(q - exact[None, None, :])))


def _orders(e):
    return math.log2(e[0] / e[1]), math.log2(e[1] / e[2])


def test_o1_is_first_order(oracle_mod):
    p1, p2 = _orders([_wave_error(oracle_mod, nx, "roe", "o1") for nx in (16, 32, 64)])
    assert 0.85 <= p1 <= 1.15 and 0.85 <= p2 <= 1.15, (p1, p2)


@pytest.mark.parametrize("scheme", ["roe", "ausmpred"])
def test_o3_is_third_order_on_coarse_grids(oracle_mod, scheme):
    p1, p2 = _orders([_wave_error(oracle_mod, nx, scheme, "o3") for nx in (16, 32, 64)])
    assert 2.7 <= p1 <= 3.3 and p2 >= 2.3, (p1, p2)


def test_o5_error_below_o3(oracle_mod):
    e5 = [_wave_error(oracle_mod, nx, "ausmpred", "o5") for nx in (16, 32, 64)]
    e3 = _wave_error(oracle_mod, 16, "ausmpred", "o3")
    p1, p2 = _orders(e5)
    assert e5[0] < 0.25 * e3 and p1 >= 1.6 and p2 >= 1.8, (e5, e3, p1, p2)


def test_o3sc_is_o3_on_smooth_flow(oracle_mod):
    """o3sc (o3_slope_var.for weighted by the shock sensor, sciacovelli.for)
    keeps the o3 slope where the flow is smooth: the same error as o3 to
    5e-5 relative, 1e-8 on the finest grid."""
    for nx, tol in ((16, 1e-4), (32, 1e-4), (64, 1e-6)):
        e3 = _wave_error(oracle_mod, nx, "ausmpred", "o3")
        esc = _wave_error(oracle_mod, nx, "ausmpred", "o3sc")
        assert abs(esc - e3) < tol * e3, (nx, e3, esc)


def test_minmod_and_senseur(oracle_mod):
    """The minmod slope clips the wave's extrema: between first and second
    order (1.2 measured); the senseur scheme (SENSOR/fluFaceEuler.for, o3,
    its dissipation switched off by the wiggle sensor on smooth data) is
    second order with an error seven times below AUSM+(P) o3's on 16 cells."""
    p1, p2 = _orders([_wave_error(oracle_mod, nx, "roe", "minmod") for nx in (16, 32, 64)])
    assert 1.0 <= p1 <= 1.5 and 1.0 <= p2 <= 1.5, (p1, p2)
    es = [_wave_error(oracle_mod, nx, "senseur", "o3") for nx in (16, 32, 64)]
    assert es[0] < 0.2 * _wave_error(oracle_mod, 16, "ausmpred", "o3")
    assert _orders(es)[1] >= 1.7, es
