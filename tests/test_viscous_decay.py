"""Viscous flux against an exact Navier-Stokes solution (oracle, CPU): the
2-d Taylor-Green vortex u = U sin x cos y, v = -U cos x sin y (pressure
U^2/4 (cos 2x + cos 2y) above the mean, T = 1, periodic box [0, 2 pi]^2,
4 cells in z) decays as exp(-2 nu t), so its kinetic energy as exp(-4 nu t).
Laminar AUSM+(P) o3 (fluvisq_3dcart_*.for, mu constant: Sutherland off),
explicit RK3, Mach 0.1, Re 100 (nu = 1e-3), to t = 20: the measured decay
rate is 4 nu within 3 % on 32 x 32 cells and 0.5 % on 64 x 64, and it
converges from above (the scheme's own dissipation vanishes with h).  On a
curvilinear (wavy, general 3-d) mesh of the same box, fluvisq_3dfull_*.for
with the full metric: within 6 % on 32 x 32 and 3 % on 64 x 64, converging.
No-slip walls (bvbs_wall_viscous_adia.for): a shear wave u = U sin(pi y)
between adiabatic walls at y = 0 and 1 decays as exp(-nu pi^2 t), its
kinetic energy as exp(-2 nu pi^2 t) (Mach 0.1, Re 50, to t = 10): the
measured rate is within 0.5 % of it on 16 cells across and 0.15 % on 32,
converging at second order."""
import math

import numpy as np

from fast_gb300 import cases, fasts


def _decay_rate(oracle_mod, n, mach=0.1, re=100.0, t_end=20.0, wavy=0.0):
    gamma = 1.4
    h = 2 * math.pi / n
    z = cases.cart_zone("tgv2d", (0.0, 0.0, 0.0), (h, h, h), (n, n, 4))
    if wavy:
        cases.wave(z, wavy, (0.0, 0.0, 0.0), (2 * math.pi, 2 * math.pi, 4 * h))
    xc, yc, _ = cases.cell_centers(z)
    u = mach * np.sin(xc) * np.cos(yc)
    v = -mach * np.cos(xc) * np.sin(yc)
    p = 1.0 / gamma + mach * mach / 4.0 * (np.cos(2 * xc) + np.cos(2 * yc))
    cases.set_conservative(z, p * gamma, u, v, np.zeros_like(u), p, gamma)
    for f in ("imin", "imax", "jmin", "jmax", "kmin", "kmax"):
        cases.add_bc(z, "per_" + f, "BCautoperiod", f)
    nsteps = int(math.ceil(t_end / ((0.3 if wavy else 0.4) * h / (mach + 1.0))))
    t = cases._tree([z], "NSLaminar",
                    {"temporal_scheme": "explicit", "rk": 3, "modulo_verif": 10 ** 6},
                    {"scheme": "ausmpred", "slope": "o3", "time_step": t_end / nsteps},
                    mach, re, gamma=gamma, prandtl=0.71, sutherland=False)
    zd = fasts.zone_data(t, fasts.prepare(t))
    assert int(zd[0]["pi"][25]) == (0 if wavy else 2)   # general / cartesian zone
    nu = float(zd[0]["pr"][11])          # mu / ro, ro = 1
    c = oracle_mod.Case(zd, ())
    c.apply_bc(0)
    c.apply_bc(1)
    pi = zd[0]["pi"]
    nip, njp, nd = int(pi[0]), int(pi[1]), int(pi[41])

    def kinetic():
        q = np.array(c.z[0]["lv"][0][:5 * nd]).reshape(5, -1, njp, nip)[:, 2:-2, 2:-2, 2:-2]
        return float(np.sum(0.5 * q[0] * (q[1] ** 2 + q[2] ** 2)))

    k0 = kinetic()
    for it in range(1, nsteps + 1):
        c.compute(it, 1, 3, 1, modulo_verif=10 ** 6)
    return -math.log(kinetic() / k0) / t_end / (4 * nu)


def test_taylor_green_2d_decay_rate(oracle_mod):
    r32 = _decay_rate(oracle_mod, 32)
    r64 = _decay_rate(oracle_mod, 64)
    assert abs(r32 - 1.0) < 0.03, r32
    assert abs(r64 - 1.0) < 0.005, r64
    assert r32 > r64


def shear_tree(ny, mach=0.1, re=50.0, t_end=10.0):
    """The shear wave between no-slip walls on 4 x ny x 4 cells and the
    number of RK3 steps to t_end."""
    gamma = 1.4
    h = 1.0 / ny
    z = cases.cart_zone("shear", (0.0, 0.0, 0.0), (h, h, h), (4, ny, 4))
    _, yc, _ = cases.cell_centers(z)
    u = mach * np.sin(math.pi * yc)
    zero = np.zeros_like(u)
    cases.set_conservative(z, np.ones_like(u), u, zero, zero, np.full_like(u, 1.0 / gamma), gamma)
    for f in ("imin", "imax", "kmin", "kmax"):
        cases.add_bc(z, "per_" + f, "BCautoperiod", f)
    cases.add_bc(z, "wall_jmin", "BCWallViscous", "jmin")
    cases.add_bc(z, "wall_jmax", "BCWallViscous", "jmax")
    nsteps = int(math.ceil(t_end / (0.4 * h / (mach + 1.0))))
    t = cases._tree([z], "NSLaminar",
                    {"temporal_scheme": "explicit", "rk": 3, "modulo_verif": 10 ** 6},
                    {"scheme": "ausmpred", "slope": "o3", "time_step": t_end / nsteps},
                    mach, re, gamma=gamma, prandtl=0.71, sutherland=False)
    return t, nsteps


def _shear_decay_rate(oracle_mod, ny, mach=0.1, re=50.0, t_end=10.0):
    t, nsteps = shear_tree(ny, mach, re, t_end)
    zd = fasts.zone_data(t, fasts.prepare(t))
    nu = float(zd[0]["pr"][11])
    c = oracle_mod.Case(zd, ())
    c.apply_bc(0)
    c.apply_bc(1)
    pi = zd[0]["pi"]
    nip, njp, nd = int(pi[0]), int(pi[1]), int(pi[41])

    def kinetic():
        q = np.array(c.z[0]["lv"][0][:5 * nd]).reshape(5, -1, njp, nip)[:, 2:-2, 2:-2, 2:-2]
        return float(np.sum(0.5 * q[0] * (q[1] ** 2 + q[2] ** 2)))

    k0 = kinetic()
    for it in range(1, nsteps + 1):
        c.compute(it, 1, 3, 1, modulo_verif=10 ** 6)
    return -math.log(kinetic() / k0) / t_end / (2 * nu * math.pi ** 2)


def test_shear_wave_between_no_slip_walls(oracle_mod):
    r16 = _shear_decay_rate(oracle_mod, 16)
    r32 = _shear_decay_rate(oracle_mod, 32)
    assert abs(r16 - 1.0) < 5e-3, r16
    assert abs(r32 - 1.0) < 1.5e-3, r32
    assert abs(r16 - 1.0) > 3.0 * abs(r32 - 1.0)


def test_taylor_green_2d_decay_rate_curvilinear(oracle_mod):
    r32 = _decay_rate(oracle_mod, 32, wavy=0.3)
    r64 = _decay_rate(oracle_mod, 64, wavy=0.3)
    assert abs(r32 - 1.0) < 0.07, r32
    assert abs(r64 - 1.0) < 0.035, r64
    assert abs(r32 - 1.0) > 1.7 * abs(r64 - 1.0)
