"""Farfield boundaries let waves out (oracle, CPU): a small right-going
acoustic pulse (a linear simple wave: dp = rho c du, drho = dp / c^2) on a
Mach 0.5 free stream leaves a tube with farfield BCs at both ends
(bvbs_farfield.for, characteristic states against the reference state);
after it has crossed the boundary, less than 0.2 % of its amplitude remains
in the tube (0.04-0.05 % measured), while extrapolation BCs at the same ends
keep over 1 % (their inflow end is not non-reflecting)."""
import math

import numpy as np
import pytest

from fast_gb300 import cases, fasts


def _left_over(oracle_mod, nx, bc, mach=0.5, t_end=0.6, amp=1e-3):
    gamma = 1.4
    h = 1.0 / nx
    z = cases.cart_zone("pulse", (0.0, 0.0, 0.0), (h, h, h), (nx, 4, 4))
    xc, _, _ = cases.cell_centers(z)
    bump = amp * np.exp(-((xc - 0.5) / 0.05) ** 2)   # T = 1, R = 1 / gamma: c = 1
    zero = np.zeros_like(xc)
    cases.set_conservative(z, 1.0 + bump, mach + bump, zero, zero, (1.0 + gamma * bump) / gamma, gamma)
    cases.add_bc(z, "b_imin", bc, "imin")
    cases.add_bc(z, "b_imax", bc, "imax")
    for f in ("jmin", "jmax", "kmin", "kmax"):
        cases.add_bc(z, "per_" + f, "BCautoperiod", f)
    nsteps = int(math.ceil(t_end / (0.4 * h / (1.0 + mach))))
    t = cases._tree([z], "Euler", {"temporal_scheme": "explicit", "rk": 3, "modulo_verif": 10 ** 6},
                    {"scheme": "ausmpred", "slope": "o3", "time_step": t_end / nsteps}, mach, 0.0,
                    gamma=gamma)
    zd = fasts.zone_data(t, fasts.prepare(t))
    c = oracle_mod.Case(zd, ())
    c.apply_bc(0)
    c.apply_bc(1)
    pi = zd[0]["pi"]
    nip, njp, nd = int(pi[0]), int(pi[1]), int(pi[41])

    def deviation():
        ro = np.array(c.z[0]["lv"][0][:nd]).reshape(-1, njp, nip)[2:-2, 2:-2, 2:-2]
        return float(np.max(np.abs(ro - 1.0)))

    d0 = deviation()
    for it in range(1, nsteps + 1):
        c.compute(it, 1, 3, 1, modulo_verif=10 ** 6)
    return deviation() / d0


def test_farfield_lets_an_acoustic_pulse_out(oracle_mod):
    assert _left_over(oracle_mod, 100, "BCFarfield") < 2e-3
    assert _left_over(oracle_mod, 100, "BCExtrapolate") > 1e-2


def test_duct_relaxes_to_the_free_stream(oracle_mod):
    """Inflow at imin (bvbs_inflow.for), outflow at imax (bvbs_outflow.for), a
    slip wall at jmin and farfield at jmax, periodic in k: a 5 % smooth
    perturbation of the free stream is carried out of the box and the state
    relaxes to the reference state itself, geometrically (5e-9 after 1500 RK3
    steps, 1e-14 after 3000)."""
    t = cases.bc_box(n=(24, 12, 4), wall="BCWallInviscid", model="Euler", perturb=0.05,
                     temporal="explicit", time_step=0.01)
    zd = fasts.zone_data(t, fasts.prepare(t))
    c = oracle_mod.Case(zd, ())
    c.apply_bc(0)
    c.apply_bc(1)
    pi, pr = zd[0]["pi"], zd[0]["pr"]
    nip, njp, nd = int(pi[0]), int(pi[1]), int(pi[41])
    free = np.array([pr[3], pr[19], pr[20], pr[21], pr[6]])   # ro, u, v, w, T of the reference state
    dev = []
    for it in range(1, 1501):
        c.compute(it, 1, 3, 1, modulo_verif=10 ** 6)
        if it % 500 == 0:
            q = np.array(c.z[0]["lv"][0][:5 * nd]).reshape(5, -1, njp, nip)[:, 2:-2, 2:-2, 2:-2]
            dev.append(float(np.max(np.abs(q - free[:, None, None, None]))))
    assert dev[0] > dev[1] > dev[2]
    assert dev[2] < 1e-7, dev


@pytest.mark.parametrize("nature", ["global", "local"])
def test_implicit_duct_relaxes_to_the_free_stream(oracle_mod, nature):
    """The same duct with implicit dual time stepping (BDF2, LU-SGS,
    ss_iteration 3, acoustic CFL about 1.6) and with the local time step
    (time_step_nature 'local', CFL 10: tstb3_impli.for, BDF1) relaxes to the
    reference state too: below 1e-4 after 200 steps (global) and 1e-7 after
    300 (local)."""
    from fast_gb300 import fastc
    from fast_gb300 import pytree as I
    t = cases.bc_box(n=(24, 12, 4), wall="BCWallInviscid", model="Euler", perturb=0.05,
                     temporal="implicit", ss_iteration=3, time_step=0.05)
    if nature == "local":
        for z in I.getZones(t):
            fastc._setNum2Zones(z, {"time_step_nature": "local", "cfl": 10.0})
    zd = fasts.zone_data(t, fasts.prepare(t))
    c = oracle_mod.Case(zd, ())
    c.apply_bc(0)
    c.apply_bc(1)
    pi, pr = zd[0]["pi"], zd[0]["pr"]
    nip, njp, nd, nss = int(pi[0]), int(pi[1]), int(pi[41]), int(pi[58])
    assert int(pi[46]) == (1 if nature == "local" else 0)
    free = np.array([pr[3], pr[19], pr[20], pr[21], pr[6]])
    nsteps, bound = (200, 1e-4) if nature == "global" else (300, 1e-7)
    for it in range(1, nsteps + 1):
        c.compute(it, 1, nss, 1, modulo_verif=10 ** 6)
    q = np.array(c.z[0]["lv"][0][:5 * nd]).reshape(5, -1, njp, nip)[:, 2:-2, 2:-2, 2:-2]
    assert float(np.max(np.abs(q - free[:, None, None, None]))) < bound
