"""Spalart-Allmaras diffusion against its linearised exact rate (oracle,
CPU): fluid at rest, no wall within reach (wall distance 1e8, so neither
production nor destruction acts), nutilde = nu_t0 (1 + 0.1 sin(2 pi x)) on a
periodic box, nu_t0 = 5 nu.  The SA equation's diffusion (1 / sigma)
div((nu + nutilde) grad nutilde) (SA/spsource_SA.for, the SA face
diffusion of AUSM/fluFaceSA.for) damps the perturbation at
(nu + nu_t0) k^2 / sigma to first order in its amplitude: measured within
0.5 % on 32 cells and 0.2 % on 64; the cb2 |grad nutilde|^2 / sigma term
raises the mean slightly (by about 1e-3 here)."""
import math

import numpy as np

from fast_gb300 import cases, fasts


def _sa_decay(oracle_mod, nx, ratio=5.0, mach=0.1, re=100.0, t_end=2.0, eps=0.1):
    gamma = 1.4
    h = 1.0 / nx
    z = cases.cart_zone("sa", (0.0, 0.0, 0.0), (h, h, h), (nx, 4, 4))
    xc, _, _ = cases.cell_centers(z)
    zero = np.zeros_like(xc)
    cases.set_conservative(z, np.ones_like(xc), zero, zero, zero, np.full_like(xc, 1.0 / gamma), gamma)
    nu = mach / re
    cases.set_spalart(z, ratio * nu * (1.0 + eps * np.sin(2 * math.pi * xc)), np.full_like(xc, 1.0e8))
    for f in ("imin", "imax", "jmin", "jmax", "kmin", "kmax"):
        cases.add_bc(z, "per_" + f, "BCautoperiod", f)
    nsteps = int(math.ceil(t_end / (0.4 * h)))
    t = cases._tree([z], "NSTurbulent",
                    {"temporal_scheme": "explicit", "rk": 3, "modulo_verif": 10 ** 6},
                    {"scheme": "ausmpred", "slope": "o3", "time_step": t_end / nsteps},
                    mach, re, gamma=gamma, prandtl=0.71, sutherland=False, nutilde_ratio=ratio)
    zd = fasts.zone_data(t, fasts.prepare(t))
    nu_lam = float(zd[0]["pr"][11])
    c = oracle_mod.Case(zd, ())
    c.apply_bc(0)
    c.apply_bc(1)
    pi = zd[0]["pi"]
    nip, njp, nd = int(pi[0]), int(pi[1]), int(pi[41])
    x = (np.arange(nx) + 0.5) * h

    def amplitude_mean():
        q = np.array(c.z[0]["lv"][0][:6 * nd]).reshape(6, -1, njp, nip)[5, 2:-2, 2:-2, 2:-2]
        return 2.0 * float(np.mean(q[0, 0, :] * np.sin(2 * math.pi * x))), float(np.mean(q))

    a0, m0 = amplitude_mean()
    for it in range(1, nsteps + 1):
        c.compute(it, 1, 3, 1, modulo_verif=10 ** 6)
    a1, m1 = amplitude_mean()
    rate = -math.log(a1 / a0) / t_end
    return rate / ((nu_lam + ratio * nu) * (2 * math.pi) ** 2 / (2.0 / 3.0)), m1 / m0


def test_sa_diffusion_rate(oracle_mod):
    r32, m32 = _sa_decay(oracle_mod, 32)
    r64, m64 = _sa_decay(oracle_mod, 64)
    assert abs(r32 - 1.0) < 5e-3, r32
    assert abs(r64 - 1.0) < 2e-3, r64
    assert 1.0 < m64 < 1.002, m64
