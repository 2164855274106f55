"""Temporal order of the time schemes (oracle, CPU): the isentropic vortex
on a fixed 24 x 24 x 4 periodic grid (Roe, o3 slope) advanced to the same
time with two time steps; against a reference run with a step eight times
smaller, the error falls by about 2^p when the step is halved: p = 1, 2, 3
for the explicit RK1, RK2, RK3 (core3ark3.for / init_rhs.for stage
coefficients) and p = 2 for the implicit dual-time BDF2 (core3as2.for; BDF1
first step; 30 LU-SGS sub-iterations, converged).  The spatial error is the
same in every run and cancels."""
import math

import numpy as np
import pytest

from fast_gb300 import cases, fasts


def _final_density(oracle_mod, rk, dt, t_end, implicit=False):
    numb = ({"temporal_scheme": "implicit", "ss_iteration": 30, "modulo_verif": 1000} if implicit
            else {"temporal_scheme": "explicit", "rk": rk, "modulo_verif": 1000})
    t = cases.isentropic_vortex(n=(24, 24, 4), numb=numb,
                                numz={"scheme": "roe", "slope": "o3", "time_step": dt})
    zd = fasts.zone_data(t, fasts.prepare(t))
    c = oracle_mod.Case(zd, ())
    c.apply_bc(0)
    c.apply_bc(1)
    nss = int(zd[0]["pi"][58])
    nsteps = int(round(t_end / dt))
    for it in range(1, nsteps + 1):
        c.compute(it, 1, nss, 1, modulo_verif=1000)
    nd = int(zd[0]["pi"][41])
    return np.array(c.z[0]["lv"][0][:nd])


@pytest.mark.parametrize("rk,lo,hi", [(1, 0.8, 1.3), (2, 1.7, 2.4), (3, 2.5, 3.7)])
def test_explicit_rk_temporal_order(oracle_mod, rk, lo, hi):
    t_end, dt = 0.8, 0.04
    ref = _final_density(oracle_mod, 3, dt / 8, t_end)
    e1 = np.max(np.abs(_final_density(oracle_mod, rk, dt, t_end) - ref))
    e2 = np.max(np.abs(_final_density(oracle_mod, rk, dt / 2, t_end) - ref))
    p = math.log2(e1 / e2)
    assert lo <= p <= hi, f"RK{rk}: observed order {p:.2f} (errors {e1:.2e}, {e2:.2e})"


def test_implicit_bdf2_temporal_order(oracle_mod):
    t_end, dt = 0.8, 0.04
    ref = _final_density(oracle_mod, 3, dt / 8, t_end, implicit=True)
    e1 = np.max(np.abs(_final_density(oracle_mod, 3, dt, t_end, implicit=True) - ref))
    e2 = np.max(np.abs(_final_density(oracle_mod, 3, dt / 2, t_end, implicit=True) - ref))
    p = math.log2(e1 / e2)
    assert 1.7 <= p <= 2.4, f"BDF2: observed order {p:.2f} (errors {e1:.2e}, {e2:.2e})"
