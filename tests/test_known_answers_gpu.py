"""The known-answer cases of the oracle tests on the GPU path: Sod's shock
tube (Roe, minmod; extrapolation BCs) and the shear wave between no-slip
walls (laminar AUSM+(P) o3) run through the C ABI give the oracle's levels
within 1e-12 per cell after every step, so the GPU path itself matches the
exact Riemann solution and the exact viscous decay rate that the oracle
tests check (tests/test_shock_tube.py, tests/test_viscous_decay.py)."""
import math

import numpy as np
import pytest

from test_gpu_parity import _check_levels, _pair
from test_shock_tube import exact_sod, sod_tree
from test_viscous_decay import shear_tree

pytestmark = pytest.mark.gpu


def _run_both(t, nsteps, oracle_mod):
    zd, ref, s = _pair(t, oracle_mod, 10 ** 6)
    for it in range(1, nsteps + 1):
        ref.compute(it, 1, 3, 1, modulo_verif=10 ** 6)
        s.compute(it, 1, 3, 1, 1)
    _check_levels(ref, s)
    s.synchronize()
    out = s.download(0, 0)
    s.close()
    return zd, out


def test_sod_shock_tube_on_gpu(oracle_mod):
    nx = 200
    t, nsteps = sod_tree(nx, "roe", "minmod")
    zd, q = _run_both(t, nsteps, oracle_mod)
    pi = zd[0]["pi"]
    nip, njp, nd = int(pi[0]), int(pi[1]), int(pi[41])
    ro = q[:nd].reshape(-1, njp, nip)[2:-2, 2:-2, 2:-2][0, 0, :]
    x = (np.arange(nx) + 0.5) / nx
    assert float(np.mean(np.abs(ro - exact_sod(x, 0.2)))) < 0.0055


def test_shear_wave_decay_on_gpu(oracle_mod):
    t, nsteps = shear_tree(16)
    zd, q = _run_both(t, nsteps, oracle_mod)
    pi = zd[0]["pi"]
    nip, njp, nd = int(pi[0]), int(pi[1]), int(pi[41])
    nu = float(zd[0]["pr"][11])
    u = q[nd:2 * nd].reshape(-1, njp, nip)[2:-2, 2:-2, 2:-2]
    u0 = 0.1 * np.sin(math.pi * (np.arange(16) + 0.5) / 16)
    decay = float(np.mean(u[:, :, 1] / u0[None, :]))   # u / u(0), every cell alike
    assert abs(decay - math.exp(-nu * math.pi ** 2 * 10.0)) < 2e-3 * decay
