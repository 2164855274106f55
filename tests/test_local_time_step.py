"""Local time stepping (time_step_nature = 'local', DTLOC = 1), implicit:
cptst3.for takes tstb3_impli.for instead of tstb3_global.for + tstb3c.for --
the spectral radii as before, then a time step per cell from the CFL number
(dtloc.for: CFL x min(convective, viscous) time step of the cell), BDF1 in
the dual-time residual (core3as2.for; Spalart-Allmaras: the first
sub-iteration's residual is coe1 x balance); explicit: tstb3_expli.for, the
same time step as coe1 of the RK3 update.  The GPU path against the
oracle at 1e-12 per cell; the oracle's coe1 against the formula on a
uniform state."""
import math

import numpy as np
import pytest

from fast_gb300 import cases, fasts

from test_gpu_parity import TOL, _check_levels, _pair


def _local(numz=None):
    z = {"time_step_nature": "local", "cfl": 5.0}
    z.update(numz or {})
    return z


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["explicit_euler", "explicit_laminar"])
def test_explicit_local_time_step_matches_oracle(oracle_mod, kind):
    """Explicit RK3 with a local time step (tstb3_expli.for: coe1 only)."""
    if kind == "explicit_euler":
        t = cases.isentropic_vortex(n=(20, 16, 6), wavy=0.3,
                                    numz=_local({"scheme": "roe_min", "slope": "minmod", "cfl": 0.5}))
    else:
        t = cases.taylor_green(n=(12, 10, 8), numb={"temporal_scheme": "explicit"},
                               numz=_local({"cfl": 0.5}))
    zd, ref, s = _pair(t, oracle_mod, 1000)
    assert int(zd[0]["pi"][46]) == 1 and int(zd[0]["pi"][29]) == 2
    for it in range(1, 4):
        ref.compute(it, 1, 3, 1, modulo_verif=1000)
        s.compute(it, 1, 3, 1, 1)
    _check_levels(ref, s)
    s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["cart", "full", "sa", "2d", "euler"])
def test_local_time_step_matches_oracle(oracle_mod, kind):
    if kind == "cart":
        t = cases.taylor_green(n=(12, 10, 8), ss_iteration=3, numz=_local())
    elif kind == "full":
        t = cases.taylor_green(n=(12, 10, 8), ss_iteration=3, wavy=0.3, numz=_local())
    elif kind == "sa":
        t = cases.bc_box(n=(12, 10, 6), model="NSTurbulent", temporal="implicit", ss_iteration=3,
                         time_step=0.02)
        from fast_gb300 import pytree as I, fastc
        for z in I.getZones(t):
            fastc._setNum2Zones(z, _local())
    elif kind == "2d":
        t = cases.isentropic_vortex(n=(20, 16, 1), two_d=True, wavy=0.3,
                                    numb={"temporal_scheme": "implicit", "ss_iteration": 3,
                                          "modulo_verif": 1},
                                    numz=_local({"scheme": "ausmpred", "slope": "o3"}))
    else:
        t = cases.isentropic_vortex(n=(16, 14, 6), numb={"temporal_scheme": "implicit",
                                                         "ss_iteration": 3, "modulo_verif": 1},
                                    numz=_local({"scheme": "roe_min", "slope": "minmod"}))
    zd, ref, s = _pair(t, oracle_mod, 1)
    assert int(zd[0]["pi"][46]) == 1
    for it in range(1, 3):
        ref.compute(it, 1, 4, 1, modulo_verif=1)
        s.compute(it, 1, 4, 1, 1)
    _check_levels(ref, s)
    s.close()


def test_oracle_local_time_step_formula(oracle_mod):
    """Uniform state on a cartesian box: coe1 = CFL min(dtconv, dtvis),
    dtconv = sqrt(d) / (|u| + c), dtvis = detj d / (2 gam1 mu) ro,
    d = 1 / sum (tc_d^2) (dtloc.for)."""
    t = cases.taylor_green(n=(8, 8, 8), ss_iteration=2, numz=_local())
    zd = fasts.zone_data(t, fasts.prepare(t))
    ref = oracle_mod.Case(zd, ())
    ref.apply_bc(0)
    ref.apply_bc(1)
    ref.compute(1, 1, 1, 1, modulo_verif=1)
    pi, pr = zd[0]["pi"], zd[0]["pr"]
    nd = int(pi[41])
    coe = ref.z[0]["coe"].reshape(-1, nd)
    ro = np.asarray(zd[0]["ro"]).reshape(5, nd)   # level n, the state the coefficients see
    nip, njp, ng, ngk = int(pi[0]), int(pi[1]), int(pi[3]), int(pi[4])
    l = (3 + ng - 1) + (4 + ng - 1) * nip + (5 + ngk - 1) * nip * njp   # interior cell (3, 4, 5)
    r, u, v, w, T = (ro[m, l] for m in range(5))
    gam, cv, prandt, cfl = pr[1], pr[2], pr[10], pr[15]
    rgp = cv * (gam - 1.)
    c = math.sqrt(gam * rgp * T)
    tc = [zd[0]["ti"][0], zd[0]["tj"][0], zd[0]["tk"][0]]
    d = 1. / sum(x * x for x in tc)
    xm = ref.z[0]["xmut"][l]
    dtvis = 0.5 * zd[0]["vol"][0] * d * (prandt / gam) / xm * r
    dtconv = math.sqrt(d) / (math.sqrt(u * u + v * v + w * w) + c)
    assert abs(coe[0, l] - cfl * min(dtconv, dtvis)) <= 1e-12 * abs(coe[0, l])
