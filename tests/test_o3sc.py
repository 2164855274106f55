"""The o3sc slope (SLOPE = 6): o3 states blended with the first-order ones by
the directional shock sensor of SENSOR/sciacovelli.for + shock_sensor.for,
recomputed on every sub-step (src_term.for:246-255); faces as
AUSM/*/fluFaceEuler_o3sc_*.for and ROE/*/fluFaceEuler_o3sc_*.for.

CPU: the oracle's sensor weights against a numpy statement of the sensor's
formula on a cartesian zone.
GPU: the sm_103a path against the oracle on cartesian, curvilinear and 2-d
zones, AUSM+(P), senseur (its wiggle flags and the o3sc weights side by
side) and Roe (with its wall-face correction), Euler / laminar /
Spalart-Allmaras, explicit RK3 and implicit LU-SGS.
"""
import numpy as np
import pytest

from conftest import rel_err
from fast_gb300 import cases, fasts


def _first_stage(oracle_mod, t):
    zd = fasts.zone_data(t, fasts.prepare(t))
    c = oracle_mod.Case(zd)
    c.apply_bc(0)
    c.apply_bc(1)
    q0 = c.z[0]["lv"][0].copy()      # the state of the first sub-step, ghosts filled
    c.compute(1, 1, 1, 1, modulo_verif=1000)
    return zd[0], c, q0


def test_sensor_cartesian_known_answer(oracle_mod):
    """wig_d = 1 - min(2 div^2 / (div^2 + rot + 1e-15) * J_d * M_d, 1) with
    central differences of the velocity (div, rot), Jameson's switch J_d of
    p = rho T and M_d = (1 - tanh(2.5 + 10 div / (tc_d c))) / 2."""
    t = cases.bc_box(n=(16, 12, 6), scheme="ausmpred", slope="o3sc", perturb=0.3,
                     wall="BCWallInviscid", model="Euler")
    z, c, q0 = _first_stage(oracle_mod, t)
    pi, pr = z["pi"], z["pr"]
    assert int(pi[25]) == 2 and int(pi[64]) == 6      # cartesian zone, o3sc
    (ni, nj, nk), nd = (16, 12, 6), int(pi[41])
    q = q0.reshape(5, nk + 4, nj + 4, ni + 4)
    tix, tjy, tkz = float(z["ti"].reshape(-1)[0]), float(z["tj"].reshape(-1)[0]), float(z["tk"].reshape(-1)[0])
    xvol = 0.5 / float(z["vol"].reshape(-1)[0])
    gam = float(pr[1])
    rgp = float(pr[2]) * (gam - 1.0)
    I = (slice(2, -2),) * 3

    def sh(a, d, s):            # a at the neighbour s cells along axis d (0 = i)
        ax = 2 - d
        idx = [slice(2, -2)] * 3
        idx[ax] = slice(2 + s, a.shape[ax] - 2 + s)
        return a[tuple(idx)]

    u, v, w = q[1], q[2], q[3]
    dx = lambda a, d: sh(a, d, 1) - sh(a, d, -1)
    div = (dx(u, 0) * tix + dx(v, 1) * tjy + dx(w, 2) * tkz) * xvol
    rotz = (dx(v, 0) * tix - dx(u, 1) * tjy) * xvol
    roty = (dx(u, 2) * tkz - dx(w, 0) * tix) * xvol
    rotx = (dx(w, 1) * tjy - dx(v, 2) * tkz) * xvol
    rot = rotx ** 2 + roty ** 2 + rotz ** 2
    snd = np.sqrt(gam * rgp * q[4][I])
    p = q[0] * q[4]
    wig = c.z[0]["wig"]
    for d, tc in enumerate((abs(tix), abs(tjy), abs(tkz))):
        m = 0.5 * (1.0 - np.tanh(2.5 + 10.0 / tc / snd * div))
        jam = np.abs(sh(p, d, -1) - 2 * p[I] + sh(p, d, 1)) / np.abs(sh(p, d, -1) + 2 * p[I] + sh(p, d, 1))
        exp = 1.0 - np.minimum(2.0 * div * div / (div * div + rot + 1e-15) * jam * m, 1.0)
        got = wig[d * nd:(d + 1) * nd].reshape(nk + 4, nj + 4, ni + 4)[I]
        assert np.max(np.abs(got - exp)) <= 1e-12, d
        assert exp.min() < 0.999         # the sensor acts on this field
    # the weights change the residual: o3sc differs from o3 on the same state
    _, c3, _ = _first_stage(oracle_mod, cases.bc_box(n=(16, 12, 6), scheme="ausmpred", slope="o3",
                                                  perturb=0.3, wall="BCWallInviscid", model="Euler"))
    a, b = c.z[0]["drodm"], c3.z[0]["drodm"]
    assert np.max(np.abs(a - b)) > 1e-6 * np.max(np.abs(b))


@pytest.mark.gpu
@pytest.mark.parametrize("scheme,n,wavy,temporal,model,wall", [
    ("ausmpred", (16, 12, 6), 0.0, "explicit", "Euler", "BCWallInviscid"),
    ("roe", (16, 12, 6), 0.0, "explicit", "NSLaminar", "BCWallViscous"),
    ("ausmpred", (12, 10, 6), 0.3, "explicit", "NSLaminar", "BCWallViscous"),
    ("ausmpred", (12, 10, 6), 0.3, "implicit", "NSLaminar", "BCWallViscous"),
    ("roe", (12, 10, 6), 0.3, "implicit", "Euler", "BCWallInviscid"),
    ("roe", (16, 12, 1), 0.3, "explicit", "NSLaminar", "BCWallViscous"),
    ("ausmpred", (16, 12, 1), 0.3, "implicit", "Euler", "BCWallInviscid"),
    ("senseur", (12, 10, 6), 0.3, "explicit", "NSLaminar", "BCWallViscous"),
    ("senseur", (16, 12, 1), 0.0, "implicit", "Euler", "BCWallInviscid"),
    ("ausmpred", (12, 10, 6), 0.3, "implicit", "NSTurbulent", "BCWallViscous"),
    ("roe", (12, 10, 6), 0.0, "explicit", "NSTurbulent", "BCWallViscous"),
    ("senseur", (16, 12, 1), 0.3, "implicit", "NSTurbulent", "BCWallViscous"),
    ("roe", (16, 12, 1), 0.3, "implicit", "NSTurbulent", "BCWallViscous"),
])
def test_o3sc_gpu_parity(oracle_mod, scheme, n, wavy, temporal, model, wall):
    from test_gpu_parity import TOL, _check_levels, _pair
    t = cases.bc_box(n=n, two_d=n[2] == 1, wall=wall, model=model, reynolds=500.0, scheme=scheme,
                     slope="o3sc", perturb=0.3, wavy=wavy, temporal=temporal, ss_iteration=3,
                     time_step=0.01 if temporal == "explicit" else 0.05)
    mv = 1000 if temporal == "explicit" else 1
    zd, ref, s = _pair(t, oracle_mod, mv)
    assert int(zd[0]["pi"][64]) == 6
    nfin = 3 if temporal == "explicit" else 4
    for it in range(1, 4):
        ref.compute(it, 1, nfin, 1, modulo_verif=mv)
        s.compute(it, 1, nfin, 1, 1)
    _check_levels(ref, s)
    if temporal == "implicit":
        nss = int(zd[0]["pi"][58])
        assert rel_err(s.residuals(0), ref.residual_norms(0, nss)) <= TOL
    s.close()
