"""Explicit Runge-Kutta of order 1 and 2 (numerics key 'rk', temporal_scheme
'explicit'): FastC packs nssiter = rk (FastC/FastC/PyTree.py:1172-1174);
the stage coefficients are init_rhs.for:58-78 (coefH: 0; 0, -1) and
core3ark3.for:64-85 (coefW: 1; 1, 0.5), the stages alternate between levels
n and n+1 as for RK3, and after the step the levels rotate for RK1 but stay
in place for RK2, whose second stage wrote level n (FastS/FastS/PyTree.py:
226-228, switchPointers__ with order nitmax%2+2).

CPU: the oracle's RK2 first stage is its RK1 step, bit for bit, and the RK2
step leaves level n-1 alone.  GPU: the device path against the oracle at
1e-12 per cell, with and without host-array steps."""
import numpy as np
import pytest

from fast_gb300 import cases, fastc, fasts
from fast_gb300 import pytree as I

from test_gpu_parity import _check_levels, _pair


def _vortex(rk, n=(20, 16, 6)):
    return cases.isentropic_vortex(n=n, numb={"temporal_scheme": "explicit", "rk": rk,
                                              "modulo_verif": 1000},
                                   numz={"scheme": "roe_min", "slope": "minmod", "time_step": 0.05})


def _laminar(rk):
    return cases.taylor_green(n=(12, 10, 8), numb={"temporal_scheme": "explicit", "rk": rk,
                                                   "modulo_verif": 1000},
                              numz={"time_step": 0.002})


def _oracle_case(t, oracle_mod):
    m = fasts.prepare(t)
    zd = fasts.zone_data(t, m)
    ref = oracle_mod.Case(zd, ())
    ref.apply_bc(0)
    ref.apply_bc(1)
    return zd, ref


@pytest.mark.parametrize("rk", [1, 2])
def test_rk_order_parameters(rk):
    t = _vortex(rk)
    fastc._buildOwnData(t)
    pi = I.getNodeFromName2(I.getZones(t)[0], "Parameter_int")[1]
    assert int(pi[fastc.RK]) == rk
    assert int(pi[fastc.NSSITER]) == rk
    assert int(pi[fastc.ITYPCP]) == 2


def test_oracle_rk2_first_stage_is_the_rk1_step(oracle_mod):
    zd1, r1 = _oracle_case(_vortex(1), oracle_mod)
    zd2, r2 = _oracle_case(_vortex(2), oracle_mod)
    m1_before = np.array(r2.z[0]["lv"][1])
    n_before = np.array(r2.z[0]["lv"][0])
    r1.compute(1, 1, 1, 1, modulo_verif=1000)
    r2.compute(1, 1, 2, 1, modulo_verif=1000)
    # RK1 rotated: its new level n is the array it wrote (level n+1 before)
    assert np.array_equal(r1.z[0]["lv"][0], r2.z[0]["lv"][2])
    assert np.array_equal(r1.z[0]["lv"][1], n_before)
    # RK2 did not rotate: level n-1 untouched, level n overwritten
    assert np.array_equal(r2.z[0]["lv"][1], m1_before)
    assert not np.array_equal(r2.z[0]["lv"][0], n_before)


def test_oracle_rk2_is_heun(oracle_mod):
    """Second stage: D2 = -D1 + R(W1), W2 = W1 + 0.5 coe D2, i.e. the
    conservative variables move by dt/2 (R(Wn) + R(W1)): with the first
    stage's residual D1 = (W1 - Wn) / coe, the density of the RK2 step is
    the mean of Wn and of an RK1 step taken from W1."""
    zd, r2 = _oracle_case(_vortex(2), oracle_mod)
    ro_n = np.array(r2.z[0]["lv"][0])
    r2.compute(1, 1, 2, 1, modulo_verif=1000)
    ro_1 = np.array(r2.z[0]["lv"][2])    # first stage (level n+1)
    ro_2 = np.array(r2.z[0]["lv"][0])    # the step's result (level n)
    # an RK1 step from W1
    zdb, rb = _oracle_case(_vortex(1), oracle_mod)
    for lvl in range(3):
        rb.z[0]["lv"][lvl][:] = ro_1
    rb.apply_bc(0)
    rb.compute(1, 1, 1, 1, modulo_verif=1000)
    ro_e = np.array(rb.z[0]["lv"][0])
    nd = int(zd[0]["pi"][41])
    pi = zd[0]["pi"]
    ni, nj, nk = int(pi[20]), int(pi[21]), int(pi[22])
    ng = int(pi[3])
    nip, njp = int(pi[0]), int(pi[1])
    ngk = int(pi[4])
    i, j, k = np.meshgrid(np.arange(ni), np.arange(nj), np.arange(nk), indexing="ij")
    l = ((i + ng) + (j + ng) * nip + (k + ngk) * nip * njp).reshape(-1)
    got = ro_2[:nd][l]
    heun = 0.5 * (ro_n[:nd][l] + ro_e[:nd][l])
    assert np.max(np.abs(got - heun)) <= 1e-13 * np.max(np.abs(heun))


@pytest.mark.gpu
@pytest.mark.parametrize("rk", [1, 2])
@pytest.mark.parametrize("kind", ["euler", "laminar"])
def test_explicit_rk_order_matches_oracle(oracle_mod, rk, kind):
    t = _vortex(rk) if kind == "euler" else _laminar(rk)
    zd, ref, s = _pair(t, oracle_mod, 1000)
    assert int(zd[0]["pi"][52]) == rk and int(zd[0]["pi"][58]) == rk
    for it in range(1, 4):
        ref.compute(it, 1, rk, 1, modulo_verif=1000)
        s.compute(it, 1, rk, 1, 1)
    _check_levels(ref, s)
    s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("rk", [1, 2])
def test_rk_order_host_array_steps_equal_resident_steps(rk):
    def run(resident):
        t = _vortex(rk, n=(24, 20, 4))
        t, tc, m = fasts.warmup(t, None, gpu_resident=resident)
        for it in range(1, 5):
            fasts._compute(t, m, it)
        if resident:
            fasts._syncHost(t)
        out = [np.array(fastc.compactArray(z, suf)) for z in I.getZones(t)
               for suf in ("", "_M1", "_P1")]
        fasts.HOOK["solver"].close()
        fasts.HOOK = None
        return out
    a = run(True)
    b = run(False)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
