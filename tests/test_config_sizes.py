"""GPU parity at the sizes of the benchmark configurations, and on the
LU-SGS schedule in which a thread takes several cells of a hyperplane.

* config 1 exactly: isentropic vortex 128 x 128 x 4, Roe + minmod, explicit
  RK3, the time step of CFL 0.5 from cpcfl3.for's local time step, 200 steps;
* an implicit Taylor-Green vortex of 64^3 cells, 4 LU-SGS sub-iterations, 2
  physical steps (levels and residual norms);
* the 48-block Spalart-Allmaras channel with its real block sizes (16 to 96
  cells a side, 2.14 M cells), 1 implicit step;
* the persistent LU-SGS sweep capped to one or two CTAs ("lu_grid"), so that
  every thread loops over several cells of the large hyperplanes, single zone
  and grouped zones, FP64 against the oracle and FP32 against the uncapped
  FP32 schedule (same cell arithmetic, so the same bits).

Bar: 1e-12 relative per cell, as in the other parity tests."""
import numpy as np
import pytest

from conftest import rel_err
from fast_gb300 import cases, fasts
from test_gpu_parity import TOL, _check_levels, _pair

pytestmark = pytest.mark.gpu


def test_config1_vortex_cfl05_200_steps(oracle_mod):
    t = cases.isentropic_vortex(cfl=0.5)
    zd, ref, s = _pair(t, oracle_mod, 1000000)
    pi = zd[0]["pi"]
    assert [int(pi[20 + d]) for d in range(3)] == [128, 128, 4]
    assert int(pi[64]) == 3 and int(pi[29]) == 2          # minmod, explicit
    assert zd[0]["pr"][0] == oracle_mod.cfl_dt(zd[0], 0.5)
    for it in range(1, 201):
        ref.compute(it, 1, 3, 1, modulo_verif=1000000)
        s.compute(it, 1, 3, 1, 1)
    _check_levels(ref, s)
    # the vortex moved: the state is not the initial one
    assert np.max(np.abs(s.download(0, 0) - zd[0]["ro"])) > 1e-3
    s.close()


def test_config1_cfl_is_half(oracle_mod):
    """The CFL statistic of the first (verified) iteration is 0.5: the GPU's
    cpcfl3 reduction on the initial state with the chosen time step."""
    t = cases.isentropic_vortex(cfl=0.5)
    zd, ref, s = _pair(t, oracle_mod, 1)
    ref.compute(1, 1, 3, 1, modulo_verif=1)
    s.compute(1, 1, 3, 1, 1)
    got, exp = s.cfl(0), ref.cfl(0)
    assert got[0] == exp[0]
    assert abs(got[0] - 0.5) <= 1e-12
    s.close()


def test_implicit_tgv64_two_steps(oracle_mod):
    t = cases.taylor_green(n=64, ss_iteration=4)
    zd, ref, s = _pair(t, oracle_mod, 1)
    for it in range(1, 3):
        ref.compute(it, 1, 5, 1, modulo_verif=1)
        s.compute(it, 1, 5, 1, 1)
    _check_levels(ref, s)
    nss = int(zd[0]["pi"][58])
    assert rel_err(s.residuals(0), ref.residual_norms(0, nss)) <= TOL
    s.close()


def test_channel_full_size_one_step(oracle_mod):
    t, tc = cases.sa_channel(ss_iteration=4, modulo_verif=1)
    zd, ref, s = _pair(t, oracle_mod, 1, tc)
    assert len(zd) == 48
    assert max(int(z["pi"][20]) for z in zd) > 60
    ref.compute(1, 1, 5, 1, modulo_verif=1)
    s.compute(1, 1, 5, 1, 1)
    for m in range(len(zd)):
        _check_levels(ref, s, zone=m)
        nss = int(zd[m]["pi"][58])
        assert rel_err(s.residuals(m), ref.residual_norms(m, nss)) <= TOL
    s.close()


def _capped_case(kind):
    if kind == "single":
        return cases.taylor_green(n=(48, 40, 36), ss_iteration=3), ()
    return cases.sa_channel(sizes=((4, 9), (4, 7), (4, 6)), first_cell=2e-2, reynolds=2000.0,
                            temporal="implicit", ss_iteration=3, time_step=0.02,
                            modulo_verif=1)


@pytest.mark.parametrize("kind", ["single", "grouped"])
@pytest.mark.parametrize("mode,cap", [(1, 1), (1, 2), (2, 1), (2, 3)])
def test_lu_grid_cap_fp64(oracle_mod, kind, mode, cap):
    """Grid-barrier sweep (mode 1): every hyperplane larger than cap x 512
    cells makes each thread loop over several cells (its multi-cell branch).
    Dataflow sweep (mode 2): one to three CTAs take every chunk in turn."""
    t, tc = _capped_case(kind)
    zd, ref, s = _pair(t, oracle_mod, 1, tc)
    s.set_option("lu_mode", mode)
    s.set_option("autotune", 0)
    s.set_option("lu_grid", cap)
    for it in range(1, 3):
        ref.compute(it, 1, 4, 1, modulo_verif=1)
        s.compute(it, 1, 4, 1, 1)
    for m in range(len(zd)):
        _check_levels(ref, s, zone=m)
    s.close()


@pytest.mark.parametrize("kind", ["single", "grouped"])
def test_lu_grid_cap_fp32_same_bits(oracle_mod, kind):
    """FP32 sweeps: the grid-barrier sweep capped to one CTA (operands
    preloaded across the barrier, several cells per thread), the uncapped
    grid-barrier sweep and the dataflow sweep give the same bits."""
    out = []
    for mode, cap in ((1, 0), (1, 1), (2, 0)):
        t, tc = _capped_case(kind)
        zd, ref, s = _pair(t, oracle_mod, 1, tc)
        s.set_option("lu_precision", 32)
        s.set_option("lu_mode", mode)
        s.set_option("autotune", 0)
        s.set_option("lu_grid", cap)
        for it in range(1, 3):
            s.compute(it, 1, 4, 1, 1)
        s.synchronize()
        out.append([s.download(m, 0) for m in range(len(zd))])
        s.close()
    for other in out[1:]:
        for a, b in zip(out[0], other):
            assert np.array_equal(a, b)


def test_grid_barrier_wait_gives_up():
    """The persistent grid-barrier sweep (lu_mode 1) with a barrier target
    that no arrival reaches ("lu_wait_skew"): its bounded wait gives up after
    4 x "lu_poll_limit" polls, the call reports FGB_ERR_DEVICE, every CTA
    returns, and a fresh solver then computes normally."""
    from fast_gb300._native import FastGB300Error, Solver
    t = cases.taylor_green(n=(12, 10, 8), ss_iteration=2)
    zd = fasts.zone_data(t, fasts.prepare(t))

    def solver():
        s = Solver(0)
        s.add_zone(zd[0]["pi"], zd[0]["pr"], zd[0]["ti"], zd[0]["tj"], zd[0]["tk"], zd[0]["vol"])
        for lvl, key in enumerate(("ro", "ro_m1", "ro_p1")):
            s.upload(0, lvl, zd[0][key])
        s.apply_bc(0)
        s.apply_bc(1)
        return s

    s = solver()
    s.set_option("lu_mode", 1)
    s.set_option("autotune", 0)
    s.set_option("lu_poll_limit", 4096)
    s.set_option("lu_wait_skew", 1)
    s.compute(1, 1, 3, 1, 1)
    with pytest.raises(FastGB300Error, match="grid barrier"):
        s.synchronize()
    s.close()
    s = solver()
    s.compute(1, 1, 3, 1, 1)
    s.synchronize()
    assert np.all(np.isfinite(s.download(0, 0)))
    s.close()


@pytest.mark.parametrize("precision", [64, 32])
def test_dataflow_wait_gives_up(precision):
    """A dependency wait of the dataflow sweep whose mark nothing publishes
    ("lu_wait_skew" raises the marks -- FP32: the tags of the increment
    words -- that the waits expect) gives up after "lu_poll_limit" polls: the
    call reports FGB_ERR_DEVICE, every warp returns, and the device stays
    usable (a fresh solver then computes normally)."""
    from fast_gb300._native import FastGB300Error
    t = cases.taylor_green(n=(12, 10, 8), ss_iteration=2)
    from fast_gb300._native import Solver
    m = fasts.prepare(t)
    zd = fasts.zone_data(t, m)

    def solver():
        s = Solver(0)
        s.add_zone(zd[0]["pi"], zd[0]["pr"], zd[0]["ti"], zd[0]["tj"], zd[0]["tk"], zd[0]["vol"])
        for lvl, key in enumerate(("ro", "ro_m1", "ro_p1")):
            s.upload(0, lvl, zd[0][key])
        s.apply_bc(0)
        s.apply_bc(1)
        return s

    s = solver()
    s.set_option("lu_mode", 2)
    s.set_option("autotune", 0)
    s.set_option("lu_precision", precision)
    s.set_option("lu_poll_limit", 4096)
    s.set_option("lu_wait_skew", 2)
    s.compute(1, 1, 3, 1, 1)
    with pytest.raises(FastGB300Error, match="gave up"):
        s.synchronize()
    s.close()
    s = solver()
    s.compute(1, 1, 3, 1, 1)
    s.synchronize()
    assert np.all(np.isfinite(s.download(0, 0)))
    s.close()


@pytest.mark.parametrize("kind", ["single", "grouped"])
def test_lu_autotuned_schedule_same_bits(oracle_mod, kind):
    """With the autotuner on (default), the first solve of each LU group
    times the grid-barrier sweep and the dataflow sweep (one and two CTAs
    per SM) and keeps the fastest: the results are those of the oracle and of
    the fixed schedules, bit for bit."""
    out = []
    for tune in (0, 1):
        t, tc = _capped_case(kind)
        zd, ref, s = _pair(t, oracle_mod, 1, tc)
        s.set_option("autotune", tune)
        for it in range(1, 3):
            if tune:
                ref.compute(it, 1, 4, 1, modulo_verif=1)
            s.compute(it, 1, 4, 1, 1)
        s.synchronize()
        out.append([s.download(m, 0) for m in range(len(zd))])
        if tune:
            for m in range(len(zd)):
                _check_levels(ref, s, zone=m)
        s.close()
    for a, b in zip(*out):
        assert np.array_equal(a, b)
