"""fgb_compute as CUDA graphs ("compute_graph", default on): a call is
recorded the second time its signature (step range, verification flags,
first_it, sweep precision) and level pointers come, and replayed from then
on.  Every case runs the same steps with recording on and off and compares
the levels and the residual norms bit for bit; the implicit single-zone case
is also held to the oracle."""
import numpy as np
import pytest

from fast_gb300 import cases, fasts

from test_gpu_parity import _check_levels, _pair

pytestmark = pytest.mark.gpu

SMALL = dict(sizes=((4, 9), (4, 7), (4, 6)), first_cell=2e-2, reynolds=2000.0)


def _make(kind):
    if kind == "implicit":
        return cases.taylor_green(n=(12, 10, 8), ss_iteration=3), None, 4, 2
    if kind == "implicit_fp32":
        return cases.taylor_green(n=(12, 10, 8), ss_iteration=3), None, 4, 2
    if kind == "implicit_grid_barrier":
        return cases.taylor_green(n=(12, 10, 8), ss_iteration=3), None, 4, 2
    if kind == "explicit_rk3":
        t = cases.isentropic_vortex(n=(20, 16, 6), numz={"scheme": "roe_min", "slope": "minmod",
                                                         "time_step": 0.05})
        return t, None, 3, 1000
    if kind == "explicit_rk2":
        t = cases.isentropic_vortex(n=(20, 16, 6), numb={"temporal_scheme": "explicit", "rk": 2,
                                                         "modulo_verif": 1000},
                                    numz={"scheme": "roe_min", "slope": "minmod", "time_step": 0.05})
        return t, None, 2, 1000
    if kind == "channel_sa":
        t, tc = cases.sa_channel(**SMALL, temporal="implicit", ss_iteration=3, time_step=0.02)
        return t, tc, 3, 3
    raise ValueError(kind)


def _run(kind, oracle_mod, graph, nsteps):
    t, tc, nss, verif = _make(kind)
    zd, ref, s = _pair(t, oracle_mod, verif, tc or ())
    s.set_option("compute_graph", graph)
    if kind == "implicit_fp32":
        s.set_option("lu_precision", 32)
    if kind == "implicit_grid_barrier":
        s.set_option("autotune", 0)
        s.set_option("lu_mode", 1)
    norms = []
    for it in range(1, nsteps + 1):
        s.compute(it, 1, nss, 1, 1)
        if not kind.startswith("explicit"):
            norms.append([s.residuals(m) for m in range(len(zd))])
    s.synchronize()
    levels = [[s.download(m, lv) for lv in range(3)] for m in range(len(zd))]
    recorded = s.get_option("step_graphs")
    return zd, ref, s, levels, norms, recorded, nss


@pytest.mark.parametrize("kind", ["implicit", "implicit_fp32", "implicit_grid_barrier",
                                  "explicit_rk3", "explicit_rk2", "channel_sa"])
def test_recorded_steps_equal_plain_steps(oracle_mod, kind):
    # 20 steps: every signature (three level rotations x the verification
    # flags) comes at least three times -- plain, recorded, replayed
    nsteps = 20
    _, _, s0, lv0, n0, rec0, _ = _run(kind, oracle_mod, 0, nsteps)
    s0.close()
    zd, ref, s1, lv1, n1, rec1, nss = _run(kind, oracle_mod, 1, nsteps)
    assert rec0 == 0
    if kind != "implicit_grid_barrier":   # (a cooperative launch may not be recordable)
        assert rec1 > 0
    for a, b in zip(lv0, lv1):
        for x, y in zip(a, b):
            assert np.array_equal(x, y)
    for a, b in zip(n0, n1):
        for x, y in zip(a, b):
            assert np.array_equal(x, y)
    if kind == "implicit":   # and the oracle, after the same steps
        for it in range(1, nsteps + 1):
            ref.compute(it, 1, nss, 1, modulo_verif=2)
        _check_levels(ref, s1)
    s1.close()


def test_changed_option_drops_recorded_steps(oracle_mod):
    t, tc, nss, verif = _make("implicit")
    zd, ref, s = _pair(t, oracle_mod, verif)
    for it in range(1, 12):   # signatures repeat after six steps
        s.compute(it, 1, nss, 1, 1)
    s.synchronize()
    assert s.get_option("step_graphs") > 0
    s.set_option("lu_precision", 64)          # unchanged: kept
    assert s.get_option("step_graphs") > 0
    s.set_option("lu_precision", 32)          # changed: dropped
    assert s.get_option("step_graphs") == 0
    s.close()
