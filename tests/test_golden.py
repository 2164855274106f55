"""Committed golden vectors (tests/golden/oracle_cases.npz, made by
tests/golden/make_golden.py from the oracle): the oracle still reproduces
them (CPU), and the GPU path reproduces them through the C ABI (GPU).
The case inputs are quantized (make_golden.quantized) so that they are the
same bits on every host; tolerance 1e-12 relative."""
import sys
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).with_name("golden")
sys.path.insert(0, str(GOLDEN))
import make_golden  # noqa: E402

TOL = 1e-12
NAMES = list(make_golden.specs())


@pytest.fixture(scope="module")
def golden():
    return dict(np.load(GOLDEN / "oracle_cases.npz"))


def _check(golden, name, q):
    """Sampled state values against the fixture, relative per value."""
    exp = golden[name + "/val"]
    got = q[golden[name + "/pos"]]
    assert np.max(np.abs(got - exp) / np.maximum(np.abs(exp), 1e-300)) <= TOL


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_golden(oracle_mod, golden, name):
    zd, q, norms = make_golden.run_oracle(name)
    _check(golden, name, q)
    sums = make_golden.interior_sums(zd[0]["pi"], q)
    exp = golden[name + "/sum"]
    assert np.allclose(sums, exp, rtol=TOL, atol=TOL * np.max(np.abs(exp)))
    en = golden[name + "/norms"]
    if en.size:
        assert np.max(np.abs(norms - en) / np.maximum(np.abs(en), 1e-300)) <= TOL


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_reproduces_golden(golden, name):
    from fast_gb300 import fasts
    from fast_gb300._native import Solver
    t, steps, nstep_fin, mv = make_golden.build_case(name)
    zd = fasts.zone_data(t, fasts.prepare(t))
    s = Solver(0)
    z = zd[0]
    s.add_zone(z["pi"], z["pr"], z["ti"], z["tj"], z["tk"], z["vol"])
    if "dist" in z:
        s.set_wall_distance(0, z["dist"])
    s.set_option("modulo_verif", mv)
    for lvl, key in enumerate(("ro", "ro_m1", "ro_p1")):
        s.upload(0, lvl, z[key])
    s.apply_bc(0)
    s.apply_bc(1)
    for it in range(1, steps + 1):
        s.compute(it, 1, nstep_fin, 1, 1)
    s.synchronize()
    q = s.download(0, 0)
    _check(golden, name, q)
    sums = make_golden.interior_sums(z["pi"], q)
    exp = golden[name + "/sum"]
    assert np.allclose(sums, exp, rtol=TOL, atol=TOL * np.max(np.abs(exp)))
    en = golden[name + "/norms"]
    if en.size:
        got = s.residuals(0)
        assert np.max(np.abs(got - en) / np.maximum(np.abs(en), 1e-300)) <= TOL
    s.close()
