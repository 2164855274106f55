"""fasts._compute with host arrays (every step uploads levels n and n-1 and
downloads the new level; the uploads are asynchronous for the page-locked
tree arrays, level n-1 joining the solver stream at the first balance) gives
the bits of the device-resident run."""
import numpy as np
import pytest

from fast_gb300 import cases, fastc, fasts
from fast_gb300 import pytree as I

pytestmark = pytest.mark.gpu


def _run(make, resident, nsteps):
    t = make()
    t, tc, m = fasts.warmup(t, None, gpu_resident=resident)
    for it in range(1, nsteps + 1):
        fasts._compute(t, m, it)
    if resident:
        fasts._syncHost(t)
    out = [np.array(fastc.compactArray(z, suf)) for z in I.getZones(t) for suf in ("", "_M1")]
    fasts.HOOK["solver"].close()
    fasts.HOOK = None
    return out


@pytest.mark.parametrize("kind", ["implicit", "explicit"])
def test_host_array_steps_equal_resident_steps(kind):
    if kind == "implicit":
        def make():
            return cases.taylor_green(n=(16, 14, 12), ss_iteration=3,
                                      numb={"temporal_scheme": "implicit", "ss_iteration": 3,
                                            "modulo_verif": 2})
    else:
        def make():
            return cases.isentropic_vortex(n=(24, 20, 4))
    a = _run(make, True, 4)
    b = _run(make, False, 4)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_upload_async_of_an_unpinned_array_is_a_plain_upload():
    from fast_gb300._native import Solver
    t = cases.taylor_green(n=(8, 8, 8), ss_iteration=2)
    zd = fasts.zone_data(t, fasts.prepare(t))
    s = Solver(0)
    s.add_zone(zd[0]["pi"], zd[0]["pr"], zd[0]["ti"], zd[0]["tj"], zd[0]["tk"], zd[0]["vol"])
    x = np.array(zd[0]["ro"])
    s.upload_async(0, 0, x)
    x[:] = -1.0   # a plain upload has already copied the values
    got = s.download(0, 0)
    assert np.array_equal(got, zd[0]["ro"])
    s.close()
