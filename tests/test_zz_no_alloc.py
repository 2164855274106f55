"""fgb_residual_norms_noalloc (the norms entry point that allocates nothing)
against fgb_residuals on the same solver state, through the C ABI.

The file name sorts last so that this also runs after every other GPU test
of the session; it passes alone in a fresh process as well.  The test
allocates the output buffer itself (with torch); the entry point allocates
nothing."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12   # the same reduction in the same order: equal in practice


def _solver(t, modulo_verif=1):
    from fast_gb300 import fasts
    from fast_gb300._native import Solver
    m = fasts.prepare(t)
    zd = fasts.zone_data(t, m)
    s = Solver(0)
    for z in zd:
        s.add_zone(z["pi"], z["pr"], z["ti"], z["tj"], z["tk"], z["vol"])
    s.set_option("modulo_verif", modulo_verif)
    for n, z in enumerate(zd):
        for lvl, key in enumerate(("ro", "ro_m1", "ro_p1")):
            s.upload(n, lvl, z[key])
    s.apply_bc(0)
    s.apply_bc(1)
    return zd, s


def test_noalloc_norms_equal_fgb_residuals():
    torch = pytest.importorskip("torch")
    from fast_gb300 import cases
    # 24 x 20 x 20 cells with 100 x 10 x 10 LU blocks: 1 x 2 x 2 blocks
    t = cases.taylor_green(n=(24, 20, 20), ss_iteration=2)
    zd, s = _solver(t)
    neq = int(zd[0]["pi"][36])
    nss = int(zd[0]["pi"][58])
    s.compute(1, 1, nss, 1, 1)   # verified step: the last sub-iteration only
    s.synchronize()              # computes (and records) the residual
    ref = s.residuals(0)[:, -1]
    assert ref.shape == (2 * neq,) and np.all(ref > 0)
    out = torch.empty(2 * neq, dtype=torch.float64, device="cuda:0")
    for _ in range(2):           # two calls in a row on the same state
        out.fill_(float("nan"))
        torch.cuda.synchronize()
        s.residual_norms_noalloc(0, out.data_ptr())
        s.synchronize()
        got = out.cpu().numpy()
        assert np.all(np.isfinite(got))
        err = float(np.max(np.abs(got - ref) / np.abs(ref)))
        assert err <= TOL, f"rel err {err:.3e}"
    s.close()


def test_noalloc_norms_reject_oversized_zone_and_host_buffer():
    torch = pytest.importorskip("torch")
    from fast_gb300 import cases
    from fast_gb300._native import FastGB300Error
    # 4 x 580 x 580 cells: 1 x 58 x 58 = 3364 LU blocks > 32768 / (2 * 5)
    t = cases.taylor_green(n=(4, 580, 580), ss_iteration=1)
    zd, s = _solver(t, modulo_verif=1000)
    out = torch.empty(10, dtype=torch.float64, device="cuda:0")
    with pytest.raises(FastGB300Error, match="FGB_NORM_PARTIALS_MAX"):
        s.residual_norms_noalloc(0, out.data_ptr())
    s.close()
    # an explicit zone has no residual to reduce
    t = cases.isentropic_vortex(n=(16, 12, 4))
    zd, s = _solver(t, modulo_verif=1000)
    with pytest.raises(FastGB300Error, match="implicit zones"):
        s.residual_norms_noalloc(0, out.data_ptr())
    s.close()
    t = cases.taylor_green(n=(12, 10, 8), ss_iteration=1)
    zd, s = _solver(t)
    host = np.zeros(10)
    with pytest.raises(FastGB300Error, match="device memory"):
        s.residual_norms_noalloc(0, host.ctypes.data)
    s.close()
