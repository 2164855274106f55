"""GPU parity: the sm_103a solve step, called through the C ABI, against the
CPU oracle on the same seeded inputs.  Bar: 1e-12 relative per cell (the
FP64 kernels are built without contraction and follow the reference's
operation order, so in practice the results are bit-identical); residual
norms, which the GPU reduces with a different summation order, to 1e-12."""
import numpy as np
import pytest

from conftest import rel_err
from fast_gb300 import cases, fasts

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _pair(t, oracle_mod, modulo_verif, tc=()):
    from fast_gb300._native import Solver
    m = fasts.prepare(t)
    zd = fasts.zone_data(t, m)
    ref = oracle_mod.Case(zd, tc)
    ref.apply_bc(0)
    ref.apply_bc(1)
    s = Solver(0)
    for n, z in enumerate(zd):
        s.add_zone(z["pi"], z["pr"], z["ti"], z["tj"], z["tk"], z["vol"])
        if "dist" in z:
            s.set_wall_distance(n, z["dist"])
    for tr in tc:
        s.add_any_transfer(tr)
    s.set_option("modulo_verif", modulo_verif)
    for n, z in enumerate(zd):
        for lvl, key in enumerate(("ro", "ro_m1", "ro_p1")):
            s.upload(n, lvl, z[key])
    s.apply_bc(0)
    s.apply_bc(1)
    return zd, ref, s


def _check_levels(ref, s, zone=0, tol=TOL):
    s.synchronize()
    for lvl in range(3):
        got = s.download(zone, lvl)
        exp = ref.z[zone]["lv"][lvl]
        err = rel_err(got, exp)
        assert err <= tol, f"level {lvl}: rel err {err:.3e}"


def _interior_mask(pi):
    ni, nj, nk = (int(pi[0]), int(pi[1]), int(pi[2]))
    m = np.zeros((nk, nj, ni), dtype=bool)
    m[2:nk - 2, 2:nj - 2, 2:ni - 2] = True
    return m.reshape(-1)


@pytest.mark.parametrize("scheme,slope", [("roe_min", "minmod"), ("roe", "o3"), ("roe", "o1"),
                                          ("ausmpred", "o3")])
def test_explicit_rk3_step(oracle_mod, scheme, slope):
    t = cases.isentropic_vortex(n=(24, 20, 6),
                                numz={"scheme": scheme, "slope": slope, "time_step": 0.05})
    zd, ref, s = _pair(t, oracle_mod, 1000)
    for it in range(1, 4):
        ref.compute(it, 1, 3, 1, modulo_verif=1000)
        s.compute(it, 1, 3, 1, 1)
    _check_levels(ref, s)
    # the stage-3 residual as well (interior cells)
    pi = zd[0]["pi"]
    nd = int(pi[41])
    mask = np.tile(_interior_mask(pi), 5)
    got = s.work(0, "drodm", 5 * nd)
    exp = ref.z[0]["drodm"]
    assert rel_err(got[mask], exp[mask]) <= TOL
    s.close()


@pytest.mark.parametrize("scheme,slope,n", [("ausmpred", "o3", (12, 10, 8)),
                                            ("roe_min", "minmod", (9, 11, 7)),
                                            ("roe", "o3", (10, 10, 10))])
def test_implicit_lusgs_step(oracle_mod, scheme, slope, n):
    t = cases.taylor_green(n=n, ss_iteration=3, scheme=scheme, slope=slope)
    zd, ref, s = _pair(t, oracle_mod, 1)
    for it in range(1, 3):
        ref.compute(it, 1, 4, 1, modulo_verif=1)
        s.compute(it, 1, 4, 1, 1)
    _check_levels(ref, s)
    pi = zd[0]["pi"]
    nd = int(pi[41])
    mask = _interior_mask(pi)
    coe = s.work(0, "coe", 5 * nd).reshape(5, nd)
    assert rel_err(coe[:, mask], ref.z[0]["coe"].reshape(5, nd)[:, mask]) <= TOL
    xm = s.work(0, "xmut", nd)
    assert rel_err(xm[mask], ref.z[0]["xmut"][:nd][mask]) <= TOL
    nss = int(pi[58])
    got = s.residuals(0)
    exp = ref.residual_norms(0, nss)
    assert got.shape == exp.shape
    assert rel_err(got, exp) <= TOL
    s.close()


def test_implicit_skipped_last_subiteration(oracle_mod):
    """Steps without verification skip the residual-only last sub-iteration
    (computePT.cpp:581-582)."""
    t = cases.taylor_green(n=(8, 8, 8), ss_iteration=2)
    zd, ref, s = _pair(t, oracle_mod, 3)
    for it in range(1, 5):
        ref.compute(it, 1, 3, 1, modulo_verif=3)
        s.compute(it, 1, 3, 1, 1)
    _check_levels(ref, s)
    s.close()


def test_nit_c_loop(oracle_mod):
    t = cases.isentropic_vortex(n=(16, 16, 4))
    zd, ref, s = _pair(t, oracle_mod, 1000)
    ref.compute(0, 1, 3, 4, modulo_verif=1000)
    s.compute(0, 1, 3, 1, 4)
    _check_levels(ref, s)
    s.close()


def test_fasts_api_roundtrip(oracle_mod):
    """warmup / _compute / display_temporal_criteria / convergence history
    through the FastS-style API, against the oracle."""
    t = cases.taylor_green(n=(10, 8, 6), ss_iteration=2)
    t2 = cases.taylor_green(n=(10, 8, 6), ss_iteration=2)
    zd, ref, _ = _pair(t2, oracle_mod, 1)
    t, tc, metrics = fasts.warmup(t, None)
    fasts._createConvergenceHistory(t, 5)
    for it in range(1, 4):
        fasts._compute(t, metrics, it)
        ref.compute(it, 1, 3, 1, modulo_verif=1)
        fasts.display_temporal_criteria(t, metrics, it, format="store")
    from fast_gb300 import fastc, pytree as I
    z = I.getZones(t)[0]
    assert rel_err(fastc.compactArray(z, "").reshape(-1), ref.z[0]["lv"][0]) <= TOL
    ch = I.getNodeFromName1(z, "ZoneConvergenceHistory")
    assert int(I.getValue(ch)) == 3


def test_errors_are_reported_not_fatal():
    from fast_gb300._native import FastGB300Error, Solver
    s = Solver(0)
    with pytest.raises(FastGB300Error):
        s.compute(1, 1, 3, 1, 1)          # no zone yet
    with pytest.raises(FastGB300Error):
        s.set_option("lu_precision", 16)
    with pytest.raises(FastGB300Error):
        s.set_option("no_such_option", 1)
    s.close()


def test_lu_persistent_equals_plane_launches(oracle_mod):
    """The dataflow sweep, the persistent grid-barrier sweep and the
    one-launch-per-hyperplane sweep give the same bits (same cell
    arithmetic, different schedules)."""
    from fast_gb300._native import Solver
    res = []
    for mode in (0, 1, 2):
        t = cases.taylor_green(n=(14, 12, 10), ss_iteration=3)
        zd, ref, s = _pair(t, oracle_mod, 1)
        s.set_option("lu_mode", mode)
        s.set_option("autotune", 0)
        for it in range(1, 3):
            s.compute(it, 1, 4, 1, 1)
        s.synchronize()
        res.append([s.download(0, lvl) for lvl in range(3)])
        s.close()
    for other in res[1:]:
        for a, b in zip(res[0], other):
            assert np.array_equal(a, b)


def test_mixed_precision_sweeps(oracle_mod):
    """FP32 LU-SGS sweeps inside the FP64 Newton loop: the residual (FP64)
    still contracts and the state stays within FP32 round-off of FP64."""
    t = cases.taylor_green(n=(16, 16, 16), ss_iteration=5)
    zd, ref, s = _pair(t, oracle_mod, 1)
    s.set_option("lu_precision", 32)
    ref.compute(1, 1, 6, 1, modulo_verif=1)
    s.compute(1, 1, 6, 1, 1)
    s.synchronize()
    r = s.residuals(0)
    assert np.all(r[:5, -1] < r[:5, 0])
    nd = int(zd[0]["pi"][41])
    mask = _interior_mask(zd[0]["pi"])
    got = s.download(0, 0).reshape(5, nd)[:, mask]
    exp = ref.z[0]["lv"][0].reshape(5, nd)[:, mask]
    # error of each variable on the scale of that variable (w starts at 0)
    scale = np.max(np.abs(exp), axis=1, keepdims=True)
    assert np.max(np.abs(got - exp) / scale) < 1e-5
    s.close()


@pytest.mark.parametrize("scheme,slope", [("roe_min", "minmod"), ("roe", "o3"), ("roe", "o1"),
                                          ("ausmpred", "o3")])
def test_curvilinear_explicit_rk3(oracle_mod, scheme, slope):
    """3-d general zone (periodic curvilinear mesh): face normals from the
    metric arrays, general Roe / AUSM+(P) faces."""
    t = cases.isentropic_vortex(n=(20, 16, 6), wavy=0.3,
                                numz={"scheme": scheme, "slope": slope, "time_step": 0.05})
    zd, ref, s = _pair(t, oracle_mod, 1000)
    assert int(zd[0]["pi"][25]) == 0
    for it in range(1, 4):
        ref.compute(it, 1, 3, 1, modulo_verif=1000)
        s.compute(it, 1, 3, 1, 1)
    _check_levels(ref, s)
    s.close()


@pytest.mark.parametrize("scheme,slope", [("ausmpred", "o3"), ("roe_min", "minmod")])
def test_curvilinear_implicit_lusgs(oracle_mod, scheme, slope):
    """LU-SGS on a 3-d general zone: B matrices from the cell normals,
    in-place upper sweep with the metric of the k+1 neighbour."""
    t = cases.taylor_green(n=(12, 10, 8), ss_iteration=3, scheme=scheme, slope=slope, wavy=0.3,
                           model="Euler")
    zd, ref, s = _pair(t, oracle_mod, 1)
    assert int(zd[0]["pi"][25]) == 0
    for it in range(1, 3):
        ref.compute(it, 1, 4, 1, modulo_verif=1)
        s.compute(it, 1, 4, 1, 1)
    _check_levels(ref, s)
    nss = int(zd[0]["pi"][58])
    assert rel_err(s.residuals(0), ref.residual_norms(0, nss)) <= TOL
    s.close()


@pytest.mark.parametrize("wall,model,scheme,slope,wavy", [
    ("BCWallInviscid", "Euler", "ausmpred", "o3", 0.0),
    ("BCWallViscous", "NSLaminar", "ausmpred", "o3", 0.0),
    ("BCWallInviscid", "Euler", "senseur", "o3", 0.3),
    ("BCWallViscous", "NSLaminar", "senseur", "o3", 0.3),
])
def test_bcs_explicit(oracle_mod, wall, model, scheme, slope, wavy):
    """Inflow, outflow, wall, farfield and periodic BCs on one zone
    (BCzone.cpp: bvbs_inflow / outflow / wall_* / farfield / periodique)."""
    t = cases.bc_box(n=(16, 12, 6), wall=wall, model=model, scheme=scheme, slope=slope,
                     wavy=wavy)
    zd, ref, s = _pair(t, oracle_mod, 1000)
    for lvl in range(2):   # ghost fill alone
        got = s.download(0, lvl)
        assert rel_err(got, ref.z[0]["lv"][lvl]) <= TOL
    for it in range(1, 4):
        ref.compute(it, 1, 3, 1, modulo_verif=1000)
        s.compute(it, 1, 3, 1, 1)
    _check_levels(ref, s)
    s.close()


@pytest.mark.parametrize("wall,model,wavy", [("BCWallViscous", "NSLaminar", 0.0),
                                             ("BCWallInviscid", "Euler", 0.3)])
def test_bcs_implicit(oracle_mod, wall, model, wavy):
    t = cases.bc_box(n=(12, 10, 6), wall=wall, model=model, wavy=wavy, temporal="implicit",
                     ss_iteration=3, scheme="ausmpred", slope="o3", time_step=0.05)
    zd, ref, s = _pair(t, oracle_mod, 1)
    for it in range(1, 3):
        ref.compute(it, 1, 4, 1, modulo_verif=1)
        s.compute(it, 1, 4, 1, 1)
    _check_levels(ref, s)
    s.close()


@pytest.mark.parametrize("scheme,slope", [("roe", "o3"), ("ausmpred", "o3")])
def test_curvilinear_viscous_explicit(oracle_mod, scheme, slope):
    """fluvisq_3dfull_{i,j,k}.for on a periodic curvilinear mesh."""
    t = cases.taylor_green(n=(12, 10, 8), wavy=0.3, reynolds=100.0, scheme=scheme, slope=slope,
                           dt=0.02, numb={"temporal_scheme": "explicit", "ss_iteration": 1,
                                          "modulo_verif": 1000})
    zd, ref, s = _pair(t, oracle_mod, 1000)
    assert int(zd[0]["pi"][25]) == 0 and int(zd[0]["pi"][27]) == 2
    for it in range(1, 4):
        ref.compute(it, 1, 3, 1, modulo_verif=1000)
        s.compute(it, 1, 3, 1, 1)
    _check_levels(ref, s)
    s.close()


def test_curvilinear_viscous_implicit_with_walls(oracle_mod):
    """Implicit LU-SGS, Navier-Stokes, curvilinear mesh, no-slip wall,
    inflow / outflow / farfield."""
    t = cases.bc_box(n=(12, 10, 6), wall="BCWallViscous", model="NSLaminar", wavy=0.3,
                     temporal="implicit", ss_iteration=3, scheme="ausmpred", slope="o3",
                     time_step=0.05, reynolds=500.0)
    zd, ref, s = _pair(t, oracle_mod, 1)
    for it in range(1, 3):
        ref.compute(it, 1, 4, 1, modulo_verif=1)
        s.compute(it, 1, 4, 1, 1)
    _check_levels(ref, s)
    s.close()


@pytest.mark.parametrize("wavy", [0.0, 0.3])
def test_senseur_explicit(oracle_mod, wavy):
    """senseur scheme: wiggle sensor (wiggle2001.for) on the first sub-step,
    AUSM faces with sensor-switched dissipation (SENSOR/fluFaceEuler.for)."""
    t = cases.taylor_green(n=(12, 10, 8), wavy=wavy, reynolds=200.0, scheme="senseur", slope="o3",
                           dt=0.02, numb={"temporal_scheme": "explicit", "ss_iteration": 1,
                                          "modulo_verif": 1000})
    zd, ref, s = _pair(t, oracle_mod, 1000)
    assert int(zd[0]["pi"][33]) == 2
    for it in range(1, 4):
        ref.compute(it, 1, 3, 1, modulo_verif=1000)
        s.compute(it, 1, 3, 1, 1)
    _check_levels(ref, s)
    s.close()


def test_senseur_implicit(oracle_mod):
    t = cases.taylor_green(n=(12, 10, 8), ss_iteration=3, scheme="senseur", slope="o3")
    zd, ref, s = _pair(t, oracle_mod, 1)
    for it in range(1, 3):
        ref.compute(it, 1, 4, 1, modulo_verif=1)
        s.compute(it, 1, 4, 1, 1)
    _check_levels(ref, s)
    s.close()


@pytest.mark.parametrize("wall,model,slope,wavy", [
    ("BCWallInviscid", "Euler", "minmod", 0.0),
    ("BCWall", "Euler", "o3", 0.3),
    ("BCWallViscous", "NSLaminar", "o3", 0.0),
    ("BCWallViscous", "NSLaminar", "minmod", 0.3),
])
def test_roe_wall_flux_correction(oracle_mod, wall, model, slope, wavy):
    """Roe with wall BCs: the balance's Euler flux at wall faces is replaced
    by the wall flux (BC/correct_flux.for, bflwallslip.for / bflwall.for)."""
    t = cases.bc_box(n=(14, 10, 6), wall=wall, model=model, scheme="roe", slope=slope, wavy=wavy)
    zd, ref, s = _pair(t, oracle_mod, 1000)
    for it in range(1, 4):
        ref.compute(it, 1, 3, 1, modulo_verif=1000)
        s.compute(it, 1, 3, 1, 1)
    _check_levels(ref, s)
    s.close()


def test_roe_wall_flux_correction_implicit(oracle_mod):
    t = cases.bc_box(n=(12, 10, 6), wall="BCWallViscous", model="NSLaminar", scheme="roe_min",
                     slope="minmod", temporal="implicit", ss_iteration=3, time_step=0.05,
                     reynolds=500.0)
    zd, ref, s = _pair(t, oracle_mod, 1)
    for it in range(1, 3):
        ref.compute(it, 1, 4, 1, modulo_verif=1)
        s.compute(it, 1, 4, 1, 1)
    _check_levels(ref, s)
    s.close()


@pytest.mark.parametrize("scheme,slope,wavy", [("roe_min", "minmod", 0.0), ("roe", "o3", 0.3),
                                               ("ausmpred", "o3", 0.3), ("senseur", "o3", 0.3)])
def test_2d_explicit(oracle_mod, scheme, slope, wavy):
    """2-d zones (ITYPZONE 3): i and j faces only, no w."""
    t = cases.isentropic_vortex(n=(24, 20, 1), two_d=True, wavy=wavy,
                                numz={"scheme": scheme, "slope": slope, "time_step": 0.05})
    zd, ref, s = _pair(t, oracle_mod, 1000)
    assert int(zd[0]["pi"][25]) == 3
    for it in range(1, 4):
        ref.compute(it, 1, 3, 1, modulo_verif=1000)
        s.compute(it, 1, 3, 1, 1)
    _check_levels(ref, s)
    s.close()


@pytest.mark.parametrize("scheme,slope,wavy", [("ausmpred", "o3", 0.0), ("roe_min", "minmod", 0.3),
                                               ("senseur", "o3", 0.3)])
def test_2d_implicit(oracle_mod, scheme, slope, wavy):
    """LU-SGS on 2-d zones (lu_{i,j}_2d.for, 2-d Newton update)."""
    t = cases.isentropic_vortex(n=(20, 16, 1), two_d=True, wavy=wavy,
                                numb={"temporal_scheme": "implicit", "ss_iteration": 3,
                                      "modulo_verif": 1},
                                numz={"scheme": scheme, "slope": slope, "time_step": 0.2})
    zd, ref, s = _pair(t, oracle_mod, 1)
    for it in range(1, 3):
        ref.compute(it, 1, 4, 1, modulo_verif=1)
        s.compute(it, 1, 4, 1, 1)
    _check_levels(ref, s)
    nss = int(zd[0]["pi"][58])
    assert rel_err(s.residuals(0), ref.residual_norms(0, nss)) <= TOL
    s.close()


@pytest.mark.parametrize("scheme,slope,temporal", [("ausmpred", "o3", "explicit"),
                                                   ("roe", "o3", "explicit"),
                                                   ("roe_min", "minmod", "implicit")])
def test_2d_bcs(oracle_mod, scheme, slope, temporal):
    """2-d zone with inflow, outflow, slip wall (Roe: wall-face correction)
    and farfield on a curvilinear mesh."""
    t = cases.bc_box(n=(16, 12, 1), two_d=True, wall="BCWallInviscid", model="Euler", scheme=scheme,
                     slope=slope, wavy=0.3, temporal=temporal, ss_iteration=3,
                     time_step=0.02 if temporal == "explicit" else 0.05)
    mv = 1000 if temporal == "explicit" else 1
    zd, ref, s = _pair(t, oracle_mod, mv)
    nfin = 3 if temporal == "explicit" else 4
    for it in range(1, 3):
        ref.compute(it, 1, nfin, 1, modulo_verif=mv)
        s.compute(it, 1, nfin, 1, 1)
    _check_levels(ref, s)
    s.close()


@pytest.mark.parametrize("wall,wavy", [("BCWallViscous", 0.0), ("BCWallViscous", 0.3),
                                       ("BCWallInviscid", 0.3)])
def test_spalart_allmaras_explicit(oracle_mod, wall, wavy):
    """Spalart-Allmaras RK3 steps with inflow / outflow / wall / farfield:
    AUSM+(P) flux of ro nutilde, nutilde diffusion, the source term of
    spsource_SA.for, the clipped update and the SA ghost fill."""
    t = cases.bc_box(n=(16, 12, 6), model="NSTurbulent", wall=wall, wavy=wavy,
                     temporal="explicit", reynolds=500.0, time_step=0.02)
    zd, ref, s = _pair(t, oracle_mod, 1000)
    pi = zd[0]["pi"]
    assert int(pi[36]) == 6
    for lvl in range(2):
        assert rel_err(s.download(0, lvl), ref.z[0]["lv"][lvl]) <= TOL
    for it in range(1, 4):
        ref.compute(it, 1, 3, 1, modulo_verif=1000)
        s.compute(it, 1, 3, 1, 1)
    _check_levels(ref, s)
    nd = int(pi[41])
    mask = _interior_mask(pi)
    xm = s.work(0, "xmut", nd)
    assert rel_err(xm[mask], ref.z[0]["xmut"][:nd][mask]) <= TOL
    s.close()


@pytest.mark.parametrize("scheme,slope,temporal,wavy", [
    ("roe", "o3", "explicit", 0.0), ("roe_min", "minmod", "explicit", 0.3),
    ("roe", "o1", "implicit", 0.3), ("roe", "o3", "implicit", 0.0),
    ("senseur", "o3", "explicit", 0.3), ("senseur", "o3", "implicit", 0.0)])
def test_spalart_allmaras_roe(oracle_mod, scheme, slope, temporal, wavy):
    """Roe with Spalart-Allmaras (ROE/*/fluFaceSA_*.for: first-order ro
    nutilde flux upwinded by the Roe-averaged normal velocity), no-slip wall
    with the Roe wall-face correction, inflow / outflow / farfield; and the
    senseur with SA (SENSOR/*/fluFaceSA_o3_*.for: the AUSM form of the ro
    nutilde flux with the sensor's interface velocity and dissipation)."""
    t = cases.bc_box(n=(14, 10, 6), model="NSTurbulent", scheme=scheme, slope=slope, wavy=wavy,
                     temporal=temporal, ss_iteration=3, reynolds=500.0,
                     time_step=0.02 if temporal == "explicit" else 0.05)
    mv = 1000 if temporal == "explicit" else 1
    zd, ref, s = _pair(t, oracle_mod, mv)
    assert int(zd[0]["pi"][36]) == 6 and int(zd[0]["pi"][33]) in (5, 2)
    nfin = 3 if temporal == "explicit" else 4
    for it in range(1, 4):
        ref.compute(it, 1, nfin, 1, modulo_verif=mv)
        s.compute(it, 1, nfin, 1, 1)
    _check_levels(ref, s)
    s.close()


@pytest.mark.parametrize("wavy", [0.0, 0.3])
def test_spalart_allmaras_implicit(oracle_mod, wavy):
    """Spalart-Allmaras with LU-SGS: coe6 from the source Jacobian, the
    sixth row of the sweeps (lu_*_SA.for), mjr_newton_SA.for."""
    t = cases.bc_box(n=(12, 10, 6), model="NSTurbulent", wavy=wavy, temporal="implicit",
                     ss_iteration=3, reynolds=500.0, time_step=0.05)
    zd, ref, s = _pair(t, oracle_mod, 1)
    for it in range(1, 3):
        ref.compute(it, 1, 4, 1, modulo_verif=1)
        s.compute(it, 1, 4, 1, 1)
    _check_levels(ref, s)
    pi = zd[0]["pi"]
    nd = int(pi[41])
    mask = _interior_mask(pi)
    coe = s.work(0, "coe", 6 * nd).reshape(6, nd)
    assert rel_err(coe[:, mask], ref.z[0]["coe"].reshape(6, nd)[:, mask]) <= TOL
    nss = int(pi[58])
    assert rel_err(s.residuals(0), ref.residual_norms(0, nss)) <= TOL
    s.close()


def test_spalart_allmaras_periodic_lusgs_plane_launches(oracle_mod):
    """Periodic SA box, persistent sweeps and one launch per hyperplane."""
    t = cases.taylor_green(n=(10, 9, 8), ss_iteration=3, model="NSTurbulent", wall_distance=2.0)
    zd, ref, s = _pair(t, oracle_mod, 1)
    s.set_option("lu_mode", 0)
    for it in range(1, 3):
        ref.compute(it, 1, 4, 1, modulo_verif=1)
        s.compute(it, 1, 4, 1, 1)
    _check_levels(ref, s)
    s.close()


def test_spalart_allmaras_mixed_precision(oracle_mod):
    """FP32 sweeps with the sixth equation: contraction and FP32-level error."""
    t = cases.bc_box(n=(16, 12, 8), model="NSTurbulent", temporal="implicit", ss_iteration=5,
                     reynolds=500.0, time_step=0.05)
    zd, ref, s = _pair(t, oracle_mod, 1)
    s.set_option("lu_precision", 32)
    ref.compute(1, 1, 6, 1, modulo_verif=1)
    s.compute(1, 1, 6, 1, 1)
    s.synchronize()
    r = s.residuals(0)
    assert np.all(r[:6, -1] < r[:6, 0])
    nd = int(zd[0]["pi"][41])
    mask = _interior_mask(zd[0]["pi"])
    got = s.download(0, 0).reshape(6, nd)[:, mask]
    exp = ref.z[0]["lv"][0].reshape(6, nd)[:, mask]
    scale = np.max(np.abs(exp), axis=1, keepdims=True)
    assert np.max(np.abs(got - exp) / scale) < 1e-5
    s.close()


def test_spalart_allmaras_refusals():
    """Unsupported SA combinations are reported, never run: AUSM+(P) with a
    minmod slope, and a compute before the wall distance is given."""
    from fast_gb300._native import Solver, FastGB300Error
    t = cases.bc_box(n=(8, 8, 6), model="NSTurbulent", scheme="ausmpred", slope="minmod",
                     temporal="explicit")
    zd = fasts.zone_data(t, fasts.prepare(t))
    s = Solver(0)
    with pytest.raises(FastGB300Error, match="Spalart-Allmaras is supported"):
        s.add_zone(zd[0]["pi"], zd[0]["pr"], zd[0]["ti"], zd[0]["tj"], zd[0]["tk"], zd[0]["vol"])
    t = cases.bc_box(n=(8, 8, 6), model="NSTurbulent", temporal="explicit")
    zd = fasts.zone_data(t, fasts.prepare(t))
    s.add_zone(zd[0]["pi"], zd[0]["pr"], zd[0]["ti"], zd[0]["tj"], zd[0]["tk"], zd[0]["vol"])
    with pytest.raises(FastGB300Error, match="wall distance"):
        s.compute(1, 1, 3, 1, 1)
    s.close()


CHANNEL = dict(sizes=((4, 9), (4, 7), (4, 6)), first_cell=2e-2, reynolds=2000.0)


@pytest.mark.parametrize("temporal", ["explicit", "implicit"])
def test_channel_sa_multiblock(oracle_mod, temporal):
    """48-block SA channel (uneven general 3-d blocks, 1-to-1 interfaces
    including the z period, inflow / outflow / no-slip walls)."""
    kw = dict(CHANNEL, temporal=temporal, ss_iteration=3,
              time_step=0.004 if temporal == "explicit" else 0.02,
              modulo_verif=1000 if temporal == "explicit" else 1)
    t, tc = cases.sa_channel(**kw)
    zd, ref, s = _pair(t, oracle_mod, kw["modulo_verif"], tc)
    assert len(zd) == 48
    nfin = 3 if temporal == "explicit" else 4
    for it in range(1, 3):
        ref.compute(it, 1, nfin, 1, modulo_verif=kw["modulo_verif"])
        s.compute(it, 1, nfin, 1, 1)
    for m in range(len(zd)):
        _check_levels(ref, s, zone=m)
        if temporal == "implicit":
            nss = int(zd[m]["pi"][58])
            assert rel_err(s.residuals(m), ref.residual_norms(m, nss)) <= TOL
    s.close()


def test_channel_inviscid_multiblock_equals_single_block():
    """On the GPU: the 48-block inviscid channel step equals the single-block
    step of the same mesh, cell for cell."""
    from fast_gb300._native import Solver
    kw = dict(CHANNEL, model="Euler", wall="BCWallInviscid", temporal="explicit",
              time_step=0.004, modulo_verif=1000)
    t, tc = cases.sa_channel(**kw)
    blocks = cases.channel_blocks(t)
    N = [max(o[d] + n[d] for _, o, n in blocks) for d in range(3)]
    t1, tc1 = cases.sa_channel(parts=[[N[0]], [N[1]], [N[2]]], **kw)
    out = []
    for tt, cc in ((t, tc), (t1, tc1)):
        zd = fasts.zone_data(tt, fasts.prepare(tt))
        s = Solver(0)
        for n, z in enumerate(zd):
            s.add_zone(z["pi"], z["pr"], z["ti"], z["tj"], z["tk"], z["vol"])
            for lvl, key in enumerate(("ro", "ro_m1", "ro_p1")):
                s.upload(n, lvl, z[key])
        for tr in cc:
            s.add_transfer(tr["dnr"], tr["rcv"], tr["dnr_idx"], tr["rcv_idx"])
        s.set_option("modulo_verif", 1000)
        s.apply_bc(0)
        s.apply_bc(1)
        for it in range(1, 4):
            s.compute(it, 1, 3, 1, 1)
        s.synchronize()
        G = np.zeros((5, N[2], N[1], N[0]))
        for m, o, n in cases.channel_blocks(tt):
            pi = zd[m]["pi"]
            ni, nj, nk = int(pi[0]), int(pi[1]), int(pi[2])
            q = s.download(m, 0).reshape(5, nk, nj, ni)[:, 2:-2, 2:-2, 2:-2]
            G[:, o[2]:o[2] + n[2], o[1]:o[1] + n[1], o[0]:o[0] + n[0]] = q
        out.append(G)
        s.close()
    assert np.array_equal(out[0], out[1])


@pytest.mark.parametrize("wavy,two_d", [(0.0, False), (0.3, False), (0.3, True)])
def test_roe_vanalbada_explicit(oracle_mod, wavy, two_d):
    """Roe + van Albada MUSCL (slope 8, the smooth limiter of the adjoint
    path) on cartesian, curvilinear and 2-d zones."""
    n = (20, 16, 1) if two_d else (20, 16, 6)
    t = cases.isentropic_vortex(n=n, wavy=wavy, two_d=two_d,
                                numz={"scheme": "roe", "slope": "vanalbada", "time_step": 0.05})
    zd, ref, s = _pair(t, oracle_mod, 1000)
    assert int(zd[0]["pi"][64]) == 8
    for it in range(1, 4):
        ref.compute(it, 1, 3, 1, modulo_verif=1000)
        s.compute(it, 1, 3, 1, 1)
    _check_levels(ref, s)
    s.close()


@pytest.mark.parametrize("case", ["tgv_implicit", "wavy_sa", "vortex_2d", "box_2d_laminar"])
def test_cfl_statistics(oracle_mod, case):
    """cpcfl3.for on the GPU (fgb_cfl) against the oracle: max and min bit
    for bit, the mean (a reduction in another order) to 1e-12."""
    if case == "tgv_implicit":
        t = cases.taylor_green(n=(12, 10, 8), ss_iteration=2)
        nfin, mv = 3, 1
    elif case == "wavy_sa":
        t = cases.bc_box(n=(12, 10, 6), model="NSTurbulent", wavy=0.3, temporal="explicit",
                         reynolds=500.0, time_step=0.02)
        nfin, mv = 3, 1
    elif case == "vortex_2d":
        t = cases.isentropic_vortex(n=(24, 20, 1), two_d=True, wavy=0.3,
                                    numz={"scheme": "roe", "slope": "o3", "time_step": 0.05})
        nfin, mv = 3, 1
    else:
        t = cases.bc_box(n=(16, 12, 1), two_d=True, model="NSLaminar", wavy=0.3,
                         temporal="explicit", reynolds=100.0, time_step=0.01)
        nfin, mv = 3, 1
    zd, ref, s = _pair(t, oracle_mod, mv)
    for it in range(1, 3):
        ref.compute(it, 1, nfin, 1, modulo_verif=mv)
        s.compute(it, 1, nfin, 1, 1)
    got, exp = s.cfl(0), ref.cfl(0)
    assert got[0] == exp[0] and got[1] == exp[1], (got, exp)
    assert abs(got[2] - exp[2]) <= 1e-12 * exp[2]
    assert 0 < exp[1] <= exp[2] <= exp[0]
    s.close()


@pytest.mark.parametrize("temporal", ["explicit", "implicit"])
def test_zone_batches_equal_per_zone_launches(oracle_mod, temporal):
    """Several zones: the per-kind zone batches (one launch of each kernel
    over the zones of one kind, face block size from the autotuner) give the
    bits of the per-zone launches."""
    kw = dict(CHANNEL, temporal=temporal, ss_iteration=3,
              time_step=0.004 if temporal == "explicit" else 0.02, modulo_verif=1)
    out = []
    for batch in (0, 1):
        t, tc = cases.sa_channel(**kw)
        zd, ref, s = _pair(t, oracle_mod, 1, tc)
        s.set_option("batch", batch)
        nfin = 3 if temporal == "explicit" else 4
        for it in range(1, 3):
            s.compute(it, 1, nfin, 1, 1)
        s.synchronize()
        out.append([s.download(m, lvl) for m in range(len(zd)) for lvl in range(3)])
        if temporal == "implicit":
            out[-1] += [s.residuals(m) for m in range(len(zd))]
        s.close()
    for a, b in zip(*out):
        assert np.array_equal(a, b)
