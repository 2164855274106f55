"""Interface connectivity from a Connector ``tc`` tree, and the overset
(non-type-0) interpolated transfers.

The reference reads its transfers from the tc donor tree
(FastS/FastS/PyTree.py:42-55; FastC/FastC/Com/setInterpTransfersFast.cpp:
440-960); the interpolation arithmetic itself is in Cassiopee Connector,
which is not part of the reference tree, so the tensor-product formulas are
restated (parity unpinned) and pinned here by known answers: every molecule
of degree >= 1 reproduces a field linear in x, y, z to round-off.  GPU tests
compare the sm_103a transfers and solve step with the oracle (1e-12 relative
per cell) and run _compute with a tc tree built by hand."""
import numpy as np
import pytest

from conftest import rel_err
from fast_gb300 import cases, connector, fasts
from fast_gb300 import pytree as I


def _face_band(tr, ni=24, nj=20):
    """Receivers of the patch's face bands (edge ghosts are then averaged
    by correct_coins.for)."""
    r = tr["rcv_idx"]
    nip, njp = ni + 4, nj + 4
    i, j = r % nip, (r // nip) % njp
    return ~(((i < 2) | (i >= ni + 2)) & ((j < 2) | (j >= nj + 2)))


@pytest.mark.parametrize("types", [(2,), (3,), (5,), (2, 3, 5)])
def test_interpolation_reproduces_linear_fields(oracle_mod, types):
    t, tc = cases.overset_patch(types=types, linear=True)
    zd = fasts.zone_data(t, fasts.prepare(t))
    c = oracle_mod.Case(zd, tc)
    c.apply_bc(0)
    z1 = I.getZones(t)[1]
    xc, yc, zc = cases.cell_centers(z1)
    X, Y, Z = (a.ravel(order="F") for a in (xc, yc, zc))
    q = c.z[1]["lv"][0].reshape(5, -1)
    r = tc[0]["rcv_idx"][_face_band(tc[0])]
    assert r.size > 100
    assert np.max(np.abs(q[0, r] - (1.0 + 0.01 * X[r] + 0.02 * Y[r] + 0.001 * Z[r]))) < 1e-14
    assert np.max(np.abs(q[1, r] - (0.5 + 0.003 * X[r]))) < 1e-14
    assert np.max(np.abs(q[2, r] - 0.002 * Y[r])) < 1e-14


@pytest.mark.parametrize("typ,exact,inexact", [(2, 1, 2), (3, 2, 4), (5, 4, None)])
def test_interpolation_polynomial_degree(oracle_mod, typ, exact, inexact):
    """Each molecule reproduces the polynomials of its degree to round-off
    and not those of the next one: trilinear (type 2) degree 1, the 27-point
    Lagrange molecule (type 3) degree 2, the 125-point one (type 5) degree 4
    in x and y."""
    def err(deg):
        t, tc = cases.overset_patch(types=(typ,), degree=deg)
        zd = fasts.zone_data(t, fasts.prepare(t))
        c = oracle_mod.Case(zd, tc)
        c.apply_bc(0)
        xc, yc, zc = cases.cell_centers(I.getZones(t)[1])
        X, Y, Z = (a.ravel(order="F") for a in (xc, yc, zc))
        q = c.z[1]["lv"][0].reshape(5, -1)
        r = tc[0]["rcv_idx"][_face_band(tc[0])]
        ro, u, v, T = cases.poly_field(X[r], Y[r], Z[r], deg)
        return max(float(np.max(np.abs(q[k, r] - f))) for k, f in ((0, ro), (1, u), (2, v), (4, T)))
    assert err(exact) < 1e-13
    if inexact is not None:
        assert err(inexact) > 1e-7


def test_tc_tree_round_trip():
    """connector.tc_tree writes the ID_ subregions FastS's tests build by
    hand; transfers_from_tc reads back the same arrays, a 1-to-1 list as
    plain copies."""
    t, tc = cases.overset_patch(types=(2, 3))
    back = connector.transfers_from_tc(t, connector.tc_tree(t, tc))
    assert len(back) == 1
    for k in ("dnr_idx", "rcv_idx", "types", "coefs"):
        assert np.array_equal(back[0][k], tc[0][k])
    t2, tc2 = cases.sa_channel(parts=[[5, 4], [6], [4]], first_cell=2e-2, reynolds=2000.0,
                               temporal="explicit", time_step=0.004, modulo_verif=1000)
    tree = connector.tc_tree(t2, tc2)
    sub = I.getNodesFromType(tree, "ZoneSubRegion_t")
    assert len(sub) == len(tc2)
    assert {c[0] for c in sub[0][2]} >= {"PointList", "PointListDonor", "InterpolantsType",
                                         "InterpolantsDonor"}
    back = connector.transfers_from_tc(t2, tree)
    assert all("types" not in b for b in back)
    key = lambda d: (d["dnr"], d["rcv"], int(d["rcv_idx"][0]))
    for a, b in zip(sorted(back, key=key), sorted(tc2, key=key)):
        assert (a["dnr"], a["rcv"]) == (b["dnr"], b["rcv"])
        assert np.array_equal(a["dnr_idx"], b["dnr_idx"]) and np.array_equal(a["rcv_idx"], b["rcv_idx"])


def test_tc_tree_rejects_unknown_types():
    t, tc = cases.overset_patch(types=(2,))
    tree = connector.tc_tree(t, tc)
    ty = I.getNodeFromName(tree, "InterpolantsType")
    ty[1] = np.full_like(ty[1], 4)
    with pytest.raises(ValueError, match="not supported"):
        connector.transfers_from_tc(t, tree)


@pytest.mark.gpu
@pytest.mark.parametrize("types", [(2,), (3,), (5,), (1, 2, 3, 5)])
def test_overset_gpu_parity(oracle_mod, types):
    from test_gpu_parity import TOL, _check_levels, _pair
    t, tc = cases.overset_patch(types=types,
                                numz={"scheme": "roe_min", "slope": "minmod", "time_step": 0.02,
                                      "cache_blocking_I": 1000000, "cache_blocking_J": 1000000,
                                      "cache_blocking_K": 1000000})
    zd, ref, s = _pair(t, oracle_mod, 1000, tc)
    for m in range(2):
        for lvl in range(2):
            assert rel_err(s.download(m, lvl), ref.z[m]["lv"][lvl]) <= TOL
    for it in range(1, 4):
        ref.compute(it, 1, 3, 1, modulo_verif=1000)
        s.compute(it, 1, 3, 1, 1)
    for m in range(2):
        _check_levels(ref, s, zone=m)
    s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["one_to_one", "overset"])
def test_compute_with_tc_tree(oracle_mod, case):
    """FastS's call sequence with a tc tree: warmup(t, tc) then
    _compute(t, metrics, it, tc), against the oracle fed the same
    transfers."""
    from fast_gb300 import fastc
    if case == "one_to_one":
        mk = lambda: cases.sa_channel(parts=[[5, 4], [6], [4]], first_cell=2e-2, reynolds=2000.0,
                                      temporal="implicit", ss_iteration=3, time_step=0.02,
                                      modulo_verif=1)
    else:
        mk = lambda: cases.overset_patch(types=(2, 3))
    t, tcl = mk()
    t2, tcl2 = mk()
    tc = connector.tc_tree(t, tcl)
    zd2 = fasts.zone_data(t2, fasts.prepare(t2))
    ref = oracle_mod.Case(zd2, tcl2)
    ref.apply_bc(0)
    ref.apply_bc(1)
    t, tc, metrics = fasts.warmup(t, tc)
    nss = fasts.HOOK["nssiter"]
    mv = 1 if case == "one_to_one" else 1000000
    for it in range(1, 3):
        fasts._compute(t, metrics, it, tc)
        ref.compute(it, 1, nss, 1, modulo_verif=mv)
    for m, z in enumerate(I.getZones(t)):
        assert rel_err(fastc.compactArray(z, "").reshape(-1), ref.z[m]["lv"][0]) <= 1e-12
    fasts.HOOK["solver"].close()
    fasts.HOOK = None
