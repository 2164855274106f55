"""BC data (nbdata > 0) and the imposed-pressure outflow BCOutpres (tag 16).

BCzone.cpp:26-53 (DEFAULT_STATE): a farfield / inflow / outflow state is the
free stream without data, values 3..7 (and 16 for nutilde) of 21 one-value
arrays, else the first values of the data; BCzone.cpp:758-792 with
BC/bvbs_outpres.for, BCOutpres_i.for and linearization_state.for: the first
ghost rank takes the imposed pressure of its face through the normal
characteristic linearised about the interior state, the next ranks copy it.

CPU: the packing of the data by _BCcompact, and known answers of the
oracle.  GPU: the sm_103a ghost fill and solve step against the oracle
(1e-12 relative per cell, as the other parity tests)."""
import numpy as np
import pytest

from conftest import rel_err
from fast_gb300 import cases, fasts
from fast_gb300 import pytree as I


def _zd(t):
    return fasts.zone_data(t, fasts.prepare(t))


def _bc_block(pi, tag):
    pt_bcs = int(pi[70])
    nb = int(pi[pt_bcs])
    for n in range(nb):
        pt = int(pi[pt_bcs + 1 + n])
        if int(pi[pt]) == tag:
            return pt, int(pi[pt_bcs + 1 + n + nb])
    raise KeyError(tag)


@pytest.mark.parametrize("form", [1, 2])
def test_outpres_data_packing(form):
    t = cases.bc_box(n=(8, 6, 4), outflow="BCOutpres", outpres_form=form)
    zd = _zd(t)
    pi, pr = zd[0]["pi"], zd[0]["pr"]
    pt, off = _bc_block(pi, 16)
    assert int(pi[pt + 8]) == form                 # nbdata
    nf = 6 * 4
    if form == 1:
        assert int(pi[pt + 9]) == nf
        p = pr[off:off + nf]
    else:
        assert (int(pi[pt + 9]), int(pi[pt + 10])) == (1, 1 + nf)
        assert pr[off] == 1.0
        p = pr[off + 1:off + 1 + nf]
    yf = (np.arange(6) + 0.5) / 6
    assert np.allclose(p.reshape(4, 6), (1.0 + 0.02 * np.sin(2 * np.pi * yf)) / 1.4, rtol=0, atol=1e-15)


def test_outpres_free_stream_known_answer(oracle_mod):
    """With the free stream and the free-stream pressure imposed, every ghost
    of the BCOutpres window holds the interior state (dqn = 0) and the flow
    stays the free stream."""
    t = cases.bc_box(n=(12, 10, 6), perturb=0.0, wall="BCWallInviscid", model="Euler",
                     outflow="BCOutpres", outpres_amp=0.0)
    zd = _zd(t)
    c = oracle_mod.Case(zd)
    c.apply_bc(0)
    pi = zd[0]["pi"]
    ni, nj, nk = (int(pi[0]), int(pi[1]), int(pi[2]))
    q = c.z[0]["lv"][0].reshape(5, nk, nj, ni)
    for g in (ni - 2, ni - 1):
        assert np.max(np.abs(q[:, 2:-2, 2:-2, g] - q[:, 2:-2, 2:-2, ni - 3])) < 1e-15
    q0 = c.z[0]["lv"][0].copy()
    c.apply_bc(1)
    for it in range(1, 4):
        c.compute(it, 1, 3, 1, modulo_verif=1000)
    assert np.max(np.abs(c.z[0]["lv"][0] - q0)) < 1e-14


def test_outpres_ghost_pressure(oracle_mod):
    """The first ghost rank carries the imposed pressure of its face
    (p = ro rgp T = pext) and the next rank repeats it."""
    t = cases.bc_box(n=(10, 8, 4), model="Euler", wall="BCWallInviscid", outflow="BCOutpres")
    zd = _zd(t)
    c = oracle_mod.Case(zd)
    c.apply_bc(0)
    pi, pr = zd[0]["pi"], zd[0]["pr"]
    ni, nj, nk = (int(pi[0]), int(pi[1]), int(pi[2]))
    q = c.z[0]["lv"][0].reshape(5, nk, nj, ni)
    rgp = pr[2] * (pr[1] - 1.0)
    p = q[0, 2:-2, 2:-2, ni - 2] * rgp * q[4, 2:-2, 2:-2, ni - 2]
    yf = (np.arange(nj - 4) + 0.5) / (nj - 4)
    pext = (1.0 + 0.02 * np.sin(2 * np.pi * yf)) / 1.4
    assert np.max(np.abs(p - pext[None, :])) < 1e-14
    assert np.array_equal(q[:, 2:-2, 2:-2, ni - 1], q[:, 2:-2, 2:-2, ni - 2])


def test_bc_state_data_known_answer(oracle_mod):
    """A farfield whose BC data state is the free stream itself leaves the
    free stream unchanged; a different data state changes the ghosts."""
    t = cases.bc_box(n=(10, 8, 4), perturb=0.0, model="Euler", wall="BCWallInviscid")
    zd0 = _zd(t)
    c0 = oracle_mod.Case(zd0)
    c0.apply_bc(0)
    t = cases.bc_box(n=(10, 8, 4), perturb=0.0, model="Euler", wall="BCWallInviscid", bc_data=True)
    zd1 = _zd(t)
    c1 = oracle_mod.Case(zd1)
    c1.apply_bc(0)
    a, b = c0.z[0]["lv"][0], c1.z[0]["lv"][0]
    assert np.max(np.abs(a - b)) > 1e-4
    pi = zd1[0]["pi"]
    pt, off = _bc_block(pi, 13)
    assert int(pi[pt + 8]) == 21


GPU_CASES = [
    dict(outflow="BCOutpres", model="Euler", wall="BCWallInviscid"),
    dict(outflow="BCOutpres", outpres_form=2, model="NSLaminar"),
    dict(outflow="BCOutpres", model="NSTurbulent", wavy=0.3),
    dict(bc_data=True, model="Euler", wall="BCWallInviscid", wavy=0.3),
    dict(bc_data=True, model="NSTurbulent"),
    dict(bc_data=True, outflow="BCOutpres", model="NSLaminar", two_d=True, n=(14, 10, 1)),
]


@pytest.mark.gpu
@pytest.mark.parametrize("kw", GPU_CASES)
@pytest.mark.parametrize("temporal", ["explicit", "implicit"])
def test_bc_data_gpu_parity(oracle_mod, kw, temporal):
    from test_gpu_parity import TOL, _check_levels, _pair
    kw = dict(kw)
    kw.setdefault("n", (14, 10, 6))
    t = cases.bc_box(temporal=temporal, ss_iteration=3, time_step=0.02 if temporal == "explicit" else 0.05,
                     **kw)
    zd, ref, s = _pair(t, oracle_mod, 1)
    for lvl in range(2):   # ghost fill alone
        assert rel_err(s.download(0, lvl), ref.z[0]["lv"][lvl]) <= TOL
    nfin = 3 if temporal == "explicit" else 4
    for it in range(1, 3):
        ref.compute(it, 1, nfin, 1, modulo_verif=1)
        s.compute(it, 1, nfin, 1, 1)
    _check_levels(ref, s)
    s.close()


@pytest.mark.gpu
def test_bc_data_refusals():
    """Data the GPU path does not read are refused, not ignored: BCOutpres
    without its pressure, and BCInflow with per-face data."""
    from fast_gb300._native import FastGB300Error, Solver
    from fast_gb300 import pytree as I
    t = cases.bc_box(n=(8, 6, 4), outflow="BCOutpres")
    bc = [b for b in I.getNodesFromType(t, "BC_t") if I.getValue(b) == "BCOutpres"][0]
    bc[2] = [c for c in bc[2] if c[3] != "BCDataSet_t"]
    zd = _zd(t)
    s = Solver(0)
    with pytest.raises(FastGB300Error, match="BCOutpres"):
        s.add_zone(zd[0]["pi"], zd[0]["pr"], zd[0]["ti"], zd[0]["tj"], zd[0]["tk"], zd[0]["vol"])
    s.close()


def test_homogeneous_k_zone_runs_as_general_zone():
    """A wall-stretched box is a zone homogeneous in k (nature_geom_dom.for
    type 1); it is solved by the general 3-d kernels on its full metric."""
    t = cases.bc_box(n=(12, 10, 6), model="NSLaminar", stretch=2.0)
    z = I.getZones(t)[0]
    assert fasts._zone_type(*fasts._coords(z), I.getZoneDim(z)[3]) == 1
    zd = _zd(t)
    assert int(zd[0]["pi"][25]) == 0


@pytest.mark.gpu
@pytest.mark.parametrize("temporal", ["explicit", "implicit"])
def test_homogeneous_k_zone_gpu_parity(oracle_mod, temporal):
    from test_gpu_parity import _check_levels, _pair
    t = cases.bc_box(n=(14, 10, 6), model="NSLaminar", stretch=2.0, temporal=temporal,
                     ss_iteration=3, time_step=0.02 if temporal == "explicit" else 0.05)
    zd, ref, s = _pair(t, oracle_mod, 1)
    nfin = 3 if temporal == "explicit" else 4
    for it in range(1, 3):
        ref.compute(it, 1, nfin, 1, modulo_verif=1)
        s.compute(it, 1, nfin, 1, 1)
    _check_levels(ref, s)
    s.close()
