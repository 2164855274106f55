"""The multi-block Spalart-Allmaras channel (48 blocks of a seeded random
box decomposition, 1-to-1 interfaces) on the CPU: the decomposition and its
interface lists, and the oracle's known answer for the 1-to-1 copy -- an
inviscid multi-block step equals the single-block step of the same mesh
cell for cell (the inviscid stencils are one-dimensional, so every value a
block reads across an interface is the neighbour's interior value)."""
import numpy as np
import pytest

from fast_gb300 import cases, fasts

SMALL = dict(sizes=((4, 9), (4, 7), (4, 6)), first_cell=2e-2, reynolds=2000.0)


def test_channel_decomposition():
    t, tc = cases.sa_channel()
    blocks = cases.channel_blocks(t)
    assert len(blocks) == 48
    for _, _, n in blocks:
        assert 16 <= n[0] <= 96 and 16 <= n[1] <= 64 and 16 <= n[2] <= 32
    zd = fasts.zone_data(t, fasts.prepare(t))
    assert {int(z["pi"][25]) for z in zd} == {0}          # general 3-d zones
    assert {int(z["pi"][36]) for z in zd} == {6}          # Spalart-Allmaras
    # every block face inside the channel or on the z period is an interface
    # (48 x 6 faces minus 12 inflow, 12 outflow, 16 + 16 wall faces), each
    # with two ghost layers of its face
    assert len(tc) == 48 * 6 - 2 * (3 * 4) - 2 * (4 * 4)
    for tr in tc:
        rz, dz = zd[tr["rcv"]], zd[tr["dnr"]]
        n = [int(v) for v in rz["pi"][20:23]]
        assert tr["rcv_idx"].size == tr["dnr_idx"].size
        assert tr["rcv_idx"].size in (2 * n[1] * n[2], 2 * n[0] * n[2], 2 * n[0] * n[1])
        assert tr["rcv_idx"].max() < int(rz["pi"][41]) and tr["dnr_idx"].max() < int(dz["pi"][41])


def _global_interior(t, zd, states):
    blocks = cases.channel_blocks(t)
    N = [max(o[d] + n[d] for _, o, n in blocks) for d in range(3)]
    nv = int(zd[0]["pi"][36])
    G = np.zeros((nv, N[2], N[1], N[0]))
    for m, o, n in blocks:
        pi = zd[m]["pi"]
        ni, nj, nk = int(pi[0]), int(pi[1]), int(pi[2])
        q = states[m].reshape(nv, nk, nj, ni)[:, 2:-2, 2:-2, 2:-2]
        G[:, o[2]:o[2] + n[2], o[1]:o[1] + n[1], o[0]:o[0] + n[0]] = q
    return G, N


def test_multiblock_equals_single_block_inviscid(oracle_mod):
    kw = dict(SMALL, model="Euler", wall="BCWallInviscid", temporal="explicit", time_step=0.004,
              modulo_verif=1000)
    t, tc = cases.sa_channel(**kw)
    zd = fasts.zone_data(t, fasts.prepare(t))
    c = oracle_mod.Case(zd, tc)
    c.apply_bc(0)
    c.apply_bc(1)
    for it in range(1, 4):
        c.compute(it, 1, 3, 1, modulo_verif=1000)
    G, N = _global_interior(t, zd, [e["lv"][0] for e in c.z])
    t1, tc1 = cases.sa_channel(parts=[[N[0]], [N[1]], [N[2]]], **kw)
    zd1 = fasts.zone_data(t1, fasts.prepare(t1))
    c1 = oracle_mod.Case(zd1, tc1)
    c1.apply_bc(0)
    c1.apply_bc(1)
    for it in range(1, 4):
        c1.compute(it, 1, 3, 1, modulo_verif=1000)
    G1, _ = _global_interior(t1, zd1, [c1.z[0]["lv"][0]])
    G0, _ = _global_interior(t1, zd1, [zd1[0]["ro"]])
    assert np.max(np.abs(G1 - G0)) > 1e-3      # the flow moved
    assert np.array_equal(G, G1)


def test_channel_sa_implicit_contracts(oracle_mod):
    t, tc = cases.sa_channel(**SMALL, temporal="implicit", ss_iteration=4, time_step=0.02)
    zd = fasts.zone_data(t, fasts.prepare(t))
    c = oracle_mod.Case(zd, tc)
    c.apply_bc(0)
    c.apply_bc(1)
    c.compute(1, 1, 4, 1, modulo_verif=1)
    # Newton residuals over all blocks (v and w start from zero, so only the
    # density, energy and nutilde residuals are expected to fall at once)
    R = np.array([c.residual_norms(m, 4)[:6] for m in range(len(zd))])
    assert np.all(np.isfinite(R))
    tot = np.sqrt((R ** 2).sum(axis=0))
    for eq in (0, 4, 5):
        assert tot[eq, -1] < tot[eq, 0] / 5
    for m in range(len(zd)):   # interior nutilde >= 0 (wall ghosts hold -nutilde)
        pi = zd[m]["pi"]
        ni, nj, nk = int(pi[0]), int(pi[1]), int(pi[2])
        assert c.z[m]["lv"][0].reshape(6, nk, nj, ni)[5, 2:-2, 2:-2, 2:-2].min() >= 0.0
