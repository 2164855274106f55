"""Differentiation of the explicit 2-d Euler solve (C-grid around a
Hicks-Henne-bumped airfoil, Roe + van Albada, RK3).

CPU: the torch mesh / metric / functional pipeline (the metric on torch
tensors equals the numpy metric bit for bit; the C-grid cells are valid).
GPU: the adjoint against the tangent (dot-product test over every input:
<lam, T d> = <A^T lam, d>), the adjoint gradient of J against the
forward-mode tangent and against central finite differences (h = 1e-6),
and the primal of the adjoint driver against fgb_compute and the oracle.
Short runs (40 steps, checkpoints every 8, so the last segment is partial
and every stage of a segment is recomputed).
"""
import numpy as np
import pytest
import torch

from fast_gb300 import adjoint as A, metric

SMALL = dict(ni=97, nj=33, nw=16, dt=4e-4, nsteps=40, ckpt=8)


@pytest.fixture(scope="module")
def case():
    return A.CGridCase(**SMALL)


def _alpha(seed=4):
    return torch.from_numpy(np.random.default_rng(seed).uniform(-0.005, 0.005, 8))


def test_cgrid_metric_torch_equals_numpy(case):
    X, Y = A.cgrid(_alpha(), case.ni, case.nj, case.nw)
    ti, tj, vol = A.metrics(X, Y)
    Xn, Yn = X.numpy(), Y.numpy()
    ref = metric._compute_2d(np.stack([Xn, Xn], axis=2), np.stack([Yn, Yn], axis=2),
                             np.stack([0 * Xn, 0 * Xn + 1.0], axis=2))
    for a, b in zip((ti, tj, vol), (ref[0], ref[1], ref[3])):
        assert np.array_equal(a.detach().numpy(), b)
    V = vol.detach().numpy().reshape(-1, case.nvi).T[:-1, :-1]
    assert V.min() > 0.0                      # no inverted cell, ghosts included


def test_cgrid_geometry(case):
    """Closed trailing edge, wake cut vertices shared by both sides, bumps
    that move the surface by the amplitudes at their peaks."""
    X, Y = A.cgrid(torch.zeros(8, dtype=torch.float64), case.ni, case.nj, case.nw)
    g = A.NG
    inner_x, inner_y = X[g:-g, g].numpy(), Y[g:-g, g].numpy()
    nw, ni = case.nw, case.ni
    assert np.allclose(inner_x[:nw + 1], inner_x[ni - nw:][::-1])
    assert np.allclose(inner_y[nw], 0.0) and np.allclose(inner_y[ni - nw], 0.0)
    x = torch.tensor([0.35], dtype=torch.float64)
    a = torch.zeros(8, dtype=torch.float64)
    a[1] = 0.004
    assert abs(float(A.airfoil_y(x, True, a) - A.airfoil_y(x, True, 0 * a)) - 0.004) < 1e-12


def test_functional_gradient_shapes(case):
    a = _alpha().requires_grad_(True)
    m = torch.tensor(0.7, dtype=torch.float64, requires_grad=True)
    ti, tj, vol, w0, st = A.inputs(case, a, m)
    J = case.functional(w0, tj)             # J of the initial state: depends on alpha only
    J.backward()
    assert a.grad is not None and torch.isfinite(a.grad).all()


@pytest.mark.gpu
def test_adjoint_primal_equals_compute(case):
    """fgb_adjoint_forward runs the product kernels: the same final state as
    fgb_compute over the same steps, bit for bit."""
    from fast_gb300._native import Solver
    ti, tj, vol, w0, st = (x.detach().numpy() for x in A.inputs(case, _alpha(),
                                                              torch.tensor(0.7, dtype=torch.float64)))
    s = case.solver(ti, tj, vol, w0, st)
    s.adjoint_forward(0, 10, 4)
    got = s.download(0, 0)
    s.close()
    s = case.solver(ti, tj, vol, w0, st)
    s.set_option("modulo_verif", 1000000)
    s.apply_bc(0)
    for it in range(1, 11):
        s.compute(it, 1, 3, 1, 1)
    s.synchronize()
    exp = s.download(0, 0)
    s.close()
    assert np.array_equal(got, exp)


@pytest.mark.gpu
def test_dot_product(case):
    """<lam, T d> = <A^T lam, d> for random lam (final state, interior) and d
    (initial state interior, ti, tj, vol, farfield state)."""
    rng = np.random.default_rng(11)
    ti, tj, vol, w0, st = (x.detach().numpy() for x in A.inputs(case, _alpha(),
                                                              torch.tensor(0.7, dtype=torch.float64)))
    nd, nvi = case.nd, case.nvi
    inner = np.zeros((5, nd), dtype=bool)
    Q = inner.reshape(5, -1, case.nip)
    Q[:, A.NG:-A.NG, A.NG:-A.NG] = True
    Q[3] = False                                # w is identically zero in 2-d
    inner = inner.reshape(-1)
    dw0 = np.where(inner, rng.standard_normal(inner.size), 0.0) * 1e-3
    dti = rng.standard_normal(ti.size) * 1e-4
    dtj = rng.standard_normal(tj.size) * 1e-4
    dvol = rng.standard_normal(vol.size) * 1e-6
    dst = np.array([1.0, 0.5, -0.3, 0.0, 0.2]) * 1e-3
    lam = np.where(inner, rng.standard_normal(inner.size), 0.0)
    s = case.solver(ti, tj, vol, w0, st)
    dW = s.tangent(0, case.nsteps, dw0, dti, dtj, dvol, dst)
    s.close()
    s = case.solver(ti, tj, vol, w0, st)
    s.adjoint_forward(0, case.nsteps, case.ckpt)
    g = s.adjoint_backward(0, lam)
    s.close()
    lhs = float(np.dot(lam, dW))
    rhs = float(np.dot(g[0], dw0) + np.dot(g[1], dti) + np.dot(g[2], dtj) + np.dot(g[3], dvol) +
                np.dot(g[4], dst))
    assert abs(lhs - rhs) <= 1e-9 * max(abs(lhs), abs(rhs)), (lhs, rhs)


@pytest.mark.gpu
def test_gradient_tangent_and_fd(case):
    alpha = _alpha()
    mach = torch.tensor(0.7, dtype=torch.float64)
    J, ga, gm = A.gradient(case, alpha, mach)
    grad = np.concatenate([ga, [gm]])
    assert np.all(np.isfinite(grad)) and np.any(grad != 0)
    # forward-mode tangent along two directions
    rng = np.random.default_rng(5)
    for _ in range(2):
        d = rng.standard_normal(9)
        dJ = A.tangent(case, alpha, mach, torch.from_numpy(d[:8]), torch.tensor(d[8], dtype=torch.float64))
        assert abs(dJ - grad @ d) <= 1e-9 * max(abs(dJ), 1e-30), (dJ, grad @ d)
    # central differences: h = 1e-6 agrees to its O(h^2) truncation (the
    # Hicks-Henne directions have large third derivatives: the FD error falls
    # as h^2 down to h = 1e-7, where it reaches 1e-7 relative); h = 1e-7 to 1e-6
    scale = np.max(np.abs(grad))
    fd6 = A.fd_gradient(case, alpha, mach, h=1e-6)
    assert np.max(np.abs(fd6 - grad)) <= 2e-5 * scale, (fd6, grad)
    fd7 = A.fd_gradient(case, alpha, mach, h=1e-7)
    assert np.max(np.abs(fd7 - grad)) <= 1e-6 * scale, (fd7, grad)


@pytest.mark.gpu
def test_graph_replay_equals_stream_launches():
    """The CUDA-graph replay of the driver loops (odd segment length: both
    lambda-buffer parities, a partial last segment) against stream launches:
    the same primal bit for bit, the same gradient to FP64-atomic reordering."""
    c = A.CGridCase(ni=97, nj=33, nw=16, dt=4e-4, nsteps=40, ckpt=7)
    ti, tj, vol, w0, st = (x.detach().numpy() for x in A.inputs(c, _alpha(),
                                                              torch.tensor(0.7, dtype=torch.float64)))
    lam = np.random.default_rng(3).standard_normal(w0.size)
    out = []
    for graph in (True, False):
        c.graph = graph
        s = c.solver(ti, tj, vol, w0, st)
        s.adjoint_forward(0, c.nsteps, c.ckpt)
        W = s.download(0, 0).copy()
        g = s.adjoint_backward(0, lam)
        g2 = s.adjoint_backward(0, lam)          # a second sweep over the same forward run
        s.close()
        out.append((W, g, g2))
    (Wg, gg, gg2), (We, ge, _) = out
    assert np.array_equal(Wg, We)
    for a, b, b2 in zip(gg, ge, gg2):
        tol = 1e-12 * max(np.max(np.abs(b)), 1e-300)
        assert np.max(np.abs(a - b)) <= tol and np.max(np.abs(b2 - b)) <= tol
