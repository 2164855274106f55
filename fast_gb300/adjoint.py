"""Gradients of the explicit 2-d Euler solve through a hand-written adjoint.

Case (the differentiation configuration): a C-grid of 385 x 129 cells (2-d
zone) around a NACA 0012-based airfoil whose upper and lower surfaces carry
eight Hicks-Henne bumps (amplitudes alpha_0..3 upper, alpha_4..7 lower,
peaks at x = 0.15, 0.35, 0.55, 0.75, width exponent 3), Mach M_inf at 2
degrees incidence, Euler, Roe + van Albada MUSCL, explicit RK3 for a fixed
number of steps.  Slip wall on the airfoil, characteristic farfield on the
outer boundary and the two wake ends, and the wake cut as a 1-to-1
interface of the zone with itself.  The functional J is the pressure force
normal to the chord on the airfoil at the final time,
J = -sum_wall p(first cell) * tj_y(wall face).

Differentiation: the mesh (from alpha), its metric (cp_tijk / cp_vol, the
same formulas on torch tensors), the initial state and the farfield state
(from M_inf) and J are torch functions; the solve is a
torch.autograd.Function whose backward is the discrete adjoint of every RK3
stage (fgb_adjoint_backward: local Jacobians of the flux, BC and update
formulas, transposed, with checkpoints every `ckpt` steps and recomputation
of each segment).  `tangent` gives the forward-mode directional derivative
(fgb_tangent) and `fd_gradient` central finite differences.

The gradient is exact for the discrete map except where it is not
differentiable: the Roe entropy fix switches (|lambda| against delta) and
the characteristic selection of the farfield BC are piecewise; both
derivative kernels take the branch of the primal state.
"""
from __future__ import annotations

import math
import time

import numpy as np
import torch

from . import fastc as FastC
from . import fasts, metric, pytree as I
from ._native import Solver

NG = 2
GAMMA = 1.4
AOA_DEG = 2.0
BUMP_PEAKS = (0.15, 0.35, 0.55, 0.75)


def hicks_henne(x, h, width=3.0):
    """sin(pi x^(ln 0.5 / ln h))^width: a bump of height 1 peaking at x = h."""
    return torch.sin(math.pi * x ** (math.log(0.5) / math.log(h))) ** width


def airfoil_y(x, upper: bool, alpha):
    """NACA 0012 (closed trailing edge) plus the Hicks-Henne bumps of one side."""
    yt = 0.6 * (0.2969 * torch.sqrt(x) - 0.1260 * x - 0.3516 * x ** 2 + 0.2843 * x ** 3
                - 0.1036 * x ** 4)
    y = yt if upper else -yt
    off = 0 if upper else 4
    for k, h in enumerate(BUMP_PEAKS):
        y = y + alpha[off + k] * hicks_henne(x, h)
    return y


def _geometric(n, first):
    """s_0..s_n of [0, 1], s_j = (q^j - 1) / (q^n - 1) with s_1 = first."""
    lo, hi = 1.0 + 1e-12, 2.0
    for _ in range(200):
        q = 0.5 * (lo + hi)
        s1 = (q - 1.0) / (q ** n - 1.0)
        if s1 > first:
            lo = q
        else:
            hi = q
    q = 0.5 * (lo + hi)
    return (q ** np.arange(n + 1) - 1.0) / (q ** n - 1.0)


def cgrid(alpha, ni=385, nj=129, nw=64, radius=10.0, wake=10.0, first=2e-3):
    """Vertex coordinates (x, y) of the C-grid, ghost vertices included
    (linear extrapolation), shape (ni + 1 + 2 NG, nj + 1 + 2 NG), float64
    torch tensors differentiable with respect to alpha (8 amplitudes)."""
    na = ni - 2 * nw
    dt = alpha.dtype
    # inner C: lower wake (x_far -> TE), airfoil (lower TE -> LE -> upper TE), upper wake
    t = torch.arange(nw, dtype=dt)
    xw_lo = 1.0 + wake * (1.0 - t / nw) ** 2
    m = torch.arange(na + 1, dtype=dt)
    theta = 2.0 * math.pi * m / na
    xi = torch.abs(theta - math.pi) / math.pi          # 0 at the leading edge, 1 at the TE
    xa = 0.25 * (1.0 - torch.cos(math.pi * xi)) + 0.5 * xi
    lower = theta < math.pi
    ya = torch.where(lower, airfoil_y(xa, False, alpha), airfoil_y(xa, True, alpha))
    xw_up = 1.0 + wake * ((torch.arange(1, nw + 1, dtype=dt)) / nw) ** 2
    xin = torch.cat([xw_lo, xa, xw_up])
    yin = torch.cat([torch.zeros(nw, dtype=dt), ya, torch.zeros(nw, dtype=dt)])
    phi = -0.5 * math.pi - math.pi * m / na
    xout = torch.cat([xw_lo, 1.0 + radius * torch.cos(phi), xw_up])
    yout = torch.cat([torch.full((nw,), -radius, dtype=dt), radius * torch.sin(phi),
                      torch.full((nw,), radius, dtype=dt)])
    s = torch.from_numpy(_geometric(nj, first / radius)).to(dt)
    X = xin[:, None] + (xout - xin)[:, None] * s[None, :]
    Y = yin[:, None] + (yout - yin)[:, None] * s[None, :]

    def pad(A):
        g = torch.arange(1, NG + 1, dtype=dt)
        lo = A[:1] - g.flip(0)[:, None] * (A[1:2] - A[:1])
        hi = A[-1:] + g[:, None] * (A[-1:] - A[-2:-1])
        A = torch.cat([lo, A, hi], dim=0)
        lo = A[:, :1] - g.flip(0)[None, :] * (A[:, 1:2] - A[:, :1])
        hi = A[:, -1:] + g[None, :] * (A[:, -1:] - A[:, -2:-1])
        return torch.cat([lo, A, hi], dim=1)

    return pad(X), pad(Y)


def metrics(X, Y):
    """(ti, tj, vol) of the 2-d zone (cp_tijk / cp_vol 2-d branch) on torch."""
    z0 = torch.zeros_like(X)
    Xk = torch.stack([X, X], dim=2)
    Yk = torch.stack([Y, Y], dim=2)
    Zk = torch.stack([z0, z0 + 1.0], dim=2)
    ti, tj, _, vol = metric._compute_2d(Xk, Yk, Zk)
    return ti, tj, vol


def free_stream(mach):
    """Primitive free stream (ro, u, v, w, T) and the conservative exterior
    state of the farfield BC (BCzone.cpp DEFAULT_STATE) for M_inf = mach."""
    a = math.radians(AOA_DEG)
    ro = torch.ones((), dtype=mach.dtype)
    u = mach * math.cos(a)
    v = mach * math.sin(a)
    p = torch.full((), 1.0 / GAMMA, dtype=mach.dtype)
    st1, st2 = u * ro, v * ro
    st4 = p / (GAMMA - 1.0) + 0.5 * (u * st1 + v * st2 + 0.0 * 0.0)
    st = torch.stack([ro, st1, st2, torch.zeros_like(ro), st4])
    return (ro, u, v, torch.zeros_like(ro), torch.ones_like(ro)), st


class CGridCase:
    """The tree (numerics, BCs, wake interface) of the C-grid case; the
    coordinates and free stream of each evaluation come from torch."""

    def __init__(self, ni=385, nj=129, nw=64, dt=4e-4, nsteps=400, ckpt=20, mach0=0.7):
        self.ni, self.nj, self.nw, self.dt, self.nsteps, self.ckpt = ni, nj, nw, dt, nsteps, ckpt
        na = ni - 2 * nw
        X, Y = cgrid(torch.zeros(8, dtype=torch.float64), ni, nj, nw)
        z = I.newZone("cgrid", [ni + 1 + 2 * NG, nj + 1 + 2 * NG, 2])
        gc = I.createChild(z, "GridCoordinates", "GridCoordinates_t")
        Xn, Yn = X.numpy(), Y.numpy()
        for nm, arr in (("CoordinateX", np.stack([Xn, Xn], axis=2)),
                        ("CoordinateY", np.stack([Yn, Yn], axis=2)),
                        ("CoordinateZ", np.stack([0 * Xn, 0 * Xn + 1.0], axis=2))):
            I.createChild(gc, nm, "DataArray_t")[1] = np.asfortranarray(arr)
        I.createChild(z, "Rind", "Rind_t", np.array([NG, NG, NG, NG, 0, 0], dtype=np.int64))
        shape = (ni + 2 * NG, nj + 2 * NG, 1)
        a = math.radians(AOA_DEG)
        from .cases import set_conservative, add_bc
        set_conservative(z, np.ones(shape), np.full(shape, mach0 * math.cos(a)),
                         np.full(shape, mach0 * math.sin(a)), np.zeros(shape),
                         np.full(shape, 1.0 / GAMMA), GAMMA)
        add_bc(z, "far_imin", "BCFarfield", "imin")
        add_bc(z, "far_imax", "BCFarfield", "imax")
        add_bc(z, "far_jmax", "BCFarfield", "jmax")
        zbc = I.getNodeFromName1(z, "ZoneBC")
        bc = I.createChild(zbc, "wall", "BC_t", "BCWallInviscid")
        rg = np.array([[NG + nw + 1, NG + nw + na + 1], [1, 1], [1, 2]], dtype=np.int64)
        I.createChild(bc, "PointRange", "IndexRange_t")[1] = np.asfortranarray(rg)
        t = I.newCGNSTree()
        b = I.newCGNSBase("Base", 3, 3, t)
        b[2].append(z)
        I.createChild(b, "FlowEquationSet", "FlowEquationSet_t")
        I.createChild(I.getNodeFromName1(b, "FlowEquationSet"), "GoverningEquations",
                      "GoverningEquations_t", "Euler")
        FastC.addReferenceState(t, mach=mach0, reynolds=0.0, gamma=GAMMA, alpha_deg=AOA_DEG)
        FastC._setNum2Base(t, {"temporal_scheme": "explicit", "ss_iteration": 1,
                               "modulo_verif": 1000000})
        FastC._setNum2Zones(t, {"scheme": "roe", "slope": "vanalbada", "time_step": dt,
                                "cache_blocking_I": 1000000, "cache_blocking_J": 1000000,
                                "cache_blocking_K": 1000000})
        self.tree = t
        zd = fasts.zone_data(t, fasts.prepare(t))[0]
        self.pi, self.pr = zd["pi"].copy(), zd["pr"].copy()
        assert int(self.pi[25]) == 3
        self.nd, self.ndm = int(self.pi[41]), int(self.pi[43])
        self.nip, self.nvi = ni + 2 * NG, ni + 1 + 2 * NG
        # wake cut: ghost (i, 1 - m) <- cell (ni + 1 - i, m), m = 1, 2
        rcv, dnr = [], []
        for m_ in (1, 2):
            for i in list(range(1, nw + 1)) + list(range(nw + na + 1, ni + 1)):
                rcv.append(self.inddm(i, 1 - m_))
                dnr.append(self.inddm(ni + 1 - i, m_))
        self.cut = (np.array(dnr, dtype=np.int64), np.array(rcv, dtype=np.int64))
        self.wall_i = np.arange(nw + 1, nw + na + 1)
        self.timing = {}
        self.graph = True       # replay the driver loops as CUDA graphs
        self.profile = False    # per-group CUDA-event timing (stream launches)

    def inddm(self, i, j):
        return (i + NG - 1) + (j + NG - 1) * self.nip

    def solver(self, ti, tj, vol, w0, st):
        s = Solver(0)
        s.set_option("graph", int(self.graph))
        s.set_option("profile", int(self.profile))
        s.add_zone(self.pi, self.pr, ti, tj, np.zeros(0), vol)
        s.add_transfer(0, 0, *self.cut)
        s.set_bc_state(0, st)
        s.upload(0, 0, w0)
        return s

    def initial_state(self, prim):
        """W0 (NEQ x NDIMDX) of a uniform primitive state (torch scalars)."""
        return torch.cat([p.reshape(1).expand(self.nd) for p in prim])

    def functional(self, W, tj):
        """J = -sum over wall faces of p(first cell) * tj_y(face)."""
        rgp = float(self.pr[2]) * (GAMMA - 1.0)
        W = W.reshape(5, self.nd)
        l = torch.as_tensor([self.inddm(i, 1) for i in self.wall_i])
        lt = torch.as_tensor([(i + NG - 1) + NG * self.nvi for i in self.wall_i])
        p = W[0, l] * W[4, l] * rgp
        return -(p * tj[self.ndm + lt]).sum()


class _Solve(torch.autograd.Function):
    """W_final = solve(ti, tj, vol, W0, st) on the GPU; backward = adjoint."""

    @staticmethod
    def forward(ctx, ti, tj, vol, w0, st, case):
        s = case.solver(ti.detach().numpy(), tj.detach().numpy(), vol.detach().numpy(),
                        w0.detach().numpy(), st.detach().numpy())
        t0 = time.perf_counter()
        s.adjoint_forward(0, case.nsteps, case.ckpt)
        s.synchronize()
        case.timing["primal_s"] = time.perf_counter() - t0
        W = torch.from_numpy(s.download(0, 0).copy())
        ctx.solver, ctx.case = s, case
        return W

    @staticmethod
    def backward(ctx, gW):
        s, case = ctx.solver, ctx.case
        t0 = time.perf_counter()
        gw0, gti, gtj, gvol, gst = s.adjoint_backward(0, gW.detach().contiguous().numpy())
        case.timing["adjoint_s"] = time.perf_counter() - t0
        if case.profile:
            case.timing["groups_ms"] = {k: v[1] for k, v in s.kernel_stats().items()}
        s.close()
        return (torch.from_numpy(gti), torch.from_numpy(gtj), torch.from_numpy(gvol),
                torch.from_numpy(gw0), torch.from_numpy(gst), None)


def inputs(case, alpha, mach):
    X, Y = cgrid(alpha, case.ni, case.nj, case.nw)
    ti, tj, vol = metrics(X, Y)
    prim, st = free_stream(mach)
    return ti, tj, vol, case.initial_state(prim), st


def objective(case, alpha, mach):
    """J(alpha, M_inf) as a torch scalar (differentiable through the adjoint)."""
    ti, tj, vol, w0, st = inputs(case, alpha, mach)
    W = _Solve.apply(ti, tj, vol, w0, st, case)
    return case.functional(W, tj)


def gradient(case, alpha, mach):
    """(J, dJ/dalpha (8), dJ/dM_inf) by the adjoint."""
    a = alpha.clone().requires_grad_(True)
    m = mach.clone().requires_grad_(True)
    J = objective(case, a, m)
    J.backward()
    return float(J.detach()), a.grad.numpy().copy(), float(m.grad)


def value(case, alpha, mach):
    with torch.no_grad():
        return float(objective(case, alpha, mach))


def fd_gradient(case, alpha, mach, h=1e-6):
    """Central finite differences of J in each amplitude and in M_inf."""
    g = np.zeros(9)
    for k in range(9):
        e = torch.zeros(9, dtype=torch.float64)
        e[k] = h
        jp = value(case, alpha + e[:8], mach + e[8])
        jm = value(case, alpha - e[:8], mach - e[8])
        g[k] = (jp - jm) / (2 * h)
    return g


def tangent(case, alpha, mach, dalpha, dmach):
    """Forward-mode dJ along (dalpha, dmach): torch jvp of the inputs, the
    GPU tangent of the solve (fgb_tangent), torch jvp of J."""
    from torch.func import jvp
    (ti, tj, vol, w0, st), (dti, dtj, dvol, dw0, dst) = jvp(
        lambda a, m: inputs(case, a, m), (alpha, mach), (dalpha, dmach))
    s = case.solver(ti.numpy(), tj.numpy(), vol.numpy(), w0.numpy(), st.numpy())
    dW = s.tangent(0, case.nsteps, dw0.numpy(), dti.numpy(), dtj.numpy(), dvol.numpy(), dst.numpy())
    s.adjoint_forward(0, case.nsteps, case.ckpt)
    W = torch.from_numpy(s.download(0, 0).copy())
    s.close()
    _, dJ = jvp(lambda w, t: case.functional(w, t), (W, tj), (torch.from_numpy(dW), dtj))
    return float(dJ)
