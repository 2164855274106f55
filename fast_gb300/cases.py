"""Synthetic cases of the benchmark configurations (meshes, initial fields,
boundary conditions), built directly as pyTrees.

Cassiopee's Generator / Initiator / Connector are not available, so the mesh
generators and initial conditions are written here from their published
definitions:

* isentropic vortex (Yee, Sandham & Djomehri, J. Comput. Phys. 150, 1999):
  du = -beta/(2 pi) (y-yc) e^{(1-r^2)/2}, dv = beta/(2 pi) (x-xc) e^{(1-r^2)/2},
  dT = -(gamma-1) beta^2 / (8 gamma pi^2) e^{1-r^2}, isentropic density,
  lengths scaled by the core radius;
* Taylor-Green vortex, with the density / pressure formula that
  FastS/test/explicitLocalTgv_t1.py:86-90 uses.

Zones carry two layers of ghost cells as after Internal.addGhostCells; BC
PointRanges follow that convention (windows extended through the ghost
layers), which FastC's getRange converts back to interior windows.
"""
from __future__ import annotations

import copy
import math

import numpy as np

from . import fastc as FastC
from . import pytree as I

NG = 2


def cart_zone(name, x0, h, n, ng=NG, ngk=None):
    """Uniform cartesian zone of n = (ni, nj, nk) interior cells, origin x0
    (first interior vertex), steps h, with ng ghost layers on every side
    (ngk in k; a 2-d zone has nk = 1 and ngk = 0)."""
    ni, nj, nk = n
    ngk = ng if ngk is None else ngk
    nv = [ni + 1 + 2 * ng, nj + 1 + 2 * ng, nk + 1 + 2 * ngk]
    z = I.newZone(name, nv)
    ii = np.arange(nv[0]) - ng
    jj = np.arange(nv[1]) - ng
    kk = np.arange(nv[2]) - ngk
    X, Y, Z = np.meshgrid(x0[0] + ii * h[0], x0[1] + jj * h[1], x0[2] + kk * h[2], indexing="ij")
    gc = I.createChild(z, "GridCoordinates", "GridCoordinates_t")
    for nm, arr in (("CoordinateX", X), ("CoordinateY", Y), ("CoordinateZ", Z)):
        I.createChild(gc, nm, "DataArray_t")[1] = np.asfortranarray(arr)
    I.createChild(z, "Rind", "Rind_t", np.array([ng, ng, ng, ng, ngk, ngk], dtype=np.int64))
    return z


def wave(z, amp, x0, L, two_d=False):
    """Periodic curvilinear mesh: displace every vertex of a uniform box by
    amp x (local step) x a product of sines of the other two coordinates,
    with the box lengths L as periods, so the mesh stays periodic (ghost
    vertices coincide with the shifted interior ones) and is a general
    3-d zone (no direction stays cartesian)."""
    gc = I.getNodeFromName1(z, "GridCoordinates")
    X, Y, Z = (I.getNodeFromName1(gc, n)[1].copy() for n in
               ("CoordinateX", "CoordinateY", "CoordinateZ"))
    hx, hy, hz = X[1, 0, 0] - X[0, 0, 0], Y[0, 1, 0] - Y[0, 0, 0], Z[0, 0, 1] - Z[0, 0, 0]
    sx, sy, sz = (2 * math.pi * (A - a0) / l for A, a0, l in ((X, x0[0], L[0]), (Y, x0[1], L[1]),
                                                              (Z, x0[2], L[2])))
    if two_d:   # in-plane displacement only: the zone stays a 2-d zone
        new = (X + amp * hx * np.sin(sy), Y + amp * hy * np.sin(sx), Z)
    else:
        new = (X + amp * hx * np.sin(sy) * np.sin(sz),
               Y + amp * hy * np.sin(sx) * np.sin(sz),
               Z + amp * hz * np.sin(sx) * np.sin(sy))
    for nm, arr in zip(("CoordinateX", "CoordinateY", "CoordinateZ"), new):
        I.getNodeFromName1(gc, nm)[1] = np.asfortranarray(arr)
    return z


def cell_centers(z):
    gc = I.getNodeFromName1(z, "GridCoordinates")
    out = []
    for nm in ("CoordinateX", "CoordinateY", "CoordinateZ"):
        a = I.getNodeFromName1(gc, nm)[1]
        c = 0.125 * (a[:-1, :-1, :-1] + a[1:, :-1, :-1] + a[:-1, 1:, :-1] + a[:-1, :-1, 1:] +
                     a[1:, 1:, :-1] + a[1:, :-1, 1:] + a[:-1, 1:, 1:] + a[1:, 1:, 1:])
        out.append(np.asfortranarray(c))
    return out


def add_bc(z, name, btype, face, ng=NG):
    """Full-face BC on face 'imin'..'kmax' with a ghost-extended PointRange."""
    nv = [int(z[1][0, 0]), int(z[1][1, 0]), int(z[1][2, 0])]
    rg = np.array([[1, nv[0]], [1, nv[1]], [1, nv[2]]], dtype=np.int64)
    d = "ijk".index(face[0])
    rg[d, :] = 1 if face[1:] == "min" else nv[d]
    zbc = I.getNodeFromName1(z, "ZoneBC") or I.createChild(z, "ZoneBC", "ZoneBC_t")
    bc = I.createChild(zbc, name, "BC_t", btype)
    I.createChild(bc, "PointRange", "IndexRange_t")[1] = np.asfortranarray(rg)
    return bc


def set_conservative(z, ro, u, v, w, p, gamma):
    sol = I.createUniqueChild(z, I.__FlowSolutionCenters__, "FlowSolution_t")
    roe = p / (gamma - 1.0) + 0.5 * ro * (u * u + v * v + w * w)
    for nm, arr in (("Density", ro), ("MomentumX", ro * u), ("MomentumY", ro * v),
                    ("MomentumZ", ro * w), ("EnergyStagnationDensity", roe)):
        I.createUniqueChild(sol, nm, "DataArray_t")[1] = np.asfortranarray(arr)


def set_spalart(z, nutilde, dist):
    """Spalart-Allmaras fields at centers: nutilde (TurbulentSANuTilde) and
    the wall distance (TurbulentDistance, which FastS requires as input)."""
    sol = I.createUniqueChild(z, I.__FlowSolutionCenters__, "FlowSolution_t")
    I.createUniqueChild(sol, "TurbulentSANuTilde", "DataArray_t")[1] = np.asfortranarray(nutilde)
    I.createUniqueChild(sol, "TurbulentDistance", "DataArray_t")[1] = np.asfortranarray(dist)


def _tree(zones, model, numb, numz, mach, reynolds, gamma=1.4, prandtl=0.72, sutherland=True,
          nutilde_ratio=0.1):
    t = I.newCGNSTree()
    b = I.newCGNSBase("Base", 3, 3, t)
    for z in zones:
        b[2].append(z)
    I.createChild(b, "FlowEquationSet", "FlowEquationSet_t")
    I.createChild(I.getNodeFromName1(b, "FlowEquationSet"), "GoverningEquations",
                  "GoverningEquations_t", model)
    FastC.addReferenceState(t, mach=mach, reynolds=reynolds, gamma=gamma, prandtl=prandtl,
                            sutherland=sutherland, nutilde_ratio=nutilde_ratio)
    FastC._setNum2Base(t, numb)
    FastC._setNum2Zones(t, numz)
    return t


def isentropic_vortex(n=(128, 128, 4), mach=0.5, beta=5.0, radius=1.0, box=10.0, gamma=1.4,
                      numb=None, numz=None, wavy=0.0, two_d=False, cfl=None):
    """Config: plain FP64, 128x128x4 periodic box [-box, box]^2, Euler vortex
    (Mach 0.5, strength 5, core radius 1), Roe + minmod, explicit RK3.
    wavy > 0: the same box on a periodic curvilinear mesh (see wave).
    cfl: the time step is the one that gives this CFL number on the initial
    field (cpcfl3.for's local time step, fasts.cfl_time_step) instead of the
    numerics' time_step."""
    ni, nj, nk = n
    if two_d:
        nk = 1
        n = (ni, nj, 1)
    h = (2 * box / ni, 2 * box / nj, 2 * box / ni)
    ng = _ghosts("roe_min", numz)
    z = cart_zone("vortex", (-box, -box, 0.0), h, n, ng=ng, ngk=0 if two_d else None)
    if wavy:
        wave(z, wavy, (-box, -box, 0.0), (2 * box, 2 * box, h[2] * nk), two_d=two_d)
    xc, yc, _ = cell_centers(z)
    x = xc / radius
    y = yc / radius
    r2 = x * x + y * y
    e = np.exp(0.5 * (1.0 - r2))
    du = -beta / (2 * math.pi) * y * e
    dv = beta / (2 * math.pi) * x * e
    T = 1.0 - (gamma - 1.0) * beta ** 2 / (8.0 * gamma * math.pi ** 2) * e * e
    ro = T ** (1.0 / (gamma - 1.0))
    p = ro * T / gamma
    set_conservative(z, ro, mach + du, dv, np.zeros_like(ro), p, gamma)
    for f in ("imin", "imax", "jmin", "jmax") + (() if two_d else ("kmin", "kmax")):
        add_bc(z, "per_" + f, "BCautoperiod", f, ng=ng)
    numb = numb or {"temporal_scheme": "explicit", "ss_iteration": 1, "modulo_verif": 1000000}
    numz = numz or {"scheme": "roe_min", "slope": "minmod", "time_step": 0.01,
                    "cache_blocking_I": 1000000, "cache_blocking_J": 1000000,
                    "cache_blocking_K": 1000000}
    t = _tree([z], "Euler", numb, numz, mach, 0.0, gamma=gamma)
    if cfl is not None:
        from . import fasts
        FastC._setNum2Zones(t, {"time_step": fasts.cfl_time_step(t, cfl)})
    return t


def _ghosts(slope, numz=None):
    """Ghost layers of a zone: three for the o5 slopes (o5, o5sc), else two."""
    sl = (numz or {}).get("slope", slope)
    return 3 if sl in ("o5", "o5sc") else NG


def taylor_green(n=256, mach=0.1, reynolds=1600.0, prandtl=0.71, gamma=1.4, ss_iteration=4,
                 dt=None, scheme="ausmpred", slope="o3", numb=None, numz=None, name="tgv",
                 wavy=0.0, model="NSLaminar", nutilde_ratio=5.0, wall_distance=1.0e8):
    """Config: laminar Taylor-Green vortex on the periodic box [0, 2 pi]^3,
    Re = 1600, Mach 0.1, Pr 0.71, mu ~ sqrt(T) (FastS Sutherland form with
    Cs = 0), AUSM+(P) o3, implicit LU-SGS dual time stepping.  model
    "NSTurbulent" adds Spalart-Allmaras with ro nutilde = nutilde_ratio x mu
    and a uniform wall distance (no wall in the periodic box)."""
    N = (n, n, n) if isinstance(n, int) else tuple(n)
    L = 1.0
    h = tuple(2 * math.pi * L / k for k in N)
    ng = _ghosts(slope, numz)
    z = cart_zone(name, (0.0, 0.0, 0.0), h, N, ng=ng)
    if wavy:
        wave(z, wavy, (0.0, 0.0, 0.0), tuple(2 * math.pi * L for _ in range(3)))
    xc, yc, zc = cell_centers(z)
    U0 = mach
    ro0, T0 = 1.0, 1.0
    p0 = ro0 * T0 / gamma
    u = U0 * np.sin(xc / L) * np.cos(yc / L) * np.cos(zc / L)
    v = -U0 * np.cos(xc / L) * np.sin(yc / L) * np.cos(zc / L)
    w = np.zeros_like(u)
    p = p0 + ro0 * U0 ** 2 / 16.0 * (np.cos(2 * xc / L) + np.cos(2 * yc / L)) * (np.cos(2 * zc / L) + 2.0)
    ro = p * gamma / T0   # T = T0 everywhere (R = 1/gamma)
    set_conservative(z, ro, u, v, w, p, gamma)
    if model == "NSTurbulent":
        set_spalart(z, nutilde_ratio * (mach / reynolds) / ro, np.full_like(ro, wall_distance))
    for f in ("imin", "imax", "jmin", "jmax", "kmin", "kmax"):
        add_bc(z, "per_" + f, "BCautoperiod", f, ng=ng)
    if dt is None:
        dt = 2.0 * h[0] / (U0 + 1.0)   # acoustic CFL 2 (implicit dual time)
    numb = numb or {"temporal_scheme": "implicit", "ss_iteration": ss_iteration,
                    "modulo_verif": 1}
    numz = numz or {"scheme": scheme, "slope": slope, "time_step": dt,
                    "cache_blocking_I": 1000000, "cache_blocking_J": 1000000,
                    "cache_blocking_K": 1000000}
    return _tree([z], model, numb, numz, mach, reynolds, gamma=gamma, prandtl=prandtl,
                 sutherland=False, nutilde_ratio=nutilde_ratio)


def add_bc_data(bc, arrays):
    """BC data as FastS reads it: DataArray_t nodes under BCDataSet_t /
    BCData_t of the BC node, in the given order (name, values)."""
    ds = I.createChild(bc, "BCDataSet", "BCDataSet_t", "Null")
    bd = I.createChild(ds, "DirichletData", "BCData_t")
    for name, val in arrays:
        I.createChild(bd, name, "DataArray_t", np.asarray(val, dtype=np.float64))
    return bc


def bc_box(n=(16, 12, 6), mach=0.3, reynolds=1.0e4, wall="BCWallViscous", model="NSLaminar",
           wavy=0.0, perturb=0.05, temporal="explicit", ss_iteration=3, scheme="ausmpred",
           slope="o3", time_step=0.02, gamma=1.4, two_d=False, nutilde_ratio=5.0,
           extrude=False, outflow="BCOutflow", outpres_form=1, outpres_amp=0.02, bc_data=False,
           stretch=0.0):
    """Box [0,1]x[0,1]x[0,dz] exercising the non-periodic BCs of the path:
    inflow at imin (BCInflow), outflow at imax (BCOutflow), a wall at jmin
    (``wall``), farfield at jmax (BCFarfield), periodic in k.  The initial
    field is the free stream with a smooth perturbation of relative size
    ``perturb`` (0 gives the free stream itself).  wavy > 0 displaces the
    vertices as in ``wave`` (periods = box lengths).  model "NSTurbulent"
    adds Spalart-Allmaras: free-stream ro nutilde = nutilde_ratio x mu, the
    same perturbation on nutilde, and the distance to the jmin wall.
    extrude (3-d only): the 2-d case extruded in k -- in-plane displacement,
    no k dependence of the initial field, w = 0.
    outflow "BCOutpres": imposed static pressure at imax instead, one value
    per face (p_inf (1 + outpres_amp sin(2 pi y))) given as BC data -- the pressure
    array alone (outpres_form 1) or after a one-value mobile_coef array
    (outpres_form 2), the two layouts bvbs_outpres reads.
    stretch > 0: the vertex y clustered at the jmin wall, y -> sinh(stretch y)
    / sinh(stretch) (a mesh homogeneous in k: zone type 1).
    bc_data: the farfield and inflow states come from BC data instead of the
    free stream (conservative ro, ro u, ro v, ro w, ro E [, ro nutilde],
    a 2-3 % departure from it): the farfield as one array of those values,
    the inflow in the 21-array layout of BCzone.cpp's DEFAULT_STATE."""
    ni, nj, nk = n
    if two_d:
        nk = 1
        n = (ni, nj, 1)
    h = (1.0 / ni, 1.0 / nj, 1.0 / ni)
    ng = _ghosts(slope)
    z = cart_zone("box", (0.0, 0.0, 0.0), h, n, ng=ng, ngk=0 if two_d else None)
    flat = two_d or extrude
    if stretch:
        gc = I.getNodeFromName1(z, "GridCoordinates")
        Y = I.getNodeFromName1(gc, "CoordinateY")[1]
        Y[:] = np.sinh(stretch * Y) / math.sinh(stretch)
    if wavy:
        wave(z, wavy, (0.0, 0.0, 0.0), (1.0, 1.0, h[2] * nk), two_d=flat)
    xc, yc, zc = cell_centers(z)
    a = perturb
    s = np.sin(2 * math.pi * xc) * np.sin(2 * math.pi * yc)
    if not flat:
        s = s * np.cos(2 * math.pi * zc / (h[2] * nk))
    ro = 1.0 + a * s
    u = mach * (1.0 + a * np.cos(2 * math.pi * yc) * np.sin(2 * math.pi * xc))
    v = mach * a * s
    w = 0.0 * xc if flat else mach * a * np.sin(2 * math.pi * xc) * np.cos(2 * math.pi * yc)
    p = (1.0 + a * 0.5 * s) / gamma
    set_conservative(z, ro, u, v, w, p, gamma)
    if model == "NSTurbulent":
        mu = mach / reynolds
        set_spalart(z, nutilde_ratio * mu * (1.0 + a * np.cos(2 * math.pi * xc) * np.sin(math.pi * yc)) / ro,
                    np.abs(yc))
    bin_ = add_bc(z, "in", "BCInflow", "imin", ng=ng)
    bout = add_bc(z, "out", outflow, "imax", ng=ng)
    add_bc(z, "wall", wall, "jmin", ng=ng)
    bfar = add_bc(z, "far", "BCFarfield", "jmax", ng=ng)
    if outflow == "BCOutpres":
        nkf = 1 if two_d else nk
        yf = (np.arange(nj) + 0.5) / nj
        pf = np.repeat((1.0 + outpres_amp * np.sin(2 * math.pi * yf))[:, None] / gamma, nkf, axis=1)
        arrays = [("Pressure", pf.ravel(order="F"))]
        if outpres_form == 2:
            arrays = [("mobile_coef", np.array([1.0]))] + arrays
        add_bc_data(bout, arrays)
    if bc_data:
        ro_e, u_e, v_e = 1.02, 1.03 * mach, 0.01 * mach
        p_e = 1.01 / gamma
        st = [ro_e, ro_e * u_e, ro_e * v_e, 0.0,
              p_e / (gamma - 1.0) + 0.5 * ro_e * (u_e * u_e + v_e * v_e)]
        if model == "NSTurbulent":
            st.append(ro_e * 1.1 * nutilde_ratio * mach / reynolds)
        add_bc_data(bfar, [("State", np.array(st))])
        st21 = [0.0] * 21
        for m_ in range(5):
            st21[3 + m_] = st[m_] * (1.0 if m_ != 1 else 0.99)
        if model == "NSTurbulent":
            st21[16] = st[5]
        add_bc_data(bin_, [("d%02d" % m_, np.array([x])) for m_, x in enumerate(st21)])
    if not two_d:
        add_bc(z, "per_kmin", "BCautoperiod", "kmin", ng=ng)
        add_bc(z, "per_kmax", "BCautoperiod", "kmax", ng=ng)
    numb = {"temporal_scheme": temporal, "ss_iteration": ss_iteration, "modulo_verif": 1}
    numz = {"scheme": scheme, "slope": slope, "time_step": time_step,
            "cache_blocking_I": 1000000, "cache_blocking_J": 1000000, "cache_blocking_K": 1000000}
    return _tree([z], model, numb, numz, mach, reynolds if model != "Euler" else 0.0, gamma=gamma,
                 nutilde_ratio=nutilde_ratio)


# ------------------------------------------------- multi-block SA channel
def _tanh_both_ends(n, first):
    """Vertex parameters s_0..s_n of [0, 1] clustered at both ends by
    s = (1 + tanh(d (eta - 1/2)) / tanh(d / 2)) / 2, d chosen (bisection) so
    that the first spacing s_1 equals `first` (uniform if that needs d <= 0)."""
    def s1(d):
        return 0.5 * (1.0 + math.tanh(d * (1.0 / n - 0.5)) / math.tanh(0.5 * d))
    eta = np.arange(n + 1) / n
    lo, hi = 1e-9, 200.0
    if s1(lo) <= first:
        return eta
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if s1(mid) > first:
            lo = mid
        else:
            hi = mid
    d = 0.5 * (lo + hi)
    return 0.5 * (1.0 + np.tanh(d * (eta - 0.5)) / math.tanh(0.5 * d))


def sa_channel(nblocks=(4, 3, 4), sizes=((16, 96), (16, 64), (16, 32)), seed=2024, mach=0.3,
               reynolds=1.0e5, bump=0.1, first_cell=1.0e-4, length=(4.0, 1.0, 1.0),
               nutilde_ratio=3.0, perturb=1.0e-3, temporal="implicit", ss_iteration=4,
               time_step=0.01, modulo_verif=1, skew=0.2, parts=None, model="NSTurbulent",
               wall="BCWallViscous"):
    """Multi-block Spalart-Allmaras channel: a seeded random box decomposition
    (nblocks = blocks per direction, 4 x 3 x 4 = 48; block sizes drawn
    uniformly in `sizes` per direction) of a channel [0, Lx] x [y_w, H]
    x [0, Lz], H = 1, with a sin^2 bump y_w = bump H sin^2(pi (x - 1))
    (3/4 + cos(2 pi z / Lz) / 4) on x in [1, 2], wall-normal tanh stretching
    at both walls (first cell
    first_cell x H), uniform in x and z.  Inflow (BCInflow) at imin, outflow
    (BCOutflow) at imax, no-slip walls (BCWallViscous) at jmin / jmax,
    periodic in z; every block face inside the channel (and the z period) is
    a 1-to-1 matching interface.  Free stream Mach `mach`, Re_H = reynolds,
    AUSM+(P) o3, ro nutilde = nutilde_ratio x mu, plus a seeded density
    perturbation of relative size `perturb`.  The x of every vertex is
    shifted by skew x (x step) x sin(2 pi z / Lz), so that no block is
    homogeneous in k (all are general 3-d zones).  The wall distance is the
    vertical distance to the nearer wall.

    `parts` (three lists of block sizes) overrides the random decomposition,
    e.g. one block per direction for the single-block version of the same
    mesh and initial field; `model` / `wall` select Euler with slip walls.

    Returns (t, tc): tc = 1-to-1 transfer lists (dicts dnr, rcv, dnr_idx,
    rcv_idx; receiver ghost cells of the face bands <- donor interior cells)."""
    rng = np.random.default_rng(seed)
    if parts is None:
        parts = [rng.integers(lo, hi + 1, size=nb) for nb, (lo, hi) in zip(nblocks, sizes)]
    parts = [np.asarray(q, dtype=np.int64) for q in parts]
    nblocks = tuple(len(q) for q in parts)
    offs = [np.concatenate([[0], np.cumsum(p)]) for p in parts]
    NI, NJ, NK = (int(o[-1]) for o in offs)
    Lx, H, Lz = length
    ng = NG
    s = _tanh_both_ends(NJ, first_cell)
    # ghost vertices: linear extrapolation in i (uniform x) and j, periodic in k
    jj = np.arange(-ng, NJ + ng + 1)
    sj = np.empty(jj.size)
    inner = (jj >= 0) & (jj <= NJ)
    sj[inner] = s[jj[inner]]
    lowj, highj = jj < 0, jj > NJ
    sj[lowj] = s[0] + jj[lowj] * (s[1] - s[0])
    sj[highj] = s[NJ] + (jj[highj] - NJ) * (s[NJ] - s[NJ - 1])

    def ywall(x, z):
        span = 0.75 + 0.25 * np.cos(2.0 * math.pi * z / Lz)
        return np.where((x >= 1.0) & (x <= 2.0),
                        bump * H * np.sin(math.pi * (x - 1.0)) ** 2 * span, 0.0)

    gamma = 1.4
    mu = mach / reynolds
    # density perturbation on the global cell grid (ghosts included), so that
    # every decomposition of the same mesh starts from the same field
    noise = np.random.default_rng(seed + 1).standard_normal((NI + 2 * ng, NJ + 2 * ng, NK + 2 * ng))
    zones, tc = [], []
    for c in range(nblocks[2]):
        for b in range(nblocks[1]):
            for a in range(nblocks[0]):
                n = (int(parts[0][a]), int(parts[1][b]), int(parts[2][c]))
                o = (int(offs[0][a]), int(offs[1][b]), int(offs[2][c]))
                ii = o[0] + np.arange(-ng, n[0] + ng + 1)
                kk = o[2] + np.arange(-ng, n[2] + ng + 1)
                x1 = Lx * ii / NI
                s1 = sj[o[1]:o[1] + n[1] + 2 * ng + 1]
                z1 = Lz * kk / NK
                shape = (ii.size, s1.size, kk.size)
                X = np.broadcast_to(x1[:, None, None] + skew * (Lx / NI) *
                                    np.sin(2.0 * math.pi * z1 / Lz)[None, None, :], shape)
                yw = ywall(X, z1[None, None, :])   # the wall under the vertices' own x
                Y = np.broadcast_to(yw + (H - yw) * s1[None, :, None], shape)
                Z = np.broadcast_to(z1[None, None, :], shape)
                z = I.newZone("blk%02d_%d_%d_%d" % (len(zones), a, b, c), list(X.shape))
                gc = I.createChild(z, "GridCoordinates", "GridCoordinates_t")
                for nm, arr in (("CoordinateX", X), ("CoordinateY", Y), ("CoordinateZ", Z)):
                    I.createChild(gc, nm, "DataArray_t")[1] = np.asfortranarray(arr)
                I.createChild(z, "Rind", "Rind_t", np.array([ng] * 6, dtype=np.int64))
                xc, yc, zc = cell_centers(z)
                ro = 1.0 + perturb * noise[o[0]:o[0] + n[0] + 2 * ng, o[1]:o[1] + n[1] + 2 * ng,
                                           o[2]:o[2] + n[2] + 2 * ng]
                u = mach + 0.0 * xc
                p = 1.0 / gamma + 0.0 * xc
                set_conservative(z, ro, u, 0.0 * xc, 0.0 * xc, p, gamma)
                if model == "NSTurbulent":
                    dist = np.minimum(np.abs(yc - ywall(xc, zc)), np.abs(H - yc))
                    set_spalart(z, nutilde_ratio * mu / ro, dist)
                if a == 0:
                    add_bc(z, "in", "BCInflow", "imin")
                if a == nblocks[0] - 1:
                    add_bc(z, "out", "BCOutflow", "imax")
                if b == 0:
                    add_bc(z, "wall_lo", wall, "jmin")
                if b == nblocks[1] - 1:
                    add_bc(z, "wall_hi", wall, "jmax")
                zones.append((z, (a, b, c), n, o))
    # 1-to-1 interfaces: the two ghost layers of every inner face (and the z
    # period) from the neighbour block's interior cells
    index = {blk: m for m, (_, blk, _, _) in enumerate(zones)}

    def inddm0(n, i, j, k):   # 0-based natural index of Fortran cell (i, j, k)
        nip, njp = n[0] + 2 * ng, n[1] + 2 * ng
        return (i + ng - 1) + (j + ng - 1) * nip + (k + ng - 1) * nip * njp

    for r, (_, blk, n, o) in enumerate(zones):
        for d in range(3):
            for side in (-1, 1):
                nb = list(blk)
                nb[d] += side
                if d == 2:
                    nb[2] %= nblocks[2]
                elif not 0 <= nb[d] < nblocks[d]:
                    continue   # physical boundary
                dn = zones[index[tuple(nb)]][2]
                rcv, dnr = [], []
                t1, t2 = [e for e in range(3) if e != d]
                for m in (1, 2):
                    for q2 in range(1, n[t2] + 1):
                        for q1 in range(1, n[t1] + 1):
                            cr = [0, 0, 0]
                            cr[t1], cr[t2] = q1, q2
                            cr[d] = 1 - m if side < 0 else n[d] + m
                            cd = list(cr)
                            cd[d] = dn[d] + 1 - m if side < 0 else m
                            rcv.append(inddm0(n, *cr))
                            dnr.append(inddm0(dn, *cd))
                tc.append(dict(dnr=index[tuple(nb)], rcv=r, dnr_idx=np.array(dnr, dtype=np.int64),
                               rcv_idx=np.array(rcv, dtype=np.int64)))
    numb = {"temporal_scheme": temporal, "ss_iteration": ss_iteration,
            "modulo_verif": modulo_verif}
    numz = {"scheme": "ausmpred", "slope": "o3", "time_step": time_step,
            "cache_blocking_I": 1000000, "cache_blocking_J": 1000000, "cache_blocking_K": 1000000}
    t = _tree([z for z, _, _, _ in zones], model, numb, numz, mach,
              reynolds if model != "Euler" else 0.0, gamma=gamma, nutilde_ratio=nutilde_ratio)
    return t, tc


def channel_blocks(t):
    """(zone index, (i0, j0, k0) global offset, (ni, nj, nk)) of the blocks
    of a sa_channel tree, in zone order, from the zone names and sizes."""
    out = []
    zs = I.getZones(t)
    dims = [tuple(int(v) - 1 - 2 * NG for v in z[1][:, 0]) for z in zs]
    pos = [tuple(int(q) for q in z[0].split("_")[1:]) for z in zs]
    nb = [max(p[d] for p in pos) + 1 for d in range(3)]
    size = [[0] * nb[d] for d in range(3)]
    for p, n in zip(pos, dims):
        for d in range(3):
            size[d][p[d]] = n[d]
    offs = [np.concatenate([[0], np.cumsum(sz)]) for sz in size]
    for m, (p, n) in enumerate(zip(pos, dims)):
        out.append((m, tuple(int(offs[d][p[d]]) for d in range(3)), n))
    return out


# ------------------------------------------- many independent Taylor-Green
def tgv_batch(ncases=64, sizes=(48, 64, 80, 96), mach=(0.05, 0.3), reynolds=(400.0, 3200.0),
              perturb=1.0e-3, seed=7, ss_iteration=4, modulo_verif=200, prandtl=0.71):
    """`ncases` independent Taylor-Green vortices in one tree (one zone each,
    periodic through BCautoperiod): sizes drawn from `sizes` (cells per side),
    Mach uniform in `mach`, Re log-uniform in `reynolds`, and seeded
    initial-phase perturbations (x, y, z phases shifted by perturb x U(-1, 1)
    times the box length / 2 pi).  Each zone carries its own ReferenceState
    and time step (acoustic CFL 2); implicit LU-SGS with ss_iteration
    sub-iterations."""
    rng = np.random.default_rng(seed)
    t = I.newCGNSTree()
    b = I.newCGNSBase("Base", 3, 3, t)
    I.createChild(b, "FlowEquationSet", "FlowEquationSet_t")
    I.createChild(I.getNodeFromName1(b, "FlowEquationSet"), "GoverningEquations",
                  "GoverningEquations_t", "NSLaminar")
    params = []
    for c in range(ncases):
        n = int(rng.choice(sizes))
        m = float(rng.uniform(*mach))
        re = float(np.exp(rng.uniform(np.log(reynolds[0]), np.log(reynolds[1]))))
        ph = perturb * rng.uniform(-1.0, 1.0, size=3)
        one = taylor_green(n=n, mach=m, reynolds=re, prandtl=prandtl, ss_iteration=ss_iteration,
                           name="tgv%02d" % c)
        z = I.getZones(one)[0]
        if np.any(ph):
            # shift the initial field's phases (the cell-centred formula of
            # taylor_green evaluated at x + phase)
            xc, yc, zc = cell_centers(z)
            gamma = 1.4
            xs, ys, zs = xc + ph[0], yc + ph[1], zc + ph[2]
            u = m * np.sin(xs) * np.cos(ys) * np.cos(zs)
            v = -m * np.cos(xs) * np.sin(ys) * np.cos(zs)
            p = 1.0 / gamma + m * m / 16.0 * (np.cos(2 * xs) + np.cos(2 * ys)) * (np.cos(2 * zs) + 2.0)
            set_conservative(z, p * gamma, u, 0.0 * u, 0.0 * u, p, gamma)
            sol = I.getNodeFromName1(z, I.__FlowSolutionCenters__)
            I.getNodeFromName1(sol, "MomentumY")[1] = np.asfortranarray(p * gamma * v)
            roe = p / (gamma - 1.0) + 0.5 * p * gamma * (u * u + v * v)
            I.getNodeFromName1(sol, "EnergyStagnationDensity")[1] = np.asfortranarray(roe)
        ref = I.getNodeFromName1(I.getBases(one)[0], "ReferenceState")
        z[2].append(ref)
        b[2].append(z)
        params.append({"n": n, "mach": m, "reynolds": re, "phase": ph.tolist()})
    FastC._setNum2Base(t, {"temporal_scheme": "implicit", "ss_iteration": ss_iteration,
                           "modulo_verif": modulo_verif})
    return t, params


# --------------------------------------------------------- overset patch
def _lagrange(x, width):
    """Lagrange weights of the nodes 0..width-1 at position x."""
    w = np.ones(width)
    for m in range(width):
        for q in range(width):
            if q != m:
                w[m] *= (x - q) / (m - q)
    return w


def poly_field(X, Y, Z, degree):
    """Density, u, v and temperature polynomial of degree `degree` in x and
    y (uniform in the periodic z, whose ghost cells then hold the same
    values), positive on [-10, 10]^2."""
    s = [X / 10.0, Y / 10.0]
    terms = [1.0, s[0], s[1]]
    if degree >= 2:
        terms += [s[0] * s[0], s[0] * s[1], s[1] * s[1]]
    if degree >= 3:
        terms += [s[0] ** 3, s[0] * s[1] ** 2]
    if degree >= 4:
        terms += [s[0] ** 4, s[0] ** 2 * s[1] ** 2, s[1] ** 4]
    def comb(c0, step):
        return c0 + sum(step * (1.0 + 0.1 * q) * tm for q, tm in enumerate(terms[1:]))
    return comb(1.0, 0.01), comb(0.5, 0.02), comb(0.0, 0.015), comb(1.0, 0.008)


def overset_patch(n=(40, 40, 4), patch=(24, 20, 4), box=10.0, mach=0.5, types=(2,), shift=0.3,
                  linear=False, numz=None, degree=None):
    """Overset (chimera) pair: zone 0 the periodic isentropic-vortex box
    [-box, box]^2 (n cells, periodic in every direction), zone 1 a finer
    cartesian patch over its centre (patch cells, steps 0.7 x zone 0's, k
    origin shifted by shift x dz, periodic in k).  Every ghost cell of the
    patch's i and j bands (edges included) receives an interpolation of
    zone 0's cell values; receiver t uses types[t % len(types)] (2:
    trilinear, 3: 27-point Lagrange, 5: 125-point Lagrange, 1: nearest
    cell), molecules anchored so that they surround the receiver.  The
    patch's i / j faces carry no BC: their ghosts are the receivers, as
    behind a BCOverlap.  linear: a field linear in x, y, z instead of the
    vortex (every interpolation reproduces it to round-off); degree d (1, 2,
    4): primitive fields polynomial of degree d in x and y (the 27- and
    125-point Lagrange molecules reproduce degree 2, the latter degree 4, to
    round-off; see poly_field).
    Returns (t, transfers) with transfers as fgb_add_interp_transfer
    takes them (one dict)."""
    t = isentropic_vortex(n=n, box=box, mach=mach, numz=numz)
    z0 = I.getZones(t)[0]
    h0 = 2 * box / n[0]
    h1 = 0.7 * h0
    ni, nj, nk = patch
    x1 = (-0.5 * ni * h1, -0.5 * nj * h1, shift * h0)
    z1 = cart_zone("patch", x1, (h1, h1, h0), patch)
    xc, yc, zc = cell_centers(z1)
    x0c, y0c, z0c = cell_centers(z0)
    if degree is not None:
        for zz, (X, Y, Z) in ((z0, (x0c, y0c, z0c)), (z1, (xc, yc, zc))):
            ro, u, v, T = poly_field(X, Y, Z, degree)
            set_conservative(zz, ro, u, v, 0.0 * X, ro * T / 1.4, 1.4)
    elif linear:
        for zz, (X, Y, Z) in ((z0, (x0c, y0c, z0c)), (z1, (xc, yc, zc))):
            ro = 1.0 + 0.01 * X + 0.02 * Y + 0.001 * Z
            set_conservative(zz, ro, 0.5 + 0.003 * X, 0.002 * Y, 0.0 * X, 1.0 / 1.4 + 0.001 * X, 1.4)
    else:
        r2 = xc * xc + yc * yc
        e = np.exp(0.5 * (1.0 - r2))
        du, dv = -5.0 / (2 * math.pi) * yc * e, 5.0 / (2 * math.pi) * xc * e
        T = 1.0 - 0.4 * 25.0 / (8.0 * 1.4 * math.pi ** 2) * e * e
        ro = T ** 2.5
        set_conservative(z1, ro, mach + du, dv, 0.0 * ro, ro * T / 1.4, 1.4)
    for f in ("kmin", "kmax"):
        add_bc(z1, "per_" + f, "BCautoperiod", f)
    I.getBases(t)[0][2].append(z1)
    z1[2].append(copy.deepcopy(I.getNodeFromName1(z0, ".Solver#define")))
    # receivers: the ghost cells of the i and j bands of the patch
    ng = NG
    nip, njp = ni + 2 * ng, nj + 2 * ng
    nip0, njp0 = n[0] + 2 * ng, n[1] + 2 * ng
    rcv, dnr, ty, co = [], [], [], []
    for k in range(ng, nk + ng):
        for j in range(njp):
            for i in range(nip):
                if ng <= i < ni + ng and ng <= j < nj + ng:
                    continue
                x, y, zz = xc[i, j, k], yc[i, j, k], zc[i, j, k]
                typ = types[len(rcv) % len(types)]
                # position in zone 0's cell-centre index space (cell l has
                # centre -box + (l - ng + 0.5) h0 in x and y, (l - ng + 0.5) dz in z)
                fx = (x + box) / h0 - 0.5 + ng
                fy = (y + box) / h0 - 0.5 + ng
                fz = zz / h0 - 0.5 + ng
                w = {1: 1, 2: 2, 3: 3, 5: 5}[typ]
                base = [int(math.floor(f)) - (w - 1) // 2 if w > 2 else int(math.floor(f))
                        for f in (fx, fy, fz)]
                if w == 1:
                    base = [int(round(f)) for f in (fx, fy, fz)]
                rel = [f - b for f, b in zip((fx, fy, fz), base)]
                if typ == 1:
                    c = [1.0]
                elif typ == 2:
                    wx, wy, wz = ([1 - r, r] for r in rel)
                    c = [wx[a] * wy[b] * wz[d] for d in range(2) for b in range(2) for a in range(2)]
                else:
                    c = np.concatenate([_lagrange(r, w) for r in rel]).tolist()
                rcv.append(i + j * nip + k * nip * njp)
                dnr.append(base[0] + base[1] * nip0 + base[2] * nip0 * njp0)
                ty.append(typ)
                co.extend(c)
    tr = dict(dnr=0, rcv=1, dnr_idx=np.array(dnr, dtype=np.int64),
              rcv_idx=np.array(rcv, dtype=np.int64), types=np.array(ty, dtype=np.int64),
              coefs=np.array(co, dtype=np.float64))
    return t, [tr]
