"""Cell-face normals and cell volumes of a structured zone (set-up, host).

Restates FastC/FastC/Metric/cp_tijk.for and cp_vol.for for the 3-d general
(ITYPZONE 0) and 3-d cartesian (ITYPZONE 2) zone types, with the array
dimensions of FastC/FastC/Metric/nature_geom_dom.for.  Like the reference,
this runs once when a zone is set up, on the host; every expression keeps
the Fortran operation order (numpy evaluates one IEEE operation per
ufunc, without contraction), so the arrays are the reference's bits.

Layout: ti, tj, tk have NEQ_IJ / NEQ_K components of NDIMDX_MTR values
each; a general zone indexes them on the vertex grid (lt = indmtr(i,j,k) =
flat Fortran index of vertex (i,j,k) including ghosts), a cartesian zone
holds one value per direction.
"""
from __future__ import annotations

import numpy as np


def dims(nijk_xyz, typ):
    """(NIJK_MTR[5], NDIMDX_MTR, NEQ_IJ, NEQ_K) of nature_geom_dom.for:284-362."""
    nvi, nvj, nvk, ng, ngk = (int(v) for v in nijk_xyz)
    if typ == 2:
        return [0, 0, 0, 0, 0], 1, 1, 1
    if typ == 0:
        return [1, nvi, nvi * nvj, ng, ngk], nvi * nvj * nvk, 3, 3
    if typ == 3:   # nature_geom_dom.for:117-126
        return [1, nvi, 0, ng, ngk], nvi * nvj, 2, 0
    raise NotImplementedError(f"zone type {typ} (3-d with a homogeneous k direction) "
                              "is not implemented: only 3-d general (0), 3-d cartesian (2) and 2-d (3)")


def _faces_i(x, y, z):
    """I-face normal*area (cp_tijk.for:91-101) from the 4 vertices
    (i,j,k), (i,j+1,k), (i,j,k+1), (i,j+1,k+1) given as slices."""
    (x0, x1, x2, x3), (y0, y1, y2, y3), (z0, z1, z2, z3) = x, y, z
    tix10 = (y1 - y0) * (z3 - z0) - (z1 - z0) * (y3 - y0)
    tiy10 = (z1 - z0) * (x3 - x0) - (x1 - x0) * (z3 - z0)
    tiz10 = (x1 - x0) * (y3 - y0) - (y1 - y0) * (x3 - x0)
    tix11 = (y2 - y3) * (z0 - z2) - (z2 - z3) * (y0 - y2)
    tiy11 = (z2 - z3) * (x0 - x2) - (x2 - x3) * (z0 - z2)
    tiz11 = (x2 - x3) * (y0 - y2) - (y2 - y3) * (x0 - x2)
    return 0.5 * (tix10 + tix11), 0.5 * (tiy10 + tiy11), 0.5 * (tiz10 + tiz11)


def _faces_j(x, y, z):
    """J-face (cp_tijk.for:103-112) from vertices (i,j,k), (i+1,j,k),
    (i,j,k+1), (i+1,j,k+1) = l0, l4, l2, l6."""
    (x0, x4, x2, x6), (y0, y4, y2, y6), (z0, z4, z2, z6) = x, y, z
    tjx10 = (y0 - y4) * (z2 - z0) - (z0 - z4) * (y2 - y0)
    tjy10 = (z0 - z4) * (x2 - x0) - (x0 - x4) * (z2 - z0)
    tjz10 = (x0 - x4) * (y2 - y0) - (y0 - y4) * (x2 - x0)
    tjx11 = (y6 - y2) * (z4 - z6) - (z6 - z2) * (y4 - y6)
    tjy11 = (z6 - z2) * (x4 - x6) - (x6 - x2) * (z4 - z6)
    tjz11 = (x6 - x2) * (y4 - y6) - (y6 - y2) * (x4 - x6)
    return 0.5 * (tjx10 + tjx11), 0.5 * (tjy10 + tjy11), 0.5 * (tjz10 + tjz11)


def _faces_k(x, y, z):
    """K-face (cp_tijk.for:114-123) from vertices (i,j,k), (i+1,j,k),
    (i,j+1,k), (i+1,j+1,k) = l0, l4, l1, l5."""
    (x0, x4, x1, x5), (y0, y4, y1, y5), (z0, z4, z1, z5) = x, y, z
    tkx10 = (y4 - y0) * (z5 - z4) - (z4 - z0) * (y5 - y4)
    tky10 = (z4 - z0) * (x5 - x4) - (x4 - x0) * (z5 - z4)
    tkz10 = (x4 - x0) * (y5 - y4) - (y4 - y0) * (x5 - x4)
    tkx11 = (y1 - y5) * (z0 - z1) - (z1 - z5) * (y0 - y1)
    tky11 = (z1 - z5) * (x0 - x1) - (x1 - x5) * (z0 - z1)
    tkz11 = (x1 - x5) * (y0 - y1) - (y1 - y5) * (x0 - x1)
    return 0.5 * (tkx10 + tkx11), 0.5 * (tky10 + tky11), 0.5 * (tkz10 + tkz11)


def _corners(a, sl_i, sl_j, sl_k):
    """The 8 vertex slices l0..l7 of cp_tijk.for:82-89 for the cells
    selected by (sl_i, sl_j, sl_k) on the vertex grid."""
    def s(di, dj, dk):
        def sh(sl, d):
            return slice(sl.start + d, sl.stop + d if sl.stop is not None else None)
        return a[sh(sl_i, di), sh(sl_j, dj), sh(sl_k, dk)]
    return (s(0, 0, 0), s(0, 1, 0), s(0, 0, 1), s(0, 1, 1),
            s(1, 0, 0), s(1, 1, 0), s(1, 0, 1), s(1, 1, 1))


def compute(x, y, z, typ, ng=2, ngk=2):
    """Metric arrays (ti, tj, tk, vol) as flat float64 arrays, for vertex
    coordinates x, y, z of shape (nvi, nvj, nvk) including ng (ngk in k)
    ghost layers.  typ: 0 (3-d general) or 2 (3-d cartesian)."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    z = np.asarray(z, dtype=np.float64)
    nvi, nvj, nvk = x.shape
    if typ == 2:
        # cp_tijk.for:291-330 / cp_vol.for:148-175 at cell (1,1,1) (lt = 1)
        c = [[a[ng + di, ng + dj, ngk + dk] for (di, dj, dk) in
              ((0, 0, 0), (0, 1, 0), (0, 0, 1), (0, 1, 1), (1, 0, 0), (1, 1, 0), (1, 0, 1), (1, 1, 1))]
             for a in (x, y, z)]
        X, Y, Z = c
        ti = _faces_i((X[0], X[1], X[2], X[3]), (Y[0], Y[1], Y[2], Y[3]), (Z[0], Z[1], Z[2], Z[3]))[0]
        tj = _faces_j((X[0], X[4], X[2], X[6]), (Y[0], Y[4], Y[2], Y[6]), (Z[0], Z[4], Z[2], Z[6]))[1]
        tk = _faces_k((X[0], X[4], X[1], X[5]), (Y[0], Y[4], Y[1], Y[5]), (Z[0], Z[4], Z[1], Z[5]))[2]
        ax = 0.25 * ((((X[4] + X[5]) + X[7]) + X[6]) * ti - (((X[0] + X[1]) + X[3]) + X[2]) * ti)
        ay = 0.25 * ((((Y[1] + Y[3]) + Y[5]) + Y[7]) * tj - (((Y[0] + Y[2]) + Y[4]) + Y[6]) * tj)
        az = 0.25 * ((((Z[2] + Z[3]) + Z[6]) + Z[7]) * tk - (((Z[0] + Z[1]) + Z[4]) + Z[5]) * tk)
        vol = max(((ax + ay) + az) / 3.0, 1.0e-30)
        return (np.array([ti]), np.array([tj]), np.array([tk]), np.array([vol]))
    if typ == 3:
        return _compute_2d(x, y, z)
    if typ != 0:
        raise NotImplementedError(f"zone type {typ}")
    shape = (nvi, nvj, nvk)
    ti = np.zeros((3,) + shape)
    tj = np.zeros((3,) + shape)
    tk = np.zeros((3,) + shape)
    cells = (slice(0, nvi - 1), slice(0, nvj - 1), slice(0, nvk - 1))
    cx, cy, cz = (_corners(a, *cells) for a in (x, y, z))
    # all cells of the zone, ghosts included (indice_omp1.h: ind_mtr)
    r = _faces_i(cx[:4], cy[:4], cz[:4])
    for c in range(3):
        ti[c][cells] = r[c]
    sel = (0, 4, 2, 6)
    r = _faces_j(tuple(cx[s] for s in sel), tuple(cy[s] for s in sel), tuple(cz[s] for s in sel))
    for c in range(3):
        tj[c][cells] = r[c]
    sel = (0, 4, 1, 5)
    r = _faces_k(tuple(cx[s] for s in sel), tuple(cy[s] for s in sel), tuple(cz[s] for s in sel))
    for c in range(3):
        tk[c][cells] = r[c]
    # last faces: i = imax+1, j = jmax+1, k = kmax+1 (cp_tijk.for:127-194)
    fi = (slice(nvi - 1, nvi), slice(0, nvj - 1), slice(0, nvk - 1))
    fx, fy, fz = (_corners(a, *fi) for a in (x, y, z))
    r = _faces_i(fx[:4], fy[:4], fz[:4])
    for c in range(3):
        ti[c][fi] = r[c]
    fj = (slice(0, nvi - 1), slice(nvj - 1, nvj), slice(0, nvk - 1))
    fx, fy, fz = (_corners_lo(a, *fj) for a in (x, y, z))
    r = _faces_j(fx, fy, fz)
    for c in range(3):
        tj[c][fj] = r[c]
    fk = (slice(0, nvi - 1), slice(0, nvj - 1), slice(nvk - 1, nvk))
    fx, fy, fz = (_corners_k(a, *fk) for a in (x, y, z))
    r = _faces_k(fx, fy, fz)
    for c in range(3):
        tk[c][fk] = r[c]
    # volumes (cp_vol.for:74-113); lip / ljp / lkp = the cell's far faces
    X, Y, Z = cx, cy, cz
    i1 = (slice(1, nvi), slice(0, nvj - 1), slice(0, nvk - 1))
    j1 = (slice(0, nvi - 1), slice(1, nvj), slice(0, nvk - 1))
    k1 = (slice(0, nvi - 1), slice(0, nvj - 1), slice(1, nvk))
    comp = []
    for c, A in enumerate((X, Y, Z)):
        s1 = ((A[4] + A[5]) + A[7]) + A[6]
        s2 = ((A[0] + A[1]) + A[3]) + A[2]
        s3 = ((A[1] + A[3]) + A[5]) + A[7]
        s4 = ((A[0] + A[2]) + A[4]) + A[6]
        s5 = ((A[2] + A[3]) + A[6]) + A[7]
        s6 = ((A[0] + A[1]) + A[4]) + A[5]
        acc = s1 * ti[c][i1] - s2 * ti[c][cells]
        acc = acc + s3 * tj[c][j1]
        acc = acc - s4 * tj[c][cells]
        acc = acc + s5 * tk[c][k1]
        acc = acc - s6 * tk[c][cells]
        comp.append(0.25 * acc)
    vol = np.zeros(shape)
    vol[cells] = np.maximum(((comp[0] + comp[1]) + comp[2]) / 3.0, 1.0e-30)
    return (np.concatenate([ti[c].reshape(-1, order="F") for c in range(3)]),
            np.concatenate([tj[c].reshape(-1, order="F") for c in range(3)]),
            np.concatenate([tk[c].reshape(-1, order="F") for c in range(3)]),
            vol.reshape(-1, order="F"))


def _corners_lo(a, sl_i, sl_j, sl_k):
    """Vertices l0, l4, l2, l6 of a j-face at the last vertex row j."""
    j = sl_j.start
    return (a[sl_i.start:sl_i.stop, j:j + 1, sl_k.start:sl_k.stop],
            a[sl_i.start + 1:sl_i.stop + 1, j:j + 1, sl_k.start:sl_k.stop],
            a[sl_i.start:sl_i.stop, j:j + 1, sl_k.start + 1:sl_k.stop + 1],
            a[sl_i.start + 1:sl_i.stop + 1, j:j + 1, sl_k.start + 1:sl_k.stop + 1])


def _corners_k(a, sl_i, sl_j, sl_k):
    """Vertices l0, l4, l1, l5 of a k-face at the last vertex plane k."""
    k = sl_k.start
    return (a[sl_i.start:sl_i.stop, sl_j.start:sl_j.stop, k:k + 1],
            a[sl_i.start + 1:sl_i.stop + 1, sl_j.start:sl_j.stop, k:k + 1],
            a[sl_i.start:sl_i.stop, sl_j.start + 1:sl_j.stop + 1, k:k + 1],
            a[sl_i.start + 1:sl_i.stop + 1, sl_j.start + 1:sl_j.stop + 1, k:k + 1])


def _is_torch(a):
    return type(a).__module__.startswith("torch")


def _zeros(shape, like):
    if _is_torch(like):
        import torch
        return torch.zeros(shape, dtype=like.dtype, device=like.device)
    return np.zeros(shape)


def _flat_f(a):
    """Fortran-order flattening of a 2-d array (numpy or torch)."""
    return a.t().reshape(-1) if _is_torch(a) else a.reshape(-1, order="F")


def _compute_2d(x, y, z):
    """2-d zone (one cell in k, no k ghosts): cp_tijk.for 2-d branch (i and
    j faces, x and y components) and cp_vol.for 2-d branch, on the vertex
    grid of the k = 1 layer (lt = flat index of vertex (i, j)).  Takes numpy
    or torch arrays (the same operations in the same order, so the same
    values; torch arrays keep the autograd graph from the coordinates)."""
    nvi, nvj, _ = x.shape
    ti = _zeros((2, nvi, nvj), x)
    tj = _zeros((2, nvi, nvj), x)
    cells = (slice(0, nvi - 1), slice(0, nvj - 1))
    def v(a, di, dj, dk):
        return a[di:nvi - 1 + di, dj:nvj - 1 + dj, dk]
    X = [v(x, *o) for o in ((0, 0, 0), (0, 1, 0), (0, 0, 1), (0, 1, 1), (1, 0, 0), (1, 1, 0), (1, 0, 1), (1, 1, 1))]
    Y = [v(y, *o) for o in ((0, 0, 0), (0, 1, 0), (0, 0, 1), (0, 1, 1), (1, 0, 0), (1, 1, 0), (1, 0, 1), (1, 1, 1))]
    Z = [v(z, *o) for o in ((0, 0, 0), (0, 1, 0), (0, 0, 1), (0, 1, 1), (1, 0, 0), (1, 1, 0), (1, 0, 1), (1, 1, 1))]
    r = _faces_i(X[:4], Y[:4], Z[:4])
    ti[0][cells], ti[1][cells] = r[0], r[1]
    sel = (0, 4, 2, 6)
    r = _faces_j(tuple(X[q] for q in sel), tuple(Y[q] for q in sel), tuple(Z[q] for q in sel))
    tj[0][cells], tj[1][cells] = r[0], r[1]
    # last faces i = imax+1, j = jmax+1
    fi = [a[nvi - 1:nvi, 0:nvj - 1, 0] for a in (x, y, z)]
    fi1 = [a[nvi - 1:nvi, 1:nvj, 0] for a in (x, y, z)]
    fi2 = [a[nvi - 1:nvi, 0:nvj - 1, 1] for a in (x, y, z)]
    fi3 = [a[nvi - 1:nvi, 1:nvj, 1] for a in (x, y, z)]
    r = _faces_i(*[(fi[c], fi1[c], fi2[c], fi3[c]) for c in range(3)])
    ti[0][nvi - 1:nvi, 0:nvj - 1], ti[1][nvi - 1:nvi, 0:nvj - 1] = r[0], r[1]
    fj = [a[0:nvi - 1, nvj - 1:nvj, 0] for a in (x, y, z)]
    fj4 = [a[1:nvi, nvj - 1:nvj, 0] for a in (x, y, z)]
    fj2 = [a[0:nvi - 1, nvj - 1:nvj, 1] for a in (x, y, z)]
    fj6 = [a[1:nvi, nvj - 1:nvj, 1] for a in (x, y, z)]
    r = _faces_j(*[(fj[c], fj4[c], fj2[c], fj6[c]) for c in range(3)])
    tj[0][0:nvi - 1, nvj - 1:nvj], tj[1][0:nvi - 1, nvj - 1:nvj] = r[0], r[1]
    i1 = (slice(1, nvi), slice(0, nvj - 1))
    j1 = (slice(0, nvi - 1), slice(1, nvj))
    comp = []
    for c, A in enumerate((X, Y)):
        s1 = ((A[4] + A[5]) + A[7]) + A[6]
        s2 = ((A[0] + A[1]) + A[3]) + A[2]
        s3 = ((A[1] + A[3]) + A[5]) + A[7]
        s4 = ((A[0] + A[2]) + A[4]) + A[6]
        acc = s1 * ti[c][i1] - s2 * ti[c][cells]
        acc = acc + s3 * tj[c][j1]
        acc = acc - s4 * tj[c][cells]
        comp.append(0.25 * acc)
    tkz10 = (X[4] - X[0]) * (Y[5] - Y[4]) - (Y[4] - Y[0]) * (X[5] - X[4])
    tkz11 = (X[1] - X[5]) * (Y[0] - Y[1]) - (Y[1] - Y[5]) * (X[0] - X[1])
    tk1 = 0.5 * (tkz10 + tkz11)
    az = 0.25 * (((((((Z[2] + Z[3]) + Z[6]) + Z[7]) - Z[0]) - Z[1]) - Z[4]) - Z[5]) * tk1
    vol = _zeros((nvi, nvj), x)
    v = ((comp[0] + comp[1]) + az) / 3.0
    vol[cells] = v.clamp_min(1.0e-30) if _is_torch(v) else np.maximum(v, 1.0e-30)
    if _is_torch(x):
        import torch
        return (torch.cat([_flat_f(ti[c]) for c in range(2)]),
                torch.cat([_flat_f(tj[c]) for c in range(2)]),
                _zeros((0,), x), _flat_f(vol))
    return (np.concatenate([ti[c].reshape(-1, order="F") for c in range(2)]),
            np.concatenate([tj[c].reshape(-1, order="F") for c in range(2)]),
            np.zeros(0),
            vol.reshape(-1, order="F"))
