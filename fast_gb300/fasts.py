"""FastS Python API of the solve step, on the GB300 library.

Same entry points, arguments and tree conventions as FastS/FastS/PyTree.py:
``warmup`` (:341), ``_compute`` (:42), ``display_temporal_criteria`` (:2039),
``_createConvergenceHistory`` (:2152), ``_extractConvergenceHistory``
(:2245) and ``allocate_metric`` (the ``fasts.allocate_metric`` C call).
The work dictionary is the module global ``HOOK`` (FastC.HOOK in the
reference); it owns the GPU solver handle.  Every numerical operation runs in
libfastgb300.so on the GPU; this module only moves the tree's compacted
time-level arrays to and from the device.
"""
from __future__ import annotations

import math
import sys

import numpy as np

from . import connector
from . import fastc as FastC
from . import metric
from . import pytree as I
from ._native import Solver

HOOK: dict | None = None
FIRST_IT = 0
PREPARED_FIRST_IT = 0   # first_iter of the last prepare (1: a restart with its _M1 level)


# --------------------------------------------------------------- metric
def _coords(z):
    gc = I.getNodeFromName1(z, "GridCoordinates")
    return [I.getNodeFromName1(gc, n)[1] for n in ("CoordinateX", "CoordinateY", "CoordinateZ")]


def allocate_metric(z, nssiter, verbose=0):
    """fasts.allocate_metric (FastS/FastS/Metric/allocate_metric.cpp:40-200):
    zone sizes into Parameter_int, zone type (FastC nature_geom_dom.for), and
    the metric list [ti|tj|tk|vol, ti0, vent, ti_df, rdm, ind_dm, it_lu, degen]
    (METRIC_* slots of FastS/FastS/param_solver.h)."""
    o = I.getNodeFromName1(z, ".Solver#ownData")
    pi = I.getNodeFromName1(o, "Parameter_int")[1]
    dims = I.getZoneDim(z)
    ni, nj, nk = dims[1], dims[2], dims[3]
    ific = 2
    pi[FastC.NIJK_XYZ:FastC.NIJK_XYZ + 5] = [ni, nj, nk, ific, 0 if nk == 2 else ific]
    pi[FastC.NIJK:FastC.NIJK + 5] = [ni - 1, nj - 1, nk - 1, ific, 0 if nk == 2 else ific]
    pi[FastC.IJKV:FastC.IJKV + 3] = [pi[0] - 2 * pi[3], pi[1] - 2 * pi[3], pi[2] - 2 * pi[4]]
    pi[FastC.NDIMDX] = pi[0] * pi[1] * pi[2]
    pi[FastC.NDIMDX_XYZ] = ni * nj * nk
    # allocate_metric.cpp:101-117: the o5 slopes (5, 7) need three ghost
    # layers (a Rind of 3 on every side), the others use two
    if int(pi[FastC.SLOPE]) in (5, 7):
        rind = I.getNodeFromName1(z, "Rind")
        need = 12 if nk == 2 else 18
        if rind is None or int(np.sum(np.asarray(rind[1])[:4 if nk == 2 else 6])) != need:
            raise ValueError("Fast: ghostcell number insufficient for o(5) slope (Rind 3 needed)")
        ific = 3
        pi[FastC.NIJK_XYZ:FastC.NIJK_XYZ + 5] = [ni, nj, nk, ific, 0 if nk == 2 else ific]
        pi[FastC.NIJK:FastC.NIJK + 5] = [ni - 1, nj - 1, nk - 1, ific, 0 if nk == 2 else ific]
        pi[FastC.IJKV:FastC.IJKV + 3] = [pi[0] - 2 * pi[3], pi[1] - 2 * pi[3], pi[2] - 2 * pi[4]]
        pi[FastC.NDIMDX] = pi[0] * pi[1] * pi[2]
    x, y, z_ = _coords(z)
    typ = _zone_type(x, y, z_, nk)
    if typ == 1:
        # A 3-d zone with a homogeneous k direction (nature_geom_dom.for's
        # type 1: z = z(k) on a constant step, x and y independent of k)
        # runs as a general 3-d zone: the reference's *_3dhomo_* variants are
        # the *_3dfull_* formulas with the vanishing metric components
        # dropped (e.g. Compute/Normale/normale_3dhomo_i.for against
        # normale_3dfull_i.for), so the general kernels, on the full metric
        # of the same mesh, compute the same quantities; the one difference
        # is a k-face norm taken as sqrt(tcz^2) instead of |tcz|, within a
        # rounding of it.
        typ = 0
    pi[FastC.ITYPZONE] = typ
    nijk_mtr, ndm, neq_ij, neq_k = metric.dims(pi[FastC.NIJK_XYZ:FastC.NIJK_XYZ + 5], typ)
    pi[FastC.NIJK_MTR:FastC.NIJK_MTR + 5] = nijk_mtr
    pi[FastC.NDIMDX_MTR] = ndm
    pi[FastC.NEQ_IJ] = neq_ij
    pi[FastC.NEQ_K] = neq_k
    itypcp = pi[FastC.ITYPCP]
    pi[FastC.NEQ] = 6 if pi[FastC.IFLOW] == 3 else 5
    pi[FastC.NEQ_COE] = (6 if pi[FastC.IFLOW] == 3 else 5) if itypcp <= 1 else 1
    pi[FastC.ITYPVENT] = 2
    pi[FastC.NEQ_VENT] = 3
    pi[FastC.NDIMDX_VENT] = 1
    # cp_tijk.for / cp_vol.for
    ti, tj, tk, vol = metric.compute(x, y, z_, typ, ng=ific, ngk=int(pi[FastC.NIJK + 4]))
    mtr = np.concatenate([ti, tj, tk, vol])
    ijkv_lu = [max(1, int(pi[FastC.IJKV + d]) // int(pi[FastC.SIZE_SSDOM + d])) for d in range(3)]
    rdm = np.zeros(int(nssiter) * int(pi[FastC.NEQ]) * 2 * ijkv_lu[0] * ijkv_lu[1] * ijkv_lu[2])
    return [mtr, None, None, None, rdm, None, None, None]


def _zone_type(x, y, z, nk, tol=2.0e-8):
    """FastC/FastC/Metric/nature_geom_dom.for: 3 = 2d (nk = 2 vertices),
    2 = 3d cartesian with constant steps, 1 = 3d with a homogeneous k
    direction (z = z(k) with a constant step, x and y independent of k),
    0 = general."""
    if nk == 2:
        return 3
    dx = np.diff(x, axis=0)
    dy = np.diff(y, axis=1)
    dz = np.diff(z, axis=2)
    cart = (np.ptp(np.diff(x, axis=1)) < tol and np.ptp(np.diff(x, axis=2)) < tol and
            np.ptp(np.diff(y, axis=0)) < tol and np.ptp(np.diff(y, axis=2)) < tol and
            np.ptp(np.diff(z, axis=0)) < tol and np.ptp(np.diff(z, axis=1)) < tol)
    cte = np.ptp(dx) < tol and np.ptp(dy) < tol and np.ptp(dz) < tol
    if cart and cte:
        return 2
    zcart = np.ptp(np.diff(z, axis=0)) < tol and np.ptp(np.diff(z, axis=1)) < tol
    if zcart and np.ptp(dz) < tol and np.ptp(np.diff(x, axis=2)) < tol and \
            np.ptp(np.diff(y, axis=2)) < tol:
        return 1
    return 0


def metric_arrays(pi, mtr):
    """Split the metric list slot into (ti, tj, tk, vol) views."""
    ndm = int(pi[FastC.NDIMDX_MTR])
    nij, nk_ = int(pi[FastC.NEQ_IJ]), int(pi[FastC.NEQ_K])
    ti = mtr[:ndm * nij]
    tj = mtr[ndm * nij:2 * ndm * nij]
    tk = mtr[2 * ndm * nij:2 * ndm * nij + ndm * nk_]
    vol = mtr[2 * ndm * nij + ndm * nk_:2 * ndm * nij + ndm * nk_ + ndm]
    return ti, tj, tk, vol


# --------------------------------------------------------------- warmup
def prepare(t):
    """Host part of warmup (no GPU): numerics packing, metric, BC block,
    primitive variables.  Returns the metric list of every zone."""
    zones = I.getZones(t)
    FastC._buildOwnData(t)
    dtloc = I.getNodeFromName1(I.getNodeFromName1(t, ".Solver#ownData"), ".Solver#dtloc")[1]
    nssiter = int(dtloc[0])
    metrics = [allocate_metric(z, nssiter) for z in zones]
    FastC._BCcompact(t)
    global PREPARED_FIRST_IT
    PREPARED_FIRST_IT = FastC._createPrimVars(t)
    return metrics


def cfl_time_step(t, cfl):
    """Global time step that gives the CFL number ``cfl`` on the tree's
    current state, by the local time-step formula of cpcfl3.for
    (FastS/FastS/Compute/cpcfl3.for:88-140, LALE = 0): per interior cell
    comp = min(vis, conv) with conv = 2 vol surf / (|u| + c), vis =
    2 ro vol^2 surf^2 Pr / (gamma mu) (Navier-Stokes only) and surf = 1 /
    max over directions of the sum of the two face-normal norms; the CFL of a
    cell is dt / comp, so dt = cfl x the smallest comp over every zone.
    Euler and laminar zones (mu from invist.for).  The tree is not
    modified: the state is read from a copy prepared as warmup does."""
    import copy
    tt = copy.deepcopy(t)
    ms = prepare(tt)
    best = math.inf
    for zd in zone_data(tt, ms):
        pi, pr = zd["pi"], zd["pr"]
        if int(pi[FastC.IFLOW]) > 2:
            raise ValueError("cfl_time_step: Euler and laminar zones only")
        nd = int(pi[FastC.NDIMDX])
        ni, nj, nk = (int(pi[FastC.IJKV + d]) for d in range(3))
        ng, ngk = int(pi[FastC.NIJK + 3]), int(pi[FastC.NIJK + 4])
        nip, njp = int(pi[FastC.NIJK]), int(pi[FastC.NIJK + 1])
        k, j, i = np.meshgrid(np.arange(1, nk + 1), np.arange(1, nj + 1), np.arange(1, ni + 1),
                              indexing="ij")
        l = ((i + ng - 1) + (j + ng - 1) * nip + (k + ngk - 1) * nip * njp).reshape(-1)
        typ = int(pi[FastC.ITYPZONE])
        ti, tj, tk, vol = zd["ti"], zd["tj"], zd["tk"], zd["vol"]
        if typ == 2:       # 3-d cartesian: one metric value per family
            dd = [np.sqrt(a[0] * a[0]) + np.sqrt(a[0] * a[0]) for a in (ti, tj, tk)]
            surf = 1.0 / max(dd)
            vv = vol[0]
        else:
            minc = [int(pi[FastC.NIJK_MTR + d]) for d in range(3)]
            mg, mgk = int(pi[FastC.NIJK_MTR + 3]), int(pi[FastC.NIJK_MTR + 4])
            ndm = int(pi[FastC.NDIMDX_MTR])
            lt = ((i + mg - 1) * minc[0] + (j + mg - 1) * minc[1] + (k + mgk - 1) * minc[2]).reshape(-1)
            ncomp = 2 if typ == 3 else 3
            dd = []
            for dd_d, a in enumerate((ti, tj, tk)):
                if typ == 3 and dd_d == 2:
                    dd.append(np.zeros(lt.size))
                    continue
                hi = lt + minc[dd_d]
                sa = sum(a[hi + c * ndm] * a[hi + c * ndm] for c in range(ncomp))
                sb = sum(a[lt + c * ndm] * a[lt + c * ndm] for c in range(ncomp))
                dd.append(np.sqrt(sa) + np.sqrt(sb))
            surf = 1.0 / np.maximum(np.maximum(dd[0], dd[1]), dd[2])
            vv = vol[lt]
        q = zd["ro"]
        r, u, v, w, temp = (q[l + m * nd] for m in range(5))
        gam = pr[FastC.GAMMA]
        rgp = pr[FastC.CVINF] * (gam - 1.0)
        c = np.sqrt(gam * rgp * temp)
        conv = 2.0 * vv * surf * (1.0 / (np.sqrt(u * u + v * v + w * w) + c))
        comp = conv
        if int(pi[FastC.IFLOW]) == 2:     # invist.for viscosity
            cs = pr[FastC.CS]
            temp01 = 1.0 / pr[FastC.TEMP0]
            coesut = pr[FastC.XMUL0] * (1.0 + cs * temp01) * math.sqrt(temp01)
            xmut = coesut * np.sqrt(temp) * temp / (temp + cs)
            vis = 2.0 * r * vv * vv * surf * surf * ((gam / pr[FastC.PRANDT]) / xmut)
            comp = np.minimum(vis, conv)
        best = min(best, float(np.min(comp)))
    return cfl * best


def zone_data(t, metrics):
    """Per zone: param_int, param_real, metric views and the three compacted
    time levels (flat float64 views into the tree)."""
    out = []
    for z, m in zip(I.getZones(t), metrics):
        o = I.getNodeFromName1(z, ".Solver#ownData")
        pi = I.getNodeFromName1(o, "Parameter_int")[1]
        pr = I.getNodeFromName1(o, "Parameter_real")[1]
        ti, tj, tk, vol = metric_arrays(pi, m[0])
        d = dict(pi=pi, pr=pr, ti=ti, tj=tj, tk=tk, vol=vol,
                 ro=FastC.compactArray(z, "").reshape(-1),
                 ro_m1=FastC.compactArray(z, "_M1").reshape(-1),
                 ro_p1=FastC.compactArray(z, "_P1").reshape(-1))
        if int(pi[FastC.NEQ]) == 6:
            sol = I.getNodeFromName1(z, I.__FlowSolutionCenters__)
            d["dist"] = np.ascontiguousarray(
                I.getNodeFromName1(sol, "TurbulentDistance")[1].ravel(order="F"), dtype=np.float64)
        out.append(d)
    return out


def transfer_list(t, tc):
    """The interface transfers of ``tc``: a Connector tc tree (ID_ zone
    subregions with PointList / PointListDonor / InterpolantsType /
    InterpolantsDonor, read by fast_gb300.connector), or a list of transfer
    dicts (dnr, rcv, dnr_idx, rcv_idx[, types, coefs]), or None."""
    if tc is None:
        return []
    if connector.is_tree(tc):
        return connector.transfers_from_tc(t, tc)
    return list(tc)


def warmup(t, tc=None, graph=None, infos_ale=None, Adjoint=False, tmy=None, list_graph=None,
           Padding=None, verbose=0, device=0, gpu_resident=False):
    """FastS/FastS/PyTree.py:341: numerics, metric, primitive variables,
    ghost cells; creates the GPU solver in HOOK.  ``tc`` is the Connector
    donor tree FastS takes (1-to-1 and overset ID_ subregions, read once
    here: the connectivity does not change between _compute calls), or a
    list of transfer dicts (see transfer_list).  With ``gpu_resident`` the state stays on the GPU between
    ``_compute`` calls and the tree is refreshed by ``_syncHost``."""
    global HOOK, FIRST_IT
    metrics = prepare(t)
    zones = I.getZones(t)
    dtloc = I.getNodeFromName1(I.getNodeFromName1(t, ".Solver#ownData"), ".Solver#dtloc")[1]
    nssiter = int(dtloc[0])
    if _temporal_scheme(t) == "explicit_local":
        # FastS prepares an explicit_local tree, but its C layer -- the one
        # this solver replaces -- refuses to compute it (PyTree.py:75-76);
        # only its Python layer, through Cassiopee's Connector transfers,
        # runs it.  No GPU solver is built; _compute raises FastS's error.
        FIRST_IT = PREPARED_FIRST_IT
        HOOK = {"solver": None, "nssiter": nssiter, "FIRST_IT": FIRST_IT,
                "gpu_resident": bool(gpu_resident), "zones": zones, "device_valid": False}
        return t, tc, metrics
    solver = Solver(device)
    for n, zd in enumerate(zone_data(t, metrics)):
        solver.add_zone(zd["pi"], zd["pr"], zd["ti"], zd["tj"], zd["tk"], zd["vol"])
        if "dist" in zd:
            solver.set_wall_distance(n, zd["dist"])
    for tr in transfer_list(t, tc):
        solver.add_any_transfer(tr)
    solver.set_option("modulo_verif", int(dtloc[1]))
    FIRST_IT = PREPARED_FIRST_IT
    solver.set_option("first_it", FIRST_IT)
    HOOK = {"solver": solver, "nssiter": nssiter, "FIRST_IT": FIRST_IT,
            "gpu_resident": bool(gpu_resident), "zones": zones, "device_valid": False}
    # the tree's time levels are what _compute copies in and out: page-lock
    # them so that those copies are DMA transfers
    for z in zones:
        for suf in ("", "_M1", "_P1"):
            arr = FastC.compactArray(z, suf).reshape(-1)
            if arr.flags.c_contiguous and arr.nbytes > 0:
                try:
                    solver.pin(arr)
                except RuntimeError:   # not page-lockable: copies stay staged by the driver
                    pass
    _upload(t)
    for lvl in (0, 1):
        solver.apply_bc(lvl)
    _download(t)
    return t, tc, metrics


def _upload(t):
    s = HOOK["solver"]
    for n, z in enumerate(I.getZones(t)):
        for lvl, suf in enumerate(("", "_M1", "_P1")):
            s.upload(n, lvl, FastC.compactArray(z, suf).reshape(-1))
    HOOK["device_valid"] = True


def _download(t):
    s = HOOK["solver"]
    for n, z in enumerate(I.getZones(t)):
        for lvl, suf in enumerate(("", "_M1", "_P1")):
            s.download(n, lvl, FastC.compactArray(z, suf).reshape(-1))


def _temporal_scheme(t):
    """.Solver#define/temporal_scheme of the tree (FastS's default: implicit)."""
    d = I.getNodeFromName1(t, ".Solver#define")
    a = I.getNodeFromName1(d, "temporal_scheme") if d is not None else None
    return I.getValue(a) if a is not None else "implicit"


def _itypcp(z):
    o = I.getNodeFromName1(z, ".Solver#ownData")
    return int(I.getNodeFromName1(o, "Parameter_int")[1][FastC.ITYPCP])


def _syncHost(t):
    """Copy the GPU state of every time level back into the tree."""
    _download(t)


def _compute(t, metrics, nitrun, tc=None, graph=None, tc2=None, graph2=None, layer="c",
             NIT=1, ucData=None, vtune=None):
    """FastS/FastS/PyTree.py:42 (layer 'c'): NIT physical steps of all the
    sub-steps through fasts._computePT -> fgb_compute, then the time-level
    rotation (done on the device; the tree arrays receive the new levels)."""
    global FIRST_IT
    if _temporal_scheme(t) == "explicit_local" and layer == "c":   # PyTree.py:73-76
        raise ValueError("compute: 'explicit_local' & 'c layer' is not implemented.")
    if HOOK is None:
        raise RuntimeError("warmup must be called before _compute")
    if layer != "c":
        raise NotImplementedError("only layer='c' is implemented")
    s = HOOK["solver"]
    zones = I.getZones(t)
    if not HOOK["gpu_resident"]:
        # inputs of the step: levels n and n-1 as the tree holds them (the
        # page-locked tree arrays are copied on a side stream; level n-1
        # arrives while the first sub-step computes its fluxes)
        for n, z in enumerate(zones):
            s.upload_async(n, 0, FastC.compactArray(z, "").reshape(-1))
            s.upload_async(n, 1, FastC.compactArray(z, "_M1").reshape(-1))
    s.set_option("first_it", HOOK["FIRST_IT"])
    s.compute(nitrun, 1, HOOK["nssiter"], 1, NIT)
    if not HOOK["gpu_resident"]:
        # the device rotated its levels after every physical step; the tree
        # does the same by swapping arrays (FastC.switchPointers__), so only
        # the new level n is copied back (into the array that becomes n)
        # (an explicit RK3 step overwrites level n with its second stage,
        # which then becomes n-1, so that level is copied back too)
        rot = NIT % 3
        explicit = HOOK["nssiter"] <= 3 and _itypcp(zones[0]) == 2
        if explicit and HOOK["nssiter"] % 2 == 0:
            # RK2 ends in level n itself and the levels keep their places
            # (PyTree.py:228, switchPointers__ order 2); level n+1 holds
            # the first stage
            for n, z in enumerate(zones):
                s.download(n, 0, FastC.compactArray(z, "").reshape(-1))
                s.download(n, 2, FastC.compactArray(z, "_P1").reshape(-1))
            HOOK["FIRST_IT"] = 1
            FIRST_IT = 1
            return None
        for n, z in enumerate(zones):
            for _ in range(rot):
                FastC.switchPointers__([z])
            s.download(n, 0, FastC.compactArray(z, "").reshape(-1))
            if rot != 1 or explicit:
                s.download(n, 1, FastC.compactArray(z, "_M1").reshape(-1))
            if rot != 1:
                s.download(n, 2, FastC.compactArray(z, "_P1").reshape(-1))
    HOOK["FIRST_IT"] = 1
    FIRST_IT = 1
    return None


# ----------------------------------------------------- convergence data
def display_temporal_criteria(t, metrics, nitrun, format=None, gmres=None, verbose="firstlast",
                              stopAtNan=True):
    """FastS/FastS/PyTree.py:2039 -> fasts.display_ss_iteration: Newton
    residual norms per zone (L2 = sqrt(sum/ncell)/dt, Loo = max/dt), printed
    (format None/'double'), stored in ZoneConvergenceHistory ('store'), or
    the stored records written out: 'flush' to residuals.bin, 'ascii' to
    residuals.dat (conv2pytree.for, lft = -1 / -2)."""
    s = HOOK["solver"]
    s.synchronize()
    zones = I.getZones(t)
    resL2, resLoo = 0.0, -1.0e15
    for n, z in enumerate(zones):
        res = s.residuals(n)
        if res.shape[1] == 0:
            continue
        # CFL_minmaxmoy of the zone's numerics (computePT.cpp:629-644),
        # printed as display_ss_iteration.cpp:100-105 does
        node = I.getNodeFromName2(z, "CFL_minmaxmoy")
        if node is not None:
            cfl = s.cfl(n)
            node[1] = np.array(cfl, dtype=np.float64)
            if (format is None or format == "double") and verbose != "none":
                print("CFL_MOY_MAX_MIN(Zone= %32.32s, nitrun=%d) %f    %f    %f " % (
                    z[0], nitrun, cfl[2], cfl[0], cfl[1]))
        neq = res.shape[0] // 2
        L2, Loo = res[:neq], res[neq:]
        resL2 += float(L2.sum())
        resLoo = max(resLoo, float(Loo.max()))
        cut = 1.0e-30
        cvg = np.concatenate([np.log10(np.maximum(L2[:, 0], cut)),
                              np.log10(np.maximum(Loo[:, 0], cut)),
                              np.log10(np.maximum(L2[:, -1], cut)) - np.log10(np.maximum(L2[:, 0], cut)),
                              np.log10(np.maximum(Loo[:, -1], cut)) - np.log10(np.maximum(Loo[:, 0], cut))])
        if format == "store":
            _store_history(z, nitrun, neq, cvg)
        elif format in ("flush", "ascii"):
            _write_history(z, neq, binary=format == "flush")
        elif format is None or format == "double":
            if verbose != "none":
                for it in range(L2.shape[1]):
                    if verbose == "firstlast" and it not in (0, L2.shape[1] - 1):
                        continue
                    print("%s it=%d ss=%d L2 %s Loo %s" % (
                        z[0], nitrun, it + 1,
                        " ".join("%7.3f" % math.log10(max(v, 1e-30)) for v in L2[:, it]),
                        " ".join("%7.3f" % math.log10(max(v, 1e-30)) for v in Loo[:, it])))
    if stopAtNan and not (np.isfinite(resL2) and np.isfinite(resLoo)):
        print("Nan in the residual: stop.")
        sys.exit(1)
    return {"L2": resL2, "Loo": resLoo}


def _createConvergenceHistory(t, nrecs):
    """FastS/FastS/PyTree.py:2152: ZoneConvergenceHistory of nrecs records."""
    for z in I.getZones(t):
        pi = I.getNodeFromName1(I.getNodeFromName1(z, ".Solver#ownData"), "Parameter_int")[1]
        neq = int(pi[FastC.NEQ])
        ch = I.createUniqueChild(z, "ZoneConvergenceHistory", "ConvergenceHistory_t", 0)
        I.createUniqueChild(ch, "IterationNumber", "DataArray_t")[1] = np.zeros(nrecs, np.int64)
        for name in ("RSD_L2", "RSD_oo", "RSD_L2_diff", "RSD_oo_diff"):
            I.createUniqueChild(ch, name, "DataArray_t")[1] = np.zeros(nrecs * neq)


def _store_history(z, nitrun, neq, cvg):
    """conv2pytree.for:56-66 (lft >= 0 branch)."""
    ch = I.getNodeFromName1(z, "ZoneConvergenceHistory")
    if ch is None:
        return
    last = int(I.getValue(ch))
    it = I.getNodeFromName1(ch, "IterationNumber")[1]
    if last >= it.size:
        return
    it[last] = nitrun
    for k, name in enumerate(("RSD_L2", "RSD_oo", "RSD_L2_diff", "RSD_oo_diff")):
        I.getNodeFromName1(ch, name)[1][last * neq:(last + 1) * neq] = cvg[k * neq:(k + 1) * neq]
    ch[1] = np.array([last + 1], dtype=np.int64)


# INTEGER_E of the reference's Fortran: 4 bytes in Cassiopee's default build
# (8 with E_DOUBLEINT); the width the residuals.bin records are written with
RESIDUALS_BIN_INT = np.int32


def _write_history(z, neq, binary, directory="."):
    """conv2pytree.for:22-55 (lft < 0): the records stored in the zone's
    ZoneConvergenceHistory appended to residuals.bin (format 'flush', lft =
    -1: one Fortran unformatted sequential record per call -- 4-byte length
    markers around zone name (40 characters, blank padded), neq, LastRec and,
    per stored iteration, its number then (L2, Loo) of every equation; the
    stored records are then released, LastRec = 0) or residuals.dat (format
    'ascii', lft = -2: the Tecplot text of the same records)."""
    import os
    ch = I.getNodeFromName1(z, "ZoneConvergenceHistory")
    if ch is None:
        return
    last = int(I.getValue(ch))
    it = I.getNodeFromName1(ch, "IterationNumber")[1]
    l2 = I.getNodeFromName1(ch, "RSD_L2")[1]
    oo = I.getNodeFromName1(ch, "RSD_oo")[1]
    name = z[0][:40].ljust(40).encode()
    if binary:
        body = bytearray(name)
        body += np.array([neq, last], dtype=RESIDUALS_BIN_INT).tobytes()
        for r in range(last):
            body += np.array([it[r]], dtype=RESIDUALS_BIN_INT).tobytes()
            pair = np.empty(2 * neq)
            pair[0::2] = l2[r * neq:(r + 1) * neq]
            pair[1::2] = oo[r * neq:(r + 1) * neq]
            body += pair.astype("<f8").tobytes()
        mark = np.array([len(body)], dtype="<i4").tobytes()
        with open(os.path.join(directory, "residuals.bin"), "ab") as f:
            f.write(mark + bytes(body) + mark)
        ch[1] = np.array([0], dtype=np.int64)
        return
    path = os.path.join(directory, "residuals.dat")
    head = not os.path.exists(path) or os.path.getsize(path) == 0
    eqs = ["Ro", "RoU", "RoV", "RoW", "RoE"] + (["Nut"] if neq == 6 else [])
    with open(path, "a") as f:
        if head:
            f.write("VARIABLES=\"It\" " + " ".join('"%s_L2"' % e for e in eqs) + " " +
                    " ".join('"%s_oo"' % e for e in eqs) + "\n")
        f.write('ZONE T="%s"\n' % z[0][:40])
        for r in range(last):
            vals = []
            for e in range(neq):
                vals += [l2[r * neq + e], oo[r * neq + e]]
            f.write("%7d" % it[r] + "".join(" %15.8E" % v for v in vals) + "\n")


def read_residuals_bin(path="residuals.bin"):
    """The records of a residuals.bin file: list of (zone name, iteration
    numbers (LastRec), L2 (LastRec, neq), Loo (LastRec, neq))."""
    out = []
    data = open(path, "rb").read()
    p = 0
    isz = np.dtype(RESIDUALS_BIN_INT).itemsize
    while p < len(data):
        n = int(np.frombuffer(data, "<i4", 1, p)[0])
        body = data[p + 4:p + 4 + n]
        p += 8 + n
        name = body[:40].decode().rstrip()
        neq, last = (int(x) for x in np.frombuffer(body, RESIDUALS_BIN_INT, 2, 40))
        q = 40 + 2 * isz
        its, l2, oo = [], [], []
        for _ in range(last):
            its.append(int(np.frombuffer(body, RESIDUALS_BIN_INT, 1, q)[0]))
            q += isz
            pair = np.frombuffer(body, "<f8", 2 * neq, q)
            q += 16 * neq
            l2.append(pair[0::2].copy())
            oo.append(pair[1::2].copy())
        out.append((name, np.array(its), np.array(l2).reshape(last, neq), np.array(oo).reshape(last, neq)))
    return out


def _extractConvergenceHistory(t, fileout):
    """FastS/FastS/PyTree.py:2245: write the stored records as residuals.dat
    (conv2pytree.for text layout: It, L2 per equation, Loo per equation)."""
    names5 = ["Ro", "RoU", "RoV", "RoW", "RoE", "Nut"]
    with open(fileout, "w") as f:
        for nd, z in enumerate(I.getZones(t)):
            ch = I.getNodeFromName1(z, "ZoneConvergenceHistory")
            if ch is None:
                continue
            last = int(I.getValue(ch))
            it = I.getNodeFromName1(ch, "IterationNumber")[1]
            l2 = I.getNodeFromName1(ch, "RSD_L2")[1]
            oo = I.getNodeFromName1(ch, "RSD_oo")[1]
            neq = l2.size // max(it.size, 1)
            if nd == 0:
                f.write("VARIABLES=\"It\" " + " ".join('"%s_L2"' % n for n in names5[:neq]) + " " +
                        " ".join('"%s_oo"' % n for n in names5[:neq]) + "\n")
            f.write('ZONE T="%s"\n' % z[0])
            for r in range(last):
                vals = [l2[r * neq + j] for j in range(neq)] + [oo[r * neq + j] for j in range(neq)]
                f.write("%7d " % it[r] + " ".join("%15.8E" % v for v in vals) + "\n")
