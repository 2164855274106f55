"""FastC services used by the solve step, restated for the GB300 build.

Mirrors the parts of FastC/FastC/PyTree.py that the FastS solve step needs:
numerics dictionaries (_setNum2Base / _setNum2Zones, keys4Base / keys4Zone,
:115-132, :929-1026), their packing into ``Parameter_int`` (137 ints) and
``Parameter_real`` (73 doubles) (_buildOwnData, :920-2045), the BC block
(_BCcompact, :2788-3038, window conversion of FastC/FastC/getRange.cpp:57-99),
primitive-variable creation (createPrimVars, :215) and the compaction of each
time level into one contiguous structure-of-arrays buffer (_compact, :2236).

Cassiopee's ReferenceState helpers are not available, so
``addReferenceState`` builds that node from Mach / Reynolds numbers with its
own documented non-dimensionalisation (rho = 1, T = 1, sound speed = 1).
"""
from __future__ import annotations

import math
import warnings

import numpy as np

from . import pytree as I

# FastS/FastS/param_solver.h index map (the part the packer fills)
NIJK, NIJK_MTR, NIJK_XYZ, IJKV = 0, 5, 10, 20
MXSSDOM_LU, ITYPZONE, ITYPVENT, IFLOW, ILES, ITYPCP, SIZE_SSDOM = 24, 25, 26, 27, 28, 29, 30
KFLUDOM, LALE, IFLAGFLT, NEQ, NEQ_IJ, NEQ_K, NEQ_COE, NEQ_VENT = 33, 34, 35, 36, 37, 38, 39, 40
NDIMDX, NDIMDX_XYZ, NDIMDX_MTR, NDIMDX_VENT, IO_THREAD, DTLOC = 41, 42, 43, 44, 45, 46
SA_INT, RK, LEVEL, EXPLOC, NSSITER, SLOPE, PT_BC, NB_RELAX, LU_MATCH = 47, 52, 53, 54, 58, 64, 70, 71, 75
DTC, GAMMA, CVINF, ROINF, PINF, VINF, TINF, MINF = 0, 1, 2, 3, 4, 5, 6, 7
REYNOLDS, PRANDT, XMUL0, TEMP0, CS, EPSI_NEWTON, CFL, PSIROE, WIG_AMP = 9, 10, 11, 12, 13, 14, 15, 34, 72
N_PARAM_INT, N_PARAM_REAL = 137, 73

# FastC/FastC/PyTree.py:29-83 (the NS subset)
tagBCDict = {
    "BCExtrapolate": 0, "BCDegenerateLine": 0, "BCFarfield": 1, "BCInflowSupersonic": 2,
    "BCWallInviscid": 3, "BCSymmetryPlane": 3, "BCWall": 4, "FamilySpecified": 5,
    "BCWallViscous": 6, "BCWallViscous_isot_fich": 7, "BC_fich": 8, "Nearmatch": 9,
    "BCOutflow": 10, "BCautoperiod": 11, "BCWallViscous_transition": 12, "BCInflow": 13,
    "BCExtrapolateRANS": 14, "BCPeriodic": 15, "BCOutpres": 16, "BCInj1": 17,
    "BCRacinf": 18, "BCInflowLund": 19, "BCInjMFR": 20, "BCOutMFR": 21, "BCOverlap": 22,
    "BCWallModel": 30, "BCWallExchange": 31, "BCWallViscousIsothermal": 32,
}

keys4Base = {
    "temporal_scheme": ["explicit", "implicit", "implicit_local", "explicit_local"],
    "ss_iteration": 0, "rk": 0, "modulo_verif": 0, "exp_local": 0, "time_begin_ale": 1,
    "omp_mode": 0, "explicit_local_type": 0,
}
keys4Zone = {
    "scheme": ["ausmpred", "senseur", "roe_min", "roe", "roe_nul", "roe_kap", "senseur_hyper"],
    "implicit_solver": ["lussor", "gmres"], "nb_relax": 0, "nb_krylov": 0, "nb_restart": 0,
    "motion": ["none", "rigid", "rigid_ext", "deformation"], "rotation": 4, "time_step": 1,
    "io_thread": 0, "sgsmodel": ["smsm", "msm", "Miles"], "wallmodel": ["musker", "power"],
    "wallmodel_sample": 0, "ransmodel": ["SA", "SA_comp", "SA_diff"], "cache_blocking_I": 0,
    "cache_blocking_J": 0, "cache_blocking_K": 0, "shiftvar": 0,
    "time_step_nature": ["local", "global"], "ssdom_IJK": 3, "lu_match": 1, "epsi_newton": 1,
    "epsi_linear": 1, "nudging_ampli": 1, "nudging_vector": 3, "inj1_newton_tol": 1,
    "inj1_newton_nit": 0, "cfl": 1, "niveaux_temps": 0, "psiroe": 1, "ausmDamping": 1,
    "coef_hyper": 4, "prandtltb": 1, "sfd": 0, "sfd_chi": 1, "sfd_delta": 1, "sfd_init_iter": 0,
    "slope": ["o1", "o3", "o5", "minmod", "o3sc", "o5sc", "vanalbada"],
    "DES": ["zdes1", "zdes1_w", "zdes2", "zdes2_w", "zdes3", "zdes3_w"], "SA_add_LowRe": 0,
    "SA_add_RotCorr": 0, "snear": 1, "DES_debug": 0, "extract_res": 0, "IBC": 3, "source": 0,
    "Cups": 4, "senseurType": 0, "ratiom": 1,
}


def checkKeys(d, keys):
    """Warn (do not fail) on unknown keys or values, as FastC.checkKeys does."""
    for c in d[2]:
        k = c[0]
        if k not in keys:
            warnings.warn(f"Fast: numerics: {k} is not a valid key.")
            continue
        allowed = keys[k]
        if isinstance(allowed, list):
            v = I.getValue(c)
            if v not in allowed:
                warnings.warn(f"Fast: numerics: {v} is not a valid value for {k}.")


def _setNum2Base(a, num):
    """FastC/FastC/PyTree.py:132: numerics of the base ('.Solver#define' of t)."""
    d = I.createUniqueChild(a, ".Solver#define", "UserDefinedData_t")
    for k, v in num.items():
        I.createUniqueChild(d, k, "DataArray_t", v)


def _setNum2Zones(a, num):
    """FastC/FastC/PyTree.py:115: numerics of every zone."""
    for z in I.getZones(a):
        d = I.createUniqueChild(z, ".Solver#define", "UserDefinedData_t")
        for k, v in num.items():
            I.createUniqueChild(d, k, "DataArray_t", v)


# ---------------------------------------------------------------- state
def addReferenceState(t, mach=0.5, reynolds=1.0e6, gamma=1.4, prandtl=0.72,
                      sutherland=True, alpha_deg=0.0, beta_deg=0.0, nutilde_ratio=0.1,
                      ts_over_tinf=1.0, cs_over_tinf=110.4 / 288.15):
    """Create the ReferenceState of every base.

    Non-dimensionalisation (own convention): free-stream density, temperature
    and speed of sound are 1, the reference length is 1.  Hence p = 1/gamma,
    R = 1/gamma, cv = R/(gamma-1), |U| = mach and the laminar viscosity
    mu = |U| / reynolds.  Sutherland: Mus = mu at Ts, Cs = 0 switches the law
    to mu ~ sqrt(T) (the FastS formula with Cs = 0, invist.for).
    """
    ro, tinf = 1.0, 1.0
    p = 1.0 / gamma
    rgas = p / (ro * tinf)
    cv = rgas / (gamma - 1.0)
    a_ = math.radians(alpha_deg)
    b_ = math.radians(beta_deg)
    u = mach * math.cos(a_) * math.cos(b_)
    v = mach * math.sin(a_) * math.cos(b_)
    w = mach * math.sin(b_)
    mu = mach / reynolds if reynolds > 0 else 0.0
    roe = p / (gamma - 1.0) + 0.5 * ro * (u * u + v * v + w * w)
    ts = ts_over_tinf * tinf
    cs = cs_over_tinf * tinf if sutherland else 0.0
    values = {
        "Density": ro, "MomentumX": ro * u, "MomentumY": ro * v, "MomentumZ": ro * w,
        "EnergyStagnationDensity": roe, "Pressure": p, "Temperature": tinf, "Cv": cv,
        "Mach": mach, "Reynolds": reynolds, "Gamma": gamma, "Rok": 0.0, "RoOmega": 0.0,
        "TurbulentSANuTildeDensity": nutilde_ratio * mu, "Mus": mu, "Cs": cs, "Ts": ts,
        "Pr": prandtl,
    }
    for b in I.getBases(t):
        ref = I.createUniqueChild(b, "ReferenceState", "ReferenceState_t")
        for k, val in values.items():
            I.createUniqueChild(ref, k, "DataArray_t", float(val))


def getState(ref):
    """The 19-entry state vector in Cassiopee's order (C.getState)."""
    g = lambda n: float(I.getValue(I.getNodeFromName1(ref, n)))
    return [g("Density"), g("MomentumX"), g("MomentumY"), g("MomentumZ"),
            g("EnergyStagnationDensity"), g("Pressure"), g("Temperature"), g("Cv"),
            g("Mach"), g("Reynolds"), g("Cs"), g("Gamma"), g("Rok"), g("RoOmega"),
            g("TurbulentSANuTildeDensity"), g("Mus"), g("Cs"), g("Ts"), g("Pr")]


# ------------------------------------------------------------- numerics
def _zone_numerics(t, b, z):
    """Defaults of FastC/FastC/PyTree.py:1290-1380 overridden by .Solver#define."""
    d0 = I.getNodeFromName1(t, ".Solver#define")
    base = dict(temporal_scheme="implicit", ss_iteration=30, rk=3, modulo_verif=200,
                exp_local=0)
    if d0 is not None:
        checkKeys(d0, keys4Base)
        for c in d0[2]:
            base[c[0]] = I.getValue(c)
    zn = dict(scheme="ausmpred", slope="o3", implicit_solver="lussor", nb_relax=1,
              lu_match=0, time_step=-0.000001, epsi_newton=0.1, psiroe=0.1, ausmDamping=1.0,
              cfl=1.0, ssdom_IJK=[240, 20, 900], time_step_nature="global", motion="none",
              cache_blocking_I=2048, cache_blocking_J=2, cache_blocking_K=7, prandtltb=None,
              io_thread=0, ratiom=10000.0, senseurType=1)
    d = I.getNodeFromName1(z, ".Solver#define")
    if d is not None:
        checkKeys(d, keys4Zone)
        for c in d[2]:
            zn[c[0]] = I.getValue(c)
    return base, zn


def _buildOwnData(t):
    """Pack numerics into .Solver#ownData/Parameter_int|real (PyTree.py:920-2045)."""
    base, _ = _zone_numerics(t, None, I.getZones(t)[0])
    temporal = base["temporal_scheme"]
    rk = int(base.get("rk", 3))
    if temporal in ("implicit", "implicit_local"):
        rk = 3
    # time level of every zone (PyTree.py:1080-1110): with explicit_local the
    # value of centers:niveaux_temps in the zone's middle cell, otherwise
    # .Solver#define/niveaux_temps (default 1)
    veclevel = [_time_level(z, temporal) for z in I.getZones(t)]
    maxlevel = max(veclevel)
    exploc = 0
    if temporal == "explicit":
        nssiter = {1: 1, 2: 2, 3: 3}[rk]
    elif temporal in ("implicit", "implicit_local"):
        nssiter = int(base["ss_iteration"]) + 1
    elif temporal == "explicit_local":   # PyTree.py:1163-1166: RK3, 4 sub-steps per level
        nssiter = 4 * maxlevel
        rk = 3
        exploc = 1
    else:
        raise NotImplementedError(f"temporal_scheme {temporal} is not supported")
    o = I.createUniqueChild(t, ".Solver#ownData", "UserDefinedData_t")
    dtloc = np.zeros(12 + 1, dtype=np.int64)
    dtloc[0] = nssiter
    dtloc[1] = int(base["modulo_verif"])
    dtloc[6] = rk
    dtloc[9] = maxlevel
    I.createUniqueChild(o, ".Solver#dtloc", "DataArray_t", dtloc)
    for ndom, (b, z) in enumerate((b, z) for b in I.getBases(t) for z in I.getZones(b)):
        _, zn = _zone_numerics(t, b, z)
        model = "Euler"
        ge = I.getNodeFromName2(z, "GoverningEquations") or I.getNodeFromName2(b, "GoverningEquations")
        if ge is not None:
            model = I.getValue(ge)
        iflow = {"Euler": 1, "euler": 1, "NSLaminar": 2, "nslaminar": 2, "NSLes": 2,
                 "nsles": 2, "NSTurbulent": 3, "nsspalart": 3}.get(model)
        if iflow is None:
            raise ValueError(f"Fast: model {model} is invalid.")
        itypcp = 2 if temporal in ("explicit", "explicit_local") else 1
        slope = zn["slope"]
        # "vanalbada" (8) is not a FastS slope: a smooth limiter for the adjoint
        islope = {"o1": 1, "o2": 4, "o3": 2, "o5": 5, "minmod": 3, "o3sc": 6, "o5sc": 7,
                  "vanalbada": 8}[slope]
        scheme = zn["scheme"]
        kfludom = {"ausmpred": 1, "senseur": 2, "dfcentre6": 3, "roe_kap": 5, "roe_min": 5,
                   "roe_nul": 5, "roe": 5, "senseur_hyper": 8}[scheme]
        if scheme == "roe_kap":
            islope = 2
        elif scheme == "roe_min":
            islope = 3
        elif scheme == "roe_nul":
            islope = 1
        lale = {"none": 0, "rigid": 1, "rigid_ext": 2, "deformation": 3}[zn["motion"]]
        dtl = 0 if zn["time_step_nature"] == "global" else 1
        size_ssdom = [100, 10, 10]
        if temporal == "implicit_local":
            size_ssdom = list(zn["ssdom_IJK"])
        ref = I.getNodeFromName1(z, "ReferenceState") or I.getNodeFromName1(b, "ReferenceState")
        adim = getState(ref) if ref is not None else None
        pi = np.full(N_PARAM_INT, -1000, dtype=np.int64)
        pi[0:25] = -1
        pi[25] = 0
        pi[26] = 0
        pi[IFLOW] = iflow
        pi[ILES] = 0
        pi[ITYPCP] = itypcp
        pi[SIZE_SSDOM:SIZE_SSDOM + 3] = size_ssdom
        pi[KFLUDOM] = kfludom
        pi[LALE] = lale
        pi[IFLAGFLT] = 0
        pi[36:45] = -1
        pi[IO_THREAD] = int(zn["io_thread"])
        pi[DTLOC] = dtl
        pi[47:52] = [0, 1, 2, 0, 0]
        pi[RK] = rk
        pi[LEVEL] = veclevel[ndom]
        pi[EXPLOC] = exploc
        pi[55] = 0
        pi[56] = 1
        pi[57] = 0
        pi[NSSITER] = nssiter
        pi[59:62] = [zn["cache_blocking_I"], zn["cache_blocking_J"], zn["cache_blocking_K"]]
        pi[62] = 0
        pi[63] = 1
        pi[SLOPE] = islope
        pi[65] = 10
        pi[66] = 0
        pi[67] = 0
        pi[68] = 0
        pi[69] = 0
        pi[PT_BC] = 0
        pi[NB_RELAX] = int(zn["nb_relax"])
        pi[72] = 1
        pi[73] = 20
        pi[74] = {"lussor": 0, "gmres": 1}[zn["implicit_solver"]]
        pi[LU_MATCH] = int(zn["lu_match"])
        pi[76:83] = 0
        pi[83] = 0
        pi[84] = 1
        pi[85] = int(zn["senseurType"])
        pi[86] = -1
        pi[87] = 0
        pi[88] = 4
        pi[132] = 0
        pi[129] = -1
        pi[130] = 0
        pi[131] = 0
        pi[134] = ndom
        pr = np.zeros(N_PARAM_REAL, dtype=np.float64)
        dtc = float(zn["time_step"])
        if dtc < 0:
            if dtl == 0:
                warnings.warn("Fast: time_step_nature global requires a time_step value. "
                              "time_step set to default value (0.0001).")
            dtc = 0.0001
        pr[DTC] = dtc
        if adim is not None:
            pr[GAMMA] = adim[11]
            pr[CVINF] = adim[7]
            pr[ROINF] = adim[0]
            pr[PINF] = adim[5]
            pr[VINF] = math.sqrt(adim[1] ** 2 + adim[2] ** 2 + adim[3] ** 2) / adim[0]
            pr[TINF] = adim[6]
            pr[MINF] = adim[8]
            pr[8] = adim[14]
            pr[REYNOLDS] = adim[9]
            pr[PRANDT] = adim[18]
            pr[XMUL0] = adim[15]
            pr[TEMP0] = adim[17]
            pr[CS] = adim[16]
            pr[19] = adim[1] / adim[0]
            pr[20] = adim[2] / adim[0]
            pr[21] = adim[3] / adim[0]
        pr[EPSI_NEWTON] = float(zn["epsi_newton"])
        pr[CFL] = float(zn["cfl"])
        pr[16], pr[17], pr[18] = 0.01, 0.2, float(zn["ratiom"])
        pr[PSIROE] = float(zn["psiroe"])
        pr[35], pr[36], pr[37] = 0.0, 1.0e15, 1.0e-5
        pr[38] = float(zn["prandtltb"]) if zn["prandtltb"] is not None else (
            adim[18] if adim is not None else 1.0)
        pr[39] = 0.01
        pr[40] = 1.0
        pr[55], pr[56] = 0.009, 0.015
        pr[57], pr[58], pr[59] = 3, 1, 0
        pr[WIG_AMP] = float(zn["ausmDamping"])
        o = I.createUniqueChild(z, ".Solver#ownData", "UserDefinedData_t")
        I.createUniqueChild(o, "Parameter_int", "DataArray_t", pi)
        I.createUniqueChild(o, "Parameter_real", "DataArray_t", pr)
        I.createUniqueChild(o, "CFL_minmaxmoy", "DataArray_t", [0.0, 0.0, 0.0])
        I.createUniqueChild(o, "model", "DataArray_t", model)
        I.createUniqueChild(o, "temporal_scheme", "DataArray_t", temporal)
    return None


def _time_level(z, temporal):
    """PyTree.py:1087-1100: the zone's time level.  explicit_local: the cell
    value at the 1-based (i, j, k) = (vertex count // 2) of each direction,
    i.e. the 0-based cell (cells + 1) // 2 - 1."""
    if temporal == "explicit_local":
        sol = I.getNodeFromName1(z, I.__FlowSolutionCenters__)
        lv = I.getNodeFromName1(sol, "niveaux_temps") if sol is not None else None
        if lv is None:
            raise ValueError("explicit_local: zone %s has no centers:niveaux_temps" % z[0])
        a = np.asarray(lv[1])
        return int(a[tuple((n + 1) // 2 - 1 for n in a.shape)])
    d = I.getNodeFromName1(z, ".Solver#define")
    a = I.getNodeFromName1(d, "niveaux_temps") if d is not None else None
    return int(I.getValue(a)) if a is not None else 1


def getRange(in_bc, pi):
    """FastC/FastC/getRange.cpp:57-99: vertex PointRange of the ghost-extended
    zone -> window of interior cell indices."""
    f = [0] * 6
    ng, ngk = pi[NIJK + 3], pi[NIJK + 4]
    if in_bc[0] == in_bc[1]:
        f[0] = in_bc[0] - 1 if in_bc[0] > 1 else in_bc[0]
        f[0] = max(1, f[0] - 2 * ng)
        f[1] = f[0]
        f[2] = max(in_bc[2] - ng, 1); f[3] = min(in_bc[3] - ng - 1, pi[IJKV + 1])
        f[4] = max(in_bc[4] - ngk, 1); f[5] = min(in_bc[5] - ngk - 1, pi[IJKV + 2])
    elif in_bc[2] == in_bc[3]:
        f[2] = in_bc[2] - 1 if in_bc[2] > 1 else in_bc[2]
        f[2] = max(1, f[2] - 2 * ng)
        f[3] = f[2]
        f[0] = max(in_bc[0] - ng, 1); f[1] = min(in_bc[1] - ng - 1, pi[IJKV])
        f[4] = max(in_bc[4] - ngk, 1); f[5] = min(in_bc[5] - ngk - 1, pi[IJKV + 2])
    elif in_bc[4] == in_bc[5]:
        f[4] = in_bc[4] - 1 if in_bc[4] > 1 else in_bc[4]
        f[4] = max(1, f[4] - 2 * ngk)
        f[5] = f[4]
        f[0] = max(in_bc[0] - ng, 1); f[1] = min(in_bc[1] - ng - 1, pi[IJKV])
        f[2] = max(in_bc[2] - ng, 1); f[3] = min(in_bc[3] - ng - 1, pi[IJKV + 1])
    return f


def getDir(ijkv, f):
    """FastC/FastC/getRange.cpp:103-111"""
    if f[0] == f[1] and f[0] == 1: return 1
    if f[0] == f[1] and f[0] == ijkv[0]: return 2
    if f[2] == f[3] and f[2] == 1: return 3
    if f[2] == f[3] and f[2] == ijkv[1]: return 4
    if f[4] == f[5] and f[4] == 1: return 5
    if f[4] == f[5] and f[4] == ijkv[2]: return 6
    return 0


def _BCcompact(t):
    """Append the BC block to Parameter_int and the BC data to
    Parameter_real (PyTree.py:2788-3038): at param_int[PT_BC]: [nb_bc,
    ptr_int(nb_bc), ptr_real(nb_bc)], then per BC [type, idir, window(6),
    nbdata, cumulative data sizes(nbdata)]; the DataArray_t nodes found
    within three levels of the BC node (BCDataSet / BCData / DataArray)
    are concatenated at the end of param_real, in that order, and the
    tree's data nodes become views of param_real, as FastC does."""
    for z in I.getZones(t):
        o = I.getNodeFromName1(z, ".Solver#ownData")
        pnode = I.getNodeFromName1(o, "Parameter_int")
        rnode = I.getNodeFromName1(o, "Parameter_real")
        pi = pnode[1]
        bcs = I.getNodesFromType2(z, "BC_t")
        nb = len(bcs)
        bcdata = [I.getNodesFromType3(bc, "DataArray_t") for bc in bcs]
        c = pi.size
        size_int = 1 + nb * 2 + 9 * nb + sum(len(d) for d in bcdata)
        size_real = sum(int(np.asarray(a[1]).size) for d in bcdata for a in d)
        data = np.zeros(c + size_int, dtype=np.int64)
        data[:c] = pi
        data[PT_BC] = c
        data[c] = nb
        cr = rnode[1].size
        real = np.zeros(cr + size_real, dtype=np.float64)
        real[:cr] = rnode[1]
        size = 1 + 2 * nb
        size_r = 0
        for n, bc in enumerate(bcs):
            pt = c + size
            data[c + 1 + n] = pt
            data[c + 1 + n + nb] = cr + size_r
            btype = I.getValue(bc)
            if btype not in tagBCDict:
                raise ValueError(f"compact: unknown BC type {btype}")
            data[pt] = tagBCDict[btype]
            rg = I.getValue(I.getNodeFromType1(bc, "IndexRange_t"))
            in_bc = [int(rg[0, 0]), int(rg[0, 1]), int(rg[1, 0]), int(rg[1, 1]),
                     int(rg[2, 0]), int(rg[2, 1])]
            f = getRange(in_bc, data)
            data[pt + 2:pt + 8] = f
            data[pt + 1] = getDir(data[IJKV:IJKV + 3], f)
            data[pt + 8] = len(bcdata[n])
            ctot = 0
            for j, arr in enumerate(bcdata[n]):
                v = np.asarray(arr[1], dtype=np.float64)
                deb = cr + size_r
                real[deb:deb + v.size] = v.ravel(order="F")
                arr[1] = real[deb:deb + v.size]
                ctot += v.size
                data[pt + 9 + j] = ctot
                size_r += v.size
            size += 9 + len(bcdata[n])
        pnode[1] = data
        rnode[1] = real


# ---------------------------------------------------------- prim vars
CONS = ["Density", "MomentumX", "MomentumY", "MomentumZ", "EnergyStagnationDensity",
        "TurbulentSANuTildeDensity"]
PRIM = ["Density", "VelocityX", "VelocityY", "VelocityZ", "Temperature"]
PRIM_SA = PRIM + ["TurbulentSANuTilde"]


def _prim_names(z):
    """Primitive variables of a zone: 5, or 6 with Spalart-Allmaras."""
    o = I.getNodeFromName1(z, ".Solver#ownData")
    pi = I.getNodeFromName1(o, "Parameter_int")[1]
    return PRIM_SA if int(pi[IFLOW]) == 3 else PRIM


def createPrimVars(t, omp_mode=0, rmConsVars=True, Adjoint=False):
    """FastC/FastC/PyTree.py:215: conservative -> primitive variables at
    centers, plus the _M1 and _P1 time levels, each level compacted into one
    contiguous (NEQ, NDIMDX) array (_compact, :2236).  Works in place and
    returns (t, first_iter, vars_zones) as the reference does: first_iter is
    1 when every zone already holds its _M1 level (a restart: the time
    levels are kept and the next step is BDF2), 0 otherwise (the levels are
    created from the current one, FastC/FastC/PyTree.py:497-509)."""
    first_iter = _createPrimVars(t, omp_mode, rmConsVars, Adjoint)
    vars_zones = [[z, _prim_names(z)] for z in I.getZones(t)]
    return t, first_iter, vars_zones


def _createPrimVars(t, omp_mode=0, rmConsVars=True, Adjoint=False):
    """In-place createPrimVars; returns FIRST_IT."""
    first_iter = 1
    for z in I.getZones(t):
        sol = I.getNodeFromName1(z, I.__FlowSolutionCenters__)
        o = I.getNodeFromName1(z, ".Solver#ownData")
        cv = float(I.getNodeFromName1(o, "Parameter_real")[1][CVINF])
        names = _prim_names(z)
        if len(names) == 6 and I.getNodeFromName1(sol, "TurbulentDistance") is None:
            raise ValueError("createPrimVars: TurbulentDistance field required at cell "
                             "centers for RANS computations.")
        if I.getNodeFromName1(sol, "VelocityX") is None:
            ro = I.getNodeFromName1(sol, "Density")[1]
            rou = I.getNodeFromName1(sol, "MomentumX")[1]
            rov = I.getNodeFromName1(sol, "MomentumY")[1]
            row = I.getNodeFromName1(sol, "MomentumZ")[1]
            roe = I.getNodeFromName1(sol, "EnergyStagnationDensity")[1]
            u, v, w = rou / ro, rov / ro, row / ro
            temp = (roe / ro - 0.5 * (u * u + v * v + w * w)) / cv
            prim = [ro, u, v, w, temp]
        else:
            prim = [I.getNodeFromName1(sol, n)[1] for n in PRIM]
        if len(names) == 6:
            # FastC/FastC/PyTree.py:484-486: nutilde from ro nutilde, else
            # the free-stream ro nutilde over the density
            nu = I.getNodeFromName1(sol, "TurbulentSANuTilde")
            if nu is not None:
                prim.append(nu[1])
            else:
                rnu = I.getNodeFromName1(sol, "TurbulentSANuTildeDensity")
                ronut_inf = float(I.getNodeFromName1(o, "Parameter_real")[1][8])
                prim.append((rnu[1] if rnu is not None else ronut_inf) / prim[0])
        shape = prim[0].shape
        n = prim[0].size
        # one mapping per level: the host gave one 512 MB huge page to each of
        # three mappings, and only one to a single mapping of three levels
        bufs = [_level_buffers(1, len(names), n)[0] for _ in range(3)]
        for suffix, buf in zip(("", "_M1", "_P1"), bufs):
            kept = [I.getNodeFromName1(sol, nm + suffix) for nm in names] if suffix else []
            if suffix and all(k is not None for k in kept):
                src = [k[1] for k in kept]          # a restart: the level is kept
            else:
                src = prim
                if suffix == "_M1":
                    first_iter = 0
            for v_, arr in enumerate(src):
                buf[v_] = np.asarray(arr, dtype=np.float64).ravel(order="F")
            for v_, name in enumerate(names):
                view = buf[v_].reshape(shape, order="F")
                I.createUniqueChild(sol, name + suffix, "DataArray_t")
                I.getNodeFromName1(sol, name + suffix)[1] = view
            o_ = I.createUniqueChild(z, ".Solver#ownData", "UserDefinedData_t")
            I.createUniqueChild(o_, "compact" + suffix, "DataArray_t")
            I.getNodeFromName1(o_, "compact" + suffix)[1] = buf
        if rmConsVars:
            sol[2] = [c for c in sol[2] if c[0] not in CONS[1:]]
    return first_iter


def _huge_page_bytes():
    try:
        with open("/sys/kernel/mm/transparent_hugepage/hpage_pmd_size") as f:
            return int(f.read())
    except (OSError, ValueError):
        return 0


def _level_buffers(count, rows, n):
    """`count` (rows, n) float64 arrays for time levels.  The solver copies
    the levels to and from the GPU every step; on Linux, levels of at least
    one transparent huge page live in one anonymous mapping advised for huge
    pages (madvise MADV_HUGEPAGE before the first touch, MADV_COLLAPSE after
    it for what fell back to base pages), so that the copy engines translate
    a few huge pages instead of one page-table entry per base page (repeated
    copies of three 0.7 GB levels in 64 KB pages missed in the translation
    caches and ran 20 times slower).  Elsewhere, or if the mapping cannot be
    made, plain numpy arrays."""
    nbytes = rows * n * 8
    hp = _huge_page_bytes()
    if hp <= 0 or nbytes < hp:
        return [np.empty((rows, n), dtype=np.float64) for _ in range(count)]
    try:
        import ctypes
        import mmap
        size = -(-count * nbytes // hp) * hp
        m = mmap.mmap(-1, size + hp, flags=mmap.MAP_PRIVATE | mmap.MAP_ANONYMOUS)
        base = ctypes.addressof(ctypes.c_char.from_buffer(m))
        start = -(-base // hp) * hp
        libc = ctypes.CDLL(None, use_errno=True)
        libc.madvise.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
        libc.madvise(ctypes.c_void_p(start), ctypes.c_size_t(size), 14)   # MADV_HUGEPAGE
        whole = np.frombuffer(m, dtype=np.float64, count=size // 8, offset=start - base)
        whole.fill(0.)   # first touch: huge pages where the kernel has them
        libc.madvise(ctypes.c_void_p(start), ctypes.c_size_t(size), 25)   # MADV_COLLAPSE (6.1+)
        return [whole[q * rows * n:(q + 1) * rows * n].reshape(rows, n) for q in range(count)]
    except (OSError, ValueError, AttributeError, TypeError):
        return [np.empty((rows, n), dtype=np.float64) for _ in range(count)]


def compactArray(z, level):
    """The contiguous (NEQ, NDIMDX) array of time level ''/_M1/_P1."""
    o = I.getNodeFromName1(z, ".Solver#ownData")
    return I.getNodeFromName1(o, "compact" + level)[1]


def switchPointers__(zones, case=3):
    """FastC/FastC/PyTree.py:2298: after a physical step the time levels
    rotate M1 <- N <- P1 (the arrays, not the values)."""
    for z in zones:
        sol = I.getNodeFromName1(z, I.__FlowSolutionCenters__)
        o = I.getNodeFromName1(z, ".Solver#ownData")
        cn, cm, cp = (I.getNodeFromName1(o, "compact" + s) for s in ("", "_M1", "_P1"))
        cn[1], cm[1], cp[1] = cp[1], cn[1], cm[1]
        for name in _prim_names(z):
            a, b, c = (I.getNodeFromName1(sol, name + s) for s in ("", "_M1", "_P1"))
            a[1], b[1], c[1] = c[1], a[1], b[1]


# ------------------------------------------------------------ restart I/O
# FastC/FastC/PyTree.py:3514-3560 (load / save) write CGNS/HDF5 files
# through Cassiopee's Converter, which is not available here (neither is
# h5py).  The same trees are written instead to a numpy .npz container that
# keeps the CGNS/Python structure node for node: "tree" holds a JSON list of
# [parent, name, type, value] entries in depth-first order (parent = index
# of the parent entry, -1 for the root; value = null, a string, or the key
# of a numpy array stored beside it in the archive, with its dtype, shape and
# Fortran order preserved).
def _tree_to_npz(t, path):
    import json
    entries, arrays = [], {}

    def walk(node, parent):
        idx = len(entries)
        v = node[1]
        if v is None:
            val = None
        elif isinstance(v, np.ndarray) and v.dtype == np.dtype("c"):
            val = {"str": b"".join(v.ravel(order="F").tolist()).decode()}
        elif isinstance(v, str):
            val = {"str": v}
        else:
            key = "a%d" % len(arrays)
            a = np.asarray(v)
            arrays[key] = a
            val = {"key": key, "fortran": bool(a.flags.f_contiguous and not a.flags.c_contiguous)}
        entries.append([parent, node[0], node[3], val])
        for c in node[2]:
            walk(c, idx)

    walk(t, -1)
    np.savez_compressed(path, tree=np.array(json.dumps(entries)), **arrays)


def _tree_from_npz(path):
    import json
    with np.load(path, allow_pickle=False) as f:
        entries = json.loads(str(f["tree"]))
        nodes = []
        for parent, name, ntype, val in entries:
            if val is None:
                v = None
            elif "str" in val:
                v = np.array([c for c in val["str"]], dtype="c")
            else:
                v = np.array(f[val["key"]])
                if val.get("fortran"):
                    v = np.asfortranarray(v)
            node = [name, v, [], ntype]
            if parent >= 0:
                nodes[parent][2].append(node)
            nodes.append(node)
    return nodes[0]


def saveTree(t, fileName="restart.npz", split="single", compress=0):
    """FastC/FastC/PyTree.py:3755: the tree without what a restart does not
    need -- the _P1 time level, the solver's own data (Parameter_int /
    Parameter_real, compacted levels), motion nodes -- written as one file
    (split = 'single'; the 'multiple' per-process layout belongs to MPI runs,
    which this solver does not have)."""
    import copy
    if split != "single":
        raise ValueError("saveTree: only split='single' is supported (one process)")
    t2 = copy.deepcopy(t)
    p1 = {n + "_P1" for n in PRIM_SA}

    def strip(node):
        node[2] = [c for c in node[2]
                   if c[0] not in (".Solver#ownData", "Displacement#0", "Motion")
                   and not (node[0] == I.__FlowSolutionCenters__ and c[0] in p1)]
        for c in node[2]:
            strip(c)

    strip(t2)
    _tree_to_npz(t2, fileName)


def loadTree(fileName="restart.npz", split="single", graph=False, exploc=0):
    """FastC/FastC/PyTree.py loadTree: the tree of a file written by
    saveTree (graph=True also returns the communication graph, None here)."""
    if split != "single":
        raise ValueError("loadTree: only split='single' is supported (one process)")
    t = _tree_from_npz(fileName)
    return (t, None) if graph else t


def save(t, fileName="restart.npz", tc=None, fileNameC="tc_restart.npz", ts=None,
         fileNameS="tstat_restart.npz", split="single", compress=0):
    """FastC/FastC/PyTree.py:3542: save t (and tc, ts when given)."""
    saveTree(t, fileName=fileName, split=split, compress=compress)
    if tc is not None:
        saveTree(tc, fileName=fileNameC, split=split, compress=compress)
    if ts is not None:
        saveTree(ts, fileName=fileNameS, split=split, compress=compress)


def load(fileName="t.npz", fileNameC=None, fileNameS=None, split="single", exploc=0):
    """FastC/FastC/PyTree.py:3514: (t, tc, ts, graph) from the files written
    by save."""
    t = loadTree(fileName=fileName, split=split, graph=False, exploc=exploc)
    if fileNameC is not None:
        tc, graph = loadTree(fileName=fileNameC, split=split, graph=True, exploc=exploc)
    else:
        tc, graph = None, None
    ts = loadTree(fileName=fileNameS, split=split) if fileNameS is not None else None
    return t, tc, ts, graph
