"""Interface connectivity as FastS receives it: the Connector ``tc`` tree.

FastS.PyTree.warmup / _compute take ``tc``, the donor tree of Cassiopee's
Connector (FastS/FastS/PyTree.py:42-55, 341), and FastC's transfers read it
every call (FastC/FastC/Com/setInterpTransfersFast.cpp:88, 440-960).  Each
donor zone of ``tc`` carries one ``ZoneSubRegion_t`` per receiver zone
(named ``ID_<receiver>``, valued with the receiver zone's name) holding

* ``PointList``: donor cell of each receiver point (linear index, ghosts
  included, 0-based, into the donor zone's arrays; for an interpolation, the
  first cell of the donor molecule),
* ``PointListDonor``: the receiver cell of each point (same indexing, into
  the receiver zone),
* ``InterpolantsType``: the interpolation of each point, and
* ``InterpolantsDonor``: the coefficients, concatenated point after point,

as FastS's own tests build them by hand (FastS/test/tgvMpi.py:136-195).
Cassiopee is not available, so this module reads and writes those nodes
directly.  Types 0 and 1 (one donor, coefficient 1) are the 1-to-1 copy;
types 2 (8-point trilinear, coefficients i fastest), 22 (4-point bilinear in
(i, j)), 3 (27-point tensor-product Lagrange, 3 + 3 + 3 coefficients) and 5
(125-point Lagrange, 5 + 5 + 5) are the overset interpolations.
"""
from __future__ import annotations

import numpy as np

from . import pytree as I

# coefficients stored per point, and donor molecule width per direction
NCOEF = {0: 1, 1: 1, 2: 8, 22: 4, 3: 9, 5: 15}
WIDTH = {0: 1, 1: 1, 2: 2, 22: 2, 3: 3, 5: 5}


def is_tree(tc) -> bool:
    """True for a CGNS/Python tree (as opposed to a list of transfer dicts)."""
    return (isinstance(tc, list) and len(tc) == 4 and isinstance(tc[0], str)
            and tc[3] == "CGNSTree_t")


def transfers_from_tc(t, tc):
    """The transfers of a ``tc`` tree as dicts: dnr, rcv (zone positions in
    t), dnr_idx, rcv_idx (int64), and for interpolations types (int64 per
    point) and coefs (float64, concatenated).  Zones are matched by name."""
    names = [z[0] for z in I.getZones(t)]
    pos = {n: k for k, n in enumerate(names)}
    out = []
    for zd in I.getZones(tc):
        if zd[0] not in pos:
            raise ValueError(f"tc: donor zone {zd[0]} is not a zone of t")
        for sr in I.getNodesFromType1(zd, "ZoneSubRegion_t"):
            rname = I.getValue(sr)
            if isinstance(rname, np.ndarray):
                rname = rname.tobytes().decode().strip("\x00 ")
            pl = I.getNodeFromName1(sr, "PointList")
            pld = I.getNodeFromName1(sr, "PointListDonor")
            if pl is None or pld is None:
                continue
            if rname not in pos:
                raise ValueError(f"tc: receiver zone {rname} is not a zone of t")
            dnr = np.asarray(pl[1], dtype=np.int64).ravel()
            rcv = np.asarray(pld[1], dtype=np.int64).ravel()
            if dnr.size != rcv.size:
                raise ValueError(f"tc: {sr[0]} of {zd[0]}: PointList and PointListDonor sizes differ")
            ty = I.getNodeFromName1(sr, "InterpolantsType")
            co = I.getNodeFromName1(sr, "InterpolantsDonor")
            types = (np.asarray(ty[1], dtype=np.int64).ravel() if ty is not None
                     else np.zeros(dnr.size, dtype=np.int64))
            coefs = (np.asarray(co[1], dtype=np.float64).ravel() if co is not None
                     else np.ones(dnr.size, dtype=np.float64))
            if types.size != dnr.size:
                raise ValueError(f"tc: {sr[0]} of {zd[0]}: one InterpolantsType per point expected")
            bad = set(np.unique(types).tolist()) - set(NCOEF)
            if bad:
                raise ValueError(f"tc: interpolation types {sorted(bad)} are not supported")
            need = int(sum(NCOEF[int(x)] for x in types))
            if coefs.size != need:
                raise ValueError(f"tc: {sr[0]} of {zd[0]}: {coefs.size} coefficients, {need} expected")
            tr = dict(dnr=pos[zd[0]], rcv=pos[rname], dnr_idx=dnr, rcv_idx=rcv)
            if np.all(types <= 1) and np.all(coefs == 1.0):
                out.append(tr)                      # the 1-to-1 copy
            else:
                tr.update(types=types, coefs=coefs)
                out.append(tr)
    return out


def tc_tree(t, transfers):
    """A ``tc`` tree holding the given transfers (dicts as returned by
    transfers_from_tc): one donor zone per zone of t, one ID_ subregion per
    (donor, receiver) pair, in the order of the list."""
    zones = I.getZones(t)
    tc = I.newCGNSTree()
    base = I.newCGNSBase("Base", 3, 3, tc)
    zc = {}
    for z in zones:
        n = I.createChild(base, z[0], "Zone_t", np.copy(z[1]))
        zc[z[0]] = n
    for tr in transfers:
        zd, zr = zones[tr["dnr"]], zones[tr["rcv"]]
        sr = I.createChild(zc[zd[0]], "ID_" + zr[0], "ZoneSubRegion_t", zr[0])
        I.createChild(sr, "ZoneRole", "DataArray_t", "Donor")
        I.createChild(sr, "GridLocation", "GridLocation_t", "CellCenter")
        n = np.asarray(tr["dnr_idx"]).size
        types = np.asarray(tr.get("types", np.ones(n, dtype=np.int64)), dtype=np.int64)
        coefs = np.asarray(tr.get("coefs", np.ones(n)), dtype=np.float64)
        I.createChild(sr, "InterpolantsDonor", "DataArray_t", coefs)
        I.createChild(sr, "InterpolantsType", "DataArray_t", types)
        I.createChild(sr, "PointListDonor", "DataArray_t", np.asarray(tr["rcv_idx"], dtype=np.int64))
        I.createChild(sr, "PointList", "DataArray_t", np.asarray(tr["dnr_idx"], dtype=np.int64))
    return tc
