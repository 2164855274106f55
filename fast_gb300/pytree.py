"""Minimal CGNS/Python tree helpers (the subset of Cassiopee Converter.Internal
that FastS's Python layer uses).

A node is the CGNS/Python list ``[name, value, children, type]``; field arrays
are Fortran-ordered numpy arrays (i fastest), exactly as in the reference's
pyTrees, so the compacted time-level arrays map one-to-one to the device
layout.
"""
from __future__ import annotations

import numpy as np

__FlowSolutionCenters__ = "FlowSolution#Centers"


def createNode(name, ntype, value=None, children=None, parent=None):
    if isinstance(value, str):
        value = np.array([c for c in value], dtype="c")
    elif isinstance(value, (int, np.integer)):
        value = np.array([value], dtype=np.int64)
    elif isinstance(value, (float, np.floating)):
        value = np.array([value], dtype=np.float64)
    elif isinstance(value, (list, tuple)):
        arr = np.asarray(value)
        value = arr.astype(np.float64) if arr.dtype.kind == "f" else arr.astype(np.int64)
    node = [name, value, children if children is not None else [], ntype]
    if parent is not None:
        parent[2].append(node)
    return node


def createChild(parent, name, ntype, value=None, children=None):
    return createNode(name, ntype, value, children, parent)


def createUniqueChild(parent, name, ntype, value=None, children=None):
    node = getNodeFromName1(parent, name)
    if node is None:
        return createChild(parent, name, ntype, value, children)
    tmp = createNode(name, ntype, value)
    node[1] = tmp[1]
    node[3] = ntype
    if children is not None:
        node[2] = children
    return node


def getValue(node):
    v = node[1]
    if isinstance(v, np.ndarray):
        if v.dtype.kind in ("S", "a", "U") or v.dtype == np.dtype("c"):
            return b"".join(v.ravel(order="F").tolist()).decode() if v.dtype == np.dtype("c") else str(v)
        if v.size == 1:
            return v.ravel()[0].item()
    return v


def setValue(node, value):
    node[1] = createNode("_", "_", value)[1]


def getNodeFromName1(node, name):
    if node is None:
        return None
    for c in node[2]:
        if c[0] == name:
            return c
    return None


def getNodeFromName2(node, name):
    if node is None:
        return None
    for c in node[2]:
        if c[0] == name:
            return c
        for cc in c[2]:
            if cc[0] == name:
                return cc
    return None


def getNodeFromName(node, name):
    if node is None:
        return None
    if node[0] == name:
        return node
    for c in node[2]:
        r = getNodeFromName(c, name)
        if r is not None:
            return r
    return None


def getNodesFromType1(node, ntype):
    return [c for c in node[2] if c[3] == ntype]


def getNodesFromType2(node, ntype):
    out = []
    for c in node[2]:
        if c[3] == ntype:
            out.append(c)
        out.extend(cc for cc in c[2] if cc[3] == ntype)
    return out


def getNodesFromType3(node, ntype):
    """Nodes of type ntype among the children, grandchildren and
    great-grandchildren of node, depth first."""
    out = []
    for c in node[2]:
        if c[3] == ntype:
            out.append(c)
        for cc in c[2]:
            if cc[3] == ntype:
                out.append(cc)
            out.extend(ccc for ccc in cc[2] if ccc[3] == ntype)
    return out


def getNodesFromType(node, ntype):
    out = [node] if node[3] == ntype else []
    for c in node[2]:
        out.extend(getNodesFromType(c, ntype))
    return out


def getNodeFromType1(node, ntype):
    for c in node[2]:
        if c[3] == ntype:
            return c
    return None


def getBases(t):
    return getNodesFromType1(t, "CGNSBase_t")


def getZones(t):
    if t[3] == "Zone_t":
        return [t]
    if t[3] == "CGNSBase_t":
        return getNodesFromType1(t, "Zone_t")
    out = []
    for b in getBases(t):
        out.extend(getNodesFromType1(b, "Zone_t"))
    return out


def getZoneDim(z):
    d = z[1]
    return ["Structured", int(d[0, 0]), int(d[1, 0]), int(d[2, 0]), 3 if int(d[2, 0]) > 2 else 2]


def newCGNSTree():
    t = createNode("CGNSTree", "CGNSTree_t")
    createChild(t, "CGNSLibraryVersion", "CGNSLibraryVersion_t", 3.1)
    return t


def newCGNSBase(name, cellDim=3, physDim=3, parent=None):
    b = createNode(name, "CGNSBase_t", np.array([cellDim, physDim], dtype=np.int64))
    if parent is not None:
        parent[2].append(b)
    return b


def newZone(name, nvertex, parent=None):
    """Structured zone with vertex dimensions nvertex = (ni, nj, nk)."""
    ni, nj, nk = nvertex
    dims = np.array([[ni, ni - 1, 0], [nj, nj - 1, 0], [nk, nk - 1, 0]], dtype=np.int64, order="F")
    z = createNode(name, "Zone_t", dims)
    createChild(z, "ZoneType", "ZoneType_t", "Structured")
    if parent is not None:
        parent[2].append(z)
    return z


def getNodeFromPath(t, path):
    node = t
    for name in [p for p in path.split("/") if p]:
        node = getNodeFromName1(node, name)
        if node is None:
            return None
    return node
