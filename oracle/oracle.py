"""ctypes binding of the CPU oracle (fast_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg.  The product package never imports it.
Parity status: unpinned by reference data (see fast_oracle.h).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "fast_oracle.c"
LIB = HERE / "_build" / "liboracle.so"
_lib = None


def build(force: bool = False) -> Path:
    """gcc -O2 -ffp-contract=off -fopenmp (no contraction: every multiply and
    add rounds separately, as in the reference's arithmetic)."""
    LIB.parent.mkdir(exist_ok=True)
    deps = [SRC, HERE / "fast_oracle.h"]
    if LIB.exists() and not force and all(d.stat().st_mtime <= LIB.stat().st_mtime for d in deps):
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
           "-o", str(tmp), str(SRC), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


class OrZone(C.Structure):
    _fields_ = [("param_int", C.POINTER(C.c_int64)), ("param_real", C.POINTER(C.c_double)),
                ("ro", C.POINTER(C.c_double)), ("ro_m1", C.POINTER(C.c_double)),
                ("ro_p1", C.POINTER(C.c_double)), ("xmut", C.POINTER(C.c_double)),
                ("drodm", C.POINTER(C.c_double)), ("coe", C.POINTER(C.c_double)),
                ("ti", C.POINTER(C.c_double)), ("tj", C.POINTER(C.c_double)),
                ("tk", C.POINTER(C.c_double)), ("vol", C.POINTER(C.c_double)),
                ("rdm", C.POINTER(C.c_double)), ("wig", C.POINTER(C.c_double)),
                ("cfl", C.POINTER(C.c_double))]


class OrTransfer(C.Structure):
    _fields_ = [("dnr_zone", C.c_int64), ("rcv_zone", C.c_int64), ("n", C.c_int64),
                ("dnr_idx", C.POINTER(C.c_int64)), ("rcv_idx", C.POINTER(C.c_int64)),
                ("types", C.POINTER(C.c_int64)), ("coefs", C.POINTER(C.c_double))]


def load():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(str(LIB))
        _lib.or_compute.restype = C.c_int
        _lib.or_cfl_dt.restype = C.c_double
    return _lib


def set_threads(n: int):
    load().or_set_threads(int(n))


def _d(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _i(a):
    assert a.dtype == np.int64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_int64))


class Case:
    """Host copies of every zone's arrays, advanced by the oracle."""

    def __init__(self, zones, transfers=()):
        """zones: list of dicts with pi, pr, ti, tj, tk, vol, ro, ro_m1, ro_p1
        (flat float64 arrays; state arrays are copied)."""
        self.z = []
        for zd in zones:
            pi = np.ascontiguousarray(zd["pi"], dtype=np.int64)
            nd, neq = int(pi[41]), int(pi[36])
            nss = int(pi[58])
            nlu = 1
            for d in range(3):
                nlu *= max(1, int(pi[20 + d]) // int(pi[30 + d]))
            e = dict(pi=pi, pr=np.ascontiguousarray(zd["pr"], dtype=np.float64),
                     ti=np.ascontiguousarray(zd["ti"], dtype=np.float64),
                     tj=np.ascontiguousarray(zd["tj"], dtype=np.float64),
                     tk=np.ascontiguousarray(zd["tk"], dtype=np.float64),
                     vol=np.ascontiguousarray(zd["vol"], dtype=np.float64),
                     lv=[np.array(zd[k], dtype=np.float64).reshape(-1) for k in ("ro", "ro_m1", "ro_p1")],
                     xmut=np.zeros(2 * nd), drodm=np.zeros(neq * nd), coe=np.zeros(neq * nd),
                     rdm=np.zeros(nss * neq * 2 * nlu), wig=np.zeros(6 * nd), cfl=np.zeros(3))
            if neq == 6:
                # Spalart-Allmaras: the wall distance follows the viscosity
                # (navier_stokes_struct passes xmut(1+NDIMDX) as dist)
                e["xmut"][nd:] = np.asarray(zd["dist"], dtype=np.float64).reshape(-1)
            self.z.append(e)
        self.tr = []
        for t in transfers:
            e = dict(dnr=int(t["dnr"]), rcv=int(t["rcv"]),
                     dnr_idx=np.ascontiguousarray(t["dnr_idx"], dtype=np.int64),
                     rcv_idx=np.ascontiguousarray(t["rcv_idx"], dtype=np.int64))
            if "types" in t:
                e["types"] = np.ascontiguousarray(t["types"], dtype=np.int64)
                e["coefs"] = np.ascontiguousarray(t["coefs"], dtype=np.float64)
            self.tr.append(e)
        self.first_it = 0

    def _structs(self):
        arr = (OrZone * len(self.z))()
        for s, e in zip(arr, self.z):
            s.param_int = _i(e["pi"]); s.param_real = _d(e["pr"])
            s.ro, s.ro_m1, s.ro_p1 = (_d(a) for a in e["lv"])
            s.xmut = _d(e["xmut"]); s.drodm = _d(e["drodm"]); s.coe = _d(e["coe"])
            s.ti = _d(e["ti"]); s.tj = _d(e["tj"]); s.tk = _d(e["tk"]); s.vol = _d(e["vol"])
            s.rdm = _d(e["rdm"]); s.wig = _d(e["wig"]); s.cfl = _d(e["cfl"])
        tr = (OrTransfer * max(1, len(self.tr)))()
        for s, t in zip(tr, self.tr):
            s.dnr_zone, s.rcv_zone, s.n = t["dnr"], t["rcv"], t["dnr_idx"].size
            s.dnr_idx = _i(t["dnr_idx"]); s.rcv_idx = _i(t["rcv_idx"])
            if "types" in t:
                s.types = _i(t["types"]); s.coefs = _d(t["coefs"])
        return arr, tr

    def apply_bc(self, level: int = 0):
        lib = load()
        arr, tr = self._structs()
        if self.tr:
            # transfers act on ro (use_p1=0) or ro_p1 (use_p1=1); for level
            # M1 the ro slot is pointed at ro_m1 for the call
            if level == 1:
                for s in arr:
                    s.ro = s.ro_m1
            lib.or_transfers(arr, tr, len(self.tr), 1 if level == 2 else 0)
        for e in self.z:
            lib.or_bc_zone(_i(e["pi"]), _d(e["pr"]), _d(e["ti"]), _d(e["tj"]), _d(e["tk"]), 0,
                           _d(e["lv"][level]))

    def compute(self, nitrun, nstep_deb, nstep_fin, nit_c=1, modulo_verif=200):
        lib = load()
        arr, tr = self._structs()
        fi = C.c_int(self.first_it)
        rc = lib.or_compute(arr, len(self.z), tr, len(self.tr), int(nitrun), int(nstep_deb),
                            int(nstep_fin), int(nit_c), int(modulo_verif), C.byref(fi))
        if rc != 0:
            raise RuntimeError(f"or_compute failed ({rc})")
        self.first_it = fi.value
        # follow the pointer rotation done by the driver
        for s, e in zip(arr, self.z):
            by_addr = {a.ctypes.data: a for a in e["lv"]}
            e["lv"] = [by_addr[C.cast(p, C.c_void_p).value] for p in (s.ro, s.ro_m1, s.ro_p1)]

    def cfl(self, zone: int):
        """(max, min, mean) CFL of the last verified iteration (cpcfl3.for)."""
        return self.z[zone]["cfl"].copy()

    def residual_norms(self, zone: int, nit: int):
        e = self.z[zone]
        neq, nss = int(e["pi"][36]), int(e["pi"][58])
        out = np.zeros(2 * neq * nit)
        load().or_residual_norms(_i(e["pi"]), _d(e["pr"]), _d(e["rdm"]), nss, nit, _d(out))
        return out.reshape(2 * neq, nit)


def cfl_dt(zd, cfl):
    """Largest dt for the given CFL (cpcfl3.for)."""
    lib = load()
    pi = np.ascontiguousarray(zd["pi"], dtype=np.int64)
    pr = np.ascontiguousarray(zd["pr"], dtype=np.float64)
    ro = np.ascontiguousarray(zd["ro"], dtype=np.float64).reshape(-1)
    xmut = np.zeros(int(pi[41]))
    ar = [np.ascontiguousarray(zd[k], dtype=np.float64) for k in ("ti", "tj", "tk", "vol")]
    return lib.or_cfl_dt(_i(pi), _d(pr), _d(ro), _d(xmut), *(_d(a) for a in ar), C.c_double(cfl))


def metric(pi, x, y, z):
    """cp_tijk.for + cp_vol.for restated in C: (ti, tj, tk, vol) for vertex
    coordinates of shape (nvi, nvj, nvk) (ghosts included)."""
    lib = load()
    pi = np.ascontiguousarray(pi, dtype=np.int64)
    ndm, nij, nk_ = int(pi[43]), int(pi[37]), int(pi[38])
    ti, tj = np.zeros(ndm * nij), np.zeros(ndm * nij)
    tk, vol = np.zeros(ndm * nk_), np.zeros(ndm)
    xs = [np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1, order="F")) for a in (x, y, z)]
    lib.or_metric(_i(pi), *(_d(a) for a in xs), _d(ti), _d(tj), _d(tk), _d(vol))
    return ti, tj, tk, vol
