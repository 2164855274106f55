"""ctypes binding of libfastgb300.so (the C ABI declared in include/fast_gb300.h).

The library is the only compute path: importing this module loads it and
raises if it is missing or cannot be loaded; nothing falls back to the CPU.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

_LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libfastgb300.so"
_lib = None

FGB_OK, FGB_ERR_ARG, FGB_ERR_CUDA, FGB_ERR_DEVICE, FGB_ERR_STATE = 0, 1, 2, 3, 4

# every exported symbol with its argument types (include/fast_gb300.h)
_P = C.c_void_p
_I64P = C.POINTER(C.c_int64)
_DP = C.POINTER(C.c_double)
SIGNATURES = {
    "fgb_last_error": ([], C.c_char_p),
    "fgb_version": ([C.POINTER(C.c_int)] * 3, C.c_int),
    "fgb_create": ([C.c_int, C.POINTER(_P)], C.c_int),
    "fgb_destroy": ([_P], C.c_int),
    "fgb_add_zone": ([_P, _I64P, C.c_int64, _DP, C.c_int64, _DP, _DP, _DP, _DP,
                      C.POINTER(C.c_int)], C.c_int),
    "fgb_add_transfer": ([_P, C.c_int, C.c_int, C.c_int64, _I64P, _I64P], C.c_int),
    "fgb_add_interp_transfer": ([_P, C.c_int, C.c_int, C.c_int64, _I64P, _I64P, _I64P, _DP,
                                 C.c_int64], C.c_int),
    "fgb_set_wall_distance": ([_P, C.c_int, _DP], C.c_int),
    "fgb_set_option": ([_P, C.c_char_p, C.c_double], C.c_int),
    "fgb_get_option": ([_P, C.c_char_p, _DP], C.c_int),
    "fgb_upload_state": ([_P, C.c_int, C.c_int, _DP], C.c_int),
    "fgb_upload_state_async": ([_P, C.c_int, C.c_int, _DP], C.c_int),
    "fgb_download_state": ([_P, C.c_int, C.c_int, _DP], C.c_int),
    "fgb_download_work": ([_P, C.c_int, C.c_char_p, _DP, C.c_int64], C.c_int),
    "fgb_compute": ([_P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int], C.c_int),
    "fgb_apply_bc": ([_P, C.c_int], C.c_int),
    "fgb_residuals": ([_P, C.c_int, _DP, C.c_int64, C.POINTER(C.c_int)], C.c_int),
    "fgb_residual_norms_noalloc": ([_P, C.c_int, _P], C.c_int),
    "fgb_set_bc_state": ([_P, C.c_int, _DP], C.c_int),
    "fgb_cfl": ([_P, C.c_int, _DP], C.c_int),
    "fgb_pin_host": ([_P, C.c_void_p, C.c_int64], C.c_int),
    "fgb_adjoint_forward": ([_P, C.c_int, C.c_int, C.c_int], C.c_int),
    "fgb_adjoint_backward": ([_P, C.c_int, _DP, _DP, _DP, _DP, _DP, _DP], C.c_int),
    "fgb_tangent": ([_P, C.c_int, C.c_int, _DP, _DP, _DP, _DP, _DP, _DP], C.c_int),
    "fgb_synchronize": ([_P], C.c_int),
    "fgb_kernel_stats": ([_P, C.c_int, C.c_char_p, C.c_int, _I64P, _DP], C.c_int),
    "fgb_launch_count": ([_P, _I64P], C.c_int),
    "fgb_stream_timer": ([_P, C.c_int, _DP], C.c_int),
    "fgb_fp64_peak": ([C.c_int, _DP], C.c_int),
}


class FastGB300Error(RuntimeError):
    pass


def lib_path() -> Path:
    return _LIB_PATH


def load():
    """Load the shared library (once) and declare every signature."""
    global _lib
    if _lib is not None:
        return _lib
    if not _LIB_PATH.exists():
        raise FastGB300Error(
            f"{_LIB_PATH} is missing: build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` (needs nvcc)")
    lib = C.CDLL(str(_LIB_PATH))
    for name, (args, res) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def _check(rc: int):
    if rc != FGB_OK:
        msg = load().fgb_last_error().decode(errors="replace")
        raise FastGB300Error(f"fast_gb300 error {rc}: {msg}")


def _dp(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_DP)


def _ip(a: np.ndarray):
    assert a.dtype == np.int64 and a.flags.c_contiguous
    return a.ctypes.data_as(_I64P)


class Solver:
    """Owner of one fgb_solver handle (one CUDA stream, all zones on one GPU)."""

    def __init__(self, device: int = 0):
        self._lib = load()
        h = _P()
        _check(self._lib.fgb_create(int(device), C.byref(h)))
        self._h = h
        self.zones = []  # (param_int, param_real) per zone
        self._pinned = []  # host arrays page-locked for this solver (kept alive)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.fgb_destroy(self._h)
            self._h = None
        self._pinned = []

    def pin(self, arr: np.ndarray):
        """Page-lock the host array (fgb_pin_host) for the state copies;
        the solver keeps it alive until close()."""
        assert arr.flags.c_contiguous
        _check(self._lib.fgb_pin_host(self._h, C.c_void_p(arr.ctypes.data), arr.nbytes))
        self._pinned.append(arr)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_zone(self, param_int, param_real, ti, tj, tk, vol) -> int:
        pi = np.ascontiguousarray(param_int, dtype=np.int64)
        pr = np.ascontiguousarray(param_real, dtype=np.float64)
        ti, tj, tk, vol = (np.ascontiguousarray(x, dtype=np.float64) for x in (ti, tj, tk, vol))
        zid = C.c_int(-1)
        _check(self._lib.fgb_add_zone(self._h, _ip(pi), pi.size, _dp(pr), pr.size, _dp(ti),
                                      _dp(tj), _dp(tk), _dp(vol), C.byref(zid)))
        self.zones.append((pi, pr))
        return zid.value

    def add_transfer(self, dnr, rcv, dnr_idx, rcv_idx):
        d = np.ascontiguousarray(dnr_idx, dtype=np.int64)
        r = np.ascontiguousarray(rcv_idx, dtype=np.int64)
        _check(self._lib.fgb_add_transfer(self._h, int(dnr), int(rcv), d.size, _ip(d), _ip(r)))

    def add_interp_transfer(self, dnr, rcv, dnr_idx, rcv_idx, types, coefs):
        """Overset interpolation (types 0/1, 2, 22, 3, 5; coefficients of
        every point concatenated)."""
        d = np.ascontiguousarray(dnr_idx, dtype=np.int64)
        r = np.ascontiguousarray(rcv_idx, dtype=np.int64)
        ty = np.ascontiguousarray(types, dtype=np.int64)
        c = np.ascontiguousarray(coefs, dtype=np.float64)
        _check(self._lib.fgb_add_interp_transfer(self._h, int(dnr), int(rcv), d.size, _ip(d), _ip(r),
                                                 _ip(ty), _dp(c), c.size))

    def add_any_transfer(self, tr):
        """A transfer dict (dnr, rcv, dnr_idx, rcv_idx[, types, coefs])."""
        if "types" in tr:
            self.add_interp_transfer(tr["dnr"], tr["rcv"], tr["dnr_idx"], tr["rcv_idx"], tr["types"],
                                     tr["coefs"])
        else:
            self.add_transfer(tr["dnr"], tr["rcv"], tr["dnr_idx"], tr["rcv_idx"])

    def set_wall_distance(self, zone: int, dist):
        """TurbulentDistance of a Spalart-Allmaras zone (NDIMDX values)."""
        d = np.ascontiguousarray(dist, dtype=np.float64).reshape(-1)
        _check(self._lib.fgb_set_wall_distance(self._h, int(zone), _dp(d)))

    def set_option(self, key: str, value: float):
        _check(self._lib.fgb_set_option(self._h, key.encode(), float(value)))

    def get_option(self, key: str) -> float:
        v = C.c_double()
        _check(self._lib.fgb_get_option(self._h, key.encode(), C.byref(v)))
        return v.value

    def upload(self, zone: int, level: int, arr: np.ndarray):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        _check(self._lib.fgb_upload_state(self._h, zone, level, _dp(a)))

    def upload_async(self, zone: int, level: int, arr: np.ndarray):
        """fgb_upload_state_async: asynchronous when ``arr`` lies in memory
        this solver page-locked (pin), which keeps it alive; the array must
        not change until the next synchronizing call."""
        if arr.dtype != np.float64 or not arr.flags.c_contiguous:
            return self.upload(zone, level, arr)
        _check(self._lib.fgb_upload_state_async(self._h, zone, level, _dp(arr)))

    def download(self, zone: int, level: int, out: np.ndarray | None = None) -> np.ndarray:
        pi = self.zones[zone][0]
        n = int(pi[36] * pi[41])
        if out is None:
            out = np.empty(n, dtype=np.float64)
        assert out.size >= n and out.flags.c_contiguous
        _check(self._lib.fgb_download_state(self._h, zone, level, _dp(out)))
        return out

    def work(self, zone: int, which: str, n: int) -> np.ndarray:
        out = np.empty(n, dtype=np.float64)
        _check(self._lib.fgb_download_work(self._h, zone, which.encode(), _dp(out), n))
        return out

    def compute(self, nitrun, nstep_deb, nstep_fin, layer_mode=1, nit_c=1):
        _check(self._lib.fgb_compute(self._h, int(nitrun), int(nstep_deb), int(nstep_fin),
                                     int(layer_mode), int(nit_c)))

    def apply_bc(self, level: int):
        _check(self._lib.fgb_apply_bc(self._h, int(level)))

    def residuals(self, zone: int):
        pi = self.zones[zone][0]
        neq, nssiter = int(pi[36]), int(pi[58])
        out = np.zeros(2 * neq * nssiter, dtype=np.float64)
        nit = C.c_int(0)
        _check(self._lib.fgb_residuals(self._h, zone, _dp(out), out.size, C.byref(nit)))
        k = nit.value
        return out[:2 * neq * k].reshape(2 * neq, k) if k else np.zeros((2 * neq, 0))

    def residual_norms_noalloc(self, zone: int, out_ptr: int):
        """Enqueue fgb_residual_norms_noalloc: 2*neq doubles (L2 then Loo)
        written to the device address out_ptr; fgb_synchronize waits."""
        _check(self._lib.fgb_residual_norms_noalloc(self._h, int(zone), C.c_void_p(int(out_ptr))))

    def cfl(self, zone: int) -> np.ndarray:
        """(max, min, mean) CFL of the last verified iteration (cpcfl3.for)."""
        out = np.zeros(3)
        _check(self._lib.fgb_cfl(self._h, int(zone), _dp(out)))
        return out

    def set_bc_state(self, zone: int, st):
        a = np.ascontiguousarray(st, dtype=np.float64)
        _check(self._lib.fgb_set_bc_state(self._h, int(zone), _dp(a)))

    def adjoint_forward(self, zone: int, nsteps: int, ckpt: int):
        _check(self._lib.fgb_adjoint_forward(self._h, int(zone), int(nsteps), int(ckpt)))

    def adjoint_backward(self, zone: int, lam_final):
        """(dJ/dW0, dJ/dti, dJ/dtj, dJ/dvol, dJ/dst) of the last forward run."""
        pi = self.zones[zone][0]
        nq, nm = int(pi[36] * pi[41]), int(pi[43])
        lf = np.ascontiguousarray(lam_final, dtype=np.float64)
        out = [np.zeros(nq), np.zeros(2 * nm), np.zeros(2 * nm), np.zeros(nm), np.zeros(5)]
        _check(self._lib.fgb_adjoint_backward(self._h, int(zone), _dp(lf), *(_dp(o) for o in out)))
        return out

    def tangent(self, zone: int, nsteps: int, dw0, dti, dtj, dvol, dst):
        pi = self.zones[zone][0]
        out = np.zeros(int(pi[36] * pi[41]))
        a = [np.ascontiguousarray(x, dtype=np.float64) for x in (dw0, dti, dtj, dvol, dst)]
        _check(self._lib.fgb_tangent(self._h, int(zone), int(nsteps), *(_dp(x) for x in a), _dp(out)))
        return out

    def synchronize(self):
        _check(self._lib.fgb_synchronize(self._h))

    def kernel_stats(self, reset: bool = False) -> dict:
        """{group name: (timed groups, total ms)} of the profiled launches."""
        buf = C.create_string_buffer(64)
        cnt, tot = C.c_int64(), C.c_double()
        out = {}
        i = 0
        while True:
            _check(self._lib.fgb_kernel_stats(self._h, i, buf, 64, C.byref(cnt), C.byref(tot)))
            if cnt.value == 0:
                break
            out[buf.value.decode()] = (cnt.value, tot.value)
            i += 1
        if reset:
            _check(self._lib.fgb_kernel_stats(self._h, -1, buf, 64, C.byref(cnt), C.byref(tot)))
        return out

    def timer_start(self):
        _check(self._lib.fgb_stream_timer(self._h, 0, None))

    def timer_stop(self) -> float:
        ms = C.c_double()
        _check(self._lib.fgb_stream_timer(self._h, 1, C.byref(ms)))
        return ms.value

    def launch_count(self) -> int:
        c = C.c_int64()
        _check(self._lib.fgb_launch_count(self._h, C.byref(c)))
        return c.value


def fp64_peak_gflops(device: int = 0) -> float:
    g = C.c_double()
    _check(load().fgb_fp64_peak(int(device), C.byref(g)))
    return g.value
