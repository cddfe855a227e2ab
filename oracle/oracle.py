"""ctypes front-end of the CPU oracle (oracle/sph_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the product package.  PARITY UNPINNED:
the oracle restates the reference's Fortran; the reference itself cannot be
built here and ships no golden vectors (see the header of sph_oracle.cpp).
tests/test_oracle.py checks it against known answers and against direct
numpy sums of each module's formula.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

from mysph_gb300 import params as P

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"

ORC_FIELD = dict(IN_DVDT=101, IN_DEDT=102, EX_DVDT=103, AV_DVDT=104,
                 AV_DEDT=105, AS_DVDT=106, TDSDT=107, ROT=108, AH_DEDT=109)

_libs: dict[bool, C.CDLL] = {}


def build(force: bool = False) -> None:
    """Compile both oracle builds with make (seconds)."""
    targets = [BUILD / "liboracle.so", BUILD / "liboracle_omp.so"]
    if force or not all(t.exists() for t in targets) or any(
            t.stat().st_mtime < (HERE / "sph_oracle.cpp").stat().st_mtime for t in targets):
        subprocess.run(["make", "-s", "-C", str(HERE), "-j2"], check=True)


def lib(omp: bool = False) -> C.CDLL:
    if omp in _libs:
        return _libs[omp]
    build()
    L = C.CDLL(str(BUILD / ("liboracle_omp.so" if omp else "liboracle.so")))
    dp, ip, vp = C.POINTER(C.c_double), C.POINTER(C.c_int32), C.c_void_p
    L.orc_create.restype = vp
    L.orc_create.argtypes = [C.POINTER(P.SphParams), C.c_int64, C.c_int64] + [dp] * 8 + [ip] * 3 + [dp]
    L.orc_destroy.argtypes = [vp]
    for name in ("orc_bggs", "orc_rates", "orc_single_step"):
        getattr(L, name).argtypes = [vp]
        getattr(L, name).restype = C.c_int
    L.orc_neighbor_total.argtypes = [vp]
    L.orc_neighbor_total.restype = C.c_int64
    L.orc_export_neighbors.argtypes = [vp, C.POINTER(C.c_int64), ip, C.c_int64]
    L.orc_advance.argtypes = [vp, C.c_int64, dp, dp]
    L.orc_info.argtypes = [vp, C.POINTER(C.c_int64), dp]
    L.orc_get_field.argtypes = [vp, C.c_int32, dp]
    L.orc_kernel.argtypes = [C.c_int32, C.c_int32, C.c_double, dp, C.c_double, dp, dp]
    L.orc_eos.argtypes = [C.POINTER(P.SphMaterial), C.c_int32, C.c_double, C.c_double, dp, dp]
    L.orc_set_search.argtypes = [vp, C.c_int32]
    L.orc_threads.argtypes = [C.c_int]
    L.orc_threads.restype = C.c_int
    _libs[omp] = L
    return L


def _dp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_int32))


class Oracle:
    """One particle system held by the C++ oracle."""

    def __init__(self, case, params: P.SphParams | None = None, omp: bool = False,
                 threads: int = 0, covering_band: bool = False):
        self.L = lib(omp)
        if omp:
            self.threads = self.L.orc_threads(threads)
        self.case = case
        self.prm = (params or case.params).copy()
        self.dim = int(self.prm.dim)
        x, v, m, rho, p, e, c, h, t, s, b, sh = case.arrays()
        self._keep = (x, v, m, rho, p, e, c, h, t, s, b, sh)
        self.h = self.L.orc_create(C.byref(self.prm), case.n_real, case.n_wall,
                                   _dp(x), _dp(v), _dp(m), _dp(rho), _dp(p), _dp(e),
                                   _dp(c), _dp(h), _ip(t), _ip(s), _ip(b), _dp(sh))
        if not self.h:
            raise RuntimeError("orc_create failed")
        if covering_band:
            # exact r < scale_k*h sets even where the reference's band of
            # int(h/cell)+1 cells falls short of 2h (test option)
            self.L.orc_set_search(self.h, 1)
        self.n_real, self.n = case.n_real, case.n

    def __del__(self):
        if getattr(self, "h", None):
            self.L.orc_destroy(self.h)
            self.h = None

    def _check(self, st: int, what: str) -> None:
        if st != 0:
            raise RuntimeError(f"oracle {what} failed with status {st}")

    def bggs(self) -> None:
        self._check(self.L.orc_bggs(self.h), "bggs")

    def neighbors(self):
        """CSR lists (offsets, 1-based indices) in the reference's order."""
        tot = self.L.orc_neighbor_total(self.h)
        off = np.zeros(self.n_real + 1, dtype=np.int64)
        lst = np.zeros(max(tot, 1), dtype=np.int32)
        self._check(self.L.orc_export_neighbors(self.h, off.ctypes.data_as(C.POINTER(C.c_int64)),
                                                _ip(lst), tot), "export")
        return off, lst[:tot]

    def rates(self) -> None:
        self._check(self.L.orc_rates(self.h), "rates")

    def step(self) -> None:
        self._check(self.L.orc_single_step(self.h), "step")

    def advance(self, n: int):
        mx, mean = C.c_double(), C.c_double()
        self._check(self.L.orc_advance(self.h, n, C.byref(mx), C.byref(mean)), "advance")
        return mx.value, mean.value

    def field(self, name: str) -> np.ndarray:
        if name in ORC_FIELD:
            fid = ORC_FIELD[name]
            count = self.n_real
            comp = {"IN_DVDT": self.dim, "EX_DVDT": self.dim, "AV_DVDT": self.dim,
                    "AS_DVDT": self.dim, "ROT": self.dim * self.dim}.get(name, 1)
            if name in ("TDSDT", "ROT"):
                count = self.n
        else:
            fid = P.FIELD[name]
            count = self.n
            comp = {"v": self.dim, "t": self.dim * self.dim, "s": 1}[P.FIELD_SHAPE[name]]
        out = np.zeros(count * comp)
        self._check(self.L.orc_get_field(self.h, fid, _dp(out)), f"field {name}")
        return out.reshape(count, comp) if comp > 1 else out

    def info(self):
        s, t = C.c_int64(), C.c_double()
        self.L.orc_info(self.h, C.byref(s), C.byref(t))
        return s.value, t.value


def kernel(skf: int, dim: int, r: float, dx, hsml: float):
    L = lib(False)
    dxa = np.ascontiguousarray(dx, dtype=np.float64)
    dw = np.zeros(dim)
    w = C.c_double()
    L.orc_kernel(skf, dim, r, _dp(dxa), hsml, C.byref(w), _dp(dw))
    return w.value, dw


def eos(material: P.SphMaterial, solid: bool, rho: float, e: float = 0.0, p0: float = 0.0,
        c0: float = 0.0):
    L = lib(False)
    p, c = C.c_double(p0), C.c_double(c0)
    L.orc_eos(C.byref(material), int(solid), rho, e, C.byref(p), C.byref(c))
    return p.value, c.value
