"""ctypes binding of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check and the
CPU-baseline leg of bench.py, never by the product.  See mlip_oracle.cpp for
the reference functions each part restates.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
TABLE_PATH = os.path.join(os.path.dirname(HERE), "lammps-mlip-package_gb300", "data",
                          "gtinv_table.txt")

_lib = None


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "mlip_oracle.cpp")
    if force or not os.path.exists(LIB_PATH) or \
            os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", HERE, "-B" if force else "all"])
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        L.orc_create.restype = P
        L.orc_create.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
        L.orc_destroy.argtypes = [P]
        L.orc_last_error.restype = ctypes.c_char_p
        L.orc_set_threads.argtypes = [P, ctypes.c_int]
        L.orc_info.argtypes = [P, ip, dp]
        L.orc_dump_itc.restype = ctypes.c_long
        L.orc_dump_itc.argtypes = [P, ip, ctypes.c_long]
        L.orc_dump_poly.restype = ctypes.c_long
        L.orc_dump_poly.argtypes = [P, ip, ctypes.c_long]
        L.orc_sph.argtypes = [P, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                              dp, dp, dp, dp]
        L.orc_radial.argtypes = [P, ctypes.c_double, dp, dp]
        L.orc_compute.restype = ctypes.c_int
        L.orc_compute.argtypes = [P, ctypes.c_int, ctypes.c_int, dp, ip, ip, ip, dp, dp, dp,
                                  dp, dp]
        L.orc_coeffs.argtypes = [P, dp]
        L.orc_features.restype = ctypes.c_int
        L.orc_features.argtypes = [P, ctypes.c_int, ctypes.c_int, dp, ip, ip, ip, dp, dp, dp, dp]
        L.orc_linear_conditioning.restype = ctypes.c_int
        L.orc_linear_conditioning.argtypes = [P, ctypes.c_int, ctypes.c_int, dp, ip, ip, ip, dp]
        L.orc_compute_centers.restype = ctypes.c_int
        L.orc_compute_centers.argtypes = [P, ctypes.c_int, ip, ctypes.c_int, dp, ip, ip, ip,
                                          dp, dp, dp, dp]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


class Oracle:
    INFO_KEYS = ["T", "TC", "F", "L", "Lh", "La", "n_irreps", "n_terms", "ITC", "D",
                 "n_coeffs", "model_type", "maxp"]

    def __init__(self, pot_path: str, threads: int = 1):
        L = lib()
        self.h = L.orc_create(pot_path.encode(), TABLE_PATH.encode())
        if not self.h:
            raise RuntimeError(L.orc_last_error().decode())
        L.orc_set_threads(self.h, threads)
        v = np.zeros(13, dtype=np.int32)
        rc = ctypes.c_double()
        L.orc_info(self.h, _ip(v), ctypes.byref(rc))
        self.info = dict(zip(self.INFO_KEYS, (int(t) for t in v)))
        self.cutoff = rc.value

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def set_threads(self, n: int):
        lib().orc_set_threads(self.h, n)

    def itc_list(self):
        n = lib().orc_dump_itc(self.h, None, 0)
        buf = np.zeros(n, dtype=np.int32)
        lib().orc_dump_itc(self.h, _ip(buf), n)
        return buf

    def poly_list(self):
        n = lib().orc_dump_poly(self.h, None, 0)
        buf = np.zeros(n, dtype=np.int32)
        lib().orc_dump_poly(self.h, _ip(buf), n)
        return buf

    def sph(self, d):
        Lh = self.info["Lh"]
        out = [np.zeros(2 * Lh) for _ in range(4)]
        lib().orc_sph(self.h, float(d[0]), float(d[1]), float(d[2]), *[_dp(o) for o in out])
        return [o[0::2] + 1j * o[1::2] for o in out]

    def radial(self, r):
        F = self.info["F"]
        fn = np.zeros(F)
        fnd = np.zeros(F)
        lib().orc_radial(self.h, float(r), _dp(fn), _dp(fnd))
        return fn, fnd

    def compute(self, sysm, want_anlm: bool = False):
        """Reference semantics on a System: returns dict(energy, f_all, virial, eatom[, anlm])."""
        x = np.ascontiguousarray(sysm.x, dtype=np.float64)
        t = np.ascontiguousarray(sysm.type, dtype=np.int32)
        off = np.ascontiguousarray(sysm.nbr_off, dtype=np.int32)
        nb = np.ascontiguousarray(sysm.nbr_idx, dtype=np.int32)
        f = np.zeros(sysm.nall * 3)
        e = ctypes.c_double()
        vir = np.zeros(6)
        eat = np.zeros(sysm.nlocal)
        an = None
        anp = None
        if want_anlm:
            i = self.info
            an = np.zeros(sysm.nlocal * i["T"] * i["F"] * i["Lh"] * 2)
            anp = _dp(an)
        lib().orc_compute(self.h, sysm.nlocal, sysm.nall, _dp(x), _ip(t), _ip(off), _ip(nb),
                          _dp(f), ctypes.byref(e), _dp(vir), _dp(eat), anp)
        out = dict(energy=e.value, f_all=f.reshape(-1, 3), virial=vir, eatom=eat)
        if want_anlm:
            i = self.info
            a = an[0::2] + 1j * an[1::2]
            out["anlm"] = a.reshape(sysm.nlocal, i["T"], i["F"], i["Lh"])
        return out

    def features(self, sysm, want=("d", "p", "ff", "sf")):
        """Training features (reference semantics): structural d [nlocal, D],
        polynomial p [nlocal, C], force ff [nlocal, C, 3] (ghost rows folded onto
        their owners) and stress sf [C, 6] (order xx yy zz yz zx xy)."""
        x = np.ascontiguousarray(sysm.x, dtype=np.float64)
        t = np.ascontiguousarray(sysm.type, dtype=np.int32)
        off = np.ascontiguousarray(sysm.nbr_off, dtype=np.int32)
        nb = np.ascontiguousarray(sysm.nbr_idx, dtype=np.int32)
        D, C = self.info["D"], self.info["n_coeffs"]
        d = np.zeros((sysm.nlocal, D)) if "d" in want else None
        p = np.zeros((sysm.nlocal, C)) if "p" in want else None
        ff = np.zeros((sysm.nall, C, 3)) if "ff" in want else None
        sf = np.zeros((C, 6)) if "sf" in want else None
        lib().orc_features(self.h, sysm.nlocal, sysm.nall, _dp(x), _ip(t), _ip(off), _ip(nb),
                           *[(_dp(a) if a is not None else None) for a in (d, p, ff, sf)])
        out = {}
        if d is not None:
            out["d"] = d
        if p is not None:
            out["p"] = p
        if ff is not None:
            folded = np.zeros((sysm.nlocal, C, 3))
            np.add.at(folded, sysm.owner, ff)
            out["ff"] = folded
        if sf is not None:
            out["sf"] = sf
        return out

    def coefficients(self):
        """The potential's regression coefficients (divided by their scales)."""
        w = np.zeros(self.info["n_coeffs"])
        lib().orc_coeffs(self.h, _dp(w))
        return w

    def linear_conditioning(self, sysm):
        """Per owned atom: sum over linear-only features of |w_f| sum_terms |c| prod |a|
        (the scale of the FP32 rounding error of those energy terms)."""
        x = np.ascontiguousarray(sysm.x, dtype=np.float64)
        t = np.ascontiguousarray(sysm.type, dtype=np.int32)
        off = np.ascontiguousarray(sysm.nbr_off, dtype=np.int32)
        nb = np.ascontiguousarray(sysm.nbr_idx, dtype=np.int32)
        out = np.zeros(sysm.nlocal)
        lib().orc_linear_conditioning(self.h, sysm.nlocal, sysm.nall, _dp(x), _ip(t), _ip(off),
                                      _ip(nb), _dp(out))
        return out

    def compute_centers(self, sysm, centers):
        """Owner-computes evaluation for a subset of centre atoms (CPU baseline)."""
        x = np.ascontiguousarray(sysm.x, dtype=np.float64)
        t = np.ascontiguousarray(sysm.type, dtype=np.int32)
        off = np.ascontiguousarray(sysm.nbr_off, dtype=np.int32)
        nb = np.ascontiguousarray(sysm.nbr_idx, dtype=np.int32)
        c = np.ascontiguousarray(centers, dtype=np.int32)
        f = np.zeros(sysm.nall * 3)
        e = ctypes.c_double()
        vir = np.zeros(6)
        eat = np.zeros(len(c))
        lib().orc_compute_centers(self.h, len(c), _ip(c), sysm.nall, _dp(x), _ip(t),
                                  _ip(off), _ip(nb), _dp(f), ctypes.byref(e), _dp(vir),
                                  _dp(eat))
        return dict(energy=e.value, f_all=f.reshape(-1, 3), virial=vir, eatom=eat)
