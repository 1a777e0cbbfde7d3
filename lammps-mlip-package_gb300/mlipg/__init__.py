"""Python binding (ctypes) of libmlipg.so, the GB300 MLIP C ABI (include/mlipg.h).

This mirrors how LAMMPS drives the reference pair style: create a handle
from a potential file (``pair_coeff`` reads it), map LAMMPS types to file
elements, then call `Potential.compute` with owned+ghost coordinates and a
full neighbour list.  There is no CPU fallback: on a machine without a GPU
the model can be inspected but every compute raises `MlipgError` with
``MLIPG_ENOGPU``.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

PREC_FP64 = 0
PREC_MIXED = 1
PREC_MIXED_A64 = 2   # mixed, with the order-parameter sums in plain FP64
PREC_FP64_NATIVE = 3  # every product and sum in native FP64 (PREC_FP64 runs the
                      # invariant/adjoint products in double-float arithmetic)
ERRORS = {1: "EINVAL", 2: "EIO", 3: "ENOMEM", 4: "ECUDA", 5: "ENOTSUP", 6: "ECAPACITY",
          7: "ENOGPU", 8: "ETIMEDOUT", 9: "EBUSY"}

_lib = None


class MlipgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "?"), code, msg))
        self.code = code


def lib():
    """Loads libmlipg.so (building it in-tree first if it is missing or stale)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build()
    L = ctypes.CDLL(path)
    P = ctypes.c_void_p
    i32 = ctypes.c_int
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    llp = ctypes.POINTER(ctypes.c_longlong)
    sig = {
        "mlipg_last_error": (ctypes.c_char_p, [P]),
        "mlipg_create": (i32, [ctypes.c_char_p, i32, ctypes.POINTER(P)]),
        "mlipg_destroy": (i32, [P]),
        "mlipg_set_precision": (i32, [P, i32]),
        "mlipg_num_elements": (i32, [P]),
        "mlipg_element_name": (ctypes.c_char_p, [P, i32]),
        "mlipg_element_mass": (ctypes.c_double, [P, i32]),
        "mlipg_cutoff": (ctypes.c_double, [P]),
        "mlipg_set_type_map": (i32, [P, i32, ctypes.POINTER(ctypes.c_char_p)]),
        "mlipg_compute": (i32, [P, i32, i32, dp, ip, i32, ip, ip, ctypes.POINTER(ip), i32, i32,
                                dp, dp, dp, dp, dp]),
        "mlipg_compute_device": (i32, [P, i32, P, P, P, P, P, P, P, P, i32, P, P, P, P]),
        "mlipg_compute_device_noalloc": (i32, [P, i32, P, P, P, P, P, P, P, P, i32, P, P, P,
                                               P]),
        "mlipg_stream": (P, [P]),
        "mlipg_device_status": (i32, [P, ip]),
        "mlipg_count_coefficients": (i32, [i32, i32, i32, i32, i32, ip, ip, i32, llp, llp]),
        "mlipg_model_info": (i32, [P, llp]),
        "mlipg_dump_itc": (ctypes.c_long, [P, ip, ctypes.c_long]),
        "mlipg_dump_poly": (ctypes.c_long, [P, ip, ctypes.c_long]),
        "mlipg_flops_per_atom_step": (ctypes.c_double, [P, i32, ctypes.c_double]),
        "mlipg_flops_per_atom_step_executed": (ctypes.c_double, [P, i32, ctypes.c_double]),
        "mlipg_nlist_build": (i32, [dp, i32, dp, ip, ctypes.c_double, ctypes.POINTER(P)]),
        "mlipg_nlist_sizes": (i32, [P, ip, llp]),
        "mlipg_nlist_copy": (i32, [P, dp, ip, ip, ip, ip, ip]),
        "mlipg_nlist_destroy": (None, [P]),
        "mlipg_set_profiling": (i32, [P, i32]),
        "mlipg_kernel_times": (i32, [P, ctypes.POINTER(ctypes.c_float), i32]),
        "mlipg_phase_cycles": (i32, [P, ctypes.POINTER(ctypes.c_ulonglong)]),
        "mlipg_md_create": (i32, [P, dp, i32, dp, dp, ip, ctypes.c_double, ctypes.POINTER(P)]),
        "mlipg_md_run": (i32, [P, i32, ctypes.c_double, i32]),
        "mlipg_md_state": (i32, [P, dp, dp, dp]),
        "mlipg_md_thermo": (i32, [P, dp]),
        "mlipg_md_destroy": (None, [P]),
        "mlipg_batch_create": (i32, [P, i32, ip, dp, dp, ip, ctypes.POINTER(P)]),
        "mlipg_batch_launch": (i32, [P]),
        "mlipg_batch_compute": (i32, [P, dp, dp, dp]),
        "mlipg_batch_sizes": (i32, [P, ip, llp]),
        "mlipg_batch_destroy": (None, [P]),
        "mlipg_batch_results": (i32, [P, dp, dp, dp]),
        "mlipg_batch_device_bytes": (ctypes.c_size_t, [P]),
        "mlipg_server_create": (i32, [ctypes.c_char_p, ctypes.c_size_t, i32, ctypes.POINTER(P)]),
        "mlipg_server_set_batch_atoms": (i32, [P, i32, i32]),
        "mlipg_server_submit": (i32, [P, i32, dp, dp, ip, i32, llp]),
        "mlipg_server_wait": (i32, [P, ctypes.c_longlong, i32, dp, dp, dp]),
        "mlipg_server_stats": (i32, [P, dp]),
        "mlipg_server_destroy": (None, [P]),
        "mlipg_measure_fma_peak": (i32, [i32, dp]),
        "mlipg_set_tiling": (i32, [P, i32, i32, i32]),
        "mlipg_get_tiling": (i32, [P, ip]),
        "mlipg_autotune": (i32, [P, i32, P, P, P, P, P, P, P, i32, P, P, i32, dp, ip]),
        "mlipg_batch_autotune": (i32, [P, i32, dp, ip]),
        "mlipg_md_autotune": (i32, [P, i32, dp, ip]),
        "mlipg_feature_sizes": (i32, [P, llp, llp]),
        "mlipg_features": (i32, [P, i32, dp, dp, ip, dp, dp, dp, dp]),
        "mlipg_dnlist_create": (i32, [P, ctypes.POINTER(P)]),
        "mlipg_dnlist_build": (i32, [P, i32, ip, dp, P, ctypes.c_double, i32]),
        "mlipg_dnlist_arrays": (i32, [P, ctypes.POINTER(P), ctypes.POINTER(P), ctypes.POINTER(P),
                                      ctypes.POINTER(P), ctypes.POINTER(P), llp, ip, ip]),
        "mlipg_dnlist_copy": (i32, [P, ip, ip, ip]),
        "mlipg_dnlist_destroy": (None, [P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def _check(rc, h=None):
    if rc != 0:
        msg = lib().mlipg_last_error(h)
        raise MlipgError(rc, msg.decode() if msg else "")


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def count_coefficients(n_types, model_type, maxp, maxl, gtinv_order, gtinv_maxl, gtinv_sym,
                       n_fn):
    """(n_coeffs, n_features) of a model specification (no GPU needed)."""
    ml = np.ascontiguousarray(list(gtinv_maxl) or [0], dtype=np.int32)
    sy = np.ascontiguousarray([int(s) for s in gtinv_sym] or [0], dtype=np.int32)
    nc = ctypes.c_longlong()
    nf = ctypes.c_longlong()
    _check(lib().mlipg_count_coefficients(n_types, model_type, maxp, maxl, gtinv_order, _ip(ml),
                                          _ip(sy), n_fn, ctypes.byref(nc), ctypes.byref(nf)))
    return nc.value, nf.value


def measure_fma_peak(fp64: bool) -> float:
    """Live FP64 / FP32 CUDA-core FMA throughput of the current device (TFLOP/s)."""
    v = ctypes.c_double()
    _check(lib().mlipg_measure_fma_peak(1 if fp64 else 0, ctypes.byref(v)))
    return v.value


def native_system(cell, cutoff: float, skin: float = 0.0):
    """`structures.System` built by the library's native neighbour builder."""
    from .structures import Cell, System
    lat = np.ascontiguousarray(cell.lattice, dtype=np.float64)
    x = np.ascontiguousarray(cell.positions, dtype=np.float64)
    t = np.ascontiguousarray(cell.types, dtype=np.int32)
    h = ctypes.c_void_p()
    _check(lib().mlipg_nlist_build(_dp(lat), len(t), _dp(x), _ip(t), cutoff + skin,
                                   ctypes.byref(h)))
    try:
        nall = ctypes.c_int()
        npairs = ctypes.c_longlong()
        _check(lib().mlipg_nlist_sizes(h, ctypes.byref(nall), ctypes.byref(npairs)))
        xa = np.zeros((nall.value, 3))
        ta = np.zeros(nall.value, dtype=np.int32)
        ow = np.zeros(nall.value, dtype=np.int32)
        im = np.zeros(nall.value, dtype=np.int32)
        off = np.zeros(len(t) + 1, dtype=np.int32)
        idx = np.zeros(max(npairs.value, 1), dtype=np.int32)
        _check(lib().mlipg_nlist_copy(h, _dp(xa), _ip(ta), _ip(ow), _ip(im), _ip(off), _ip(idx)))
    finally:
        lib().mlipg_nlist_destroy(h)
    s = System(cell=Cell(lat, xa[:len(t)].copy(), t), x=xa, type=ta, owner=ow.astype(np.int64),
               nbr_off=off, nbr_idx=idx[:npairs.value], nlocal=len(t), cutoff=cutoff)
    s.image = im
    return s


class Potential:
    """A loaded potential on the current CUDA device (one handle, one stream)."""

    INFO = ["T", "F", "L", "Lh", "n_irreps", "n_terms", "n_folded_terms", "ITC", "D",
            "n_coeffs", "model_type", "maxp", "max_nonlinear_itc"]

    def __init__(self, path: str, precision: int = PREC_FP64):
        import weakref
        self._children = weakref.WeakSet()   # batches / MD runs built on this handle
        h = ctypes.c_void_p()
        _check(lib().mlipg_create(os.fsencode(path), precision, ctypes.byref(h)))
        self.h = h
        self.precision = precision
        v = (ctypes.c_longlong * 13)()
        _check(lib().mlipg_model_info(self.h, v), self.h)
        self.info = dict(zip(self.INFO, list(v)))
        self.elements = [lib().mlipg_element_name(self.h, k).decode()
                         for k in range(lib().mlipg_num_elements(self.h))]
        self.masses = [lib().mlipg_element_mass(self.h, k) for k in range(len(self.elements))]
        self.cutoff = lib().mlipg_cutoff(self.h)

    def close(self):
        # objects that use this handle's stream go first (in a garbage-collected
        # cycle the handle may be finalized before them)
        for child in list(getattr(self, "_children", ())):
            child.close()
        if getattr(self, "h", None):
            lib().mlipg_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def set_precision(self, precision: int):
        _check(lib().mlipg_set_precision(self.h, precision), self.h)
        self.precision = precision

    def set_type_map(self, names):
        arr = (ctypes.c_char_p * len(names))(*[n.encode() for n in names])
        _check(lib().mlipg_set_type_map(self.h, len(names), arr), self.h)

    def stream(self) -> int:
        return lib().mlipg_stream(self.h) or 0

    def set_tiling(self, irr_chunk: int = 24, warp_order: int = 0, ctas_per_sm: int = 0):
        _check(lib().mlipg_set_tiling(self.h, irr_chunk, warp_order, ctas_per_sm), self.h)

    def tiling(self):
        o = (ctypes.c_int * 3)()
        _check(lib().mlipg_get_tiling(self.h, o), self.h)
        return {"irr_chunk": o[0], "warp_order": o[1], "ctas_per_sm": o[2]}

    def autotune_device(self, ncenters, x4, centers, nbr_off, nbr_idx, f, out8, img=0, cell=0,
                        center_cell=0, nb_cap=0):
        """Autotunes on device buffers (pointers, as for compute_device)."""
        rep = np.zeros(4 * 64)
        n = ctypes.c_int()
        _check(lib().mlipg_autotune(self.h, ncenters, x4, centers, nbr_off, nbr_idx,
                                    img or None, cell or None, center_cell or None, nb_cap, f,
                                    out8, 64, _dp(rep), ctypes.byref(n)), self.h)
        return _tiling_rows(rep, n.value)

    def itc_list(self):
        n = lib().mlipg_dump_itc(self.h, None, 0)
        b = np.zeros(n, dtype=np.int32)
        lib().mlipg_dump_itc(self.h, _ip(b), n)
        return b

    def poly_list(self):
        n = lib().mlipg_dump_poly(self.h, None, 0)
        b = np.zeros(n, dtype=np.int32)
        lib().mlipg_dump_poly(self.h, _ip(b), n)
        return b

    def flops_per_atom_step(self, elem: int, nbar: float, executed: bool = False) -> float:
        fn = lib().mlipg_flops_per_atom_step_executed if executed else \
            lib().mlipg_flops_per_atom_step
        return fn(self.h, elem, nbar)

    def compute_lammps(self, nlocal, nall, x, lmp_type, ilist, numneigh, firstneigh_arrays,
                       eatom=True, vatom=False):
        """LAMMPS-shaped call: x[nall,3], 1-based types, per-atom neighbour arrays.

        Returns (energy, f_all[nall,3], virial6 LAMMPS order, eatom[nlocal]) and, with
        vatom=True, vatom[nlocal, 6] as a fifth element.
        """
        x = np.ascontiguousarray(x, dtype=np.float64)
        t = np.ascontiguousarray(lmp_type, dtype=np.int32)
        il = np.ascontiguousarray(ilist, dtype=np.int32)
        nn = np.ascontiguousarray(numneigh, dtype=np.int32)
        keep = [np.ascontiguousarray(a, dtype=np.int32) for a in firstneigh_arrays]
        fp = (ctypes.POINTER(ctypes.c_int) * max(nall, 1))()
        for i, a in enumerate(keep):
            fp[i] = _ip(a)
        f = np.zeros((nall, 3))
        e = ctypes.c_double()
        vir = np.zeros(6)
        ea = np.zeros(max(nlocal, 1)) if eatom else None
        va = np.zeros((max(nlocal, 1), 6)) if vatom else None
        _check(lib().mlipg_compute(self.h, nlocal, nall, _dp(x), _ip(t), len(il), _ip(il),
                                   _ip(nn), fp, 1, 1, _dp(f), ctypes.byref(e), _dp(vir),
                                   _dp(ea) if eatom else None, _dp(va) if vatom else None),
               self.h)
        out = (e.value, f, vir, (ea[:nlocal] if eatom else None))
        return out + (va[:nlocal],) if vatom else out

    def compute(self, system, eatom=True, vatom=False):
        """Evaluates a `structures.System` through the LAMMPS-shaped C ABI."""
        off = system.nbr_off
        lists = [system.nbr_idx[off[i]:off[i + 1]] for i in range(system.nlocal)]
        nn = np.diff(off).astype(np.int32)
        r = self.compute_lammps(system.nlocal, system.nall, system.x, system.type + 1,
                                np.arange(system.nlocal), nn, lists, eatom, vatom)
        out = dict(energy=r[0], f_all=r[1], virial=r[2], eatom=r[3])
        if vatom:
            out["vatom"] = r[4]
        return out

    def compute_device(self, ncenters, x4, centers, nbr_off, nbr_idx, f, out8, eatom=None,
                       img=None, cell=None, center_cell=None, fold=None, nb_cap=256,
                       vatom=None):
        """Stream-ordered call on device pointers (ints); see mlipg_compute_device."""
        _check(lib().mlipg_compute_device(self.h, ncenters, x4, centers, nbr_off, nbr_idx,
                                          img, cell, center_cell, fold, nb_cap, f, eatom, vatom,
                                          out8), self.h)

    def features(self, cell, want=("d", "p", "ff", "sf")):
        """Training features of a periodic cell (see mlipg_features): structural d
        [natoms, D], polynomial p [natoms, C], force ff [natoms, C, 3] and stress
        sf [C, 6] (order xx yy zz yz zx xy), with E = p.sum(0) . w, F = ff . w and
        the virial sf . w for the coefficients w."""
        nd, nc = ctypes.c_longlong(), ctypes.c_longlong()
        _check(lib().mlipg_feature_sizes(self.h, ctypes.byref(nd), ctypes.byref(nc)), self.h)
        D, C, n = nd.value, nc.value, cell.natoms
        out = {"d": np.zeros((n, D)) if "d" in want else None,
               "p": np.zeros((n, C)) if "p" in want else None,
               "ff": np.zeros((n, C, 3)) if "ff" in want else None,
               "sf": np.zeros((C, 6)) if "sf" in want else None}
        lat = np.ascontiguousarray(cell.lattice, dtype=np.float64)
        x = np.ascontiguousarray(cell.positions, dtype=np.float64)
        t = np.ascontiguousarray(cell.types, dtype=np.int32)
        _check(lib().mlipg_features(self.h, n, _dp(lat), _dp(x), _ip(t),
                                    *[(_dp(out[k]) if out[k] is not None else None)
                                      for k in ("d", "p", "ff", "sf")]), self.h)
        return {k: v for k, v in out.items() if v is not None}

    def set_profiling(self, on: bool):
        _check(lib().mlipg_set_profiling(self.h, 1 if on else 0), self.h)

    def kernel_times(self, cap: int = 4096):
        buf = (ctypes.c_float * cap)()
        n = lib().mlipg_kernel_times(self.h, buf, cap)
        return [buf[k] for k in range(max(n, 0))]

    def compute_device_noalloc(self, ncenters, x4, centers, nbr_off, nbr_idx, f, out8,
                               eatom=None, img=None, cell=None, center_cell=None, fold=None,
                               nb_cap=256, vatom=None):
        """mlipg_compute_device_noalloc: same as compute_device, allocates nothing."""
        _check(lib().mlipg_compute_device_noalloc(self.h, ncenters, x4, centers, nbr_off,
                                                  nbr_idx, img, cell, center_cell, fold, nb_cap,
                                                  f, eatom, vatom, out8), self.h)

    PHASES = ["compaction", "order_parameters", "nonlinear_polynomial", "invariants_batched",
              "invariants_single", "forces_reduction"]

    def phase_cycles(self):
        buf = (ctypes.c_ulonglong * 8)()
        _check(lib().mlipg_phase_cycles(self.h, buf), self.h)
        return dict(zip(self.PHASES, [int(buf[k]) for k in range(6)]))

    def device_status(self) -> int:
        b = ctypes.c_int()
        _check(lib().mlipg_device_status(self.h, ctypes.byref(b)), self.h)
        return b.value


class MD:
    """NVE molecular dynamics of one periodic cell on the device (metal units)."""

    THERMO = ["pe", "ke", "temp", "etotal", "press", "pxx", "pyy", "pzz", "pxy", "pxz", "pyz",
              "rebuilds"]

    def __init__(self, potential: Potential, cell, velocities=None, skin: float = 1.0):
        self.pot = potential
        self.n = cell.natoms
        lat = np.ascontiguousarray(cell.lattice, dtype=np.float64)
        x = np.ascontiguousarray(cell.positions, dtype=np.float64)
        t = np.ascontiguousarray(cell.types, dtype=np.int32)
        v = None if velocities is None else np.ascontiguousarray(velocities, dtype=np.float64)
        h = ctypes.c_void_p()
        rc = lib().mlipg_md_create(potential.h, _dp(lat), self.n, _dp(x),
                                   _dp(v) if v is not None else None, _ip(t), skin,
                                   ctypes.byref(h))
        if rc != 0:
            raise MlipgError(rc, lib().mlipg_last_error(potential.h).decode())
        self.h = h
        potential._children.add(self)

    def run(self, nsteps: int, dt: float = 0.001, graph: bool = True):
        rc = lib().mlipg_md_run(self.h, nsteps, dt, 1 if graph else 0)
        if rc != 0:
            raise MlipgError(rc, lib().mlipg_last_error(self.pot.h).decode())

    def autotune(self):
        """Picks the potential's tile shape for this system; returns the timing table."""
        rep = np.zeros(4 * 64)
        n = ctypes.c_int()
        _check(lib().mlipg_md_autotune(self.h, 64, _dp(rep), ctypes.byref(n)), self.pot.h)
        return _tiling_rows(rep, n.value)

    def state(self):
        x = np.zeros((self.n, 3))
        v = np.zeros((self.n, 3))
        f = np.zeros((self.n, 3))
        _check(lib().mlipg_md_state(self.h, _dp(x), _dp(v), _dp(f)))
        return x, v, f

    def thermo(self):
        o = np.zeros(12)
        _check(lib().mlipg_md_thermo(self.h, _dp(o)))
        return dict(zip(self.THERMO, o.tolist()))

    def close(self):
        if getattr(self, "h", None):
            lib().mlipg_md_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


def maxwell_boltzmann(masses, temperature, rng):
    """Velocities (A/ps, metal units) at `temperature` K, zero total momentum,
    rescaled to exactly that temperature with dof = 3N - 3."""
    kb, mvv2e = 8.617343e-5, 1.0364269e-4
    m = np.asarray(masses, dtype=np.float64)
    v = rng.normal(size=(len(m), 3)) * np.sqrt(kb * temperature / (m * mvv2e))[:, None]
    v -= (m[:, None] * v).sum(0) / m.sum()
    ke = 0.5 * (m[:, None] * v * v).sum() * mvv2e
    t = 2 * ke / ((3 * len(m) - 3) * kb)
    return v * np.sqrt(temperature / t) if t > 0 else v


def _tiling_rows(rep, n):
    r = rep.reshape(-1, 4)[:min(n, 64)]
    return [{"irr_chunk": int(a), "warp_order": int(b), "ctas_per_sm": int(c), "ms": float(d)}
            for a, b, c, d in r]


class Batch:
    """Many periodic cells evaluated in one persistent launch (see mlipg_batch_*)."""

    def __init__(self, potential: Potential, cells):
        self.pot = potential
        self.ncells = len(cells)
        n = np.array([c.natoms for c in cells], dtype=np.int32)
        lat = np.ascontiguousarray(np.stack([c.lattice for c in cells]), dtype=np.float64)
        x = np.ascontiguousarray(np.concatenate([c.positions for c in cells]), dtype=np.float64)
        t = np.ascontiguousarray(np.concatenate([c.types for c in cells]), dtype=np.int32)
        self.natoms = n
        self.offsets = np.concatenate([[0], np.cumsum(n)])
        h = ctypes.c_void_p()
        rc = lib().mlipg_batch_create(potential.h, self.ncells, _ip(n), _dp(lat), _dp(x), _ip(t),
                                      ctypes.byref(h))
        if rc != 0:
            raise MlipgError(rc, "mlipg_batch_create failed")
        self.h = h
        potential._children.add(self)
        na = ctypes.c_int()
        npairs = ctypes.c_longlong()
        lib().mlipg_batch_sizes(self.h, ctypes.byref(na), ctypes.byref(npairs))
        self.total_atoms, self.npairs = na.value, npairs.value

    def launch(self):
        _check(lib().mlipg_batch_launch(self.h))

    def autotune(self):
        """Picks the potential's tile shape for this batch; returns the timing table."""
        rep = np.zeros(4 * 64)
        n = ctypes.c_int()
        _check(lib().mlipg_batch_autotune(self.h, 64, _dp(rep), ctypes.byref(n)), self.pot.h)
        return _tiling_rows(rep, n.value)

    def compute(self):
        e = np.zeros(self.ncells)
        f = np.zeros((self.total_atoms, 3))
        v = np.zeros((self.ncells, 6))
        rc = lib().mlipg_batch_compute(self.h, _dp(e), _dp(f), _dp(v))
        if rc != 0:
            raise MlipgError(rc, lib().mlipg_last_error(self.pot.h).decode())
        return e, f, v

    def close(self):
        if getattr(self, "h", None):
            lib().mlipg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


class Server:
    """Continuous-batching request loop (see mlipg_server_*)."""

    STATS = ["completed", "p50_ms", "p99_ms", "atom_steps_per_s", "batches", "device_bytes",
             "queued", "in_flight"]

    def __init__(self, path: str, budget_bytes: int = 64 << 30, max_batch_atoms: int = 65536,
                 max_batch_atoms_fp64: int = 0):
        lib()
        h = ctypes.c_void_p()
        _check(lib().mlipg_server_create(os.fsencode(path), budget_bytes, max_batch_atoms,
                                         ctypes.byref(h)))
        self.h = h
        self.natoms = {}
        if max_batch_atoms_fp64 > 0:
            _check(lib().mlipg_server_set_batch_atoms(self.h, PREC_FP64, max_batch_atoms_fp64))

    def submit(self, cell, precision: int) -> int:
        lat = np.ascontiguousarray(cell.lattice, dtype=np.float64)
        x = np.ascontiguousarray(cell.positions, dtype=np.float64)
        t = np.ascontiguousarray(cell.types, dtype=np.int32)
        tk = ctypes.c_longlong()
        _check(lib().mlipg_server_submit(self.h, cell.natoms, _dp(lat), _dp(x), _ip(t),
                                         precision, ctypes.byref(tk)))
        self.natoms[tk.value] = cell.natoms
        return tk.value

    def wait(self, ticket: int, timeout_ms: int = 60000):
        n = self.natoms.get(ticket, 0)
        e = ctypes.c_double()
        f = np.zeros((n, 3))
        v = np.zeros(6)
        rc = lib().mlipg_server_wait(self.h, ticket, timeout_ms, ctypes.byref(e), _dp(f), _dp(v))
        if rc != 0:
            raise MlipgError(rc, "mlipg_server_wait")
        del self.natoms[ticket]
        return e.value, f, v

    def stats(self):
        o = np.zeros(8)
        _check(lib().mlipg_server_stats(self.h, _dp(o)))
        return dict(zip(self.STATS, o.tolist()))

    def close(self):
        if getattr(self, "h", None):
            lib().mlipg_server_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


class DeviceNeighbourList:
    """Image-coded full lists of many cells built on the device (mlipg_dnlist_*).

    `build` takes a device pointer to double4 positions + element of all cells
    (wrapped into their cells in place)."""

    def __init__(self, stream: int = 0):
        h = ctypes.c_void_p()
        _check(lib().mlipg_dnlist_create(stream or None, ctypes.byref(h)))
        self.h = h
        self.natoms = 0

    def build(self, natoms, lattices, x4_ptr: int, rlist: float, headroom_pct: int = 0):
        n = np.ascontiguousarray(natoms, dtype=np.int32)
        lat = np.ascontiguousarray(lattices, dtype=np.float64).reshape(-1, 9)
        _check(lib().mlipg_dnlist_build(self.h, len(n), _ip(n), _dp(lat), x4_ptr, rlist,
                                        headroom_pct))
        self.natoms = int(n.sum())
        return self.info()

    def info(self):
        ptrs = [ctypes.c_void_p() for _ in range(5)]
        npairs = ctypes.c_longlong()
        maxn = ctypes.c_int()
        gen = ctypes.c_int()
        _check(lib().mlipg_dnlist_arrays(self.h, *[ctypes.byref(p) for p in ptrs],
                                         ctypes.byref(npairs), ctypes.byref(maxn),
                                         ctypes.byref(gen)))
        keys = ["off", "idx", "img", "center_cell", "cells"]
        out = {k: p.value or 0 for k, p in zip(keys, ptrs)}
        out.update(npairs=npairs.value, max_neigh=maxn.value, generation=gen.value)
        return out

    def copy(self):
        info = self.info()
        off = np.zeros(self.natoms + 1, dtype=np.int32)
        idx = np.zeros(max(info["npairs"], 1), dtype=np.int32)
        img = np.zeros(max(info["npairs"], 1), dtype=np.int32)
        _check(lib().mlipg_dnlist_copy(self.h, _ip(off), _ip(idx), _ip(img)))
        return off, idx[:info["npairs"]], img[:info["npairs"]]

    def close(self):
        if getattr(self, "h", None):
            lib().mlipg_dnlist_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()
