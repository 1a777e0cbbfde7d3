"""Regenerate the golden fixtures in this directory from the reference package.

Run in an environment where the reference sources are present (they are not
on the GPU host; the outputs of this script are committed):

    python tests/golden/make_golden.py /path/to/reference

What it writes:
* ``gtinv-{197,820,434}.mlip.gz``, ``pair-{60,17}.mlip.gz`` -- the
  reference's regression potentials (test/regression/*.mlip), gzip-compressed,
  unchanged (the pair potentials drive its `pair_style mlip_pair` runs).
* ``structure*.lammps`` -- the reference's 32-atom TiAl3 cell and the 64-atom
  conventional / triclinic cells (test/regression/).
* ``golden.json`` --
  - thermo values at step 0 read from the reference's LAMMPS logs
    (E_pair, Press, Pxx..Pyz), with the log line they come from;
  - model-structure fingerprints (irreps/term/feature/coefficient counts and
    SHA-256 of the irreps x typecomb list and of the polynomial index) and
    the scaled coefficients' checksum, computed by the reference's OWN
    parser / enumeration code compiled from its sources (oracle/_ref,
    built by oracle/build_ref.sh);
  - spherical harmonics Y_lm and dY_lm/dx,y,z (l <= 12) at fixed directions
    from the reference's host spherical-harmonics class;
  - half-list pair counts of the reference's neighbour builder for the cells;
  - the unit-test known answers of test/test_mlip_features.cpp.
"""
from __future__ import annotations

import ctypes
import gzip
import hashlib
import json
import os
import re
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
POTS = ["gtinv-197", "gtinv-820", "gtinv-434"]
PAIR_POTS = ["pair-60", "pair-17"]
STRUCTS = ["structure.lammps", "structure_00064_conventional.lammps",
           "structure_00064_triclinic.lammps"]
DUMPS = ["dump.atom.gtinv-197", "dump.atom.gtinv-820", "dump.atom.gtinv-434",
         "dump.atom.pair-60", "dump.atom.pair-17"]
SH_DIRS = [(0.3, -0.4, 1.2), (-1.1, 0.2, -0.5), (0.7, 0.7, 0.0), (0.0, 0.0, 2.0),
           (1e-3, -2e-3, -1.5), (-0.25, -0.9, 0.35)]


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.int64).tobytes()).hexdigest()


def thermo_rows(log_path):
    """All thermo rows of the first run block: {step: {column: value}}."""
    lines = open(log_path).read().splitlines()
    for i, ln in enumerate(lines):
        if ln.strip().startswith("Step "):
            head = ln.split()
            rows = {}
            for k in range(i + 1, len(lines)):
                if lines[k].startswith("Loop time"):
                    break
                vals = lines[k].split()
                rows[int(float(vals[0]))] = dict(zip(head, map(float, vals)))
                rows[int(float(vals[0]))]["cite"] = "test/regression/%s:%d" % (
                    os.path.basename(log_path), k + 1)
            return rows
    raise ValueError("no thermo block in " + log_path)


def thermo_step0(log_path):
    lines = open(log_path).read().splitlines()
    for i, ln in enumerate(lines):
        if ln.strip().startswith("Step "):
            head = ln.split()
            vals = lines[i + 1].split()
            return dict(zip(head, map(float, vals))), i + 2
    raise ValueError("no thermo block in " + log_path)


def ref_lib(ref_root):
    so = os.path.join(REPO, "oracle", "_ref", "libmlipref.so")
    env = dict(os.environ, REF_SRC=os.path.join(ref_root, "src", "USER-MLIP"))
    subprocess.check_call(["sh", os.path.join(REPO, "oracle", "build_ref.sh")], env=env)
    L = ctypes.CDLL(so)
    ip = ctypes.POINTER(ctypes.c_int)
    dp = ctypes.POINTER(ctypes.c_double)
    L.ref_load.argtypes = [ctypes.c_char_p]
    L.ref_info.argtypes = [ip]
    L.ref_dump_itc.restype = ctypes.c_long
    L.ref_dump_itc.argtypes = [ip, ctypes.c_long]
    L.ref_dump_poly.restype = ctypes.c_long
    L.ref_dump_poly.argtypes = [ip, ctypes.c_long]
    L.ref_dump_terms.restype = ctypes.c_long
    L.ref_dump_terms.argtypes = [dp, ctypes.c_long]
    L.ref_coeffs.argtypes = [dp]
    L.ref_sph.argtypes = [ctypes.c_int] + [ctypes.c_double] * 3 + [dp] * 4
    L.ref_count_half_pairs.restype = ctypes.c_long
    L.ref_count_half_pairs.argtypes = [ctypes.c_int, dp, dp, ctypes.c_double]
    return L


def model_fingerprint(L, path):
    ip = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    L.ref_load(path.encode())
    info = np.zeros(7, dtype=np.int32)
    L.ref_info(ip(info))
    n = L.ref_dump_itc(None, 0)
    itc = np.zeros(n, dtype=np.int32)
    L.ref_dump_itc(ip(itc), n)
    n = L.ref_dump_poly(None, 0)
    poly = np.zeros(n, dtype=np.int32)
    L.ref_dump_poly(ip(poly), n)
    n = L.ref_dump_terms(None, 0)
    terms = np.zeros(n)
    L.ref_dump_terms(dp(terms), n)
    co = np.zeros(int(info[4]))
    L.ref_coeffs(dp(co))
    keys = ["n_irreps", "n_terms", "ITC", "D", "n_coeffs", "T", "F"]
    out = dict(zip(keys, (int(v) for v in info)))
    out.update(itc_sha256=sha(itc), poly_sha256=sha(poly), itc_len=int(itc.size),
               poly_len=int(poly.size), coeff_sum=float(co.sum()),
               coeff_abs_sum=float(np.abs(co).sum()), coeff_first=[float(v) for v in co[:4]],
               term_coeff_sum=float(terms.sum()))
    return out


def main():
    if len(sys.argv) < 2:
        sys.exit("usage: make_golden.py <reference package root (with test/regression)>")
    ref = sys.argv[1]
    reg = os.path.join(ref, "test", "regression")
    sys.path.insert(0, os.path.join(REPO, "lammps-mlip-package_gb300"))
    from mlipg.structures import read_lammps_data

    for p in POTS + PAIR_POTS:
        with open(os.path.join(reg, p + ".mlip"), "rb") as fi, \
                gzip.open(os.path.join(HERE, p + ".mlip.gz"), "wb", 9) as fo:
            shutil.copyfileobj(fi, fo)
    for s in STRUCTS + DUMPS:
        shutil.copy(os.path.join(reg, s), os.path.join(HERE, s))

    gold = {"source": "quantum-mtl/lammps-mlip-package test/regression and test/*.cpp"}
    logs = {}
    for name, log in [("gtinv-197", "log.lammps.gtinv-197"),
                      ("gtinv-820", "log.lammps.gtinv-820"),
                      ("gtinv-434", "log.lammps.gtinv-434"),
                      ("gtinv-197-stress", "log.lammps.gtinv-197.stress.ev_tally"),
                      ("gtinv-197-conv64", "log.lammps.gtinv-197.conv64"),
                      ("pair-60", "log.lammps.pair-60"),
                      ("pair-17", "log.lammps.pair-17")]:
        vals, line = thermo_step0(os.path.join(reg, log))
        vals["cite"] = "test/regression/%s:%d" % (log, line)
        logs[name] = vals
    gold["thermo_step0"] = logs
    # NVE trajectories: thermo at every printed step (100 steps, dt 1 fs; the
    # stress run uses dt 5 fs and prints every 50 steps)
    traj = {}
    for name, log, dt in [("gtinv-197", "log.lammps.gtinv-197", 0.001),
                          ("gtinv-820", "log.lammps.gtinv-820", 0.001),
                          ("gtinv-434", "log.lammps.gtinv-434", 0.001),
                          ("gtinv-197-stress", "log.lammps.gtinv-197.stress.ev_tally", 0.005),
                          ("pair-60", "log.lammps.pair-60", 0.001),
                          ("pair-17", "log.lammps.pair-17", 0.001)]:
        rows = thermo_rows(os.path.join(reg, log))
        traj[name] = {"dt": dt, "rows": {str(k): v for k, v in rows.items()}}
    gold["nve"] = traj

    L = ref_lib(ref)
    gold["model"] = {p: model_fingerprint(L, os.path.join(reg, p + ".mlip")) for p in POTS}

    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    lmax = 12
    lh = (lmax + 1) * (lmax + 2) // 2
    sh = []
    for d in SH_DIRS:
        bufs = [np.zeros(2 * lh) for _ in range(4)]
        L.ref_sph(lmax, d[0], d[1], d[2], *[dp(b) for b in bufs])
        sh.append({"dir": d, "ylm": bufs[0].tolist(), "dx": bufs[1].tolist(),
                   "dy": bufs[2].tolist(), "dz": bufs[3].tolist()})
    gold["sph_lmax12"] = {"cite": "src/USER-MLIP/mlipkk_spherical_harmonics.cpp", "cases": sh}

    pairs = {}
    for s, rc in [("structure.lammps", 8.0), ("structure.lammps", 6.0),
                  ("structure_00064_triclinic.lammps", 8.0)]:
        c = read_lammps_data(os.path.join(reg, s))
        pos = np.ascontiguousarray(c.positions)
        lat = np.ascontiguousarray(c.lattice)
        pairs["%s@%g" % (s, rc)] = int(L.ref_count_half_pairs(c.natoms, dp(pos), dp(lat), rc))
    gold["half_pairs_reference_builder"] = {"cite": "src/USER-MLIP/mlipkk_cell.cpp:218-307",
                                            "counts": pairs}

    text = open(os.path.join(ref, "test", "test_mlip_features.cpp")).read()
    gold["unit_kat"] = {
        "cite": "test/test_mlip_features.cpp:27-42,80-100",
        "ylm_theta0": "Y_l0(theta=0) = sqrt((2l+1)/(4 pi)), Y_lm = 0 for m != 0",
        "fn_r2_rc4_beta_ln2": {"mu": [0.0, 2.0], "fn": [0.03125, 0.5]},
        "present": bool(re.search(r"0\.03125", text)),
    }
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(gold, f, indent=1)
    print("wrote", os.path.join(HERE, "golden.json"))


if __name__ == "__main__":
    main()
