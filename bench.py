#!/usr/bin/env python
"""Throughput benchmark of the linearized-MLIP energy/force/virial path on GB300.

One step = one evaluation of energy, forces and virial of every atom of the
workload (the hot path behind `pair_style mlip_gtinv`).  Default workload:
the 1,048,576-atom ternary fcc alloy (64^3 conventional cells, a = 4.0 A,
1/3 of each element, jitter N(0, 0.1 A)) with the order-4 / l <= [12, 8, 4]
potential (15 Gaussians, rc 6 A, model_type 3, 68,535 seeded coefficients),
mixed precision.  Inputs are synthetic and seeded.

Reported (one JSON line on rank 0):
  value      atom-steps/s, inputs resident in HBM (positions, CSR full list)
  e2e        the same through mlipg_compute with LAMMPS-shaped host arrays,
             host->device and device->host copies inside the timed region
  fp64       MLIPG_PREC_FP64 (double-float invariant/adjoint products) on all
             centres of the same structure, and the mixed/FP64 speed ratio
  fp64_native  the all-FP64 form on a bounded subset of the centres
  accuracy   mixed vs FP64 (GPU) on a 4,000-atom cell of the same workload
  roofline   algorithmic FLOPs per fused-kernel launch / its CUDA-event time,
             against the live FP32 FMA peak of the device; also on the folded
             table the kernel executes and against the FP32 pipe's arithmetic
             rate at the measured clock
  cpu_baseline  the CPU oracle (restatement of the reference algorithm) on a
             bounded sample of centres, all host threads
`--impl reference` times that CPU implementation alone on the same workload.
Under torchrun each rank evaluates its own replica (weak scaling).
"""
from __future__ import annotations

import os

if "LOCAL_RANK" in os.environ and "CUDA_VISIBLE_DEVICES" not in os.environ:
    os.environ["CUDA_VISIBLE_DEVICES"] = os.environ["LOCAL_RANK"]

import argparse
import json
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "lammps-mlip-package_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

from mlipg import replicas  # noqa: E402

METRIC = "atom-steps/s E+F, mixed vs FP64 at force RMS err≤1e-4 eV/Å; p99 latency"
UNIT = "atom-steps/s"

WORKLOADS = {
    "fcc-ternary-1m": dict(lattice="fcc", n=64, a=4.0, ntypes=3, jitter=0.1,
                           pot="fcc-ternary-1m"),
    "bcc-binary-16k": dict(lattice="bcc", n=20, a=3.2, ntypes=2, jitter=0.05,
                           pot="bcc-binary-16k"),
    "fcc-al-256": dict(lattice="fcc", n=4, a=4.05, ntypes=1, jitter=0.05, pot="fcc-al-256"),
    # 4096 random triclinic cells, 8..512 atoms (log-uniform), one persistent launch
    "triclinic-batch-4096": dict(kind="batch", cells=4096, lo=8, hi=512, density=0.06,
                                 ntypes=2, pot="triclinic-batch"),
    # Poisson stream of requests (16..8192 atoms, FP64/mixed 50/50) at 80% of capacity
    "serve-poisson": dict(kind="serve", requests=20000, lo=16, hi=8192, density=0.06,
                          ntypes=2, pot="triclinic-batch", load=0.8, budget=64 << 30),
    # 256-atom fcc Al at 300 K (run it with --steps 100: 100 NVE steps, dt 1 fs), each
    # step a CUDA graph
    "md-fcc-al-256": dict(kind="md", lattice="fcc", n=4, a=4.05, ntypes=1, jitter=0.05,
                          pot="fcc-al-256", temperature=300.0, dt=0.001),
    # 16,000-atom binary bcc at 300 K (run it with --steps 100): the same NVE run in
    # mixed and in FP64 precision, each step a CUDA graph
    "md-bcc-binary-16k": dict(kind="md", lattice="bcc", n=20, a=3.2, ntypes=2, jitter=0.05,
                              pot="bcc-binary-16k", temperature=300.0, dt=0.001, fp64=True),
    # 50 NVE steps of the 1M-atom ternary alloy at 300 K, each step a CUDA graph
    "md-fcc-ternary-1m": dict(kind="md", lattice="fcc", n=64, a=4.0, ntypes=3, jitter=0.1,
                              pot="fcc-ternary-1m", temperature=300.0, dt=0.001),
}
POT_DESC = {
    "fcc-ternary-1m": "3 elements, rc 6, 15 Gaussians, gtinv order 4 l<=[12,8,4], "
                      "model_type 3 max_p 2, 68535 coefficients ~N(0,1e-3)",
    "bcc-binary-16k": "2 elements, rc 6, 15 Gaussians, gtinv order 4 l<=[12,8,4], "
                      "model_type 3 max_p 2, 14340 coefficients ~N(0,1e-3)",
    "fcc-al-256": "1 element, rc 6, 10 Gaussians, gtinv order 3 l<=[4,4], model_type 2 "
                  "max_p 2, 20300 coefficients ~N(0,1e-3)",
    "triclinic-batch": "2 elements, rc 6, 15 Gaussians, gtinv order 3 l<=[12,8], "
                       "model_type 3 max_p 2, 11805 coefficients ~N(0,1e-3)",
}
SKIN = 1.0
PRECISIONS = {"mixed": 1, "fp64": 0, "mixed_a64": 2, "fp64_native": 3}   # mlipg.PREC_* values
PRECISION_DESC = ("mixed (MLIPG_PREC_MIXED): FP32 radial functions, Y_lm, invariant and adjoint "
                  "products; order-parameter neighbour sums in Kahan-compensated FP32 (the "
                  "mixed_a64 record times the same kernel with plain FP64 sums); the "
                  "polynomial's input features and their energy, forces, per-atom and total "
                  "energies and the virial in FP64")
GOLDEN = os.path.join(REPO, "tests", "golden")
SOLO = {"rank": 0, "world": 1}   # rank 0's own sub-records (no collectives)


def make_cell(spec, n=None, seed=1):
    from mlipg.structures import bcc_cell, fcc_cell, jitter, random_types
    rng = np.random.default_rng(seed)
    n = n or spec["n"]
    cell = (fcc_cell if spec["lattice"] == "fcc" else bcc_cell)(n, n, n, spec["a"])
    cell = jitter(cell, spec["jitter"], rng)
    if spec["ntypes"] > 1:
        cell = random_types(cell, spec["ntypes"], rng)
    return cell


class ClockSampler:
    """nvidia-smi samples (200 ms) of SM clock and throttle reasons."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thr = threading.Thread(target=self._read, daemon=True)
            self.thr.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([v.strip() for v in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm = [float(r[0]) for r in self.rows if len(r) >= 7 and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) >= 7 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows if len(r) >= 7
                          for k in range(4) if r[3 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(sm)}


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_baseline(pot_path, sysm, seconds=15.0, seed=0):
    """Times the CPU oracle (all host threads) on a random sample of centres."""
    from oracle import Oracle
    nth = host_threads()
    o = Oracle(pot_path, threads=nth)
    rng = np.random.default_rng(seed)
    n = max(nth, 16)
    t = 0.0
    while True:
        centres = rng.choice(sysm.nlocal, size=min(n, sysm.nlocal), replace=False)
        t0 = time.perf_counter()
        o.compute_centers(sysm, centres)
        t = time.perf_counter() - t0
        if t >= seconds / 4 or n >= sysm.nlocal:
            break
        n = min(sysm.nlocal, int(n * max(2.0, 0.6 * seconds / max(t, 1e-3))))
    return {"value": len(centres) / t, "unit": UNIT, "cores": nth, "kind": "port",
            "sample": "%d random centre atoms of the %d-atom workload, one evaluation each "
                      "(energy, adjoint, pair forces; %.1f s)" % (len(centres), sysm.nlocal, t)}


def profiled_traffic(workload):
    """DRAM bytes (read + write) of one full launch of the fused kernel, from
    the ncu summary committed for this workload (`traffic_bytes_per_launch:`
    line)."""
    import re
    path = os.path.join(REPO, "profiles", "fused_kernel_%s.md" % workload)
    if not os.path.exists(path):
        return {"traffic": None}
    m = re.search(r"^traffic_bytes_per_launch:\s*(\d+)", open(path).read(), re.M)
    return {"traffic": int(m.group(1)) if m else None,
            "traffic_source": os.path.relpath(path, REPO)}


def mean_neighbours_in_cutoff(sysm, rc):
    d = sysm.x[sysm.nbr_idx] - np.repeat(sysm.x[:sysm.nlocal], np.diff(sysm.nbr_off), axis=0)
    inside = np.einsum("ij,ij->i", d, d) <= rc * rc
    per = np.add.reduceat(inside.astype(np.int64), sysm.nbr_off[:-1]) \
        if sysm.npairs else np.zeros(sysm.nlocal)
    out = {}
    for t in np.unique(sysm.type[:sysm.nlocal]):
        out[int(t)] = (int(np.sum(sysm.type[:sysm.nlocal] == t)),
                       float(per[sysm.type[:sysm.nlocal] == t].mean()))
    return out


def run_reference(args, dist):
    """--impl reference: the CPU implementation of the path on the host cores."""
    import mlipg
    from mlipg.potential import workload_potential
    if dist["rank"] != 0:
        return
    spec = WORKLOADS[args.workload]
    if spec.get("kind") in ("batch", "serve"):
        return run_reference_cells(args, dist, spec)
    with tempfile.TemporaryDirectory() as d:
        pot = os.path.join(d, "pot.mlip")
        workload_potential(pot, spec["pot"])
        cell = make_cell(spec)
        sysm = mlipg.native_system(cell, 6.0, SKIN)
        from oracle import Oracle
        nth = host_threads()
        o = Oracle(pot, threads=nth)
        rng = np.random.default_rng(123)
        # size each step's sample to a few seconds of CPU work
        probe = rng.choice(sysm.nlocal, size=nth, replace=False)
        t0 = time.perf_counter()
        o.compute_centers(sysm, probe)
        tp = time.perf_counter() - t0
        per_step = int(min(sysm.nlocal, max(nth, nth * 8.0 / max(tp, 1e-3))))
        for _ in range(args.warmup):
            o.compute_centers(sysm, rng.choice(sysm.nlocal, size=nth, replace=False))
        t0 = time.perf_counter()
        for _ in range(args.steps):
            o.compute_centers(sysm, rng.choice(sysm.nlocal, size=per_step, replace=False))
        el = time.perf_counter() - t0
        v = per_step * args.steps / el
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT,
                "n_gpus": dist["world"], "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": el / args.steps * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": args.workload, "atoms": sysm.nlocal,
                           "potential": POT_DESC[spec["pot"]],
                           "sample_per_step": per_step},
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": nth, "kind": "port",
                                 "sample": "%d random centres per step of the %d-atom workload"
                                           % (per_step, sysm.nlocal)},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)


def run_reference_cells(args, dist, spec):
    """--impl reference for the many-cell workloads: the CPU implementation on
    whole cells drawn from the workload, each step a bounded time slice."""
    from mlipg.potential import workload_potential
    with tempfile.TemporaryDirectory() as d:
        pot = os.path.join(d, "pot.mlip")
        workload_potential(pot, spec["pot"])
        n = 256 if spec["kind"] == "batch" else 64
        cells = triclinic_cells(n, spec["lo"], spec["hi"], spec["density"], spec["ntypes"],
                                seed=7 if spec["kind"] == "batch" else 17)
        per_step = max(1.0, min(8.0, 90.0 / max(args.steps + args.warmup, 1)))
        for w in range(args.warmup):
            cpu_baseline_cells(pot, cells, 0.5, seed=100 + w)
        vals = [cpu_baseline_cells(pot, cells, per_step, seed=w) for w in range(args.steps)]
        atoms_per_s = float(np.mean([v["value"] for v in vals]))
        line = {"impl": "reference", "metric": METRIC, "value": atoms_per_s, "unit": UNIT,
                "n_gpus": dist["world"], "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": per_step * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": args.workload, "potential": POT_DESC[spec["pot"]],
                           "sample_per_step": "%.1f s of whole cells" % per_step},
                "cpu_baseline": dict(vals[0], value=atoms_per_s),
                "e2e": {"value": atoms_per_s, "unit": UNIT, "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)


def run_ours(args, dist):
    import torch

    import mlipg
    from mlipg.potential import workload_potential

    spec = WORKLOADS[args.workload]
    rank = dist["rank"]
    tmp = tempfile.mkdtemp()
    pot = os.path.join(tmp, "pot.mlip")
    workload_potential(pot, spec["pot"])
    cell = make_cell(spec, seed=1 + rank)
    rc = 6.0
    sysm = mlipg.native_system(cell, rc, SKIN)
    natoms = sysm.nlocal
    nbar = mean_neighbours_in_cutoff(sysm, rc)

    # CPU baseline first (before the GPU is touched), rank 0 only
    cpu = cpu_baseline(pot, sysm, seconds=args.cpu_seconds) \
        if rank == 0 and args.cpu_seconds > 0 else None

    dev = torch.device("cuda", 0)
    g = mlipg.Potential(pot, PRECISIONS[args.precision])
    stream = torch.cuda.ExternalStream(g.stream(), device=dev)
    x4 = np.zeros((sysm.nall, 4))
    x4[:, :3] = sysm.x
    x4[:, 3] = sysm.type
    d_x4 = torch.from_numpy(x4).to(dev)
    d_cent = torch.arange(natoms, dtype=torch.int32, device=dev)
    d_off = torch.from_numpy(sysm.nbr_off).to(dev)
    d_idx = torch.from_numpy(sysm.nbr_idx).to(dev)
    d_f = torch.zeros((sysm.nall, 3), dtype=torch.float64, device=dev)
    d_out = torch.zeros(8, dtype=torch.float64, device=dev)
    d_eat = torch.zeros(natoms, dtype=torch.float64, device=dev)
    nb_cap = int(np.diff(sysm.nbr_off).max())
    torch.cuda.synchronize()

    ncent_main = min(natoms, args.centres) if args.centres > 0 else natoms
    tune = None
    if args.tiling:
        g.set_tiling(*[int(v) for v in args.tiling.split(",")])
        tune = {"table": None, "picked": g.tiling()}
    if args.autotune:
        tune = {"table": g.autotune_device(natoms, d_x4.data_ptr(), d_cent.data_ptr(),
                                           d_off.data_ptr(), d_idx.data_ptr(), d_f.data_ptr(),
                                           d_out.data_ptr(), nb_cap=nb_cap),
                "picked": g.tiling()}

    def step(ncent=None):
        ncent = ncent_main if ncent is None else ncent
        with torch.cuda.stream(stream):
            d_f.zero_()
        g.compute_device(ncent, d_x4.data_ptr(), d_cent.data_ptr(), d_off.data_ptr(),
                         d_idx.data_ptr(), d_f.data_ptr(), d_out.data_ptr(),
                         eatom=d_eat.data_ptr(), nb_cap=nb_cap)

    def barrier():
        replicas.barrier(dist)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    g.kernel_times()
    g.set_profiling(True)
    clocks = ClockSampler(0)
    clocks.start()
    barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        step()
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    g.set_profiling(False)
    el_ms = ev0.elapsed_time(ev1)
    ktimes = g.kernel_times()
    phases = g.phase_cycles()
    ptot = max(sum(phases.values()), 1)
    phase_share = {k: round(v / ptot, 4) for k, v in phases.items()}
    el_max = el_ms
    el_max = replicas.max_over_ranks(el_ms, dist)
    value = ncent_main * args.steps * dist["world"] / (el_max * 1e-3)
    e_mixed = float(d_out[0].item())
    if args.device_only:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "partial": True,
                              "config": {"workload": args.workload, "centres": ncent_main,
                                         "precision": args.precision},
                              "kernel_ms_per_launch": ktimes, "phase_share": phase_share,
                              "clocks": clk}), flush=True)
        g.close()
        return

    # ---------------- e2e through the LAMMPS-shaped C ABI (host arrays)
    off = sysm.nbr_off
    lists = [sysm.nbr_idx[off[i]:off[i + 1]] for i in range(natoms)]
    numneigh = np.diff(off).astype(np.int32)
    ilist = np.arange(natoms, dtype=np.int32)
    ltype = (sysm.type + 1).astype(np.int32)
    import ctypes
    fp = (ctypes.POINTER(ctypes.c_int) * natoms)()
    for i, a in enumerate(lists):
        fp[i] = a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    xh = np.ascontiguousarray(sysm.x)
    fh = np.zeros((sysm.nall, 3))
    e = ctypes.c_double()
    vir = np.zeros(6)
    L = mlipg.lib()
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    ip = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))

    def e2e_step():
        fh[:] = 0.0
        rcode = L.mlipg_compute(g.h, natoms, sysm.nall, dp(xh), ip(ltype), natoms, ip(ilist),
                                ip(numneigh), fp, 1, 1, dp(fh), ctypes.byref(e), dp(vir), None,
                                None)
        if rcode != 0:
            raise RuntimeError(L.mlipg_last_error(g.h).decode())

    e2e_step()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e2e_el = time.perf_counter() - t0
    e2e_el = replicas.max_over_ranks(e2e_el, dist)
    e2e = {"value": natoms * args.steps * dist["world"] / e2e_el, "unit": UNIT,
           "h2d_bytes_per_step": int(32 * sysm.nall + 4 * natoms + 4 * (natoms + 1) +
                                     4 * sysm.npairs),
           "d2h_bytes_per_step": int(24 * sysm.nall + 8 * 8 + 4),
           "api": "mlipg_compute (LAMMPS-shaped host arrays)"}

    # ---------------- FP64 (MLIPG_PREC_FP64: the invariant/adjoint products in
    # double-float arithmetic) on all centres, and the all-FP64 form
    # (MLIPG_PREC_FP64_NATIVE) on a bounded subset of them, with their own
    # tile shape (autotuned for FP64 unless one is fixed)
    mixed_tiling = g.tiling()
    g.set_precision(mlipg.PREC_FP64)
    fp64_tiling = None
    if args.autotune:
        g.autotune_device(min(ncent_main, 9728), d_x4.data_ptr(), d_cent.data_ptr(),
                          d_off.data_ptr(), d_idx.data_ptr(), d_f.data_ptr(), d_out.data_ptr(),
                          nb_cap=nb_cap)
        fp64_tiling = g.tiling()

    def timed_launches(ncent, n):
        step(ncent)
        torch.cuda.synchronize()
        g.kernel_times()
        g.set_profiling(True)
        ck = ClockSampler(0)
        ck.start()
        ev0.record(stream)
        for _ in range(n):
            step(ncent)
        ev1.record(stream)
        torch.cuda.synchronize()
        c = ck.stop()
        g.set_profiling(False)
        kt_ = [t for t in g.kernel_times() if t > 0]
        return ncent * n / (ev0.elapsed_time(ev1) * 1e-3), c, float(np.mean(kt_)) if kt_ else None

    fp64_v, clk64, kms64 = timed_launches(ncent_main, 2)
    e_fp64 = float(d_out[0].item())
    g.set_precision(mlipg.PREC_FP64_NATIVE)
    # a bounded subset (at least 1,024 centres when there are that many; never
    # more centres than the workload has)
    nsub = min(ncent_main, max(1024, int(ncent_main * args.fp64_fraction)))
    nat_v, clk_nat, kms_nat = timed_launches(nsub, 2)
    g.set_precision(mlipg.PREC_MIXED)
    g.set_tiling(mixed_tiling["irr_chunk"], mixed_tiling["warp_order"],
                 mixed_tiling["ctas_per_sm"])

    # ---------------- the mixed form with plain FP64 order-parameter sums
    # (MLIPG_PREC_MIXED_A64), same tile shape, 2 launches over all centres
    g.set_precision(mlipg.PREC_MIXED_A64)
    step()
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(2):
        step()
    ev1.record(stream)
    torch.cuda.synchronize()
    a64_v = ncent_main * 2 * dist["world"] / (replicas.max_over_ranks(ev0.elapsed_time(ev1), dist)
                                              * 1e-3)
    g.set_precision(mlipg.PREC_MIXED)

    # ---------------- accuracy of mixed vs FP64 on a 4,000-atom cell
    small = mlipg.native_system(make_cell(spec, n=10 if spec["lattice"] == "fcc" else 13,
                                          seed=11), rc, SKIN)
    g.set_precision(mlipg.PREC_FP64)
    r64 = g.compute(small)
    g.set_precision(mlipg.PREC_MIXED)
    r32 = g.compute(small)
    F64, F32 = small.fold_forces(r64["f_all"]), small.fold_forces(r32["f_all"])
    acc = {"atoms": small.nlocal,
           "force_rms_err_eV_per_A": float(np.sqrt(np.mean((F32 - F64) ** 2))),
           "force_rms_eV_per_A": float(np.sqrt(np.mean(F64 ** 2))),
           "energy_err_eV_per_atom": abs(r32["energy"] - r64["energy"]) / small.nlocal,
           "virial_rel_err": float(np.abs(r32["virial"] - r64["virial"]).max() /
                                   max(np.abs(r64["virial"]).max(), 1e-300))}
    g.set_precision(mlipg.PREC_MIXED_A64)
    ra = g.compute(small)
    g.set_precision(mlipg.PREC_MIXED)
    Fa = small.fold_forces(ra["f_all"])
    acc_a64 = {"force_rms_err_eV_per_A": float(np.sqrt(np.mean((Fa - F64) ** 2))),
               "energy_err_eV_per_atom": abs(ra["energy"] - r64["energy"]) / small.nlocal}
    acc_fitted = fitted_accuracy() if rank == 0 else None

    # ---------------- roofline of the fused kernel
    flops = sum(cnt * g.flops_per_atom_step(t, nb) for t, (cnt, nb) in nbar.items())
    kt = [t for t in ktimes if t > 0]
    kmean = float(np.mean(kt)) if kt else float("nan")
    peak = mlipg.measure_fma_peak(False)
    achieved = flops / (kmean * 1e-3) / 1e12
    roof = {"bound": "fp32-cuda-core", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "traffic": None,
            "peak_source": "live FP32 FMA microkernel on this GPU (mlipg_measure_fma_peak); "
                           "the machine's measured peaks cover HBM copy and bf16 tensor only",
            "kernel": "fused_kernel<12> (mixed)", "kernel_ms": kmean,
            "algorithmic_flops_per_launch": flops,
            "flops_per_atom": flops / natoms,
            # positions+element, centre, CSR offsets and indices read; forces written
            "algorithmic_bytes_per_launch": int(32 * sysm.nall + 8 * natoms + 4 * sysm.npairs +
                                                24 * sysm.nall)}
    # the kernels run the folded table (each conjugate pair of terms once):
    # the same FLOP model on it, and the FP32 pipe's arithmetic rate
    # (SMs x 128 lanes x 2 FLOP x the SM clock seen during the timed launches)
    flops_exec = sum(cnt * g.flops_per_atom_step(t, nb, executed=True)
                     for t, (cnt, nb) in nbar.items())
    nsm = torch.cuda.get_device_properties(0).multi_processor_count
    arith = nsm * 128 * 2 * (clk.get("sm_mhz") or 0) * 1e6 / 1e12
    ach_exec = flops_exec / (kmean * 1e-3) / 1e12
    roof.update({"executed_flops_per_launch": flops_exec,
                 "achieved_executed": ach_exec, "frac_executed": ach_exec / peak,
                 "arith_peak_fp32": arith,
                 "frac_arith": achieved / arith if arith > 0 else None,
                 "frac_executed_arith": ach_exec / arith if arith > 0 else None})
    roof.update(profiled_traffic(args.workload))

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist["world"],
                "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": el_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic",
                "config": {"workload": args.workload, "atoms_per_gpu": natoms,
                           "potential": POT_DESC[spec["pot"]],
                           "precision": PRECISION_DESC,
                           "neighbours_in_cutoff_per_atom":
                               {str(k): v[1] for k, v in nbar.items()},
                           "neighbour_list": "full, rc+%.1f A skin, %d pairs (%.0f MB)"
                                             % (SKIN, sysm.npairs, sysm.npairs * 4 / 1e6),
                           "l2": "inputs larger than L2 (positions + neighbour list %.0f MB)"
                                 % ((32 * sysm.nall + 4 * sysm.npairs) / 1e6),
                           "step": "energy + forces + virial of all atoms, one fused launch",
                           "tiling": tune},
                "e2e": e2e,
                "fp64": {"value": fp64_v, "unit": UNIT, "centres": ncent_main,
                         "what": "MLIPG_PREC_FP64: FP64 order parameters, polynomial, forces; "
                                 "invariant/adjoint products in double-float arithmetic, "
                                 "adjoint in exact fixed point",
                         "kernel_ms": kms64, "energy_eV": e_fp64, "tiling": fp64_tiling,
                         "mixed_over_fp64": value / dist["world"] / fp64_v, "clocks": clk64},
                "fp64_native": {"value": nat_v, "unit": UNIT, "centres": nsub,
                                "what": "MLIPG_PREC_FP64_NATIVE: every product and sum in FP64",
                                "kernel_ms": kms_nat,
                                "fp64_over_native": fp64_v / nat_v, "clocks": clk_nat},
                "mixed_a64": {"value": a64_v, "unit": UNIT,
                              "what": "MLIPG_PREC_MIXED_A64: order-parameter sums in plain FP64",
                              "accuracy_vs_fp64": acc_a64},
                "accuracy_mixed_vs_fp64": acc,
                "accuracy_fitted_potentials": acc_fitted,
                "energy_eV": e_mixed,
                "roofline": roof, "cpu_baseline": cpu, "clocks": clk,
                "gpu_launches": 2 * args.steps,
                "kernel_ms_per_launch": kt, "phase_share": phase_share}
    g.close()
    if rank == 0 and not args.no_sub_records:
        # short records of the batched-cell and serving configurations, so that
        # their rates and latencies are measured in every default run
        sub = argparse.Namespace(**vars(args))
        sub.cpu_seconds = 0.0
        sub.steps, sub.warmup = 3, 1
        line["batch_4096"] = batch_record(sub, SOLO, "triclinic-batch-4096")
        sub.requests = 2000
        line["serving"] = serve_record(sub, SOLO, "serve-poisson")
        # the NVE configurations: 100 steps of the 256-atom cell, and 100 steps
        # of the 16K binary in mixed and FP64
        sub.steps, sub.warmup = 100, 3
        line["md_256"] = md_record(sub, SOLO, "md-fcc-al-256")
        line["md_16k"] = md_record(sub, SOLO, "md-bcc-binary-16k")
    if rank == 0:
        print(json.dumps(line), flush=True)


def fitted_accuracy():
    """Mixed (and mixed_a64) against the FP64 path (itself within 1e-10 of the
    oracle) on the reference's fitted regression potentials and their 32-atom
    TiAl3 cell: energy error per atom, relative energy error, force RMS error."""
    import gzip
    import shutil

    import mlipg
    from mlipg.structures import read_lammps_data
    out = {}
    cell = read_lammps_data(os.path.join(GOLDEN, "structure.lammps"))
    with tempfile.TemporaryDirectory() as d:
        for name in ("gtinv-197", "gtinv-820", "gtinv-434"):
            pot = os.path.join(d, name + ".mlip")
            with gzip.open(os.path.join(GOLDEN, name + ".mlip.gz"), "rb") as fi, \
                    open(pot, "wb") as fo:
                shutil.copyfileobj(fi, fo)
            g = mlipg.Potential(pot, mlipg.PREC_FP64)
            s = mlipg.native_system(cell, g.cutoff, 2.0)
            r64 = g.compute(s)
            F64 = s.fold_forces(r64["f_all"])
            rec = {"atoms": s.nlocal, "energy_eV": r64["energy"]}
            for key, prec in (("mixed", mlipg.PREC_MIXED), ("mixed_a64", mlipg.PREC_MIXED_A64)):
                g.set_precision(prec)
                r = g.compute(s)
                F = s.fold_forces(r["f_all"])
                rec[key] = {"energy_err_eV_per_atom": abs(r["energy"] - r64["energy"]) / s.nlocal,
                            "energy_rel_err": abs(r["energy"] - r64["energy"]) /
                                              abs(r64["energy"]),
                            "force_rms_err_eV_per_A": float(np.sqrt(np.mean((F - F64) ** 2)))}
            g.close()
            out[name] = rec
    return out


# ---------------------------------------------------------------- other configurations

def triclinic_cells(count, lo, hi, density, ntypes, seed):
    """`count` random triclinic cells, atom counts log-uniform in [lo, hi]."""
    from mlipg.structures import random_triclinic_cell
    rng = np.random.default_rng(seed)
    sizes = np.minimum(hi, np.exp(rng.uniform(np.log(lo), np.log(hi + 1), count)).astype(int))
    return [random_triclinic_cell(int(k), density, ntypes, rng) for k in sizes]


def cpu_baseline_cells(pot_path, cells, seconds, seed=0):
    """CPU oracle (all host threads) on whole cells drawn at random from `cells`."""
    import mlipg
    from oracle import Oracle
    nth = host_threads()
    o = Oracle(pot_path, threads=nth)
    rng = np.random.default_rng(seed)
    atoms, t, ncell = 0, 0.0, 0
    for k in rng.permutation(len(cells)):
        sysm = mlipg.native_system(cells[k], 6.0, 0.0)
        t0 = time.perf_counter()
        o.compute(sysm)
        t += time.perf_counter() - t0
        atoms += sysm.nlocal
        ncell += 1
        if t >= seconds:
            break
    return {"value": atoms / t, "unit": UNIT, "cores": nth, "kind": "port",
            "sample": "%d whole cells (%d atoms) of the workload, one evaluation each "
                      "(%.1f s)" % (ncell, atoms, t)}


def type_flops(g, cells_types, nb_mean):
    t = np.concatenate(cells_types)
    return sum(int(np.sum(t == k)) * g.flops_per_atom_step(int(k), nb_mean) for k in np.unique(t))


def run_batch(args, dist):
    line = batch_record(args, dist, args.workload)
    if line is not None:
        print(json.dumps(line), flush=True)


def batch_record(args, dist, workload):
    """Every cell of the batch evaluated (energy, forces, stress) in one launch."""
    import torch

    import mlipg
    from mlipg.potential import workload_potential
    spec = WORKLOADS[workload]
    rank = dist["rank"]
    tmp = tempfile.mkdtemp()
    pot = os.path.join(tmp, "pot.mlip")
    workload_potential(pot, spec["pot"])
    cells = triclinic_cells(spec["cells"], spec["lo"], spec["hi"], spec["density"],
                            spec["ntypes"], seed=7 + rank)
    natoms = sum(c.natoms for c in cells)
    cpu = cpu_baseline_cells(pot, cells, args.cpu_seconds) \
        if rank == 0 and args.cpu_seconds > 0 else None
    dev = torch.device("cuda", 0)
    res, rates, kms, create_s, tune = {}, {}, {}, {}, {}
    clk = None
    for prec in (mlipg.PREC_FP64, mlipg.PREC_MIXED):
        g = mlipg.Potential(pot, prec)
        stream = torch.cuda.ExternalStream(g.stream(), device=dev)
        t0 = time.perf_counter()
        b = mlipg.Batch(g, cells)
        create_s[prec] = time.perf_counter() - t0
        tune[prec] = {"table": b.autotune(), "picked": g.tiling()} if args.autotune else None
        for _ in range(args.warmup):
            b.launch()
        torch.cuda.synchronize()
        g.kernel_times()
        g.set_profiling(True)
        clocks = ClockSampler(0)
        clocks.start()
        torch.cuda.synchronize()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(args.steps):
            b.launch()
        ev1.record(stream)
        torch.cuda.synchronize()
        c = clocks.stop()
        g.set_profiling(False)
        el = ev0.elapsed_time(ev1)
        el = replicas.max_over_ranks(el, dist)
        rates[prec] = natoms * args.steps * dist["world"] / (el * 1e-3)
        kt = [t for t in g.kernel_times() if t > 0]
        kms[prec] = float(np.mean(kt)) if kt else float("nan")
        res[prec] = b.compute()
        npairs = b.npairs
        if prec == mlipg.PREC_MIXED:
            clk = c
            el_mixed = el
            # e2e: the public batch API from host cells each step (neighbour
            # lists, upload, launch, results back)
            t0 = time.perf_counter()
            ne2e = max(1, min(args.steps, 3))
            for _ in range(ne2e):
                bb = mlipg.Batch(g, cells)
                bb.compute()
                bb.close()
            e2e_s = (time.perf_counter() - t0) / ne2e
            nb_mean = npairs / natoms
            flops = type_flops(g, [c.types for c in cells], nb_mean)
            peak = mlipg.measure_fma_peak(False)
            ach = flops / (kms[prec] * 1e-3) / 1e12
            roof = {"bound": "fp32-cuda-core", "achieved": ach, "peak": peak,
                    "unit": "TFLOP/s", "frac": ach / peak, "traffic": None,
                    "peak_source": "live FP32 FMA microkernel on this GPU",
                    "kernel": "fused kernel (mixed), all cells", "kernel_ms": kms[prec],
                    "algorithmic_flops_per_launch": flops}
        b.close()
        g.close()
    e64, f64, v64 = res[mlipg.PREC_FP64]
    e32, f32, v32 = res[mlipg.PREC_MIXED]
    n = np.array([c.natoms for c in cells])
    acc = {"force_rms_err_eV_per_A": float(np.sqrt(np.mean((f32 - f64) ** 2))),
           "force_rms_eV_per_A": float(np.sqrt(np.mean(f64 ** 2))),
           "energy_err_eV_per_atom_max": float(np.max(np.abs(e32 - e64) / n)),
           "virial_err_max_eV": float(np.abs(v32 - v64).max())}
    if rank == 0:
        # device-resident inputs of a launch: positions+element, centres, list
        # offsets, list entries and image codes, cell lattices and ids
        dev_in = natoms * (32 + 4 + 4) + 8 * npairs + len(cells) * (72 + 4)
        # per e2e step over the bus: positions+element, cell offsets and
        # lattices up; the list size (12 B), energies, forces and virials back
        h2d = natoms * 32 + (len(cells) + 1) * 4 + len(cells) * 72
        d2h = 12 + 24 * natoms + 56 * len(cells)
        line = {"metric": METRIC, "value": rates[mlipg.PREC_MIXED], "unit": UNIT,
                "n_gpus": dist["world"], "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": el_mixed / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": workload, "cells": len(cells), "atoms": natoms,
                           "atoms_per_cell": "log-uniform [%d, %d], mean %.1f"
                                             % (spec["lo"], spec["hi"], natoms / len(cells)),
                           "cells_desc": "random triclinic, angles U(60,120) deg, density "
                                         "0.06/A^3, 1.8 A minimum distance, 2 species",
                           "potential": POT_DESC[spec["pot"]],
                           "neighbours_per_atom": npairs / natoms,
                           "l2": "inputs larger than L2 (%.0f MB)" % (dev_in / 1e6),
                           "step": "one persistent launch over all cells + per-cell sums",
                           "tiling": {"mixed": tune[mlipg.PREC_MIXED],
                                      "fp64": tune[mlipg.PREC_FP64]}},
                "fp64": {"value": rates[mlipg.PREC_FP64], "unit": UNIT,
                         "kernel_ms": kms[mlipg.PREC_FP64],
                         "mixed_over_fp64": rates[mlipg.PREC_MIXED] / rates[mlipg.PREC_FP64]},
                "accuracy_mixed_vs_fp64": acc,
                "e2e": {"value": natoms * dist["world"] / e2e_s, "unit": UNIT,
                        "h2d_bytes_per_step": int(h2d),
                        "d2h_bytes_per_step": int(d2h),
                        "api": "mlipg_batch_create + mlipg_batch_compute from host cells "
                               "(positions up, neighbour lists built on the device each "
                               "step, results back)",
                        "host_setup_s": create_s[mlipg.PREC_MIXED]},
                "roofline": roof, "cpu_baseline": cpu, "clocks": clk,
                "gpu_launches": 3 * args.steps}
        return line
    return None


def run_serve(args, dist):
    line = serve_record(args, dist, args.workload)
    if line is not None:
        print(json.dumps(line), flush=True)


def serve_record(args, dist, workload):
    """Poisson request stream against the continuous-batching server."""
    import mlipg
    from mlipg.potential import workload_potential
    spec = WORKLOADS[workload]
    rank = dist["rank"]
    tmp = tempfile.mkdtemp()
    pot = os.path.join(tmp, "pot.mlip")
    workload_potential(pot, spec["pot"])
    nreq = args.requests or spec["requests"]
    pool = triclinic_cells(args.pool, spec["lo"], spec["hi"], spec["density"], spec["ntypes"],
                           seed=17 + rank)
    rng = np.random.default_rng(5 + rank)
    pick = rng.integers(0, len(pool), nreq)
    prec = np.where(rng.random(nreq) < 0.5, mlipg.PREC_FP64, mlipg.PREC_MIXED)
    cpu = cpu_baseline_cells(pot, pool, args.cpu_seconds) \
        if rank == 0 and args.cpu_seconds > 0 else None

    def burst(srv, idx):
        t0 = time.perf_counter()
        tk = [srv.submit(pool[pick[k]], int(prec[k])) for k in idx]
        for t in tk:
            srv.wait(t, 600000)
        return time.perf_counter() - t0

    # capacity: a closed burst of requests drawn like the stream
    srv = mlipg.Server(pot, budget_bytes=spec["budget"], max_batch_atoms=args.max_batch_atoms,
                       max_batch_atoms_fp64=args.max_batch_atoms_fp64)
    burst(srv, range(min(nreq, 4 * args.warmup)))
    ncap = min(nreq, max(200, nreq // 20))
    tcap = burst(srv, range(ncap))
    cap_atoms = sum(pool[pick[k]].natoms for k in range(ncap)) / tcap
    cap_req = ncap / tcap
    srv.close()

    # the stream: exponential inter-arrival gaps at `load` x capacity
    lam = spec["load"] * cap_req
    arrivals = np.cumsum(rng.exponential(1.0 / lam, nreq))
    srv = mlipg.Server(pot, budget_bytes=spec["budget"], max_batch_atoms=args.max_batch_atoms,
                       max_batch_atoms_fp64=args.max_batch_atoms_fp64)
    tickets = [None] * nreq
    clocks = ClockSampler(0)
    clocks.start()
    t0 = time.perf_counter()

    def submitter():
        for k in range(nreq):
            d = t0 + arrivals[k] - time.perf_counter()
            if d > 0:
                time.sleep(d)
            tickets[k] = srv.submit(pool[pick[k]], int(prec[k]))

    th = threading.Thread(target=submitter)
    th.start()
    for k in range(nreq):
        while tickets[k] is None:
            time.sleep(0.0005)
        srv.wait(tickets[k], 600000)
    el = time.perf_counter() - t0
    th.join()
    clk = clocks.stop()
    st = srv.stats()
    srv.close()
    atoms = int(sum(pool[pick[k]].natoms for k in range(nreq)))
    # roofline: algorithmic FLOPs of every served atom-step (counting rule of
    # the fused kernel, per element at the pool's mean neighbour count) over
    # the wall time of the stream, against the FP32 FMA peak (FP64 requests
    # run their invariant/adjoint products in double-float arithmetic on the
    # FP32 pipe, about 15 FP32 operations per FP64-class FMA, so their FLOPs
    # are also reported apart)
    g = mlipg.Potential(pot, mlipg.PREC_MIXED)
    nb_mean = 4.18879 * 6.0 ** 3 * spec["density"]
    fl = np.array([sum(int(np.sum(pool[pick[k]].types == t)) * g.flops_per_atom_step(int(t), nb_mean)
                       for t in range(spec["ntypes"])) for k in range(nreq)])
    g.close()
    peak = mlipg.measure_fma_peak(False)
    ach = fl.sum() / el / 1e12
    roof = {"bound": "fp32-cuda-core (mixed requests: FP32 products; FP64 requests: "
                     "double-float products)", "achieved": ach,
            "peak": peak, "unit": "TFLOP/s", "frac": ach / peak, "traffic": None,
            "fp64_share_of_flops": float(fl[prec == mlipg.PREC_FP64].sum() / fl.sum()),
            "note": "whole-stream average at %.0f%% offered load (the GPU idles between "
                    "arrivals)" % (100 * spec["load"])}
    if rank == 0:
        # per request over the bus: positions+element (32 B/atom), lattice and
        # cell offset up (lists are built on the device); forces, energy and
        # virial back
        h2d = atoms / nreq * 32 + 76
        line = {"metric": METRIC, "value": st["atom_steps_per_s"] * dist["world"], "unit": UNIT,
                "n_gpus": dist["world"], "steps": nreq, "warmup": args.warmup,
                "ms_per_step": el / nreq * 1e3, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64+f32", "data": "synthetic",
                "config": {"workload": workload, "requests": nreq,
                           "atoms_per_request": "log-uniform [%d, %d], mean %.0f"
                                                % (spec["lo"], spec["hi"], atoms / nreq),
                           "structures": "pool of %d random triclinic cells (density 0.06/A^3,"
                                         " 1.8 A minimum distance, 2 species), drawn at "
                                         "random per request" % len(pool),
                           "precision_mix": "FP64 / mixed 50/50 per request",
                           "potential": POT_DESC[spec["pot"]],
                           "budget_bytes": spec["budget"],
                           "max_batch_atoms": args.max_batch_atoms,
                           "max_batch_atoms_fp64": args.max_batch_atoms_fp64 or
                                                   min(8192, args.max_batch_atoms),
                           "offered_load": spec["load"],
                           "step": "one request (energy + forces + stress)"},
                "latency_ms": {"p50": st["p50_ms"], "p99": st["p99_ms"]},
                "capacity": {"atom_steps_per_s": cap_atoms, "requests_per_s": cap_req,
                             "burst_requests": ncap},
                "offered_requests_per_s": lam, "batches": st["batches"],
                "e2e": {"value": atoms / el, "unit": UNIT,
                        "h2d_bytes_per_step": int(h2d),
                        "d2h_bytes_per_step": int(24 * atoms / nreq + 56),
                        "api": "mlipg_server_submit / mlipg_server_wait with host arrays"},
                "roofline": roof, "cpu_baseline": cpu, "clocks": clk,
                "gpu_launches": int(3 * st["batches"])}
        return line
    return None


def run_md(args, dist):
    """NVE molecular dynamics (velocity Verlet), each step one CUDA graph."""
    line = md_record(args, dist, args.workload)
    if dist["rank"] == 0:
        print(json.dumps(line), flush=True)


def md_record(args, dist, workload):
    import torch

    import mlipg
    from mlipg.potential import workload_potential
    spec = WORKLOADS[workload]
    rank = dist["rank"]
    tmp = tempfile.mkdtemp()
    pot = os.path.join(tmp, "pot.mlip")
    workload_potential(pot, spec["pot"])
    cell = make_cell(spec, seed=1 + rank)
    g = mlipg.Potential(pot, mlipg.PREC_MIXED)
    masses = np.array(g.masses)[cell.types]
    v = mlipg.maxwell_boltzmann(masses, spec["temperature"], np.random.default_rng(3 + rank))
    t0 = time.perf_counter()
    md = mlipg.MD(g, cell, v, skin=SKIN)
    setup_s = time.perf_counter() - t0
    tune = {"table": md.autotune(), "picked": g.tiling()} if args.autotune else None
    md.run(args.warmup, spec["dt"], True)
    th0 = md.thermo()
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    t0 = time.perf_counter()
    md.run(args.steps, spec["dt"], True)
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    clk = clocks.stop()
    th1 = md.thermo()
    x_mixed = md.state()[0]
    el = replicas.max_over_ranks(el, dist)
    n = cell.natoms
    value = n * args.steps * dist["world"] / el
    fp64_rec = None
    if spec.get("fp64"):
        # the same run (cell, velocities, warm-up and timed steps) in FP64
        g64 = mlipg.Potential(pot, mlipg.PREC_FP64)
        md64 = mlipg.MD(g64, cell, v, skin=SKIN)
        md64.run(args.warmup, spec["dt"], True)
        th0_64 = md64.thermo()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        md64.run(args.steps, spec["dt"], True)
        torch.cuda.synchronize()
        el64 = replicas.max_over_ranks(time.perf_counter() - t0, dist)
        th1_64 = md64.thermo()
        d = x_mixed - md64.state()[0]
        fr = d @ np.linalg.inv(cell.lattice)
        d = (fr - np.round(fr)) @ cell.lattice     # minimum image
        md64.close()
        g64.close()
        v64 = n * args.steps * dist["world"] / el64
        fp64_rec = {"value": v64, "unit": UNIT, "ms_per_step": el64 / args.steps * 1e3,
                    "what": "MLIPG_PREC_FP64 (double-float invariant/adjoint products)",
                    "energy_drift_eV_per_atom": (th1_64["etotal"] - th0_64["etotal"]) / n,
                    "mixed_over_fp64": value / v64,
                    "mixed_vs_fp64_max_displacement_A": float(np.abs(d).max()),
                    "mixed_vs_fp64_pe_eV_per_atom": abs(th1["pe"] - th1_64["pe"]) / n}
    per_cell = 4 if spec["lattice"] == "fcc" else 2   # atoms per conventional cell
    nb = per_cell * 4.0 / 3.0 * np.pi * 6.0 ** 3 / spec["a"] ** 3
    flops = type_flops(g, [cell.types], nb)
    peak = mlipg.measure_fma_peak(False)
    ach = flops / (el / args.steps) / 1e12
    md.close()
    g.close()
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist["world"],
                "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": el / args.steps * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": workload, "atoms": n,
                           "potential": POT_DESC[spec["pot"]],
                           "md": "NVE velocity Verlet, dt %.3f ps, %g K Maxwell-Boltzmann, "
                                 "skin %.1f A, list rebuilt when an atom moves skin/2"
                                 % (spec["dt"], spec["temperature"], SKIN),
                           "step": "one CUDA graph per step (integrate, forces, integrate, "
                                   "displacement check)",
                           "tiling": tune},
                "thermo_start": th0, "thermo_end": th1,
                "energy_drift_eV_per_atom": (th1["etotal"] - th0["etotal"]) / n,
                "e2e": {"value": n * args.steps * dist["world"] / (el + setup_s), "unit": UNIT,
                        "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 8,
                        "api": "mlipg_md_create + mlipg_md_run (setup amortised over the run)"},
                "roofline": {"bound": "fp32-cuda-core", "achieved": ach, "peak": peak,
                             "unit": "TFLOP/s", "frac": ach / peak, "traffic": None,
                             "note": "whole MD step time (upper bound of the force kernel)"},
                "fp64": fp64_rec,
                "cpu_baseline": None, "clocks": clk,
                # per step one graph of 5 kernels (first half-kick, fused force kernel,
                # finalize, second half-kick, displacement check); list rebuilds
                # in the timed region add the device list builder's kernels
                "gpu_launches": 5 * args.steps,
                "graph_launches": args.steps,
                "list_rebuilds": int(th1["rebuilds"] - th0["rebuilds"])}
        return line
    return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="fcc-ternary-1m", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--fp64-fraction", type=float, default=1.0 / 8)
    ap.add_argument("--centres", type=int, default=0,
                    help="evaluate only the first N centres per step (profiling runs)")
    ap.add_argument("--device-only", action="store_true",
                    help="time the device-resident step only (no e2e/FP64/accuracy/CPU legs)")
    ap.add_argument("--requests", type=int, default=0,
                    help="serving: number of requests (default: the workload's)")
    ap.add_argument("--pool", type=int, default=256,
                    help="serving: distinct structures the requests are drawn from")
    ap.add_argument("--max-batch-atoms", type=int, default=65536)
    ap.add_argument("--max-batch-atoms-fp64", type=int, default=0,
                    help="serving: FP64 batch cap (0: the server's default)")
    ap.add_argument("--no-sub-records", action="store_true",
                    help="skip the short batch and serving records of the default run")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="keep the default tile shape instead of autotuning it")
    ap.add_argument("--tiling", default="",
                    help="fixed tile shape 'terms,order,ctas_per_sm' (implies --no-autotune)")
    ap.add_argument("--precision", default="mixed", choices=sorted(PRECISIONS),
                    help="precision of the device-only step (profiling runs; the full run "
                         "always reports mixed with its FP64 and mixed_a64 legs)")
    args = ap.parse_args()
    if args.tiling:
        args.autotune = False
    if args.precision != "mixed" and not args.device_only:
        ap.error("--precision applies to --device-only runs")
    dist = replicas.init("gloo")
    try:
        kind = WORKLOADS[args.workload].get("kind", "cell")
        if args.impl == "reference":
            run_reference(args, dist)
        elif kind == "batch":
            run_batch(args, dist)
        elif kind == "serve":
            run_serve(args, dist)
        elif kind == "md":
            run_md(args, dist)
        else:
            run_ours(args, dist)
    finally:
        replicas.finish(dist)


if __name__ == "__main__":
    main()
