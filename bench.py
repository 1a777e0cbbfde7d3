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
  fp64       the plain FP64 path on a bounded subset of centres of the same
             structure, and the mixed/FP64 speed ratio
  accuracy   mixed vs FP64 (GPU) on a 4,000-atom cell of the same workload
  roofline   algorithmic FLOPs per fused-kernel launch / its CUDA-event time,
             against the live FP32 FMA peak of the device
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

METRIC = "atom-steps/s E+F, mixed vs FP64 at force RMS err≤1e-4 eV/Å; p99 latency"
UNIT = "atom-steps/s"

WORKLOADS = {
    "fcc-ternary-1m": dict(lattice="fcc", n=64, a=4.0, ntypes=3, jitter=0.1,
                           pot="fcc-ternary-1m"),
    "bcc-binary-16k": dict(lattice="bcc", n=20, a=3.2, ntypes=2, jitter=0.05,
                           pot="bcc-binary-16k"),
    "fcc-al-256": dict(lattice="fcc", n=4, a=4.05, ntypes=1, jitter=0.05, pot="fcc-al-256"),
}
POT_DESC = {
    "fcc-ternary-1m": "3 elements, rc 6, 15 Gaussians, gtinv order 4 l<=[12,8,4], "
                      "model_type 3 max_p 2, 68535 coefficients ~N(0,1e-3)",
    "bcc-binary-16k": "2 elements, rc 6, 15 Gaussians, gtinv order 4 l<=[12,8,4], "
                      "model_type 3 max_p 2, 14340 coefficients ~N(0,1e-3)",
    "fcc-al-256": "1 element, rc 6, 10 Gaussians, gtinv order 3 l<=[4,4], model_type 2 "
                  "max_p 2, 20300 coefficients ~N(0,1e-3)",
}
SKIN = 1.0


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
                           "potential": POT_DESC[args.workload],
                           "sample_per_step": per_step},
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": nth, "kind": "port",
                                 "sample": "%d random centres per step of the %d-atom workload"
                                           % (per_step, sysm.nlocal)},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0,
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
    g = mlipg.Potential(pot, mlipg.PREC_MIXED)
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

    def step(ncent=None):
        ncent = ncent_main if ncent is None else ncent
        with torch.cuda.stream(stream):
            d_f.zero_()
        g.compute_device(ncent, d_x4.data_ptr(), d_cent.data_ptr(), d_off.data_ptr(),
                         d_idx.data_ptr(), d_f.data_ptr(), d_out.data_ptr(),
                         eatom=d_eat.data_ptr(), nb_cap=nb_cap)

    def barrier():
        if dist["world"] > 1:
            torch.distributed.barrier()

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
    if dist["world"] > 1:
        t = torch.tensor([el_ms], dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        el_max = float(t.item())
    value = ncent_main * args.steps * dist["world"] / (el_max * 1e-3)
    e_mixed = float(d_out[0].item())
    if args.device_only:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "partial": True,
                              "config": {"workload": args.workload, "centres": ncent_main},
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
    if dist["world"] > 1:
        t = torch.tensor([e2e_el], dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_el = float(t.item())
    e2e = {"value": natoms * args.steps * dist["world"] / e2e_el, "unit": UNIT,
           "h2d_bytes_per_step": int(32 * sysm.nall + 4 * natoms + 4 * (natoms + 1) +
                                     4 * sysm.npairs),
           "d2h_bytes_per_step": int(24 * sysm.nall + 8 * 8 + 4),
           "api": "mlipg_compute (LAMMPS-shaped host arrays)"}

    # ---------------- plain FP64 path on a bounded subset of centres
    g.set_precision(mlipg.PREC_FP64)
    nsub = max(1024, min(natoms, int(natoms * args.fp64_fraction)))
    step(nsub)
    torch.cuda.synchronize()
    ev0.record(stream)
    for _ in range(2):
        step(nsub)
    ev1.record(stream)
    torch.cuda.synchronize()
    fp64_v = nsub * 2 / (ev0.elapsed_time(ev1) * 1e-3)
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
            "flops_per_atom": flops / natoms}
    prof = os.path.join(REPO, "profiles", "traffic_" + args.workload + ".json")
    if os.path.exists(prof):
        with open(prof) as f:
            roof["traffic"] = json.load(f).get("dram_bytes_per_launch")

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist["world"],
                "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": el_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic",
                "config": {"workload": args.workload, "atoms_per_gpu": natoms,
                           "potential": POT_DESC[args.workload],
                           "precision": "mixed: FP32 radial/Y_lm/invariant/adjoint products, "
                                        "FP64 a_nlm sums, forces, energies, virial",
                           "neighbours_in_cutoff_per_atom":
                               {str(k): v[1] for k, v in nbar.items()},
                           "neighbour_list": "full, rc+%.1f A skin, %d pairs (%.0f MB)"
                                             % (SKIN, sysm.npairs, sysm.npairs * 4 / 1e6),
                           "l2": "inputs larger than L2 (positions + neighbour list %.0f MB)"
                                 % ((32 * sysm.nall + 4 * sysm.npairs) / 1e6),
                           "step": "energy + forces + virial of all atoms, one fused launch"},
                "e2e": e2e,
                "fp64": {"value": fp64_v, "unit": UNIT, "centres": nsub,
                         "mixed_over_fp64": value / dist["world"] / fp64_v},
                "accuracy_mixed_vs_fp64": acc,
                "energy_eV": e_mixed,
                "roofline": roof, "cpu_baseline": cpu, "clocks": clk,
                "gpu_launches": 2 * args.steps,
                "kernel_ms_per_launch": kt, "phase_share": phase_share}
        print(json.dumps(line), flush=True)
    g.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="fcc-ternary-1m", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--fp64-fraction", type=float, default=1.0 / 32)
    ap.add_argument("--centres", type=int, default=0,
                    help="evaluate only the first N centres per step (profiling runs)")
    ap.add_argument("--device-only", action="store_true",
                    help="time the device-resident step only (no e2e/FP64/accuracy/CPU legs)")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    dist = {"world": world, "rank": rank}
    if world > 1:
        import torch.distributed
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        torch.distributed.init_process_group("gloo")
    try:
        if args.impl == "reference":
            run_reference(args, dist)
        else:
            run_ours(args, dist)
    finally:
        if world > 1:
            import torch.distributed
            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
