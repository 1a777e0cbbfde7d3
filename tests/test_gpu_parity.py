"""GPU path (through the C ABI) against the CPU oracle and the golden logs.

Tolerances:
* FP64 precisions: energy, every force component and the virial agree with
  the oracle to 1e-10 relative (to the largest magnitude of each quantity).
  MLIPG_PREC_FP64_NATIVE differs from the oracle only in summation order;
  MLIPG_PREC_FP64 runs the invariant and adjoint products in double-float
  arithmetic (a few 2^-47 per operation) and agrees to ~1e-13.
* mixed path: force RMS error <= 1e-4 eV/A against the FP64 oracle on every
  potential.  Energy: the polynomial's input features and their whole
  energy (linear and polynomial terms) are evaluated in FP64, so a potential
  whose features all enter the polynomial (gtinv-197) matches to 1e-9
  eV/atom; the other, "linear-only", features are FP32 products of FP32
  order parameters (the stated precision split), whose error is a few FP32
  ulps of their conditioning C = sum_f |w_f| sum_terms |c| prod |a| (the
  oracle computes C per atom).  The bound is 1e-6 eV/atom plus 4 ulps
  (2^-22) of C: the synthetic workload potentials (C of order 1e-2 eV per
  atom) stay within 1e-6 eV/atom; the fitted regression potentials, whose
  linear terms reach C ~ 450-610 eV per atom against energies of -4.2 eV per
  atom, are bounded by about 1e-4 eV/atom and measure 1e-6 - 1e-5.
"""
import numpy as np
import pytest

import mlipg
from conftest import structure
from mlipg.potential import workload_potential
from mlipg.structures import (bcc_cell, build_system, fcc_cell, jitter, random_triclinic_cell,
                              random_types)
from oracle import Oracle

pytestmark = pytest.mark.gpu

REL = 1e-10


def rel_err(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def check_fp64(gpu, ref, sysm):
    assert abs(gpu["energy"] - ref["energy"]) <= REL * abs(ref["energy"])
    assert rel_err(gpu["f_all"], ref["f_all"]) <= REL
    assert rel_err(gpu["virial"], ref["virial"]) <= REL
    assert rel_err(gpu["eatom"], ref["eatom"]) <= REL
    assert rel_err(sysm.fold_forces(gpu["f_all"]), sysm.fold_forces(ref["f_all"])) <= REL


@pytest.fixture(scope="module")
def ref_cache():
    return {}


@pytest.mark.parametrize("prec", [mlipg.PREC_FP64, mlipg.PREC_FP64_NATIVE])
@pytest.mark.parametrize("pot", ["gtinv-197", "gtinv-820", "gtinv-434"])
def test_regression_potentials_fp64(potdir, golden, pot, prec):
    o = Oracle(potdir[pot], threads=16)
    s = build_system(structure("structure.lammps"), o.cutoff, skin=2.0)
    ref = o.compute(s)
    g = mlipg.Potential(potdir[pot], prec)
    got = g.compute(s)
    check_fp64(got, ref, s)
    gl = golden["thermo_step0"][pot]
    assert got["energy"] == pytest.approx(gl["E_pair"], abs=6e-6)
    assert s.pressure(got["virial"]) == pytest.approx(gl["Press"], abs=6e-4)


@pytest.mark.parametrize("pot", ["pair-60", "pair-17"])
def test_pair_descriptor(potdir, golden, pot):
    """Radial-only potentials (des_type pair, the reference's pair_style
    mlip_pair; pair-60 has 20 radial functions and a third-order polynomial
    of 22,910 terms): the FP64 kernel matches the oracle to 1e-10 and the
    reference's step-0 log; every precision runs that FP64 kernel."""
    o = Oracle(potdir[pot], threads=16)
    s = build_system(structure("structure.lammps"), o.cutoff, skin=2.0)
    ref = o.compute(s)
    gl = golden["thermo_step0"][pot]
    for prec in (mlipg.PREC_FP64, mlipg.PREC_MIXED):
        got = mlipg.Potential(potdir[pot], prec).compute(s, vatom=True)
        check_fp64(got, ref, s)
        assert got["energy"] == pytest.approx(gl["E_pair"], abs=6e-6)
        assert s.pressure(got["virial"]) == pytest.approx(gl["Press"], abs=6e-4)
        np.testing.assert_allclose(got["vatom"].sum(0), got["virial"], rtol=1e-12, atol=1e-12)


def test_stress_and_triclinic_fp64(potdir, golden):
    g = mlipg.Potential(potdir["gtinv-197"], mlipg.PREC_FP64)
    s = build_system(structure("structure.lammps"), g.cutoff, skin=2.0)
    p = s.pressure_tensor(g.compute(s)["virial"])
    gl = golden["thermo_step0"]["gtinv-197-stress"]
    np.testing.assert_allclose(p, [gl[k] for k in ["Pxx", "Pyy", "Pzz", "Pxy", "Pxz", "Pyz"]],
                               atol=2e-3, rtol=0)
    gc = golden["thermo_step0"]["gtinv-197-conv64"]
    for name in ["structure_00064_conventional.lammps", "structure_00064_triclinic.lammps"]:
        s = build_system(structure(name), g.cutoff, skin=2.0)
        r = g.compute(s)
        assert r["energy"] == pytest.approx(gc["E_pair"], abs=6e-6)
        assert s.pressure(r["virial"]) == pytest.approx(gc["Press"], abs=0.1)


def mixed_energy_bound(o, s):
    """1e-6 eV/atom plus 4 FP32 ulps of the linear-only terms' conditioning."""
    return 1e-6 * s.nlocal + 2.0 ** -22 * o.linear_conditioning(s).sum()


@pytest.mark.parametrize("prec", [mlipg.PREC_MIXED, mlipg.PREC_MIXED_A64])
@pytest.mark.parametrize("name", ["structure.lammps", "structure_00064_conventional.lammps"])
@pytest.mark.parametrize("pot", ["gtinv-197", "gtinv-820", "gtinv-434"])
def test_regression_potentials_mixed(potdir, pot, name, prec):
    o = Oracle(potdir[pot], threads=16)
    s = build_system(structure(name), o.cutoff, skin=2.0)
    ref = o.compute(s)
    got = mlipg.Potential(potdir[pot], prec).compute(s)
    F, Fr = s.fold_forces(got["f_all"]), s.fold_forces(ref["f_all"])
    assert np.sqrt(np.mean((F - Fr) ** 2)) <= 1e-4
    de = abs(got["energy"] - ref["energy"])
    cond = o.linear_conditioning(s)
    if cond.sum() == 0.0:
        # every feature enters the polynomial: all of the energy is FP64
        assert de / s.nlocal <= 1e-9
    assert de <= mixed_energy_bound(o, s)


def workload_system(name, rng):
    if name == "fcc-al-256":
        cell = jitter(fcc_cell(4, 4, 4, 4.05), 0.05, rng)
    elif name == "bcc-binary-16k":      # 3x3x3 bcc cell of the same alloy
        cell = random_types(jitter(bcc_cell(3, 3, 3, 3.2), 0.05, rng), 2, rng)
    elif name == "fcc-ternary-1m":      # 2x2x2 fcc cell of the same alloy
        cell = random_types(jitter(fcc_cell(2, 2, 2, 4.0), 0.1, rng), 3, rng)
    elif name == "triclinic-batch":
        cell = random_triclinic_cell(24, 0.06, 2, rng)
    return cell


@pytest.mark.parametrize("name", ["fcc-al-256", "bcc-binary-16k", "fcc-ternary-1m",
                                  "triclinic-batch"])
def test_workload_potentials(tmp_path, name):
    rng = np.random.default_rng(7)
    path = str(tmp_path / (name + ".mlip"))
    workload_potential(path, name, seed=3)
    cell = workload_system(name, rng)
    o = Oracle(path, threads=16)
    s = build_system(cell, o.cutoff, skin=1.0)
    ref = o.compute(s)
    got = mlipg.Potential(path, mlipg.PREC_FP64).compute(s)
    check_fp64(got, ref, s)
    mix = mlipg.Potential(path, mlipg.PREC_MIXED).compute(s)
    F, Fr = s.fold_forces(mix["f_all"]), s.fold_forces(ref["f_all"])
    assert np.sqrt(np.mean((F - Fr) ** 2)) <= 1e-4
    assert abs(mix["energy"] - ref["energy"]) / s.nlocal <= 1e-6
    assert abs(mix["energy"] - ref["energy"]) <= mixed_energy_bound(o, s)


HIGH_L = {
    # order-2 terms to l = 16 and order-3 terms to l = 10 (the table's limit),
    # two elements: the kernel's l <= 16 instantiation
    "l16": dict(elements=["A", "B"], maxl=16, gtinv_maxl=[16, 10]),
    # order-2 terms to l = 20 (the table's limit), one element: the l <= 20
    # instantiation (with two elements its FP64 form exceeds shared memory)
    "l20": dict(elements=["A"], maxl=20, gtinv_maxl=[20, 10]),
}


@pytest.mark.parametrize("spec", sorted(HIGH_L))
def test_high_l_potentials(tmp_path, spec):
    """Potentials with max_l 13-16 and 17-20 (the coupling table holds order-2
    terms to l = 20 and order-3 terms to l = 10): FP64 against the oracle at
    1e-10, mixed within the stated bounds."""
    from mlipg.potential import gaussian_params, write_potential
    h = HIGH_L[spec]
    path = str(tmp_path / (spec + ".mlip"))
    write_potential(path, h["elements"], 5.0, gaussian_params(6, 5.0), 3, 2, h["maxl"], 3,
                    h["gtinv_maxl"], [0, 0], masses=[27.0] * len(h["elements"]), seed=11)
    rng = np.random.default_rng(5)
    cell = jitter(fcc_cell(2, 2, 2, 3.6), 0.05, rng)
    if len(h["elements"]) > 1:
        cell = random_types(cell, len(h["elements"]), rng)
    o = Oracle(path, threads=16)
    s = build_system(cell, o.cutoff, skin=1.0)
    ref = o.compute(s)
    g = mlipg.Potential(path, mlipg.PREC_FP64)
    assert g.info["L"] == h["maxl"]
    check_fp64(g.compute(s), ref, s)
    mix = mlipg.Potential(path, mlipg.PREC_MIXED).compute(s)
    F, Fr = s.fold_forces(mix["f_all"]), s.fold_forces(ref["f_all"])
    assert np.sqrt(np.mean((F - Fr) ** 2)) <= 1e-4
    assert abs(mix["energy"] - ref["energy"]) <= mixed_energy_bound(o, s)


@pytest.mark.parametrize("name", ["fcc-ternary-1m", "fcc-al-256"])
def test_dense_neighbourhoods(tmp_path, name):
    """Compressed fcc (a = 3.3 A, about 100 neighbours inside 6 A): the mixed
    path stages the order-parameter sums in windows of 64 neighbours, so here
    every neighbourhood spans two windows and elements straddle the boundary."""
    rng = np.random.default_rng(11)
    path = str(tmp_path / (name + ".mlip"))
    workload_potential(path, name, seed=5)
    cell = jitter(fcc_cell(3, 3, 3, 3.3), 0.05, rng)
    o = Oracle(path, threads=16)
    if o.info["T"] > 1:
        cell = random_types(cell, o.info["T"], rng)
    s = build_system(cell, o.cutoff, skin=1.0)
    ref = o.compute(s)
    got = mlipg.Potential(path, mlipg.PREC_FP64).compute(s)
    check_fp64(got, ref, s)
    mix = mlipg.Potential(path, mlipg.PREC_MIXED).compute(s)
    F, Fr = s.fold_forces(mix["f_all"]), s.fold_forces(ref["f_all"])
    assert np.sqrt(np.mean((F - Fr) ** 2)) <= 1e-4
    assert abs(mix["energy"] - ref["energy"]) / s.nlocal <= 1e-6


@pytest.mark.parametrize("name", ["bcc-binary-16k", "fcc-ternary-1m", "triclinic-batch"])
def test_mixed_fp64_sums(tmp_path, name):
    """MLIPG_PREC_MIXED_A64 (order-parameter sums in plain FP64) meets the
    mixed bounds against the oracle, and the compensated FP32 sums of
    MLIPG_PREC_MIXED agree with it to far inside them."""
    rng = np.random.default_rng(7)
    path = str(tmp_path / (name + ".mlip"))
    workload_potential(path, name, seed=3)
    cell = workload_system(name, rng)
    o = Oracle(path, threads=16)
    s = build_system(cell, o.cutoff, skin=1.0)
    ref = o.compute(s)
    a64 = mlipg.Potential(path, mlipg.PREC_MIXED_A64).compute(s)
    mix = mlipg.Potential(path, mlipg.PREC_MIXED).compute(s)
    Fr = s.fold_forces(ref["f_all"])
    Fa, Fm = s.fold_forces(a64["f_all"]), s.fold_forces(mix["f_all"])
    assert np.sqrt(np.mean((Fa - Fr) ** 2)) <= 1e-4
    assert abs(a64["energy"] - ref["energy"]) / s.nlocal <= 1e-6
    assert np.sqrt(np.mean((Fm - Fa) ** 2)) <= 1e-6
    assert abs(mix["energy"] - a64["energy"]) / s.nlocal <= 1e-8


def test_edge_cases(potdir):
    g = mlipg.Potential(potdir["gtinv-820"], mlipg.PREC_FP64)
    o = Oracle(potdir["gtinv-820"])
    # empty system
    e, f, vir, ea = g.compute_lammps(0, 0, np.zeros((0, 3)), [], [], [], [])
    assert e == 0.0 and np.all(vir == 0)
    # isolated atoms (no neighbours inside the cutoff) and a NULL-mapped type
    cell = structure("structure.lammps")
    s = build_system(cell, g.cutoff, skin=2.0)
    g.set_type_map(["Ti", "Al", "NULL"])
    t = s.type.copy() + 1
    t[5] = 3                       # atom 5 (and its images) not handled by this style
    t[s.owner == 5] = 3
    off = s.nbr_off
    lists = [s.nbr_idx[off[i]:off[i + 1]] for i in range(s.nlocal)]
    e, f, vir, ea = g.compute_lammps(s.nlocal, s.nall, s.x, t, np.arange(s.nlocal),
                                     np.diff(off), lists)
    assert ea[5] == 0.0
    tt = s.type.copy()
    tt[s.owner == 5] = -1
    s2 = type(s)(**{**s.__dict__, "type": tt})
    ref = o.compute(s2)
    assert abs(e - ref["energy"]) <= REL * abs(ref["energy"])
    assert rel_err(f, ref["f_all"]) <= REL
    # a subset of centres via ilist
    g.set_type_map(["Ti", "Al"])
    il = np.arange(0, s.nlocal, 3)
    e2, f2, _, ea2 = g.compute_lammps(s.nlocal, s.nall, s.x, s.type + 1, il, np.diff(off), lists)
    full = o.compute(s)
    assert e2 == pytest.approx(full["eatom"][il].sum(), rel=1e-10)


@pytest.mark.parametrize("prec,ftol", [(mlipg.PREC_FP64, 1e-12), (mlipg.PREC_MIXED, 1e-12)])
def test_repeatability(potdir, prec, ftol):
    """Energies are bitwise reproducible (fixed summation order; the mixed
    path's adjoint sums are exact fixed point); forces differ between runs
    only through the order of the FP64 force scatter, at FP64 rounding."""
    g = mlipg.Potential(potdir["gtinv-820"], prec)
    s = build_system(structure("structure.lammps"), g.cutoff, skin=2.0)
    a = g.compute(s)
    b = g.compute(s)
    assert a["energy"] == b["energy"]
    np.testing.assert_array_equal(a["eatom"], b["eatom"])
    scale = np.abs(a["f_all"]).max()
    np.testing.assert_allclose(a["f_all"], b["f_all"], rtol=0, atol=ftol * scale)


@pytest.mark.parametrize("ncent", [1, 2, 32])
def test_device_api_totals_match_per_atom(potdir, ncent):
    """out8 (energy, virial) of mlipg_compute_device equals the per-atom sums."""
    import torch
    g = mlipg.Potential(potdir["gtinv-820"], mlipg.PREC_FP64)
    s = build_system(structure("structure.lammps"), g.cutoff, skin=2.0)
    dev = torch.device("cuda")
    x4 = np.zeros((s.nall, 4))
    x4[:, :3] = s.x
    x4[:, 3] = s.type
    cents = list(range(ncent))
    offs = np.zeros(ncent + 1, dtype=np.int32)
    idx = []
    for k, i in enumerate(cents):
        lst = s.nbr_idx[s.nbr_off[i]:s.nbr_off[i + 1]]
        idx.append(lst)
        offs[k + 1] = offs[k] + len(lst)
    t = {k: torch.from_numpy(v).to(dev) for k, v in
         dict(x4=x4, c=np.array(cents, np.int32), o=offs, i=np.concatenate(idx)).items()}
    f = torch.zeros((s.nall, 3), dtype=torch.float64, device=dev)
    out = torch.full((8,), -7.0, dtype=torch.float64, device=dev)
    ea = torch.zeros(ncent, dtype=torch.float64, device=dev)
    for _ in range(2):
        g.compute_device(ncent, t["x4"].data_ptr(), t["c"].data_ptr(), t["o"].data_ptr(),
                         t["i"].data_ptr(), f.data_ptr(), out.data_ptr(), eatom=ea.data_ptr(),
                         nb_cap=512)
    torch.cuda.synchronize()
    ref = Oracle(potdir["gtinv-820"]).compute_centers(s, np.array(cents))
    assert out[0].item() == pytest.approx(ea.sum().item(), rel=1e-12)
    assert out[0].item() == pytest.approx(ref["energy"], rel=1e-10)
    v = out.cpu().numpy()[1:7]
    # kernel order xx yy zz yz zx xy vs oracle's LAMMPS order xx yy zz xy xz yz
    np.testing.assert_allclose(v[[0, 1, 2, 5, 4, 3]], ref["virial"], rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("prec", [mlipg.PREC_FP64, mlipg.PREC_FP64_NATIVE])
def test_sparse_neighbourhoods(tmp_path, prec):
    """Dilute random cells (0.004 atoms per cubic angstrom: a few neighbours
    each, mostly near the cutoff) make the order parameters, and with them
    the adjoint flushes, orders of magnitude smaller than in a dense cell:
    the double-float kernel's fixed-point scale adapts to them (and caps at
    2^100) without leaving FP64 parity."""
    p = str(tmp_path / "sparse.mlip")
    workload_potential(p, "triclinic-batch", seed=6)
    g = mlipg.Potential(p, prec)
    o = Oracle(p, threads=8)
    rng = np.random.default_rng(21)
    for n in (6, 20):
        cell = random_triclinic_cell(n, 0.004, 2, rng, min_dist=3.0)
        s = build_system(cell, o.cutoff, skin=1.0)
        got = g.compute(s)
        check_fp64(got, o.compute(s), s)
        assert g.device_status() == 0
    g.close()


SINGLE_TUPLE = {
    # more than three elements: every irreps runs one element tuple per unit
    "4el-order3": dict(elements=["A", "B", "C", "D"], maxl=4, order=3, gtinv_maxl=[4, 2]),
    # orders 5 and 6 (the table's l <= 1 terms): single-tuple units beside the
    # batched ones of orders <= 4
    "2el-order6": dict(elements=["A", "B"], maxl=4, order=6, gtinv_maxl=[4, 2, 2, 1, 1]),
}


@pytest.mark.parametrize("spec", sorted(SINGLE_TUPLE))
def test_single_tuple_units(tmp_path, spec):
    """The single-tuple units (run_unit: any order up to 6, any number of
    elements) in every precision: FP64 and all-FP64 against the oracle at
    1e-10, mixed within the stated bounds."""
    from mlipg.potential import gaussian_params, write_potential
    h = SINGLE_TUPLE[spec]
    path = str(tmp_path / (spec + ".mlip"))
    ne = len(h["elements"])
    write_potential(path, h["elements"], 5.0, gaussian_params(6, 5.0), 3, 2, h["maxl"],
                    h["order"], h["gtinv_maxl"], [0] * (h["order"] - 1),
                    masses=[27.0] * ne, seed=13)
    rng = np.random.default_rng(17)
    cell = random_types(jitter(fcc_cell(2, 2, 2, 3.6), 0.05, rng), ne, rng)
    o = Oracle(path, threads=16)
    s = build_system(cell, o.cutoff, skin=1.0)
    ref = o.compute(s)
    for prec in (mlipg.PREC_FP64, mlipg.PREC_FP64_NATIVE):
        g = mlipg.Potential(path, prec)
        check_fp64(g.compute(s), ref, s)
        assert g.device_status() == 0
        g.close()
    mix = mlipg.Potential(path, mlipg.PREC_MIXED).compute(s)
    F, Fr = s.fold_forces(mix["f_all"]), s.fold_forces(ref["f_all"])
    assert np.sqrt(np.mean((F - Fr) ** 2)) <= 1e-4
    assert abs(mix["energy"] - ref["energy"]) <= mixed_energy_bound(o, s)
