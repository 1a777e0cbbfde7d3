"""The CPU oracle against the reference's golden vectors (no GPU needed).

Pins: step-0 thermo of the reference's regression logs (energy to the 8
printed digits, pressure and stress tensor to their printed digits), the
triclinic / conventional 64-atom cells, force sums, and finite differences.
"""
import numpy as np
import pytest

from conftest import structure
from mlipg.structures import build_system
from oracle import Oracle

CASES = [("gtinv-197", "gtinv-197"), ("gtinv-820", "gtinv-820"), ("gtinv-434", "gtinv-434"),
         # the radial-only descriptor (pair_style mlip_pair of the reference)
         ("pair-60", "pair-60"), ("pair-17", "pair-17")]


@pytest.mark.parametrize("pot,log", CASES)
def test_step0_energy_pressure(potdir, golden, pot, log):
    o = Oracle(potdir[pot], threads=4)
    s = build_system(structure("structure.lammps"), o.cutoff, skin=2.0)
    r = o.compute(s)
    g = golden["thermo_step0"][log]
    assert r["energy"] == pytest.approx(g["E_pair"], abs=6e-6)
    assert s.pressure(r["virial"]) == pytest.approx(g["Press"], abs=6e-5 * 10)
    assert np.abs(s.fold_forces(r["f_all"]).sum(0)).max() < 1e-10


def test_stress_tensor_gtinv197(potdir, golden):
    o = Oracle(potdir["gtinv-197"], threads=4)
    s = build_system(structure("structure.lammps"), o.cutoff, skin=2.0)
    p = s.pressure_tensor(o.compute(s)["virial"])
    g = golden["thermo_step0"]["gtinv-197-stress"]
    ref = [g[k] for k in ["Pxx", "Pyy", "Pzz", "Pxy", "Pxz", "Pyz"]]
    np.testing.assert_allclose(p, ref, atol=2e-3, rtol=0)


@pytest.mark.parametrize("name", ["structure_00064_conventional.lammps",
                                  "structure_00064_triclinic.lammps"])
def test_conv64_and_triclinic(potdir, golden, name):
    o = Oracle(potdir["gtinv-197"], threads=8)
    s = build_system(structure(name), o.cutoff, skin=2.0)
    r = o.compute(s)
    g = golden["thermo_step0"]["gtinv-197-conv64"]
    assert r["energy"] == pytest.approx(g["E_pair"], abs=6e-6)
    # the reference's triclinic test allows 0.1 bar (test/regression/regression.py:85)
    assert s.pressure(r["virial"]) == pytest.approx(g["Press"], abs=0.1)
    if "conventional" in name:
        # perfect lattice: log.lammps.gtinv-197.conv64 reports Fmax 2.7e-14
        assert np.abs(s.fold_forces(r["f_all"])).max() < 1e-9


def test_model_structure_matches_reference(potdir, golden):
    import hashlib
    for pot, fp in golden["model"].items():
        o = Oracle(potdir[pot])
        for k in ["n_irreps", "n_terms", "ITC", "D", "n_coeffs", "T", "F"]:
            assert o.info[k] == fp[k], (pot, k)
        itc = o.itc_list().astype(np.int64)
        poly = o.poly_list().astype(np.int64)
        assert hashlib.sha256(itc.tobytes()).hexdigest() == fp["itc_sha256"]
        assert hashlib.sha256(poly.tobytes()).hexdigest() == fp["poly_sha256"]


def test_spherical_harmonics_match_reference_host_twin(golden, potdir, tmp_path):
    # a minimal potential with max_l = 12 to expose the l <= 12 harmonics
    from mlipg.potential import write_potential
    p = tmp_path / "l12.mlip"
    write_potential(str(p), ["A"], cutoff=6.0, params=[(1.0, 0.0)], model_type=3, maxp=1,
                    maxl=12, gtinv_order=2, gtinv_maxl=[12], gtinv_sym=[0], coeffs=None)
    o = Oracle(str(p))
    for case in golden["sph_lmax12"]["cases"]:
        y, dx, dy, dz = o.sph(case["dir"])
        for got, key in [(y, "ylm"), (dx, "dx"), (dy, "dy"), (dz, "dz")]:
            ref = np.array(case[key])
            ref = ref[0::2] + 1j * ref[1::2]
            np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-13)


def test_radial_kat(tmp_path):
    # test/test_mlip_features.cpp:80-100: r=2, rc=4, beta=ln2, mu in {0, 2}
    from mlipg.potential import write_potential
    p = tmp_path / "kat.mlip"
    write_potential(str(p), ["A"], cutoff=4.0, params=[(np.log(2.0), 0.0), (np.log(2.0), 2.0)],
                    model_type=3, maxp=1, maxl=0, gtinv_order=2, gtinv_maxl=[0],
                    gtinv_sym=[0], coeffs=None)
    fn, _ = Oracle(str(p)).radial(2.0)
    np.testing.assert_allclose(fn, [0.03125, 0.5], rtol=1e-15)


@pytest.mark.parametrize("pot", ["gtinv-820", "pair-17"])
def test_finite_difference_forces_and_virial(potdir, pot):
    o = Oracle(potdir[pot], threads=8)
    cell = structure("structure.lammps")
    s = build_system(cell, o.cutoff, skin=1.0)
    r = o.compute(s)
    F = s.fold_forces(r["f_all"])
    h = 1e-5
    rng = np.random.default_rng(0)
    for _ in range(3):
        a, k = int(rng.integers(cell.natoms)), int(rng.integers(3))
        e = []
        for sgn in (1, -1):
            c2 = structure("structure.lammps")
            c2.positions[a, k] += sgn * h
            e.append(o.compute(build_system(c2, o.cutoff, skin=1.0))["energy"])
        assert F[a, k] == pytest.approx(-(e[0] - e[1]) / (2 * h), abs=2e-5)
    # virial from a homogeneous strain: W_xx = -dE/d eps_xx
    e = []
    for sgn in (1, -1):
        c2 = structure("structure.lammps")
        m = np.eye(3)
        m[0, 0] += sgn * h
        c2.lattice = c2.lattice @ m
        c2.positions = c2.positions @ m
        e.append(o.compute(build_system(c2, o.cutoff, skin=1.0))["energy"])
    assert r["virial"][0] == pytest.approx(-(e[0] - e[1]) / (2 * h), rel=1e-5, abs=1e-4)


@pytest.mark.parametrize("maxl, order, gl", [(20, 2, [20]), (16, 3, [16, 6]), (20, 3, [20, 4])])
def test_high_l_models(tmp_path, maxl, order, gl):
    """Potentials with l up to 20 (the coupling table's limit): the library
    builds the model and a schedule for every autotuner tile shape with the
    coefficient count of the file, and the oracle's forces at l = 20 match
    finite differences of its energy."""
    import mlipg
    from mlipg.potential import gaussian_params, write_potential
    from mlipg.structures import fcc_cell, jitter
    path = str(tmp_path / "high_l.mlip")
    nc = write_potential(path, ["A"], 5.0, gaussian_params(6, 5.0), 1, 1, maxl, order, gl,
                         [0] * len(gl), masses=[27.0], seed=2)
    g = mlipg.Potential(path, mlipg.PREC_MIXED)
    for chunk in (12, 24, 48):
        for worder in (0, 1, 2):
            g.set_tiling(chunk, worder, 1)
    g.close()
    o = Oracle(path, threads=8)
    assert o.info["L"] == maxl and o.info["n_coeffs"] == nc
    rng = np.random.default_rng(3)
    cell = jitter(fcc_cell(2, 2, 2, 4.05), 0.05, rng)
    r = o.compute(build_system(cell, o.cutoff, skin=1.0))
    F = build_system(cell, o.cutoff, skin=1.0).fold_forces(r["f_all"])
    h = 1e-5
    for a, k in ((0, 0), (5, 2)):
        e = []
        for sgn in (1, -1):
            c2 = jitter(fcc_cell(2, 2, 2, 4.05), 0.05, np.random.default_rng(3))
            c2.positions[a, k] += sgn * h
            e.append(o.compute(build_system(c2, o.cutoff, skin=1.0))["energy"])
        assert F[a, k] == pytest.approx(-(e[0] - e[1]) / (2 * h), abs=1e-6)


@pytest.mark.parametrize("pot", ["gtinv-820", "gtinv-434"])
def test_training_features_identities(potdir, pot):
    """The oracle's training features (the reference's prepare_features:
    structural, polynomial, force and stress features) reproduce its energy,
    forces and virial through the linear model: E = sum_i P_i . w,
    F = FF . w, virial = SF . w."""
    o = Oracle(potdir[pot], threads=8)
    s = build_system(structure("structure.lammps"), o.cutoff, skin=2.0)
    ft = o.features(s)
    ref = o.compute(s)
    w = o.coefficients()
    assert ft["p"].sum(0) @ w == pytest.approx(ref["energy"], rel=1e-12)
    np.testing.assert_allclose(ft["p"] @ w, ref["eatom"], rtol=0, atol=1e-10)
    F = np.einsum("ipk,p->ik", ft["ff"], w)
    Fr = s.fold_forces(ref["f_all"])
    assert np.abs(F - Fr).max() <= 1e-11 * np.abs(Fr).max()
    v = w @ ft["sf"]                       # xx yy zz yz zx xy
    vr = ref["virial"]                     # xx yy zz xy xz yz
    assert np.abs(v[[0, 1, 2, 5, 4, 3]] - vr).max() <= 1e-10 * np.abs(vr).max()
